"""CPU restatement of the learned-guess network (test infrastructure only: the checker of the
U-Net kernels in drd_application_gb300/csrc/drd_unet.cu, never a product path).

The network has no counterpart in the reference (DRD_application's solves start from the
previous step's field, microfluidics_complex_domain/PhSolve.f90:62-74); this file restates
the library's own definition so that its forward pass and gradients can be checked:

  enc l (l = 0..3): conv3x3(C_in_l -> C_l) + ReLU, conv3x3(C_l -> C_l) + ReLU = e_l,
                    2x2 average pool between levels (C_l = 32 << l)
  dec l (l = 2..0): conv3x3(up2(d_{l+1}) -> C_l) + ReLU, concatenated with e_l,
                    conv3x3(2C_l -> C_l) + ReLU, conv3x3(C_l -> C_l) + ReLU = d_l   (d_3 = e_3)
  out:              1x1 conv(C_0 -> out_ch)
  loss:             mean squared error over the caller's H x W grid

on the grid padded to multiples of 8 (input zero outside H x W).  With `rounding=True` the
values are rounded to bfloat16 (round to nearest even) where the kernels store BF16: the
packed input, the 3x3 weights, every stored activation, the pooled maps and the
pre-activation gradients that feed the tensor-core kernels.  With `rounding=False` everything
is float64, which is what the finite-difference checks of this file's backward pass use.
"""
import numpy as np

LEVELS = 4
BASE = 32
CIN_PAD = 16


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layer_table():
    """(cin, cout, level, up) of the 17 3x3 layers in parameter order."""
    L = []
    for l in range(LEVELS):
        L.append((CIN_PAD if l == 0 else BASE << (l - 1), BASE << l, l, 0))
        L.append((BASE << l, BASE << l, l, 0))
    for l in range(LEVELS - 2, -1, -1):
        L.append((BASE << (l + 1), BASE << l, l, 1))
        L.append((2 * BASE << l, BASE << l, l, 0))
        L.append((BASE << l, BASE << l, l, 0))
    return L


def param_count(out_ch):
    return sum(9 * ci * co + co for ci, co, _, _ in layer_table()) + out_ch * BASE + out_ch


def unpack(params, out_ch):
    """Views (w[9][cout][cin], b[cout]) per layer, and (wo[out][32], bo[out])."""
    p = np.asarray(params, dtype=np.float64)
    off, W = 0, []
    for ci, co, _, _ in layer_table():
        w = p[off:off + 9 * co * ci].reshape(9, co, ci)
        off += 9 * co * ci
        W.append((w, p[off:off + co]))
        off += co
    wo = p[off:off + out_ch * BASE].reshape(out_ch, BASE)
    off += out_ch * BASE
    bo = p[off:off + out_ch]
    off += out_ch
    assert off == p.size, (off, p.size)
    return W, wo, bo


def _shift(x, dy, dx):
    """y[:, i, j] = x[:, i + dy, j + dx] with zeros outside (NHWC)."""
    B, H, W, C = x.shape
    y = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    y[:, ys:ye, xs:xe] = x[:, ys + dy:ye + dy, xs + dx:xe + dx]
    return y


def _up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def _up_bwd(d):
    B, H, W, C = d.shape
    return d.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def _pool(x):
    B, H, W, C = x.shape
    return 0.25 * x.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


class UNetOracle:
    def __init__(self, H, W, in_ch, out_ch, rounding=True):
        self.H0, self.W0, self.cin, self.cout = H, W, in_ch, out_ch
        self.Hp, self.Wp = -(-H // 8) * 8, -(-W // 8) * 8
        self.rounding = rounding

    def _r(self, a):
        return bf16(a) if self.rounding else np.asarray(a, dtype=np.float64)

    def _conv(self, x, w, b, up):
        xin = _up(x) if up else x
        out = np.zeros(xin.shape[:3] + (w.shape[1],))
        for tap in range(9):
            out += _shift(xin, tap // 3 - 1, tap % 3 - 1) @ self._r(w[tap]).T
        return np.maximum(out + b, 0.0)

    def forward(self, params, x):
        """x: (B, in_ch, H, W).  Returns y (B, out_ch, H, W) and the activations."""
        Wl, wo, bo = unpack(params, self.cout)
        B = x.shape[0]
        xin = np.zeros((B, self.Hp, self.Wp, CIN_PAD))
        xin[:, :self.H0, :self.W0, :self.cin] = np.transpose(x, (0, 2, 3, 1))
        xin = self._r(xin)
        a = {"xin": xin}
        h = xin
        for l in range(LEVELS):
            a[f"ea{l}"] = self._r(self._conv(h, *Wl[2 * l], 0))
            a[f"e{l}"] = self._r(self._conv(a[f"ea{l}"], *Wl[2 * l + 1], 0))
            if l < LEVELS - 1:
                a[f"pool{l + 1}"] = self._r(_pool(a[f"e{l}"]))
                h = a[f"pool{l + 1}"]
        below = a[f"e{LEVELS - 1}"]
        for k, l in enumerate(range(LEVELS - 2, -1, -1)):
            li = 8 + 3 * k
            a[f"dup{l}"] = self._r(self._conv(below, *Wl[li], 1))
            a[f"cat{l}"] = np.concatenate([a[f"dup{l}"], a[f"e{l}"]], axis=3)
            a[f"db{l}"] = self._r(self._conv(a[f"cat{l}"], *Wl[li + 1], 0))
            a[f"d{l}"] = self._r(self._conv(a[f"db{l}"], *Wl[li + 2], 0))
            below = a[f"d{l}"]
        d0 = a["d0"][:, :self.H0, :self.W0]
        y = d0 @ wo.T + bo
        return np.transpose(y, (0, 3, 1, 2)), a

    # -------------------------------------------------------------------------------------
    def _conv_bwd(self, xin_eff, G, w):
        """Weight, bias and input gradients of one 3x3 layer (input as the conv reads it)."""
        dw = np.zeros_like(w)
        for tap in range(9):
            xs = _shift(xin_eff, tap // 3 - 1, tap % 3 - 1)
            dw[tap] = np.einsum("bhwo,bhwi->oi", G, xs)
        db = G.sum(axis=(0, 1, 2))
        dx = np.zeros(xin_eff.shape)
        for tap in range(9):
            dx += _shift(G, -(tap // 3 - 1), -(tap % 3 - 1)) @ self._r(w[tap])
        return dw, db, dx

    def gradients(self, params, x, target):
        """Loss and flat parameter gradient, in the kernels' order of operations."""
        Wl, wo, bo = unpack(params, self.cout)
        y, a = self.forward(params, x)
        n = y.size
        loss = float(((y - target) ** 2).sum() / n)
        dy = 2.0 * (y - target) / n  # (B, out, H0, W0)
        B = x.shape[0]
        dyp = np.zeros((B, self.Hp, self.Wp, self.cout))
        dyp[:, :self.H0, :self.W0] = np.transpose(dy, (0, 2, 3, 1))
        grads = [None] * 17
        dwo = np.einsum("bhwo,bhwc->oc", dyp, a["d0"])
        dbo = dyp.sum(axis=(0, 1, 2))
        r = self._r
        G = r((a["d0"] > 0) * (dyp @ wo))
        below_name = {2: f"e{LEVELS - 1}", 1: "d2", 0: "d1"}
        # decoder, top level first
        dcat = {}
        for l in range(0, LEVELS - 1):
            li = 8 + 3 * (LEVELS - 2 - l)
            C = BASE << l
            dw, db, dx = self._conv_bwd(a[f"db{l}"], G, Wl[li + 2][0])
            grads[li + 2] = (dw, db)
            G = r((a[f"db{l}"] > 0) * dx)
            dw, db, dx = self._conv_bwd(a[f"cat{l}"], G, Wl[li + 1][0])
            grads[li + 1] = (dw, db)
            dcat[l] = dx
            G = r((a[f"cat{l}"][..., :C] > 0) * dx[..., :C])
            below = a[below_name[l]]
            dw, db, dx = self._conv_bwd(_up(below), G, Wl[li][0])
            grads[li] = (dw, db)
            G = r((below > 0) * _up_bwd(dx))
        # encoder, bottom level first
        for l in range(LEVELS - 1, -1, -1):
            dw, db, dx = self._conv_bwd(a[f"ea{l}"], G, Wl[2 * l + 1][0])
            grads[2 * l + 1] = (dw, db)
            G = r((a[f"ea{l}"] > 0) * dx)
            xin = a["xin"] if l == 0 else a[f"pool{l}"]
            dw, db, dx = self._conv_bwd(xin, G, Wl[2 * l][0])
            grads[2 * l] = (dw, db)
            if l == 0:
                break
            Cp = BASE << (l - 1)
            dpool = dx
            e = a[f"e{l - 1}"]
            G = r((e > 0) * (dcat[l - 1][..., Cp:] + 0.25 * _up(dpool)))
        flat = []
        for dw, db in grads:
            flat.append(dw.ravel())
            flat.append(db)
        flat.append(dwo.ravel())
        flat.append(dbo)
        return loss, np.concatenate(flat)

    def loss(self, params, x, target):
        y, _ = self.forward(params, x)
        return float(((y - target) ** 2).sum() / y.size)


def he_init(out_ch, in_ch, seed):
    """He-normal weights of the same shapes (numpy's generator, for oracle-only checks)."""
    rng = np.random.default_rng(seed)
    p = []
    for ci, co, _, _ in layer_table():
        real = in_ch if ci == CIN_PAD else ci
        w = rng.standard_normal((9, co, ci)) * np.sqrt(2.0 / (9 * real))
        if ci == CIN_PAD:
            w[:, :, in_ch:] = 0.0
        p += [w.ravel(), np.zeros(co)]
    p += [rng.standard_normal(out_ch * BASE) * 0.1 * np.sqrt(2.0 / BASE), np.zeros(out_ch)]
    return np.concatenate(p)
