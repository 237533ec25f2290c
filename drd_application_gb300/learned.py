"""The learned initial guess of the CH solve: the U-Net of csrc/drd_unet.cu over the C-ABI,
the training pairs the solver itself emits, the training loop and the guess.

System.  PhSolve solves A mu = rhs (microfluidics_complex_domain/PhSolve.f90:62-74) starting
from the previous step's mu^n, the plain guess.  Over a run, the error of that guess is
e_n = mu^{n+1} - mu^n and its residual r_n = A e_n (A is the library's FP64 operator
DRD_OP_CH_MATVEC; the coefficients do not change within a run without particles).

Pairs.  With s_n = RMS(r_n), the network input is (r_n / s_n, bdr_ph, ph^n) on the nz x nr
interior (packed CH order: H = nz rows of W = nr) and the target is e_n / s_n.

Guess.  x0 = mu^n + s * net(r / s, bdr_ph, ph^n), r = b - A mu^n.  The plain guess stays the
fallback: when the learned guess's FP64 residual is not below the plain one's, the plain
guess is returned.  The solve that follows is unchanged, so the result meets the same FP64
tolerance either way; what the network changes is the iteration count.  The same holds with
the cubic extrapolation (guess_mode 3) as the base guess (base="cubic").

    python -m drd_application_gb300.learned [--base plain|cubic] [--train-seeds 24] ...

generates the pairs on the GPU, trains the network and reports, on held-out seeds, the
relative error of each guess and the mixed-precision CH iterations to the FP64 residual 1e-8.
"""
import ctypes as C
import time

import numpy as np

from . import abi, _lib
from .api import DRDContext

F = abi


class UNetError(RuntimeError):
    pass


def _p(a):
    """Pointer of a contiguous float32 numpy array or of a CUDA torch tensor."""
    if isinstance(a, np.ndarray):
        if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"]:
            raise ValueError("expected a C-contiguous float32 array")
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous() or str(a.dtype) != "torch.float32":
            raise ValueError("expected a contiguous float32 tensor")
        return C.c_void_p(a.data_ptr())
    raise TypeError(type(a))


class UNet:
    """drd_unet_*: the network on an H x W grid, in_ch -> out_ch fields, batches <= max_batch."""

    def __init__(self, H, W, in_ch=3, out_ch=1, max_batch=8, seed=0, lib=None):
        self.L = lib or _lib.load()
        h = C.c_void_p()
        rc = self.L.drd_unet_create(int(H), int(W), int(in_ch), int(out_ch), int(max_batch), int(seed), C.byref(h))
        if rc != 0:
            raise UNetError(f"drd_unet_create failed with {rc}")
        self.h, self.H, self.W, self.in_ch, self.out_ch, self.max_batch = h, H, W, in_ch, out_ch, max_batch
        self.nparam = int(self.L.drd_unet_param_count(h))

    def close(self):
        if getattr(self, "h", None):
            self.L.drd_unet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _rc(self, rc, what):
        if rc != 0:
            msg = self.L.drd_unet_last_error(self.h)
            raise UNetError(f"{what} failed with {rc}: {msg.decode() if msg else ''}")

    def get_params(self):
        p = np.zeros(self.nparam, dtype=np.float32)
        self._rc(self.L.drd_unet_get_params(self.h, _p(p)), "drd_unet_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.shape != (self.nparam,):
            raise ValueError(f"expected {self.nparam} parameters")
        self._rc(self.L.drd_unet_set_params(self.h, _p(p)), "drd_unet_set_params")

    def _batch(self, x, ch):
        b = x.shape[0]
        if tuple(x.shape[1:]) != (ch, self.H, self.W) or not 1 <= b <= self.max_batch:
            raise ValueError(f"expected (batch<={self.max_batch}, {ch}, {self.H}, {self.W}), got {tuple(x.shape)}")
        return b

    def forward(self, x, out=None):
        b = self._batch(x, self.in_ch)
        if out is None:
            out = np.zeros((b, self.out_ch, self.H, self.W), dtype=np.float32)
        self._rc(self.L.drd_unet_forward(self.h, b, _p(x), _p(out)), "drd_unet_forward")
        return out

    def gradients(self, x, target):
        b = self._batch(x, self.in_ch)
        self._batch(target, self.out_ch)
        loss = np.zeros(1, dtype=np.float32)
        g = np.zeros(self.nparam, dtype=np.float32)
        self._rc(self.L.drd_unet_gradients(self.h, b, _p(x), _p(target), _p(loss), _p(g)), "drd_unet_gradients")
        return float(loss[0]), g

    def train_step(self, x, target, lr):
        b = self._batch(x, self.in_ch)
        self._batch(target, self.out_ch)
        loss = np.zeros(1, dtype=np.float32)
        self._rc(self.L.drd_unet_train_step(self.h, b, _p(x), _p(target), C.c_float(lr), _p(loss)),
                 "drd_unet_train_step")
        return float(loss[0])


# ------------------------------------------------------------------------------------------
def _interior(a):
    return np.ascontiguousarray(a[1:-1, 1:-1])


def _rms(v):
    return float(np.sqrt(np.mean(v * v)))


def cubic_guess(hist):
    """4 mu^n - 6 mu^{n-1} + 4 mu^{n-2} - mu^{n-3} (guess_mode 3) from [mu^{n-3}, .., mu^n]."""
    return 4 * hist[-1] - 6 * hist[-2] + 4 * hist[-3] - hist[-4]


def ch_run_pairs(case, nsteps, warmup=0, precision=F.DRD_PREC_MIXED, base="plain"):
    """Runs warmup + nsteps steps of `case` on the GPU and returns the CH pairs of the last nsteps:
    dict(x=(n,3,nz,nr) float32 inputs, y=(n,1,nz,nr) float32 targets, s=(n,) scales,
    mu0=(n, nr*nz) base guesses, mu1=(n, nr*nz) solutions, b=(n, nr*nz) right-hand sides).
    base: "plain" (mu^n) or "cubic" (cubic_guess; needs warmup >= 3)."""
    if base == "cubic" and warmup < 3:
        raise ValueError("the cubic guess needs three earlier steps")
    P = case.params.copy()
    P.precision = precision
    nr, nz = P.nr, P.nz
    ctx = DRDContext(P)
    try:
        ctx.set_case(case)
        ctx.upload_state(case.state)
        bdr = _interior(case.coefs["bdr_ph"])
        t = 0.0
        mus, phs = [], []
        first = warmup - 3 if base == "cubic" else warmup
        for s in range(warmup + nsteps + 1):
            if s >= first:
                st = ctx.download_state([F.F_RMU, F.F_PH])
                mus.append(_interior(st[F.F_RMU]).reshape(-1))
                phs.append(_interior(st[F.F_PH]))
            if s == warmup + nsteps:
                break
            stats = ctx.step(s == 0, t)
            if stats.ch.info != 0:
                raise UNetError(f"CH solve did not converge at step {s} (info {stats.ch.info})")
            t += P.dt
        n, o = nsteps, 3 if base == "cubic" else 0
        X = np.zeros((n, 3, nz, nr), dtype=np.float32)
        Y = np.zeros((n, 1, nz, nr), dtype=np.float32)
        S = np.zeros(n)
        B = np.zeros((n, nr * nz))
        G = np.zeros((n, nr * nz))
        for k in range(n):
            j = k + o
            G[k] = cubic_guess(mus[j - 3:j + 1]) if base == "cubic" else mus[j]
            e = mus[j + 1] - G[k]
            r = ctx.op_apply(F.DRD_OP_CH_MATVEC, e, bdf=2)
            B[k] = ctx.op_apply(F.DRD_OP_CH_MATVEC, mus[j + 1], bdf=2)
            sc = max(_rms(r), 1e-300)
            S[k] = sc
            X[k, 0] = (r / sc).reshape(nz, nr)
            X[k, 1] = bdr
            X[k, 2] = phs[j]
            Y[k, 0] = (e / sc).reshape(nz, nr)
        return dict(x=X, y=Y, s=S, mu0=G, mu1=np.array(mus[o + 1:o + n + 1]), b=B)
    finally:
        ctx.close()


def concat_pairs(parts):
    return {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}


def train(net, data, steps, batch=8, lr=1e-3, lr_final=1e-4, seed=0, log_every=0):
    """Adam on random minibatches of `data` (dict x, y) with a geometric learning-rate decay.
    Returns the list of losses."""
    rng = np.random.default_rng(seed)
    n = data["x"].shape[0]
    losses = []
    batch = min(batch, net.max_batch, n)
    for it in range(steps):
        idx = rng.choice(n, size=batch, replace=False)
        rate = lr * (lr_final / lr) ** (it / max(steps - 1, 1))
        loss = net.train_step(np.ascontiguousarray(data["x"][idx]), np.ascontiguousarray(data["y"][idx]), rate)
        losses.append(loss)
        if log_every and (it % log_every == 0 or it == steps - 1):
            print(f"  train step {it}: loss {loss:.4e} lr {rate:.2e}", flush=True)
    return losses


def ch_guess(ctx, net, b, mu0, bdr, ph, judge="residual"):
    """The learned guess for A x = b from the base guess mu0 (packed), or mu0 itself when the
    learned one is judged worse.  judge: "residual" compares the FP64 residual norms ||b - A x||
    (the default), "precond" compares ||M^-1 r|| (M^-1 = PSolve_CG, an estimate of the error),
    "none" always takes the learned guess.  Returns (x0, used_learned, measure_base,
    measure_learned)."""
    nr, nz = ctx.nr, ctx.nz
    r = b - ctx.op_apply(F.DRD_OP_CH_MATVEC, mu0, bdf=2)
    sc = max(_rms(r), 1e-300)
    x = np.zeros((1, 3, nz, nr), dtype=np.float32)
    x[0, 0] = (r / sc).reshape(nz, nr)
    x[0, 1] = bdr
    x[0, 2] = ph
    y = net.forward(x)
    x0 = mu0 + sc * y[0, 0].reshape(-1).astype(np.float64)
    if judge == "none":
        return x0, True, 0.0, 0.0
    r1 = b - ctx.op_apply(F.DRD_OP_CH_MATVEC, x0, bdf=2)
    if judge == "precond":
        r = ctx.op_apply(F.DRD_OP_CH_PSOLVE, r, bdf=2)
        r1 = ctx.op_apply(F.DRD_OP_CH_PSOLVE, r1, bdf=2)
    n0, n1 = float(np.linalg.norm(r)), float(np.linalg.norm(r1))
    if not n1 < n0:
        return mu0.copy(), False, n0, n1
    return x0, True, n0, n1


def evaluate_ch(case, net, pairs, precision=F.DRD_PREC_MIXED, tol=1e-8, judge="residual"):
    """Iterations and wall time of the CH solves of `pairs` (from ch_run_pairs on `case`) to the
    FP64 relative residual `tol`, from the plain guess and from the learned one."""
    P = case.params.copy()
    P.precision = precision
    P.tol = tol
    ctx = DRDContext(P)
    try:
        ctx.set_case(case)
        bdr = _interior(case.coefs["bdr_ph"])
        out = dict(iters_plain=[], iters_learned=[], res_plain=[], res_learned=[], used=[], t_plain=[],
                   t_learned=[], t_guess=[], true_resid_plain=[], true_resid_learned=[])
        for k in range(pairs["b"].shape[0]):
            b, mu0 = pairs["b"][k], pairs["mu0"][k]
            ph = pairs["x"][k, 2]
            t0 = time.perf_counter()
            _, st = ctx.solve(F.DRD_SYS_CH, b, mu0)
            t1 = time.perf_counter()
            x0, used, n0, n1 = ch_guess(ctx, net, b, mu0, bdr, ph, judge)
            t2 = time.perf_counter()
            _, st2 = ctx.solve(F.DRD_SYS_CH, b, x0)
            t3 = time.perf_counter()
            out["iters_plain"].append(st.iter)
            out["iters_learned"].append(st2.iter)
            out["res_plain"].append(n0)
            out["res_learned"].append(n1)
            out["used"].append(used)
            out["t_plain"].append(t1 - t0)
            out["t_guess"].append(t2 - t1)
            out["t_learned"].append(t3 - t2)
            out["true_resid_plain"].append(st.true_resid)
            out["true_resid_learned"].append(st2.true_resid)
        return {k: np.array(v) for k, v in out.items()}
    finally:
        ctx.close()


# ------------------------------------------------------------------------------------------
# The learned blend inside the CH preconditioner.
#
# PSolve_CG (microfluidics_complex_domain/PhSolve.f90:296-313) inverts the CH operator with unit
# mobility everywhere.  The library's blended form y = q + w (x - q) (drd_set_ch_blend) adds the
# identity where the mobilities vanish, which is what the operator tends to in the solid.  The
# best per-cell w of a geometry is fitted on the GPU from Rademacher probes
# (drd_ch_blend_probe); the network learns the map from the mobility fields to that fit, so a
# geometry gets its weights from one forward pass, and the network's fit, trained on many
# geometries, carries less probe noise than a fit from one geometry's probes.
#
# Inputs, 3 channels on the nz x nr interior: (log10 M0)/12 + 1, (log10 Mi)/12 + 1 (M clamped to
# >= 1e-12) and M0.  Target: 1 + ln(w + BLEND_FLOOR) / ln(1/BLEND_FLOOR), so that an error in the
# output is a relative error in w, and the fluid's w = 0 comes out within a few 1e-5 of zero (a
# weight of 1e-2 in the fluid would undo most of the gain).

BLEND_FLOOR = 1e-4
_BLEND_SCALE = float(np.log(1.0 / BLEND_FLOOR))


def blend_features(M0, Mi):
    """(3, nz, nr) float32 network input from the CELL mobility fields."""
    m0, mi = _interior(M0), _interior(Mi)
    x = np.empty((3,) + m0.shape, dtype=np.float32)
    x[0] = np.log10(np.maximum(m0, 1e-12)) / 12.0 + 1.0
    x[1] = np.log10(np.maximum(mi, 1e-12)) / 12.0 + 1.0
    x[2] = m0
    return x


def blend_target(w):
    """Network target of weights w (any shape)."""
    return (1.0 + np.log(np.asarray(w, dtype=np.float64) + BLEND_FLOOR) / _BLEND_SCALE).astype(np.float32)


def blend_weights(y):
    """Weights in [0, 1] (FP64) from network outputs y."""
    y = np.asarray(y, dtype=np.float64)
    return np.clip(np.exp((y - 1.0) * _BLEND_SCALE) - BLEND_FLOOR, 0.0, 1.0)


def blend_pairs(cases, nprobe=64, seed=0):
    """Probe-fitted blend weights of each case's mobilities (one GPU context, the cases share
    their grid and parameters): dict(x=(n,3,nz,nr) inputs, y=(n,1,nz,nr) targets, w=(n, nr*nz)
    weights)."""
    P = cases[0].params.copy()
    ctx = DRDContext(P)
    try:
        X, Y, W = [], [], []
        for k, case in enumerate(cases):
            M0, Mi = case.coefs["M0"], case.coefs["Mi"]
            ctx.set_coefs(ph_M_0=M0, ph_M_inner=Mi)
            w = ctx.ch_blend_probe(nprobe, seed + k, install=False)
            X.append(blend_features(M0, Mi))
            Y.append(blend_target(w).reshape(1, P.nz, P.nr))
            W.append(w)
        return dict(x=np.stack(X), y=np.stack(Y), w=np.stack(W))
    finally:
        ctx.close()


def flip_augment(data):
    """Adds the mirror images along x, along z and along both (the CH operator, its Neumann
    sides and the DCT-I preconditioner are symmetric under both reflections)."""
    xs, ys = [data["x"]], [data["y"]]
    for ax in ((-1,), (-2,), (-2, -1)):
        xs.append(np.ascontiguousarray(np.flip(data["x"], ax)))
        ys.append(np.ascontiguousarray(np.flip(data["y"], ax)))
    return dict(x=np.concatenate(xs), y=np.concatenate(ys))


def learned_blend(net, M0, Mi):
    """The network's blend weights (packed nr*nz, FP64) for the CELL mobility fields."""
    x = blend_features(M0, Mi)[None]
    y = net.forward(np.ascontiguousarray(x))
    return blend_weights(y[0, 0]).reshape(-1)


def train_blend(train_cases, steps=800, nprobe=64, batch=8, lr=1e-3, lr_final=1e-4, seed=0, log_every=0):
    """Fits the blend weights of `train_cases` on the GPU and trains a network on them (with
    mirror images).  Returns (net, info)."""
    t0 = time.perf_counter()
    data = flip_augment(blend_pairs(train_cases, nprobe, seed=1 << 20))
    t1 = time.perf_counter()
    P = train_cases[0].params
    net = UNet(P.nz, P.nr, 3, 1, max_batch=batch, seed=seed)
    losses = train(net, data, steps, batch=batch, lr=lr, lr_final=lr_final, seed=seed, log_every=log_every)
    t2 = time.perf_counter()
    info = {"geometries": len(train_cases), "samples": int(data["x"].shape[0]), "probes": nprobe,
            "adam_steps": steps, "data_s": t1 - t0, "train_s": t2 - t1,
            "loss_first": float(np.mean(losses[:10])), "loss_last": float(np.mean(losses[-20:]))}
    return net, info


def evaluate_blend(case, weights, warmup=4, steps=8):
    """Steps of `case` (mixed, the case's guess mode) for each entry of `weights` (name -> packed
    weights, or None for PSolve_CG alone): mean CH iterations and CH solve seconds over the last
    `steps` steps, and the largest FP64 true residual."""
    out = {}
    for name, w in weights.items():
        P = case.params.copy()
        P.precision = F.DRD_PREC_MIXED
        ctx = DRDContext(P)
        try:
            ctx.set_case(case)
            ctx.upload_state(case.state)
            if w is not None:
                ctx.set_ch_blend(w)
            its, secs, tr, ok = [], [], [], 0
            t = 0.0
            for k in range(warmup + steps):
                st = ctx.step(k == 0, t)
                t += P.dt
                if k >= warmup:
                    its.append(st.ch.iter)
                    secs.append(st.ch.seconds)
                    tr.append(st.ch.true_resid)
                    ok += int(st.ch.info == 0 and st.ch.true_resid <= P.tol)
            out[name] = {"ch_iters": float(np.mean(its)), "ch_solve_ms": 1e3 * float(np.mean(secs)),
                         "max_true_resid": float(np.max(tr)), "converged": f"{ok}/{steps}"}
        finally:
            ctx.close()
    return out


def blend_main(a):
    from .workloads import make_case

    train_cases = [make_case("c2", seed=1000 + s, nr=a.nr, nz=a.nz, precision=F.DRD_PREC_MIXED, guess_mode=3)
                   for s in range(a.train_seeds)]
    net, info = train_blend(train_cases, steps=a.steps, nprobe=a.probes, log_every=max(a.steps // 8, 1))
    print(f"blend network: {info}", flush=True)
    if a.save:
        np.save(a.save, net.get_params())
    for s in range(a.eval_seeds):
        case = make_case("c2", seed=2000 + s, nr=a.nr, nz=a.nz, precision=F.DRD_PREC_MIXED, guess_mode=3)
        ref = blend_pairs([case], a.probes, seed=7)
        w_net = learned_blend(net, case.coefs["M0"], case.coefs["Mi"])
        err = float(np.sqrt(np.mean((blend_target(w_net) - blend_target(ref["w"][0])) ** 2)))
        ev = evaluate_blend(case, {"PSolve_CG": None, "probe fit": ref["w"][0], "learned": w_net})
        print(f"held-out seed {2000 + s}: target-space RMS error of the learned weights {err:.3f}", flush=True)
        for name, r in ev.items():
            print(f"  {name:10s} CH iterations {r['ch_iters']:6.1f}  CH solve {r['ch_solve_ms']:6.2f} ms  "
                  f"converged {r['converged']}  max true residual {r['max_true_resid']:.2e}", flush=True)
    net.close()


def _layers():
    """(cin, cout, level) of the 17 3x3 layers, as drd_unet_create builds them."""
    L = []
    for l in range(4):
        L.append((16 if l == 0 else 32 << (l - 1), 32 << l, l))
        L.append((32 << l, 32 << l, l))
    for l in (2, 1, 0):
        L += [(32 << (l + 1), 32 << l, l), (64 << l, 32 << l, l), (32 << l, 32 << l, l)]
    return L


def conv_flops(Hp, Wp, batch, train=True):
    """Tensor-core FLOPs (2 per multiply-add) of the 3x3 layers on the padded Hp x Wp grid for
    one forward pass, or with train=True one training step (forward, data gradient, weight
    gradient; the first layer has no data gradient)."""
    total = 0.0
    for i, (ci, co, l) in enumerate(_layers()):
        f = 2.0 * 9 * ci * co * (Hp >> l) * (Wp >> l) * batch
        total += f * ((2 if i == 0 else 3) if train else 1)
    return total


def main(argv=None):
    import argparse

    from .workloads import make_case

    ap = argparse.ArgumentParser(description="train and evaluate the learned CH guess on C2 runs")
    ap.add_argument("--base", choices=("plain", "cubic"), default="plain")
    ap.add_argument("--train-seeds", type=int, default=24, help="C2 geometries 1000.. used for training")
    ap.add_argument("--per-seed", type=int, default=12, help="pairs per training run")
    ap.add_argument("--warmup", type=int, default=10, help="steps before the first pair of a run")
    ap.add_argument("--steps", type=int, default=1500, help="Adam steps (batch 8)")
    ap.add_argument("--eval-seeds", type=int, default=2, help="held-out geometries 2000..")
    ap.add_argument("--eval-pairs", type=int, default=8)
    ap.add_argument("--nr", type=int, default=420)
    ap.add_argument("--nz", type=int, default=180)
    ap.add_argument("--save", default=None, help="write the trained parameters (.npy)")
    ap.add_argument("--lowpass", type=float, nargs="*", default=[],
                    help="also evaluate the learned and the exact corrections with only the lowest fraction "
                         "of their DCT-II modes kept along each axis (evaluation only)")
    ap.add_argument("--blend", action="store_true",
                    help="train and evaluate the learned blend of the CH preconditioner instead of the guess")
    ap.add_argument("--probes", type=int, default=64, help="Rademacher probes per geometry (--blend)")
    a = ap.parse_args(argv)
    if a.blend:
        return blend_main(a)
    t0 = time.perf_counter()
    parts = [ch_run_pairs(make_case("c2", seed=1000 + s, nr=a.nr, nz=a.nz), a.per_seed, a.warmup, base=a.base)
             for s in range(a.train_seeds)]
    data = concat_pairs(parts)
    t1 = time.perf_counter()
    net = UNet(a.nz, a.nr, 3, 1, max_batch=8, seed=0)
    losses = train(net, data, a.steps, batch=8)
    t2 = time.perf_counter()
    fl = conv_flops(-(-a.nz // 8) * 8, -(-a.nr // 8) * 8, 8) * a.steps
    print(f"pairs {data['x'].shape[0]} in {t1 - t0:.1f} s; {a.steps} Adam steps in {t2 - t1:.1f} s "
          f"({fl / (t2 - t1) / 1e12:.1f} TFLOP/s in the 3x3 layers); loss {np.mean(losses[:20]):.3e} -> "
          f"{np.mean(losses[-50:]):.3e}", flush=True)
    if a.save:
        np.save(a.save, net.get_params())
    for s in range(a.eval_seeds):
        case = make_case("c2", seed=2000 + s, nr=a.nr, nz=a.nz)
        pr = ch_run_pairs(case, a.eval_pairs, a.warmup, base=a.base)
        y = np.concatenate([net.forward(np.ascontiguousarray(pr["x"][k:k + 1])) for k in range(pr["x"].shape[0])])
        rel = np.sqrt(((y - pr["y"]) ** 2).sum(axis=(1, 2, 3)) / (pr["y"] ** 2).sum(axis=(1, 2, 3)))
        print(f"held-out seed {2000 + s}: error of the learned guess / error of the {a.base} guess: "
              f"mean {rel.mean():.3f}", flush=True)
        for judge in ("none", "residual"):
            ev = evaluate_ch(case, net, pr, judge=judge)
            print(f"  judge {judge}: mixed CH iterations to 1e-8: {a.base} {ev['iters_plain'].mean():.1f}, "
                  f"learned {ev['iters_learned'].mean():.1f}; learned guess taken {int(ev['used'].sum())}/"
                  f"{ev['used'].size}; max true residual {ev['true_resid_learned'].max():.2e}", flush=True)
        for frac in a.lowpass:
            _lowpass_rows(case, net, pr, frac)
    net.close()


def _lowpass_rows(case, net, pr, frac):
    """Mixed CH iterations from the base guess plus the learned, or the exact, correction with
    only its lowest `frac` of DCT-II modes kept along each axis."""
    import scipy.fft as sf

    nz, nr = case.nz, case.nr

    def lp(v):
        c = sf.dctn(v.reshape(nz, nr), type=2, norm="ortho")
        c[int(nz * frac):, :] = 0.0
        c[:, int(nr * frac):] = 0.0
        return sf.idctn(c, type=2, norm="ortho").reshape(-1)

    P = case.params.copy()
    P.precision = F.DRD_PREC_MIXED
    P.tol = 1e-8
    ctx = DRDContext(P)
    try:
        ctx.set_case(case)
        bdr = _interior(case.coefs["bdr_ph"])
        its = {"learned": [], "exact": []}
        errs = {"learned": [], "exact": []}
        for k in range(pr["b"].shape[0]):
            b, g0, mu1 = pr["b"][k], pr["mu0"][k], pr["mu1"][k]
            xl, _, _, _ = ch_guess(ctx, net, b, g0, bdr, pr["x"][k, 2], judge="none")
            for name, corr in (("learned", xl - g0), ("exact", mu1 - g0)):
                x0 = g0 + lp(corr)
                _, st = ctx.solve(F.DRD_SYS_CH, b, x0)
                its[name].append(st.iter)
                errs[name].append(np.linalg.norm(x0 - mu1) / np.linalg.norm(mu1 - g0))
        for name in its:
            print(f"  {name} correction low-passed to {frac}: error ratio {np.mean(errs[name]):.3f}, "
                  f"iterations {np.mean(its[name]):.1f}", flush=True)
    finally:
        ctx.close()


if __name__ == "__main__":
    main()
