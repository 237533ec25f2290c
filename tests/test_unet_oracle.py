"""Pins of the CPU restatement of the learned-guess network (oracle/unet_oracle.py), CPU only.

  * its bfloat16 rounding equals torch's float32 -> bfloat16 conversion (round to nearest even);
  * its parameter layout has the documented size (include/drd_gb300.h, drd_unet_*);
  * its backward pass agrees with central finite differences of its own FP64 forward pass,
    layer by layer (directional derivatives along random directions within each layer).
"""
import numpy as np
import pytest

from oracle.unet_oracle import UNetOracle, bf16, he_init, layer_table, param_count


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(20000) * 10.0 ** rng.uniform(-20, 20, 20000)).astype(np.float32)
    x[:4] = [0.0, -0.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8]  # exact ties round to even
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(bf16(x).astype(np.float32), ref)


def test_parameter_layout():
    L = layer_table()
    assert len(L) == 17
    assert [c[1] for c in L[:8]] == [32, 32, 64, 64, 128, 128, 256, 256]
    assert [(c[0], c[1], c[3]) for c in L[8:11]] == [(256, 128, 1), (256, 128, 0), (128, 128, 0)]
    # 3x3 weights 9 * 238080, biases 1632, output layer 32 + 1
    assert param_count(1) == 9 * 238080 + 1632 + 33
    assert param_count(2) == param_count(1) + 33


def _layer_slices(out_ch):
    off, out = 0, []
    for ci, co, _, _ in layer_table():
        n = 9 * ci * co + co
        out.append(slice(off, off + n))
        off += n
    out.append(slice(off, off + out_ch * 33))
    return out


@pytest.mark.parametrize("H,W", [(16, 16), (13, 19), (8, 7)])
def test_backward_matches_finite_differences(H, W):
    o = UNetOracle(H, W, 3, 1, rounding=False)
    p = he_init(1, 3, seed=1)
    p[-33:] *= 10.0  # a larger output layer, so that every layer's gradient is well above round-off
    rng = np.random.default_rng(2)
    # non-zero biases: with zero biases the zero-padded cells sit exactly on the ReLU kink,
    # where the loss has no derivative for finite differences to approximate
    for (ci, co, _, _), s in zip(layer_table(), _layer_slices(1)):
        p[s.stop - co:s.stop] = 0.1 * rng.standard_normal(co)
    x = rng.standard_normal((2, 3, H, W))
    t = rng.standard_normal((2, 1, H, W))
    _, g = o.gradients(p, x, t)
    sl = _layer_slices(1)
    for li in (0, 1, 6, 7, 8, 9, 13, 14, 16, 17):
        v = np.zeros_like(p)
        v[sl[li]] = rng.standard_normal(sl[li].stop - sl[li].start)
        if li == 0:
            v[sl[0]] = v[sl[0]] * (p[sl[0]] != 0)  # the padded input channels carry no signal
        v /= np.linalg.norm(v)
        eps = 1e-6
        fd = (o.loss(p + eps * v, x, t) - o.loss(p - eps * v, x, t)) / (2 * eps)
        an = float(g @ v)
        assert abs(fd - an) <= 1e-4 * max(abs(an), 1e-3), (li, fd, an)


def test_harness_layer_table_and_flops_match_the_oracle():
    """learned.py's FLOP model walks the same 17 layers as the oracle (and drd_unet_create)."""
    from drd_application_gb300 import learned

    assert learned._layers() == [(ci, co, lev) for ci, co, lev, _ in layer_table()]
    # one forward pass on an 8 x 16 padded grid: 2 * 9 * cin * cout * pixels of the layer's level
    want = sum(2.0 * 9 * ci * co * (8 >> lev) * (16 >> lev) for ci, co, lev, _ in layer_table())
    assert learned.conv_flops(8, 16, 1, train=False) == want
    # training adds a data gradient (not for the first layer) and a weight gradient
    first = 2.0 * 9 * 16 * 32 * 8 * 16
    assert learned.conv_flops(8, 16, 1) == 3 * want - first


def test_cubic_guess_is_exact_for_cubics():
    from drd_application_gb300.learned import cubic_guess

    t = np.arange(4.0)
    hist = [np.array([1.0 + 2 * s - 0.5 * s ** 2 + 0.25 * s ** 3]) for s in t]
    s = 4.0
    assert np.allclose(cubic_guess(hist), 1.0 + 2 * s - 0.5 * s ** 2 + 0.25 * s ** 3)
