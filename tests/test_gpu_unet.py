"""The learned-guess network's kernels (csrc/drd_unet.cu) against the CPU restatement
(oracle/unet_oracle.py), through the C-ABI: the forward pass, every layer's gradient, the
Adam loop, host and device buffers.

Tolerances: the kernels and the oracle round the same values to BF16, but the kernels sum in
FP32 in another order, so an element near a rounding boundary can round the other way; such
flips (2^-8 relative) spread through the 17 layers.  Forward outputs agree to 2e-2 in the
relative 2-norm.  Weight gradients are sums over pixels with heavy cancellation, so BF16
rounding alone moves them 7-22% from their FP64 values on these random-target cases; the
check is that every layer's kernel gradient is closer to the rounded oracle than 0.8 of the
rounded oracle's distance to FP64, and within 0.2 of it, against differences of order 1 for
a wrong layout, tap or transposition."""
import numpy as np
import pytest

from oracle.unet_oracle import UNetOracle, layer_table, param_count

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _slices(out_ch):
    off, out = 0, []
    for ci, co, _, _ in layer_table():
        n = 9 * ci * co + co
        out.append(slice(off, off + n))
        off += n
    out.append(slice(off, off + out_ch * 33))
    return out


def _net(H, W, cin, cout, seed, bias=True):
    from drd_application_gb300.learned import UNet

    net = UNet(H, W, cin, cout, max_batch=4, seed=seed)
    if bias:  # non-zero biases, so that the check also covers them
        p = net.get_params()
        rng = np.random.default_rng(seed)
        for (ci, co, _, _), s in zip(layer_table(), _slices(cout)):
            p[s.stop - co:s.stop] = 0.05 * rng.standard_normal(co)
        net.set_params(p)
    return net


@pytest.mark.parametrize("H,W,cin,cout", [(16, 16, 3, 1), (13, 30, 3, 1), (21, 11, 4, 2)])
def test_forward_matches_oracle(cuda_lib, H, W, cin, cout):
    net = _net(H, W, cin, cout, seed=H)
    assert net.nparam == param_count(cout)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, cin, H, W)).astype(np.float32)
    y = net.forward(x)
    yo, _ = UNetOracle(H, W, cin, cout).forward(net.get_params().astype(np.float64), x.astype(np.float64))
    assert _rel(y, yo) < 2e-2
    net.close()


@pytest.mark.parametrize("H,W", [(16, 16), (13, 30)])
def test_gradients_match_oracle(cuda_lib, H, W):
    net = _net(H, W, 3, 1, seed=7)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((2, 3, H, W)).astype(np.float32)
    t = rng.standard_normal((2, 1, H, W)).astype(np.float32)
    loss, g = net.gradients(x, t)
    p, x64, t64 = net.get_params().astype(np.float64), x.astype(np.float64), t.astype(np.float64)
    lo, go = UNetOracle(H, W, 3, 1).gradients(p, x64, t64)
    _, g64 = UNetOracle(H, W, 3, 1, rounding=False).gradients(p, x64, t64)
    assert abs(loss - lo) <= 1e-3 * lo
    for li, s in enumerate(_slices(1)):
        noise = _rel(go[s], g64[s])
        assert _rel(g[s], go[s]) < min(0.8 * noise, 0.2), (li, _rel(g[s], go[s]), noise)
    net.close()


def test_device_buffers_match_host(cuda_lib):
    torch = pytest.importorskip("torch")
    net = _net(16, 24, 3, 1, seed=2)
    x = np.random.default_rng(4).standard_normal((3, 3, 16, 24)).astype(np.float32)
    yh = net.forward(x)
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros((3, 1, 16, 24), dtype=torch.float32, device="cuda")
    net.forward(xd, out=yd)
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), yh)
    net.close()


def test_training_fits_a_smooth_map(cuda_lib):
    """Adam through the library's own backward pass fits a fixed smooth map of the inputs."""
    from drd_application_gb300.learned import UNet

    H, W = 32, 48
    net = UNet(H, W, 3, 1, max_batch=4, seed=11)
    rng = np.random.default_rng(5)
    x = rng.standard_normal((4, 3, H, W)).astype(np.float32)
    k = np.array([0.25, 0.5, 0.25])
    sm = x[:, 0]
    for ax in (1, 2):
        sm = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), ax, sm)
    t = (sm + 0.5 * x[:, 1] * (x[:, 2] > 0))[:, None].astype(np.float32)
    l0 = net.gradients(x, t)[0]
    for it in range(300):
        loss = net.train_step(x, t, 1e-3)
    assert loss < 0.05 * l0, (l0, loss)
    net.close()


@pytest.mark.parametrize("H,W", [(16, 16), (37, 70), (64, 128)])
def test_tensor_core_convolutions_match_the_mma_sync_kernels(cuda_lib, H, W):
    """The tcgen05 convolutions (DRD_UNET_TC=1) against the mma.sync kernels (the default) on
    the same parameters: forward outputs and gradients.  Both accumulate in FP32 from BF16
    operands; only the summation order differs, so BF16 rounding flips are the only source of
    difference."""
    import os

    rng = np.random.default_rng(H)
    x = rng.standard_normal((3, 3, H, W)).astype(np.float32)
    tg = rng.standard_normal((3, 1, H, W)).astype(np.float32)
    out = []
    for tc in ("1", "0"):
        os.environ["DRD_UNET_TC"] = tc
        try:
            net = _net(H, W, 3, 1, seed=5)
        finally:
            os.environ.pop("DRD_UNET_TC", None)
        y = net.forward(x)
        loss, g = net.gradients(x, tg)
        out.append((y, loss, g))
        net.close()
    (y1, l1, g1), (y0, l0, g0) = out
    assert _rel(y1, y0) < 2e-2 and abs(l1 - l0) <= 2e-2 * abs(l0)
    assert _rel(g1, g0) < 5e-2
