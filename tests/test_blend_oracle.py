"""The solid-blended CH preconditioner in the oracle (CPU): the probe generator, the limits
w = 0 and w = 1, the mirror symmetry that the network's data augmentation relies on, the probe
fit's shape and its gain over PSolve_CG alone, and the network's target transform."""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.learned import BLEND_FLOOR, blend_features, blend_target, blend_weights, flip_augment
from tests.helpers import advanced_case, pack_cell

M64 = (1 << 64) - 1


def _splitmix_sign(seed, probe, n, q):
    z = (seed + (probe * n + q + 1) * 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    z = z ^ (z >> 31)
    return -1.0 if z >> 63 else 1.0


@pytest.fixture(scope="module")
def small():
    from oracle.oracle import Oracle

    case, st, _ = advanced_case("c2", seed=3, nr=84, nz=36, steps=2)
    return case, st, Oracle(case.params)


def test_probe_signs_follow_splitmix64(small):
    _, _, orc = small
    n = 84 * 36
    for seed, p, q in ((0, 0, 0), (7, 3, 100), (2 ** 40 + 5, 15, n - 1), (M64 - 3, 1, 17)):
        assert orc.L.orc_probe_sign(seed, p, n, q) == _splitmix_sign(seed, p, n, q)
    s = np.array([orc.L.orc_probe_sign(11, 2, n, q) for q in range(n)])
    assert set(np.unique(s)) == {-1.0, 1.0}
    assert abs(s.mean()) < 0.05


def test_blend_limits(small):
    case, _, orc = small
    rng = np.random.default_rng(0)
    x = rng.standard_normal(case.nr * case.nz)
    q = orc.ch_psolve(x)
    assert np.array_equal(orc.ch_psolve_blend(None, x), q)
    assert np.array_equal(orc.ch_psolve_blend(np.zeros_like(x), x), q)
    assert np.allclose(orc.ch_psolve_blend(np.ones_like(x), x), x, rtol=0, atol=1e-14 * np.abs(x).max())
    w = rng.uniform(0, 1, x.size)
    assert np.allclose(orc.ch_psolve_blend(w, x), q + w * (x - q), rtol=1e-15, atol=1e-15 * np.abs(q).max())


def test_operator_and_preconditioner_mirror_symmetry(small):
    """A(flip M) flip x = flip (A(M) x) and P flip x = flip P x along both axes, so a mirrored
    geometry's blend weights are the mirrored weights (the network's augmentation)."""
    case, _, orc = small
    nr, nz = case.nr, case.nz
    rng = np.random.default_rng(1)
    x = rng.standard_normal(nr * nz)
    M0, Mi = case.coefs["M0"], case.coefs["Mi"]
    for ax in (0, 1):
        fM0 = np.ascontiguousarray(np.flip(M0, ax))
        fMi = np.ascontiguousarray(np.flip(Mi, ax))
        fx = np.ascontiguousarray(np.flip(x.reshape(nz, nr), ax)).reshape(-1)
        a = orc.ch_matvec(fM0, fMi, fx)
        b = np.flip(orc.ch_matvec(M0, Mi, x).reshape(nz, nr), ax).reshape(-1)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
        a = orc.ch_psolve(fx)
        b = np.flip(orc.ch_psolve(x).reshape(nz, nr), ax).reshape(-1)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()


def test_probe_fit_shape_and_gain(small):
    case, st, orc = small
    M0, Mi = case.coefs["M0"], case.coefs["Mi"]
    w = orc.ch_blend_probe(M0, Mi, 32, 9)
    bdr = pack_cell(case.coefs["bdr_ph"])
    assert w.min() >= 0.0 and w.max() <= 1.0
    assert w[bdr < 0.5].max() < 0.02  # the fluid keeps PSolve_CG
    assert w[bdr > 0.999].mean() > 0.5  # the solid takes mostly the identity
    b, x0, _ = orc.ch_system(st[abi.F_U], st[abi.F_V], st[abi.F_PH], st[abi.F_RMU], case.coefs["bdr_ph"],
                             case.coefs["bdr_ph_grad"], Mi)
    orc.P.tol = 1e-8
    x_ref, s_ref = orc.ch_solve_blend(M0, Mi, None, b, x0)
    x_bl, s_bl = orc.ch_solve_blend(M0, Mi, w, b, x0)
    assert s_ref.info == 0 and s_bl.info == 0
    assert s_bl.iter <= 0.6 * s_ref.iter, (s_bl.iter, s_ref.iter)
    for x in (x_ref, x_bl):
        assert np.linalg.norm(b - orc.ch_matvec(M0, Mi, x)) <= 1.0001e-8 * np.linalg.norm(b)


def test_blend_target_round_trip():
    w = np.concatenate([np.zeros(5), np.logspace(-6, 0, 50), np.ones(3)])
    y = blend_target(w)
    assert y.dtype == np.float32
    back = blend_weights(y)
    assert np.all(back >= 0) and np.all(back <= 1)
    assert np.abs(back - w).max() <= 1e-6
    # an output error of 0.01 moves w by ~9 % and the fluid's zero by < 1e-5
    assert blend_weights(blend_target(np.zeros(1)) + 0.01)[0] < 1e-5 + BLEND_FLOOR * 0.1
    r = blend_weights(blend_target(np.array([0.5])) + 0.01)[0] / 0.5
    assert 1.05 < r < 1.12


def test_blend_features_and_augment(small):
    case, _, _ = small
    x = blend_features(case.coefs["M0"], case.coefs["Mi"])
    assert x.shape == (3, case.nz, case.nr) and x.dtype == np.float32
    assert x[:2].min() >= 0.0 and x[:2].max() <= 1.0 + 1e-6
    d = flip_augment({"x": x[None], "y": x[None, :1]})
    assert d["x"].shape == (4, 3, case.nz, case.nr) and d["y"].shape == (4, 1, case.nz, case.nr)
    assert np.array_equal(d["x"][1], np.flip(x, -1)) and np.array_equal(d["x"][3], np.flip(x, (-2, -1)))
