"""Pins of the oracle's ESOLP_x momentum preconditioner (CPU only).

Precipitation_dynamics/VeloSolve_combined.f90:800-806 preconditions the momentum system with
ESOLP_x (Precipitation_dynamics/ESOLP.f90): per block of the packed vector, VCOST along x, one
tridiagonal solve (rfords, setup.f90:327-354) along y per x mode, VCOST along x again, with the
coefficients of setup.f90:157-235.  No reference output exists, so the restatement is pinned by
  * an independent numpy construction of those coefficients (t1 = pi/2 when they are formed);
  * the defining identity: with C the scaled DCT-I (scipy's type-1 DCT / sqrt(2(L-1))) and T_k
    the tridiagonal matrix of mode k, ESOLP(x) = z satisfies T_k (C z)_k = (C x)_k;
  * the momentum solve preconditioned with ESOLP_x reaching the same answer as with Jacobi.
"""
import numpy as np
import pytest
import scipy.fft as sf

from drd_application_gb300 import abi
from oracle.oracle import Oracle
from tests.helpers import advanced_case, rel_err


def _params(nr=23, nz=11):
    p = abi.default_params(nr, nz)
    p.dr, p.dz = 3.0 / nr, 1.2 / nz
    p.dt = 2.0e-3
    return p


def _coefs_np(P, bdf):
    """setup.f90:157-235 for the no-slip deck (xlsB = xlsT = 0, slip ratio 1)."""
    nr, nz, dt, dz2, dr2 = P.nr, P.nz, P.dt, P.dz ** 2, P.dr ** 2
    m = 1.5 if bdf == 2 else 1.0
    t1 = np.pi / 2  # the fmx loops leave t1 at pi*nr/nr/2
    xls = (2 * P.xlsB - P.dz) / (2 * P.xlsB + P.dz)
    fu = 4 * dt * np.sin(np.pi * np.arange(nr + 1) / nr / 2) ** 2 / dr2
    ua = np.full((nr + 1, nz), -dt / dz2)
    uc = np.full((nr + 1, nz), -dt / dz2)
    ub = t1 * m + (2 * dt / dz2 + fu[:, None]) * np.ones((1, nz))
    ua[:, 0] = 0.0
    uc[:, -1] = 0.0
    ub[:, 0] = ub[:, -1] = t1 * m + ((2 - xls) * dt / dz2 + fu)
    fv = 4 * dt * np.sin(np.pi * np.arange(nr) / (nr - 1) / 2) ** 2 / dr2
    va = np.full((nr, nz - 1), -dt / dz2)
    vc = np.full((nr, nz - 1), -dt / dz2)
    vb = t1 * m + 2 * dt / dz2 + fv[:, None] * np.ones((1, nz - 1))
    va[:, 0] = 0.0
    vc[:, -1] = 0.0
    return (ua, ub, uc), (va, vb, vc)


@pytest.mark.parametrize("bdf", [1, 2])
def test_esolp_coefficients_match_setup(oracle_build, bdf):
    P = _params()
    o = Oracle(P)
    (u, v), (un, vn) = o.esolp_coefs(bdf), _coefs_np(P, bdf)
    for a, b in zip(u + v, un + vn):
        assert a.shape == b.shape
        assert rel_err(a, b) < 1e-14


def _vcost(x):
    n = x.shape[-1]
    return sf.dct(x, type=1, axis=-1) / np.sqrt(2 * (n - 1))


def _tri_apply(a, b, c, y):
    """Row j of mode k: a_j y_{j-1} + b_j y_j + c_j y_{j+1}; y is (rows, modes), a..c (modes, rows)."""
    out = b.T * y
    out[1:] += a.T[1:] * y[:-1]
    out[:-1] += c.T[:-1] * y[1:]
    return out


@pytest.mark.parametrize("nr,nz", [(23, 11), (16, 9), (40, 21)])
@pytest.mark.parametrize("bdf", [1, 2])
def test_esolp_inverts_vcost_tridiagonal(oracle_build, nr, nz, bdf):
    P = _params(nr, nz)
    o = Oracle(P)
    mu = (nr + 1) * nz
    x = np.random.default_rng(nr + bdf).standard_normal(mu + nr * (nz - 1))
    z = o.uv_psolve_esolp(bdf, x)
    (ua, ub, uc), (va, vb, vc) = _coefs_np(P, bdf)
    for (a, b, c), L, rows, sl in (((ua, ub, uc), nr + 1, nz, slice(0, mu)),
                                   ((va, vb, vc), nr, nz - 1, slice(mu, None))):
        xb, zb = x[sl].reshape(rows, L), z[sl].reshape(rows, L)
        assert rel_err(_tri_apply(a, b, c, _vcost(zb)), _vcost(xb)) < 1e-12


def test_velosolve_esolp_matches_jacobi(oracle_build):
    case, st, t = advanced_case("c2", seed=4, nr=40, nz=20, steps=1)
    F = abi
    k = case.coefs
    outs = []
    for pre in (F.DRD_UV_JACOBI, F.DRD_UV_ESOLP):
        P = case.params.copy()
        P.tol = 1e-12
        P.uv_precond = pre
        o = Oracle(P)
        outs.append(o.velosolve(2, st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE], st[F.F_U], st[F.F_V_PRE], st[F.F_V],
                                st[F.F_P], k["rho"], k["eta"], k["bdr_ph"], k["bdr_pen"], k["bdr_used"], st[F.F_PH],
                                st[F.F_RMU], t, st[F.F_PF1], st[F.F_PF2]))
    (uj, vj, _, _, sj), (ue, ve, _, _, se) = outs
    assert sj.info == 0 and se.info == 0
    assert se.true_resid <= 1e-11
    assert rel_err(ue, uj) < 1e-8 and rel_err(ve, vj) < 1e-8


@pytest.mark.parametrize("bdf", [1, 2])
def test_esolp_scaled_definition(oracle_build, bdf):
    """DRD_UV_ESOLP_SCALED: s = sqrt(D0 / D) from the Jacobi diagonals (D0 at rho = eta = 1),
    y = s ESOLP_x(s x); with rho = eta = 1 the scaling is the identity."""
    case, st, _ = advanced_case("c2", seed=2, nr=48, nz=24, steps=1)
    P = case.params.copy()
    orc = Oracle(P)
    rho, eta = case.coefs["rho"], case.coefs["eta"]
    one = np.ones_like(rho)
    n = (P.nr + 1) * P.nz + P.nr * (P.nz - 1)
    s = orc.uv_esolp_scale(bdf, rho, eta)
    d = orc.uv_psolve(bdf, rho, eta, np.ones(n))
    d0 = orc.uv_psolve(bdf, one, one, np.ones(n))
    assert np.allclose(s, np.sqrt(d / d0), rtol=1e-14, atol=0)
    assert s.min() > 0 and s.max() <= 1.0 + 1e-12  # rho, eta >= 1 here: D >= D0
    x = np.random.default_rng(bdf).standard_normal(n)
    y = orc.uv_psolve_esolp_scaled(bdf, s, x)
    assert rel_err(y, s * orc.uv_psolve_esolp(bdf, s * x)) <= 1e-15
    assert np.allclose(orc.uv_esolp_scale(bdf, one, one), 1.0, rtol=1e-15, atol=0)


def test_esolp_scaled_fewer_iterations(oracle_build):
    """With the two-fluid coefficients (viscosity ratio 5) the scaled form needs fewer momentum
    iterations than ESOLP_x to the same FP64 residual."""
    case, st, _ = advanced_case("c2", seed=4, nr=84, nz=36, steps=2)
    c = case.coefs
    from tests.helpers import pack_uv

    x_true = pack_uv(st[abi.F_U], st[abi.F_V])
    its = {}
    for pre in (abi.DRD_UV_ESOLP, abi.DRD_UV_ESOLP_SCALED):
        P = case.params.copy()
        P.uv_precond = pre
        P.tol = 1e-10
        orc = Oracle(P)
        b = orc.uv_matvec(2, c["rho"], c["eta"], c["bdr_pen"], x_true)
        x, stt = orc.solve(1, 2, c, b)
        assert stt.info == 0
        assert np.linalg.norm(b - orc.uv_matvec(2, c["rho"], c["eta"], c["bdr_pen"], x)) <= 1.0001e-10 * np.linalg.norm(b)
        its[pre] = stt.iter
    assert its[abi.DRD_UV_ESOLP_SCALED] < its[abi.DRD_UV_ESOLP], its
