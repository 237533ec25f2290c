"""Pins of the FP64 CPU oracle (CPU only).

No reference test or reference output exists for this path, so the oracle is pinned against:
  * scipy.fft's DCT-I / DCT-II / DCT-III, the published definitions of vfftpack VCOST
    (lib/vfftpack.f:689-704, with the 1/sqrt(2(N-1)) scaling) and FFTW REDFT10 / REDFT01;
  * the manufactured Poisson case of microfluidics_complex_domain/PreSolve_2.f90:32-67;
  * operator identities of the reference's discretisation (Neumann null spaces, symmetry,
    Jacobi = diagonal of the operator, self-inverse VCOST);
  * BiCGSTAB exit semantics of lib/BiCGSTABREVCOM.f;
  * the committed golden vectors (tests/golden/, made by make_golden.py).
"""
import os

import numpy as np
import pytest
import scipy.fft as sf

from drd_application_gb300 import abi
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import advanced_case, rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
F = abi


@pytest.fixture(scope="module")
def orc(oracle_build):
    return Oracle(abi.default_params(16, 8))


@pytest.mark.parametrize("n", [2, 3, 5, 16, 31, 179, 180, 420])
def test_vcost_is_scaled_dct1(orc, n):
    x = np.random.default_rng(n).standard_normal((3, n))
    ref = sf.dct(x, type=1, axis=-1) / np.sqrt(2 * (n - 1))
    # VCOST uses pi = 3.14159265358979 (PIMACH, lib/vfftpack.f:294): ~3e-15 relative at most
    assert rel_err(orc.vcost(x), ref) < 2e-14
    assert rel_err(orc.vcost(orc.vcost(x)), x) < 1e-12  # self-inverse (:698-701)


@pytest.mark.parametrize("n", [1, 2, 7, 64, 180, 420])
def test_redft10_redft01_are_dct2_dct3(orc, n):
    x = np.random.default_rng(n + 1).standard_normal((4, n))
    assert rel_err(orc.redft10(x), sf.dct(x, type=2, axis=-1)) < 1e-13
    assert rel_err(orc.redft01(x), sf.dct(x, type=3, axis=-1)) < 1e-13
    assert rel_err(orc.redft01(orc.redft10(x)) / (2 * n), x) < 1e-12  # round trip scales by 2n


def test_manufactured_poisson_case(oracle_build):
    """microfluidics_complex_domain/PreSolve_2.f90:32-67: p = cos(20 pi x/slen) cos(10 pi y/shig);
    the pressure step applied to u = grad_x p, v = grad_y p returns p (up to the mean mode)."""
    case = make_case("c2", seed=0, nr=120, nz=60)
    P = case.params
    o = Oracle(P)
    nr, nz = P.nr, P.nz
    slen, shig = P.dr * nr, P.dz * nz
    x = (np.arange(-1, nr + 1) + 0.5) * P.dr
    z = (np.arange(-1, nz + 1) + 0.5) * P.dz
    p = np.cos(20 * np.pi * x[None, :] / slen) * np.cos(10 * np.pi * z[:, None] / shig)
    u = np.zeros((nz + 2, nr + 3))
    v = np.zeros((nz + 1, nr + 2))
    u[:, 1:nr + 2] = (p[:, 1:] - p[:, :-1]) / P.dr
    v[:, 1:-1] = (p[1:, 1:-1] - p[:-1, 1:-1]) / P.dz
    psi = o.presolve(u, v, 1.0)
    a = psi[1:-1, 1:-1] - psi[1:-1, 1:-1].mean()
    b = p[1:-1, 1:-1] - p[1:-1, 1:-1].mean()
    assert rel_err(a, b) < 1e-10
    # Neumann ghosts of dct_fftw (:175-183)
    assert np.array_equal(psi[:, 0], psi[:, 1]) and np.array_equal(psi[0, :], psi[1, :])


def test_op_double_gradient_neumann_null_space_and_symmetry(oracle_build):
    case = make_case("c2", seed=1, nr=30, nz=14)
    P = case.params
    o = Oracle(P)
    mo = case.coefs["M0"] + 0.1
    ones = np.ones((P.nz + 2, P.nr + 2))
    assert np.abs(o.op_double_gradient_neum(ones, mo)).max() < 1e-9  # constants are in the null space
    rng = np.random.default_rng(0)
    a = rng.standard_normal(ones.shape)
    b = rng.standard_normal(ones.shape)
    La = o.op_double_gradient_neum(a, mo)[1:-1, 1:-1]
    Lb = o.op_double_gradient_neum(b, mo)[1:-1, 1:-1]
    lhs = (La * b[1:-1, 1:-1]).sum()
    rhs = (Lb * a[1:-1, 1:-1]).sum()
    assert abs(lhs - rhs) < 1e-9 * abs(lhs)  # zero-flux operator is symmetric


def test_jacobi_is_the_operator_diagonal_for_u_rows(oracle_build):
    """PSolve_uv_2_CG's diagonal (VeloSolve_2_combined.f90:662-686) equals the u-u diagonal of
    MatrixVector_uv_2_CG minus its penalty term (the reference's Jacobi omits the penalty)."""
    case = make_case("c2", seed=2, nr=12, nz=8)
    P = case.params.copy()
    P.penalty_k = 0.0
    o = Oracle(P)
    k = case.coefs
    n = (P.nr + 1) * P.nz + P.nr * (P.nz - 1)
    mn = (P.nr + 1) * P.nz
    diag = np.zeros(n)
    for q in range(mn):
        e = np.zeros(n)
        e[q] = 1.0
        diag[q] = o.uv_matvec(2, k["rho"], k["eta"], k["bdr_pen"], e)[q]
    inv = o.uv_psolve(2, k["rho"], k["eta"], np.ones(n))
    # x-boundary u rows (i = 0, nr) couple to their reflected ghosts and differ by design
    rows = [q for q in range(mn) if 0 < q % (P.nr + 1) < P.nr]
    assert rel_err(1.0 / inv[rows], diag[rows]) < 1e-13


def test_ch_psolve_inverts_the_constant_coefficient_ch_operator(oracle_build):
    """PSolve_CG's DCT-I diagonalisation (setup.f90:134-155, DCT.f90) is the exact inverse of the
    CH operator on the (nr-1) x (nz-1)-interval vertex grid; applied to a smooth field it is a good
    approximation of the cell-grid operator with unit mobility."""
    case = make_case("c1", seed=0, nr=32, nz=16)
    P = case.params
    o = Oracle(P)
    one = np.ones((P.nz + 2, P.nr + 2))
    xs = np.cos(np.pi * np.arange(P.nr) / (P.nr - 1))[None, :] * np.cos(np.pi * np.arange(P.nz) / (P.nz - 1))[:, None]
    y = o.ch_matvec(one, one, xs.reshape(-1))
    z = o.ch_psolve(y)
    assert rel_err(z, xs.reshape(-1)) < 0.05


def test_bicgstab_exit_semantics(oracle_build):
    """INFO and ITER as lib/BiCGSTABREVCOM.f returns them."""
    case, st, t = advanced_case("c2", seed=4, nr=24, nz=12, steps=1)
    P = case.params.copy()
    k = case.coefs
    o = Oracle(P)
    r, p, s = o.phsolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], k["bdr_ph"], k["bdr_ph_grad"], k["M0"], k["Mi"])
    assert s.info == 0 and s.resid <= P.tol and s.true_resid <= 1.01 * P.tol
    # ITER cap of 1: not converged, INFO = 1 (:376-379)
    P1 = P.copy()
    P1.ch_maxit = 1
    s1 = Oracle(P1).phsolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], k["bdr_ph"], k["bdr_ph_grad"], k["M0"], k["Mi"])[2]
    assert s1.info == 1 and s1.iter == 1
    # initial guess already the solution: the absolute x0 test (:248) ends with ITER = MAXIT, RESID = TOL
    P2 = P.copy()
    P2.tol = 1e6
    s2 = Oracle(P2).phsolve(st[F.F_U], st[F.F_V], st[F.F_PH], r, k["bdr_ph"], k["bdr_ph_grad"], k["M0"], k["Mi"])[2]
    assert s2.info == 0 and s2.iter == P2.ch_maxit and s2.resid == P2.tol and (s2.flags & F.DRD_FLAG_EARLY_X0)


def test_golden_fixtures_reproduce(oracle_build):
    g = np.load(os.path.join(HERE, "golden", "mf_24x12.npz"))
    P = abi.default_params(int(g["param_nr"]), int(g["param_nz"]))
    for name, _ in abi.drd_params._fields_:
        if "param_" + name in g:
            v = g["param_" + name]
            setattr(P, name, int(v) if v.dtype.kind in "iu" else float(v))
    o = Oracle(P)
    c = {n: g["coef_" + n] for n in ("rho", "eta", "bdr_ph", "bdr_ph_grad", "M0", "Mi", "bdr_pen", "bdr_used")}
    r, p, s = o.phsolve(g["in_u"], g["in_v"], g["in_ph"], g["in_rmu"], c["bdr_ph"], c["bdr_ph_grad"], c["M0"], c["Mi"])
    assert rel_err(r, g["ph_rmu_after"]) < 1e-9 and rel_err(p, g["ph_ph_after"]) < 1e-11
    assert abs(int(s.iter) - int(g["ph_iter"])) <= 1
    psi = o.presolve(g["in_u"], g["in_v"], float(g["pre_coef"]))
    assert rel_err(psi, g["pre_psi"]) < 1e-12
    assert rel_err(o.ch_psolve(g["op_x_ch"]), g["op_ch_psolve"]) < 1e-12
    assert rel_err(o.uv_matvec(2, c["rho"], c["eta"], c["bdr_pen"], g["op_x_uv"]), g["op_uv_matvec2"]) < 1e-13
    assert abs(o.mass(g["in_ph"]) - float(g["mass"])) < 1e-13


def test_interpolate_coef_formula(oracle_build):
    case = make_case("c2", seed=5, nr=40, nz=20)
    o = Oracle(case.params)
    fpd, rho, eta = o.interpolate_coef(case.dist, case.coefs["bdr_ph"])
    assert rel_err(fpd, case.coefs["fpd"]) < 1e-14
    assert rel_err(eta, 1.0 + (case.params.lambda_eta - 1.0) * fpd) < 1e-14
    assert np.allclose(rho, 1.0 + (case.params.lambda_rho - 1.0) * fpd)


def test_two_phase_coef_formula(oracle_build):
    """The two-fluid coefficients (two_phase_flow_complex_domain/interpolate_coef.f90:91-112):
    the oracle equals the workload's numpy form bit for bit, the drops carry lambda_eta, the
    matrix fluid 1, the solid at least 1 + (lambda_eta - 1) fpd_ph, and the clipped branches."""
    case = make_case("c2", seed=5, nr=84, nz=36)
    P = case.params
    assert P.two_fluid == 1 and P.lambda_eta == 5.0
    o = Oracle(P)
    ph, fpd = case.state[abi.F_PH], case.coefs["fpd"]
    rho, eta = o.two_phase_coef(fpd, ph)
    assert np.array_equal(eta, case.coefs["eta"]) and np.array_equal(rho, case.coefs["rho"])
    assert np.all(eta >= 1.0 + 4.0 * fpd) and np.all(eta >= 1.0 + 4.0 * np.clip(ph, -1, 1))
    drop = (ph > 0.5) & (fpd < 1e-6)
    assert drop.any() and np.allclose(eta[drop], 1.0 + 4.0 * ph[drop])
    x = np.linspace(-1.5, 1.5, ph.size).reshape(ph.shape)
    _, e2 = o.two_phase_coef(np.zeros_like(x), x)
    assert np.all(e2[x >= 1.0] == 5.0) and np.all(e2[x <= -1.0] == 1.0)
