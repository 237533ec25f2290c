"""Parity of the CUDA library (through its C-ABI) with the FP64 CPU oracle.

Operator level: every operator of the three Krylov systems and the pressure transform agree
with the oracle to 1e-12 relative in FP64 (the FP32 operators of the mixed mode to 2e-6).
Solve level: two correct BiCGSTABs whose dot products are summed in different orders stop at
slightly different iterates, so solves are compared (a) with a tolerance of 1e-12, where the
fields must agree to 1e-9 relative, and (b) at the reference deck tolerance, where both must
meet it and the fields agree to 1e-6 relative.
"""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from oracle.oracle import Oracle
from tests.helpers import advanced_case, pack_cell, pack_uv, rel_err

pytestmark = pytest.mark.gpu

F = abi


@pytest.fixture(scope="module")
def mf_case(cuda_lib, oracle_build):
    return advanced_case("c2", seed=3, nr=48, nz=24, steps=2)


@pytest.fixture(scope="module")
def tp_case(cuda_lib, oracle_build):
    return advanced_case("tp", seed=5, nr=40, nz=32, steps=2)


def _ctx(case, **kw):
    P = case.params.copy()
    for k, v in kw.items():
        setattr(P, k, v)
    ctx = DRDContext(P)
    ctx.set_case(case)
    return ctx, Oracle(P)


# ---------------------------------------------------------------------------------- operators
@pytest.mark.parametrize("bdf", [1, 2])
def test_uv_operators_fp64(mf_case, bdf):
    case, st, _ = mf_case
    ctx, orc = _ctx(case)
    k = case.coefs
    rng = np.random.default_rng(1)
    x = rng.standard_normal(ctx.L.drd_op_length(ctx.h, F.DRD_OP_UV_MATVEC))
    y = ctx.op_apply(F.DRD_OP_UV_MATVEC, x, bdf=bdf)
    yo = orc.uv_matvec(bdf, k["rho"], k["eta"], k["bdr_pen"], x)
    assert rel_err(y, yo) < 1e-12
    z = ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=bdf)
    zo = orc.uv_psolve(bdf, k["rho"], k["eta"], x)
    assert rel_err(z, zo) < 1e-13
    # the solution field itself as input (smooth, non-trivial)
    xs = pack_uv(st[F.F_U], st[F.F_V])
    assert rel_err(ctx.op_apply(F.DRD_OP_UV_MATVEC, xs, bdf=bdf), orc.uv_matvec(bdf, k["rho"], k["eta"], k["bdr_pen"], xs)) < 1e-12
    ctx.close()


def test_ch_operators_fp64(mf_case):
    case, st, _ = mf_case
    ctx, orc = _ctx(case)
    k = case.coefs
    rng = np.random.default_rng(2)
    n = case.nr * case.nz
    for x in (rng.standard_normal(n), pack_cell(st[F.F_RMU])):
        y = ctx.op_apply(F.DRD_OP_CH_MATVEC, x)
        assert rel_err(y, orc.ch_matvec(k["M0"], k["Mi"], x)) < 1e-12
        z = ctx.op_apply(F.DRD_OP_CH_PSOLVE, x)
        assert rel_err(z, orc.ch_psolve(x)) < 1e-12
    ctx.close()


def test_operators_fp32_close(mf_case):
    case, st, _ = mf_case
    ctx, orc = _ctx(case)
    k = case.coefs
    rng = np.random.default_rng(3)
    x = rng.standard_normal(case.nr * case.nz)
    assert rel_err(ctx.op_apply(F.DRD_OP_CH_MATVEC, x, precision=F.DRD_PREC_MIXED), orc.ch_matvec(k["M0"], k["Mi"], x)) < 2e-6
    assert rel_err(ctx.op_apply(F.DRD_OP_CH_PSOLVE, x, precision=F.DRD_PREC_MIXED), orc.ch_psolve(x)) < 2e-5
    xu = rng.standard_normal(ctx.L.drd_op_length(ctx.h, F.DRD_OP_UV_MATVEC))
    assert rel_err(ctx.op_apply(F.DRD_OP_UV_MATVEC, xu, precision=F.DRD_PREC_MIXED),
                   orc.uv_matvec(2, k["rho"], k["eta"], k["bdr_pen"], xu)) < 2e-6
    ctx.close()


@pytest.mark.parametrize("nr,nz", [(97, 53), (130, 17), (420, 180)])
def test_ch_operator_fp32_tiles(cuda_lib, oracle_build, nr, nz):
    """The FP32 CH operator (one tiled pass over 64 x 8 cells) on grids of several tiles with
    ragged right and top edges, against the oracle's FP64 operator."""
    from drd_application_gb300.workloads import make_case

    case = make_case("c2", seed=nr, nr=nr, nz=nz)
    ctx, orc = _ctx(case)
    try:
        k = case.coefs
        rng = np.random.default_rng(nz)
        for x in (rng.standard_normal(nr * nz), np.sin(np.arange(nr * nz) * 0.01)):
            y = ctx.op_apply(F.DRD_OP_CH_MATVEC, x, precision=F.DRD_PREC_MIXED)
            assert rel_err(y, orc.ch_matvec(k["M0"], k["Mi"], x)) < 2e-6
    finally:
        ctx.close()


def test_phmu_operators_fp64(tp_case):
    case, st, t = tp_case
    ctx, orc = _ctx(case)
    k = case.coefs
    # the coupled operator uses the M0 that ph_mu_solve recomputes from phi; run one solve to set it
    ang = np.full(case.nr + 1, case.params.angle)
    ph_after, rmu_after, M0, cbt, _ = ctx.ph_mu_solve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], t)
    _, _, M0o, cbto, _ = orc.ph_mu_solve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], k["bdr_ph"], k["bdr_used"],
                                         k["bdr_ph_grad"], k["Mi"], ang, ang)
    assert rel_err(M0, M0o) < 1e-14
    assert np.allclose(cbt, cbto)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(2 * case.nr * case.nz)
    y = ctx.op_apply(F.DRD_OP_PHMU_MATVEC, x)
    assert rel_err(y, orc.phmu_matvec(M0o, k["Mi"], k["bdr_used"], x, cbto[0], cbto[1])) < 1e-12
    z = ctx.op_apply(F.DRD_OP_PHMU_PSOLVE, x)
    assert rel_err(z, orc.phmu_psolve(x)) < 1e-13
    ctx.close()


# ------------------------------------------------------------------------------------ pressure
def test_presolve_matches_oracle(mf_case):
    case, st, _ = mf_case
    ctx, orc = _ctx(case)
    coef = 3 * case.params.re / 2.0 / case.params.dt
    psi = ctx.PreSolve_2(st[F.F_U], st[F.F_V], coef)
    psio = orc.presolve(st[F.F_U], st[F.F_V], coef)
    assert rel_err(psi, psio) < 1e-12
    ctx.close()


def test_presolve_manufactured_case(cuda_lib):
    """The known-answer check kept in microfluidics_complex_domain/PreSolve_2.f90:32-67:
    p = cos(20 pi x/slen) cos(10 pi y/shig); a velocity whose divergence is lap(p) must give
    psi = p up to the mean mode the reference keeps (Pre_Lcc(0,0) = -1)."""
    from drd_application_gb300.workloads import make_case

    case = make_case("c2", seed=0, nr=96, nz=48)
    P = case.params
    nr, nz = P.nr, P.nz
    slen, shig = P.dr * nr, P.dz * nz
    ctx = DRDContext(P)
    x = (np.arange(-1, nr + 1) + 0.5) * P.dr
    z = (np.arange(-1, nz + 1) + 0.5) * P.dz
    p = np.cos(20 * np.pi * x[None, :] / slen) * np.cos(10 * np.pi * z[:, None] / shig)
    # u(i,k) = (p(i,k) - p(i-1,k))/dr, v(i,k) = (p(i,k) - p(i,k-1))/dz gives div u = lap_h(p)
    u = np.zeros(ctx.us)
    v = np.zeros(ctx.vs)
    u[:, 1:nr + 2] = (p[:, 1:] - p[:, :-1]) / P.dr
    v[:, 1:-1] = (p[1:, 1:-1] - p[:-1, 1:-1]) / P.dz
    psi = ctx.PreSolve_2(u, v, 1.0)
    inner = psi[1:-1, 1:-1] - psi[1:-1, 1:-1].mean()
    ref = p[1:-1, 1:-1] - p[1:-1, 1:-1].mean()
    assert rel_err(inner, ref) < 1e-10
    ctx.close()


# --------------------------------------------------------------------------------------- solves
def _phsolve_both(case, st, t, tol):
    ctx, orc = _ctx(case, tol=tol)
    k = case.coefs
    r_g, p_g, s_g = ctx.PhSolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], t)
    r_o, p_o, s_o = orc.phsolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], k["bdr_ph"], k["bdr_ph_grad"], k["M0"], k["Mi"])
    ctx.close()
    return (r_g, p_g, s_g), (r_o, p_o, s_o)


def test_phsolve_tight(mf_case):
    case, st, t = mf_case
    (r_g, p_g, s_g), (r_o, p_o, s_o) = _phsolve_both(case, st, t, 1e-12)
    assert s_g.info == 0 and s_o.info == 0
    assert s_g.true_resid <= 1e-11
    assert rel_err(r_g, r_o) < 1e-9
    assert rel_err(p_g, p_o) < 1e-11


def test_phsolve_deck_tol(mf_case):
    case, st, t = mf_case
    (r_g, p_g, s_g), (r_o, p_o, s_o) = _phsolve_both(case, st, t, case.params.tol)
    assert s_g.info == 0
    assert s_g.true_resid <= 1.01 * case.params.tol
    assert abs(s_g.iter - s_o.iter) <= 2
    assert rel_err(r_g, r_o) < 1e-6
    assert rel_err(p_g, p_o) < 1e-8


@pytest.mark.parametrize("bdf", [1, 2])
def test_velosolve_tight(mf_case, bdf):
    case, st, t = mf_case
    ctx, orc = _ctx(case, tol=1e-12)
    k = case.coefs
    ph_after, rmu_after = st[F.F_PH], st[F.F_RMU]
    o = orc.velosolve(bdf, st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE], st[F.F_U], st[F.F_V_PRE], st[F.F_V], st[F.F_P],
                      k["rho"], k["eta"], k["bdr_ph"], k["bdr_pen"], k["bdr_used"], ph_after, rmu_after, t,
                      st[F.F_PF1], st[F.F_PF2])
    if bdf == 1:
        g = ctx.VeloSolve_combined(None, st[F.F_U], st[F.F_V], st[F.F_P], rmu_after, ph_after, t, st[F.F_PF1], st[F.F_PF2])
    else:
        g = ctx.VeloSolve_2_combined(st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE], st[F.F_U], st[F.F_V_PRE], st[F.F_V],
                                     st[F.F_P], None, ph_after, None, rmu_after, t, st[F.F_PF1], st[F.F_PF2])
    assert g[4].info == 0 and o[4].info == 0
    assert g[4].true_resid <= 1e-11
    assert rel_err(g[0], o[0]) < 1e-9
    assert rel_err(g[1], o[1]) < 1e-9
    nz = case.nz
    assert rel_err(g[2][:nz], o[2][:nz]) < 1e-14
    ctx.close()


def test_ph_mu_solve_tight(tp_case):
    """The Jacobi-preconditioned coupled system is ill-conditioned (about 1400 iterations for a
    relative residual of 1e-10 and 3200 for 1e-11), so two iterates at residual 1e-10 can differ
    by cond * 1e-10 in the fields.  Parity is therefore checked on the system itself: the GPU's
    fields must satisfy the oracle's own discretisation (rhs and operator rebuilt by the
    oracle from the same inputs) to the tolerance."""
    case, st, t = tp_case
    ctx, orc = _ctx(case, tol=1e-10)
    k = case.coefs
    ang = np.full(case.nr + 1, case.params.angle)
    inputs = (st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU])
    g = ctx.ph_mu_solve(*inputs, t)
    o = orc.ph_mu_solve(*inputs, k["bdr_ph"], k["bdr_used"], k["bdr_ph_grad"], k["Mi"], ang, ang)
    assert g[4].info == 0 and o[4].info == 0
    assert g[4].true_resid <= 1.01e-10
    assert orc.phmu_residual(inputs, k, ang, ang, g[0], g[1]) <= 1.01e-10
    assert orc.phmu_residual(inputs, k, ang, ang, o[0], o[1]) <= 1.01e-10
    assert rel_err(g[2], o[2]) < 1e-14  # ph_M_0 recomputed from phi, no solve involved
    # ghost rows of phi follow the wall condition from the interior (ph_mu_solve.f90:174-177)
    assert rel_err(g[0][0, 1:-1] - g[0][1, 1:-1], o[0][0, 1:-1] - o[0][1, 1:-1]) < 1e-3
    ctx.close()


def test_phsolve_solution_satisfies_oracle_system(mf_case):
    """Residual-based parity at the deck tolerance: the GPU's mu satisfies the oracle's CH system."""
    case, st, t = mf_case
    ctx, orc = _ctx(case)
    inputs = (st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU])
    r_g, p_g, s_g = ctx.PhSolve(*inputs, t)
    assert orc.ch_residual(inputs, case.coefs, r_g) <= 1.01 * case.params.tol
    ctx.close()


# ---------------------------------------------------------------------------------- mixed mode
def test_mixed_phsolve_reaches_fp64_tolerance(mf_case):
    case, st, t = mf_case
    ctx64, orc = _ctx(case)
    ctxmx, _ = _ctx(case, precision=F.DRD_PREC_MIXED)
    r64, p64, s64 = ctx64.PhSolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], t)
    rmx, pmx, smx = ctxmx.PhSolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], t)
    assert smx.info == 0, smx.as_dict()
    assert smx.true_resid <= case.params.tol
    assert smx.refinements >= 1
    assert rel_err(rmx, r64) < 1e-5
    ctx64.close()
    ctxmx.close()


def test_mixed_velosolve_reaches_fp64_tolerance(mf_case):
    case, st, t = mf_case
    ctx, _ = _ctx(case, precision=F.DRD_PREC_MIXED)
    g = ctx.VeloSolve_2_combined(st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE], st[F.F_U], st[F.F_V_PRE], st[F.F_V],
                                 st[F.F_P], None, st[F.F_PH], None, st[F.F_RMU], t)
    assert g[4].info == 0, g[4].as_dict()
    assert g[4].true_resid <= case.params.tol
    ctx.close()


@pytest.mark.parametrize("gm", [1, 2, 3])
def test_drop_in_guess_extrapolation_keeps_the_answer(mf_case, gm):
    """guess_mode 1 / 2 on the per-routine calls: PhSolve extrapolates rmu through the previous
    calls' rmu, VeloSolve_2_combined u through u_pre (and the previous call's u_pre).  Only the
    starting guess changes, so at tol 1e-12 the answers agree with guess_mode 0 to 1e-9."""
    case, st, t = mf_case
    out = []
    for g in (0, gm):
        ctx, _ = _ctx(case, tol=1e-12, guess_mode=g)
        for _ in range(3):  # earlier calls: the history the quadratic and cubic guesses read
            ctx.PhSolve(st[F.F_U_PRE], st[F.F_V_PRE], st[F.F_PH_PRE], st[F.F_RMU_PRE], t - case.params.dt)
            ctx.VeloSolve_2_combined(st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE], st[F.F_U], st[F.F_V_PRE], st[F.F_V],
                                     st[F.F_P], None, st[F.F_PH], None, st[F.F_RMU], t)
        r, p, s1 = ctx.PhSolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], t)
        g = ctx.VeloSolve_2_combined(st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE], st[F.F_U], st[F.F_V_PRE], st[F.F_V],
                                     st[F.F_P], None, p, None, r, t)
        assert s1.info == 0 and g[4].info == 0
        out.append((r, p, g[0], g[1]))
        ctx.close()
    for a, b in zip(*out):
        assert rel_err(b, a) < 1e-9


# ------------------------------------------------------------------------------- step sequence
@pytest.mark.parametrize("precision,guess", [(abi.DRD_PREC_FP64, 0), (abi.DRD_PREC_MIXED, 0), (abi.DRD_PREC_MIXED, 1),
                                             (abi.DRD_PREC_MIXED, 2), (abi.DRD_PREC_FP64, 2),
                                             (abi.DRD_PREC_MIXED, 3), (abi.DRD_PREC_FP64, 3)])
def test_step_sequence_matches_oracle(cuda_lib, oracle_build, precision, guess):
    """Four mcl6 steps on the resident state against the oracle at tol 1e-12, where the result
    no longer depends on the Krylov guess (guess_mode 1 extrapolates it)."""
    from drd_application_gb300.workloads import make_case

    case = make_case("c2", seed=7, nr=48, nz=24)
    P = case.params.copy()
    P.tol = 1e-12
    P.precision = precision
    P.guess_mode = guess
    ctx = DRDContext(P)
    ctx.set_case(case)
    ctx.upload_state(case.state)
    orc = Oracle(P)
    st = case.copy_state()
    t = 0.0
    for s in range(4):
        stats = ctx.step(s == 0, t)
        so = orc.step(st, case.coefs, s == 0, t)
        assert stats.ch.info == 0 and stats.uv.info == 0
        t += P.dt
    g = ctx.download_state()
    tol = 1e-8 if precision == abi.DRD_PREC_FP64 else 1e-6
    for fid in (F.F_U, F.F_V, F.F_PH, F.F_RMU, F.F_P, F.F_PSI2):
        assert rel_err(g[fid], st[fid]) < tol, fid
    assert abs(stats.mass - orc.mass(st[F.F_PH])) < 1e-12 * max(1.0, abs(stats.mass))
    ctx.close()


def test_interpolate_coef_from_distance(cuda_lib, oracle_build):
    """drd_interpolate_coef (microfluidics_complex_domain/interpolate_coef.f90:4-92) from a
    caller's distance field: fpd_ph, rho, eta against the oracle, and they become the
    coefficients of the momentum operator."""
    from drd_application_gb300.workloads import make_case

    case = make_case("c2", seed=9, nr=64, nz=32, two_fluid=0, lambda_rho=2.0)
    ctx = DRDContext(case.params)
    ctx.set_case(case)
    rng = np.random.default_rng(5)
    dist = case.dist + 0.01 * rng.standard_normal(case.dist.shape)
    fpd, rho, eta = ctx.interpolate_coef(dist)
    orc = Oracle(case.params)
    fo, ro, eo = orc.interpolate_coef(dist, case.coefs["bdr_ph"])
    assert rel_err(fpd, fo) < 1e-14 and rel_err(rho, ro) < 1e-14 and rel_err(eta, eo) < 1e-14
    x = rng.standard_normal(ctx.L.drd_op_length(ctx.h, F.DRD_OP_UV_MATVEC))
    y = ctx.op_apply(F.DRD_OP_UV_MATVEC, x, bdf=2)
    assert rel_err(y, orc.uv_matvec(2, ro, eo, case.coefs["bdr_pen"], x)) < 1e-12
    ctx.close()
