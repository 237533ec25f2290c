"""Parity of the ESOLP_x momentum preconditioner (drd_params.uv_precond = DRD_UV_ESOLP) with
the FP64 CPU oracle, through the C-ABI: the operator in FP64 and FP32, and whole momentum
solves (Precipitation_dynamics/VeloSolve_combined.f90:800-806)."""
import os

import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from oracle.oracle import Oracle
from tests.helpers import advanced_case, rel_err

pytestmark = pytest.mark.gpu

F = abi


@pytest.fixture(scope="module")
def mf_case(cuda_lib, oracle_build):
    return advanced_case("c2", seed=3, nr=48, nz=24, steps=2)


def _ctx(case, **kw):
    P = case.params.copy()
    P.uv_precond = F.DRD_UV_ESOLP
    for k, v in kw.items():
        setattr(P, k, v)
    ctx = DRDContext(P)
    ctx.set_case(case)
    return ctx, Oracle(P)


@pytest.mark.parametrize("nr,nz", [(48, 24), (97, 53), (420, 180)])
@pytest.mark.parametrize("bdf", [1, 2])
def test_esolp_operator(cuda_lib, oracle_build, nr, nz, bdf):
    P = abi.default_params(nr, nz)
    P.dr, P.dz, P.dt = 3.5 / nr, 1.5 / nz, 1e-3
    P.uv_precond = F.DRD_UV_ESOLP
    ctx, orc = DRDContext(P), Oracle(P)
    x = np.random.default_rng(nr + bdf).standard_normal(ctx.L.drd_op_length(ctx.h, F.DRD_OP_UV_PSOLVE))
    zo = orc.uv_psolve_esolp(bdf, x)
    assert rel_err(ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=bdf), zo) < 1e-12
    assert rel_err(ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=bdf, precision=F.DRD_PREC_MIXED), zo) < 2e-5
    if ctx.persistent_solver()[0]:  # the persistent solver's own code: row passes, scanned Thomas sweeps
        zp = ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=bdf, precision=F.DRD_OP_PERSISTENT)
        assert rel_err(zp, zo) < 2e-5, rel_err(zp, zo)
    ctx.close()


@pytest.mark.parametrize("bdf", [1, 2])
def test_velosolve_esolp_tight(mf_case, bdf):
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
    assert abs(g[4].iter - o[4].iter) <= 4  # rounding moves the count by a few at this tolerance
    assert rel_err(g[0], o[0]) < 1e-9
    assert rel_err(g[1], o[1]) < 1e-9
    ctx.close()


def _mixed_esolp_steps(case, st, t, persist, nsteps=2, pre=F.DRD_UV_ESOLP):
    os.environ["DRD_PERSIST"] = "1" if persist else "0"
    try:
        ctx, _ = _ctx(case, precision=F.DRD_PREC_MIXED, uv_precond=pre)
    finally:
        del os.environ["DRD_PERSIST"]
    try:
        ctx.upload_state(st)
        rows = [ctx.step(False, t + s * case.params.dt) for s in range(nsteps)]
        g = ctx.download_state([F.F_U, F.F_V, F.F_PH])
        return rows, g, ctx.persistent_solver()[0]
    finally:
        ctx.close()


@pytest.mark.parametrize("pre", [F.DRD_UV_ESOLP, F.DRD_UV_ESOLP_SCALED])
def test_mixed_step_with_esolp_meets_tolerance(mf_case, pre):
    """Mixed-precision steps with ESOLP_x (plain and scaled), in the persistent solver and in the
    kernel-per-phase loop: both reach the FP64 tolerance and agree to the level it allows."""
    case, st, t = mf_case
    r1, g1, on = _mixed_esolp_steps(case, st, t, True, pre=pre)
    r0, g0, _ = _mixed_esolp_steps(case, st, t, False, pre=pre)
    assert on
    for rows in (r1, r0):
        for stats in rows:
            assert stats.uv.info == 0 and stats.ch.info == 0
            assert stats.uv.true_resid <= case.params.tol
    for fid in (F.F_U, F.F_V, F.F_PH):
        assert rel_err(g1[fid], g0[fid]) < 1e-6


def test_persistent_esolp_cuts_momentum_iterations(cuda_lib):
    """At 420x180 the persistent momentum solve with ESOLP_x needs well under half of Jacobi's
    FP32 iterations to the same FP64 residual."""
    from drd_application_gb300.workloads import make_case
    from tests.helpers import pack_uv

    case = make_case("c2", seed=2, precision=F.DRD_PREC_MIXED)
    orc = Oracle(case.params)
    st = case.copy_state()
    orc.step(st, case.coefs, True, 0.0)
    x_true = pack_uv(st[F.F_U], st[F.F_V])
    c = case.coefs
    b = orc.uv_matvec(2, c["rho"], c["eta"], c["bdr_pen"], x_true)
    its = {}
    for pre in (F.DRD_UV_JACOBI, F.DRD_UV_ESOLP):
        P = case.params.copy()
        P.uv_precond = pre
        ctx = DRDContext(P)
        try:
            ctx.set_case(case)
            assert ctx.persistent_solver()[0]
            x, s = ctx.solve(F.DRD_SYS_UV, b, np.zeros_like(b), bdf=2)
        finally:
            ctx.close()
        assert s.info == 0, s.as_dict()
        assert np.linalg.norm(b - orc.uv_matvec(2, c["rho"], c["eta"], c["bdr_pen"], x)) <= 1.0001e-8 * np.linalg.norm(b)
        its[pre] = s.iter
    assert its[F.DRD_UV_ESOLP] <= 0.5 * its[F.DRD_UV_JACOBI], its


@pytest.mark.parametrize("bdf", [1, 2])
def test_esolp_scaled_operator(cuda_lib, oracle_build, bdf):
    """DRD_UV_ESOLP_SCALED's preconditioner (the scaling from the context's rho and eta) in FP64,
    FP32 and the persistent solver's own code, against the oracle."""
    case, _, _ = advanced_case("c2", seed=6, nr=96, nz=48, steps=1)
    ctx, orc = _ctx(case, uv_precond=F.DRD_UV_ESOLP_SCALED)
    try:
        n = ctx.L.drd_op_length(ctx.h, F.DRD_OP_UV_PSOLVE)
        x = np.random.default_rng(bdf).standard_normal(n)
        s = orc.uv_esolp_scale(bdf, case.coefs["rho"], case.coefs["eta"])
        zo = orc.uv_psolve_esolp_scaled(bdf, s, x)
        assert rel_err(ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=bdf), zo) < 1e-12
        assert rel_err(ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=bdf, precision=F.DRD_PREC_MIXED), zo) < 2e-5
        if ctx.persistent_solver()[0]:
            zp = ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=bdf, precision=F.DRD_OP_PERSISTENT)
            assert rel_err(zp, zo) < 2e-5, rel_err(zp, zo)
    finally:
        ctx.close()


@pytest.mark.parametrize("bdf", [1, 2])
def test_velosolve_esolp_scaled_tight(mf_case, bdf):
    case, st, t = mf_case
    ctx, orc = _ctx(case, tol=1e-12, uv_precond=F.DRD_UV_ESOLP_SCALED)
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
    assert abs(g[4].iter - o[4].iter) <= 4
    assert rel_err(g[0], o[0]) < 1e-9
    assert rel_err(g[1], o[1]) < 1e-9
    ctx.close()


def test_persistent_esolp_scaled_cuts_iterations(cuda_lib):
    """At 420x180 with the two-fluid coefficients the scaled form needs fewer persistent mixed
    momentum iterations than ESOLP_x, and both reach the FP64 residual."""
    from drd_application_gb300.workloads import make_case
    from tests.helpers import pack_uv

    case = make_case("c2", seed=2, precision=F.DRD_PREC_MIXED)
    orc = Oracle(case.params)
    st = case.copy_state()
    orc.step(st, case.coefs, True, 0.0)
    x_true = pack_uv(st[F.F_U], st[F.F_V])
    c = case.coefs
    b = orc.uv_matvec(2, c["rho"], c["eta"], c["bdr_pen"], x_true)
    its = {}
    for pre in (F.DRD_UV_ESOLP, F.DRD_UV_ESOLP_SCALED):
        P = case.params.copy()
        P.uv_precond = pre
        ctx = DRDContext(P)
        try:
            ctx.set_case(case)
            assert ctx.persistent_solver()[0]
            x, s = ctx.solve(F.DRD_SYS_UV, b, np.zeros_like(b), bdf=2)
        finally:
            ctx.close()
        assert s.info == 0, s.as_dict()
        assert np.linalg.norm(b - orc.uv_matvec(2, c["rho"], c["eta"], c["bdr_pen"], x)) <= 1.0001e-8 * np.linalg.norm(b)
        its[pre] = s.iter
    assert its[F.DRD_UV_ESOLP_SCALED] < its[F.DRD_UV_ESOLP], its


@pytest.mark.parametrize("nr,nz", [(512, 256), (1024, 512)])
@pytest.mark.parametrize("pre", [F.DRD_UV_ESOLP, F.DRD_UV_ESOLP_SCALED])
def test_persistent_esolp_operator_large(cuda_lib, oracle_build, nr, nz, pre):
    """The persistent solver's ESOLP_x where the row transforms span several K chunks (512x256:
    K = 257, resident B panels) and where the tiles outnumber the blocks (1024x512: B streamed)."""
    P = abi.default_params(nr, nz)
    P.dr, P.dz, P.dt = 3.5 / nr, 1.5 / nz, 1e-3
    P.uv_precond = pre
    P.precision = F.DRD_PREC_MIXED
    rng = np.random.default_rng(nr)
    cs = (nr + 2) * (nz + 2)
    rho = (1.0 + rng.uniform(0, 1, cs)).reshape(nz + 2, nr + 2)
    eta = (1.0 + 4.0 * rng.uniform(0, 1, cs)).reshape(nz + 2, nr + 2)
    ctx, orc = DRDContext(P), Oracle(P)
    try:
        ctx.set_coefs(rho=rho, eta=eta)
        if not ctx.persistent_solver()[0]:
            pytest.skip("persistent solver not in use")
        x = rng.standard_normal(ctx.L.drd_op_length(ctx.h, F.DRD_OP_UV_PSOLVE))
        if pre == F.DRD_UV_ESOLP_SCALED:
            zo = orc.uv_psolve_esolp_scaled(2, orc.uv_esolp_scale(2, rho, eta), x)
        else:
            zo = orc.uv_psolve_esolp(2, x)
        zp = ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=2, precision=F.DRD_OP_PERSISTENT)
        assert rel_err(zp, zo) < 2e-5, rel_err(zp, zo)
    finally:
        ctx.close()
