"""Parity of the ESOLP_x momentum preconditioner (drd_params.uv_precond = DRD_UV_ESOLP) with
the FP64 CPU oracle, through the C-ABI: the operator in FP64 and FP32, and whole momentum
solves (Precipitation_dynamics/VeloSolve_combined.f90:800-806)."""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext, DRDError
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
    with pytest.raises(DRDError):  # the persistent momentum solver applies Jacobi only
        ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=bdf, precision=F.DRD_OP_PERSISTENT)
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


def test_mixed_step_with_esolp_meets_tolerance(mf_case):
    """A mixed-precision step with ESOLP_x: the momentum solve runs the FP32 BiCGSTAB of the
    kernel-per-phase loop (not the persistent solver) and still reaches the FP64 tolerance."""
    case, st, t = mf_case
    ctx, _ = _ctx(case, precision=F.DRD_PREC_MIXED)
    ctx.upload_state(st)
    for s in range(2):
        stats = ctx.step(False, t + s * case.params.dt)
        assert stats.uv.info == 0 and stats.ch.info == 0
        assert stats.uv.true_resid <= case.params.tol
    ctx.close()
