"""Full-size (420x180) and odd-size checks of the transform kernels and the solves.

Every tile configuration of the transform GEMMs (the autotuner may pick any of them for a
given grid) is forced in turn and checked against the oracle's DCT-I preconditioner; the CH
solve at 420x180 must meet the deck tolerance in both arithmetic modes.
"""
import os

import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu
F = abi


N_CFG_FP32, N_CFG_FP64 = 9, 14  # configurations 9-13: the FP64-only double-float kernels


@pytest.mark.parametrize("nr,nz", [(420, 180), (97, 53)])
def test_every_gemm_config_matches_oracle(cuda_lib, oracle_build, nr, nz):
    case = make_case("c2", seed=1, nr=nr, nz=nz)
    orc = Oracle(case.params)
    x = np.random.default_rng(nr).standard_normal(nr * nz)
    ref = orc.ch_psolve(x)
    bad = []
    for cfg in range(N_CFG_FP64):
        # FP64 GEMM configurations serve the FP64 mode; the double-float ones (9-11) serve the
        # mixed mode's FP64 transforms, so they are checked from a mixed-mode context
        os.environ["DRD_GEMM_CFG"] = str(cfg)
        P = case.params.copy()
        if cfg >= N_CFG_FP32:
            P.precision = F.DRD_PREC_MIXED
        try:
            ctx = DRDContext(P)
            ctx.set_case(case)
            e64 = rel_err(ctx.op_apply(F.DRD_OP_CH_PSOLVE, x), ref)
            e32 = rel_err(ctx.op_apply(F.DRD_OP_CH_PSOLVE, x, precision=F.DRD_PREC_MIXED), ref)
            ctx.close()
        finally:
            del os.environ["DRD_GEMM_CFG"]
        if not (e64 < 1e-12 and e32 < 5e-5):
            bad.append((cfg, e64, e32))
    assert not bad, bad


@pytest.mark.parametrize("precision", [abi.DRD_PREC_FP64, abi.DRD_PREC_MIXED])
def test_fullsize_first_step_solves_meet_tolerance(cuda_lib, oracle_build, precision):
    case = make_case("c2", seed=0, precision=precision)
    P = case.params
    ctx = DRDContext(P)
    ctx.set_case(case)
    st = case.state
    inputs = (st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU])
    r, p, s = ctx.PhSolve(*inputs, P.dt)
    assert s.info == 0, s.as_dict()
    assert s.true_resid <= P.tol
    assert not (s.flags & F.DRD_FLAG_FALLBACK64)  # FP32 carries the 420x180 CH system
    orc = Oracle(P)
    assert orc.ch_residual(inputs, case.coefs, r) <= 1.01 * P.tol
    u, v, _, _, s2 = ctx.VeloSolve_combined(None, st[F.F_U], st[F.F_V], st[F.F_P], r, p, P.dt)
    assert s2.info == 0 and s2.true_resid <= P.tol, s2.as_dict()
    ctx.close()


def test_c5_mixed_step_solves_ch_in_fp64_and_conserves_mass(cuda_lib):
    """2048x1024 with 64 fibers and 32 drops.  The CH system there is too stiff for FP32 Krylov
    vectors (stiffness estimate 0.42 > 0.1), so the mixed mode solves it with the FP64 solver
    and flags it; the momentum solve stays mixed.  Size-independent checks: the momentum solve
    meets the tolerance, the CH residual falls below 1e-6 within the reference's 500
    iterations, the fields stay finite and the phase-field mass moves by < 1e-6 relative."""
    case = make_case("c5", seed=0, precision=abi.DRD_PREC_MIXED)
    ctx = DRDContext(case.params)
    ctx.set_case(case)
    ctx.upload_state(case.state)
    m0 = ctx.mass(case.state[F.F_PH])
    st = ctx.step(True, 0.0)
    assert st.ch.flags & F.DRD_FLAG_FALLBACK64
    assert st.ch.true_resid < 1e-6, st.ch.as_dict()
    assert st.uv.info == 0 and st.uv.true_resid <= case.params.tol, st.uv.as_dict()
    assert not (st.uv.flags & F.DRD_FLAG_FALLBACK64)
    assert abs(st.mass - m0) / m0 < 1e-6
    out = ctx.download_state([F.F_U, F.F_V, F.F_PH, F.F_P])
    assert all(np.isfinite(a).all() for a in out.values())
    ctx.close()


def test_c5_mixed_step_with_blend_solves_ch_in_fp32(cuda_lib):
    """The same step with the probe-fitted blend in the CH preconditioner and the scaled ESOLP_x:
    with the blend the FP32 inner CH solves converge at this stiffness (the library raises the
    limit while weights are installed), and both solves reach the FP64 tolerance that PSolve_CG
    alone does not reach within the reference's 500 iterations."""
    case = make_case("c5", seed=0, precision=abi.DRD_PREC_MIXED, uv_precond=abi.DRD_UV_ESOLP_SCALED)
    ctx = DRDContext(case.params)
    ctx.set_case(case)
    ctx.ch_blend_probe(64, 11, install=True)
    ctx.upload_state(case.state)
    m0 = ctx.mass(case.state[F.F_PH])
    st = ctx.step(True, 0.0)
    assert not (st.ch.flags & F.DRD_FLAG_FALLBACK64)
    assert st.ch.info == 0 and st.ch.true_resid <= case.params.tol, st.ch.as_dict()
    assert st.uv.info == 0 and st.uv.true_resid <= case.params.tol, st.uv.as_dict()
    assert abs(st.mass - m0) / m0 < 1e-6
    ctx.set_ch_blend(None)  # without weights the stiffness rule sends it back to the FP64 solver
    st2 = ctx.step(False, case.params.dt)
    assert st2.ch.flags & F.DRD_FLAG_FALLBACK64
    ctx.close()


@pytest.mark.parametrize("precision", [abi.DRD_PREC_FP64, abi.DRD_PREC_MIXED])
def test_c1_steps_match_oracle(cuda_lib, oracle_build, precision):
    """The C1 configuration at its own size (128x64, one drop, no solid, tol 1e-10): five
    resident mcl6 steps against the oracle's five steps."""
    case = make_case("c1", seed=0)
    P = case.params.copy()
    P.precision = precision
    ctx = DRDContext(P)
    ctx.set_case(case)
    ctx.upload_state(case.state)
    orc = Oracle(P)
    st = case.copy_state()
    t = 0.0
    for s in range(5):
        g = ctx.step(s == 0, t)
        orc.step(st, case.coefs, s == 0, t)
        t += P.dt
        assert g.ch.info == 0 and g.uv.info == 0, (g.ch.as_dict(), g.uv.as_dict())
        assert g.ch.true_resid <= P.tol and g.uv.true_resid <= P.tol
    out = ctx.download_state([F.F_U, F.F_V, F.F_PH, F.F_RMU, F.F_P])
    lim = 1e-6 if precision == abi.DRD_PREC_FP64 else 1e-4
    for fid, a in out.items():
        assert rel_err(a, st[fid]) < lim, fid
    ctx.close()


def test_direct_launch_mode_matches_graph_mode(cuda_lib):
    """DRD_DIRECT_LAUNCH=1 (per-kernel launches, host-run loops; used for profiling) computes
    exactly what the captured graphs compute: the reductions are in a fixed order."""
    case = make_case("c2", seed=4, nr=64, nz=32, precision=abi.DRD_PREC_MIXED)
    out = []
    for direct in (False, True):
        if direct:
            os.environ["DRD_DIRECT_LAUNCH"] = "1"
        try:
            ctx = DRDContext(case.params)
            ctx.set_case(case)
            ctx.upload_state(case.state)
            t = 0.0
            for s in range(3):
                st = ctx.step(s == 0, t)
                t += case.params.dt
            out.append((ctx.download_state([F.F_U, F.F_PH, F.F_P]), st.ch.iter, st.uv.iter))
            ctx.close()
        finally:
            os.environ.pop("DRD_DIRECT_LAUNCH", None)
    (a, ia, ja), (b, ib, jb) = out
    assert (ia, ja) == (ib, jb)
    for fid in a:
        assert np.array_equal(a[fid], b[fid]), fid
