"""The persistent cooperative FP32 inner solver against the kernel-per-phase graph loop.

Both run the same BiCGSTAB steps (lib/BiCGSTABREVCOM.f) for the inner solves of the mixed CH
solve; the refined FP64 result of each must meet the FP64 tolerance, agree with the other to
the level that tolerance allows, and take a comparable number of inner iterations.
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


def _solve(case, persist):
    os.environ["DRD_PERSIST"] = "1" if persist else "0"
    try:
        ctx = DRDContext(case.params)
    finally:
        del os.environ["DRD_PERSIST"]
    ctx.set_case(case)
    st = case.state
    inputs = (st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU])
    r, p, s = ctx.PhSolve(*inputs, case.params.dt)
    on, why = ctx.persistent_solver()
    ctx.close()
    return inputs, r, p, s, on, why


@pytest.mark.parametrize("nr,nz", [(420, 180), (97, 53)])
def test_persistent_inner_solver(cuda_lib, oracle_build, nr, nz):
    case = make_case("c2", seed=3, nr=nr, nz=nz, precision=abi.DRD_PREC_MIXED)
    inputs, r1, p1, s1, on1, why1 = _solve(case, True)
    _, r0, p0, s0, on0, _ = _solve(case, False)
    assert on1, f"persistent solver not in use: {why1}"
    assert not on0
    for s in (s1, s0):
        assert s.info == 0, s.as_dict()
        assert s.true_resid <= case.params.tol
    orc = Oracle(case.params)
    assert orc.ch_residual(inputs, case.coefs, r1) <= 1.01 * case.params.tol
    assert rel_err(p1, p0) < 1e-6
    # FP32 BiCGSTAB iteration counts swing with rounding (both ways across seeds); only a gross
    # difference would point at a wrong step
    assert s1.iter <= 3 * s0.iter + 20


@pytest.mark.parametrize("nr,nz", [(420, 180), (97, 53), (64, 33)])
def test_persistent_operators_match_oracle(cuda_lib, oracle_build, nr, nz):
    """The persistent solver's own FP32 operator code (x-pass / z-divide-z / x-pass transform,
    stencils, Jacobi) against the FP64 oracle and the kernel-per-phase FP32 operators."""
    from tests.helpers import advanced_case

    case, st, t = advanced_case("c2", seed=2, nr=nr, nz=nz, steps=1)
    P = case.params.copy()
    P.precision = abi.DRD_PREC_MIXED
    ctx = DRDContext(P)
    ctx.set_case(case)
    orc = Oracle(P)
    on, why = ctx.persistent_solver()
    assert on, why
    rng = np.random.default_rng(nr)
    for op in (F.DRD_OP_CH_PSOLVE, F.DRD_OP_CH_MATVEC, F.DRD_OP_UV_MATVEC, F.DRD_OP_UV_PSOLVE):
        x = rng.standard_normal(ctx.L.drd_op_length(ctx.h, op))
        p32 = ctx.op_apply(op, x, precision=F.DRD_OP_PERSISTENT)
        g32 = ctx.op_apply(op, x, precision=F.DRD_PREC_MIXED)
        g64 = ctx.op_apply(op, x, precision=F.DRD_PREC_FP64)
        assert rel_err(g64, _oracle_op(orc, case, op, x)) < 1e-12, op
        assert rel_err(p32, g64) < 5e-5, (op, rel_err(p32, g64))
        assert rel_err(p32, g32) < 5e-5, (op, rel_err(p32, g32))
    ctx.close()


def _oracle_op(orc, case, op, x):
    k = case.coefs
    if op == F.DRD_OP_CH_PSOLVE:
        return orc.ch_psolve(x)
    if op == F.DRD_OP_CH_MATVEC:
        return orc.ch_matvec(k["M0"], k["Mi"], x)
    if op == F.DRD_OP_UV_MATVEC:
        return orc.uv_matvec(2, k["rho"], k["eta"], k["bdr_pen"], x)
    return orc.uv_psolve(2, k["rho"], k["eta"], x)


def test_grid_barrier_wait_is_bounded(cuda_lib):
    """Failure detection without a fault: a block that never reaches the persistent solver's grid
    barrier makes the waiting block give up after its bounded wait and report DRD_ERR_TIMEOUT;
    the context stays usable afterwards."""
    import time

    P = abi.default_params(64, 32)
    ctx = DRDContext(P)
    assert ctx.barrier_selftest(-1) == 0
    t0 = time.time()
    assert ctx.barrier_selftest(1) == abi.DRD_ERR_TIMEOUT
    assert time.time() - t0 < 60.0
    x = np.ones(64 * 32)
    y = ctx.op_apply(abi.DRD_OP_CH_PSOLVE, x)
    assert np.all(np.isfinite(y))
    assert ctx.barrier_selftest(-1) == 0
    ctx.close()
