"""The persistent cooperative FP32 inner solver against the kernel-per-phase graph loop.

Both run the same BiCGSTAB steps (lib/BiCGSTABREVCOM.f) for the inner solves of the mixed CH
solve; the refined FP64 result of each must meet the FP64 tolerance, agree with the other to
the level that tolerance allows, and take a similar number of inner iterations.
"""
import os

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
    assert abs(s1.iter - s0.iter) <= 0.25 * s0.iter + 10
