"""drd_solve: A x = b for the step's Krylov systems on a caller's right-hand side (the C3 batch
of independent momentum solves, and the CH mu system).

CPU: the oracle's solve meets its tolerance on the C3 operators and the C3 generator is
deterministic.  GPU: the library's solve agrees with the oracle's (FP64 at tol 1e-12), and the
mixed mode reaches the FP64 tolerance, on C3 cases and on the CH system of the 420x180-style
workload.
"""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.workloads import make_c3_solve, make_case
from oracle.oracle import Oracle
from tests.helpers import rel_err

F = abi


def test_c3_generator_is_seeded(oracle_build):
    p1, c1, b1, m1 = make_c3_solve(3, 7)
    p2, c2, b2, m2 = make_c3_solve(3, 7)
    assert (p1.nr, p1.nz) == (p2.nr, p2.nz) and np.array_equal(b1, b2) and m1 == m2
    assert np.array_equal(b1, b1.astype(np.float32).astype(np.float64))  # stored FP32
    assert abs(b1.std() - 1.0) < 1e-3


@pytest.mark.parametrize("size", [(64, 32), (128, 64)])
def test_oracle_c3_solve_meets_tolerance(oracle_build, size):
    P, coefs, b, _ = make_c3_solve(0, 1, size=size, precision=abi.DRD_PREC_FP64)
    P.tol = 1e-10
    o = Oracle(P)
    x, st = o.solve(1, 2, coefs, b)
    assert st.info == 0
    r = b - o.uv_matvec(2, coefs["rho"], coefs["eta"], coefs["bdr_pen"], x)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("size", [(64, 32), (128, 64), (420, 180)])
def test_gpu_c3_solve_matches_oracle(cuda_lib, oracle_build, size):
    from drd_application_gb300.api import DRDContext

    P, coefs, b, _ = make_c3_solve(1, 2, size=size, precision=abi.DRD_PREC_FP64)
    P.tol = 1e-12
    ctx = DRDContext(P)
    ctx.set_coefs(coefs["rho"], coefs["eta"], coefs["bdr_ph"], coefs["bdr_ph_grad"], coefs["M0"], coefs["Mi"])
    x, st = ctx.solve(F.DRD_SYS_UV, b)
    xo, so = Oracle(P).solve(1, 2, coefs, b)
    assert st.info == 0 and so.info == 0
    assert st.true_resid <= 1e-11
    assert rel_err(x, xo) < 1e-9
    # the mixed mode from the same context parameters reaches the FP64 tolerance
    P.precision = F.DRD_PREC_MIXED
    P.tol = 1e-8
    ctx.set_params(P)
    xm, sm = ctx.solve(F.DRD_SYS_UV, b)
    assert sm.info == 0 and sm.true_resid <= 1e-8
    assert rel_err(xm, xo) < 1e-6
    ctx.close()


@pytest.mark.gpu
def test_gpu_ch_system_solve_matches_oracle(cuda_lib, oracle_build):
    from drd_application_gb300.api import DRDContext

    case = make_case("c2", seed=2, nr=97, nz=53)
    P = case.params.copy()
    P.tol = 1e-12
    ctx = DRDContext(P)
    ctx.set_case(case)
    b = np.random.default_rng(4).standard_normal(P.nr * P.nz)
    x, st = ctx.solve(F.DRD_SYS_CH, b)
    xo, so = Oracle(P).solve(0, 1, case.coefs, b)
    assert st.info == 0 and so.info == 0
    assert rel_err(x, xo) < 1e-9
    ctx.close()
