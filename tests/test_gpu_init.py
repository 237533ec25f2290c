"""PhSolve_ori and finit's wall smoothing on the GPU against the oracle
(microfluidics_complex_domain/PhSolve_ori.f90, finit.f90:120-189), through the C-ABI."""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from drd_application_gb300.layout import u_shape, v_shape
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _params(nr, nz, tol=1e-12, precision=abi.DRD_PREC_FP64):
    p = abi.default_params(nr, nz, tol=tol)
    p.dr, p.dz = 3.5 / nr, 1.5 / nz
    p.dt = 1.0e-4  # finit.f90:151
    p.precision = precision
    return p


@pytest.mark.parametrize("precision", [abi.DRD_PREC_FP64, abi.DRD_PREC_MIXED])
def test_phsolve_ori(cuda_lib, oracle_build, precision):
    P = _params(84, 36, precision=precision)
    case = make_case("c2", seed=4, nr=P.nr, nz=P.nz)
    ph = 2.0 * case.coefs["bdr_ph"] - 1.0
    rng = np.random.default_rng(2)
    u, v = 0.1 * rng.standard_normal(u_shape(P.nr, P.nz)), 0.1 * rng.standard_normal(v_shape(P.nr, P.nz))
    angB, angT = rng.uniform(30, 150, P.nr + 1), rng.uniform(30, 150, P.nr + 1)
    ctx = DRDContext(P)
    rmu_g, ph_g, st = ctx.PhSolve_ori(u, v, ph, angB, angT, 0.3)
    rmu_o, ph_o, st_o = Oracle(P).phsolve_ori(u, v, ph, angB, angT, 0.3)
    assert st.info == 0 and st_o.info == 0
    tol = 1e-9 if precision == abi.DRD_PREC_FP64 else 1e-7
    assert rel_err(ph_g, ph_o) < tol and rel_err(rmu_g, rmu_o) < 1e3 * tol
    assert st.true_resid <= P.tol * 1.0001
    ctx.close()


def test_finit_wall(cuda_lib, oracle_build):
    P = _params(84, 36, tol=1e-10)
    case = make_case("c2", seed=6, nr=P.nr, nz=P.nz)
    sharp = (case.coefs["bdr_ph"] > 0.5).astype(np.float64)
    ctx = DRDContext(P)
    b_g, ph_g, rmu_g, info = ctx.finit_wall(sharp, 6)
    b_o, ph_o, rmu_o, info_o = Oracle(P).finit_wall(sharp, 6)
    assert info == 0 and info_o == 0
    assert rel_err(ph_g, ph_o) < 1e-8 and rel_err(b_g, b_o) < 1e-8
    assert rel_err(rmu_g, rmu_o) < 1e-6
    ctx.close()
