"""dissipation's diagnostics and reinint_by_PhSolve on the GPU against the oracle, through the
C-ABI (microfluidics_complex_domain/dissipation.f90:1-122,
two_phase_flow_complex_domain/reinint_by_PhSolve.f90:1-91)."""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from drd_application_gb300.layout import neumann_ghosts_cell
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import advanced_case, rel_err

pytestmark = pytest.mark.gpu
F = abi


@pytest.mark.parametrize("nr,nz", [(48, 24), (420, 180)])
def test_dissipation_matches_oracle(cuda_lib, oracle_build, nr, nz):
    if nr <= 64:
        case, st, _ = advanced_case("c2", seed=6, nr=nr, nz=nz, steps=2)
    else:
        case = make_case("c2", seed=6)
        st = case.copy_state()
        rng = np.random.default_rng(1)
        st[F.F_U] = rng.standard_normal(st[F.F_U].shape)
        st[F.F_V] = rng.standard_normal(st[F.F_V].shape)
    P = case.params
    ctx = DRDContext(P)
    orc = Oracle(P)
    rng = np.random.default_rng(nr)
    angB, angT = rng.uniform(30, 150, nr + 1), rng.uniform(30, 150, nr + 1)
    for ang in ((None, None), (angB, angT)):
        g = ctx.dissipation(5.0e4, st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], *ang).as_tuple()
        o = orc.dissipation(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], 5.0e4, *ang)
        for name, a, b in zip(("e1", "e2", "e3", "e4", "dissip", "mass"), g, o):
            assert abs(a - b) <= 1e-12 * max(abs(b), 1e-300), (name, a, b)
    # the resident fields (NULL arrays) give the same numbers
    ctx.upload_state(st)
    r = ctx.dissipation(5.0e4).as_tuple()
    assert rel_err(np.array(r), np.array(o if angB is None else orc.dissipation(
        st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], 5.0e4))) < 1e-12
    ctx.close()


def test_reinint_by_phsolve_matches_oracle(cuda_lib, oracle_build):
    case = make_case("tp", seed=3, nr=84, nz=36)
    P = case.params.copy()
    P.dt, P.tol = 1.0e-4, 1e-13
    sharp = np.where(case.coefs["bdr_ph"] > 0.5, 1.0, -1.0)
    neumann_ghosts_cell(sharp)
    ctx = DRDContext(P)
    b, pen, info = ctx.reinint_by_PhSolve(sharp)
    bo, peno, info_o = Oracle(P).reinint_by_phsolve(sharp)
    assert info == 0 and info_o == 0
    # 51 smoothing steps from a sharp mask: the oracle against itself, tol 1e-13 against 1e-14,
    # moves bdr_ph by 1.8e-7 here (its unclipped ghost rows carry the largest values)
    assert rel_err(b, bo) < 1e-7
    decided = np.abs(bo - 0.5) > 1e-6
    assert np.array_equal(pen[decided], peno[decided])
    # both became the context's: the TP momentum operator now penalises with the new mask
    x = np.random.default_rng(2).standard_normal(ctx.L.drd_op_length(ctx.h, F.DRD_OP_UV_MATVEC))
    y = ctx.op_apply(F.DRD_OP_UV_MATVEC, x, bdf=2)
    yo = Oracle(P).uv_matvec(2, np.ones_like(b), np.ones_like(b), pen, x)
    ctx.close()
    assert rel_err(y, yo) < 1e-12
