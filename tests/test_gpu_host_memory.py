"""Page-locked host arrays (drd_host_register) and caller-supplied output arrays of the drop-in
routines: the results are the same as with pageable arrays and fresh outputs."""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext, pin, unpin
from tests.helpers import advanced_case

pytestmark = pytest.mark.gpu
F = abi


def test_pinned_inputs_and_out_buffers(cuda_lib, oracle_build):
    case, st, t = advanced_case("c2", seed=8, nr=96, nz=48, steps=2)
    ctx = DRDContext(case.params)
    try:
        ctx.set_case(case)
        args = [st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU]]
        r0, p0, s0 = ctx.PhSolve(*args, t)
        pinned = [pin(np.array(a)) for a in args]
        outs = (pin(np.full(ctx.cs, np.nan)), pin(np.full(ctx.cs, np.nan)))
        r1, p1, s1 = ctx.PhSolve(*pinned, t, out=outs)
        assert r1 is outs[0] and p1 is outs[1]
        assert s0.info == 0 and s1.info == 0
        assert np.array_equal(r0, r1) and np.array_equal(p0, p1)
        psi = pin(np.full(ctx.cs, np.nan))
        assert np.array_equal(ctx.PreSolve_2(pinned[0], pinned[1], 2.0, out=psi), ctx.PreSolve_2(args[0], args[1], 2.0))
        for a in pinned + list(outs) + [psi]:
            unpin(a)
        with pytest.raises(ValueError):
            ctx.PhSolve(*args, t, out=(np.zeros(ctx.cs, dtype=np.float32), np.zeros(ctx.cs)))
    finally:
        ctx.close()


def test_pinned_velosolve_coef_and_mixed_inputs(cuda_lib, oracle_build):
    """VeloSolve_2_combined and the two-fluid coefficients with page-locked inputs and outputs
    (copied by the calls' gather and scatter launches), with a mix of page-locked and pageable
    inputs in one call, and with pageable arrays (DMA copies): the same results bit for bit."""
    case, st, t = advanced_case("c2", seed=9, nr=96, nz=48, steps=2)
    ctx = DRDContext(case.params)
    try:
        ctx.set_case(case)
        rmu_a, ph_a, _ = ctx.PhSolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], t)
        args = [st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE], st[F.F_U], st[F.F_V_PRE], st[F.F_V], st[F.F_P],
                st[F.F_PH_PRE], ph_a, st[F.F_RMU_PRE], rmu_a]
        ref = ctx.VeloSolve_2_combined(*args, t)
        assert ref[4].info == 0
        pinned = [pin(np.array(a)) for a in args]
        outs = (pin(np.full(ctx.us, np.nan)), pin(np.full(ctx.vs, np.nan)), pin(np.full(ctx.nz + 1, np.nan)),
                pin(np.full(ctx.nz + 1, np.nan)))
        mixed_in = [p if i % 2 else np.array(a) for i, (a, p) in enumerate(zip(args, pinned))]
        try:
            for inputs in (pinned, mixed_in):
                got = ctx.VeloSolve_2_combined(*inputs, t, out=outs)
                assert got[4].info == 0
                for g, r in zip(got[:2], ref[:2]):
                    assert np.array_equal(g, r)
                assert np.array_equal(got[2][:ctx.nz], ref[2][:ctx.nz])
            ro, eo = pin(np.full(ctx.cs, np.nan)), pin(np.full(ctx.cs, np.nan))
            try:
                rho1, eta1 = ctx.two_phase_coef(None, pinned[8], out=(ro, eo))
                assert rho1 is ro and eta1 is eo
                rho2, eta2 = ctx.two_phase_coef(None, ph_a)
                assert np.array_equal(rho1, rho2) and np.array_equal(eta1, eta2)
            finally:
                unpin(ro)
                unpin(eo)
        finally:
            for a in pinned + list(outs):
                unpin(a)
    finally:
        ctx.close()
