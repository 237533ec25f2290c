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
