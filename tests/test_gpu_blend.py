"""The solid-blended CH preconditioner on the GPU, through the C-ABI, against the oracle: the
blended PSolve_CG in FP64, FP32 and in the persistent solver's own code, the probe fit, a
blended FP64 BiCGSTAB solve, the removal of the weights with new mobilities, the iteration
gain of the probe fit in the mixed time step, and the learned weights' gain on a held-out
geometry (the network trained on the GPU by the library's own kernels)."""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from drd_application_gb300.learned import evaluate_blend, learned_blend, train_blend
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import advanced_case, rel_err

pytestmark = pytest.mark.gpu


def _ctx(case, precision):
    P = case.params.copy()
    P.precision = precision
    ctx = DRDContext(P)
    ctx.set_case(case)
    return ctx


@pytest.fixture(scope="module")
def small(cuda_lib, oracle_build):
    case, st, _ = advanced_case("c2", seed=5, nr=96, nz=48, steps=2)
    return case, st, Oracle(case.params)


def test_blend_psolve_matches_oracle(small):
    case, _, orc = small
    n = case.nr * case.nz
    rng = np.random.default_rng(2)
    w = rng.uniform(0.0, 1.0, n)
    x = rng.standard_normal(n)
    ref = orc.ch_psolve_blend(w, x)
    for prec, tol in ((abi.DRD_PREC_FP64, 1e-12), (abi.DRD_PREC_MIXED, 2e-5)):
        ctx = _ctx(case, prec)
        try:
            ctx.set_ch_blend(w)
            y = ctx.op_apply(abi.DRD_OP_CH_PSOLVE, x, precision=prec)
            assert rel_err(y, ref) <= tol, (prec, rel_err(y, ref))
            if prec == abi.DRD_PREC_MIXED and ctx.persistent_solver()[0]:
                yp = ctx.op_apply(abi.DRD_OP_CH_PSOLVE, x, precision=abi.DRD_OP_PERSISTENT)
                assert rel_err(yp, ref) <= tol, rel_err(yp, ref)
            ctx.set_ch_blend(None)
            y0 = ctx.op_apply(abi.DRD_OP_CH_PSOLVE, x, precision=prec)
            assert rel_err(y0, orc.ch_psolve(x)) <= tol
        finally:
            ctx.close()


def test_blend_probe_matches_oracle(small):
    case, _, orc = small
    ref = orc.ch_blend_probe(case.coefs["M0"], case.coefs["Mi"], 16, 5)
    # FP64 transforms (FP64 context) and double-float transforms (mixed context)
    for prec, tol in ((abi.DRD_PREC_FP64, 1e-9), (abi.DRD_PREC_MIXED, 1e-6)):
        ctx = _ctx(case, prec)
        try:
            w = ctx.ch_blend_probe(16, 5, install=False)
            assert np.abs(w - ref).max() <= tol, (prec, np.abs(w - ref).max())
        finally:
            ctx.close()


def test_blend_solve_matches_oracle(small):
    case, st, orc = small
    M0, Mi = case.coefs["M0"], case.coefs["Mi"]
    b, x0, _ = orc.ch_system(st[abi.F_U], st[abi.F_V], st[abi.F_PH], st[abi.F_RMU], case.coefs["bdr_ph"],
                             case.coefs["bdr_ph_grad"], Mi)
    P = case.params.copy()
    P.precision = abi.DRD_PREC_FP64
    P.tol = 1e-11
    o = Oracle(P)
    ctx = DRDContext(P)
    try:
        ctx.set_case(case)
        w = ctx.ch_blend_probe(16, 3, install=True)
        xg, sg = ctx.solve(abi.DRD_SYS_CH, b, x0)
        xo, so = o.ch_solve_blend(M0, Mi, w, b, x0)
        assert sg.info == 0 and so.info == 0
        assert abs(sg.iter - so.iter) <= 2, (sg.iter, so.iter)
        assert rel_err(xg, xo) <= 1e-8
        _, s_ref = o.ch_solve_blend(M0, Mi, None, b, x0)
        assert so.iter < s_ref.iter
    finally:
        ctx.close()


def test_new_mobilities_remove_the_weights(small):
    case, _, orc = small
    n = case.nr * case.nz
    x = np.random.default_rng(4).standard_normal(n)
    ctx = _ctx(case, abi.DRD_PREC_FP64)
    try:
        ctx.set_ch_blend(np.full(n, 0.5))
        ctx.set_coefs(ph_M_0=case.coefs["M0"], ph_M_inner=case.coefs["Mi"])
        y = ctx.op_apply(abi.DRD_OP_CH_PSOLVE, x)
        assert rel_err(y, orc.ch_psolve(x)) <= 1e-12
    finally:
        ctx.close()


def test_probe_blend_cuts_mixed_step_iterations(cuda_lib):
    case = make_case("c2", seed=1, nr=210, nz=90, precision=abi.DRD_PREC_MIXED, guess_mode=3)
    ctx = _ctx(case, abi.DRD_PREC_MIXED)
    try:
        w = ctx.ch_blend_probe(32, 1, install=False)
    finally:
        ctx.close()
    ev = evaluate_blend(case, {"ref": None, "probe": w}, warmup=4, steps=4)
    for r in ev.values():
        assert r["converged"] == "4/4" and r["max_true_resid"] <= case.params.tol
    assert ev["probe"]["ch_iters"] <= 0.5 * ev["ref"]["ch_iters"], ev


def test_learned_blend_gain_on_held_out_geometry(cuda_lib):
    """The network, trained on the probe fits of four geometries, gives an unseen geometry
    weights that cut the mixed CH iterations well below PSolve_CG's."""
    nr, nz = 128, 56
    train = [make_case("c2", seed=100 + s, nr=nr, nz=nz, precision=abi.DRD_PREC_MIXED, guess_mode=3)
             for s in range(4)]
    net, info = train_blend(train, steps=300, nprobe=32)
    try:
        assert info["loss_last"] < 0.25 * info["loss_first"], info
        case = make_case("c2", seed=7, nr=nr, nz=nz, precision=abi.DRD_PREC_MIXED, guess_mode=3)
        w = learned_blend(net, case.coefs["M0"], case.coefs["Mi"])
        assert w.shape == (nr * nz,) and w.min() >= 0.0 and w.max() <= 1.0
        ev = evaluate_blend(case, {"ref": None, "learned": w}, warmup=4, steps=4)
        for r in ev.values():
            assert r["converged"] == "4/4" and r["max_true_resid"] <= case.params.tol
        assert ev["learned"]["ch_iters"] <= 0.6 * ev["ref"]["ch_iters"], ev
    finally:
        net.close()
