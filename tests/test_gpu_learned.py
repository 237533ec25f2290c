"""The learned CH guess end to end on a small C2 grid: pairs emitted by the solver's own GPU
runs, training by the library's kernels, evaluation on a held-out geometry.

What the trained network gains over the method without it: the error of the learned guess on
held-out steps is a small fraction of the error of the plain guess mu^n (it predicts
mu^{n+1} - mu^n).  What it does not change: the solve still reaches the FP64 tolerance from
either guess, and the FP64-residual judge returns the plain guess whenever the learned one's
residual is larger, so the iteration count never rises under that judge."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_learned_guess_gain_on_held_out_geometry(cuda_lib):
    from drd_application_gb300 import learned as LN
    from drd_application_gb300.workloads import make_case

    nr, nz = 96, 48
    data = LN.concat_pairs([LN.ch_run_pairs(make_case("c2", seed=1000 + s, nr=nr, nz=nz), 8, warmup=6)
                            for s in range(6)])
    net = LN.UNet(nz, nr, 3, 1, max_batch=8, seed=0)
    losses = LN.train(net, data, 400, batch=8, lr=1e-3, lr_final=1e-4)
    assert np.mean(losses[-20:]) < 0.05 * np.mean(losses[:5])
    case = make_case("c2", seed=2000, nr=nr, nz=nz)
    pr = LN.ch_run_pairs(case, 4, warmup=6)
    y = np.concatenate([net.forward(np.ascontiguousarray(pr["x"][k:k + 1])) for k in range(4)])
    # error of the learned guess relative to the error of the plain guess, per held-out step
    rel = np.sqrt(((y - pr["y"]) ** 2).sum(axis=(1, 2, 3)) / (pr["y"] ** 2).sum(axis=(1, 2, 3)))
    assert rel.max() < 0.3, rel
    for judge in ("none", "residual"):
        ev = LN.evaluate_ch(case, net, pr, judge=judge)
        assert (ev["true_resid_learned"] <= 1e-8).all() and (ev["true_resid_plain"] <= 1e-8).all()
        if judge == "residual":
            assert (ev["iters_learned"][~ev["used"]] == ev["iters_plain"][~ev["used"]]).all()
    net.close()
