"""The batched solver (drd_batch_*): independent momentum and pressure Poisson systems of
uneven sizes in one persistent launch, checked against the FP64 operators and solves of the
oracle, through the C-ABI."""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.batch import Batch
from drd_application_gb300.workloads import make_c3_pressure, make_c3_solve
from oracle.oracle import Oracle
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

SIZES = [(64, 32), (128, 64), (256, 128), (420, 180), (512, 256), (96, 40)]


def _systems(seed, sizes):
    out = []
    for j, sz in enumerate(sizes):
        P, c, b, _ = make_c3_solve(seed, j, size=sz)
        out.append(("uv", P, {"rho": c["rho"], "eta": c["eta"], "bdr_ph": c["bdr_ph"]}, b))
        P, bdr, bp, _ = make_c3_pressure(seed, j, size=sz)
        out.append(("pressure", P, bdr, bp))
    return out


def _true_resid(orc, kind, sysd, x):
    if kind == "uv":
        c = sysd[2]
        Ax = orc.uv_matvec(2, c["rho"], c["eta"], c["bdr_ph"], x)
    else:
        Ax = orc.pressure_matvec(sysd[2], x)
    b = sysd[3]
    return float(np.linalg.norm(b - Ax) / np.linalg.norm(b))


def test_batch_solves_reach_fp64_tolerance(cuda_lib, oracle_build):
    systems = _systems(7, SIZES)
    bt = Batch(systems, autotune=False)
    sec = bt.run()
    assert sec > 0
    for i, s in enumerate(systems):
        x, st = bt.result(i)
        assert st.info == 0, (i, s[0], s[1].nr, s[1].nz, st.as_dict())
        tr = _true_resid(Oracle(s[1]), s[0], s, x)
        assert tr <= 1.0001e-8, (i, s[0], tr)
        assert abs(tr - st.true_resid) <= 1e-3 * tr + 1e-15
    bt.close()


def test_batch_matches_oracle_solutions(cuda_lib, oracle_build):
    """A sample against the oracle's own solves (reference BiCGSTAB, FP64, tol 1e-11)."""
    systems = _systems(3, [(64, 32), (96, 40)])
    bt = Batch(systems, autotune=False)
    bt.run()
    for i, s in enumerate(systems):
        x, st = bt.result(i)
        P = s[1].copy()
        P.tol = 1e-11
        P.uv_maxit = 4000
        orc = Oracle(P)
        if s[0] == "uv":
            c = s[2]
            k = {"rho": c["rho"], "eta": c["eta"], "bdr_pen": c["bdr_ph"], "M0": c["rho"], "Mi": c["rho"]}
            xo, so = orc.solve(abi.DRD_SYS_UV, 2, k, s[3])
            assert so.info == 0
        else:
            xo, so, info = orc.pressure_solve(s[2], s[3])
            assert info == 0
            # the constant null space: compare zero-mean parts
            x, xo = x - x.mean(), xo - xo.mean()
        assert rel_err(x, xo) < 1e-6, (i, s[0], rel_err(x, xo))
    bt.close()


def test_batch_runs_are_repeatable_and_autotuned(cuda_lib, oracle_build):
    systems = _systems(11, [(64, 32), (128, 64), (180, 84)])
    bt = Batch(systems, autotune=True)
    info = bt.info()
    assert info["threads"] in (256, 512, 1024) and info["blocks_per_sm"] >= 1
    bt.run()
    a = [bt.result(i)[0] for i in range(len(systems))]
    bt.run()
    b = [bt.result(i)[0] for i in range(len(systems))]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert bt.info()["bytes_last_run"] > 0
    bt.close()


def test_batch_rejects_bad_systems(cuda_lib):
    P, bdr, b, _ = make_c3_pressure(1, 0, size=(64, 32))
    P2 = P.copy()
    P2.nr = 67  # 67 is prime: no FFT plan for the pressure preconditioner
    with pytest.raises(Exception):
        Batch([("pressure", P2, np.zeros((P.nz + 2, 69)), np.zeros(67 * P.nz))], autotune=False)
