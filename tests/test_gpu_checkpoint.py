"""Checkpoint of the resident state (drd_checkpoint_async): the file written while the GPU
runs on equals `output` of the fields downloaded at the same point of the step sequence."""
import numpy as np
import pytest

from drd_application_gb300 import abi, fileio
from drd_application_gb300.api import DRDContext
from drd_application_gb300.workloads import make_case

pytestmark = pytest.mark.gpu


def test_checkpoint_async_matches_download(cuda_lib, tmp_path):
    case = make_case("c2", seed=2, nr=60, nz=30, particles=True)
    P = case.params
    parts = case.meta["particles"]
    ctx = DRDContext(P)
    ctx.set_case(case)
    ctx.upload_state(case.state)
    ctx.particles_set(parts["pp"], parts["points"], parts["bdr_dist"])
    t = 0.0
    for s in range(2):
        ctx.step(s == 0, t)
        t += P.dt
    path = tmp_path / "data001"
    ctx.checkpoint_async(path, t)
    g = ctx.download_state()            # same point: after step 2, before step 3
    fpd, _, _ = ctx.interpolate_coef_particles()
    ctx.step(False, t)                  # runs while the file is written
    ctx.checkpoint_wait()
    ref = tmp_path / "ref001"
    fileio.output(ref, P.nr, P.nz, P.dr, P.dz, g[abi.F_U], g[abi.F_V], g[abi.F_P], fpd, g[abi.F_PH], t)
    assert open(path, "rb").read() == open(ref, "rb").read()
    assert fileio.read_time(path, P.nr, P.nz) == t
    ctx.close()
