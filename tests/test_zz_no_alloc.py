"""The allocation-free pressure step (drd_presolve_2_noalloc) against drd_presolve_2 and the
oracle.

drd_presolve_2_noalloc exists for callers that cannot let the library call cudaMalloc: an
application whose device memory all belongs to its own pool allocator, or a driver issuing
the pressure step from code where allocation is not allowed.  It keeps its intermediates in a
fixed-size __device__ array instead, and the caller passes device buffers for u, v and psi.
This file is collected last (tests/test_zz_*), and each case checks two calls in a row, since
every call reuses the same array.
"""
import ctypes as C

import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import advanced_case, rel_err

pytestmark = pytest.mark.gpu


def _noalloc(lib, P, u, v, coef):
    import torch

    du = torch.from_numpy(u).cuda()
    dv = torch.from_numpy(v).cuda()
    dpsi = torch.full((P.nz + 2, P.nr + 2), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.drd_presolve_2_noalloc(P.nr, P.nz, P.dr, P.dz, C.c_void_p(du.data_ptr()), C.c_void_p(dv.data_ptr()),
                                    coef, C.c_void_p(dpsi.data_ptr()), None)
    torch.cuda.synchronize()
    assert rc == 0
    return dpsi.cpu().numpy()


@pytest.mark.parametrize("nr,nz", [(48, 24), (420, 180)])
def test_noalloc_presolve_matches_presolve_2_twice(cuda_lib, oracle_build, nr, nz):
    case, st, _ = advanced_case("c2", seed=9, nr=nr, nz=nz, steps=1) if nr <= 64 else (make_case("c2", seed=9, nr=nr, nz=nz), None, 0.0)
    P = case.params
    ctx = DRDContext(P)
    orc = Oracle(P)
    rng = np.random.default_rng(nr)
    for call in range(2):
        if st is not None and call == 0:
            u, v = st[abi.F_U].copy(), st[abi.F_V].copy()
        else:
            u = rng.standard_normal(ctx.us)
            v = rng.standard_normal(ctx.vs)
        coef = 3 * P.re / 2.0 / P.dt * (1.0 + call)
        ref = ctx.PreSolve_2(u, v, coef)
        got = _noalloc(cuda_lib, P, u, v, coef)
        assert np.isfinite(got).all()
        assert rel_err(got, ref) < 1e-12, (call, rel_err(got, ref))
        # and against the oracle's PreSolve_2 + dct_fftw directly
        assert rel_err(got, orc.presolve(u, v, coef)) < 1e-12, call
    ctx.close()


def test_noalloc_rejects_grids_beyond_its_scratch(cuda_lib):
    P = abi.default_params(2048, 1024)
    one = C.c_void_p(1)  # never dereferenced: the size check comes first
    rc = cuda_lib.drd_presolve_2_noalloc(P.nr, P.nz, P.dr, P.dz, one, one, 1.0, one, None)
    assert rc == abi.DRD_ERR_TOO_LARGE
