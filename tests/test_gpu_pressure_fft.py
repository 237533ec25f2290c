"""PreSolve_2 by FFT (drd_pressure_fft.cu) on the GPU: against the oracle's direct transforms,
against the GEMM-form transforms the library keeps for grids whose sides are not of the form
2^a 3^b 5^c 7^d (DRD_PRESSURE_FFT=0 forces them), and the kernel bench's cold-L2 timings."""
import os

import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from oracle.oracle import Oracle
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _params(nr, nz):
    P = abi.default_params(nr, nz)
    P.dr, P.dz = 3.5 / nr, 1.5 / nz
    return P


def _uv(P, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((P.nz + 2, P.nr + 3)), rng.standard_normal((P.nz + 1, P.nr + 2))


def _presolve(P, u, v, coef, fft):
    if not fft:
        os.environ["DRD_PRESSURE_FFT"] = "0"
    try:
        ctx = DRDContext(P)
    finally:
        os.environ.pop("DRD_PRESSURE_FFT", None)
    psi = ctx.PreSolve_2(u, v, coef)
    ctx.close()
    return psi


@pytest.mark.parametrize("nr,nz", [(420, 180), (48, 24), (128, 64), (210, 98)])
def test_fft_presolve_matches_oracle(cuda_lib, oracle_build, nr, nz):
    P = _params(nr, nz)
    u, v = _uv(P, nr)
    coef = 3 * P.re / 2.0 / P.dt
    psi = _presolve(P, u, v, coef, True)
    ref = Oracle(P).presolve(u, v, coef)
    assert rel_err(psi, ref) < 1e-13


@pytest.mark.parametrize("nr,nz", [(512, 256), (2048, 1024)])
def test_fft_presolve_matches_gemm_form(cuda_lib, nr, nz):
    """At sizes where the O(n^2) oracle is slow, the FFT and GEMM forms agree with each other."""
    P = _params(nr, nz)
    u, v = _uv(P, nz)
    a = _presolve(P, u, v, 1.0, True)
    b = _presolve(P, u, v, 1.0, False)
    assert rel_err(a, b) < 1e-12


def test_fft_kernel_bench_cold(cuda_lib):
    P = _params(420, 180)
    ctx = DRDContext(P)
    for kb in (abi.DRD_KB_PRESSURE_FFT64, abi.DRD_KB_DCT2_FFT32):
        us, by, _ = ctx.kernel_bench(kb, reps=5)
        assert us > 0 and by > 0
    ctx.close()
    ctx = DRDContext(_params(97, 53))  # prime sides: no FFT plan
    with pytest.raises(Exception):
        ctx.kernel_bench(abi.DRD_KB_DCT2_FFT32, reps=2)
    ctx.close()
