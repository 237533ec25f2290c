"""The tensor-core transform GEMM (3xTF32 tcgen05, GEMM configuration kGemmTcCfg = 14) in the
FP32 passes of the kernel-per-phase loop, forced with DRD_GEMM_CFG: the CH preconditioner
(folded DCT-I passes along x and z, the division by Ph_Lcc in an epilogue) and ESOLP_x's row
passes, against the oracle's FP64 operators at FP32 accuracy.  Both stagings of the data
operand run: TMA boxes (k_gemm_tc_tma: straight from the data where rows are 16-byte aligned,
else from the operand pre-folded into aligned scratch, as at 97x53 and for ESOLP_x's u rows of
nr + 1) and the register staging (k_gemm_tc, the fallback; DRD_GEMM_TC_NOTMA forces it)."""
import contextlib
import os

import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext
from oracle.oracle import Oracle
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu
F = abi


def _ctx(P):
    os.environ["DRD_GEMM_CFG"] = "14"
    try:
        return DRDContext(P)
    finally:
        del os.environ["DRD_GEMM_CFG"]


@contextlib.contextmanager
def _staging(tma):
    if not tma:
        os.environ["DRD_GEMM_TC_NOTMA"] = "1"
    try:
        yield
    finally:
        os.environ.pop("DRD_GEMM_TC_NOTMA", None)


@pytest.mark.parametrize("tma", [True, False])
@pytest.mark.parametrize("nr,nz", [(97, 53), (420, 180), (512, 256), (128, 97)])
def test_tc_ch_psolve_matches_oracle(cuda_lib, oracle_build, nr, nz, tma):
    """(128, 97): the z pass's fold has its middle point k = L / 2 = 48 inside a TMA chunk."""
    P = abi.default_params(nr, nz)
    P.dr, P.dz, P.dt = 3.5 / nr, 1.5 / nz, 1e-3
    P.precision = F.DRD_PREC_MIXED
    with _staging(tma):
        _check_psolve(P, nr, nz)


def _check_psolve(P, nr, nz):
    ctx, orc = _ctx(P), Oracle(P)
    try:
        x = np.random.default_rng(nr).standard_normal(nr * nz)
        y = ctx.op_apply(F.DRD_OP_CH_PSOLVE, x, precision=F.DRD_PREC_MIXED)
        assert np.isfinite(y).all()
        assert rel_err(y, orc.ch_psolve(x)) < 2e-5, rel_err(y, orc.ch_psolve(x))
    finally:
        ctx.close()


@pytest.mark.parametrize("tma", [True, False])
@pytest.mark.parametrize("nr,nz", [(97, 53), (420, 180)])
def test_tc_esolp_rows_match_oracle(cuda_lib, oracle_build, nr, nz, tma):
    P = abi.default_params(nr, nz)
    P.dr, P.dz, P.dt = 3.5 / nr, 1.5 / nz, 1e-3
    P.precision = F.DRD_PREC_MIXED
    P.uv_precond = F.DRD_UV_ESOLP
    with _staging(tma):
        _check_esolp(P, nz)


def _check_esolp(P, nz):
    ctx, orc = _ctx(P), Oracle(P)
    try:
        x = np.random.default_rng(nz).standard_normal(ctx.L.drd_op_length(ctx.h, F.DRD_OP_UV_PSOLVE))
        y = ctx.op_apply(F.DRD_OP_UV_PSOLVE, x, bdf=2, precision=F.DRD_PREC_MIXED)
        assert rel_err(y, orc.uv_psolve_esolp(2, x)) < 2e-5
    finally:
        ctx.close()
