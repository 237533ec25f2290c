"""Standalone rates of the solver's bandwidth- and GEMM-bound kernels at several grid sizes.

    python -m drd_application_gb300.kernel_bench [--grids 420x180 2048x1024 4096x2048]

Each kernel runs `reps` times back to back in one captured graph between CUDA events on the
context stream (drd_kernel_bench), except the FFT transforms, which run after a 512 MiB L2 flush
each and are timed launch by launch; the rates use the algorithmic bytes and flops that
drd_kernel_bench reports for one launch (compulsory inputs and outputs only), against the
measured HBM copy rate of MEASURED_PEAKS.json (6.8 TB/s when that file is absent).
"""
import argparse
import json
import os

from . import abi
from .api import DRDContext

KERNELS = (
    (abi.DRD_KB_UV_MATVEC_FP32, "momentum stencil FP32"),
    (abi.DRD_KB_CH_MATVEC_FP32, "CH stencil FP32"),
    (abi.DRD_KB_UV_MATVEC_FP64, "momentum stencil FP64"),
    (abi.DRD_KB_DCT_X_FP32, "DCT-I x pass FP32"),
    (abi.DRD_KB_DCT_Z_FP32, "DCT-I z pass FP32"),
    (abi.DRD_KB_DCT_X_FP64, "DCT-I x pass FP64"),
    (abi.DRD_KB_PRESSURE_FFT64, "PreSolve_2 FFT FP64"),
    (abi.DRD_KB_DCT2_FFT32, "DCT-II/III FFT FP32"),
)
COLD = (abi.DRD_KB_PRESSURE_FFT64, abi.DRD_KB_DCT2_FFT32)  # timed with L2 flushed before each launch


def hbm_peak():
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"])
    except Exception:
        return 6800.0


def main(argv=None):
    ap = argparse.ArgumentParser(description="standalone kernel rates (drd_kernel_bench)")
    ap.add_argument("--grids", nargs="*", default=["420x180", "2048x1024", "4096x2048"])
    a = ap.parse_args(argv)
    peak = hbm_peak()
    for g in a.grids:
        nr, nz = (int(v) for v in g.lower().split("x"))
        ctx = DRDContext(abi.default_params(nr, nz, precision=abi.DRD_PREC_MIXED))
        print(f"{nr}x{nz}", flush=True)
        for kid, name in KERNELS:
            stencil = "stencil" in name
            reps = 10 if kid in COLD else (100 if stencil else (20 if nr <= 2048 else 3))
            try:
                us, by, fl = ctx.kernel_bench(kid, reps=reps)
            except Exception as e:  # e.g. an FFT transform on a grid whose sides it does not factor
                print(f"  {name:22s} n/a ({e})", flush=True)
                continue
            gbs = by / us / 1e3
            print(f"  {name:22s} {us:10.2f} us  {gbs:8.1f} GB/s ({100 * gbs / peak:5.1f} % of {peak:.0f})  "
                  f"{fl / us / 1e6:7.2f} TFLOP/s", flush=True)
        ctx.close()


if __name__ == "__main__":
    main()
