"""The C-ABI library loads without a GPU, exports every symbol include/drd_gb300.h declares,
and the ctypes mirror of its structs has the header's layout (checked with gcc)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from drd_application_gb300 import _lib, abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "drd_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(drd_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_reference_entry_points():
    names = header_functions()
    for must in ("drd_create", "drd_phsolve", "drd_ph_mu_solve", "drd_velosolve_combined",
                 "drd_velosolve_2_combined", "drd_presolve_2", "drd_interpolate_coef", "drd_mass", "drd_step"):
        assert must in names


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = C.CDLL(path)  # loads without a GPU: CUDA is only touched by the entry points
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(header_functions()) <= set(_lib.SIGNATURES), "ctypes signatures must cover the header"
    assert _lib.load().drd_abi_version() == abi.DRD_ABI_VERSION


def _c_layout(struct, fields):
    prog = "#include <stdio.h>\n#include <stddef.h>\n#include \"drd_gb300.h\"\nint main(void){\n"
    prog += f'printf("%zu\\n", sizeof({struct}));\n'
    for f in fields:
        prog += f'printf("%zu\\n", offsetof({struct}, {f}));\n'
    prog += "return 0;}\n"
    d = os.path.join(ROOT, "oracle", "build")
    os.makedirs(d, exist_ok=True)
    src = os.path.join(d, f"layout_{struct}.c")
    exe = src[:-2]
    open(src, "w").write(prog)
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    return [int(x) for x in out]


@pytest.mark.parametrize("cls,name", [(abi.drd_params, "drd_params"), (abi.drd_status, "drd_status"),
                                      (abi.drd_step_stats, "drd_step_stats"),
                                      (abi.drd_particle_params, "drd_particle_params"),
                                      (abi.drd_deck, "drd_deck"), (abi.drd_diagnostics, "drd_diagnostics")])
def test_struct_layout_matches_header(cls, name):
    fields = [f for f, _ in cls._fields_]
    got = _c_layout(name, fields)
    assert got[0] == C.sizeof(cls)
    for f, off in zip(fields, got[1:]):
        assert getattr(cls, f).offset == off, f


def test_bad_arguments_are_rejected_without_a_gpu():
    lib = _lib.load()
    h = C.c_void_p()
    p = abi.default_params(2, 2)  # below the minimum grid: rejected before any CUDA call
    assert lib.drd_create(C.byref(p), C.byref(h)) == abi.DRD_ERR_BADARG
    p = abi.default_params(16, 8, xlsB=0.1)  # slip walls have no solve in the reference
    assert lib.drd_create(C.byref(p), C.byref(h)) == abi.DRD_ERR_UNSUPPORTED
    assert lib.drd_destroy(None) == abi.DRD_ERR_BADARG
    # the host-only particle helpers need no GPU and match the Python defaults bit for bit
    pp = abi.drd_particle_params()
    assert lib.drd_particle_params_default(C.byref(pp), 3.5, 1.5) == 0
    assert bytes(pp) == bytes(abi.default_particle_params(3.5, 1.5))
    pts = (C.c_double * 18)()
    assert lib.drd_particle_initialize(C.byref(pp), 1.75, 0.42, pts) == 0
    assert list(pts) == [x for row in abi.particle_chain(pp, 1.75, 0.42) for x in row]
    assert lib.drd_particles_set(None, C.byref(pp), pts, pts) == abi.DRD_ERR_BADARG


def test_unet_bad_arguments_are_rejected_without_a_gpu():
    """drd_unet_create validates its arguments before any CUDA call; null handles are rejected."""
    lib = _lib.load()
    h = C.c_void_p()
    for H, W, cin, cout, mb in ((4, 64, 3, 1, 1), (64, 7, 3, 1, 1), (64, 64, 0, 1, 1), (64, 64, 17, 1, 1),
                                (64, 64, 3, 0, 1), (64, 64, 3, 5, 1), (64, 64, 3, 1, 0)):
        assert lib.drd_unet_create(H, W, cin, cout, mb, 0, C.byref(h)) == abi.DRD_ERR_BADARG
    assert lib.drd_unet_create(64, 64, 3, 1, 1, 0, None) == abi.DRD_ERR_BADARG
    assert lib.drd_unet_param_count(None) == -1
    assert lib.drd_unet_forward(None, 1, None, None) == abi.DRD_ERR_BADARG
    assert lib.drd_unet_train_step(None, 1, None, None, C.c_float(1e-3), None) == abi.DRD_ERR_BADARG
    assert lib.drd_unet_destroy(None) == 0
