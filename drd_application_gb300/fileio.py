"""The reference driver's files through the C library: the `input` deck
(microfluidics_complex_domain/mcl6.f90:68-99), the checkpoint records of `output` / `input`
(inout.f90:1-60) and `output_particles` (particles_move.f90:312-323).

Arrays use the shapes of layout.py (CELL, UFACE, VFACE); the grids x, y are NODE arrays of
shape (nz+1, nr+1).
"""
import ctypes as C

import numpy as np

from . import _lib, abi
from .layout import cell_shape, ptr, u_shape, v_shape


def node_shape(nr, nz):
    return (nz + 1, nr + 1)


def read_deck(path):
    """drd_read_deck -> abi.drd_deck (raises ValueError with the parser's message)."""
    L = _lib.load()
    d = abi.drd_deck()
    err = C.create_string_buffer(256)
    rc = L.drd_read_deck(str(path).encode(), C.byref(d), err, len(err))
    if rc != 0:
        raise ValueError(err.value.decode())
    return d


def params_from_deck(deck, nr, nz, variant=abi.DRD_VARIANT_MF):
    L = _lib.load()
    p = abi.drd_params()
    if L.drd_params_from_deck(C.byref(deck), nr, nz, variant, C.byref(p)) != 0:
        raise ValueError("deck does not describe a grid (slen, shig > 0 and nr, nz >= 3 needed)")
    return p


def output(path, nr, nz, dr, dz, u, v, p, f, f2, t, x=None, y=None):
    """output(M,N,x,y,u,v,p,f,f2,t,fname); x, y default to the cell-centre grids."""
    L = _lib.load()
    a = [np.ascontiguousarray(z, dtype=np.float64) if z is not None else None for z in (x, y, u, v, p, f, f2)]
    rc = L.drd_output(str(path).encode(), nr, nz, dr, dz, *[ptr(z) for z in a], t)
    if rc != 0:
        raise OSError(f"drd_output failed for {path}")


def input(path, nr, nz):  # noqa: A001 - the reference routine's name
    """input(M,N,x,y,u,v,p,f,t,fname) -> dict; t is what the reference reads (f2(0,0))."""
    L = _lib.load()
    out = {"x": np.zeros(node_shape(nr, nz)), "y": np.zeros(node_shape(nr, nz)), "u": np.zeros(u_shape(nr, nz)),
           "v": np.zeros(v_shape(nr, nz)), "p": np.zeros(cell_shape(nr, nz)), "f": np.zeros(cell_shape(nr, nz))}
    t = C.c_double()
    rc = L.drd_input(str(path).encode(), nr, nz, *[ptr(out[k]) for k in ("x", "y", "u", "v", "p", "f")], C.byref(t))
    if rc != 0:
        raise OSError(f"drd_input failed for {path}")
    out["t"] = t.value
    return out


def read_time(path, nr, nz):
    L = _lib.load()
    t = C.c_double()
    if L.drd_read_time(str(path).encode(), nr, nz, C.byref(t)) != 0:
        raise OSError(f"drd_read_time failed for {path}")
    return t.value


def output_particles(path, points):
    L = _lib.load()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    if L.drd_output_particles(str(path).encode(), pts.shape[1], ptr(pts)) != 0:
        raise OSError(f"drd_output_particles failed for {path}")


def write_fort23(path, t, diss, lib=None):
    """Append dissipation's fort.23 record (t, e1, e2, e3, e4, dissip in format 6e14.7)."""
    L = lib or _lib.load()
    if L.drd_write_fort23(str(path).encode(), float(t), C.byref(diss)) != 0:
        raise OSError(f"drd_write_fort23 failed for {path}")


def write_fort22(path, kcount, dt, diss, lib=None):
    """Append mcl6's fort.22 record (kcount, dt*dissip, mass)."""
    L = lib or _lib.load()
    if L.drd_write_fort22(str(path).encode(), int(kcount), float(dt), C.byref(diss)) != 0:
        raise OSError(f"drd_write_fort22 failed for {path}")
