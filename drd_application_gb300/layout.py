"""Fortran ghosted array shapes as numpy arrays.

The reference declares (microfluidics_complex_domain/global.f90:42-47)
    u(-1:nr+1,-1:nz), v(-1:nr,0:nz), ph/rmu/p/rho/eta/...(-1:nr,-1:nz)
column-major with i fastest.  A C-ordered numpy array of shape (nz_extent, nr_extent)
indexed [k - k0, i - i0] has exactly that memory layout, so these arrays can be handed
to the C-ABI (and to a Fortran caller) without copies.
"""
import numpy as np


def cell_shape(nr, nz):
    return (nz + 2, nr + 2)


def u_shape(nr, nz):
    return (nz + 2, nr + 3)


def v_shape(nr, nz):
    return (nz + 1, nr + 2)


SHAPES = {"cell": cell_shape, "u": u_shape, "v": v_shape}


def empty(kind, nr, nz, fill=0.0):
    return np.full(SHAPES[kind](nr, nz), fill, dtype=np.float64)


class Fort2D:
    """Index a Fortran-shaped array with the reference's own bounds: a[i, k]."""

    def __init__(self, arr, i0, k0):
        self.a, self.i0, self.k0 = arr, i0, k0

    def __getitem__(self, ik):
        i, k = ik
        return self.a[self._k(k), self._i(i)]

    def __setitem__(self, ik, val):
        i, k = ik
        self.a[self._k(k), self._i(i)] = val

    def _i(self, i):
        if isinstance(i, slice):
            return slice(None if i.start is None else i.start - self.i0,
                         None if i.stop is None else i.stop - self.i0, i.step)
        return i - self.i0

    def _k(self, k):
        if isinstance(k, slice):
            return slice(None if k.start is None else k.start - self.k0,
                         None if k.stop is None else k.stop - self.k0, k.step)
        return k - self.k0


def cell(a):
    return Fort2D(a, -1, -1)


def ufield(a):
    return Fort2D(a, -1, -1)


def vfield(a):
    return Fort2D(a, -1, 0)


def interior_cell(a):
    """View of the (0:nr-1, 0:nz-1) interior as [k, i]."""
    return a[1:-1, 1:-1]


def neumann_ghosts_cell(a):
    """Ghost copies used throughout the reference for CELL fields (e.g. bcd.f90:25-39)."""
    a[1:-1, 0] = a[1:-1, 1]
    a[1:-1, -1] = a[1:-1, -2]
    a[0, :] = a[1, :]
    a[-1, :] = a[-2, :]
    return a


def ptr(a):
    """ctypes double* of a contiguous float64 array (None passes through)."""
    import ctypes as C

    if a is None:
        return None
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]):
        raise TypeError("expected a C-contiguous float64 numpy array")
    return a.ctypes.data_as(C.POINTER(C.c_double))
