"""Batches of independent solves in one persistent launch (drd_batch_* of the C-ABI).

    from drd_application_gb300.batch import Batch
    b = Batch([("uv", params, coefs, rhs), ("pressure", params, bdr_ph, rhs), ...])
    seconds = b.run()            # one graph launch solves every system
    x, status = b.result(3)

Each system carries its own grid size and coefficients; all are uploaded once at creation.
"""
import ctypes as C

import numpy as np

from . import _lib, abi
from .layout import cell_shape, ptr


class BatchError(RuntimeError):
    pass


class Batch:
    def __init__(self, systems, autotune=True, lib=None):
        """systems: tuples ("uv", params, coefs, b[, x0, bdf]) with coefs holding the CELL arrays
        "rho", "eta", "bdr_ph", or ("pressure", params, bdr_ph, b[, x0])."""
        self.L = lib or _lib.load()
        n = len(systems)
        arr = (abi.drd_batch_problem * n)()
        self._keep = []
        self.meta = []
        for i, s in enumerate(systems):
            kind, P = s[0], s[1]
            q = arr[i]
            q.params = P.copy()
            cs = cell_shape(P.nr, P.nz)
            if kind == "uv":
                coefs, b = s[2], s[3]
                x0 = s[4] if len(s) > 4 else None
                q.system, q.bdf = abi.DRD_SYS_UV, (s[5] if len(s) > 5 else 2)
                arrays = [np.ascontiguousarray(coefs[k], dtype=np.float64) for k in ("rho", "eta", "bdr_ph")]
                for a in arrays:
                    if a.shape != cs:
                        raise ValueError("coefficients must be CELL arrays")
                q.rho, q.eta, q.bdr_ph = (ptr(a) for a in arrays)
            elif kind == "pressure":
                bdr, b = s[2], s[3]
                x0 = s[4] if len(s) > 4 else None
                q.system, q.bdf = abi.DRD_SYS_PRESSURE, 2
                arrays = [np.ascontiguousarray(bdr, dtype=np.float64)]
                if arrays[0].shape != cs:
                    raise ValueError("bdr_ph must be a CELL array")
                q.bdr_ph = ptr(arrays[0])
            else:
                raise ValueError(f"unknown system kind {kind!r}")
            length = self.L.drd_batch_length(q.system, P.nr, P.nz)
            b = np.ascontiguousarray(b, dtype=np.float64)
            if b.shape != (length,):
                raise ValueError(f"system {i}: b has {b.size} entries, expected {length}")
            q.b = ptr(b)
            arrays.append(b)
            if x0 is not None:
                x0 = np.ascontiguousarray(x0, dtype=np.float64)
                q.x0 = ptr(x0)
                arrays.append(x0)
            self._keep.append(arrays)
            self.meta.append((kind, P.nr, P.nz, length))
        h = C.c_void_p()
        rc = self.L.drd_batch_create(n, arr, int(bool(autotune)), C.byref(h))
        self._keep = None  # uploaded: the host arrays are no longer referenced
        if rc != 0:
            raise BatchError(f"drd_batch_create failed with {rc}")
        self.h = h
        self.n = n

    def run(self):
        """Solve every system (one persistent launch); returns its device seconds."""
        sec = C.c_double()
        rc = self.L.drd_batch_run(self.h, C.byref(sec))
        if rc != 0:
            raise BatchError(f"drd_batch_run failed with {rc}: {self.L.drd_batch_last_error(self.h)}")
        return sec.value

    def result(self, i):
        x = np.zeros(self.meta[i][3])
        st = abi.drd_status()
        self.L.drd_batch_result(self.h, i, ptr(x), C.byref(st))
        return x, st

    def status(self, i):
        st = abi.drd_status()
        self.L.drd_batch_result(self.h, i, None, C.byref(st))
        return st

    def info(self):
        t, b, by = C.c_int(), C.c_int(), C.c_double()
        self.L.drd_batch_info(self.h, C.byref(t), C.byref(b), C.byref(by))
        return {"threads": t.value, "blocks_per_sm": b.value, "bytes_last_run": by.value}

    def close(self):
        if getattr(self, "h", None):
            self.L.drd_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
