"""Python mirror of the reference's per-step subroutine interface over the C-ABI.

Method names and argument order follow the Fortran subroutines
(microfluidics_complex_domain/PhSolve.f90:1, VeloSolve_combined.f90:5,
VeloSolve_2_combined.f90:4, PreSolve_2.f90:1, two_phase_flow_complex_domain/ph_mu_solve.f90:3);
the module-global inputs those subroutines read are set once with set_coefs /
set_tp_fields or passed explicitly.  Arrays are numpy float64 with the Fortran ghosted
shapes of drd_application_gb300.layout.  Every call runs the CUDA library; a missing
library raises.
"""
import ctypes as C

import numpy as np

from . import abi, _lib
from .layout import cell_shape, ptr, u_shape, v_shape


class DRDError(RuntimeError):
    pass


def _check_shape(a, shape, name):
    if a is None:
        return None
    if not isinstance(a, np.ndarray) or a.shape != shape or a.dtype != np.float64:
        raise ValueError(f"{name}: expected float64 array of shape {shape}")
    return np.ascontiguousarray(a)


def _out(a, shape, name):
    """A caller-supplied output array (written in place), or a new one."""
    if a is None:
        return np.zeros(shape)
    if not isinstance(a, np.ndarray) or a.shape != shape or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise ValueError(f"{name}: expected a C-contiguous float64 array of shape {shape}")
    return a


def pin(a, lib=None):
    """Page-lock and map a numpy array's memory (drd_host_register): the per-routine calls then
    read or write it in their one gather / scatter launch.  Unpin it (unpin) before it is freed."""
    L = lib or _lib.load()
    if not isinstance(a, np.ndarray) or not a.flags["C_CONTIGUOUS"]:
        raise ValueError("pin: expected a C-contiguous numpy array")
    rc = L.drd_host_register(C.c_void_p(a.ctypes.data), a.nbytes)
    if rc != 0:
        raise DRDError(f"drd_host_register failed with {rc}")
    return a


def unpin(a, lib=None):
    L = lib or _lib.load()
    rc = L.drd_host_unregister(C.c_void_p(a.ctypes.data))
    if rc != 0:
        raise DRDError(f"drd_host_unregister failed with {rc}")


class DRDContext:
    """One GPU context for an nr x nz grid (drd_create / drd_destroy)."""

    def __init__(self, params, lib=None):
        self.L = lib or _lib.load()
        self.P = params.copy()
        h = C.c_void_p()
        rc = self.L.drd_create(C.byref(self.P), C.byref(h))
        if rc != 0:
            raise DRDError(f"drd_create failed with {rc}")
        self.h = h
        self.nr, self.nz = params.nr, params.nz
        self.cs, self.us, self.vs = cell_shape(self.nr, self.nz), u_shape(self.nr, self.nz), v_shape(self.nr, self.nz)

    def close(self):
        if getattr(self, "h", None):
            self.L.drd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -------------------------------------------------------------------------------------
    def _rc(self, rc, what, allow_info=True):
        if rc == 0:
            return rc
        if allow_info and (rc > 0 or rc in (-10, -11)):
            return rc  # BiCGSTAB INFO: the reference prints it and continues
        msg = self.L.drd_last_error(self.h)
        raise DRDError(f"{what} failed with {rc}: {msg.decode() if msg else ''}")

    def set_params(self, params):
        self.P = params.copy()
        self._rc(self.L.drd_set_params(self.h, C.byref(self.P)), "drd_set_params", False)

    def set_coefs(self, rho=None, eta=None, bdr_ph=None, bdr_ph_grad=None, ph_M_0=None, ph_M_inner=None):
        a = [_check_shape(x, self.cs, n) for x, n in ((rho, "rho"), (eta, "eta"), (bdr_ph, "bdr_ph"),
                                                        (bdr_ph_grad, "bdr_ph_grad"), (ph_M_0, "ph_M_0"),
                                                        (ph_M_inner, "ph_M_inner"))]
        self._rc(self.L.drd_set_coefs(self.h, *[ptr(x) for x in a]), "drd_set_coefs", False)

    def set_tp_fields(self, bdr_ph_used=None, bdr_ph_penalty=None, angleB=None, angleT=None):
        a = [_check_shape(bdr_ph_used, self.cs, "bdr_ph_used"), _check_shape(bdr_ph_penalty, self.cs, "bdr_ph_penalty")]
        ang = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (angleB, angleT)]
        for x in ang:
            if x is not None and x.shape != (self.nr + 1,):
                raise ValueError("angle arrays have nr+1 entries")
        self._rc(self.L.drd_set_tp_fields(self.h, ptr(a[0]), ptr(a[1]), ptr(ang[0]), ptr(ang[1])),
                 "drd_set_tp_fields", False)

    def set_ch_blend(self, w):
        """Install the solid-blend weights of the CH preconditioner (packed nr*nz, in [0, 1]), or
        remove them (None): drd_set_ch_blend."""
        if w is not None:
            w = np.ascontiguousarray(w, dtype=np.float64).reshape(-1)
            if w.shape != (self.nr * self.nz,):
                raise ValueError(f"blend weights have nr*nz = {self.nr * self.nz} entries")
        self._rc(self.L.drd_set_ch_blend(self.h, ptr(w)), "drd_set_ch_blend", False)

    def ch_blend_probe(self, nprobe=32, seed=0, install=True):
        """Fit the blend weights of the current mobilities with `nprobe` Rademacher probes on the
        GPU (drd_ch_blend_probe); returns them (packed nr*nz) and installs them if asked."""
        w = np.zeros(self.nr * self.nz)
        self._rc(self.L.drd_ch_blend_probe(self.h, int(nprobe), int(seed), int(bool(install)), ptr(w)),
                 "drd_ch_blend_probe", False)
        return w

    def set_case(self, case):
        """Load the coefficient fields of a workloads.Case (with two_fluid, also its indicator
        fpd_ph, which every step combines with the phase field)."""
        k = case.coefs
        self.set_coefs(k["rho"], k["eta"], k["bdr_ph"], k["bdr_ph_grad"], k["M0"], k["Mi"])
        if self.P.variant == abi.DRD_VARIANT_TP:
            self.set_tp_fields(k["bdr_used"], k["bdr_pen"])
        if self.P.two_fluid:
            self.two_phase_coef(k["fpd"], case.state[abi.F_PH])

    def two_phase_coef(self, fpd_ph=None, ph=None, out=None):
        """The two-fluid rho, eta of interpolate_coef (two_phase_flow_complex_domain/
        interpolate_coef.f90:91-112, commented out there) -> (rho, eta); they also replace the
        context's coefficients.  fpd_ph None keeps the context's indicator, ph None uses the
        resident phase field."""
        f = _check_shape(fpd_ph, self.cs, "fpd_ph")
        ph = _check_shape(ph, self.cs, "ph")
        o = out or (None, None)
        rho, eta = _out(o[0], self.cs, "rho"), _out(o[1], self.cs, "eta")
        self._rc(self.L.drd_two_phase_coef(self.h, ptr(f), ptr(ph), ptr(rho), ptr(eta)), "two_phase_coef", False)
        return rho, eta

    # ---- the reference subroutines --------------------------------------------------------
    def interpolate_coef(self, dist):
        dist = np.ascontiguousarray(dist, dtype=np.float64)
        if dist.shape != (self.nz, self.nr):
            raise ValueError("dist has shape (nz, nr)")
        fpd, rho, eta = (np.zeros(self.cs) for _ in range(3))
        self._rc(self.L.drd_interpolate_coef(self.h, ptr(dist), ptr(fpd), ptr(rho), ptr(eta)), "interpolate_coef", False)
        return fpd, rho, eta

    # ---- initialisation (finit.f90) -------------------------------------------------------
    def PhSolve_ori(self, u, v, ph, angleB=None, angleT=None, alpha_s=0.0):
        """PhSolve_ori(rmu_after, ph_after, t) -> (rmu_after, ph_after, status)."""
        u, v = _check_shape(u, self.us, "u"), _check_shape(v, self.vs, "v")
        ph = _check_shape(ph, self.cs, "ph")
        ang = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (angleB, angleT)]
        for a in ang:
            if a is not None and a.shape != (self.nr + 1,):
                raise ValueError("angle arrays have nr+1 entries")
        rmu_after, ph_after = np.zeros(self.cs), np.zeros(self.cs)
        st = abi.drd_status()
        rc = self.L.drd_phsolve_ori(self.h, ptr(u), ptr(v), ptr(ph), ptr(ang[0]), ptr(ang[1]), alpha_s,
                                    ptr(rmu_after), ptr(ph_after), C.byref(st))
        self._rc(rc, "PhSolve_ori")
        return rmu_after, ph_after, st

    def finit_wall(self, bdr_ph, nsteps=51):
        """finit's wall smoothing -> (bdr_ph, ph, rmu, info)."""
        bdr_ph = _check_shape(bdr_ph, self.cs, "bdr_ph")
        out = [np.zeros(self.cs) for _ in range(3)]
        rc = self.L.drd_finit_wall(self.h, ptr(bdr_ph), nsteps, *[ptr(a) for a in out])
        self._rc(rc, "finit_wall")
        return out[0], out[1], out[2], rc

    def reinint_by_PhSolve(self, bdr_ph):
        """reinint_by_PhSolve (two_phase_flow_complex_domain/reinint_by_PhSolve.f90) ->
        (bdr_ph, bdr_ph_penalty, info); both also become the context's."""
        bdr_ph = _check_shape(bdr_ph, self.cs, "bdr_ph")
        b, pen = np.zeros(self.cs), np.zeros(self.cs)
        rc = self.L.drd_reinint_by_phsolve(self.h, ptr(bdr_ph), ptr(b), ptr(pen))
        self._rc(rc, "reinint_by_phsolve")
        return b, pen, rc

    def dissipation(self, vs, u=None, v=None, ph=None, rmu=None, angleB=None, angleT=None):
        """dissipation's diagnostics -> abi.drd_diagnostics (e1, e2, e3, e4, dissip, mass).
        Fields left None are the resident ones."""
        a = [_check_shape(u, self.us, "u"), _check_shape(v, self.vs, "v"), _check_shape(ph, self.cs, "ph"),
             _check_shape(rmu, self.cs, "rmu")]
        ang = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (angleB, angleT)]
        for x in ang:
            if x is not None and x.shape[0] < self.nr:
                raise ValueError("angle arrays need nr entries")
        out = abi.drd_diagnostics()
        self._rc(self.L.drd_dissipation(self.h, *[ptr(x) for x in a], ptr(ang[0]), ptr(ang[1]), float(vs),
                                        C.byref(out)), "dissipation", False)
        return out

    # ---- fiber particles (particles_move.f90) --------------------------------------------
    def particles_set(self, pp, points=None, bdr_dist=None):
        """Make a bead chain resident (drd_particles_set); points is a (2, Np) array (x row, y
        row: the column-major Fortran points(0:Np-1,0:1)), bdr_dist a CELL array."""
        self.pp = pp.copy()
        pts = None if points is None else np.ascontiguousarray(points, dtype=np.float64)
        if pts is not None and pts.shape != (2, pp.np):
            raise ValueError("points has shape (2, np)")
        bd = _check_shape(bdr_dist, self.cs, "bdr_dist")
        self._rc(self.L.drd_particles_set(self.h, C.byref(self.pp), ptr(pts), ptr(bd)), "drd_particles_set", False)

    def particles_get(self):
        """(points, tot_F), both (2, Np)."""
        n = self.pp.np if getattr(self, "pp", None) is not None else 0
        pts, tot = np.zeros((2, n)), np.zeros((2, n))
        self._rc(self.L.drd_particles_get(self.h, ptr(pts), ptr(tot)), "drd_particles_get", False)
        return pts, tot

    def force_caculation_vel(self, dt, t):
        """force_caculation_vel -> (particle_force1, particle_force2) CELL arrays."""
        pf1, pf2 = np.zeros(self.cs), np.zeros(self.cs)
        self._rc(self.L.drd_force_caculation_vel(self.h, dt, t, ptr(pf1), ptr(pf2)), "force_caculation_vel", False)
        return pf1, pf2

    def update_position_vel(self, u, v, dt):
        u, v = _check_shape(u, self.us, "u"), _check_shape(v, self.vs, "v")
        self._rc(self.L.drd_update_position_vel(self.h, ptr(u), ptr(v), dt), "update_position_vel", False)

    def interpolate_coef_particles(self):
        """interpolate_coef with fpd_dist of the resident beads -> (fpd_ph, rho, eta)."""
        fpd, rho, eta = (np.zeros(self.cs) for _ in range(3))
        self._rc(self.L.drd_interpolate_coef_particles(self.h, ptr(fpd), ptr(rho), ptr(eta)),
                 "interpolate_coef_particles", False)
        return fpd, rho, eta

    # ---- checkpoint of the resident state (inout.f90 output) -------------------------------
    def checkpoint_async(self, path, t):
        self._rc(self.L.drd_checkpoint_async(self.h, str(path).encode(), t), "drd_checkpoint_async", False)

    def checkpoint_wait(self):
        self._rc(self.L.drd_checkpoint_wait(self.h), "drd_checkpoint_wait", False)

    def PhSolve(self, u, v, ph, rmu, t, out=None):
        """PhSolve(rmu_after, ph_after, t) -> (rmu_after, ph_after, status).  out: optional
        (rmu_after, ph_after) arrays to write."""
        u, v = _check_shape(u, self.us, "u"), _check_shape(v, self.vs, "v")
        ph, rmu = _check_shape(ph, self.cs, "ph"), _check_shape(rmu, self.cs, "rmu")
        o = out or (None, None)
        rmu_after, ph_after = _out(o[0], self.cs, "rmu_after"), _out(o[1], self.cs, "ph_after")
        st = abi.drd_status()
        self._rc(self.L.drd_phsolve(self.h, ptr(u), ptr(v), ptr(ph), ptr(rmu), t, ptr(rmu_after), ptr(ph_after),
                                    C.byref(st)), "PhSolve")
        return rmu_after, ph_after, st

    def ph_mu_solve(self, u, v, ph, rmu, t):
        """ph_mu_solve(ph_after, rmu_after, t) -> (ph_after, rmu_after, ph_M_0, (coef_bot, coef_top), status)."""
        u, v = _check_shape(u, self.us, "u"), _check_shape(v, self.vs, "v")
        ph, rmu = _check_shape(ph, self.cs, "ph"), _check_shape(rmu, self.cs, "rmu")
        ph_after, rmu_after, M0 = np.zeros(self.cs), np.zeros(self.cs), np.zeros(self.cs)
        cbt = np.zeros(2)
        st = abi.drd_status()
        self._rc(self.L.drd_ph_mu_solve(self.h, ptr(u), ptr(v), ptr(ph), ptr(rmu), t, ptr(ph_after), ptr(rmu_after),
                                        ptr(M0), ptr(cbt), C.byref(st)), "ph_mu_solve")
        return ph_after, rmu_after, M0, tuple(cbt), st

    def VeloSolve_combined(self, psi, u, v, p, rmu_after, ph_after, t, particle_force1=None, particle_force2=None):
        """VeloSolve_combined(psi, u_after, v_after, rmu_after, ph_after, t, pf1, pf2)
        -> (u_after, v_after, uL, uR, status)."""
        args = [_check_shape(x, s, n) for x, s, n in ((u, self.us, "u"), (v, self.vs, "v"), (p, self.cs, "p"),
                                                       (rmu_after, self.cs, "rmu_after"), (ph_after, self.cs, "ph_after"))]
        pf = [_check_shape(x, self.cs, "particle_force") for x in (particle_force1, particle_force2)]
        u_after, v_after = np.zeros(self.us), np.zeros(self.vs)
        uL, uR = np.zeros(self.nz + 1), np.zeros(self.nz + 1)
        st = abi.drd_status()
        self._rc(self.L.drd_velosolve_combined(self.h, ptr(_check_shape(psi, self.cs, "psi")), *[ptr(x) for x in args],
                                               t, ptr(pf[0]), ptr(pf[1]), ptr(u_after), ptr(v_after), ptr(uL), ptr(uR),
                                               C.byref(st)), "VeloSolve_combined")
        return u_after, v_after, uL, uR, st

    def VeloSolve_2_combined(self, psi1, psi2, u_pre, u, v_pre, v, p, ph_pre, ph_after, rmu_pre, rmu_after, t,
                             particle_force1=None, particle_force2=None, out=None):
        """VeloSolve_2_combined(psi1, psi2, u_pre, u_after, v_pre, v_after, ph_pre, ph_after, rmu_pre,
        rmu_after, t, pf1, pf2) -> (u_after, v_after, uL, uR, status).  out: optional (u_after,
        v_after, uL, uR) arrays to write."""
        cs, us, vs = self.cs, self.us, self.vs
        a = [_check_shape(x, s, n) for x, s, n in (
            (psi1, cs, "psi1"), (psi2, cs, "psi2"), (u_pre, us, "u_pre"), (u, us, "u"), (v_pre, vs, "v_pre"),
            (v, vs, "v"), (p, cs, "p"), (ph_pre, cs, "ph_pre"), (ph_after, cs, "ph_after"), (rmu_pre, cs, "rmu_pre"),
            (rmu_after, cs, "rmu_after"))]
        pf = [_check_shape(x, cs, "particle_force") for x in (particle_force1, particle_force2)]
        o = out or (None, None, None, None)
        u_after, v_after = _out(o[0], us, "u_after"), _out(o[1], vs, "v_after")
        uL, uR = _out(o[2], (self.nz + 1,), "uL"), _out(o[3], (self.nz + 1,), "uR")
        st = abi.drd_status()
        self._rc(self.L.drd_velosolve_2_combined(self.h, *[ptr(x) for x in a], t, ptr(pf[0]), ptr(pf[1]),
                                                 ptr(u_after), ptr(v_after), ptr(uL), ptr(uR), C.byref(st)),
                 "VeloSolve_2_combined")
        return u_after, v_after, uL, uR, st

    def PreSolve_2(self, u, v, coef, out=None):
        """PreSolve_2(plan, plan_back, psi, coef) -> psi (the FFTW plans live in the context).
        out: optional psi array to write."""
        u, v = _check_shape(u, self.us, "u"), _check_shape(v, self.vs, "v")
        psi = _out(out, self.cs, "psi")
        st = abi.drd_status()
        self._rc(self.L.drd_presolve_2(self.h, ptr(u), ptr(v), coef, ptr(psi), C.byref(st)), "PreSolve_2", False)
        return psi

    def mass(self, ph):
        ph = _check_shape(ph, self.cs, "ph")
        m = C.c_double()
        self._rc(self.L.drd_mass(self.h, ptr(ph), C.byref(m)), "mass", False)
        return m.value

    # ---- resident state --------------------------------------------------------------------
    def upload_state(self, state):
        for fid, arr in state.items():
            shape = {"u": self.us, "v": self.vs, "cell": self.cs}[abi.FIELD_KIND[fid]]
            self._rc(self.L.drd_state_upload(self.h, fid, ptr(_check_shape(arr, shape, f"field {fid}"))),
                     "state_upload", False)

    def download_state(self, fields=None):
        out = {}
        for fid in (fields if fields is not None else range(abi.F_COUNT)):
            shape = {"u": self.us, "v": self.vs, "cell": self.cs}[abi.FIELD_KIND[fid]]
            a = np.zeros(shape)
            self._rc(self.L.drd_state_download(self.h, fid, ptr(a)), "state_download", False)
            out[fid] = a
        return out

    def step(self, first, t, stats=True):
        st = abi.drd_step_stats() if stats else None
        self._rc(self.L.drd_step(self.h, int(first), t, C.byref(st) if st is not None else None), "drd_step", False)
        return st

    def steps_async(self, first, t, n):
        self._rc(self.L.drd_steps_async(self.h, int(first), t, int(n)), "drd_steps_async", False)

    def synchronize(self):
        self._rc(self.L.drd_synchronize(self.h), "drd_synchronize", False)

    def barrier_selftest(self, absent):
        """Status of the grid barrier with block `absent` (1) or none (-1) missing: 0 or DRD_ERR_TIMEOUT."""
        st = C.c_int(0)
        self._rc(self.L.drd_barrier_selftest(self.h, int(absent), C.byref(st)), "drd_barrier_selftest", False)
        return st.value

    def solve(self, system, b, x0=None, bdf=2):
        """A x = b for DRD_SYS_CH or DRD_SYS_UV with the context's coefficients -> (x, status)."""
        op = abi.DRD_OP_CH_MATVEC if system == abi.DRD_SYS_CH else abi.DRD_OP_UV_MATVEC
        n = self.L.drd_op_length(self.h, op)
        b = np.ascontiguousarray(b, dtype=np.float64)
        if b.shape != (n,):
            raise ValueError(f"system {system} has {n} unknowns")
        x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
        st = abi.drd_status()
        self._rc(self.L.drd_solve(self.h, system, bdf, ptr(b), ptr(x), C.byref(st)), "drd_solve")
        return x, st

    def op_apply(self, op, x, bdf=2, precision=abi.DRD_PREC_FP64):
        """y = op(x) for one of the DRD_OP_* operators (verification access)."""
        n = self.L.drd_op_length(self.h, op)
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != (n,):
            raise ValueError(f"operator {op} acts on vectors of length {n}")
        y = np.zeros(n)
        self._rc(self.L.drd_op_apply(self.h, op, bdf, precision, ptr(x), ptr(y)), "drd_op_apply", False)
        return y

    def kernel_bench(self, which, reps=200):
        """(us per launch, algorithmic bytes per launch, flops per launch) of kernel `which`."""
        us, by, fl = C.c_double(), C.c_double(), C.c_double()
        self._rc(self.L.drd_kernel_bench(self.h, which, reps, C.byref(us), C.byref(by), C.byref(fl)),
                 "drd_kernel_bench", False)
        return us.value, by.value, fl.value

    def flush_l2(self, nbytes=512 << 20):
        self._rc(self.L.drd_flush_l2(self.h, int(nbytes)), "drd_flush_l2", False)

    def persistent_solver(self):
        """(in use, why not) of the persistent cooperative FP32 inner solver."""
        why = C.create_string_buffer(512)
        on = self.L.drd_persistent_solver(self.h, why, len(why))
        return bool(on == 1), why.value.decode()

    def kernel_launches(self):
        return int(self.L.drd_kernel_launches(self.h))

    def stream(self):
        return self.L.drd_stream(self.h)
