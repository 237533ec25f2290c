"""ctypes binding of the FP64 CPU oracle (oracle/drd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline legs as the checker.  The product library never loads it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from drd_application_gb300 import abi
from drd_application_gb300.layout import ptr

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "liboracle.so")
LIB_OMP = os.path.join(BUILD, "liboracle_omp.so")
SRC = os.path.join(HERE, "drd_oracle.c")
HDR = os.path.join(HERE, "drd_oracle.h")


def build(force=False):
    """Compile the oracle with gcc: a serial library (the checker and the single-thread CPU
    baseline, like the reference's serial build) and an OpenMP one for all-core timing."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [SRC, HDR, os.path.join(HERE, "..", "include", "drd_gb300.h")]
    newest = max(os.path.getmtime(d) for d in deps)
    for out, extra in ((LIB, []), (LIB_OMP, ["-fopenmp", "-DORC_OPENMP"])):
        if force or not os.path.exists(out) or os.path.getmtime(out) < newest:
            cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", *extra, "-o", out + ".tmp", SRC, "-lm"]
            subprocess.run(cmd, check=True)
            os.replace(out + ".tmp", out)
    return LIB


_libs = {}


def lib(openmp=False):
    path = LIB_OMP if openmp else LIB
    if path not in _libs:
        build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        P = C.POINTER(abi.drd_params)
        S = C.POINTER(abi.drd_status)
        L.orc_setup_tables.argtypes = [P, dp, dp]
        for f in ("orc_vcost", "orc_redft10", "orc_redft01"):
            getattr(L, f).argtypes = [C.c_int, C.c_int, dp, C.c_long, C.c_long]
        L.orc_op_double_gradient_neum.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, dp, dp, dp]
        L.orc_ch_matvec.argtypes = [P, dp, dp, C.c_double, dp, C.c_double, dp]
        L.orc_ch_psolve.argtypes = [P, dp, dp, dp]
        L.orc_ch_psolve_blend.argtypes = [P, dp, dp, dp, dp]
        L.orc_probe_sign.argtypes = [C.c_uint64, C.c_long, C.c_long, C.c_long]
        L.orc_probe_sign.restype = C.c_double
        L.orc_ch_blend_probe.argtypes = [P, dp, dp, dp, C.c_int, C.c_uint64, dp]
        L.orc_ch_solve_blend.argtypes = [P, dp, dp, dp, dp, dp, dp, S]
        L.orc_uv_matvec.argtypes = [P, C.c_int, dp, dp, dp, C.c_double, dp, C.c_double, dp]
        L.orc_uv_psolve.argtypes = [P, C.c_int, dp, dp, dp, dp]
        L.orc_uv_psolve_esolp.argtypes = [P, C.c_int, dp, dp]
        L.orc_uv_esolp_scale.argtypes = [P, C.c_int, dp, dp, dp]
        L.orc_uv_psolve_esolp_scaled.argtypes = [P, C.c_int, dp, dp, dp]
        L.orc_solve_system.argtypes = [P, C.c_int, C.c_int, dp, dp, dp, dp, dp, dp, dp, dp, S]
        L.orc_esolp_coefs.argtypes = [P, C.c_int, dp, dp, dp, dp, dp, dp]
        L.orc_phmu_matvec.argtypes = [P, dp, dp, dp, C.c_double, C.c_double, C.c_double, dp, C.c_double, dp]
        L.orc_phmu_psolve.argtypes = [P, dp, dp]
        L.orc_ch_system.argtypes = [P, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_phmu_system.argtypes = [P, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_phsolve.argtypes = [P, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, S]
        L.orc_phsolve.restype = C.c_int
        L.orc_ph_mu_solve.argtypes = [P, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, S]
        L.orc_ph_mu_solve.restype = C.c_int
        L.orc_velosolve.argtypes = [P, C.c_int] + [dp] * 14 + [C.c_double, dp, dp, dp, dp, dp, dp, S]
        L.orc_velosolve.restype = C.c_int
        L.orc_presolve.argtypes = [P, dp, dp, dp, C.c_double, dp]
        L.orc_interpolate_coef.argtypes = [P, dp, dp, dp, dp, dp]
        L.orc_two_phase_coef.argtypes = [P, dp, dp, dp, dp]
        L.orc_pressure_matvec.argtypes = [P, dp, dp, dp]
        L.orc_pressure_psolve.argtypes = [P, dp, dp, dp]
        L.orc_pressure_solve.argtypes = [P, dp, dp, dp, dp, S]
        L.orc_pressure_solve.restype = C.c_int
        L.orc_reinint_by_phsolve.argtypes = [P, dp, dp, dp, dp]
        L.orc_reinint_by_phsolve.restype = C.c_int
        L.orc_dissipation.argtypes = [P, dp, dp, dp, dp, dp, dp, C.c_double, dp]
        L.orc_mass.argtypes = [P, dp]
        L.orc_mass.restype = C.c_double
        L.orc_ori_coef.argtypes = [P, C.c_double]
        L.orc_ori_coef.restype = C.c_double
        L.orc_ori_matvec.argtypes = [P, C.c_double, C.c_double, C.c_double, dp, C.c_double, dp]
        L.orc_ori_system.argtypes = [P, dp, dp, dp, dp, dp, C.c_double, dp, dp, dp, dp, dp]
        L.orc_phsolve_ori.argtypes = [P, dp, dp, dp, dp, dp, dp, C.c_double, dp, dp, S]
        L.orc_phsolve_ori.restype = C.c_int
        L.orc_finit_wall.argtypes = [P, dp, dp, C.c_int, dp, dp, dp]
        L.orc_finit_wall.restype = C.c_int
        PP = C.POINTER(abi.drd_particle_params)
        L.orc_particle_forces.argtypes = [P, PP, dp, dp, dp]
        L.orc_force_caculation_vel.argtypes = [P, PP, dp, dp, dp, dp, dp]
        L.orc_update_position_vel.argtypes = [P, PP, dp, dp, dp, C.c_double]
        L.orc_fpd_dist_field.argtypes = [P, PP, dp, dp]
        L.drd_particle_params_default.argtypes = [PP, C.c_double, C.c_double]
        L.drd_particle_initialize.argtypes = [PP, C.c_double, C.c_double, dp]
        _libs[path] = L
    return _libs[path]


class OrcParticles(C.Structure):
    _fields_ = [("pp", abi.drd_particle_params)] + [
        (n, C.POINTER(C.c_double)) for n in ("points", "tot_F", "bdr_dist", "fpd_ph", "rho", "eta")
    ]


class OrcState(C.Structure):
    _fields_ = [("f", C.POINTER(C.c_double) * abi.F_COUNT)] + [
        (n, C.POINTER(C.c_double)) for n in ("rho", "eta", "bdr_ph", "bdr_ph_grad", "M0", "Mi", "bdr_pen", "bdr_used")
    ] + [("parts", C.POINTER(OrcParticles)), ("fpd_ph", C.POINTER(C.c_double))]


def abi_uv_len(nr, nz):
    return (nr + 1) * nz + nr * (nz - 1)


class Oracle:
    """FP64 CPU restatement bound to one drd_params."""

    def __init__(self, params, openmp=False):
        self.P = params.copy()
        self.L = lib(openmp)
        nr, nz = self.P.nr, self.P.nz
        self.ph_lcc = np.zeros(nr * nz)
        self.pre_lcc = np.zeros((nr + 1) * (nz + 1))
        self.L.orc_setup_tables(C.byref(self.P), ptr(self.ph_lcc), ptr(self.pre_lcc))
        self.L.orc_step.argtypes = [C.POINTER(abi.drd_params), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(OrcState), C.c_int, C.c_double, C.POINTER(abi.drd_status)]

    # -- transforms on arrays of sequences --------------------------------------------------
    def vcost(self, x, axis=-1):
        return self._transform(self.L.orc_vcost, x, axis)

    def redft10(self, x, axis=-1):
        return self._transform(self.L.orc_redft10, x, axis)

    def redft01(self, x, axis=-1):
        return self._transform(self.L.orc_redft01, x, axis)

    @staticmethod
    def _transform(fn, x, axis):
        y = np.ascontiguousarray(np.moveaxis(np.array(x, dtype=np.float64), axis, -1))
        n = y.shape[-1]
        m = y.size // n
        fn(n, m, ptr(y), n, 1)
        return np.moveaxis(y, -1, axis)

    # -- operators ---------------------------------------------------------------------------
    def op_double_gradient_neum(self, x, mo):
        out = np.zeros_like(x)
        self.L.orc_op_double_gradient_neum(self.P.nr, self.P.nz, self.P.dr ** 2, self.P.dz ** 2,
                                           ptr(np.ascontiguousarray(x)), ptr(np.ascontiguousarray(mo)), ptr(out))
        return out

    def ch_matvec(self, M0, Mi, x, alpha=1.0, beta=0.0, y=None):
        y = np.zeros_like(x) if y is None else np.array(y, dtype=np.float64)
        self.L.orc_ch_matvec(C.byref(self.P), ptr(M0), ptr(Mi), alpha, ptr(np.ascontiguousarray(x)), beta, ptr(y))
        return y

    def ch_psolve(self, x):
        y = np.zeros_like(x)
        self.L.orc_ch_psolve(C.byref(self.P), ptr(self.ph_lcc), ptr(np.ascontiguousarray(x)), ptr(y))
        return y

    def ch_psolve_blend(self, w, x):
        """y = q + w (x - q), q = PSolve_CG(x) (w None: PSolve_CG alone)."""
        y = np.zeros_like(x)
        self.L.orc_ch_psolve_blend(C.byref(self.P), ptr(self.ph_lcc), None if w is None else ptr(np.ascontiguousarray(w)),
                                   ptr(np.ascontiguousarray(x)), ptr(y))
        return y

    def ch_blend_probe(self, M0, Mi, nprobe, seed):
        """The probe-fitted blend weights (packed nr x nz) of the CH operator with mobilities M0, Mi."""
        w = np.zeros(self.P.nr * self.P.nz)
        self.L.orc_ch_blend_probe(C.byref(self.P), ptr(self.ph_lcc), ptr(M0), ptr(Mi), int(nprobe), int(seed), ptr(w))
        return w

    def ch_solve_blend(self, M0, Mi, w, b, x0=None):
        """BiCGSTAB on the CH system with the blended preconditioner; returns (x, status)."""
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        st = abi.drd_status()
        self.L.orc_ch_solve_blend(C.byref(self.P), ptr(self.ph_lcc), ptr(M0), ptr(Mi),
                                  None if w is None else ptr(np.ascontiguousarray(w)), ptr(np.ascontiguousarray(b)),
                                  ptr(x), C.byref(st))
        return x, st

    def uv_matvec(self, bdf, rho, eta, pen, x, alpha=1.0, beta=0.0, y=None):
        y = np.zeros_like(x) if y is None else np.array(y, dtype=np.float64)
        self.L.orc_uv_matvec(C.byref(self.P), bdf, ptr(rho), ptr(eta), ptr(pen), alpha,
                             ptr(np.ascontiguousarray(x)), beta, ptr(y))
        return y

    def uv_psolve(self, bdf, rho, eta, x):
        y = np.zeros_like(x)
        self.L.orc_uv_psolve(C.byref(self.P), bdf, ptr(rho), ptr(eta), ptr(np.ascontiguousarray(x)), ptr(y))
        return y

    def solve(self, system, bdf, coefs, b, x0=None):
        """A x = b for system 0 (CH mu) or 1 (momentum) -> (x, status).  coefs: M0, Mi (CH) or
        rho, eta, bdr_pen (momentum), CELL shaped."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        z = np.zeros(1)
        g = lambda k: ptr(np.ascontiguousarray(coefs[k])) if k in coefs else ptr(z)
        st = abi.drd_status()
        self.L.orc_solve_system(C.byref(self.P), system, bdf, ptr(self.ph_lcc), g("M0"), g("Mi"), g("rho"), g("eta"),
                                g("bdr_pen"), ptr(b), ptr(x), C.byref(st))
        return x, st

    def uv_psolve_esolp(self, bdf, x):
        """ESOLP_x on a packed momentum vector (Precipitation_dynamics/VeloSolve_combined.f90:800-806)."""
        y = np.zeros_like(x)
        self.L.orc_uv_psolve_esolp(C.byref(self.P), bdf, ptr(np.ascontiguousarray(x)), ptr(y))
        return y

    def uv_esolp_scale(self, bdf, rho, eta):
        """s = sqrt(D0 / D) of DRD_UV_ESOLP_SCALED (packed momentum unknowns)."""
        s = np.zeros(abi_uv_len(self.P.nr, self.P.nz))
        self.L.orc_uv_esolp_scale(C.byref(self.P), bdf, ptr(rho), ptr(eta), ptr(s))
        return s

    def uv_psolve_esolp_scaled(self, bdf, s, x):
        y = np.zeros_like(x)
        self.L.orc_uv_psolve_esolp_scaled(C.byref(self.P), bdf, ptr(np.ascontiguousarray(s)),
                                          ptr(np.ascontiguousarray(x)), ptr(y))
        return y

    def esolp_coefs(self, bdf):
        """(ua, ub, uc) as (nr+1, nz) arrays [mode, row] and (va, vb, vc) as (nr, nz-1)."""
        nr, nz = self.P.nr, self.P.nz
        u = [np.zeros((nr + 1) * nz) for _ in range(3)]
        v = [np.zeros(nr * (nz - 1)) for _ in range(3)]
        self.L.orc_esolp_coefs(C.byref(self.P), bdf, *[ptr(a) for a in u + v])
        return [a.reshape(nr + 1, nz) for a in u], [a.reshape(nr, nz - 1) for a in v]

    def phmu_matvec(self, M0, Mi, used, x, coef_bot=1.0, coef_top=1.0, alpha=1.0, beta=0.0, y=None):
        y = np.zeros_like(x) if y is None else np.array(y, dtype=np.float64)
        self.L.orc_phmu_matvec(C.byref(self.P), ptr(M0), ptr(Mi), ptr(used), coef_bot, coef_top, alpha,
                               ptr(np.ascontiguousarray(x)), beta, ptr(y))
        return y

    def phmu_psolve(self, x):
        y = np.zeros_like(x)
        self.L.orc_phmu_psolve(C.byref(self.P), ptr(np.ascontiguousarray(x)), ptr(y))
        return y

    # -- systems and residuals -----------------------------------------------------------------
    def ch_system(self, u, v, ph, rmu, bdr_ph, bdr_ph_grad, Mi):
        n = self.P.nr * self.P.nz
        f2, b, x0 = np.zeros_like(ph), np.zeros(n), np.zeros(n)
        self.L.orc_ch_system(C.byref(self.P), ptr(u), ptr(v), ptr(ph), ptr(rmu), ptr(bdr_ph), ptr(bdr_ph_grad),
                             ptr(Mi), ptr(f2), ptr(b), ptr(x0))
        return b, x0, f2

    def ch_residual(self, inputs, coefs, rmu_after):
        """||b - A x|| / ||b|| of the PhSolve system for a solution field rmu_after (CELL)."""
        u, v, ph, rmu = inputs
        b, _, _ = self.ch_system(u, v, ph, rmu, coefs["bdr_ph"], coefs["bdr_ph_grad"], coefs["Mi"])
        x = np.ascontiguousarray(rmu_after[1:-1, 1:-1]).reshape(-1)
        r = b - self.ch_matvec(coefs["M0"], coefs["Mi"], x)
        return float(np.linalg.norm(r) / np.linalg.norm(b))

    def phmu_system(self, u, v, ph, rmu, bdr_ph, bdr_used, bdr_grad, angleB, angleT):
        nr, nz = self.P.nr, self.P.nz
        M0 = np.zeros_like(ph)
        b, x0 = np.zeros(2 * nr * nz), np.zeros(2 * nr * nz)
        pnb, pnt, cbt = np.zeros(nr), np.zeros(nr), np.zeros(2)
        self.L.orc_phmu_system(C.byref(self.P), ptr(u), ptr(v), ptr(ph), ptr(rmu), ptr(bdr_ph), ptr(bdr_used),
                               ptr(bdr_grad), ptr(np.ascontiguousarray(angleB, dtype=np.float64)),
                               ptr(np.ascontiguousarray(angleT, dtype=np.float64)), ptr(M0), ptr(b), ptr(x0),
                               ptr(pnb), ptr(pnt), ptr(cbt))
        return b, x0, M0, cbt

    def phmu_residual(self, inputs, coefs, angleB, angleT, ph_after, rmu_after):
        """||b - A x|| / ||b|| of the ph_mu_solve system for solution fields (CELL)."""
        u, v, ph, rmu = inputs
        b, _, M0, cbt = self.phmu_system(u, v, ph, rmu, coefs["bdr_ph"], coefs["bdr_used"], coefs["bdr_ph_grad"],
                                         angleB, angleT)
        x = np.concatenate([ph_after[1:-1, 1:-1].reshape(-1), rmu_after[1:-1, 1:-1].reshape(-1)])
        r = b - self.phmu_matvec(M0, coefs["Mi"], coefs["bdr_used"], x, cbt[0], cbt[1])
        return float(np.linalg.norm(r) / np.linalg.norm(b))

    # -- per-step routines -------------------------------------------------------------------
    def phsolve(self, u, v, ph, rmu, bdr_ph, bdr_ph_grad, M0, Mi):
        rmu_after = np.zeros_like(ph)
        ph_after = np.zeros_like(ph)
        st = abi.drd_status()
        self.L.orc_phsolve(C.byref(self.P), ptr(self.ph_lcc), ptr(u), ptr(v), ptr(ph), ptr(rmu), ptr(bdr_ph),
                           ptr(bdr_ph_grad), ptr(M0), ptr(Mi), ptr(rmu_after), ptr(ph_after), C.byref(st))
        return rmu_after, ph_after, st

    def ph_mu_solve(self, u, v, ph, rmu, bdr_ph, bdr_used, bdr_grad, Mi, angleB, angleT):
        M0 = np.zeros_like(ph)
        ph_after = np.zeros_like(ph)
        rmu_after = np.zeros_like(ph)
        cbt = np.zeros(2)
        st = abi.drd_status()
        self.L.orc_ph_mu_solve(C.byref(self.P), ptr(u), ptr(v), ptr(ph), ptr(rmu), ptr(bdr_ph), ptr(bdr_used),
                               ptr(bdr_grad), ptr(Mi), ptr(angleB), ptr(angleT), ptr(M0), ptr(ph_after),
                               ptr(rmu_after), ptr(cbt), C.byref(st))
        return ph_after, rmu_after, M0, cbt, st

    def velosolve(self, bdf, psi1, psi2, u_pre, u, v_pre, v, p, rho, eta, bdr_ph, bdr_pen, bdr_used,
                  ph_after, rmu_after, t, pf1, pf2):
        u_after = np.zeros_like(u)
        v_after = np.zeros_like(v)
        nz = self.P.nz
        uL = np.zeros(nz + 1)
        uR = np.zeros(nz + 1)
        st = abi.drd_status()
        rc = self.L.orc_velosolve(C.byref(self.P), bdf, ptr(psi1), ptr(psi2), ptr(u_pre), ptr(u), ptr(v_pre),
                                  ptr(v), ptr(p), ptr(rho), ptr(eta), ptr(bdr_ph), ptr(bdr_pen), ptr(bdr_used),
                                  ptr(ph_after), ptr(rmu_after), t, ptr(pf1), ptr(pf2), ptr(u_after),
                                  ptr(v_after), ptr(uL), ptr(uR), C.byref(st))
        if rc == abi.DRD_ERR_UNSUPPORTED:
            raise ValueError("slip walls (xlsB >= 1e-8) have no solve in the reference")
        return u_after, v_after, uL, uR, st

    def presolve(self, u, v, coef):
        psi = np.zeros(((self.P.nz + 2), (self.P.nr + 2)))
        self.L.orc_presolve(C.byref(self.P), ptr(self.pre_lcc), ptr(u), ptr(v), coef, ptr(psi))
        return psi

    def interpolate_coef(self, dist, bdr_ph):
        fpd = np.zeros_like(bdr_ph)
        rho = np.zeros_like(bdr_ph)
        eta = np.zeros_like(bdr_ph)
        self.L.orc_interpolate_coef(C.byref(self.P), ptr(np.ascontiguousarray(dist)), ptr(bdr_ph), ptr(fpd),
                                    ptr(rho), ptr(eta))
        return fpd, rho, eta

    def pressure_matvec(self, bdr_ph, x):
        """The batched solves' variable-coefficient pressure Poisson operator."""
        y = np.zeros_like(x)
        self.L.orc_pressure_matvec(C.byref(self.P), ptr(bdr_ph), ptr(np.ascontiguousarray(x)), ptr(y))
        return y

    def pressure_psolve(self, x):
        """PreSolve_2's DCT solve on packed cells (the pressure systems' preconditioner)."""
        y = np.zeros_like(x)
        self.L.orc_pressure_psolve(C.byref(self.P), ptr(self.pre_lcc), ptr(np.ascontiguousarray(x)), ptr(y))
        return y

    def pressure_solve(self, bdr_ph, b, x0=None):
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
        st = abi.drd_status()
        info = self.L.orc_pressure_solve(C.byref(self.P), ptr(self.pre_lcc), ptr(bdr_ph), ptr(b), ptr(x), C.byref(st))
        return x, st, info

    def two_phase_coef(self, fpd_ph, ph):
        """The two-fluid rho, eta (two_phase_flow_complex_domain/interpolate_coef.f90:91-112)."""
        rho, eta = np.zeros_like(ph), np.zeros_like(ph)
        self.L.orc_two_phase_coef(C.byref(self.P), ptr(fpd_ph), ptr(ph), ptr(rho), ptr(eta))
        return rho, eta

    def reinint_by_phsolve(self, bdr_ph):
        """reinint_by_PhSolve -> (bdr_ph, bdr_ph_penalty, info)."""
        b, pen = np.zeros_like(bdr_ph), np.zeros_like(bdr_ph)
        info = self.L.orc_reinint_by_phsolve(C.byref(self.P), ptr(self.ph_lcc), ptr(bdr_ph), ptr(b), ptr(pen))
        return b, pen, info

    def dissipation(self, u, v, ph, rmu, vs, angleB=None, angleT=None):
        """dissipation's (e1, e2, e3, e4, dissip, mass)."""
        out = np.zeros(6)
        self.L.orc_dissipation(C.byref(self.P), ptr(u), ptr(v), ptr(ph), ptr(rmu), ptr(angleB), ptr(angleT), vs,
                               ptr(out))
        return tuple(float(x) for x in out)

    def mass(self, ph):
        return self.L.orc_mass(C.byref(self.P), ptr(ph))

    # -- PhSolve_ori and finit's wall smoothing (PhSolve_ori.f90, finit.f90:120-189) ---------
    def ori_coef(self, alpha_s=0.0):
        return self.L.orc_ori_coef(C.byref(self.P), alpha_s)

    def ori_matvec(self, x, alpha_s=0.0, alpha=1.0, beta=0.0, y=None):
        y = np.zeros_like(x) if y is None else y.copy()
        cb = self.ori_coef(alpha_s)
        self.L.orc_ori_matvec(C.byref(self.P), cb, cb, alpha, ptr(x), beta, ptr(y))
        return y

    def ori_system(self, u, v, ph, angleB=None, angleT=None, alpha_s=0.0):
        nr, nz = self.P.nr, self.P.nz
        f2 = np.zeros_like(ph)
        rhs, x0, pnb, pnt = np.zeros(nr * nz), np.zeros(nr * nz), np.zeros(nr), np.zeros(nr)
        self.L.orc_ori_system(C.byref(self.P), ptr(u), ptr(v), ptr(ph), ptr(angleB), ptr(angleT), alpha_s,
                              ptr(f2), ptr(rhs), ptr(x0), ptr(pnb), ptr(pnt))
        return rhs, x0, pnb, pnt

    def phsolve_ori(self, u, v, ph, angleB=None, angleT=None, alpha_s=0.0):
        rmu_after, ph_after = np.zeros_like(ph), np.zeros_like(ph)
        st = abi.drd_status()
        self.L.orc_phsolve_ori(C.byref(self.P), ptr(self.ph_lcc), ptr(u), ptr(v), ptr(ph), ptr(angleB), ptr(angleT),
                               alpha_s, ptr(rmu_after), ptr(ph_after), C.byref(st))
        return rmu_after, ph_after, st

    def finit_wall(self, bdr_ph, nsteps=51):
        out = [np.zeros_like(bdr_ph) for _ in range(3)]
        info = self.L.orc_finit_wall(C.byref(self.P), ptr(self.ph_lcc), ptr(bdr_ph), nsteps, *[ptr(a) for a in out])
        return out[0], out[1], out[2], info

    # -- fiber particles (particles_move.f90) -----------------------------------------------
    def particle_forces(self, pp, points, bdr_dist):
        tot_f = np.zeros_like(points)
        self.L.orc_particle_forces(C.byref(self.P), C.byref(pp), ptr(points), ptr(bdr_dist), ptr(tot_f))
        return tot_f

    def force_caculation_vel(self, pp, points, bdr_dist):
        tot_f = np.zeros_like(points)
        pf1 = np.zeros_like(bdr_dist)
        pf2 = np.zeros_like(bdr_dist)
        self.L.orc_force_caculation_vel(C.byref(self.P), C.byref(pp), ptr(points), ptr(bdr_dist), ptr(tot_f),
                                        ptr(pf1), ptr(pf2))
        return tot_f, pf1, pf2

    def update_position_vel(self, pp, points, u, v, dt):
        out = np.array(points, dtype=np.float64, copy=True)
        self.L.orc_update_position_vel(C.byref(self.P), C.byref(pp), ptr(out), ptr(u), ptr(v), dt)
        return out

    def fpd_dist_field(self, pp, points):
        dist = np.zeros((self.P.nz, self.P.nr))
        self.L.orc_fpd_dist_field(C.byref(self.P), C.byref(pp), ptr(points), ptr(dist))
        return dist

    def step(self, state, coefs, first, t, particles=None):
        """state: dict field-id -> array (updated in place); coefs: dict of coefficient arrays.
        particles: None (held fixed) or a dict with "pp", "points" (POINTS array, moved in place)
        and "bdr_dist"; the step then writes "tot_F", "fpd", "rho" and "eta" into it."""
        S = OrcState()
        for fid in range(abi.F_COUNT):
            S.f[fid] = ptr(state[fid])
        for name in ("rho", "eta", "bdr_ph", "bdr_ph_grad", "M0", "Mi", "bdr_pen", "bdr_used"):
            setattr(S, name, ptr(coefs[name]))
        if "fpd" in coefs:
            S.fpd_ph = ptr(coefs["fpd"])
        X = None
        if particles is not None:
            shape = coefs["rho"].shape
            for key in ("fpd", "rho", "eta"):
                particles.setdefault(key, np.zeros(shape))
            particles.setdefault("tot_F", np.zeros_like(particles["points"]))
            X = OrcParticles()
            X.pp = particles["pp"]
            X.points = ptr(particles["points"])
            X.tot_F = ptr(particles["tot_F"])
            X.bdr_dist = ptr(particles["bdr_dist"])
            X.fpd_ph, X.rho, X.eta = ptr(particles["fpd"]), ptr(particles["rho"]), ptr(particles["eta"])
            S.parts = C.pointer(X)
        st = (abi.drd_status * 2)()
        self.L.orc_step(C.byref(self.P), ptr(self.ph_lcc), ptr(self.pre_lcc), C.byref(S), int(first), t, st)
        return st[0], st[1]
