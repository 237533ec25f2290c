"""ctypes mirror of include/drd_gb300.h (structs, constants).

The structs here must match the C header field for field; tests/test_abi.py checks the
sizes and offsets against the header's own layout rules.
"""
import ctypes as C

DRD_ABI_VERSION = 1

DRD_VARIANT_MF = 0
DRD_VARIANT_TP = 1
DRD_PREC_FP64 = 0
DRD_PREC_MIXED = 1

DRD_OK = 0
DRD_ERR_BADARG = -100
DRD_ERR_CUDA = -101
DRD_ERR_TIMEOUT = -102
DRD_ERR_UNSUPPORTED = -103
DRD_ERR_NONFINITE = -104
DRD_ERR_NOMEM = -105
DRD_ERR_TOO_LARGE = -106

DRD_FLAG_EARLY_S = 1
DRD_FLAG_EARLY_X0 = 2
DRD_FLAG_REFINED = 4
DRD_FLAG_FALLBACK64 = 8

DRD_OP_CH_MATVEC, DRD_OP_CH_PSOLVE, DRD_OP_UV_MATVEC, DRD_OP_UV_PSOLVE, DRD_OP_PHMU_MATVEC, DRD_OP_PHMU_PSOLVE = range(6)
DRD_OP_PERSISTENT = 2  # op_apply precision: the persistent solver's FP32 operator code
DRD_SYS_CH, DRD_SYS_UV = 0, 1  # drd_solve systems
DRD_UV_JACOBI, DRD_UV_ESOLP, DRD_UV_ESOLP_SCALED = 0, 1, 2  # drd_params.uv_precond

(DRD_KB_UV_MATVEC_FP64, DRD_KB_UV_MATVEC_FP32, DRD_KB_DCT_X_FP64, DRD_KB_DCT_X_FP32, DRD_KB_DCT_Z_FP64,
 DRD_KB_DCT_Z_FP32, DRD_KB_CH_MATVEC_FP32, DRD_KB_PRESSURE_FFT64, DRD_KB_DCT2_FFT32) = range(9)
KB_NAMES = {
    DRD_KB_UV_MATVEC_FP64: "k_uv_mv<double> (momentum stencil)",
    DRD_KB_UV_MATVEC_FP32: "k_uv_mv<float> (momentum stencil)",
    DRD_KB_DCT_X_FP64: "k_gemm<double> DCT-I x pass",
    DRD_KB_DCT_X_FP32: "k_gemm<float> DCT-I x pass",
    DRD_KB_DCT_Z_FP64: "k_gemm<double> DCT-I z pass",
    DRD_KB_DCT_Z_FP32: "k_gemm<float> DCT-I z pass",
    DRD_KB_CH_MATVEC_FP32: "k_ch_mv2<float> (CH stencil)",
    DRD_KB_PRESSURE_FFT64: "k_pfft_* PreSolve_2 by FFT, FP64 (cold L2)",
    DRD_KB_DCT2_FFT32: "k_pfft_* REDFT10 / Pre_Lcc / REDFT01, FP32 (cold L2)",
}

# resident-state fields (DRD_F_*)
F_U, F_V, F_U_PRE, F_V_PRE, F_PH, F_RMU, F_PH_PRE, F_RMU_PRE, F_P, F_PSI1, F_PSI2, F_PF1, F_PF2 = range(13)
F_COUNT = 13
FIELD_KIND = {
    F_U: "u", F_V: "v", F_U_PRE: "u", F_V_PRE: "v", F_PH: "cell", F_RMU: "cell", F_PH_PRE: "cell",
    F_RMU_PRE: "cell", F_P: "cell", F_PSI1: "cell", F_PSI2: "cell", F_PF1: "cell", F_PF2: "cell",
}


class drd_params(C.Structure):
    _fields_ = [
        ("nr", C.c_int32), ("nz", C.c_int32), ("variant", C.c_int32), ("precision", C.c_int32),
        ("phi_mode", C.c_int32), ("lr_bd_type", C.c_int32), ("ch_maxit", C.c_int32),
        ("uv_maxit", C.c_int32), ("phmu_maxit", C.c_int32), ("guess_mode", C.c_int32),
        ("dr", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
        ("xld", C.c_double), ("re", C.c_double), ("ca", C.c_double),
        ("I_thickness", C.c_double), ("s_implicit", C.c_double), ("tol", C.c_double),
        ("ggx", C.c_double), ("ggz", C.c_double), ("uwT", C.c_double), ("uwB", C.c_double),
        ("UU", C.c_double), ("twall", C.c_double), ("bdr_upp", C.c_double), ("bdr_low", C.c_double),
        ("angle", C.c_double), ("xlsB", C.c_double), ("penalty_k", C.c_double),
        ("lambda_rho", C.c_double), ("lambda_eta", C.c_double), ("bdr_ph_used_adjust", C.c_double),
        ("mixed_inner_tol", C.c_double), ("mixed_max_refine", C.c_int32), ("uv_precond", C.c_int32),
        ("two_fluid", C.c_int32), ("reserved1", C.c_int32),
    ]

    def copy(self):
        out = drd_params()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(drd_params))
        return out

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if not name.startswith("reserved")}


class drd_diagnostics(C.Structure):
    """dissipation()'s diagnostics (microfluidics_complex_domain/dissipation.f90:1-122)."""
    _fields_ = [(n, C.c_double) for n in ("e1", "e2", "e3", "e4", "dissip", "mass")]

    def as_tuple(self):
        return (self.e1, self.e2, self.e3, self.e4, self.dissip, self.mass)


DRD_SYS_PRESSURE = 2  # batched variable-coefficient pressure Poisson systems
DRD_BATCH_MAX_LINE = 2048


class drd_batch_problem(C.Structure):
    """One system of a batch (drd_batch_create)."""
    _fields_ = [("system", C.c_int32), ("bdf", C.c_int32), ("params", drd_params)] + [
        (n, C.POINTER(C.c_double)) for n in ("rho", "eta", "bdr_ph", "b", "x0")]


PARTICLES_MAX = 64


class drd_particle_params(C.Structure):
    """module particles_params (microfluidics_complex_domain/particles_params.f90)."""
    _fields_ = [
        ("np", C.c_int32), ("reserved0", C.c_int32), ("lx", C.c_double), ("ly", C.c_double),
        ("fpd_radius", C.c_double), ("l0", C.c_double), ("ks", C.c_double), ("kb", C.c_double),
        ("theta0", C.c_double), ("k0_inter", C.c_double), ("k0_inter_bdr", C.c_double),
        ("fpd_fpd_dist", C.c_double), ("fpd_bdr_dist", C.c_double),
    ]

    def copy(self):
        out = drd_particle_params()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(drd_particle_params))
        return out


def default_particle_params(lx, ly, np_beads=9):
    """The reference's fiber parameters (particles_params.f90:74-98), same arithmetic as
    drd_particle_params_default in the C library."""
    pp = drd_particle_params()
    pp.np = np_beads
    pp.lx, pp.ly = lx, ly
    pp.fpd_radius = 0.05 / 2.0
    pp.l0 = 2 * (pp.fpd_radius + 0.00)
    pp.ks = 5.0
    pp.kb = 0.0025 * 100
    pp.theta0 = 0.0
    pp.k0_inter = 2.5
    pp.k0_inter_bdr = 2.5 * 10
    pp.fpd_fpd_dist = pp.fpd_radius + pp.fpd_radius + 0.01
    pp.fpd_bdr_dist = pp.fpd_radius + 0.02
    return pp


def particle_chain(pp, xc, yc):
    """particle_initialize's straight vertical chain (particles_move.f90:50-68) as a POINTS
    array: Np x 2 column-major, returned as shape (2, Np)."""
    np_ = pp.np
    pts = [[0.0] * np_, [0.0] * np_]
    if np_ > 2:
        mid = np_ // 2
        pts[0][mid], pts[1][mid] = xc, yc
        for i in range(mid):
            pts[0][i], pts[1][i] = xc, yc + (mid - i) * pp.l0
            pts[0][np_ - i - 1], pts[1][np_ - i - 1] = xc, yc - (mid - i) * pp.l0
    return pts


class drd_deck(C.Structure):
    """The `input` deck (microfluidics_complex_domain/mcl6.f90:68-99)."""
    _fields_ = [(n, C.c_double) for n in ("xld", "re", "ca", "vs", "xlsT", "xlsB", "xlsL", "xlsR", "uwT", "uwB",
                                          "slen", "shig", "angle", "slipratio")] + [
        ("iflag", C.c_int32), ("istep", C.c_int32)] + [
        (n, C.c_double) for n in ("tf", "I_thickness", "s_implicit", "tol", "ggz", "ggx", "time_step_change",
                                  "lambda_rho", "lambda_eta", "UU")] + [
        (n, C.c_char) for n in ("lr_bd_type", "top_type_ph", "bot_type_ph", "top_type_u", "bot_type_u",
                                "is_complex_domain")] + [
        ("pad", C.c_char * 2), ("entries", C.c_int32), ("reserved", C.c_int32)]


class drd_status(C.Structure):
    _fields_ = [
        ("info", C.c_int32), ("iter", C.c_int32), ("resid", C.c_double), ("true_resid", C.c_double),
        ("refinements", C.c_int32), ("flags", C.c_uint32), ("seconds", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class drd_step_stats(C.Structure):
    _fields_ = [("ch", drd_status), ("uv", drd_status), ("pre", drd_status), ("mass", C.c_double),
                ("t", C.c_double), ("seconds", C.c_double)]


def default_params(nr, nz, **kw):
    """Parameters of the reference deck (microfluidics_complex_domain/input:1-31, global.f90:91,
    mcl6.f90:151, finit.f90:106-107,397) on an nr x nz grid of slen x shig = 3.5 x 1.5."""
    p = drd_params()
    p.nr, p.nz = nr, nz
    p.variant = DRD_VARIANT_MF
    p.precision = DRD_PREC_FP64
    p.phi_mode = 1
    p.lr_bd_type = ord("d")
    p.ch_maxit, p.uv_maxit, p.phmu_maxit = 500, 800, 5000
    slen, shig = 3.5, 1.5
    p.dr, p.dz = slen / nr, shig / nz
    p.xld, p.re, p.ca = 5.0e-2, 1.0, 100.0
    p.I_thickness, p.s_implicit, p.tol = 0.005, 1.5, 1.0e-8
    p.ggx, p.ggz = 0.0, 0.0
    p.uwT, p.uwB = 0.0, 0.0
    p.UU, p.twall = 1.0, 0.1
    p.bdr_upp, p.bdr_low = 0.6725, 0.1725
    p.angle, p.xlsB = 135.0, 0.0
    p.penalty_k = 1.0e5
    p.lambda_rho, p.lambda_eta = 1.0, 100.0
    p.bdr_ph_used_adjust = 1.0e-6
    p.dt = min(p.dr, p.dz) * 0.1
    p.mixed_inner_tol = 0.2
    p.mixed_max_refine = 30
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(f"drd_params has no field {k!r}")
        setattr(p, k, ord(v) if k == "lr_bd_type" and isinstance(v, str) else v)
    return p
