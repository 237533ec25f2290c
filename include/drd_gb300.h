/*
 * drd_gb300.h — C-ABI of the GB300 (sm_103a) per-time-step solver core of DRD-Micro.
 *
 * The reference is a serial Fortran program whose per-step solver subroutines
 * take explicit-shape REAL(8) arrays by reference and read everything else from
 * `module global` (microfluidics_complex_domain/global.f90:1-129).  This header
 * is what a Fortran `iso_c_binding` interface (or ctypes) binds instead: every
 * hidden module input becomes an explicit argument or a field of drd_params,
 * every array keeps its Fortran ghosted shape and column-major order, so the
 * Fortran side passes its arrays unchanged.
 *
 * Array shapes (Fortran bounds, i fastest, no padding):
 *   CELL  (-1:nr, -1:nz)     element (i,k) at [(i+1) + (k+1)*(nr+2)], (nr+2)*(nz+2) doubles
 *   UFACE (-1:nr+1, -1:nz)   element (i,k) at [(i+1) + (k+1)*(nr+3)], (nr+3)*(nz+2) doubles
 *   VFACE (-1:nr, 0:nz)      element (i,k) at [(i+1) +  k   *(nr+2)], (nr+2)*(nz+1) doubles
 *   DIST  (0:nr-1, 0:nz-1)   element (i,k) at [i + k*nr],             nr*nz doubles
 *   ZLINE (0:nz)             uL / uR inlet profiles, nz+1 doubles (entries 0..nz-1 written)
 *   XLINE (0:nr)             angleB / angleT contact angles (TP), nr+1 doubles
 *
 * Host pointers are caller-owned and only read/written during the call.
 * Device buffers are owned by the context.  One context per host thread; a
 * context owns one CUDA stream and its CUDA graphs.
 *
 * Return codes: DRD_OK, a BiCGSTAB INFO value (>0 not converged, -10/-11
 * breakdown, exactly as lib/BiCGSTABREVCOM.f:64-90 defines them), or a
 * negative DRD_ERR_* code for argument, CUDA or timeout errors.  The reference
 * prints INFO and continues (microfluidics_complex_domain/PhSolve.f90:75-79);
 * callers of this library may do the same: outputs are always written.
 */
#ifndef DRD_GB300_H
#define DRD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DRD_ABI_VERSION 1

/* Which application's copy of the solver routines to follow. */
#define DRD_VARIANT_MF 0 /* microfluidics_complex_domain/ (README example, headline)   */
#define DRD_VARIANT_TP 1 /* two_phase_flow_complex_domain/ (ph_mu_solve, sharp penalty) */

/* Arithmetic of the Krylov solves. */
#define DRD_PREC_FP64 0  /* every operator in FP64: the reference's arithmetic           */
#define DRD_PREC_MIXED 1 /* FP32 operators and preconditioners inside FP64 iterative
                            refinement; FP64 inner products and true-residual recompute  */

/* Momentum preconditioners (drd_params.uv_precond). */
#define DRD_UV_JACOBI 0 /* PSolve_uv_2_CG (microfluidics_complex_domain/VeloSolve_2_combined.f90:649-711) */
#define DRD_UV_ESOLP 1  /* ESOLP_x: DCT-I along x, tridiagonal along y (microfluidics_complex_domain/
                           ESOLP.f90:1-82, applied in Precipitation_dynamics/VeloSolve_combined.f90:795-808) */
#define DRD_UV_ESOLP_SCALED 2 /* ESOLP_x between two diagonal scalings (an extension): y = s E(s x),
                                 s = sqrt(D0 / D) per unknown, D the Jacobi diagonal of PSolve_uv_2_CG
                                 with the context's rho and eta, D0 the same with rho = eta = 1 (the
                                 coefficients ESOLP_x's constant operator has).  MF only. */

/* Return codes besides BiCGSTAB INFO values. */
#define DRD_OK 0
#define DRD_ERR_BADARG (-100)
#define DRD_ERR_CUDA (-101)
#define DRD_ERR_TIMEOUT (-102)
#define DRD_ERR_UNSUPPORTED (-103)
#define DRD_ERR_NONFINITE (-104)
#define DRD_ERR_NOMEM (-105)
#define DRD_ERR_TOO_LARGE (-106)

/* Status flags. */
#define DRD_FLAG_EARLY_S 1u      /* stopped at the absolute ||s|| <= tol test (BiCGSTABREVCOM.f:313) */
#define DRD_FLAG_EARLY_X0 2u     /* stopped at the absolute ||b - A x0|| <= tol test (:248)          */
#define DRD_FLAG_REFINED 4u      /* mixed mode: result produced by FP64 iterative refinement         */
#define DRD_FLAG_FALLBACK64 8u   /* mixed mode: the CH system is too stiff for FP32 vectors (the    */
                                 /* grid's stiffness estimate); it was solved with the FP64 solver */

/*
 * Scalars that the reference keeps in `module global` and the input deck
 * (microfluidics_complex_domain/mcl6.f90:68-101, global.f90:30-91).
 */
typedef struct drd_params {
    int32_t nr, nz;        /* cells in x (r) and y (z); global.f90:18-19                          */
    int32_t variant;       /* DRD_VARIANT_*                                                        */
    int32_t precision;     /* DRD_PREC_*                                                           */
    int32_t phi_mode;      /* TP: 1 = phi in [0,1], 2 = phi in [-1,1] (TP/mcl6.f90:156)            */
    int32_t lr_bd_type;    /* TP: 'd' Dirichlet inlet or 'n' Neumann sides (TP/VeloSolve_2:272)   */
    int32_t ch_maxit;      /* PhSolve ITER, 500 (PhSolve.f90:72)                                   */
    int32_t uv_maxit;      /* VeloSolve ITER, 800 MF (VeloSolve_2_combined.f90:398), 2000 TP       */
    int32_t phmu_maxit;    /* ph_mu_solve ITER, 5000 (TP/ph_mu_solve.f90:156)                      */
    int32_t guess_mode;    /* initial guess of the CH and momentum solves: 0 = the previous step's */
                           /* field (the reference); 1, 2, 3 = the polynomial extrapolation of   */
                           /* that order through the last 2, 3, 4 steps (lower orders until the  */
                           /* steps are held): 2 x^n - x^(n-1); 3 x^n - 3 x^(n-1) + x^(n-2);     */
                           /* 4 x^n - 6 x^(n-1) + 4 x^(n-2) - x^(n-3).  drd_step keeps the      */
                           /* history on the device; drd_velosolve_2_combined extrapolates from  */
                           /* u_pre and earlier calls' u_pre, drd_phsolve from earlier calls' rmu */
    double dr, dz, dt;     /* grid spacing and time step (finit.f90:25-28,397)                    */
    double xld, re, ca;    /* 1/Pe, Reynolds, capillary number (input deck lines 1-3)             */
    double I_thickness;    /* interface thickness epsilon (deck line 18)                           */
    double s_implicit;     /* stabilisation s (deck line 19)                                       */
    double tol;            /* BiCGSTAB tolerance (deck line 20)                                    */
    double ggx, ggz;       /* body force (deck lines 21-22)                                        */
    double uwT, uwB;       /* wall speeds (deck lines 9-10)                                        */
    double UU, twall;      /* inlet amplitude (deck line 26), ramp time 0.1 (mcl6.f90:151)         */
    double bdr_upp, bdr_low; /* inlet extent (finit.f90:106-107)                                   */
    double angle;          /* contact angle in degrees (deck line 13)                              */
    double xlsB;           /* bottom slip length; only the no-slip branch (< 1e-8) is on the path  */
    double penalty_k;      /* DRD resistance coefficient (global.f90:91, 1e5)                      */
    double lambda_rho, lambda_eta; /* density / viscosity ratios (deck lines 24-25)                */
    double bdr_ph_used_adjust;     /* TP: 1e-6 (TP/finit.f90:572)                                  */
    double mixed_inner_tol;        /* mixed mode: relative residual reduction per FP32 inner solve; */
                                   /* a sweep that gains < 10 % tightens it tenfold (to 1.5e-4)     */
    int32_t mixed_max_refine;      /* mixed mode: maximum FP64 refinement sweeps                   */
    int32_t uv_precond;            /* momentum preconditioner: DRD_UV_JACOBI (the MF reference),    */
                                   /* DRD_UV_ESOLP (ESOLP_x, used by the PD application) or         */
                                   /* DRD_UV_ESOLP_SCALED (ESOLP_x with the variable-coefficient     */
                                   /* diagonal scaling)                                             */
    int32_t two_fluid;             /* 0: rho, eta follow the solid/particle indicator fpd_ph only   */
                                   /* (interpolate_coef.f90:84-89).  1: the two-fluid form that     */
                                   /* two_phase_flow_complex_domain/interpolate_coef.f90:91-112     */
                                   /* keeps commented out: rho = rho(ph), eta = max(eta(fpd_ph),    */
                                   /* eta(ph)), rebuilt by drd_step after every CH solve from ph    */
                                   /* before the swap, where mcl6 calls interpolate_coef            */
    int32_t reserved1;
} drd_params;

typedef struct drd_status {
    int32_t info;        /* BiCGSTAB INFO on exit (lib/BiCGSTAB.f:99-124)                         */
    int32_t iter;        /* ITER on exit: iterations performed (FP32 iterations summed in mixed)  */
    double resid;        /* RESID on exit                                                          */
    double true_resid;   /* ||b - A x||_2 / ||b||_2 recomputed in FP64 from the returned x         */
    int32_t refinements; /* mixed mode: FP64 refinement sweeps                                     */
    uint32_t flags;      /* DRD_FLAG_*                                                             */
    double seconds;      /* device time of the call (CUDA events)                                  */
} drd_status;

typedef struct drd_ctx drd_ctx;

/* ---- life cycle ------------------------------------------------------------------------ */

/* Replaces setup() (microfluidics_complex_domain/setup.f90:106-155: Ph_Lcc, Pre_Lcc tables)
 * and PreSolve_init() (microfluidics_complex_domain/PreSolve_init.f90:1-16: the FFTW
 * REDFT10/REDFT01 plans).  Allocates all device memory for an nr x nz grid. */
int drd_create(const drd_params* params, drd_ctx** ctx_out);
int drd_destroy(drd_ctx* ctx);
/* Re-derives the dt-dependent tables after dt changes (setup() is re-run in mcl6.f90:201). */
int drd_set_params(drd_ctx* ctx, const drd_params* params);
const char* drd_last_error(drd_ctx* ctx);
int drd_abi_version(void);

/* ---- hidden module inputs --------------------------------------------------------------- */

/* rho, eta, bdr_ph, bdr_ph_grad, ph_M_0, ph_M_inner: CELL arrays of module global
 * (microfluidics_complex_domain/global.f90:47,81-85).  Any pointer may be NULL to keep the
 * value on the device. */
int drd_set_coefs(drd_ctx* ctx, const double* rho, const double* eta, const double* bdr_ph,
                  const double* bdr_ph_grad, const double* ph_M_0, const double* ph_M_inner);
/* TP-only module inputs: bdr_ph_used, bdr_ph_penalty (CELL), angleB, angleT (XLINE)
 * (two_phase_flow_complex_domain/global.f90:44,95-98). */
int drd_set_tp_fields(drd_ctx* ctx, const double* bdr_ph_used, const double* bdr_ph_penalty,
                      const double* angleB, const double* angleT);

/* ---- the solid-blended CH preconditioner (an extension; the reference has no counterpart) --
 * PSolve_CG (microfluidics_complex_domain/PhSolve.f90:296-313) inverts the CH operator with
 * unit mobility everywhere.  In the solid the mobilities ph_M_0, ph_M_inner vanish and the
 * operator tends to the identity, which that solve resolves worst.  With weights w installed
 * (packed nr x nz, the CH unknowns' order, values in [0, 1]) every CH preconditioner
 * application becomes y = q + w (x - q), q = PSolve_CG(x): a fixed linear operator, so
 * BiCGSTAB is unchanged and the solve still ends on the reference's residual test.  MF only.
 * The weights belong to the mobilities: drd_set_coefs with new ph_M_0 or ph_M_inner removes them. */

/* Installs w (host or device memory), or removes the weights when w is NULL. */
int drd_set_ch_blend(drd_ctx* ctx, const double* w);
/* Fits the weights of the current mobilities with `nprobe` Rademacher probes e (entries +-1, the
 * sign of the top bit of splitmix64(seed + (probe nr nz + q + 1) 0x9E3779B97F4A7C15)): r = A e,
 * q = PSolve_CG(r), d = r - q, t = e - q, w = clamp(sum t d / sum d d, 0, 1) per cell (0 where
 * sum d d = 0), in FP64.  Installs them when `install` is non-zero; writes them to w_out (host or
 * device, may be NULL). */
int drd_ch_blend_probe(drd_ctx* ctx, int nprobe, uint64_t seed, int install, double* w_out);

/* ---- the per-step solver core (drop-in for the reference subroutines) ------------------ */

/* interpolate_coef (microfluidics_complex_domain/interpolate_coef.f90:4-92).  `dist` is the
 * particle distance dist(r(i,k), z(i,k)) of every interior cell (DIST shape); fpd_ph, rho,
 * eta (CELL) are written and rho/eta also replace the context's coefficients. */
int drd_interpolate_coef(drd_ctx* ctx, const double* dist, double* fpd_ph, double* rho, double* eta);
/* The two-fluid coefficients of interpolate_coef, in the form two_phase_flow_complex_domain/
 * interpolate_coef.f90:91-112 leaves commented out (its "TODO: two-phase viscosity/density
 * ratio"): with x = ph, rho = 1 (x <= -1), lambda_rho (x >= 1), else 1 + (lambda_rho - 1) x; the
 * same for eta_ph with lambda_eta; eta = max(1 + (lambda_eta - 1) fpd_ph, eta_ph).  fpd_ph (CELL)
 * becomes the context's indicator (NULL keeps the one from the last interpolate_coef, particle
 * step or call of this routine); ph (CELL, NULL = the resident phase field).  rho, eta (CELL)
 * are written (each may be NULL) and replace the context's coefficients.  drd_step does the
 * same on the device after each CH solve when params.two_fluid = 1. */
int drd_two_phase_coef(drd_ctx* ctx, const double* fpd_ph, const double* ph, double* rho, double* eta);

/* ---- initialisation: finit's wall smoothing ------------------------------------------- */

/* PhSolve_ori(rmu_after, ph_after, t) (microfluidics_complex_domain/PhSolve_ori.f90:1-214):
 * the phi in [-1,1] Cahn-Hilliard step with unit mobility and the wall-energy rows at the
 * bottom and top, solved by BiCGSTAB with the PhSolve DCT-I preconditioner.  Inputs u (UFACE),
 * v (VFACE), ph (CELL); angleB, angleT (XLINE, degrees; NULL = 0) and alpha_s are the module
 * globals of its wall terms.  Left/right are Neumann and the wall rows take the non-dynamic
 * branch: finit forces lr_bd_type = top/bot_type_ph = 'n' around its calls (finit.f90:144-147).
 * The context's dt, tol and ch_maxit are the solve's (finit runs it with dt = 1e-4). */
int drd_phsolve_ori(drd_ctx* ctx, const double* u, const double* v, const double* ph, const double* angleB,
                    const double* angleT, double alpha_s, double* rmu_after, double* ph_after, drd_status* st);
/* finit's wall smoothing (finit.f90:120-189): ph = bdr_ph (CELL, interior read) with Neumann
 * ghosts, rmu from ph, then `nsteps` PhSolve_ori steps with u = v = 0 and zero angles and
 * alpha_s (finit sets those after the loop, finit.f90:364-374), then
 * bdr_ph = (ph + 1)/2 clipped to [0, 1] on the interior.  The reference runs 51 steps
 * (finit.f90:172) on a context whose dt is 1e-4 (finit.f90:151).  bdr_ph_out, ph_out, rmu_out
 * (CELL) may be NULL.  The context's resident u, v, ph and rmu fields are overwritten.
 * Returns the last solve's INFO. */
int drd_finit_wall(drd_ctx* ctx, const double* bdr_ph_in, int nsteps, double* bdr_ph_out, double* ph_out,
                   double* rmu_out);
/* reinint_by_PhSolve() (two_phase_flow_complex_domain/reinint_by_PhSolve.f90:1-91): the same
 * 51 PhSolve_ori steps from ph = bdr_ph (unit mobility, Neumann sides and walls, on a context
 * whose dt is 1e-4, :34-56), bdr_ph = (ph + 1)/2 clipped to [0, 1] on the interior (:58-70),
 * then bdr_ph_penalty = 1 where bdr_ph > 0.5, else 0, over the whole ghosted array (:78-86).
 * bdr_ph_in, bdr_ph_out, bdr_ph_penalty_out are CELL (outputs may be NULL).  Like the
 * reference, which rewrites these module globals, it makes the results the context's bdr_ph
 * and penalty mask; the resident u, v, ph and rmu are overwritten.  The mobilities are left as
 * they are (the reference sets ph_M_0 = ph_M_inner = 1 for its loop): a caller rebuilds them
 * and bdr_ph_grad from the new bdr_ph with drd_set_coefs.  Any variant. */
int drd_reinint_by_phsolve(drd_ctx* ctx, const double* bdr_ph_in, double* bdr_ph_out, double* bdr_ph_penalty_out);

/* ---- fiber particles coupled to the flow (microfluidics_complex_domain/particles_move.f90) --
 *
 * A fiber is a chain of Np beads (module particles: points(0:Np-1,0:1)).  Per step the driver
 * (mcl6.f90:394-402) computes the chain forces, spreads them onto the grid as
 * particle_force1/2, moves the beads with the fluid and rebuilds fpd_ph, rho and eta from the
 * new bead positions.  Point arrays are POINTS shaped: Np x 2, column-major like the Fortran
 * points(0:Np-1,0:1) (x of bead b at [b], y at [Np + b]).  Swimmers are not modelled: the
 * reference fixes Np_swm = 0 (particles_params.f90:61). */
#define DRD_PARTICLES_MAX 64

/* The parameters of module particles_params (microfluidics_complex_domain/particles_params.f90). */
typedef struct drd_particle_params {
    int32_t np;            /* beads Np (:78); 0 = no particles, else 3..DRD_PARTICLES_MAX      */
    int32_t reserved0;
    double lx, ly;         /* periodic box: slen, shig (mcl6.f90:397)                         */
    double fpd_radius;     /* bead radius (:80)                                               */
    double l0;             /* rest length between beads (:83)                                 */
    double ks, kb;         /* stretching and bending stiffness (:74-75)                       */
    double theta0;         /* rest bending angle (:76)                                        */
    double k0_inter;       /* bead-bead repulsion (:93)                                       */
    double k0_inter_bdr;   /* wall repulsion (:94)                                            */
    double fpd_fpd_dist;   /* bead-bead repulsion range (:97)                                 */
    double fpd_bdr_dist;   /* wall repulsion range (:98)                                      */
} drd_particle_params;

/* Fills `pp` with the reference's values (Np = 9, radius 0.025, ks 5, kb 0.25, ...) for a box
 * of lx x ly. */
int drd_particle_params_default(drd_particle_params* pp, double lx, double ly);
/* particle_initialize's fiber placement (particles_move.f90:50-68): a straight vertical chain
 * centred on (xc, yc), bead spacing l0.  Host-only; writes POINTS. */
int drd_particle_initialize(const drd_particle_params* pp, double xc, double yc, double* points);
/* Makes the chain resident: parameters, POINTS and bdr_ph_dist (CELL; the distance to the
 * walls that interaction_force_bdr samples, global.f90:83).  pp->np == 0 turns the coupling
 * off.  While np > 0, drd_step runs the particle coupling of mcl6.f90:394-402 every step. */
int drd_particles_set(drd_ctx* ctx, const drd_particle_params* pp, const double* points, const double* bdr_dist);
/* Current bead positions and the last computed total bead forces tot_F (both POINTS; either
 * may be NULL). */
int drd_particles_get(drd_ctx* ctx, double* points, double* tot_F);
/* force_caculation_vel (particles_move.f90:758-868 with force_caculation :421-627): chain,
 * bead-bead and wall forces, spread onto the grid as particle_force1/2 (CELL, written). */
int drd_force_caculation_vel(drd_ctx* ctx, double dt, double t, double* particle_force1, double* particle_force2);
/* update_position_vel (particles_move.f90:872-980): moves every bead by dt times the
 * indicator-weighted mean of u (UFACE) and v (VFACE), wrapping periodically. */
int drd_update_position_vel(drd_ctx* ctx, const double* u, const double* v, double dt);
/* interpolate_coef with dist = fpd_dist of the resident beads (particles_move.f90:361-391,
 * dist.f90): fpd_ph, rho, eta (CELL) written (each may be NULL); rho/eta also replace the
 * context's coefficients. */
int drd_interpolate_coef_particles(drd_ctx* ctx, double* fpd_ph, double* rho, double* eta);

/* PhSolve(rmu_after, ph_after, t) (microfluidics_complex_domain/PhSolve.f90:1-126).
 * Inputs u (UFACE), v (VFACE), ph, rmu (CELL) are the module globals it reads. */
int drd_phsolve(drd_ctx* ctx, const double* u, const double* v, const double* ph, const double* rmu,
                double t, double* rmu_after, double* ph_after, drd_status* st);

/* ph_mu_solve(ph_after, rmu_after, t) (two_phase_flow_complex_domain/ph_mu_solve.f90:3-197).
 * ph_M_0 is recomputed inside the reference (:31-35) and written back (CELL, may be NULL);
 * coef_bot_top[2] receives the global side outputs coef_bot, coef_top (may be NULL). */
int drd_ph_mu_solve(drd_ctx* ctx, const double* u, const double* v, const double* ph, const double* rmu,
                    double t, double* ph_after, double* rmu_after, double* ph_M_0_out,
                    double* coef_bot_top, drd_status* st);

/* VeloSolve_combined(psi, u_after, v_after, rmu_after, ph_after, t, pf1, pf2)
 * (microfluidics_complex_domain/VeloSolve_combined.f90:5-511): first-step backward Euler.
 * u, v (module globals), p (CELL), psi (unused by the reference, may be NULL).  uL, uR
 * (ZLINE) receive the global inlet profiles (may be NULL). */
int drd_velosolve_combined(drd_ctx* ctx, const double* psi, const double* u, const double* v,
                           const double* p, const double* rmu_after, const double* ph_after, double t,
                           const double* particle_force1, const double* particle_force2,
                           double* u_after, double* v_after, double* uL, double* uR, drd_status* st);

/* VeloSolve_2_combined(psi1, psi2, u_pre, u_after, v_pre, v_after, ph_pre, ph_after,
 * rmu_pre, rmu_after, t, pf1, pf2) (microfluidics_complex_domain/VeloSolve_2_combined.f90:4-510
 * and two_phase_flow_complex_domain/VeloSolve_2_combined.f90): BDF2 momentum with the DRD
 * penalty.  ph_pre and rmu_pre are unused by the reference (may be NULL). */
int drd_velosolve_2_combined(drd_ctx* ctx, const double* psi1, const double* psi2,
                             const double* u_pre, const double* u, const double* v_pre, const double* v,
                             const double* p, const double* ph_pre, const double* ph_after,
                             const double* rmu_pre, const double* rmu_after, double t,
                             const double* particle_force1, const double* particle_force2,
                             double* u_after, double* v_after, double* uL, double* uR, drd_status* st);

/* PreSolve_2(plan, plan_back, psi, coef) (microfluidics_complex_domain/PreSolve_2.f90:1-130 with
 * dct_fftw :135-186): div u -> DCT-II -> / Pre_Lcc -> DCT-III -> / (4 nr nz) -> Neumann ghosts
 * -> * coef.  u (UFACE), v (VFACE) are the module globals it reads; psi is CELL. */
int drd_presolve_2(drd_ctx* ctx, const double* u, const double* v, double coef, double* psi,
                   drd_status* st);

/* Mass sum of dissipation() (microfluidics_complex_domain/dissipation.f90:116-122), FP64. */
int drd_mass(drd_ctx* ctx, const double* ph, double* mass);

/* The diagnostics of dissipation(ph_pre, dissip, mass, t) (microfluidics_complex_domain/
 * dissipation.f90:1-122), in FP64 on the device with a fixed summation order:
 *   e1 = xld ca dr dz sum_cells |grad rmu|^2          (central differences over rmu's ghosts, :39-47)
 *   e2 = vs ca eps^2 dr sum_i (wall residual of the contact-angle condition)^2 at the top and
 *        bottom rows, with cf = sqrt2 cos(angle pi/180)/3 pi/2/eps (:49-57)
 *   e3 = dr dz sum_{i=0..nr, k=0..nz} Cx Cz (u_x^2 + v_z^2 + u_z^2 + v_x^2), Cx, Cz = 1/2 at
 *        the ends (:59-88), u_z and v_z one-sided in the wall rows as :68-77 writes them
 *   e4 = 0: the slip term (:91-99) runs only for xlsB >= 1e-8, which this library rejects
 *   dissip = e1 + e2 + e3 + e4; mass = sum ph dr dz (:113-122)
 * The reference's e3 is not fully defined: it passes v to dif1x through a dummy of u's shape
 * (leading dimension nr+3 instead of nr+2) and sums vvb where only its two wall rows were
 * assigned.  Here every derivative is taken on the field's own grid: v_x and v_z by central
 * differences on v(-1:nr, 0:nz), one-sided at i = nr and in the wall rows.
 * u (UFACE), v (VFACE), ph, rmu (CELL) may be NULL for the resident fields; angleB, angleT
 * (XLINE, degrees) NULL for params.angle everywhere; vs is the deck's slip coefficient (line 4). */
typedef struct drd_diagnostics {
    double e1, e2, e3, e4, dissip, mass;
} drd_diagnostics;
int drd_dissipation(drd_ctx* ctx, const double* u, const double* v, const double* ph, const double* rmu,
                    const double* angleB, const double* angleT, double vs, drd_diagnostics* out);
/* The two diagnostic records mcl6 appends per output step: fort.23's `write(23,110) t, e1, e2,
 * e3, e4, dissip` with format 6e14.7 (dissipation.f90:103-105), and fort.22's
 * `write(22,*) kcount, dt*dissip, mass` (mcl6.f90:235, :361), written here as one integer and
 * two values in E format with 16 significant digits (list-directed layout is the compiler's
 * choice).  Each call appends one line to `path`. */
int drd_write_fort23(const char* path, double t, const drd_diagnostics* d);
int drd_write_fort22(const char* path, int kcount, double dt, const drd_diagnostics* d);

/* ---- resident-state time stepping (the mcl6 step sequence on device) ------------------- */

/* Fields of the resident state; the same arrays mcl6 keeps (mcl6.f90:22-31, global.f90:42-47). */
#define DRD_F_U 0        /* UFACE */
#define DRD_F_V 1        /* VFACE */
#define DRD_F_U_PRE 2    /* UFACE */
#define DRD_F_V_PRE 3    /* VFACE */
#define DRD_F_PH 4       /* CELL  */
#define DRD_F_RMU 5      /* CELL  */
#define DRD_F_PH_PRE 6   /* CELL  */
#define DRD_F_RMU_PRE 7  /* CELL  */
#define DRD_F_P 8        /* CELL  */
#define DRD_F_PSI1 9     /* CELL  */
#define DRD_F_PSI2 10    /* CELL  */
#define DRD_F_PF1 11     /* CELL  particle_force1 */
#define DRD_F_PF2 12     /* CELL  particle_force2 */
#define DRD_F_COUNT 13

int drd_state_upload(drd_ctx* ctx, int field, const double* host);
int drd_state_download(drd_ctx* ctx, int field, double* host);
/* Device pointer of a resident field (for callers that keep data on the GPU). */
int drd_state_device_ptr(drd_ctx* ctx, int field, double** dptr);

typedef struct drd_step_stats {
    drd_status ch;   /* PhSolve or ph_mu_solve; .seconds = device time of its Krylov solve        */
    drd_status uv;   /* VeloSolve(_2)_combined; .seconds = device time of its Krylov solve        */
    drd_status pre;  /* PreSolve_2              */
    double mass;     /* sum(ph) dr dz after the step (FP64)  */
    double t;        /* time after the step     */
    double seconds;  /* device time of the whole step (CUDA events around the step's launch)     */
} drd_step_stats;

/* One pass of the mcl6 time loop body (microfluidics_complex_domain/mcl6.f90:378-486, the
 * first step :239-306 when `first` != 0): CH solve -> [particle coupling] -> momentum ->
 * swaps -> pressure -> p += psi2, on the resident state.  The particle coupling
 * (force_caculation_vel, update_position_vel, interpolate_coef) runs when drd_particles_set
 * made a chain resident; otherwise the coefficients stay as last set.
 * t is the time before the step; solves see t + dt as in the reference.  `stats` may be NULL;
 * when non-NULL the call waits for the step and fills it. */
int drd_step(drd_ctx* ctx, int first, double t, drd_step_stats* stats);
/* Enqueue `nsteps` steps without host synchronisation (stats are not collected). */
int drd_steps_async(drd_ctx* ctx, int first, double t, int nsteps);
int drd_synchronize(drd_ctx* ctx);

/* ---- input deck and checkpoint files --------------------------------------------------- */

/* The `input` deck that mcl6 reads line by line with list-directed READ
 * (microfluidics_complex_domain/mcl6.f90:68-99; the TP deck adds is_complex_domain,
 * two_phase_flow_complex_domain/mcl6.f90:100).  Only the first value of each line is read,
 * as list-directed input does; the rest of the line (the deck's '!' notes) is ignored. */
typedef struct drd_deck {
    double xld, re, ca, vs, xlsT, xlsB, xlsL, xlsR, uwT, uwB, slen, shig, angle, slipratio;
    int32_t iflag, istep;
    double tf, I_thickness, s_implicit, tol, ggz, ggx, time_step_change, lambda_rho, lambda_eta, UU;
    char lr_bd_type, top_type_ph, bot_type_ph, top_type_u, bot_type_u, is_complex_domain;
    char pad[2];
    int32_t entries;       /* values read: 31 for an MF deck, 32 for a TP deck */
    int32_t reserved;
} drd_deck;
/* Parses a deck file.  Returns DRD_OK, or DRD_ERR_BADARG with a message in `err` (may be NULL,
 * `err_len` bytes) when the file cannot be read or a value does not parse. */
int drd_read_deck(const char* path, drd_deck* deck, char* err, int err_len);
/* drd_params of an nr x nz grid from a deck, as finit and mcl6 derive them: dr = slen/nr,
 * dz = shig/nz (finit.f90:25-26), dt = min(dr,dz) * time_step_change (finit.f90:395-397),
 * twall = 0.1 (mcl6.f90:140), penalty_k = 1e5 (global.f90:91), bdr_low/upp = 0.1725/0.6725
 * (finit.f90:104-105); `variant` selects the application. */
int drd_params_from_deck(const drd_deck* deck, int nr, int nz, int variant, drd_params* params);

/* output(M,N,x,y,u,v,p,f,f2,t,fname) (microfluidics_complex_domain/inout.f90:1-19): a Fortran
 * unformatted sequential file (4-byte record markers) with the records
 * ((a(i,k),k=0,nz),i=0,nr) of x, y, u, v, p, f, f2 and the record t.  x and y are NODE shaped,
 * (nr+1)*(nz+1) doubles with element (i,k) at [i + k*(nr+1)] (the grids r(0:nr,0:nz),
 * z(0:nr,0:nz)); u UFACE, v VFACE, p, f, f2 CELL.  mcl6 writes fpd_ph as f and ph as f2
 * (mcl6.f90:352).  x or y NULL writes the cell-centre grid (i+0.5)dr, (k+0.5)dz. */
int drd_output(const char* path, int nr, int nz, double dr, double dz, const double* x, const double* y,
               const double* u, const double* v, const double* p, const double* f, const double* f2, double t);
/* input(M,N,x,y,u,v,p,f,t,fname) (inout.f90:41-60): reads the six field records and then t
 * from the NEXT record, which in a file written by output is f2's, so t receives f2(0,0) as
 * in the reference.  drd_read_time returns the true t of the last record instead.  Any array
 * may be NULL (skipped). */
int drd_input(const char* path, int nr, int nz, double* x, double* y, double* u, double* v, double* p, double* f,
              double* t);
int drd_read_time(const char* path, int nr, int nz, double* t);
/* output_particles (particles_move.f90:312-323): one record ((points(i,k),i=0,Np-1),k=0,1). */
int drd_output_particles(const char* path, int np, const double* points);
/* The output of the resident state: u, v, p, the context's fpd_ph (from the last
 * interpolate_coef or particle step) and ph, written as drd_output does.  The device copies
 * are ordered after the work already enqueued and before any later step, and the file is
 * written by a host thread while the GPU runs on; drd_checkpoint_wait joins it (and reports
 * its status).  One checkpoint may be in flight per context. */
int drd_checkpoint_async(drd_ctx* ctx, const char* path, double t);
int drd_checkpoint_wait(drd_ctx* ctx);

/* ---- pressure step without device allocation ------------------------------------------- */

/* Largest grid drd_presolve_2_noalloc accepts. */
#define DRD_NOALLOC_MAX_CELLS (512 * 256) /* nr * nz */
#define DRD_NOALLOC_MAX_LINE 1024         /* nr and nz each */

/* The pressure step of drd_presolve_2 for callers that cannot let the library call
 * cudaMalloc (an application whose device memory all belongs to its own pool allocator, or a
 * driver issuing the step from code where allocation is not allowed).  No context: u (UFACE),
 * v (VFACE) and psi (CELL) are device pointers owned by the caller, and the kernels run on
 * `stream` (a cudaStream_t, NULL for the default stream).  All intermediates live in one
 * fixed __device__ array of about 3.2 MB, held by every GPU that loads the library until the
 * process exits; grids beyond DRD_NOALLOC_MAX_* return DRD_ERR_TOO_LARGE.  Every call looks up
 * that array's device address in the current context (cudaGetSymbolAddress), so the call stays
 * valid after a cudaDeviceReset; the first call on a device loads the library's module and
 * should therefore come before any stream capture on that device.
 * Calls share the array: each call writes every intermediate before reading it, but calls that
 * overlap on the GPU race on it.
 * No counterpart in the reference (its PreSolve_2 allocates nothing on a device because it has
 * none). */
int drd_presolve_2_noalloc(int nr, int nz, double dr, double dz, const double* u, const double* v, double coef,
                           double* psi, void* stream);

/* ---- operator access (verification) ---------------------------------------------------- */

/* Operators of the three Krylov systems on packed vectors (the reference's Atob orders):
 *   DRD_OP_CH_MATVEC   MATRIX_VECTOR_CG (microfluidics_complex_domain/PhSolve.f90:240-292)
 *   DRD_OP_CH_PSOLVE   PSolve_CG -> DCT (PhSolve.f90:296-313, DCT.f90:1-57)
 *   DRD_OP_UV_MATVEC   MatrixVector_uv_2_CG / MatrixVector_uv_CG (bdf 2 / 1)
 *   DRD_OP_UV_PSOLVE   PSolve_uv_2_CG / PSolve_uv_CG Jacobi (identity for TP bdf 2)
 *   DRD_OP_PHMU_MATVEC MATRIX_VECTOR_PH_MU_CG (two_phase_flow_complex_domain/ph_mu_solve.f90:203-299)
 *   DRD_OP_PHMU_PSOLVE PSolve_PH_MU_CG (:304-380)
 * y = op(x) with the context's current coefficients, in FP64 (precision DRD_PREC_FP64) or
 * with the FP32 operators of the mixed mode (DRD_PREC_MIXED; x and y stay FP64 arrays). */
#define DRD_OP_CH_MATVEC 0
#define DRD_OP_CH_PSOLVE 1
#define DRD_OP_UV_MATVEC 2
#define DRD_OP_UV_PSOLVE 3
#define DRD_OP_PHMU_MATVEC 4
#define DRD_OP_PHMU_PSOLVE 5
/* `precision` DRD_OP_PERSISTENT evaluates the FP32 CH / momentum operators with the device code
 * of the persistent inner solver (one cooperative launch), for checking it against the others. */
#define DRD_OP_PERSISTENT 2
int drd_op_apply(drd_ctx* ctx, int op, int bdf, int precision, const double* x, double* y);
/* Length of the packed vector of operator `op`. */
long drd_op_length(drd_ctx* ctx, int op);

/* Systems of drd_solve. */
#define DRD_SYS_CH 0 /* the mu system of PhSolve (MATRIX_VECTOR_CG, PSolve_CG), MF variant      */
#define DRD_SYS_UV 1 /* the momentum system of VeloSolve_combined (bdf 1) / _2_combined (bdf 2) */

/* A x = b for one of the Krylov systems of the step, with the context's coefficients
 * (drd_set_coefs) and parameters: the BiCGSTAB solve of PhSolve.f90:62-74 or
 * VeloSolve_2_combined.f90:398-401 (tol, ch_maxit / uv_maxit, the precision mode, the mixed
 * mode's stiffness rule) on a caller's packed right-hand side.  x: the initial guess in, the
 * solution out; both of length drd_op_length of the system's operator.  For batches of
 * independent solves that do not come from a time step. */
int drd_solve(drd_ctx* ctx, int system, int bdf, const double* b, double* x, drd_status* st);

/* ---- batches of independent solves in one persistent launch --------------------------------
 *
 * Many independent systems of uneven grid sizes (no time step between them) are uploaded once
 * and solved by ONE persistent kernel launch, captured in a CUDA graph: each thread block takes
 * the next unsolved system from a device-side queue (largest first) and runs its whole
 * mixed-precision solve (FP64 iterative refinement around FP32 BiCGSTAB, the refinement policy
 * of the context solves: inner tolerance mixed_inner_tol, tenfold tighter after a sweep that
 * gains less than 10 %, FP64 true residual judged against tol, at most mixed_max_refine sweeps
 * and uv_maxit FP32 iterations per sweep).  Systems:
 *   DRD_SYS_UV        the momentum operator of VeloSolve_2_combined (bdf 2) / VeloSolve_combined
 *                     (bdf 1), MF variant, from rho, eta and the penalty mask bdr_ph, with the
 *                     Jacobi preconditioner of PSolve_uv_2_CG (VeloSolve_2_combined.f90:515-711)
 *   DRD_SYS_PRESSURE  a variable-coefficient pressure Poisson operator that the reference does
 *                     not have (its PreSolve_2 is a direct DCT solve): A psi = d/dx(beta dpsi/dx)
 *                     + d/dz(beta dpsi/dz) on the nr x nz cells, beta = 1/(1 + penalty_k dt
 *                     bdr_ph), face values the mean of the two cells, zero flux through the
 *                     domain faces; preconditioned by PreSolve_2's DCT solve (dct_fftw.f90:3-54:
 *                     REDFT10, / Pre_Lcc, REDFT01, / 4 nr nz), in FP32 by FFT.  The constant
 *                     field is its null space: b must sum to zero.
 * Packed vectors: DRD_SYS_UV the Atob_uv order (drd_op_length); DRD_SYS_PRESSURE nr*nz, i fastest.
 * Limits: nr, nz <= DRD_BATCH_MAX_LINE; pressure grids need nr and nz of the form 2^a 3^b 5^c 7^d. */
#define DRD_SYS_PRESSURE 2
#define DRD_BATCH_MAX_LINE 2048
typedef struct drd_batch_problem {
    int32_t system;     /* DRD_SYS_UV or DRD_SYS_PRESSURE                                           */
    int32_t bdf;        /* DRD_SYS_UV: 1 or 2                                                       */
    drd_params params;  /* nr, nz, dr, dz, dt, re, penalty_k, tol, mixed_inner_tol,
                           mixed_max_refine, uv_maxit; variant MF                                   */
    const double* rho;    /* CELL; DRD_SYS_UV only                                                  */
    const double* eta;    /* CELL; DRD_SYS_UV only                                                  */
    const double* bdr_ph; /* CELL: the penalty mask (DRD_SYS_UV) or the resistance giving beta     */
    const double* b;      /* packed right-hand side                                                  */
    const double* x0;     /* packed initial guess, NULL = zero                                       */
} drd_batch_problem;
typedef struct drd_batch drd_batch;
/* Uploads every system (coefficients in FP64 and FP32, right-hand sides, guesses) and builds the
 * FFT plans and tables; tunes the launch shape (threads per block, blocks per SM) by timing the
 * candidates on the batch itself when `autotune` is nonzero. */
int drd_batch_create(int nprob, const drd_batch_problem* probs, int autotune, drd_batch** out);
/* Solves every system from its x0 in one persistent launch (a captured graph) on the batch's
 * stream; *seconds receives the device time of the launch (CUDA events). */
int drd_batch_run(drd_batch* b, double* seconds);
/* Solution and status of system i after drd_batch_run (x: packed, may be NULL). */
int drd_batch_result(drd_batch* b, int i, double* x, drd_status* st);
/* Launch shape in use: threads per block, blocks per SM; algorithmic bytes of the last run. */
int drd_batch_info(drd_batch* b, int* threads, int* blocks_per_sm, double* bytes_last_run);
int drd_batch_destroy(drd_batch* b);
const char* drd_batch_last_error(drd_batch* b);
/* Packed length of a batch system. */
long drd_batch_length(int system, int nr, int nz);

/* ---- learned initial guess ---------------------------------------------------------------
 * A 4-level U-Net (channels 32/64/128/256, 3x3 convolutions with ReLU, 2x2 average pooling,
 * nearest upsampling, concatenated skips, a 1x1 output convolution) in BF16 weights and
 * activations with FP32 accumulation, run and trained by the library's own tensor-core
 * kernels.  It maps in_ch input fields on an H x W grid (for the CH system: the residual of
 * the plain guess divided by its RMS, the resistance bdr_ph and the phase field, each as the
 * packed nr x nz interior, H = nz rows of W = nr) to out_ch fields (the correction of the
 * guess in the same units).  No counterpart exists in the reference: this is the learned
 * guess its solves (PhSolve.f90:62-74, VeloSolve_2_combined.f90:388-407) can start from, with
 * the plain guess as the fallback that the FP64 true residual judges.
 *
 * Arrays are FP32, (batch, channels, H, W) C order, in host or device memory.  Parameters are
 * one FP32 vector of drd_unet_param_count floats: per 3x3 layer the weights [tap][Cout][Cin]
 * then the bias, the 17 layers in the order enc0a enc0b enc1a enc1b enc2a enc2b enc3a enc3b,
 * then per decoder level 2, 1, 0: upconv, conv(concat), conv; then the output layer's
 * weights [out_ch][32] and bias.  The first layer's Cin is 16 (inputs zero-padded). */
typedef struct drd_unet drd_unet;
int drd_unet_create(int H, int W, int in_ch, int out_ch, int max_batch, uint64_t seed, drd_unet** net);
int drd_unet_destroy(drd_unet* net);
int64_t drd_unet_param_count(drd_unet* net);
const char* drd_unet_last_error(drd_unet* net);
int drd_unet_get_params(drd_unet* net, float* params);
/* Sets the parameters and resets the Adam state. */
int drd_unet_set_params(drd_unet* net, const float* params);
int drd_unet_forward(drd_unet* net, int batch, const float* x, float* y);
/* Mean squared error of forward(x) against target over the H x W grid, and its gradient
 * with respect to every parameter (no update).  loss / grads may be NULL. */
int drd_unet_gradients(drd_unet* net, int batch, const float* x, const float* target, float* loss, float* grads);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) at learning rate lr on that loss. */
int drd_unet_train_step(drd_unet* net, int batch, const float* x, const float* target, float lr, float* loss);
/* The network's CUDA stream (cudaStream_t). */
int drd_unet_stream(drd_unet* net, void** stream);

/* ---- performance instrumentation ------------------------------------------------------- */

/* Kernels that drd_kernel_bench can time in isolation on the context's current data. */
#define DRD_KB_UV_MATVEC_FP64 0   /* MatrixVector_uv_2_CG stencil, FP64                    */
#define DRD_KB_UV_MATVEC_FP32 1   /* the same in FP32 (mixed mode inner solves)            */
#define DRD_KB_DCT_X_FP64 2       /* one x-axis DCT-I pass of PSolve_CG (GEMM form), FP64  */
#define DRD_KB_DCT_X_FP32 3       /* the same in FP32                                       */
#define DRD_KB_DCT_Z_FP64 4       /* one z-axis DCT-I pass, FP64                            */
#define DRD_KB_DCT_Z_FP32 5       /* the same in FP32                                       */
#define DRD_KB_CH_MATVEC_FP32 6   /* MATRIX_VECTOR_CG second stencil pass, FP32             */
#define DRD_KB_PRESSURE_FFT64 7   /* PreSolve_2 by FFT, FP64: u, v -> psi (three passes)     */
#define DRD_KB_DCT2_FFT32 8       /* REDFT10, / Pre_Lcc, REDFT01 of an nr x nz FP32 field    */
#define DRD_KB_COUNT 9
/* DRD_KB_PRESSURE_FFT64 and DRD_KB_DCT2_FFT32 write 512 MiB of scratch before every launch (L2
 * cold, the inputs come from HBM) and report the mean of the per-launch event times; they need
 * nr and nz of the form 2^a 3^b 5^c 7^d (DRD_ERR_UNSUPPORTED otherwise). */
/* Launches kernel `which` `reps` times back to back (one captured graph) between CUDA events
 * on the context stream.  Returns the average device time per launch and the algorithmic
 * bytes and flops one launch moves / performs (compulsory inputs and outputs only). */
int drd_kernel_bench(drd_ctx* ctx, int which, int reps, double* us_per_launch, double* bytes_per_launch,
                     double* flops_per_launch);
/* Writes `bytes` of scratch memory on the context stream (evicts L2 between timed steps). */
int drd_flush_l2(drd_ctx* ctx, int64_t bytes);

/* Page-locks and maps `bytes` of the caller's host memory at p (cudaHostRegister, mapped) and
 * records the range with its device address: the per-routine calls then move every array
 * argument that lies in a recorded range in one gather launch in and one scatter launch out
 * through the mapped addresses (other arrays, including memory page-locked by other means:
 * cudaMemcpyAsync); a driver that registers its module arrays once after allocating them makes
 * every later call's copies faster.  Unregister (which drops the record) before freeing. */
int drd_host_register(void* p, int64_t bytes);
int drd_host_unregister(void* p);

/* 1 when the mixed mode runs each whole CH and momentum solve (the FP64 refinement and its
 * FP32 iterations) as one persistent cooperative launch with grid-wide barriers between the
 * phases of an iteration; 0 when it runs the captured kernel-per-phase loop (no cooperative
 * launch support, DRD_PERSIST=0 in the environment, or a graph that could not take the
 * cooperative launch).  `why` receives the reason for whatever does not use it, including a
 * grid past the CH solve's resident shared-memory plan, or past the resident row-transform
 * panels of the momentum solve with ESOLP_x, whose solve then uses the loop. */
int drd_persistent_solver(drd_ctx* ctx, char* why, int len);
/* With DRD_PERSIST_PROF=1 in the environment at drd_create, the persistent solver records
 * %globaltimer (ns) at entry and exit of each grid barrier of its third iteration, as seen by
 * block 0: ns[2k], ns[2k+1] for barrier k (up to 62 barriers; zero where none ran).  Returns
 * the number of entries copied. */
int drd_persist_profile(drd_ctx* ctx, int64_t* ns, int n);
/* Failure detection of the persistent solver's grid barrier, without a fault: two blocks run
 * the barrier; with absent = 1 the second block never arrives, and the first gives up after
 * its bounded wait (a few seconds) and reports DRD_ERR_TIMEOUT in *status, as the solver
 * would.  With absent = -1 both arrive and *status is 0.  The context stays usable. */
int drd_barrier_selftest(drd_ctx* ctx, int absent, int* status);

/* Number of kernels this library has launched on the context (graph nodes counted per
 * execution), cumulative. */
int64_t drd_kernel_launches(drd_ctx* ctx);
/* Raw CUDA stream of the context (cudaStream_t), for callers timing with events. */
void* drd_stream(drd_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* DRD_GB300_H */
