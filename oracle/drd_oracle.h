/*
 * drd_oracle.h — FP64 CPU restatement of the DRD-Micro per-time-step solver core.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline legs may load this library; the product path never does.
 *
 * Parity status: the reference (Fortran + prebuilt FFTW + MKL) cannot be compiled here or
 * on the GPU host, and it ships no tests or reference outputs for these routines, so this
 * restatement is "parity unpinned" against reference-run outputs.  It is pinned instead
 * against (1) scipy.fft's DCT-I/II/III, which define vfftpack VCOST and FFTW
 * REDFT10/REDFT01, (2) the manufactured Poisson case the reference keeps in
 * microfluidics_complex_domain/PreSolve_2.f90:32-67, and (3) operator identities
 * (symmetry, Neumann null spaces, round trips) checked in tests/.
 *
 * Layouts are the Fortran ones documented in include/drd_gb300.h (CELL, UFACE, VFACE).
 */
#ifndef DRD_ORACLE_H
#define DRD_ORACLE_H

#include "../include/drd_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Tables of setup() (microfluidics_complex_domain/setup.f90:106-155).
 * ph_lcc: nr*nz (i fastest), pre_lcc: (nr+1)*(nz+1) (i fastest). */
void orc_setup_tables(const drd_params* P, double* ph_lcc, double* pre_lcc);

/* Transforms on `m` sequences of length n; sequence s element j at x[s*seq_stride + j*elem_stride]. */
void orc_vcost(int n, int m, double* x, long seq_stride, long elem_stride);   /* lib/vfftpack.f:643-704 */
void orc_redft10(int n, int m, double* x, long seq_stride, long elem_stride); /* FFTW REDFT10 */
void orc_redft01(int n, int m, double* x, long seq_stride, long elem_stride); /* FFTW REDFT01 */

/* op_double_gradient_Neum (microfluidics_complex_domain/matrix_tool.f90:178-219) on CELL arrays. */
void orc_op_double_gradient_neum(int nr, int nz, double dr2, double dz2, const double* x,
                                 const double* mo, double* out);

/* Operators of the CH system on packed vectors of length nr*nz (Atob order). */
void orc_ch_matvec(const drd_params* P, const double* M0, const double* Mi, double alpha,
                   const double* x, double beta, double* y);              /* PhSolve.f90:240-292 */
void orc_ch_psolve(const drd_params* P, const double* ph_lcc, const double* x, double* y); /* :296-313 */
/* The solid-blended CH preconditioner y = q + w (x - q), q = PSolve_CG(x), its probe fit and
 * BiCGSTAB with it (an extension; no reference counterpart). */
void orc_ch_psolve_blend(const drd_params* P, const double* ph_lcc, const double* w, const double* x, double* y);
double orc_probe_sign(uint64_t seed, long probe, long n, long q);
void orc_ch_blend_probe(const drd_params* P, const double* ph_lcc, const double* M0, const double* Mi, int nprobe,
                        uint64_t seed, double* w);
int orc_ch_solve_blend(const drd_params* P, const double* ph_lcc, const double* M0, const double* Mi, const double* w,
                       const double* b, double* x, drd_status* st);

/* Operators of the momentum system on packed vectors of length (nr+1)nz + nr(nz-1). */
void orc_uv_matvec(const drd_params* P, int bdf, const double* rho, const double* eta,
                   const double* bdr_pen, double alpha, const double* x, double beta, double* y);
void orc_uv_psolve(const drd_params* P, int bdf, const double* rho, const double* eta,
                   const double* x, double* y);

/* Coupled [phi; mu] operators (two_phase_flow_complex_domain/ph_mu_solve.f90:203-380). */
void orc_phmu_matvec(const drd_params* P, const double* M0, const double* Mi, const double* bdr_used,
                     double coef_bot, double coef_top, double alpha, const double* x, double beta,
                     double* y);
void orc_phmu_psolve(const drd_params* P, const double* x, double* y);

/* RHS builders of the three Krylov systems (packed rhs and initial guess). */
void orc_ch_system(const drd_params* P, const double* u, const double* v, const double* ph, const double* rmu,
                   const double* bdr_ph, const double* bdr_ph_grad, const double* Mi, double* f2, double* rhs,
                   double* x0);
void orc_phmu_system(const drd_params* P, const double* u, const double* v, const double* ph, const double* rmu,
                     const double* bdr_ph, const double* bdr_ph_used, const double* bdr_ph_grad, const double* angleB,
                     const double* angleT, double* M0, double* rhs, double* x0, double* pnb, double* pnt,
                     double* coef_bot_top);

/* BiCGSTAB of lib/BiCGSTAB.f + lib/BiCGSTABREVCOM.f + lib/STOPTEST2.f. */
typedef void (*orc_matvec_fn)(void* ctx, double alpha, const double* x, double beta, double* y);
typedef void (*orc_psolve_fn)(void* ctx, const double* x, double* y);
int orc_bicgstab(long n, const double* b, double* x, int maxit, double tol, orc_matvec_fn mv,
                 orc_psolve_fn ps, void* ctx, drd_status* st);

/* The per-step routines.  All arrays are Fortran-shaped; see include/drd_gb300.h. */
int orc_phsolve(const drd_params* P, const double* ph_lcc, const double* u, const double* v,
                const double* ph, const double* rmu, const double* bdr_ph, const double* bdr_ph_grad,
                const double* M0, const double* Mi, double* rmu_after, double* ph_after, drd_status* st);

int orc_ph_mu_solve(const drd_params* P, const double* u, const double* v, const double* ph,
                    const double* rmu, const double* bdr_ph, const double* bdr_ph_used,
                    const double* bdr_ph_grad, const double* Mi, const double* angleB,
                    const double* angleT, double* M0_out, double* ph_after, double* rmu_after,
                    double* coef_bot_top, drd_status* st);

/* bdf = 1: VeloSolve_combined; bdf = 2: VeloSolve_2_combined. */
int orc_velosolve(const drd_params* P, int bdf, const double* psi1, const double* psi2,
                  const double* u_pre, const double* u, const double* v_pre, const double* v,
                  const double* p, const double* rho, const double* eta, const double* bdr_ph,
                  const double* bdr_pen, const double* bdr_used, const double* ph_after,
                  const double* rmu_after, double t, const double* pf1, const double* pf2,
                  double* u_after, double* v_after, double* uL, double* uR, drd_status* st);

void orc_presolve(const drd_params* P, const double* pre_lcc, const double* u, const double* v,
                  double coef, double* psi);

void orc_interpolate_coef(const drd_params* P, const double* dist, const double* bdr_ph,
                          double* fpd_ph, double* rho, double* eta);

int orc_reinint_by_phsolve(const drd_params* P, const double* ph_lcc, const double* bdr_in, double* bdr_out,
                           double* pen_out);
void orc_dissipation(const drd_params* P, const double* u, const double* v, const double* ph, const double* rmu,
                     const double* angB, const double* angT, double vs, double* out);
void orc_pressure_matvec(const drd_params* P, const double* bdr_ph, const double* x, double* y);
void orc_pressure_psolve(const drd_params* P, const double* pre_lcc, const double* x, double* y);
int orc_pressure_solve(const drd_params* P, const double* pre_lcc, const double* bdr_ph, const double* b, double* x,
                       drd_status* st);
void orc_two_phase_coef(const drd_params* P, const double* fpd_ph, const double* ph, double* rho, double* eta);
double orc_mass(const drd_params* P, const double* ph);

/* ESOLP_x momentum preconditioner (microfluidics_complex_domain/ESOLP.f90, setup.f90:157-235). */
void orc_esolp_coefs(const drd_params* P, int bdf, double* ua, double* ub, double* uc, double* va, double* vb,
                     double* vc);
void orc_uv_psolve_esolp(const drd_params* P, int bdf, const double* x, double* y);
/* DRD_UV_ESOLP_SCALED (an extension): s = sqrt(D0 / D) and y = s ESOLP_x(s x). */
void orc_uv_esolp_scale(const drd_params* P, int bdf, const double* rho, const double* eta, double* s);
void orc_uv_psolve_esolp_scaled(const drd_params* P, int bdf, const double* s, const double* x, double* y);

/* A x = b for system 0 (CH mu) or 1 (momentum, bdf 1/2) with the reference BiCGSTAB. */
int orc_solve_system(const drd_params* P, int system, int bdf, const double* ph_lcc, const double* M0,
                     const double* Mi, const double* rho, const double* eta, const double* pen, const double* b,
                     double* x, drd_status* st);

/* PhSolve_ori and finit's wall smoothing (microfluidics_complex_domain/PhSolve_ori.f90,
 * finit.f90:120-189).  angleB/angleT may be NULL (zeros, as during finit's loop). */
double orc_ori_coef(const drd_params* P, double alpha_s);
void orc_ori_matvec(const drd_params* P, double coef_bot, double coef_top, double alpha, const double* x,
                    double beta, double* y);
void orc_ori_system(const drd_params* P, const double* u, const double* v, const double* ph, const double* angleB,
                    const double* angleT, double alpha_s, double* f2, double* rhs, double* x0, double* pnb,
                    double* pnt);
int orc_phsolve_ori(const drd_params* P, const double* ph_lcc, const double* u, const double* v, const double* ph,
                    const double* angleB, const double* angleT, double alpha_s, double* rmu_after, double* ph_after,
                    drd_status* st);
int orc_finit_wall(const drd_params* P, const double* ph_lcc, const double* bdr_in, int nsteps, double* bdr_out,
                   double* ph_out, double* rmu_out);

/* Fiber particles (microfluidics_complex_domain/particles_move.f90; POINTS arrays as in
 * include/drd_gb300.h).  drd_particle_params_default and drd_particle_initialize are also
 * defined here with the library's signatures, so the oracle can set up a chain by itself. */
void orc_particle_forces(const drd_params* P, const drd_particle_params* pp, const double* points,
                         const double* bdr_dist, double* tot_F);                      /* :421-627 */
void orc_force_caculation_vel(const drd_params* P, const drd_particle_params* pp, const double* points,
                              const double* bdr_dist, double* tot_F, double* pf1, double* pf2); /* :758-868 */
void orc_update_position_vel(const drd_params* P, const drd_particle_params* pp, double* points,
                             const double* u, const double* v, double dt);            /* :872-980 */
void orc_fpd_dist_field(const drd_params* P, const drd_particle_params* pp, const double* points,
                        double* dist);                                                /* :361-391 */
typedef struct orc_particles {
    drd_particle_params pp;
    double* points;          /* POINTS, moved by each step */
    double* tot_F;           /* POINTS, written */
    const double* bdr_dist;  /* CELL */
    double* fpd_ph;          /* CELL, written */
    double* rho;             /* CELL, written; the step's momentum solve uses these */
    double* eta;             /* CELL, written */
} orc_particles;
void orc_particles_step(const drd_params* P, orc_particles* X, const double* u, const double* v,
                        const double* bdr_ph, double* pf1, double* pf2);

/* The mcl6 loop body on a state held by the caller (same field order as DRD_F_*); coefficient
 * arrays as in orc_velosolve.  Returns the CH status in st[0], momentum in st[1]. */
typedef struct orc_state {
    double* f[DRD_F_COUNT];
    const double* rho;
    const double* eta;
    const double* bdr_ph;
    const double* bdr_ph_grad;
    double* M0; /* ph_mu_solve rewrites it (two_phase_flow_complex_domain/ph_mu_solve.f90:31-35) */
    const double* Mi;
    const double* bdr_pen;
    const double* bdr_used;
    orc_particles* parts;   /* NULL: particles held fixed; else the coupling of mcl6.f90:394-402 */
    const double* fpd_ph;   /* indicator of interpolate_coef for params.two_fluid (NULL: bdr_ph)  */
} orc_state;
int orc_step(const drd_params* P, const double* ph_lcc, const double* pre_lcc, orc_state* S,
             int first, double t, drd_status* st2);

#ifdef __cplusplus
}
#endif
#endif
