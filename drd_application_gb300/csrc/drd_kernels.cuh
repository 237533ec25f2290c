// drd_kernels.cuh — host launchers of the solver-core kernels (defined in drd_kernels.cu).
#pragma once

#include "drd_common.cuh"
#include "drd_fft.cuh"

namespace drd {

typedef unsigned long long ull;

// Gate of a kernel on the Krylov state: always run, run while the solve is running, or run
// while running and the initial guess is nonzero (the ||x0|| != 0 branch of
// lib/BiCGSTABREVCOM.f:230).
enum Gate : int { G_ALWAYS = 0, G_RUNNING = 1, G_XNZ = 2, G_EARLY_OR_RUNNING = 3 };

// Scalars of the operators in the precision T of the Krylov vectors.
template <typename T>
struct OpScal {
    T dt, xld, eps, s, idr2, idz2, dtxld, re, pk, dr, dz, dr2, dz2, adjust;
    T idrdz;   // 1 / (dr dz): the FP32 momentum operator multiplies where FP64 divides
    T cb, ct;  // ph_mu_solve coef_bot / coef_top
    int nr, nz, variant, lr_neumann, bdf, phi_mode;
};

struct Dots {
    double* part;      // partials buffer, slot s at part + s*DRD_MAXB
    int G;             // blocks of the reduction grid
};

// ---- transforms (GEMM form) -----------------------------------------------------------
enum Epi : int { EPI_STORE = 0, EPI_DIV_TAB = 1, EPI_PRE_FINAL = 2, EPI_SCALE = 3 };
template <typename T>
struct GemmArgs {
    int M, N, K;
    const T* A; long lda;   // row-major M x K
    const T* B; long ldb;   // row-major K x N
    T* C; long ldc;         // row-major M x N (EPI_PRE_FINAL: CELL field, ldc ignored)
    const T* tab; long ldt; // EPI_DIV_TAB: C = acc / tab[m*ldt + n]
    const CallArgs* ca;     // EPI_PRE_FINAL: coef
    double scale;           // EPI_PRE_FINAL: divisor 4 nr nz; EPI_SCALE: multiplier
    int nr;
    const KState* ks; int gate;
    ull* ctr;
    // DCT-I even/odd folding (C[o][L-j] = (-1)^o C[o][j]): the output parity is blockIdx.z
    // (split-K: blockIdx.z / KS).  FOLD_A: A is the data X (lda), loaded as X[m][j] +- X[m][L-j],
    // B / B_odd the even / odd-column matrices, N / N_odd their widths, output column 2n+p.
    // FOLD_B: B is the data, loaded as X[j][n] +- X[L-j][n], A / A_odd the even / odd-row
    // matrices, M / M_odd their heights, output row 2m+p.  K is floor(L/2)+1.
    int fold; int Lf;
    const T* A_odd; const T* B_odd; int M_odd, N_odd;
    int* err;  // the tensor-core GEMM: set when a wait gave up (may be null)
    // the tensor-core GEMM: the constant operand (B of FOLD_A, A of FOLD_B) pre-split into TF32
    // high and low parts and laid out as the CTA's 32 KB shared-memory blocks (gemm_tc_pack),
    // brought in by one bulk copy per K chunk; null: staged by the threads like the data
    const float* packed;
    int pk_tiles, pk_chunks;
    // the tensor-core GEMM, FOLD_A with rows TMA cannot address (a row stride or row length not a
    // multiple of 16 bytes): scratch of pad_cap floats for the folded even and odd operands, laid
    // out for TMA by a pre-pass (null: the register-staged kernel runs)
    float* pad;
    long pad_cap;
};
// Packs the constant operand of a folded transform for k_gemm_tc: rows r (its N for FOLD_A, its
// M for FOLD_B) of the even and odd matrices, K values each; b_style: the matrices are K x rows
// (B of FOLD_A, row stride ld), else rows x K (A of FOLD_B).  Returns the floats written, or the
// floats needed when out is null; *tiles and *chunks receive the 128-row tiles and 32-K chunks of
// the layout.
long gemm_tc_pack(const float* even, const float* odd, int rows_e, int rows_o, int K, long ld, int b_style,
                  float* out, int* tiles, int* chunks, cudaStream_t s);
enum Fold : int { FOLD_NONE = 0, FOLD_A = 1, FOLD_B = 2 };
int gemm_config_count(int fp64);
// FP32 transform GEMM configuration that runs on the tensor cores (3xTF32 tcgen05); the FP32
// autotuner times it beside the SIMT configurations [0, gemm_config_count(0)).
constexpr int kGemmTcCfg = 14;
const char* gemm_config_name(int cfg);
template <typename T>
void launch_gemm(int cfg, int epi, const GemmArgs<T>& a, cudaStream_t s);

// ---- CH (microfluidics_complex_domain/PhSolve.f90) -------------------------------------
void launch_ch_f2(const DevParams& P, const double* u, const double* v, const double* ph, double* f2, ull* ctr, cudaStream_t s);
void launch_ch_rhs(const DevParams& P, const double* ph, const double* rmu, const double* rmu_pre,
                   const double* rmu_pre2, const double* rmu_pre3, const double* bdr, const double* grad,
                   const double* Mi, const double* f2, double* b, double* x, ull* ctr, cudaStream_t s);
template <typename T>
void launch_ch_matvec(const OpScal<T>& o, const T* M0, const T* Mi, T alpha, const T* x, T beta, T* y, T* ff1,
                      const T* dot1, int self2, const Dots& d, int slot1, const KState* ks, int gate, ull* ctr,
                      cudaStream_t s);
void launch_ch_fin(const DevParams& P, const double* x, const double* f2, const double* M0, double* rmu_after,
                   double* ph_after, ull* ctr, cudaStream_t s);

// ---- ESOLP_x tridiagonal stage (microfluidics_complex_domain/ESOLP.f90) --------------------
// One block of an ESOLP_x momentum vector: `rows` rows of `len` values, row j mode k at
// w[k + len*j]; the precomputed Thomas factors (multiplier, pivot, super-diagonal) likewise.
template <typename T>
struct TriBlock {
    int len, rows;
    const T *rm, *bp, *cc;
    T* w;
};
template <typename T>
void launch_tridiag(const TriBlock<T>& b0, const TriBlock<T>& b1, const KState* ks, int gate, ull* ctr, cudaStream_t s);

// ---- PhSolve_ori (microfluidics_complex_domain/PhSolve_ori.f90), finit's wall smoothing ---
void launch_ori_rhs(const DevParams& P, const double* ph, const double* f2, const double* cfb, const double* cft,
                    double alpha_s, double* b, double* x, double* pnb, double* pnt, ull* ctr, cudaStream_t s);
template <typename T>
void launch_ori_matvec(const OpScal<T>& o, T alpha, const T* x, T beta, T* y, T* ff1, const T* dot1, int self2,
                       const Dots& d, int slot1, const KState* ks, int gate, ull* ctr, cudaStream_t s);
void launch_ori_fin(const DevParams& P, const double* x, const double* pnb, const double* pnt, double cb, double ct,
                    double* ph_after, double* rmu_after, ull* ctr, cudaStream_t s);
void launch_ori_rmu0(const DevParams& P, const double* ph, double* rmu, ull* ctr, cudaStream_t s);
void launch_ori_bdr(int nr, int nz, const double* ph, double* bdr, ull* ctr, cudaStream_t s);

// ---- coupled CH (two_phase_flow_complex_domain/ph_mu_solve.f90) -----------------------
void launch_phmu_prep(const DevParams& P, const double* u, const double* v, const double* ph, const double* bdr,
                      const double* used, double* M0, double* f2, ull* ctr, cudaStream_t s);
void launch_phmu_rhs(const DevParams& P, const double* ph, const double* rmu, const double* ph_pre,
                     const double* rmu_pre, const double* bdr, const double* grad, const double* f2, const double* cfB,
                     const double* cfT, double* b, double* x, double* pnb, double* pnt, ull* ctr, cudaStream_t s);
template <typename T>
void launch_phmu_matvec(const OpScal<T>& o, const T* M0, const T* Mi, const T* used, T alpha, const T* x, T beta, T* y,
                        const T* dot1, int self2, const Dots& d, int slot1, const KState* ks, int gate, ull* ctr,
                        cudaStream_t s);
template <typename T>
void launch_phmu_diag(const OpScal<T>& o, T* diag, ull* ctr, cudaStream_t s);
void launch_phmu_fin(const DevParams& P, const double* x, const double* pnb, const double* pnt, double cb, double ct,
                     double* ph_after, double* rmu_after, ull* ctr, cudaStream_t s);

// ---- momentum (microfluidics_complex_domain/VeloSolve_2_combined.f90) -----------------
void launch_uv_rhs(const DevParams& P, int bdf, const CallArgs* ca, const double* psi1, const double* psi2,
                   const double* u_pre, const double* u, const double* v_pre, const double* v, const double* p,
                   const double* rho, const double* eta, const double* bdr, const double* used, const double* ph_after,
                   const double* rmu_after, const double* pf1, const double* pf2, double* b, double* x, double* uL,
                   int extrap, const double* u_pre2, const double* v_pre2,
                   const double* u_pre3, const double* v_pre3, ull* ctr, cudaStream_t s);
template <typename T>
void launch_uv_matvec(const OpScal<T>& o, const T* rho, const T* eta, const T* pen, T alpha, const T* x, T beta, T* y,
                      const T* dot1, int self2, const Dots& d, int slot1, const KState* ks, int gate, ull* ctr,
                      cudaStream_t s);
template <typename T>
void launch_uv_diag(const OpScal<T>& o, const T* rho, const T* eta, T* diag, ull* ctr, cudaStream_t s);
void launch_uv_fin(const DevParams& P, const double* x, const double* uL, double* u_after, double* v_after, ull* ctr,
                   cudaStream_t s);

// ---- pressure (microfluidics_complex_domain/PreSolve_2.f90) -----------------------------
void launch_pre_div(const DevParams& P, const double* u, const double* v, double* w, ull* ctr, cudaStream_t s);
void launch_fill_neumann(int nr, int nz, double* a, double* b, ull* ctr, cudaStream_t s);
void launch_cell_add(long n, const double* x, double* y, ull* ctr, cudaStream_t s);  // y = x + y

// ---- interpolate_coef / mass ----------------------------------------------------------
void launch_interp_coef(const DevParams& P, const double* dist, const double* bdr, double* fpd, double* rho, double* eta,
                        ull* ctr, cudaStream_t s);
// dissipation() diagnostics (microfluidics_complex_domain/dissipation.f90): out[6] = e1, e2, e3,
// e4, dissip, mass; uses partial slots 0-3.
struct DissipArgs {
    int nr, nz;
    double dr, dz, xld, ca, eps, vs, angle;
};
void launch_dissipation(const DissipArgs& a, const double* u, const double* v, const double* ph, const double* rmu,
                        const double* angB, const double* angT, const Dots& d, double* out, ull* ctr, cudaStream_t s);
// PreSolve_2 by FFT (drd_pressure_fft.cu): plans for lengths of the form 2^a 3^b 5^c 7^d;
// whether a grid fits the passes' shared memory with reals of `real_bytes`; the kernels'
// shared-memory opt-in (once per context, outside stream capture); the FP64 step (u, v -> psi
// interior, * ca->coef) and the FP32 2-D pair on plain arrays.
bool pfft_plan(int n, FftPlan& pl);
bool pfft_fits(int nr, int nz, int real_bytes);
cudaError_t pfft_prepare(int nr, int nz);
cudaError_t launch_pressure_fft(int nr, int nz, double dr, double dz, const FftPlan& px, const FftPlan& pz,
                                const void* twx, const void* twz, const double* u, const double* v, double* T,
                                const double* pre_lcc, double* psi, const CallArgs* ca, ull* ctr, cudaStream_t s);
cudaError_t launch_pressure_fft32(int nr, int nz, const FftPlan& px, const FftPlan& pz, const void* twx,
                                  const void* twz, const float* x, float* T, const float* lcc, float* out, ull* ctr,
                                  cudaStream_t s);
void launch_threshold(long n, const double* x, double t, double* y, ull* ctr, cudaStream_t s);  // y = x > t
void launch_two_phase_coef(const DevParams& P, long cs, const double* fpd, const double* ph, double* rho, double* eta,
                           float* rho32, float* eta32, ull* ctr, cudaStream_t s);

// Up to kHostCopyMax copies of FP64 arrays in one launch, each src[i] -> dst[i] of len[i] values
// (one row of blocks per copy).  The per-routine calls use it for the caller's page-locked host
// arrays, read or written through their mapped device addresses over the host link, in place of
// one DMA copy per array.
constexpr int kHostCopyMax = 16;
struct HostCopies {
    int n;
    const double* src[kHostCopyMax];
    double* dst[kHostCopyMax];
    long len[kHostCopyMax];
};
void launch_host_copies(const HostCopies& h, ull* ctr, cudaStream_t s);

// ---- persistent cooperative BiCGSTAB (FP32 inner solves of the CH and momentum systems) ---
struct GridBar {
    unsigned count, gen;
    int err, pad;
};
enum PersistKind : int { PK_CH = 0, PK_UV = 1 };
enum PersistMode : int { PM_SOLVE = 0, PM_PSOLVE = 1, PM_MATVEC = 2, PM_REFINE = 3 };
struct PersistArgs {
    int kind;                             // PK_CH or PK_UV
    int mode;                             // PM_SOLVE, or one application x = op(b)
    int nr, nz;
    long n;                               // unknowns
    OpScal<float> o;
    // CH: mobilities (CELL), packed Ph_Lcc, folded DCT-I operands
    const float *M0, *Mi, *lcc;
    const float* pcw;  // solid-blend weights of the CH preconditioner (packed), or null
    const float *fxe, *fxo, *fze, *fzo;
    int Kx, Nxe, Nxo, Kz, Mze, Mzo;
    // momentum: rho, eta, penalty mask (CELL), Jacobi diagonal; ident = identity preconditioner
    const float *rho, *eta, *pen, *diag;
    int ident;
    // momentum with ESOLP_x: the folded VCOST operands of length nr+1 (u block, Ku x Nue; the v
    // block uses the CH x-pass operands of length nr), the Thomas factors of the bdf (u block
    // rm, bp, cc, then the v block), the tridiagonal phase's modes per batch
    int esolp;  // 1: ESOLP_x, 2: ESOLP_x between the diagonal scalings held in diag
    const float *fue, *fuo, *esf;
    int Ku, Nue, Nuo;
    float *x, *b, *r, *rtld, *p, *v, *phat, *shat, *t, *ff1, *w1, *w2;
    // PM_REFINE: the FP64 system (b64, x64 in place), its residual and stencil scratch, the
    // FP64 operators' scalars and coefficients, the refinement tolerance and sweep limit
    const double* b64;
    double *x64, *r64, *f64;
    OpScal<double> od;
    const double *M0d, *Mid, *rhod, *etad, *pend;
    double outer_tol;
    int max_refine;
    double* part;
    KState* ks;
    const KState* parent;
    GridBar* bar;
    double tol;
    int maxit;
    ull* ctr;
    unsigned long long* prof;  // optional: barrier entry/exit times (ns) of block 0 in iteration 3
    // CH shared-memory plan (floats): work area, resident z operands, resident x-pass B panel
    long work_off, z_off, b_off;
    int z_res, b_res;
    size_t smem_bytes;
};
struct PbPlan {
    long work_off, z_off, b_off;
    int z_res, b_res;
    size_t bytes;
};
PbPlan persist_ch_plan(int nr, int nz, int grid, size_t budget);
PbPlan persist_esolp_plan(int nr, int nz, int grid, size_t budget);
int persist_threads();
const void* persist_kernel(int kind);
cudaError_t launch_bicg_persist(const PersistArgs& a, int grid, cudaStream_t s);
void launch_bar_reset(GridBar* b, ull* ctr, cudaStream_t s);
void launch_stamp(KState* ks, int end, ull* ctr, cudaStream_t s);
void launch_bar_selftest(GridBar* bar, int absent, int* out, ull* ctr, cudaStream_t s);

// ---- fiber particles (microfluidics_complex_domain/particles_move.f90), drd_particles.cu --
constexpr int PT_GX = 64;  // blocks per bead in the per-bead sums
struct PartParams {
    int np, nr, nz, pad;
    double lx, ly, radius, l0, ks, kb, theta0, k0, k0b, eq_pp, eq_bdr;
    double dr, dz, eps, dt, lambda_rho, lambda_eta;
    double skip_d2;  // (radius + 20 sqrt(2) eps)^2: beyond it the bead indicator is < 4.3e-18
};
void launch_pt_force(const PartParams& Q, double* pts, double* pts_old, double* totF, const double* bdist, ull* ctr,
                     cudaStream_t s);
void launch_pt_sums(const PartParams& Q, const double* pts, const double* u, const double* v, double* part, ull* ctr,
                    cudaStream_t s);
void launch_pt_finish(const PartParams& Q, const double* part, double* psum, double* pts, int move, ull* ctr,
                      cudaStream_t s);
void launch_pt_spread(const PartParams& Q, int mode, const double* pts_old, const double* pts, const double* totF,
                      const double* psum, const double* bdr, double* pf1, double* pf2, double* fpd, double* rho,
                      double* eta, float* rho32, float* eta32, ull* ctr, cudaStream_t s);
void launch_mass_partial(int nr, int nz, const double* ph, const Dots& d, int slot, ull* ctr, cudaStream_t s);
void launch_mass_final(const Dots& d, int slot, double drdz, double* out, ull* ctr, cudaStream_t s);

// ---- BiCGSTAB (lib/BiCGSTABREVCOM.f) ----------------------------------------------------
template <typename T>
void launch_bi_init1(long n, const T* b, const T* x, T* r, const Dots& d, ull* ctr, cudaStream_t s);
void launch_bi_init2(KState* ks, const Dots& d, double tol, int maxit, const KState* parent, ull* ctr, cudaStream_t s);
void launch_bi_init3(KState* ks, const Dots& d, ull* ctr, cudaStream_t s);
template <typename T>
void launch_bi_init4(long n, const T* r, T* rtld, const Dots& d, const KState* ks, ull* ctr, cudaStream_t s);
template <typename T>
void launch_bi_p(long n, const T* r, const T* v, T* p, T* phat, const T* diag, int ident, KState* ks, const Dots& d,
                 ull* ctr, cudaStream_t s);
template <typename T>
void launch_bi_s(long n, const T* v, T* r, KState* ks, const Dots& d, ull* ctr, cudaStream_t s);
void launch_bi_snorm(KState* ks, const Dots& d, ull* ctr, cudaStream_t s);
template <typename T>
void launch_pc_blend(long n, const T* x, const T* w, T* y, const KState* ks, int gate, ull* ctr, cudaStream_t s);
template <typename T>
void launch_uv_esolp_scale(const OpScal<T>& o, const T* rho, const T* eta, long n, T* sc, ull* ctr, cudaStream_t s);
template <typename T>
void launch_vmul(long n, const T* a, const T* sc, T* out, const KState* ks, int gate, ull* ctr, cudaStream_t s);
void launch_probe_fill(long n, unsigned long long seed, long probe, double* e, ull* ctr, cudaStream_t s);
void launch_probe_acc(long n, unsigned long long seed, long probe, const double* r, const double* qv, double* num,
                      double* den, int first, ull* ctr, cudaStream_t s);
void launch_probe_final(long n, const double* num, const double* den, double* w, float* w32, ull* ctr,
                        cudaStream_t s);
template <typename T>
void launch_bi_diag_apply(long n, const T* x, const T* diag, int ident, T* y, const KState* ks, int gate, ull* ctr,
                          cudaStream_t s);
template <typename T>
void launch_bi_xr(long n, const T* phat, const T* shat, const T* t, const T* rtld, T* x, T* r, KState* ks,
                  const Dots& d, ull* ctr, cudaStream_t s);
void launch_bi_end(KState* ks, const Dots& d, cudaGraphConditionalHandle h, int use_graph, ull* ctr, cudaStream_t s);
void launch_bi_true_resid(KState* ks, const Dots& d, ull* ctr, cudaStream_t s);
void launch_arm_while(const KState* ks, cudaGraphConditionalHandle h, ull* ctr, cudaStream_t s);

// ---- mixed precision: FP32 BiCGSTAB with FP64 reliable updates ---------------------------
void launch_mr_init(KState* ks, const Dots& d, double tol, int maxit, ull* ctr, cudaStream_t s);
template <typename T>
void launch_mr_reset(long n, const double* r64, T* r, T* rtld, const Dots& d, const KState* ks, ull* ctr,
                     cudaStream_t s);
void launch_mr_end(KState* ks, const Dots& d, cudaGraphConditionalHandle hw, cudaGraphConditionalHandle hif, ull* ctr,
                   cudaStream_t s);
template <typename T>
void launch_mr_fold(long n, T* x32, double* x64, ull* ctr, cudaStream_t s);
void launch_mr_check(KState* ks, const Dots& d, cudaGraphConditionalHandle hw, ull* ctr, cudaStream_t s);

// ---- vectors ---------------------------------------------------------------------------
template <typename T>
void launch_copy(long n, const T* x, T* y, ull* ctr, cudaStream_t s);
template <typename TO, typename TI>
void launch_convert_scale(long n, const TI* x, double scale, TO* y, ull* ctr, cudaStream_t s);  // y = scale * x
void launch_axpy_f2d(long n, const KState* ks, const float* d, double* x, ull* ctr, cudaStream_t s);
template <typename T>
void launch_norm2_partial(long n, const T* x, const Dots& d, int slot, ull* ctr, cudaStream_t s);

// ---- mixed-precision refinement control -------------------------------------------------
void launch_mx_init(KState* outer, const Dots& d, double tol, int max_refine, double itol, ull* ctr,
                    cudaStream_t s);
void launch_mx_inner_setup(KState* inner, const KState* outer, double inner_tol, int inner_maxit, ull* ctr,
                           cudaStream_t s);
void launch_mx_check(KState* outer, const KState* inner, const Dots& d, cudaGraphConditionalHandle h, int use_graph,
                     ull* ctr, cudaStream_t s);
template <typename TO>
void launch_mx_scale(long n, const double* r, const KState* o, TO* y, TO* zero, ull* ctr, cudaStream_t s);

}  // namespace drd
