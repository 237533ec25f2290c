// drd_solver.cu — context, solve sequences, CUDA-graph capture and the extern "C" entry
// points of include/drd_gb300.h.
//
// Each reference subroutine becomes one captured CUDA graph: its RHS kernels, a BiCGSTAB
// whose iteration loop is a device-side WHILE conditional node (the loop never returns to
// the host; the last kernel of each iteration decides whether another one runs), and the
// finalisation kernels.  A full time step (drd_step) is one graph holding all three solves.
// In mixed precision the FP32 BiCGSTAB is nested in a second WHILE loop of FP64 iterative
// refinement (true residual b - A x recomputed in FP64 at every restart).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "drd_kernels.cuh"

using namespace drd;

namespace {

enum SysKind { SYS_CH = 0, SYS_UV = 1, SYS_PHMU = 2, SYS_ORI = 3 };
enum { KS_CH = 0, KS_UV = 1, KS_PHMU = 2, KS_INNER = 3, KS_PRE = 4, KS_MASS = 5, KS_COUNT = 6 };

template <typename T>
struct KVecs {
    T *x, *b, *r, *rtld, *p, *v, *t, *phat, *shat, *tmp, *diag, *ff1;
};

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kPimach = 3.14159265358979;  // lib/vfftpack.f:294

}  // namespace

struct drd_ctx {
    drd_params P;
    DevParams dp;
    int nr = 0, nz = 0;
    long cs = 0, us = 0, vs = 0, nc = 0, nuv = 0, nphmu = 0, nmax = 0;
    cudaStream_t s = nullptr, s2 = nullptr, s3 = nullptr;
    int device = 0;
    char* arena = nullptr;
    size_t arena_bytes = 0, arena_used = 0;
    // coefficients (CELL)
    double *rho, *eta, *bdr, *grad, *M0, *Mi, *pen, *used;
    float *rho32, *eta32, *pen32, *M032, *Mi32, *used32;
    // tables and transform matrices
    double *ph_lcc, *pre_lcc;
    float* ph_lcc32;
    // the solid-blended CH preconditioner: per-cell weights (FP64 and FP32, packed), the probe
    // accumulators; allocated on first use, pc_on when weights are installed
    double *pcw = nullptr, *pnum = nullptr, *pden = nullptr;
    float* pcw32 = nullptr;
    int pc_on = 0;
    double *m2xT, *m2z, *m3xT, *m3z;
    // folded DCT-I (VCOST) matrices of the CH preconditioner: x pass B operands (even / odd
    // output columns, Kx x Nxe each) and z pass A operands (even / odd output rows, Mze x Kz)
    double *f1xe, *f1xo, *f1ze, *f1zo;
    float *f1xe32, *f1xo32, *f1ze32, *f1zo32;
    int Kx = 0, Kz = 0, Nxe = 0, Nxo = 0, Mze = 0, Mzo = 0;
    // ESOLP_x momentum preconditioner: folded DCT-I of length nr+1 for the u block (the v
    // block's length nr reuses f1xe/f1xo), Thomas factors per bdf [rm|bp|c of u, rm|bp|c of v]
    // and a momentum-length scratch vector
    double *f1ue, *f1uo, *es64[2], *esw;
    float *f1ue32, *f1uo32, *es32[2], *esw32;
    // the persistent solver's form of the ESOLP_x factors: r_j, 1/b'_j and c_j/b'_j per mode and row
    float* esq32[2];
    int Ku = 0, Nue = 0, Nuo = 0;
    double *cfB, *cfT;
    // PreSolve_2 by FFT (nr and nz of the form 2^a 3^b 5^c 7^d): plans and twiddle tables in
    // FP64 (the pressure step) and FP32 (the transform's kernel bench)
    int pfft = 0, pfft_ok = 0;
    FftPlan fpx{}, fpz{};
    double *ftwx, *ftwz;
    float *ftwx32, *ftwz32;
    // resident state and scratch
    double* fld[DRD_F_COUNT];
    double *u_after, *v_after, *ph_after, *rmu_after, *f2, *uL, *pnb, *pnt, *dist, *fpd, *w, *t1, *t2;
    float *t1f, *t2f;
    KVecs<double> k64;
    KVecs<float> k32;
    double* part;
    // fiber particles (particles_move.f90): POINTS arrays (np x 2, column-major) and scratch
    drd_particle_params pp{};
    double *pts, *pts_old, *totF, *psum, *ppart, *bdist;
    // PhSolve_ori: wall-energy prefactors cf of angleB / angleT (XLINE) and alpha_s
    double *ori_cfb, *ori_cft;
    // drd_phsolve with guess_mode 1: the rmu of the previous call (the x^(n-1) of the next one)
    double *rmu_prev, *rmu_prev2, *rmu_prev3;
    int rmu_hist = 0;  // how many of rmu_prev.. hold earlier calls' rmu
    // guess_mode 2 / 3: the fields two and three steps back (rmu, u, v), and how many steps of
    // history exist (uv_hist: earlier calls' u_pre held by the per-routine momentum solve)
    double *rmu_pre2, *u_pre2, *v_pre2, *rmu_pre3, *u_pre3, *v_pre3;
    int hist = 0, uv_hist = 0;
    double ori_alpha = 0.0;
    // persistent cooperative inner solver (FP32 CH): grid size, barrier state, on/off
    int persist = 0, pgrid = 0;
    int persist_ch = 0;  // the CH solve too: only when its transform operands stay in shared memory
    int persist_esolp = 0;      // the momentum kernel can run ESOLP_x (its shared-memory work area fits)
    int persist_esolp_solve = 0;  // ... and the momentum solve with ESOLP_x uses it (resident B panels)
    PbPlan eplan{};
    // mixed mode: the CH system is too stiff for FP32 Krylov vectors and is solved in FP64
    int ch_fp64 = 0;
    double ch_stiff = 0.0;
    PbPlan pplan{};
    GridBar* bar = nullptr;
    std::string persist_err;
    int* tcerr = nullptr;  // device: set by the tensor-core transform GEMM when a wait gave up
    // the tensor-core GEMM's packed constant operands: CH x pass (also ESOLP_x's v rows), CH z
    // pass, ESOLP_x's u rows; tiles and K chunks of each
    float *pk_x = nullptr, *pk_z = nullptr, *pk_u = nullptr;
    int pkx_t = 0, pkx_c = 0, pkz_t = 0, pkz_c = 0, pku_t = 0, pku_c = 0;
    // its scratch for the pre-folded operand of x passes whose rows TMA cannot address
    float* tc_pad = nullptr;
    long tc_pad_cap = 0;
    unsigned long long* pprof = nullptr;  // DRD_PERSIST_PROF=1: barrier timestamps of block 0
    int pprof_on = 0;
    KState* ks;      // device, KS_COUNT entries
    CallArgs* ca;    // device
    double* d_mass;  // device
    double* d_diag;  // device: the dissipation diagnostics (e1, e2, e3, e4, dissip, mass)
    KState* h_ks;    // pinned
    CallArgs* h_ca;  // pinned
    double* h_mass;  // pinned
    unsigned long long* ctr;
    int G = 1;
    int gcfg[2][2] = {{-1, -1}, {-1, -1}};  // [fp32?][z-pass?]
    // the mixed mode's FP64 transforms (pressure, a stiff CH system): double-float kernels
    int gcfg_df[2] = {-1, -1};
    std::map<long, cudaGraphExec_t> graphs;
    std::string err;
    int use_graph = 1;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // the per-routine calls' copies of page-locked host arrays, gathered into one launch each way
    HostCopies hq_up{}, hq_down{};
    cudaEvent_t tev0 = nullptr, tev1 = nullptr;  // autotuner timing
    // asynchronous checkpoint: pinned staging, its copy stream and events, the writer thread
    cudaStream_t sck = nullptr;
    cudaEvent_t eck0 = nullptr, eck1 = nullptr;
    double* h_stage = nullptr;
    std::thread ckpt;
    int ckpt_rc = 0;
};

namespace {

#define CK(call)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            c->err = std::string(#call) + ": " + cudaGetErrorString(e_);           \
            return DRD_ERR_CUDA;                                                   \
        }                                                                          \
    } while (0)

template <typename T>
T* carve(drd_ctx* c, long n) {
    size_t bytes = ((size_t)(n > 0 ? n : 1) * sizeof(T) + 255) & ~(size_t)255;
    T* p = (T*)(c->arena + c->arena_used);
    c->arena_used += bytes;
    return p;
}

size_t arena_need(long cs, long us, long vs, long nc, long nr, long nz, long nmax) {
    size_t b = 0;
    auto add = [&](size_t n, size_t sz) { b += ((n > 0 ? n : 1) * sz + 255) & ~(size_t)255; };
    for (int i = 0; i < 8; ++i) add(cs, 8);      // coefficients
    for (int i = 0; i < 6; ++i) add(cs, 4);      // FP32 coefficients
    add(nc, 8); add((nr + 1) * (nz + 1), 8); add(nc, 4);
    add(nr * nr, 8); add(nz * nz, 8); add(nr * nr, 8); add(nz * nz, 8);
    for (int i = 0; i < 4; ++i) { add((nr / 2 + 1) * (nr / 2 + 1), 8); add((nz / 2 + 1) * (nz / 2 + 1), 8); }
    for (int i = 0; i < 4; ++i) { add((nr / 2 + 1) * (nr / 2 + 1), 4); add((nz / 2 + 1) * (nz / 2 + 1), 4); }
    add(nr + 1, 8); add(nr + 1, 8);
    for (int f = 0; f < DRD_F_COUNT; ++f) add(std::max(us, cs), 8);
    add(us, 8); add(vs, 8); add(cs, 8); add(cs, 8); add(cs, 8); add(nz + 1, 8); add(nr, 8); add(nr, 8);
    add(nc, 8); add(cs, 8); add(nc, 8); add(nc, 8); add(nc, 8); add(nc, 4); add(nc, 4);
    for (int i = 0; i < 12; ++i) add(nmax, 8);
    for (int i = 0; i < 12; ++i) add(nmax, 4);
    add(DRD_NDOT * DRD_MAXB, 8);
    add(KS_COUNT * sizeof(KState), 1); add(sizeof(CallArgs), 1); add(1, 8); add(1, 8);
    for (int i = 0; i < 4; ++i) add(2 * DRD_PARTICLES_MAX, 8);  // pts, pts_old, totF, psum
    add(3 * DRD_PARTICLES_MAX * PT_GX, 8); add(cs, 8);          // ppart, bdist
    add(nr + 1, 8); add(nr + 1, 8);                            // ori_cfb, ori_cft
    add(cs, 8); add(cs, 8); add(cs, 8);                        // rmu_prev, rmu_prev2, rmu_prev3
    add(cs, 8); add(us, 8); add(vs, 8);                        // rmu_pre2, u_pre2, v_pre2
    add(cs, 8); add(us, 8); add(vs, 8);                        // rmu_pre3, u_pre3, v_pre3
    add(sizeof(GridBar), 1);                                   // bar
    add(128, 8);                                               // pprof
    add(8, 8);                                                 // d_diag
    add(1, 8);                                                 // tcerr
    add(4 * nr, 8); add(4 * nz, 8); add(4 * nr, 4); add(4 * nz, 4);  // FFT tables (complex, 2n each)
    const long fu = (nr / 2 + 1) * (nr / 2 + 2), nes = 3 * (us + vs);
    add(fu, 8); add(fu, 8); add(fu, 4); add(fu, 4);            // f1ue, f1uo (+ FP32)
    for (int i = 0; i < 2; ++i) { add(nes, 8); add(nes, 4); add(nes, 4); }  // es64, es32, esq32
    add(nmax, 8); add(nmax, 4);                                // esw, esw32
    return b + 4096;
}

DevParams make_dev_params(const drd_params& P) {
    DevParams d{};
    d.nr = P.nr; d.nz = P.nz; d.variant = P.variant; d.phi_mode = P.phi_mode;
    d.lr_neumann = (P.variant == DRD_VARIANT_TP && P.lr_bd_type == 'n');
    d.dr = P.dr; d.dz = P.dz; d.dr2 = P.dr * P.dr; d.dz2 = P.dz * P.dz;
    d.idr2 = 1.0 / d.dr2; d.idz2 = 1.0 / d.dz2;
    d.dt = P.dt; d.xld = P.xld; d.re = P.re; d.ca = P.ca; d.eps = P.I_thickness; d.s = P.s_implicit;
    d.ggx = P.ggx; d.ggz = P.ggz; d.uwT = P.uwT; d.uwB = P.uwB; d.UU = P.UU; d.twall = P.twall;
    d.bdr_upp = P.bdr_upp; d.bdr_low = P.bdr_low;
    d.cang = std::cos(P.angle * kPi / 180);
    d.penalty_k = P.penalty_k; d.lambda_rho = P.lambda_rho; d.lambda_eta = P.lambda_eta;
    d.adjust = P.bdr_ph_used_adjust;
    return d;
}

template <typename T>
OpScal<T> make_op(const drd_ctx* c, int bdf) {
    const DevParams& d = c->dp;
    OpScal<T> o{};
    o.dt = (T)d.dt; o.xld = (T)d.xld; o.eps = (T)d.eps; o.s = (T)d.s; o.idr2 = (T)d.idr2; o.idz2 = (T)d.idz2;
    o.dtxld = (T)(d.dt * d.xld); o.re = (T)d.re; o.pk = (T)d.penalty_k; o.dr = (T)d.dr; o.dz = (T)d.dz;
    o.dr2 = (T)d.dr2; o.dz2 = (T)d.dz2; o.adjust = (T)d.adjust; o.idrdz = (T)(1.0 / (d.dr * d.dz));
    const double tmp = d.eps / d.dz;
    o.cb = (T)((d.eps / d.dz) / tmp);  // coef_bot = (I/dz)/tmp (ph_mu_solve.f90:123)
    o.ct = o.cb;
    o.nr = d.nr; o.nz = d.nz; o.variant = d.variant; o.lr_neumann = d.lr_neumann; o.bdf = bdf; o.phi_mode = d.phi_mode;
    return o;
}

// coef_bot = coef_top of PhSolve_ori's non-dynamic wall branch
// (microfluidics_complex_domain/PhSolve_ori.f90:71-74, :111-113).
double ori_coef(const drd_ctx* c) {
    const double tmp1 = c->P.I_thickness / c->P.dz + 0.5 * c->ori_alpha;
    return (c->P.I_thickness / c->P.dz - 0.5 * c->ori_alpha) / tmp1;
}

// setup() tables (microfluidics_complex_domain/setup.f90:106-155), FP64 on the host.
void host_tables(const drd_params& P, std::vector<double>& ph_lcc, std::vector<double>& pre_lcc) {
    const int nr = P.nr, nz = P.nz;
    const double dr2 = P.dr * P.dr, dz2 = P.dz * P.dz;
    pre_lcc.assign((size_t)(nr + 1) * (nz + 1), 0.0);
    ph_lcc.assign((size_t)nr * nz, 0.0);
    for (int j = 0; j <= nz; ++j) {
        double t1 = kPi * j / 2.0 / nz, fmy = 4.0 * (std::sin(t1) * std::sin(t1)) / dz2;
        for (int i = 0; i <= nr; ++i) {
            double t0 = kPi * i / 2.0 / nr, fmx = 4.0 * (std::sin(t0) * std::sin(t0)) / dr2;
            pre_lcc[i + (size_t)j * (nr + 1)] = -(fmx + fmy);
        }
    }
    pre_lcc[0] = -1.0;
    for (int j = 0; j < nz; ++j) {
        double t1 = kPi * j / 2.0 / (nz - 1), fmy = 4.0 * (std::sin(t1) * std::sin(t1)) / dz2;
        for (int i = 0; i < nr; ++i) {
            double t0 = kPi * i / 2.0 / (nr - 1), fmx = 4.0 * (std::sin(t0) * std::sin(t0)) / dr2;
            double temp = fmx + fmy;
            ph_lcc[i + (size_t)j * nr] =
                1. + P.xld * P.dt * P.s_implicit * temp / P.I_thickness + P.xld * P.I_thickness * P.dt * (temp * temp);
        }
    }
}

// ESOLP_x coefficients of setup (Precipitation_dynamics/setup.f90:157-235), factored for the
// Thomas sweep (rfords) of k_tridiag.  Per mode k of a block with `rows` rows, the system along
// j has sub-diagonal a_j, diagonal b_j = t1 m + (2 dt/dz^2 + fmx_k) (m = 1.5 for bdf 2, the
// *_2 set), super-diagonal c_j; the u block's wall rows carry (2 - xls) dt/dz^2 with xls =
// (2 xlsB - dz)/(2 xlsB + dz) for both walls (xlsT = xlsB, slip ratio 1 on the no-slip deck).
// t1 holds pi/2 when these lines run: the fmx loops before them overwrite the Re-based value
// (:159, :166-169, :202-205).  Output [rm|bp|c of u ((nr+1) x nz), rm|bp|c of v (nr x (nz-1))],
// row j of mode k at [k + len*j]; rm_j = -a_j / b'_{j-1}, b'_j = b_j + rm_j c_{j-1}, b'_0 = b_0.
void host_esolp(const drd_params& P, int bdf, std::vector<double>& out) {
    const int nr = P.nr, nz = P.nz;
    const double dt = P.dt, dr2 = P.dr * P.dr, dz2 = P.dz * P.dz, dz = P.dz;
    const double m = (bdf == 2) ? 1.5 : 1.0;
    double xls = P.xlsB * (1.0 + 1.0) / 2.0;
    xls = (2.0 * xls - dz) / (2.0 * xls + dz);
    const long mu = (long)(nr + 1) * nz, mv = (long)nr * (nz - 1);
    out.assign(3 * (mu + mv), 0.0);
    auto factor = [&](int len, int rows, double* base, const std::vector<double>& a, const std::vector<double>& b,
                      const std::vector<double>& cc, int k) {
        double* rm = base;
        double* bp = base + (long)len * rows;
        double* cv = base + 2L * len * rows;
        double piv = b[0];
        rm[k] = 0.0;
        bp[k] = piv;
        cv[k] = cc[0];
        for (int j = 1; j < rows; ++j) {
            const double r = -a[j] / piv;
            piv = b[j] + r * cc[j - 1];
            rm[k + (long)len * j] = r;
            bp[k + (long)len * j] = piv;
            cv[k + (long)len * j] = cc[j];
        }
    };
    std::vector<double> a, b, cc;
    // u block: modes 0..nr of VCOST length nr+1, rows 0..nz-1 (:166-199)
    const double t1u = kPi * nr / nr / 2.;
    for (int k = 0; k <= nr; ++k) {
        const double sk = std::sin(kPi * k / nr / 2.), fmx = 4.0 * dt * sk * sk / dr2;
        a.assign(nz, -dt / dz2); b.assign(nz, t1u * m + (2.0 * dt / dz2 + fmx)); cc.assign(nz, -dt / dz2);
        a[0] = 0.0; cc[nz - 1] = 0.0;
        b[0] = t1u * m + ((2.0 - xls) * dt / dz2 + fmx);
        b[nz - 1] = t1u * m + ((2.0 - xls) * dt / dz2 + fmx);
        factor(nr + 1, nz, out.data(), a, b, cc, k);
    }
    // v block: modes 0..nr-1 of VCOST length nr, rows 1..nz-1 of v (:202-235)
    const int rv = nz - 1;
    const double t1v = kPi * (nr - 1) / (nr - 1) / 2.;
    for (int k = 0; k < nr; ++k) {
        const double sk = std::sin(kPi * k / (nr - 1) / 2.), fmx = 4.0 * dt * sk * sk / dr2;
        a.assign(rv, -dt / dz2); b.assign(rv, t1v * m + 2.0 * dt / dz2 + fmx); cc.assign(rv, -dt / dz2);
        a[0] = 0.0; cc[rv - 1] = 0.0;
        factor(nr, rv, out.data() + 3 * mu, a, b, cc, k);
    }
}

// Transform matrices.  D1[o][j]: VCOST of length n (lib/vfftpack.f:689-704, pi = PIMACH);
// D2[o][j]: REDFT10; D3[o][j]: REDFT01 (FFTW manual).  Entries use an exact periodic table.
void host_dct_mats(int n, std::vector<double>& d1, std::vector<double>& d2, std::vector<double>& d3) {
    d1.assign((size_t)n * n, 0.0);
    d2.assign((size_t)n * n, 0.0);
    d3.assign((size_t)n * n, 0.0);
    if (n >= 2) {
        const long per = 2L * (n - 1);
        std::vector<double> tab(per);
        for (long q = 0; q < per; ++q) tab[q] = std::cos((double)q * kPimach / (double)(n - 1));
        const double sc = std::sqrt(2.0 * (n - 1));
        for (int o = 0; o < n; ++o)
            for (int j = 0; j < n; ++j) {
                double w = (j == 0) ? 1.0 : (j == n - 1 ? ((o & 1) ? -1.0 : 1.0) : 2.0 * tab[((long)o * j) % per]);
                d1[(size_t)o * n + j] = w / sc;
            }
    }
    const long per4 = 4L * n;
    std::vector<double> t4(per4);
    for (long q = 0; q < per4; ++q) t4[q] = std::cos(kPi * (double)q / (2.0 * n));
    for (int o = 0; o < n; ++o)
        for (int j = 0; j < n; ++j) {
            d2[(size_t)o * n + j] = 2.0 * t4[((long)(2 * j + 1) * o) % per4];
            d3[(size_t)o * n + j] = (j == 0) ? 1.0 : 2.0 * t4[((long)j * (2 * o + 1)) % per4];
        }
}

std::vector<double> transpose(const std::vector<double>& a, int n) {
    std::vector<double> t(a.size());
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) t[(size_t)j * n + i] = a[(size_t)i * n + j];
    return t;
}

template <typename T>
KVecs<T> carve_vecs(drd_ctx* c) {
    KVecs<T> k;
    T** f[] = {&k.x, &k.b, &k.r, &k.rtld, &k.p, &k.v, &k.t, &k.phat, &k.shat, &k.tmp, &k.diag, &k.ff1};
    for (auto* pp : f) *pp = carve<T>(c, c->nmax);
    return k;
}

Dots dots(drd_ctx* c) { return Dots{c->part, c->G}; }
KVecs<double>& vecs(drd_ctx* c, double*) { return c->k64; }
KVecs<float>& vecs(drd_ctx* c, float*) { return c->k32; }

// ---- transforms --------------------------------------------------------------------------
// folded DCT-I operands: 0 x-even, 1 x-odd, 2 z-even, 3 z-odd
template <typename T>
const T* fmat(const drd_ctx* c, int which);
template <>
const double* fmat<double>(const drd_ctx* c, int w) {
    const double* m[] = {c->f1xe, c->f1xo, c->f1ze, c->f1zo};
    return m[w];
}
template <>
const float* fmat<float>(const drd_ctx* c, int w) {
    const float* m[] = {c->f1xe32, c->f1xo32, c->f1ze32, c->f1zo32};
    return m[w];
}

template <typename T>
T* tmp1(drd_ctx* c);
template <>
double* tmp1<double>(drd_ctx* c) { return c->t1; }
template <>
float* tmp1<float>(drd_ctx* c) { return c->t1f; }
template <typename T>
T* tmp2(drd_ctx* c);
template <>
double* tmp2<double>(drd_ctx* c) { return c->t2; }
template <>
float* tmp2<float>(drd_ctx* c) { return c->t2f; }

template <typename T>
GemmArgs<T> gargs(drd_ctx* c, int M, int N, int K, const T* A, long lda, const T* B, long ldb, T* C, long ldc,
                  const KState* ks, int gate) {
    GemmArgs<T> a{};
    a.M = M; a.N = N; a.K = K; a.A = A; a.lda = lda; a.B = B; a.ldb = ldb; a.C = C; a.ldc = ldc;
    a.nr = c->nr; a.ks = ks; a.gate = gate; a.ctr = c->ctr; a.ca = c->ca; a.scale = 1.0;
    a.err = c->tcerr;
    return a;
}

template <typename T>
int gcfg(drd_ctx* c, int zpass) {
    // FP64 transforms: true FP64 GEMMs in the FP64 mode (the reference's arithmetic), the
    // double-float kernels in the mixed mode, where they are never the precision that limits
    if (sizeof(T) == 8 && c->P.precision == DRD_PREC_MIXED) return c->gcfg_df[zpass];
    return c->gcfg[sizeof(T) == 4][zpass];
}

// The folded DCT-I passes of the CH preconditioner.  x pass: out[m][o] = sum_j X[m][j] C_x[o][j]
// over nr columns; z pass: out[o][n] = sum_j C_z[o][j] X[j][n] over nz rows.  Each pass folds
// X's j and L-j (C[o][L-j] = (-1)^o C[o][j]) and computes even and odd outputs as the two
// halves of one launch, halving the multiply-adds.
template <typename T>
GemmArgs<T> dct1_xpass(drd_ctx* c, const T* X, T* out, const KState* ks, int gate) {
    GemmArgs<T> a = gargs<T>(c, c->nz, c->Nxe, c->Kx, X, c->nr, fmat<T>(c, 0), c->Nxe, out, c->nr, ks, gate);
    a.fold = FOLD_A;
    a.Lf = c->nr - 1;
    a.B_odd = fmat<T>(c, 1);
    a.N_odd = c->Nxo;
    if (sizeof(T) == 4) {
        a.packed = c->pk_x; a.pk_tiles = c->pkx_t; a.pk_chunks = c->pkx_c;
        a.pad = (float*)c->tc_pad; a.pad_cap = c->tc_pad_cap;
    }
    return a;
}
template <typename T>
GemmArgs<T> dct1_zpass(drd_ctx* c, const T* X, T* out, const KState* ks, int gate) {
    GemmArgs<T> a = gargs<T>(c, c->Mze, c->nr, c->Kz, fmat<T>(c, 2), c->Kz, X, c->nr, out, c->nr, ks, gate);
    a.fold = FOLD_B;
    a.Lf = c->nz - 1;
    a.A_odd = fmat<T>(c, 3);
    a.M_odd = c->Mzo;
    if (sizeof(T) == 4) { a.packed = c->pk_z; a.pk_tiles = c->pkz_t; a.pk_chunks = c->pkz_c; }
    return a;
}

// PSolve_CG (microfluidics_complex_domain/PhSolve.f90:296-313): y = C (C x ./ Ph_Lcc) with the
// separable 2-D DCT-I C = VCOST_x VCOST_z, as four folded GEMM passes (x, z, x, z).
template <typename T>
void enq_ch_psolve(drd_ctx* c, const T* x, T* y, const KState* ks, int gate, cudaStream_t s) {
    T* t1 = tmp1<T>(c);
    T* t2 = tmp2<T>(c);
    const T* tab = (sizeof(T) == 8) ? (const T*)c->ph_lcc : (const T*)c->ph_lcc32;
    launch_gemm<T>(gcfg<T>(c, 0), EPI_STORE, dct1_xpass<T>(c, x, t1, ks, gate), s);
    auto a2 = dct1_zpass<T>(c, t1, t2, ks, gate);
    a2.tab = tab;
    a2.ldt = c->nr;
    launch_gemm<T>(gcfg<T>(c, 1), EPI_DIV_TAB, a2, s);
    launch_gemm<T>(gcfg<T>(c, 0), EPI_STORE, dct1_xpass<T>(c, t2, t1, ks, gate), s);
    launch_gemm<T>(gcfg<T>(c, 1), EPI_STORE, dct1_zpass<T>(c, t1, y, ks, gate), s);
}

// The row pass of ESOLP_x over one block: VCOST of length L along each of M rows (row
// stride L), folded like the CH x pass.  L = nr+1 (u block) uses f1ue/f1uo, L = nr (v) f1xe/f1xo.
template <typename T>
GemmArgs<T> esolp_rows(drd_ctx* c, int M, int L, const T* X, T* out, const KState* ks, int gate) {
    const bool u = (L == c->nr + 1);
    const T* be = u ? (sizeof(T) == 8 ? (const T*)c->f1ue : (const T*)c->f1ue32) : fmat<T>(c, 0);
    const T* bo = u ? (sizeof(T) == 8 ? (const T*)c->f1uo : (const T*)c->f1uo32) : fmat<T>(c, 1);
    const int K = u ? c->Ku : c->Kx, Ne = u ? c->Nue : c->Nxe, No = u ? c->Nuo : c->Nxo;
    GemmArgs<T> a = gargs<T>(c, M, Ne, K, X, L, be, Ne, out, L, ks, gate);
    a.fold = FOLD_A;
    a.Lf = L - 1;
    a.B_odd = bo;
    a.N_odd = No;
    if (sizeof(T) == 4) {
        a.packed = u ? c->pk_u : c->pk_x;
        a.pk_tiles = u ? c->pku_t : c->pkx_t;
        a.pk_chunks = u ? c->pku_c : c->pkx_c;
        a.pad = (float*)c->tc_pad;
        a.pad_cap = c->tc_pad_cap;
    }
    return a;
}

// PSolve_CG with ESOLP_x (Precipitation_dynamics/VeloSolve_combined.f90:800-806, ESOLP.f90):
// per block (u: nr+1 x nz, v: nr x nz-1 of the packed vector) VCOST along x, a tridiagonal
// solve along y per x mode, VCOST along x.  Five launches: two row passes, one Thomas sweep
// over both blocks, two row passes.
template <typename T>
void enq_esolp(drd_ctx* c, int bdf, const T* x, T* y, const KState* ks, int gate, cudaStream_t s) {
    const int nr = c->nr, nz = c->nz;
    const long mu = (long)(nr + 1) * nz, mv = (long)nr * (nz - 1);
    T* w = (sizeof(T) == 8) ? (T*)c->esw : (T*)c->esw32;
    const T* f = (sizeof(T) == 8) ? (const T*)c->es64[bdf - 1] : (const T*)c->es32[bdf - 1];
    launch_gemm<T>(gcfg<T>(c, 0), EPI_STORE, esolp_rows<T>(c, nz, nr + 1, x, w, ks, gate), s);
    launch_gemm<T>(gcfg<T>(c, 0), EPI_STORE, esolp_rows<T>(c, nz - 1, nr, x + mu, w + mu, ks, gate), s);
    const T* fv = f + 3 * mu;
    TriBlock<T> bu{nr + 1, nz, f, f + mu, f + 2 * mu, w};
    TriBlock<T> bv{nr, nz - 1, fv, fv + mv, fv + 2 * mv, w + mu};
    launch_tridiag<T>(bu, bv, ks, gate, c->ctr, s);
    launch_gemm<T>(gcfg<T>(c, 0), EPI_STORE, esolp_rows<T>(c, nz, nr + 1, w, y, ks, gate), s);
    launch_gemm<T>(gcfg<T>(c, 0), EPI_STORE, esolp_rows<T>(c, nz - 1, nr, w + mu, y + mu, ks, gate), s);
}

// ---- generic system operations -------------------------------------------------------------
struct Sys {
    int kind;
    int bdf;
    long n;
    int jacobi;  // diagonal preconditioner in k.diag
    int ident;   // identity preconditioner
    int esolp;   // ESOLP_x preconditioner (momentum)
    int scaled;  // ESOLP_x between the diagonal scalings s = sqrt(D0 / D), held in k.diag
};

template <typename T>
const T* coef(drd_ctx* c, int which);  // 0 rho 1 eta 2 pen 3 M0 4 Mi 5 used
template <>
const double* coef<double>(drd_ctx* c, int w) {
    const double* a[] = {c->rho, c->eta, c->pen, c->M0, c->Mi, c->used};
    return a[w];
}
template <>
const float* coef<float>(drd_ctx* c, int w) {
    const float* a[] = {c->rho32, c->eta32, c->pen32, c->M032, c->Mi32, c->used32};
    return a[w];
}

template <typename T>
void enq_matvec(drd_ctx* c, const Sys& S, T alpha, const T* x, T beta, T* y, const T* dot1, int self2, int slot1,
                const KState* ks, int gate, cudaStream_t s) {
    Dots d = dots(c);
    KVecs<T>& k = vecs(c, (T*)nullptr);
    if (S.kind == SYS_CH) {
        launch_ch_matvec<T>(make_op<T>(c, 0), coef<T>(c, 3), coef<T>(c, 4), alpha, x, beta, y, k.ff1, dot1, self2, d,
                            slot1, ks, gate, c->ctr, s);
    } else if (S.kind == SYS_ORI) {
        OpScal<T> o = make_op<T>(c, 0);
        const double cb = ori_coef(c);
        o.cb = (T)cb;
        o.ct = (T)cb;
        launch_ori_matvec<T>(o, alpha, x, beta, y, k.ff1, dot1, self2, d, slot1, ks, gate, c->ctr, s);
    } else if (S.kind == SYS_UV) {
        launch_uv_matvec<T>(make_op<T>(c, S.bdf), coef<T>(c, 0), coef<T>(c, 1), coef<T>(c, 2), alpha, x, beta, y,
                            dot1, self2, d, slot1, ks, gate, c->ctr, s);
    } else {
        launch_phmu_matvec<T>(make_op<T>(c, 0), coef<T>(c, 3), coef<T>(c, 4), coef<T>(c, 5), alpha, x, beta, y, dot1,
                              self2, d, slot1, ks, gate, c->ctr, s);
    }
}

template <typename T>
void enq_psolve(drd_ctx* c, const Sys& S, const T* x, T* y, const KState* ks, int gate, cudaStream_t s) {
    KVecs<T>& k = vecs(c, (T*)nullptr);
    if (S.kind == SYS_CH || S.kind == SYS_ORI) {
        enq_ch_psolve<T>(c, x, y, ks, gate, s);
        if (S.kind == SYS_CH && c->pc_on)
            launch_pc_blend<T>(S.n, x, (sizeof(T) == 8) ? (const T*)c->pcw : (const T*)c->pcw32, y, ks, gate, c->ctr, s);
    } else if (S.esolp && S.scaled) {  // y = s E(s x)
        launch_vmul<T>(S.n, x, k.diag, k.ff1, ks, gate, c->ctr, s);
        enq_esolp<T>(c, S.bdf, k.ff1, y, ks, gate, s);
        launch_vmul<T>(S.n, y, k.diag, y, ks, gate, c->ctr, s);
    } else if (S.esolp) enq_esolp<T>(c, S.bdf, x, y, ks, gate, s);
    else launch_bi_diag_apply<T>(S.n, x, S.jacobi ? k.diag : nullptr, S.ident, y, ks, gate, c->ctr, s);
}

// Preconditioner diagonal for the systems that use one (set up once per solve).
template <typename T>
void enq_sys_setup(drd_ctx* c, const Sys& S, cudaStream_t s) {
    KVecs<T>& k = vecs(c, (T*)nullptr);
    if (S.kind == SYS_UV && S.jacobi) launch_uv_diag<T>(make_op<T>(c, S.bdf), coef<T>(c, 0), coef<T>(c, 1), k.diag, c->ctr, s);
    if (S.kind == SYS_UV && S.esolp && S.scaled)
        launch_uv_esolp_scale<T>(make_op<T>(c, S.bdf), coef<T>(c, 0), coef<T>(c, 1), S.n, k.diag, c->ctr, s);
    if (S.kind == SYS_PHMU) launch_phmu_diag<T>(make_op<T>(c, 0), k.diag, c->ctr, s);
}

// One BiCGSTAB iteration (lib/BiCGSTABREVCOM.f:257-388) up to the X/R update.
template <typename T>
void enq_bicg_body(drd_ctx* c, const Sys& S, KVecs<T>& k, KState* ks, cudaStream_t s) {
    Dots d = dots(c);
    const long n = S.n;
    if (S.kind == SYS_CH || S.kind == SYS_ORI || S.esolp) {
        launch_bi_p<T>(n, k.r, k.v, k.p, k.phat, nullptr, 0, ks, d, c->ctr, s);
        enq_psolve<T>(c, S, k.p, k.phat, ks, G_RUNNING, s);
    } else {
        launch_bi_p<T>(n, k.r, k.v, k.p, k.phat, S.jacobi ? k.diag : nullptr, S.ident || !S.jacobi, ks, d, c->ctr, s);
    }
    enq_matvec<T>(c, S, T(1), k.phat, T(0), k.v, k.rtld, 0, 4, ks, G_RUNNING, s);
    launch_bi_s<T>(n, k.v, k.r, ks, d, c->ctr, s);
    launch_bi_snorm(ks, d, c->ctr, s);
    enq_psolve<T>(c, S, k.r, k.shat, ks, G_RUNNING, s);
    enq_matvec<T>(c, S, T(1), k.shat, T(0), k.t, k.r, 1, 6, ks, G_RUNNING, s);
    launch_bi_xr<T>(n, k.phat, k.shat, k.t, k.rtld, k.x, k.r, ks, d, c->ctr, s);
}

template <typename T>
void enq_bicg_iter(drd_ctx* c, const Sys& S, KVecs<T>& k, KState* ks, cudaGraphConditionalHandle h, int use_graph,
                   cudaStream_t s) {
    enq_bicg_body<T>(c, S, k, ks, s);
    launch_bi_end(ks, dots(c), h, use_graph && c->use_graph, c->ctr, s);
}

// Start of the solve with the guess already in k.x (:229-255).
template <typename T>
void enq_bicg_setup(drd_ctx* c, const Sys& S, KVecs<T>& k, KState* ks, double tol, int maxit, const KState* parent,
                    cudaStream_t s) {
    Dots d = dots(c);
    launch_bi_init1<T>(S.n, k.b, k.x, k.r, d, c->ctr, s);
    launch_bi_init2(ks, d, tol, maxit, parent, c->ctr, s);
    enq_matvec<T>(c, S, T(-1), k.x, T(1), k.r, nullptr, 1, -1, ks, G_XNZ, s);
    launch_bi_init3(ks, d, c->ctr, s);
    launch_bi_init4<T>(S.n, k.r, k.rtld, d, ks, c->ctr, s);
}

// Appends a WHILE conditional node looping on state `ks` to the graph being captured on `s`
// (preceded by a kernel that arms its condition from ks) and captures body(stream, handle)
// into its body graph on `sb`.
int capture_while(drd_ctx* c, cudaStream_t s, cudaStream_t sb, const KState* ks,
                  const std::function<void(cudaStream_t, cudaGraphConditionalHandle)>& body) {
    if (!c->use_graph) {
        // direct launches (profiling / debugging): the host runs the loop, reading the state's
        // phase after every body; the body's own cap (MAXIT) still bounds it
        (void)sb;
        int* hp = &c->h_ks[KS_COUNT - 1].phase;  // scratch slot of the pinned states
        for (int guard = 0; guard < (1 << 20); ++guard) {
            CK(cudaMemcpyAsync(hp, &ks->phase, sizeof(int), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (*hp != PH_RUNNING) break;
            body(s, cudaGraphConditionalHandle{});
        }
        return DRD_OK;
    }
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
    if (st != cudaStreamCaptureStatusActive) { c->err = "capture_while: stream not capturing"; return DRD_ERR_CUDA; }
    cudaGraphConditionalHandle h;
    CK(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    launch_arm_while(ks, h, c->ctr, s);
    CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t bg = p.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(sb, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    body(sb, h);
    cudaGraph_t out;
    CK(cudaStreamEndCapture(sb, &out));
    return DRD_OK;
}

// Creates an IF conditional handle in the graph being captured on `s`.
int make_if_handle(drd_ctx* c, cudaStream_t s, cudaGraphConditionalHandle* h) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr));
    CK(cudaGraphConditionalHandleCreate(h, g, 0, 0));
    return DRD_OK;
}

// Appends an IF conditional node on handle h (set by an already captured kernel) to the graph
// being captured on `s`, and captures body(stream) into its body graph on `sb`.
int capture_if(drd_ctx* c, cudaStream_t s, cudaStream_t sb, cudaGraphConditionalHandle h,
               const std::function<void(cudaStream_t)>& body) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t bg = p.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(sb, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    body(sb);
    cudaGraph_t out;
    CK(cudaStreamEndCapture(sb, &out));
    return DRD_OK;
}

// The persistent cooperative inner solver needs cooperative launch support and one resident
// block per SM; DRD_PERSIST=0 in the environment turns it off (the graph-loop path is used).
int setup_persist(drd_ctx* c) {
    c->persist = 0;
    const char* env = std::getenv("DRD_PERSIST");
    if (env && std::atoi(env) == 0) return DRD_OK;
    int coop = 0, sms = 0;
    CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    if (!coop || sms < 1) { c->persist_err = "no cooperative launch on this device"; return DRD_OK; }
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    const int grid = std::min(sms, DRD_MAXB);
    c->pplan = persist_ch_plan(c->nr, c->nz, grid, (size_t)std::max(0, optin - 4096));
    c->eplan = persist_esolp_plan(c->nr, c->nz, grid, (size_t)std::max(0, optin - 4096));
    for (int kind = PK_CH; kind <= PK_UV; ++kind) {
        const size_t sm = kind == PK_CH ? c->pplan.bytes : 0;
        if (sm > (size_t)optin) { c->persist_err = "persistent solver needs more shared memory"; return DRD_OK; }
        int occ = 0;
        CK(cudaFuncSetAttribute(persist_kernel(kind), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, persist_kernel(kind), persist_threads(), sm));
        if (occ < 1) { c->persist_err = "persistent solver does not fit one block per SM"; return DRD_OK; }
    }
    c->pgrid = grid;
    c->persist = 1;
    // the momentum kernel's ESOLP_x work area (the Jacobi path launches it without one)
    c->persist_esolp = 0;
    if (c->eplan.bytes <= (size_t)optin &&
        cudaFuncSetAttribute(persist_kernel(PK_UV), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->eplan.bytes) ==
            cudaSuccess) {
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, persist_kernel(PK_UV), persist_threads(),
                                                          c->eplan.bytes) == cudaSuccess && occ >= 1)
            c->persist_esolp = 1;
    }
    cudaGetLastError();
    // Past the resident plan (more x-pass tiles than blocks, streamed operands) the persistent CH
    // solve is slower than the kernel-per-phase loop's tuned GEMMs: 2048x1024 took about 10 ms
    // per FP32 iteration against 2 ms.
    c->persist_ch = c->pplan.b_res && c->pplan.z_res;
    if (!c->persist_ch) c->persist_err = "CH: the grid exceeds the resident shared-memory plan; the CH solve uses the kernel-per-phase loop";
    // The same for the momentum solve with ESOLP_x: past the resident row-transform panels its
    // persistent row passes stream their operands, and the kernel-per-phase loop's tuned GEMMs
    // (the tensor-core passes at large grids) win: at 2048x1024 a solve took 85-92 ms there
    // against 261-266 ms in the persistent kernel.
    c->persist_esolp_solve = c->persist_esolp && c->eplan.b_res;
    if (c->persist_esolp && !c->persist_esolp_solve)
        c->persist_err += std::string(c->persist_err.empty() ? "" : "; ") +
                          "momentum: the row-transform panels exceed shared memory; the ESOLP_x solve uses the kernel-per-phase loop";
    const char* pe = std::getenv("DRD_PERSIST_PROF");
    c->pprof_on = pe && std::atoi(pe) != 0;
    return DRD_OK;
}

// Arguments of the persistent FP32 inner solve of system S (the k32 vectors, FP32 coefficients).
PersistArgs persist_args(drd_ctx* c, const Sys& S, KState* in, const KState* parent, double tol, int maxit) {
    PersistArgs a{};
    a.kind = (S.kind == SYS_CH) ? PK_CH : PK_UV;
    a.nr = c->nr; a.nz = c->nz; a.n = S.n;
    a.o = make_op<float>(c, S.kind == SYS_UV ? S.bdf : 0);
    a.M0 = c->M032; a.Mi = c->Mi32; a.lcc = c->ph_lcc32;
    a.pcw = (S.kind == SYS_CH && c->pc_on) ? c->pcw32 : nullptr;
    a.fxe = c->f1xe32; a.fxo = c->f1xo32; a.fze = c->f1ze32; a.fzo = c->f1zo32;
    a.Kx = c->Kx; a.Nxe = c->Nxe; a.Nxo = c->Nxo; a.Kz = c->Kz; a.Mze = c->Mze; a.Mzo = c->Mzo;
    KVecs<float>& f = c->k32;
    a.rho = c->rho32; a.eta = c->eta32; a.pen = c->pen32; a.diag = f.diag; a.ident = S.ident || !S.jacobi;
    a.esolp = (S.kind == SYS_UV && S.esolp) ? (S.scaled ? 2 : 1) : 0;
    a.fue = c->f1ue32; a.fuo = c->f1uo32; a.Ku = c->Ku; a.Nue = c->Nue; a.Nuo = c->Nuo;
    a.esf = a.esolp ? c->esq32[S.bdf - 1] : nullptr;
    a.x = f.x; a.b = f.b; a.r = f.r; a.rtld = f.rtld; a.p = f.p; a.v = f.v; a.phat = f.phat; a.shat = f.shat;
    a.t = f.t; a.ff1 = f.ff1; a.w1 = c->t1f; a.w2 = c->t2f;
    a.part = c->part; a.ks = in; a.parent = parent; a.bar = c->bar; a.tol = tol; a.maxit = maxit; a.ctr = c->ctr;
    a.prof = c->pprof_on ? c->pprof : nullptr;
    a.work_off = c->pplan.work_off; a.z_off = c->pplan.z_off; a.b_off = c->pplan.b_off;
    a.z_res = c->pplan.z_res; a.b_res = c->pplan.b_res;
    a.smem_bytes = a.kind == PK_CH ? c->pplan.bytes : 0;
    if (a.esolp) {  // the momentum kernel's own plan
        a.work_off = c->eplan.work_off; a.b_off = c->eplan.b_off; a.b_res = c->eplan.b_res;
        a.z_res = 0;
        a.smem_bytes = c->eplan.bytes;
    }
    return a;
}

// A whole Krylov solve of system S for k64.b with guess k64.x (FP64 result in k64.x).
// FP64 mode: the reference's BiCGSTAB.  Mixed mode: FP64 iterative refinement around an FP32
// BiCGSTAB with the same preconditioner.  `ks_slot` receives the status.
int enq_solve(drd_ctx* c, const Sys& S, int ks_slot, double tol, int maxit, int mixed, cudaStream_t s) {
    KState* ks = c->ks + ks_slot;
    KVecs<double>& k = c->k64;
    Dots d = dots(c);
    int rc = DRD_OK;
    const bool persistent =
        mixed && c->persist && ((S.kind == SYS_CH && c->persist_ch) || (S.kind == SYS_UV && (!S.esolp || c->persist_esolp_solve)));
    if (!persistent) launch_stamp(ks, 0, c->ctr, s);
    if (!mixed) {
        enq_sys_setup<double>(c, S, s);
        enq_bicg_setup<double>(c, S, k, ks, tol, maxit, nullptr, s);
        rc = capture_while(c, s, c->s2, ks, [&](cudaStream_t sb, cudaGraphConditionalHandle h) {
            enq_bicg_iter<double>(c, S, k, ks, h, 1, sb);
        });
        if (rc) return rc;
    } else if (persistent) {
        // the whole mixed solve (FP64 refinement and its FP32 inner solves) in one cooperative
        // launch; it leaves the FP64 true residual of the returned x in the state
        enq_sys_setup<float>(c, S, s);
        launch_bar_reset(c->bar, c->ctr, s);
        PersistArgs a = persist_args(c, S, ks, nullptr, c->P.mixed_inner_tol, maxit);
        a.mode = PM_REFINE;
        a.b64 = k.b;
        a.x64 = k.x;
        a.r64 = k.r;
        a.f64 = k.ff1;
        a.od = make_op<double>(c, S.kind == SYS_UV ? S.bdf : 0);
        a.M0d = coef<double>(c, 3); a.Mid = coef<double>(c, 4);
        a.rhod = coef<double>(c, 0); a.etad = coef<double>(c, 1); a.pend = coef<double>(c, 2);
        a.outer_tol = tol;
        a.max_refine = c->P.mixed_max_refine;
        cudaError_t e = launch_bicg_persist(a, c->pgrid, s);
        if (e != cudaSuccess) {
            c->err = std::string("persistent solver launch: ") + cudaGetErrorString(e);
            return DRD_ERR_CUDA;
        }
        return DRD_OK;
    } else {
        // FP64 iterative refinement around an FP32 BiCGSTAB: each sweep solves A d = r / ||r||
        // from a zero guess to mixed_inner_tol, then x += ||r|| d and r = b - A x in FP64.
        // (A single FP32 sequence with residual replacement is not used: the FP32 transforms'
        // rounding makes the preconditioner slightly input-dependent and long sequences drift.)
        KVecs<float>& f = c->k32;
        KState* in = c->ks + KS_INNER;
        enq_sys_setup<float>(c, S, s);
        launch_copy<double>(S.n, k.b, k.r, c->ctr, s);
        enq_matvec<double>(c, S, -1.0, k.x, 1.0, k.r, nullptr, 1, -1, nullptr, G_ALWAYS, s);
        launch_norm2_partial<double>(S.n, k.b, d, 3, c->ctr, s);
        const double itol = c->P.mixed_inner_tol;
        launch_mx_init(ks, d, tol, c->P.mixed_max_refine, itol, c->ctr, s);
        rc = capture_while(c, s, c->s2, ks, [&](cudaStream_t sb, cudaGraphConditionalHandle ho) {
            launch_mx_scale<float>(S.n, k.r, ks, f.b, f.x, c->ctr, sb);
            enq_bicg_setup<float>(c, S, f, in, itol, maxit, ks, sb);
            int rc2 = capture_while(c, sb, c->s3, in, [&](cudaStream_t si, cudaGraphConditionalHandle hi) {
                enq_bicg_iter<float>(c, S, f, in, hi, 1, si);
            });
            if (rc2) rc = rc2;
            launch_axpy_f2d(S.n, ks, f.x, k.x, c->ctr, sb);
            launch_copy<double>(S.n, k.b, k.r, c->ctr, sb);
            enq_matvec<double>(c, S, -1.0, k.x, 1.0, k.r, nullptr, 1, -1, nullptr, G_ALWAYS, sb);
            launch_mx_check(ks, in, d, ho, c->use_graph, c->ctr, sb);
        });
        if (rc) return rc;
    }
    // true FP64 residual of the returned x
    launch_copy<double>(S.n, k.b, k.tmp, c->ctr, s);
    enq_matvec<double>(c, S, -1.0, k.x, 1.0, k.tmp, nullptr, 1, -1, nullptr, G_ALWAYS, s);
    launch_bi_true_resid(ks, d, c->ctr, s);
    launch_stamp(ks, 1, c->ctr, s);
    return DRD_OK;
}

// ---- the per-step routines as graph segments ------------------------------------------------
Sys sys_of(drd_ctx* c, int kind, int bdf) {
    Sys S{};
    S.kind = kind;
    S.bdf = bdf;
    if (kind == SYS_CH || kind == SYS_ORI) S.n = c->nc;
    else if (kind == SYS_PHMU) { S.n = c->nphmu; S.jacobi = 1; }
    else {
        S.n = c->nuv;
        const bool tp_ident = (c->P.variant == DRD_VARIANT_TP && bdf == 2);
        S.esolp = (c->P.uv_precond == DRD_UV_ESOLP || c->P.uv_precond == DRD_UV_ESOLP_SCALED);
        S.scaled = (c->P.uv_precond == DRD_UV_ESOLP_SCALED);
        S.jacobi = !tp_ident && !S.esolp;
        S.ident = tp_ident && !S.esolp;
    }
    return S;
}

int mixed_of(drd_ctx* c) { return c->P.precision == DRD_PREC_MIXED; }
// Whether the solve that reports into status slot `slot` runs mixed (the CH slot may not).
int mixed_for(drd_ctx* c, int slot) { return mixed_of(c) && !(slot == KS_CH && c->ch_fp64); }

// PhSolve (microfluidics_complex_domain/PhSolve.f90:1-126) on fld[U,V,PH,RMU] -> rmu_after, ph_after.
// extrap: the initial guess is 2 rmu - rmu_pre (1), 3 rmu - 3 rmu_pre + rmu_pre2 (2) or
// 4 rmu - 6 rmu_pre + 4 rmu_pre2 - rmu_pre3 (3).
int enq_ch(drd_ctx* c, cudaStream_t s, int extrap = 0) {
    const DevParams& P = c->dp;
    launch_ch_f2(P, c->fld[DRD_F_U], c->fld[DRD_F_V], c->fld[DRD_F_PH], c->f2, c->ctr, s);
    launch_ch_rhs(P, c->fld[DRD_F_PH], c->fld[DRD_F_RMU], extrap ? c->fld[DRD_F_RMU_PRE] : nullptr,
                  extrap >= 2 ? c->rmu_pre2 : nullptr, extrap == 3 ? c->rmu_pre3 : nullptr, c->bdr, c->grad, c->Mi,
                  c->f2, c->k64.b, c->k64.x, c->ctr, s);
    int rc = enq_solve(c, sys_of(c, SYS_CH, 0), KS_CH, c->P.tol, c->P.ch_maxit, mixed_for(c, KS_CH), s);
    if (rc) return rc;
    launch_ch_fin(P, c->k64.x, c->f2, c->M0, c->rmu_after, c->ph_after, c->ctr, s);
    return DRD_OK;
}

// PhSolve_ori (microfluidics_complex_domain/PhSolve_ori.f90:1-214) on fld[U,V,PH] ->
// ph_after, rmu_after, with the wall prefactors and alpha_s last set by set_ori_walls.
int enq_ori(drd_ctx* c, cudaStream_t s) {
    const DevParams& P = c->dp;
    launch_ch_f2(P, c->fld[DRD_F_U], c->fld[DRD_F_V], c->fld[DRD_F_PH], c->f2, c->ctr, s);
    launch_ori_rhs(P, c->fld[DRD_F_PH], c->f2, c->ori_cfb, c->ori_cft, c->ori_alpha, c->k64.b, c->k64.x, c->pnb, c->pnt,
                   c->ctr, s);
    int rc = enq_solve(c, sys_of(c, SYS_ORI, 0), KS_CH, c->P.tol, c->P.ch_maxit, mixed_for(c, KS_CH), s);
    if (rc) return rc;
    const double cb = ori_coef(c);
    launch_ori_fin(P, c->k64.x, c->pnb, c->pnt, cb, cb, c->ph_after, c->rmu_after, c->ctr, s);
    return DRD_OK;
}

// ph_mu_solve (two_phase_flow_complex_domain/ph_mu_solve.f90:3-197).
int enq_phmu(drd_ctx* c, cudaStream_t s, int extrap = 0) {
    const DevParams& P = c->dp;
    launch_phmu_prep(P, c->fld[DRD_F_U], c->fld[DRD_F_V], c->fld[DRD_F_PH], c->bdr, c->used, c->M0, c->f2, c->ctr, s);
    launch_convert_scale<float, double>(c->cs, c->M0, 1.0, c->M032, c->ctr, s);
    launch_phmu_rhs(P, c->fld[DRD_F_PH], c->fld[DRD_F_RMU], extrap ? c->fld[DRD_F_PH_PRE] : nullptr,  // linear only
                    extrap ? c->fld[DRD_F_RMU_PRE] : nullptr, c->bdr, c->grad, c->f2, c->cfB, c->cfT, c->k64.b,
                    c->k64.x, c->pnb, c->pnt, c->ctr, s);
    int rc = enq_solve(c, sys_of(c, SYS_PHMU, 0), KS_PHMU, c->P.tol, c->P.phmu_maxit, mixed_of(c), s);
    if (rc) return rc;
    OpScal<double> o = make_op<double>(c, 0);
    launch_phmu_fin(P, c->k64.x, c->pnb, c->pnt, o.cb, o.ct, c->ph_after, c->rmu_after, c->ctr, s);
    return DRD_OK;
}

// VeloSolve_combined (bdf 1) / VeloSolve_2_combined (bdf 2) -> u_after, v_after.
// extrap (BDF2 only): the guess extrapolates u through u_pre, u_pre2, u_pre3 linearly (1),
// quadratically (2) or cubically (3); v likewise.
int enq_uv(drd_ctx* c, int bdf, cudaStream_t s, int extrap = 0) {
    const DevParams& P = c->dp;
    double** f = c->fld;
    launch_uv_rhs(P, bdf, c->ca, f[DRD_F_PSI1], f[DRD_F_PSI2], f[DRD_F_U_PRE], f[DRD_F_U], f[DRD_F_V_PRE], f[DRD_F_V],
                  f[DRD_F_P], c->rho, c->eta, c->bdr, c->used, c->ph_after, c->rmu_after, f[DRD_F_PF1], f[DRD_F_PF2],
                  c->k64.b, c->k64.x, c->uL, bdf == 2 ? extrap : 0, c->u_pre2, c->v_pre2, c->u_pre3, c->v_pre3,
                  c->ctr, s);
    int rc = enq_solve(c, sys_of(c, SYS_UV, bdf), KS_UV, c->P.tol, c->P.uv_maxit, mixed_of(c), s);
    if (rc) return rc;
    launch_uv_fin(P, c->k64.x, c->uL, c->u_after, c->v_after, c->ctr, s);
    return DRD_OK;
}

// PreSolve_2 + dct_fftw (microfluidics_complex_domain/PreSolve_2.f90:1-186) on fld[U,V] -> out.
void enq_pre(drd_ctx* c, double* out, cudaStream_t s) {
    const int nr = c->nr, nz = c->nz;
    if (c->pfft) {  // three FFT passes (drd_pressure_fft.cu), then the ghosts
        launch_pressure_fft(nr, nz, c->P.dr, c->P.dz, c->fpx, c->fpz, c->ftwx, c->ftwz, c->fld[DRD_F_U],
                            c->fld[DRD_F_V], c->t1, c->pre_lcc, out, c->ca, c->ctr, s);
        launch_fill_neumann(nr, nz, out, nullptr, c->ctr, s);
        return;
    }
    launch_pre_div(c->dp, c->fld[DRD_F_U], c->fld[DRD_F_V], c->w, c->ctr, s);
    launch_gemm<double>(gcfg<double>(c, 0), EPI_STORE, gargs<double>(c, nz, nr, nr, c->w, nr, c->m2xT, nr, c->t1, nr, nullptr, G_ALWAYS), s);
    auto a2 = gargs<double>(c, nz, nr, nz, c->m2z, nz, c->t1, nr, c->t2, nr, nullptr, G_ALWAYS);
    a2.tab = c->pre_lcc; a2.ldt = nr + 1;
    launch_gemm<double>(gcfg<double>(c, 1), EPI_DIV_TAB, a2, s);
    launch_gemm<double>(gcfg<double>(c, 0), EPI_STORE, gargs<double>(c, nz, nr, nr, c->t2, nr, c->m3xT, nr, c->t1, nr, nullptr, G_ALWAYS), s);
    auto a4 = gargs<double>(c, nz, nr, nz, c->m3z, nz, c->t1, nr, out, 0, nullptr, G_ALWAYS);
    a4.scale = 4.0 * nr * nz;
    launch_gemm<double>(gcfg<double>(c, 1), EPI_PRE_FINAL, a4, s);
    launch_fill_neumann(nr, nz, out, nullptr, c->ctr, s);
}

void enq_mass(drd_ctx* c, const double* ph, cudaStream_t s) {
    Dots d = dots(c);
    launch_mass_partial(c->nr, c->nz, ph, d, 0, c->ctr, s);
    launch_mass_final(d, 0, c->P.dr * c->P.dz, c->d_mass, c->ctr, s);
}

PartParams part_params(const drd_ctx* c) {
    PartParams q{};
    q.np = c->pp.np; q.nr = c->nr; q.nz = c->nz;
    q.lx = c->pp.lx; q.ly = c->pp.ly; q.radius = c->pp.fpd_radius; q.l0 = c->pp.l0;
    q.ks = c->pp.ks; q.kb = c->pp.kb; q.theta0 = c->pp.theta0;
    q.k0 = c->pp.k0_inter; q.k0b = c->pp.k0_inter_bdr; q.eq_pp = c->pp.fpd_fpd_dist; q.eq_bdr = c->pp.fpd_bdr_dist;
    q.dr = c->P.dr; q.dz = c->P.dz; q.eps = c->P.I_thickness; q.dt = c->P.dt;
    q.lambda_rho = c->P.lambda_rho; q.lambda_eta = c->P.lambda_eta;
    const double cut = c->pp.fpd_radius + 20.0 * std::sqrt(2.0) * c->P.I_thickness;
    q.skip_d2 = cut * cut;
    return q;
}

// The particle block of the mcl6 loop (mcl6.f90:394-402).  PT_FORCE: force_caculation_vel
// (tot_F, particle_force1/2 at the positions on entry); PT_MOVE: update_position_vel with u, v;
// PT_COEF: interpolate_coef at the positions after the move.
enum { PT_FORCE = 1, PT_MOVE = 2, PT_COEF = 4 };
void enq_particles(drd_ctx* c, int what, const double* u, const double* v, cudaStream_t s) {
    const PartParams q = part_params(c);
    if (q.np > 0 && (what & (PT_FORCE | PT_MOVE))) {
        if (what & PT_FORCE) launch_pt_force(q, c->pts, c->pts_old, c->totF, c->bdist, c->ctr, s);
        launch_pt_sums(q, c->pts, (what & PT_MOVE) ? u : nullptr, (what & PT_MOVE) ? v : nullptr, c->ppart, c->ctr, s);
        launch_pt_finish(q, c->ppart, c->psum, c->pts, (what & PT_MOVE) ? 1 : 0, c->ctr, s);
    }
    const int mode = ((what & PT_FORCE) && q.np > 0 ? 1 : 0) | ((what & PT_COEF) ? 2 : 0);
    if (mode)
        launch_pt_spread(q, mode, c->pts_old, c->pts, c->totF, c->psum, c->bdr, c->fld[DRD_F_PF1], c->fld[DRD_F_PF2],
                         c->fpd, c->rho, c->eta, c->rho32, c->eta32, c->ctr, s);
}

// The mcl6 step (microfluidics_complex_domain/mcl6.f90:239-306 first, :378-486 loop).
// extrap: 0 = x^n, 1 = linear, 2 = quadratic extrapolation of the solves' initial guesses.
int enq_step(drd_ctx* c, int first, int extrap, cudaStream_t s) {
    double** f = c->fld;
    const size_t cb = sizeof(double) * c->cs, ub = sizeof(double) * c->us, vb = sizeof(double) * c->vs;
    int rc = (c->P.variant == DRD_VARIANT_TP) ? enq_phmu(c, s, extrap != 0) : enq_ch(c, s, extrap);
    if (rc) return rc;
    if (c->pp.np > 0) enq_particles(c, PT_FORCE | PT_MOVE | PT_COEF, f[DRD_F_U], f[DRD_F_V], s);
    // interpolate_coef's place in the loop (mcl6.f90:401, :254): the two-fluid coefficients
    // from ph before the swap
    if (c->P.two_fluid)
        launch_two_phase_coef(c->dp, c->cs, c->fpd, f[DRD_F_PH], c->rho, c->eta, c->rho32, c->eta32, c->ctr, s);
    rc = enq_uv(c, first ? 1 : 2, s, extrap);
    if (rc) return rc;
    if (c->P.guess_mode == 3) {  // the fields three steps back, for the next step's guess
        CK(cudaMemcpyAsync(c->u_pre3, c->u_pre2, ub, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(c->v_pre3, c->v_pre2, vb, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(c->rmu_pre3, c->rmu_pre2, cb, cudaMemcpyDeviceToDevice, s));
    }
    if (c->P.guess_mode >= 2) {  // the fields two steps back
        CK(cudaMemcpyAsync(c->u_pre2, f[DRD_F_U_PRE], ub, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(c->v_pre2, f[DRD_F_V_PRE], vb, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(c->rmu_pre2, f[DRD_F_RMU_PRE], cb, cudaMemcpyDeviceToDevice, s));
    }
    CK(cudaMemcpyAsync(f[DRD_F_U_PRE], f[DRD_F_U], ub, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(f[DRD_F_V_PRE], f[DRD_F_V], vb, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(f[DRD_F_U], c->u_after, ub, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(f[DRD_F_V], c->v_after, vb, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(f[DRD_F_PH_PRE], f[DRD_F_PH], cb, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(f[DRD_F_RMU_PRE], f[DRD_F_RMU], cb, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(f[DRD_F_PH], c->ph_after, cb, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(f[DRD_F_RMU], c->rmu_after, cb, cudaMemcpyDeviceToDevice, s));
    if (!first) CK(cudaMemcpyAsync(f[DRD_F_PSI1], f[DRD_F_PSI2], cb, cudaMemcpyDeviceToDevice, s));
    enq_pre(c, f[DRD_F_PSI2], s);
    launch_cell_add(c->cs, f[DRD_F_PSI2], f[DRD_F_P], c->ctr, s);
    enq_mass(c, f[DRD_F_PH], s);
    return DRD_OK;
}

// Graph keys
enum GraphKind { GK_CH = 1, GK_UV = 2, GK_PHMU = 3, GK_PRE = 4, GK_STEP = 5, GK_ORI = 6, GK_SOLVE = 7 };
long gkey(int kind, int a, int b) { return (long)kind * 100 + a * 10 + b; }

int get_graph(drd_ctx* c, long key, const std::function<int(cudaStream_t)>& build, cudaGraphExec_t* out) {
    auto it = c->graphs.find(key);
    if (it != c->graphs.end()) { *out = it->second; return DRD_OK; }
    CK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    int rc = build(c->s);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->s, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { c->err = std::string("capture: ") + cudaGetErrorString(e); return DRD_ERR_CUDA; }
    cudaGraphExec_t ex;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { c->err = std::string("instantiate: ") + cudaGetErrorString(e); return DRD_ERR_CUDA; }
    c->graphs[key] = ex;
    *out = ex;
    return DRD_OK;
}

void clear_graphs(drd_ctx* c) {
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
}

// ---- GEMM tile autotuner: times each tile configuration on the context's transform shapes --
template <typename T>
int tune_pass(drd_ctx* c, int zpass, int lo, int hi, int extra = -1) {
    const int nr = c->nr, nz = c->nz;
    const char* env = std::getenv("DRD_GEMM_CFG");
    if (env) { int v = std::atoi(env); if ((v >= lo && v < hi) || v == extra) return v; }
    int best = lo;
    float best_ms = 1e30f;
    T* t1 = tmp1<T>(c);
    T* t2 = tmp2<T>(c);
    for (int i = lo; i < hi + (extra >= 0 ? 1 : 0); ++i) {
        const int cfg = i < hi ? i : extra;
        auto a = zpass ? dct1_zpass<T>(c, t1, t2, nullptr, G_ALWAYS) : dct1_xpass<T>(c, t1, t2, nullptr, G_ALWAYS);
        a.ctr = nullptr;
        launch_gemm<T>(cfg, EPI_STORE, a, c->s);  // warm-up
        cudaEventRecord(c->tev0, c->s);
        for (int r = 0; r < 5; ++r) launch_gemm<T>(cfg, EPI_STORE, a, c->s);
        cudaEventRecord(c->tev1, c->s);
        cudaEventSynchronize(c->tev1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->tev0, c->tev1);
        if (cudaGetLastError() != cudaSuccess) continue;
        if (ms < best_ms) { best_ms = ms; best = cfg; }
    }
    return best;
}

int ensure_tuned(drd_ctx* c) {
    if (c->gcfg[0][0] >= 0) return DRD_OK;
    CK(cudaMemsetAsync(c->t1, 0, sizeof(double) * c->nc, c->s));
    CK(cudaMemsetAsync(c->t1f, 0, sizeof(float) * c->nc, c->s));
    const int nx = gemm_config_count(0), nd = gemm_config_count(1);  // configs [nx, nd): double-float
    c->gcfg[0][0] = tune_pass<double>(c, 0, 0, nx);
    c->gcfg[0][1] = tune_pass<double>(c, 1, 0, nx);
    c->gcfg_df[0] = tune_pass<double>(c, 0, nx, nd);
    c->gcfg_df[1] = tune_pass<double>(c, 1, nx, nd);
    c->gcfg[1][0] = tune_pass<float>(c, 0, 0, nx, kGemmTcCfg);
    c->gcfg[1][1] = tune_pass<float>(c, 1, 0, nx, kGemmTcCfg);
    CK(cudaStreamSynchronize(c->s));
    return DRD_OK;
}

int run_graph(drd_ctx* c, long key, const std::function<int(cudaStream_t)>& build, double t, double coef) {
    int rc = ensure_tuned(c);
    if (rc) return rc;
    c->h_ca->t = t;
    c->h_ca->cf = 1.0 - std::exp(-t / c->P.twall);
    c->h_ca->coef = coef;
    CK(cudaMemcpyAsync(c->ca, c->h_ca, sizeof(CallArgs), cudaMemcpyHostToDevice, c->s));
    if (!c->use_graph) return build(c->s);  // direct launches (DRD_DIRECT_LAUNCH=1)
    cudaGraphExec_t ex;
    rc = get_graph(c, key, build, &ex);
    if (rc == DRD_ERR_CUDA && c->persist) {
        // a graph that cannot hold the cooperative inner solver: record why, use the graph loop
        c->persist_err = c->err;
        c->persist = 0;
        cudaGetLastError();
        clear_graphs(c);
        rc = get_graph(c, key, build, &ex);
    }
    if (rc) return rc;
    CK(cudaGraphLaunch(ex, c->s));
    return DRD_OK;
}

void fill_status(drd_ctx* c, int slot, const KState& k, drd_status* st, double secs) {
    if (!st) return;
    const int mixed = mixed_for(c, slot);
    st->info = k.info;
    st->iter = mixed ? k.inner_total : k.iter;
    st->resid = k.resid;
    st->true_resid = k.true_resid;
    st->refinements = mixed ? k.outer : 0;
    st->flags = k.flags;
    if (mixed_of(c) && !mixed) st->flags |= DRD_FLAG_FALLBACK64;
    st->seconds = secs;
}

int check_ctx(drd_ctx* c) { return c ? DRD_OK : DRD_ERR_BADARG; }

int up(drd_ctx* c, double* dst, const double* src, long n) {
    if (!src) return DRD_OK;
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, c->s));
    return DRD_OK;
}
int down(drd_ctx* c, double* dst, const double* src, long n) {
    if (!dst) return DRD_OK;
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
    return DRD_OK;
}

// The host ranges page-locked and mapped through drd_host_register: start -> (bytes, device
// address of start).  A per-routine call looks its arrays up here, without a driver call.
struct HostRange {
    size_t bytes;
    char* dev;
};
std::mutex g_host_mu;
std::map<uintptr_t, HostRange> g_host_ranges;

// The device address of host array [p, p + n) when the whole range lies in one range
// registered by drd_host_register, else null.
double* mapped_range(const double* p, long n) {
    if (n <= 0) return nullptr;
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    std::lock_guard<std::mutex> lock(g_host_mu);
    auto it = g_host_ranges.upper_bound(a);
    if (it == g_host_ranges.begin()) return nullptr;
    --it;
    if (a + sizeof(double) * (size_t)n > it->first + it->second.bytes) return nullptr;
    return reinterpret_cast<double*>(it->second.dev + (a - it->first));
}

// Host-to-device copy of a per-routine call's input: queued for the call's one gather launch
// (flush_up) when the host array is mapped, page-locked memory, else an immediate DMA copy.  The
// queue must be flushed before any work that reads dst.
int up_q(drd_ctx* c, double* dst, const double* src, long n) {
    if (!src) return DRD_OK;
    HostCopies& h = c->hq_up;
    const double* m = h.n < kHostCopyMax ? mapped_range(src, n) : nullptr;
    if (!m) return up(c, dst, src, n);
    h.src[h.n] = m;
    h.dst[h.n] = dst;
    h.len[h.n] = n;
    ++h.n;
    return DRD_OK;
}
// Device-to-host copy of a call's output, queued likewise (flush_down after the work that
// writes src).
int down_q(drd_ctx* c, double* dst, const double* src, long n) {
    if (!dst) return DRD_OK;
    HostCopies& h = c->hq_down;
    double* m = h.n < kHostCopyMax ? mapped_range(dst, n) : nullptr;
    if (!m) return down(c, dst, src, n);
    h.src[h.n] = src;
    h.dst[h.n] = m;
    h.len[h.n] = n;
    ++h.n;
    return DRD_OK;
}
int flush_q(drd_ctx* c, HostCopies& h) {
    launch_host_copies(h, c->ctr, c->s);
    h.n = 0;
    CK(cudaGetLastError());
    return DRD_OK;
}
void reset_q(drd_ctx* c) { c->hq_up.n = c->hq_down.n = 0; }

int refresh_fp32(drd_ctx* c) {
    launch_convert_scale<float, double>(c->cs, c->rho, 1.0, c->rho32, nullptr, c->s);
    launch_convert_scale<float, double>(c->cs, c->eta, 1.0, c->eta32, nullptr, c->s);
    launch_convert_scale<float, double>(c->cs, c->pen, 1.0, c->pen32, nullptr, c->s);
    launch_convert_scale<float, double>(c->cs, c->M0, 1.0, c->M032, nullptr, c->s);
    launch_convert_scale<float, double>(c->cs, c->Mi, 1.0, c->Mi32, nullptr, c->s);
    launch_convert_scale<float, double>(c->cs, c->used, 1.0, c->used32, nullptr, c->s);
    CK(cudaGetLastError());
    return DRD_OK;
}

// FP32 rounding of the preconditioned direction, |z| 2^-24 spread over all modes by the last
// DCT-I (a length-K sum: about sqrt(K) roundings), comes back multiplied by the CH operator's
// largest eigenvalue, which the table's largest entry estimates.  Measured on GB300: with this
// estimate at 0.004 (420x180), 0.031, 0.040 and 0.069 the mixed CH solves reach 1e-8; at 0.169
// (1400x600) and 0.42 (2048x1024) the FP64 refinement stalls or diverges.  Above 0.1 the mixed
// mode solves the CH system with the FP64 solver.
constexpr double kChStiffLimit = 0.1;
// With the solid-blended preconditioner the FP32 inner solves of a stiffer system still converge
// (2048x1024, estimate 0.42: 269-296 iterations to the FP64 residual 1e-8 where PSolve_CG's
// diverged), so the limit is raised while weights are installed.
constexpr double kChStiffLimitBlend = 1.0;
// Whether the mixed mode solves the CH system with the FP64 solver: the stiffness estimate
// against the limit for the preconditioner in use (DRD_CH_STIFF_LIMIT in the environment
// replaces both limits).
void update_ch_mode(drd_ctx* c) {
    const char* sl = std::getenv("DRD_CH_STIFF_LIMIT");
    const double lim = sl ? std::atof(sl) : (c->pc_on ? kChStiffLimitBlend : kChStiffLimit);
    c->ch_fp64 = c->ch_stiff > lim;
}

double ch_stiffness(const drd_ctx* c, const std::vector<double>& ph_lcc) {
    double lmax = 0.0;
    for (double v : ph_lcc) lmax = std::max(lmax, v);
    return std::ldexp(1.0, -24) * std::sqrt((double)std::max(c->Kx, c->Kz)) * lmax;
}

int upload_tables(drd_ctx* c) {
    std::vector<double> ph, pre;
    host_tables(c->P, ph, pre);
    c->ch_stiff = ch_stiffness(c, ph);
    update_ch_mode(c);
    CK(cudaMemcpy(c->ph_lcc, ph.data(), sizeof(double) * ph.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->pre_lcc, pre.data(), sizeof(double) * pre.size(), cudaMemcpyHostToDevice));
    launch_convert_scale<float, double>(c->nc, c->ph_lcc, 1.0, c->ph_lcc32, nullptr, c->s);
    // FFT twiddles: tw[m] = e^(-2 pi i m/n), then tq[k] = e^(-i pi k/2n) (drd_fft.cuh).
    // DRD_PRESSURE_FFT=0 in the environment keeps the GEMM-form pressure transforms.
    const char* pe = std::getenv("DRD_PRESSURE_FFT");
    c->pfft_ok = pfft_fits(c->nr, c->nz, 8) && pfft_plan(c->nr, c->fpx) && pfft_plan(c->nz, c->fpz);
    c->pfft = c->pfft_ok && !(pe && pe[0] == '0');
    if (c->pfft_ok) {
        CK(pfft_prepare(c->nr, c->nz));
        for (int ax = 0; ax < 2; ++ax) {
            const int n = ax ? c->nz : c->nr;
            std::vector<double> t(4L * n);
            std::vector<float> t32(4L * n);
            for (int m = 0; m < n; ++m) {
                const double a = -2.0 * kPi * m / n, b = -kPi * m / (2.0 * n);
                t[2 * m] = std::cos(a); t[2 * m + 1] = std::sin(a);
                t[2 * (n + m)] = std::cos(b); t[2 * (n + m) + 1] = std::sin(b);
            }
            for (size_t q = 0; q < t.size(); ++q) t32[q] = (float)t[q];
            CK(cudaMemcpy(ax ? c->ftwz : c->ftwx, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(ax ? c->ftwz32 : c->ftwx32, t32.data(), sizeof(float) * t32.size(), cudaMemcpyHostToDevice));
        }
    }
    for (int bdf = 1; bdf <= 2; ++bdf) {
        std::vector<double> f;
        host_esolp(c->P, bdf, f);
        CK(cudaMemcpy(c->es64[bdf - 1], f.data(), sizeof(double) * f.size(), cudaMemcpyHostToDevice));
        launch_convert_scale<float, double>((long)f.size(), c->es64[bdf - 1], 1.0, c->es32[bdf - 1], nullptr, c->s);
        // r_j, 1/b'_j (0 at the last row when |b'| <= 1e-12, as rfords' back substitution), c_j/b'_j
        std::vector<float> q(f.size());
        const long mu = (long)(c->nr + 1) * c->nz, mv = (long)c->nr * (c->nz - 1);
        for (int blk = 0; blk < 2; ++blk) {
            const long base = blk ? 3 * mu : 0, rb = blk ? mv : mu;
            const int len = blk ? c->nr : c->nr + 1, rows = blk ? c->nz - 1 : c->nz;
            for (long e = 0; e < rb; ++e) {
                const long j = e / len;
                const double rm = f[base + e], bp = f[base + rb + e], cc = f[base + 2 * rb + e];
                const bool last = j == rows - 1;
                q[base + e] = (float)rm;
                q[base + rb + e] = (float)((last && std::fabs(bp) <= 1.0E-12) ? 0.0 : 1.0 / bp);
                q[base + 2 * rb + e] = (float)(last ? 0.0 : cc / bp);
            }
        }
        CK(cudaMemcpy(c->esq32[bdf - 1], q.data(), sizeof(float) * q.size(), cudaMemcpyHostToDevice));
    }
    CK(cudaStreamSynchronize(c->s));
    return DRD_OK;
}

int setup_context(drd_ctx* c) {
    const int nr = c->nr, nz = c->nz;
    CK(cudaGetDevice(&c->device));
    CK(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->s2, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->s3, cudaStreamNonBlocking));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    CK(cudaEventCreate(&c->tev0));
    CK(cudaEventCreate(&c->tev1));
    c->arena_bytes = arena_need(c->cs, c->us, c->vs, c->nc, nr, nz, c->nmax);
    CK(cudaMalloc(&c->arena, c->arena_bytes));
    CK(cudaMemset(c->arena, 0, c->arena_bytes));
    double** cf[] = {&c->rho, &c->eta, &c->bdr, &c->grad, &c->M0, &c->Mi, &c->pen, &c->used};
    for (auto* pp : cf) *pp = carve<double>(c, c->cs);
    float** cf32[] = {&c->rho32, &c->eta32, &c->pen32, &c->M032, &c->Mi32, &c->used32};
    for (auto* pp : cf32) *pp = carve<float>(c, c->cs);
    c->ph_lcc = carve<double>(c, c->nc);
    c->pre_lcc = carve<double>(c, (long)(nr + 1) * (nz + 1));
    c->ph_lcc32 = carve<float>(c, c->nc);
    c->m2xT = carve<double>(c, (long)nr * nr); c->m2z = carve<double>(c, (long)nz * nz);
    c->m3xT = carve<double>(c, (long)nr * nr); c->m3z = carve<double>(c, (long)nz * nz);
    c->Kx = (nr - 1) / 2 + 1; c->Nxe = (nr + 1) / 2; c->Nxo = nr / 2;
    c->Kz = (nz - 1) / 2 + 1; c->Mze = (nz + 1) / 2; c->Mzo = nz / 2;
    const long fx = (long)c->Kx * c->Nxe, fz = (long)c->Mze * c->Kz;
    c->f1xe = carve<double>(c, fx); c->f1xo = carve<double>(c, fx);
    c->f1ze = carve<double>(c, fz); c->f1zo = carve<double>(c, fz);
    c->f1xe32 = carve<float>(c, fx); c->f1xo32 = carve<float>(c, fx);
    c->f1ze32 = carve<float>(c, fz); c->f1zo32 = carve<float>(c, fz);
    c->cfB = carve<double>(c, nr + 1); c->cfT = carve<double>(c, nr + 1);
    for (int f = 0; f < DRD_F_COUNT; ++f) c->fld[f] = carve<double>(c, std::max(c->us, c->cs));
    c->u_after = carve<double>(c, c->us); c->v_after = carve<double>(c, c->vs);
    c->ph_after = carve<double>(c, c->cs); c->rmu_after = carve<double>(c, c->cs); c->f2 = carve<double>(c, c->cs);
    c->uL = carve<double>(c, nz + 1); c->pnb = carve<double>(c, nr); c->pnt = carve<double>(c, nr);
    c->dist = carve<double>(c, c->nc); c->fpd = carve<double>(c, c->cs); c->w = carve<double>(c, c->nc);
    c->t1 = carve<double>(c, c->nc); c->t2 = carve<double>(c, c->nc);
    c->t1f = carve<float>(c, c->nc); c->t2f = carve<float>(c, c->nc);
    c->k64 = carve_vecs<double>(c);
    c->k32 = carve_vecs<float>(c);
    c->part = carve<double>(c, DRD_NDOT * DRD_MAXB);
    c->ks = (KState*)carve<char>(c, KS_COUNT * sizeof(KState));
    c->ca = (CallArgs*)carve<char>(c, sizeof(CallArgs));
    c->d_mass = carve<double>(c, 1);
    c->tcerr = (int*)carve<double>(c, 1);
    c->ctr = (unsigned long long*)carve<double>(c, 1);
    c->pts = carve<double>(c, 2 * DRD_PARTICLES_MAX); c->pts_old = carve<double>(c, 2 * DRD_PARTICLES_MAX);
    c->totF = carve<double>(c, 2 * DRD_PARTICLES_MAX); c->psum = carve<double>(c, 2 * DRD_PARTICLES_MAX);
    c->ppart = carve<double>(c, 3 * DRD_PARTICLES_MAX * PT_GX); c->bdist = carve<double>(c, c->cs);
    c->ori_cfb = carve<double>(c, nr + 1); c->ori_cft = carve<double>(c, nr + 1);
    c->rmu_prev = carve<double>(c, c->cs); c->rmu_prev2 = carve<double>(c, c->cs); c->rmu_prev3 = carve<double>(c, c->cs);
    c->rmu_pre2 = carve<double>(c, c->cs); c->u_pre2 = carve<double>(c, c->us); c->v_pre2 = carve<double>(c, c->vs);
    c->rmu_pre3 = carve<double>(c, c->cs); c->u_pre3 = carve<double>(c, c->us); c->v_pre3 = carve<double>(c, c->vs);
    c->bar = (GridBar*)carve<char>(c, sizeof(GridBar));
    c->pprof = (unsigned long long*)carve<double>(c, 128);
    c->d_diag = carve<double>(c, 8);
    c->ftwx = carve<double>(c, 4L * nr); c->ftwz = carve<double>(c, 4L * nz);
    c->ftwx32 = carve<float>(c, 4L * nr); c->ftwz32 = carve<float>(c, 4L * nz);
    c->Ku = nr / 2 + 1; c->Nue = (nr + 2) / 2; c->Nuo = (nr + 1) / 2;
    const long fu = (long)c->Ku * c->Nue, nes = 3 * ((long)(nr + 1) * nz + (long)nr * (nz - 1));
    c->f1ue = carve<double>(c, fu); c->f1uo = carve<double>(c, fu);
    c->f1ue32 = carve<float>(c, fu); c->f1uo32 = carve<float>(c, fu);
    for (int b = 0; b < 2; ++b) {
        c->es64[b] = carve<double>(c, nes);
        c->es32[b] = carve<float>(c, nes);
        c->esq32[b] = carve<float>(c, nes);
    }
    c->esw = carve<double>(c, c->nmax); c->esw32 = carve<float>(c, c->nmax);
    if (c->arena_used > c->arena_bytes) { c->err = "arena overflow"; return DRD_ERR_NOMEM; }
    CK(cudaMallocHost(&c->h_ks, KS_COUNT * sizeof(KState)));
    CK(cudaMallocHost(&c->h_ca, sizeof(CallArgs)));
    CK(cudaMallocHost(&c->h_mass, sizeof(double)));
    memset(c->h_ks, 0, KS_COUNT * sizeof(KState));
    memset(c->h_ca, 0, sizeof(CallArgs));
    // default coefficients: no solid, unit density / viscosity / mobility
    std::vector<double> ones(c->cs, 1.0), zeros(c->cs, 0.0);
    CK(cudaMemcpy(c->rho, ones.data(), sizeof(double) * c->cs, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->eta, ones.data(), sizeof(double) * c->cs, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->M0, ones.data(), sizeof(double) * c->cs, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->Mi, ones.data(), sizeof(double) * c->cs, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->used, ones.data(), sizeof(double) * c->cs, cudaMemcpyHostToDevice));
    // transform matrices: x-pass operands transposed (B[j][o] = D[o][j]), z-pass as is
    std::vector<double> d1, d2, d3, e1, e2, e3;
    host_dct_mats(nr, d1, d2, d3);
    host_dct_mats(nz, e1, e2, e3);
    auto put = [&](double* dst, const std::vector<double>& v) {
        return cudaMemcpy(dst, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice);
    };
    CK(put(c->m2xT, transpose(d2, nr)));
    CK(put(c->m3xT, transpose(d3, nr)));
    CK(put(c->m2z, e2));
    CK(put(c->m3z, e3));
    {
        // x pass B operands: B_p[j][n] = D1x[2n+p][j]; z pass A operands: A_p[m][j] = D1z[2m+p][j]
        std::vector<double> xe((size_t)c->Kx * c->Nxe, 0.0), xo(xe.size(), 0.0);
        for (int j = 0; j < c->Kx; ++j)
            for (int n = 0; n < c->Nxe; ++n) {
                xe[(size_t)j * c->Nxe + n] = d1[(size_t)(2 * n) * nr + j];
                if (n < c->Nxo) xo[(size_t)j * c->Nxe + n] = d1[(size_t)(2 * n + 1) * nr + j];
            }
        std::vector<double> ze((size_t)c->Mze * c->Kz, 0.0), zo(ze.size(), 0.0);
        for (int m = 0; m < c->Mze; ++m)
            for (int j = 0; j < c->Kz; ++j) {
                ze[(size_t)m * c->Kz + j] = e1[(size_t)(2 * m) * nz + j];
                if (m < c->Mzo) zo[(size_t)m * c->Kz + j] = e1[(size_t)(2 * m + 1) * nz + j];
            }
        CK(put(c->f1xe, xe));
        CK(put(c->f1xo, xo));
        CK(put(c->f1ze, ze));
        CK(put(c->f1zo, zo));
        launch_convert_scale<float, double>((long)xe.size(), c->f1xe, 1.0, c->f1xe32, nullptr, c->s);
        launch_convert_scale<float, double>((long)xo.size(), c->f1xo, 1.0, c->f1xo32, nullptr, c->s);
        launch_convert_scale<float, double>((long)ze.size(), c->f1ze, 1.0, c->f1ze32, nullptr, c->s);
        launch_convert_scale<float, double>((long)zo.size(), c->f1zo, 1.0, c->f1zo32, nullptr, c->s);
        // ESOLP_x u block: VCOST of length nr+1, the same folded x-pass operands
        const int L = nr + 1;
        std::vector<double> g1, g2, g3;
        host_dct_mats(L, g1, g2, g3);
        std::vector<double> ue((size_t)c->Ku * c->Nue, 0.0), uo(ue.size(), 0.0);
        for (int j = 0; j < c->Ku; ++j)
            for (int n = 0; n < c->Nue; ++n) {
                ue[(size_t)j * c->Nue + n] = g1[(size_t)(2 * n) * L + j];
                if (n < c->Nuo) uo[(size_t)j * c->Nue + n] = g1[(size_t)(2 * n + 1) * L + j];
            }
        CK(put(c->f1ue, ue));
        CK(put(c->f1uo, uo));
        launch_convert_scale<float, double>((long)ue.size(), c->f1ue, 1.0, c->f1ue32, nullptr, c->s);
        launch_convert_scale<float, double>((long)uo.size(), c->f1uo, 1.0, c->f1uo32, nullptr, c->s);
    }
    {
        // the tensor-core GEMM's packed constant operands (TF32 hi / lo, shared-memory block order)
        auto pack = [&](const float* ev, const float* od, int re, int ro, int K, long ld, int bst, float** out,
                        int* tiles, int* chunks) -> int {
            const long n = gemm_tc_pack(ev, od, re, ro, K, ld, bst, nullptr, tiles, chunks, c->s);
            CK(cudaMalloc(out, sizeof(float) * n));
            gemm_tc_pack(ev, od, re, ro, K, ld, bst, *out, nullptr, nullptr, c->s);
            return DRD_OK;
        };
        // the pre-folded operand: even and odd rows of up to nz + 1 rows (the u block) of the
        // longest folded row rounded up to 4 values
        const int kmax = std::max(c->Kx, c->Ku);
        c->tc_pad_cap = 2L * (nz + 1) * ((kmax + 3) & ~3);
        CK(cudaMalloc(&c->tc_pad, sizeof(float) * c->tc_pad_cap));
        int rc = pack(c->f1xe32, c->f1xo32, c->Nxe, c->Nxo, c->Kx, c->Nxe, 1, &c->pk_x, &c->pkx_t, &c->pkx_c);
        rc |= pack(c->f1ze32, c->f1zo32, c->Mze, c->Mzo, c->Kz, c->Kz, 0, &c->pk_z, &c->pkz_t, &c->pkz_c);
        rc |= pack(c->f1ue32, c->f1uo32, c->Nue, c->Nuo, c->Ku, c->Nue, 1, &c->pk_u, &c->pku_t, &c->pku_c);
        if (rc) return DRD_ERR_CUDA;
        CK(cudaGetLastError());
    }
    std::vector<double> cfa(nr + 1, std::cos(c->P.angle * kPi / 180.0) / std::sqrt(2.0));
    CK(put(c->cfB, cfa));
    CK(put(c->cfT, cfa));
    int rc = upload_tables(c);
    if (rc) return rc;
    rc = setup_persist(c);
    if (rc) return rc;
    rc = refresh_fp32(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->s));
    // DRD_DIRECT_LAUNCH=1 launches every kernel directly on the stream with the Krylov loops
    // run by the host (for per-kernel profilers and debugging); the default is one CUDA graph
    // per routine or step with device-side WHILE loops.
    const char* g = std::getenv("DRD_DIRECT_LAUNCH");
    c->use_graph = !(g && g[0] == '1');
    return DRD_OK;
}

int validate(const drd_params* p, std::string& why) {
    if (!p) { why = "params is NULL"; return DRD_ERR_BADARG; }
    if (p->nr < 3 || p->nz < 3) { why = "nr and nz must be >= 3"; return DRD_ERR_BADARG; }
    if ((long)p->nr * p->nz > (1L << 26)) { why = "grid too large"; return DRD_ERR_BADARG; }
    if (!(p->dr > 0) || !(p->dz > 0) || !(p->dt > 0)) { why = "dr, dz, dt must be positive"; return DRD_ERR_BADARG; }
    if (!(p->I_thickness > 0)) { why = "I_thickness must be positive"; return DRD_ERR_BADARG; }
    if (p->variant != DRD_VARIANT_MF && p->variant != DRD_VARIANT_TP) { why = "unknown variant"; return DRD_ERR_BADARG; }
    if (p->precision != DRD_PREC_FP64 && p->precision != DRD_PREC_MIXED) { why = "unknown precision"; return DRD_ERR_BADARG; }
    if (p->variant == DRD_VARIANT_TP && p->phi_mode != 1 && p->phi_mode != 2) { why = "phi_mode must be 1 or 2"; return DRD_ERR_BADARG; }
    if (p->ch_maxit <= 0 || p->uv_maxit <= 0 || p->phmu_maxit <= 0) { why = "maxit must be positive"; return DRD_ERR_BADARG; }
    if (p->xlsB >= 1.e-8) { why = "slip walls (xlsB >= 1e-8) have no solve in the reference"; return DRD_ERR_UNSUPPORTED; }
    if (p->guess_mode < 0 || p->guess_mode > 3) { why = "guess_mode must be 0 to 3"; return DRD_ERR_BADARG; }
    if (p->uv_precond != DRD_UV_JACOBI && p->uv_precond != DRD_UV_ESOLP && p->uv_precond != DRD_UV_ESOLP_SCALED) {
        why = "unknown uv_precond";
        return DRD_ERR_BADARG;
    }
    if (p->uv_precond == DRD_UV_ESOLP_SCALED && p->variant != DRD_VARIANT_MF) {
        why = "DRD_UV_ESOLP_SCALED scales by VeloSolve_2_combined's (MF) Jacobi diagonal";
        return DRD_ERR_UNSUPPORTED;
    }
    if (p->two_fluid != 0 && p->two_fluid != 1) { why = "two_fluid must be 0 or 1"; return DRD_ERR_BADARG; }
    if (p->precision == DRD_PREC_MIXED && (!(p->mixed_inner_tol > 0) || p->mixed_max_refine <= 0)) {
        why = "mixed precision needs mixed_inner_tol > 0 and mixed_max_refine > 0";
        return DRD_ERR_BADARG;
    }
    return DRD_OK;
}

int finish_call(drd_ctx* c, int slot, drd_status* st, bool has_solve) {
    if (has_solve) CK(cudaMemcpyAsync(c->h_ks + slot, c->ks + slot, sizeof(KState), cudaMemcpyDeviceToHost, c->s));
    CK(cudaEventRecord(c->ev1, c->s));
    CK(cudaStreamSynchronize(c->s));
    CK(cudaGetLastError());
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    if (has_solve) {
        fill_status(c, slot, c->h_ks[slot], st, ms * 1e-3);
        return c->h_ks[slot].info;
    }
    if (st) { memset(st, 0, sizeof(*st)); st->seconds = ms * 1e-3; }
    return DRD_OK;
}

extern "C" int set_ori_walls(drd_ctx* c, const double* angleB, const double* angleT, double alpha_s);

// finit's wall smoothing (finit.f90:120-189; reinint_by_PhSolve.f90:12-70 repeats it): ph =
// bdr_in with Neumann ghosts, rmu from ph, nsteps PhSolve_ori steps, then the clipped
// (ph + 1)/2 in c->w.
int wall_smoothing(drd_ctx* c, const double* bdr_in, int nsteps, double* bdr_out, double* ph_out, double* rmu_out) {
    int rc = set_ori_walls(c, nullptr, nullptr, 0.0);
    if (rc) return rc;
    double* ph = c->fld[DRD_F_PH];
    double* rmu = c->fld[DRD_F_RMU];
    const size_t cb = sizeof(double) * c->cs;
    if (up(c, ph, bdr_in, c->cs)) return DRD_ERR_CUDA;                   // finit.f90:123-133
    launch_fill_neumann(c->nr, c->nz, ph, nullptr, c->ctr, c->s);
    CK(cudaMemsetAsync(c->fld[DRD_F_U], 0, sizeof(double) * c->us, c->s));  // u = v = 0 (mcl6.f90:143)
    CK(cudaMemsetAsync(c->fld[DRD_F_V], 0, sizeof(double) * c->vs, c->s));
    CK(cudaMemsetAsync(rmu, 0, cb, c->s));
    launch_ori_rmu0(c->dp, ph, rmu, c->ctr, c->s);                        // finit.f90:163-169
    int info = 0;
    for (int it = 0; it < nsteps; ++it) {                                 // finit.f90:172-176
        rc = run_graph(c, gkey(GK_ORI, mixed_of(c), 0), [&](cudaStream_t s) { return enq_ori(c, s); }, 0.0, 0.0);
        if (rc) return rc;
        CK(cudaMemcpyAsync(rmu, c->rmu_after, cb, cudaMemcpyDeviceToDevice, c->s));
        CK(cudaMemcpyAsync(ph, c->ph_after, cb, cudaMemcpyDeviceToDevice, c->s));
    }
    launch_ori_bdr(c->nr, c->nz, ph, c->w, c->ctr, c->s);                 // finit.f90:178-189
    CK(cudaGetLastError());
    if (down(c, bdr_out, c->w, c->cs) | down(c, ph_out, ph, c->cs) | down(c, rmu_out, rmu, c->cs)) return DRD_ERR_CUDA;
    CK(cudaMemcpyAsync(c->h_ks + KS_CH, c->ks + KS_CH, sizeof(KState), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    if (nsteps > 0) info = c->h_ks[KS_CH].info;
    return info;
}

}  // namespace

// ============================================================================================
// extern "C"
// ============================================================================================
extern "C" {

int drd_abi_version(void) { return DRD_ABI_VERSION; }

int drd_create(const drd_params* params, drd_ctx** out) {
    if (!out) return DRD_ERR_BADARG;
    *out = nullptr;
    std::string why;
    int rc = validate(params, why);
    if (rc) { std::fprintf(stderr, "drd_create: %s\n", why.c_str()); return rc; }
    drd_ctx* c = new drd_ctx();
    c->P = *params;
    c->dp = make_dev_params(c->P);
    c->nr = params->nr;
    c->nz = params->nz;
    c->cs = (long)(c->nr + 2) * (c->nz + 2);
    c->us = (long)(c->nr + 3) * (c->nz + 2);
    c->vs = (long)(c->nr + 2) * (c->nz + 1);
    c->nc = (long)c->nr * c->nz;
    c->nuv = (long)(c->nr + 1) * c->nz + (long)c->nr * (c->nz - 1);
    c->nphmu = 2 * c->nc;
    c->nmax = std::max(c->nuv, c->nphmu);
    long g = (c->nmax + 2L * DRD_TPB - 1) / (2L * DRD_TPB);
    c->G = (int)std::max(1L, std::min<long>(DRD_MAXB, g));
    rc = setup_context(c);
    if (rc) {
        std::fprintf(stderr, "drd_create: %s\n", c->err.c_str());
        drd_destroy(c);
        return rc;
    }
    *out = c;
    return DRD_OK;
}

int drd_destroy(drd_ctx* c) {
    if (!c) return DRD_ERR_BADARG;
    if (c->ckpt.joinable()) c->ckpt.join();
    if (c->s) cudaStreamSynchronize(c->s);
    if (c->sck) cudaStreamDestroy(c->sck);
    if (c->eck0) cudaEventDestroy(c->eck0);
    if (c->eck1) cudaEventDestroy(c->eck1);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    clear_graphs(c);
    if (c->arena) cudaFree(c->arena);
    if (c->pk_x) cudaFree(c->pk_x);
    if (c->pk_z) cudaFree(c->pk_z);
    if (c->pk_u) cudaFree(c->pk_u);
    if (c->tc_pad) cudaFree(c->tc_pad);
    if (c->pcw) cudaFree(c->pcw);
    if (c->pcw32) cudaFree(c->pcw32);
    if (c->pnum) cudaFree(c->pnum);
    if (c->pden) cudaFree(c->pden);
    if (c->h_ks) cudaFreeHost(c->h_ks);
    if (c->h_ca) cudaFreeHost(c->h_ca);
    if (c->h_mass) cudaFreeHost(c->h_mass);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->tev0) cudaEventDestroy(c->tev0);
    if (c->tev1) cudaEventDestroy(c->tev1);
    if (c->s) cudaStreamDestroy(c->s);
    if (c->s2) cudaStreamDestroy(c->s2);
    if (c->s3) cudaStreamDestroy(c->s3);
    delete c;
    return DRD_OK;
}

const char* drd_last_error(drd_ctx* c) { return c ? c->err.c_str() : "null context"; }

int drd_set_params(drd_ctx* c, const drd_params* p) {
    if (!c) return DRD_ERR_BADARG;
    std::string why;
    int rc = validate(p, why);
    if (rc) { c->err = why; return rc; }
    if (p->nr != c->nr || p->nz != c->nz) { c->err = "grid size cannot change"; return DRD_ERR_BADARG; }
    CK(cudaStreamSynchronize(c->s));
    c->P = *p;
    c->dp = make_dev_params(c->P);
    clear_graphs(c);
    rc = upload_tables(c);
    if (rc) return rc;
    std::vector<double> cfa(c->nr + 1, std::cos(c->P.angle * kPi / 180.0) / std::sqrt(2.0));
    CK(cudaMemcpy(c->cfB, cfa.data(), sizeof(double) * cfa.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->cfT, cfa.data(), sizeof(double) * cfa.size(), cudaMemcpyHostToDevice));
    return DRD_OK;
}

int drd_set_coefs(drd_ctx* c, const double* rho, const double* eta, const double* bdr_ph, const double* bdr_ph_grad,
                  const double* ph_M_0, const double* ph_M_inner) {
    if (!c) return DRD_ERR_BADARG;
    int rc = 0;
    rc |= up(c, c->rho, rho, c->cs);
    rc |= up(c, c->eta, eta, c->cs);
    rc |= up(c, c->bdr, bdr_ph, c->cs);
    rc |= up(c, c->grad, bdr_ph_grad, c->cs);
    rc |= up(c, c->M0, ph_M_0, c->cs);
    rc |= up(c, c->Mi, ph_M_inner, c->cs);
    if (rc) return DRD_ERR_CUDA;
    // blend weights belong to the mobilities they were fitted for
    if ((ph_M_0 || ph_M_inner) && c->pc_on) {
        c->pc_on = 0;
        update_ch_mode(c);
        clear_graphs(c);
    }
    // MF penalises with bdr_ph itself (VeloSolve_2_combined.f90:580); TP keeps its own mask
    if (bdr_ph && c->P.variant == DRD_VARIANT_MF)
        CK(cudaMemcpyAsync(c->pen, c->bdr, sizeof(double) * c->cs, cudaMemcpyDeviceToDevice, c->s));
    rc = refresh_fp32(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->s));
    return DRD_OK;
}

// ---- the solid-blended CH preconditioner ----------------------------------------------------
int pc_alloc(drd_ctx* c) {
    if (c->pcw) return DRD_OK;
    CK(cudaMalloc(&c->pcw, sizeof(double) * c->nc));
    CK(cudaMalloc(&c->pcw32, sizeof(float) * c->nc));
    CK(cudaMalloc(&c->pnum, sizeof(double) * c->nc));
    CK(cudaMalloc(&c->pden, sizeof(double) * c->nc));
    return DRD_OK;
}

// Turns the blend on or off; the step and solve graphs hold the choice, so a change drops them.
void pc_switch(drd_ctx* c, int on) {
    if (c->pc_on == on) return;
    c->pc_on = on;
    update_ch_mode(c);
    clear_graphs(c);
}

int drd_set_ch_blend(drd_ctx* c, const double* w) {
    if (!c) return DRD_ERR_BADARG;
    if (c->P.variant != DRD_VARIANT_MF) { c->err = "the blended preconditioner belongs to PhSolve (MF)"; return DRD_ERR_UNSUPPORTED; }
    if (!w) { pc_switch(c, 0); return DRD_OK; }
    int rc = pc_alloc(c);
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->pcw, w, sizeof(double) * c->nc, cudaMemcpyDefault, c->s));
    launch_convert_scale<float, double>(c->nc, c->pcw, 1.0, c->pcw32, nullptr, c->s);
    CK(cudaStreamSynchronize(c->s));
    CK(cudaGetLastError());
    pc_switch(c, 1);
    return DRD_OK;
}

int drd_ch_blend_probe(drd_ctx* c, int nprobe, uint64_t seed, int install, double* w_out) {
    if (!c || nprobe < 1) return DRD_ERR_BADARG;
    if (c->P.variant != DRD_VARIANT_MF) { c->err = "the blended preconditioner belongs to PhSolve (MF)"; return DRD_ERR_UNSUPPORTED; }
    int rc = ensure_tuned(c);
    if (rc) return rc;
    rc = pc_alloc(c);
    if (rc) return rc;
    const long n = c->nc;
    Sys S = sys_of(c, SYS_CH, 0);
    KVecs<double>& k = c->k64;
    // the probes see the reference preconditioner alone: fit the weights, then install them
    for (int p = 0; p < nprobe; ++p) {
        launch_probe_fill(n, seed, p, k.tmp, c->ctr, c->s);
        enq_matvec<double>(c, S, 1.0, k.tmp, 0.0, k.v, nullptr, 0, 0, nullptr, G_ALWAYS, c->s);
        enq_ch_psolve<double>(c, k.v, k.phat, nullptr, G_ALWAYS, c->s);
        launch_probe_acc(n, seed, p, k.v, k.phat, c->pnum, c->pden, p == 0, c->ctr, c->s);
    }
    double* wd = install ? c->pcw : k.tmp;  // not installing: the probe vector's buffer holds the fit
    float* w32 = install ? c->pcw32 : c->k32.tmp;
    launch_probe_final(n, c->pnum, c->pden, wd, w32, c->ctr, c->s);
    if (w_out) CK(cudaMemcpyAsync(w_out, wd, sizeof(double) * n, cudaMemcpyDefault, c->s));
    CK(cudaStreamSynchronize(c->s));
    CK(cudaGetLastError());
    if (install) pc_switch(c, 1);
    return DRD_OK;
}

int drd_set_tp_fields(drd_ctx* c, const double* bdr_ph_used, const double* bdr_ph_penalty, const double* angleB,
                      const double* angleT) {
    if (!c) return DRD_ERR_BADARG;
    int rc = 0;
    rc |= up(c, c->used, bdr_ph_used, c->cs);
    rc |= up(c, c->pen, bdr_ph_penalty, c->cs);
    if (rc) return DRD_ERR_CUDA;
    auto cf = [&](double* dst, const double* ang) -> int {
        if (!ang) return DRD_OK;
        std::vector<double> v(c->nr + 1);
        for (int i = 0; i <= c->nr; ++i) v[i] = std::cos(ang[i] * kPi / 180.0) / std::sqrt(2.0);
        CK(cudaMemcpy(dst, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice));
        return DRD_OK;
    };
    rc = cf(c->cfB, angleB);
    if (rc) return rc;
    rc = cf(c->cfT, angleT);
    if (rc) return rc;
    rc = refresh_fp32(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->s));
    return DRD_OK;
}

int drd_interpolate_coef(drd_ctx* c, const double* dist, double* fpd_ph, double* rho, double* eta) {
    if (!c || !dist) return DRD_ERR_BADARG;
    CK(cudaEventRecord(c->ev0, c->s));
    if (up(c, c->dist, dist, c->nc)) return DRD_ERR_CUDA;
    launch_interp_coef(c->dp, c->dist, c->bdr, c->fpd, c->rho, c->eta, c->ctr, c->s);
    int rc = refresh_fp32(c);
    if (rc) return rc;
    rc = down(c, fpd_ph, c->fpd, c->cs) | down(c, rho, c->rho, c->cs) | down(c, eta, c->eta, c->cs);
    if (rc) return DRD_ERR_CUDA;
    return finish_call(c, 0, nullptr, false);
}

int drd_two_phase_coef(drd_ctx* c, const double* fpd_ph, const double* ph, double* rho, double* eta) {
    if (!c) return DRD_ERR_BADARG;
    reset_q(c);
    CK(cudaEventRecord(c->ev0, c->s));
    if (up_q(c, c->fpd, fpd_ph, c->cs)) return DRD_ERR_CUDA;
    const double* dph = c->fld[DRD_F_PH];
    if (ph) {
        if (up_q(c, c->ph_after, ph, c->cs)) return DRD_ERR_CUDA;  // scratch until the next solve
        dph = c->ph_after;
    }
    if (flush_q(c, c->hq_up)) return DRD_ERR_CUDA;
    launch_two_phase_coef(c->dp, c->cs, c->fpd, dph, c->rho, c->eta, c->rho32, c->eta32, c->ctr, c->s);
    CK(cudaGetLastError());
    if (down_q(c, rho, c->rho, c->cs) | down_q(c, eta, c->eta, c->cs) | flush_q(c, c->hq_down)) return DRD_ERR_CUDA;
    return finish_call(c, 0, nullptr, false);
}

int drd_particle_params_default(drd_particle_params* pp, double lx, double ly) {
    if (!pp) return DRD_ERR_BADARG;
    memset(pp, 0, sizeof(*pp));
    pp->np = 9;                                                 // particles_params.f90:78
    pp->lx = lx;
    pp->ly = ly;
    pp->fpd_radius = 0.05 / 2.0;                                // :80
    pp->l0 = 2 * (pp->fpd_radius + 0.00);                       // :83 (fpd_inter_dist = 0, :81)
    pp->ks = 5;                                                 // :74
    pp->kb = 0.0025 * 100;                                      // :75
    pp->theta0 = 0.0;                                           // :76
    pp->k0_inter = 2.5;                                         // :93
    pp->k0_inter_bdr = 2.5 * 10;                                // :94
    pp->fpd_fpd_dist = pp->fpd_radius + pp->fpd_radius + 0.01;  // :97
    pp->fpd_bdr_dist = pp->fpd_radius + 0.02;                   // :98
    return DRD_OK;
}

int drd_particle_initialize(const drd_particle_params* pp, double xc, double yc, double* points) {
    // particle_initialize, fibers: particles_move.f90:50-68
    if (!pp || !points || pp->np < 0 || pp->np > DRD_PARTICLES_MAX) return DRD_ERR_BADARG;
    const int np = pp->np;
    if (np > 2) {
        const int mid = (int)std::floor(np / 2.0);
        points[mid] = xc;
        points[np + mid] = yc;
        for (int i = 0; i < mid; ++i) {
            points[i] = xc;
            points[np + i] = yc + (mid - i) * pp->l0;
            points[np - i - 1] = xc;
            points[np + np - i - 1] = yc - (mid - i) * pp->l0;
        }
    }
    return DRD_OK;
}

int drd_particles_set(drd_ctx* c, const drd_particle_params* pp, const double* points, const double* bdr_dist) {
    if (!c || !pp) return DRD_ERR_BADARG;
    if (pp->np != 0 && (pp->np < 3 || pp->np > DRD_PARTICLES_MAX || !points || !bdr_dist || !(pp->lx > 0) ||
                        !(pp->ly > 0) || !(pp->fpd_radius > 0))) {
        c->err = "drd_particles_set: np must be 0 or 3..DRD_PARTICLES_MAX with points, bdr_dist and a positive box";
        return DRD_ERR_BADARG;
    }
    const int changed = std::memcmp(pp, &c->pp, sizeof(*pp)) != 0;
    c->pp = *pp;
    if (pp->np > 0) {
        CK(cudaMemcpyAsync(c->pts, points, sizeof(double) * 2 * pp->np, cudaMemcpyHostToDevice, c->s));
        CK(cudaMemcpyAsync(c->pts_old, points, sizeof(double) * 2 * pp->np, cudaMemcpyHostToDevice, c->s));
        CK(cudaMemsetAsync(c->totF, 0, sizeof(double) * 2 * DRD_PARTICLES_MAX, c->s));
        if (up(c, c->bdist, bdr_dist, c->cs)) return DRD_ERR_CUDA;
    }
    CK(cudaStreamSynchronize(c->s));
    if (changed) clear_graphs(c);  // the step graph holds the particle launches and their parameters
    return DRD_OK;
}

int drd_particles_get(drd_ctx* c, double* points, double* tot_F) {
    if (!c) return DRD_ERR_BADARG;
    const size_t b = sizeof(double) * 2 * c->pp.np;
    if (b && points) CK(cudaMemcpyAsync(points, c->pts, b, cudaMemcpyDeviceToHost, c->s));
    if (b && tot_F) CK(cudaMemcpyAsync(tot_F, c->totF, b, cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    return DRD_OK;
}

int drd_force_caculation_vel(drd_ctx* c, double dt, double t, double* pf1, double* pf2) {
    (void)t;  // only the swimmers' tumbling clock reads t (particles_move.f90:600), and Np_swm = 0
    if (!c || !pf1 || !pf2) return DRD_ERR_BADARG;
    if (c->pp.np <= 0) { c->err = "no resident particles (drd_particles_set)"; return DRD_ERR_BADARG; }
    CK(cudaEventRecord(c->ev0, c->s));
    const double dt_keep = c->P.dt;
    c->P.dt = dt;
    enq_particles(c, PT_FORCE, nullptr, nullptr, c->s);
    c->P.dt = dt_keep;
    CK(cudaGetLastError());
    if (down(c, pf1, c->fld[DRD_F_PF1], c->cs) | down(c, pf2, c->fld[DRD_F_PF2], c->cs)) return DRD_ERR_CUDA;
    return finish_call(c, 0, nullptr, false);
}

int drd_update_position_vel(drd_ctx* c, const double* u, const double* v, double dt) {
    if (!c || !u || !v) return DRD_ERR_BADARG;
    if (c->pp.np <= 0) { c->err = "no resident particles (drd_particles_set)"; return DRD_ERR_BADARG; }
    CK(cudaEventRecord(c->ev0, c->s));
    if (up(c, c->u_after, u, c->us) | up(c, c->v_after, v, c->vs)) return DRD_ERR_CUDA;
    const double dt_keep = c->P.dt;
    c->P.dt = dt;
    enq_particles(c, PT_MOVE, c->u_after, c->v_after, c->s);
    c->P.dt = dt_keep;
    CK(cudaGetLastError());
    return finish_call(c, 0, nullptr, false);
}

int drd_interpolate_coef_particles(drd_ctx* c, double* fpd_ph, double* rho, double* eta) {
    if (!c) return DRD_ERR_BADARG;
    CK(cudaEventRecord(c->ev0, c->s));
    enq_particles(c, PT_COEF, nullptr, nullptr, c->s);
    CK(cudaGetLastError());
    if (down(c, fpd_ph, c->fpd, c->cs) | down(c, rho, c->rho, c->cs) | down(c, eta, c->eta, c->cs)) return DRD_ERR_CUDA;
    return finish_call(c, 0, nullptr, false);
}

// Wall prefactors cf = sqrt(2) cos(angle pi/180)/3 pi/2 of PhSolve_ori (:48, :87) and alpha_s.
// The captured graphs read cf from device memory but take alpha_s by value, so a new alpha_s
// drops the PhSolve_ori graphs.
int set_ori_walls(drd_ctx* c, const double* angleB, const double* angleT, double alpha_s) {
    std::vector<double> cb(c->nr + 1), ct(c->nr + 1);
    for (int i = 0; i <= c->nr; ++i) {
        const double aB = angleB ? angleB[i] : 0.0, aT = angleT ? angleT[i] : 0.0;
        cb[i] = std::sqrt(2.0) * std::cos(aB * kPi / 180.0) / 3.0 * kPi / 2.;
        ct[i] = std::sqrt(2.0) * std::cos(aT * kPi / 180.0) / 3.0 * kPi / 2.;
    }
    CK(cudaMemcpyAsync(c->ori_cfb, cb.data(), sizeof(double) * cb.size(), cudaMemcpyHostToDevice, c->s));
    CK(cudaMemcpyAsync(c->ori_cft, ct.data(), sizeof(double) * ct.size(), cudaMemcpyHostToDevice, c->s));
    CK(cudaStreamSynchronize(c->s));  // the host vectors go out of scope
    if (alpha_s != c->ori_alpha) {
        c->ori_alpha = alpha_s;
        for (int m = 0; m < 2; ++m) {
            auto it = c->graphs.find(gkey(GK_ORI, m, 0));
            if (it != c->graphs.end()) { cudaGraphExecDestroy(it->second); c->graphs.erase(it); }
        }
    }
    return DRD_OK;
}

int drd_phsolve_ori(drd_ctx* c, const double* u, const double* v, const double* ph, const double* angleB,
                    const double* angleT, double alpha_s, double* rmu_after, double* ph_after, drd_status* st) {
    if (!c || !u || !v || !ph || !rmu_after || !ph_after) return DRD_ERR_BADARG;
    if (c->P.variant != DRD_VARIANT_MF) { c->err = "PhSolve_ori belongs to the MF variant"; return DRD_ERR_BADARG; }
    int rc = set_ori_walls(c, angleB, angleT, alpha_s);
    if (rc) return rc;
    CK(cudaEventRecord(c->ev0, c->s));
    rc = up(c, c->fld[DRD_F_U], u, c->us) | up(c, c->fld[DRD_F_V], v, c->vs) | up(c, c->fld[DRD_F_PH], ph, c->cs);
    if (rc) return DRD_ERR_CUDA;
    rc = run_graph(c, gkey(GK_ORI, mixed_of(c), 0), [&](cudaStream_t s) { return enq_ori(c, s); }, 0.0, 0.0);
    if (rc) return rc;
    if (down(c, rmu_after, c->rmu_after, c->cs) | down(c, ph_after, c->ph_after, c->cs)) return DRD_ERR_CUDA;
    return finish_call(c, KS_CH, st, true);
}

int drd_finit_wall(drd_ctx* c, const double* bdr_in, int nsteps, double* bdr_out, double* ph_out, double* rmu_out) {
    if (!c || !bdr_in || nsteps < 0) return DRD_ERR_BADARG;
    if (c->P.variant != DRD_VARIANT_MF) { c->err = "finit's wall smoothing belongs to the MF variant"; return DRD_ERR_BADARG; }
    return wall_smoothing(c, bdr_in, nsteps, bdr_out, ph_out, rmu_out);
}

int drd_reinint_by_phsolve(drd_ctx* c, const double* bdr_in, double* bdr_out, double* pen_out) {
    if (!c || !bdr_in) return DRD_ERR_BADARG;
    // reinint_by_PhSolve.f90:34-70: the wall smoothing of finit, 51 PhSolve_ori steps
    const int info = wall_smoothing(c, bdr_in, 51, nullptr, nullptr, nullptr);
    if (info < 0 && info != -10 && info != -11) return info;
    // the smoothed indicator becomes bdr_ph, and :78-86 the penalty mask over the ghosted array
    CK(cudaMemcpyAsync(c->bdr, c->w, sizeof(double) * c->cs, cudaMemcpyDeviceToDevice, c->s));
    launch_threshold(c->cs, c->bdr, 0.5, c->pen, c->ctr, c->s);
    CK(cudaGetLastError());
    int rc = refresh_fp32(c);
    if (rc) return rc;
    if (down(c, bdr_out, c->bdr, c->cs) | down(c, pen_out, c->pen, c->cs)) return DRD_ERR_CUDA;
    CK(cudaStreamSynchronize(c->s));
    return info;
}

int drd_dissipation(drd_ctx* c, const double* u, const double* v, const double* ph, const double* rmu,
                    const double* angleB, const double* angleT, double vs, drd_diagnostics* out) {
    if (!c || !out) return DRD_ERR_BADARG;
    CK(cudaEventRecord(c->ev0, c->s));
    // caller arrays go to scratch that the next solve rewrites; NULL keeps the resident field
    const double* du = u ? c->u_after : c->fld[DRD_F_U];
    const double* dv = v ? c->v_after : c->fld[DRD_F_V];
    const double* dph = ph ? c->ph_after : c->fld[DRD_F_PH];
    const double* drmu = rmu ? c->rmu_after : c->fld[DRD_F_RMU];
    if (up(c, c->u_after, u, c->us) | up(c, c->v_after, v, c->vs) | up(c, c->ph_after, ph, c->cs) |
        up(c, c->rmu_after, rmu, c->cs) | up(c, c->pnb, angleB, c->nr) | up(c, c->pnt, angleT, c->nr))
        return DRD_ERR_CUDA;
    DissipArgs a{};
    a.nr = c->nr; a.nz = c->nz; a.dr = c->P.dr; a.dz = c->P.dz; a.xld = c->P.xld; a.ca = c->P.ca;
    a.eps = c->P.I_thickness; a.vs = vs; a.angle = c->P.angle;
    launch_dissipation(a, du, dv, dph, drmu, angleB ? c->pnb : nullptr, angleT ? c->pnt : nullptr, dots(c), c->d_diag,
                       c->ctr, c->s);
    CK(cudaGetLastError());
    double h[6];
    CK(cudaMemcpyAsync(h, c->d_diag, sizeof(h), cudaMemcpyDeviceToHost, c->s));
    int rc = finish_call(c, 0, nullptr, false);
    if (rc) return rc;
    out->e1 = h[0]; out->e2 = h[1]; out->e3 = h[2]; out->e4 = h[3]; out->dissip = h[4]; out->mass = h[5];
    return DRD_OK;
}


int drd_checkpoint_wait(drd_ctx* c) {
    if (!c) return DRD_ERR_BADARG;
    if (c->ckpt.joinable()) c->ckpt.join();
    const int rc = c->ckpt_rc;
    c->ckpt_rc = 0;
    return rc;
}

int drd_checkpoint_async(drd_ctx* c, const char* path, double t) {
    if (!c || !path) return DRD_ERR_BADARG;
    int rc = drd_checkpoint_wait(c);
    if (rc) return rc;
    const long us = c->us, vs = c->vs, cs = c->cs;
    if (!c->h_stage) {
        CK(cudaMallocHost(&c->h_stage, sizeof(double) * (us + vs + 3 * cs)));
        CK(cudaStreamCreateWithFlags(&c->sck, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->eck0, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->eck1, cudaEventDisableTiming));
    }
    double* hu = c->h_stage;
    double* hv = hu + us;
    double* hp = hv + vs;
    double* hf = hp + cs;
    double* hph = hf + cs;
    // the copies start after the work already on the context stream, and later work on that
    // stream (the next step rewrites these fields) waits for them
    CK(cudaEventRecord(c->eck0, c->s));
    CK(cudaStreamWaitEvent(c->sck, c->eck0, 0));
    CK(cudaMemcpyAsync(hu, c->fld[DRD_F_U], sizeof(double) * us, cudaMemcpyDeviceToHost, c->sck));
    CK(cudaMemcpyAsync(hv, c->fld[DRD_F_V], sizeof(double) * vs, cudaMemcpyDeviceToHost, c->sck));
    CK(cudaMemcpyAsync(hp, c->fld[DRD_F_P], sizeof(double) * cs, cudaMemcpyDeviceToHost, c->sck));
    CK(cudaMemcpyAsync(hf, c->fpd, sizeof(double) * cs, cudaMemcpyDeviceToHost, c->sck));
    CK(cudaMemcpyAsync(hph, c->fld[DRD_F_PH], sizeof(double) * cs, cudaMemcpyDeviceToHost, c->sck));
    CK(cudaEventRecord(c->eck1, c->sck));
    CK(cudaStreamWaitEvent(c->s, c->eck1, 0));
    const std::string file(path);
    const int nr = c->nr, nz = c->nz, dev = c->device;
    const double dr = c->P.dr, dz = c->P.dz;
    cudaEvent_t done = c->eck1;
    c->ckpt = std::thread([=]() {
        int r = DRD_OK;
        if (cudaSetDevice(dev) != cudaSuccess || cudaEventSynchronize(done) != cudaSuccess) r = DRD_ERR_CUDA;
        else r = drd_output(file.c_str(), nr, nz, dr, dz, nullptr, nullptr, hu, hv, hp, hf, hph, t);
        c->ckpt_rc = r;
    });
    return DRD_OK;
}

int drd_phsolve(drd_ctx* c, const double* u, const double* v, const double* ph, const double* rmu, double t,
                double* rmu_after, double* ph_after, drd_status* st) {
    if (!c || !u || !v || !ph || !rmu || !rmu_after || !ph_after) return DRD_ERR_BADARG;
    if (c->P.variant != DRD_VARIANT_MF) { c->err = "PhSolve belongs to the MF variant"; return DRD_ERR_BADARG; }
    reset_q(c);
    CK(cudaEventRecord(c->ev0, c->s));
    // guess_mode 1 / 2: the guess extrapolates rmu through the rmu of the previous one or two
    // calls (x^(n-1), x^(n-2) when the calls are successive time steps; otherwise only the
    // starting guess is poorer)
    const size_t cb = sizeof(double) * c->cs;
    const int gm = c->P.guess_mode;
    const int extrap = std::min(gm, c->rmu_hist);
    if (extrap >= 1) CK(cudaMemcpyAsync(c->fld[DRD_F_RMU_PRE], c->rmu_prev, cb, cudaMemcpyDeviceToDevice, c->s));
    if (extrap >= 2) CK(cudaMemcpyAsync(c->rmu_pre2, c->rmu_prev2, cb, cudaMemcpyDeviceToDevice, c->s));
    if (extrap == 3) CK(cudaMemcpyAsync(c->rmu_pre3, c->rmu_prev3, cb, cudaMemcpyDeviceToDevice, c->s));
    int rc = up_q(c, c->fld[DRD_F_U], u, c->us) | up_q(c, c->fld[DRD_F_V], v, c->vs) |
             up_q(c, c->fld[DRD_F_PH], ph, c->cs) | up_q(c, c->fld[DRD_F_RMU], rmu, c->cs);
    rc |= flush_q(c, c->hq_up);
    if (rc) return DRD_ERR_CUDA;
    if (gm >= 1) {
        if (gm == 3) CK(cudaMemcpyAsync(c->rmu_prev3, c->rmu_prev2, cb, cudaMemcpyDeviceToDevice, c->s));
        if (gm >= 2) CK(cudaMemcpyAsync(c->rmu_prev2, c->rmu_prev, cb, cudaMemcpyDeviceToDevice, c->s));
        CK(cudaMemcpyAsync(c->rmu_prev, c->fld[DRD_F_RMU], cb, cudaMemcpyDeviceToDevice, c->s));
        c->rmu_hist = std::min(c->rmu_hist + 1, 3);
    }
    rc = run_graph(c, gkey(GK_CH, mixed_of(c), extrap), [&](cudaStream_t s) { return enq_ch(c, s, extrap); }, t, 0.0);
    if (rc) return rc;
    rc = down_q(c, rmu_after, c->rmu_after, c->cs) | down_q(c, ph_after, c->ph_after, c->cs);
    rc |= flush_q(c, c->hq_down);
    if (rc) return DRD_ERR_CUDA;
    return finish_call(c, KS_CH, st, true);
}

int drd_ph_mu_solve(drd_ctx* c, const double* u, const double* v, const double* ph, const double* rmu, double t,
                    double* ph_after, double* rmu_after, double* ph_M_0_out, double* coef_bot_top, drd_status* st) {
    if (!c || !u || !v || !ph || !rmu || !rmu_after || !ph_after) return DRD_ERR_BADARG;
    if (c->P.variant != DRD_VARIANT_TP) { c->err = "ph_mu_solve belongs to the TP variant"; return DRD_ERR_BADARG; }
    CK(cudaEventRecord(c->ev0, c->s));
    int rc = up(c, c->fld[DRD_F_U], u, c->us) | up(c, c->fld[DRD_F_V], v, c->vs) | up(c, c->fld[DRD_F_PH], ph, c->cs) |
             up(c, c->fld[DRD_F_RMU], rmu, c->cs);
    if (rc) return DRD_ERR_CUDA;
    rc = run_graph(c, gkey(GK_PHMU, mixed_of(c), 0), [&](cudaStream_t s) { return enq_phmu(c, s); }, t, 0.0);
    if (rc) return rc;
    rc = down(c, ph_after, c->ph_after, c->cs) | down(c, rmu_after, c->rmu_after, c->cs) |
         down(c, ph_M_0_out, c->M0, c->cs);
    if (rc) return DRD_ERR_CUDA;
    if (coef_bot_top) {
        OpScal<double> o = make_op<double>(c, 0);
        coef_bot_top[0] = o.cb;
        coef_bot_top[1] = o.ct;
    }
    return finish_call(c, KS_PHMU, st, true);
}

static int velo_common(drd_ctx* c, int bdf, const double* psi1, const double* psi2, const double* u_pre,
                       const double* u, const double* v_pre, const double* v, const double* p, const double* ph_after,
                       const double* rmu_after, double t, const double* pf1, const double* pf2, double* u_after,
                       double* v_after, double* uL, double* uR, drd_status* st) {
    if (!c || !u || !v || !p || !ph_after || !rmu_after || !u_after || !v_after) return DRD_ERR_BADARG;
    if (bdf == 2 && (!psi1 || !psi2 || !u_pre || !v_pre)) return DRD_ERR_BADARG;
    reset_q(c);
    CK(cudaEventRecord(c->ev0, c->s));
    int rc = up_q(c, c->fld[DRD_F_U], u, c->us) | up_q(c, c->fld[DRD_F_V], v, c->vs) |
             up_q(c, c->fld[DRD_F_P], p, c->cs) | up_q(c, c->ph_after, ph_after, c->cs) |
             up_q(c, c->rmu_after, rmu_after, c->cs);
    if (bdf == 2)
        rc |= up_q(c, c->fld[DRD_F_PSI1], psi1, c->cs) | up_q(c, c->fld[DRD_F_PSI2], psi2, c->cs) |
              up_q(c, c->fld[DRD_F_U_PRE], u_pre, c->us) | up_q(c, c->fld[DRD_F_V_PRE], v_pre, c->vs);
    if (pf1) rc |= up_q(c, c->fld[DRD_F_PF1], pf1, c->cs);
    else CK(cudaMemsetAsync(c->fld[DRD_F_PF1], 0, sizeof(double) * c->cs, c->s));
    if (pf2) rc |= up_q(c, c->fld[DRD_F_PF2], pf2, c->cs);
    else CK(cudaMemsetAsync(c->fld[DRD_F_PF2], 0, sizeof(double) * c->cs, c->s));
    rc |= flush_q(c, c->hq_up);
    if (rc) return DRD_ERR_CUDA;
    // guess_mode 1 / 2 (BDF2): the momentum solve starts from 2 u - u_pre, or from 3 u - 3 u_pre +
    // u_pre2 with u_pre2 the u_pre of the previous call; v likewise
    const int gm = c->P.guess_mode;
    const int extrap = (bdf != 2 || gm == 0) ? 0 : std::min(gm, 1 + c->uv_hist);
    rc = run_graph(c, gkey(GK_UV, mixed_of(c), bdf + 2 * extrap), [&](cudaStream_t s) { return enq_uv(c, bdf, s, extrap); },
                   t, 0.0);
    if (rc) return rc;
    if (gm >= 2 && bdf == 2) {  // this call's u_pre is the next call's u_pre2
        const size_t ub = sizeof(double) * c->us, vb = sizeof(double) * c->vs;
        if (gm == 3) {
            CK(cudaMemcpyAsync(c->u_pre3, c->u_pre2, ub, cudaMemcpyDeviceToDevice, c->s));
            CK(cudaMemcpyAsync(c->v_pre3, c->v_pre2, vb, cudaMemcpyDeviceToDevice, c->s));
        }
        CK(cudaMemcpyAsync(c->u_pre2, c->fld[DRD_F_U_PRE], ub, cudaMemcpyDeviceToDevice, c->s));
        CK(cudaMemcpyAsync(c->v_pre2, c->fld[DRD_F_V_PRE], vb, cudaMemcpyDeviceToDevice, c->s));
        c->uv_hist = std::min(c->uv_hist + 1, 2);
    }
    if (rc) return rc;
    rc = down_q(c, u_after, c->u_after, c->us) | down_q(c, v_after, c->v_after, c->vs);
    const bool dirichlet = !(c->P.variant == DRD_VARIANT_TP && c->P.lr_bd_type == 'n');
    if (dirichlet) rc |= down_q(c, uL, c->uL, c->nz) | down_q(c, uR, c->uL, c->nz);
    rc |= flush_q(c, c->hq_down);
    if (rc) return DRD_ERR_CUDA;
    return finish_call(c, KS_UV, st, true);
}

int drd_velosolve_combined(drd_ctx* c, const double* psi, const double* u, const double* v, const double* p,
                           const double* rmu_after, const double* ph_after, double t, const double* pf1,
                           const double* pf2, double* u_after, double* v_after, double* uL, double* uR, drd_status* st) {
    (void)psi;  // VeloSolve_combined ignores psi (temp_p = p, VeloSolve_combined.f90:182)
    return velo_common(c, 1, nullptr, nullptr, nullptr, u, nullptr, v, p, ph_after, rmu_after, t, pf1, pf2, u_after,
                       v_after, uL, uR, st);
}

int drd_velosolve_2_combined(drd_ctx* c, const double* psi1, const double* psi2, const double* u_pre,
                             const double* u, const double* v_pre, const double* v, const double* p,
                             const double* ph_pre, const double* ph_after, const double* rmu_pre,
                             const double* rmu_after, double t, const double* pf1, const double* pf2, double* u_after,
                             double* v_after, double* uL, double* uR, drd_status* st) {
    (void)ph_pre;
    (void)rmu_pre;
    return velo_common(c, 2, psi1, psi2, u_pre, u, v_pre, v, p, ph_after, rmu_after, t, pf1, pf2, u_after, v_after,
                       uL, uR, st);
}

int drd_presolve_2(drd_ctx* c, const double* u, const double* v, double coef, double* psi, drd_status* st) {
    if (!c || !u || !v || !psi) return DRD_ERR_BADARG;
    reset_q(c);
    CK(cudaEventRecord(c->ev0, c->s));
    int rc = up_q(c, c->fld[DRD_F_U], u, c->us) | up_q(c, c->fld[DRD_F_V], v, c->vs);
    rc |= flush_q(c, c->hq_up);
    if (rc) return DRD_ERR_CUDA;
    rc = run_graph(c, gkey(GK_PRE, 0, 0), [&](cudaStream_t s) { enq_pre(c, c->fld[DRD_F_PSI2], s); return DRD_OK; },
                   0.0, coef);
    if (rc) return rc;
    if (down_q(c, psi, c->fld[DRD_F_PSI2], c->cs) | flush_q(c, c->hq_down)) return DRD_ERR_CUDA;
    return finish_call(c, 0, st, false);
}

int drd_solve(drd_ctx* c, int system, int bdf, const double* b, double* x, drd_status* st) {
    if (!c || !b || !x || (system != DRD_SYS_CH && system != DRD_SYS_UV) || (bdf != 1 && bdf != 2))
        return DRD_ERR_BADARG;
    if (system == DRD_SYS_CH && c->P.variant != DRD_VARIANT_MF) {
        c->err = "the CH system belongs to the MF variant";
        return DRD_ERR_BADARG;
    }
    int rc = ensure_tuned(c);
    if (rc) return rc;
    const int slot = system == DRD_SYS_CH ? KS_CH : KS_UV;
    const long n = system == DRD_SYS_CH ? c->nc : c->nuv;
    CK(cudaEventRecord(c->ev0, c->s));
    rc = up(c, c->k64.b, b, n) | up(c, c->k64.x, x, n);
    if (rc) return DRD_ERR_CUDA;
    const int mixed = mixed_for(c, slot);
    rc = run_graph(c, gkey(GK_SOLVE, mixed, 3 * system + bdf), [&](cudaStream_t s) {
        const Sys S = sys_of(c, system == DRD_SYS_CH ? SYS_CH : SYS_UV, bdf);
        return enq_solve(c, S, slot, c->P.tol, system == DRD_SYS_CH ? c->P.ch_maxit : c->P.uv_maxit, mixed, s);
    }, 0.0, 0.0);
    if (rc) return rc;
    if (down(c, x, c->k64.x, n)) return DRD_ERR_CUDA;
    return finish_call(c, slot, st, true);
}

int drd_mass(drd_ctx* c, const double* ph, double* mass) {
    if (!c || !ph || !mass) return DRD_ERR_BADARG;
    CK(cudaEventRecord(c->ev0, c->s));
    if (up(c, c->ph_after, ph, c->cs)) return DRD_ERR_CUDA;
    enq_mass(c, c->ph_after, c->s);
    CK(cudaMemcpyAsync(c->h_mass, c->d_mass, sizeof(double), cudaMemcpyDeviceToHost, c->s));
    int rc = finish_call(c, 0, nullptr, false);
    *mass = *c->h_mass;
    return rc;
}

int drd_state_upload(drd_ctx* c, int field, const double* host) {
    if (!c || field < 0 || field >= DRD_F_COUNT || !host) return DRD_ERR_BADARG;
    const long n = (field == DRD_F_U || field == DRD_F_U_PRE) ? c->us : (field == DRD_F_V || field == DRD_F_V_PRE) ? c->vs : c->cs;
    CK(cudaMemcpyAsync(c->fld[field], host, sizeof(double) * n, cudaMemcpyHostToDevice, c->s));
    CK(cudaStreamSynchronize(c->s));
    c->hist = 0;  // a new state: no step history for the extrapolated guesses
    return DRD_OK;
}

int drd_state_download(drd_ctx* c, int field, double* host) {
    if (!c || field < 0 || field >= DRD_F_COUNT || !host) return DRD_ERR_BADARG;
    const long n = (field == DRD_F_U || field == DRD_F_U_PRE) ? c->us : (field == DRD_F_V || field == DRD_F_V_PRE) ? c->vs : c->cs;
    CK(cudaMemcpyAsync(host, c->fld[field], sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    return DRD_OK;
}

int drd_state_device_ptr(drd_ctx* c, int field, double** dptr) {
    if (!c || field < 0 || field >= DRD_F_COUNT || !dptr) return DRD_ERR_BADARG;
    *dptr = c->fld[field];
    return DRD_OK;
}

int drd_steps_async(drd_ctx* c, int first, double t, int nsteps) {
    if (!c || nsteps < 0) return DRD_ERR_BADARG;
    for (int k = 0; k < nsteps; ++k) {
        const int fst = (first && k == 0);
        const double gamma1 = std::min(1.0, c->P.lambda_rho);
        const double coef = fst ? c->P.re * gamma1 / c->P.dt : 3 * c->P.re * gamma1 / 2. / c->P.dt;
        const double tt = t + k * c->P.dt + c->P.dt;
        // the guess of this step: the polynomial of order guess_mode through the steps held
        const int gm = c->P.guess_mode;
        const int extrap = (fst || gm == 0) ? 0 : std::min(gm, std::max(c->hist, 1));
        int rc = run_graph(c, gkey(GK_STEP, mixed_of(c), fst + 2 * extrap),
                           [&](cudaStream_t s) { return enq_step(c, fst, extrap, s); }, tt, coef);
        if (rc) return rc;
        c->hist = fst ? 1 : std::min(c->hist + 1, 3);
    }
    return DRD_OK;
}

int drd_step(drd_ctx* c, int first, double t, drd_step_stats* stats) {
    if (!c) return DRD_ERR_BADARG;
    CK(cudaEventRecord(c->ev0, c->s));
    int rc = drd_steps_async(c, first, t, 1);
    if (rc) return rc;
    if (!stats) return DRD_OK;
    CK(cudaMemcpyAsync(c->h_ks, c->ks, KS_COUNT * sizeof(KState), cudaMemcpyDeviceToHost, c->s));
    CK(cudaMemcpyAsync(c->h_mass, c->d_mass, sizeof(double), cudaMemcpyDeviceToHost, c->s));
    CK(cudaEventRecord(c->ev1, c->s));
    CK(cudaStreamSynchronize(c->s));
    CK(cudaGetLastError());
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    // a solve's own device time: %globaltimer stamps at its start and end
    auto solve_s = [](const KState& k) { return k.t_end > k.t_begin ? 1e-9 * (double)(k.t_end - k.t_begin) : 0.0; };
    const int sch = c->P.variant == DRD_VARIANT_TP ? KS_PHMU : KS_CH;
    fill_status(c, sch, c->h_ks[sch], &stats->ch, solve_s(c->h_ks[sch]));
    fill_status(c, KS_UV, c->h_ks[KS_UV], &stats->uv, solve_s(c->h_ks[KS_UV]));
    stats->seconds = ms * 1e-3;
    memset(&stats->pre, 0, sizeof(stats->pre));
    stats->mass = *c->h_mass;
    stats->t = t + c->P.dt;
    return DRD_OK;
}

int drd_synchronize(drd_ctx* c) {
    if (!c) return DRD_ERR_BADARG;
    CK(cudaStreamSynchronize(c->s));
    CK(cudaGetLastError());
    return DRD_OK;
}

long drd_op_length(drd_ctx* c, int op) {
    if (!c) return -1;
    if (op == DRD_OP_CH_MATVEC || op == DRD_OP_CH_PSOLVE) return c->nc;
    if (op == DRD_OP_UV_MATVEC || op == DRD_OP_UV_PSOLVE) return c->nuv;
    if (op == DRD_OP_PHMU_MATVEC || op == DRD_OP_PHMU_PSOLVE) return c->nphmu;
    return -1;
}

int drd_op_apply(drd_ctx* c, int op, int bdf, int precision, const double* x, double* y) {
    if (!c || !x || !y) return DRD_ERR_BADARG;
    const long n = drd_op_length(c, op);
    if (n < 0 || (bdf != 1 && bdf != 2)) return DRD_ERR_BADARG;
    int rc = ensure_tuned(c);
    if (rc) return rc;
    const int kind = (op <= DRD_OP_CH_PSOLVE) ? SYS_CH : (op <= DRD_OP_UV_PSOLVE) ? SYS_UV : SYS_PHMU;
    const bool mv = (op % 2) == 0;
    Sys S = sys_of(c, kind, bdf);
    KVecs<double>& k = c->k64;
    CK(cudaMemcpyAsync(k.tmp, x, sizeof(double) * n, cudaMemcpyHostToDevice, c->s));
    if (precision == DRD_OP_PERSISTENT && (kind == SYS_CH || kind == SYS_UV)) {
        // the persistent solver's own operator code: x = op(b) in one cooperative launch
        if (!c->persist) { c->err = "persistent solver not in use: " + c->persist_err; return DRD_ERR_UNSUPPORTED; }
        if (S.esolp && !c->persist_esolp) { c->err = "the persistent momentum solver cannot hold ESOLP_x's work area"; return DRD_ERR_UNSUPPORTED; }
        KVecs<float>& f = c->k32;
        enq_sys_setup<float>(c, S, c->s);
        launch_convert_scale<float, double>(n, k.tmp, 1.0, f.b, c->ctr, c->s);
        PersistArgs a = persist_args(c, S, c->ks + KS_INNER, nullptr, 0.0, 0);
        a.mode = mv ? PM_MATVEC : PM_PSOLVE;
        launch_bar_reset(c->bar, c->ctr, c->s);
        CK(launch_bicg_persist(a, c->pgrid, c->s));
        launch_convert_scale<double, float>(n, f.x, 1.0, k.v, c->ctr, c->s);
    } else if (precision == DRD_PREC_FP64) {
        enq_sys_setup<double>(c, S, c->s);
        if (mv) enq_matvec<double>(c, S, 1.0, k.tmp, 0.0, k.v, nullptr, 0, 0, nullptr, G_ALWAYS, c->s);
        else enq_psolve<double>(c, S, k.tmp, k.v, nullptr, G_ALWAYS, c->s);
    } else {
        KVecs<float>& f = c->k32;
        enq_sys_setup<float>(c, S, c->s);
        launch_convert_scale<float, double>(n, k.tmp, 1.0, f.tmp, c->ctr, c->s);
        if (mv) enq_matvec<float>(c, S, 1.0f, f.tmp, 0.0f, f.v, nullptr, 0, 0, nullptr, G_ALWAYS, c->s);
        else enq_psolve<float>(c, S, f.tmp, f.v, nullptr, G_ALWAYS, c->s);
        launch_convert_scale<double, float>(n, f.v, 1.0, k.v, c->ctr, c->s);
    }
    CK(cudaMemcpyAsync(y, k.v, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    CK(cudaGetLastError());
    return DRD_OK;
}

int drd_kernel_bench(drd_ctx* c, int which, int reps, double* us, double* bytes, double* flops) {
    if (!c || which < 0 || which >= DRD_KB_COUNT || reps <= 0 || !us) return DRD_ERR_BADARG;
    int rc = ensure_tuned(c);
    if (rc) return rc;
    const int nr = c->nr, nz = c->nz;
    Sys S = sys_of(c, SYS_UV, 2);
    double by = 0.0, fl = 0.0;
    auto enqueue = [&](cudaStream_t s) {
        switch (which) {
            case DRD_KB_UV_MATVEC_FP64:
                launch_uv_matvec<double>(make_op<double>(c, 2), c->rho, c->eta, c->pen, 1.0, c->k64.p, 0.0, c->k64.v,
                                         nullptr, 0, dots(c), 0, nullptr, G_ALWAYS, nullptr, s);
                break;
            case DRD_KB_UV_MATVEC_FP32:
                launch_uv_matvec<float>(make_op<float>(c, 2), c->rho32, c->eta32, c->pen32, 1.0f, c->k32.p, 0.0f,
                                        c->k32.v, nullptr, 0, dots(c), 0, nullptr, G_ALWAYS, nullptr, s);
                break;
            case DRD_KB_DCT_X_FP64: {
                auto a = dct1_xpass<double>(c, c->k64.p, c->t1, nullptr, G_ALWAYS);
                a.ctr = nullptr;
                launch_gemm<double>(gcfg<double>(c, 0), EPI_STORE, a, s);
                break;
            }
            case DRD_KB_DCT_X_FP32: {
                auto a = dct1_xpass<float>(c, c->k32.p, c->t1f, nullptr, G_ALWAYS);
                a.ctr = nullptr;
                launch_gemm<float>(gcfg<float>(c, 0), EPI_STORE, a, s);
                break;
            }
            case DRD_KB_DCT_Z_FP64: {
                auto a = dct1_zpass<double>(c, c->k64.p, c->t1, nullptr, G_ALWAYS);
                a.ctr = nullptr;
                launch_gemm<double>(gcfg<double>(c, 1), EPI_STORE, a, s);
                break;
            }
            case DRD_KB_DCT_Z_FP32: {
                auto a = dct1_zpass<float>(c, c->k32.p, c->t1f, nullptr, G_ALWAYS);
                a.ctr = nullptr;
                launch_gemm<float>(gcfg<float>(c, 1), EPI_STORE, a, s);
                break;
            }
            case DRD_KB_PRESSURE_FFT64:
                launch_pressure_fft(nr, nz, c->P.dr, c->P.dz, c->fpx, c->fpz, c->ftwx, c->ftwz, c->fld[DRD_F_U],
                                    c->fld[DRD_F_V], c->t1, c->pre_lcc, c->fld[DRD_F_PSI2], c->ca, nullptr, s);
                break;
            case DRD_KB_DCT2_FFT32:
                launch_pressure_fft32(nr, nz, c->fpx, c->fpz, c->ftwx32, c->ftwz32, c->k32.p, c->t1f, c->t2f,
                                      c->k32.v, nullptr, s);
                break;
            default:
                launch_ch_matvec<float>(make_op<float>(c, 0), c->M032, c->Mi32, 1.0f, c->k32.p, 0.0f, c->k32.v,
                                        c->k32.ff1, nullptr, 0, dots(c), 0, nullptr, G_ALWAYS, nullptr, s);
                break;
        }
    };
    const bool cold = (which == DRD_KB_PRESSURE_FFT64 || which == DRD_KB_DCT2_FFT32);
    if (cold && !c->pfft_ok) return DRD_ERR_UNSUPPORTED;
    switch (which) {
        case DRD_KB_UV_MATVEC_FP64: by = 8.0 * (2.0 * S.n + 3.0 * c->cs); fl = 45.0 * S.n; break;
        case DRD_KB_UV_MATVEC_FP32: by = 4.0 * (2.0 * S.n + 3.0 * c->cs); fl = 45.0 * S.n; break;
        // folded passes: K = floor((N-1)/2)+1 multiply-adds per output
        case DRD_KB_DCT_X_FP64: by = 8.0 * (2.0 * c->nc + 2.0 * c->Kx * c->Nxe); fl = 2.0 * c->nc * c->Kx; break;
        case DRD_KB_DCT_X_FP32: by = 4.0 * (2.0 * c->nc + 2.0 * c->Kx * c->Nxe); fl = 2.0 * c->nc * c->Kx; break;
        case DRD_KB_DCT_Z_FP64: by = 8.0 * (2.0 * c->nc + 2.0 * c->Mze * c->Kz); fl = 2.0 * c->nc * c->Kz; break;
        case DRD_KB_DCT_Z_FP32: by = 4.0 * (2.0 * c->nc + 2.0 * c->Mze * c->Kz); fl = 2.0 * c->nc * c->Kz; break;
        // u, v read, psi written; the table and the intermediate round trips are not counted
        case DRD_KB_PRESSURE_FFT64: by = 8.0 * (c->us + c->vs + c->cs); fl = 0.0; break;
        case DRD_KB_DCT2_FFT32: by = 4.0 * 3.0 * c->nc; fl = 0.0; break;
        default: by = 4.0 * (3.0 * c->nc + 2.0 * c->cs); fl = 40.0 * c->nc; break;
    }
    if (cold) {
        // an nr x nz Pre_Lcc table in FP32 for the FP32 pair; zero inputs are enough, the
        // transforms' cost does not depend on the values
        std::vector<float> l32(c->nc);
        std::vector<double> ph, pre;
        host_tables(c->P, ph, pre);
        for (int k = 0; k < nz; ++k)
            for (int i = 0; i < nr; ++i) l32[i + (size_t)nr * k] = (float)pre[i + (size_t)(nr + 1) * k];
        CK(cudaMemcpy(c->t2f, l32.data(), sizeof(float) * l32.size(), cudaMemcpyHostToDevice));
        CK(cudaMemsetAsync(c->k32.p, 0, sizeof(float) * c->nmax, c->s));
        const int64_t flush = 512ll << 20;
        int rc2 = drd_flush_l2(c, flush);
        if (rc2) return rc2;
        enqueue(c->s);  // warm-up
        CK(cudaGetLastError());
        float total = 0.f;
        for (int r = 0; r < reps; ++r) {
            rc2 = drd_flush_l2(c, flush);
            if (rc2) return rc2;
            CK(cudaEventRecord(c->ev0, c->s));
            enqueue(c->s);
            CK(cudaEventRecord(c->ev1, c->s));
            CK(cudaEventSynchronize(c->ev1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            total += ms;
        }
        CK(cudaGetLastError());
        *us = 1e3 * total / reps;
        if (bytes) *bytes = by;
        if (flops) *flops = fl;
        return DRD_OK;
    }
    CK(cudaMemsetAsync(c->k64.p, 0, sizeof(double) * c->nmax, c->s));
    CK(cudaMemsetAsync(c->k32.p, 0, sizeof(float) * c->nmax, c->s));
    enqueue(c->s);  // warm-up
    CK(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal));
    for (int r = 0; r < reps; ++r) enqueue(c->s);
    cudaGraph_t g;
    CK(cudaStreamEndCapture(c->s, &g));
    cudaGraphExec_t ex;
    CK(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    CK(cudaGraphLaunch(ex, c->s));  // warm-up of the graph
    CK(cudaEventRecord(c->ev0, c->s));
    CK(cudaGraphLaunch(ex, c->s));
    CK(cudaEventRecord(c->ev1, c->s));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    cudaGraphExecDestroy(ex);
    *us = 1e3 * ms / reps;
    if (bytes) *bytes = by;
    if (flops) *flops = fl;
    return DRD_OK;
}

int drd_host_register(void* p, int64_t bytes) {
    if (!p || bytes <= 0) return DRD_ERR_BADARG;
    cudaError_t e = cudaHostRegister(p, (size_t)bytes, cudaHostRegisterMapped);
    if (e != cudaSuccess) { cudaGetLastError(); return DRD_ERR_CUDA; }
    void* dev = nullptr;
    e = cudaHostGetDevicePointer(&dev, p, 0);
    if (e != cudaSuccess || dev == nullptr) {
        cudaGetLastError();  // page-locked but not mapped: the calls copy it by DMA
        return DRD_OK;
    }
    std::lock_guard<std::mutex> lock(g_host_mu);
    g_host_ranges[reinterpret_cast<uintptr_t>(p)] = HostRange{(size_t)bytes, static_cast<char*>(dev)};
    return DRD_OK;
}

int drd_host_unregister(void* p) {
    if (!p) return DRD_ERR_BADARG;
    {
        std::lock_guard<std::mutex> lock(g_host_mu);
        g_host_ranges.erase(reinterpret_cast<uintptr_t>(p));
    }
    const cudaError_t e = cudaHostUnregister(p);
    if (e != cudaSuccess) { cudaGetLastError(); return DRD_ERR_CUDA; }
    return DRD_OK;
}

int drd_flush_l2(drd_ctx* c, int64_t bytes) {
    if (!c || bytes < 0) return DRD_ERR_BADARG;
    static thread_local void* buf = nullptr;
    static thread_local int64_t have = 0;
    if (have < bytes) {
        if (buf) cudaFree(buf);
        buf = nullptr;
        have = 0;
        CK(cudaMalloc(&buf, (size_t)bytes));
        have = bytes;
    }
    CK(cudaMemsetAsync(buf, have & 0xff, (size_t)bytes, c->s));
    return DRD_OK;
}

int drd_persist_profile(drd_ctx* c, int64_t* ns, int n) {
    if (!c || !ns || n <= 0) return DRD_ERR_BADARG;
    const int m = std::min(n, 128);
    std::vector<unsigned long long> h(m);
    CK(cudaStreamSynchronize(c->s));
    CK(cudaMemcpy(h.data(), c->pprof, sizeof(unsigned long long) * m, cudaMemcpyDeviceToHost));
    for (int i = 0; i < m; ++i) ns[i] = (int64_t)h[i];
    return m;
}

int drd_barrier_selftest(drd_ctx* c, int absent, int* status) {
    if (!c || !status || (absent != -1 && absent != 1)) return DRD_ERR_BADARG;
    int* d_out = reinterpret_cast<int*>(c->pprof + 120);  // scratch: two ints of the profile buffer
    launch_bar_selftest(c->bar, absent, d_out, c->ctr, c->s);
    int h[2] = {0, 0};
    CK(cudaMemcpyAsync(h, d_out, sizeof(h), cudaMemcpyDeviceToHost, c->s));
    CK(cudaStreamSynchronize(c->s));
    CK(cudaGetLastError());
    *status = (absent == 1) ? h[0] : (h[0] != 0 ? h[0] : h[1]);
    return DRD_OK;
}

int drd_persistent_solver(drd_ctx* c, char* why, int len) {
    if (!c) return DRD_ERR_BADARG;
    if (why && len > 0) std::snprintf(why, (size_t)len, "%s", c->persist_err.c_str());
    return c->persist;
}

int64_t drd_kernel_launches(drd_ctx* c) {
    if (!c) return -1;
    unsigned long long v = 0;
    cudaStreamSynchronize(c->s);
    cudaMemcpy(&v, c->ctr, sizeof(v), cudaMemcpyDeviceToHost);
    return (int64_t)v;
}

void* drd_stream(drd_ctx* c) { return c ? (void*)c->s : nullptr; }

}  // extern "C"
