/*
 * drd_oracle.c — FP64 CPU restatement of the DRD-Micro per-time-step solver core.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the checker for the CUDA library.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline legs load it; nothing in the
 * product path calls it.  Parity is "unpinned" against reference-run outputs (none exist
 * and the Fortran reference cannot be built); see drd_oracle.h for the pins used instead.
 *
 * Each routine cites the reference lines it restates.  Arithmetic follows the Fortran
 * left-to-right evaluation order of those lines so that a faithful build of the
 * reference would agree to rounding.  Transforms are evaluated by direct summation of
 * their published definitions (vfftpack VCOST prologue, FFTW REDFT10/REDFT01).
 */
#include "drd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define CI(i, k) ((long)((i) + 1) + (long)((k) + 1) * (nr + 2)) /* CELL  (-1:nr,  -1:nz) */
#define UI(i, k) ((long)((i) + 1) + (long)((k) + 1) * (nr + 3)) /* UFACE (-1:nr+1,-1:nz) */
#define VI(i, k) ((long)((i) + 1) + (long)(k) * (nr + 2))       /* VFACE (-1:nr,   0:nz) */

static const double kPi = 3.14159265358979323846264338327950288; /* global.f90:27 */
static const double kPimach = 3.14159265358979;                  /* lib/vfftpack.f:294 PIMACH */
static const double kBreakTol = 1.2325951644078309e-32;           /* GETBREAK = DLAMCH('E')**2 */

static long cell_size(int nr, int nz) { return (long)(nr + 2) * (nz + 2); }
static long u_size(int nr, int nz) { return (long)(nr + 3) * (nz + 2); }
static long v_size(int nr, int nz) { return (long)(nr + 2) * (nz + 1); }
static long uv_len(int nr, int nz) { return (long)(nr + 1) * nz + (long)nr * (nz - 1); }

static double* dalloc(long n) { return (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

/* The OpenMP build (-DORC_OPENMP, used for the all-cores CPU timing) splits the independent
 * sequences of a transform across threads; every output is still summed by one thread in
 * the serial order, so both builds give identical results. */
#ifdef ORC_OPENMP
#define ORC_PARALLEL _Pragma("omp parallel")
#define ORC_FOR _Pragma("omp for schedule(static)")
#else
#define ORC_PARALLEL
#define ORC_FOR
#endif

/* ---------------------------------------------------------------------------------------
 * BLAS-1 (the MKL routines BiCGSTABREVCOM calls), sequential order.
 * ------------------------------------------------------------------------------------- */
static double ddot(long n, const double* x, const double* y) {
    double s = 0.0;
    for (long i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}
static double dnrm2(long n, const double* x) { return sqrt(ddot(n, x, x)); }
static void daxpy(long n, double a, const double* x, double* y) {
    for (long i = 0; i < n; ++i) y[i] += a * x[i];
}

/* ---------------------------------------------------------------------------------------
 * setup() tables: microfluidics_complex_domain/setup.f90:106-155.
 * ------------------------------------------------------------------------------------- */
void orc_setup_tables(const drd_params* P, double* ph_lcc, double* pre_lcc) {
    const int nr = P->nr, nz = P->nz;
    const double dr2 = P->dr * P->dr, dz2 = P->dz * P->dz;
    /* Pre_Lcc(0:nr,0:nz) = -(fmx(i)+fmy(j)), fmx(i) = 4 sin^2(pi i/(2 nr))/dr2; Pre_Lcc(0,0) = -1 */
    for (int j = 0; j <= nz; ++j) {
        double t1 = kPi * j / 2.0 / nz;
        double fmy = 4.0 * (sin(t1) * sin(t1)) / dz2;
        for (int i = 0; i <= nr; ++i) {
            double t0 = kPi * i / 2.0 / nr;
            double fmx = 4.0 * (sin(t0) * sin(t0)) / dr2;
            pre_lcc[i + (long)j * (nr + 1)] = -(fmx + fmy);
        }
    }
    pre_lcc[0] = -1.0; /* setup.f90:131 */
    /* Ph_Lcc(0:nr-1,0:nz-1) with the eigenvalues of the (nr-1, nz-1)-interval grid (:134-155) */
    for (int j = 0; j < nz; ++j) {
        double t1 = kPi * j / 2.0 / (nz - 1);
        double fmy = 4.0 * (sin(t1) * sin(t1)) / dz2;
        for (int i = 0; i < nr; ++i) {
            double t0 = kPi * i / 2.0 / (nr - 1);
            double fmx = 4.0 * (sin(t0) * sin(t0)) / dr2;
            double temp = fmx + fmy;
            ph_lcc[i + (long)j * nr] = 1. + P->xld * P->dt * P->s_implicit * temp / P->I_thickness +
                                       P->xld * P->I_thickness * P->dt * (temp * temp);
        }
    }
}

/* ---------------------------------------------------------------------------------------
 * Transforms by direct summation of their definitions.
 * ------------------------------------------------------------------------------------- */

/* VCOST (lib/vfftpack.f:689-704):
 *   X_i = ( x_1 + (-1)^(i-1) x_N + sum_{k=2}^{N-1} 2 x_k cos((k-1)(i-1) pi/(N-1)) ) / sqrt(2(N-1))
 * with pi = PIMACH.  Self-inverse. */
void orc_vcost(int n, int m, double* x, long seq_stride, long elem_stride) {
    if (n < 2 || m <= 0) return;
    const long period = 2L * (n - 1);
    double* tab = dalloc(period);
    double* in = dalloc(n);
    for (long q = 0; q < period; ++q) tab[q] = cos((double)q * kPimach / (double)(n - 1));
    const double scale = sqrt(2.0 * (n - 1));
    free(in);
    ORC_PARALLEL
    {
        double* buf = dalloc(n);
        ORC_FOR
        for (int s = 0; s < m; ++s) {
            double* xs = x + (long)s * seq_stride;
            for (int j = 0; j < n; ++j) buf[j] = xs[j * elem_stride];
            for (int i = 0; i < n; ++i) {
                double acc = buf[0] + ((i & 1) ? -buf[n - 1] : buf[n - 1]);
                long idx = 0;
                for (int k = 1; k < n - 1; ++k) {
                    idx += i;
                    if (idx >= period) idx -= period * (idx / period);
                    acc += 2.0 * buf[k] * tab[idx];
                }
                xs[i * elem_stride] = acc / scale;
            }
        }
        free(buf);
    }
    free(tab);
}

/* REDFT10 (DCT-II, FFTW manual): Y_k = 2 sum_{j=0}^{n-1} X_j cos(pi (j+1/2) k / n). */
void orc_redft10(int n, int m, double* x, long seq_stride, long elem_stride) {
    if (n < 1 || m <= 0) return;
    const long period = 4L * n;
    double* tab = dalloc(period);
    double* in = dalloc(n);
    for (long q = 0; q < period; ++q) tab[q] = cos(kPi * (double)q / (2.0 * n));
    free(in);
    ORC_PARALLEL
    {
        double* buf = dalloc(n);
        ORC_FOR
        for (int s = 0; s < m; ++s) {
            double* xs = x + (long)s * seq_stride;
            for (int j = 0; j < n; ++j) buf[j] = xs[j * elem_stride];
            for (int k = 0; k < n; ++k) {
                double acc = 0.0;
                for (int j = 0; j < n; ++j) acc += buf[j] * tab[((long)(2 * j + 1) * k) % period];
                xs[k * elem_stride] = 2.0 * acc;
            }
        }
        free(buf);
    }
    free(tab);
}

/* REDFT01 (DCT-III, FFTW manual): Y_k = X_0 + 2 sum_{j=1}^{n-1} X_j cos(pi j (k+1/2) / n). */
void orc_redft01(int n, int m, double* x, long seq_stride, long elem_stride) {
    if (n < 1 || m <= 0) return;
    const long period = 4L * n;
    double* tab = dalloc(period);
    double* in = dalloc(n);
    for (long q = 0; q < period; ++q) tab[q] = cos(kPi * (double)q / (2.0 * n));
    free(in);
    ORC_PARALLEL
    {
        double* buf = dalloc(n);
        ORC_FOR
        for (int s = 0; s < m; ++s) {
            double* xs = x + (long)s * seq_stride;
            for (int j = 0; j < n; ++j) buf[j] = xs[j * elem_stride];
            for (int k = 0; k < n; ++k) {
                double acc = 0.0;
                for (int j = 1; j < n; ++j) acc += buf[j] * tab[((long)j * (2 * k + 1)) % period];
                xs[k * elem_stride] = buf[0] + 2.0 * acc;
            }
        }
        free(buf);
    }
    free(tab);
}

/* ---------------------------------------------------------------------------------------
 * op_double_gradient_Neum: microfluidics_complex_domain/matrix_tool.f90:178-219.
 * out = 0 everywhere, then the variable-coefficient 5-point operator on the interior with
 * zero flux through the domain faces.  Reads no ghost values.
 * ------------------------------------------------------------------------------------- */
void orc_op_double_gradient_neum(int nr, int nz, double dx2, double dy2, const double* x,
                                 const double* mo, double* out) {
    memset(out, 0, sizeof(double) * cell_size(nr, nz));
    for (int j = 0; j < nz; ++j) {
        for (int i = 0; i < nr; ++i) {
            double moL, moR, acc = 0.0;
            if (i == 0) {
                moL = (mo[CI(i, j)] + mo[CI(i, j)]) / 2.0;
                moR = (mo[CI(i, j)] + mo[CI(i + 1, j)]) / 2.0;
                acc = acc + 1.0 / dx2 * (moL * x[CI(i, j)] + moR * x[CI(i + 1, j)] - (moL + moR) * x[CI(i, j)]);
            } else if (i == nr - 1) {
                moL = (mo[CI(i - 1, j)] + mo[CI(i, j)]) / 2.0;
                moR = (mo[CI(i, j)] + mo[CI(i, j)]) / 2.0;
                acc = acc + 1.0 / dx2 * (moL * x[CI(i - 1, j)] + moR * x[CI(i, j)] - (moL + moR) * x[CI(i, j)]);
            } else {
                moL = (mo[CI(i - 1, j)] + mo[CI(i, j)]) / 2.0;
                moR = (mo[CI(i, j)] + mo[CI(i + 1, j)]) / 2.0;
                acc = acc + 1.0 / dx2 * (moL * x[CI(i - 1, j)] + moR * x[CI(i + 1, j)] - (moL + moR) * x[CI(i, j)]);
            }
            if (j == 0) {
                moL = (mo[CI(i, j)] + mo[CI(i, j)]) / 2.0;
                moR = (mo[CI(i, j)] + mo[CI(i, j + 1)]) / 2.0;
                acc = acc + 1.0 / dy2 * (moL * x[CI(i, j)] + moR * x[CI(i, j + 1)] - (moL + moR) * x[CI(i, j)]);
            } else if (j == nz - 1) {
                moL = (mo[CI(i, j - 1)] + mo[CI(i, j)]) / 2.0;
                moR = (mo[CI(i, j)] + mo[CI(i, j)]) / 2.0;
                acc = acc + 1.0 / dy2 * (moL * x[CI(i, j - 1)] + moR * x[CI(i, j)] - (moL + moR) * x[CI(i, j)]);
            } else {
                moL = (mo[CI(i, j - 1)] + mo[CI(i, j)]) / 2.0;
                moR = (mo[CI(i, j)] + mo[CI(i, j + 1)]) / 2.0;
                acc = acc + 1.0 / dy2 * (moL * x[CI(i, j - 1)] + moR * x[CI(i, j + 1)] - (moL + moR) * x[CI(i, j)]);
            }
            out[CI(i, j)] = acc;
        }
    }
}

/* ---------------------------------------------------------------------------------------
 * Pack / unpack: microfluidics_complex_domain/matrix_tool.f90:5-173.
 * ------------------------------------------------------------------------------------- */
static void atob_cell(int nr, int nz, const double* f, double* b) { /* Atob(nr-1,nz-1,...) :142-155 */
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i) b[i + (long)nr * j] = f[CI(i, j)];
}
static void btoa_cell(int nr, int nz, double* f, const double* b) { /* btoA(nr-1,nz-1,...) :160-173 */
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i) f[CI(i, j)] = b[i + (long)nr * j];
}
static void atob_uv(int nr, int nz, const double* f1, const double* f2, double* b) { /* :5-26 */
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i <= nr; ++i) b[i + (long)(nr + 1) * j] = f1[UI(i, j)];
    const long mn = (long)(nr + 1) * nz;
    for (int j = 1; j < nz; ++j)
        for (int i = 0; i < nr; ++i) b[i + (long)nr * (j - 1) + mn] = f2[VI(i, j)];
}
static void btoa_uv(int nr, int nz, double* f1, double* f2, const double* b) { /* :32-75 */
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i <= nr; ++i) f1[UI(i, j)] = b[i + (long)(nr + 1) * j];
    const long mn = (long)(nr + 1) * nz;
    for (int j = 1; j < nz; ++j)
        for (int i = 0; i < nr; ++i) f2[VI(i, j)] = b[i + (long)nr * (j - 1) + mn];
    for (int i = 0; i <= nr; ++i) {
        f1[UI(i, -1)] = -f1[UI(i, 0)];
        f1[UI(i, nz)] = -f1[UI(i, nz - 1)];
    }
    for (int j = -1; j <= nz; ++j) {
        f1[UI(-1, j)] = f1[UI(1, j)];
        f1[UI(nr + 1, j)] = f1[UI(nr - 1, j)];
    }
    for (int i = 0; i < nr; ++i) {
        f2[VI(i, 0)] = 0;
        f2[VI(i, nz)] = 0;
    }
    for (int j = 0; j <= nz; ++j) {
        f2[VI(-1, j)] = f2[VI(0, j)];
        f2[VI(nr, j)] = f2[VI(nr - 1, j)];
    }
}
static void atob_ph_mu(int nr, int nz, const double* f1, const double* f2, double* b) { /* :82-98 */
    const long mn = (long)nr * nz;
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i) {
            b[i + (long)nr * j] = f1[CI(i, j)];
            b[i + (long)nr * j + mn] = f2[CI(i, j)];
        }
}
static void btoa_ph_mu(int nr, int nz, double* f1, double* f2, const double* b) { /* :104-136 */
    const long mn = (long)nr * nz;
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i) {
            f1[CI(i, j)] = b[i + (long)nr * j];
            f2[CI(i, j)] = b[i + (long)nr * j + mn];
        }
    for (int i = 0; i < nr; ++i) {
        f1[CI(i, -1)] = f1[CI(i, 0)];
        f1[CI(i, nz)] = f1[CI(i, nz - 1)];
        f2[CI(i, -1)] = f2[CI(i, 0)];
        f2[CI(i, nz)] = f2[CI(i, nz - 1)];
    }
    for (int j = -1; j <= nz; ++j) {
        f1[CI(-1, j)] = f1[CI(0, j)];
        f1[CI(nr, j)] = f1[CI(nr - 1, j)];
        f2[CI(-1, j)] = f2[CI(0, j)];
        f2[CI(nr, j)] = f2[CI(nr - 1, j)];
    }
}

/* ---------------------------------------------------------------------------------------
 * BiCGSTAB: lib/BiCGSTAB.f:153-217 driving lib/BiCGSTABREVCOM.f:150-418 with
 * lib/STOPTEST2.f:281-290.  Right preconditioning, absolute early tests at :248 and
 * :313, relative final test in STOPTEST2, breakdown at |rho|,|omega| < eps^2.
 * ------------------------------------------------------------------------------------- */
int orc_bicgstab(long n, const double* b, double* x, int maxit, double tol, orc_matvec_fn mv,
                 orc_psolve_fn ps, void* ctx, drd_status* st) {
    drd_status local;
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    if (n < 0) { st->info = -1; return -1; }
    if (maxit <= 0) { st->info = -3; return -3; }
    double* r = dalloc(n);
    double* rtld = dalloc(n);
    double* p = dalloc(n);
    double* v = dalloc(n);
    double* t = dalloc(n);
    double* phat = dalloc(n);
    double* shat = dalloc(n);
    int info = 0, iter = maxit;
    double resid = tol, rho = 0.0, rho1 = 0.0, alpha = 0.0, omega = 0.0, bnrm2;

    memcpy(r, b, sizeof(double) * n);
    if (dnrm2(n, x) != 0.0) {
        mv(ctx, -1.0, x, 1.0, r);
        if (dnrm2(n, r) <= tol) { st->flags |= DRD_FLAG_EARLY_X0; goto done; }
    }
    memcpy(rtld, r, sizeof(double) * n);
    bnrm2 = dnrm2(n, b);
    if (bnrm2 == 0.0) bnrm2 = 1.0;
    iter = 0;
    for (;;) {
        iter = iter + 1;
        rho = ddot(n, rtld, r);
        if (fabs(rho) < kBreakTol) { info = -10; goto done; }
        if (iter > 1) {
            double beta = (rho / rho1) * (alpha / omega);
            daxpy(n, -omega, v, p);
            for (long q = 0; q < n; ++q) p[q] = beta * p[q];
            daxpy(n, 1.0, r, p);
        } else {
            memcpy(p, r, sizeof(double) * n);
        }
        ps(ctx, p, phat);
        mv(ctx, 1.0, phat, 0.0, v);
        alpha = rho / ddot(n, rtld, v);
        daxpy(n, -alpha, v, r); /* s = r - alpha v, s aliases r */
        if (dnrm2(n, r) <= tol) {
            daxpy(n, alpha, phat, x);
            resid = dnrm2(n, r) / bnrm2;
            st->flags |= DRD_FLAG_EARLY_S;
            info = 0;
            goto done;
        }
        ps(ctx, r, shat);
        mv(ctx, 1.0, shat, 0.0, t);
        omega = ddot(n, t, r) / ddot(n, t, t);
        daxpy(n, alpha, phat, x);
        daxpy(n, omega, shat, x);
        daxpy(n, -omega, t, r);
        resid = dnrm2(n, r) / bnrm2; /* STOPTEST2 */
        if (resid <= tol) { info = 0; goto done; }
        if (iter == maxit) { info = 1; goto done; }
        if (fabs(omega) < kBreakTol) { info = (fabs(rho) < kBreakTol) ? -10 : -11; goto done; }
        rho1 = rho;
    }
done:
    st->info = info;
    st->iter = iter;
    st->resid = resid;
    /* true residual of the returned x (not part of the reference; reported alongside) */
    {
        memcpy(t, b, sizeof(double) * n);
        mv(ctx, -1.0, x, 1.0, t);
        double bn = dnrm2(n, b);
        st->true_resid = dnrm2(n, t) / (bn == 0.0 ? 1.0 : bn);
    }
    free(r); free(rtld); free(p); free(v); free(t); free(phat); free(shat);
    return info;
}

/* ---------------------------------------------------------------------------------------
 * CH operators: microfluidics_complex_domain/PhSolve.f90:240-313.
 * ------------------------------------------------------------------------------------- */
void orc_ch_matvec(const drd_params* P, const double* M0, const double* Mi, double alpha,
                   const double* x, double beta, double* y) {
    const int nr = P->nr, nz = P->nz;
    const double dr2 = P->dr * P->dr, dz2 = P->dz * P->dz;
    const long cs = cell_size(nr, nz);
    double* f1 = dalloc(cs);
    double* ff1 = dalloc(cs);
    double* ff2 = dalloc(cs);
    btoa_cell(nr, nz, f1, x);
    orc_op_double_gradient_neum(nr, nz, dr2, dz2, f1, M0, ff1);
    for (long q = 0; q < cs; ++q) ff1[q] = -(P->dt * P->xld * ff1[q]);
    orc_op_double_gradient_neum(nr, nz, dr2, dz2, ff1, Mi, ff2);
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i) {
            long c = CI(i, j), q = i + (long)nr * j;
            double a = P->s_implicit * ff1[c] / P->I_thickness - P->I_thickness * ff2[c];
            double av = f1[c] + a;
            y[q] = (beta == 0.0) ? alpha * av : alpha * av + beta * y[q];
        }
    free(f1); free(ff1); free(ff2);
}

/* PSolve_CG -> DCT(nr-1, nz-1, f1, f2, Ph_Lcc, ...) (microfluidics_complex_domain/DCT.f90:1-57):
 * VCOST along z, VCOST along x, divide by Ph_Lcc, VCOST along z, VCOST along x. */
void orc_ch_psolve(const drd_params* P, const double* ph_lcc, const double* x, double* y) {
    const int nr = P->nr, nz = P->nz;
    const long n = (long)nr * nz;
    double* w = dalloc(n);
    memcpy(w, x, sizeof(double) * n);
    orc_vcost(nz, nr, w, 1, nr); /* sequences along z: one per i */
    orc_vcost(nr, nz, w, nr, 1); /* sequences along x: one per k */
    for (long q = 0; q < n; ++q) w[q] = w[q] / ph_lcc[q];
    orc_vcost(nz, nr, w, 1, nr);
    orc_vcost(nr, nz, w, nr, 1);
    memcpy(y, w, sizeof(double) * n);
    free(w);
}

typedef struct { const drd_params* P; const double* M0; const double* Mi; const double* lcc; } ch_ctx;
static void ch_mv_cb(void* c, double a, const double* x, double b, double* y) {
    ch_ctx* C = (ch_ctx*)c;
    orc_ch_matvec(C->P, C->M0, C->Mi, a, x, b, y);
}
static void ch_ps_cb(void* c, const double* x, double* y) {
    ch_ctx* C = (ch_ctx*)c;
    orc_ch_psolve(C->P, C->lcc, x, y);
}

/* ch_bulk_energy: microfluidics_complex_domain/ch_bulk_energy.f90:4-28 (localised double well). */
static double bulk_mf(double phi, double psi) {
    double aa = (phi * phi) * ((1.0 - phi) * (1.0 - phi));
    aa = 1.0 - sqrt(aa / (aa + 1.0E-2)) * psi;
    return 0.5 * phi * (1.0 - phi) * (1.0 - 2.0 * phi) * aa;
}

/* RHS of PhSolve (microfluidics_complex_domain/PhSolve.f90:26-63): f2 (CELL), the packed
 * rhs -f1 + s f2/eps - eps L_Mi(f2) and the packed initial guess rmu. */
void orc_ch_system(const drd_params* P, const double* u, const double* v, const double* ph, const double* rmu,
                   const double* bdr_ph, const double* bdr_ph_grad, const double* Mi, double* f2, double* rhs,
                   double* x0) {
    const int nr = P->nr, nz = P->nz;
    const double dr = P->dr, dz = P->dz, dt = P->dt, eps = P->I_thickness, s = P->s_implicit;
    const double dr2 = dr * dr, dz2 = dz * dz;
    const long cs = cell_size(nr, nz);
    double* f1 = dalloc(cs);
    double* ff = dalloc(cs);
    memcpy(f2, ph, sizeof(double) * cs); /* :26 */
    for (int k = 0; k < nz; ++k)        /* :29-34 */
        for (int i = 0; i < nr; ++i)
            f2[CI(i, k)] = f2[CI(i, k)] -
                           dt * (u[UI(i + 1, k)] + u[UI(i, k)]) / 2.0 * (ph[CI(i + 1, k)] - ph[CI(i - 1, k)]) / 2.0 / dr -
                           dt * (v[VI(i, k + 1)] + v[VI(i, k)]) / 2.0 * (ph[CI(i, k + 1)] - ph[CI(i, k - 1)]) / 2.0 / dz;
    const double cang = cos(P->angle * kPi / 180);
    for (int k = 0; k < nz; ++k) /* :37-42 */
        for (int i = 0; i < nr; ++i) {
            double p0 = ph[CI(i, k)];
            f1[CI(i, k)] = s * p0 / eps - bulk_mf(p0, bdr_ph[CI(i, k)]) / eps -
                           p0 * (p0 - 1.0) * bdr_ph_grad[CI(i, k)] * cang / sqrt(2.0);
        }
    orc_op_double_gradient_neum(nr, nz, dr2, dz2, f2, Mi, ff); /* :47 */
    for (int k = 0; k < nz; ++k)                               /* :48 (interior is what Atob reads) */
        for (int i = 0; i < nr; ++i) {
            long c = CI(i, k);
            f1[c] = -f1[c] + s * f2[c] / eps - eps * ff[c];
        }
    atob_cell(nr, nz, f1, rhs); /* :62-63 */
    atob_cell(nr, nz, rmu, x0);
    free(f1);
    free(ff);
}

/* PhSolve: microfluidics_complex_domain/PhSolve.f90:1-126. */
int orc_phsolve(const drd_params* P, const double* ph_lcc, const double* u, const double* v,
                const double* ph, const double* rmu, const double* bdr_ph, const double* bdr_ph_grad,
                const double* M0, const double* Mi, double* rmu_after, double* ph_after, drd_status* st) {
    const int nr = P->nr, nz = P->nz;
    const double dr2 = P->dr * P->dr, dz2 = P->dz * P->dz, dt = P->dt;
    const long cs = cell_size(nr, nz), n = (long)nr * nz;
    double* f2 = dalloc(cs);
    double* ff = dalloc(cs);
    double* rhs = dalloc(n);
    double* x = dalloc(n);
    orc_ch_system(P, u, v, ph, rmu, bdr_ph, bdr_ph_grad, Mi, f2, rhs, x);
    ch_ctx C = {P, M0, Mi, ph_lcc};
    int info = orc_bicgstab(n, rhs, x, P->ch_maxit, P->tol, ch_mv_cb, ch_ps_cb, &C, st); /* :72-74 */
    memcpy(rmu_after, rmu, sizeof(double) * cs);
    btoa_cell(nr, nz, rmu_after, x); /* :85 */
    for (int i = 0; i < nr; ++i) {   /* :88-96 */
        rmu_after[CI(i, -1)] = rmu_after[CI(i, 0)];
        rmu_after[CI(i, nz)] = rmu_after[CI(i, nz - 1)];
    }
    for (int k = -1; k <= nz; ++k) {
        rmu_after[CI(-1, k)] = rmu_after[CI(0, k)];
        rmu_after[CI(nr, k)] = rmu_after[CI(nr - 1, k)];
    }
    orc_op_double_gradient_neum(nr, nz, dr2, dz2, rmu_after, M0, ff); /* :100-101 */
    for (long q = 0; q < cs; ++q) ph_after[q] = f2[q] + dt * P->xld * ff[q];
    for (int i = 0; i < nr; ++i) { /* :111-124 */
        ph_after[CI(i, -1)] = ph_after[CI(i, 0)];
        ph_after[CI(i, nz)] = ph_after[CI(i, nz - 1)];
    }
    for (int k = -1; k <= nz; ++k) {
        ph_after[CI(-1, k)] = ph_after[CI(0, k)];
        ph_after[CI(nr, k)] = ph_after[CI(nr - 1, k)];
    }
    free(f2); free(ff); free(rhs); free(x);
    return info;
}

/* ---------------------------------------------------------------------------------------
 * PhSolve_ori: microfluidics_complex_domain/PhSolve_ori.f90 (phi in [-1,1], constant
 * mobility, wall-energy boundary rows), the solve finit repeats to smooth the wall indicator
 * (finit.f90:120-189).  Neumann left/right (laplace_nn) and the non-dynamic wall branch, which
 * is what finit selects (finit.f90:144-147).
 * ------------------------------------------------------------------------------------- */
/* laplace_nn (PhSolve_ori.f90:463-487): writes a's Neumann ghosts, then the 5-point Laplacian. */
static void laplace_nn(int nr, int nz, double dr2, double dz2, double* a, double* b) {
    for (int i = 0; i < nr; ++i) {
        a[CI(i, -1)] = a[CI(i, 0)];
        a[CI(i, nz)] = a[CI(i, nz - 1)];
    }
    for (int j = -1; j <= nz; ++j) {
        a[CI(-1, j)] = a[CI(0, j)];
        a[CI(nr, j)] = a[CI(nr - 1, j)];
    }
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i)
            b[CI(i, j)] = (a[CI(i + 1, j)] + a[CI(i - 1, j)] - 2 * a[CI(i, j)]) / dr2 +
                          (a[CI(i, j + 1)] + a[CI(i, j - 1)] - 2 * a[CI(i, j)]) / dz2;
}

/* coef_bot = coef_top of the non-dynamic branch (PhSolve_ori.f90:71-74, :111-113). */
double orc_ori_coef(const drd_params* P, double alpha_s) {
    const double tmp1 = P->I_thickness / P->dz + 0.5 * alpha_s;
    return (P->I_thickness / P->dz - 0.5 * alpha_s) / tmp1;
}

typedef struct { const drd_params* P; double cb, ct; const double* lcc; } ori_ctx;

/* MATRIX_VECTOR_CG_ori (PhSolve_ori.f90:368-421). */
void orc_ori_matvec(const drd_params* P, double coef_bot, double coef_top, double alpha, const double* x,
                    double beta, double* y) {
    const int nr = P->nr, nz = P->nz;
    const long cs = cell_size(nr, nz);
    const double dr2 = P->dr * P->dr, dz2 = P->dz * P->dz, eps = P->I_thickness;
    double* f1 = dalloc(cs);
    double* ff1 = dalloc(cs);
    double* ff2 = dalloc(cs);
    btoa_cell(nr, nz, f1, x);
    laplace_nn(nr, nz, dr2, dz2, f1, ff1);
    for (long q = 0; q < cs; ++q) ff1[q] = -eps * ff1[q];
    for (int i = 0; i < nr; ++i) {
        int j = 0;
        ff1[CI(i, j)] = ff1[CI(i, j)] + eps / dz2 * (f1[CI(i, j - 1)] - coef_bot * f1[CI(i, j)]);
        j = nz - 1;
        ff1[CI(i, j)] = ff1[CI(i, j)] + eps / dz2 * (f1[CI(i, j + 1)] - coef_top * f1[CI(i, j)]);
    }
    for (long q = 0; q < cs; ++q) ff1[q] = ff1[q] + f1[q] * P->s_implicit / eps;
    laplace_nn(nr, nz, dr2, dz2, ff1, ff2);
    for (long q = 0; q < cs; ++q) ff2[q] = -(P->dt * P->xld * ff2[q]);
    for (long q = 0; q < cs; ++q) ff2[q] = f1[q] + ff2[q];
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i) {
            const long q = i + (long)nr * j;
            y[q] = alpha * ff2[CI(i, j)] + beta * y[q];
        }
    free(f1); free(ff1); free(ff2);
}
static void ori_mv_cb(void* c, double a, const double* x, double b, double* y) {
    ori_ctx* C = (ori_ctx*)c;
    orc_ori_matvec(C->P, C->cb, C->ct, a, x, b, y);
}
static void ori_ps_cb(void* c, const double* x, double* y) {
    ori_ctx* C = (ori_ctx*)c;
    orc_ch_psolve(C->P, C->lcc, x, y); /* PSolve_CG_ori: the same DCT preconditioner (:426-441) */
}

/* RHS of PhSolve_ori (:23-139): f2 (CELL), packed rhs and guess Atob(ph), wall terms pnb/pnt. */
void orc_ori_system(const drd_params* P, const double* u, const double* v, const double* ph, const double* angleB,
                    const double* angleT, double alpha_s, double* f2, double* rhs, double* x0, double* pnb,
                    double* pnt) {
    const int nr = P->nr, nz = P->nz;
    const double dr = P->dr, dz = P->dz, dt = P->dt, eps = P->I_thickness, s = P->s_implicit;
    const double dr2 = dr * dr, dz2 = dz * dz;
    const long cs = cell_size(nr, nz);
    double* f1 = dalloc(cs);
    double* ff = dalloc(cs);
    memcpy(f2, ph, sizeof(double) * cs); /* :23 */
    for (int k = 0; k < nz; ++k)        /* :26-32 */
        for (int i = 0; i < nr; ++i)
            f2[CI(i, k)] = f2[CI(i, k)] -
                           dt * (u[UI(i + 1, k)] + u[UI(i, k)]) / 2.0 * (ph[CI(i + 1, k)] - ph[CI(i - 1, k)]) / 2.0 / dr -
                           dt * (v[VI(i, k + 1)] + v[VI(i, k)]) / 2.0 * (ph[CI(i, k + 1)] - ph[CI(i, k - 1)]) / 2.0 / dz;
    for (int k = 0; k < nz; ++k) /* :35-39 */
        for (int i = 0; i < nr; ++i) {
            const double p0 = ph[CI(i, k)];
            f1[CI(i, k)] = ((1. + s) * p0 - p0 * p0 * p0) / eps;
        }
    const double tmp1 = eps / dz + 0.5 * alpha_s;
    for (int i = 0; i < nr; ++i) { /* :44-49, :71-78 */
        const int k = 0;
        const double cf = sqrt(2.0) * cos((angleB ? angleB[i] : 0.0) * kPi / 180.0) / 3.0 * kPi / 2.;
        const double tmp = (ph[CI(i, k - 1)] + ph[CI(i, k)]) / 2.0;
        pnb[i] = cf * cos(tmp * kPi / 2) + alpha_s * tmp;
        pnb[i] = pnb[i] / tmp1;
        f1[CI(i, k)] = f1[CI(i, k)] + pnb[i] * eps / dz2;
    }
    for (int i = 0; i < nr; ++i) { /* :84-89, :110-118 */
        const int k = nz - 1;
        const double cf = sqrt(2.0) * cos((angleT ? angleT[i] : 0.0) * kPi / 180.0) / 3.0 * kPi / 2.;
        const double tmp = (ph[CI(i, k)] + ph[CI(i, k + 1)]) / 2.0;
        pnt[i] = cf * cos(tmp * kPi / 2) + alpha_s * tmp;
        pnt[i] = pnt[i] / tmp1;
        f1[CI(i, k)] = f1[CI(i, k)] + pnt[i] * eps / dz2;
    }
    laplace_nn(nr, nz, dr2, dz2, f1, ff); /* :126-130 */
    for (long q = 0; q < cs; ++q) f2[q] = f2[q] - dt * P->xld * ff[q];
    atob_cell(nr, nz, f2, rhs); /* :137-138 */
    atob_cell(nr, nz, ph, x0);
    free(f1); free(ff);
}

/* rmu from ph with its ghosts (PhSolve_ori.f90:187-194, finit.f90:163-169), interior. */
static void ori_rmu(int nr, int nz, double dr2, double dz2, double eps, const double* ph, double* rmu) {
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) {
            const double p0 = ph[CI(i, k)];
            rmu[CI(i, k)] = -eps * ((ph[CI(i + 1, k)] + ph[CI(i - 1, k)] - 2 * p0) / dr2 +
                                    (ph[CI(i, k + 1)] + ph[CI(i, k - 1)] - 2 * p0) / dz2) -
                            p0 / eps + p0 * p0 * p0 / eps;
        }
}

/* PhSolve_ori(rmu_after, ph_after, t) (PhSolve_ori.f90:1-214); t is unused by the routine. */
int orc_phsolve_ori(const drd_params* P, const double* ph_lcc, const double* u, const double* v, const double* ph,
                    const double* angleB, const double* angleT, double alpha_s, double* rmu_after, double* ph_after,
                    drd_status* st) {
    const int nr = P->nr, nz = P->nz;
    const double dr2 = P->dr * P->dr, dz2 = P->dz * P->dz;
    const long cs = cell_size(nr, nz), n = (long)nr * nz;
    double* f2 = dalloc(cs);
    double* rhs = dalloc(n);
    double* x = dalloc(n);
    double* pnb = dalloc(nr);
    double* pnt = dalloc(nr);
    orc_ori_system(P, u, v, ph, angleB, angleT, alpha_s, f2, rhs, x, pnb, pnt);
    const double cb = orc_ori_coef(P, alpha_s);
    ori_ctx C = {P, cb, cb, ph_lcc};
    int info = orc_bicgstab(n, rhs, x, P->ch_maxit, P->tol, ori_mv_cb, ori_ps_cb, &C, st); /* :146-147 */
    memset(ph_after, 0, sizeof(double) * cs);
    btoa_cell(nr, nz, ph_after, x); /* :156 */
    for (int i = 0; i < nr; ++i) {  /* :159-162 */
        ph_after[CI(i, -1)] = ph_after[CI(i, 0)] * cb + pnb[i];
        ph_after[CI(i, nz)] = ph_after[CI(i, nz - 1)] * cb + pnt[i];
    }
    for (int k = -1; k <= nz; ++k) { /* :169-173 */
        ph_after[CI(-1, k)] = ph_after[CI(0, k)];
        ph_after[CI(nr, k)] = ph_after[CI(nr - 1, k)];
    }
    memset(rmu_after, 0, sizeof(double) * cs);
    ori_rmu(nr, nz, dr2, dz2, P->I_thickness, ph_after, rmu_after); /* :178-184 */
    for (int i = 0; i < nr; ++i) {                                  /* :186-189 */
        rmu_after[CI(i, -1)] = rmu_after[CI(i, 0)];
        rmu_after[CI(i, nz)] = rmu_after[CI(i, nz - 1)];
    }
    for (int k = -1; k <= nz; ++k) { /* :197-201 */
        rmu_after[CI(-1, k)] = rmu_after[CI(0, k)];
        rmu_after[CI(nr, k)] = rmu_after[CI(nr - 1, k)];
    }
    free(f2); free(rhs); free(x); free(pnb); free(pnt);
    return info;
}

/* finit's wall smoothing (finit.f90:120-189): ph = bdr_ph with Neumann ghosts, rmu from ph,
 * `nsteps` PhSolve_ori solves with u = v = 0, then bdr_ph = (ph + 1)/2 clipped to [0, 1] on the
 * interior.  The context's dt is finit's (1e-4, finit.f90:151); angleB/angleT and alpha_s are
 * zero there (finit.f90:364-374 sets them after this loop). */
int orc_finit_wall(const drd_params* P, const double* ph_lcc, const double* bdr_in, int nsteps, double* bdr_out,
                   double* ph_out, double* rmu_out) {
    const int nr = P->nr, nz = P->nz;
    const long cs = cell_size(nr, nz);
    const long us = u_size(nr, nz), vs = v_size(nr, nz);
    double* u = dalloc(us);
    double* v = dalloc(vs);
    double* ph = dalloc(cs);
    double* rmu = dalloc(cs);
    double* pa = dalloc(cs);
    double* ra = dalloc(cs);
    memcpy(ph, bdr_in, sizeof(double) * cs); /* :123-133 */
    for (int j = 0; j < nz; ++j) {
        ph[CI(-1, j)] = ph[CI(0, j)];
        ph[CI(nr, j)] = ph[CI(nr - 1, j)];
    }
    for (int i = -1; i <= nr; ++i) {
        ph[CI(i, -1)] = ph[CI(i, 0)];
        ph[CI(i, nz)] = ph[CI(i, nz - 1)];
    }
    ori_rmu(nr, nz, P->dr * P->dr, P->dz * P->dz, P->I_thickness, ph, rmu); /* :163-169 */
    int info = 0;
    for (int it = 0; it < nsteps; ++it) { /* :172-176 */
        drd_status st;
        info = orc_phsolve_ori(P, ph_lcc, u, v, ph, NULL, NULL, 0.0, ra, pa, &st);
        memcpy(rmu, ra, sizeof(double) * cs);
        memcpy(ph, pa, sizeof(double) * cs);
    }
    for (long q = 0; q < cs; ++q) bdr_out[q] = (ph[q] + 1.0) / 2.0; /* :178 */
    for (int j = 0; j < nz; ++j)                                     /* :181-189 */
        for (int i = 0; i < nr; ++i) {
            double* b = &bdr_out[CI(i, j)];
            if (*b >= 1.0) *b = 1.0;
            else if (*b <= 0.0) *b = 0.0;
        }
    if (ph_out) memcpy(ph_out, ph, sizeof(double) * cs);
    if (rmu_out) memcpy(rmu_out, rmu, sizeof(double) * cs);
    free(u); free(v); free(ph); free(rmu); free(pa); free(ra);
    return info;
}

/* ---------------------------------------------------------------------------------------
 * Coupled CH: two_phase_flow_complex_domain/ph_mu_solve.f90:3-380, ch_bulk_energy.f90:32-67,
 * ch_bdr_condition.f90:3-27.
 * ------------------------------------------------------------------------------------- */
static double bulk_tp(double phi, double psi, int mode) {
    if (mode == 1) return 0.5 * phi * (1.0 - phi) * (1.0 - 2.0 * phi) * (1 - psi);
    return (phi * phi * phi - phi) * (1 - psi);
}
static double bdr_cond_tp(double angle, double phi, int mode) {
    double cf = cos(angle * kPi / 180.0) / sqrt(2.0);
    if (mode == 1) return cf * (1.0 - phi) * phi;
    return cf * (1.0 - phi * phi);
}

void orc_phmu_matvec(const drd_params* P, const double* M0, const double* Mi, const double* bdr_used,
                     double coef_bot, double coef_top, double alpha, const double* x, double beta,
                     double* y) {
    const int nr = P->nr, nz = P->nz;
    const double dr2 = P->dr * P->dr, dz2 = P->dz * P->dz, eps = P->I_thickness;
    const long cs = cell_size(nr, nz), mn = (long)nr * nz;
    double* f1 = dalloc(cs);
    double* f2 = dalloc(cs);
    double* ff1 = dalloc(cs);
    double* ff2 = dalloc(cs);
    btoa_ph_mu(nr, nz, f1, f2, x);
    orc_op_double_gradient_neum(nr, nz, dr2, dz2, f1, Mi, ff1); /* :214 */
    for (int j = 0; j < nz; ++j)                                  /* :216-224 */
        for (int i = 0; i < nr; ++i) {
            long c = CI(i, j);
            ff1[c] = P->s_implicit * f1[c] / eps - eps * ff1[c] - f2[c] * bdr_used[c];
        }
    for (int i = 0; i < nr; ++i) { /* :227-233 */
        ff1[CI(i, 0)] = ff1[CI(i, 0)] + eps / dz2 * (f1[CI(i, -1)] - coef_bot * f1[CI(i, 0)]);
        ff1[CI(i, nz - 1)] = ff1[CI(i, nz - 1)] + eps / dz2 * (f1[CI(i, nz)] - coef_top * f1[CI(i, nz - 1)]);
    }
    orc_op_double_gradient_neum(nr, nz, dr2, dz2, f2, M0, ff2); /* :245 */
    for (int j = 0; j < nz; ++j)                                  /* :247-253 */
        for (int i = 0; i < nr; ++i) {
            long c = CI(i, j);
            ff2[c] = f1[c] * (bdr_used[c] + P->bdr_ph_used_adjust) - P->dt * P->xld * ff2[c];
        }
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i) {
            long c = CI(i, j), q = i + (long)nr * j;
            y[q] = (beta == 0.0) ? alpha * ff1[c] : alpha * ff1[c] + beta * y[q];
            y[q + mn] = (beta == 0.0) ? alpha * ff2[c] : alpha * ff2[c] + beta * y[q + mn];
        }
    free(f1); free(f2); free(ff1); free(ff2);
}

/* PSolve_PH_MU_CG Jacobi (:304-356), including `j == nr-1` in the x test and `i == 0` in the
 * z test exactly as written there. */
void orc_phmu_psolve(const drd_params* P, const double* x, double* y) {
    const int nr = P->nr, nz = P->nz;
    const double dr2 = P->dr * P->dr, dz2 = P->dz * P->dz, eps = P->I_thickness;
    const long mn = (long)nr * nz;
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nr; ++i) {
            double tmpx = (i == 0 || j == nr - 1) ? 1.0 / dr2 : 2.0 / dr2;
            double tmpz = (i == 0 || j == nz - 1) ? 1.0 / dz2 : 2.0 / dz2;
            long q = i + (long)nr * j;
            y[q] = x[q] / ((tmpx + tmpz) * eps + P->s_implicit / eps);
            y[q + mn] = x[q + mn] / (P->dt * P->xld * (tmpx + tmpz));
        }
}

typedef struct {
    const drd_params* P; const double* M0; const double* Mi; const double* used; double cb, ct;
} phmu_ctx;
static void phmu_mv_cb(void* c, double a, const double* x, double b, double* y) {
    phmu_ctx* C = (phmu_ctx*)c;
    orc_phmu_matvec(C->P, C->M0, C->Mi, C->used, C->cb, C->ct, a, x, b, y);
}
static void phmu_ps_cb(void* c, const double* x, double* y) {
    phmu_ctx* C = (phmu_ctx*)c;
    orc_phmu_psolve(C->P, x, y);
}

/* RHS of ph_mu_solve (two_phase_flow_complex_domain/ph_mu_solve.f90:31-153): M0 (CELL,
 * recomputed from phi), packed rhs [f1; f2], packed guess [phi; mu], wall values pnb/pnt and
 * coef_bot/top. */
void orc_phmu_system(const drd_params* P, const double* u, const double* v, const double* ph, const double* rmu,
                     const double* bdr_ph, const double* bdr_ph_used, const double* bdr_ph_grad, const double* angleB,
                     const double* angleT, double* M0, double* rhs, double* x0, double* pnb, double* pnt,
                     double* coef_bot_top) {
    const int nr = P->nr, nz = P->nz, mode = P->phi_mode;
    const double dr = P->dr, dz = P->dz, dt = P->dt, eps = P->I_thickness, s = P->s_implicit;
    const double dz2 = dz * dz;
    const long cs = cell_size(nr, nz);
    double* f1 = dalloc(cs);
    double* f2 = dalloc(cs);
    for (long q = 0; q < cs; ++q) { /* :31-35 */
        double p0 = ph[q];
        if (mode == 1) M0[q] = (1.0 - bdr_ph[q]) * (p0 * p0) * ((p0 - 1.0) * (p0 - 1.0));
        else M0[q] = (1.0 - bdr_ph[q]) * ((p0 * p0 - 1.0) * (p0 * p0 - 1.0));
    }
    for (long q = 0; q < cs; ++q) f2[q] = ph[q] * (bdr_ph_used[q] + P->bdr_ph_used_adjust); /* :40 */
    for (int k = 0; k < nz; ++k) /* :43-51 */
        for (int i = 0; i < nr; ++i)
            f2[CI(i, k)] = f2[CI(i, k)] -
                           dt * (u[UI(i + 1, k)] + u[UI(i, k)]) / 2.0 *
                               (ph[CI(i + 1, k)] * bdr_ph_used[CI(i + 1, k)] - ph[CI(i - 1, k)] * bdr_ph_used[CI(i - 1, k)]) / 2.0 / dr -
                           dt * (v[VI(i, k + 1)] + v[VI(i, k)]) / 2.0 *
                               (ph[CI(i, k + 1)] * bdr_ph_used[CI(i, k + 1)] - ph[CI(i, k - 1)] * bdr_ph_used[CI(i, k - 1)]) / 2.0 / dz;
    const double cang = cos(P->angle * kPi / 180);
    for (int k = 0; k < nz; ++k) /* :55-77 */
        for (int i = 0; i < nr; ++i) {
            double p0 = ph[CI(i, k)];
            double wet = (mode == 1) ? p0 * (p0 - 1.0) : (p0 * p0 - 1.0);
            f1[CI(i, k)] = s * p0 / eps - bulk_tp(p0, bdr_ph[CI(i, k)], mode) / eps -
                           wet * bdr_ph_grad[CI(i, k)] * cang / sqrt(2.0);
        }
    double coef_bot = 1.0, coef_top = 1.0;
    for (int i = 0; i < nr; ++i) { /* :109-127 */
        double tmp = (ph[CI(i, -1)] + ph[CI(i, 0)]) / 2.0;
        pnb[i] = bdr_cond_tp(angleB[i], tmp, mode);
    }
    for (int i = 0; i < nr; ++i) {
        double tmp = eps / dz;
        coef_bot = (eps / dz) / tmp;
        pnb[i] = pnb[i] / tmp;
        f1[CI(i, 0)] = f1[CI(i, 0)] + pnb[i] * eps / dz2;
    }
    for (int i = 0; i < nr; ++i) { /* :130-149 */
        double tmp = (ph[CI(i, nz - 1)] + ph[CI(i, nz)]) / 2.0;
        pnt[i] = bdr_cond_tp(angleT[i], tmp, mode);
    }
    for (int i = 0; i < nr; ++i) {
        double tmp = eps / dz;
        coef_top = (eps / dz) / tmp;
        pnt[i] = pnt[i] / tmp;
        f1[CI(i, nz - 1)] = f1[CI(i, nz - 1)] + pnt[i] * eps / dz2;
    }
    atob_ph_mu(nr, nz, f1, f2, rhs); /* :152-153 */
    atob_ph_mu(nr, nz, ph, rmu, x0);
    if (coef_bot_top) { coef_bot_top[0] = coef_bot; coef_bot_top[1] = coef_top; }
    free(f1);
    free(f2);
}

int orc_ph_mu_solve(const drd_params* P, const double* u, const double* v, const double* ph,
                    const double* rmu, const double* bdr_ph, const double* bdr_ph_used,
                    const double* bdr_ph_grad, const double* Mi, const double* angleB,
                    const double* angleT, double* M0, double* ph_after, double* rmu_after,
                    double* coef_bot_top, drd_status* st) {
    const int nr = P->nr, nz = P->nz;
    const long cs = cell_size(nr, nz), n = 2L * nr * nz;
    double* rhs = dalloc(n);
    double* x = dalloc(n);
    double* pnb = dalloc(nr);
    double* pnt = dalloc(nr);
    double cbt[2];
    orc_phmu_system(P, u, v, ph, rmu, bdr_ph, bdr_ph_used, bdr_ph_grad, angleB, angleT, M0, rhs, x, pnb, pnt, cbt);
    phmu_ctx C = {P, M0, Mi, bdr_ph_used, cbt[0], cbt[1]};
    int info = orc_bicgstab(n, rhs, x, P->phmu_maxit, P->tol, phmu_mv_cb, phmu_ps_cb, &C, st);
    memcpy(ph_after, ph, sizeof(double) * cs);
    memcpy(rmu_after, rmu, sizeof(double) * cs);
    btoa_ph_mu(nr, nz, ph_after, rmu_after, x); /* :173-177 */
    for (int i = 0; i < nr; ++i) {
        ph_after[CI(i, -1)] = ph_after[CI(i, 0)] * cbt[0] + pnb[i];
        ph_after[CI(i, nz)] = ph_after[CI(i, nz - 1)] * cbt[1] + pnt[i];
    }
    if (coef_bot_top) { coef_bot_top[0] = cbt[0]; coef_bot_top[1] = cbt[1]; }
    free(rhs); free(x); free(pnb); free(pnt);
    return info;
}

/* ---------------------------------------------------------------------------------------
 * Momentum operators: microfluidics_complex_domain/VeloSolve_2_combined.f90:515-711 (bdf 2),
 * VeloSolve_combined.f90:516-760 (bdf 1), two_phase_flow_complex_domain/VeloSolve_2_combined.f90
 * (TP: penalty field bdr_ph_penalty, lr_bd_type, identity preconditioner).
 * ------------------------------------------------------------------------------------- */
static void uv_unpack_for_matvec(const drd_params* P, const double* x, double* f1, double* f2) {
    const int nr = P->nr, nz = P->nz;
    btoa_uv(nr, nz, f1, f2, x);
    const int tp_neumann = (P->variant == DRD_VARIANT_TP && P->lr_bd_type == 'n');
    if (!tp_neumann) {
        for (int k = 0; k < nz; ++k) { /* :536-539 */
            f1[UI(-1, k)] = -f1[UI(1, k)];
            f1[UI(nr + 1, k)] = -f1[UI(nr - 1, k)];
        }
    } else {
        for (int k = -1; k <= nz; ++k) {
            f1[UI(-1, k)] = f1[UI(1, k)];
            f1[UI(nr + 1, k)] = f1[UI(nr - 1, k)];
        }
    }
    for (int k = 0; k <= nz; ++k) { /* :540-543 */
        f2[VI(-1, k)] = f2[VI(0, k)];
        f2[VI(nr, k)] = f2[VI(nr - 1, k)];
    }
    for (int i = -1; i <= nr + 1; ++i) { /* :545-548 */
        f1[UI(i, -1)] = -f1[UI(i, 0)];
        f1[UI(i, nz)] = -f1[UI(i, nz - 1)];
    }
    for (int i = -1; i <= nr; ++i) { /* :550-553 */
        f2[VI(i, 0)] = 0.0;
        f2[VI(i, nz)] = 0.0;
    }
}

void orc_uv_matvec(const drd_params* P, int bdf, const double* rho, const double* eta,
                   const double* bdr_pen, double alpha, const double* x, double beta, double* y) {
    const int nr = P->nr, nz = P->nz;
    const double dr = P->dr, dz = P->dz, dt = P->dt, re = P->re, pk = P->penalty_k;
    const double dr2 = dr * dr, dz2 = dz * dz;
    double* f1 = dalloc(u_size(nr, nz));
    double* f2 = dalloc(v_size(nr, nz));
    double* f11 = dalloc(u_size(nr, nz));
    double* f22 = dalloc(v_size(nr, nz));
    const long N = uv_len(nr, nz);
    double* zz = dalloc(N);
    uv_unpack_for_matvec(P, x, f1, f2);
    for (int k = 0; k < nz; ++k) /* u: :577-584 */
        for (int i = 0; i <= nr; ++i) {
            if (bdf == 2)
                f11[UI(i, k)] = f1[UI(i, k)] * 1.5 * re * (rho[CI(i, k)] + rho[CI(i - 1, k)]) / 2.0 +
                                f1[UI(i, k)] * pk * (bdr_pen[CI(i, k)] + bdr_pen[CI(i - 1, k)]) / 2.0 * dt;
            else
                f11[UI(i, k)] = f1[UI(i, k)] * re * (rho[CI(i, k)] + rho[CI(i - 1, k)]) / 2.0;
        }
    for (int k = 0; k < nz; ++k) /* :587-594 */
        for (int i = 0; i <= nr; ++i) {
            double cr = eta[CI(i, k)], cl = eta[CI(i - 1, k)];
            f11[UI(i, k)] = f11[UI(i, k)] -
                            2.0 * dt * (cr * f1[UI(i + 1, k)] + cl * f1[UI(i - 1, k)] - (cl + cr) * f1[UI(i, k)]) / dr2;
        }
    for (int k = 0; k < nz; ++k) /* :597-607 */
        for (int i = 0; i <= nr; ++i) {
            double cr = (eta[CI(i, k + 1)] + eta[CI(i - 1, k + 1)] + eta[CI(i, k)] + eta[CI(i - 1, k)]) / 4.0;
            double cl = (eta[CI(i, k)] + eta[CI(i - 1, k)] + eta[CI(i, k - 1)] + eta[CI(i - 1, k - 1)]) / 4.0;
            f11[UI(i, k)] = f11[UI(i, k)] - dt * (cr * f1[UI(i, k + 1)] + cl * f1[UI(i, k - 1)] - (cl + cr) * f1[UI(i, k)]) / dz2;
            f11[UI(i, k)] = f11[UI(i, k)] -
                            dt * (cr * (f2[VI(i, k + 1)] - f2[VI(i - 1, k + 1)]) - cl * (f2[VI(i, k)] - f2[VI(i - 1, k)])) / dr / dz;
        }
    for (int k = 1; k < nz; ++k) /* v: :610-617 */
        for (int i = 0; i < nr; ++i) {
            if (bdf == 2)
                f22[VI(i, k)] = f2[VI(i, k)] * 1.5 * re * (rho[CI(i, k)] + rho[CI(i, k - 1)]) / 2.0 +
                                f2[VI(i, k)] * pk * (bdr_pen[CI(i, k)] + bdr_pen[CI(i, k - 1)]) / 2.0 * dt;
            else
                f22[VI(i, k)] = f2[VI(i, k)] * re * (rho[CI(i, k)] + rho[CI(i, k - 1)]) / 2.0;
        }
    for (int k = 1; k < nz; ++k) /* :620-627 */
        for (int i = 0; i < nr; ++i) {
            double cr = eta[CI(i, k)], cl = eta[CI(i, k - 1)];
            f22[VI(i, k)] = f22[VI(i, k)] -
                            2.0 * dt * (cr * f2[VI(i, k + 1)] + cl * f2[VI(i, k - 1)] - (cl + cr) * f2[VI(i, k)]) / dz2;
        }
    for (int k = 1; k < nz; ++k) /* :630-640 */
        for (int i = 0; i < nr; ++i) {
            double cr = (eta[CI(i + 1, k)] + eta[CI(i, k)] + eta[CI(i + 1, k - 1)] + eta[CI(i, k - 1)]) / 4.0;
            double cl = (eta[CI(i, k)] + eta[CI(i - 1, k)] + eta[CI(i, k - 1)] + eta[CI(i - 1, k - 1)]) / 4.0;
            f22[VI(i, k)] = f22[VI(i, k)] - dt * (cr * f2[VI(i + 1, k)] + cl * f2[VI(i - 1, k)] - (cl + cr) * f2[VI(i, k)]) / dr2;
            f22[VI(i, k)] = f22[VI(i, k)] -
                            dt * (cr * (f1[UI(i + 1, k)] - f1[UI(i + 1, k - 1)]) - cl * (f1[UI(i, k)] - f1[UI(i, k - 1)])) / dr / dz;
        }
    atob_uv(nr, nz, f11, f22, zz); /* :644-645 */
    for (long q = 0; q < N; ++q) y[q] = (beta == 0.0) ? alpha * zz[q] : alpha * zz[q] + beta * y[q];
    free(f1); free(f2); free(f11); free(f22); free(zz);
}

/* Jacobi of PSolve_uv_2_CG (:649-711) / PSolve_uv_CG; identity for TP (TP :779-780). */
void orc_uv_psolve(const drd_params* P, int bdf, const double* rho, const double* eta,
                   const double* x, double* y) {
    const int nr = P->nr, nz = P->nz;
    const double dt = P->dt, re = P->re, dr2 = P->dr * P->dr, dz2 = P->dz * P->dz;
    const long N = uv_len(nr, nz), mn = (long)(nr + 1) * nz;
    if (P->variant == DRD_VARIANT_TP && bdf == 2) { /* the first-step TP solve keeps Jacobi */
        memcpy(y, x, sizeof(double) * N);
        return;
    }
    const double m = (bdf == 2) ? 1.5 * re : re;
    for (int j = 0; j < nz; ++j)
        for (int i = 0; i <= nr; ++i) {
            double tmp = m * (rho[CI(i, j)] + rho[CI(i - 1, j)]) / 2.0;
            double cr = eta[CI(i, j)], cl = eta[CI(i - 1, j)];
            tmp = tmp + 2.0 * dt * (cl + cr) / dr2;
            cr = (eta[CI(i, j + 1)] + eta[CI(i - 1, j + 1)] + eta[CI(i, j)] + eta[CI(i - 1, j)]) / 4.0;
            cl = (eta[CI(i, j)] + eta[CI(i - 1, j)] + eta[CI(i, j - 1)] + eta[CI(i - 1, j - 1)]) / 4.0;
            if (j == 0) tmp = tmp + dt * (cl + (cl + cr)) / dz2;
            else if (j == nz - 1) tmp = tmp + dt * (cr + (cl + cr)) / dz2;
            else tmp = tmp + dt * (cl + cr) / dz2;
            long q = i + (long)(nr + 1) * j;
            y[q] = x[q] / tmp;
        }
    for (int j = 1; j < nz; ++j)
        for (int i = 0; i < nr; ++i) {
            double tmp = m * (rho[CI(i, j)] + rho[CI(i - 1, j)]) / 2.0; /* rho(i-1,j) as written (:690) */
            double cr = eta[CI(i, j)], cl = eta[CI(i, j - 1)];
            tmp = tmp + 2.0 * dt * (cl + cr) / dz2;
            cr = (eta[CI(i + 1, j)] + eta[CI(i, j)] + eta[CI(i + 1, j - 1)] + eta[CI(i, j - 1)]) / 4.0;
            cl = (eta[CI(i, j)] + eta[CI(i - 1, j)] + eta[CI(i, j - 1)] + eta[CI(i - 1, j - 1)]) / 4.0;
            if (i == 0) tmp = tmp + dt * cr / dr2;
            else if (i == nr - 1) tmp = tmp + dt * cl / dr2;
            else tmp = tmp + dt * (cl + cr) / dr2;
            long q = i + (long)nr * (j - 1) + mn;
            y[q] = x[q] / tmp;
        }
}

/* ---------------------------------------------------------------------------------------
 * ESOLP_x preconditioner of the momentum system: DCT-I (VCOST) along x, a tridiagonal solve
 * along y per x mode, DCT-I along x (microfluidics_complex_domain/ESOLP.f90:1-82), with the
 * coefficients ua..vc of setup (setup.f90:157-235) and the Thomas solver rfords
 * (Precipitation_dynamics/setup.f90:327-354).  The reference applies it to the u and v blocks
 * of the momentum vector in Precipitation_dynamics/VeloSolve_combined.f90:795-808.
 * ------------------------------------------------------------------------------------- */
/* rfords: forward elimination on copies of b and f, then back substitution into ff. */
static void rfords(int n, double* ff, const double* a, const double* bb, const double* c) {
    double* b = dalloc(n);
    double* f = dalloc(n);
    memcpy(b, bb, sizeof(double) * n);
    memcpy(f, ff, sizeof(double) * n);
    for (int j = 1; j < n; ++j) {
        const double r = -a[j] / b[j - 1];
        b[j] = b[j] + r * c[j - 1];
        f[j] = f[j] + r * f[j - 1];
    }
    if (fabs(b[n - 1]) <= 1.0E-12) ff[n - 1] = 0.0;
    else ff[n - 1] = f[n - 1] / b[n - 1];
    for (int j = n - 2; j >= 0; --j) ff[j] = (f[j] - c[j] * ff[j + 1]) / b[j];
    free(b);
    free(f);
}

/* setup()'s ua, ub, uc (nz rows x (nr+1) modes) and va, vb, vc ((nz-1) x nr), element
 * (row j, mode k) at [j + rows*k]; bdf 2 takes the *_2 set (mass term 1.5 t1).  t1 is pi/2:
 * the fmx loops overwrite it before use (setup.f90:159,166-169,202-205).  The slip lengths
 * enter through (2 xls_ave - dz)/(2 xls_ave + dz) with xlsT = xlsB (the no-slip deck). */
void orc_esolp_coefs(const drd_params* P, int bdf, double* ua, double* ub, double* uc, double* va, double* vb,
                     double* vc) {
    const int nr = P->nr, nz = P->nz;
    const double dt = P->dt, dr2 = P->dr * P->dr, dz2 = P->dz * P->dz, dz = P->dz;
    const double kPiG = kPi; /* global.f90:27 */
    double t1 = 0.0, xls = P->xlsB * (1.0 + 1.0) / 2.0;
    xls = (2.0 * xls - dz) / (2.0 * xls + dz);
    const double m = (bdf == 2) ? 1.5 : 1.0;
    double* fmx = dalloc(nr + 1);
    for (int i = 0; i <= nr; ++i) {
        t1 = kPiG * i / nr / 2.;
        fmx[i] = 4.0 * dt * sin(t1) * sin(t1) / dr2;
    }
    for (int k = 0; k <= nr; ++k) {
        for (int j = 0; j < nz; ++j) {
            const long q = j + (long)nz * k;
            if (j == 0) {
                ua[q] = 0.0;
                ub[q] = t1 * m + ((2.0 - xls) * dt / dz2 + fmx[k]);
                uc[q] = (-1.0 * dt / dz2);
            } else if (j == nz - 1) {
                ua[q] = (-1.0 * dt / dz2);
                ub[q] = t1 * m + ((2.0 - xls) * dt / dz2 + fmx[k]);
                uc[q] = 0.0;
            } else {
                ua[q] = (-dt / dz2);
                ub[q] = t1 * m + (2.0 * dt / dz2 + fmx[k]);
                uc[q] = (-dt / dz2);
            }
        }
    }
    for (int i = 0; i < nr; ++i) {
        t1 = kPiG * i / (nr - 1) / 2.;
        fmx[i] = 4.0 * dt * sin(t1) * sin(t1) / dr2;
    }
    const int nv = nz - 1;
    for (int k = 0; k < nr; ++k)
        for (int j = 0; j < nv; ++j) {
            const long q = j + (long)nv * k;
            va[q] = (j == 0) ? 0.0 : -dt / dz2;
            vb[q] = t1 * m + 2.0 * dt / dz2 + fmx[k];
            vc[q] = (j == nv - 1) ? 0.0 : -1.0 * dt / dz2;
        }
    free(fmx);
}

/* ESOLP_x on one block: `rows` rows of `len` values (row j, element k at [k + len*j]), in place. */
static void esolp_block(int len, int rows, double* w, const double* pa, const double* pb, const double* pc) {
    orc_vcost(len, rows, w, len, 1); /* along x, one sequence per row (ESOLP.f90:21-30) */
    double* col = dalloc(rows);
    for (int k = 0; k < len; ++k) { /* tridiagonal along y per mode (:36-57) */
        for (int j = 0; j < rows; ++j) col[j] = w[k + (long)len * j];
        rfords(rows, col, pa + (long)rows * k, pb + (long)rows * k, pc + (long)rows * k);
        for (int j = 0; j < rows; ++j) w[k + (long)len * j] = col[j];
    }
    free(col);
    orc_vcost(len, rows, w, len, 1); /* (:64-73) */
}

/* The ESOLP_x preconditioner on a packed momentum vector (Atob_uv order). */
void orc_uv_psolve_esolp(const drd_params* P, int bdf, const double* x, double* y) {
    const int nr = P->nr, nz = P->nz;
    const long N = uv_len(nr, nz), mn = (long)(nr + 1) * nz;
    double* ua = dalloc(mn); double* ub = dalloc(mn); double* uc = dalloc(mn);
    const long vn = (long)nr * (nz - 1);
    double* va = dalloc(vn); double* vb = dalloc(vn); double* vc = dalloc(vn);
    orc_esolp_coefs(P, bdf, ua, ub, uc, va, vb, vc);
    memcpy(y, x, sizeof(double) * N);
    esolp_block(nr + 1, nz, y, ua, ub, uc);
    esolp_block(nr, nz - 1, y + mn, va, vb, vc);
    free(ua); free(ub); free(uc); free(va); free(vb); free(vc);
}

/* The diagonal scaling of DRD_UV_ESOLP_SCALED (an extension of ESOLP_x): s = sqrt(D0 / D) per
 * unknown with D the Jacobi diagonal of PSolve_uv_2_CG (orc_uv_psolve's divisor) for rho, eta and
 * D0 the same for rho = eta = 1, the coefficients of ESOLP_x's constant operator. */
void orc_uv_esolp_scale(const drd_params* P, int bdf, const double* rho, const double* eta, double* s) {
    const int nr = P->nr, nz = P->nz;
    const long N = uv_len(nr, nz), cs = (long)(nr + 2) * (nz + 2);
    double* one = dalloc(cs);
    double* e = dalloc(N);
    double* d = dalloc(N);
    double* d0 = dalloc(N);
    for (long q = 0; q < cs; ++q) one[q] = 1.0;
    for (long q = 0; q < N; ++q) e[q] = 1.0;
    orc_uv_psolve(P, bdf, rho, eta, e, d);  /* 1 / D */
    orc_uv_psolve(P, bdf, one, one, e, d0); /* 1 / D0 */
    for (long q = 0; q < N; ++q) s[q] = sqrt(d[q] / d0[q]);
    free(one); free(e); free(d); free(d0);
}

/* y = s ESOLP_x(s x). */
void orc_uv_psolve_esolp_scaled(const drd_params* P, int bdf, const double* s, const double* x, double* y) {
    const long N = uv_len(P->nr, P->nz);
    double* t = dalloc(N);
    for (long q = 0; q < N; ++q) t[q] = s[q] * x[q];
    orc_uv_psolve_esolp(P, bdf, t, y);
    for (long q = 0; q < N; ++q) y[q] = s[q] * y[q];
    free(t);
}

typedef struct {
    const drd_params* P; int bdf; const double* rho; const double* eta; const double* pen; double* scale;
} uv_ctx;
static void uv_mv_cb(void* c, double a, const double* x, double b, double* y) {
    uv_ctx* C = (uv_ctx*)c;
    orc_uv_matvec(C->P, C->bdf, C->rho, C->eta, C->pen, a, x, b, y);
}
static void uv_ps_cb(void* c, const double* x, double* y) {
    uv_ctx* C = (uv_ctx*)c;
    if (C->P->uv_precond == DRD_UV_ESOLP) orc_uv_psolve_esolp(C->P, C->bdf, x, y);
    else if (C->P->uv_precond == DRD_UV_ESOLP_SCALED) orc_uv_psolve_esolp_scaled(C->P, C->bdf, C->scale, x, y);
    else orc_uv_psolve(C->P, C->bdf, C->rho, C->eta, x, y);
}

/* A x = b for the CH mu system (system 0: MATRIX_VECTOR_CG with PSolve_CG, ph_lcc the
 * Ph_Lcc table) or the momentum system (system 1, bdf 1/2) with the reference BiCGSTAB
 * (PhSolve.f90:72-74, VeloSolve_2_combined.f90:398-401); x: guess in, solution out. */
int orc_solve_system(const drd_params* P, int system, int bdf, const double* ph_lcc, const double* M0,
                     const double* Mi, const double* rho, const double* eta, const double* pen, const double* b,
                     double* x, drd_status* st) {
    if (system == 0) {
        ch_ctx C = {P, M0, Mi, ph_lcc};
        return orc_bicgstab((long)P->nr * P->nz, b, x, P->ch_maxit, P->tol, ch_mv_cb, ch_ps_cb, &C, st);
    }
    uv_ctx C = {P, bdf, rho, eta, pen, NULL};
    if (P->uv_precond == DRD_UV_ESOLP_SCALED) {
        C.scale = dalloc(uv_len(P->nr, P->nz));
        orc_uv_esolp_scale(P, bdf, rho, eta, C.scale);
    }
    const int info = orc_bicgstab(uv_len(P->nr, P->nz), b, x, P->uv_maxit, P->tol, uv_mv_cb, uv_ps_cb, &C, st);
    free(C.scale);
    return info;
}

/* ---------------------------------------------------------------------------------------
 * The solid-blended CH preconditioner (an extension of PSolve_CG, PhSolve.f90:296-313; the
 * reference has no counterpart): y = q + w (x - q) with q = PSolve_CG(x) and a per-cell weight
 * w in [0, 1] on the packed nr x nz cells.  In the solid the mobilities vanish and the CH
 * operator tends to the identity, which the constant-mobility DCT-I solve does not resolve;
 * w blends the identity in there.  The fitted weight of a geometry comes from Rademacher
 * probes e (entries +-1): r = A e, q = PSolve_CG(r), d = r - q, t = e - q and per cell
 * w = clamp(sum t d / sum d d, 0, 1) (0 where sum d d = 0), the least-squares weight that maps
 * the probes' d onto their t.
 * ------------------------------------------------------------------------------------- */
void orc_ch_psolve_blend(const drd_params* P, const double* ph_lcc, const double* w, const double* x, double* y) {
    const long n = (long)P->nr * P->nz;
    orc_ch_psolve(P, ph_lcc, x, y);
    if (!w) return;
    for (long q = 0; q < n; ++q) y[q] = y[q] + w[q] * (x[q] - y[q]);
}

/* Entry q of probe `probe`: +1 or -1 from the top bit of splitmix64(seed + (probe n + q + 1) G),
 * G = 0x9E3779B97F4A7C15 (the same integer arithmetic as the device generator). */
double orc_probe_sign(uint64_t seed, long probe, long n, long q) {
    uint64_t z = seed + (uint64_t)(probe * n + q + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return (z >> 63) ? -1.0 : 1.0;
}

void orc_ch_blend_probe(const drd_params* P, const double* ph_lcc, const double* M0, const double* Mi, int nprobe,
                        uint64_t seed, double* w) {
    const long n = (long)P->nr * P->nz;
    double* e = dalloc(n);
    double* r = dalloc(n);
    double* q = dalloc(n);
    double* num = dalloc(n);
    double* den = dalloc(n);
    for (long i = 0; i < n; ++i) num[i] = den[i] = 0.0;
    for (int p = 0; p < nprobe; ++p) {
        for (long i = 0; i < n; ++i) e[i] = orc_probe_sign(seed, p, n, i);
        orc_ch_matvec(P, M0, Mi, 1.0, e, 0.0, r);
        orc_ch_psolve(P, ph_lcc, r, q);
        for (long i = 0; i < n; ++i) {
            const double d = r[i] - q[i], t = e[i] - q[i];
            num[i] += t * d;
            den[i] += d * d;
        }
    }
    for (long i = 0; i < n; ++i) {
        const double v = den[i] > 0.0 ? num[i] / den[i] : 0.0;
        w[i] = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
    }
    free(e); free(r); free(q); free(num); free(den);
}

typedef struct { const drd_params* P; const double* M0; const double* Mi; const double* lcc; const double* w; } chb_ctx;
static void chb_mv_cb(void* c, double a, const double* x, double b, double* y) {
    chb_ctx* C = (chb_ctx*)c;
    orc_ch_matvec(C->P, C->M0, C->Mi, a, x, b, y);
}
static void chb_ps_cb(void* c, const double* x, double* y) {
    chb_ctx* C = (chb_ctx*)c;
    orc_ch_psolve_blend(C->P, C->lcc, C->w, x, y);
}

/* PhSolve's BiCGSTAB (lib/BiCGSTAB.f) with the blended preconditioner. */
int orc_ch_solve_blend(const drd_params* P, const double* ph_lcc, const double* M0, const double* Mi, const double* w,
                       const double* b, double* x, drd_status* st) {
    chb_ctx C = {P, M0, Mi, ph_lcc, w};
    return orc_bicgstab((long)P->nr * P->nz, b, x, P->ch_maxit, P->tol, chb_mv_cb, chb_ps_cb, &C, st);
}

/* The variable-coefficient pressure Poisson operator of the batched solves (no reference
 * counterpart: PreSolve_2 is a direct DCT solve): y = d/dx(beta dx/dx) + d/dz(beta dx/dz) on the
 * packed nr x nz cells, beta = 1/(1 + penalty_k dt bdr_ph), face values the mean of the two
 * cells, zero flux through the domain faces. */
void orc_pressure_matvec(const drd_params* P, const double* bdr_ph, const double* x, double* y) {
    const int nr = P->nr, nz = P->nz;
    const double idr2 = 1.0 / (P->dr * P->dr), idz2 = 1.0 / (P->dz * P->dz);
    double* beta = dalloc((long)nr * nz);
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) beta[i + (long)nr * k] = 1.0 / (1.0 + P->penalty_k * P->dt * bdr_ph[CI(i, k)]);
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) {
            const long q = i + (long)nr * k;
            const double c = x[q], bc = beta[q];
            double fx = 0.0, fz = 0.0;
            if (i + 1 < nr) fx += (bc + beta[q + 1]) * 0.5 * (x[q + 1] - c);
            if (i > 0) fx -= (bc + beta[q - 1]) * 0.5 * (c - x[q - 1]);
            if (k + 1 < nz) fz += (bc + beta[q + nr]) * 0.5 * (x[q + nr] - c);
            if (k > 0) fz -= (bc + beta[q - nr]) * 0.5 * (c - x[q - nr]);
            y[q] = fx * idr2 + fz * idz2;
        }
    free(beta);
}

/* PreSolve_2's DCT solve as a preconditioner (dct_fftw.f90:3-54): y = REDFT01(REDFT10(x) /
 * Pre_Lcc) / (4 nr nz) on the packed cells. */
void orc_pressure_psolve(const drd_params* P, const double* pre_lcc, const double* x, double* y) {
    const int nr = P->nr, nz = P->nz;
    const long n = (long)nr * nz;
    memcpy(y, x, sizeof(double) * n);
    orc_redft10(nr, nz, y, nr, 1);
    orc_redft10(nz, nr, y, 1, nr);
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) y[i + (long)nr * k] = y[i + (long)nr * k] / pre_lcc[i + (long)(nr + 1) * k];
    orc_redft01(nr, nz, y, nr, 1);
    orc_redft01(nz, nr, y, 1, nr);
    const double scale = 4.0 * nr * nz;
    for (long q = 0; q < n; ++q) y[q] = y[q] / scale;
}

typedef struct { const drd_params* P; const double* pre_lcc; const double* bdr; double* tmp; } pr_ctx;
static void pr_mv_cb(void* c, double a, const double* x, double b, double* y) {
    pr_ctx* C = (pr_ctx*)c;
    const long n = (long)C->P->nr * C->P->nz;
    orc_pressure_matvec(C->P, C->bdr, x, C->tmp);
    for (long q = 0; q < n; ++q) y[q] = a * C->tmp[q] + (b == 0.0 ? 0.0 : b * y[q]);
}
static void pr_ps_cb(void* c, const double* x, double* y) {
    pr_ctx* C = (pr_ctx*)c;
    orc_pressure_psolve(C->P, C->pre_lcc, x, y);
}

/* A x = b for the pressure Poisson system with the reference BiCGSTAB (lib/BiCGSTABREVCOM.f),
 * P->uv_maxit iterations, tolerance P->tol; x: guess in, solution out. */
int orc_pressure_solve(const drd_params* P, const double* pre_lcc, const double* bdr_ph, const double* b, double* x,
                       drd_status* st) {
    pr_ctx C = {P, pre_lcc, bdr_ph, dalloc((long)P->nr * P->nz)};
    const int info = orc_bicgstab((long)P->nr * P->nz, b, x, P->uv_maxit, P->tol, pr_mv_cb, pr_ps_cb, &C, st);
    free(C.tmp);
    return info;
}

/* VeloSolve_combined (bdf 1) / VeloSolve_2_combined (bdf 2). */
int orc_velosolve(const drd_params* P, int bdf, const double* psi1, const double* psi2,
                  const double* u_pre, const double* u, const double* v_pre, const double* v,
                  const double* p, const double* rho, const double* eta, const double* bdr_ph,
                  const double* bdr_pen, const double* bdr_used, const double* ph_after,
                  const double* rmu_after, double t, const double* pf1, const double* pf2,
                  double* u_after, double* v_after, double* uL, double* uR, drd_status* st) {
    const int nr = P->nr, nz = P->nz;
    const double dr = P->dr, dz = P->dz, dt = P->dt, re = P->re, ca = P->ca;
    const double dr2 = dr * dr, dz2 = dz * dz;
    const int tp = (P->variant == DRD_VARIANT_TP);
    const int dirichlet = !tp || P->lr_bd_type != 'n';
    if (P->xlsB >= 1.E-8) return DRD_ERR_UNSUPPORTED; /* the slip branch is commented out (:299-369) */
    const long us = u_size(nr, nz), vs = v_size(nr, nz), cs = cell_size(nr, nz), N = uv_len(nr, nz);
    double* fu = dalloc(us);
    double* fv = dalloc(vs);
    double* ut = dalloc(us);
    double* vt = dalloc(vs);
    double* tp_ = dalloc(cs);
    double* rhs = dalloc(N);
    double* x = dalloc(N);
    /* surface tension ca*mu*grad(phi) (:62-86; TP :64-90) */
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i <= nr; ++i) {
            if (!tp)
                fu[UI(i, k)] = ca * (rmu_after[CI(i, k)] + rmu_after[CI(i - 1, k)]) / 2.0 *
                               (ph_after[CI(i, k)] - ph_after[CI(i - 1, k)]) / dr *
                               (1.0 - (bdr_ph[CI(i, k)] + bdr_ph[CI(i - 1, k)]) / 2.0);
            else
                fu[UI(i, k)] = ca * (rmu_after[CI(i, k)] + rmu_after[CI(i - 1, k)]) / 2.0 *
                               (ph_after[CI(i, k)] * bdr_used[CI(i, k)] - ph_after[CI(i - 1, k)] * bdr_used[CI(i - 1, k)]) / dr;
        }
    for (int k = 1; k < nz; ++k)
        for (int i = 0; i < nr; ++i) {
            if (!tp)
                fv[VI(i, k)] = ca * (rmu_after[CI(i, k)] + rmu_after[CI(i, k - 1)]) / 2.0 *
                               (ph_after[CI(i, k)] - ph_after[CI(i, k - 1)]) / dz *
                               (1.0 - (bdr_ph[CI(i, k)] + bdr_ph[CI(i, k - 1)]) / 2.0);
            else
                fv[VI(i, k)] = ca * (rmu_after[CI(i, k)] + rmu_after[CI(i, k - 1)]) / 2.0 *
                               (ph_after[CI(i, k)] * bdr_used[CI(i, k)] - ph_after[CI(i, k - 1)] * bdr_used[CI(i, k - 1)]) / dz;
        }
    /* advection with u~ = 2u - u_pre (bdf 2, :98-113) or u (bdf 1) */
    for (long q = 0; q < us; ++q) ut[q] = (bdf == 2) ? 2.0 * u[q] - u_pre[q] : u[q];
    for (long q = 0; q < vs; ++q) vt[q] = (bdf == 2) ? 2.0 * v[q] - v_pre[q] : v[q];
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i <= nr; ++i)
            fu[UI(i, k)] = fu[UI(i, k)] -
                           re * (rho[CI(i, k)] + rho[CI(i - 1, k)]) / 2.0 *
                               (ut[UI(i, k)] * (ut[UI(i + 1, k)] - ut[UI(i - 1, k)]) / 2.0 / dr +
                                (vt[VI(i, k)] + vt[VI(i - 1, k)] + vt[VI(i, k + 1)] + vt[VI(i - 1, k + 1)]) / 4.0 *
                                    (ut[UI(i, k + 1)] - ut[UI(i, k - 1)]) / 2.0 / dz);
    for (int k = 1; k < nz; ++k)
        for (int i = 0; i < nr; ++i)
            fv[VI(i, k)] = fv[VI(i, k)] -
                           re * (rho[CI(i, k)] + rho[CI(i, k - 1)]) / 2.0 *
                               ((ut[UI(i, k)] + ut[UI(i + 1, k)] + ut[UI(i, k - 1)] + ut[UI(i + 1, k - 1)]) / 4.0 *
                                    (vt[VI(i + 1, k)] - vt[VI(i - 1, k)]) / 2.0 / dr +
                                vt[VI(i, k)] * (vt[VI(i, k + 1)] - vt[VI(i, k - 1)]) / 2.0 / dz);
    /* pressure gradient, mass and body force (:187-210) */
    for (long q = 0; q < cs; ++q) tp_[q] = (bdf == 2) ? p[q] + 4 * psi2[q] / 3.0 - psi1[q] / 3.0 : p[q];
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i <= nr; ++i) {
            double g = (tp && bdf == 2) ? (ph_after[CI(i, k)] + ph_after[CI(i - 1, k)]) / 2.0 * P->ggx : P->ggx;
            double mass = (bdf == 2) ? 2.0 * u[UI(i, k)] * re / dt - u_pre[UI(i, k)] * re / 2.0 / dt + g
                                     : u[UI(i, k)] * re / dt + g;
            fu[UI(i, k)] = fu[UI(i, k)] - (tp_[CI(i, k)] - tp_[CI(i - 1, k)]) / dr +
                           (rho[CI(i, k)] + rho[CI(i - 1, k)]) / 2.0 * mass;
        }
    for (int k = 1; k < nz; ++k)
        for (int i = 0; i < nr; ++i) {
            /* TP weights ggz with (ph(i,k)+ph(i-1,k))/2 as written (TP :219) */
            double g = (tp && bdf == 2) ? (ph_after[CI(i, k)] + ph_after[CI(i - 1, k)]) / 2.0 * P->ggz : P->ggz;
            double mass = (bdf == 2) ? 2.0 * v[VI(i, k)] * re / dt - v_pre[VI(i, k)] * re / 2.0 / dt + g
                                     : v[VI(i, k)] * re / dt + g;
            fv[VI(i, k)] = fv[VI(i, k)] - (tp_[CI(i, k)] - tp_[CI(i, k - 1)]) / dz +
                           (rho[CI(i, k)] + rho[CI(i, k - 1)]) / 2.0 * mass;
        }
    /* particle force (:229-239) and the dt scaling (:242-252) */
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i <= nr; ++i) fu[UI(i, k)] = fu[UI(i, k)] + (pf1[CI(i, k)] + pf1[CI(i - 1, k)]) / 2.0;
    for (int k = 1; k < nz; ++k)
        for (int i = 0; i < nr; ++i) fv[VI(i, k)] = fv[VI(i, k)] + (pf2[CI(i, k)] + pf2[CI(i, k - 1)]) / 2.0;
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i <= nr; ++i) fu[UI(i, k)] = fu[UI(i, k)] * dt;
    for (int k = 1; k < nz; ++k)
        for (int i = 0; i < nr; ++i) fv[VI(i, k)] = fv[VI(i, k)] * dt;
    /* inlet / outlet Dirichlet profiles (:262-295) */
    double* uLl = dalloc(nz + 1);
    double* uRl = dalloc(nz + 1);
    if (dirichlet) {
        double cf = 1.0 - exp(-t / P->twall);
        double hig = P->bdr_upp - P->bdr_low;
        for (int k = 0; k < nz; ++k) {
            double z = (k + 0.5) * dz;
            if (z > P->bdr_low && z < P->bdr_upp) {
                double d = z - P->bdr_low - hig / 2;
                uLl[k] = P->UU * (-(d * d) / hig / hig * 4 + 1) * cf;
            } else {
                uLl[k] = 0.0;
            }
            fu[UI(0, k)] = fu[UI(0, k)] + 2.0 * uLl[k] * eta[CI(0, k)] * 2.0 * dt / dr2;
        }
        for (int k = 0; k < nz; ++k) {
            uRl[k] = uLl[k];
            fu[UI(nr, k)] = fu[UI(nr, k)] + 2.0 * uRl[k] * eta[CI(nr, k)] * 2.0 * dt / dr2;
        }
    }
    /* no-slip wall terms (:377-385) */
    for (int i = 0; i <= nr; ++i) {
        int k = 0;
        double etay = (eta[CI(i, k)] + eta[CI(i - 1, k)] + eta[CI(i, k - 1)] + eta[CI(i - 1, k - 1)]) / 4.0;
        fu[UI(i, k)] = fu[UI(i, k)] + dt * (2.0 * P->uwB / dz2 * etay);
        k = nz - 1;
        etay = (eta[CI(i, k + 1)] + eta[CI(i - 1, k + 1)] + eta[CI(i, k)] + eta[CI(i - 1, k)]) / 4.0;
        fu[UI(i, k)] = fu[UI(i, k)] + dt * (2.0 * P->uwT / dz2 * etay);
    }
    atob_uv(nr, nz, fu, fv, rhs); /* :388-389 */
    atob_uv(nr, nz, u, v, x);
    uv_ctx C = {P, bdf, rho, eta, bdr_pen, NULL};
    if (P->uv_precond == DRD_UV_ESOLP_SCALED) {
        C.scale = dalloc(N);
        orc_uv_esolp_scale(P, bdf, rho, eta, C.scale);
    }
    int info = orc_bicgstab(N, rhs, x, P->uv_maxit, P->tol, uv_mv_cb, uv_ps_cb, &C, st); /* :398-401 */
    free(C.scale);
    btoa_uv(nr, nz, u_after, v_after, x); /* :411 */
    if (dirichlet) {
        for (int k = 0; k < nz; ++k) u_after[UI(-1, k)] = 2.0 * uLl[k] - u_after[UI(1, k)];
        for (int k = 0; k < nz; ++k) u_after[UI(nr + 1, k)] = 2.0 * uRl[k] - u_after[UI(nr - 1, k)];
    } else {
        for (int k = 0; k <= nz; ++k) { /* TP :437-440 */
            u_after[UI(-1, k)] = u_after[UI(1, k)];
            u_after[UI(nr + 1, k)] = u_after[UI(nr - 1, k)];
        }
    }
    for (int i = -1; i <= nr + 1; ++i) {
        u_after[UI(i, -1)] = P->uwB * 2.0 - u_after[UI(i, 0)];
        u_after[UI(i, nz)] = P->uwT * 2.0 - u_after[UI(i, nz - 1)];
    }
    for (int i = -1; i <= nr; ++i) {
        v_after[VI(i, 0)] = 0.0;
        v_after[VI(i, nz)] = 0.0;
    }
    for (int k = 1; k < nz; ++k) {
        v_after[VI(-1, k)] = v_after[VI(0, k)];
        v_after[VI(nr, k)] = v_after[VI(nr - 1, k)];
    }
    if (dirichlet) {
        if (uL) memcpy(uL, uLl, sizeof(double) * nz);
        if (uR) memcpy(uR, uRl, sizeof(double) * nz);
    }
    free(fu); free(fv); free(ut); free(vt); free(tp_); free(rhs); free(x); free(uLl); free(uRl);
    return info;
}

/* ---------------------------------------------------------------------------------------
 * PreSolve_2 + dct_fftw: microfluidics_complex_domain/PreSolve_2.f90:1-130,135-186.
 * ------------------------------------------------------------------------------------- */
void orc_presolve(const drd_params* P, const double* pre_lcc, const double* u, const double* v,
                  double coef, double* psi) {
    const int nr = P->nr, nz = P->nz;
    const long n = (long)nr * nz, cs = cell_size(nr, nz);
    double* w = dalloc(n);
    for (int k = 0; k < nz; ++k) /* :16-21 */
        for (int i = 0; i < nr; ++i)
            w[i + (long)nr * k] = (u[UI(i + 1, k)] - u[UI(i, k)]) / P->dr + (v[VI(i, k + 1)] - v[VI(i, k)]) / P->dz;
    orc_redft10(nr, nz, w, nr, 1); /* dfftw_execute_r2r(plan): REDFT10 in both dimensions */
    orc_redft10(nz, nr, w, 1, nr);
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) w[i + (long)nr * k] = w[i + (long)nr * k] / pre_lcc[i + (long)(nr + 1) * k];
    orc_redft01(nr, nz, w, nr, 1); /* plan_back: REDFT01 in both dimensions */
    orc_redft01(nz, nr, w, 1, nr);
    const double scale = 4.0 * nr * nz; /* :47 */
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) psi[CI(i, k)] = w[i + (long)nr * k] / scale;
    for (int k = 0; k < nz; ++k) { /* :175-183 */
        psi[CI(-1, k)] = psi[CI(0, k)];
        psi[CI(nr, k)] = psi[CI(nr - 1, k)];
    }
    for (int i = -1; i <= nr; ++i) {
        psi[CI(i, -1)] = psi[CI(i, 0)];
        psi[CI(i, nz)] = psi[CI(i, nz - 1)];
    }
    for (long q = 0; q < cs; ++q) psi[q] = psi[q] * coef; /* :125 */
    free(w);
}

/* interpolate_coef: microfluidics_complex_domain/interpolate_coef.f90:55-89. */
void orc_interpolate_coef(const drd_params* P, const double* dist, const double* bdr_ph,
                          double* fpd_ph, double* rho, double* eta) {
    const int nr = P->nr, nz = P->nz;
    const long cs = cell_size(nr, nz);
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i)
            fpd_ph[CI(i, k)] = tanh(-1.0 * dist[i + (long)nr * k] / sqrt(2.0) / P->I_thickness);
    for (long q = 0; q < cs; ++q) fpd_ph[q] = (fpd_ph[q] + 1.0) / 2.0;
    for (long q = 0; q < cs; ++q) fpd_ph[q] = fpd_ph[q] + bdr_ph[q];
    for (int k = 0; k < nz; ++k) {
        fpd_ph[CI(-1, k)] = fpd_ph[CI(0, k)];
        fpd_ph[CI(nr, k)] = fpd_ph[CI(nr - 1, k)];
    }
    for (int i = -1; i <= nr; ++i) {
        fpd_ph[CI(i, -1)] = fpd_ph[CI(i, 0)];
        fpd_ph[CI(i, nz)] = fpd_ph[CI(i, nz - 1)];
    }
    for (long q = 0; q < cs; ++q) {
        rho[q] = 1.0 + (P->lambda_rho - 1.0) * fpd_ph[q];
        eta[q] = 1.0 + (P->lambda_eta - 1.0) * fpd_ph[q];
    }
}

/* reinint_by_PhSolve (two_phase_flow_complex_domain/reinint_by_PhSolve.f90:1-91): finit's wall
 * smoothing (51 PhSolve_ori steps, :12-70), then bdr_ph_penalty = 1 where bdr_ph > 0.5 over
 * the whole ghosted array (:78-86). */
int orc_reinint_by_phsolve(const drd_params* P, const double* ph_lcc, const double* bdr_in, double* bdr_out,
                           double* pen_out) {
    const int info = orc_finit_wall(P, ph_lcc, bdr_in, 51, bdr_out, NULL, NULL);
    const long cs = cell_size(P->nr, P->nz);
    for (long q = 0; q < cs; ++q) pen_out[q] = bdr_out[q] > 0.5 ? 1.0 : 0.0;
    return info;
}

/* dissipation (microfluidics_complex_domain/dissipation.f90:1-122) with setup's derivative
 * coefficients xa1 = -1/2/dr, xb1 = 0, xc1 = -xa1 (setup.f90:9-19) in dif1x / dif1y's
 * expression ua u(i-1) + ub u(i) + uc u(i+1) (setup.f90:269-307).  Where the reference is not
 * defined (v handed to dif1x through a dummy of u's shape, vvb summed where only its wall rows
 * were assigned), v_x and v_z are taken on v's own grid, one-sided at i = nr and in the wall
 * rows like u_z (:68-77).  angB/angT NULL: P->angle everywhere.  out: e1 e2 e3 e4 dissip mass. */
void orc_dissipation(const drd_params* P, const double* u, const double* v, const double* ph, const double* rmu,
                     const double* angB, const double* angT, double vs, double* out) {
    const int nr = P->nr, nz = P->nz;
    const double dr = P->dr, dz = P->dz, eps = P->I_thickness;
    const double pi = 3.14159265358979323846264338327950288; /* global.f90:27 */
    const double xa1 = -1.0 / 2.0 / dr, xb1 = 0.0, xc1 = -xa1;
    const double ya1 = -1.0 / 2.0 / dz, yb1 = 0.0, yc1 = -ya1;
#define UA(i, k) u[(long)((i) + 1) + (long)((k) + 1) * (nr + 3)]
#define VA(i, k) v[(long)((i) + 1) + (long)(k) * (nr + 2)]
    double e1 = 0.;
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) {
            const double gx = (rmu[CI(i + 1, k)] - rmu[CI(i - 1, k)]) / 2.0 / dr;
            const double gz = (rmu[CI(i, k + 1)] - rmu[CI(i, k - 1)]) / 2.0 / dz;
            e1 = e1 + (gx * gx + gz * gz);
        }
    e1 = e1 * P->xld * P->ca * dr * dz;
    double e2 = 0.;
    for (int i = 0; i < nr; ++i) {
        double cf = sqrt(2.0) * cos((angT ? angT[i] : P->angle) * pi / 180.0) / 3.0 * pi / 2. / eps;
        double g = (ph[CI(i, nz)] - ph[CI(i, nz - 1)]) / dz - cf * cos(pi * (ph[CI(i, nz)] + ph[CI(i, nz - 1)]) / 2.0 / 2.);
        e2 = e2 + g * g;
        cf = sqrt(2.0) * cos((angB ? angB[i] : P->angle) * pi / 180.0) / 3.0 * pi / 2. / eps;
        g = (ph[CI(i, -1)] - ph[CI(i, 0)]) / dz - cf * cos(pi * (ph[CI(i, 0)] + ph[CI(i, -1)]) / 2.0 / 2.);
        e2 = e2 + g * g;
    }
    e2 = e2 * vs * P->ca * (eps * eps) * dr;
    double e3 = 0.;
    for (int k = 0; k <= nz; ++k)
        for (int i = 0; i <= nr; ++i) {
            const double uua = xa1 * UA(i - 1, k) + xb1 * UA(i, k) + xc1 * UA(i + 1, k);
            double uub, vvb, vva;
            if (k == 0) {
                uub = (UA(i, k + 1) - UA(i, k)) / dz;
                vvb = (VA(i, k + 1) - VA(i, k)) / dz;
            } else if (k == nz) {
                uub = (UA(i, k) - UA(i, k - 1)) / dz;
                vvb = (VA(i, k) - VA(i, k - 1)) / dz;
            } else {
                uub = ya1 * UA(i, k - 1) + yb1 * UA(i, k) + yc1 * UA(i, k + 1);
                vvb = ya1 * VA(i, k - 1) + yb1 * VA(i, k) + yc1 * VA(i, k + 1);
            }
            if (i < nr) vva = xa1 * VA(i - 1, k) + xb1 * VA(i, k) + xc1 * VA(i + 1, k);
            else vva = (VA(nr, k) - VA(nr - 1, k)) / dr;
            const double cx = (i == 0 || i == nr) ? 0.5 : 1.0, cz = (k == 0 || k == nz) ? 0.5 : 1.0;
            e3 = e3 + cx * cz * ((uua * uua + vvb * vvb) + uub * uub + vva * vva);
        }
    e3 = e3 * dr * dz;
#undef UA
#undef VA
    const double e4 = 0.0; /* :91-99 runs only for xlsB >= 1e-8 */
    double m = 0.0;
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) m = m + ph[CI(i, k)];
    out[0] = e1; out[1] = e2; out[2] = e3; out[3] = e4;
    out[4] = e1 + e2 + e3 + e4;
    out[5] = m * dr * dz;
}

/* The two-fluid coefficients that two_phase_flow_complex_domain/interpolate_coef.f90:91-112
 * keeps commented out: rho and eta_tmp piecewise in ph (1 at ph <= -1, the ratio at ph >= 1,
 * 1 + (ratio - 1) ph between), then eta = max(eta, eta_tmp) with eta = 1 + (lambda_eta - 1)
 * fpd_ph as computed above it (:84-89). */
void orc_two_phase_coef(const drd_params* P, const double* fpd_ph, const double* ph, double* rho, double* eta) {
    const long cs = cell_size(P->nr, P->nz);
    for (long q = 0; q < cs; ++q) {
        const double x = ph[q];
        double r, e;
        if (x <= -1.0) {
            r = 1.0;
            e = 1.0;
        } else if (x >= 1.0) {
            r = P->lambda_rho;
            e = P->lambda_eta;
        } else {
            r = 1.0 + (P->lambda_rho - 1.0) * x;
            e = 1.0 + (P->lambda_eta - 1.0) * x;
        }
        const double es = 1.0 + (P->lambda_eta - 1.0) * fpd_ph[q];
        rho[q] = r;
        eta[q] = es > e ? es : e;
    }
}

/* Mass sum of dissipation(): microfluidics_complex_domain/dissipation.f90:116-122. */
double orc_mass(const drd_params* P, const double* ph) {
    const int nr = P->nr, nz = P->nz;
    double e4 = 0.0;
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) e4 = e4 + ph[CI(i, k)];
    return e4 * P->dr * P->dz;
}

/* ---------------------------------------------------------------------------------------
 * Fiber particles: microfluidics_complex_domain/particles_move.f90 (Np_swm = 0, so the
 * swimmer and phantom loops of those routines are empty and not restated).
 * POINTS arrays are Np x 2 column-major: x of bead b at [b], y at [np + b].
 * ------------------------------------------------------------------------------------- */
int drd_particle_params_default(drd_particle_params* pp, double lx, double ly) {
    if (!pp) return DRD_ERR_BADARG;
    memset(pp, 0, sizeof(*pp));
    pp->np = 9;                                       /* particles_params.f90:78 */
    pp->lx = lx;
    pp->ly = ly;
    pp->fpd_radius = 0.05 / 2.0;                      /* :80 */
    pp->l0 = 2 * (pp->fpd_radius + 0.00);             /* :83, fpd_inter_dist = 0 (:81) */
    pp->ks = 5;                                       /* :74 */
    pp->kb = 0.0025 * 100;                            /* :75 */
    pp->theta0 = 0.0;                                 /* :76 */
    pp->k0_inter = 2.5;                               /* :93 */
    pp->k0_inter_bdr = 2.5 * 10;                      /* :94 */
    pp->fpd_fpd_dist = pp->fpd_radius + pp->fpd_radius + 0.01; /* :97 */
    pp->fpd_bdr_dist = pp->fpd_radius + 0.02;         /* :98 */
    return DRD_OK;
}

/* particle_initialize, fibers: particles_move.f90:50-68. */
int drd_particle_initialize(const drd_particle_params* pp, double xc, double yc, double* points) {
    if (!pp || !points || pp->np < 0 || pp->np > DRD_PARTICLES_MAX) return DRD_ERR_BADARG;
    const int np = pp->np;
    if (np > 2) {
        const int mid = (int)floor(np / 2.0);
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

/* MirrorDistance: particles_move.f90:1055-1065. */
static double mirror_distance(double d, double l) {
    if (d < -0.5 * l) return d + l;
    if (d > 0.5 * l) return d - l;
    return d;
}

/* fpd_dist_periodic: particles_move.f90:326-357. */
static double fpd_dist_periodic(double x, double y, double lx, double ly, double rx, double ry, double r) {
    double xd = 0.0, yd = 0.0;
    if (rx < r) xd = -lx;
    else if (lx - rx < r) xd = lx;
    if (ry < r) yd = -ly;
    else if (ly - ry < r) yd = ly;
    double d = sqrt((x - rx) * (x - rx) + (y - ry) * (y - ry)) - r;
    d = fmin(d, sqrt((x + xd - rx) * (x + xd - rx) + (y - ry) * (y - ry)) - r);
    d = fmin(d, sqrt((x - rx) * (x - rx) + (y + yd - ry) * (y + yd - ry)) - r);
    d = fmin(d, sqrt((x + xd - rx) * (x + xd - rx) + (y + yd - ry) * (y + yd - ry)) - r);
    return d;
}

/* The smoothed bead indicator (tanh(-dd/sqrt(2)/eps) + 1)/2 of particles_move.f90:786-787. */
static double bead_indicator(double dd, double eps) { return (tanh(-1.0 * dd / sqrt(2.0) / eps) + 1.0) / 2.0; }

/* interaction_force: particles_move.f90:1010-1053. */
static void interaction_force(double p1x, double p1y, double p2x, double p2y, double eq, double k, double f[2],
                              double lx, double ly) {
    double dx = mirror_distance(p1x - p2x, lx);
    double dy = mirror_distance(p1y - p2y, ly);
    const double d = sqrt(dx * dx + dy * dy);
    if (d < eq) {
        dx = dx / d;
        dy = dy / d;
        f[0] = -(k / (eq * eq) * (d - eq) * dx);
        f[1] = -(k / (eq * eq) * (d - eq) * dy);
    } else {
        f[0] = 0.0;
        f[1] = 0.0;
    }
}

/* Flat CELL index of bdr_dist(i,j) as the Fortran column-major array addresses it, clamped to
 * the array: interaction_force_bdr reads bdr_dist(i-1,j) with i = -1 for a bead within half a
 * cell of x = 0, which column-major storage maps to bdr_dist(nr, j-1). */
static long bdr_flat(int nr, int nz, int i, int j) {
    long q = (long)(i + 1) + (long)(j + 1) * (nr + 2);
    const long cs = cell_size(nr, nz);
    return q < 0 ? 0 : (q >= cs ? cs - 1 : q);
}

/* interaction_force_bdr: particles_move.f90:1069-1103. */
static void interaction_force_bdr(int nr, int nz, double dr, double dz, const double* bd, double px, double py,
                                  double eq, double k, double f[2]) {
    const int i = (int)floor((px - dr * 0.5) / dr);
    const int j = (int)floor((py - dz * 0.5) / dz);
    const double d = bd[bdr_flat(nr, nz, i, j)];
    double dx = (bd[bdr_flat(nr, nz, i + 1, j)] - bd[bdr_flat(nr, nz, i - 1, j)]) / 2.0 / dr;
    double dy = (bd[bdr_flat(nr, nz, i, j + 1)] - bd[bdr_flat(nr, nz, i, j - 1)]) / 2.0 / dz;
    const double di = sqrt(dx * dx + dy * dy);
    dx = dx / di;
    dy = dy / di;
    if (d < eq) {
        f[0] = -(k / (eq * eq) * (d - eq) * dx);
        f[1] = -(k / (eq * eq) * (d - eq) * dy);
    } else {
        f[0] = 0.0;
        f[1] = 0.0;
    }
}

/* force_caculation, fiber part: particles_move.f90:421-549 and :589-594 (tot_F). */
void orc_particle_forces(const drd_params* P, const drd_particle_params* pp, const double* pts,
                         const double* bdr_dist, double* tot_F) {
    const int np = pp->np;
    const double lx = pp->lx, ly = pp->ly, l0 = pp->l0, ks = pp->ks, kb = pp->kb;
    const double PI = 4.0 * atan(1.0); /* particles_params.f90:4 */
    double rdiff[DRD_PARTICLES_MAX] = {0}, tv[DRD_PARTICLES_MAX][2] = {{0}}, nv[DRD_PARTICLES_MAX][2] = {{0}};
    double theta[DRD_PARTICLES_MAX] = {0}, G[DRD_PARTICLES_MAX] = {0};
    for (int i = 0; i < np - 1; ++i) {                                  /* :445-459 */
        const double dX = mirror_distance(pts[i + 1] - pts[i], lx);
        const double dY = mirror_distance(pts[np + i + 1] - pts[np + i], ly);
        rdiff[i] = sqrt(dX * dX + dY * dY);
        tv[i][0] = dX / rdiff[i];
        tv[i][1] = dY / rdiff[i];
        nv[i][0] = -dY / rdiff[i];
        nv[i][1] = dX / rdiff[i];
        theta[i] = atan2(tv[i][1], tv[i][0]);
        if (theta[i] < 0) theta[i] = theta[i] + 2 * PI;
    }
    for (int i = 0; i < np - 2; ++i) {                                  /* :471-481 */
        double a = theta[i + 1] - theta[i];
        a = mirror_distance(a, 2 * PI);
        G[i] = a - pp->theta0;
    }
    const double kl = ks / (l0 * l0);
    for (int i = 0; i < np; ++i) {                                      /* :483-516 */
        double Fs[2], Fb[2];
        for (int c = 0; c < 2; ++c) {
            if (i == 0) {
                Fs[c] = kl * (rdiff[i] - l0) * tv[i][c];
                Fb[c] = -(kb * G[i] / rdiff[i] * nv[i][c]);
            } else if (i == 1) {
                Fs[c] = kl * ((rdiff[i] - l0) * tv[i][c] - (rdiff[i - 1] - l0) * tv[i - 1][c]);
                Fb[c] = kb * (G[i - 1] / rdiff[i - 1] * nv[i - 1][c] - (G[i] - G[i - 1]) / rdiff[i] * nv[i - 1][c]);
            } else if (i == np - 1) {
                Fs[c] = -kl * (rdiff[i - 1] - l0) * tv[i - 1][c];
                Fb[c] = -(kb * (G[i - 2] / rdiff[i - 1] * nv[i - 1][c]));
            } else if (i == np - 2) {
                Fs[c] = kl * ((rdiff[i] - l0) * tv[i][c] - (rdiff[i - 1] - l0) * tv[i - 1][c]);
                Fb[c] = kb * ((G[i - 1] - G[i - 2]) / rdiff[i - 1] * nv[i - 1][c] + G[i - 1] / rdiff[i] * nv[i - 1][c]);
            } else {
                Fs[c] = kl * ((rdiff[i] - l0) * tv[i][c] - (rdiff[i - 1] - l0) * tv[i - 1][c]);
                Fb[c] = kb * ((G[i - 1] - G[i - 2]) / rdiff[i - 1] * nv[i - 1][c] - (G[i] - G[i - 1]) / rdiff[i] * nv[i][c]);
            }
            tot_F[i + (long)np * c] = Fs[c] + Fb[c];                    /* :518 */
        }
    }
    double f[2];
    for (int i = 0; i < np; ++i)                                        /* :532-539 */
        for (int j = i + 1; j < np; ++j) {
            interaction_force(pts[i], pts[np + i], pts[j], pts[np + j], pp->fpd_fpd_dist, pp->k0_inter, f, lx, ly);
            tot_F[i] = tot_F[i] + f[0];
            tot_F[np + i] = tot_F[np + i] + f[1];
            tot_F[j] = tot_F[j] - f[0];
            tot_F[np + j] = tot_F[np + j] - f[1];
        }
    for (int i = 0; i < np; ++i) {                                      /* :574-579 */
        interaction_force_bdr(P->nr, P->nz, P->dr, P->dz, bdr_dist, pts[i], pts[np + i], pp->fpd_bdr_dist,
                              pp->k0_inter_bdr, f);
        tot_F[i] = tot_F[i] + f[0];
        tot_F[np + i] = tot_F[np + i] + f[1];
    }
}

/* force_caculation_vel: particles_move.f90:758-815 (fiber beads; grid r = (i+0.5)dr,
 * z = (k+0.5)dz as finit.f90:34-35 sets it).  pf1/pf2 are CELL with zero ghosts. */
void orc_force_caculation_vel(const drd_params* P, const drd_particle_params* pp, const double* pts,
                              const double* bdr_dist, double* tot_F, double* pf1, double* pf2) {
    const int nr = P->nr, nz = P->nz, np = pp->np;
    const long cs = cell_size(nr, nz);
    orc_particle_forces(P, pp, pts, bdr_dist, tot_F);
    for (long q = 0; q < cs; ++q) { pf1[q] = 0.0; pf2[q] = 0.0; }
    double* w = dalloc((long)nr * nz);
    for (int b = 0; b < np; ++b) {
        double sum = 0.0;
        for (int k = 0; k < nz; ++k)
            for (int i = 0; i < nr; ++i) {
                const double dd = bead_indicator(
                    fpd_dist_periodic((i + 0.5) * P->dr, (k + 0.5) * P->dz, pp->lx, pp->ly, pts[b], pts[np + b],
                                      pp->fpd_radius), P->I_thickness);
                w[i + (long)nr * k] = dd;
                sum = sum + dd;
            }
        sum = sum * P->dr * P->dz;
        for (int k = 0; k < nz; ++k)
            for (int i = 0; i < nr; ++i) {
                const double dd = w[i + (long)nr * k];
                pf1[CI(i, k)] = pf1[CI(i, k)] + (tot_F[b] * dd) / sum;
                pf2[CI(i, k)] = pf2[CI(i, k)] + (tot_F[np + b] * dd) / sum;
            }
    }
    free(w);
}

/* update_position_vel: particles_move.f90:872-924 (fiber beads). */
void orc_update_position_vel(const drd_params* P, const drd_particle_params* pp, double* pts, const double* u,
                             const double* v, double dt) {
    const int nr = P->nr, nz = P->nz, np = pp->np;
    for (int b = 0; b < np; ++b) {
        double ua = 0., va = 0., sum = 0.0;
        for (int k = 0; k < nz; ++k)
            for (int i = 0; i < nr; ++i) {
                const double dd = bead_indicator(
                    fpd_dist_periodic((i + 0.5) * P->dr, (k + 0.5) * P->dz, pp->lx, pp->ly, pts[b], pts[np + b],
                                      pp->fpd_radius), P->I_thickness);
                ua = ua + (u[UI(i, k)] + u[UI(i, k + 1)]) / 2.0 * dd; /* u averaged over k, as :902 */
                va = va + (v[VI(i, k)] + v[VI(i, k + 1)]) / 2.0 * dd;
                sum = sum + dd;
            }
        ua = ua / sum;
        va = va / sum;
        pts[b] = pts[b] + ua * dt;
        pts[np + b] = pts[np + b] + va * dt;
        if (pts[b] > pp->lx) pts[b] = pts[b] - pp->lx;
        else if (pts[b] < 0) pts[b] = pts[b] + pp->lx;
        if (pts[np + b] > pp->ly) pts[np + b] = pts[np + b] - pp->ly;
        else if (pts[np + b] < 0) pts[np + b] = pts[np + b] + pp->ly;
    }
}

/* dist(r(i,k), z(i,k)) = fpd_dist (dist.f90 -> particles_move.f90:361-391): distance to the
 * nearest bead surface, not periodic, 1e10 without beads.  DIST shaped. */
void orc_fpd_dist_field(const drd_params* P, const drd_particle_params* pp, const double* pts, double* dist) {
    const int nr = P->nr, nz = P->nz, np = pp->np;
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nr; ++i) {
            const double x = (i + 0.5) * P->dr, y = (k + 0.5) * P->dz;
            double d = 1.0E10;
            for (int b = 0; b < np; ++b)
                d = fmin(d, sqrt((x - pts[b]) * (x - pts[b]) + (y - pts[np + b]) * (y - pts[np + b])) - pp->fpd_radius);
            dist[i + (long)nr * k] = d;
        }
}

/* The particle block of the mcl6 loop (mcl6.f90:394-402): forces and spreading with the beads
 * where they are, then the move with the current u, v, then interpolate_coef at the new
 * positions. */
void orc_particles_step(const drd_params* P, orc_particles* X, const double* u, const double* v,
                        const double* bdr_ph, double* pf1, double* pf2) {
    orc_force_caculation_vel(P, &X->pp, X->points, X->bdr_dist, X->tot_F, pf1, pf2);
    orc_update_position_vel(P, &X->pp, X->points, u, v, P->dt);
    double* dist = dalloc((long)P->nr * P->nz);
    orc_fpd_dist_field(P, &X->pp, X->points, dist);
    orc_interpolate_coef(P, dist, bdr_ph, X->fpd_ph, X->rho, X->eta);
    free(dist);
}

/* ---------------------------------------------------------------------------------------
 * The mcl6 step: microfluidics_complex_domain/mcl6.f90:239-306 (first) and :378-486 (loop).
 * ------------------------------------------------------------------------------------- */
int orc_step(const drd_params* P, const double* ph_lcc, const double* pre_lcc, orc_state* S,
             int first, double t, drd_status* st2) {
    const int nr = P->nr, nz = P->nz;
    const long cs = cell_size(nr, nz), us = u_size(nr, nz), vs = v_size(nr, nz);
    double** f = S->f;
    double* rmu_after = dalloc(cs);
    double* ph_after = dalloc(cs);
    double* u_after = dalloc(us);
    double* v_after = dalloc(vs);
    drd_status st[2];
    memset(st, 0, sizeof(st));
    const double gamma1 = fmin(1.0, P->lambda_rho);
    int rc = 0;
    if (P->variant == DRD_VARIANT_TP) {
        /* TP step: the angle arrays are uniform (TP/finit.f90:581) */
        double* ang = dalloc(nr + 1);
        for (int i = 0; i <= nr; ++i) ang[i] = P->angle;
        rc = orc_ph_mu_solve(P, f[DRD_F_U], f[DRD_F_V], f[DRD_F_PH], f[DRD_F_RMU], S->bdr_ph, S->bdr_used,
                             S->bdr_ph_grad, S->Mi, ang, ang, S->M0, ph_after, rmu_after, NULL, &st[0]);
        free(ang);
    } else {
        /* guess_mode 1: the Krylov guess is 2 rmu - rmu_pre (the rhs only reads rmu through it) */
        double* guess = f[DRD_F_RMU];
        double* ext = NULL;
        if (!first && P->guess_mode == 1) {
            ext = dalloc(cs);
            for (long q = 0; q < cs; ++q) ext[q] = 2.0 * f[DRD_F_RMU][q] - f[DRD_F_RMU_PRE][q];
            guess = ext;
        }
        rc = orc_phsolve(P, ph_lcc, f[DRD_F_U], f[DRD_F_V], f[DRD_F_PH], guess, S->bdr_ph, S->bdr_ph_grad,
                         S->M0, S->Mi, rmu_after, ph_after, &st[0]);
        free(ext);
    }
    (void)rc;
    const double* rho = S->rho;
    const double* eta = S->eta;
    if (S->parts && S->parts->pp.np > 0) { /* mcl6.f90:394-402 */
        orc_particles_step(P, S->parts, f[DRD_F_U], f[DRD_F_V], S->bdr_ph, f[DRD_F_PF1], f[DRD_F_PF2]);
        rho = S->parts->rho;
        eta = S->parts->eta;
    }
    double *rho2 = NULL, *eta2 = NULL;
    if (P->two_fluid) { /* interpolate_coef's two-fluid form, from ph before the swap */
        const double* fpd = (S->parts && S->parts->pp.np > 0) ? S->parts->fpd_ph : S->fpd_ph;
        if (!fpd) fpd = S->bdr_ph; /* no particles and no indicator given: the solid alone */
        rho2 = dalloc(cs);
        eta2 = dalloc(cs);
        orc_two_phase_coef(P, fpd, f[DRD_F_PH], rho2, eta2);
        rho = rho2;
        eta = eta2;
    }
    orc_velosolve(P, first ? 1 : 2, f[DRD_F_PSI1], f[DRD_F_PSI2], f[DRD_F_U_PRE], f[DRD_F_U], f[DRD_F_V_PRE],
                  f[DRD_F_V], f[DRD_F_P], rho, eta, S->bdr_ph, S->bdr_pen, S->bdr_used, ph_after,
                  rmu_after, t + P->dt, f[DRD_F_PF1], f[DRD_F_PF2], u_after, v_after, NULL, NULL, &st[1]);
    memcpy(f[DRD_F_U_PRE], f[DRD_F_U], sizeof(double) * us);
    memcpy(f[DRD_F_V_PRE], f[DRD_F_V], sizeof(double) * vs);
    memcpy(f[DRD_F_U], u_after, sizeof(double) * us);
    memcpy(f[DRD_F_V], v_after, sizeof(double) * vs);
    memcpy(f[DRD_F_PH_PRE], f[DRD_F_PH], sizeof(double) * cs);
    memcpy(f[DRD_F_RMU_PRE], f[DRD_F_RMU], sizeof(double) * cs);
    memcpy(f[DRD_F_PH], ph_after, sizeof(double) * cs);
    memcpy(f[DRD_F_RMU], rmu_after, sizeof(double) * cs);
    double coef;
    if (first) {
        coef = P->re * gamma1 / P->dt;
    } else {
        memcpy(f[DRD_F_PSI1], f[DRD_F_PSI2], sizeof(double) * cs);
        coef = 3 * P->re * gamma1 / 2. / P->dt;
    }
    orc_presolve(P, pre_lcc, f[DRD_F_U], f[DRD_F_V], coef, f[DRD_F_PSI2]);
    for (long q = 0; q < cs; ++q) f[DRD_F_P][q] = f[DRD_F_PSI2][q] + f[DRD_F_P][q];
    if (st2) { st2[0] = st[0]; st2[1] = st[1]; }
    free(rmu_after); free(ph_after); free(u_after); free(v_after); free(rho2); free(eta2);
    return 0;
}
