// drd_particles.cu — fiber particles coupled to the flow: the per-step block
// force_caculation_vel -> update_position_vel -> interpolate_coef of
// microfluidics_complex_domain/mcl6.f90:394-402 (routines in particles_move.f90).
//
// Four launches per step, all FP64 like the reference:
//   k_pt_force   one thread: chain, bead-bead and wall forces of every bead (tot_F), and a copy
//                of the bead positions the forces and the spreading are evaluated at;
//   k_pt_sums    grid (blocks x beads): per bead the indicator sum S = sum dd and the weighted
//                velocity sums of update_position_vel, as fixed-slot block partials;
//   k_pt_finish  one block: deterministic reduction of the partials, then the bead move;
//   k_pt_spread  grid over CELL: particle_force1/2 = sum_b tot_F(b) dd_b / (S_b dr dz) at the old
//                positions, and fpd_ph, rho, eta (FP64 and the FP32 copies the mixed solver
//                reads) from fpd_dist at the new positions.
// The bead indicator dd = (tanh(-d/sqrt(2)/eps)+1)/2 is below 4.3e-18 once d > 20 sqrt(2) eps;
// the sums and the spreading skip those cells (the reference adds them: the difference is
// below 1e-14 of S at any grid size this library accepts).  fpd_dist_periodic's minimum of
// four square roots is taken as the square root of the minimum of the four squares, which is
// the same number because a correctly rounded sqrt is monotonic.
#include "drd_kernels.cuh"

namespace drd {

namespace {

__device__ __forceinline__ double mirror_distance(double d, double l) {
    // MirrorDistance: particles_move.f90:1055-1065
    if (d < -0.5 * l) return d + l;
    if (d > 0.5 * l) return d - l;
    return d;
}

// Squared distance from (x, y) to the bead centre and its periodic images, the images chosen
// as fpd_dist_periodic does (particles_move.f90:326-357).
struct BeadImg {
    double rx, ry, xd, yd;
};
__device__ __forceinline__ BeadImg bead_img(double rx, double ry, double r, double lx, double ly) {
    BeadImg b{rx, ry, 0.0, 0.0};
    if (rx < r) b.xd = -lx;
    else if (lx - rx < r) b.xd = lx;
    if (ry < r) b.yd = -ly;
    else if (ly - ry < r) b.yd = ly;
    return b;
}
__device__ __forceinline__ double bead_d2(const BeadImg& b, double x, double y) {
    const double ax = x - b.rx, ay = y - b.ry;
    double m = ax * ax + ay * ay;
    if (b.xd != 0.0) {
        const double bx = x + b.xd - b.rx;
        m = fmin(m, bx * bx + ay * ay);
    }
    if (b.yd != 0.0) {
        const double by = y + b.yd - b.ry;
        m = fmin(m, ax * ax + by * by);
        if (b.xd != 0.0) {
            const double bx = x + b.xd - b.rx;
            m = fmin(m, bx * bx + by * by);
        }
    }
    return m;
}
__device__ __forceinline__ double bead_indicator(double d2, double r, double eps) {
    // particles_move.f90:786-787
    const double dd = sqrt(d2) - r;
    return (tanh(-1.0 * dd / sqrt(2.0) / eps) + 1.0) / 2.0;
}

__device__ __forceinline__ void repulsion(double dx, double dy, double d, double eq, double k, double f[2]) {
    // interaction_force / interaction_force_bdr tail (particles_move.f90:1040-1050, :1091-1098)
    if (d < eq) {
        f[0] = -(k / (eq * eq) * (d - eq) * dx);
        f[1] = -(k / (eq * eq) * (d - eq) * dy);
    } else {
        f[0] = 0.0;
        f[1] = 0.0;
    }
}

// Flat CELL index of bdr_dist(i,j) as column-major Fortran storage addresses it, clamped to the
// array: for a bead within half a cell of x = 0, interaction_force_bdr reads bdr_dist(-2, j),
// which is bdr_dist(nr, j-1) in memory.
__device__ __forceinline__ long bdr_flat(int nr, int nz, int i, int j) {
    const long q = (long)(i + 1) + (long)(j + 1) * (nr + 2);
    const long cs = (long)(nr + 2) * (nz + 2);
    return q < 0 ? 0 : (q >= cs ? cs - 1 : q);
}

}  // namespace

// force_caculation (particles_move.f90:421-594), fiber beads; one thread in the reference's
// order of operations.  np in [3, DRD_PARTICLES_MAX] (checked on the host).
__global__ void k_pt_force(PartParams Q, double* __restrict__ pts, double* __restrict__ pts_old,
                           double* __restrict__ totF, const double* __restrict__ bd, ull* ctr) {
    count_launch(ctr);
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int np = Q.np;
    const double lx = Q.lx, ly = Q.ly, l0 = Q.l0, ks = Q.ks, kb = Q.kb;
    const double PI = 4.0 * atan(1.0);
    double rdiff[DRD_PARTICLES_MAX], tv0[DRD_PARTICLES_MAX], tv1[DRD_PARTICLES_MAX];
    double nv0[DRD_PARTICLES_MAX], nv1[DRD_PARTICLES_MAX], theta[DRD_PARTICLES_MAX], G[DRD_PARTICLES_MAX];
    for (int i = 0; i < np; ++i) {
        rdiff[i] = tv0[i] = tv1[i] = nv0[i] = nv1[i] = theta[i] = G[i] = 0.0;
        pts_old[i] = pts[i];
        pts_old[np + i] = pts[np + i];
    }
    for (int i = 0; i < np - 1; ++i) {  // :445-459
        const double dX = mirror_distance(pts[i + 1] - pts[i], lx);
        const double dY = mirror_distance(pts[np + i + 1] - pts[np + i], ly);
        rdiff[i] = sqrt(dX * dX + dY * dY);
        tv0[i] = dX / rdiff[i];
        tv1[i] = dY / rdiff[i];
        nv0[i] = -dY / rdiff[i];
        nv1[i] = dX / rdiff[i];
        theta[i] = atan2(tv1[i], tv0[i]);
        if (theta[i] < 0) theta[i] = theta[i] + 2 * PI;
    }
    for (int i = 0; i < np - 2; ++i) {  // :471-481
        double a = theta[i + 1] - theta[i];
        a = mirror_distance(a, 2 * PI);
        G[i] = a - Q.theta0;
    }
    const double kl = ks / (l0 * l0);
    for (int i = 0; i < np; ++i) {  // :483-518
        for (int c = 0; c < 2; ++c) {
            const double* tv = c ? tv1 : tv0;
            const double* nv = c ? nv1 : nv0;
            double Fs, Fb;
            if (i == 0) {
                Fs = kl * (rdiff[i] - l0) * tv[i];
                Fb = -(kb * G[i] / rdiff[i] * nv[i]);
            } else if (i == 1) {
                Fs = kl * ((rdiff[i] - l0) * tv[i] - (rdiff[i - 1] - l0) * tv[i - 1]);
                Fb = kb * (G[i - 1] / rdiff[i - 1] * nv[i - 1] - (G[i] - G[i - 1]) / rdiff[i] * nv[i - 1]);
            } else if (i == np - 1) {
                Fs = -kl * (rdiff[i - 1] - l0) * tv[i - 1];
                Fb = -(kb * (G[i - 2] / rdiff[i - 1] * nv[i - 1]));
            } else if (i == np - 2) {
                Fs = kl * ((rdiff[i] - l0) * tv[i] - (rdiff[i - 1] - l0) * tv[i - 1]);
                Fb = kb * ((G[i - 1] - G[i - 2]) / rdiff[i - 1] * nv[i - 1] + G[i - 1] / rdiff[i] * nv[i - 1]);
            } else {
                Fs = kl * ((rdiff[i] - l0) * tv[i] - (rdiff[i - 1] - l0) * tv[i - 1]);
                Fb = kb * ((G[i - 1] - G[i - 2]) / rdiff[i - 1] * nv[i - 1] - (G[i] - G[i - 1]) / rdiff[i] * nv[i]);
            }
            totF[i + np * c] = Fs + Fb;
        }
    }
    double f[2];
    for (int i = 0; i < np; ++i)  // :532-539 bead-bead repulsion
        for (int j = i + 1; j < np; ++j) {
            const double dx = mirror_distance(pts[i] - pts[j], lx);
            const double dy = mirror_distance(pts[np + i] - pts[np + j], ly);
            const double d = sqrt(dx * dx + dy * dy);
            repulsion(dx / d, dy / d, d, Q.eq_pp, Q.k0, f);
            totF[i] = totF[i] + f[0];
            totF[np + i] = totF[np + i] + f[1];
            totF[j] = totF[j] - f[0];
            totF[np + j] = totF[np + j] - f[1];
        }
    const int nr = Q.nr, nz = Q.nz;
    for (int b = 0; b < np; ++b) {  // :574-579 wall repulsion, interaction_force_bdr :1069-1103
        const int i = (int)floor((pts[b] - Q.dr * 0.5) / Q.dr);
        const int j = (int)floor((pts[np + b] - Q.dz * 0.5) / Q.dz);
        const double d = bd[bdr_flat(nr, nz, i, j)];
        double dx = (bd[bdr_flat(nr, nz, i + 1, j)] - bd[bdr_flat(nr, nz, i - 1, j)]) / 2.0 / Q.dr;
        double dy = (bd[bdr_flat(nr, nz, i, j + 1)] - bd[bdr_flat(nr, nz, i, j - 1)]) / 2.0 / Q.dz;
        const double di = sqrt(dx * dx + dy * dy);
        dx = dx / di;
        dy = dy / di;
        repulsion(dx, dy, d, Q.eq_bdr, Q.k0b, f);
        totF[b] = totF[b] + f[0];
        totF[np + b] = totF[np + b] + f[1];
    }
}

// Per-bead sums over the interior cells (particles_move.f90:781-791 and :897-906): slot
// (3b + 0) sum dd, (3b + 1) sum (u(i,k)+u(i,k+1))/2 dd, (3b + 2) the same for v (0 when u is
// null).  Grid (PT_GX, np); block partials at part[slot * PT_GX + blockIdx.x].
__global__ void k_pt_sums(PartParams Q, const double* __restrict__ pts, const double* __restrict__ u,
                          const double* __restrict__ v, double* __restrict__ part, ull* ctr) {
    count_launch(ctr);
    const int nr = Q.nr, nz = Q.nz, np = Q.np, b = blockIdx.y;
    const BeadImg bi = bead_img(pts[b], pts[np + b], Q.radius, Q.lx, Q.ly);
    const long n = (long)nr * nz;
    double s = 0.0, su = 0.0, sv = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % nr), k = (int)(q / nr);
        const double d2 = bead_d2(bi, (i + 0.5) * Q.dr, (k + 0.5) * Q.dz);
        if (d2 > Q.skip_d2) continue;
        const double dd = bead_indicator(d2, Q.radius, Q.eps);
        s += dd;
        if (u) {
            su += (u[uidx(nr, i, k)] + u[uidx(nr, i, k + 1)]) / 2.0 * dd;  // u averaged over k, as :902
            sv += (v[vidx(nr, i, k)] + v[vidx(nr, i, k + 1)]) / 2.0 * dd;
        }
    }
    __shared__ double sm[32];
    const double rs = block_sum<DRD_TPB>(s, sm);
    const double ru = block_sum<DRD_TPB>(su, sm);
    const double rv = block_sum<DRD_TPB>(sv, sm);
    if (threadIdx.x == 0) {
        part[(3 * b + 0) * PT_GX + blockIdx.x] = rs;
        part[(3 * b + 1) * PT_GX + blockIdx.x] = ru;
        part[(3 * b + 2) * PT_GX + blockIdx.x] = rv;
    }
}

// Reduces the partials (one warp per bead, fixed order) into psum[b] = S_b dr dz (the
// force_caculation_vel denominator, :793) and, when `move`, advances bead b by dt times the
// weighted mean velocity with the periodic wrap of update_position_vel (:907-924).
__global__ void k_pt_finish(PartParams Q, const double* __restrict__ part, double* __restrict__ psum,
                            double* __restrict__ pts, int move, ull* ctr) {
    count_launch(ctr);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5, np = Q.np;
    for (int b = w; b < np; b += nw) {
        double a[3];
        for (int j = 0; j < 3; ++j) {
            double x = 0.0;
            for (int g = lane; g < PT_GX; g += 32) x += part[(3 * b + j) * PT_GX + g];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            a[j] = x;
        }
        if (lane == 0) {
            psum[b] = a[0] * Q.dr * Q.dz;
            if (move) {
                const double ua = a[1] / a[0], va = a[2] / a[0];
                double x = pts[b] + ua * Q.dt, y = pts[np + b] + va * Q.dt;
                if (x > Q.lx) x = x - Q.lx;
                else if (x < 0) x = x + Q.lx;
                if (y > Q.ly) y = y - Q.ly;
                else if (y < 0) y = y + Q.ly;
                pts[b] = x;
                pts[np + b] = y;
            }
        }
    }
}

// mode bit 1: particle_force1/2 (CELL, zero ghosts) from tot_F, psum and the positions in
// pts_old (force_caculation_vel :795-813).  mode bit 2: interpolate_coef with fpd_dist of the
// positions in pts (interpolate_coef.f90:55-89, particles_move.f90:361-391).
__global__ void k_pt_spread(PartParams Q, int mode, const double* __restrict__ pts_old,
                            const double* __restrict__ pts, const double* __restrict__ totF,
                            const double* __restrict__ psum, const double* __restrict__ bdr, double* __restrict__ pf1,
                            double* __restrict__ pf2, double* __restrict__ fpd, double* __restrict__ rho,
                            double* __restrict__ eta, float* __restrict__ rho32, float* __restrict__ eta32,
                            ull* ctr) {
    count_launch(ctr);
    __shared__ BeadImg s_img[DRD_PARTICLES_MAX];
    __shared__ double s_f[DRD_PARTICLES_MAX][3];
    __shared__ double s_p[DRD_PARTICLES_MAX][2];
    const int nr = Q.nr, nz = Q.nz, np = Q.np;
    for (int b = threadIdx.x; b < np; b += blockDim.x) {
        s_img[b] = bead_img(pts_old[b], pts_old[np + b], Q.radius, Q.lx, Q.ly);
        s_f[b][0] = totF[b];
        s_f[b][1] = totF[np + b];
        s_f[b][2] = psum[b];
        s_p[b][0] = pts[b];
        s_p[b][1] = pts[np + b];
    }
    __syncthreads();
    const long cs = (long)(nr + 2) * (nz + 2);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < cs; q += (long)gridDim.x * blockDim.x) {
        const int i = (int)(q % (nr + 2)) - 1, k = (int)(q / (nr + 2)) - 1;
        if (mode & 1) {
            double p1 = 0.0, p2 = 0.0;
            if (i >= 0 && i < nr && k >= 0 && k < nz) {
                const double x = (i + 0.5) * Q.dr, y = (k + 0.5) * Q.dz;
                for (int b = 0; b < np; ++b) {
                    const double d2 = bead_d2(s_img[b], x, y);
                    if (d2 > Q.skip_d2) continue;
                    const double dd = bead_indicator(d2, Q.radius, Q.eps);
                    p1 = p1 + (s_f[b][0] * dd) / s_f[b][2];
                    p2 = p2 + (s_f[b][1] * dd) / s_f[b][2];
                }
            }
            pf1[q] = p1;
            pf2[q] = p2;
        }
        if (mode & 2) {
            const int si = i < 0 ? 0 : (i > nr - 1 ? nr - 1 : i);
            const int sk = k < 0 ? 0 : (k > nz - 1 ? nz - 1 : k);
            const double x = (si + 0.5) * Q.dr, y = (sk + 0.5) * Q.dz;
            double m = -1.0;
            for (int b = 0; b < np; ++b) {
                const double ax = x - s_p[b][0], ay = y - s_p[b][1];
                const double d2 = ax * ax + ay * ay;
                m = (m < 0.0) ? d2 : fmin(m, d2);
            }
            const double dist = (np > 0) ? fmin(1.0E10, sqrt(m) - Q.radius) : 1.0E10;
            double f = tanh(-1.0 * dist / sqrt(2.0) / Q.eps);
            f = (f + 1.0) / 2.0;
            f = f + bdr[cidx(nr, si, sk)];
            const double r = 1.0 + (Q.lambda_rho - 1.0) * f;
            const double e = 1.0 + (Q.lambda_eta - 1.0) * f;
            fpd[q] = f;
            rho[q] = r;
            eta[q] = e;
            rho32[q] = (float)r;
            eta32[q] = (float)e;
        }
    }
}

void launch_pt_force(const PartParams& Q, double* pts, double* pts_old, double* totF, const double* bdist, ull* ctr,
                     cudaStream_t s) {
    k_pt_force<<<1, 32, 0, s>>>(Q, pts, pts_old, totF, bdist, ctr);
}
void launch_pt_sums(const PartParams& Q, const double* pts, const double* u, const double* v, double* part, ull* ctr,
                    cudaStream_t s) {
    k_pt_sums<<<dim3(PT_GX, Q.np), DRD_TPB, 0, s>>>(Q, pts, u, v, part, ctr);
}
void launch_pt_finish(const PartParams& Q, const double* part, double* psum, double* pts, int move, ull* ctr,
                      cudaStream_t s) {
    k_pt_finish<<<1, DRD_TPB, 0, s>>>(Q, part, psum, pts, move, ctr);
}
void launch_pt_spread(const PartParams& Q, int mode, const double* pts_old, const double* pts, const double* totF,
                      const double* psum, const double* bdr, double* pf1, double* pf2, double* fpd, double* rho,
                      double* eta, float* rho32, float* eta32, ull* ctr, cudaStream_t s) {
    const long cs = (long)(Q.nr + 2) * (Q.nz + 2);
    long g = (cs + DRD_TPB - 1) / DRD_TPB;
    if (g > 4096) g = 4096;
    k_pt_spread<<<(int)g, DRD_TPB, 0, s>>>(Q, mode, pts_old, pts, totF, psum, bdr, pf1, pf2, fpd, rho, eta, rho32,
                                           eta32, ctr);
}

}  // namespace drd
