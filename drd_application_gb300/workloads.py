"""Seeded synthetic workloads with the reference's shapes and field construction.

No reference output data exists, so every workload is built here from a seed, the way
microfluidics_complex_domain/finit.f90 builds its fields:

* bdr_ph: the solid indicator in [0, 1] (1 in solid), Neumann ghosts;
* bdr_ph_grad = |grad bdr_ph| by central differences on the interior, 0 on ghosts
  (finit.f90:346-352); ph_M_0 = ph_M_inner = 1 - bdr_ph (finit.f90:358-359);
* phi in [0, 1] from tanh profiles, clipped by 1 - bdr_ph (finit.f90:274-288);
* rmu = -eps lap(phi) - phi/eps + phi^3/eps with Neumann ghosts (finit.f90:315-329);
* fpd_ph / rho / eta from interpolate_coef (interpolate_coef.f90:55-89) with the particle
  distance field of rigid rectangular fibers.

Workloads:
  "c1"  128x64 channel, one drop, no solid (lambda ratios 1), tol 1e-10, dt 1e-3.
  "c2"  420x180 serpentine channel (seeded sinusoidal walls, amplitude 30, period 140 cells,
        half-width 45 cells), resistance penalty 1e4, walls smoothed by tanh(d / 2 cells),
        3 rigid fibers of 40x4 cells at seeded poses, two drops of radius 15 cells,
        viscosity ratio 5 between the drops and the matrix fluid (two_fluid = 1: eta =
        max(1 + 4 fpd_ph, 1 + 4 ph), rebuilt every step from ph), Re 0.5, Ca 0.05.
  "tp"  the two_phase_flow_complex_domain variant (phi in [-1,1], ph_mu_solve, sharp penalty).
  "c5"  2048x1024 serpentine channel (amplitude 150, period 680 cells, half-width 0.35 nz),
        64 rigid fibers of 60x6 cells and 32 drops of radius U(20, 60) cells at seeded
        positions in the channel, viscosity ratio 10 (two-fluid, as c2), Re 1, Ca 0.02,
        dr = dz = 1/512.
Any workload can be built at another grid size; geometry lengths scale with the grid.

  C3 (make_c3_solve, make_c3_pressure): independent momentum solves, A x = b with the
        VeloSolve_2_combined operator, and pressure Poisson solves, div(beta grad psi) = b with
        beta = 1/(1 + penalty_k dt mask), on a grid drawn from {64x32, 128x64, 256x128, 420x180,
        512x256}; the solid is 2 to 6 disks of radius 5 to 25 cells, eta = 1 + 99 mask; b is a
        Gaussian random field (white noise filtered by exp(-k^2 l^2 / 2), l = 8 cells, unit
        variance, rounded to FP32; zero mean for the pressure systems).
"""
import math

import numpy as np

from . import abi
from .layout import cell_shape, neumann_ghosts_cell, u_shape, v_shape


def _grad_mag(b, dr, dz):
    g = np.zeros_like(b)
    g[1:-1, 1:-1] = np.sqrt(((b[1:-1, 2:] - b[1:-1, :-2]) / 2.0 / dr) ** 2.0 +
                            ((b[2:, 1:-1] - b[:-2, 1:-1]) / 2.0 / dz) ** 2.0)
    return g


def _rmu_init(ph, eps, dr, dz):
    r = np.zeros_like(ph)
    p = ph
    r[1:-1, 1:-1] = (-eps * ((p[1:-1, 2:] + p[1:-1, :-2] - 2 * p[1:-1, 1:-1]) / dr ** 2 +
                             (p[2:, 1:-1] + p[:-2, 1:-1] - 2 * p[1:-1, 1:-1]) / dz ** 2)
                     - p[1:-1, 1:-1] / eps + p[1:-1, 1:-1] ** 3 / eps)
    return neumann_ghosts_cell(r)


def _rect_sdf(x, y, cx, cy, half_l, half_w, ang):
    """Signed distance to a rotated rectangle (negative inside)."""
    c, s = math.cos(ang), math.sin(ang)
    lx = (x - cx) * c + (y - cy) * s
    ly = -(x - cx) * s + (y - cy) * c
    qx = np.abs(lx) - half_l
    qy = np.abs(ly) - half_w
    outside = np.sqrt(np.maximum(qx, 0.0) ** 2 + np.maximum(qy, 0.0) ** 2)
    inside = np.minimum(np.maximum(qx, qy), 0.0)
    return outside + inside


def _c5_channel(rng, p, nr, nz, X, Z, bdr, meta):
    """Serpentine walls (amplitude 150, period 680 cells at 2048x1024, scaled with the grid) and
    64 rigid 60x6-cell fibers at seeded poses inside the channel."""
    sx, sz = nr / 2048.0, nz / 1024.0
    dr, dz = p.dr, p.dz
    xi = np.arange(nr) + 0.5
    zk = np.arange(nz) + 0.5
    phase = rng.uniform(0, 2 * math.pi)
    amp, period, half = 150.0 * sz, 680.0 * sx, 0.35 * nz
    yc = nz / 2.0 + amp * np.sin(2 * math.pi * xi / period + phase)
    slope = amp * 2 * math.pi / period * np.cos(2 * math.pi * xi / period + phase)
    d_cells = (half - np.abs(zk[:, None] - yc[None, :])) / np.sqrt(1.0 + slope[None, :] ** 2)
    smooth = max(2.0 * min(sx, sz), 0.75)
    bdr[1:-1, 1:-1] = 0.5 * (1.0 - np.tanh(d_cells / smooth))
    neumann_ghosts_cell(bdr)
    p.bdr_low = (yc[0] - half) * dz
    p.bdr_upp = (yc[0] + half) * dz
    sdf = np.full((nz, nr), np.inf)
    fibers = []
    for f in range(64):
        cxc = rng.uniform(0, nr)
        ic = int(min(max(round(cxc - 0.5), 0), nr - 1))
        czc = yc[ic] + rng.uniform(-0.7, 0.7) * half
        ang = rng.uniform(0, math.pi)
        fibers.append((cxc, czc, ang))
        sdf = np.minimum(sdf, _rect_sdf(X / dr, Z / dz, cxc, czc, 30.0 * sx, 3.0 * sz, ang))
    meta.update(phase=phase, amp=amp, period=period, half=half, fibers=fibers)
    return bdr, sdf * min(dr, dz), yc, half


def _c5_drops(rng, ph, nr, nz, dr, dz, eps, X, Z, yc, half, meta):
    """32 drops of radius U(20, 60) cells (scaled with the grid) inside the channel."""
    s = min(nr / 2048.0, nz / 1024.0)
    drops = []
    h = min(dr, dz)
    for j in range(32):
        R = rng.uniform(20.0, 60.0) * s
        cxd = rng.uniform(0, nr)
        ic = int(min(max(round(cxd), 0), nr - 1))
        czd = yc[ic] + rng.uniform(-0.6, 0.6) * half
        drops.append((cxd, czd, R))
        d = np.sqrt((X / dr - cxd) ** 2 + (Z / dz - czd) ** 2) * h
        ph[1:-1, 1:-1] = np.maximum(ph[1:-1, 1:-1], 0.5 * (1.0 + np.tanh((R * h - d) / (math.sqrt(2.0) * eps))))
    meta["drops"] = drops


C3_SIZES = ((64, 32), (128, 64), (256, 128), (420, 180), (512, 256))


def _grf(rng, shape, ell=8.0):
    """Gaussian random field: white N(0,1) filtered by exp(-k^2 ell^2 / 2) (k in radians per
    cell), unit variance, rounded to FP32."""
    w = rng.standard_normal(shape)
    ky = 2 * np.pi * np.fft.fftfreq(shape[0])[:, None]
    kx = 2 * np.pi * np.fft.fftfreq(shape[1])[None, :]
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * np.exp(-(kx ** 2 + ky ** 2) * ell ** 2 / 2.0)))
    f = (f - f.mean()) / f.std()
    return f.astype(np.float32).astype(np.float64)


def _c3_params_mask(rng, size, precision, overrides):
    """Grid (drawn from C3_SIZES unless given), parameters and the seeded mask of 2 to 6 disks of
    radius 5 to 25 cells, smoothed by tanh over 0.75 cells."""
    nr, nz = size if size is not None else C3_SIZES[int(rng.integers(len(C3_SIZES)))]
    p = abi.default_params(nr, nz, re=0.5, ca=0.05, lambda_rho=1.0, lambda_eta=1.0, penalty_k=1.0e4)
    p.dr, p.dz = 1.0 / nz, 1.0 / nz
    p.dt = 0.1 * p.dr
    p.precision = precision
    for k, v in overrides.items():
        setattr(p, k, v)
    X, Z = np.meshgrid(np.arange(nr) + 0.5, np.arange(nz) + 0.5)
    d = np.full((nz, nr), np.inf)
    disks = []
    for _ in range(int(rng.integers(2, 7))):
        r = rng.uniform(5.0, 25.0)
        cx, cz = rng.uniform(0, nr), rng.uniform(0, nz)
        disks.append((cx, cz, r))
        d = np.minimum(d, np.hypot(X - cx, Z - cz) - r)
    bdr = np.zeros(cell_shape(nr, nz))
    bdr[1:-1, 1:-1] = 0.5 * (1.0 - np.tanh(d / 0.75))
    neumann_ghosts_cell(bdr)
    return p, bdr, disks


def make_c3_pressure(seed, index, size=None, precision=abi.DRD_PREC_MIXED, **overrides):
    """Pressure system `index` of the seeded C3 batch: (params, bdr_ph, b) for the batched
    variable-coefficient Poisson solve (DRD_SYS_PRESSURE).  b is a Gaussian random field rounded to
    FP32, then its mean is removed in FP64 so that it lies in the operator's range."""
    rng = np.random.default_rng([seed, index, 2])
    p, bdr, disks = _c3_params_mask(rng, size, precision, overrides)
    b = _grf(rng, (p.nz, p.nr)).ravel()
    b = b - b.mean()
    return p, bdr, b, {"disks": disks}


def make_c3_solve(seed, index, size=None, precision=abi.DRD_PREC_MIXED, **overrides):
    """Solve `index` of the seeded C3 batch: (params, coefs, b) for DRDContext.solve(DRD_SYS_UV)."""
    rng = np.random.default_rng([seed, index])
    p, bdr, disks = _c3_params_mask(rng, size, precision, overrides)
    nr, nz = p.nr, p.nz
    M = 1.0 - bdr
    coefs = {"rho": np.ones(cell_shape(nr, nz)), "eta": 1.0 + 99.0 * bdr, "bdr_ph": bdr,
             "bdr_ph_grad": _grad_mag(bdr, dr=p.dr, dz=p.dz), "M0": M.copy(), "Mi": M.copy(), "bdr_pen": bdr.copy(),
             "bdr_used": M.copy()}
    b = np.concatenate([_grf(rng, (nz, nr + 1)).ravel(), _grf(rng, (nz - 1, nr)).ravel()])
    return p, coefs, b, {"disks": disks}


def interpolate_coef_host(params, dist, bdr_ph):
    """numpy form of interpolate_coef (interpolate_coef.f90:55-89) used to prepare inputs."""
    eps = params.I_thickness
    fpd = np.zeros_like(bdr_ph)
    fpd[1:-1, 1:-1] = np.tanh(-1.0 * dist / math.sqrt(2.0) / eps)
    fpd = (fpd + 1.0) / 2.0 + bdr_ph
    neumann_ghosts_cell(fpd)
    rho = 1.0 + (params.lambda_rho - 1.0) * fpd
    eta = 1.0 + (params.lambda_eta - 1.0) * fpd
    return fpd, rho, eta


def two_phase_coef_host(params, fpd, ph):
    """numpy form of the two-fluid coefficients (two_phase_flow_complex_domain/
    interpolate_coef.f90:91-112, commented out there), evaluated like drd_two_phase_coef."""
    lr, le = params.lambda_rho - 1.0, params.lambda_eta - 1.0
    rho = np.where(ph <= -1.0, 1.0, np.where(ph >= 1.0, params.lambda_rho, 1.0 + lr * ph))
    eta_ph = np.where(ph <= -1.0, 1.0, np.where(ph >= 1.0, params.lambda_eta, 1.0 + le * ph))
    eta = np.maximum(1.0 + le * fpd, eta_ph)
    return rho, eta


class Case:
    """A workload: parameters, resident-state fields and coefficient fields."""

    def __init__(self, name, params, state, coefs, dist, meta):
        self.name, self.params, self.state, self.coefs, self.dist, self.meta = name, params, state, coefs, dist, meta

    @property
    def nr(self):
        return self.params.nr

    @property
    def nz(self):
        return self.params.nz

    def copy_state(self):
        return {k: v.copy() for k, v in self.state.items()}


def _empty_state(nr, nz):
    st = {}
    for fid, kind in abi.FIELD_KIND.items():
        shape = {"u": u_shape, "v": v_shape, "cell": cell_shape}[kind](nr, nz)
        st[fid] = np.zeros(shape)
    return st


def fpd_dist_host(pp, points, nr, nz, dr, dz):
    """dist(r(i,k), z(i,k)) = fpd_dist of the beads (particles_move.f90:361-391), shape (nz, nr)."""
    X = ((np.arange(nr) + 0.5) * dr)[None, :]
    Z = ((np.arange(nz) + 0.5) * dz)[:, None]
    d = np.full((nz, nr), 1.0e10)
    for b in range(pp.np):
        d = np.minimum(d, np.sqrt((X - points[0, b]) ** 2 + (Z - points[1, b]) ** 2) - pp.fpd_radius)
    return d


def make_case(name="c2", seed=0, nr=None, nz=None, precision=abi.DRD_PREC_FP64, particles=False, **overrides):
    rng = np.random.default_rng(seed)
    name = name.lower()
    if name == "c1":
        nr = nr or 128
        nz = nz or 64
        slen, shig = 2.0, 1.0
        p = abi.default_params(nr, nz, xld=0.01, re=1.0, ca=0.1, I_thickness=0.02, s_implicit=1.5, tol=1e-10,
                               lambda_rho=1.0, lambda_eta=1.0, penalty_k=1.0e5, ggx=1.0, UU=1.0)
        p.dr, p.dz = slen / nr, shig / nz
        p.dt = 1.0e-3
        p.bdr_low, p.bdr_upp = 0.0, shig
    elif name == "c5":
        nr = nr or 2048
        nz = nz or 1024
        p = abi.default_params(nr, nz, re=1.0, ca=0.02, lambda_rho=1.0, lambda_eta=10.0, penalty_k=1.0e4,
                               two_fluid=1)
        p.dr, p.dz = 4.0 / nr, 2.0 / nz
        p.dt = min(p.dr, p.dz) * 0.1
    elif name in ("c2", "tp"):
        nr = nr or (420 if name == "c2" else 128)
        nz = nz or (180 if name == "c2" else 128)
        slen, shig = 3.5, 1.5
        p = abi.default_params(nr, nz, re=0.5, ca=0.05, lambda_rho=1.0, lambda_eta=5.0, penalty_k=1.0e4,
                               two_fluid=1 if name == "c2" else 0)
        p.dr, p.dz = slen / nr, shig / nz
        p.dt = min(p.dr, p.dz) * 0.1
    else:
        raise ValueError(f"unknown workload {name!r}")
    p.precision = precision
    for k, v in overrides.items():
        setattr(p, k, ord(v) if k == "lr_bd_type" and isinstance(v, str) else v)
    dr, dz, eps = p.dr, p.dz, p.I_thickness
    # cell-centre coordinates r(i,k) = (i+0.5) dr, z(i,k) = (k+0.5) dz (finit.f90:34-35)
    xi = (np.arange(nr) + 0.5)
    zk = (np.arange(nz) + 0.5)
    X, Z = np.meshgrid(xi * dr, zk * dz)  # [k, i]
    bdr = np.zeros(cell_shape(nr, nz))
    dist = np.full((nz, nr), 10.0)  # no particles: far away
    meta = {"seed": seed, "nr": nr, "nz": nz}
    sx, sz = nr / 420.0, nz / 180.0
    if name == "c5":
        bdr, dist, yc, half = _c5_channel(rng, p, nr, nz, X, Z, bdr, meta)
    if name in ("c2", "tp"):
        phase = rng.uniform(0, 2 * math.pi)
        amp, period, half = 30.0 * sz, 140.0 * sx, 45.0 * sz
        yc = nz / 2.0 + amp * np.sin(2 * math.pi * xi / period + phase)  # cells, per column
        slope = amp * 2 * math.pi / period * np.cos(2 * math.pi * xi / period + phase)
        d_cells = (half - np.abs(zk[:, None] - yc[None, :])) / np.sqrt(1.0 + slope[None, :] ** 2)
        smooth = max(2.0 * min(sx, sz), 0.75)
        bdr[1:-1, 1:-1] = 0.5 * (1.0 - np.tanh(d_cells / smooth))
        neumann_ghosts_cell(bdr)
        p.bdr_low = (yc[0] - half) * dz
        p.bdr_upp = (yc[0] + half) * dz
        meta.update(phase=phase, amp=amp, period=period, half=half)
        # rigid fibers 40 x 4 cells at seeded poses inside the channel
        fibers = []
        sdf = np.full((nz, nr), np.inf)
        for f in range(3):
            cxc = (f + 0.5) * nr / 3.0 + rng.uniform(-0.1, 0.1) * nr / 3.0
            ic = int(min(max(round(cxc - 0.5), 0), nr - 1))
            czc = yc[ic] + rng.uniform(-0.25, 0.25) * half
            ang = rng.uniform(0, math.pi)
            fibers.append((cxc, czc, ang))
            sdf = np.minimum(sdf, _rect_sdf(X / dr, Z / dz, cxc, czc, 20.0 * sx, 2.0 * sz, ang))
        dist = sdf * min(dr, dz)
        meta["fibers"] = fibers
    if particles:
        # the reference's fiber instead of the rigid fibers: a chain of Np = 9 beads placed by
        # particle_initialize (particles_move.f90:50-68) at mid-length on the channel centre line
        # (mcl6.f90:178 places it at (slen/2, 0.42) in its own channel), and bdr_ph_dist = the
        # distance to the walls inside the channel, 0 in the solid (global.f90:83)
        lx, ly = nr * dr, nz * dz
        pp = abi.default_particle_params(lx, ly)
        if name in ("c2", "tp"):
            ic = nr // 2
            ycen = yc[ic] * dz
            bd_cells = np.maximum(d_cells, 0.0) * min(dr, dz)
        else:
            ycen = ly / 2.0
            bd_cells = np.minimum(Z, ly - Z)
        points = np.array(abi.particle_chain(pp, lx / 2.0, ycen), dtype=np.float64)
        bdr_dist = np.zeros(cell_shape(nr, nz))
        bdr_dist[1:-1, 1:-1] = bd_cells
        neumann_ghosts_cell(bdr_dist)
        dist = fpd_dist_host(pp, points, nr, nz, dr, dz)
        meta["particles"] = {"pp": pp, "points": points, "bdr_dist": bdr_dist}
        meta.pop("fibers", None)
    fpd, rho, eta = interpolate_coef_host(p, dist, bdr)
    # phase field: drops (phi = 1 inside), clipped by the solid (finit.f90:288)
    ph = np.zeros(cell_shape(nr, nz))
    if name == "c5":
        _c5_drops(rng, ph, nr, nz, dr, dz, eps, X, Z, yc, half, meta)
    elif name == "c1":
        R = 12.0 * sz
        cx = nr / 2.0 + rng.uniform(-2, 2)
        cz = nz / 2.0 + rng.uniform(-2, 2)
        d = np.sqrt((X / dr - cx) ** 2 + (Z / dz - cz) ** 2) * dr
        ph[1:-1, 1:-1] = 0.5 * (1.0 + np.tanh((R * dr - d) / (math.sqrt(2.0) * eps)))
        meta["drops"] = [(cx, cz, R)]
    else:
        R = 15.0 * sz
        drops = []
        ymid = meta["phase"]
        for j in range(2):
            cxd = (j + 0.5) * nr / 2.0 + rng.uniform(-0.05, 0.05) * nr
            ic = int(min(max(round(cxd), 0), nr - 1))
            czd = yc[ic] + rng.uniform(-0.2, 0.2) * half
            drops.append((cxd, czd, R))
            d = np.sqrt((X / dr - cxd) ** 2 + (Z / dz - czd) ** 2) * min(dr, dz)
            ph[1:-1, 1:-1] = np.maximum(ph[1:-1, 1:-1],
                                        0.5 * (1.0 + np.tanh((R * min(dr, dz) - d) / (math.sqrt(2.0) * eps))))
        del ymid
        meta["drops"] = drops
    ph = np.minimum(1.0 - bdr, ph)
    neumann_ghosts_cell(ph)
    if name == "tp":
        # two_phase_flow_complex_domain: phi in [-1, 1], bdr_ph_used = 1 - bdr_ph, sharp penalty mask
        p.variant = abi.DRD_VARIANT_TP
        p.phi_mode = 2
        p.lr_bd_type = ord("d")
        p.uv_maxit = 2000
        p.penalty_k = 1.0e8
        ph = 2.0 * ph - 1.0
        neumann_ghosts_cell(ph)
    state = _empty_state(nr, nz)
    state[abi.F_PH] = ph
    state[abi.F_RMU] = _rmu_init(ph, eps, dr, dz)
    M = 1.0 - bdr
    coefs = {
        "rho": rho, "eta": eta, "fpd": fpd, "bdr_ph": bdr, "bdr_ph_grad": _grad_mag(bdr, dr, dz),
        "M0": M.copy(), "Mi": M.copy(), "bdr_pen": bdr.copy(), "bdr_used": 1.0 - bdr,
    }
    if p.two_fluid:
        # the drops carry the viscosity ratio (eta = lambda_eta inside them, 1 in the matrix fluid)
        coefs["rho"], coefs["eta"] = two_phase_coef_host(p, fpd, ph)
    if name == "tp":
        coefs["bdr_pen"] = (bdr > 0.5).astype(np.float64)
        coefs["M0"] = (1.0 - bdr) * (ph ** 2 - 1.0) ** 2
    return Case(name, p, state, coefs, dist, meta)


def load_reference_geometry(path):
    """The reference's serpentine geometry (a domain_snake_420_180.npz fixture holding the raw
    domain_snake_420_180.bin and _dist.bin values, each a [nr][nz] array as read_var reads
    them, microfluidics_complex_domain/inout.f90:75-86) -> (mask, dist) as [k][i] arrays."""
    z = np.load(path)
    return np.ascontiguousarray(z["mask"].T), np.ascontiguousarray(z["dist"].T)


def mask_cell(mask):
    """finit's ph = bdr_ph from the mask (finit.f90:121-141): interior from the file, Neumann
    ghosts; the input of drd_finit_wall."""
    nz, nr = mask.shape
    a = np.zeros(cell_shape(nr, nz))
    a[1:-1, 1:-1] = mask
    return neumann_ghosts_cell(a)


def make_reference_snake(bdr_ph, wall_dist, precision=abi.DRD_PREC_FP64, **overrides):
    """The reference's own microfluidics example on its own geometry: the MF deck
    (microfluidics_complex_domain/input), bdr_ph = finit's smoothed wall indicator (CELL, the
    output of drd_finit_wall on the domain_snake mask), bdr_ph_dist = the distance file
    (interior; the ghosts keep the zero of the module array), the 9-bead fiber at
    (slen/2, (0.17 + 0.67)/2) (mcl6.f90:178), and the fluid stripe of finit.f90:222-233:
    ph = min(tanh((r - 0.4 slen - 0.2)/(sqrt2 eps)), tanh(-(r - 0.6 slen - 0.2)/(sqrt2 eps))),
    rescaled to [0, 1] and clipped by 1 - bdr_ph; rmu, bdr_ph_grad, ph_M_0 = ph_M_inner =
    1 - bdr_ph as finit.f90:244-278 computes them."""
    nz, nr = bdr_ph.shape[0] - 2, bdr_ph.shape[1] - 2
    p = abi.default_params(nr, nz)
    p.precision = precision
    for k, v in overrides.items():
        setattr(p, k, v)
    dr, dz, eps = p.dr, p.dz, p.I_thickness
    slen = nr * dr
    bdr = np.array(bdr_ph, dtype=np.float64, copy=True)
    pp = abi.default_particle_params(slen, nz * dz)
    points = np.array(abi.particle_chain(pp, slen / 2.0, (0.17 + 0.67) / 2.0), dtype=np.float64)
    bdr_dist = np.zeros(cell_shape(nr, nz))
    bdr_dist[1:-1, 1:-1] = wall_dist
    dist = fpd_dist_host(pp, points, nr, nz, dr, dz)
    fpd, rho, eta = interpolate_coef_host(p, dist, bdr)
    r = ((np.arange(nr) + 0.5) * dr)[None, :] * np.ones((nz, 1))
    s2 = math.sqrt(2.0) * eps
    ph = np.zeros(cell_shape(nr, nz))
    ph[1:-1, 1:-1] = np.minimum(np.tanh((r - 0.4 * slen - 0.2) / s2), np.tanh(-(r - 0.6 * slen - 0.2) / s2))
    ph = (ph + 1.0) / 2.0
    ph = np.minimum(1.0 - bdr, ph)
    neumann_ghosts_cell(ph)
    state = _empty_state(nr, nz)
    state[abi.F_PH] = ph
    state[abi.F_RMU] = _rmu_init(ph, eps, dr, dz)
    M = 1.0 - bdr
    coefs = {"rho": rho, "eta": eta, "fpd": fpd, "bdr_ph": bdr, "bdr_ph_grad": _grad_mag(bdr, dr, dz),
             "M0": M.copy(), "Mi": M.copy(), "bdr_pen": bdr.copy(), "bdr_used": 1.0 - bdr}
    meta = {"particles": {"pp": pp, "points": points, "bdr_dist": bdr_dist}, "nr": nr, "nz": nz}
    return Case("reference_snake", p, state, coefs, dist, meta)
