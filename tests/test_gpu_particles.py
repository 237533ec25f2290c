"""Fiber particles on the GPU against the oracle (particles_move.f90, mcl6.f90:394-402).

Each reference routine is called through the C-ABI with the same inputs as the oracle:
force_caculation_vel (tot_F and the spread particle_force1/2), update_position_vel (bead
moves), interpolate_coef with fpd_dist, and the particle-coupled mcl6 step sequence.  All
arithmetic is FP64 on both sides; tolerances are stated per check.
"""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.api import DRDContext, DRDError
from drd_application_gb300.layout import u_shape, v_shape
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu
F = abi


def _setup(name="c2", nr=84, nz=36, seed=3, where="bent"):
    case = make_case(name, seed=seed, nr=nr, nz=nz, particles=True)
    parts = case.meta["particles"]
    pp = parts["pp"]
    pts = parts["points"].copy()
    rng = np.random.default_rng(seed)
    pts += rng.uniform(-0.3, 0.3, size=pts.shape) * pp.l0
    bdr_dist = parts["bdr_dist"]
    if where == "periodic":
        pts[0] += pp.lx - pts[0].max() + 0.01
        pts[0] = np.where(pts[0] > pp.lx, pts[0] - pp.lx, pts[0])
    elif where == "wall":
        pts[1] -= pts[1].min() - 0.03  # bottom bead inside the wall-repulsion range
    return case, pp, pts, bdr_dist


@pytest.mark.parametrize("name,where", [("c2", "bent"), ("c1", "periodic"), ("c1", "wall")])
def test_force_caculation_vel(cuda_lib, oracle_build, name, where):
    case, pp, pts, bd = _setup(name, where=where)
    P = case.params
    ctx = DRDContext(P)
    ctx.set_case(case)
    ctx.particles_set(pp, pts, bd)
    pf1, pf2 = ctx.force_caculation_vel(P.dt, 0.0)
    _, tot = ctx.particles_get()
    o = Oracle(P)
    tot_o, pf1_o, pf2_o = o.force_caculation_vel(pp, pts, bd)
    # one thread in the reference's order: libm differences (atan2, sqrt are exact) only
    assert rel_err(tot, tot_o) < 1e-12
    if where == "wall":
        assert abs(tot_o[1, 8]) > 1.0
    # tree-ordered sums and CUDA tanh against sequential sums and glibc tanh
    assert rel_err(pf1, pf1_o) < 1e-12 and rel_err(pf2, pf2_o) < 1e-12
    ctx.close()


def test_update_position_vel(cuda_lib, oracle_build):
    case, pp, pts, bd = _setup("c2", seed=5)
    P = case.params
    rng = np.random.default_rng(8)
    u = rng.standard_normal(u_shape(P.nr, P.nz))
    v = rng.standard_normal(v_shape(P.nr, P.nz))
    ctx = DRDContext(P)
    ctx.set_case(case)
    ctx.particles_set(pp, pts, bd)
    dt = 0.05  # large enough that the move is far above rounding
    ctx.update_position_vel(u, v, dt)
    got, _ = ctx.particles_get()
    exp = Oracle(P).update_position_vel(pp, pts, u, v, dt)
    assert np.abs(got - exp).max() < 1e-13
    assert np.abs(got - pts).max() > 1e-4
    ctx.close()


def test_interpolate_coef_particles(cuda_lib, oracle_build):
    case, pp, pts, bd = _setup("c2", seed=6)
    P = case.params
    ctx = DRDContext(P)
    ctx.set_case(case)
    ctx.particles_set(pp, pts, bd)
    fpd, rho, eta = ctx.interpolate_coef_particles()
    o = Oracle(P)
    fpd_o, rho_o, eta_o = o.interpolate_coef(o.fpd_dist_field(pp, pts), case.coefs["bdr_ph"])
    assert rel_err(fpd, fpd_o) < 1e-14 and rel_err(rho, rho_o) < 1e-14 and rel_err(eta, eta_o) < 1e-14
    ctx.close()


def test_particles_set_rejects_bad_counts(cuda_lib):
    case, pp, pts, bd = _setup("c1", nr=32, nz=16)
    ctx = DRDContext(case.params)
    bad = pp.copy()
    bad.np = 2
    with pytest.raises(DRDError):
        ctx.particles_set(bad, pts[:, :2], bd)
    bad.np = abi.PARTICLES_MAX + 1
    with pytest.raises(DRDError):
        ctx.particles_set(bad, np.zeros((2, bad.np)), bd)
    ctx.close()


@pytest.mark.parametrize("precision", [abi.DRD_PREC_FP64, abi.DRD_PREC_MIXED])
def test_step_sequence_with_particles(cuda_lib, oracle_build, precision):
    """Four particle-coupled mcl6 steps (PhSolve, the particle block, momentum, pressure) on the
    resident state against the oracle at Krylov tol 1e-12: bead positions, forces and fields."""
    case, pp, pts, bd = _setup("c2", nr=48, nz=24, seed=7)
    P = case.params.copy()
    P.tol = 1e-12
    P.precision = precision
    # a 5-bead chain scaled to the small grid so that each bead covers a few cells
    pp.np = 5
    pp.fpd_radius, pp.l0 = 0.05, 0.1
    pp.fpd_fpd_dist, pp.fpd_bdr_dist = 0.12, 0.09
    pts = np.array(abi.particle_chain(pp, 1.7, case.meta["particles"]["points"][1, 4]))
    pts += np.random.default_rng(1).uniform(-0.02, 0.02, size=pts.shape)
    ctx = DRDContext(P)
    ctx.set_case(case)
    ctx.upload_state(case.state)
    ctx.particles_set(pp, pts, bd)
    orc = Oracle(P)
    st = case.copy_state()
    X = {"pp": pp, "points": pts.copy(), "bdr_dist": bd}
    t = 0.0
    for s in range(4):
        stats = ctx.step(s == 0, t)
        orc.step(st, case.coefs, s == 0, t, particles=X)
        assert stats.ch.info == 0 and stats.uv.info == 0
        t += P.dt
    g = ctx.download_state()
    got_pts, got_tot = ctx.particles_get()
    fp64 = precision == abi.DRD_PREC_FP64
    tol = 1e-8 if fp64 else 1e-6
    # positions integrate u dt (dt = 6e-3): their error is the velocity error times dt
    assert np.abs(got_pts - X["points"]).max() < (1e-11 if fp64 else 1e-9)
    assert rel_err(got_tot, X["tot_F"]) < (1e-8 if fp64 else 1e-6)
    for fid in (F.F_U, F.F_V, F.F_PH, F.F_RMU, F.F_P, F.F_PSI2, F.F_PF1, F.F_PF2):
        assert rel_err(g[fid], st[fid]) < tol, fid
    assert np.abs(g[F.F_PF1]).max() > 0
    ctx.close()
