"""Pins of the oracle's fiber-particle routines (CPU only).

The reference ships no test or output for microfluidics_complex_domain/particles_move.f90, so
the oracle's restatement is pinned by
  * known answers: a straight chain at rest spacing feels only the bead-bead repulsion of its
    two end beads (particles_move.f90:1040-1046); a uniform flow moves every bead by u dt;
  * an independent vectorised numpy restatement of fpd_dist_periodic, the spreading of
    force_caculation_vel and the averages of update_position_vel;
  * conservation: each bead's spread force integrates to tot_F over the grid.
"""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.layout import cell_shape, ptr, u_shape, v_shape
from drd_application_gb300.workloads import fpd_dist_host, make_case
from oracle.oracle import Oracle
from tests.helpers import rel_err


def _grid(P):
    x = ((np.arange(P.nr) + 0.5) * P.dr)[None, :]
    z = ((np.arange(P.nz) + 0.5) * P.dz)[:, None]
    return x, z


def _indicator_np(P, pp, bx, by):
    """(tanh(-d/sqrt(2)/eps)+1)/2 of fpd_dist_periodic (particles_move.f90:326-357, :786-787)."""
    x, z = _grid(P)
    xd = -pp.lx if bx < pp.fpd_radius else (pp.lx if pp.lx - bx < pp.fpd_radius else 0.0)
    yd = -pp.ly if by < pp.fpd_radius else (pp.ly if pp.ly - by < pp.fpd_radius else 0.0)
    d = np.sqrt((x - bx) ** 2 + (z - by) ** 2) - pp.fpd_radius
    d = np.minimum(d, np.sqrt((x + xd - bx) ** 2 + (z - by) ** 2) - pp.fpd_radius)
    d = np.minimum(d, np.sqrt((x - bx) ** 2 + (z + yd - by) ** 2) - pp.fpd_radius)
    d = np.minimum(d, np.sqrt((x + xd - bx) ** 2 + (z + yd - by) ** 2) - pp.fpd_radius)
    return (np.tanh(-1.0 * d / np.sqrt(2.0) / P.I_thickness) + 1.0) / 2.0


def _case(seed=3, nr=96, nz=48, name="c1"):
    case = make_case(name, seed=seed, nr=nr, nz=nz, particles=True)
    return case, case.meta["particles"]


def _bent(pts, pp, seed):
    rng = np.random.default_rng(seed)
    out = pts.copy()
    out += rng.uniform(-0.3, 0.3, size=pts.shape) * pp.l0
    return out


def test_default_params_and_chain(oracle_build):
    pp = abi.default_particle_params(3.5, 1.5)
    assert (pp.np, pp.fpd_radius, pp.l0, pp.ks, pp.kb) == (9, 0.025, 0.05, 5.0, 0.25)
    assert pp.fpd_fpd_dist == 0.025 + 0.025 + 0.01 and pp.fpd_bdr_dist == 0.025 + 0.02
    pts = np.array(abi.particle_chain(pp, 1.75, 0.42))
    assert np.all(pts[0] == 1.75)
    # particles_move.f90:58-64: bead 4 at the centre, bead i at yc + (4-i) l0
    assert pts[1, 4] == 0.42 and abs(pts[1, 0] - (0.42 + 4 * 0.05)) < 1e-15 and abs(pts[1, 8] - (0.42 - 0.2)) < 1e-15
    # the C library's own helpers (same arithmetic) agree bit for bit
    L = oracle_build.lib()
    q = abi.drd_particle_params()
    L.drd_particle_params_default(q, 3.5, 1.5)
    assert bytes(q) == bytes(pp)
    out = np.zeros((2, 9))
    L.drd_particle_initialize(q, 1.75, 0.42, ptr(out))
    assert np.array_equal(out, pts)


def test_straight_chain_forces_known_answer(oracle_build):
    """At rest spacing l0 with zero bending, only neighbour repulsion acts (l0 = 0.05 is inside
    fpd_fpd_dist = 0.06): interior beads cancel, the end beads are pushed apart with
    k0_inter (eq - l0) / eq^2."""
    case, parts = _case()
    o = Oracle(case.params)
    pp = parts["pp"]
    tot = o.particle_forces(pp, parts["points"], parts["bdr_dist"])
    mag = pp.k0_inter * (pp.fpd_fpd_dist - pp.l0) / pp.fpd_fpd_dist ** 2
    expect = np.zeros((2, 9))
    expect[1, 0], expect[1, 8] = mag, -mag
    assert np.abs(tot - expect).max() < 1e-9


def test_wall_force_pushes_away(oracle_build):
    """interaction_force_bdr (particles_move.f90:1069-1103): a bead closer to the wall than
    fpd_bdr_dist is pushed along the gradient of the wall distance (away from the wall)."""
    case, parts = _case()
    o = Oracle(case.params)
    pp = parts["pp"]
    pts = parts["points"].copy()
    pts[1] -= pts[1, 8] - 0.03  # lowest bead 0.03 above the bottom (distance field min(z, ly - z))
    tot = o.particle_forces(pp, pts, parts["bdr_dist"])
    free = o.particle_forces(pp, parts["points"], parts["bdr_dist"])
    assert tot[1, 8] - free[1, 8] > 1.0  # upward push on the bottom bead
    assert np.abs(tot[:, :8] - free[:, :8]).max() < 1e-9


@pytest.mark.parametrize("where", ["inside", "periodic_x", "periodic_y"])
def test_spreading_matches_numpy_restatement(oracle_build, where):
    case, parts = _case(seed=5)
    P = case.params
    o = Oracle(P)
    pp = parts["pp"]
    pts = _bent(parts["points"], pp, 11)
    if where == "periodic_x":
        pts[0] += pp.lx - pts[0].max() + 0.01  # beads straddle x = lx
        pts[0] = np.where(pts[0] > pp.lx, pts[0] - pp.lx, pts[0])
    bdr_dist = parts["bdr_dist"]
    if where == "periodic_y":
        pts[1] -= pts[1].min() - 0.01  # beads straddle y = 0; no walls in this box
        bdr_dist = np.ones_like(bdr_dist)
    tot, pf1, pf2 = o.force_caculation_vel(pp, pts, bdr_dist)
    e1 = np.zeros(cell_shape(P.nr, P.nz))
    e2 = np.zeros_like(e1)
    for b in range(pp.np):
        dd = _indicator_np(P, pp, pts[0, b], pts[1, b])
        s = dd.sum() * P.dr * P.dz
        e1[1:-1, 1:-1] += tot[0, b] * dd / s
        e2[1:-1, 1:-1] += tot[1, b] * dd / s
    assert rel_err(pf1, e1) < 1e-12 and rel_err(pf2, e2) < 1e-12
    # conservation: each spread force integrates to the bead force
    assert abs(pf1.sum() * P.dr * P.dz - tot[0].sum()) < 1e-10 * max(1.0, np.abs(tot).sum())
    assert abs(pf2.sum() * P.dr * P.dz - tot[1].sum()) < 1e-10 * max(1.0, np.abs(tot).sum())


def test_update_position_uniform_flow_and_wrap(oracle_build):
    case, parts = _case(seed=2)
    P = case.params
    o = Oracle(P)
    pp = parts["pp"]
    pts = parts["points"].copy()
    pts[0] = pp.lx - 0.004  # the move below carries every bead across x = lx
    u = np.full(u_shape(P.nr, P.nz), 3.0)
    v = np.full(v_shape(P.nr, P.nz), -1.5)
    dt = 0.002
    out = o.update_position_vel(pp, pts, u, v, dt)
    assert np.abs(out[0] - (pts[0] + 3.0 * dt - pp.lx)).max() < 1e-13
    assert np.abs(out[1] - (pts[1] - 1.5 * dt)).max() < 1e-13


def test_update_position_matches_numpy_restatement(oracle_build):
    case, parts = _case(seed=4)
    P = case.params
    o = Oracle(P)
    pp = parts["pp"]
    pts = _bent(parts["points"], pp, 4)
    rng = np.random.default_rng(9)
    u = rng.standard_normal(u_shape(P.nr, P.nz))
    v = rng.standard_normal(v_shape(P.nr, P.nz))
    dt = 1e-3
    out = o.update_position_vel(pp, pts, u, v, dt)
    nr, nz = P.nr, P.nz
    # u(i,k) at [k+1, i+1] of the UFACE array; the reference averages u(i,k) and u(i,k+1)
    ua = (u[1:nz + 1, 1:nr + 1] + u[2:nz + 2, 1:nr + 1]) / 2.0
    va = (v[0:nz, 1:nr + 1] + v[1:nz + 1, 1:nr + 1]) / 2.0
    for b in range(pp.np):
        dd = _indicator_np(P, pp, pts[0, b], pts[1, b])
        ex = pts[0, b] + (ua * dd).sum() / dd.sum() * dt
        ey = pts[1, b] + (va * dd).sum() / dd.sum() * dt
        assert abs(out[0, b] - ex) < 1e-14 and abs(out[1, b] - ey) < 1e-14


def test_fpd_dist_field(oracle_build):
    case, parts = _case(seed=6)
    P = case.params
    o = Oracle(P)
    pp = parts["pp"]
    pts = _bent(parts["points"], pp, 6)
    d = o.fpd_dist_field(pp, pts)
    assert np.array_equal(d, fpd_dist_host(pp, pts, P.nr, P.nz, P.dr, P.dz))


def test_step_with_particles_moves_chain(oracle_build):
    """The mcl6 loop with the particle block (mcl6.f90:394-402): the chain moves, rho and eta
    follow it, particle forces are spread."""
    case, parts = _case(name="c2", nr=84, nz=36, seed=1)
    o = Oracle(case.params)
    st = case.copy_state()
    X = {"pp": parts["pp"], "points": parts["points"].copy(), "bdr_dist": parts["bdr_dist"]}
    t = 0.0
    for s in range(3):
        o.step(st, case.coefs, s == 0, t, particles=X)
        t += case.params.dt
    assert np.isfinite(X["points"]).all() and np.isfinite(st[abi.F_U]).all()
    assert not np.array_equal(X["points"], parts["points"])
    assert np.abs(st[abi.F_PF2]).max() > 0
    fpd = X["fpd"]
    assert rel_err(X["rho"], 1.0 + (case.params.lambda_rho - 1.0) * fpd) < 1e-15
