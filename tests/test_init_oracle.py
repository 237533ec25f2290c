"""Pins of the oracle's PhSolve_ori and finit wall smoothing (CPU only).

microfluidics_complex_domain/PhSolve_ori.f90 and finit.f90:120-189 have no reference test or
output, so the restatement is pinned by
  * an independent numpy restatement of MATRIX_VECTOR_CG_ori's stencil (:368-421);
  * a dense direct solve of the same system: BiCGSTAB's answer must agree with it;
  * known answers: a uniform phase (phi = 1 everywhere) is a fixed point of the smoothing.
"""
import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.layout import u_shape, v_shape
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import rel_err


def _params(nr=14, nz=9, tol=1e-12):
    p = abi.default_params(nr, nz, tol=tol)
    p.dr, p.dz = 3.5 / nr, 1.5 / nz
    p.dt = 1.0e-4  # finit.f90:151
    return p


def _lap_nn(a, dr2, dz2):
    """laplace_nn (PhSolve_ori.f90:463-487) of an (nz, nr) interior array."""
    g = np.pad(a, 1, mode="edge")
    return (g[1:-1, 2:] + g[1:-1, :-2] - 2 * a) / dr2 + (g[2:, 1:-1] + g[:-2, 1:-1] - 2 * a) / dz2


def _ori_matvec_np(P, x, cb):
    nr, nz = P.nr, P.nz
    dr2, dz2, eps = P.dr ** 2, P.dz ** 2, P.I_thickness
    f1 = x.reshape(nz, nr)
    ff1 = -eps * _lap_nn(f1, dr2, dz2)
    ff1[0] += eps / dz2 * (f1[0] - cb * f1[0])
    ff1[-1] += eps / dz2 * (f1[-1] - cb * f1[-1])
    ff1 = ff1 + f1 * P.s_implicit / eps
    ff2 = f1 - P.dt * P.xld * _lap_nn(ff1, dr2, dz2)
    return ff2.reshape(-1)


@pytest.mark.parametrize("alpha_s", [0.0, 0.37])
def test_ori_matvec_matches_numpy(oracle_build, alpha_s):
    P = _params()
    o = Oracle(P)
    x = np.random.default_rng(3).standard_normal(P.nr * P.nz)
    cb = o.ori_coef(alpha_s)
    assert abs(cb - (P.I_thickness / P.dz - 0.5 * alpha_s) / (P.I_thickness / P.dz + 0.5 * alpha_s)) < 1e-15
    assert rel_err(o.ori_matvec(x, alpha_s), _ori_matvec_np(P, x, cb)) < 1e-13


def test_phsolve_ori_matches_dense_solve(oracle_build):
    P = _params()
    o = Oracle(P)
    nr, nz, n = P.nr, P.nz, P.nr * P.nz
    case = make_case("c2", seed=1, nr=nr, nz=nz)
    ph = 2.0 * case.coefs["bdr_ph"] - 1.0
    rng = np.random.default_rng(5)
    u, v = 0.1 * rng.standard_normal(u_shape(nr, nz)), 0.1 * rng.standard_normal(v_shape(nr, nz))
    angB, angT = rng.uniform(30, 150, nr + 1), rng.uniform(30, 150, nr + 1)
    rhs, _, pnb, pnt = o.ori_system(u, v, ph, angB, angT, 0.2)
    A = np.stack([o.ori_matvec(np.eye(n)[j], 0.2) for j in range(n)], axis=1)
    x = np.linalg.solve(A, rhs)
    rmu_after, ph_after, st = o.phsolve_ori(u, v, ph, angB, angT, 0.2)
    assert st.info == 0
    assert rel_err(ph_after[1:-1, 1:-1].reshape(-1), x) < 1e-9
    cb = o.ori_coef(0.2)
    # ghost rows (PhSolve_ori.f90:159-162) and Neumann columns
    assert rel_err(ph_after[0, 1:-1], ph_after[1, 1:-1] * cb + pnb) < 1e-14
    assert rel_err(ph_after[-1, 1:-1], ph_after[-2, 1:-1] * cb + pnt) < 1e-14
    assert np.array_equal(ph_after[:, 0], ph_after[:, 1]) and np.array_equal(ph_after[:, -1], ph_after[:, -2])
    # rmu_after = -eps lap(ph_after) - ph/eps + ph^3/eps (:178-184), using the ghosts just set
    eps = P.I_thickness
    pa = ph_after
    lap = (pa[1:-1, 2:] + pa[1:-1, :-2] - 2 * pa[1:-1, 1:-1]) / P.dr ** 2 + \
          (pa[2:, 1:-1] + pa[:-2, 1:-1] - 2 * pa[1:-1, 1:-1]) / P.dz ** 2
    expect = -eps * lap - pa[1:-1, 1:-1] / eps + pa[1:-1, 1:-1] ** 3 / eps
    assert rel_err(rmu_after[1:-1, 1:-1], expect) < 1e-12


def test_finit_wall_uniform_phase_is_fixed(oracle_build):
    P = _params()
    o = Oracle(P)
    bdr = np.ones((P.nz + 2, P.nr + 2))  # ph = 1: bulk minimum, zero wall flux at angle 0 up to cos(pi/2)
    out, ph, rmu, info = o.finit_wall(bdr, 3)
    assert info == 0
    assert np.abs(out[1:-1, 1:-1] - 1.0).max() < 1e-12
    assert np.abs(ph[1:-1, 1:-1] - 1.0).max() < 1e-12


def test_finit_wall_smooths_the_indicator(oracle_build):
    P = _params(nr=40, nz=24, tol=1e-10)
    o = Oracle(P)
    case = make_case("c2", seed=2, nr=40, nz=24)
    sharp = (case.coefs["bdr_ph"] > 0.5).astype(np.float64)
    out, ph, rmu, info = o.finit_wall(sharp, 10)
    assert info == 0
    inner = out[1:-1, 1:-1]
    assert inner.min() >= 0.0 and inner.max() <= 1.0
    # the step is spread over a few cells: intermediate values appear next to the walls
    assert ((inner > 0.05) & (inner < 0.95)).sum() > 0
    assert rel_err(out[1:-1, 1:-1], np.clip((ph[1:-1, 1:-1] + 1.0) / 2.0, 0.0, 1.0)) < 1e-15
