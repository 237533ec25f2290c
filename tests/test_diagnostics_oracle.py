"""dissipation's diagnostics and reinint_by_PhSolve in the oracle, and the fort.22 / fort.23
records, on the CPU.

The oracle's dissipation (oracle/drd_oracle.c) is checked against an independent numpy
restatement of microfluidics_complex_domain/dissipation.f90:1-122 and against closed forms;
the record writers against hand-formatted Fortran E fields."""
import math

import numpy as np
import pytest

from drd_application_gb300 import abi, fileio
from drd_application_gb300.layout import neumann_ghosts_cell, u_shape, v_shape
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle
from tests.helpers import advanced_case


def numpy_dissipation(P, u, v, ph, rmu, vs, angB=None, angT=None):
    """dissipation.f90 in numpy, arrays as [k + k0, i + i0]: e1 (:39-47), e2 (:49-57), e3 (:59-88)
    with v's derivatives on its own grid, e4 = 0 (no slip), mass (:113-122)."""
    nr, nz, dr, dz, eps = P.nr, P.nz, P.dr, P.dz, P.I_thickness
    pi = math.pi
    R = lambda i, k: rmu[k + 1, i + 1]  # noqa: E731
    I = np.arange(nr)[None, :]
    K = np.arange(nz)[:, None]
    gx = (R(I + 1, K) - R(I - 1, K)) / 2.0 / dr
    gz = (R(I, K + 1) - R(I, K - 1)) / 2.0 / dz
    e1 = float(np.sum(gx ** 2 + gz ** 2)) * P.xld * P.ca * dr * dz
    aT = np.full(nr, P.angle) if angT is None else angT[:nr]
    aB = np.full(nr, P.angle) if angB is None else angB[:nr]
    top, top1 = ph[nz + 1, 1:nr + 1], ph[nz, 1:nr + 1]
    bot, bot0 = ph[0, 1:nr + 1], ph[1, 1:nr + 1]
    cfT = math.sqrt(2.0) * np.cos(aT * pi / 180.0) / 3.0 * pi / 2.0 / eps
    cfB = math.sqrt(2.0) * np.cos(aB * pi / 180.0) / 3.0 * pi / 2.0 / eps
    e2 = float(np.sum(((top - top1) / dz - cfT * np.cos(pi * (top + top1) / 4.0)) ** 2 +
                      ((bot - bot0) / dz - cfB * np.cos(pi * (bot0 + bot) / 4.0)) ** 2)) * vs * P.ca * eps ** 2 * dr
    U = lambda i, k: u[k + 1, i + 1]  # noqa: E731
    V = lambda i, k: v[k, i + 1]  # noqa: E731
    In = np.arange(nr + 1)[None, :]
    Kn = np.arange(nz + 1)[:, None]
    uua = (U(In + 1, Kn) - U(In - 1, Kn)) / 2.0 / dr
    uub = np.empty((nz + 1, nr + 1))
    vvb = np.empty((nz + 1, nr + 1))
    Ki = np.arange(1, nz)[:, None]
    uub[1:nz] = (U(In, Ki + 1) - U(In, Ki - 1)) / 2.0 / dz
    vvb[1:nz] = (V(In, Ki + 1) - V(In, Ki - 1)) / 2.0 / dz
    uub[0], uub[nz] = (U(In[0], 1) - U(In[0], 0)) / dz, (U(In[0], nz) - U(In[0], nz - 1)) / dz
    vvb[0], vvb[nz] = (V(In[0], 1) - V(In[0], 0)) / dz, (V(In[0], nz) - V(In[0], nz - 1)) / dz
    vva = np.empty((nz + 1, nr + 1))
    Ii = np.arange(nr)[None, :]
    vva[:, :nr] = (V(Ii + 1, Kn) - V(Ii - 1, Kn)) / 2.0 / dr
    vva[:, nr] = (V(nr, Kn[:, 0]) - V(nr - 1, Kn[:, 0])) / dr
    cx = np.ones(nr + 1); cx[0] = cx[-1] = 0.5
    cz = np.ones(nz + 1); cz[0] = cz[-1] = 0.5
    e3 = float(np.sum(cz[:, None] * cx[None, :] * (uua ** 2 + vvb ** 2 + uub ** 2 + vva ** 2))) * dr * dz
    mass = float(np.sum(ph[1:-1, 1:-1])) * dr * dz
    return e1, e2, e3, 0.0, e1 + e2 + e3, mass


def test_oracle_dissipation_matches_numpy(oracle_build):
    case, st, _ = advanced_case("c2", seed=4, nr=40, nz=20, steps=2)
    P = case.params
    rng = np.random.default_rng(3)
    angB, angT = rng.uniform(30, 150, P.nr + 1), rng.uniform(30, 150, P.nr + 1)
    o = Oracle(P)
    for a in ((None, None), (angB, angT)):
        got = o.dissipation(st[abi.F_U], st[abi.F_V], st[abi.F_PH], st[abi.F_RMU], 5.0e4, *a)
        ref = numpy_dissipation(P, st[abi.F_U], st[abi.F_V], st[abi.F_PH], st[abi.F_RMU], 5.0e4, *a)
        for g, r in zip(got, ref):
            assert abs(g - r) <= 1e-12 * max(abs(r), 1e-300)
    assert got[2] > 0 and got[0] > 0


def test_oracle_dissipation_closed_forms(oracle_build):
    """Rest state with a uniform phase field: e1 = e3 = 0; e2 is the wall residual of a uniform
    ph alone, 2 nr (cf cos(pi ph/2))^2 vs ca eps^2 dr; a linear shear u = z gives
    e3 = (nr+1 - 1)(trapezoid) ... checked as dr dz sum Cx Cz over the nodes of u_z^2 = 1."""
    P = abi.default_params(24, 12)
    o = Oracle(P)
    u, v = np.zeros(u_shape(24, 12)), np.zeros(v_shape(24, 12))
    ph = np.full((14, 26), 0.3)
    rmu = np.full((14, 26), 2.0)
    e1, e2, e3, e4, dis, m = o.dissipation(u, v, ph, rmu, 1.0)
    cf = math.sqrt(2.0) * math.cos(P.angle * math.pi / 180.0) / 3.0 * math.pi / 2.0 / P.I_thickness
    e2_ref = 2 * 24 * (cf * math.cos(math.pi * 0.6 / 4.0)) ** 2 * P.ca * P.I_thickness ** 2 * P.dr
    assert e1 == 0.0 and e3 == 0.0 and e4 == 0.0
    assert abs(e2 - e2_ref) <= 1e-12 * e2_ref and abs(m - 0.3 * 24 * 12 * P.dr * P.dz) < 1e-14
    # u(i,k) = z_k = (k + 0.5) dz on every row including the ghosts: u_z = 1 at every node
    z = (np.arange(-1, 13) + 0.5) * P.dz
    u = np.repeat(z[:, None], 27, axis=1)
    e3 = o.dissipation(u, v, ph, rmu, 1.0)[2]
    assert abs(e3 - 24 * 12 * P.dr * P.dz) <= 1e-12


def test_reinint_oracle(oracle_build):
    case = make_case("tp", seed=3, nr=40, nz=20)
    P = case.params.copy()
    P.dt, P.tol = 1.0e-4, 1e-11
    sharp = np.where(case.coefs["bdr_ph"] > 0.5, 1.0, -1.0)
    neumann_ghosts_cell(sharp)
    o = Oracle(P)
    b, pen, info = o.reinint_by_phsolve(sharp)
    b2, _, _, _ = o.finit_wall(sharp, 51)
    assert info == 0 and np.array_equal(b, b2)
    assert np.array_equal(pen, (b > 0.5).astype(np.float64))
    assert b[1:-1, 1:-1].min() >= 0.0 and b[1:-1, 1:-1].max() <= 1.0


@pytest.mark.parametrize("x,s", [(1.0, " 0.1000000E+01"), (-0.000123456789, "-0.1234568E-03"), (0.0, " 0.0000000E+00"),
                                 (0.99999999, " 0.1000000E+01"), (1.5e-120, " 0.1500000-119"), (123456.75, " 0.1234568E+06")])
def test_fort23_record_format(tmp_path, x, s):
    d = abi.drd_diagnostics(x, 0.0, 0.0, 0.0, 0.0, 0.0)
    path = tmp_path / "fort.23"
    fileio.write_fort23(path, 2.5, d)
    line = open(path).read().rstrip("\n")
    assert len(line) == 6 * 14
    assert line[:14] == " 0.2500000E+01" and line[14:28] == s


def test_fort22_record(tmp_path):
    d = abi.drd_diagnostics(0, 0, 0, 0, 2.0, 0.125)
    path = tmp_path / "fort.22"
    fileio.write_fort22(path, 7, 0.001, d)
    fileio.write_fort22(path, 8, 0.001, d)
    rows = [r.split() for r in open(path).read().splitlines()]
    assert len(rows) == 2 and rows[0][0] == "7" and rows[1][0] == "8"
    assert float(rows[0][1]) == 0.002 and float(rows[0][2]) == 0.125
