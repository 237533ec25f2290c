"""The batched solves' pressure Poisson system in the oracle (CPU): its operator and the
PreSolve_2 DCT preconditioner, pinned by closed forms, and the batch inputs."""
import numpy as np

from drd_application_gb300 import abi
from drd_application_gb300.layout import cell_shape
from drd_application_gb300.workloads import make_c3_pressure, make_c3_solve
from oracle.oracle import Oracle


def test_pressure_operator_properties(oracle_build):
    P, bdr, b, _ = make_c3_pressure(1, 0, size=(64, 32))
    o = Oracle(P)
    rng = np.random.default_rng(0)
    x, y = rng.standard_normal(P.nr * P.nz), rng.standard_normal(P.nr * P.nz)
    Ax, Ay = o.pressure_matvec(bdr, x), o.pressure_matvec(bdr, y)
    assert abs(np.dot(Ax, y) - np.dot(x, Ay)) < 1e-9 * abs(np.dot(Ax, y))          # symmetric
    assert np.abs(o.pressure_matvec(bdr, np.ones_like(x))).max() < 1e-9            # constants: null space
    assert np.dot(x, Ax) < 0                                                        # negative semidefinite
    assert abs(Ax.sum()) < 1e-9 * np.abs(Ax).sum()                                  # range: zero-mean fields


def test_dct_preconditioner_inverts_constant_coefficient_operator(oracle_build):
    """With no solid (beta = 1) PreSolve_2's DCT solve is the exact inverse of the operator on
    zero-mean fields: M^-1 A x = x - mean(x)."""
    P = abi.default_params(48, 20)
    P.dt = 1e-3
    o = Oracle(P)
    x = np.random.default_rng(1).standard_normal(P.nr * P.nz)
    y = o.pressure_psolve(o.pressure_matvec(np.zeros(cell_shape(P.nr, P.nz)), x))
    assert np.abs(y - (x - x.mean())).max() < 1e-10 * np.abs(x).max()


def test_pressure_solve_oracle(oracle_build):
    P, bdr, b, _ = make_c3_pressure(2, 5, size=(64, 32), tol=1e-10)
    o = Oracle(P)
    x, st, info = o.pressure_solve(bdr, b)
    r = b - o.pressure_matvec(bdr, x)
    assert info == 0 and np.linalg.norm(r) / np.linalg.norm(b) < 1e-9
    assert abs(b.sum()) < 1e-10 * np.abs(b).sum()


def test_c3_inputs_unchanged_by_the_shared_mask_builder():
    """The momentum systems keep their seeded inputs: the mask and rhs of solve 3 of seed 0."""
    p, c, b, m = make_c3_solve(0, 3)
    assert (p.nr, p.nz) == (256, 128) and b.shape == (65408,)
    assert len(m["disks"]) in range(2, 7) and np.allclose(c["eta"], 1.0 + 99.0 * c["bdr_ph"])
