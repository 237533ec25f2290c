"""Shared helpers of the tests: packing in the reference's Atob orders, error measures and
states advanced by the oracle (so that operator and solve checks see non-trivial fields)."""
import numpy as np

from drd_application_gb300 import abi
from drd_application_gb300.workloads import make_case
from oracle.oracle import Oracle


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def pack_cell(a):
    """Atob (microfluidics_complex_domain/matrix_tool.f90:142-155) of a CELL array."""
    return np.ascontiguousarray(a[1:-1, 1:-1]).reshape(-1)


def pack_uv(u, v):
    """Atob_uv (matrix_tool.f90:5-26): u(0:nr,0:nz-1) then v(0:nr-1,1:nz-1)."""
    nz = u.shape[0] - 2
    nr = u.shape[1] - 3
    return np.concatenate([u[1:nz + 1, 1:nr + 2].reshape(-1), v[1:nz, 1:nr + 1].reshape(-1)])


def advanced_case(name="c2", seed=0, nr=48, nz=24, steps=2, **kw):
    """A workload advanced `steps` time steps by the oracle; returns (case, state, t)."""
    case = make_case(name, seed=seed, nr=nr, nz=nz, **kw)
    orc = Oracle(case.params)
    st = case.copy_state()
    t = 0.0
    for s in range(steps):
        orc.step(st, case.coefs, s == 0, t)
        t += case.params.dt
    return case, st, t


def solve_inputs(case, st):
    """Arguments the per-step routines read, taken from a resident state."""
    F = abi
    return dict(u=st[F.F_U], v=st[F.F_V], u_pre=st[F.F_U_PRE], v_pre=st[F.F_V_PRE], ph=st[F.F_PH], rmu=st[F.F_RMU],
                p=st[F.F_P], psi1=st[F.F_PSI1], psi2=st[F.F_PSI2], pf1=st[F.F_PF1], pf2=st[F.F_PF2])
