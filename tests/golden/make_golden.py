"""Generate the committed golden vectors of tests/golden/ from the FP64 CPU oracle.

    python tests/golden/make_golden.py

The reference publishes no outputs and cannot be built here (Fortran + prebuilt FFTW + MKL),
so these fixtures are produced by the oracle (oracle/drd_oracle.c) from seeded workloads
(drd_application_gb300.workloads) after the oracle itself was pinned against scipy's DCT
definitions and the reference's manufactured Poisson case (tests/test_oracle_pins.py).
They freeze the oracle's results so that the CUDA path and oracle builds on other machines
are checked against the same numbers.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from drd_application_gb300 import abi  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402
from tests.helpers import advanced_case  # noqa: E402

F = abi


def params_dict(P):
    return {k: np.array(v) for k, v in P.as_dict().items()}


def make_mf(path, seed=21, nr=24, nz=12):
    case, st, t = advanced_case("c2", seed=seed, nr=nr, nz=nz, steps=2)
    P = case.params
    orc = Oracle(P)
    k = case.coefs
    out = {"t": np.array(t)}
    for name, fid in (("u", F.F_U), ("v", F.F_V), ("u_pre", F.F_U_PRE), ("v_pre", F.F_V_PRE), ("ph", F.F_PH),
                      ("rmu", F.F_RMU), ("p", F.F_P), ("psi1", F.F_PSI1), ("psi2", F.F_PSI2)):
        out["in_" + name] = st[fid]
    for name in ("rho", "eta", "bdr_ph", "bdr_ph_grad", "M0", "Mi", "bdr_pen", "bdr_used"):
        out["coef_" + name] = k[name]
    r, p, s = orc.phsolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], k["bdr_ph"], k["bdr_ph_grad"], k["M0"], k["Mi"])
    out.update(ph_rmu_after=r, ph_ph_after=p, ph_iter=np.array(s.iter), ph_info=np.array(s.info))
    for bdf in (1, 2):
        u, v, uL, uR, s = orc.velosolve(bdf, st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE], st[F.F_U], st[F.F_V_PRE],
                                        st[F.F_V], st[F.F_P], k["rho"], k["eta"], k["bdr_ph"], k["bdr_pen"],
                                        k["bdr_used"], p, r, t + P.dt, st[F.F_PF1], st[F.F_PF2])
        out[f"uv{bdf}_u_after"], out[f"uv{bdf}_v_after"], out[f"uv{bdf}_uL"] = u, v, uL
        out[f"uv{bdf}_iter"] = np.array(s.iter)
    coef = 3 * P.re / 2.0 / P.dt
    out["pre_coef"] = np.array(coef)
    out["pre_psi"] = orc.presolve(st[F.F_U], st[F.F_V], coef)
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(P.nr * P.nz)
    out["op_x_ch"] = x
    out["op_ch_matvec"] = orc.ch_matvec(k["M0"], k["Mi"], x)
    out["op_ch_psolve"] = orc.ch_psolve(x)
    xu = rng.standard_normal((P.nr + 1) * P.nz + P.nr * (P.nz - 1))
    out["op_x_uv"] = xu
    out["op_uv_matvec2"] = orc.uv_matvec(2, k["rho"], k["eta"], k["bdr_pen"], xu)
    out["op_uv_psolve2"] = orc.uv_psolve(2, k["rho"], k["eta"], xu)
    out["mass"] = np.array(orc.mass(st[F.F_PH]))
    out.update({"param_" + kk: vv for kk, vv in params_dict(P).items()})
    np.savez_compressed(path, **out)


def make_tp(path, seed=22, nr=20, nz=16):
    case, st, t = advanced_case("tp", seed=seed, nr=nr, nz=nz, steps=2)
    P = case.params
    orc = Oracle(P)
    k = case.coefs
    ang = np.full(P.nr + 1, P.angle)
    out = {"t": np.array(t)}
    for name, fid in (("u", F.F_U), ("v", F.F_V), ("ph", F.F_PH), ("rmu", F.F_RMU)):
        out["in_" + name] = st[fid]
    for name in ("rho", "eta", "bdr_ph", "bdr_ph_grad", "M0", "Mi", "bdr_pen", "bdr_used"):
        out["coef_" + name] = k[name]
    ph_after, rmu_after, M0, cbt, s = orc.ph_mu_solve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], k["bdr_ph"],
                                                      k["bdr_used"], k["bdr_ph_grad"], k["Mi"], ang, ang)
    out.update(phmu_ph_after=ph_after, phmu_rmu_after=rmu_after, phmu_M0=M0, phmu_cbt=cbt, phmu_iter=np.array(s.iter))
    out.update({"param_" + kk: vv for kk, vv in params_dict(P).items()})
    np.savez_compressed(path, **out)


if __name__ == "__main__":
    make_mf(os.path.join(HERE, "mf_24x12.npz"))
    make_tp(os.path.join(HERE, "tp_20x16.npz"))
    print("golden fixtures written")
