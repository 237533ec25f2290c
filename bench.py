"""Benchmark of the GB300 per-time-step solver core.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: 420x180 complex-domain two-phase flow -- a seeded serpentine channel (sinusoidal
walls, amplitude 30 and period 140 cells, resistance penalty 1e4, walls smoothed by tanh over
2 cells), three rigid 40x4-cell fibers at seeded poses, two drops of radius 15 cells,
viscosity ratio 5, Re 0.5, Ca 0.05.  A step is one pass of the reference's time loop body
(CH solve -> momentum solve -> pressure solve -> p += psi), every Krylov solve to the deck
tolerance 1e-8 (relative FP64 residual).  Inputs are synthetic (seeded), as no dataset exists.

value: time-steps/s of the learned + mixed path (FP32 Krylov solves inside FP64 iterative
refinement; the CH preconditioner blended per cell by weights that a U-Net, trained before the
timed region on other seeded geometries, predicts from the mobility fields) with the state
resident in HBM, device-timed with CUDA events per step, L2 flushed between steps.  The plain
FP64 path (the reference's arithmetic, guess and preconditioner) is timed the same way and
reported beside it, with arms that split the ratio into its factors.  e2e: the same
metric through the drop-in C-ABI routines with host arrays (PhSolve, VeloSolve_2_combined,
PreSolve_2 each step, host<->device copies inside the timed region).

Multi-GPU: the path does not shard a grid; N ranks run N independent replicas (weak scaling)
and value = steps of all ranks / max elapsed over ranks.

--impl reference times the reference's algorithm on the host cores: the FP64 CPU
restatement (oracle/, OpenMP over transform lines), since the Fortran reference cannot be
built without a Fortran compiler, MKL and the prebuilt FFTW.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-steps/s and solves/s to FP64 resid 1e-8: learned+FP32 vs plain FP64, 1 GB300"
# DRAM bytes (read + write) of one launch of the persistent CH solve kernel, from an ncu capture
# of this workload (dram__bytes_read.sum + dram__bytes_write.sum of one launch)
TRAFFIC_CH = 4348160 + 304640
# the same for one launch of the persistent momentum solve kernel with the scaled ESOLP_x (the
# same capture)
TRAFFIC_UV = 8695808 + 1454592
# relative residual reduction of each FP32 inner solve in the mixed mode's FP64 refinement (every
# mixed leg of the GPU arm)
INNER_TOL = 0.1
WORKLOAD = ("420x180 serpentine channel (amp 30, period 140 cells, penalty 1e4), 3 rigid fibers 40x4, "
            "2 drops R=15, lambda_eta 5, Re 0.5, Ca 0.05; CH + momentum + pressure per step, tol 1e-8")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=None, help="timed steps of the plain FP64 path")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--c3-solves", type=int, default=512,
                    help="independent momentum and pressure systems of the C3 batch (0: skip)")
    ap.add_argument("--c5-steps", type=int, default=2,
                    help="steps of the 2048x1024 C5 comparison, mixed against FP64 (0: skip)")
    ap.add_argument("--learned-steps", type=int, default=600,
                    help="Adam steps of the learned CH guess leg (0: skip)")
    ap.add_argument("--blend-steps", type=int, default=800,
                    help="Adam steps of the blend network that drives the headline (0: PSolve_CG alone)")
    ap.add_argument("--blend-geometries", type=int, default=16, help="training geometries of the blend network")
    ap.add_argument("--nr", type=int, default=420)
    ap.add_argument("--nz", type=int, default=180)
    return ap.parse_args()


# ------------------------------------------------------------------------------ distributed
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, local):
    if ws <= 1:
        return None
    import torch
    import torch.distributed as dist

    dist.init_process_group("nccl", device_id=torch.device("cuda", 0))
    return dist


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples (clocks and throttle reasons) while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu, self.rows, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler is delivering (at most 5 s of waiting)
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for j, nm in enumerate(names):
                if len(r) > 4 + j and r[4 + j].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------ CPU baseline
def cpu_model():
    """The host CPU's model name (lscpu), or the machine type when lscpu has none."""
    import platform

    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.machine()


def cpu_baseline(steps=2, nr=420, nz=180):
    """The FP64 CPU restatement on the host cores, on a bounded sample of the same workload:
    one untimed step, then `steps` steps with OpenMP over the transform lines on every core
    (the reported value), then one step of the serial build on one core (the reference's own
    build is serial) beside it."""
    from oracle.oracle import Oracle
    from drd_application_gb300.workloads import make_case

    case = make_case("c2", seed=0, nr=nr, nz=nz)
    orc = Oracle(case.params, openmp=True)
    st = case.copy_state()
    dt = case.params.dt
    orc.step(st, case.coefs, True, 0.0)
    t = dt
    t0 = time.perf_counter()
    for s in range(steps):
        orc.step(st, case.coefs, False, t)
        t += dt
    elapsed = time.perf_counter() - t0
    t1 = time.perf_counter()
    Oracle(case.params, openmp=False).step(st, case.coefs, False, t)
    serial = time.perf_counter() - t1
    cores = os.cpu_count()
    return {"value": steps / elapsed, "unit": "time-steps/s", "cores": cores, "kind": "port", "cpu_model": cpu_model(),
            "single_thread": {"value": 1.0 / serial, "unit": "time-steps/s", "cores": 1,
                              "sample": f"step {steps + 2} of the same workload, serial FP64 oracle, {serial:.1f} s"},
            "sample": f"steps 2-{steps + 1} of the same {nr}x{nz} workload (step 1 untimed), FP64 oracle "
                      f"(oracle/drd_oracle.c, OpenMP over transform lines, {cores} threads), {elapsed:.1f} s"}


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    from oracle import oracle

    oracle.build()
    from drd_application_gb300.workloads import make_case
    from oracle.oracle import Oracle

    case = make_case("c2", seed=0, nr=args.nr, nz=args.nz)
    orc = Oracle(case.params, openmp=True)
    st = case.copy_state()
    t = 0.0
    # the requested warm-up steps, bounded to 60 s of host time; w is the number done
    w, t_w = 0, time.perf_counter()
    while w < args.warmup and time.perf_counter() - t_w < 60.0:
        orc.step(st, case.coefs, w == 0, t)
        t += case.params.dt
        w += 1
    timed, elapsed = 0, 0.0
    budget = 150.0
    for s in range(args.steps):
        t0 = time.perf_counter()
        orc.step(st, case.coefs, (w + s) == 0, t)
        elapsed += time.perf_counter() - t0
        t += case.params.dt
        timed += 1
        if elapsed > budget:
            break
    v = timed / elapsed
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "time-steps/s", "n_gpus": args.gpus,
        "steps": timed, "warmup": w, "ms_per_step": 1e3 * elapsed / timed, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nr": args.nr, "nz": args.nz,
                   "reference_code": "FP64 CPU restatement of the reference routines "
                                     "(Fortran reference not buildable: no Fortran compiler)"},
        "cpu_baseline": {"value": v, "unit": "time-steps/s", "cores": cores, "kind": "port", "cpu_model": cpu_model(),
                         "sample": f"{timed} timed steps after {w} warm-up, OpenMP over transform lines, {cores} threads"},
        "e2e": {"value": v, "unit": "time-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------------- GPU arm
def time_c5(steps, seed=0):
    """C5: the 2048x1024 workload (serpentine channel, 64 rigid fibers, 32 drops, viscosity ratio
    10 between the fluids), `steps` resident steps in the mixed mode (cubic guess) and in the plain
    FP64 mode (the reference's arithmetic and guess) from the same state: wall time per step,
    iterations and convergence of every solve, the phase-field mass drift per step and the
    velocity and phase fields of the mixed run against the FP64 run."""
    import numpy as np

    from drd_application_gb300 import abi
    from drd_application_gb300.api import DRDContext
    from drd_application_gb300.workloads import make_case

    out, fields = {}, {}
    J, ES = abi.DRD_UV_JACOBI, abi.DRD_UV_ESOLP_SCALED
    for name, prec, gm, pc, uvp in (("mixed", abi.DRD_PREC_MIXED, 3, None, J),
                                    ("mixed_probe_blend_esolp_scaled", abi.DRD_PREC_MIXED, 3, 64, ES),
                                    ("fp64", abi.DRD_PREC_FP64, 0, None, J)):
        case = make_case("c5", seed=seed, precision=prec, guess_mode=gm, uv_precond=uvp)
        ctx = DRDContext(case.params)
        ctx.set_case(case)
        fit_s = None
        if pc:  # this geometry's probe-fitted blend of the CH preconditioner (the network is per grid)
            t0 = time.perf_counter()
            ctx.ch_blend_probe(pc, 11, install=True)
            fit_s = time.perf_counter() - t0
        ctx.upload_state(case.state)
        m0 = ctx.mass(case.state[abi.F_PH])
        t, rows = 0.0, []
        for s_ in range(steps):
            rows.append(ctx.step(s_ == 0, t))
            t += case.params.dt
        g = ctx.download_state([abi.F_U, abi.F_V, abi.F_PH])
        fields[name] = g
        ctx.close()
        out[name] = {
            "ms_per_step": [1e3 * r.seconds for r in rows],
            "ch": [{"info": r.ch.info, "iter": r.ch.iter, "true_resid": r.ch.true_resid,
                    "fp64_fallback": bool(r.ch.flags & abi.DRD_FLAG_FALLBACK64)} for r in rows],
            "uv": [{"info": r.uv.info, "iter": r.uv.iter, "true_resid": r.uv.true_resid} for r in rows],
            "mass_drift_per_step": (rows[-1].mass - m0) / abs(m0) / steps,
        }
        if fit_s is not None:
            out[name]["probe_fit_s"] = fit_s
    rel = lambda a, b: float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))  # noqa: E731
    for name in ("mixed", "mixed_probe_blend_esolp_scaled"):
        out[name + "_vs_fp64"] = {"u": rel(fields[name][abi.F_U], fields["fp64"][abi.F_U]),
                                  "v": rel(fields[name][abi.F_V], fields["fp64"][abi.F_V]),
                                  "ph": rel(fields[name][abi.F_PH], fields["fp64"][abi.F_PH])}
    out["steps"] = steps
    out["workload"] = "c5 2048x1024: serpentine channel (amp 150, period 680), 64 fibers 60x6, 32 drops, lambda_eta 10"
    return out


def c3_systems(n_solves, seed):
    """The C3 batch: n_solves independent systems on grids drawn from five sizes, alternately the
    momentum operator of VeloSolve_2_combined (2 to 6 disks, eta = 1 + 99 mask) and the
    variable-coefficient pressure Poisson operator (beta = 1/(1 + penalty dt mask)), each with a
    Gaussian-random-field right-hand side."""
    from drd_application_gb300.workloads import make_c3_pressure, make_c3_solve

    systems = []
    for i in range(n_solves):
        if i % 2 == 0:
            P, c, b, _ = make_c3_solve(seed, i)
            systems.append(("uv", P, {"rho": c["rho"], "eta": c["eta"], "bdr_ph": c["bdr_ph"]}, b))
        else:
            P, bdr, b, _ = make_c3_pressure(seed, i)
            systems.append(("pressure", P, bdr, b))
    return systems


def time_c3(n_solves, seed, runs=3):
    """The C3 batch solved by ONE persistent launch under a CUDA graph (drd_batch_run): every
    system's coefficients and right-hand side are uploaded once at creation (which also tunes the
    launch shape and team sizes); each timed run solves all systems from a zero guess.  Device
    time by CUDA events; the roofline uses the algorithmic bytes of the run's iterations."""
    from drd_application_gb300.batch import Batch

    systems = c3_systems(n_solves, seed)
    t0 = time.perf_counter()
    bt = Batch(systems, autotune=True)
    create_s = time.perf_counter() - t0
    bt.run()  # warm-up
    secs = [bt.run() for _ in range(runs)]
    info = bt.info()
    st = [bt.status(i) for i in range(n_solves)]
    ok = sum(int(s.info == 0 and s.true_resid <= systems[i][1].tol) for i, s in enumerate(st))
    sec = statistics.median(secs)
    kinds = {}
    for (kind, P, *_), s in zip(systems, st):
        kinds.setdefault(kind, []).append(s.iter)
    bt.close()
    return {"solves": n_solves, "seconds": sec, "solves_per_s": n_solves / sec, "runs_s": secs,
            "launch": "one persistent cooperative launch in a CUDA graph",
            "threads_per_block": info["threads"], "blocks_per_sm": info["blocks_per_sm"],
            "create_and_tune_s": create_s, "achieved_GBps": info["bytes_last_run"] / secs[-1] / 1e9,
            "iters_mean": {k: statistics.mean(v) for k, v in kinds.items()},
            "systems": {k: len(v) for k, v in kinds.items()},
            "solves_to_fp64_1e-8": f"{ok}/{n_solves}",
            "sizes": sorted({f"{P.nr}x{P.nz}" for _, P, *_ in systems})}


def cpu_c3_sample(seed, n=4, budget_s=20.0):
    """The FP64 CPU restatement on the first systems of the same C3 batch (host cores, OpenMP
    over transform lines; Jacobi-preconditioned momentum, DCT-preconditioned pressure), up to
    budget_s."""
    from oracle.oracle import Oracle

    done, elapsed = 0, 0.0
    for kind, P, a, b in c3_systems(n, seed):
        orc = Oracle(P, openmp=True)
        t0 = time.perf_counter()
        if kind == "uv":
            orc.solve(1, 2, {"rho": a["rho"], "eta": a["eta"], "bdr_pen": a["bdr_ph"]}, b)
        else:
            orc.pressure_solve(a, b)
        elapsed += time.perf_counter() - t0
        done += 1
        if elapsed > budget_s:
            break
    return {"value": done / elapsed, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port", "cpu_model": cpu_model(),
            "sample": f"first {done} systems of the same C3 batch, FP64 oracle, {elapsed:.1f} s"}


def time_learned(steps, nr, nz, train_seeds=8, per_seed=12):
    """The learned CH guess beside the headline: the U-Net trained by the library's kernels on
    CH pairs from this workload's own runs (geometries 1000..), then evaluated on a held-out
    geometry (2000): mixed CH iterations to the FP64 residual 1e-8 from the plain guess x^n and
    from the learned one (taken unconditionally, and under the FP64-residual judge)."""
    import numpy as np

    from drd_application_gb300 import learned as LN
    from drd_application_gb300.workloads import make_case

    t0 = time.perf_counter()
    data = LN.concat_pairs([LN.ch_run_pairs(make_case("c2", seed=1000 + s, nr=nr, nz=nz), per_seed, warmup=10)
                            for s in range(train_seeds)])
    t1 = time.perf_counter()
    import torch

    net = LN.UNet(nz, nr, 3, 1, max_batch=8, seed=0)
    rng = np.random.default_rng(0)
    n = data["x"].shape[0]
    # the pairs stay in HBM; each step gathers its batch there (torch's stream, synchronised
    # before the network's own stream reads it)
    X, Y = torch.from_numpy(data["x"]).cuda(), torch.from_numpy(data["y"]).cuda()
    xb = torch.empty((8,) + tuple(X.shape[1:]), dtype=torch.float32, device="cuda")
    yb = torch.empty((8,) + tuple(Y.shape[1:]), dtype=torch.float32, device="cuda")

    def batch():
        idx = torch.from_numpy(rng.choice(n, size=8, replace=False)).cuda()
        torch.index_select(X, 0, idx, out=xb)
        torch.index_select(Y, 0, idx, out=yb)
        torch.cuda.synchronize()

    for k in range(3):  # warm-up at learning rate 0
        batch()
        net.train_step(xb, yb, 0.0)
    losses, step_s = [], []
    for k in range(steps):
        lr = 1e-3 * (5e-2) ** (k / max(steps - 1, 1))
        batch()
        a = time.perf_counter()
        losses.append(net.train_step(xb, yb, lr))
        step_s.append(time.perf_counter() - a)
    t2 = time.perf_counter()
    case = make_case("c2", seed=2000, nr=nr, nz=nz)
    pr = LN.ch_run_pairs(case, 6, warmup=10)
    y = np.concatenate([net.forward(np.ascontiguousarray(pr["x"][k:k + 1])) for k in range(6)])
    rel = np.sqrt(((y - pr["y"]) ** 2).sum(axis=(1, 2, 3)) / (pr["y"] ** 2).sum(axis=(1, 2, 3)))
    ev = {j: LN.evaluate_ch(case, net, pr, judge=j) for j in ("none", "residual")}
    net.close()
    med = statistics.median(step_s)
    fl = LN.conv_flops(-(-nz // 8) * 8, -(-nr // 8) * 8, 8)
    return {
        "network": "U-Net 4 levels, 32 base channels, 3x3, BF16 weights/activations, FP32 accumulate "
                   "(mma.sync m16n8k16 kernels)",
        "inputs": "residual of x^n / its RMS, bdr_ph, ph; target (x^(n+1) - x^n) / RMS",
        "train_pairs": n, "adam_steps": steps, "batch": 8,
        "train_step": "median wall time of one Adam step (forward, backward, update, loss read-back) on a batch "
                      "resident in HBM",
        "data_s": t1 - t0, "train_s": t2 - t1, "loss_first": float(np.mean(losses[:10])),
        "loss_last": float(np.mean(losses[-20:])),
        "train_step_ms": 1e3 * med, "conv_tflops": fl / med / 1e12,
        "held_out_error_ratio": float(rel.mean()),
        "iters_plain": float(ev["none"]["iters_plain"].mean()),
        "iters_learned": float(ev["none"]["iters_learned"].mean()),
        # wall time per solve through drd_solve with host arrays, and of building the learned
        # guess (residual, network, update) before it
        "solve_ms_plain": 1e3 * float(ev["none"]["t_plain"].mean()),
        "solve_ms_learned": 1e3 * float(ev["none"]["t_learned"].mean()),
        "guess_ms": 1e3 * float(ev["none"]["t_guess"].mean()),
        "iters_learned_residual_judge": float(ev["residual"]["iters_learned"].mean()),
        "learned_taken_residual_judge": f"{int(ev['residual']['used'].sum())}/{ev['residual']['used'].size}",
        "max_true_resid": float(max(ev["none"]["true_resid_learned"].max(), ev["none"]["true_resid_plain"].max())),
    }


def time_resident(ctx, case, warmup, steps, flush_bytes):
    """Per-step device time (CUDA events inside drd_step) with the state resident in HBM."""
    from drd_application_gb300 import abi

    ctx.upload_state(case.state)
    dt = case.params.dt
    t = 0.0
    for s in range(warmup):
        ctx.step(s == 0, t)
        t += dt
    ctx.synchronize()
    launches0 = ctx.kernel_launches()
    per, ch_it, uv_it, refine, resid, ok, ch_solve, ch_ref = [], [], [], [], [], 0, [], []
    uv_solve, uv_ref = [], []
    for s in range(steps):
        ctx.flush_l2(flush_bytes)
        ctx.synchronize()
        st = ctx.step(False, t)
        t += dt
        per.append(st.seconds)
        ch_solve.append(st.ch.seconds)
        ch_it.append(st.ch.iter)
        uv_it.append(st.uv.iter)
        refine.append(st.ch.refinements + st.uv.refinements)
        ch_ref.append(st.ch.refinements)
        uv_solve.append(st.uv.seconds)
        uv_ref.append(st.uv.refinements)
        resid.append(max(st.ch.true_resid, st.uv.true_resid))
        ok += int(st.ch.info == 0 and st.ch.true_resid <= case.params.tol * 1.0001) + \
            int(st.uv.info == 0 and st.uv.true_resid <= case.params.tol * 1.0001)
    launches = ctx.kernel_launches() - launches0
    del abi
    return {"seconds": sum(per), "per_step_ms": [1e3 * x for x in per], "ch_iters": ch_it, "uv_iters": uv_it,
            "refinements": refine, "max_true_resid": max(resid), "solves_ok": ok, "solves": 2 * steps,
            "launches": launches, "t_end": t, "ch_solve_s": ch_solve, "ch_refinements": ch_ref,
            "uv_solve_s": uv_solve, "uv_refinements": uv_ref}


def time_e2e(ctx, case, warmup, steps, flush_bytes):
    """The drop-in path: per-routine C-ABI calls with host arrays, mcl6 swaps on the host.  The
    host arrays are page-locked once (drd_host_register), as a driver that registers its module
    arrays at start-up would have them, and each call writes its outputs into page-locked arrays
    that no state entry holds (the ones the swaps freed)."""
    import numpy as np

    from drd_application_gb300 import abi
    from drd_application_gb300.api import pin, unpin

    P = case.params
    F = abi
    pinned = []

    def new(shape):
        a = np.zeros(shape)
        pin(a)
        pinned.append(a)
        return a

    st = {}
    for k, v in case.state.items():
        st[k] = new(v.shape)
        st[k][...] = v
    pool, taken = {}, []

    def take(shape):
        for a in pool.setdefault(shape, []):
            if not any(a is x for x in st.values()) and not any(a is x for x in taken):
                taken.append(a)
                return a
        a = new(shape)
        pool[shape].append(a)
        taken.append(a)
        return a

    cs, us, vs = st[F.F_PH].shape, st[F.F_U].shape, st[F.F_V].shape
    rho_o, eta_o, uL, uR = new(cs), new(cs), new((P.nz + 1,)), new((P.nz + 1,))
    gamma1 = min(1.0, P.lambda_rho)
    t = 0.0
    nb_cell = st[F.F_PH].nbytes
    nb_u = st[F.F_U].nbytes
    nb_v = st[F.F_V].nbytes
    h2d = (nb_u + nb_v + 2 * nb_cell) + (5 * nb_cell + 2 * nb_u + 2 * nb_v) + (nb_u + nb_v)
    d2h = (2 * nb_cell) + (nb_u + nb_v + 2 * 8 * (P.nz + 1)) + nb_cell
    if P.two_fluid:  # interpolate_coef's two-fluid rho, eta from ph each step: ph in, rho and eta out
        h2d += nb_cell
        d2h += 2 * nb_cell

    def one(first, t):
        taken.clear()
        rmu_after, ph_after, s1 = ctx.PhSolve(st[F.F_U], st[F.F_V], st[F.F_PH], st[F.F_RMU], t + P.dt,
                                              out=(take(cs), take(cs)))
        if P.two_fluid:
            ctx.two_phase_coef(None, st[F.F_PH], out=(rho_o, eta_o))
        if first:
            u_after, v_after, _, _, s2 = ctx.VeloSolve_combined(None, st[F.F_U], st[F.F_V], st[F.F_P], rmu_after,
                                                                ph_after, t + P.dt)
        else:
            u_after, v_after, _, _, s2 = ctx.VeloSolve_2_combined(st[F.F_PSI1], st[F.F_PSI2], st[F.F_U_PRE],
                                                                  st[F.F_U], st[F.F_V_PRE], st[F.F_V], st[F.F_P],
                                                                  st[F.F_PH_PRE], ph_after, st[F.F_RMU_PRE],
                                                                  rmu_after, t + P.dt,
                                                                  out=(take(us), take(vs), uL, uR))
        st[F.F_U_PRE], st[F.F_V_PRE] = st[F.F_U], st[F.F_V]
        st[F.F_U], st[F.F_V] = u_after, v_after
        st[F.F_PH_PRE], st[F.F_RMU_PRE] = st[F.F_PH], st[F.F_RMU]
        st[F.F_PH], st[F.F_RMU] = ph_after, rmu_after
        if first:
            coef = P.re * gamma1 / P.dt
        else:
            st[F.F_PSI1] = st[F.F_PSI2]
            coef = 3 * P.re * gamma1 / 2.0 / P.dt
        st[F.F_PSI2] = ctx.PreSolve_2(st[F.F_U], st[F.F_V], coef, out=take(cs))
        np.add(st[F.F_PSI2], st[F.F_P], out=st[F.F_P])
        return s1, s2

    try:
        for s in range(warmup):
            one(s == 0, t)
            t += P.dt
        total = 0.0
        for s in range(steps):
            ctx.flush_l2(flush_bytes)
            ctx.synchronize()
            t0 = time.perf_counter()
            one(False, t)
            total += time.perf_counter() - t0
            t += P.dt
    finally:
        for a in pinned:
            unpin(a)
    return {"seconds": total, "h2d": h2d, "d2h": d2h}


def run_gpu(args, ws, rank, local):
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import __graft_entry__

    __graft_entry__.build()
    dist = dist_init(ws, local)
    from drd_application_gb300 import abi
    from drd_application_gb300.api import DRDContext
    from drd_application_gb300.workloads import make_case

    flush = 512 << 20  # > 129 MB L2
    K, W = args.steps, max(3, args.warmup)
    K64 = args.fp64_steps if args.fp64_steps is not None else max(3, K // 4)
    # the mixed leg and the drop-in e2e leg (same context) start each solve from the cubic
    # extrapolation 4 x^n - 6 x^(n-1) + 4 x^(n-2) - x^(n-3) (guess_mode 3); the FP64 leg starts
    # from x^n as the reference does
    # the momentum solves of the headline and of the e2e leg use ESOLP_x (the reference's DCT /
    # tridiagonal momentum preconditioner, Precipitation_dynamics/ESOLP.f90) between the diagonal
    # scalings of the variable coefficients, in the persistent solver; the FP64 legs keep
    # VeloSolve_2_combined's Jacobi, and arms isolate each choice
    case = make_case("c2", seed=rank, nr=args.nr, nz=args.nz, precision=abi.DRD_PREC_MIXED, guess_mode=3,
                     uv_precond=abi.DRD_UV_ESOLP_SCALED, mixed_inner_tol=INNER_TOL)

    # the learned blend of the CH preconditioner: a U-Net trained, before any timed region, on
    # the probe fits of other seeded geometries (seeds 1000.., never a rank's own), then asked
    # for this geometry's weights in one forward pass
    blend_net, blend = None, None
    if args.blend_steps > 0:
        from drd_application_gb300.learned import learned_blend, train_blend

        train_cases = [make_case("c2", seed=1000 + g, nr=args.nr, nz=args.nz, precision=abi.DRD_PREC_MIXED,
                                 guess_mode=3) for g in range(args.blend_geometries)]
        blend_net, blend = train_blend(train_cases, steps=args.blend_steps, nprobe=64)
        del train_cases

    def install_blend(c, k):
        if blend_net is None:
            return None
        t0 = time.perf_counter()
        w = learned_blend(blend_net, k.coefs["M0"], k.coefs["Mi"])
        c.set_ch_blend(w)
        return time.perf_counter() - t0

    # learned + mixed (headline) path, resident state
    ctx = DRDContext(case.params)
    ctx.set_case(case)
    if blend is not None:
        blend["inference_and_install_s"] = install_blend(ctx, case)
    persist = ctx.persistent_solver()
    clocks = ClockSampler(int(local) if ws == 1 else 0)
    barrier(dist)
    clocks.start()
    wall0 = time.perf_counter()
    mx = time_resident(ctx, case, W, K, flush)
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    sec = max_over_ranks(dist, mx["seconds"])
    barrier(dist)

    # roofline of the dominant kernel, timed live (CUDA events, back-to-back launches)
    kb = {}
    for kid in (abi.DRD_KB_DCT_X_FP32, abi.DRD_KB_DCT_Z_FP32, abi.DRD_KB_UV_MATVEC_FP32, abi.DRD_KB_CH_MATVEC_FP32,
                abi.DRD_KB_DCT_X_FP64, abi.DRD_KB_UV_MATVEC_FP64):
        us, by, fl = ctx.kernel_bench(kid, reps=200)
        kb[kid] = (us, by, fl)

    # e2e through the drop-in C-ABI routines (host arrays)
    e2e = time_e2e(ctx, case, W, K, flush)
    e2e_sec = max_over_ranks(dist, e2e["seconds"])
    e2e_steps = K
    ctx.close()

    # the same mixed step with the fiber coupling of the reference loop (a 9-bead chain moved by
    # the flow, its forces spread onto the grid, rho/eta rebuilt every step) in place of the
    # rigid fibers: reported beside the headline, not part of it
    casep = make_case("c2", seed=rank, nr=args.nr, nz=args.nz, precision=abi.DRD_PREC_MIXED, guess_mode=3,
                      particles=True, uv_precond=abi.DRD_UV_ESOLP_SCALED, mixed_inner_tol=INNER_TOL)
    ctxp = DRDContext(casep.params)
    ctxp.set_case(casep)
    install_blend(ctxp, casep)
    parts = casep.meta["particles"]
    ctxp.particles_set(parts["pp"], parts["points"], parts["bdr_dist"])
    pt = time_resident(ctxp, casep, W, K, flush)
    pt_sec = max_over_ranks(dist, pt["seconds"])
    ctxp.close()

    # the C3 batch of independent momentum solves (reported beside the headline)
    c3 = time_c3(args.c3_solves, rank) if args.c3_solves > 0 else None
    if c3 is not None:
        c3["solves_per_s"] = args.c3_solves * ws / max_over_ranks(dist, c3["seconds"])
        c3["hbm_frac"] = c3["achieved_GBps"] / float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get(
            "hbm_gbs", 6800.0)) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
        if rank == 0 and not args.no_cpu:
            c3["cpu_baseline"] = cpu_c3_sample(rank)

    # the learned CH guess (rank 0 only: it is reported beside the headline)
    learned = time_learned(args.learned_steps, args.nr, args.nz) if (args.learned_steps > 0 and rank == 0) else None

    # C5 at 2048x1024, mixed against FP64 (rank 0 only, reported beside the headline)
    c5 = time_c5(args.c5_steps, rank) if (args.c5_steps > 0 and rank == 0) else None

    # plain FP64 path, resident state (--fp64-steps 0 skips it, e.g. for profiler runs), and the
    # arms that split mixed_over_fp64 into its factors on the same workload: FP64 with the cubic
    # guess (the guess), mixed with the cubic guess in the kernel-per-phase graph loop that the
    # FP64 path also uses (the arithmetic), and the headline's persistent solves (the launch
    # structure)
    f64, f64_sec, arms = None, None, {}
    if K64 > 0:
        case64 = make_case("c2", seed=rank, nr=args.nr, nz=args.nz, precision=abi.DRD_PREC_FP64)
        ctx64 = DRDContext(case64.params)
        ctx64.set_case(case64)
        f64 = time_resident(ctx64, case64, W, K64, flush)
        f64_sec = max_over_ranks(dist, f64["seconds"])
        ctx64.close()
        J, E, ES = abi.DRD_UV_JACOBI, abi.DRD_UV_ESOLP, abi.DRD_UV_ESOLP_SCALED
        legs = [("fp64_cubic", abi.DRD_PREC_FP64, None, K64, None, J),
                ("mixed_cubic_graph_loop", abi.DRD_PREC_MIXED, "0", K, None, J),
                ("mixed_cubic_persistent_psolve_cg", abi.DRD_PREC_MIXED, None, K, None, J)]
        if blend_net is not None:
            legs += [("mixed_cubic_persistent_learned_blend_jacobi", abi.DRD_PREC_MIXED, None, K, "learned", J),
                     ("mixed_cubic_persistent_learned_blend_esolp", abi.DRD_PREC_MIXED, None, K, "learned", E),
                     ("mixed_cubic_persistent_probe_blend_esolp_scaled", abi.DRD_PREC_MIXED, None, K, "probe", ES)]
        for name, prec, persist_env, nsteps, pc, uvp in legs:
            casea = make_case("c2", seed=rank, nr=args.nr, nz=args.nz, precision=prec, guess_mode=3, uv_precond=uvp,
                              **({"mixed_inner_tol": INNER_TOL} if prec == abi.DRD_PREC_MIXED else {}))
            if persist_env is not None:
                os.environ["DRD_PERSIST"] = persist_env
            try:
                ctxa = DRDContext(casea.params)
            finally:
                os.environ.pop("DRD_PERSIST", None)
            ctxa.set_case(casea)
            if pc == "probe":  # this geometry's own probe fit (64 probes) in place of the network's
                ctxa.ch_blend_probe(64, 7, install=True)
            elif pc == "learned":
                install_blend(ctxa, casea)
            ra = time_resident(ctxa, casea, W, nsteps, flush)
            ctxa.close()
            sa = max_over_ranks(dist, ra["seconds"])
            arms[name] = {"steps_per_s": nsteps * ws / sa, "ms_per_step": 1e3 * sa / nsteps, "steps": nsteps,
                          "ch_iters_mean": statistics.mean(ra["ch_iters"]),
                          "uv_iters_mean": statistics.mean(ra["uv_iters"]),
                          "solves_to_fp64_1e-8": f"{ra['solves_ok']}/{ra['solves']}"}
    if blend_net is not None:
        blend_net.close()

    if rank != 0:
        return 0
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    # the roofline line reports the persistent solve kernel with the larger share of the step
    # (each is one cooperative launch per step, timed by the CUDA events the step records around
    # it; the other is reported beside it).  Algorithmic bytes of one launch:
    # CH: 29 N_c FP32 words per BiCGSTAB iteration (the minimum of a fully fused iteration: 23
    #   vector passes, two mobility reads, one Ph_Lcc read), plus 4 N_c with the blend (the
    #   weights and the preconditioner's input, read once per preconditioner application), and per
    #   refinement sweep the FP64 residual (x, b, r and the two mobility fields) and the FP32 scale
    #   / FP64 update passes.
    # momentum with ESOLP_x: 36 n + 6 N_c FP32 words per iteration (n = nuv unknowns: the two
    #   preconditioner applications 9 n each -- input read and output written in each of the three
    #   phases, the three factor arrays read in the tridiagonal one; the two operators 2 n each plus
    #   rho, eta and the penalty at N_c each; the S pass 4 n; the X / R / P pass 10 n; 4 n more for
    #   the diagonal scalings of the scaled form), and per sweep the FP64 residual (x, b, r and the
    #   three coefficient fields) and the scale / update passes.
    nc = args.nr * args.nz
    cs = (args.nr + 2) * (args.nz + 2)
    nuv = (args.nr + 1) * args.nz + args.nr * (args.nz - 1)
    ch_words = 29.0 + (4.0 if blend_net is not None else 0.0)
    kernels = {
        "ch": {"name": "k_bicg_persist<CH> (whole mixed CH solve)", "traffic": TRAFFIC_CH,
               "iters": sum(mx["ch_iters"]), "sec": sum(mx["ch_solve_s"]), "launches": len(mx["ch_solve_s"]),
               "bytes": ch_words * nc * 4 * sum(mx["ch_iters"]) +
               sum(mx["ch_refinements"]) * (8.0 * (4 * nc + 2 * cs) + 4.0 * 4 * nc + 20.0 * nc)},
        "uv": {"name": "k_bicg_persist<UV> (whole mixed momentum solve)", "traffic": TRAFFIC_UV,
               "iters": sum(mx["uv_iters"]), "sec": sum(mx["uv_solve_s"]), "launches": len(mx["uv_solve_s"]),
               "bytes": (40.0 * nuv + 6.0 * nc) * 4 * sum(mx["uv_iters"]) +
               sum(mx["uv_refinements"]) * (8.0 * (3 * nuv + 3 * cs) + 4.0 * 3 * nuv + 20.0 * nuv)},
    }
    for kd in kernels.values():
        n_l = max(1, kd["launches"])
        kd["achieved"] = kd["bytes"] / kd["sec"] / 1e9 if kd["sec"] > 0 else 0.0
        kd["us"] = 1e6 * kd["sec"] / n_l
        kd["by"] = kd["bytes"] / n_l
        kd["ipl"] = kd["iters"] / n_l
    dom = "ch" if kernels["ch"]["sec"] >= kernels["uv"]["sec"] else "uv"
    other = "uv" if dom == "ch" else "ch"

    def roof(kd):
        return {"bound": "hbm", "kernel": kd["name"], "achieved": kd["achieved"], "peak": hbm_peak, "unit": "GB/s",
                "frac": kd["achieved"] / hbm_peak, "traffic": kd["traffic"], "bytes_per_launch": kd["by"],
                "us_per_launch": kd["us"], "iterations_per_launch": kd["ipl"],
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst)" if peaks else "fallback 6800 GB/s"}
    fl = None
    steps_total = K * ws
    value = steps_total / sec
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "time-steps/s",
        "n_gpus": ws,
        "steps": K,
        "warmup": W,
        "ms_per_step": 1e3 * sec / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded geometry, fibers and drops per rank)",
        "config": {
            "workload": WORKLOAD, "nr": args.nr, "nz": args.nz,
            "path": ("learned + mixed: FP32 BiCGSTAB in FP64 refinement, one persistent launch per solve; the CH "
                     "preconditioner PSolve_CG blended per cell, y = q + w (x - q), with weights w predicted by "
                     "the U-Net from the mobility fields (learned_blend); the momentum preconditioner ESOLP_x "
                     "between diagonal scalings; initial guesses by cubic extrapolation. The learned initial "
                     "guess is measured beside it (learned_guess) and does not drive the timed step")
            if blend_net is not None else
            "mixed + cubic guess: FP32 BiCGSTAB in FP64 refinement, PSolve_CG, initial guesses by cubic "
            "extrapolation",
            "learned_blend": blend,
            "initial_guess": "mixed and e2e legs: cubic extrapolation 4x^n - 6x^(n-1) + 4x^(n-2) - x^(n-3) (guess_mode 3); fp64 leg: x^n",
            "momentum_preconditioner": "mixed and e2e legs: ESOLP_x between the diagonal scalings sqrt(D0/D) "
                                       "(uv_precond 2); fp64 legs: Jacobi (PSolve_uv_2_CG)",
            "mixed_inner_tol": INNER_TOL,
            "inner_ch_solver": "persistent cooperative kernel" if persist[0] else
            f"kernel-per-phase graph loop ({persist[1] or 'persistent solver off'})",
            "parallelism": f"replicas x{ws}", "l2": "flushed between timed steps (512 MiB write)",
            "solves_per_s": 2 * steps_total / sec,
            "solves_to_fp64_1e-8": f"{mx['solves_ok']}/{mx['solves']}",
            "max_true_resid": mx["max_true_resid"],
            "ch_iters_mean": statistics.mean(mx["ch_iters"]), "uv_iters_mean": statistics.mean(mx["uv_iters"]),
            "refinements_mean": statistics.mean(mx["refinements"]),
            "wall_s_timed_region": wall,
            "fp64": None if f64 is None else {
                "steps_per_s": K64 * ws / f64_sec, "ms_per_step": 1e3 * f64_sec / K64, "steps": K64,
                "ch_iters_mean": statistics.mean(f64["ch_iters"]), "uv_iters_mean": statistics.mean(f64["uv_iters"]),
                "solves_to_fp64_1e-8": f"{f64['solves_ok']}/{f64['solves']}"},
            "mixed_over_fp64": None if f64 is None else (value / (K64 * ws / f64_sec)),
            "arms": arms,
            "mixed_over_fp64_factors": None if not arms else {
                "guess (fp64 x^n -> fp64 cubic)": arms["fp64_cubic"]["steps_per_s"] / (K64 * ws / f64_sec),
                "arithmetic (fp64 cubic -> mixed cubic, both graph loops)":
                    arms["mixed_cubic_graph_loop"]["steps_per_s"] / arms["fp64_cubic"]["steps_per_s"],
                "launch structure (graph loop -> persistent solves)":
                    arms["mixed_cubic_persistent_psolve_cg"]["steps_per_s"] / arms["mixed_cubic_graph_loop"]["steps_per_s"],
                **({"learned blend (PSolve_CG -> learned blend, persistent, Jacobi)":
                    arms["mixed_cubic_persistent_learned_blend_jacobi"]["steps_per_s"] /
                    arms["mixed_cubic_persistent_psolve_cg"]["steps_per_s"],
                    "momentum preconditioner (Jacobi -> ESOLP_x, persistent, learned blend)":
                    arms["mixed_cubic_persistent_learned_blend_esolp"]["steps_per_s"] /
                    arms["mixed_cubic_persistent_learned_blend_jacobi"]["steps_per_s"],
                    "variable-coefficient scaling (ESOLP_x -> scaled ESOLP_x)":
                    value / arms["mixed_cubic_persistent_learned_blend_esolp"]["steps_per_s"]}
                   if blend_net is not None else
                   {"momentum preconditioner (Jacobi -> scaled ESOLP_x, persistent)":
                    value / arms["mixed_cubic_persistent_psolve_cg"]["steps_per_s"]})},
            "kernels_us": {abi.KB_NAMES[k]: round(v[0], 3) for k, v in kb.items()},
            "with_particles": {"steps_per_s": K * ws / pt_sec, "ms_per_step": 1e3 * pt_sec / K, "beads": 9,
                               "solves_to_fp64_1e-8": f"{pt['solves_ok']}/{pt['solves']}"},
            "c3_batch": c3,
            "c5": c5,
            "learned_guess": learned,
        },
        "roofline": roof(kernels[dom]),
        "roofline_other_solve": roof(kernels[other]),
        "e2e": {"value": e2e_steps * ws / e2e_sec, "unit": "time-steps/s", "h2d_bytes_per_step": e2e["h2d"],
                "d2h_bytes_per_step": e2e["d2h"], "host_memory": "page-locked (drd_host_register)"},
        "clocks": clk,
        "gpu_launches": mx["launches"],
    }
    if not args.no_cpu and ws == 1:
        line["cpu_baseline"] = cpu_baseline(steps=2, nr=args.nr, nz=args.nz)
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
