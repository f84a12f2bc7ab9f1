"""Throughput benchmark of the GB300 MPM substep (MPM_Simulator_WARP.p2g2p).

Workload (default): the large sand column -- 1,048,576 sand particles,
128^3 grid (dx = 1/128), column [0.35,0.65]^2 x [0.05,0.85], Drucker-Prager
E = 2e5, nu = 0.3, friction 30 deg, density 2200, gravity (0,0,-9.8),
sticky floor + slip walls, dt = 5e-5.  Seeded synthetic particles (the
reference's sampling data is not available).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on rank 0.  A "step" is one substep of every particle.
  value  -- particle-substeps/s with the state resident in HBM, substeps
            replayed from a CUDA graph, timed with CUDA events (max over ranks)
  e2e    -- the same metric through the C ABI with host buffers: each step
            loads u, v, stress from pinned host memory (load_uvstress_from_tensor),
            runs the substep and reads u, v, F_disp, stress back to pinned host
            memory (export_uvFstress_from_warp)
  extra keys of the default line (skipped with --no-extras / --no-adjoint /
            --no-surrogate): metal_block_1m, reduced_1m, decoder_1m, batch_64,
            adjoint, surrogate -- each also runs alone with --workload
  --workload reduced_1m -- the reduced sampled-quadrature substep
            (p2g2p_reduced) on the same column with 4,096 sample points
  --workload decoder_1m -- the substep with the reference's stress decoder
            (NetDec) decoding every particle's stress first
  --impl reference -- the CPU restatement of the reference's algorithm (the
            reference is Python + Warp and cannot be installed here) on all
            host cores, on a bounded particle sample per step.
Multi-GPU: independent replicas, one per rank (the substep has no
cross-GPU exchange); value sums all ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALG_BYTES = {"sand": 284, "jelly": 284, "metal": 288}  # per particle-substep
METRIC = "particle-substeps/s (1M sand, fp32)"


def workload_config(sc, world: int) -> dict:
    return {"workload": f"{sc.name}: {sc.n_particles} particles, {sc.n_grid}^3 grid, dt {sc.dt}, "
                        f"{sc.material}, sticky floor + slip walls",
            "particles": sc.n_particles, "grid": sc.n_grid, "parallelism": f"replicas x{world}"}


KERNEL_BYTES = {"p2g": 116, "g2p": 192}  # algorithmic particle bytes per launch unit


def timing_label(K: int, gsize: int, repeats: int) -> str:
    """What the timed region ran, in words."""
    parts = []
    if K // gsize:
        parts.append(f"{K // gsize} replay(s) of a CUDA graph of {gsize} substeps")
    if K % gsize:
        parts.append(f"{K % gsize} eager substep(s)")
    return (f"{repeats} x {K} substeps ({' + '.join(parts)}), CUDA events on the launching stream, "
            "max over ranks")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="sand_column_1m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the forward+adjoint measurement")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the learned-stress measurement")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the metal, reduced, decoder and batched workloads in the default line")
    return ap.parse_args()


def _events_ms(fn, reps: int) -> float:
    """Mean milliseconds of fn() over reps calls, CUDA events on the current stream."""
    import torch

    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        fn()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def adjoint_extra(device) -> dict:
    """Differentiable rollout (131,072 sand particles, 96^3, 100 substeps, dt
    1e-4, v0 ~ N(0, 0.1^2)): forward time, forward + hand-written adjoint
    time (checkpoints every 10 substeps, grid tape), and the gradients of
    the MSE to a target rollout (E = 3e5, friction 35 deg) and of a linear
    functional of the final positions with respect to E, the friction angle
    and 16 random unit directions of v0 against central differences with
    relative step 1e-3.  The differences come from
    the committed fixture tests/golden/adjoint_fd_sand_rollout_131k.json
    (the same rollout restated in float64, with its float64 target): at this
    step the loss moves by about 1e-6 of itself, below what the float32
    forward resolves, so differences of the float32 forward (also reported)
    measure its rounding.  The forward uses the ordered P2G (deterministic
    sums), in both timings."""
    import json

    import numpy as np
    import torch

    from reduced_mpm_stress_training_gb300 import scenarios as S
    from reduced_mpm_stress_training_gb300.adjoint import SandRollout

    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden")
    with open(os.path.join(golden, "adjoint_fd_sand_rollout_131k.json")) as f:
        ref = json.load(f)
    sc = S.sand_rollout_131k()
    disp = np.load(os.path.join(golden, "adjoint_target_sand_rollout_131k.npz"))["displacement"]
    target = torch.from_numpy(sc.particles()[0].astype(np.float64) + disp.astype(np.float64)).to(device)
    sand = SandRollout(sc, checkpoint_every=10, device=device)
    v0 = sand.v0_default
    E, phi = sc.E, sc.friction_angle

    def fwd():
        sand.forward(v0, E, phi, keep=False)

    state = {}

    def fwd_adj():
        x = sand.positions(sand.forward(v0, E, phi, keep=True))
        state["g"] = sand.backward((2.0 * (x.double() - target) / x.numel()).float())

    fwd()
    fwd_adj()
    t_f = _events_ms(fwd, 3)
    t_fa = _events_ms(fwd_adj, 3)
    rng = np.random.default_rng(ref["direction_seed"])
    dirs = rng.standard_normal((ref["n_directions"], sc.n_particles, 3))
    dirs /= np.linalg.norm(dirs.reshape(ref["n_directions"], -1), axis=1)[:, None, None]

    def directional(v0b, Eb, phib):
        g = v0b.double().cpu().numpy()
        out = {"E": float(Eb), "friction_angle": float(phib)}
        for k in range(ref["n_directions"]):
            out[f"v0_direction_{k}"] = float((g * dirs[k]).sum())
        return out

    got = directional(*state["g"])
    checks = {k: (got[k], f) for k, f in ref["fd"].items()}
    # the adjoint itself: a linear functional of the final positions, whose
    # gradient does not pass through the MSE's small residual
    w = np.random.default_rng(ref["linear_seed"]).standard_normal((sc.n_particles, 3))
    sand.forward(v0, E, phi, keep=True)
    got_lin = directional(*sand.backward(torch.from_numpy(w / w.size).to(device, torch.float32)))
    lin = {k: (got_lin[k], f) for k, f in ref["fd_linear"].items()}

    def J(v, e_, p_):
        x = sand.positions(sand.forward(v, e_, p_, keep=False))
        return float(((x.double() - target) ** 2).mean())

    rh = float(ref["relative_step"])
    f32 = {"E": (J(v0, E * (1 + rh), phi) - J(v0, E * (1 - rh), phi)) / (2 * rh * E),
           "friction_angle": (J(v0, E, phi * (1 + rh)) - J(v0, E, phi * (1 - rh))) / (2 * rh * phi)}
    h = rh * v0.norm().item()
    for k in range(ref["n_directions"]):
        d = torch.from_numpy(dirs[k]).to(device, torch.float32)
        f32[f"v0_direction_{k}"] = (J(v0 + h * d, E, phi) - J(v0 - h * d, E, phi)) / (2 * h)
    return {"workload": f"sand_rollout_131k: {sc.n_particles} particles, {sc.n_grid}^3 grid, "
                        f"{sc.substeps} substeps, dt {sc.dt}, checkpoints every 10",
            "forward_p2g": "ordered (mpm_p2g_ordered: deterministic sums)" if sand.engine.ordered else "atomic",
            "forward_ms": round(t_f, 3), "forward_adjoint_ms": round(t_fa, 3),
            "ratio": round(t_fa / t_f, 3),
            "fd_relative_step": rh,
            "fd_forward": ref["forward"],
            "gradient_vs_fd_linear_functional": {k: {"adjoint": a, "fd": f, "rel_err": abs(a - f) / abs(f)}
                                                 for k, (a, f) in lin.items()},
            "max_rel_err_linear_functional": max(abs(a - f) / abs(f) for a, f in lin.values()),
            "gradient_vs_fd": {k: {"adjoint": a, "fd": f, "rel_err": abs(a - f) / abs(f)}
                               for k, (a, f) in checks.items()},
            "max_rel_err": max(abs(a - f) / abs(f) for a, f in checks.values()),
            "mse_note": "float32 rollouts end 1.8e-7 RMS from the float64 rollout against an 8.3e-6 RMS "
                        "MSE residual (2 %), which bounds any float32 gradient of the MSE loss",
            "float32_forward_fd_max_rel_err": max(abs(got[k] - f) / abs(f) for k, f in f32.items())}


def surrogate_extra(device) -> dict:
    """Learned stress: the network trained by the library's kernels (8M
    tuples, Adam lr 1e-3, batch 65,536, 60,000 steps), then the 1M sand
    column substep with the surrogate stress stage against the plain
    return-map substep, from the same state after 2,000 plain substeps."""
    import torch

    from reduced_mpm_stress_training_gb300 import _capi as A
    from reduced_mpm_stress_training_gb300 import scenarios as S
    from reduced_mpm_stress_training_gb300 import surrogate as SU

    t0 = time.perf_counter()
    roll = SU.rollout_F_trial(S.sand_column_32k(), 600, 60, device=device)
    x, y = SU.build_training_set(8_000_000, device=device, seed=0, rollout=roll)
    net = SU.StressMLP(device, seed=0)
    t1 = time.perf_counter()
    log = SU.train(net, x, y, steps=60000, batch=65536, lr=1e-3, lr_min=1e-5, log_every=20000)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    del x, y
    sc = S.sand_column_1m()
    sim = S.build_simulator(sc, device=device)
    eng = sim.engine
    for k in range(2):
        sim.p2g2p(k, sc.dt)
    g = eng.graph(200, 0.0, sc.dt)
    for _ in range(10):
        g.replay()
    torch.cuda.synchronize()
    snap = eng.snapshot()
    eng.restore(snap)
    eng.substep_raw(0.0, sc.dt)
    tau_plain = eng.export(A.FIELD_STRESS).reshape(-1, 9).clone()
    sur = SU.StressSurrogate(net)
    eng.set_stress_surrogate(sur)
    eng.restore(snap)
    eng.substep_raw(0.0, sc.dt)
    tau_sur = eng.export(A.FIELD_STRESS).reshape(-1, 9).clone()
    counts = sur.outcome_counts()
    err = SU.stress_errors(tau_sur, tau_plain)

    def timed(surrogate):
        eng.set_stress_surrogate(surrogate)
        eng.restore(snap)
        eng.substep_raw(0.0, sc.dt)
        gg = eng.graph(20, 0.0, sc.dt)
        gg.replay()
        return _events_ms(gg.replay, 3) / 20

    t_sur = timed(sur)
    t_plain = timed(None)
    n = sc.n_particles
    acc = counts["elastic"] + counts["plastic"]
    return {"workload": "sand_column_1m after 2,002 plain substeps (settling column)",
            "plain_step_ms": round(t_plain, 4), "surrogate_step_ms": round(t_sur, 4),
            "surrogate_over_plain": round(t_sur / t_plain, 3),
            "stress_rel_l2_vs_plain": err["rel_l2"],
            "accepted_fraction": acc / n, "outcomes": counts,
            "training": {"tuples": 8_000_000, "steps": 60000, "batch": 65536, "seconds": round(t_train, 1),
                         "data_seconds": round(t1 - t0, 1), "loss": log[-1][1],
                         "kernels": "tcgen05 forward and backward (tensor-memory accumulators), Adam",
                         # forward 2 (12*128 + 2*128*128 + 128*6) flop per row, the backward twice that
                         "tflops": round(3 * 2.0 * (12 * 128 + 2 * 128 * 128 + 128 * 6) * 65536 * 60000
                                         / t_train / 1e12, 1),
                         "peak_tflops": measured_peak_bf16()}}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value: float, world: int, device) -> float:
    """Max of a host float over all ranks (identity for one rank)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int, device=None):
    if world > 1:
        import torch.distributed as dist

        if device is not None and device.type == "cuda":
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, copy)"
    except Exception:
        return 6800.0, "fallback (6.8 TB/s)"


def measured_peak_bf16():
    """Dense bf16 TFLOP/s: the burst figure (a kernel timed alone) and the
    sustained one (a kernel inside a long loop), from MEASURED_PEAKS.json."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return {"burst": float(d["bf16_tflops"]), "sustained": float(d["bf16_tflops_sustained"]),
                "source": "measured (MEASURED_PEAKS.json, cuBLAS bf16)"}
    except Exception:
        return {"burst": 1900.0, "sustained": 1700.0, "source": "fallback"}


def profiled_traffic(workload: str):
    """Per-substep DRAM bytes from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"dram_traffic_{workload}.json")
    try:
        return json.load(open(p))
    except Exception:
        return None


# ---------------------------------------------------------------------------
def cpu_port_rate(sc, n_sample: int, min_seconds: float, max_steps: int, steps: int | None = None):
    """Particle-substeps/s of the CPU restatement (all host threads) on the
    first n_sample particles of the scene's seeded set."""
    from oracle import oracle as O

    x0, v0, vol, mass = sc.particles()
    x0, v0, vol, mass = (a[:n_sample].copy() for a in (x0, v0, vol, mass))
    m = O.make_model(sc.n_grid, sc.grid_lim, material=sc.material, E=sc.E, nu=sc.nu,
                     friction_angle=sc.friction_angle, gravity=sc.gravity)
    cols = [O.surface_collider(**kw) if k == "surface" else O.bounding_box(**kw)
            for k, kw in sc.colliders()]
    sim = O.OracleSim(m, x0, mass, vol, v0, bits=32, colliders=cols,
                      yield_stress=sc.yield_stress if sc.material == "metal" else None)
    nt = O.max_threads()
    sim.p2g2p(sc.dt, nthreads_p2g=nt)  # warm
    done, t0 = 0, time.perf_counter()
    while True:
        sim.p2g2p(sc.dt, nthreads_p2g=nt)
        done += 1
        el = time.perf_counter() - t0
        if steps is not None:
            if done >= steps:
                break
        elif (el >= min_seconds and done >= 2) or done >= max_steps:
            break
    return n_sample * done / el, nt, done, el


def reference_arm(args, sc, world, rank):
    if rank != 0:
        return
    # bound the per-step sample so K steps end within about two minutes
    from oracle import oracle as O  # noqa: F401

    probe = 65536
    rate, nt, _, _ = cpu_port_rate(sc, probe, 0.0, 2, steps=2)
    per_step_budget = 120.0 / max(1, args.steps + args.warmup)
    n_sample = int(max(4096, min(sc.n_particles, rate * per_step_budget)))
    n_sample = 1 << int(math.log2(n_sample))
    rate, nt, done, el = cpu_port_rate(sc, n_sample, 0.0, 0, steps=args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate,
        "unit": "particle-substeps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / done, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(sc, args.gpus),
        "l2": "not applicable (host cores)",
        "timing": {"method": f"{args.steps} substeps of the bounded sample, wall clock (perf_counter)",
                   "repeats": 1, "substeps_timed": done, "timed_region_s": round(el, 4)},
        "cpu_baseline": {"value": rate, "unit": "particle-substeps/s", "cores": nt, "kind": "port",
                         "sample": f"first {n_sample} particles of the seeded {sc.n_particles}-particle "
                                   f"column on the {sc.n_grid}^3 grid, one substep per step "
                                   "(C restatement of the reference's Warp kernels, float32, OpenMP)"},
        "e2e": {"value": rate, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "reference is Python + NVIDIA Warp; warp-lang is not installable offline, "
                "so the reference arm times the project's C restatement of its algorithm",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def gb300_arm(args, sc, world, rank, local):
    import torch

    from reduced_mpm_stress_training_gb300 import _capi as A
    from reduced_mpm_stress_training_gb300.scenarios import build_simulator

    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    sim = build_simulator(sc, device=device)
    eng = sim._engine
    n = sc.n_particles
    dt = sc.dt
    W = max(3, args.warmup)
    for k in range(W):
        sim.p2g2p(k, dt)
    torch.cuda.synchronize()
    sim.check_status()

    K = args.steps
    gsize = max(1, min(32, K))
    graph = eng.graph(gsize, float(sim.time), dt)
    graph.replay()  # untimed: the first replay uploads the graph
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()

    def k_substeps():
        # exactly K substeps: K // gsize graph replays, the remainder eagerly
        for _ in range(K // gsize):
            graph.replay()
        for _ in range(K % gsize):
            eng.substep_raw(float(sim.time), dt)

    # the timed region repeats the K-substep block R times so it lasts at least
    # half a second (the clock sampler then sees several samples under load)
    t_block = _events_ms(k_substeps, 1) / 1e3
    repeats = max(1, min(1000, math.ceil(0.5 / max(t_block, 1e-6))))
    repeats = int(max_over_ranks(float(repeats), world, device))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(device.index if world == 1 else local)
    barrier(world, device)
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(st)
    for _ in range(repeats):
        k_substeps()
    ev1.record(st)
    torch.cuda.synchronize()
    barrier(world, device)
    clk = clocks.stop()
    t = ev0.elapsed_time(ev1) / 1e3
    t_max = max_over_ranks(t, world, device)
    status = eng.status()
    launches_per_substep = 6  # scan_tiles, scan_finish, scatter, p2g, grid, g2p
    timed_substeps = repeats * K
    value = world * n * timed_substeps / t_max
    ms_per_step = 1e3 * t_max / timed_substeps

    # per-stage times, eager, CUDA events on the launching stream
    stage_ms = {"sort": 0.0, "p2g": 0.0, "grid": 0.0, "g2p": 0.0}
    reps = 32
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    for k in range(reps):
        evs[0].record(st)
        eng.stage("sort")
        evs[1].record(st)
        eng.stage("p2g", dt=dt)
        evs[2].record(st)
        eng.stage("grid", time=float(sim.time), dt=dt)
        evs[3].record(st)
        eng.stage("g2p", dt=dt)
        evs[4].record(st)
        torch.cuda.synchronize()
        for i, kname in enumerate(stage_ms):
            stage_ms[kname] += evs[i].elapsed_time(evs[i + 1]) / reps

    # end to end through the C ABI with pinned host buffers
    hu = torch.empty(n * 3, dtype=torch.float32).pin_memory()
    hv = torch.empty(n * 3, dtype=torch.float32).pin_memory()
    hs = torch.empty(n * 9, dtype=torch.float32).pin_memory()
    eng.export(A.FIELD_U, hu)
    eng.export(A.FIELD_V, hv)
    eng.export(A.FIELD_STRESS, hs)
    outs = tuple(torch.empty(n * c, dtype=torch.float32).pin_memory() for c in (3, 3, 9, 9))
    k_e2e = max(3, min(K, 100))

    def e2e_step():
        # load_uvstress_from_tensor, p2g2p, export_uvFstress_from_warp through the C ABI;
        # the output copy is left in flight (the next step's input copy overlaps it) and
        # the timed region ends with a synchronize, after the last step's copy landed
        eng.load_uvstress(hu, hv, hs)
        eng.substep_raw(float(sim.time), dt)
        eng.export_uvFstress(outs, wait=False)

    for _ in range(3):
        e2e_step()
    torch.cuda.synchronize()
    barrier(world, device)
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        e2e_step()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world, device)
    e2e_value = world * n * k_e2e / t_e2e
    status |= eng.status()

    if rank != 0:
        return
    peak, peak_src = measured_peak_hbm()
    alg = ALG_BYTES[sc.material]
    achieved = alg * n / (t_max / timed_substeps) / 1e9
    traffic = profiled_traffic(sc.name)
    kern = {}
    for kname, b in KERNEL_BYTES.items():
        ms = stage_ms[kname]
        gbs = b * n / (ms * 1e-3) / 1e9
        kern[kname] = {"ms": round(ms, 4), "algorithmic_bytes": b * n, "achieved_gbs": round(gbs, 1),
                       "frac": round(gbs / peak, 4)}
    for kname in ("sort", "grid"):
        kern[kname] = {"ms": round(stage_ms[kname], 4)}
    line = {
        "metric": METRIC, "value": value,
        "unit": "particle-substeps/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform particles in the column; reference sampling data absent)",
        "config": workload_config(sc, world),
        "l2": "state larger than L2 (2 x %.0f MB particle buffers + grid); no flush" % (eng.plan.state_bytes / 1e6),
        "timing": {"method": timing_label(K, gsize, repeats), "repeats": repeats,
                   "substeps_timed": timed_substeps, "timed_region_s": round(t_max, 4)},
        "roofline": {"bound": "hbm", "kernel": "substep (sort + p2g + grid + g2p)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": None if traffic is None else traffic.get("bytes_per_substep"),
                     "traffic_source": None if traffic is None else
                     "profiles/dram_traffic_%s.json (ncu dram__bytes_read+write, one substep)" % sc.name,
                     "algorithmic_bytes_per_unit": alg, "unit_count": n, "peak_source": peak_src},
        "roofline_kernels": kern,
        "e2e": {"value": e2e_value, "unit": "particle-substeps/s", "h2d_bytes_per_step": 60 * n,
                "d2h_bytes_per_step": 96 * n, "steps": k_e2e},
        "gpu_launches": int(round(timed_substeps * launches_per_substep)),
        "clocks": clk,
        "status": status,
    }
    if world == 1 and not args.no_extras:
        # the other workloads, recorded in the same line; one failing keeps the headline
        for key, fn in (("metal_block_1m", metal_result), ("reduced_1m", reduced_result),
                        ("decoder_1m", decoder_result), ("batch_64", batched_result)):
            try:
                line[key] = fn(args, device)
            except Exception as exc:  # noqa: BLE001
                line[key] = {"error": repr(exc)}
    if not args.no_adjoint:
        line["adjoint"] = adjoint_extra(device)
    if not args.no_surrogate:
        line["surrogate"] = surrogate_extra(device)
    if not args.no_cpu_baseline:
        rate, nt, done, el = cpu_port_rate(sc, sc.n_particles, 10.0, 30)
        line["cpu_baseline"] = {"value": rate, "unit": "particle-substeps/s", "cores": nt,
                                "kind": "port",
                                "sample": f"{done} substeps of the full {sc.n_particles}-particle "
                                          f"column ({el:.1f} s), C restatement (float32, OpenMP)"}
    print(json.dumps(line), flush=True)


def metal_result(args, device) -> dict:
    """The von Mises metal block variant of the large column: 1,048,576 particles,
    128^3 grid, E = 1e7, yield stress 1e5, density 2700, v0 = (0, 0, -1), dt 5e-5;
    substeps replayed from a CUDA graph (CUDA events) after a warm-up."""
    import torch

    from reduced_mpm_stress_training_gb300 import scenarios as S

    sc = S.metal_block_1m()
    sim = S.build_simulator(sc, device=device)
    eng = sim.engine
    for k in range(max(3, args.warmup)):
        sim.p2g2p(k, sc.dt)
    sim.check_status()
    gsize = 32
    graph = eng.graph(gsize, float(sim.time), sc.dt)
    graph.replay()
    reps = 8
    t = _events_ms(graph.replay, reps) / 1e3 / gsize
    n = sc.n_particles
    peak, peak_src = measured_peak_hbm()
    achieved = ALG_BYTES["metal"] * n / t / 1e9
    return {"metric": "particle-substeps/s (1M von Mises metal, fp32)", "value": n / t,
            "unit": "particle-substeps/s", "ms_per_step": 1e3 * t, "steps": reps * gsize,
            "timing": f"{reps} replays of a CUDA graph of {gsize} substeps, CUDA events",
            "config": workload_config(sc, 1),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "algorithmic_bytes_per_unit": ALG_BYTES["metal"],
                         "peak_source": peak_src},
            "status": eng.status()}


def batched_result(args, device) -> dict:
    """64 scenes (sand and metal, N log-uniform in [1e4, 2e5], grids 48/64/96) in one
    batched launch per stage, replayed from a CUDA graph, over the workload's full 500
    substeps (warm-up and graph upload included), against the same scenes stepped one
    by one.  The status word and the finiteness of every scene are checked at the end."""
    import torch

    from reduced_mpm_stress_training_gb300 import _capi as A
    from reduced_mpm_stress_training_gb300 import scenarios as S
    from reduced_mpm_stress_training_gb300.batched import BatchedMPM, time_chunk_size

    scenes = S.batch_64()
    b = BatchedMPM(scenes, device=device, chunk_size="auto")
    dt = scenes[0].dt
    total = scenes[0].substeps
    W = max(3, args.warmup)
    for _ in range(W):
        b.step(dt)
    gsize = 32
    graph = b.graph(gsize, dt)
    graph.replay()
    torch.cuda.synchronize()
    done = W + gsize
    K = (total - done) // gsize * gsize
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(K // gsize):
        graph.replay()
    e1.record(st)
    torch.cuda.synchronize()
    done += K
    for _ in range(total - done):
        b.step(dt)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / K
    finite = bool(torch.isfinite(b.engine.export(A.FIELD_U)).all()) and bool(
        torch.isfinite(b.engine.export(A.FIELD_STRESS)).all())
    seq = sum(time_chunk_size([s], b.chunk_size, device, steps=16) for s in scenes)
    n = b.n_particles
    return {"metric": "particle-substeps/s (64-scene batch, fp32)", "value": n / t,
            "unit": "particle-substeps/s", "steps": K, "warmup": W, "ms_per_step": 1e3 * t,
            "substeps_run": total, "timing": f"{K // gsize} replays of a CUDA graph of {gsize} substeps of all "
                                              "64 scenes, CUDA events",
            "config": {"workload": "batch_64: 64 scenes, N log-uniform [1e4, 2e5], grids 48/64/96, 25 % metal "
                                   "(E log-uniform [1e5, 1e6]), dt 1e-4, 500 substeps",
                       "scenes": len(scenes), "particles": n, "chunk_size": b.chunk_size},
            "one_by_one": {"value": n / seq, "ms_per_step": 1e3 * seq},
            "speedup_vs_one_by_one": seq / t, "status": b.engine.status(), "finite_after_500": finite}


def batched_arm(args):
    import torch

    import __graft_entry__ as g

    g.build()
    d = batched_result(args, torch.device("cuda:0"))
    d.update(n_gpus=1, higher_is_better=True, dtype="f32", data="synthetic")
    print(json.dumps(d), flush=True)


def reduced_result(args, device) -> dict:
    """The reduced sampled-quadrature substep (MPM_Simulator_WARP.p2g2p_reduced) on the
    large sand column after two plain substeps, with 4,096 seeded sample points:
    every particle is scanned, the marked ones scatter, and the dense 128^3 grid is
    written.  Substeps are replayed from a CUDA graph and timed with CUDA events."""
    import ctypes as C

    import numpy as np
    import torch

    from reduced_mpm_stress_training_gb300 import MPM_Simulator_WARP
    from reduced_mpm_stress_training_gb300 import _capi as A
    from reduced_mpm_stress_training_gb300 import scenarios as S

    sc = S.sand_column_1m()
    n, ng, dt = sc.n_particles, sc.n_grid, sc.dt
    x0, v0, vol, mass = sc.particles()
    sim = MPM_Simulator_WARP(n, n_grid=ng, grid_lim=sc.grid_lim, device=device)
    sim.set_parameters(material=sc.material, E=sc.E, nu=sc.nu, friction_angle=sc.friction_angle,
                       gravity=sc.gravity)
    sim.load_x_initial_from_tensor(torch.from_numpy(x0))
    sim.load_vol_from_tensor(torch.from_numpy(vol))
    sim.set_parameters(density=sc.density)
    sim.load_v_from_tensor(torch.from_numpy(v0))
    for kind, kw in sc.colliders():
        sim.add_surface_collider(**kw) if kind == "surface" else sim.add_bounding_box(**kw)
    for k in range(2):
        sim.p2g2p(k, dt)
    n_samples = 4096
    sample = np.random.default_rng(0).choice(n, n_samples, replace=False).astype(np.int32)
    sim.load_sample_particle_index_from_tensor(torch.from_numpy(sample))
    for k in range(max(3, args.warmup)):
        sim.p2g2p_reduced(k, dt)
    sim.check_status()
    rg = sim._reduced_grid()
    rg.f_disp = sim._f_disp_state()
    gs = rg.struct(sim.engine)
    lib, buf = A.load(), sim.engine.buf
    gsize = 16
    graph, side = torch.cuda.CUDAGraph(), torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        hs = torch.cuda.current_stream().cuda_stream
        for _ in range(gsize):  # time and moving colliders are fixed: the scene has none that move
            A.check(lib.mpm_p2g2p_reduced(C.byref(buf), C.byref(gs), float(sim.time), dt, hs),
                    "mpm_p2g2p_reduced")
    graph.replay()
    torch.cuda.synchronize()
    K = max(gsize, min(args.steps, 2000) // gsize * gsize)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(K // gsize):
        graph.replay()
    e1.record(st)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / K
    # algorithmic bytes of one reduced substep: every particle's x_initial, u and the mark
    # of its base cell (28 B); a marked particle's F_disp, density, v, mass read and F
    # written (92 B); every node's scratch cleared and read, both marks cleared, the mark
    # read, grid_m, grid_v_in, grid_v_out written (76 B)
    x = sim.engine.export(A.FIELD_X).reshape(n, 3)
    base = torch.trunc(x * np.float32(ng) - 0.5).long()
    marked = int((rg.neighboring_cells[base[:, 0], base[:, 1], base[:, 2]] > 0).sum())
    alg = 28 * n + 92 * marked + 76 * ng ** 3
    peak, peak_src = measured_peak_hbm()
    achieved = alg / t / 1e9
    # CPU restatement of the same step (single-threaded), one substep on the same state
    from oracle import oracle as O

    m = O.make_model(ng, sc.grid_lim, material=sc.material, E=sc.E, nu=sc.nu,
                     friction_angle=sc.friction_angle, gravity=sc.gravity)
    cols = [O.surface_collider(**kw) if k == "surface" else O.bounding_box(**kw) for k, kw in sc.colliders()]
    ref = O.OracleSim(m, x0, mass, vol, v0, bits=32, colliders=cols)
    ref.u[:] = sim.engine.export(A.FIELD_U).reshape(n, 3).cpu().numpy()
    ref.v[:] = sim.engine.export(A.FIELD_V).reshape(n, 3).cpu().numpy()
    ref.F_disp[:] = rg.f_disp.reshape(n, 9).cpu().numpy()
    ref.density[:] = sc.density
    ref.sample_particle_index_short = sample
    nt = O.max_threads()
    t0 = time.perf_counter()
    ref.p2g2p_reduced(dt, nthreads_p2g=nt)
    cpu_t = time.perf_counter() - t0
    return {
        "metric": "particle-substeps/s (reduced sampled-quadrature substep, 1M sand, 4096 samples, fp32)",
        "value": n / t, "unit": "particle-substeps/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"sand_column_1m after 2 substeps: {n} particles, {ng}^3 grid, "
                               f"{n_samples} sample points, p2g2p_reduced",
                   "marked_particles": marked, "marked_cells": int(rg.neighboring_cells.sum()),
                   "l2": "inputs and dense grids larger than L2"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src, "scope": "whole substep",
                     "alg_bytes_per_step": alg},
        "cpu_baseline": {"value": n / cpu_t, "unit": "particle-substeps/s", "cores": nt, "kind": "port",
                         "sample": "one reduced substep of the same state (oracle, float32, OpenMP)"},
        "status": sim.engine.status()}


def reduced_arm(args):
    import torch

    import __graft_entry__ as g

    g.build()
    print(json.dumps(reduced_result(args, torch.device("cuda:0"))), flush=True)


def decoder_result(args, device) -> dict:
    """The reduced-order loop's substep with the reference's stress decoder as the
    stress source (NetDec 10 -> 30 x 5 -> 6, ELU, seeded reference initialisation):
    each step decodes every particle's stress into the state (mpm_decoder_stress)
    and runs the substep, on the large sand column.  CUDA events."""
    import numpy as np
    import torch

    from reduced_mpm_stress_training_gb300 import MPM_Simulator_WARP
    from reduced_mpm_stress_training_gb300 import scenarios as S
    from reduced_mpm_stress_training_gb300.decoder import StressDecoder

    sc = S.sand_column_1m()
    n, dt = sc.n_particles, sc.dt
    x0, v0, vol, mass = sc.particles()
    sim = MPM_Simulator_WARP(n, n_grid=sc.n_grid, grid_lim=sc.grid_lim, device=device)
    sim.set_parameters(material=sc.material, E=sc.E, nu=sc.nu, friction_angle=sc.friction_angle,
                       gravity=sc.gravity)
    sim.load_x_initial_from_tensor(torch.from_numpy(x0))
    sim.load_vol_from_tensor(torch.from_numpy(vol))
    sim.load_mass_from_tensor(torch.from_numpy(mass))
    sim.load_v_from_tensor(torch.from_numpy(v0))
    for kind, kw in sc.colliders():
        sim.add_surface_collider(**kw) if kind == "surface" else sim.add_bounding_box(**kw)
    dec = StressDecoder.random(seed=0, x_stats=((0.5, 0.5, 0.45), (0.09, 0.09, 0.23)),
                               q_stats=((0.0,) * 6, (50.0,) * 6), device=device)
    label = torch.from_numpy(np.random.default_rng(0).normal(0, 1, 6).astype(np.float32)).to(device)
    mu = torch.full((n, 1), sc.friction_angle, dtype=torch.float32, device=device)
    eng = sim.engine

    def decode():
        dec.stress_into(eng, label, mu)

    def step():
        decode()
        eng.substep_raw(float(sim.time), dt)

    for _ in range(max(3, args.warmup)):
        step()
        sim.time += dt
    sim.check_status()
    K = max(16, min(args.steps, 1000))
    t_dec = _events_ms(decode, K) / 1e3
    t_step = _events_ms(step, K) / 1e3
    sim.time += K * dt
    flops = 2 * (3 * dec.hidden + dec.mu_dim * dec.hidden + 4 * dec.hidden ** 2 + 6 * dec.hidden) * n
    # CPU: the NumPy float32 restatement of the decoder (BLAS threads) on a 262,144-row sample
    from oracle import decoder as OD

    m_cpu = 262_144
    rows = np.concatenate([np.tile(label.cpu().numpy(), (m_cpu, 1)), x0[:m_cpu],
                           np.full((m_cpu, 1), sc.friction_angle, np.float32)], 1)
    blob = dec.params.cpu().numpy()
    t0 = time.perf_counter()
    OD.forward(blob, rows, dec.label_dim, dec.mu_dim, dec.hidden, False, dec.omega_0, dtype=np.float32)
    cpu_rate = m_cpu / (time.perf_counter() - t0)
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    fp32_peak = sms * 128 * 2 * 2.07e9 / 1e12
    return {
        "metric": "particle-substeps/s (decoded-stress substep: NetDec stress + p2g2p, 1M sand, fp32)",
        "value": n / t_step, "unit": "particle-substeps/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded reference initialisation of the decoder)",
        "config": {"workload": f"sand_column_1m: {n} particles, {sc.n_grid}^3 grid; NetDec label 6, "
                               f"hidden {dec.hidden}, ELU",
                   "l2": "state larger than L2"},
        "decoder": {"ms": 1e3 * t_dec, "tflops": flops / t_dec / 1e12, "flops_per_particle": flops / n,
                    "fp32_peak_nominal_tflops": fp32_peak, "frac_of_nominal": flops / t_dec / 1e12 / fp32_peak,
                    "cpu_baseline": {"value": cpu_rate, "unit": "particles decoded/s", "cores": os.cpu_count(),
                                     "kind": "port", "sample": f"{m_cpu} rows, NumPy float32 (BLAS threads)"}},
        "status": eng.status()}


def decoder_arm(args):
    import torch

    import __graft_entry__ as g

    g.build()
    print(json.dumps(decoder_result(args, torch.device("cuda:0"))), flush=True)


def main():
    args = parse()
    world, rank, local = dist_env()
    from reduced_mpm_stress_training_gb300 import scenarios as S

    if args.workload == "batch_64":
        if rank == 0 and args.impl == "gb300":
            batched_arm(args)
        return
    if args.workload == "decoder_1m":
        if rank == 0 and args.impl == "gb300":
            decoder_arm(args)
        return
    if args.workload == "reduced_1m":
        if rank == 0 and args.impl == "gb300":
            reduced_arm(args)
        return
    sc = S.SCENES[args.workload]()
    if world > 1:
        import torch
        import torch.distributed as dist

        if args.impl == "reference":
            if rank != 0:
                return
        else:
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    if args.impl == "reference":
        reference_arm(args, sc, world, rank)
        return
    if world == 1:
        import __graft_entry__ as g

        g.build()
    gb300_arm(args, sc, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
