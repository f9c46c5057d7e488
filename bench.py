"""XPBI substep throughput on GB300: particle-substeps/s.

One step = one XPBI substep over every particle of the workload (all scenes
of a batched handle in one graph replay). Default workload: the dam-breach
scene mix at 4M particles (four 1M-particle dam-breach scenes, seeds 0-3:
water 600k PBF + Drucker-Prager sand 400k each, 15 XPBI + 4 PBF
iterations, dt=1e-4). Inputs are synthetic, seeded lattices.

Arms:
  --impl xpbi       libxpbi (this repo) through its C ABI
  --impl reference  the reference's kernels on the host cores: its WGSL
                    translated mechanically to C++ (oracle/wgsl_ref.py; a
                    WebGPU adapter exists on neither machine), or the CPU
                    oracle port where that translation is not built
"""
from __future__ import annotations

import argparse
import datetime
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-substeps/s at equal residual, learned warm-start vs plain, 1 GB300"
UNIT = "particle-substeps/s"

# Algorithmic bytes per particle for one launch of each kernel (compulsory
# traffic, minimal layout), as (solid particle, water particle):
#   solveA  solid: reads pos 16, vel 16, F 36, L 36, state 4, lambda 4, writes
#           lambda 4, the 64-byte neighbour record and the 16-byte own dv
#           = 196; water: reads pos 16 and exits.
#   solveB  solid: reads pos 16, vel 16, its record 64 and own dv 16 (every
#           record is read by its neighbours; compulsory once), writes vel 16
#           = 128; water: pos, vel in, vel out = 48.
#   pbfA    pos 16, predicted position 16, writes the multiplier 4 = 36.
#   pbfB    predicted position 16, multiplier 4, vel in 16, vel out 16 = 52.
#   computeL pos 16, vel 16, writes L 36 = 68.   xsph pos, vel in, vel out = 48.
#   updateF+integrate solid: reads pos 16, vel 16, F 36, L 36, state 4,
#           writes pos 16, vel 16, F 36, state 4 = 180; water: no L = 144.
ALGO_BYTES = {"solveA": (196, 16), "solveB": (128, 48), "pbfA": (36, 36), "pbfB": (52, 52),
              "computeL": (68, 68), "xsph": (48, 48), "updateF+integrate": (180, 144),
              "reorder": (148, 148), "count": (20, 20), "fill": (8, 8), "scan": (8, 8)}

# DRAM bytes per particle per launch (dram__bytes_read.sum +
# dram__bytes_write.sum over particles) from an ncu --set full capture of the
# current kernels on the 1M-particle dam breach 100 plain substeps in (the
# bench's loaded state; profiles/stencil_kernels_full_dam_breach_1M.md); the
# traffic of a launch grows with the particle count, so the bench scales it
# by the workload's.
NCU_TRAFFIC_PER_PARTICLE = {"solveB": 145.6, "solveA": 213.2, "pbfA": 107.2, "computeL": 169.7}


def workload(name: str, rank: int = 0, world: int = 1):
    """(package, this rank's scenes, scaling) of a named workload. The job's
    batch is built once and split across ranks by the particle-count
    bin-pack of shard.py (disjoint shards, no data-path collective):
      dam_mix<S>   S one-million-particle dam breaches per rank (seeds
                   0..S*world-1; dam_mix4 is the 4M benchmark mix): weak
      batch256     the 256-scene mixed batch (seed 0), fixed in total: strong
      dam_breach, nacc_snowball, sand_column   one scene per rank (seed =
                   rank): weak"""
    xp = importlib.import_module("xpbi-webgpu_gb300")
    shard = importlib.import_module("xpbi-webgpu_gb300.shard")
    if name.startswith("dam_mix") and name[7:].isdigit() and int(name[7:]) > 0:
        count = int(name[7:])
        batch = xp.scenes.config_dam_mix(seeds=tuple(range(count * world)))
        return xp, shard.shard(batch, rank, world), "weak"
    if name == "batch256":
        return xp, shard.shard(xp.scenes.config_batch(seed=0), rank, world), "strong"
    if name == "dam_breach":
        scenes = [xp.scenes.config_dam_breach(seed=rank)]
    elif name == "nacc_snowball":
        scenes = [xp.scenes.config_nacc_snowball(seed=rank)]
    elif name == "sand_column":
        scenes = [xp.scenes.config_sand_column(seed=rank)]
    else:
        raise SystemExit(f"unknown workload {name}")
    return xp, scenes, "weak"


class Clocks:
    """nvidia-smi sampling during the timed region: samples every 50 ms,
    started before the region (the sampler needs a moment to come up) and
    kept only where their timestamps fall inside it."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.p = None
        self.t0 = self.t1 = 0.0

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        time.sleep(0.3)
        self.t0 = time.time()

    def stop(self) -> dict:
        self.t1 = time.time()
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        return self.summarise(out, self.t0, self.t1)

    @staticmethod
    def summarise(out: str, t0: float, t1: float) -> dict:
        rows = []
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(f[2]), float(f[3]), f[6:10]))
            except ValueError:
                continue
        inside = [r for r in rows if t0 - 0.05 <= r[0] <= t1 + 0.05]
        use = inside or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = {n for r in use for n, v in zip(names, r[3]) if v.lower().startswith("active")}
        return {"sm_mhz": statistics.median(r[1] for r in use) if use else None,
                "sm_max_mhz": max(r[2] for r in use) if use else None,
                "reasons": sorted(reasons), "samples": len(use), "samples_in_region": len(inside)}


def standalone_scenes():
    """scenes.py (the seeded scene factories, NumPy only) loaded by file path,
    without importing the package, so the CPU leg touches no part of the
    library under test."""
    import importlib.util
    path = os.path.join(ROOT, "xpbi-webgpu_gb300", "scenes.py")
    spec = importlib.util.spec_from_file_location("xpbi_cpu_scenes", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def cpu_path():
    """(kind, substep function, description) of the CPU path timed beside
    the GPU: the reference's own kernels (its WGSL translated to C++ by
    oracle/wgsl_ref.py) where they are built, else the oracle port."""
    from oracle import oracle as O
    from oracle import wgsl_ref as W
    try:
        if W.build() is not None:
            W.lib()
            return "reference", W.substep, "the reference's WGSL kernels translated to C++"
    except (OSError, RuntimeError) as e:
        print(f"reference kernels unavailable ({e}); timing the oracle port", file=sys.stderr)
    return "port", O.substep, "f32 oracle port"


def cpu_sample_name(scale: float, preroll: int) -> str:
    return f"dam_breach scale {scale:g} seed 0 after {preroll} plain substeps"


class CpuSample:
    """The CPU path on the benchmark's sample: one dam-breach scene (seed 0)
    with its z extent scaled by `scale`, rolled `preroll` plain substeps
    forward by the CPU path itself (the state the GPU workload's scenes are
    timed from, at a size the host cores finish in minutes). Uniforms come
    from oracle/uniforms.py and scenes from scenes.py loaded standalone: no
    part of libxpbi runs here."""

    def __init__(self, scale: float, preroll: int, threads: int):
        from oracle import oracle as O
        from oracle import uniforms as U
        self.kind, self.fn, self.desc = cpu_path()
        S = standalone_scenes()
        sc = S.config_dam_breach(seed=0, scale=scale)
        self.pw, self.mw = U.pack(sc, U.frame_params(sc))
        self.it, self.pbf = sc["iterations"], sc["pbfIterations"]
        self.n = len(sc["positions"])
        self.threads = threads
        self.name = cpu_sample_name(scale, preroll)
        t0 = time.perf_counter()
        self.st = O.initial_state(sc)
        if preroll:
            self.st = self.fn(self.pw, self.mw, self.st, self.it, True, self.pbf, substeps=preroll,
                              threads=threads)
        self.preroll_s = time.perf_counter() - t0

    def step(self) -> float:
        """One substep from the current state; returns its seconds."""
        t0 = time.perf_counter()
        self.st = self.fn(self.pw, self.mw, self.st, self.it, True, self.pbf, substeps=1, threads=self.threads)
        return time.perf_counter() - t0


def cpu_baseline(scale: float, preroll: int, threads: int, substeps: int, budget_s: float):
    """Consecutive substeps of the CPU sample until `substeps` ran or
    budget_s seconds were spent (at least one). Returns (particle-substeps/s,
    cpu_baseline dict)."""
    smp = CpuSample(scale, preroll, threads)
    dt, done = 0.0, 0
    while done < substeps:
        dt += smp.step()
        done += 1
        if budget_s > 0 and dt >= budget_s:
            break
    v = smp.n * done / dt
    return v, {"value": v, "unit": UNIT, "cores": threads, "kind": smp.kind,
               "sample": f"{smp.desc}: {smp.name} ({smp.n} particles, 15 XPBI + 4 PBF iterations per "
                         f"substep), {done} consecutive substeps in {dt:.1f} s on {threads} threads"}


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, rank: int, world: int):
    """The reference's kernels on the host cores (rank 0 only), one substep
    of the CPU sample per step, consecutive from the prerolled state."""
    if rank != 0:
        return
    threads = host_threads()
    smp = CpuSample(args.cpu_scale, args.preroll, threads)
    for _ in range(args.warmup):
        smp.step()
    total = sum(smp.step() for _ in range(args.steps))
    value = smp.n * args.steps / total
    sample = (f"{smp.desc}: {smp.name} ({smp.n} particles), one substep (15 XPBI + 4 PBF iterations) "
              f"per step, {threads} threads")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": args.workload, "solver": "plain", "cpu_sample": smp.name,
                       "cpu_sample_particles": smp.n, "preroll_seconds": round(smp.preroll_s, 1)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": smp.kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def make_sim(xp, scenes, stream, preroll: int):
    """A handle over the workload, rolled forward `preroll` plain substeps
    (deterministic: equal inputs give equal states)."""
    sim = xp.Simulation(scenes if len(scenes) > 1 else scenes[0])
    sim.set_stream(stream.cuda_stream)
    has_water = any(s["hasWater"] for s in scenes)
    for k, s in enumerate(scenes):
        sim.write_params(xp.params_for(s), scene=k)
        sim.set_schedule(k, s["iterations"], s["hasWater"])
    if preroll:
        sim.set_solver(0, 0.0, False, True)  # carries multipliers for the warm start
        sim.step(preroll, -1, has_water)
    sim.synchronize()
    return sim, has_water


def max_over_ranks(x: float, dist, device: str = "cuda") -> float:
    """The job's time is its slowest rank's: all-reduce MAX (NCCL tensors
    live on the GPU, gloo ones on the host)."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_particles(n_rank: int, dist, device: str = "cuda") -> int:
    """Particles of the whole job: every rank's shard (all-reduce SUM)."""
    if not dist:
        return n_rank
    import torch
    t = torch.tensor([n_rank], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())


def job_throughput(job_particles_: int, steps: int, seconds: float) -> float:
    """Whole-job particle-substeps/s: every rank's particles over the slowest
    rank's time."""
    return job_particles_ * steps / seconds


def timed_steps(sim, has_water, steps, stream, dist):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    sim.step(steps, -1, has_water)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    sim.synchronize()
    return max_over_ranks(ms, dist)


def residual_stats(sim, has_water, n_scenes, substeps):
    """Final constraint and contact residuals relative to their starting
    values, and iterations applied, over `substeps` tracked substeps of every
    scene."""
    rel, relc, used = [], [], []
    sim.fallbacks = []
    for _ in range(substeps):
        sim.step(1, -1, has_water)
        for k in range(n_scenes):
            r, u = sim.read_residuals(k)
            c = sim.read_contact_residuals(k)
            sim.fallbacks.append(sim.read_fallback(k))
            if r[0] > 0:  # a scene with constraints (its contact entry pairs with it; 0 with no contact)
                rel.append(float(r[-1] / r[0]))  # the final state's residual, re-measured over every particle
                relc.append(float(c[-1] / c[0]) if c[0] > 0 else 0.0)
            used.append(u)
    return rel, relc, used


def profile_kernels(sim, has_water, substeps: int) -> dict:
    """Per-launch times (CUDA events around each launch) of `substeps`
    enqueued substeps: label -> list of milliseconds."""
    per = {}
    for _ in range(max(1, substeps)):
        for line in sim.profile_substep(-1, has_water).splitlines():
            if ":" not in line:
                continue
            name, t = line.rsplit(":", 1)
            per.setdefault(name.strip(), []).append(float(t.strip().replace("ms", "")))
    return per


def reached_fraction(rel, relc, tau: float, tau_c: float) -> float:
    """Fraction of tracked (scene, substep) solves whose final constraint AND
    contact residuals (relative to their starting values) are both within
    the plain solve's tolerances (0.01% slack for the f64 sums' rounding)."""
    r = np.asarray(rel, np.float64)
    c = np.asarray(relc, np.float64)
    return float(np.mean((r <= tau * 1.0001) & (c <= tau_c * 1.0001))) if len(r) else 0.0


def other_configs(xp, stream, args) -> dict:
    """The plain solve of the other benchmark configs, measured in the same
    run (one GPU): the 16k sand column (10 iterations), the 113k NACC
    snowball (20), the 256-scene mixed batch (~4.4M particles, 10-20 per
    scene), each from its initial state, autotuned, `args.steps` graph
    replays timed with CUDA events after `args.warmup`."""
    out = {}
    for name, scenes in (("sand_column_16k", [xp.scenes.config_sand_column()]),
                         ("nacc_snowball_113k", [xp.scenes.config_nacc_snowball()]),
                         ("batch256", xp.scenes.config_batch(seed=0))):
        n = sum(len(s["positions"]) for s in scenes)
        sim, hw = make_sim(xp, scenes, stream, 0)
        sim.set_solver(0, 0.0, False, False)
        tuned_o = sim.autotune(-1, hw, repeats=3)
        sim.step(args.warmup, -1, hw)
        sim.synchronize()
        ms = timed_steps(sim, hw, args.steps, stream, None)
        sim.close()
        its = sorted({s["iterations"] for s in scenes})
        out[name] = {"value": n * args.steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / args.steps,
                     "particles": n, "scenes": len(scenes), "solver": "plain",
                     "iterations": its if len(its) > 1 else its[0],
                     "autotuned_variants": {"solveA": tuned_o["solveA"], "solveB": tuned_o["solveB"],
                                            "solveA_ms": [round(x, 4) for x in tuned_o["solveA_ms"]],
                                            "solveB_ms": [round(x, 4) for x in tuned_o["solveB_ms"]]}}
    return out


def run_xpbi(args, rank: int, world: int):
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    xp, scenes, scaling = workload(args.workload, rank, world)
    n_rank = sum(len(s["positions"]) for s in scenes)
    n_job = job_particles(n_rank, dist)
    stream = torch.cuda.Stream()
    learned = args.solver == "learned"

    # ---- plain solve (the reference's fixed iteration budget)
    sim, has_water = make_sim(xp, scenes, stream, args.preroll)
    sim.set_solver(0, 0.0, False, False)
    tuned = sim.autotune(-1, has_water, repeats=5)  # launch shapes timed on this workload
    sim.step(args.warmup, -1, has_water)  # graph capture happens here
    sim.synchronize()
    clocks = Clocks(local)
    clocks.start()
    ms_plain = timed_steps(sim, has_water, args.steps, stream, dist)
    clk = clocks.stop()
    per_plain = profile_kernels(sim, has_water, args.profile_substeps)
    value_plain = job_throughput(n_job, args.steps, ms_plain / 1e3)
    launches = sim.launches_per_substep(-1, has_water)
    solvers = {"plain": {"value": value_plain, "ms_per_step": ms_plain / args.steps,
                         "iterations": [s["iterations"] for s in scenes][:4]}}
    ms, value = ms_plain, value_plain
    if learned:
        # equal residual: the plain solve's own final constraint and contact
        # residuals, relative to their starting values, median over tracked
        # substeps and scenes; the early-stopped solves stop once both are
        # reached
        sim.set_solver(0, 0.0, True, True)
        rel, relc, _ = residual_stats(sim, has_water, len(scenes), args.residual_substeps)
        tau = float(np.median(rel))
        tau_c = float(np.median(relc)) if relc else 1.0
        sim.close()
        solvers["plain"]["final_rel_residual_median"] = tau
        solvers["plain"]["final_rel_contact_residual_median"] = tau_c
        tw = importlib.import_module("xpbi-webgpu_gb300.train_warm")
        net = tw.load_weights()
        n_solid_rank = sum(int(sum(1 for m in s["matIds"] if s["materials"][m]["kind"] != 6)) for s in scenes)

        def early_stopped(mode, share, keep=False):
            """An early-stopped solve at the plain tolerances: mode 1 = the
            network's warm start, 0 = the zero start; share > 0 = with the
            active set. Returns (its solver record, the handle if keep)."""
            h, _ = make_sim(xp, scenes, stream, args.preroll)
            h.set_variants(tuned["solveA"], tuned["solveB"])
            if mode == 1:
                h.set_network(net)
            h.set_active_set(share)
            h.set_max_iterations(args.max_iterations)
            h.set_solver(mode, tau, False, False, contact_rel_tol=tau_c)
            h.step(args.warmup, -1, has_water)
            h.synchronize()
            ck = Clocks(local)
            ck.start()
            t = timed_steps(h, has_water, args.steps, stream, dist)
            c = ck.stop()
            h.set_solver(mode, tau, True, False, contact_rel_tol=tau_c)
            rel_l, relc_l, used_l = residual_stats(h, has_water, len(scenes), args.residual_substeps)
            act_a, act_b = h.read_active_counts()
            h.set_solver(mode, tau, False, False, contact_rel_tol=tau_c)
            rec = {"value": job_throughput(n_job, args.steps, t / 1e3), "ms_per_step": t / args.steps,
                   "network": mode == 1, "active_share": share, "max_iterations": args.max_iterations,
                   "rel_tol": tau, "contact_rel_tol": tau_c,
                   "final_rel_residual_median": float(np.median(rel_l)),
                   "final_rel_contact_residual_median": float(np.median(relc_l)) if relc_l else None,
                   "iterations_mean": float(np.mean(used_l)),
                   "reached_tol_fraction": reached_fraction(rel_l, relc_l, tau, tau_c),
                   "resolved_plainly_fraction": float(np.mean(h.fallbacks)) if h.fallbacks else 0.0}
            if share > 0:
                K = max(max(s["iterations"] for s in scenes), args.max_iterations)
                rec["active_fraction_per_iteration"] = {
                    "solveA": [1.0, 1.0] + [round(int(x) / max(n_solid_rank, 1), 4) for x in act_a[2:K]],
                    "solveB": [1.0, 1.0] + [round(int(x) / max(n_rank, 1), 4) for x in act_b[2:K]],
                    "of": "solids (solveA), all particles (solveB); last tracked substep"}
            return rec, (h, c) if keep else h.close()

        solvers["learned"], (sim, clk) = early_stopped(1, args.active_share, keep=True)
        value, ms = solvers["learned"]["value"], solvers["learned"]["ms_per_step"] * args.steps
        launches = sim.launches_per_substep(-1, has_water)
        if args.active_share > 0:
            # the graph runs the iterations after the last PBF pass as a device
            # loop: 6 launches (two compactions, solveA, solveB, the residual,
            # the loop step) per iteration it runs plus one to start it, in
            # place of the 5 per iteration up to the cap that an enqueued
            # substep issues
            pbf = [p_.get("pbfIterations", 0) or 0 for p_ in (xp.params_for(s_) for s_ in scenes)]
            k0 = max(1, max(pbf))
            cap = max(args.max_iterations, max(s_["iterations"] for s_ in scenes))
            it = solvers["learned"]["iterations_mean"]
            if cap - k0 >= 2:
                launches = launches - 5 * (cap - k0) + 1 + 6 * max(0.0, it - k0)
        if not args.no_ablation:
            # what each part gains: the network without the active set, and
            # the active set without the network (zero start)
            if args.active_share > 0:
                solvers["learned_without_active_set"], _ = early_stopped(1, 0.0)
                solvers["plain_start_with_active_set"], _ = early_stopped(0, args.active_share)

    # ---- end to end through the public API with host buffers: per step the
    # frame's writeParams from host memory, one substep, and the positions
    # read back into pinned host memory (asynchronously, like the
    # reference's mapAsync: a step's read-back overlaps the next substep;
    # all are complete when the final synchronize returns)
    pinned = [torch.empty((len(s["positions"]), 4), dtype=torch.float32, pin_memory=True).numpy()
              for s in scenes]
    params = [xp.params_for(s) for s in scenes]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for k in range(len(scenes)):
            sim.write_params(params[k], scene=k)
        sim.step(1, -1, has_water)
        for k in range(len(scenes)):
            sim.read_pos_async(k, pinned[k])
    sim.synchronize()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e = job_throughput(n_job, args.steps, e2e_s)
    # uniforms uploaded per step: SceneDev (244 B) + MatDev table (8 x 48 B)
    # + packed material words (8 x 64 B) per scene
    h2d = len(scenes) * (244 + 8 * 48 + 8 * 64)
    d2h = 16 * n_rank

    # ---- per-kernel times (events around each launch) for the roofline: of
    # the plain solve (every kernel over every particle); the learned
    # solve's time per kernel and substep is reported beside it
    per = per_plain
    if learned:
        per_l = profile_kernels(sim, has_water, args.profile_substeps)
        reps = max(1, args.profile_substeps)
        solvers["learned"]["substep_ms_by_kernel"] = {k: round(sum(v) / reps, 4) for k, v in per_l.items()}
    total_ms = sum(sum(v) for v in per.values())
    dom = max(per, key=lambda k: sum(per[k]))
    dom_avg_ms = statistics.mean(per[dom])
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    n_water = sum(int(sum(1 for m in s["matIds"] if s["materials"][m]["kind"] == 6)) for s in scenes)
    n_solid = n_rank - n_water
    bs, bw = ALGO_BYTES.get(dom, (0, 0))
    algo = bs * n_solid + bw * n_water  # bytes per launch
    achieved = algo / (dom_avg_ms / 1e3) / 1e9
    tpp = NCU_TRAFFIC_PER_PARTICLE.get(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_src,
                "traffic": None if tpp is None else tpp * n_rank,
                "traffic_source": "ncu capture of the 1M-particle dam breach (100 substeps in) scaled by particle count",
                "algo_bytes_per_launch": algo, "solid_particles": n_solid, "water_particles": n_water,
                "share": sum(per[dom]) / total_ms,
                "kernel_ms": {k: round(statistics.mean(v), 4) for k, v in per.items()}}
    # every kernel with a byte model: its algorithmic bytes per launch over its
    # own event time; and the substep's (all launches' bytes over the graph's
    # time per substep)
    reps = max(1, args.profile_substeps)
    kern, sub_bytes = {}, 0.0
    for k, v in per.items():
        if k not in ALGO_BYTES:
            continue
        b_s, b_w = ALGO_BYTES[k]
        # the scan moves 8 bytes per cell (cell counts in, starts out)
        nbytes = 8 * sim.num_cells if k == "scan" else b_s * n_solid + b_w * n_water
        sub_bytes += nbytes * len(v) / reps
        gbs = nbytes / (statistics.mean(v) / 1e3) / 1e9
        kern[k] = {"launches_per_substep": len(v) // reps, "achieved": round(gbs, 1), "frac": round(gbs / peak, 4)}
    roofline["kernels"] = kern
    sub_gbs = sub_bytes / (ms / args.steps / 1e3) / 1e9
    roofline["substep"] = {"algo_bytes": sub_bytes, "achieved": round(sub_gbs, 1), "frac": round(sub_gbs / peak, 4)}
    sim.close()

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": scaling,
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": args.workload, "particles_per_gpu": n_rank, "particles_job": n_job,
                      "scenes": len(scenes),
                      "solver": args.solver, "preroll_substeps": args.preroll,
                      "iterations": [s["iterations"] for s in scenes][:4],
                      "autotuned_variants": {"solveA": tuned["solveA"], "solveB": tuned["solveB"],
                                             "solveA_ms": [round(x, 4) for x in tuned["solveA_ms"]],
                                             "solveB_ms": [round(x, 4) for x in tuned["solveB_ms"]]},
                      "l2": "inputs larger than L2 (state ~1.3 GB per 4M particles)",
                      "cpu_sample": cpu_sample_name(args.cpu_scale, args.preroll)},
           "solvers": solvers,
           "roofline": roofline, "clocks": clk, "gpu_launches": int(round(launches * args.steps)),
           "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}}
    if world == 1 and not args.no_other_configs:
        out["other_configs"] = other_configs(xp, stream, args)
    if rank == 0 and not args.no_cpu_baseline:
        _, out["cpu_baseline"] = cpu_baseline(args.cpu_scale, args.preroll, host_threads(), args.cpu_substeps,
                                              args.cpu_budget)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


def run_profile_region(args):
    """For ncu --profile-from-start off: the learned solve of the workload set
    up as the bench line's (plain preroll, the plain solve's tolerances from
    tracked substeps, network warm start, active set, iteration cap), three
    warm-up substeps from its graph, then two substeps inside
    cudaProfilerStart/Stop, replayed from the graph (`graph`; ncu times it
    whole) or enqueued launch by launch (`eager`; the same kernels, with the
    iterations past the stop enqueued as launches that find nothing to do).
    `plain`: the plain solve (autotuned as the bench line's) after the same
    preroll, one substep enqueued launch by launch inside the region."""
    import torch
    torch.cuda.set_device(0)
    xp, scenes, _ = workload(args.workload, 0, 1)
    stream = torch.cuda.Stream()
    sim, has_water = make_sim(xp, scenes, stream, args.preroll)
    if args.profile_region == "plain":
        sim.set_solver(0, 0.0, False, False)
        tuned = sim.autotune(-1, has_water, repeats=3)
        sim.step(3, -1, has_water)
        sim.synchronize()
        torch.cuda.profiler.start()
        sim.encode_substep(-1, has_water)
        sim.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"profile_region": "plain", "workload": args.workload, "variants": tuned}))
        return
    sim.set_solver(0, 0.0, True, True)
    rel, relc, _ = residual_stats(sim, has_water, len(scenes), args.residual_substeps)
    tau, tau_c = float(np.median(rel)), float(np.median(relc))
    tw = importlib.import_module("xpbi-webgpu_gb300.train_warm")
    sim.set_network(tw.load_weights())
    sim.set_active_set(args.active_share)
    sim.set_max_iterations(args.max_iterations)
    sim.set_solver(1, tau, False, False, contact_rel_tol=tau_c)
    sim.step(3, -1, has_water)
    sim.synchronize()
    torch.cuda.profiler.start()
    for _ in range(2):
        if args.profile_region == "graph":
            sim.step(1, -1, has_water)
        else:
            sim.encode_substep(-1, has_water)
    sim.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"profile_region": args.profile_region, "workload": args.workload, "rel_tol": tau,
                      "contact_rel_tol": tau_c}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xpbi", choices=["xpbi", "reference"])
    ap.add_argument("--workload", default="dam_mix4")
    ap.add_argument("--cpu-scale", type=float, default=0.25)
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds after which the CPU baseline sample stops (at least one substep)")
    ap.add_argument("--cpu-substeps", type=int, default=30,
                    help="substeps of the CPU baseline sample (about 10 s on 16 cores)")
    ap.add_argument("--profile-substeps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--solver", default=None, choices=["learned", "plain"],
                    help="learned warm start at the plain solve's residual (default for the dam-breach mix)")
    ap.add_argument("--preroll", type=int, default=None, help="untimed plain substeps before warm-up")
    ap.add_argument("--residual-substeps", type=int, default=4)
    ap.add_argument("--active-share", type=float, default=0.25,
                    help="active set of the learned solve: share of the residual budget settled particles may "
                         "hold (0: no work skipping)")
    ap.add_argument("--max-iterations", type=int, default=30,
                    help="iteration cap of the early-stopped solves (they stop once both residuals reach the plain "
                         "solve's; the plain solve runs its fixed 15)")
    ap.add_argument("--profile-region", choices=["graph", "eager", "plain"], default=None,
                    help="set up the learned solve (graph, eager: two substeps) or the plain one (plain: one substep) "
                         "and run it between cudaProfilerStart/Stop (for ncu "
                         "--profile-from-start off); prints no bench line")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the plain solve of the sand column, snowball and 256-scene batch configs")
    ap.add_argument("--no-ablation", action="store_true",
                    help="skip the learned solve's ablation lines (network alone, active set alone)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.solver is None:
        args.solver = "learned" if args.workload in ("dam_mix4", "dam_breach") else "plain"
    if args.preroll is None:
        args.preroll = 100 if (args.solver == "learned" or args.impl == "reference") else 0
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    if args.profile_region:
        if args.preroll is None or args.preroll == 0:
            args.preroll = 100
        run_profile_region(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_xpbi(args, rank, world)


if __name__ == "__main__":
    main()
