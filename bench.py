#!/usr/bin/env python
"""Batched contact-path throughput on GB300.

Workload (one GPU): 4,096 independent worlds with body counts log-uniform in
[8, 512] (box pyramids with base 4-16 and random-hull piles as in the 1,000-hull
drop), each with its own static plate; dt 1/60, one substep, 10 PGS velocity
iterations + 1 position iteration, warm start on, sleeping off.  A step advances
every world by one timeStep.

Reported (one JSON line on rank 0):
  value      batched body-steps/s with the state resident in HBM, device time
             (CUDA events on the library's stream) of exactly --steps graph-
             launched steps after --warmup untimed ones
  e2e        the same through the C ABI with host buffers: every step writes
             the full body state from pinned host memory, steps, and reads the
             full state back
  plain      body-steps/s of the plain path (each world as its own
             single-world device batch) on an evenly spaced sample of worlds;
             vs_plain = value / plain
  roofline   dominant kernel: algorithmic bytes / its measured time against the
             measured HBM copy bandwidth (MEASURED_PEAKS.json)
  cpu_baseline  the reference engine (compiled from its own sources) on the
             box's host cores, one engine per thread, on a bounded sample of
             the same worlds and steps

--impl reference times only the reference engine on that sample and prints
its line.  Under torchrun each rank takes its own 4,096 worlds (weak scaling,
no collective on the data path); rank 0 prints the max-time line.
"""
import argparse
import concurrent.futures
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

from constraintphysics_gb300 import scenes  # noqa: E402

METRIC = "batched body-steps/s vs plain GPU path @ <=1e-3 m drift; p50/p99 step latency"
UNIT = "body-steps/s"
WORKLOAD = "batched_4096_worlds"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=60)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--worlds", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--cpu-budget-s", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-only", action="store_true", help="build the batch, run warmup + steps, no extras")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="duration of each serving run (0: none)")
    ap.add_argument("--serve-rates", default="2000,20", help="Poisson request rates (requests/s) of the serving runs")
    ap.add_argument("--workload", default=WORKLOAD,
                    choices=[WORKLOAD, "hull_drop_1000", "terrain_20k", "chains_1024"],
                    help="the headline batched workload (default) or one of the other configurations")
    ap.add_argument("--tune-steps", type=int, default=3,
                    help="trial steps per candidate schedule of the batch autotuner (0: the hand-set schedule)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def shard_seed(seed, rank):
    """The seed of a rank's own worlds: every rank steps a different draw of
    the workload (world-sharded, no data-path collective)."""
    return seed + 1000 * rank


def across_ranks(world_size, maxes=(), sums=()):
    """(max over the ranks of each of `maxes`, sum over the ranks of each of
    `sums`); on one rank the values themselves.  The process group's backend
    chooses the tensors' device (NCCL: the GPU, gloo: the host)."""
    maxes, sums = [float(x) for x in maxes], [float(x) for x in sums]
    if world_size == 1:
        return maxes, sums
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    m = torch.tensor(maxes or [0.0], dtype=torch.float64, device=dev)
    s = torch.tensor(sums or [0.0], dtype=torch.float64, device=dev)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    return m.tolist()[:len(maxes)], s.tolist()[:len(sums)]


def build_worlds(ws_scenes, make_world):
    worlds = []
    for sc in ws_scenes:
        w = make_world()
        scenes.apply(sc, w)
        worlds.append(w)
    return worlds


def dynamic_bodies(ws_scenes):
    return sum(sc.n_bodies - 1 for sc in ws_scenes)   # every world has one fixed plate


def hull_sizes(ws_scenes):
    """Mean vertices / faces / edges over the scenes' hulls (boxes: 8/6/12)."""
    v = f = e = n = 0
    for sc in ws_scenes:
        for op in sc.ops:
            if op[0] == "hull":
                nv, nf = len(op[1]), len(op[2])
                v, f, e, n = v + nv, f + nf, e + nv + nf - 2, n + 1
            elif op[0] == "box":
                v, f, e, n = v + 8, f + 6, e + 12, n + 1
    return v / n, f / n, e / n


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.gpu = gpu_index
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if len(r) > 8]
        mx = [float(r[2]) for r in rows if len(r) > 8]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_traffic(stage, worlds):
    """DRAM bytes per launch of the stage's dominant kernel, from the committed
    summary of an ncu capture of the current build (profiles/pgs_traffic.txt:
    lines `stage bytes worlds`, the bytes scaled to the workload's world count
    from a smaller capture, as the file states), or None."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", "pgs_traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 3 and not line.startswith("#") and parts[0] == stage and int(parts[2]) == worlds:
                    return int(parts[1])
    except OSError:
        pass
    return None


def algorithmic_bytes(stage, counts, nbodies, vfe, params):
    """Algorithmic bytes of one launch of a stage (each datum read/written once)."""
    V, F, E = vfe
    npairs, ncont = counts["pairs"], counts["contacts"]
    iv, ip = params["pgs_vel"], params["pgs_pos"]
    if stage == "narrowphase":
        # both poses + both hulls (vertices, face planes, arcs) + manifold out
        return npairs * (2 * (32 + 16 * V + 16 * F + 4 * E) + 112)
    if stage == "pgs":
        # per contact: each velocity sweep reads 3 rows (48 B each) and
        # read-modify-writes 2 bodies' velocity deltas; each position sweep 1 row + 2 deltas
        return ncont * (iv * (3 * 48 + 2 * 48) + ip * (48 + 2 * 48))
    if stage == "rows":
        return ncont * (64 + 3 * 48)
    if stage == "integrate":
        return nbodies * (92 + 52)
    if stage == "pairs":
        return nbodies * 32 + npairs * 8
    return None


def run_serving(cg, rates, duration, seed, budget_bytes=150 << 30, epoch_steps=10, n_templates=48):
    """Serving workload: Poisson arrivals; each request is a world of
    floor(exp(U[ln 16, ln 2048])) bodies (pile or pyramid, generated as the
    batched workload) advanced K ~ U{30..300} steps, admitted under the
    device-memory budget into the continuously re-formed batch.  Requests are
    cloned from a pool of seeded template worlds.  Latency = completion minus
    arrival (wall clock)."""
    rng = np.random.default_rng(seed + 4242)
    pool = scenes.HullPool(seed + 5, size=128)
    temps = []
    for _ in range(n_templates):
        w = cg.world()
        scenes.apply(scenes.batched_world(rng, pool, 16, 2048), w)
        temps.append(w)
    out = []
    for rate in rates:
        srv = cg.Server(budget_bytes, epoch_steps)
        arr, t = [], 0.0
        while True:
            t += rng.exponential(1.0 / rate)
            if t > duration:
                break
            arr.append(t)
        meta, lat, offered, i = {}, [], 0, 0
        start = time.perf_counter()
        while True:
            now = time.perf_counter() - start
            while i < len(arr) and arr[i] <= now:
                tmp = temps[int(rng.integers(len(temps)))]
                k = int(rng.integers(30, 301))
                meta[srv.submit(cg.clone(tmp), k)] = arr[i]
                offered += k * (tmp.n_bodies - 1)
                i += 1
            if now > duration:
                break
            srv.advance(5)
            tn = time.perf_counter() - start
            for tok in srv.poll():
                lat.append(tn - meta.pop(tok))
        wall = time.perf_counter() - start
        st = srv.stats()
        srv.close()
        lat = np.array(lat) if lat else np.zeros(1)
        out.append({"rate_per_s": rate, "duration_s": duration, "arrived": len(arr), "completed": int(len(lat)),
                    "offered_body_steps_per_s": offered / duration, "served_body_steps_per_s": st["body_steps"] / wall,
                    "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
                    "reforms": st["reforms"], "reform_s": st["reform_ms"] / 1e3,
                    "device_gb": st["device_bytes"] / 1e9, "running_bodies_at_end": st["running_bodies"],
                    "budget_gb": budget_bytes / 1e9})
    return out


def run_reference_sample(ws_scenes, warmup, steps, budget_s, threads):
    """The reference engine on an evenly spaced sample of worlds: one engine per
    worker thread (ctypes releases the GIL), `warmup` untimed then `steps` timed
    steps per world.  Returns (body_steps_per_s, sample description, cores)."""
    import oracle
    if not oracle.ref_available():
        oracle.build()
    abi = oracle.ref_abi()
    step_untraced = abi._lib.cpref_step_untraced
    import ctypes
    step_untraced.restype = ctypes.c_int
    step_untraced.argtypes = [ctypes.c_void_p, ctypes.c_int]
    # probe one world to size the sample
    idx = list(range(0, len(ws_scenes), max(1, len(ws_scenes) // 512)))
    probe = oracle.ref_world()
    scenes.apply(ws_scenes[idx[0]], probe)
    step_untraced(probe.h, warmup)
    t = time.perf_counter()
    step_untraced(probe.h, steps)
    per_body_step = (time.perf_counter() - t) / max(1, steps * (ws_scenes[idx[0]].n_bodies - 1))
    est_total = per_body_step * steps * sum(ws_scenes[i].n_bodies - 1 for i in idx) / threads
    keep = max(threads, int(len(idx) * min(1.0, budget_s / max(est_total, 1e-9))))
    idx = idx[:: max(1, len(idx) // keep)][:keep]
    worlds = []
    for i in idx:
        w = oracle.ref_world()
        scenes.apply(ws_scenes[i], w)
        worlds.append((w, ws_scenes[i].n_bodies - 1))

    def warm(item):
        step_untraced(item[0].h, warmup)

    def timed(item):
        t0 = time.perf_counter()
        step_untraced(item[0].h, steps)
        return time.perf_counter() - t0

    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        list(ex.map(warm, worlds))
        t0 = time.perf_counter()
        list(ex.map(timed, worlds))
        wall = time.perf_counter() - t0
    body_steps = sum(n for _, n in worlds) * steps
    sample = (f"{len(worlds)} of {len(ws_scenes)} worlds (every {len(ws_scenes) // max(1, len(idx))}th), "
              f"{sum(n for _, n in worlds)} dynamic bodies, {warmup} untimed + {steps} timed steps each, "
              f"one single-threaded reference engine per thread")
    return body_steps / wall, sample, wall


def _f32_state(st):
    return {k: np.asarray(v, np.float32).astype(np.float64) for k, v in st.items()}


def measure_drift(cg, ws_scenes, n_per_kind=4, steps=300, max_bodies=400):
    """Position drift against the reference engine after `steps` steps, per
    scene kind (box pyramids, hull piles), on an evenly spaced sample of the
    worlds with at most `max_bodies` bodies, each side stepping the scene from
    scratch; per dynamic body the distance between the two centres of mass.
    Beside the device (FP32) two controls run on the CPU: the FP64
    restatement (mass properties within 1e-12 of the reference's, nothing else
    different) and the same restatement with its state rounded to FP32 after
    every step (FP64 arithmetic, FP32 storage: the smallest perturbation any
    FP32 implementation makes).  On chaotic scenes all three drift alike."""
    import oracle
    pick = []
    for kind in ("pyramid", "pile"):
        idx = [i for i, sc in enumerate(ws_scenes) if sc.name.startswith(kind) and sc.n_bodies <= max_bodies]
        pick += [(kind, i) for i in idx[:: max(1, len(idx) // n_per_kind)][:n_per_kind]]
    acc = {}
    for kind, i in pick:
        sc = ws_scenes[i]
        g = cg.world()
        scenes.apply(sc, g)
        g.step(steps)
        r = oracle.ref_world()
        scenes.apply(sc, r)
        r.step(steps)
        p = oracle.port_world()
        scenes.apply(sc, p)
        p.step(steps)
        q = oracle.port_world()
        scenes.apply(sc, q)
        for _ in range(steps):
            q.set_state(**_f32_state(q.state()))
            q.step(1)
        dyn = np.array([m == scenes.DYNAMIC for m in sc.movements()])
        rc = r.state()["com"][dyn]
        for name, w in (("device", g), ("fp64_control", p), ("fp32_state_control", q)):
            acc.setdefault(kind, {}).setdefault(name, []).append(np.linalg.norm(w.state()["com"][dyn] - rc, axis=1))

    def stats(x):
        x = np.concatenate(x)
        return {"median_m": float(np.median(x)), "p95_m": float(np.percentile(x, 95)), "max_m": float(x.max()),
                "frac_within_1e-3_m": float(np.mean(x <= 1e-3)), "bodies": int(x.size)}
    out = {kind: {name: stats(v) for name, v in m.items()} for kind, m in acc.items()}
    out.update(worlds=len(pick), steps=steps,
               note="per scene kind, every dynamic body; device FP32 vs the reference engine FP64 from the same "
                    "scene; fp64_control = the FP64 restatement, fp32_state_control = the restatement with its "
                    "state rounded to FP32 after every step; hull piles are chaotic at rounding level")
    return out


SECONDARY = {
    "hull_drop_1000": "1,000 random hulls (8-32 points, scale U[0.5,1.5] m) on a 10x10x10 grid dropped on the plate; "
                      "one world (the plain single-world path), dt 1/60, 1 substep, PGS (10,1,1)",
    "terrain_20k": "20,000 mixed bodies (40% boxes, 20% spheres, 20% cylinders, 20% hulls) dropped on a 256x256 "
                   "value-noise heightfield mesh (131,072 triangles); one world, PGS (20,1,1)",
    "chains_1024": "1,024 articulated chains of 16-64 unit boxes (link mass log-uniform [0.1,100] kg), ball-socket and "
                   "hinge joints, 50 fixed spheres each; one batch, 8 substeps, PGS (4,1,1) with the block solve",
}


def run_secondary(a):
    """One of the other configurations: device body-steps/s (state in HBM),
    per-stage times and roofline, the reference engine on the machine's host
    cores on a bounded sample, and (1,000 hulls) the 600-step drift."""
    import constraintphysics_gb300 as cg
    import oracle
    threads = max(1, os.cpu_count() or 1)
    if a.workload == "hull_drop_1000":
        scs = [scenes.hull_drop(seed=a.seed, n_side=10)]
        params = {"pgs_vel": 10, "pgs_pos": 1, "substeps": 1}
    elif a.workload == "terrain_20k":
        scs = [scenes.terrain_drop(seed=a.seed, n_grid=256, n_side=50, n_layers=8)]
        params = {"pgs_vel": 20, "pgs_pos": 1, "substeps": 1}
    else:
        rng = np.random.default_rng(a.seed)
        scs = [scenes.chain_world(rng) for _ in range(1024)]
        params = {"pgs_vel": 4, "pgs_pos": 1, "substeps": 8}
    n_dyn = sum(sum(1 for m in sc.movements() if m == scenes.DYNAMIC) for sc in scs)
    t0 = time.perf_counter()
    worlds = build_worlds(scs, cg.world)
    batch = cg.Batch(worlds)
    setup_s = time.perf_counter() - t0
    batch.step(a.warmup)
    sampler = ClockSampler(0)
    dev_ms = batch.step_timed(a.steps)
    stage_ms, counts = batch.profile(a.steps)
    clocks = sampler.stop()
    stage_ms = {k: v / a.steps for k, v in stage_ms.items()}
    value = n_dyn * a.steps / (dev_ms / 1e3)
    peak, peak_kind = measured_peaks()
    dominant = max(stage_ms, key=stage_ms.get)
    has_hulls = any(op[0] in ("hull", "box") for sc in scs for op in sc.ops)
    vfe = hull_sizes(scs) if has_hulls else (8, 6, 12)
    roof = None
    b = algorithmic_bytes(dominant, counts, batch.n_bodies, vfe, params)
    if b is not None:
        roof = {"bound": "hbm", "kernel": dominant, "achieved": b / (stage_ms[dominant] / 1e3) / 1e9, "peak": peak,
                "unit": "GB/s", "peak_kind": peak_kind, "algorithmic_bytes_per_launch": b,
                "launch_ms": stage_ms[dominant], "traffic": None}
        roof["frac"] = roof["achieved"] / peak
    # the reference engine on a bounded sample of the same scenes
    idx = list(range(len(scs)))[:: max(1, len(scs) // 64)]
    ref_steps = 3 if a.workload == "terrain_20k" else 10
    ref = []
    for i in idx:
        w = oracle.ref_world()
        scenes.apply(scs[i], w)
        ref.append((w, sum(1 for m in scs[i].movements() if m == scenes.DYNAMIC)))
    import ctypes
    step_untraced = oracle.ref_abi()._lib.cpref_step_untraced
    step_untraced.restype = ctypes.c_int
    step_untraced.argtypes = [ctypes.c_void_p, ctypes.c_int]
    with concurrent.futures.ThreadPoolExecutor(min(threads, len(ref))) as ex:
        list(ex.map(lambda it: step_untraced(it[0].h, 1), ref))
        tc = time.perf_counter()
        list(ex.map(lambda it: step_untraced(it[0].h, ref_steps), ref))
        wall = time.perf_counter() - tc
    cpu = {"value": sum(n for _, n in ref) * ref_steps / wall, "unit": UNIT, "cores": min(threads, len(ref)),
           "kind": "reference", "sample": f"{len(ref)} of {len(scs)} worlds, {ref_steps} timed steps after 1, "
                                         f"one single-threaded reference engine per thread"}
    drift = None
    if a.workload == "hull_drop_1000":
        g = cg.world()
        scenes.apply(scs[0], g)
        g.step(600)
        r = oracle.ref_world()
        scenes.apply(scs[0], r)
        r.step(600)
        dyn = np.array([m == scenes.DYNAMIC for m in scs[0].movements()])
        d = np.linalg.norm(g.state()["com"][dyn] - r.state()["com"][dyn], axis=1)
        drift = {"steps": 600, "median_m": float(np.median(d)), "p95_m": float(np.percentile(d, 95)),
                 "frac_within_1e-3_m": float(np.mean(d <= 1e-3)),
                 "note": "device FP32 vs the reference FP64 from the same scene; a 1,000-hull drop is chaotic"}
    line = {"metric": "body-steps/s", "value": value, "unit": UNIT, "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": dev_ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded scenes)",
            "config": {"workload": a.workload, "description": SECONDARY[a.workload], "dynamic_bodies": n_dyn,
                       "seed": a.seed},
            "roofline": roof, "cpu_baseline": cpu, "clocks": clocks, "stage_ms": stage_ms, "counts": counts,
            "setup_s": setup_s, "drift": drift, "gpu_launches": batch.launches_per_step() * a.steps}
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.workload != WORKLOAD:
        return run_secondary(a)
    rank, world_size, local_rank = dist_env()
    t_setup = time.perf_counter()
    ws_scenes = scenes.batched_worlds(seed=shard_seed(a.seed, rank), n_worlds=a.worlds)
    params = {"pgs_vel": 10, "pgs_pos": 1, "substeps": 1}
    n_dyn = dynamic_bodies(ws_scenes)
    config = {"workload": WORKLOAD, "worlds": a.worlds, "bodies_per_world": "log-uniform [8, 512]",
              "dynamic_bodies": n_dyn, "dt": 1 / 60, "substeps": 1, "pgs": [10, 1, 1],
              "scenes": "box pyramids (base 4-16) and random-hull piles (8-32 vertices), own plate per world",
              "seed": a.seed, "parallelism": f"world-sharded x{world_size}" if world_size > 1 else "single GPU"}
    threads = max(1, os.cpu_count() or 1)

    if a.impl == "reference":
        if rank != 0:
            return
        bsps, sample, wall = run_reference_sample(ws_scenes, a.warmup, a.steps, a.cpu_budget_s, threads)
        line = {"impl": "reference", "metric": METRIC, "value": bsps, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": config,
                "cpu_baseline": {"value": bsps, "unit": UNIT, "cores": threads, "kind": "reference", "sample": sample},
                "e2e": {"value": bsps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import constraintphysics_gb300 as cg
    if world_size > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    worlds = build_worlds(ws_scenes, cg.world)
    batch = cg.Batch(worlds)
    setup_s = time.perf_counter() - t_setup

    def barrier():
        if world_size > 1:
            import torch.distributed as dist
            dist.barrier()

    batch.step(a.warmup)
    # the autotuner chooses the schedule from the warmed-up state (its trial
    # steps are undone: the timed steps continue from the same state)
    t_tune = time.perf_counter()
    if a.tune_steps > 0 and not a.profile_only:
        batch.tune(a.tune_steps)
    schedule = dict(batch.schedule(), tune_s=time.perf_counter() - t_tune)
    if a.profile_only:
        batch.step(a.steps)
        print(json.dumps({"profile_only": True, "steps": a.steps, "warmup": a.warmup}), flush=True)
        return
    sampler = ClockSampler(local_rank)
    barrier()
    dev_ms = batch.step_timed(a.steps)
    barrier()
    # end to end through the C ABI with pinned host buffers, on the steps
    # right after the timed ones (the scenes' later steps carry more
    # contacts, so the two numbers are taken on neighbouring states)
    try:
        import torch
        host = torch.empty((batch.n_bodies, 16), dtype=torch.float32, pin_memory=True)
        host_desc = "pinned"
    except Exception:
        host = np.empty((batch.n_bodies, 16), dtype=np.float32)
        host_desc = "pageable"
    batch.read_state(host)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        batch.write_state(host)
        batch.step(1)
        batch.read_state(host)
    e2e_s = time.perf_counter() - t0
    # per-step latency distribution over another `steps` steps
    lat = [batch.step_timed(1) for _ in range(a.steps)]
    # per-stage device times over another `steps` steps launched stage by
    # stage with CUDA events on every part's stream (one step at a time, the
    # parts concurrent): each stage's time is the union of the parts'
    # intervals in it
    stage_ms, counts = batch.profile(a.steps)
    clocks = sampler.stop()
    # FP64 momentum / energy audit: steps with the audit kernel at the end of
    # each, interleaved with steps without it for its cost, then --steps
    # audited steps for the report
    plain_ms = audit_ms = 0.0
    for _ in range(5):
        plain_ms += batch.step_timed(2)
        batch.set_audit(True)
        audit_ms += batch.step_timed(2)
        batch.set_audit(False)
    batch.set_audit(True)
    batch.step(a.steps)
    av = batch.read_audit()
    batch.set_audit(False)
    audit = {"steps": int(av[0, 9]), "ms_per_step_added": (audit_ms - plain_ms) / 10,
             "total_kinetic_J": float(av[:, 6].sum()), "total_potential_J": float(av[:, 7].sum()),
             "max_step_energy_gain_J": float(av[:, 8].max()),
             "worlds_gaining_energy": int((av[:, 8] > 1e-6 * (np.abs(av[:, 6]) + np.abs(av[:, 7]) + 1.0)).sum()),
             "note": "per world, FP64 sums over the FP32 state after every step (cpgpu_batch_set_audit); "
                     "max_step_energy_gain_J is the largest one-step increase of kinetic + potential energy"}
    info = batch.info()
    # whole job: the units every rank processed over the slowest rank's time
    (dev_ms, e2e_s), (n_dyn_all, contacts_all) = across_ranks(world_size, [dev_ms, e2e_s], [n_dyn, info["contacts"]])
    value = n_dyn_all * a.steps / (dev_ms / 1e3)
    state_bytes = batch.n_bodies * 64
    e2e = {"value": n_dyn_all * a.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": state_bytes,
           "d2h_bytes_per_step": state_bytes, "host_buffers": host_desc,
           "call": "cpgpu_batch_write_state + cpgpu_batch_step + cpgpu_batch_read_state per step",
           "steps": "the --steps steps right after the timed ones"}

    stage_ms = {k: v / a.steps for k, v in stage_ms.items()}
    dominant = max(stage_ms, key=stage_ms.get)
    vfe = hull_sizes(ws_scenes)
    peak, peak_kind = measured_peaks()
    roof = None
    for stage in [dominant] + [s for s in ("pgs", "narrowphase") if s != dominant]:
        b = algorithmic_bytes(stage, counts, batch.n_bodies, vfe, params)
        if b is not None:
            achieved = b / (stage_ms[stage] / 1e3) / 1e9
            roof = {"bound": "hbm", "kernel": stage, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_kind": peak_kind, "traffic": measured_traffic(stage, a.worlds),
                    "algorithmic_bytes_per_launch": b, "launch_ms": stage_ms[stage],
                    "note": ("dominant stage (k_pgs_big with k_pgs_small beside it, every part); launch_ms is the "
                             "time some part spends in it per step (union of the parts' intervals), CUDA events "
                             "on every part's stream over --steps steps")
                    if stage == dominant else f"dominant stage {dominant} has no byte model"}
            break

    # plain single-world path on an evenly spaced sample of the same worlds
    plain = None
    if a.plain_sample > 0:
        step = max(1, a.worlds // a.plain_sample)
        pw = build_worlds([ws_scenes[i] for i in range(0, a.worlds, step)][: a.plain_sample], cg.world)
        total_bs, total_ms = 0, 0.0
        for w, i in zip(pw, range(0, a.worlds, step)):
            b1 = cg.Batch([w])
            b1.step(a.warmup)
            total_ms += b1.step_timed(a.steps)
            total_bs += (ws_scenes[i].n_bodies - 1) * a.steps
            b1.close()
        plain = total_bs / (total_ms / 1e3)

    serving = None
    launches = batch.launches_per_step() * a.steps
    batch_bodies = batch.n_bodies
    if a.serve_seconds > 0 and rank == 0:
        batch.close()
        serving = run_serving(cg, [float(r) for r in a.serve_rates.split(",") if r], a.serve_seconds, a.seed)

    cpu = None
    if not a.no_cpu and rank == 0:
        bsps, sample, wall = run_reference_sample(ws_scenes, a.warmup, a.steps, a.cpu_budget_s, threads)
        cpu = {"value": bsps, "unit": UNIT, "cores": threads, "kind": "reference", "sample": sample,
               "drift_300": measure_drift(cg, ws_scenes)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": dev_ms / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes)",
                "config": config,
                "l2": "state larger than L2 (%.0f MB resident)" % (batch_bodies * 600 / 1e6),
                "contacts": info["contacts"],
                "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
                "contacts_per_s": contacts_all / (dev_ms / a.steps / 1e3),
                "plain": {"value": plain, "unit": UNIT, "sample_worlds": a.plain_sample,
                          "vs_plain": (value / world_size / plain) if plain else None},
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks, "audit": audit,
                "gpu_launches": launches, "schedule": schedule,
                "stage_ms": stage_ms, "counts": counts, "setup_s": setup_s, "serving": serving}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
