"""Benchmark: agent-steps/s of the plain per-frame pipeline (sort -> cell ranges -> physics).

Default workload (one GPU): 1,048,576 spheres, N = 1024 cells per side, uniform
positions, N(0, 1) m/s velocities, rigid response, dt = 1/60 (runs as 0.016).
A "step" is one frame of the pipeline over the whole scene.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload P-1M|P-small|P-4M|batch|serving|sort|segments|render]
                    [--cpu-seconds S] [--sort rank|counting|onesweep]
                    [--tuning field=value,...]

``--sort`` / ``--tuning`` set the world workloads' mb_tuning (default: the
library's, rank placement); the JSON line's config names the sort used.

Timing: W untimed frames, then K frames, each bracketed by CUDA events on the
world's stream; L2 is flushed (a 256 MB write, then a 256 MB read so that no dirty
flush lines are left to write back) before every timed frame, outside
the events.  Per-stage times come from the library's own event nodes inside the
frame graph.  ``e2e`` goes through the public API with host buffers: upload the
scene from pinned memory, run INIT + F frames, download the state.

Under torchrun (N > 1) every rank runs its own independent scene (weak scaling,
no collective on the data path); only the barrier and the max over ranks of the
elapsed time use torch.distributed.

``--impl reference`` times the CPU restatement of the reference pipeline (the
oracle; the reference itself is Rust + wgpu and cannot run here) on the host
cores, same workload, same metric.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# Algorithmic bytes per agent and frame (each array touched once; neighbour and
# cell-table gathers counted as cache hits):
#   physics: read own state 32 + perm 4, write state 32 + key 4      = 72 B/agent
#   sort:    3 x (8 read + 8 write) + histogram read 4                = 52 B/agent
#   cells:   read sorted keys 4 + write start/close 8                 = 12 B/agent, + 4 B/cell
PHYSICS_BYTES_PER_AGENT = 72
FRAME_BYTES_PER_AGENT = 136
FRAME_BYTES_PER_CELL = 4
SORTS = {"counting": 0, "onesweep": 1, "rank": 2}  # mb_tuning.sort_algorithm


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str, workload: str):
    """DRAM bytes per launch from a committed ncu summary, or None."""
    f = ROOT / "profiles" / f"{kernel}_{workload}.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle_run(scene, frames_budget_s: float, max_frames: int | None = None, threads: int | None = None):
    """Time the oracle (CPU restatement) on the scene: INIT untimed, then LOOP frames
    until the time budget is spent.  Returns (agent-steps/s, frames, seconds, threads)."""
    import oracle

    threads = threads or oracle.hardware_threads()
    ow = oracle.OracleWorld(scene.plugin.to_c(), threads=threads)
    ow.set_state(scene.pos_scale, scene.vfme)
    ow.step(1)  # INIT frame
    frames, t0 = 0, time.perf_counter()
    while True:
        ow.step(1)
        frames += 1
        el = time.perf_counter() - t0
        if el >= frames_budget_s or (max_frames is not None and frames >= max_frames):
            break
    ow.close()
    return scene.n * frames / el, frames, el, threads


def workload_desc(name, sc):
    p = sc.plugin
    return (f"{name}: {sc.n:,} spheres, N={p.number_of_grids_one_dimension}, grid_size={p.grid_size}, "
            f"H={p.half_map_height}, {'spring' if p.enable_spring else 'rigid'}, dt=1/60 (runs 0.016)")


def run_reference(args, rank, world_size):
    """CPU restatement of the reference pipeline on the host cores (the oracle port)."""
    if rank != 0:
        return 0
    from bevy_millions_ball_gb300 import scenes

    sc = scenes.workload(args.workload)
    import oracle

    threads = oracle.hardware_threads()
    ow = oracle.OracleWorld(sc.plugin.to_c(), threads=threads)
    ow.set_state(sc.pos_scale, sc.vfme)
    ow.step(1)  # INIT
    for _ in range(args.warmup):
        ow.step(1)
    budget = args.reference_seconds
    times = []
    t_all = time.perf_counter()
    for k in range(args.steps):
        t0 = time.perf_counter()
        ow.step(1)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > budget:
            break
    total = sum(times)
    v = sc.n * len(times) / total
    sample = (f"{len(times)} of {args.steps} requested frames of the full scene (time budget {budget:.0f} s), "
              f"{threads} threads")
    line = {
        "impl": "reference", "metric": "agent-steps/s", "value": v, "unit": "agent-steps/s",
        "n_gpus": world_size, "steps": len(times), "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_desc(args.workload, sc), "n": sc.n, "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": "agent-steps/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "agent-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference is Rust + wgpu (no Rust toolchain or graphics stack here): timed its CPU restatement",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, rank, world_size, local_rank):
    import numpy as np
    import torch

    from bevy_millions_ball_gb300 import World, scenes

    torch.cuda.set_device(local_rank)
    dist = None
    if world_size > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    sc = scenes.workload(args.workload, seed=rank)
    n = sc.n
    p = sc.plugin
    cells = p.number_of_grids_one_dimension ** 2
    stream = torch.cuda.current_stream()
    w = World(p, stream=stream.cuda_stream)
    if args.sort != "default":
        w.set_tuning(sort_algorithm=SORTS[args.sort])
    if args.tuning:
        w.set_tuning(**{k: int(v) for k, v in (kv.split("=") for kv in args.tuning.split(","))})
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    flush_read = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB

    def flush_l2():
        # write 256 MB, then read 256 MB: L2 (129 MB) ends up holding clean lines of
        # the read buffer, so the frame neither hits in L2 nor pays for writing the
        # flush's dirty lines back to HBM
        flush.zero_()
        flush_read.amax()

    w.set_state(sc.pos_scale, sc.vfme)
    w.step(1)  # INIT frame
    for _ in range(max(args.warmup, 3)):
        w.step(1)
    w.sync()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    smi_index = int(vis.split(",")[local_rank]) if vis and vis.split(",")[0].isdigit() else local_rank
    with ClockSampler(smi_index) as clocks:
        for k in range(args.steps):
            flush_l2()
            ev[k][0].record(stream)
            w.step(1)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    w.sync()
    if dist:
        dist.barrier()
    per = np.array([a.elapsed_time(b) for a, b in ev])  # ms
    total_ms = float(per.sum())
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())

    # stage split (sort / cell offsets / physics kernel durations): event nodes inside
    # the frame graph cost a few microseconds each, so they run in a second pass of
    # the same frames right after the timed region, not inside it
    prof_frames = min(args.steps, 200)
    stage = np.zeros((prof_frames, 3))
    prof_ms = 0.0
    w.set_profiling(True)
    for k in range(prof_frames):
        flush_l2()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        w.step(1)
        b.record(stream)
        stage[k] = w.last_frame_times()  # waits for this frame
        prof_ms += a.elapsed_time(b)
    w.set_profiling(False)
    value = world_size * n * args.steps / (total_ms * 1e-3)
    kernels = w.kernels_per_frame
    # candidate pairs the physics pass tests per frame (the last profiled frame's cell ranges)
    from bevy_millions_ball_gb300 import stats as mbstats
    dbg = w.debug()
    pair_tests = mbstats.candidate_tests(dbg["start"], dbg["close"], p.number_of_grids_one_dimension)

    # e2e through the public API with host buffers (pinned)
    e2e = None
    if rank == 0 or world_size > 1:
        F = args.e2e_frames
        pin_p = torch.from_numpy(sc.pos_scale).pin_memory()
        pin_q = torch.from_numpy(sc.vfme.view(np.int32)).pin_memory()
        out_p = torch.empty_like(pin_p).pin_memory()
        out_q = torch.empty_like(pin_q).pin_memory()
        lib = w._lib

        def job():
            w._check(lib.mb_set_state(w._h, pin_p.data_ptr(), pin_q.data_ptr(), 0))
            w.step(1 + F)
            w._check(lib.mb_get_state(w._h, out_p.data_ptr(), out_q.data_ptr(), 0))

        job()
        reps = max(3, args.e2e_reps)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            job()
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        e2e = {"value": world_size * n * F * reps / el, "unit": "agent-steps/s",
               "h2d_bytes_per_step": int(pin_p.numel() * 4 + pin_q.numel() * 4),
               "d2h_bytes_per_step": int(out_p.numel() * 4 + out_q.numel() * 4),
               "frames_per_step": F,
               "what": f"per step: upload {n:,} spheres from pinned host memory, INIT + {F} frames, download state"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        w.close()
        return 0

    hbm, peak_kind = peaks()
    phys_ms = float(stage[:, 2].mean())
    phys_bytes = PHYSICS_BYTES_PER_AGENT * n
    achieved = phys_bytes / (phys_ms * 1e-3) / 1e9
    frame_bytes = FRAME_BYTES_PER_AGENT * n + FRAME_BYTES_PER_CELL * cells
    roofline = {
        "bound": "hbm", "kernel": "k_physics_frame", "achieved": achieved, "peak": hbm, "unit": "GB/s",
        "frac": achieved / hbm, "peak_kind": peak_kind,
        "traffic": ncu_traffic("k_physics_frame", args.workload),
        "traffic_from": f"profiles/k_physics_frame_{args.workload}.txt (one ncu capture; its header names the frame)",
        "algorithmic_bytes_per_launch": phys_bytes,
        "frame": {"algorithmic_bytes": frame_bytes,
                  "achieved_gbs": frame_bytes / (total_ms / args.steps * 1e-3) / 1e9,
                  "frac": frame_bytes / (total_ms / args.steps * 1e-3) / 1e9 / hbm},
    }
    # pair-test rate of the physics pass against an issue ceiling: one candidate
    # test is at least 10 lane-instructions (3 differences, the squared distance
    # in 3 multiply/FMA steps, the bound FMA, compare, mask), and an SM issues 4
    # warp-instructions (128 lane-instructions) per clock
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    sm_mhz = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("sm_max_mhz", 2070.0)) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else 2070.0
    test_ceiling = props.multi_processor_count * 128 * sm_mhz * 1e6 / 10.0
    pairs = {"tests_per_frame": pair_tests, "tests_per_sphere": pair_tests / n,
             "achieved_per_s": pair_tests / (phys_ms * 1e-3), "ceiling_per_s": test_ceiling,
             "frac": pair_tests / (phys_ms * 1e-3) / test_ceiling,
             "how": "candidate pairs of the 3 x 3 cell neighbourhoods from the last profiled frame's cell "
                    "ranges, over the physics kernel's mean event time; ceiling = SMs x 128 lane-instructions "
                    "per clock x max SM clock / 10 lane-instructions per test"}
    cpu = None
    if world_size == 1 and not args.no_cpu_baseline:
        v, frames, el, thr = cpu_oracle_run(sc, args.cpu_seconds)
        v1, frames1, el1, _ = cpu_oracle_run(sc, max(args.cpu_seconds / 4.0, 1.0), threads=1)
        cpu = {"value": v, "unit": "agent-steps/s", "cores": thr, "kind": "port",
               "sample": f"{frames} LOOP frames of the same {n:,}-sphere scene ({el:.1f} s wall), oracle, {thr} threads",
               "one_thread": {"value": v1, "sample": f"{frames1} LOOP frames ({el1:.1f} s wall), 1 thread"}}
    line = {
        "metric": "agent-steps/s", "value": value, "unit": "agent-steps/s", "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": workload_desc(args.workload, sc), "n": n, "grids": p.number_of_grids_one_dimension,
                   "cells": cells, "parallelism": f"replicas{world_size}" if world_size > 1 else "single",
                   "l2": "flushed before every timed frame (256 MB write then 256 MB read, outside the events)",
                   "digit_bits_max": w.tuning.digit_bits_max, "collide_block": w.tuning.collide_block,
                   "sort_algorithm": {v: k for k, v in SORTS.items()}[w.tuning.sort_algorithm],
                   "scatter_agents": max(w.tuning.scatter_agents, 1)},
        "stages_ms": {"sort": float(stage[:, 0].mean()), "cells": float(stage[:, 1].mean()),
                      "physics": phys_ms, "frames": prof_frames,
                      "ms_per_step_with_stage_events": prof_ms / prof_frames,
                      "how": "CUDA events inside the frame graph, on the world's stream, in a second pass of "
                             f"{prof_frames} frames right after the timed region"},
        "roofline": roofline,
        "pair_tests": pairs,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(kernels * args.steps),
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    w.close()
    if dist:
        dist.destroy_process_group()
    return 0


def run_batch(args, rank=0, world_size=1, local_rank=0):
    """Batching workload: independent scenes (log-uniform sizes) stepped together vs one at a time.
    Under N ranks every rank steps its own share of the scenes (sharding.partition_by_size) on its
    own GPU; nothing is exchanged but the timing (max over ranks)."""
    import numpy as np
    import torch

    from bevy_millions_ball_gb300 import Batch, World, scenes
    from bevy_millions_ball_gb300.sharding import my_scenes

    torch.cuda.set_device(local_rank)
    dist = None
    if world_size > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    all_scs = scenes.batch(count=args.batch_scenes, seed=0)
    mine = my_scenes([s.n for s in all_scs], rank, world_size)
    scs = [all_scs[i] for i in mine]
    total = sum(s.n for s in all_scs)
    stream = torch.cuda.current_stream()
    K = args.steps
    b = Batch([s.plugin for s in scs], stream=stream.cuda_stream)
    for i, s in enumerate(scs):
        b.set_state(i, s.pos_scale, s.vfme)
    b.step(1 + max(args.warmup, 3))
    b.sync()
    # frames per graph launch and physics tile from the batch autotuner (states restored)
    tuned = b.autotune(frames=8)
    b.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    b.step(K)
    e1.record(stream)
    b.sync()
    t_batch = e0.elapsed_time(e1) * 1e-3
    if dist:
        t = torch.tensor([t_batch], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_batch = float(t.item())
    mem = b.memory()
    b.close()
    # the plain loop: each scene in its own world, one after the other
    worlds = []
    for s in scs:
        w = World(s.plugin, stream=stream.cuda_stream)
        w.set_state(s.pos_scale, s.vfme)
        w.step(1 + max(args.warmup, 3))
        worlds.append(w)
    torch.cuda.synchronize()
    e0.record(stream)
    for w in worlds:
        w.step(K)
    e1.record(stream)
    torch.cuda.synchronize()
    t_plain = e0.elapsed_time(e1) * 1e-3
    for w in worlds:
        w.close()
    if dist:
        t = torch.tensor([t_plain], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_plain = float(t.item())
        dist.destroy_process_group()
    if rank != 0:
        return 0
    sizes = np.array([s.n for s in all_scs])
    line = {
        "metric": "agent-steps/s (batched scenes)", "value": total * K / t_batch, "unit": "agent-steps/s",
        "n_gpus": world_size, "steps": K, "warmup": args.warmup, "ms_per_step": 1e3 * t_batch / K,
        "higher_is_better": True, "scaling": "strong" if world_size > 1 else "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batch: {len(scs)} scenes, n log-uniform [1024, 262144], total {total:,} spheres, "
                               "N = next_pow2(sqrt n), H in {4,8,16}, e in [0.5,0.95], half spring",
                   "spheres_total": int(total), "median_scene": int(np.median(sizes)), "pool_bytes": int(mem),
                   "tuning": dict(tuned["best"], how="mb_batch_autotune, 8 frames per candidate"),
                   "l2": "pool larger than L2",
                   "parallelism": f"scene shards x{world_size} (no collective)" if world_size > 1 else "single"},
        "plain_loop": {"value": total * K / t_plain, "ms_per_step": 1e3 * t_plain / K,
                       "what": "same scenes, each in its own world, stepped one after the other"},
        "speedup_vs_plain_loop": t_plain / t_batch,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_sort(args):
    """Stage workload: mb_sort_and_hash (stable sort of u32 cell keys with iota values, then the
    start/close cell tables) on 2^24 random keys over 2^24 cells, the reference's largest
    hashing known-answer size (src/physics/spatial_hashing.rs:536-632)."""
    import numpy as np
    import torch

    from bevy_millions_ball_gb300 import SortPlan

    torch.cuda.set_device(0)
    n = cells = 1 << 24
    plan = SortPlan(max_keys=n, max_cells=cells)
    keys_np = np.random.default_rng(0).integers(0, cells, n).astype(np.uint32)
    keys = torch.from_numpy(keys_np.view(np.int32)).cuda()
    sk = torch.empty(n, dtype=torch.int32, device="cuda")
    sv = torch.empty_like(sk)
    st = torch.empty(cells, dtype=torch.int32, device="cuda")
    cl = torch.empty_like(st)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    run = lambda: plan.run(keys.data_ptr(), None, n, cells, sk.data_ptr(), sv.data_ptr(), st.data_ptr(),
                           cl.data_ptr(), stream.cuda_stream)
    for _ in range(max(args.warmup, 3)):
        run()
    torch.cuda.synchronize()
    assert np.array_equal(sk.cpu().numpy().view(np.uint32), np.sort(keys_np))
    K = min(args.steps, 50)
    total = 0.0
    for _ in range(K):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run()
        b.record(stream)
        torch.cuda.synchronize()
        total += a.elapsed_time(b)
    plan.close()
    ms = total / K
    hbm, peak_kind = peaks()
    # byte model: histogram read 4, 3 passes x (8 read + 8 write), sorted keys read 4, start/close
    # write 8 per key, offsets write 4 per cell
    model = 4 * n + 3 * 16 * n + 4 * n + 8 * cells + 4 * cells
    achieved = model / (ms * 1e-3) / 1e9
    line = {
        "metric": "keys/s (stable sort + cell ranges)", "value": n / (ms * 1e-3), "unit": "keys/s", "n_gpus": 1,
        "steps": K, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "stage: 16,777,216 uniform random keys < 2^24, iota values, 2^24 cells, 3 x 8-bit passes",
                   "l2": "flushed before every timed call (256 MB write, outside the events)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "model_bytes": model},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_serving(args):
    """Serving workload: Poisson arrivals of create / advance(k) requests; latency p50/p99."""
    import math
    import threading as th

    import numpy as np
    import torch

    from bevy_millions_ball_gb300 import Server, World, scenes

    torch.cuda.set_device(0)
    rng = np.random.default_rng(1)
    R, rate = args.serve_requests, args.serve_rate
    # request stream: the first creates, then 25% creates / 75% advances
    reqs, n_scenes = [], 0
    t = 0.0
    for r in range(R):
        t += rng.exponential(1.0 / rate)
        if n_scenes < 4 or rng.random() < 0.25:
            n = int(round(math.exp(rng.uniform(math.log(4096), math.log(1 << 20)))))
            grids = scenes.next_pow2(math.isqrt(n - 1) + 1)
            sc = scenes.plain_uniform(n, grids, half_map_height=int(rng.choice([4, 8, 16])),
                                      seed=int(rng.integers(0, 2**31)), spring=bool(rng.integers(0, 2)),
                                      e=float(rng.uniform(0.5, 0.95)))
            reqs.append(("create", t, sc))
            n_scenes += 1
        else:
            reqs.append(("advance", t, int(rng.integers(0, n_scenes)), int(rng.integers(1, 65))))
    # batched server
    srv = Server(budget_bytes=120 << 30, max_scenes=max(64, n_scenes))
    lat = [None] * R
    handles = {}
    ids = [None] * R
    t0 = time.perf_counter()
    for i, rq in enumerate(reqs):
        now = time.perf_counter() - t0
        if rq[1] > now:
            time.sleep(rq[1] - now)
        if rq[0] == "create":
            handles[len(handles)], ids[i] = srv.create(rq[2].plugin, rq[2].pos_scale, rq[2].vfme)
        else:
            ids[i] = srv.advance(handles[rq[2]], rq[3])
    for i in range(R):
        lat[i] = srv.wait(ids[i])
    t_end = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    serve_value = st.agent_steps / t_end
    # plain loop: the same stream served one request at a time, each scene its own world
    worlds, plain_lat, clock, steps_done = {}, [], 0.0, 0
    stream = torch.cuda.current_stream()
    tp0 = time.perf_counter()
    for rq in reqs:
        clock = max(clock, rq[1])
        s0 = time.perf_counter()
        if rq[0] == "create":
            w = World(rq[2].plugin, stream=stream.cuda_stream)
            w.set_state(rq[2].pos_scale, rq[2].vfme)
            w.step(1)
            worlds[len(worlds)] = w
        else:
            w = worlds[rq[2]]
            w.step(rq[3])
            steps_done += w.n * rq[3]
        torch.cuda.synchronize()
        clock += time.perf_counter() - s0
        plain_lat.append(clock - rq[1])
    t_plain = clock
    for w in worlds.values():
        w.close()
    line = {
        "metric": "agent-steps/s (serving)", "value": serve_value, "unit": "agent-steps/s", "n_gpus": 1,
        "steps": R, "warmup": 0, "ms_per_step": 1e3 * t_end / R, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"serving: {R} Poisson requests at {rate}/s, creates n log-uniform "
                               "[4096, 1048576], advances k ~ U{1..64}, 120 GB budget",
                   "scenes": n_scenes},
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "busy": {"value": st.agent_steps / max(st.busy_seconds, 1e-9), "seconds": st.busy_seconds,
                 "what": "agent-steps over the time the server's worker had frames on the GPU"},
        "plain_loop": {"value": steps_done / t_plain,
                       "latency_s": {"p50": float(np.percentile(plain_lat, 50)),
                                     "p99": float(np.percentile(plain_lat, 99))},
                       "what": "same request stream served one at a time, each scene in its own world"},
        "speedup_vs_plain_loop": serve_value / (steps_done / t_plain),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_segments(args):
    """Stage workload: mb_assemble_segments (segment starts, key->segment map and
    count) over 16,777,216 sorted keys drawn uniformly below 2^24 (sorted once by
    the stage sort, outside the timing); the reference's segment assembly
    (src/physics/assemble_segs.rs:314-430) at its largest hashing-test size."""
    import numpy as np
    import torch

    from bevy_millions_ball_gb300 import SortPlan

    torch.cuda.set_device(0)
    n = cells = 1 << 24
    plan = SortPlan(max_keys=n, max_cells=cells)
    keys_np = np.random.default_rng(0).integers(0, cells, n).astype(np.uint32)
    keys = torch.from_numpy(keys_np.view(np.int32)).cuda()
    sk = torch.empty(n, dtype=torch.int32, device="cuda")
    sv = torch.empty_like(sk)
    segs = torch.empty(n, dtype=torch.int32, device="cuda")
    kmap = torch.empty(cells, dtype=torch.int32, device="cuda")
    num = torch.empty(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    plan.run(keys.data_ptr(), None, n, cells, sk.data_ptr(), sv.data_ptr(), None, None, stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    run = lambda: plan.assemble_segments(sk.data_ptr(), n, segs.data_ptr(), kmap.data_ptr(), num.data_ptr(),
                                         stream.cuda_stream)
    for _ in range(max(args.warmup, 3)):
        run()
    torch.cuda.synchronize()
    sorted_np = np.sort(keys_np)
    starts = np.flatnonzero(np.r_[True, sorted_np[1:] != sorted_np[:-1]]).astype(np.uint32)
    m = int(num.cpu().numpy()[0])
    assert m == starts.size and np.array_equal(segs[:m].cpu().numpy().view(np.uint32), starts)
    K = min(args.steps, 50)
    total = 0.0
    for _ in range(K):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run()
        b.record(stream)
        torch.cuda.synchronize()
        total += a.elapsed_time(b)
    plan.close()
    ms = total / K
    hbm, peak_kind = peaks()
    # byte model: sorted keys read once (4 B/key), segment start and map entry written (8 B/segment)
    model = 4 * n + 8 * m
    achieved = model / (ms * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:  # the same assembly restated in numpy, one thread
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < min(args.cpu_seconds, 10.0) or reps == 0:
            st = np.flatnonzero(np.r_[True, sorted_np[1:] != sorted_np[:-1]])
            km = np.empty(cells, np.uint32)
            km[sorted_np[st]] = np.arange(st.size, dtype=np.uint32)
            reps += 1
        dt = (time.perf_counter() - t0) / reps
        cpu = {"value": n / dt, "unit": "keys/s", "cores": 1, "kind": "port",
               "sample": f"{reps} numpy runs of the same 16,777,216 sorted keys, one thread"}
    line = {
        "metric": "keys/s (segment table)", "value": n / (ms * 1e-3), "unit": "keys/s", "n_gpus": 1,
        "steps": K, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"stage: 16,777,216 sorted keys, uniform below 2^24 ({m:,} segments)",
                   "l2": "flushed before every timed call (256 MB write, outside the events)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "model_bytes": model},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_render(args):
    """Headless impostor render (mb_render_topdown) of the settled 1,048,576-sphere
    scene (P-1M after 300 frames) into a 2048 x 2048 RGBA8 image + height map in
    device memory, the whole 1024 x 1024 map in view."""
    import ctypes as C

    import numpy as np
    import torch

    from bevy_millions_ball_gb300 import World, scenes
    from bevy_millions_ball_gb300._abi import MB_DEVICE

    torch.cuda.set_device(0)
    sc = scenes.workload("P-1M")
    stream = torch.cuda.current_stream()
    W = H = 2048
    w = World(sc.plugin, stream=stream.cuda_stream)
    w.set_state(sc.pos_scale, sc.vfme)
    w.step(300)
    w.sync()
    img = torch.empty(W * H, dtype=torch.int32, device="cuda")
    hmap = torch.empty(W * H, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    run = lambda: w._check(w._lib.mb_render_topdown(w._h, W, H, -512.0, -512.0, 512.0, 512.0, img.data_ptr(),
                                                    hmap.data_ptr(), MB_DEVICE))
    for _ in range(max(args.warmup, 3)):
        run()
    torch.cuda.synchronize()
    K = min(args.steps, 50)
    total = 0.0
    for _ in range(K):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run()
        b.record(stream)
        torch.cuda.synchronize()
        total += a.elapsed_time(b)
    ms = total / K
    # the reference's own perspective view of the same state (mb_render_view), 1920 x 1080
    VW, VH = 1920, 1080
    vimg = torch.empty(VW * VH, dtype=torch.int32, device="cuda")
    vdep = torch.empty(VW * VH, dtype=torch.float32, device="cuda")
    vrun = lambda: w._check(w._lib.mb_render_view(w._h, VW, VH, None, None, 0.0, vimg.data_ptr(), vdep.data_ptr(),
                                                  MB_DEVICE))
    for _ in range(max(args.warmup, 3)):
        vrun()
    torch.cuda.synchronize()
    vtotal = 0.0
    for _ in range(K):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        vrun()
        b.record(stream)
        torch.cuda.synchronize()
        vtotal += a.elapsed_time(b)
    vms = vtotal / K
    pos, _ = w.get_state()
    s_ = w.settings
    w.close()
    hbm, peak_kind = peaks()
    px = W * H
    # byte model: spheres read once (16 B), z-buffer cleared, each covered pixel's
    # atomic max (read + write 16 B; pi r^2 pixels per sphere at 2 px per unit),
    # then per pixel the z-buffer read, the winning sphere read and 8 B written
    covered = int(sc.n * np.pi * 0.25 * (W / 1024.0) ** 2)
    model = 16 * sc.n + 8 * px + 16 * covered + px * (8 + 16 + 8)
    achieved = model / (ms * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        import oracle

        t0 = time.perf_counter()
        oracle.render_topdown(pos, W, H, -512.0, -512.0, 512.0, 512.0)
        dt = time.perf_counter() - t0
        cpu = {"value": 1.0 / dt, "unit": "images/s", "cores": 1, "kind": "port",
               "sample": "one oracle render of the same state and image size, one thread"}
        t0 = time.perf_counter()
        oracle.render_view(pos, VW, VH, s_.number_of_grids_one_dimension * s_.grid_size / 2.0,
                           2.0 * s_.half_map_height)
        vcpu = 1.0 / (time.perf_counter() - t0)
    else:
        vcpu = None
    line = {
        "metric": "images/s (headless impostor render)", "value": 1e3 / ms, "unit": "images/s", "n_gpus": 1,
        "steps": K, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "P-1M state after 300 frames, 2048 x 2048 top-down image of the whole map",
                   "l2": "flushed before every timed call (256 MB write, outside the events)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": peak_kind, "model_bytes": model},
        "cpu_baseline": cpu,
        "view": {"what": "mb_render_view: the reference camera (eye (0, 64, 64) onto the origin, 45 degrees) of "
                         "the same state, 1920 x 1080, L2 flushed before every call",
                 "images_per_s": 1e3 / vms, "ms": vms, "cpu_images_per_s_1_thread": vcpu},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="P-1M",
                    choices=["P-small", "P-1M", "P-4M", "batch", "serving", "sort", "segments", "render"])
    ap.add_argument("--batch-scenes", type=int, default=512)
    ap.add_argument("--serve-requests", type=int, default=300)
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--reference-seconds", type=float, default=120.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-frames", type=int, default=100)
    ap.add_argument("--e2e-reps", type=int, default=5)
    ap.add_argument("--sort", choices=["default", *SORTS], default="default",
                    help="frame sort of the world workloads (default: the library's)")
    ap.add_argument("--tuning", default="",
                    help="other mb_tuning fields of the world workloads, e.g. scatter_agents=2,collide_block=256")
    args = ap.parse_args()
    rank, world_size, local_rank = env_rank()
    if args.impl == "reference":
        if args.workload in ("batch", "serving", "sort", "segments", "render"):
            why = ("the reference's sort and segment passes run only as wgpu compute passes (no graphics stack "
                   "on this box)" if args.workload in ("sort", "segments") else
                   "the reference's impostor pass is a wgpu fragment shader: unavailable on this box"
                   if args.workload == "render" else
                   "the reference runs one scene per app; batching/serving have no reference implementation")
            print(json.dumps({"impl": "reference", "unavailable": why}))
            return 0
        return run_reference(args, rank, world_size)
    from __graft_entry__ import build

    build()
    if args.workload == "batch":
        return run_batch(args, rank, world_size, local_rank)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "sort":
        return run_sort(args)
    if args.workload == "segments":
        return run_segments(args)
    if args.workload == "render":
        return run_render(args)
    return run_ours(args, rank, world_size, local_rank)


if __name__ == "__main__":
    sys.exit(main())
