#!/usr/bin/env python
"""Benchmark of the chunk relight + mesh path on one GB300 (or N replicas under torchrun).

A step relights and meshes every chunk of the scale workload: 32 x 8 x 32 = 8,192 chunks of seeded
value-noise terrain with caves and glowstone (plus a ring of lit all-air chunks so each has 26
neighbours), resident in the device chunk pool. The timed form is the batched persistent
work-stealing kernel replayed as a CUDA graph; the plain one-launch-per-chunk form is timed beside
it. The default line (N = 1) adds, as sub-objects, the same measurement on the batched uneven
mixture (16,384 chunks), the edit + relight + remesh workload and the serving loop at 2k-20k
requests/s. Beside each batched workload the reference's own CPU mesher (compiled from its sources)
is timed on a seeded sample of the same chunks, and the GPU's meshes of a second seeded sample are
compared byte for byte with the reference's.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload scale|mixture|edits|serve]
                  [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

PEAKS_FILE = os.path.join(REPO, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
DESC_BYTES = 48
E2E_SETS = 3  # pools and plans in flight in the end-to-end measurement
RESULT_BYTES = 20
CPU_SAMPLE = 2048      # chunks per CPU-baseline step
CPU_SEED = 1           # step k of a CPU baseline samples with seed CPU_SEED + k (both arms)
PARITY_SAMPLE = 512    # chunks compared byte for byte with the reference's CPU mesher
PARITY_SEED = 2024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="scale", choices=["scale", "mixture", "edits", "serve"])
    ap.add_argument("--rates", default="2000,5000,10000,20000", help="serving: Poisson arrival rates (requests/s)")
    ap.add_argument("--seconds", type=float, default=3.0, help="--workload serve: trace length per rate")
    ap.add_argument("--ctas", type=int, default=4, help="serving: CTAs meshing one chunk together (1, 2, 4, 8)")
    ap.add_argument("--serve-seconds", type=float, default=1.5, help="default line: serving trace length per rate "
                                                                     "(0: no serving sub-object)")
    ap.add_argument("--size", default="", help="override grid as NXxNYxNZ (profiling runs)")
    ap.add_argument("--no-plain", action="store_true", help="skip the per-chunk form (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and the reference parity sample")
    ap.add_argument("--no-extra", action="store_true", help="default line without the mixture, edits and serving "
                                                            "sub-objects")
    ap.add_argument("--variant", default="auto", help="persistent variant: auto-tuned, or pinned by index "
                    "(profiling runs: a profiler's per-launch cost distorts the autotuner's timing)")
    return ap.parse_args()


def dims(workload, size=""):
    if size:
        return tuple(int(x) for x in size.lower().split("x"))
    return (32, 8, 32) if workload == "scale" else (32, 16, 32)


def make_world(workload, size, rank):
    from hypercraft_gb300 import worldgen
    nx, ny, nz = dims(workload, size)
    seed = worldgen.WORLD_SEED + 7919 * rank
    if workload == "scale":
        return worldgen.scale_world(nx, ny, nz, seed=seed)
    return worldgen.mixture_world(nx, ny, nz, seed=seed)


def workload_name(workload, size=""):
    nx, ny, nz = dims(workload, size)
    if workload == "scale":
        return (f"scale: {nx}x{ny}x{nz}={nx * ny * nz} chunks of seeded 2D value-noise terrain with 3D value-noise "
                f"caves (~15% of underground) and 2% glowstone torches, 5% leaves, ring of lit air chunks")
    return (f"mixture: {nx}x{ny}x{nz}={nx * ny * nz} chunks, seeded 30% air / 20% stone / 35% terrain / "
            f"10% random fill / 5% checkerboard, shuffled, ring of lit air chunks")


# DRAM bytes (read + write) of one mesher launch per default workload, each from one ncu capture
# of that launch (--metrics dram__bytes_read.sum,dram__bytes_write.sum, one pass) on the same
# source; other workloads: null.
MESH_TRAFFIC = {
    "scale:32x8x32": {"bytes": 1.644e9, "capture": "k_mesh_batch, 3rd launch of "
                      "`bench.py --steps 2 --warmup 3 --no-plain --no-e2e --no-cpu --no-extra --variant 0`"},
    "mixture:32x16x32": {"bytes": 13.563e9, "capture": "k_mesh_batch, 3rd launch of "
                         "`bench.py --workload mixture --steps 2 --warmup 3 --no-plain --no-e2e --no-cpu --no-extra "
                         "--variant 0`"},
}

# What bounds the mesher instead of DRAM, from one ncu --set full capture per workload (a
# 16 x 8 x 16 grid of the same world): issue-slot, ALU-pipe, DRAM and warp-occupancy fractions.
MESH_LIMITER = {
    "scale": {"issue_active_frac": 0.499, "alu_pipe_frac": 0.435, "dram_throughput_frac": 0.098,
              "warps_active_frac": 0.499, "capture": "ncu --set full, k_mesh_batch, scale 16x8x16"},
    "mixture": {"issue_active_frac": 0.620, "alu_pipe_frac": 0.592, "dram_throughput_frac": 0.124,
                "warps_active_frac": 0.500, "capture": "ncu --set full, k_mesh_batch, mixture 16x8x16"},
}


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.proc, self.lines = device, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()  # the sampler is running before the timed region starts
            while not self.lines and time.perf_counter() - t0 < 2.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)  # one more sample after the timed region
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------------------------ CPU leg

def cpu_runner():
    """The reference's own relight + mesher compiled from its sources (oracle/_ref), else the
    restatement, with the reason on stderr."""
    from oracle import bind
    try:
        ref = bind.reference()
    except Exception as e:  # noqa: BLE001 - a failed build is reported, then the restatement runs
        print(f"bench: the reference's CPU mesher did not build ({e}); timing the restatement", file=sys.stderr)
        ref = None
    if ref is not None:
        return ref, "reference", None
    why = "no reference sources or bundle on this host"
    print(f"bench: {why}; the CPU baseline is the restatement (oracle/hc_oracle.cpp)", file=sys.stderr)
    return bind.oracle(), "port", why


def cpu_time(runner, w, chunks, nbr, threads):
    from oracle import bind
    t0 = time.perf_counter()
    q, m = bind.mesh_many(runner, w.blocks, w.heights, nbr, threads)
    return time.perf_counter() - t0, q, m


def cpu_leg(w, chunks, nbr, arena, runner, kind, why):
    """CPU baseline on a seeded sample (all host threads, the reference client's default 3/4 of them,
    one thread) and the byte-exact check of a second seeded sample against the GPU arena."""
    from oracle import bind
    threads = os.cpu_count() or 1
    n = len(chunks)
    pick = bind.sample_positions(n, CPU_SAMPLE, CPU_SEED)
    dt, q, _ = cpu_time(runner, w, chunks[pick], nbr[pick], threads)
    ref_threads = max(1, threads * 3 // 4)  # client/src/Application.cpp:248
    dt3, _, _ = cpu_time(runner, w, chunks[pick], nbr[pick], ref_threads)
    one = pick[:min(len(pick), 64)]
    dt1, _, _ = cpu_time(runner, w, chunks[one], nbr[one], 1)
    base = {"value": len(pick) / dt, "unit": "chunks/s", "cores": threads, "kind": kind,
            "sample": f"{len(pick)} seeded random chunks (seed {CPU_SEED}) of the {n} workload chunks, "
                      f"{threads} threads, {q} quads",
            "quads_per_s": q / dt, "reference_default_threads": ref_threads,
            "chunks_per_s_at_default_threads": len(pick) / dt3,
            "single_thread_ms_per_chunk": 1e3 * dt1 / len(one)}
    if why:
        base["why_not_reference"] = why
    parity = None
    if arena is not None:
        pp = bind.sample_positions(n, PARITY_SAMPLE, PARITY_SEED)
        got = arena.sample_meshes(pp)
        want = bind.mesh_rows(runner, w.blocks, w.heights, nbr[pp], threads)
        bad = [int(i) for i, ref in zip(pp, want) if len(got[int(i)]) != len(ref)
               or not all(a == b for a, b in zip(got[int(i)], ref))]
        parity = {"byte_exact": not bad, "chunks": len(pp), "against": kind, "seed": PARITY_SEED,
                  "mismatched": bad[:8]}
        assert not bad, f"GPU meshes differ from the CPU {kind} on chunks {bad[:8]}"
    return base, parity


def reference_arm(args):
    """The reference's CPU path on the host cores: oracle/_ref, built from the reference sources (or
    from the bundle copied out of them), else the CPU restatement. Same workload, metric and seeded
    samples as the GPU arm's CPU leg."""
    from oracle import bind
    rank, world, _ = dist_setup(args)
    if rank != 0:
        return
    from hypercraft_gb300.build import build
    build()
    runner, kind, why = cpu_runner()
    w = make_world(args.workload, args.size, 0)
    chunks = w.meshable()
    nbr = w.neighbour_table(chunks)
    threads = os.cpu_count() or 1
    # a bounded amount of CPU work in all, whatever the step count
    sample = min(len(chunks), CPU_SAMPLE, max(128, 40960 // (args.warmup + args.steps)))
    times, quads = [], 0
    for step in range(args.warmup + args.steps):
        pick = bind.sample_positions(len(chunks), sample, CPU_SEED + step)
        dt, q, _ = cpu_time(runner, w, chunks[pick], nbr[pick], threads)
        if step >= args.warmup:
            times.append(dt)
            quads += q
    total = sum(times)
    value = sample * args.steps / total
    ref_threads = max(1, threads * 3 // 4)  # client/src/Application.cpp:248
    dt3, _, _ = cpu_time(runner, w, chunks[pick], nbr[pick], ref_threads)
    one = pick[:min(sample, 64)]
    dt1, _, _ = cpu_time(runner, w, chunks[one], nbr[one], 1)
    cpu = {"value": value, "unit": "chunks/s", "cores": threads, "kind": kind,
           "sample": f"{sample} seeded random chunks per step (seeds {CPU_SEED}..{CPU_SEED + args.warmup + args.steps - 1})"
                     f" of the {len(chunks)} workload chunks, {threads} threads",
           "reference_default_threads": ref_threads, "chunks_per_s_at_default_threads": sample / dt3,
           "single_thread_ms_per_chunk": 1e3 * dt1 / len(one)}
    if why:
        cpu["why_not_reference"] = why
    line = {
        "impl": "reference", "metric": "chunks/s", "value": value, "unit": "chunks/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16", "data": "synthetic",
        "config": {"workload": workload_name(args.workload, args.size), "sample_chunks_per_step": sample},
        "quads_per_s": quads / total, "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------- GPU arm

def ctypes_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


def measure_batch(args, ctx, workload, rank, world, local, *, plain=True, e2e=True, cpu=True):
    """Batched plan on one workload: throughput with the pool resident, stage times, roofline, the
    plain form, end to end through the C ABI with host buffers, and the CPU leg."""
    import torch
    from hypercraft_gb300 import batch
    dev = torch.device("cuda", local)
    size = args.size if workload == args.workload else ""
    w = make_world(workload, size, rank)
    rw = batch.upload_world(ctx, w)
    n = len(rw.chunks)
    stream = torch.cuda.Stream(device=dev)  # all work and timing events on one non-default stream
    torch.cuda.set_stream(stream)
    sp = ctypes_stream(stream)

    # size the arena from a counting run, then allocate it with a margin
    probe = batch.Arena(1, 1, n, local)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, probe, batch.PERSISTENT)
    plan.launch(sp)
    need_q, need_m, _ = plan.result(check=False)
    plan.close()
    arena = batch.Arena(int(need_q * 1.02) + 1024, int(need_m * 1.02) + 64, n, local)
    mode = batch.AUTO if args.variant == "auto" else batch.variant_mode(int(args.variant))
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena, mode)
    variant, variant_name, variant_ms = plan.variant()

    for _ in range(args.warmup):
        plan.launch(sp)
    quads, meshes, failed = plan.result()
    assert failed == 0, f"{failed} chunks failed"

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            plan.launch(sp)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    ms_total = ev0.elapsed_time(ev1)
    assert plan.result() == (quads, meshes, 0)
    ms_total = max_over_ranks(ms_total, world, dev)
    chunks_all = sum_over_ranks(n * args.steps, world, dev)
    quads_all = sum_over_ranks(quads * args.steps, world, dev)
    value = chunks_all / (ms_total / 1e3)
    ms_step = ms_total / args.steps

    # the dominant kernel alone: CUDA events recorded inside the plan's graph around its stages,
    # on the plan's stream, read after each of K further launches
    stages = np.zeros(3)
    for _ in range(args.steps):
        plan.launch(sp)
        stages += plan.stage_ms()
    stages /= args.steps
    mesh_ms = float(stages[2])
    algo_bytes = n * (65536 + 1024 + RESULT_BYTES) + 44 * quads + DESC_BYTES * meshes
    peak, peak_kind = hbm_peak()
    achieved = algo_bytes / (mesh_ms / 1e3) / 1e9
    nx, ny, nz = dims(workload, size)
    traffic = MESH_TRAFFIC.get(f"{workload}:{nx}x{ny}x{nz}") if variant == 0 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic["bytes"] if traffic else None,
                "traffic_capture": traffic["capture"] if traffic else None,
                "peak_source": f"{peak_kind} ({'MEASURED_PEAKS.json hbm_gbs' if peak_kind == 'measured' else 'fallback'})",
                "kernel": "k_mesh_cluster" if variant in (2, 3) else "k_mesh_batch", "kernel_ms": mesh_ms,
                "stage_ms": {"planes": float(stages[0]), "light_pass": float(stages[1]), "mesh": float(stages[2])},
                "algorithmic_bytes_per_launch": algo_bytes,
                "step_frac": algo_bytes / (ms_step / 1e3) / 1e9 / peak,
                "hbm_target_0p5_met": achieved / peak >= 0.5,
                "limiter": MESH_LIMITER.get(workload) if variant == 0 else None}

    # plain form: one kernel launch per chunk, same arena layout; the batched form's meshes of
    # every chunk must equal the plain form's (per-chunk counts here; bytes on the reference sample)
    plain_value = None
    if plain:
        parena = batch.Arena(arena.quad_capacity, arena.mesh_capacity, n, local)
        pplan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, parena, batch.PER_CHUNK)
        pplan.launch(sp)
        pplan.result()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        pplan.launch(sp)
        e1.record(stream)
        torch.cuda.synchronize()
        assert pplan.result() == (quads, meshes, 0)
        rb = arena.results_host(n)[:, [0, 1, 3, 4]]
        rp = parena.results_host(n)[:, [0, 1, 3, 4]]
        assert np.array_equal(rb, rp), "batched and per-chunk forms differ"
        plain_value = n / (e0.elapsed_time(e1) / 1e3)
        pplan.close()
        del parena

    # end to end through the C ABI with host buffers: every step uploads the world from pinned
    # memory, meshes it and reads every quad, mesh descriptor and per-chunk result back to pinned
    # memory. E2E_SETS pools and plans take the steps in turn on their own streams, so a step's
    # upload and download overlap the others' meshing (hc_batch_plan_download_async); the serial
    # form (one step at a time, each waited for) is reported beside it.
    e2e_line = None
    if e2e:
        hb = torch.from_numpy(w.blocks.view(np.int16)).pin_memory()
        hh = torch.from_numpy(w.heights).pin_memory()
        lib = rw.pool.lib

        def outputs():
            return (torch.empty(quads * 8, dtype=torch.int32).pin_memory(),
                    torch.empty(quads * 6, dtype=torch.int16).pin_memory(),
                    torch.empty(meshes * 12, dtype=torch.int32).pin_memory(),
                    torch.empty(n * 5, dtype=torch.int32).pin_memory())

        extra = []  # the other pools, arenas, plans and streams in flight
        for _ in range(E2E_SETS - 1):
            pool_x = batch.Pool(ctx, w.n_chunks)
            arena_x = batch.Arena(arena.quad_capacity, arena.mesh_capacity, n, local)
            plan_x = batch.BatchPlan(ctx, pool_x, rw.neighbours, arena_x, batch.variant_mode(variant))
            extra.append((pool_x, arena_x, plan_x, torch.cuda.Stream(device=dev)))
        sets = [(rw.pool, plan, sp, outputs())] + [(px, plx, ctypes_stream(stx), outputs()) for px, _, plx, stx in extra]

        def issue(k):
            pool_k, plan_k, st_k, (ov, oi, od, orr) = sets[k % len(sets)]
            ctx.check(lib.hc_pool_upload(pool_k.handle, 0, w.n_chunks, hb.data_ptr(), hh.data_ptr(), 0, st_k), "upload")
            plan_k.launch(st_k)
            ctx.check(lib.hc_batch_plan_download_async(plan_k.handle, quads, meshes, ov.data_ptr(), oi.data_ptr(),
                                                       od.data_ptr(), orr.data_ptr(), st_k), "download")

        def serial_step():
            ctx.check(lib.hc_pool_upload(rw.pool.handle, 0, w.n_chunks, hb.data_ptr(), hh.data_ptr(), 0, sp), "upload")
            plan.launch(sp)
            q, m, f = plan.result()
            ov, oi, od, orr = sets[0][3]
            ctx.check(lib.hc_batch_plan_download(plan.handle, q, m, ov.data_ptr(), oi.data_ptr(), od.data_ptr(),
                                                 orr.data_ptr()), "download")

        def timed(fn, k_steps):
            for k in range(max(1, args.warmup)):
                fn(k)
            torch.cuda.synchronize()
            barrier(world)
            t0 = time.perf_counter()
            for k in range(k_steps):
                fn(k)
            torch.cuda.synchronize()
            barrier(world)
            return max_over_ranks(time.perf_counter() - t0, world, dev)

        t_pipe = timed(issue, args.steps)
        # every set produced the whole output: the same per-chunk counts (arena placement may differ)
        for _, plan_k, _, _ in sets:
            assert plan_k.result() == (quads, meshes, 0)
        r0 = sets[0][3][3].view(-1, 5)[:, [0, 1, 3, 4]]
        assert all(torch.equal(r0, x[3][3].view(-1, 5)[:, [0, 1, 3, 4]]) for x in sets[1:]), "pipelined sets differ"
        t_serial = timed(lambda k: serial_step(), args.steps)
        e2e_line = {"value": chunks_all / t_pipe, "unit": "chunks/s",
                    "h2d_bytes_per_step": int(w.n_chunks * (65536 + 1024)),
                    "d2h_bytes_per_step": int(quads * 44 + meshes * DESC_BYTES + n * RESULT_BYTES),
                    "form": f"{E2E_SETS} pools and plans in flight on {E2E_SETS} streams: a step's copies overlap "
                            "the others' meshing",
                    "serial_value": chunks_all / t_serial}
        for pool_x, arena_x, plan_x, _ in extra:
            plan_x.close()
            pool_x.close()
        del extra, sets, hb, hh
        # the arena of set 0 holds the last step's output again (the serial steps ran last)

    cpu_line, parity = None, None
    if cpu and rank == 0:
        runner, kind, why = cpu_runner()
        cpu_line, parity = cpu_leg(w, rw.chunks, rw.neighbours, arena, runner, kind, why)

    out = {"workload": workload_name(workload, size), "chunks": n, "value": value, "unit": "chunks/s",
           "ms_per_step": ms_step, "quads_per_s": quads_all / (ms_total / 1e3), "quads_per_step": quads,
           "meshes_per_step": meshes, "plain_chunks_per_s": plain_value,
           "batched_vs_plain": (value / world / plain_value) if plain_value else None,
           "autotuned_variant": variant_name, "variant_ms": dict(zip(batch.VARIANTS, variant_ms)),
           "roofline": roofline, "e2e": e2e_line, "cpu_baseline": cpu_line, "parity_vs_cpu_sample": parity,
           "gpu_launches": args.steps * batch.launches_per_run(variant),
           "clocks": clk.summary(),
           "l2": f"inputs larger than L2: pool {w.n_chunks * 66560 / 1e6:.0f} MB, output {(44 * quads) / 1e6:.0f} MB "
                 f"per step"}
    plan.close()
    rw.pool.close()
    del arena, plan, rw
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def edits_measure(args, ctx):
    """Edit workload: 4,096 seeded edits (half stone, half air, 10% glowstone, within 48 voxels of the
    centre) on 7 x 5 x 7 chunks of terrain; a step applies them, recomputes the sunlight heights and
    relights + remeshes every chunk they touch. The world is restored (outside the timed region)
    before each step. CPU: the reference's kMesh runner over the same remeshed chunks."""
    import torch
    from hypercraft_gb300 import batch, world as hw
    w = hw.edit_world()
    edits = hw.seeded_edits(4096, seed=7)
    rw = hw.ResidentWorld(ctx, w)
    arena = batch.Arena(4_000_000, 8192, w.n_chunks)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = ctypes_stream(stream)
    by_cluster = {}
    cells = quads = None
    for cluster in (1, 4):
        rw.set_cluster(cluster)
        times = []
        for step in range(args.warmup + args.steps):
            rw.pool.upload(0, w.blocks, w.heights, sp)
            rw.touch(sp)
            rw.remesh(arena, sp)  # nothing marked: rebuilds the restored chunks' planes only
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rw.apply_edits(edits, sp)
            cells, quads, meshes = rw.remesh(arena, sp)
            torch.cuda.synchronize()
            if step >= args.warmup:
                times.append(time.perf_counter() - t0)
        by_cluster[cluster] = {"median_ms": 1e3 * float(np.median(times)), "p99_ms": 1e3 * float(np.percentile(times, 99))}
    best = min(by_cluster, key=lambda c: by_cluster[c]["median_ms"])
    ms = by_cluster[best]["median_ms"]
    wc = hw.edit_world()
    from oracle import edits as oe
    oe.apply_edits(wc, edits)
    nbr = wc.neighbour_table(cells)
    runner, kind, why = cpu_runner()
    threads = os.cpu_count() or 1
    dt, q, _ = cpu_time(runner, wc, cells, nbr, threads)
    rw.close()
    line = {"workload": "edits: 4096 seeded edits within 48 voxels of the centre of 7x5x7 terrain chunks "
                        "(50% stone, 50% air, 10% glowstone); apply, recompute heights, relight + remesh the "
                        "touched chunks", "metric": "edits/s", "value": len(edits) / (ms / 1e3), "unit": "edits/s",
            "remesh_latency_ms": ms, "remeshed_chunks_per_step": int(len(cells)), "quads_per_step": int(quads),
            "chunks_per_s": len(cells) / (ms / 1e3), "latency_ms_by_ctas_per_chunk": by_cluster,
            "cpu_baseline": {"value": len(edits) / dt, "unit": "edits/s", "cores": threads, "kind": kind,
                             "kmesh_ms": 1e3 * dt, "sample": f"kMesh of the same {len(cells)} chunks, edit "
                                                            "application excluded"}}
    if why:
        line["cpu_baseline"]["why_not_reference"] = why
    return line


def _pct(x, q):
    return float(np.percentile(x, q)) if len(x) else None


def serve_rates(ctx, rates, seconds, ctas):
    """Replays the seeded serving trace at each rate on a fresh server; one result row per rate."""
    from hypercraft_gb300 import server as hs
    lib = hs.ChunkLibrary(16, 8, 16, seed=0x5E7E)
    rows = []
    names = {hs.REQ_EDIT: "edit", hs.REQ_FILL: "fill", hs.REQ_LOAD: "load", hs.REQ_UNLOAD: "unload"}
    # warm-up (not reported): a short trace on a throwaway server, so that one-time costs of the
    # process (the first launches of each kernel, first-use allocations) fall outside every rate
    wl = hs.ServingWorkload(lib, seed=1)
    init = wl.initial_loads()
    reqs, times = wl.trace(rates[0], 0.3)
    srv = hs.Server(ctx, wl.grid, wl.origin, pool_capacity=0, tick_us=1000, depth=3, max_edits_per_tick=16384,
                    max_loads_per_tick=512, arena_quads=8 << 20, arena_meshes=1 << 16, ctas_per_chunk=ctas)
    srv.submit(init)
    srv.drain()
    srv.start()
    srv.replay(reqs, times)
    srv.stop()
    srv.close()
    for rate in rates:
        wl = hs.ServingWorkload(lib, seed=int(rate))
        init = wl.initial_loads()
        reqs, times = wl.trace(rate, seconds)
        srv = hs.Server(ctx, wl.grid, wl.origin, pool_capacity=0, tick_us=1000, depth=3, max_edits_per_tick=16384,
                        max_loads_per_tick=512, arena_quads=8 << 20, arena_meshes=1 << 16, ctas_per_chunk=ctas)
        srv.submit(init)
        srv.drain()
        st0 = srv.stats()
        srv.start()
        with Clocks(0) as clk:
            lat, elapsed = srv.replay(reqs, times)
        srv.stop()
        st1 = srv.stats()
        secs = elapsed / 1e9
        lat_ms = lat / 1e6
        row = {"rate": rate, "requests": int(len(reqs)), "seconds": secs,
               "requests_per_s": len(reqs) / secs,
               "chunks_per_s": (st1["chunks_remeshed"] - st0["chunks_remeshed"]) / secs,
               "quads_per_s": (st1["quads"] - st0["quads"]) / secs,
               "ticks": st1["ticks"] - st0["ticks"],
               "gpu_busy": (st1["gpu_ns_total"] - st0["gpu_ns_total"]) / elapsed,
               "gpu_ms_max_pass": (st1["gpu_ns_max"]) / 1e6,
               "requeued": st1["chunks_requeued"] - st0["chunks_requeued"],
               "pool_capacity": st1["pool_capacity"], "resident": st1["resident"],
               "p50_ms": _pct(lat_ms, 50), "p99_ms": _pct(lat_ms, 99), "clocks": clk.summary()}
        for k, name in names.items():
            sel = lat_ms[reqs["kind"] == k]
            row[f"{name}_n"] = int(len(sel))
            row[f"{name}_p50_ms"] = _pct(sel, 50)
            row[f"{name}_p99_ms"] = _pct(sel, 99)
        rows.append(row)
        srv.close()
    return rows


SERVE_DOC = ("serve: device pool sized by free HBM (at most 65,536 chunks) over a 96x32x96 chunk grid; a player "
             "takes a seeded random walk and the view sphere of radius 16 chunks stays resident; Poisson arrivals: "
             "70% single-block edits within 48 voxels of the player, 25% loads of chunks entering the view (mixture "
             "chunks), 5% 16^3 region fills; unloads of chunks leaving the view go in before the loads; 1 ms ticks, "
             "three passes in flight; latency = arrival to completion of the request's pass")


def ours(args):
    import torch
    rank, world, local = dist_setup(args)
    torch.cuda.set_device(local)
    from hypercraft_gb300.build import build
    if rank == 0:
        build()
    barrier(world)
    from hypercraft_gb300 import mesher
    ctx = mesher.Context(local)
    main = measure_batch(args, ctx, args.workload, rank, world, local, plain=not args.no_plain, e2e=not args.no_e2e,
                         cpu=not args.no_cpu)
    extra = rank == 0 and world == 1 and not args.no_extra and args.workload == "scale" and not args.size
    mixture = edits = serving = None
    if extra:
        mixture = measure_batch(args, ctx, "mixture", rank, world, local, plain=not args.no_plain,
                                e2e=not args.no_e2e, cpu=not args.no_cpu)
        edits = edits_measure(args, ctx)
        if args.serve_seconds > 0:
            rows = serve_rates(ctx, [float(r) for r in args.rates.split(",")], args.serve_seconds, args.ctas)
            head = next((r for r in rows if r["rate"] == 10000.0), rows[-1])
            serving = {"workload": SERVE_DOC, "seconds_per_rate": args.serve_seconds, "ctas_per_chunk": args.ctas,
                       "edit_p50_ms": head["edit_p50_ms"], "edit_p99_ms": head["edit_p99_ms"],
                       "p50_ms": head["p50_ms"], "p99_ms": head["p99_ms"], "at_rate": head["rate"], "rates": rows}

    if rank == 0:
        line = {
            "metric": "chunks/s", "value": main["value"], "unit": "chunks/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u16",
            "data": "synthetic: seeded worlds generated in-process (the reference publishes no benchmark data)",
            "config": {"workload": main["workload"], "chunks_per_gpu": main["chunks"],
                       "form": "batched persistent work-stealing kernel, CUDA graph",
                       "autotuned_variant": main["autotuned_variant"], "variant_ms": main["variant_ms"],
                       "parallelism": f"replicas x{world}", "l2": main["l2"]},
            "quads_per_s": main["quads_per_s"], "quads_per_step": main["quads_per_step"],
            "meshes_per_step": main["meshes_per_step"], "plain_chunks_per_s": main["plain_chunks_per_s"],
            "batched_vs_plain": main["batched_vs_plain"], "parity_vs_cpu_sample": main["parity_vs_cpu_sample"],
            "roofline": main["roofline"], "cpu_baseline": main["cpu_baseline"], "e2e": main["e2e"],
            "gpu_launches": main["gpu_launches"], "clocks": main["clocks"],
            "mixture": mixture, "edits": edits, "serving": serving,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def edits_bench(args):
    from hypercraft_gb300 import mesher
    from hypercraft_gb300.build import build
    build()
    line = edits_measure(args, mesher.Context(0))
    line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": line["remesh_latency_ms"],
                 "higher_is_better": True})
    print(json.dumps(line), flush=True)


def serve_bench(args):
    from hypercraft_gb300 import mesher
    from hypercraft_gb300.build import build
    build()
    ctx = mesher.Context(0)
    rows = serve_rates(ctx, [float(r) for r in args.rates.split(",")], args.seconds, args.ctas)
    for row in rows:
        print(json.dumps({"serve_rate": row}), flush=True)
    head = next((r for r in rows if r["rate"] == 10000.0), rows[-1])
    line = {"metric": "p99 single-edit relight+remesh latency at 10k requests/s", "value": head["edit_p99_ms"],
            "unit": "ms", "n_gpus": 1, "steps": len(rows), "warmup": 0, "ms_per_step": None,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
            "data": "synthetic: seeded serving trace (the reference publishes no benchmark data)",
            "config": {"workload": SERVE_DOC, "rates": [r["rate"] for r in rows], "seconds_per_rate": args.seconds,
                       "tick_us": 1000, "passes_in_flight": 3, "ctas_per_chunk": args.ctas},
            "rates": rows, "clocks": head["clocks"]}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "edits":
        edits_bench(args)
        return
    if args.workload == "serve":
        serve_bench(args)
        return
    if args.impl == "reference":
        reference_arm(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
