#!/usr/bin/env python
"""Benchmark of the chunk relight + mesh path on one GB300 (or N replicas under torchrun).

A step relights and meshes every chunk of the scale workload: 32 x 8 x 32 = 8,192 chunks of seeded
value-noise terrain with caves and glowstone (plus a ring of lit all-air chunks so each has 26
neighbours), resident in the device chunk pool. The timed form is the batched persistent
work-stealing kernel replayed as a CUDA graph; the plain one-launch-per-chunk form is timed beside
it. Output is byte-identical to the reference (tests/); a sample is re-checked here.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload scale|mixture] [--impl reference]
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="scale", choices=["scale", "mixture", "edits", "serve"])
    ap.add_argument("--rates", default="2000,5000,10000,20000", help="serve: Poisson arrival rates (requests/s)")
    ap.add_argument("--seconds", type=float, default=3.0, help="serve: trace length per rate")
    ap.add_argument("--ctas", type=int, default=4, help="serve: CTAs meshing one chunk together (1, 2, 4, 8)")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="default line: serving trace length (0: skip)")
    ap.add_argument("--size", default="", help="override grid as NXxNYxNZ (profiling runs)")
    ap.add_argument("--no-plain", action="store_true", help="skip the per-chunk form (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--variant", default="auto", choices=["auto", "0", "1", "2", "3"],
                    help="persistent variant: auto-tuned, or pinned (profiling runs: a profiler's per-launch cost "
                         "distorts the autotuner's timing)")
    return ap.parse_args()


def dims(args):
    if args.size:
        return tuple(int(x) for x in args.size.lower().split("x"))
    return (32, 8, 32) if args.workload == "scale" else (32, 16, 32)


def make_world(args, rank):
    from hypercraft_gb300 import worldgen
    nx, ny, nz = dims(args)
    seed = worldgen.WORLD_SEED + 7919 * rank
    if args.workload == "scale":
        return worldgen.scale_world(nx, ny, nz, seed=seed)
    return worldgen.mixture_world(nx, ny, nz, seed=seed)


def workload_name(args):
    nx, ny, nz = dims(args)
    if args.workload == "scale":
        return (f"scale: {nx}x{ny}x{nz}={nx * ny * nz} chunks of seeded 2D value-noise terrain with 3D value-noise "
                f"caves (~15% of underground) and 2% glowstone torches, 5% leaves, ring of lit air chunks")
    return (f"mixture: {nx}x{ny}x{nz}={nx * ny * nz} chunks, seeded 30% air / 20% stone / 35% terrain / "
            f"10% random fill / 5% checkerboard, shuffled, ring of lit air chunks")


# DRAM bytes (read + write) of one k_mesh_batch launch on the default scale workload, from one
# ncu capture (profiles/k_mesh_batch_scale32x8x32_dram.md gives the command); other workloads: null
MESH_TRAFFIC_BYTES = {"scale:32x8x32": 1.496e9}


def mesh_traffic(args):
    nx, ny, nz = dims(args)
    return MESH_TRAFFIC_BYTES.get(f"{args.workload}:{nx}x{ny}x{nz}")


# What bounds k_mesh_batch instead of DRAM: its instruction issue and ALU pipe utilisation from one
# ncu --set full capture of the same scale terrain at 16x8x16 (profiles/k_mesh_batch_scale16x8x16.md
# gives the command); the integer merge and light-key work keeps the SMs busy while DRAM idles.
MESH_ISSUE = {"issue_active_frac": 0.559, "alu_pipe_frac": 0.486, "dram_throughput_frac": 0.074,
              "warps_active_frac": 0.500, "source": "ncu --set full, k_mesh_batch, scale 16x8x16"}


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


def cpu_run(world_obj, chunks, nbr, runner, threads):
    from oracle import bind
    t0 = time.perf_counter()
    q, m = bind.mesh_many(runner, world_obj.blocks, world_obj.heights, nbr, threads)
    return time.perf_counter() - t0, q, m


def reference_arm(args):
    """The reference's CPU path on the host cores: oracle/_ref where it was built from the reference
    sources here, else the CPU restatement (oracle/hc_oracle.cpp)."""
    from oracle import bind
    rank, world, _ = dist_setup(args)
    if rank != 0:
        return
    import __graft_entry__  # noqa: F401
    from hypercraft_gb300.build import build
    build()
    ref = bind.reference()
    runner, kind = (ref, "reference") if ref is not None else (bind.oracle(), "port")
    w = make_world(args, 0)
    chunks = w.meshable()
    nbr = w.neighbour_table(chunks)
    threads = os.cpu_count()
    # about 40k chunks of CPU work in all, whatever the step count (~10 s on 16 cores)
    sample = min(len(chunks), 2048, max(128, 40960 // (args.warmup + args.steps)))
    rng = np.random.default_rng(1)
    times, quads = [], 0
    for step in range(args.warmup + args.steps):
        pick = np.sort(rng.choice(len(chunks), sample, replace=False))
        dt, q, _ = cpu_run(w, chunks[pick], nbr[pick], runner, threads)
        if step >= args.warmup:
            times.append(dt)
            quads += q
    total = sum(times)
    value = sample * args.steps / total
    # the reference client's own worker count (hardware_concurrency * 3 / 4, client/src/Application.cpp:248)
    # and one runner's per-chunk latency, on bounded samples of the same chunks
    ref_threads = max(1, threads * 3 // 4)
    dt3, _, _ = cpu_run(w, chunks[pick], nbr[pick], runner, ref_threads)
    one = min(sample, 128)
    dt1, _, _ = cpu_run(w, chunks[pick[:one]], nbr[pick[:one]], runner, 1)
    line = {
        "impl": "reference", "metric": "chunks/s", "value": value, "unit": "chunks/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16", "data": "synthetic",
        "config": {"workload": workload_name(args), "sample_chunks_per_step": sample},
        "quads_per_s": quads / total,
        "cpu_baseline": {"value": value, "unit": "chunks/s", "cores": threads, "kind": kind,
                         "sample": f"{sample} random chunks of the workload per step, {threads} threads",
                         "reference_default_threads": ref_threads,
                         "chunks_per_s_at_default_threads": sample / dt3,
                         "single_thread_ms_per_chunk": 1e3 * dt1 / one},
        "e2e": {"value": value, "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def ours(args):
    import torch
    rank, world, local = dist_setup(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from hypercraft_gb300.build import build
    if rank == 0:
        build()
    barrier(world)
    from hypercraft_gb300 import batch, mesher

    ctx = mesher.Context(local)
    w = make_world(args, rank)
    rw = batch.upload_world(ctx, w)
    n = len(rw.chunks)
    # all work (library calls and timing events) on one dedicated non-default stream
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sp = ctypes_stream(stream)

    # size the arena from a counting run, then allocate it with a margin
    probe = batch.Arena(1, 1, n, local)
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, probe, batch.PERSISTENT)
    plan.launch(sp)
    need_q, need_m, _ = plan.result(check=False)
    plan.close()
    arena = batch.Arena(int(need_q * 1.05) + 1024, int(need_m * 1.05) + 64, n, local)
    # the autotuner times the persistent variants on this batch and keeps the fastest
    plan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, arena,
                           batch.AUTO if args.variant == "auto" else batch.variant_mode(int(args.variant)))
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
    q2, m2, f2 = plan.result()
    assert (q2, m2, f2) == (quads, meshes, 0)
    ms_total = max_over_ranks(ms_total, world, dev)
    chunks_all = sum_over_ranks(n * args.steps, world, dev)
    quads_all = sum_over_ranks(quads * args.steps, world, dev)
    value = chunks_all / (ms_total / 1e3)
    ms_step = ms_total / args.steps

    # the dominant kernel alone: CUDA events recorded inside the plan's graph around its stages,
    # read after each of K further launches
    stages = np.zeros(3)
    for _ in range(args.steps):
        plan.launch(sp)
        stages += plan.stage_ms()
    stages /= args.steps
    mesh_ms = float(stages[2])

    algo_bytes = n * (65536 + 1024 + RESULT_BYTES) + 44 * quads + DESC_BYTES * meshes
    peak, peak_kind = hbm_peak()
    achieved = algo_bytes / (mesh_ms / 1e3) / 1e9

    # plain form: one kernel launch per chunk, same arena layout
    plain_value = None
    plain_checked = None
    if not args.no_plain:
        parena = batch.Arena(arena.quad_capacity, arena.mesh_capacity, n, local)
        pplan = batch.BatchPlan(ctx, rw.pool, rw.neighbours, parena, batch.PER_CHUNK)
        pplan.launch(sp)
        pplan.result()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        pplan.launch(sp)
        e1.record(stream)
        torch.cuda.synchronize()
        pq, pm, pf = pplan.result()
        plain_value = n / (e0.elapsed_time(e1) / 1e3)
        # byte-exact check of a sample of chunks between the two forms
        hb, hp = arena.host(), parena.host()
        rng = np.random.default_rng(3)
        sample = rng.choice(n, min(n, 256), replace=False)
        plain_checked = (pq, pm, pf) == (quads, meshes, 0) and all(
            a == b for i in sample for a, b in zip(arena.chunk_meshes(int(i), hb), parena.chunk_meshes(int(i), hp)))
        assert plain_checked, "batched and per-chunk forms differ"
        pplan.close()
        del parena

    # end to end through the C ABI with host buffers: every step uploads the world from pinned
    # memory, meshes it and reads every quad, mesh descriptor and per-chunk result back to pinned
    # memory. E2E_SETS pools and plans take the steps in turn on their own streams, so a step's
    # upload and download overlap the others' meshing (hc_batch_plan_download_async); the serial
    # form (one step at a time, each waited for) is reported beside it.
    e2e = None
    if not args.no_e2e:
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
        # both sets produced the whole output: the same per-chunk counts (arena placement may differ)
        for _, plan_k, _, _ in sets:
            assert plan_k.result() == (quads, meshes, 0)
        r0 = sets[0][3][3].view(-1, 5)[:, [0, 1, 3, 4]]
        assert all(torch.equal(r0, x[3][3].view(-1, 5)[:, [0, 1, 3, 4]]) for x in sets[1:]), "pipelined sets differ"
        t_serial = timed(lambda k: serial_step(), args.steps)
        e2e = {"value": chunks_all / t_pipe, "unit": "chunks/s",
               "h2d_bytes_per_step": int(w.n_chunks * (65536 + 1024)),
               "d2h_bytes_per_step": int(quads * 44 + meshes * DESC_BYTES + n * RESULT_BYTES),
               "form": f"{E2E_SETS} pools and plans in flight on {E2E_SETS} streams: a step's copies overlap "
                       "the others' meshing",
               "serial_value": chunks_all / t_serial}
        for pool_x, arena_x, plan_x, _ in extra:
            plan_x.close()
            pool_x.close()
        del extra

    serving = None
    if rank == 0 and world == 1 and args.serve_seconds > 0:
        rows, _ = serve_rates(ctx, [10000.0], args.serve_seconds, args.ctas)
        r = rows[0]
        serving = {"workload": "serve: seeded trace at 10,000 requests/s (70% edits, 25% view loads along a "
                               "random walk, 5% 16^3 fills), 1 ms ticks, pool sized by free HBM",
                   "edit_p50_ms": r["edit_p50_ms"], "edit_p99_ms": r["edit_p99_ms"], "p50_ms": r["p50_ms"],
                   "p99_ms": r["p99_ms"], "requests_per_s": r["requests_per_s"], "chunks_per_s": r["chunks_per_s"],
                   "seconds": r["seconds"], "ctas_per_chunk": args.ctas}

    cpu = None
    if rank == 0 and world >= 1 and not args.no_cpu:
        from oracle import bind
        sample = min(n, 2048)
        threads = os.cpu_count()
        dt, q, _ = cpu_run(w, rw.chunks[:sample], rw.neighbours[:sample], bind.oracle(), threads)
        cpu = {"value": sample / dt, "unit": "chunks/s", "cores": threads, "kind": "port",
               "sample": f"first {sample} of the {n} workload chunks, {threads} threads, {q} quads"}

    if rank == 0:
        nx, ny, nz = dims(args)
        line = {
            "metric": "chunks/s", "value": value, "unit": "chunks/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u16",
            "data": "synthetic: seeded worlds generated in-process (the reference publishes no benchmark data)",
            "config": {"workload": workload_name(args), "chunks_per_gpu": n, "form": "batched persistent "
                       "work-stealing kernel, CUDA graph", "autotuned_variant": variant_name,
                       "variant_ms": dict(zip(batch.VARIANTS, variant_ms)), "parallelism": f"replicas x{world}",
                       "l2": f"inputs larger than L2: pool {w.n_chunks * 66560 / 1e6:.0f} MB, output "
                             f"{(44 * quads) / 1e6:.0f} MB per step"},
            "quads_per_s": quads_all / (ms_total / 1e3),
            "quads_per_step": quads, "meshes_per_step": meshes,
            "plain_chunks_per_s": plain_value,
            "batched_vs_plain": (value / world / plain_value) if plain_value else None,
            "byte_exact_vs_plain_sample": plain_checked,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": mesh_traffic(args),
                         "peak_source": f"{peak_kind} ({'MEASURED_PEAKS.json hbm_gbs' if peak_kind == 'measured' else 'fallback'})",
                         "kernel": "k_mesh_batch" if variant < 2 else "k_mesh_cluster",
                         "kernel_ms": mesh_ms,
                         "stage_ms": {"planes": float(stages[0]), "light_pass": float(stages[1]),
                                      "mesh": float(stages[2])},
                         "algorithmic_bytes_per_launch": algo_bytes,
                         "issue": MESH_ISSUE if args.workload == "scale" and variant == 0 else None},
            "serving": serving,
            # per step the plan's graph runs the plane refresh, the blank test (one-CTA variants), 15 light
            # levels (light-pass variant only) and the mesher
            "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": args.steps * (18 if variant == 0 else (3 if variant == 1 else 2)),
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def edits_bench(args):
    """Edit workload: 4,096 seeded edits (half stone, half air, 10% glowstone, within 48 voxels of the
    centre) on 7 x 5 x 7 chunks of terrain; a step applies them, recomputes the sunlight heights and
    relights + remeshes every chunk they touch. The world is restored (outside the timed region)
    before each step."""
    import torch
    from hypercraft_gb300 import batch, mesher, world as hw
    from hypercraft_gb300.build import build
    from oracle import bind
    build()
    ctx = mesher.Context(0)
    w = hw.edit_world()
    edits = hw.seeded_edits(4096, seed=7)
    rw = hw.ResidentWorld(ctx, w)
    arena = batch.Arena(4_000_000, 8192, w.n_chunks)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = ctypes_stream(stream)
    by_cluster = {}
    for cluster in (1, 4):
        rw.set_cluster(cluster)
        times, cells = [], None
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
        by_cluster[cluster] = 1e3 * float(np.median(times))
    ms = min(by_cluster.values())
    # CPU: the reference's kMesh runner over the same remeshed chunks, all host cores
    wc = hw.edit_world()
    from oracle import edits as oe
    oe.apply_edits(wc, edits)
    nbr = wc.neighbour_table(cells)
    threads = os.cpu_count()
    ref = bind.reference()
    runner, kind = (ref, "reference") if ref is not None else (bind.oracle(), "port")
    dt, q, _ = cpu_run(wc, cells, nbr, runner, threads)
    line = {"metric": "edits/s", "value": len(edits) / (ms / 1e3), "unit": "edits/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "workload": "edits: 4096 seeded edits within 48 voxels of the centre of 7x5x7 terrain chunks",
            "remeshed_chunks_per_step": int(len(cells)), "quads_per_step": int(quads),
            "remesh_latency_ms": ms, "latency_ms_by_ctas_per_chunk": by_cluster,
            "cpu_baseline": {"value": len(edits) / dt, "unit": "edits/s", "cores": threads, "kind": kind,
                             "sample": f"kMesh of the same {len(cells)} chunks ({dt * 1e3:.1f} ms), edit application excluded"}}
    print(json.dumps(line), flush=True)


def _pct(x, q):
    return float(np.percentile(x, q)) if len(x) else None


def serve_rates(ctx, rates, seconds, ctas):
    """Replays the seeded serving trace at each rate on a fresh server; one result row per rate."""
    from hypercraft_gb300 import server as hs
    lib = hs.ChunkLibrary(16, 8, 16, seed=0x5E7E)
    rows, clocks = [], None
    names = {hs.REQ_EDIT: "edit", hs.REQ_FILL: "fill", hs.REQ_LOAD: "load", hs.REQ_UNLOAD: "unload"}
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
        if rate == 10000.0 or clocks is None:
            clocks = clk.summary()
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
               "p50_ms": _pct(lat_ms, 50), "p99_ms": _pct(lat_ms, 99)}
        for k, name in names.items():
            sel = lat_ms[reqs["kind"] == k]
            row[f"{name}_n"] = int(len(sel))
            row[f"{name}_p50_ms"] = _pct(sel, 50)
            row[f"{name}_p99_ms"] = _pct(sel, 99)
        rows.append(row)
        srv.close()
    return rows, clocks


def serve_bench(args):
    """Serving workload: a device pool sized by free HBM (at most 65,536 chunks) over a 96 x 32 x 96
    chunk grid; a player takes a seeded random walk and the chunks of a view sphere of radius 16
    chunks around it are resident. Poisson arrivals at each rate: 70% single-block edits within
    48 voxels of the player, 25% loads of chunks entering the view (mixture chunks: 30% air, 20%
    stone, 35% terrain, 10% random fill, 5% checkerboard), 5% 16^3 region fills; unloads of the
    chunks leaving the view go in before the loads. 1 ms ticks, three passes in flight. Latency =
    arrival to completion of the request's pass; the initial view is loaded before timing."""
    from hypercraft_gb300 import mesher
    from hypercraft_gb300.build import build
    build()
    ctx = mesher.Context(0)
    rows, clocks = serve_rates(ctx, [float(r) for r in args.rates.split(",")], args.seconds, args.ctas)
    for row in rows:
        print(json.dumps({"serve_rate": row}), flush=True)
    head = next((r for r in rows if r["rate"] == 10000.0), rows[-1])
    line = {"metric": "p99 single-edit relight+remesh latency at 10k requests/s", "value": head["edit_p99_ms"],
            "unit": "ms", "n_gpus": 1, "steps": len(rows), "warmup": 0, "ms_per_step": None,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
            "data": "synthetic: seeded serving trace (the reference publishes no benchmark data)",
            "config": {"workload": "serve: " + (serve_bench.__doc__ or "").split("\n")[0],
                       "rates": [r["rate"] for r in rows], "seconds_per_rate": args.seconds,
                       "tick_us": 1000, "passes_in_flight": 3, "ctas_per_chunk": args.ctas},
            "rates": rows, "clocks": clocks}
    print(json.dumps(line), flush=True)


def ctypes_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


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
