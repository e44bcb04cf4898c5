"""Benchmark: PSkel iterative stencils on one GB300.

Default workload (the headline configuration): Game of Life, Moore mask,
uint8 cells Bernoulli(0.3) from a seed, 8192 x 8192 grid, 1000 generations
per step, temporally blocked passes. A "step" is one full 1000-generation run
over the grid.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload life|jacobi|jacobi_bf16|advect|advect_bf16|heat3d|heat3d_bf16|batch|batch_bf16]

Prints ONE JSON line. ``value`` is GCells/s (cell updates per second) with the
grid resident in HBM; ``e2e`` is the same metric through the host entry point
(pskel_run2d_host: host->device copy from pinned memory, the run, the copy
back). ``--impl reference`` times the reference's own OpenMP runIterativeCPU
(oracle/_ref/pskel_ref, built from the reference headers) on the host cores,
every timed step running the whole workload.

A single-GPU run of the headline workload also measures every other workload
(at most 5 timed steps each, a smaller CPU sample) and reports them under
``others``; ``--no-others`` skips that.

Under torchrun (N > 1) every rank runs an independent replica of the
workload on its own GPU (the path has no cross-grid exchange); the timing is
the max over ranks and ``value`` counts the cells of all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GCells/s"
WORKLOADS = {
    "life": dict(desc="Game of Life 2D Moore 8-neighbour mask, uint8 Bernoulli(0.3), 8192x8192, 1000 iterations",
                 W=8192, H=8192, iters=1000, dtype="u8", T=17, b_alg=2),
    "jacobi": dict(desc="Jacobi 2D 5-point (4 neighbours, weight 0.25), float32 1024x1024, zero ring, 100 iterations",
                   W=1024, H=1024, iters=100, dtype="f32", T=13, b_alg=8),
    "jacobi_bf16": dict(desc="Jacobi 2D 5-point, bf16 storage / fp32 arithmetic, 1024x1024, 100 iterations",
                        W=1024, H=1024, iters=100, dtype="bf16", T=13, b_alg=4),
    "advect": dict(desc="advection-diffusion 2D, float32 4096x4096, winds N(0,0.1), K 0.1, dt 0.2, 500 iterations",
                   W=4096, H=4096, iters=500, dtype="f32", T=5, b_alg=16),
    "advect_bf16": dict(desc="advection-diffusion 2D, bf16 storage / fp32 arithmetic, 4096x4096, 500 iterations",
                        W=4096, H=4096, iters=500, dtype="bf16", T=1, b_alg=8),
    "heat3d": dict(desc="3D 7-point heat (Mask3D), float32 512^3, zero halo, 50 iterations, fp64 residual every 10",
                   W=512, H=512, D=512, iters=50, dtype="f32", T=2, b_alg=8, every=10),
    "heat3d_bf16": dict(desc="3D 7-point heat, bf16 storage / fp32 arithmetic, 512^3, 50 iterations, "
                             "fp64 residual every 10", W=512, H=512, D=512, iters=50, dtype="bf16", T=1, b_alg=4,
                        every=10),
    "batch": dict(desc="batched Jacobi 2D 5-point, float32, 256 grids, sides log-uniform [64,2048], iterations "
                       "uniform [10,500], one persistent launch in a CUDA graph, MLP-picked steps per pass",
                  grids=256, train_grids=64, dtype="f32", batch=True, W=1024, H=1024, iters=100),
    "batch_bf16": dict(desc="batched Jacobi 2D 5-point, bf16 storage / fp32 arithmetic, 256 grids, sides "
                            "log-uniform [64,2048], iterations uniform [10,500], one persistent launch in a CUDA "
                            "graph, MLP-picked steps per pass",
                       grids=256, train_grids=64, dtype="bf16", batch=True, W=1024, H=1024, iters=100),
}


L2_NOTE = ("every timed step starts from freshly written inputs; the GPU arm also writes 512 MB (more than the "
           "L2) between timed steps")


def workload_config(wl, world):
    """The workload as both arms run it (the GPU arm's schedule is reported beside it)."""
    grid = [wl["H"], wl["W"]] + ([wl["D"]] if "D" in wl else [])
    return {"workload": wl["desc"], "grid": grid, "iterations_per_step": wl["iters"], "l2": L2_NOTE,
            "parallelism": "one replica per rank" if world > 1 else "single replica"}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
            # the timed region starts once the sampler is producing samples
            t0 = time.time()
            while time.time() - t0 < 5 and self.proc.poll() is None and os.path.getsize(self.file.name) == 0:
                time.sleep(0.02)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def dist_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- our arm

def make_inputs(wl):
    from pskel_gb300 import synth as S
    name = wl["name"]
    W, H = wl["W"], wl["H"]
    if name == "life":
        a, b = S.life(W, H, seed=1)
        return {"in": a, "out": b}
    if name.startswith("jacobi") or name.startswith("batch"):
        a, b = S.jacobi2d(W, H, seed=1)
        if wl["dtype"] == "bf16":
            a, b = S.f32_to_bf16(a), S.f32_to_bf16(b)
        return {"in": a, "out": b}
    if name.startswith("heat3d"):
        a, b = S.heat3d(W, H, wl["D"], seed=1)
        if wl["dtype"] == "bf16":
            a, b = S.f32_to_bf16(a), S.f32_to_bf16(b)
        return {"in": a, "out": b}
    if name.startswith("advect"):
        a, b, u, v = S.advect2d(W, H, seed=1)
        if wl["dtype"] == "bf16":
            a, b, u, v = (S.f32_to_bf16(x) for x in (a, b, u, v))
        return {"in": a, "out": b, "u": u, "v": v}
    raise ValueError(name)


def stencil_for(wl, P, S, keep, wind=(None, None)):
    name = wl["name"]
    if name == "life":
        return P.make_stencil(P.OP_LIFE, "u8", S.MOORE8_OFFSETS, keep=keep)
    if name.startswith("jacobi"):
        return P.make_stencil(P.OP_LINEAR, wl["dtype"], S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    if name.startswith("heat3d"):
        return P.make_stencil(P.OP_LINEAR, wl["dtype"], S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, keep=keep)
    return P.make_stencil(P.OP_ADVECT, wl["dtype"], S.JACOBI4_OFFSETS, wind=wind, K=S.ADVECT_K, dt=S.ADVECT_DT,
                          inv_dx=S.ADVECT_INV_DX, keep=keep)


def run_ours(args, wl, world, rank, local):
    import torch

    import pskel_gb300 as P
    from pskel_gb300 import synth as S

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    x = make_inputs(wl)
    W, H, iters = wl["W"], wl["H"], wl["iters"]
    D = wl.get("D", 1)
    tview = (lambda a: torch.from_numpy(a.view(np.int16))) if wl["dtype"] == "bf16" else torch.from_numpy
    src0 = tview(x["in"]).to(dev)
    out0 = tview(x["out"]).to(dev)
    a = src0.clone()
    b = out0.clone()
    keep = P._Keep()
    wind_dev = (None, None)
    if "u" in x:
        ud, vd = tview(x["u"]).to(dev), tview(x["v"]).to(dev)
        wind_dev = (ud.data_ptr(), vd.data_ptr())
    st = stencil_for(wl, P, S, keep, wind_dev)
    sch = P.Schedule(time_steps=args.time_steps or wl["T"], tile_w=0, tile_h=args.tile_h, tile_d=0, ctas=0)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)  # 512 MB > L2

    is3d = "D" in wl
    every = wl.get("every", 0)
    res_dev = torch.zeros(max(1, iters // every if every else 1), dtype=torch.float64, device=dev)

    def one_step():
        if is3d:
            P.iterate3d(st, a, b, iters, sched=sch, residual_every=every, residuals=res_dev if every else None,
                        stream=stream.cuda_stream)
        else:
            P.iterate2d(st, a, b, iters, sched=sch, stream=stream.cuda_stream)

    def reset():
        with torch.cuda.stream(stream):
            a.copy_(src0)
            b.copy_(out0)
            flush.fill_(1)

    for _ in range(args.warmup):
        reset()
        one_step()
    P.sync(stream.cuda_stream)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    dist_barrier(world)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            reset()
            starts[k].record(stream)
            one_step()
            ends[k].record(stream)
        P.sync(stream.cuda_stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    dist_barrier(world)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    t_dev = dist_max(sum(step_ms) / 1e3, world)
    cells = W * H * D * iters
    value = world * cells * args.steps / t_dev / 1e9

    # "plain": the same run with one step per pass (no temporal blocking, the
    # structure of the reference's runIterativeGPU), timed the same way; its
    # result must equal the tuned run's bit for bit (schedules change speed only)
    final_tuned = (b if iters % 2 == 1 else a).clone()
    plain = None
    if sch.time_steps != 1:
        sch1 = P.Schedule(time_steps=1)

        def plain_step():
            if is3d:
                P.iterate3d(st, a, b, iters, sched=sch1, residual_every=every, residuals=res_dev if every else None,
                            stream=stream.cuda_stream)
            else:
                P.iterate2d(st, a, b, iters, sched=sch1, stream=stream.cuda_stream)

        reset()
        plain_step()
        P.sync(stream.cuda_stream)
        same_plain = bool(torch.equal((b if iters % 2 == 1 else a), final_tuned))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        torch.cuda.synchronize()
        dist_barrier(world)
        for s0, e0 in ev:
            reset()
            s0.record(stream)
            plain_step()
            e0.record(stream)
        P.sync(stream.cuda_stream)
        torch.cuda.synchronize()
        dist_barrier(world)
        t_plain = dist_max(sum(s0.elapsed_time(e0) for s0, e0 in ev) / 1e3, world)
        plain = {"value": round(world * cells * args.steps / t_plain / 1e9, 3), "unit": "GCells/s",
                 "time_steps_per_pass": 1, "ms_per_step": round(t_plain / args.steps * 1e3, 4),
                 "results_identical_to_tuned": same_plain}

    if is3d:
        passes = len(plan_any(iters, sch.time_steps))
        launches = (passes + (iters // every if every else 0)) * args.steps  # + residual reductions
        dom = passes  # launches of the dominant kernel per step: one per pass
    else:
        # the library reports the kernel launches of its last 2D call: Life runs
        # every pass in one persistent launch between two bit planes (plus two
        # packs and an unpack); grids of few tiles per pass run every pass in one
        # persistent launch; larger grids launch once per pass
        reset()
        one_step()
        P.sync(stream.cuda_stream)
        per_call = int(P.lib.pskel_last_launches2d())
        launches = per_call * args.steps
        passes = 1 if wl["name"] == "life" else P.lib.pskel_plan_passes(iters, sch.time_steps, None, 0)
        dom = 1 if (wl["name"] == "life" or per_call == 1) else per_call

    # kernel-only launch timing for the roofline: average duration of a launch
    # of the dominant kernel (a pass, or every pass in one persistent launch)
    per_launch_ms = sum(step_ms) / args.steps / dom

    # ---- end to end through the host entry point, pinned host buffers
    pin_in = torch.from_numpy(x["in"].view(np.int16) if wl["dtype"] == "bf16" else x["in"]).pin_memory()
    pin_out0 = torch.from_numpy(x["out"].view(np.int16) if wl["dtype"] == "bf16" else x["out"]).pin_memory()
    pin_out = pin_out0.clone().pin_memory()
    wind_host = (None, None)
    if "u" in x:
        pu = torch.from_numpy(x["u"].view(np.int16) if wl["dtype"] == "bf16" else x["u"]).pin_memory()
        pv = torch.from_numpy(x["v"].view(np.int16) if wl["dtype"] == "bf16" else x["v"]).pin_memory()
        wind_host = (pu.data_ptr(), pv.data_ptr())
    st_h = stencil_for(wl, P, S, keep, wind_host)
    esz = pin_in.element_size()
    r = 1  # ring of the 2D workloads (mask range 1)
    if is3d:
        h2d = W * H * D * esz  # the 3D output's initial contents are never read
        d2h = W * H * D * esz + 8 * (iters // every if every else 0)
    else:
        h2d = W * H * esz * (3 if "u" in x else 1)
        # the output array's ring goes to the device too (read by every second step)
        h2d += (2 * r * W + 2 * r * (H - 2 * r)) * esz
        d2h = W * H * esz
    res_host = np.zeros(max(1, iters // every if every else 1), dtype=np.float64)

    def host_call():
        if is3d:
            return P.lib.pskel_run3d_host(P.C.byref(st_h), pin_in.data_ptr(), pin_out.data_ptr(), W, H, D, iters,
                                          P.C.byref(sch), every, res_host.ctypes.data)
        return P.lib.pskel_run2d_host(P.C.byref(st_h), pin_in.data_ptr(), pin_out.data_ptr(), W, H, iters,
                                      P.C.byref(sch))

    def reset_out():
        # Only what the call reads of the output array is restored between
        # steps: its ring in 2D (the last run left the result's ring there),
        # nothing in 3D (never read). Rewriting the whole pinned array from the
        # CPU before each call would leave its lines dirty in the Grace caches
        # and slow the device's coherent writes of the result into them.
        if not is3d:
            pin_out[:r].copy_(pin_out0[:r])
            pin_out[-r:].copy_(pin_out0[-r:])
            pin_out[:, :r].copy_(pin_out0[:, :r])
            pin_out[:, -r:].copy_(pin_out0[:, -r:])

    def e2e_step():
        reset_out()
        host_call()

    for _ in range(max(1, args.warmup)):
        e2e_step()
    times = []
    for _ in range(args.steps):
        reset_out()
        t1 = time.perf_counter()
        rc = host_call()
        times.append(time.perf_counter() - t1)
        if rc != 0:
            raise RuntimeError(P.lib.pskel_last_error().decode())
    t_e2e = dist_max(sum(times), world)
    e2e_value = world * cells * args.steps / t_e2e / 1e9
    # the e2e result equals the device-resident run's result
    final_dev = (b if iters % 2 == 1 else a).cpu()
    # (the device run was reset between steps, so its final state is one run)
    same = bool(torch.equal(final_dev, pin_out))

    peak, peak_kind = load_peaks()
    b_alg = wl["b_alg"]
    achieved = b_alg * W * H * D * (iters / dom) / (per_launch_ms / 1e3) / 1e9
    # the launch's own compulsory traffic: read + write the grid once per pass
    pass_bytes = b_alg * W * H * D * (passes / dom)
    if wl["name"] == "life":
        pass_bytes = 3 * W * H  # HBM: pack reads both byte grids, unpack writes one; the bit planes stay in L2
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GCells/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_dev / args.steps * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": wl["dtype"], "data": "synthetic (seeded SplitMix64)",
        "config": workload_config(wl, world),
        "schedule": {"time_steps_per_pass": sch.time_steps, "passes": passes},
        "e2e": {"value": round(e2e_value, 3), "unit": "GCells/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "matches_device_run": same},
        "plain": plain if plain is not None else {"note": "the tuned schedule is one step per pass"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 3), "traffic": None,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s",
                     "algorithmic_bytes_per_launch": b_alg * W * H * D * (iters / dom),
                     "per_launch_ms": round(per_launch_ms, 5),
                     "pass_compulsory_frac": round(pass_bytes / (per_launch_ms / 1e3) / 1e9 / peak, 3),
                     "note": "achieved = B_alg per cell update x cell updates per launch / launch time; "
                             "temporal blocking fuses time_steps updates per HBM round trip, so frac can exceed 1; "
                             "pass_compulsory_frac = one read + one write of the grid per pass / time / peak"},
        "wall_s": round(wall, 3),
    }
    return line, clk.summary()


# ------------------------------------------------- batched workload

def batch_pool(torch, dev, shapes, dtype, seed):
    """All grids of a batch in one device pool (each buffer 256-byte aligned,
    rows padded to 16 bytes); returns the pool, its pristine copy and per-grid
    (in view, out view, pitch)."""
    from pskel_gb300 import synth as S
    esz = 2 if dtype == "bf16" else 4
    offs, total = [], 0
    for W, H, _ in shapes:
        pitch = -(-W * esz // 16) * 16 // esz
        n = pitch * H
        a_off = total
        total += -(-n * esz // 256) * 256 // esz
        b_off = total
        total += -(-n * esz // 256) * 256 // esz
        offs.append((a_off, b_off, pitch))
    host = np.zeros(total, dtype=np.int16 if dtype == "bf16" else np.float32)
    for k, ((W, H, _), (a_off, b_off, pitch)) in enumerate(zip(shapes, offs)):
        a, b = S.jacobi2d(W, H, seed=seed * 100003 + k)
        if dtype == "bf16":
            a, b = S.f32_to_bf16(a).view(np.int16), S.f32_to_bf16(b).view(np.int16)
        host[a_off:a_off + pitch * H].reshape(H, pitch)[:, :W] = a
        host[b_off:b_off + pitch * H].reshape(H, pitch)[:, :W] = b
    pool0 = torch.from_numpy(host).to(dev)
    pool = pool0.clone()
    views = [(pool[a:a + p * H].view(H, p), pool[b:b + p * H].view(H, p), p)
             for (W, H, _), (a, b, p) in zip(shapes, offs)]
    return host, pool, pool0, views


def run_batch(args, wl, world, rank, local):
    """256 Jacobi grids of uneven shapes and iteration counts in one
    persistent launch (a CUDA graph). The per-grid steps per pass come from the
    MLP cost model (trained here on timings the measured tuner takes on a
    separate set of grids); the same batch with the exhaustive tuner's picks,
    and the GA-tuned plain per-grid launches, are timed beside it."""
    import torch

    import pskel_gb300 as P
    import pskel_gb300.tuner as T
    from pskel_gb300 import synth as S

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dtype = wl["dtype"]
    esz = 2 if dtype == "bf16" else 4
    keep = P._Keep()
    st = P.make_stencil(P.OP_LINEAR, dtype, S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, keep=keep)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    shapes = S.batch_shapes(wl["grids"], seed=1 + rank)
    cells = sum(W * H * it for W, H, it in shapes)
    host, pool, pool0, views = batch_pool(torch, dev, shapes, dtype, seed=1 + rank)

    def cands(W, H, it):  # the batched kernel's space: steps per pass on the 128 x 66 tile
        return [c for c in T.candidates(st, W, H, it) if c.tile_h == 0]

    # ---- tuning (untimed). The measured tuner times each grid's candidates
    # inside a batched launch (copies of the grid filling the GPU, buffers from
    # a scratch pool): the exhaustive per-grid pick on the benchmark's grids.
    scratch = torch.empty(160 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)
    t0 = time.perf_counter()
    exh, exh_ms = [], []
    for W, H, it in shapes:
        cs = cands(W, H, it)
        ms, _ = T.time_in_batch(st, scratch, W, H, it, cs, reps=3, stream=sp)
        exh.append(cs[int(np.argmin(ms))].time_steps)
        exh_ms.append(float(ms.min()))
    t_exh = time.perf_counter() - t0
    # training set: the same tuner's timings on a separate draw of grids
    t0 = time.perf_counter()
    tshapes = S.batch_shapes(wl["train_grids"], seed=1000 + rank)
    X, Y = [], []
    for W, H, it in tshapes:
        cs = cands(W, H, it)
        ms, _ = T.time_in_batch(st, scratch, W, H, it, cs, reps=3, stream=sp)
        for c, m in zip(cs, ms):
            X.append(T.features(st, W, H, it, c))
            Y.append(np.log(m))
    del scratch
    X = np.stack(X)
    Y = np.array(Y, dtype=np.float32)
    model = T.CostModel(hidden=64, layers=3, seed=1)
    y_mean = float(Y.mean())
    loss = model.train(X, Y - y_mean, epochs=4000, lr=3e-3)
    t_train = time.perf_counter() - t0
    if args.save_model and rank == 0:
        model.save(args.save_model)
    learned = []
    for W, H, it in shapes:
        cs = cands(W, H, it)
        pred = model.predict(np.stack([T.features(st, W, H, it, c) for c in cs]))
        learned.append(cs[int(np.argmin(pred))].time_steps)
    model.close()
    ga = [T.ga_schedule(st, W, H, it, seed=1)[0] for W, H, it in shapes]

    def make(ts):
        return P.Batch(st, [(x, y, it, t, p, W) for (W, H, it), (x, y, p), t in zip(shapes, views, ts)])

    b_learned = make(learned)
    b_exh = make(exh)
    b_default = make([0] * len(shapes))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)

    def reset():
        with torch.cuda.stream(stream):
            pool.copy_(pool0)
            flush.fill_(1)

    def ga_plain():
        for (W, H, it), (x, y, p), s in zip(shapes, views, ga):
            P.iterate2d(st, x, y, it, sched=s, pitch=p, width=W, height=H, stream=sp)

    def timed(fn, steps, warm):
        for _ in range(warm):
            reset()
            fn()
        P.sync(sp)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize()
        dist_barrier(world)
        for s, e in ev:
            reset()
            s.record(stream)
            fn()
            e.record(stream)
        P.sync(sp)
        torch.cuda.synchronize()
        dist_barrier(world)
        return dist_max(sum(s.elapsed_time(e) for s, e in ev) / 1e3, world)

    with ClockSampler(local) as clk:
        t_learned = timed(lambda: b_learned.run(sp), args.steps, args.warmup)
    t_exh_b = timed(lambda: b_exh.run(sp), args.steps, args.warmup)
    t_def = timed(lambda: b_default.run(sp), args.steps, args.warmup)
    t_ga = timed(ga_plain, max(1, args.steps // 2), 1)
    ga_steps = max(1, args.steps // 2)

    # uniform steps per pass for the whole batch, every odd value: the best
    # uniform schedule is the other exhaustive reference point
    uniform = {}
    for t in range(1, 16, 2):
        bu = make([t] * len(shapes))
        uniform[t] = world * cells * 3 / timed(lambda: bu.run(sp), 3, 1) / 1e9
        bu.close()
    t_uni = max(uniform, key=uniform.get)

    # result check: the learned and exhaustive batches leave identical results
    # (each grid's result buffer; the other buffer holds a schedule-dependent
    # intermediate state)
    def results():
        return [(y if it % 2 else x)[:, :W].clone() for (W, H, it), (x, y, p) in zip(shapes, views)]

    reset()
    b_learned.run(sp)
    P.sync(sp)
    res_l = results()
    reset()
    b_exh.run(sp)
    P.sync(sp)
    same = all(bool(torch.equal(a, b)) for a, b in zip(res_l, results()))
    del res_l

    # ---- end to end: pinned host grids in, one graph launch, results out
    pin_src = torch.from_numpy(host).pin_memory()
    pin_res = torch.empty_like(pin_src).pin_memory()

    def e2e_step():
        with torch.cuda.stream(stream):
            pool.copy_(pin_src, non_blocking=True)
        b_learned.run(sp)
        with torch.cuda.stream(stream):
            pin_res.copy_(pool, non_blocking=True)
        stream.synchronize()

    for _ in range(args.warmup):
        e2e_step()
    tt = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        e2e_step()
        tt.append(time.perf_counter() - t1)
    t_e2e = dist_max(sum(tt), world)
    pool_bytes = pool.numel() * esz

    value = world * cells * args.steps / t_learned / 1e9
    v_exh = world * cells * args.steps / t_exh_b / 1e9
    v_def = world * cells * args.steps / t_def / 1e9
    v_ga = world * cells * ga_steps / t_ga / 1e9
    peak, peak_kind = load_peaks()
    # one launch per step: algorithmic bytes = B_alg x every cell update of the batch
    b_alg = 2 * esz
    per_launch = t_learned / args.steps
    achieved = b_alg * cells / per_launch / 1e9
    passes = sum(P.lib.pskel_plan_passes(it, t, None, 0) for (W, H, it), t in zip(shapes, learned))
    pass_bytes = sum(2 * esz * W * H * P.lib.pskel_plan_passes(it, t, None, 0)
                     for (W, H, it), t in zip(shapes, learned))
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GCells/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_learned / args.steps * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded SplitMix64)",
        "config": {"workload": wl["desc"], "grids": len(shapes), "cell_updates_per_step": cells, "l2": L2_NOTE,
                   "parallelism": "one replica per rank" if world > 1 else "single replica"},
        "tuning": {"learned_batch": round(value, 3), "exhaustive_batch": round(v_exh, 3),
                   "default_batch": round(v_def, 3), "ga_plain_launches": round(v_ga, 3),
                   "uniform_batch": {str(t): round(v, 3) for t, v in uniform.items()},
                   "best_uniform": {"time_steps": t_uni, "value": round(uniform[t_uni], 3)},
                   "learned_vs_exhaustive": round(value / v_exh, 4),
                   "learned_vs_best_uniform": round(value / uniform[t_uni], 4),
                   "learned_vs_ga_plain": round(value / v_ga, 4),
                   "picks_equal_exhaustive": int(sum(a == b for a, b in zip(learned, exh))),
                   "exhaustive_tuning_s": round(t_exh, 2), "training_s": round(t_train, 2),
                   "training_samples": int(X.shape[0]), "training_loss": round(float(loss), 5),
                   "results_identical": same},
        "e2e": {"value": round(world * cells * args.steps / t_e2e / 1e9, 3), "unit": "GCells/s",
                "h2d_bytes_per_step": pool_bytes, "d2h_bytes_per_step": pool_bytes},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 3), "traffic": None,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s",
                     "algorithmic_bytes_per_launch": b_alg * cells,
                     "per_launch_ms": round(per_launch * 1e3, 4), "passes_per_launch": passes,
                     "pass_compulsory_frac": round(pass_bytes / per_launch / 1e9 / peak, 3),
                     "note": "one persistent launch runs every pass of every grid; achieved = B_alg x cell "
                             "updates / launch time; pass_compulsory_frac = one read + one write of each grid per "
                             "pass / launch time / peak"},
    }
    for b in (b_learned, b_exh, b_default):
        b.close()
    return line, clk.summary()


def plan_any(iters, T):
    """Pass lengths of a 3D run (mirror of the library's plan for fully written grids)."""
    p = [T] * (iters // T) + ([iters % T] if iters % T else [])
    if len(p) % 2 != iters % 2:
        for i, v in enumerate(p):
            if v >= 2:
                p[i:i + 1] = [v // 2, v - v // 2]
                break
    return p


def load_counters(name):
    """ncu counters of the workload's dominant kernel, per launch, from the
    committed summary (profiles/counters.json): DRAM bytes, warp instructions
    issued and ALU-pipe warp instructions, with the summary they come from."""
    p = ROOT / "profiles" / "counters.json"
    if p.exists():
        return json.loads(p.read_text()).get(name, {})
    return {}


ISSUE_PER_SM_CLK = 4  # warp instructions an SM issues per clock (four schedulers)
ALU_PER_SM_CLK = 2    # ALU-pipe warp instructions an SM completes per clock (16 lanes per scheduler)


def finish_roofline(line, name, clocks, sms):
    """Picks the roof of the dominant kernel. Its HBM figure (algorithmic bytes
    per launch / launch time / measured copy bandwidth) is the roofline when
    the kernel moves about its algorithmic bytes. A kernel whose DRAM traffic
    (ncu) is far below them -- temporal blocking keeps the grid on chip -- is
    bound by an SM resource instead: instruction issue (warp instructions per
    launch from ncu / launch time against SMs x 4 schedulers x the SM clock
    sampled during the timed region), or the ALU pipe (ALU-pipe warp
    instructions against SMs x 2 per clock: the bit-sliced Life kernel), which
    ever is the larger fraction. The HBM figure is kept beside it."""
    rf = line["roofline"]
    c = load_counters(name)
    rf["traffic"] = c.get("dram_bytes")
    alg = rf.pop("algorithmic_bytes_per_launch")
    if not (c.get("dram_bytes") is not None and c.get("warp_instructions") and c["dram_bytes"] < 0.5 * alg):
        rf["counters_from"] = c.get("profile")
        return
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not mhz:
        return
    t = rf["per_launch_ms"] / 1e3
    hbm = {k: rf[k] for k in ("achieved", "peak", "unit", "frac", "peak_source")}
    clk = f"{mhz:.0f} MHz (median SM clock sampled during the timed region)"
    issue = c["warp_instructions"] / t / 1e9
    issue_peak = sms * ISSUE_PER_SM_CLK * mhz * 1e6 / 1e9
    roofs = {"issue": (issue, issue_peak, "G warp instructions/s", f"{sms} SMs x {ISSUE_PER_SM_CLK} schedulers x {clk}")}
    if c.get("alu_warp_instructions"):
        alu = c["alu_warp_instructions"] / t / 1e9
        roofs["alu"] = (alu, sms * ALU_PER_SM_CLK * mhz * 1e6 / 1e9, "G ALU-pipe warp instructions/s",
                        f"{sms} SMs x {ALU_PER_SM_CLK} ALU-pipe warp instructions per clock x {clk}")
    bound = max(roofs, key=lambda k: roofs[k][0] / roofs[k][1])
    ach, peak, unit, src = roofs[bound]
    line["roofline"] = {
        "bound": bound, "achieved": round(ach, 1), "peak": round(peak, 1), "unit": unit,
        "frac": round(ach / peak, 3), "traffic": c["dram_bytes"], "peak_source": src,
        "per_launch_ms": rf["per_launch_ms"],
        "warp_instructions_per_launch": c["warp_instructions"], "counters_from": c.get("profile"),
        "other_roofs": {k: round(v[0] / v[1], 3) for k, v in roofs.items() if k != bound},
        "hbm_algorithmic": dict(hbm, note="algorithmic bytes per launch / launch time; above 1 because the grid "
                                          "stays on chip between steps (bytes_avoided_factor = frac)"),
        "bytes_avoided_factor": hbm["frac"],
        "dram_frac_of_algorithmic": round(c["dram_bytes"] / alg, 6),
    }
    for k in ("pass_compulsory_frac", "passes_per_launch"):
        if k in rf:
            line["roofline"][k] = rf[k]


# ------------------------------------------------------- CPU baselines

def cpu_sample(wl, threads, iters_sample, use_ref=True):
    """Time the reference's runIterativeCPU (or the oracle port) on a sample."""
    import oracle
    x = make_inputs(wl)
    W, H = wl["W"], wl["H"]
    if use_ref and oracle.have_ref():
        from pskel_gb300 import synth as S
        env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="close", OMP_PLACES="cores")
        with tempfile.TemporaryDirectory() as d:
            d = Path(d)
            npt = x["in"].dtype
            for k, v in x.items():
                np.ascontiguousarray(v).tofile(d / k)
            if wl["name"] == "life":
                cmd = ["life", W, H, iters_sample, threads, d / "in", d / "out", d / "res"]
            elif wl["name"].startswith("heat3d"):
                with open(d / "m.txt", "w") as f:
                    f.write("7 3\n" + "".join(f"{o[0]} {o[1]} {o[2]} {w!r}\n" for o, w in zip(S.HEAT7_OFFSETS,
                                                                                              S.HEAT7_WEIGHTS)))
                cmd = ["lin3d", wl["dtype"], W, H, wl["D"], iters_sample, threads, d / "m.txt", "0.0", d / "in",
                       d / "out", d / "res"]
            elif wl["name"].startswith(("jacobi", "batch")):
                with open(d / "m.txt", "w") as f:
                    f.write("4 2\n" + "".join(f"{o[0]} {o[1]} {w!r}\n" for o, w in zip(S.JACOBI4_OFFSETS,
                                                                                     S.JACOBI4_WEIGHTS)))
                cmd = ["lin2d", wl["dtype"], W, H, iters_sample, threads, d / "m.txt", d / "in", d / "out", d / "res"]
            else:
                cmd = ["advect", wl["dtype"], W, H, iters_sample, threads, repr(S.ADVECT_K), repr(S.ADVECT_DT),
                       repr(S.ADVECT_INV_DX), d / "in", d / "out", d / "u", d / "v", d / "res"]
            out = subprocess.run([str(oracle.REF_BIN)] + [str(c) for c in cmd], capture_output=True, text=True,
                                 env=env, check=True).stdout
            wall = json.loads([l for l in out.splitlines() if l.startswith("{")][-1])["wall_s"]
            del npt
        return W * H * wl.get("D", 1) * iters_sample / wall / 1e9, "reference", wall
    oracle.build()
    t0 = time.perf_counter()
    if wl["name"] == "life":
        oracle.life(x["in"], x["out"], iters_sample)
    elif wl["name"].startswith(("jacobi", "batch")):
        from pskel_gb300 import synth as S
        oracle.lin2d(x["in"], x["out"], S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, iters_sample, dtype=wl["dtype"])
    elif wl["name"].startswith("heat3d"):
        from pskel_gb300 import synth as S
        oracle.lin3d(x["in"], x["out"], S.HEAT7_OFFSETS, S.HEAT7_WEIGHTS, iters_sample, dtype=wl["dtype"])
    else:
        from pskel_gb300 import synth as S
        oracle.advect(x["in"], x["out"], x["u"], x["v"], iters_sample, S.ADVECT_K, S.ADVECT_DT, S.ADVECT_INV_DX,
                      dtype=wl["dtype"])
    wall = time.perf_counter() - t0
    return W * H * wl.get("D", 1) * iters_sample / wall / 1e9, "port", wall


def sample_iters(wl, updates=2e10):
    # a bounded sample: about `updates` cell updates (3D: 60 % of it), 10-15 s
    # of the reference's OpenMP loop on the 16 host cores of a GB300 node
    cells = wl["W"] * wl["H"] * wl.get("D", 1)
    return max(1, int((0.6 * updates if "D" in wl else updates) // cells))


def reference_gpu_path(wl):
    """The reference's own GPU path on the same workload, beside its CPU arm:
    ``runIterativeGPU`` (one kernel launch per step, 32 x 4 threads per block
    as in the reference's test scripts, a device synchronisation after each
    step; PSkelStencil.hpp:1046-1097). Two runs (the workload's iterations and
    a tenth of them) give the per-step time of the step loop alone by their
    difference; ``e2e`` is the reference's own GPU_time of the full run
    (copies in and out included). Only the 2D workloads it runs as shipped
    (Life u8, Jacobi f32)."""
    import oracle
    if wl["name"] not in ("life", "jacobi"):
        return None
    if not oracle.have_ref_gpu() or not Path("/dev/nvidiactl").exists():
        return {"unavailable": "no GPU or oracle/_ref/pskel_ref_gpu not built"}
    from pskel_gb300 import synth as S
    x = make_inputs(wl)
    full = wl["iters"]
    short = max(2, full // 10)
    runs = {}
    try:
        for its in (short, full):
            if wl["name"] == "life":
                _, t = oracle.ref_gpu_life(x["in"], x["out"], its)
            else:
                _, t = oracle.ref_gpu_lin2d(x["in"], x["out"], S.JACOBI4_OFFSETS, S.JACOBI4_WEIGHTS, its)
            runs[its] = t
    except (subprocess.CalledProcessError, OSError, ValueError, KeyError, IndexError) as e:
        # the CPU arm stands on its own; the GPU path is context
        return {"unavailable": f"the reference's runIterativeGPU did not run: {type(e).__name__}"}
    cells = wl["W"] * wl["H"]
    per_step = (runs[full]["gpu_time_s"] - runs[short]["gpu_time_s"]) / (full - short)
    return {"impl": "runIterativeGPU (stencilTilingCU, one launch per step), blocks 32x4",
            "value": round(cells / per_step / 1e9, 4), "unit": "GCells/s", "ms_per_iteration": round(per_step * 1e3, 4),
            "e2e": round(cells * full / runs[full]["gpu_time_s"] / 1e9, 4),
            "gpu_time_s": {str(k): round(v["gpu_time_s"], 6) for k, v in runs.items()},
            "note": "value: the step loop alone (difference of the two runs); e2e: the reference's GPU_time of the "
                    "full run, host copies included"}


def run_reference_arm(args, wl, world, rank):
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    # every timed step runs the whole workload (Life 8192^2 x 1000: about
    # 30 s on 16 Grace cores), so the arm's config is the GPU arm's; the
    # untimed warm-up steps run a tenth of the iterations (they only page in
    # the binary and the inputs)
    its = wl["iters"]
    vals, kind, walls = [], None, []
    for _ in range(args.warmup):
        cpu_sample(wl, threads, max(1, its // 10))
    for _ in range(args.steps):
        v, kind, w = cpu_sample(wl, threads, its)
        vals.append(v)
        walls.append(w)
    cells = wl["W"] * wl["H"] * wl.get("D", 1) * its * args.steps
    value = cells / sum(walls) / 1e9
    shape = "x".join(str(v) for v in ([wl["H"], wl["W"]] + ([wl["D"]] if "D" in wl else [])))
    sample = (f"{shape} grid, {its} iterations per step (of {wl['iters']}), {threads} OpenMP threads"
              if its < wl["iters"] else f"{shape} grid, the whole workload per step, {threads} OpenMP threads")
    if wl.get("batch"):
        sample = (f"one {shape} grid of the same stencil, {its} iterations per step (the reference has no batched "
                  f"path: runIterativeCPU runs grid by grid), {threads} OpenMP threads")
    return {"metric": METRIC, "value": round(value, 4), "unit": "GCells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(sum(walls) / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": wl["dtype"], "data": "synthetic (seeded SplitMix64)",
            "config": workload_config(wl, world),
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 4), "unit": "GCells/s", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "GCells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_path": reference_gpu_path(wl)}


OTHERS = ["jacobi", "jacobi_bf16", "advect", "advect_bf16", "heat3d", "heat3d_bf16", "batch", "batch_bf16"]


def cpu_baseline(wl, updates):
    """The reference's runIterativeCPU on the host cores: runs of at most the
    workload's iterations (the whole workload when it is small, repeated up to
    10 times), about `updates` cell updates in all."""
    total = sample_iters(wl, updates)
    its = min(wl["iters"], total)
    reps = min(10, max(1, total // its))
    shape = "x".join(str(v) for v in ([wl["H"], wl["W"]] + ([wl["D"]] if "D" in wl else [])))
    kind, wall = None, 0.0
    for _ in range(reps):
        _, kind, w = cpu_sample(wl, os.cpu_count() or 1, its)
        wall += w
    v = wl["W"] * wl["H"] * wl.get("D", 1) * its * reps / wall / 1e9
    sample = f"{shape} grid, {reps} run(s) of {its} iterations (of {wl['iters']}), {wall:.2f} s"
    if wl.get("batch"):
        sample = f"one {shape} grid of the same stencil (the reference runs grid by grid), " + sample[len(shape) + 7:]
    return {"value": round(v, 4), "unit": "GCells/s", "cores": os.cpu_count() or 1, "kind": kind, "sample": sample}


FP64_ERRORS = Path(__file__).resolve().parent / "tests" / "golden" / "fp64_errors.json"


def fp64_error(wl):
    """The workload's error against an FP64 oracle. The results are
    bit-identical to the oracle's fp32 / bf16 restatement on these inputs (the
    -m gpu suite checks the full-size runs), so the error is that of the
    restatement against the same algorithm in double precision, computed once
    on the CPU by tests/golden/make_fp64_errors.py."""
    if wl["name"] == "life":
        return {"kind": "integer", "note": "bit-exact against the reference; no floating point"}
    try:
        e = json.loads(FP64_ERRORS.read_text())[wl["name"]]
    except (OSError, KeyError, ValueError):
        return None
    return {"max_abs": e["max_abs"], "max_rel": e["max_rel"], "rel_l2": e["rel_l2"],
            "source": "tests/golden/fp64_errors.json (the oracle's bit-identical restatement against FP64 on the "
                      "same inputs)"}


def run_workload(name, args, world, rank, local, cpu_updates):
    import torch
    wl = dict(WORKLOADS[name], name=name)
    runner = run_batch if wl.get("batch") else run_ours
    line, clocks = runner(args, wl, world, rank, local)
    line["clocks"] = clocks
    line["fp64_error"] = fp64_error(wl)
    finish_roofline(line, name, clocks, torch.cuda.get_device_properties(local).multi_processor_count)
    if rank == 0 and cpu_updates:
        line["cpu_baseline"] = cpu_baseline(wl, cpu_updates)
    return line


def compact(line):
    """The keys of another workload's line that the headline line carries."""
    out = {k: line[k] for k in ("value", "unit", "ms_per_step", "steps", "warmup", "dtype", "config", "schedule",
                                "gpu_launches", "roofline", "cpu_baseline", "clocks", "fp64_error") if k in line}
    out["plain"] = line["plain"].get("value") if isinstance(line.get("plain"), dict) else None
    out["e2e"] = line["e2e"]["value"]
    if "tuning" in line:
        out["tuning"] = {k: line["tuning"][k] for k in ("learned_vs_exhaustive", "learned_vs_ga_plain",
                                                        "learned_vs_best_uniform", "exhaustive_batch",
                                                        "ga_plain_launches", "best_uniform", "results_identical")}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="life", choices=sorted(WORKLOADS))
    ap.add_argument("--time-steps", type=int, default=0)
    ap.add_argument("--tile-h", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-others", action="store_true",
                    help="only the chosen workload (by default a single-GPU run of the headline workload also "
                         "measures every other workload, with at most 5 timed steps each, under `others`)")
    ap.add_argument("--save-model", default="", help="batch workloads: write the trained cost model here")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        line = run_reference_arm(args, dict(WORKLOADS[args.workload], name=args.workload), world, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    line = run_workload(args.workload, args, world, rank, local, 0 if args.no_cpu_baseline else 2e10)
    if world == 1 and args.workload == "life" and not args.no_others and not args.time_steps and not args.tile_h:
        import torch
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.warmup = min(args.steps, 5), 3
        others = {}
        for name in OTHERS:
            others[name] = compact(run_workload(name, sub, world, rank, local,
                                                0 if args.no_cpu_baseline else 5e9))
            torch.cuda.empty_cache()
        line["others"] = others
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
