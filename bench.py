"""Benchmark of the self_contact_sparse cloth step on GB300.

Workload (one "step" = one frame of every cloth): 512 independent square
cloths in one device arena, grid side uniform in 11..81 vertices (1.3 M
vertices in total), 1 m sheets dropped from 0.3-1.5 m onto spheres of radius
0.1-0.4 m, rotated about z, material lambda = mu = 1, bending 1e-3, dt 0.02,
clearance 0.01, CG tolerance 1e-6 (the reference's Solve_CG: ILU(0) meets
non-positive pivots on the finer sheets).  Inputs are synthetic and seeded.

Metric: vertex-steps/s (cloth vertices advanced one frame per second, whole
job), with p50 / p99 frame latency.  `value` is timed with CUDA events on the
library's stream with the state resident in HBM; `e2e` goes through the C ABI
with the state copied from pinned host memory and back every frame.

    python bench.py [--steps K] [--warmup W] [--impl native|reference] [--cloths N]
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "vertex-steps/s batched vs plain GPU path at 1e-6 err; p50/p99 step latency"
UNIT = "vertex-steps/s"


def workload_config(n_cloths: int, nv: int) -> dict:
    return {
        "workload": f"{n_cloths} cloths in one arena, grid side U{{11..81}} (1 m), drop 0.3-1.5 m onto "
                    f"spheres r 0.1-0.4 m, CG tol 1e-6, dt 0.02",
        "cloths": n_cloths,
        "vertices": nv,
        "l2": "inputs larger than L2 (FP64 block matrix of the arena > 1 GB)",
    }


def workload_vertices(cloths) -> int:
    return int(sum(c.np for c in cloths))


def read_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return {"hbm_gbs": float(p["hbm_gbs"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_figures() -> dict:
    """Figures from the committed ncu summaries that the bench cannot measure
    itself: lines of the form `bench-figure <kernel> <name> <value>` in
    profiles/*.md, e.g. the ratio of DRAM bytes to algorithmic bytes of a kernel
    (scaled here to a launch of this run) or its FP64-pipe activity."""
    out = {}
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return out
    for fn in sorted(os.listdir(d)):
        if not fn.endswith(".md"):
            continue
        with open(os.path.join(d, fn)) as f:
            for line in f:
                p = line.strip().strip("`").split()
                if len(p) == 4 and p[0] == "bench-figure":
                    try:
                        out[(p[1], p[2])] = float(p[3])
                    except ValueError:
                        pass
    return out


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------------------
# algorithmic bytes of the kernels we report a roofline for (FP64 values 8 B, indices 4 B)
# SpMV over a cloth of N vertices and B off-diagonal blocks: blocks + column indices,
# diagonal blocks, x read, y written, row pointers.
def spmv_bytes(nv: int, nb: int, s: int = 8) -> int:
    return nb * (9 * s + 4) + nv * (9 * s + 6 * s + 4)


def run_cpu_baseline(cloths, budget_s: float = 12.0) -> dict:
    """The oracle restatement (single core) on a bounded sample of the workload."""
    from oracle import oracle as O
    O.build("port")
    lib = O.OracleLib("port")
    done_vs, t_used, frames = 0, 0.0, 0
    used = 0
    for c in cloths:
        sim = O.OracleCloth(lib, c)
        t0 = time.perf_counter()
        sim.step(2)
        dt = time.perf_counter() - t0
        t_used += dt
        done_vs += 2 * c.np
        frames += 2
        used += 1
        sim.close()
        if t_used > budget_s:
            break
    return {"value": done_vs / t_used, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle restatement, first {used} cloths of the workload x 2 frames each "
                      f"({done_vs} vertex-steps in {t_used:.1f} s), 1 host core"}


# --------------------------------------------------------------------------------------
def timed_batch(ctx, steps, warmup, stream, nv, tune_frames=2, profile_window=False):
    """W untimed frames, then K frames of every cloth in the context timed with
    per-frame CUDA events on the library's stream (no per-kernel profiling).
    Returns (per-frame ms list, launches, start state of the timed frames)."""
    import torch

    ctx.step(warmup)
    ctx.synchronize()
    # launch shapes timed on two frames from here (the state is restored)
    tune = ctx.autotune(tune_frames) if tune_frames else None
    torch.cuda.synchronize()
    # the state at the start of the timed frames (the end-to-end and profiled
    # passes replay the same frames from it)
    x0 = np.empty(3 * nv)
    v0 = np.empty(3 * nv)
    ctx.get_states(x0, v0)
    launches0 = ctx.launch_count()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    if profile_window:
        torch.cuda.cudart().cudaProfilerStart()
    ev[0].record(stream)
    for k in range(steps):
        ctx.step(1)
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    ctx.synchronize()
    if profile_window:
        torch.cuda.cudart().cudaProfilerStop()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
    return step_ms, ctx.launch_count() - launches0, (x0, v0), tune


def profiled_replay(ctx, steps, start, profile_names=()):
    """The timed frames once more from their start state, with CUDA events around
    every kernel launch: per-class kernel time and launches, and the device
    counters (contacts, FP64 tests, algorithmic bytes of the solver)."""
    ctx.set_states(start[0], start[1])
    ctx.profile(True)
    ctx.step(steps)
    ctx.synchronize()
    prof = {name: ctx.profile_read(name) for name in profile_names}
    counts = {}
    counts["spmv32_bytes"], counts["spmv64_bytes"] = ctx.profile_bytes()
    for k in ("pairs", "candidates", "contacts", "detections", "fp64_fv_prx", "fp64_ee_prx", "fp64_fv_ccd",
              "fp64_ee_ccd", "persist_bytes"):
        counts[k] = ctx.profile_read(k)[1]
    ctx.profile(False)
    return prof, counts


PROFILED = ("cg_spmv", "cg_update", "cg_direction", "tri_elements", "slot_reduce", "rhs", "refit", "traverse",
            "narrow", "impulse", "pcg", "ilu_factor", "mx_spmv", "mx_update", "mx_direction", "mx_residual",
            "mx_persist", "narrow_filter", "narrow_fv", "narrow_ee", "narrow_ccd64", "sort")


NESTED = ("narrow_filter", "narrow_fv", "narrow_ee", "narrow_ccd64")


def plain_one_per_launch(cloths, device, steps: int, warmup: int, start, budget_s: float = 8.0) -> dict:
    """The plain FP64 path, one cloth per arena and launch sequence, on the timed
    frames of the batched run (frames warmup+1 .. warmup+steps, from the batched
    FP64 run's start state), for a sample of cloths spread over the workload."""
    import torch

    from cloth_sim_self_collision_gb300.context import ClothContext
    ctx = ClothContext(device, "fp64")
    stream = torch.cuda.ExternalStream(ctx.stream(), device=device)
    offs = np.concatenate([[0], np.cumsum([3 * c.np for c in cloths])])
    stride = 37 if len(cloths) % 37 else 41
    order = [(k * stride) % len(cloths) for k in range(len(cloths))]
    vs, ms, used = 0, 0.0, 0
    for i in order:
        c = cloths[i]
        cid = ctx.add_cloth(c)
        ctx.set_states(start[0][offs[i]:offs[i + 1]].copy(), start[1][offs[i]:offs[i + 1]].copy())
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
        vs += c.np * steps
        used += 1
        ctx.remove_cloth(cid)
        if ms / 1e3 > budget_s:
            break
    ctx.close()
    return {"value": vs / (ms / 1e3), "unit": UNIT,
            "sample": f"{used} cloths spread over the workload (every {stride}th), each alone in its own arena "
                      f"(FP64, tree-summed inner products), on the batched line's timed frames "
                      f"{warmup + 1}..{warmup + steps} from the batched FP64 run's start state"}


def small_config(device: int, frames: int = 300) -> dict:
    """The reference's own small case (21 x 21 sheet of 1 m over a sphere of
    radius 0.3, ILU(0)-PCG tol 1e-6, 300 frames) on the plain FP64 GPU path, the
    oracle restatement of the reference's CPU path timed beside it on one core."""
    import torch

    from cloth_sim_self_collision_gb300 import scene
    from cloth_sim_self_collision_gb300.context import ClothContext
    from oracle import oracle as O
    c = scene.config_small()
    ctx = ClothContext(device, "fp64")
    try:
        cid = ctx.add_cloth(c)
        ctx.set_state(cid, c.X0, np.zeros_like(c.X0))
        stream = torch.cuda.ExternalStream(ctx.stream(), device=device)
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.step(frames)
        e1.record(stream)
        torch.cuda.synchronize()
        gms = e0.elapsed_time(e1)
    finally:
        ctx.close()
    O.build("port")
    orc = O.OracleCloth(O.OracleLib("port"), c)
    t0 = time.perf_counter()
    orc.step(frames)
    cs = time.perf_counter() - t0
    return {"workload": f"21x21 sheet, 1 m, z 0.5 over a sphere of radius 0.3, ILU(0)-PCG tol 1e-6, "
                        f"{frames} frames from rest",
            "gpu_fp64": {"value": c.np * frames / (gms / 1e3), "ms_per_step": gms / frames},
            "cpu_port_1core": {"value": c.np * frames / cs, "ms_per_step": 1e3 * cs / frames}}


def serving(device: int, scenes: int, rate: float, steps: int, seed: int = 1, plain_budget_s: float = 40.0,
            plain: bool = True) -> dict:
    """The serving workload: scenes of log-uniform size (1e2..1e5 vertices) arriving
    as a Poisson process, each run for `steps` frames by the native server (one
    arena, continuous batching, admission by a 150 GB device-byte budget).
    Throughput counts the vertex-steps of scenes that finished; scenes whose frames
    blew up (CS_ERR_DIVERGED) are counted apart.  The plain FP64 path runs the
    same scenes, in arrival order, one per context for the same `steps` frames,
    until `plain_budget_s` of device time is used."""
    import torch

    from cloth_sim_self_collision_gb300 import _native as N
    from cloth_sim_self_collision_gb300 import scene
    from cloth_sim_self_collision_gb300.context import ClothContext
    from cloth_sim_self_collision_gb300.serve import Server
    cl = scene.config_serving(scenes)
    arr = np.cumsum(np.random.default_rng(seed).exponential(1.0 / rate, scenes))
    infos, diverged = [], 0
    with Server(device, "mixed", 150e9) as srv:
        reqs = []
        t0 = time.perf_counter()
        for c, a in zip(cl, arr):
            wait = a - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            reqs.append(srv.submit(c, steps))
        for c, r in zip(cl, reqs):
            try:
                infos.append((c, srv.wait(r, timeout=900.0)[2]))
            except N.CsError as e:
                if e.code != N.CS_ERR_DIVERGED:
                    raise
                diverged += 1
        st = srv.stats()
    done = [(c, i) for c, i in infos]
    span = max(i["t_done"] for _, i in done) - min(i["t_submit"] for _, i in done) if done else float("nan")
    vsteps = sum(c.np * steps for c, _ in done)
    out = {
        "workload": f"{scenes} scenes, vertex count log-uniform 1e2..1e5 (square grids), Poisson arrivals at "
                    f"{rate}/s, {steps} frames each, 150 GB admission budget, mixed precision",
        "rate_per_s": rate,
        "vertex_steps_per_s": vsteps / span if done else None, "completed": len(done), "diverged": diverged,
        "p50_step_ms": st["step_ms_p50"], "p99_step_ms": st["step_ms_p99"], "max_step_ms": st["step_ms_max"],
        "admit_ms_p50": st["admit_ms_p50"], "admit_ms_p99": st["admit_ms_p99"],
        "p50_request_s": float(np.percentile([i["t_done"] - i["t_submit"] for _, i in done], 50)) if done else None,
        "p99_request_s": float(np.percentile([i["t_done"] - i["t_submit"] for _, i in done], 99)) if done else None,
        "frames": st["frames"], "arena_swaps": st["rebuilds"], "build_ms_total": st["build_ms_total"],
        "swap_ms_total": st["install_ms_total"], "peak_bytes": st["peak_bytes"],
    }
    if not plain:
        return out
    # the plain FP64 path, one scene per context, on a sample of the same scenes
    ctx = ClothContext(device, "fp64")
    stream = torch.cuda.ExternalStream(ctx.stream(), device=device)
    pv, pms, used, tried = 0, 0.0, 0, 0
    for c in cl:
        cid = ctx.add_cloth(c)
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        tried += 1
        ms = e0.elapsed_time(e1)
        if not ctx.stats(cid)["diverged"]:
            pms += ms
            pv += c.np * steps
            used += 1
        ctx.remove_cloth(cid)
        if pms / 1e3 > plain_budget_s:
            break
    ctx.close()
    out["plain_gpu_fp64_one_per_launch"] = {
        "value": pv / (pms / 1e3) if pms > 0 else None, "unit": UNIT,
        "sample": f"first {tried} scenes in arrival order ({used} that did not blow up), each alone in its "
                  f"own arena for its {steps} frames"}
    if out["vertex_steps_per_s"] and out["plain_gpu_fp64_one_per_launch"]["value"]:
        out["vs_plain_gpu"] = out["vertex_steps_per_s"] / out["plain_gpu_fp64_one_per_launch"]["value"]
    return out


def single_cloths(device: int, frames: int = 5, warmup: int = 2) -> dict:
    """The single-cloth configurations (101x101 sheet of 2 m, 256x256 sheet of
    2 m): mixed precision against the plain FP64 path on the same cloth, frames
    warmup+1 .. warmup+frames, CUDA events on the library's stream."""
    import torch

    from cloth_sim_self_collision_gb300 import scene
    from cloth_sim_self_collision_gb300.context import ClothContext
    out = {}
    for name, make in (("single_101", scene.config_single_101), ("single_256", scene.config_single_256)):
        row = {}
        for prec in ("mixed", "fp64"):
            c = make()
            ctx = ClothContext(device, prec)
            cid = ctx.add_cloth(c)
            ctx.step(warmup)
            ctx.synchronize()
            stream = torch.cuda.ExternalStream(ctx.stream(), device=device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.step(frames)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            row[prec] = {"value": c.np * frames / (ms / 1e3), "ms_per_step": ms / frames,
                         "solver_iterations_last": ctx.stats(cid)["solver_iterations"]}
            ctx.close()
        row["vertices"] = c.np
        row["mixed_vs_fp64"] = row["mixed"]["value"] / row["fp64"]["value"]
        out[name] = row
    return out


def barrier(world):
    """All ranks meet here (torch.distributed over gloo when there are several)."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value, world):
    """The largest value over the ranks: a job's time is its slowest rank's."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def native(args):
    import torch

    from cloth_sim_self_collision_gb300 import build as B
    from cloth_sim_self_collision_gb300 import scene
    from cloth_sim_self_collision_gb300.context import ClothContext

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # replicas: each rank steps its own copy of the workload; the side
        # measurements (plain path, single cloths, serving, CPU sample) are
        # taken at one GPU only
        import torch.distributed as dist
        dist.init_process_group("gloo")
        args.no_plain = args.no_single = args.no_serve = args.no_cpu = args.no_small = True
    B.build()
    torch.cuda.set_device(local)
    cloths = scene.config_batch(count=args.cloths)

    results = {}
    for prec in (["mixed", "fp64"] if args.precision == "both" else [args.precision]):
        ctx = ClothContext(local, prec)
        ctx.frame_mode(args.frame_mode == "graph")
        ids = [ctx.add_cloth(c) for c in cloths]
        nv = ctx.num_vertices()
        nb_total = sum(int(ctx.pattern(i)[0][-1]) for i in ids)
        stream = torch.cuda.ExternalStream(ctx.stream(), device=local)
        clocks = ClockSampler(local)
        barrier(world)
        clocks.start()
        step_ms, launches, start, tune = timed_batch(ctx, args.steps, args.warmup, stream, nv,
                                                     0 if args.no_tune else 2, args.profile_window)
        clk = clocks.stop()
        barrier(world)
        total_ms = max_over_ranks(sum(step_ms), world)
        res = {"value": world * nv * args.steps / (total_ms / 1e3), "ms_per_step": total_ms / args.steps,
               "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
               "launches": launches, "clocks": clk, "nv": nv, "nb": nb_total, "start": start, "tune": tune,
               "frames": ctx.frame_counts()}
        if not results:
            # end to end through the C ABI, on the same frames: pinned host state
            # in, frame, state out
            xs = torch.empty(3 * nv, dtype=torch.float64, pin_memory=True)
            vs = torch.empty(3 * nv, dtype=torch.float64, pin_memory=True)
            xs.numpy()[:] = start[0]
            vs.numpy()[:] = start[1]
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            barrier(world)
            e0.record(stream)
            for _ in range(args.steps):
                ctx.set_states(xs.numpy(), vs.numpy())
                ctx.step(1)
                ctx.get_states(xs.numpy(), vs.numpy())
            e1.record(stream)
            torch.cuda.synchronize()
            barrier(world)
            e2e_ms = max_over_ranks(e0.elapsed_time(e1), world)
            res["e2e"] = {"value": world * nv * args.steps / (e2e_ms / 1e3), "unit": UNIT,
                          "h2d_bytes_per_step": 2 * 3 * nv * 8, "d2h_bytes_per_step": 2 * 3 * nv * 8}
            results["headline"] = prec
        # per-kernel times and device counters: a profiled replay of the timed frames
        res["prof"], res["counts"] = profiled_replay(ctx, args.steps, start, PROFILED)
        results[prec] = res
        ctx.close()
    head = results[results["headline"]]
    plain = None
    if not args.no_plain:
        st = results["fp64"]["start"] if "fp64" in results else head["start"]
        plain = plain_one_per_launch(cloths, local, args.steps, args.warmup, st)

    # Roofline: the solver kernel (HBM-bound; in mixed precision the persistent inner
    # CG, one launch per refinement cycle) with its algorithmic bytes counted on the
    # device per processed tile / row; the kernel with the largest share is reported
    # beside it (the FP64 narrow phase is bound by the FP64 pipe, not by HBM).
    prof = head["prof"]
    # the narrow phase's three kernels are timed both as one class and apart
    outer = {k: v for k, v in prof.items() if k not in NESTED}
    top = max(outer, key=lambda k: outer[k][0])
    total_kernel_ms = sum(v[0] for v in outer.values())
    peaks = read_peaks()
    figs = profile_figures()
    if results["headline"] == "mixed":
        spmv = "mx_persist" if prof["mx_persist"][1] else "mx_spmv"
    else:
        spmv = "cg_spmv"
    ms, n = prof[spmv]
    alg = head["counts"][{"mx_persist": "persist_bytes", "mx_spmv": "spmv32_bytes", "cg_spmv": "spmv64_bytes"}[spmv]]
    ratio = figs.get((spmv, "dram_per_algorithmic_byte"))
    roof = {"kernel": spmv, "bound": "hbm", "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "peak_source": peaks["source"], "launches": n, "avg_launch_us": 1e3 * ms / max(n, 1),
            "bytes_per_launch": alg / max(n, 1),
            "traffic": ratio * alg / max(n, 1) if ratio else None,
            "traffic_source": (f"ncu dram bytes / algorithmic bytes = {ratio} on a smaller arena "
                               f"(profiles/), scaled to this run's bytes per launch") if ratio else None,
            "achieved": (alg / max(n, 1)) / (ms / max(n, 1) / 1e3) / 1e9 if ms > 0 else None,
            "timing": "CUDA events around each launch on the library's stream, in a profiled replay of the "
                      "timed frames",
            "share_of_kernel_time": ms / total_kernel_ms if total_kernel_ms else None}
    roof["frac"] = roof["achieved"] / roof["peak"] if roof["achieved"] else None
    dominant = {"kernel": top, "share_of_kernel_time": prof[top][0] / total_kernel_ms if total_kernel_ms else None,
                "launches": prof[top][1], "avg_launch_us": 1e3 * prof[top][0] / max(prof[top][1], 1)}
    fp64_frac = figs.get((top, "fp64_pipe_active"))
    if fp64_frac is not None:
        dominant["bound"] = "fp64 pipe"
        dominant["fp64_pipe_active_frac"] = fp64_frac
        dominant["fp64_pipe_source"] = "sm__pipe_fp64_cycles_active from one ncu capture (profiles/)"

    if rank != 0:
        return
    hp = results["headline"]
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if hp == "mixed" else "f64", "data": "synthetic",
        "precision": hp,
        "config": workload_config(len(cloths), head["nv"]),
        "p50_step_ms": head["p50_step_ms"], "p99_step_ms": head["p99_step_ms"],
        "e2e": head["e2e"], "roofline": roof, "dominant_kernel": dominant,
        "gpu_launches": int(head["launches"]), "clocks": head["clocks"],
        "frame_graph": {"frames": head["frames"],
                        "note": "gpu_launches counts host-issued launches: one CUDA graph launch per graph "
                                "frame (kernels inside the graph are not counted), plus the launches of "
                                "frames re-run host-driven"},
        "autotune": head["tune"],
        "kernel_ms": {k: [round(v[0], 3), v[1]] for k, v in prof.items() if v[1]},
        "contact_counts": head["counts"],
    }
    for prec in ("mixed", "fp64"):
        if prec in results and prec != hp:
            r = results[prec]
            line[f"batched_{prec}"] = {"value": r["value"], "ms_per_step": r["ms_per_step"],
                                       "p50_step_ms": r["p50_step_ms"], "p99_step_ms": r["p99_step_ms"],
                                       "kernel_ms": {k: [round(v[0], 3), v[1]] for k, v in r["prof"].items() if v[1]}}
            # the FP64 SpMV of the FP64 path: its device-counted algorithmic bytes over
            # its time, as a fraction of HBM (it is bound by the FP64 pipe: the row's
            # blocks are added in the reference's order on one lane)
            ms64, n64 = r["prof"].get("cg_spmv", (0.0, 0))
            b64 = r["counts"].get("spmv64_bytes", 0)
            if ms64 > 0 and b64 > 0:
                ach = b64 / (ms64 / 1e3) / 1e9
                line[f"batched_{prec}"]["roofline_cg_spmv"] = {
                    "kernel": "cg_spmv", "bound": "fp64 pipe", "launches": n64,
                    "bytes_per_launch": b64 / max(n64, 1), "achieved": ach, "unit": "GB/s",
                    "hbm_frac": ach / peaks["hbm_gbs"]}
    if plain is not None:
        line["plain_gpu_fp64_one_per_launch"] = plain
        line["vs_plain_gpu"] = head["value"] / plain["value"]
    if not args.no_small:
        line["small_21"] = small_config(local)
    if not args.no_single:
        line["single_cloth"] = single_cloths(local)
    if not args.no_serve:
        line["serving"] = serving(local, args.serve_scenes, args.serve_rate, args.serve_steps)
        if args.serve_rates:
            # the latency / throughput curve over the arrival rate (the plain path
            # is the one measured above: the same scenes in the same order)
            pl = line["serving"]["plain_gpu_fp64_one_per_launch"]["value"]
            sweep = []
            for r in (float(t) for t in args.serve_rates.split(",")):
                row = serving(local, args.serve_scenes, r, args.serve_steps, plain=False)
                if row["vertex_steps_per_s"] and pl:
                    row["vs_plain_gpu"] = row["vertex_steps_per_s"] / pl
                sweep.append(row)
            line["serving_sweep"] = sweep
    if not args.no_cpu:
        line["cpu_baseline"] = run_cpu_baseline(cloths)
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------
_W = {}


def _ref_init(lib_kind, cloth_args):
    from cloth_sim_self_collision_gb300 import scene
    from oracle import oracle as O
    lib = O.OracleLib(lib_kind)
    allc = scene.config_batch(count=cloth_args[0])
    _W["sims"] = [O.OracleCloth(lib, allc[i]) for i in cloth_args[1]]


def _ref_step(_):
    t0 = time.perf_counter()
    n = 0
    for s in _W["sims"]:
        s.step(1)
        n += s.n
    return n, time.perf_counter() - t0


def reference(args):
    """The reference's CPU path on the host cores: the reference build where it
    exists on this machine, else the oracle restatement; cloths spread over all
    cores, one frame of each per step."""
    import multiprocessing as mp

    from cloth_sim_self_collision_gb300 import scene
    from oracle import oracle as O
    if int(os.environ.get("RANK", "0")) != 0:
        return
    kind = "reference" if O.ref_available() else "port"
    lib_kind = "ref" if kind == "reference" else "port"
    if kind == "port":
        O.build("port")
    cores = os.cpu_count() or 1
    n = args.ref_cloths
    groups = [list(range(w, n, cores)) for w in range(cores)]
    groups = [g for g in groups if g]
    ctx = mp.get_context("spawn")
    pools = [ctx.Pool(1, initializer=_ref_init, initargs=(lib_kind, (args.cloths, g))) for g in groups]
    try:
        def one_step():
            t0 = time.perf_counter()
            res = [p.apply_async(_ref_step, (0,)) for p in pools]
            out = [r.get() for r in res]
            return sum(o[0] for o in out), time.perf_counter() - t0

        for _ in range(args.warmup):
            one_step()
        vs, t = 0, 0.0
        step_s = []
        for _ in range(args.steps):
            a, b = one_step()
            vs += a
            t += b
            step_s.append(b)
    finally:
        for p in pools:
            p.terminate()
    value = vs / t
    sample = (f"{n} of the workload's cloths, one frame each per step, spread over {len(groups)} processes "
              f"on {cores} host cores ({'reference sources' if kind == 'reference' else 'oracle restatement'})")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "precision": "fp64 (CPU)",
        "config": workload_config(args.cloths, workload_vertices(scene.config_batch(count=args.cloths))),
        "p50_step_ms": 1e3 * float(np.percentile(step_s, 50)), "p99_step_ms": 1e3 * float(np.percentile(step_s, 99)),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": len(groups), "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--cloths", type=int, default=512)
    ap.add_argument("--ref-cloths", type=int, default=512)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-cloth-per-launch FP64 sample")
    ap.add_argument("--precision", default="both", choices=["both", "mixed", "fp64"],
                    help="both: mixed is the headline, FP64 batched reported beside it")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving workload")
    ap.add_argument("--no-single", action="store_true", help="skip the single-cloth configurations")
    ap.add_argument("--no-small", action="store_true", help="skip the 21x21 ILU(0)-PCG sheet")
    ap.add_argument("--frame-mode", default="graph", choices=["graph", "host"],
                    help="frames as one captured CUDA graph each (default) or host-driven (profilers that "
                         "cannot see into conditional graph nodes)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes (no autotuning)")
    ap.add_argument("--profile-window", action="store_true",
                    help="cudaProfilerStart/Stop around the timed frames (ncu --profile-from-start off)")
    ap.add_argument("--serve-scenes", type=int, default=24)
    ap.add_argument("--serve-rate", type=float, default=2.0, help="Poisson arrival rate, scenes per second")
    ap.add_argument("--serve-steps", type=int, default=200)
    ap.add_argument("--serve-rates", default="",
                    help="comma-separated Poisson arrival rates for a latency / throughput sweep of the server")
    args = ap.parse_args()
    if args.warmup < 0 or args.steps < 1:
        raise SystemExit("need --steps >= 1 and --warmup >= 0")
    if args.impl == "reference":
        reference(args)
    else:
        native(args)


if __name__ == "__main__":
    main()
