#!/usr/bin/env python
"""Benchmark of the ghost-update + red-black SOR path on one GB300.

Workload (the configuration the headline metric is quoted on): the two-level
octree -- a 4x4x4 root grid over [0,1]^3 refined to level 3 where blocks meet
the sphere |x - (0.5,0.5,0.5)| = 0.3, 2:1 balanced -- with 16^3 cells per
block and a 2-cell virtual layer, FP32, right-hand side a seeded Gaussian blob
(sigma 0.1) plus uniform[-0.01,0.01] noise, Dirichlet 0 on the outer faces.

One step = 500 red-black SOR iterations at omega = 1.8 (sor2's scheme), each
followed by the ghost update over all same-level, F2C and C2F faces.  The
field plus the source are 284 MB (padded bricks), larger than the 129 MB L2.
The same workload runs again in FP64 (the reference's own precision for this
scheme) and is reported beside the FP32 headline under "fp64"; short samples
of C1's structure at flat level 5 and of the C3 mixed-precision solve follow
under "other_workloads" (--no-side leaves them out).

  value  Gcell-updates/s with data resident in HBM (CUDA events on the stream)
  e2e    same metric through the public API from pinned host buffers, with the
         upload of f and s and the download of f inside every timed step
  cpu_baseline / --impl reference   the reference's own OpenMP CPU path,
         compiled from its sources (oracle/_ref/refbench: sor2's Solver sweep
         and Dirichlet code, BlockManager + Scalar3DUpdater<double> ghost
         update), FP64, on all host cores (and one core for cpu_baseline),
         same mesh and source, a bounded sample of iterations per step; the
         oracle's C port where that binary was not built.

With torchrun (N > 1) every rank runs an independent replica (the path has
no cross-GPU exchange on one rank per GPU); value sums all replicas' cells
over the slowest rank's time.
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

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ITERS_PER_STEP = 500
OMEGA = 1.8
N_CELL = 16
VC = 2


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


L2_BYTES = 120e6  # GB300 L2 (126 MB) less headroom: the batched sets' working-set bound


def profile_traffic(name: str):
    """Per-launch DRAM bytes of the named kernel from a committed ncu summary."""
    p = ROOT / "profiles" / f"{name}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_full_workload:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.proc, self.lines = device, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(ms: float, pg, device: str = "cpu") -> float:
    """Slowest rank's time (all-reduce MAX); the local value without a group."""
    if pg is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cells_per_rank: int, iters_per_step: int, steps: int, world: int,
                   ms_max: float) -> float:
    """Gcell-updates/s of all replicas over the slowest rank's time (weak scaling)."""
    return cells_per_rank * iters_per_step * steps * world / (ms_max / 1e3) / 1e9


def make_problem(workload_dtype="f32"):
    import bcmtools_gb300 as bg
    from bcmtools_gb300 import workloads as W
    w = W.two_level_sphere(n=N_CELL, vc=VC)
    dt = np.float32 if workload_dtype == "f32" else np.float64
    s_host = W.rhs_gaussian(w, seed=2, dtype=dt)
    bct, bcv = w.dirichlet(0.0)
    coef = bg.sor2_coef(w.tree.cell_sizes(w.n))
    return w, s_host, bct, bcv, coef


WORKLOAD_NAME = ("two_level_sphere: root 4^3, sphere r=0.3 to level 3, 2:1 balanced, "
                 "16^3 cells/block, vc=2, RB-SOR omega=1.8")


# --------------------------------------------------------------------------
# CPU legs: the reference's own compiled path (oracle/_ref/refbench: sor2's
# Solver sweep and Dirichlet code, BlockManager + Scalar3DUpdater<double>
# ghost update, OpenMP), FP64 as the reference's sor2 is; the oracle's C port
# where that binary was not built.
def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_sample(w, s64, threads: int, seconds: float, max_iters: int = ITERS_PER_STEP):
    """Iterations of the reference path on the full mesh sized to about
    `seconds`: (Gcell-updates/s, iterations, seconds)."""
    from oracle import refbench_io
    t1, _ = refbench_io.run(w.tree, w.n, w.vc, s64, OMEGA, threads, 0, 1)
    iters = max(1, min(max_iters, int(seconds / max(t1, 1e-6))))
    sec, _ = refbench_io.run(w.tree, w.n, w.vc, s64, OMEGA, threads, 1, iters)
    return w.cells * iters / sec / 1e9, iters, sec


def port_sample(w, s_host, bct, bcv, coef, seconds: float):
    """The oracle's C restatement (OpenMP over blocks and faces)."""
    from oracle import pyoracle as po
    ld, nid, sf, _ = w.neighbors()
    m = po.OracleMesh(ld, nid, sf, w.n, w.vc)
    f = np.zeros(m.shape, s_host.dtype)
    m.vc_update(f)
    m.dirichlet(f, bct, bcv, 0)
    t0 = time.perf_counter()
    m.sor_run(f, coef, OMEGA, 2, 1, 1, bct, bcv, 0, s=s_host)
    t1 = time.perf_counter() - t0
    iters = max(1, min(ITERS_PER_STEP, int(seconds / max(t1, 1e-6))))
    t0 = time.perf_counter()
    m.sor_run(f, coef, OMEGA, 2, 1, iters, bct, bcv, 0, s=s_host)
    el = time.perf_counter() - t0
    return w.cells * iters / el / 1e9, iters, po.num_threads()


def cpu_baseline_sample(w, s64, bct, bcv, coef):
    """rank 0, N = 1: the reference path on all host cores and on one core
    (about 12 s and 8 s of CPU work), else the port on all cores."""
    from oracle import refbench_io
    if refbench_io.available():
        cores = host_cores()
        v, it, _ = reference_sample(w, s64, cores, 12.0)
        v1, it1, _ = reference_sample(w, s64, 1, 8.0)
        return {"value": v, "unit": "Gcell/s", "cores": cores, "kind": "reference",
                "dtype": "f64",
                "sample": f"{it} RB-SOR iterations (sweep + Dirichlet + ghost update) of the full "
                          f"{w.nb}-block mesh, FP64, the reference's compiled sor2 Solver sweep "
                          f"and BlockManager/Scalar3DUpdater<double> (oracle/_ref/refbench), "
                          f"OpenMP on {cores} threads",
                "single_core": {"value": v1, "cores": 1, "iterations": it1}}
    v, it, cores = port_sample(w, s64.astype(np.float32), bct, bcv, coef, 12.0)
    return {"value": v, "unit": "Gcell/s", "cores": cores, "kind": "port", "dtype": "f32",
            "sample": f"{it} RB-SOR iterations of the full {w.nb}-block mesh, FP32, "
                      "oracle/bcm_oracle.c with OpenMP (the reference's compiled path was not "
                      "built on this host)"}


def run_reference(args):
    """Reference arm: the reference's own compiled CPU path on every host
    core, FP64 (its sor2 Solver is Scalar3D<double> only), same mesh and
    source; one step = a bounded sample of iterations of the full mesh."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import refbench_io
    w, s64, bct, bcv, coef = make_problem("f64")
    cores = host_cores()
    if refbench_io.available():
        t1, _ = refbench_io.run(w.tree, w.n, w.vc, s64, OMEGA, cores, 0, 1)
        budget = 120.0 / max(1, args.steps + args.warmup)
        per_step = max(1, min(ITERS_PER_STEP, int(budget / max(t1, 1e-6))))
        sec, _ = refbench_io.run(w.tree, w.n, w.vc, s64, OMEGA, cores,
                                 args.warmup * per_step, args.steps * per_step)
        kind, dtype = "reference", "f64"
        how = ("the reference's compiled sor2 Solver sweep + Dirichlet ghosts and "
               "BlockManager/Scalar3DUpdater<double> ghost update (oracle/_ref/refbench), "
               f"OpenMP on {cores} threads, FP64")
    else:
        import time as _t
        from oracle import pyoracle as po
        s32 = s64.astype(np.float32)
        ld, nid, sf, _ = w.neighbors()
        m = po.OracleMesh(ld, nid, sf, w.n, w.vc)
        f = np.zeros(m.shape, np.float32)
        m.vc_update(f)
        m.dirichlet(f, bct, bcv, 0)
        t0 = _t.perf_counter()
        m.sor_run(f, coef, OMEGA, 2, 1, 1, bct, bcv, 0, s=s32)
        t1 = _t.perf_counter() - t0
        budget = 120.0 / max(1, args.steps + args.warmup)
        per_step = max(1, min(ITERS_PER_STEP, int(budget / max(t1, 1e-6))))
        m.sor_run(f, coef, OMEGA, 2, 1, args.warmup * per_step, bct, bcv, 0, s=s32)
        t0 = _t.perf_counter()
        m.sor_run(f, coef, OMEGA, 2, 1, args.steps * per_step, bct, bcv, 0, s=s32)
        sec = _t.perf_counter() - t0
        kind, dtype, cores = "port", "f32", po.num_threads()
        how = ("the oracle's C restatement of the reference path (oracle/bcm_oracle.c, OpenMP), "
               "FP32: the reference's compiled path was not built on this host")
    v = w.cells * per_step * args.steps / sec / 1e9
    sample = f"{per_step} RB-SOR iterations of the full {w.nb}-block mesh per step, {how}"
    line = {"metric": "Gcell-updates/s", "value": v, "unit": "Gcell/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded Gaussian blob + noise RHS)", "impl": "reference",
            "config": {"workload": WORKLOAD_NAME, "blocks": w.nb, "cells": w.cells,
                       "iters_per_step": per_step, "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": v, "unit": "Gcell/s", "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": v, "unit": "Gcell/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def first_layer_ghosts(w, bct) -> int:
    """Ghost cells of the first layer that have a value source: every face
    with a neighbour (same level, coarser, or finer: the four F2C subfaces
    cover it) or a Dirichlet condition.  The pull-form fused sweep pulls
    exactly these per launch; its deeper layers are written only by the
    ghost update that closes a run."""
    ld, nid, _, _ = w.neighbors()
    n = w.n
    has = (nid >= 0).any(axis=2) | (np.asarray(bct) == 1)
    return int(has.sum()) * n * n


def ghost_cells_per_update(w, bct) -> int:
    """Ghost cells one full VC update + Dirichlet writes (face-table box sizes)."""
    ld, nid, _, _ = w.neighbors()
    n, vc = w.n, w.vc
    has = nid >= 0
    same = ((ld == 0) & has[:, :, 0]).sum() * vc * n * n
    c2f = ((ld == -1) & has[:, :, 0]).sum() * vc * n * n
    f2c = ((ld == 1)[:, :, None] & has).sum() * vc * (n // 2) ** 2
    dirichlet = (np.asarray(bct) == 1).sum() * n * n
    return int(same + c2f + f2c + dirichlet)


SHAPES = {6: "fused RB-SOR, pull-form ghosts, persistent pipeline (sweep_pipe_kernel, 2 stages), "
             "shape 6",
          7: "fused RB-SOR, pull-form ghosts, one CTA per block (sweep_pipe_kernel, 1 stage), "
             "shape 7"}


def measure_sor(args, bm, w, s_host, bct, coef, dtype, stream, world, pg, local, variant):
    """One precision of the benchmark: the timed region (data resident), the
    per-kernel breakdown, the roofline of the SOR kernel and the end-to-end
    number through the public API from pinned host buffers."""
    import torch

    import bcmtools_gb300 as bg
    sh = stream.cuda_stream
    es = 4 if dtype == "f32" else 8
    tdt = torch.float32 if dtype == "f32" else torch.float64
    f = bm.setDataClass(dtype, w.vc)
    s = bm.setDataClass(dtype, w.vc)
    bm.prepareForVCUpdate(f, 100, bg.VCUpdateMethod.AtOnce)
    s.upload(s_host)

    def step():
        bm.sor_run(f, coef, OMEGA, form=2, n_inner=1, n_outer=ITERS_PER_STEP, s=s, stream=sh)

    def barrier():
        if pg is not None:
            pg.barrier()

    f.fill(0.0, stream=sh)
    bm.imposeBoundaryCondition(f, stream=sh)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    l0 = bm.launch_count()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = bm.launch_count() - l0
    clk = clocks.stop()
    ms_max = max_over_ranks(ms, pg, f"cuda:{local}" if pg is not None and
                            pg.get_backend() == "nccl" else "cpu")
    value = whole_job_rate(w.cells, ITERS_PER_STEP, args.steps, world, ms_max)

    # per-kernel device time (events around each launch, separate pass)
    bm.profile_begin()
    for _ in range(max(1, min(args.steps, 5))):
        step()
    prof = bm.profile_end()
    sor_ms, sor_n = prof["sor_rb"]
    tot_ms = sum(v[0] for v in prof.values())
    # algorithmic bytes of one launch: read f, read s, write f per interior
    # cell, plus the first ghost layer the pull-form kernel reads from its
    # neighbours (the deeper layers are written only by the closing update)
    ghosts = first_layer_ghosts(w, bct) if variant in SHAPES else ghost_cells_per_update(w, bct)
    bytes_per_launch = 3 * es * w.cells + es * ghosts
    # average SOR launch duration over the timed region: its events' time per
    # iteration, less the share of the other kernels (source packing, the
    # closing ghost update) measured in the per-kernel pass.  Consecutive
    # launches of a run overlap their start with the previous one's end
    # (programmatic dependent launch), which events around every launch in the
    # per-kernel pass would prevent.
    sor_share = sor_ms / tot_ms if tot_ms else 1.0
    avg_s = ms / 1e3 / args.steps / ITERS_PER_STEP * sor_share
    achieved = bytes_per_launch / avg_s / 1e9
    peak, peak_kind = load_peaks()
    traffic = profile_traffic(f"sor_rb_two_level_sphere{'' if dtype == 'f32' else '_f64'}")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "dram_frac": (traffic / avg_s / 1e9 / peak) if traffic else None,
                "kernel": SHAPES.get(variant, f"fused RB-SOR + ghost push, shape {variant}"),
                "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": bytes_per_launch,
                "first_layer_ghosts": ghosts,
                "avg_launch_us": avg_s * 1e6,
                "isolated_launch_us": sor_ms / max(sor_n, 1) * 1e3}
    kernels = {k: {"ms": v[0], "launches": v[1], "share": (v[0] / tot_ms if tot_ms else 0.0)}
               for k, v in prof.items() if v[1]}
    if dtype == "f64":
        # the FP64 sweep is bound by GB300's FP64 pipe, not by HBM: sor2's
        # update is 13 separately rounded FP64 adds and multiplies per cell
        # (no contraction, for bit parity with the reference), against a
        # nominal 1.25 TFLOP/s (0.625 T adds or multiplies per second)
        roofline["fp64_pipe"] = {"ops_per_cell": 13,
                                 "achieved_tops": 13 * w.cells / avg_s / 1e12,
                                 "nominal_tops": 0.625,
                                 "frac": 13 * w.cells / avg_s / 1e12 / 0.625}

    # end to end through the public API from pinned host buffers
    f_pin = torch.empty(f.shape, dtype=tdt, pin_memory=True).numpy()
    s_pin = torch.empty(s.shape, dtype=tdt, pin_memory=True).numpy()
    s_pin[...] = s_host
    f_pin[...] = 0.0
    e2e_steps = max(1, min(args.steps, 3))
    lib, ctx = bm.lib, bm.ctx
    e0.record(stream)
    for _ in range(e2e_steps):
        lib.bcmg_field_upload(ctx, f.id, f_pin.ctypes.data, sh)
        lib.bcmg_field_upload(ctx, s.id, s_pin.ctypes.data, sh)
        bm.imposeBoundaryCondition(f, stream=sh)
        step()
        lib.bcmg_field_download(ctx, f.id, f_pin.ctypes.data, sh)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    e2e = {"value": w.cells * ITERS_PER_STEP * e2e_steps / (e2e_ms / 1e3) / 1e9,
           "unit": "Gcell/s", "h2d_bytes_per_step": int(f_pin.nbytes + s_pin.nbytes),
           "d2h_bytes_per_step": int(f_pin.nbytes), "steps": e2e_steps}
    padded_mb = 2 * f_pin.nbytes / 1e6
    bm.destroy(f)
    bm.destroy(s)
    return {"value": value, "ms_per_step": ms_max / args.steps, "gpu_launches": launches,
            "clocks": clk, "roofline": roofline, "kernels": kernels, "e2e": e2e,
            "padded_mb": padded_mb}


def run_ours(args):
    import torch

    import bcmtools_gb300 as bg

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if dist.is_nccl_available() else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist

    w, s32, bct, bcv, coef = make_problem("f32")
    _, s64, _, _, _ = make_problem("f64")
    bm = bg.BlockManager(local)
    bm.register_octree(w.tree, w.n)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    stream = torch.cuda.Stream(device=local)
    sh = stream.cuda_stream

    if args.profile:
        # short case for ncu: a few fused SOR iterations of one kernel shape
        dt = "f64" if args.dtype == "f64" else "f32"
        f = bm.setDataClass(dt, w.vc)
        s = bm.setDataClass(dt, w.vc)
        bm.prepareForVCUpdate(f, 100, bg.VCUpdateMethod.AtOnce)
        s.upload(s64 if dt == "f64" else s32)
        f.fill(0.0, stream=sh)
        bm.imposeBoundaryCondition(f, stream=sh)
        bm.set_sor_variant(args.variant)
        # (10 iterations: runs of 8 or more read the packed source, as the bench does)
        bm.sor_run(f, coef, OMEGA, form=2, n_inner=1, n_outer=10, s=s, stream=sh)
        torch.cuda.synchronize()
        print(f"profile case done: 10 {dt} SOR iterations of the benchmark mesh, "
              f"shape {args.variant}")
        return 0
    # kernel shape: forced, tuned on a copy of f (--autotune; setup, outside
    # the timed region), or the library's default for this shape (the pull
    # form one CTA per block, shape 7) -- the default keeps a profiled run on
    # the same kernels as a plain one
    variant_us = None
    if args.sor_shape:
        bm.set_sor_variant(args.sor_shape)
        variant = args.sor_shape
    elif args.autotune:
        tf = bm.setDataClass("f32", w.vc)
        ts = bm.setDataClass("f32", w.vc)
        ts.upload(s32)
        variant, variant_us = bm.autotune_sor(tf, coef, OMEGA, form=2, s=ts, iters=20)
        bm.destroy(tf)
        bm.destroy(ts)
    else:
        variant = 7
    r32 = measure_sor(args, bm, w, s32, bct, coef, "f32", stream, world, pg, local, variant)
    r64 = None if args.dtype == "f32" else measure_sor(args, bm, w, s64, bct, coef, "f64", stream,
                                                       world, pg, local, variant)

    if rank == 0:
        cpu = cpu_baseline_sample(w, s64, bct, bcv, coef) if world == 1 else None
        side = side_workloads(local) if world == 1 and not args.no_side else None
        line = {"metric": "Gcell-updates/s", "value": r32["value"], "unit": "Gcell/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": r32["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded Gaussian blob + noise RHS)",
                "config": {"workload": WORKLOAD_NAME,
                           "blocks": w.nb, "cells": w.cells, "iters_per_step": ITERS_PER_STEP,
                           "l2": "inputs larger than L2 (f + s padded = "
                                 f"{r32['padded_mb']:.0f} MB in FP32, "
                                 f"{2 * r32['padded_mb']:.0f} MB in FP64)",
                           "parallelism": f"replicas x{world}",
                           "sor_kernel_shape": variant, "tuned_us_per_iter": variant_us},
                "gpu_launches": r32["gpu_launches"] + (r64["gpu_launches"] if r64 else 0),
                "clocks": r32["clocks"], "roofline": r32["roofline"],
                "kernels": r32["kernels"], "e2e": r32["e2e"], "cpu_baseline": cpu}
        if r64:
            line["fp64"] = {"value": r64["value"], "unit": "Gcell/s", "dtype": "f64",
                            "ms_per_step": r64["ms_per_step"], "e2e": r64["e2e"],
                            "roofline": r64["roofline"], "kernels": r64["kernels"],
                            "clocks": r64["clocks"], "gpu_launches": r64["gpu_launches"],
                            "note": "same workload in FP64, bit-exact with the reference's "
                                    "sor2 scheme (the reference's own dtype)"}
        if side:
            line["other_workloads"] = side
        print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()
    return 0


def side_workloads(local: int) -> dict:
    """The other configurations measured in the default run, one short
    sample each, so that the default line carries them too: C1's structure at
    flat level 5 (32768 blocks of 16^3, 134 M cells: 200 fused Jacobi sweeps
    with the ghost update, one CUDA-graph replay) and C3 (the mixed-precision
    BiCGSTAB on the level-5 points mesh to 1e-10, its error against the FP64
    CPU oracle's solution)."""
    import torch

    import bcmtools_gb300 as bg
    from bcmtools_gb300 import workloads as W
    out = {}
    peak, _ = load_peaks()
    # C1 structure at level 5
    w = W.plain_poisson(n=16, vc=1, level=5)
    bm = bg.BlockManager(local)
    bm.register_octree(w.tree, w.n)
    bct, bcv = w.dirichlet(0.0)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    x, b = bm.setDataClass("f32", 1), bm.setDataClass("f32", 1)
    b.upload(W.rhs_uniform(w, seed=1, dtype=np.float32))
    op = bm.op_const(bg.laplace_coef(w.tree.cell_sizes(w.n)))
    stream = torch.cuda.Stream(device=local)
    sh = stream.cuda_stream
    x.fill(0.0, stream=sh)
    bm.imposeBoundaryCondition(x, stream=sh)
    bm.jacobi_run(op, x, b, 1.0, 200, use_graph=True, stream=sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    bm.jacobi_run(op, x, b, 1.0, 200, use_graph=True, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    bpl = 3 * 4 * w.cells + 4 * first_layer_ghosts(w, bct)
    out["c1_level5_jacobi"] = {
        "workload": "flat level 5, 32768 blocks of 16^3 (134 M cells), vc=1, FP32, 200 fused "
                    "Jacobi sweeps + ghost update per step (one CUDA-graph replay)",
        "gcell_updates_per_s": w.cells * 200 / (ms / 1e3) / 1e9, "ms_per_sweep": ms / 200,
        "hbm_frac": bpl / (ms / 1e3 / 200) / 1e9 / peak,
        "algorithmic_bytes_per_sweep": bpl}
    bm.close()
    del bm
    # C3
    w = W.points_level5()
    bm = bg.BlockManager(local)
    bm.register_octree(w.tree, w.n)
    t, v = w.dirichlet(0.0)
    bm.set_boundary(t, v, bg.DIRICHLET_SOR)
    op = bm.op_const(bg.laplace_coef(w.tree.cell_sizes(w.n)))
    x, b = bm.setDataClass("f64", 1), bm.setDataClass("f64", 1)
    b.fill(0.0)
    b.fill_random(3)

    def solve(max_outer):
        x.fill(0.0)
        bm.imposeBoundaryCondition(x)
        return bm.bicgstab_mixed(op, x, b, omega=0.8, n_pre=2, max_inner=200, eps_inner=1e-2,
                                 max_outer=max_outer, eps=1e-10)

    solve(1)  # first use: work vectors, kernels
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    info = solve(60)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    c3 = {"workload": f"mixed-precision BiCGSTAB, points_level5: {w.nb} blocks of 32^3 "
                      f"({w.cells} cells), vc=1, to 1e-10",
          "seconds": secs, "iterations": info.iterations, "refinements": info.refinements,
          "fp64_iterations": info.fp64_iterations, "true_residual": info.true_residual,
          "effective_GBps": (26 + 6 * 2) * 4 * w.cells * info.iterations / secs / 1e9}
    fx = ROOT / "tests" / "golden" / "c3_points_level5_fp64.npz"
    if fx.exists():
        g = np.load(fx)
        if int(g["nb"]) == w.nb and np.array_equal(g["pedigrees"], w.tree.pedigrees):
            xi = x.download()[:, 1:-1, 1:-1, 1:-1]
            c3["max_rel_error_vs_cpu_oracle"] = float(
                np.abs(xi[g["sample_ids"]] - g["sample_blocks"]).max() / float(g["xmax"]))
    out["c3_mixed_bicgstab"] = c3
    bm.close()
    return out


def run_jacobi(args):
    """Plain single-level Poisson (512 blocks of 16^3, vc=1, FP32, RHS uniform
    [-1,1] minus its mean, Dirichlet 0): one step = 200 Jacobi sweeps, each
    with the ghost update and Dirichlet ghosts of the new iterate (fused, one
    launch per sweep, replayed as one CUDA graph).  --workload
    plain_poisson_l5 runs the same structure at flat level 5 (32768 blocks,
    134 M cells, 1.6 GB per sweep) so the sweep streams from HBM."""
    import torch

    import bcmtools_gb300 as bg
    from bcmtools_gb300 import workloads as W
    level = 5 if args.workload == "plain_poisson_l5" else 3
    sweeps = 200
    w = W.plain_poisson(n=16, vc=1, level=level)
    torch.cuda.set_device(0)
    bm = bg.BlockManager(0)
    bm.register_octree(w.tree, w.n)
    bct, bcv = w.dirichlet(0.0)
    bm.set_boundary(bct, bcv, bg.DIRICHLET_SOR)
    bm.set_jacobi_shape(args.jacobi_shape)
    x, b = bm.setDataClass("f32", 1), bm.setDataClass("f32", 1)
    b.upload(W.rhs_uniform(w, seed=1, dtype=np.float32))
    op = bm.op_const(bg.laplace_coef(w.tree.cell_sizes(w.n)))
    stream = torch.cuda.Stream(device=0)
    sh = stream.cuda_stream
    x.fill(0.0, stream=sh)
    bm.imposeBoundaryCondition(x, stream=sh)
    # fused-Jacobi kernel choice: forced, tuned on a copy of x (--autotune;
    # setup, outside the timed region), or the library's default by mesh size
    # (push form up to 1024 blocks, pull form one CTA per block beyond)
    if args.jacobi_shape:
        choice, choice_us = {1: 2, 2: 3}[args.jacobi_shape], None
    elif args.autotune:
        choice, choice_us = bm.autotune_jacobi(op, x, b, 1.0, iters=20)
    else:
        choice, choice_us = (1 if w.nb <= 1024 else 2), None
    if args.profile:
        # short case for ncu: a few fused Jacobi sweeps
        bm.jacobi_run(op, x, b, 1.0, 5, use_graph=False, stream=sh)
        torch.cuda.synchronize()
        print(f"profile case done: 5 Jacobi sweeps, {args.workload}")
        return 0
    for _ in range(args.warmup):
        bm.jacobi_run(op, x, b, 1.0, sweeps, use_graph=True, stream=sh)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = bm.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        bm.jacobi_run(op, x, b, 1.0, sweeps, use_graph=True, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = bm.launch_count() - l0
    clk = clocks.stop()
    bm.profile_begin()
    bm.jacobi_run(op, x, b, 1.0, 20, use_graph=False, stream=sh)
    prof = bm.profile_end()
    jms, jn = prof["jacobi"]
    bytes_per_launch = 3 * 4 * w.cells + 4 * ghost_cells_per_update(w, bct)
    avg_s = jms / max(jn, 1) / 1e3
    peak, peak_kind = load_peaks()
    rr = bm.calc_r2(op, x, b)
    value = w.cells * sweeps * args.steps / (ms / 1e3) / 1e9
    resident = "L2-resident" if w.cells * 12 < 100e6 else "larger than L2"
    line = {"metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded uniform RHS, mean removed)",
            "config": {"workload": f"{args.workload}: flat level {level}, {w.nb} blocks of 16^3, "
                                   f"vc=1, {sweeps} Jacobi sweeps + ghost update per step",
                       "cells": w.cells, "l2": f"working set {resident}"},
            "gpu_launches": launches, "clocks": clk,
            "roofline": {"bound": "hbm", "achieved": bytes_per_launch / avg_s / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": bytes_per_launch / avg_s / 1e9 / peak,
                         "traffic": (profile_traffic("jacobi_plain_poisson_l5")
                                     if level == 5 and choice == 2 else None),
                         "kernel": {1: "fused Jacobi, push-form ghosts (jacobi_tile_kernel)",
                                    2: "fused Jacobi, pull-form ghosts, one CTA per block "
                                       "(jacobi_tile_kernel)",
                                    3: "fused Jacobi, pull-form ghosts, persistent pipeline "
                                       "(sweep_pipe_kernel)"}.get(choice, "separate launches"),
                         "tuned_us_per_sweep": choice_us,
                         "peak_source": peak_kind, "avg_launch_us": avg_s * 1e6,
                         "algorithmic_bytes_per_launch": bytes_per_launch},
            "residual_l2": float(np.sqrt(rr))}
    print(json.dumps(line))
    return 0


def run_batched(args):
    """Batched instances: 256 seeded instances (seeds 1000..1255; blocks
    log-uniform in [64, 4096]; block edge drawn from {8, 16, 32}; RHS uniform
    [-1,1]; Dirichlet 0), one block set per block edge streamed from HBM
    (bcmtools_gb300.batch.plan_block_sets; with --l2-sets the 8^3 instances
    go into L2-sized sets instead: measured slower, as were L2-sized sets of
    16^3 and 32^3 blocks, a couple of waves of CTAs each), its fused-Jacobi
    kernel autotuned on the set (bcmg_autotune_jacobi); each set swept by a
    CUDA-graph-replayed fused Jacobi run, one set after another on one stream;
    against the same instances solved one after another, each in its own
    context.  A step = `--batch-iters` Jacobi sweeps + ghost update of every
    instance."""
    import torch

    import bcmtools_gb300 as bg
    from bcmtools_gb300 import workloads as W
    from bcmtools_gb300.batch import Batch, brick_bytes, group_by_shape, plan_block_sets
    torch.cuda.set_device(0)
    iters = args.batch_iters
    seeds = list(range(1000, 1256))
    ws = [W.random_instance(s) for s in seeds]
    seed_of = {id(w): s for w, s in zip(ws, seeds)}
    cells = sum(w.cells for w in ws)
    # ---- batched: block sets per block edge, on --batch-streams streams ------
    runs = []
    stream = torch.cuda.Stream(device=0)
    for (n, vc), grp in sorted(group_by_shape(ws).items()):
        # one set per block edge; --l2-sets packs L2-sized sets where one holds
        # 2048 blocks or more (8^3 here), measured slower on this mix
        for chunk in plan_block_sets(grp, L2_BYTES,
                                     min_set_blocks=2048 if args.l2_sets else 1 << 40):
            bt = Batch(chunk)
            bt.set_dirichlet(0.0)
            op = bt.laplace_op()
            x, b = bt.bm.setDataClass("f32", vc), bt.bm.setDataClass("f32", vc)
            bt.fill_rhs(b, [seed_of[id(w)] for w in chunk], stream=stream.cuda_stream)
            x.fill(0.0, stream=stream.cuda_stream)
            bt.bm.imposeBoundaryCondition(x, stream=stream.cuda_stream)
            hbm = sum(brick_bytes(w) for w in chunk) > L2_BYTES
            runs.append((bt, op, x, b, stream, f"n={n} {'HBM' if hbm else 'L2'}"))
    torch.cuda.synchronize()
    # the fused-Jacobi kernel of each set tuned on it (set-up, outside the
    # timed region; x is left as it was): per block edge, the tiling
    tuned = {}
    for bt, op, x, b, _, label in runs:
        best, us = bt.bm.autotune_jacobi(op, x, b, 1.0, iters=10)
        tuned[label] = {"choice": {0: "separate launches", 1: "push form",
                                   2: "pull form, one CTA per block",
                                   3: "pull form, pipelined"}.get(best, str(best)),
                        "us_per_sweep": round(us, 1)}
    torch.cuda.synchronize()
    # sets spread over the streams largest first, each to the stream with the
    # fewest cells so far: the sets on different streams overlap on the device
    nstreams = max(1, args.batch_streams)
    streams = [stream] + [torch.cuda.Stream(device=0) for _ in range(nstreams - 1)]
    load = [0] * nstreams
    order = sorted(range(len(runs)), key=lambda i: -runs[i][0].cells)
    on = {}
    for i in order:
        k = load.index(min(load))
        on[i] = streams[k]
        load[k] += runs[i][0].cells

    def batched_step():
        for i, (bt, op, x, b, _, _) in enumerate(runs):
            bt.bm.jacobi_run(op, x, b, 1.0, iters, use_graph=True, stream=on[i].cuda_stream)

    for _ in range(args.warmup):
        batched_step()
    torch.cuda.synchronize()
    l0 = sum(r[0].bm.launch_count() for r in runs)
    clocks = ClockSampler(0)
    clocks.start()
    start = torch.cuda.Event(enable_timing=True)
    start.record()
    ends = []
    for st in streams:
        st.wait_event(start)
    for _ in range(args.steps):
        batched_step()
    for st in streams:
        e = torch.cuda.Event(enable_timing=True)
        e.record(st)
        ends.append(e)
    torch.cuda.synchronize()
    ms_batched = max(start.elapsed_time(e) for e in ends)
    clk = clocks.stop()
    launches = sum(r[0].bm.launch_count() for r in runs) - l0
    # ---- sequential: each instance alone in its own context ------------------
    alone = []
    stream = torch.cuda.Stream(device=0)
    sh = stream.cuda_stream
    for w in ws:
        bm = bg.BlockManager(0)
        bm.register_octree(w.tree, w.n)
        t, v = w.dirichlet(0.0)
        bm.set_boundary(t, v, bg.DIRICHLET_SOR)
        op = bm.op_const(bg.laplace_coef(w.tree.cell_sizes(w.n)))
        x, b = bm.setDataClass("f32", w.vc), bm.setDataClass("f32", w.vc)
        b.fill(0.0, stream=sh)
        b.fill_random(seed_of[id(w)], stream=sh)
        x.fill(0.0, stream=sh)
        bm.imposeBoundaryCondition(x, stream=sh)
        alone.append((bm, op, x, b))
    for _ in range(args.warmup):  # warm-up (and graph capture): as many runs as the batch had
        for bm, op, x, b in alone:
            bm.jacobi_run(op, x, b, 1.0, iters, use_graph=True, stream=sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        for bm, op, x, b in alone:
            bm.jacobi_run(op, x, b, 1.0, iters, use_graph=True, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_seq = e0.elapsed_time(e1)
    # ---- where the time goes: a short pass with events around each set and
    # each instance (not the timed figures) ------------------------------------
    bi = max(1, iters // 10)
    split = {}

    def timed_pass(items):
        evs = []
        for bm_, op_, x_, b_, st_, label in items:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st_)
            bm_.jacobi_run(op_, x_, b_, 1.0, bi, use_graph=False, stream=st_.cuda_stream)
            e1.record(st_)
            evs.append((label, e0, e1))
        torch.cuda.synchronize()
        out = {}
        for k, e0, e1 in evs:
            out[k] = out.get(k, 0.0) + e0.elapsed_time(e1) * iters / bi
        return out
    bst = runs[0][4]
    split["batched_ms_by_set"] = timed_pass(
        [(r[0].bm, r[1], r[2], r[3], bst, r[5]) for r in runs])
    split["sequential_ms_by_edge"] = timed_pass(
        [(bm, op, x, b, stream, f"n={w.n}") for (bm, op, x, b), w in zip(alone, ws)])
    # ---- the same values alone and in the batch (a sample of instances) -----
    check = [k for k, w in enumerate(ws) if w.cells <= 2_000_000][:24]
    worst = 0.0
    for k in check:
        w = ws[k]
        grp = next(r for r in runs if id(w) in map(id, r[0].workloads))
        idx = [id(u) for u in grp[0].workloads].index(id(w))
        xb = grp[0].instance(grp[2].download(), idx)
        xa = alone[k][2].download()
        worst = max(worst, float(np.abs(xb.astype(np.float64) - xa).max()))
    value = cells * iters * args.steps / (ms_batched / 1e3) / 1e9
    seq = cells * iters * args.steps / (ms_seq / 1e3) / 1e9
    line = {"metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_batched / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded instances and uniform RHS)",
            "config": {"workload": f"batched: {len(ws)} instances (seeds 1000..1255), blocks "
                                   "log-uniform [64, 4096], n in {8,16,32}, vc=1, "
                                   f"{iters} Jacobi sweeps + ghost update per step",
                       "cells": cells,
                       "groups": {f"n={n}": {"instances": sum(len(r[0].workloads) for r in runs
                                                              if r[0].n == n),
                                               "block_sets": sum(1 for r in runs if r[0].n == n),
                                               "blocks": sum(r[0].nb for r in runs if r[0].n == n)}
                                  for n in sorted({r[0].n for r in runs})},
                       "streams": nstreams, "tuned": tuned,
                       "block_sets": ("L2-sized (x, work copy and b <= "
                                      f"{L2_BYTES / 1e6:.0f} MB) where one holds >= 2048 "
                                      "blocks, the rest one set per block edge"
                                      if args.l2_sets else "one set per block edge")},
            "gpu_launches": launches, "clocks": clk,
            "sequential": {"value": seq, "unit": "Gcell/s", "ms_per_step": ms_seq / args.steps,
                           "what": "the same instances one after another, one context each, "
                                   "same API call"},
            "batched_over_sequential": value / seq,
            "breakdown": {"what": f"one pass of {bi} sweeps, events around each set / "
                                  f"instance, scaled to {iters}; launches not graph-replayed",
                          **{k: {kk: round(vv, 1) for kk, vv in v.items()}
                             for k, v in split.items()}},
            "alone_vs_batched_max_abs_diff": worst, "checked_instances": len(check)}
    print(json.dumps(line))
    return 0


def run_served(args):
    """Served stream: `--requests` requests with Poisson arrivals at 200/s
    (seed 5), cells log-uniform in [1e4, 1e8], block edge 16 or 32, maximum
    level 2..6, seeded uniform RHS, Dirichlet 0, each solved by the
    mixed-precision BiCGSTAB to a 1e-8 relative residual.  Served: continuous
    batching (serve.BatchServer: requests admitted as a worker and memory free
    up, packed with waiting requests of the same block edge and similar size
    into one block set, each a segment advanced by every launch; 4 workers,
    150 GB budget).  Against the one-at-a-time loop over the same list.
    Latency includes queueing and the mesh set-up, which runs on the device
    (octree, 2:1 balance, neighbour and face tables from each request's
    divider); the stream generator's choice of each request's divider (a
    radius bisected on host trees to hit its cell count) is made before the
    timed runs, as a request arriving with its mesh description."""
    import dataclasses

    import torch

    from bcmtools_gb300 import serve
    torch.cuda.set_device(0)
    reqs = serve.poisson_stream(args.requests, 200.0, seed=5)
    warm = serve.poisson_stream(4, 200.0, seed=99, cells=(3e5, 6e5))
    for r in reqs + warm:
        r.mesh_spec()
    serve.BatchServer(workers=2).run(warm)  # module load, first-use costs
    clocks = ClockSampler(0)
    clocks.start()
    srv = serve.BatchServer(budget_bytes=150e9, workers=4)
    served = srv.run(reqs)
    clk = clocks.stop()
    plain = serve.one_at_a_time(reqs)
    s, p = serve.summary(served), serve.summary(plain)
    cells = np.array([r.cells for r in plain], dtype=np.float64)
    busy = np.array([r.finish - r.start for r in plain])
    order = np.argsort(cells)
    dec = np.array_split(order, 10)
    # The plain path: the FP64 BiCGSTAB, one request at a time, run on every
    # k-th request by size (a systematic sample over the size range; all of
    # them at k = 1).  Its total solve time over the stream is estimated by
    # the ratio of FP64 to mixed solve time on the sample.
    k = max(1, args.plain_sample)
    by_rid = {r.rid: r for r in reqs}
    sample = [dataclasses.replace(by_rid[plain[i].rid], arrival=0.0)
              for i in order[k // 2::k]]
    fp64 = serve.one_at_a_time(sample, solver=serve.solve_plain)
    f64_busy = sum(r.finish - r.start for r in fp64)
    mix_busy = sum(plain[i].finish - plain[i].start for i in order[k // 2::k])
    est_busy = f64_busy * busy.sum() / mix_busy
    plain64 = {"what": "FP64 BiCGSTAB (the reference's precision), one request at a time, "
                       "same systems, preconditioner and 1e-8 target",
               "sample_every": k, "sampled_requests": len(fp64),
               "sample_busy_s": f64_busy, "sample_mixed_busy_s": mix_busy,
               "estimated_busy_s_all": est_busy,
               "solves_per_s": len(reqs) / est_busy,
               "max_residual": float(max(r.residual for r in fp64)),
               "failed": int(sum(1 for r in fp64 if r.status != 0)),
               "iterations_mean": float(np.mean([r.iterations for r in fp64]))}
    line = {"metric": "solves/s", "value": s["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
            "steps": 1, "warmup": 1, "ms_per_step": s["makespan_s"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded Poisson arrivals, meshes and RHS)",
            "config": {"workload": f"served: {len(reqs)} requests, Poisson 200/s, cells "
                                   "log-uniform [1e4, 1e8], n in {16, 32}, levels 2..6, "
                                   "mixed-precision BiCGSTAB to 1e-8, budget 150 GB, continuous "
                                   "batching on 4 workers",
                       "cells": s["cells"]},
            "clocks": clk, "served": s, "one_at_a_time": p, "batches": srv.batches,
            "served_over_one_at_a_time": s["solves_per_s"] / p["solves_per_s"],
            "plain_fp64_one_at_a_time": plain64,
            "served_over_plain_fp64": s["solves_per_s"] / plain64["solves_per_s"],
            "plain_time_share_by_size_decile": [float(busy[d].sum() / busy.sum()) for d in dec],
            "plain_cells_by_size_decile": [float(cells[d].mean()) for d in dec],
            "errors": getattr(srv, "errors", [])}
    print(json.dumps(line))
    return 0


def run_mixed(args):
    """Mixed-precision BiCGSTAB on the level-5 octree around 16 seeded points
    (32^3 cells per block, vc=1, ~96 M cells), seeded uniform RHS, Dirichlet 0:
    FP32 vectors and stencil in the correction solves, FP64 residual, inner
    products and refinement, to a 1e-10 relative residual.  Reference: the
    FP64 BiCGSTAB on the same system to 1e-12; the error is reported against
    it (the FP64 CPU oracle pins both at small sizes in the tests)."""
    import torch

    import bcmtools_gb300 as bg
    from bcmtools_gb300 import workloads as W
    torch.cuda.set_device(0)
    if args.profile:
        # short case for ncu: 4 FP32 BiCGSTAB iterations on the same kind of
        # mesh with smaller balls (about 1 GB of vectors)
        w = W.points_level5(radius=0.02)
        bm = bg.BlockManager(0)
        bm.register_octree(w.tree, w.n)
        t, v = w.dirichlet(0.0)
        bm.set_boundary(t, v, bg.DIRICHLET_SOR)
        op = bm.op_const(bg.laplace_coef(w.tree.cell_sizes(w.n)))
        x32, b32 = bm.setDataClass("f32", 1), bm.setDataClass("f32", 1)
        b32.fill(0.0)
        b32.fill_random(3)
        x32.fill(0.0)
        bm.imposeBoundaryCondition(x32)
        bm.bicgstab(op, x32, b32, omega=0.8, n_pre=2, max_iter=4, eps=1e-30)
        torch.cuda.synchronize()
        print(f"profile case done: 4 FP32 BiCGSTAB iterations, {w.nb} blocks of 32^3")
        return 0
    w = W.points_level5()
    bm = bg.BlockManager(0)
    bm.register_octree(w.tree, w.n)
    t, v = w.dirichlet(0.0)
    bm.set_boundary(t, v, bg.DIRICHLET_SOR)
    op = bm.op_const(bg.laplace_coef(w.tree.cell_sizes(w.n)))
    x, b = bm.setDataClass("f64", 1), bm.setDataClass("f64", 1)
    b.fill(0.0)
    b.fill_random(3)
    omega, n_pre = 0.8, 2

    def solve_mixed():
        x.fill(0.0)
        bm.imposeBoundaryCondition(x)
        return bm.bicgstab_mixed(op, x, b, omega=omega, n_pre=n_pre, max_inner=args.max_inner,
                                 eps_inner=args.eps_inner, max_outer=60, eps=1e-10)

    solve_mixed()  # warm-up (work fields, first launches)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    info = solve_mixed()
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    clk = clocks.stop()
    xm = x.download()
    x.fill(0.0)
    bm.imposeBoundaryCondition(x)
    t1 = time.perf_counter()
    ref = bm.bicgstab(op, x, b, omega=omega, n_pre=n_pre, max_iter=4000, eps=1e-12)
    torch.cuda.synchronize()
    secs64 = time.perf_counter() - t1
    xr = x.download()
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    err = float(np.abs(xm[inner] - xr[inner]).max() / np.abs(xr[inner]).max())
    per_iter = (26 + 6 * n_pre) * 4 * w.cells  # algorithmic bytes of one FP32 iteration
    # the error against the FP64 CPU oracle's solution of the same system
    # (tests/golden/make_c3_fixture.py): every block's interior norm and
    # eight whole blocks
    cpu = None
    fx = ROOT / "tests" / "golden" / "c3_points_level5_fp64.npz"
    if fx.exists():
        g = np.load(fx)
        if int(g["nb"]) == w.nb and np.array_equal(g["pedigrees"], w.tree.pedigrees):
            xi = xm[inner]
            ids = g["sample_ids"]
            ref_blocks = g["sample_blocks"]
            blk_err = float(np.abs(xi[ids] - ref_blocks).max() / float(g["xmax"]))
            norms = np.sqrt((xi.astype(np.float64) ** 2).sum(axis=(1, 2, 3)))
            ref_norms = np.sqrt(g["block_sumsq"])
            norm_err = float(np.abs(norms - ref_norms).max() / ref_norms.max())
            cpu = {"max_rel_error_sampled_blocks": blk_err,
                   "max_rel_error_block_norms": norm_err,
                   "cpu_iterations": int(g["iterations"]), "cpu_residual": float(g["residual"]),
                   "cpu_seconds": float(g["cpu_seconds"]), "cpu_threads": int(g["cpu_threads"])}
    # one FP32 BiCGSTAB of 30 iterations under per-launch events: where the
    # time of an iteration goes, by kernel kind
    x32, b32 = bm.setDataClass("f32", 1), bm.setDataClass("f32", 1)
    b32.fill(0.0)
    b32.fill_random(3)
    x32.fill(0.0)
    bm.imposeBoundaryCondition(x32)
    bm.bicgstab(op, x32, b32, omega=omega, n_pre=n_pre, max_iter=3, eps=1e-30)
    torch.cuda.synchronize()
    x32.fill(0.0)
    bm.imposeBoundaryCondition(x32)
    t2 = time.perf_counter()
    it32 = bm.bicgstab(op, x32, b32, omega=omega, n_pre=n_pre, max_iter=30, eps=1e-30)
    torch.cuda.synchronize()
    it_ms = (time.perf_counter() - t2) * 1e3 / max(1, it32.iterations)
    x32.fill(0.0)
    bm.imposeBoundaryCondition(x32)
    bm.profile_begin()
    bm.bicgstab(op, x32, b32, omega=omega, n_pre=n_pre, max_iter=30, eps=1e-30)
    prof = bm.profile_end()
    kern = {k: {"ms_per_iter": v[0] / 30, "launches_per_iter": v[1] / 30}
            for k, v in prof.items() if v[1]}
    line = {"metric": "solve_seconds", "value": secs, "unit": "s", "n_gpus": 1, "steps": 1,
            "warmup": 1, "ms_per_step": secs * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 vectors, f64 residual",
            "data": "synthetic (seeded uniform RHS)",
            "config": {"workload": f"mixed-precision BiCGSTAB: points_level5, {w.nb} blocks of "
                                   f"32^3, vc=1, Jacobi preconditioner {n_pre} passes at "
                                   f"omega {omega}, FP32 correction solves to "
                                   f"{args.eps_inner:g} or {args.max_inner} iterations, "
                                   "target 1e-10", "cells": w.cells},
            "clocks": clk,
            "mixed": {"iterations": info.iterations, "refinements": info.refinements,
                      "true_residual": info.true_residual, "status": info.status,
                      "effective_GBps": per_iter * info.iterations / secs / 1e9},
            "fp64": {"seconds": secs64, "iterations": ref.iterations,
                     "residual": ref.true_residual, "status": ref.status},
            "max_rel_error_vs_fp64": err, "fp64_over_mixed_time": secs64 / secs,
            "vs_cpu_oracle": cpu,
            "fp32_iteration": {"ms": it_ms, "effective_GBps": per_iter / it_ms / 1e6,
                               "kernels": kern}}
    print(json.dumps(line))
    return 0


def run_vc_only(args):
    """The ghost update alone on the two-level sphere mesh (16^3 cells, vc=2):
    `--vc-updates` updates of each face kind (same level, F2C, C2F) timed with
    CUDA events, FP32 and FP64; ghosts/s and algorithmic GB/s per kind.  Bytes
    per ghost: one write plus its unique sources -- 1 (same level), 8 (F2C),
    and for C2F the coarse cells of each fine face's source region,
    (vc/2 + 2) (n/2 + 2)^2 per face, counted from the mesh."""
    import torch

    import bcmtools_gb300 as bg
    from bcmtools_gb300 import workloads as W
    torch.cuda.set_device(0)
    w = W.two_level_sphere()
    n, vc = w.n, w.vc
    ld, nid, _, _ = w.neighbors()
    has = nid >= 0
    n_same = int(((ld == 0) & has[:, :, 0]).sum())
    n_c2f = int(((ld == -1) & has[:, :, 0]).sum())
    n_f2c = int(((ld == 1)[:, :, None] & has).sum())
    kinds = {"same_level": (2, n_same * vc * n * n, 1.0),
             "f2c": (4, n_f2c * vc * (n // 2) ** 2, 8.0),
             "c2f": (1, n_c2f * vc * n * n, None)}
    c2f_src = n_c2f * (vc // 2 + 2) * (n // 2 + 2) ** 2
    bm = bg.BlockManager(0)
    bm.register_octree(w.tree, n)
    stream = torch.cuda.Stream(device=0)
    sh = stream.cuda_stream
    out = {}
    for dt, es in (("f32", 4), ("f64", 8)):
        f = bm.setDataClass(dt, vc)
        bm.prepareForVCUpdate(f)
        f.fill_random(9, stream=sh)
        res = {}
        for name, (ldbit, ghosts, srcs) in kinds.items():
            for _ in range(5):
                bm.beginUpdateVC(f, 7, ldbit, stream=sh)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.vc_updates):
                bm.beginUpdateVC(f, 7, ldbit, stream=sh)
            e1.record(stream)
            torch.cuda.synchronize()
            us = e0.elapsed_time(e1) * 1e3 / args.vc_updates
            nbytes = ghosts * es + (ghosts * srcs * es if srcs else c2f_src * es)
            res[name] = {"ghosts": ghosts, "us_per_update": us, "Gghosts_per_s": ghosts / us / 1e3,
                         "algorithmic_GBps": nbytes / us / 1e3}
        bm.destroy(f)
        out[dt] = res
    peak, peak_kind = load_peaks()
    line = {"metric": "Gghosts/s", "value": out["f32"]["same_level"]["Gghosts_per_s"],
            "unit": "Gghosts/s", "n_gpus": 1, "steps": args.vc_updates, "warmup": 5,
            "ms_per_step": out["f32"]["same_level"]["us_per_update"] / 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64",
            "data": "synthetic (seeded uniform field)",
            "config": {"workload": f"vc_only: two_level_sphere, {w.nb} blocks of 16^3, vc=2, "
                                   "each face kind updated alone"},
            "by_kind": out, "peak_GBps": peak, "peak_source": peak_kind}
    print(json.dumps(line))
    return 0


def run_mesh_setup(args):
    """Mesh set-up, host against device: building the octree of a divider,
    its 2:1 balance, the neighbour table and the registration with its face
    tables -- on the host (Octree.build + neighbors + register_blocks, whose
    face tables are built on the device) and on the device
    (BlockManager.build_mesh: everything on the GPU).  Meshes: the two-level
    sphere (C2, 4432 blocks), the level-5 points mesh (C3, 2920 blocks), a
    flat level-6 mesh (262,144 blocks), and the 100 meshes of the served
    stream as one batch (BlockManager.build_mesh_batch against host trees
    concatenated).  Best of 3 wall-clock times each, after one untimed run."""
    import torch

    import bcmtools_gb300 as bg
    from bcmtools_gb300 import serve
    from bcmtools_gb300.batch import Batch
    from bcmtools_gb300.serve import _Mesh
    torch.cuda.set_device(0)
    pts = np.random.default_rng(3).uniform(0.0, 1.0, size=(16, 3))
    cases = [("two_level_sphere", bg.RootGrid(4, 4, 4, root_length=0.25),
              bg.Divider.sphere_surface((0.5, 0.5, 0.5), 0.3, 3), 16),
             ("points_level5", bg.RootGrid(1, 1, 1), bg.Divider.balls(pts, 0.05, 5), 32),
             ("flat_level6", bg.RootGrid(1, 1, 1), bg.Divider.flat(6), 16)]

    def best(fn, reps=3):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    out = {}
    for name, rg, div, n in cases:
        def host():
            tree = bg.Octree.build(rg, div, "Z")
            ld, nid, sf, _ = tree.neighbors()
            bm = bg.BlockManager(0)
            bm.register_blocks(ld, nid, sf, n)
            bm.close()
            return tree.num_leaves

        def dev():
            bm = bg.BlockManager(0)
            bm.build_mesh(rg, div, n)
            bm.close()
        nb = host()
        out[name] = {"blocks": nb, "host_s": best(host), "device_s": best(dev)}
        out[name]["host_over_device"] = out[name]["host_s"] / out[name]["device_s"]
    reqs = serve.poisson_stream(100, 200.0, seed=5)
    by_n = {}
    for r in reqs:
        by_n.setdefault(r.n, []).append(r)
    specs = {k: [r.mesh_spec() for r in v] for k, v in by_n.items()}

    def host_batch():
        for k, sp in specs.items():
            b = Batch([_Mesh(bg.Octree.build(rg, d, "Z"), k) for rg, d in sp])
            b.bm.close()

    def dev_batch():
        for k, sp in specs.items():
            b = Batch.from_dividers(sp, k)
            b.bm.close()
    nblocks = sum(Batch.from_dividers(sp, k).nb for k, sp in specs.items())
    out["served_stream_meshes"] = {"meshes": len(reqs), "blocks": nblocks,
                                   "host_s": best(host_batch, 2), "device_s": best(dev_batch, 2)}
    out["served_stream_meshes"]["host_over_device"] = (out["served_stream_meshes"]["host_s"] /
                                                       out["served_stream_meshes"]["device_s"])
    line = {"metric": "mesh set-up seconds", "value": out["served_stream_meshes"]["device_s"],
            "unit": "s", "n_gpus": 1, "steps": 3, "warmup": 1,
            "ms_per_step": out["served_stream_meshes"]["device_s"] * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "int",
            "data": "synthetic (dividers of the bench meshes and the served stream)",
            "config": {"workload": "mesh_setup: octree, 2:1 balance, neighbour and face tables, "
                                   "host against device"},
            "by_mesh": out}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--profile", action="store_true",
                    help="short run for an ncu capture (two_level_sphere: 10 SOR iterations "
                         "of --variant in --dtype; mixed_bicgstab: 4 FP32 BiCGSTAB iterations "
                         "on a smaller points mesh), no timing")
    ap.add_argument("--workload", default="two_level_sphere",
                    choices=["two_level_sphere", "plain_poisson", "plain_poisson_l5",
                             "batched", "served", "mixed_bicgstab", "vc_only", "mesh_setup"])
    ap.add_argument("--vc-updates", type=int, default=1000,
                    help="ghost updates per face kind of the vc_only workload")
    ap.add_argument("--max-inner", type=int, default=200,
                    help="iteration cap of each FP32 correction solve (mixed_bicgstab)")
    ap.add_argument("--eps-inner", type=float, default=1e-2,
                    help="relative target of each FP32 correction solve (mixed_bicgstab)")
    ap.add_argument("--requests", type=int, default=200,
                    help="requests of the served workload")
    ap.add_argument("--l2-sets", action="store_true",
                    help="batched: L2-sized block sets where one holds >= 2048 blocks")
    ap.add_argument("--batch-streams", type=int, default=1,
                    help="batched: streams the block sets are spread over")
    ap.add_argument("--plain-sample", type=int, default=1,
                    help="served: the FP64 plain path runs every k-th request by size "
                         "(1, the default: all of them)")
    ap.add_argument("--batch-iters", type=int, default=20,
                    help="Jacobi sweeps per step of the batched workload")
    ap.add_argument("--jacobi-shape", type=int, default=0,
                    help="pull-form Jacobi kernel (0 auto, 1 one CTA per block, 2 pipelined)")
    ap.add_argument("--autotune", action="store_true",
                    help="time every kernel shape on a copy of the field first and keep the fastest")
    ap.add_argument("--sor-shape", type=int, default=0,
                    help="fused-SOR kernel shape for the timed run (0: autotuned)")
    ap.add_argument("--variant", type=int, default=7,
                    help="kernel shape for --profile (bcmg_set_sor_variant)")
    ap.add_argument("--no-side", action="store_true",
                    help="two_level_sphere: skip the short C1-level-5 and C3 samples the "
                         "default line carries")
    ap.add_argument("--dtype", default="both", choices=["f32", "f64", "both"],
                    help="two_level_sphere: FP32 headline alone, or with the FP64 run beside "
                         "it (both); --profile: the precision of the short case")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload.startswith("plain_poisson"):
        return run_jacobi(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "served":
        return run_served(args)
    if args.workload == "mixed_bicgstab":
        return run_mixed(args)
    if args.workload == "vc_only":
        return run_vc_only(args)
    if args.workload == "mesh_setup":
        return run_mesh_setup(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
