#!/usr/bin/env python3
"""Benchmark: TGV leaf-iterations per second of the sm_103a Stage-6 solver.

One step = one full coarse-to-fine solve (setup + every level, fixed iteration
count per level) over one synthetic workload with inputs resident in HBM.  The
default workload, three64, has the shape of the "plain method at scale"
configuration: a sphere, a box and a torus seen by 64 cameras at 1920x1080,
cubes to depth 11 (6.2M with seed 0), 10-bin histograms from this package's
own kernels, alpha1 = 1, alpha0 = 2, 1000 iterations per level.  The first
warm-up step lets the online autotuner pick each level's schedule; later steps
capture the level loop into a CUDA graph and relaunch it.

Also reported in the same JSON line:
  e2e           the same metric through the public host-buffer C ABI call
                (tgvg_tgv_minimize) from pinned host memory, copies included
  roofline      the dominant iteration kernel timed per launch with CUDA events
                on the library's stream, against MEASURED_PEAKS.json
  cpu_baseline  the CPU oracle port on a bounded sample of the same workload
  histograms    the Stage-5 pass (pyramids + binning) on the same workload
  surface       extract_surface + compute_normals of the solved state through
                the host-buffer C ABI call, beside the CPU oracle on a slice
  warm_start    time to relative residual 1e-4 on held-out small scenes from
                the zero start, from the trained warm-start network
                (tgvreconclaude_gb300/data/warmstart_nb10.npz) and from the
                reference's initialisation

`--impl reference` times the CPU implementation of the path (the oracle port of
the reference's tgv.cpp, all host threads) on a bounded sample of the same
workload and prints the same metric.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import glob
import json
import math
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "TGV leaf-iter/s"
UNIT = "leaf-iter/s"
BYTES_DUAL = 100     # per cube: bars 16 + neighbour ids 12 + p/q 36 read, p/q 36 written
BYTES_PRIMAL = 104   # per cube: u/v 16 + p/q 36 + data 8 + neighbour ids 12 read, u/v 16 + bars 16 written
BYTES_ITER = 168     # algorithmic bytes per leaf-iteration (one fused pass)


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_cube():
    """dram bytes per cube per launch from the committed ncu summaries
    (lines 'traffic_per_cube <kernel> <bytes>')."""
    out = {}
    for p in glob.glob(os.path.join(HERE, "profiles", "*.md")) + glob.glob(os.path.join(HERE, "profiles", "*.txt")):
        with open(p) as f:
            for line in f:
                m = re.match(r"\s*traffic_per_cube\s+(\w+)\s+([0-9.eE+]+)", line)
                if m:
                    out[m.group(1)] = float(m.group(2))
    return out


class Clocks:
    """nvidia-smi sampling (200 ms) during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        for r in rows:
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("TGV_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
        pg = dist
    return ws, rank, local, pg


def allreduce_max(x, pg, torch):
    if pg is None:
        return x
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x, pg, torch):
    if pg is None:
        return x
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    pg.all_reduce(t)
    return float(t.item())


def cpu_sample(w, n_sample: int, iters: int):
    """A contiguous Morton-ordered slice of the workload (a spatially compact
    region, like one treetop chunk)."""
    n = min(n_sample, len(w.cubes))
    start = max(0, (len(w.cubes) - n) // 2)
    return w.cubes[start:start + n].copy(), w.hists[start:start + n].copy()


def time_cpu_oracle(cubes, hists, iters, nthreads, repeats=1):
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle
    oracle.build()
    best = None
    li = 0
    out = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        out, st = oracle.tgv_solve(cubes, hists, None, "inmem", 2.0, 1.0, iters, nthreads=nthreads)
        dt = time.perf_counter() - t0
        li = sum(s["active"] * s["iters_run"] for s in st)
        best = dt if best is None else min(best, dt)
    return li / best, best, li, out


def run_reference(args):
    """CPU implementation of the path on the host cores: the oracle port of the
    reference's tgv_minimize (bit-identical to the reference compiled from its
    own sources, which exist only where the reference is checked out, not on
    the GPU host), on the same cube slice and iteration count as the FP64
    check of this package's arm.  All host threads; a single-thread step (the
    reference's own threading) is reported beside it."""
    import torch
    ws, rank, local, pg = dist_setup()
    if rank != 0:
        return 0
    from tgvreconclaude_gb300 import workloads
    torch.cuda.set_device(local)
    # Scene and cubes come from torch on the GPU (input preparation only); the
    # sample's histograms come from the CPU oracle, so no kernel of this
    # package runs on this arm.
    w = workloads.build(args.workload, seed=args.seed, device="cuda", histograms=False)
    threads = os.cpu_count() or 1
    cubes, _ = cpu_sample(w, args.ref_sample or args.cpu_sample, args.cpu_iters)
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle
    oracle.build()
    maps = []
    for c, d in zip(w.cams, w.depths):
        maps.append(dict(depth=d, rt_inv=np.array(c.rt_inv[:], np.float32).reshape(4, 4), fx=c.fx, fy=c.fy, cx=c.cx,
                         cy=c.cy, lidar=bool(c.lidar)))
    hists = oracle.compute_histograms(cubes, maps, w.cfg["origin"], w.cfg["r_root"], nbins=w.cfg["nbins"],
                                      nthreads=threads)
    for _ in range(max(0, args.warmup)):
        time_cpu_oracle(cubes, hists, args.cpu_iters, threads)
    vals, tot_li, tot_t = [], 0, 0.0
    for _ in range(args.steps):
        v, dt, li, _ = time_cpu_oracle(cubes, hists, args.cpu_iters, threads)
        vals.append(v)
        tot_li += li
        tot_t += dt
    value = tot_li / tot_t
    v1, dt1, _, _ = time_cpu_oracle(cubes, hists, args.cpu_iters, 1)
    sample = f"{len(cubes)} contiguous Morton-ordered cubes of {args.workload}, {args.cpu_iters} iterations per level, in-memory semantics, {threads} threads"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "cubes_sample": len(cubes), "iters_per_level": args.cpu_iters,
                       "semantics": "tgv_minimize"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "single_thread": {"value": v1, "unit": UNIT, "cores": 1, "seconds": dt1,
                              "what": "the same step on one thread (the reference is single-threaded)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def measure_e2e(args, w, ctx, prm, mode, leaves, out_t, stream):
    """The same solve through the public host-buffer call (tgvg_tgv_minimize):
    cubes and histograms copied from pinned host memory, state copied back,
    every step."""
    import ctypes as C
    import torch
    from tgvreconclaude_gb300 import _native as N, api, formats as F
    n, nbins = len(w.cubes), w.hists.shape[1]
    pin_c = torch.from_numpy(w.cubes.view(np.int32).reshape(n, 4).copy()).pin_memory()
    pin_h = torch.from_numpy(w.hists.view(np.int32).copy()).pin_memory()
    pin_o = torch.empty((n, 13), dtype=torch.float32).pin_memory()
    c_np = pin_c.numpy().view(F.CUBE_DTYPE).reshape(n)
    h_np = pin_h.numpy().view(np.uint32)
    o_np = pin_o.numpy().view(F.STATE_DTYPE).reshape(n)
    lv = None if leaves is None else np.ascontiguousarray(leaves, F.LEAF_DTYPE)
    p = prm.struct()
    stt = N.Stats()
    steps = max(1, min(args.steps, args.e2e_steps))

    def call():
        rc = ctx.lib.tgvg_tgv_minimize(ctx.h, c_np.ctypes.data, h_np.ctypes.data, n, nbins, api._p(lv),
                                       0 if lv is None else len(lv), api.MODES[mode], C.byref(p), None,
                                       o_np.ctypes.data, C.byref(stt))
        ctx.check(rc, "tgvg_tgv_minimize")
        return stt.leaf_iters

    # warm-up: the first call is the problem's first sighting without per-launch
    # timing, the second captures its level-loop graph; the timed calls replay it
    for _ in range(2):
        call()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    t_w = time.perf_counter()
    li = sum(call() for _ in range(steps))
    f1.record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_w
    t = max(f0.elapsed_time(f1) / 1e3, 1e-9)
    same = bool(np.array_equal(o_np.view(np.float32).reshape(n, 13), out_t.cpu().numpy()))
    return {"value": li / t, "unit": UNIT, "h2d_bytes_per_step": int(16 * n + 4 * nbins * n),
            "d2h_bytes_per_step": int(52 * n), "steps": steps, "wall_s": t_wall, "matches_device_run": same}


def histogram_kernel_eval(ctx, w, cubes_t, nbins, expect, stream, reps=5):
    """The binning kernel alone (tgvg_compute_histograms_dev) on device-resident
    pyramids and cubes, timed with CUDA events on the library's stream, with its
    algorithmic bytes: per pair one texel (4 B), per cube its record (16 B) and
    histogram row (4 B per bin) once."""
    import ctypes as C
    import torch
    from tgvreconclaude_gb300 import _native as N, api
    lib, cams = ctx.lib, w.cams
    ncam, n = len(cams), len(w.cubes)
    sizes = []
    for c in cams:
        dims = (C.c_int32 * 26)()
        nl = lib.tgvg_pyramid_dims(c.width, c.height, dims)
        sizes.append(sum(dims[2 * k] * dims[2 * k + 1] for k in range(nl)))
    levels = [np.empty(sz, np.float32) for sz in sizes]
    arr = (N.Camera * ncam)(*cams)
    basep = (C.c_void_p * ncam)(*[np.ascontiguousarray(d, np.float32).ctypes.data for d in w.depths])
    outp = (C.c_void_p * ncam)(*[lv.ctypes.data for lv in levels])
    ctx.check(lib.tgvg_build_pyramids(ctx.h, arr, ncam, basep, outp), "tgvg_build_pyramids")
    tex = torch.from_numpy(np.concatenate(levels)).cuda()
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    d_out = torch.empty((n, nbins), dtype=torch.int32, device="cuda")
    o = np.asarray(w.cfg["origin"], np.float32)

    def call():
        ctx.check(lib.tgvg_compute_histograms_dev(ctx.h, cubes_t.data_ptr(), n, arr, ncam, tex.data_ptr(), api._p(off),
                                                  api._p(o), float(w.cfg["r_root"]), nbins, d_out.data_ptr()),
                  "tgvg_compute_histograms_dev")

    call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    pairs = n * ncam
    nbytes = 4 * pairs + n * (16 + 4 * nbins)
    hbm, peak_kind = peaks()
    return {"kernel": "k_histograms", "ms": ms, "pairs_per_s": pairs / (ms * 1e-3),
            "algorithmic_bytes": nbytes, "achieved_gbs": nbytes / (ms * 1e-3) / 1e9,
            "frac": nbytes / (ms * 1e-3) / 1e9 / hbm, "peak_kind": peak_kind,
            "texels_on_device_mb": 4 * int(off[-1]) / 1e6,
            "matches_host_call": bool(np.array_equal(d_out.cpu().numpy().view(np.uint32), expect))}


def histogram_oracle_check(w, hh, n_sample: int):
    """Bit-exact check of the GPU histograms against the CPU oracle on a seeded
    random subset of the workload's cubes, against every depth map."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as O
    n = len(w.cubes)
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(n, min(n, n_sample), replace=False))
    maps = [dict(depth=np.ascontiguousarray(d, np.float32), rt_inv=np.array(list(c.rt_inv), np.float32).reshape(4, 4),
                 fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy, lidar=bool(c.lidar)) for c, d in zip(w.cams, w.depths)]
    t0 = time.perf_counter()
    ref = O.compute_histograms(w.cubes[idx], maps, w.cfg["origin"], w.cfg["r_root"], hh.shape[1],
                               nthreads=os.cpu_count() or 1)
    dt = time.perf_counter() - t0
    bad = int((ref != hh[idx]).any(1).sum())
    return {"cubes": int(len(idx)), "maps": len(maps), "rows_differing": bad, "bit_exact": bad == 0,
            "votes": int(ref.sum()), "oracle_s": round(dt, 2), "oracle_threads": os.cpu_count() or 1}


def surface_eval(args, w, out_t):
    """Surface extraction (extract_surface with has_data and normals) of the
    solved state through the host-buffer C ABI call, and the CPU oracle on a
    bounded contiguous Morton slice of the same input."""
    import torch
    from tgvreconclaude_gb300 import api, formats as F
    n = len(w.cubes)
    # inputs in pinned host memory, as for the solver's e2e
    state = torch.empty(out_t.shape, dtype=out_t.dtype, pin_memory=True)
    state.copy_(out_t)
    state = state.numpy().view(F.STATE_DTYPE).reshape(n)
    has = torch.from_numpy((w.hists.sum(1) > 0).astype(np.uint8)).pin_memory().numpy()
    cubes = torch.from_numpy(w.cubes.view(np.int32).reshape(n, 4).copy()).pin_memory().numpy()
    cubes = cubes.view(F.CUBE_DTYPE).reshape(n)
    o, r = np.float32(w.cfg["origin"]), float(w.cfg["r_root"])
    api.extract_surface(cubes[:1000], state[:1000], o, r, has_data=has[:1000], normals=True)  # warm-up
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        v, f, _ = api.extract_surface(cubes, state, o, r, has_data=has, normals=True)
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    res = {"cubes": n, "vertices": int(len(v)), "triangles": int(len(f)), "ms_e2e": 1e3 * t,
           "cubes_per_s_e2e": n / t, "what": "extract_surface + compute_normals, inputs in pinned host memory, mesh returned in host arrays"}
    if not args.skip_cpu:
        sys.path.insert(0, os.path.join(HERE, "oracle"))
        import oracle as O
        m = min(n, args.cpu_sample)
        t0 = time.perf_counter()
        O.extract_surface(w.cubes[:m], state[:m], o, r, has_data=has[:m], normals=True)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": m / dt, "unit": "cubes/s", "cores": 1, "kind": "port",
                               "sample": f"first {m} Morton-ordered cubes of the solved {args.workload} state"}
    return res


def stages13_eval(args, w):
    """Stages 1-3 on the workload's depth maps through the host-buffer C ABI
    calls: cubes from every map, their merge, and the 2:1 balance of the merged
    list; the CPU oracle, and a GPU/oracle equality check, on the first two maps."""
    from tgvreconclaude_gb300 import api
    if not w.depths:
        return {"unavailable": "workload loaded from a cache without depth maps"}
    o, r = np.float32(w.cfg["origin"]), float(w.cfg["r_root"])

    def as_map(cam, d):
        rt = np.linalg.inv(np.asarray(cam.rt_inv[:], np.float64).reshape(4, 4)).astype(np.float32)
        return dict(depth=d, rt=rt, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy)

    import torch
    pinned = [torch.from_numpy(np.ascontiguousarray(d, np.float32)).pin_memory().numpy() for d in w.depths]
    maps = [as_map(c, d) for c, d in zip(w.cams, pinned)]  # depth maps in pinned host memory
    api.build_cubes(maps[0], o, r)  # warm-up
    t0 = time.perf_counter()
    arrs = [api.build_cubes(m, o, r) for m in maps]
    t1 = time.perf_counter()
    merged = api.merge_cubes(arrs)
    t2 = time.perf_counter()
    bal = api.balance_cubes(merged, r)
    t3 = time.perf_counter()
    px = int(sum(m["depth"].size for m in maps))
    n1 = int(sum(len(a) for a in arrs))
    res = {"maps": len(maps), "pixels": px, "stage1_cubes": n1, "merged": int(len(merged)), "balanced": int(len(bal)),
           "ms_e2e": {"stage1": 1e3 * (t1 - t0), "merge": 1e3 * (t2 - t1), "balance": 1e3 * (t3 - t2)},
           "stage1_pixels_per_s_e2e": px / (t1 - t0), "merge_cubes_per_s_e2e": n1 / (t2 - t1),
           "balance_cubes_per_s_e2e": len(merged) / (t3 - t2),
           "what": "build_cubes per map (depth maps in pinned host memory), merge_cubes, balance_cubes; "
                   "host arrays in and out"}
    if not args.skip_cpu:
        sys.path.insert(0, os.path.join(HERE, "oracle"))
        import oracle as O
        s_maps = maps[:2]
        c0 = time.perf_counter()
        s_arrs = [O.build_cubes(m, o, r) for m in s_maps]
        c1 = time.perf_counter()
        s_merged = O.merge_cubes(s_arrs)
        c2 = time.perf_counter()
        s_bal = O.balance_cubes(s_merged, r)
        c3 = time.perf_counter()
        s_px = int(sum(m["depth"].size for m in s_maps))
        g_arrs = [api.build_cubes(m, o, r) for m in s_maps]
        g_merged = api.merge_cubes(g_arrs)
        same = (all(a.tobytes() == b.tobytes() for a, b in zip(g_arrs, s_arrs))
                and g_merged.tobytes() == s_merged.tobytes()
                and api.balance_cubes(g_merged, r).tobytes() == s_bal.tobytes())
        res["cpu_baseline"] = {
            "stage1_pixels_per_s": s_px / (c1 - c0),
            "merge_cubes_per_s": sum(map(len, s_arrs)) / (c2 - c1),
            "balance_cubes_per_s": len(s_merged) / (c3 - c2), "cores": 1, "kind": "port",
            "sample": f"the first 2 depth maps of {args.workload} ({s_px} pixels, {len(s_merged)} merged cubes)"}
        res["matches_oracle_on_sample"] = bool(same)
    return res


def warm_start_eval(args):
    """Time to relative residual 1e-4 (at most 6000 iterations per level) on
    held-out small scenes: zero start, trained network, reference initialisation."""
    from tgvreconclaude_gb300 import warmstart as WS
    if not os.path.exists(WS.WEIGHTS):
        return {"unavailable": "no trained weights at tgvreconclaude_gb300/data/warmstart_nb10.npz"}
    mlp = WS.WarmStartMLP.load(WS.WEIGHTS)
    recs, summary = WS.evaluate(mlp, range(1000, 1000 + args.warm_seeds), tol=1e-4)
    return {"tol": 1e-4, "max_iters_per_level": 6000, "scenes": len(recs), "graphs": "off (direct launches)",
            "scene": "16 cameras at 320x240, torus (depth 7) / three objects (depth 8), held-out seeds 1000+",
            **summary, "records": recs}


def time_to_gap_eval(args):
    """The batched-chunks configuration with 12 primitives (prims256: 256 cameras
    at 2048x1536, 128 chunks, streaming semantics) solved to relative residual
    1e-4 (at most 6000 iterations per level) on the device from the zero start,
    from the learned warm start and from the reference's initialisation; device
    time per solve (CUDA events on the library stream), prediction included."""
    import torch
    from tgvreconclaude_gb300 import api, warmstart as WS, workloads
    t0 = time.time()
    w = workloads.build(args.ttg_workload, seed=args.seed, device="cuda")
    gen_s = time.time() - t0
    torch.cuda.empty_cache()
    ctx = api.context()
    n = len(w.cubes)
    cubes_t = torch.from_numpy(w.cubes.view(np.int32).reshape(n, 4)).cuda()
    hists_t = torch.from_numpy(w.hists.view(np.int32)).cuda()
    out_t = torch.empty((n, 13), dtype=torch.float32, device="cuda")
    prm = api.TGVParams(alpha0=2.0, alpha1=1.0, iters=6000, tol=1e-4, check_every=10)
    res = {"workload": args.ttg_workload, "cubes": n, "chunks": int(len(w.leaves)), "cameras": len(w.cams),
           "image": f"{w.cfg['width']}x{w.cfg['height']}",
           "levels": {int(k): int(v) for k, v in enumerate(np.bincount(w.cubes["depth"], minlength=22)) if v},
           "gen_s": round(gen_s, 1), "tol": 1e-4, "max_iters_per_level": 6000, "graphs": "off (direct launches)"}
    # Stage 5 on the same workload: the binning kernel alone, and a bit-exact
    # check of its histograms against the oracle on a sample of cubes
    hs = histogram_kernel_eval(ctx, w, cubes_t, w.hists.shape[1], w.hists, torch.cuda.ExternalStream(ctx.stream))
    hs["oracle_check"] = histogram_oracle_check(w, w.hists, args.hist_sample // 4)
    res["histograms"] = hs
    ctx.set_graphs(False)
    try:
        starts = {"zero": torch.zeros((n, 13), dtype=torch.float32, device="cuda")}
        pred_ms = 0.0
        if os.path.exists(WS.WEIGHTS):
            mlp = WS.WarmStartMLP.load(WS.WEIGHTS)
            u_t = torch.empty(n, dtype=torch.float32, device="cuda")
            st = torch.cuda.ExternalStream(ctx.stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            lv = np.ascontiguousarray(w.leaves)
            e0.record(st)
            ctx.check(ctx.lib.tgvg_mlp_warm_start_dev(ctx.h, mlp.h, cubes_t.data_ptr(), hists_t.data_ptr(), n,
                                                      w.hists.shape[1], lv.ctypes.data, len(lv), u_t.data_ptr()),
                      "tgvg_mlp_warm_start_dev")
            with torch.cuda.stream(st):
                rec = torch.zeros((n, 13), dtype=torch.float32, device="cuda")
                rec[:, 0] = u_t
            e1.record(st)
            torch.cuda.synchronize()
            pred_ms = e0.elapsed_time(e1)
            starts["warm"] = rec
        for name in ("zero", "warm", "reference"):
            if name == "reference":
                st = api.tgv_solve_device(cubes_t, hists_t, out_t, w.leaves, "stream", prm)
            elif name in starts:
                st = api.tgv_solve_device(cubes_t, hists_t, out_t, w.leaves, "stream", prm,
                                          state_init_t=starts[name])
            else:
                continue
            ms = st["total_ms"] + (pred_ms if name == "warm" else 0.0)
            res[name] = {"ms": round(ms, 2), "leaf_iters": int(st["leaf_iters"]), "iters": st["iters_run"],
                         "active": [int(a) for a in st["active"]],
                         "capped_levels": int(sum(i >= prm.iters for i in st["iters_run"]))}
        if "warm" in res:
            res["warm"]["predict_ms"] = round(pred_ms, 3)
            res["time_ratio_zero_over_warm"] = res["zero"]["ms"] / res["warm"]["ms"]
            res["time_ratio_reference_over_warm"] = res["reference"]["ms"] / res["warm"]["ms"]
    finally:
        ctx.set_graphs(True)
    return res


def run_ours(args):
    import torch
    ws, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    from tgvreconclaude_gb300 import _native as N, api, workloads, formats as F
    t0 = time.time()
    if args.cache and os.path.exists(args.cache):
        w = workloads.load(args.cache)
    else:
        w = workloads.build(args.workload, seed=args.seed + rank, device="cuda", verbose=rank == 0,
                            max_cubes=args.max_cubes or None)
        if args.cache:
            workloads.save(w, args.cache)
    t_gen = time.time() - t0
    torch.cuda.empty_cache()  # drop the generator's temporaries before timing
    cfg = w.cfg
    ctx = api.context()
    n = len(w.cubes)
    nbins = w.hists.shape[1]
    cubes_t = torch.from_numpy(w.cubes.view(np.int32).reshape(n, 4)).cuda()
    hists_t = torch.from_numpy(w.hists.view(np.int32)).cuda()
    out_t = torch.empty((n, 13), dtype=torch.float32, device="cuda")
    prm = api.TGVParams(alpha0=2.0, alpha1=1.0, iters=args.iters or cfg["iters"])
    tune_prm = prm
    if args.tol > 0:  # time to tolerance: the stopped solves reuse the schedules a fixed-count solve tuned
        prm = api.TGVParams(alpha0=2.0, alpha1=1.0, iters=args.max_iters, tol=args.tol, check_every=10)
    mode = "stream" if cfg["chunks"] > 1 else "inmem"
    leaves = w.leaves if mode == "stream" else None
    stream = torch.cuda.ExternalStream(ctx.stream)
    # fixed schedules per size class (floor(log2 cubes)) instead of the online
    # autotuner: a profiler's serialised launches would skew the tuner's timings
    for item in filter(None, args.schedules.split(",")):
        cls, sched = (int(v) for v in item.split(":"))
        ctx.set_schedule(mode, cls, sched)

    # warm-up: the first step autotunes every level's schedule (direct launches);
    # with per-launch timing on, the third captures the level loop into a CUDA
    # graph (the second solve of the same problem does) that the timed steps relaunch
    for k in range(args.warmup):
        ctx.lib.tgvg_set_timing(ctx.h, int(k > 0))
        api.tgv_solve_device(cubes_t, hists_t, out_t, leaves, mode, tune_prm if k == 0 else prm)
    ctx.lib.tgvg_set_timing(ctx.h, 1)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    clocks = Clocks(local)
    clocks.start()
    k0 = ctx.kernel_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    li, kt_d, kt_p, kt_n, kt_active = 0, 0.0, 0.0, 0, 0
    for _ in range(args.steps):
        st = api.tgv_solve_device(cubes_t, hists_t, out_t, leaves, mode, prm)
        li += st["leaf_iters"]
        kt_d += st["kt_dual_ms"]
        kt_p += st["kt_primal_ms"]
        kt_n += st["kt_launches"]
        kt_active = st["kt_active"]
        last_st = st
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.kernel_count() - k0
    clk = clocks.stop()
    ctx.lib.tgvg_set_timing(ctx.h, 0)
    if pg:
        pg.barrier()
    elapsed = allreduce_max(e0.elapsed_time(e1) / 1e3, pg, torch)
    li_all = allreduce_sum(li, pg, torch)
    value = li_all / elapsed

    # ---- roofline of the dominant iteration kernel (per launch, CUDA events)
    hbm, peak_kind = peaks()
    dual_ms, primal_ms = kt_d / max(1, kt_n), kt_p / max(1, kt_n)
    if last_st.get("kt_fused"):  # one fused or wavefront launch per iteration (its time is in kt_dual_ms)
        dom, ms, bpc = ("k_wave" if last_st["kt_fused"] == 2 else "k_fused"), dual_ms, BYTES_ITER
    else:
        dom, ms, bpc = ("k_dual", dual_ms, BYTES_DUAL) if kt_d >= kt_p else ("k_primal", primal_ms, BYTES_PRIMAL)
    achieved = bpc * kt_active / (ms * 1e-3) / 1e9 if ms > 0 else None
    tpc = traffic_per_cube().get(dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": (achieved / hbm) if achieved else None, "peak_kind": peak_kind,
            "traffic": (tpc * kt_active) if tpc else None,
            "bytes_per_launch": bpc * kt_active, "avg_launch_ms": ms, "active_cubes": kt_active,
            "iteration_achieved": BYTES_ITER * kt_active / ((dual_ms + primal_ms) * 1e-3) / 1e9
            if dual_ms + primal_ms > 0 else None,
            "other_kernel_ms": 0.0 if dom in ("k_fused", "k_wave") else (primal_ms if dom == "k_dual" else dual_ms)}

    result = None
    if rank == 0:
        e2e = {} if args.skip_e2e else measure_e2e(args, w, ctx, prm, mode, leaves, out_t, stream)

        # ---- Stage 5 on the same workload: pyramids + binning, host buffers in/out
        # (depth maps and cubes in pinned host memory, as for the solver's e2e)
        hs = {}
        if not args.skip_hist:
            pin_maps = [torch.from_numpy(np.ascontiguousarray(d, np.float32)).pin_memory().numpy() for d in w.depths]
            pin_cubes = torch.from_numpy(w.cubes.view(np.int32).reshape(n, 4).copy()).pin_memory().numpy()
            pin_cubes = pin_cubes.view(F.CUBE_DTYPE).reshape(n)
            h_t0 = time.perf_counter()
            hh = api.compute_histograms_from_maps(pin_cubes, w.cams, pin_maps, cfg["origin"], cfg["r_root"], nbins)
            h_dt = time.perf_counter() - h_t0
            pairs = n * len(w.cams)
            hs = {"pairs_per_s_e2e": pairs / h_dt, "ms_e2e": 1e3 * h_dt, "pairs": pairs,
                  "oracle_check": histogram_oracle_check(w, hh, args.hist_sample)}
            if w.cams:
                hs["device"] = histogram_kernel_eval(ctx, w, cubes_t, nbins, hh, stream)

        # ---- CPU oracle baseline on a bounded sample (1 thread), and the error
        # of this package's FP32 result against an FP64 run of the same solver
        cb, f64 = {}, {}
        if not args.skip_cpu:
            cubes_s, hists_s = cpu_sample(w, args.cpu_sample, args.cpu_iters)
            v, dt, lis, ref32 = time_cpu_oracle(cubes_s, hists_s, args.cpu_iters, 1)
            cb = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "seconds": dt, "host_cores": os.cpu_count(),
                  "sample": f"{len(cubes_s)} contiguous Morton-ordered cubes of {args.workload}, {args.cpu_iters} iterations per "
                            f"level, in-memory semantics, single thread"}
            import oracle as O
            ref64, _ = O.tgv_solve(cubes_s, hists_s, None, "inmem", 2.0, 1.0, args.cpu_iters, fp64=True,
                                   nthreads=os.cpu_count() or 1)
            gpu32, _ = api.tgv_solve(cubes_s, hists_s, None, "inmem",
                                     api.TGVParams(alpha0=2.0, alpha1=1.0, iters=args.cpu_iters))
            du = np.abs(gpu32["u"].astype(np.float64) - ref64[:, 0])
            bounded = np.abs(ref64[:, 0]) <= 1.0
            f64 = {"cubes": int(len(cubes_s)), "iters_per_level": args.cpu_iters, "max_abs_du": float(du.max()),
                   "rms_du": float(np.sqrt(np.mean(du ** 2))), "max_abs_du_bounded": float(du[bounded].max()),
                   "what": "this package's FP32 u against the oracle's FP64 run on the same slice",
                   "fp32_bit_exact": gpu32.tobytes() == ref32.tobytes(),
                   "fp32_what": "the whole 13-float state against the oracle's FP32 run timed as cpu_baseline"}

        surf = {} if args.skip_surface else surface_eval(args, w, out_t)
        s13 = {} if args.skip_stages13 else stages13_eval(args, w)
        ws_eval = {} if args.skip_warm else warm_start_eval(args)
        ttg = {} if args.skip_ttg else time_to_gap_eval(args)

        depth_hist = np.bincount(w.cubes["depth"], minlength=22)
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "cubes": n, "cameras": len(w.cams),
                       "image": f"{cfg['width']}x{cfg['height']}", "max_depth": cfg["max_depth"], "nbins": nbins,
                       "iters_per_level": prm.iters, "alpha1": prm.alpha1, "alpha0": prm.alpha0,
                       "tol": prm.tol, "check_every": prm.check_every if prm.tol > 0 else None,
                       "semantics": "tgv_minimize" if mode == "inmem" else "tgv_minimize_streaming (batched)",
                       "chunks": len(w.leaves), "levels": {int(k): int(v) for k, v in enumerate(depth_hist) if v},
                       "l2": "inputs larger than L2 (about 100 B of state per cube)",
                       "schedules": args.schedules or "autotuned",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
            "e2e": e2e, "roofline": roof, "cpu_baseline": cb, "fp64_check": f64, "histograms": hs, "surface": surf,
            "stages_1_3": s13,
            "warm_start": ws_eval,
            "time_to_gap": ttg,
            "clocks": clk, "graph": last_st["graph"],
            "gpu_launches": int(launches), "leaf_iters_per_step": int(li_all / args.steps),
            "levels_detail": [{"depth": d, "active": int(a), "ms": round(m, 3), "schedule": s, "iters": it,
                               "residual": r, "energy": en}
                              for d, a, m, s, it, r, en in zip(last_st["depth"], last_st["active"],
                                                              last_st["level_ms"], last_st["schedule"],
                                                              last_st["iters_run"], last_st["residual"],
                                                              last_st["energy"])],
            "gen_s": round(t_gen, 1),
        }
        print(json.dumps(result), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="three64")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--iters", type=int, default=0, help="override iterations per level")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-sample", type=int, default=1000000)
    ap.add_argument("--cpu-iters", type=int, default=50)
    ap.add_argument("--ref-sample", type=int, default=0, help="reference-arm slice (0: the --cpu-sample slice)")
    ap.add_argument("--hist-sample", type=int, default=200000, help="cubes checked bit-exact against the oracle")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-hist", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-warm", action="store_true")
    ap.add_argument("--skip-surface", action="store_true")
    ap.add_argument("--skip-stages13", action="store_true")
    ap.add_argument("--tol", type=float, default=0.0,
                    help="solve each level to this relative residual (time to tolerance) instead of a fixed count")
    ap.add_argument("--max-iters", type=int, default=6000, help="iteration cap per level with --tol")
    ap.add_argument("--warm-seeds", type=int, default=20)
    ap.add_argument("--skip-ttg", action="store_true", help="skip the time-to-gap solves of --ttg-workload")
    ap.add_argument("--ttg-workload", default="prims256")
    ap.add_argument("--max-cubes", type=int, default=0, help="truncate the workload (profiling runs)")
    ap.add_argument("--cache", default="", help="load the workload from / save it to this .npz (profiling runs)")
    ap.add_argument("--schedules", default="", help="fix schedules, e.g. 17:15,21:14 (size class:schedule; profiling runs)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
