"""Run every kernel family of the library once on one mid-size workload, for a
profiler's launch list (per-kernel time and DRAM traffic).

    python -m tgvreconclaude_gb300.kernel_tour [--workload torus16] [--iters 20]

Stages, in order: cubes from the first depth maps (Stage 1); pyramids and
histograms (Stage 5) from the workload's depth maps; the TGV solve (Stage 6) under the in-memory, OC and streaming semantics
with each schedule family forced in turn (per-sweep launches, band order, two
cubes per thread, persistent, cluster, fused, fused with TMA staging); surface
extraction with normals; the warm-start network's features, forward pass,
gradient and one training epoch.  Prints one line per stage.
"""
from __future__ import annotations

import argparse
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="torus16")
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--max-cubes", type=int, default=0)
    a = ap.parse_args(argv)
    from . import api, workloads as W, warmstart as WS

    t0 = time.time()
    w = W.build(a.workload, seed=0, histograms=False, max_cubes=a.max_cubes or None)
    cfg = w.cfg
    o, r = np.float32(cfg["origin"]), float(cfg["r_root"])
    nc = 0
    for cam, d in list(zip(w.cams, w.depths))[:4]:
        rt = np.linalg.inv(np.asarray(cam.rt_inv[:], np.float64).reshape(4, 4)).astype(np.float32)
        nc += len(api.build_cubes(dict(depth=d, rt=rt, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy), o, r))
    print(f"stage 1: {nc} cubes from 4 depth maps", flush=True)
    hists = api.compute_histograms_from_maps(w.cubes, w.cams, w.depths, cfg["origin"], cfg["r_root"], cfg["nbins"])
    print(f"histograms: {len(w.cubes)} cubes x {len(w.cams)} cameras, {int(hists.sum())} votes "
          f"({time.time() - t0:.1f} s with generation)", flush=True)

    ctx = api.context()
    ctx.set_graphs(False)
    leaves = W.chunk_leaves(w.cubes, 8, np.random.default_rng(0)) if cfg["chunks"] <= 1 else w.leaves
    prm = api.TGVParams(alpha0=2.0, alpha1=1.0, iters=a.iters)
    state = None
    for mode in ("inmem", "oc", "stream"):
        for cfg_id in (0, 14, 16, 3, 11, 18, 19):
            ctx.set_schedule(mode, -1, cfg_id)
            out, st = api.tgv_solve(w.cubes, hists, None if mode == "inmem" else leaves, mode, prm)
            if mode == "inmem" and cfg_id == 0:
                state = out
        ctx.set_schedule(mode, -1, -1)
        print(f"tgv {mode}: levels {st['depth']}, schedules {sorted(set(st['schedule']))}", flush=True)
    stop = api.TGVParams(alpha0=2.0, alpha1=1.0, iters=4 * a.iters, tol=1e-3, check_every=10)
    api.tgv_solve(w.cubes, hists, None, "inmem", stop)
    ctx.set_graphs(True)

    has = (hists.sum(1) > 0).astype(np.uint8)
    v, f, _ = api.extract_surface(w.cubes, state, o, r, has_data=has, normals=True)
    vs, fs = api.extract_surface_leaves(w.cubes, state, hists, leaves, o, r)
    print(f"surface: {len(v)} vertices, {len(f)} triangles; streaming semantics {len(fs)} triangles", flush=True)

    m = WS.WarmStartMLP.load(WS.WEIGHTS)
    X = m.features(w.cubes, hists)
    u0 = m.warm_start(w.cubes, hists)
    t = (state["u"] - WS.median_start(hists)).astype(np.float32)
    loss, _ = m.grad(X[:65536], t[:65536])
    m.train(X[:65536], t[:65536], epochs=1, batch=4096, lr=1e-4, seed=0)
    print(f"warm start: {len(u0)} predictions, loss {loss:.3g}, one training epoch", flush=True)


if __name__ == "__main__":
    main()
