"""Run every kernel family of the library once on one mid-size workload, for a
profiler's launch list (per-kernel time and DRAM traffic).

    python -m tgvreconclaude_gb300.kernel_tour [--workload torus16] [--iters 20]
        [--max-cubes N] [--maps K] [--cache PATH]

Stages, in order: cubes from the first depth maps (Stage 1), their merge
(Stage 2) and its 2:1 balance (Stage 3); pyramids and histograms (Stage 5)
from the workload's depth maps (the first K with --maps); the TGV solve (Stage 6) under the in-memory, OC and streaming semantics
with each schedule family forced in turn (per-sweep launches, band order, two
cubes per thread, persistent, cluster and single block on the small levels
they are for, fused, fused with TMA staging, ordered
wavefront through L2 and through L1); surface
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
    ap.add_argument("--maps", type=int, default=0, help="depth maps used by Stages 1-5 (0: all)")
    ap.add_argument("--cache", default="", help="workload file: written if absent, else read (no generation)")
    a = ap.parse_args(argv)
    from . import api, workloads as W, warmstart as WS

    t0 = time.time()
    w = load_or_build(a, W)
    cfg = w.cfg
    o, r = np.float32(cfg["origin"]), float(cfg["r_root"])
    arrs = []
    for cam, d in list(zip(w.cams, w.depths))[:4]:
        rt = np.linalg.inv(np.asarray(cam.rt_inv[:], np.float64).reshape(4, 4)).astype(np.float32)
        arrs.append(api.build_cubes(dict(depth=d, rt=rt, fx=cam.fx, fy=cam.fy, cx=cam.cx, cy=cam.cy), o, r))
    merged = api.merge_cubes(arrs)
    bal = api.balance_cubes(merged, r)
    print(f"stages 1-3: {sum(map(len, arrs))} cubes from {len(arrs)} depth maps, {len(merged)} merged, "
          f"{len(bal)} balanced", flush=True)
    hists = api.compute_histograms_from_maps(w.cubes, w.cams, w.depths, cfg["origin"], cfg["r_root"], cfg["nbins"])
    print(f"histograms: {len(w.cubes)} cubes x {len(w.cams)} cameras, {int(hists.sum())} votes "
          f"({time.time() - t0:.1f} s with generation)", flush=True)

    ctx = api.context()
    ctx.set_graphs(False)
    leaves = W.chunk_leaves(w.cubes, 8, np.random.default_rng(0)) if cfg["chunks"] <= 1 else w.leaves
    prm = api.TGVParams(alpha0=2.0, alpha1=1.0, iters=a.iters)
    state = None
    for mode in ("inmem", "oc", "stream"):
        for cfg_id in (0, 14, 16, 3, 11, 22, 18, 19, 20, 21):
            ctx.set_schedule(mode, -1, 14 if cfg_id in (11, 22) else cfg_id)
            if cfg_id in (11, 22):  # the small-level schedules on the levels they are for
                for cls in range(13 if cfg_id == 22 else 17):
                    ctx.set_schedule(mode, cls, cfg_id)
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


def load_or_build(a, W):
    """The workload, with its depth maps and cameras (the first --maps of them)."""
    import os
    from . import _native as N
    if a.cache and os.path.exists(a.cache):
        d = np.load(a.cache)
        w = W.Workload(str(d["name"]), dict(W.CONFIGS[str(d["name"])]), [], list(d["depths"]), d["cubes"],
                       d["hists"], d["leaves"], {})
        for row in d["cams"]:
            cam = N.Camera()
            cam.rt_inv[:] = [float(v) for v in row[:16]]
            cam.fx, cam.fy, cam.cx, cam.cy = (float(v) for v in row[16:20])
            cam.width, cam.height, cam.lidar = int(row[20]), int(row[21]), int(row[22])
            w.cams.append(cam)
        return w
    w = W.build(a.workload, seed=0, histograms=False, max_cubes=a.max_cubes or None)
    if a.maps:
        w.cams, w.depths = w.cams[:a.maps], w.depths[:a.maps]
    if a.cache:
        cams = np.array([list(c.rt_inv) + [c.fx, c.fy, c.cx, c.cy, c.width, c.height, c.lidar] for c in w.cams],
                        np.float64)
        np.savez(a.cache, name=w.name, cubes=w.cubes, hists=w.hists, leaves=w.leaves, depths=np.stack(w.depths),
                 cams=cams)
    return w


if __name__ == "__main__":
    main()
