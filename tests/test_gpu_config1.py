"""The CPU-runnable benchmark configuration end to end on the GPU, against the
oracle at full size (not a sample): a seeded torus (R = 1, r = 0.3,
N(0, 0.005) noise) seen by 16 cameras on a radius-3 sphere at 640x480, cubes
to depth 8 (about 0.27 M with seed 0), the reference's 8-bin histograms, TGV alpha1 = 1,
alpha0 = 2, 300 iterations per level (reference src/histogram.cpp:127-163,
src/tgv.cpp:356-419).

Bars: every histogram row bit-exact; the TGV state bit-exact with the oracle
(which is bit-exact with the reference); the FP32 u within 1e-4 of an FP64 run
of the same solver."""
import os

import numpy as np
import pytest

from tgvreconclaude_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu


def oracle_maps(w):
    maps = []
    for c, d in zip(w.cams, w.depths):
        rt_inv = np.array(list(c.rt_inv), np.float32).reshape(4, 4)
        maps.append(dict(depth=np.ascontiguousarray(d, np.float32), rt_inv=rt_inv, fx=c.fx, fy=c.fy, cx=c.cx,
                         cy=c.cy, lidar=bool(c.lidar)))
    return maps


def test_config1_histograms_and_tgv_full_size(oracle_lib):
    w = W.build("torus16", seed=0, device="cuda", keep_depths=True, histograms=False)
    cfg = w.cfg
    n = len(w.cubes)
    assert 150_000 < n < 900_000, n
    nt = os.cpu_count() or 1
    h_gpu = api.compute_histograms_from_maps(w.cubes, w.cams, w.depths, cfg["origin"], cfg["r_root"], 8)
    h_ref = oracle_lib.compute_histograms(w.cubes, oracle_maps(w), cfg["origin"], cfg["r_root"], 8, nthreads=nt)
    assert h_gpu.shape == (n, 8) and int(h_ref.sum()) > 0
    assert np.array_equal(h_gpu, h_ref), f"{int((h_gpu != h_ref).any(1).sum())} of {n} rows differ"

    out, st = api.tgv_solve(w.cubes, h_gpu, None, "inmem", api.TGVParams(alpha0=2.0, alpha1=1.0, iters=300))
    ref, _ = oracle_lib.tgv_solve(w.cubes, h_ref, None, "inmem", 2.0, 1.0, 300, nthreads=nt)
    assert st["leaf_iters"] == 300 * n
    du = float(np.abs(out["u"].astype(np.float64) - ref["u"]).max())
    assert out.tobytes() == ref.tobytes(), f"state differs from the oracle (max|du| = {du})"

    f64, _ = oracle_lib.tgv_solve(w.cubes, h_ref, None, "inmem", 2.0, 1.0, 300, fp64=True, nthreads=nt)
    err = np.abs(out["u"].astype(np.float64) - f64[:, 0])
    print(f"config 1: {n} cubes, max|u32 - u64| = {err.max():.3e}, rms {np.sqrt(np.mean(err ** 2)):.3e}")
    assert float(err.max()) <= 1e-4, f"max|u32 - u64| = {err.max()} (rms {np.sqrt(np.mean(err ** 2))})"
