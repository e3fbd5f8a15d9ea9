"""GPU parity of the whole-state warm start (tgvg_tgv_minimize_state): every
cube starts its own level from the caller's (u, v, p, q) record instead of the
reference's parent copy, and holds the reference's initial state until then.
The oracle restates the same rule (level_init); states must agree bit for bit
in all three semantics, under every iteration schedule, with and without the
stopping test.  Also: solves of different problems back to back on one context
(pooled buffers hold the previous solve's p/q) give the oracle's state."""
import ctypes as C

import numpy as np
import pytest

from tgvreconclaude_gb300 import _native as N, api, formats as F, scenes as S

pytestmark = pytest.mark.gpu


def random_state(rng, n, scale=0.5):
    s = np.zeros(n, F.STATE_DTYPE)
    s["u"] = rng.uniform(-1, 1, n)
    s["v"] = rng.normal(0, 0.1 * scale, (n, 3))
    s["p"] = rng.normal(0, scale, (n, 3))
    s["q"] = rng.normal(0, scale, (n, 6))
    return s


def same(gpu, ref, what):
    du = float(np.abs(gpu["u"].astype(np.float64) - ref["u"]).max()) if len(ref) else 0.0
    assert du <= 1e-4, f"{what}: max|du| = {du}"
    assert gpu.tobytes() == ref.tobytes(), f"{what}: not bit-identical (max|du| = {du})"


@pytest.mark.parametrize("seed", range(4))
def test_state_start_random_vs_oracle(oracle_lib, seed):
    rng = np.random.default_rng(900 + seed)
    nbins = 10 if seed % 2 else 8
    cubes = S.random_octree(rng, dmin=seed % 3, dmax=4 + seed % 3, target=4000 + 3000 * seed,
                            shape=["sphere", "plane", "random"][seed % 3])
    hists = S.random_histograms(rng, len(cubes), nbins=nbins)
    leaves = S.split_leaves(len(cubes), 1 + 2 * seed, rng, cubes, aligned=seed % 2 == 0)
    s0 = random_state(rng, len(cubes))
    for mode in ("inmem", "oc", "stream"):
        ref, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 23, level_init=s0)
        out, _ = api.tgv_solve(cubes, hists, leaves, mode, api.TGVParams(2.0, 1.0, 23), state_init=s0)
        same(out, ref, f"seed {seed} {mode}")
        ref, rst = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 300, tol=1e-3, check_every=10,
                                        level_init=s0)
        out, st = api.tgv_solve(cubes, hists, leaves, mode,
                                api.TGVParams(2.0, 1.0, 300, tol=1e-3, check_every=10), state_init=s0)
        same(out, ref, f"seed {seed} {mode} stopping")
        assert st["iters_run"] == [r["iters_run"] for r in rst]


def test_zero_state_start(oracle_lib):
    """All-zero records: a zero start of every level of the reference's problem;
    on a one-level octree that is the reference's zero initialisation."""
    rng = np.random.default_rng(5)
    cubes = S.random_octree(rng, dmin=2, dmax=6, target=8000, shape="sphere")
    hists = S.random_histograms(rng, len(cubes), nbins=10)
    z = np.zeros(len(cubes), F.STATE_DTYPE)
    ref, _ = oracle_lib.tgv_solve(cubes, hists, None, "inmem", 2.0, 1.0, 60, level_init=z)
    out, _ = api.tgv_solve(cubes, hists, None, "inmem", api.TGVParams(2.0, 1.0, 60), state_init=z)
    same(out, ref, "zero records")
    one = cubes[cubes["depth"] == 5]
    h1 = hists[cubes["depth"] == 5]
    ref, _ = oracle_lib.tgv_solve(one, h1, None, "inmem", 2.0, 1.0, 60, init="zero")
    out, _ = api.tgv_solve(one, h1, None, "inmem", api.TGVParams(2.0, 1.0, 60), state_init=z[:len(one)])
    same(out, ref, "one level, zero records vs zero initialisation")


@pytest.mark.parametrize("mode", ["inmem", "stream"])
def test_state_start_every_schedule(oracle_lib, mode):
    ctx = api.context()
    rng = np.random.default_rng(43)
    cubes = S.random_octree(rng, dmin=1, dmax=6, target=12000, shape="sphere")
    hists = S.random_histograms(rng, len(cubes), nbins=8, empty_frac=0.0)
    leaves = S.split_leaves(len(cubes), 5, rng, cubes, aligned=True)
    s0 = random_state(rng, len(cubes))
    ref, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 40, nthreads=8, level_init=s0)
    try:
        for cfg in range(25):
            ctx.set_schedule(mode, -1, cfg)
            out, _ = api.tgv_solve(cubes, hists, leaves, mode, api.TGVParams(2.0, 1.0, 40), state_init=s0)
            same(out, ref, f"schedule {cfg} {mode}")
    finally:
        ctx.set_schedule(mode, -1, -1)


@pytest.mark.parametrize("mode", ["inmem", "oc", "stream"])
def test_back_to_back_solves_on_one_context(oracle_lib, mode):
    """A whole-state solve leaves nonzero p/q in every pooled buffer (both
    ping-pong sets of the fused schedules too); the next solve, of a different
    problem of the same size, must not see them.  Run under every schedule."""
    ctx = api.context()
    rng = np.random.default_rng(61)
    a = S.random_octree(rng, dmin=1, dmax=6, target=10000, shape="sphere")
    b = S.random_octree(rng, dmin=2, dmax=6, target=10000, shape="plane")
    n = min(len(a), len(b))
    a, b = a[:n], b[:n]
    ha = S.random_histograms(rng, n, nbins=8, empty_frac=0.0)
    hb = S.random_histograms(rng, n, nbins=8, empty_frac=0.1)
    la = S.split_leaves(n, 3, rng, a, aligned=True)
    lb = S.split_leaves(n, 4, rng, b, aligned=True)
    sa = random_state(rng, n, scale=1.0)
    ref_b, _ = oracle_lib.tgv_solve(b, hb, lb, mode, 2.0, 1.0, 30, nthreads=8)
    try:
        for cfg in range(25):
            ctx.set_schedule(mode, -1, cfg)
            api.tgv_solve(a, ha, la, mode, api.TGVParams(2.0, 1.0, 30), state_init=sa)
            out, _ = api.tgv_solve(b, hb, lb, mode, api.TGVParams(2.0, 1.0, 30))
            same(out, ref_b, f"schedule {cfg} {mode} after a whole-state solve")
    finally:
        ctx.set_schedule(mode, -1, -1)


def test_state_start_errors():
    rng = np.random.default_rng(1)
    cubes = S.random_octree(rng, dmin=2, dmax=4, target=500)
    hists = S.random_histograms(rng, len(cubes))
    ctx = api.context()
    out = np.zeros(len(cubes), F.STATE_DTYPE)
    prm = api.TGVParams(2.0, 1.0, 5, init="state").struct()
    st = N.Stats()
    # the plain entry has no state array to read
    assert ctx.lib.tgvg_tgv_minimize(ctx.h, cubes.ctypes.data, hists.ctypes.data, len(cubes), 8, None, 0, 0,
                                     C.byref(prm), None, out.ctypes.data, C.byref(st)) == -1
    # the state entry wants init = state and a state array
    prm2 = api.TGVParams(2.0, 1.0, 5).struct()
    s0 = np.zeros(len(cubes), F.STATE_DTYPE)
    assert ctx.lib.tgvg_tgv_minimize_state(ctx.h, cubes.ctypes.data, hists.ctypes.data, len(cubes), 8, None, 0,
                                           0, C.byref(prm2), s0.ctypes.data, out.ctypes.data, C.byref(st)) == -1
    assert ctx.lib.tgvg_tgv_minimize_state(ctx.h, cubes.ctypes.data, hists.ctypes.data, len(cubes), 8, None, 0,
                                           0, C.byref(prm), None, out.ctypes.data, C.byref(st)) == -1
