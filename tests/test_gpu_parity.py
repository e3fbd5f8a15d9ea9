"""GPU parity: the sm_103a path through the C ABI against the oracle and the
reference's golden fixtures.

Bars: histograms and pyramids bit-exact; TGV states bit-exact with the oracle
(which is itself bit-exact with the reference), and always within the stated
tolerance max|du| <= 1e-4.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_maps, load_golden
from tgvreconclaude_gb300 import _native as N, api, formats as F, scenes as S

pytestmark = pytest.mark.gpu
TOL_U = 1e-4

TGV_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "tgv_*.npz")))
HIST_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "hist_*.npz")))


def cams_from(maps):
    out = []
    for m in maps:
        c = N.Camera()
        c.rt_inv[:] = [float(v) for v in np.asarray(m["rt_inv"], np.float32).reshape(16)]
        c.fx, c.fy, c.cx, c.cy = m["fx"], m["fy"], m["cx"], m["cy"]
        h, w = m["depth"].shape
        c.width, c.height = w, h
        c.lidar = int(bool(m.get("lidar", False)))
        out.append(c)
    return out


def render_maps(scene, rig, seed=0, lidar_every=0):
    maps = []
    for i, c in enumerate(rig):
        d = S.render_depth(scene, c, seed=seed + i).numpy()
        rt_inv = np.linalg.inv(np.asarray(c["rt"], np.float64)).astype(np.float32)
        maps.append(dict(depth=d, rt=c["rt"], rt_inv=rt_inv, fx=c["fx"], fy=c["fy"], cx=c["cx"], cy=c["cy"],
                         lidar=bool(lidar_every and i % lidar_every == 0)))
    return maps


def assert_state_equal(gpu, ref, what=""):
    du = np.abs(gpu["u"].astype(np.float64) - ref["u"]).max() if len(ref) else 0.0
    assert du <= TOL_U, f"{what}: max|du| = {du}"
    assert gpu.tobytes() == ref.tobytes(), f"{what}: not bit-identical (max|du| = {du})"


# ------------------------------------------------------------- Stage 5 ---

@pytest.mark.parametrize("case", HIST_CASES)
def test_histograms_match_golden(case):
    g = load_golden(case)
    maps = golden_maps(g)
    bins = api.compute_histograms_from_maps(g["cubes"], cams_from(maps), [m["depth"] for m in maps], g["origin"],
                                            float(g["r_root"]))
    assert np.array_equal(bins, g["bins"])


def test_pyramids_bitexact(oracle_lib):
    rng = np.random.default_rng(5)
    for (h, w) in [(37, 50), (1, 9), (64, 2), (480, 640), (1080, 1920), (5, 5)]:
        d = rng.uniform(0.5, 5.0, (h, w)).astype(np.float32)
        d[rng.random((h, w)) < 0.2] = np.nan
        d[rng.random((h, w)) < 0.05] = -1.0
        d[rng.random((h, w)) < 0.02] = np.inf
        d[rng.random((h, w)) < 0.02] = 0.0
        mm = api.DepthMipmap().build(api.DepthMap(w, h, d))
        ref, dims = oracle_lib.pyramid(d)
        assert mm.dims == dims
        assert mm._flat.view(np.uint32).tobytes() == ref.view(np.uint32).tobytes(), (h, w)


@pytest.mark.parametrize("nbins", [8, 10])
def test_histograms_random_scenes(oracle_lib, nbins):
    rng = np.random.default_rng(11 + nbins)
    scene = S.three_objects_scene(rng)
    maps = render_maps(scene, S.sphere_rig(12, 6.0, width=160, height=120, half_fov_deg=28), 40, lidar_every=5)
    cubes = S.random_octree(rng, dmin=3, dmax=9, target=60000, shape="sphere", r_root=3.0)
    cubes["r_c"][:8] = [0.0, -2.0, np.nan, np.inf, 1e9, 1e-30, -0.0, 5.0]
    ref = oracle_lib.compute_histograms(cubes, maps, (-3.0, -3.0, -3.0), 3.0, nbins=nbins, nthreads=8)
    gpu = api.compute_histograms_from_maps(cubes, cams_from(maps), [m["depth"] for m in maps], (-3.0, -3.0, -3.0),
                                           3.0, nbins=nbins)
    assert ref.sum() > 0
    assert np.array_equal(gpu, ref)


def test_histograms_via_depth_mipmap(oracle_lib):
    """The DepthMipmap route (pyramids built on the GPU, then compute_histograms)."""
    rng = np.random.default_rng(2)
    rig = S.sphere_rig(5, 3.0, width=120, height=90)
    maps = render_maps(S.torus_scene(), rig, 7, lidar_every=2)
    mms = []
    for m in maps:
        mm = api.DepthMipmap().build(api.DepthMap(120, 90, m["depth"], K=np.array(
            [[m["fx"], 0, m["cx"]], [0, m["fy"], m["cy"]], [0, 0, 1]], np.float32), Rt=m["rt"]), m["lidar"])
        m["rt_inv"] = mm.Rt_inv
        mms.append(mm)
    cubes = S.random_octree(rng, dmin=3, dmax=8, target=20000, r_root=1.5)
    gpu = api.compute_histograms(cubes, mms, (-1.5, -1.5, -1.5), 1.5)
    ref = oracle_lib.compute_histograms(cubes, maps, (-1.5, -1.5, -1.5), 1.5)
    assert np.array_equal(gpu, ref)
    # project / depth_at mirror the reference's per-point API (test_stage5.cpp:45-80)
    c = F.cube_keys(cubes[:50])
    for i in range(50):
        x, y, z = (int(v) for v in F.morton_decode(np.uint64(c[i])))
        d = int(cubes["depth"][i]); cs = 3.0 / (1 << d)
        P = [-1.5 + ((v >> (21 - d)) + 0.5) * cs for v in (x, y, z)]
        assert mms[0].project(P, float(cubes["r_c"][i]))[0] == oracle_lib.project(maps[0], P, float(cubes["r_c"][i]))[0]


def test_histograms_empty_and_no_cameras():
    e = api.compute_histograms_from_maps(np.zeros(0, F.CUBE_DTYPE), [], [], (0, 0, 0), 1.0)
    assert e.shape == (0, 8)
    rng = np.random.default_rng(0)
    cubes = S.random_octree(rng, 2, 4, 100)
    z = api.compute_histograms_from_maps(cubes, [], [], (0, 0, 0), 1.0)
    assert z.shape == (len(cubes), 8) and z.sum() == 0


def test_histograms_oc_file(tmp_path, oracle_lib):
    """compute_histograms_oc: cube file + leaves in, TGVH out (histogram.cpp:222-256)."""
    g = load_golden("hist_torus.npz")
    maps = golden_maps(g)
    cp, hp = tmp_path / "c.bin", tmp_path / "h.bin"
    F.save_cubes(cp, g["cubes"], float(g["r_root"]))
    leaves = S.split_leaves(len(g["cubes"]), 5, np.random.default_rng(1), g["cubes"])
    mms = []
    for m in maps:
        mm = api.DepthMipmap().build(api.DepthMap(m["depth"].shape[1], m["depth"].shape[0], m["depth"], K=np.array(
            [[m["fx"], 0, m["cx"]], [0, m["fy"], m["cy"]], [0, 0, 1]], np.float32), Rt=m["rt"]), m["lidar"])
        mm.Rt_inv = m["rt_inv"]
        mms.append(mm)
    api.compute_histograms_oc(cp, leaves, mms, g["origin"], float(g["r_root"]), hp)
    assert np.array_equal(F.load_histograms(hp), g["bins"])


# ------------------------------------------------------------- Stage 6 ---

@pytest.mark.parametrize("case", TGV_CASES)
@pytest.mark.parametrize("mode", ["inmem", "oc", "stream"])
def test_tgv_matches_golden(case, mode):
    g = load_golden(case)
    a0, a1 = (float(x) for x in g["params"])
    prm = api.TGVParams(alpha0=a0, alpha1=a1, iters=int(g["iters"]))
    out, st = api.tgv_solve(g["cubes"], g["hists"], g["leaves"], mode, prm)
    assert_state_equal(out, g[mode], f"{case}/{mode}")
    assert st["leaf_iters"] == len(g["cubes"]) * int(g["iters"])  # golden leaves cover every cube


@pytest.mark.parametrize("seed", range(6))
def test_tgv_random_vs_oracle(oracle_lib, seed):
    rng = np.random.default_rng(500 + seed)
    nbins = 10 if seed % 3 == 2 else 8
    cubes = S.random_octree(rng, dmin=seed % 3, dmax=3 + seed % 4, target=3000 + 2000 * seed,
                            shape=["sphere", "plane", "random"][seed % 3])
    hists = S.random_histograms(rng, len(cubes), nbins=nbins)
    leaves = S.split_leaves(len(cubes), 1 + 2 * seed, rng, cubes, aligned=seed % 2 == 0)
    init = ["median", "zero", "given"][seed % 3]
    u0 = rng.uniform(-1, 1, len(cubes)).astype(np.float32) if init == "given" else None
    for mode in ("inmem", "oc", "stream"):
        a0, a1 = [(0.02, 0.04), (2.0, 1.0), (0.3, 0.1)][seed % 3]
        ref, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, a0, a1, 17, init=init, u_init=u0)
        out, _ = api.tgv_solve(cubes, hists, leaves, mode, api.TGVParams(a0, a1, 17, init=init), u_init=u0)
        assert_state_equal(out, ref, f"seed {seed} {mode}")


def test_tgv_autotuned_schedules_are_exact(oracle_lib):
    """800 iterations: the first solve tunes each level's schedule online
    (per-sweep launches with and without register cap and L2 prefetch vs one
    cooperative launch per level, several grid sizes), the second reuses the
    tuned table; both stay bit-identical."""
    rng = np.random.default_rng(77)
    cubes = S.random_octree(rng, dmin=1, dmax=7, target=60000, shape="sphere")
    hists = S.random_histograms(rng, len(cubes), nbins=8, empty_frac=0.05)
    leaves = S.split_leaves(len(cubes), 5, rng, cubes, aligned=True)
    for mode in ("inmem", "stream"):
        ref, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, alpha0=2.0, alpha1=1.0, iters=800, nthreads=8)
        for _ in range(2):
            out, st = api.tgv_solve(cubes, hists, leaves, mode, api.TGVParams(alpha0=2.0, alpha1=1.0, iters=800))
            assert_state_equal(out, ref, f"autotuned {mode}")


@pytest.mark.parametrize("mode", ["inmem", "oc", "stream"])
def test_tgv_every_schedule_is_exact(oracle_lib, mode):
    """Each of the twenty-five iteration schedules (per-sweep launches with and
    without register cap / L2 prefetch / swapped sweep directions / band order /
    two cubes per thread, the fused tile kernel plain and TMA-staged, the ordered
    wavefront through L2 and through L1 (these four run band order in OC
    semantics), six persistent grid sizes, clusters of 8 and 16 CTAs, a single
    block reading through L1 or holding the state in shared memory, a cluster
    holding it in distributed shared memory), forced for every level,
    with and without the stopping test, gives the oracle's state bit for bit."""
    ctx = api.context()
    rng = np.random.default_rng(41)
    cubes = S.random_octree(rng, dmin=1, dmax=6, target=12000, shape="sphere")
    hists = S.random_histograms(rng, len(cubes), nbins=8, empty_frac=0.0)
    leaves = S.split_leaves(len(cubes), 5, rng, cubes, aligned=True)
    fixed, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 40, nthreads=8)
    stop, rst = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 300, tol=1e-3, check_every=10,
                                     nthreads=8)
    try:
        for cfg in range(25):
            ctx.set_schedule(mode, -1, cfg)
            out, st = api.tgv_solve(cubes, hists, leaves, mode, api.TGVParams(alpha0=2.0, alpha1=1.0, iters=40))
            want = 14 if (18 <= cfg <= 21 and mode == "oc") else cfg
            if cfg == 23:  # units above 2048 cubes run the single-block kernel without shared-memory state
                assert set(st["schedule"]) <= {22, 23} and 23 in st["schedule"], (cfg, mode)
            else:
                assert set(st["schedule"]) == {want}, (cfg, mode)
            assert_state_equal(out, fixed, f"schedule {cfg} {mode}")
            out, st = api.tgv_solve(cubes, hists, leaves, mode,
                                    api.TGVParams(alpha0=2.0, alpha1=1.0, iters=300, tol=1e-3, check_every=10))
            assert_state_equal(out, stop, f"schedule {cfg} {mode} stopping")
            assert st["iters_run"] == [r["iters_run"] for r in rst]
    finally:
        ctx.set_schedule(mode, -1, -1)


@pytest.mark.parametrize("mode", ["inmem", "oc", "stream"])
def test_tgv_graph_capture_and_replay(oracle_lib, mode):
    """With the schedule fixed, the second solve of a problem captures the
    whole level loop into one CUDA graph (graph = 1) and later solves relaunch
    it (graph = 2).  A tolerance-stopped solve: graphs off, first sighting,
    captured and replayed all give the oracle's state and per-level iteration
    counts bit for bit.  A fixed-count solve after resetting the schedule
    table: the first call autotunes with direct launches (graph = 0), the next
    is a first sighting, then capture and replay."""
    ctx = api.context()
    rng = np.random.default_rng(31)
    cubes = S.random_octree(rng, dmin=1, dmax=6, target=20000, shape="sphere")
    hists = S.random_histograms(rng, len(cubes), nbins=10, empty_frac=0.0)
    leaves = S.split_leaves(len(cubes), 7, rng, cubes, aligned=True)
    ref, rst = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 400, tol=1e-4, check_every=10,
                                    nthreads=8)
    prm = api.TGVParams(alpha0=2.0, alpha1=1.0, iters=400, tol=1e-4, check_every=10)
    try:
        runs = []
        for graphs in (False, True, True, True):
            ctx.set_graphs(graphs)
            runs.append(api.tgv_solve(cubes, hists, leaves, mode, prm))
        assert [st["graph"] for _, st in runs] == [0, 0, 1, 2]
        for out, st in runs:
            assert_state_equal(out, ref, f"graph {st['graph']} {mode}")
            assert st["iters_run"] == [r["iters_run"] for r in rst]
        assert runs[2][1]["kernel_launches"] == runs[3][1]["kernel_launches"] > 0

        ref, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 800, nthreads=8)
        ctx.set_schedule(mode, -1, -1)
        prm = api.TGVParams(alpha0=2.0, alpha1=1.0, iters=800)
        runs = [api.tgv_solve(cubes, hists, leaves, mode, prm) for _ in range(4)]
        assert [st["graph"] for _, st in runs] == [0, 0, 1, 2]
        for out, st in runs:
            assert_state_equal(out, ref, f"tuned graph {st['graph']} {mode}")
        assert runs[1][1]["schedule"] == runs[2][1]["schedule"] == runs[3][1]["schedule"]
    finally:
        ctx.set_graphs(True)


def test_tgv_unsorted_inmem_and_leaf_gaps(oracle_lib):
    """In-memory semantics need no ordering; leaves may leave cubes uncovered."""
    rng = np.random.default_rng(9)
    cubes = S.random_octree(rng, 2, 6, 4000)
    perm = rng.permutation(len(cubes))
    cu, h = cubes[perm], S.random_histograms(rng, len(cubes))
    ref, _ = oracle_lib.tgv_solve(cu, h, None, "inmem", 0.5, 0.5, 15)
    out, _ = api.tgv_solve(cu, h, None, "inmem", api.TGVParams(0.5, 0.5, 15))
    assert_state_equal(out, ref, "unsorted inmem")
    leaves = S.split_leaves(len(cubes), 4, rng, cubes)
    leaves = leaves[[0, 2, 3]]  # leaf 1's cubes are in no leaf
    leaves = leaves[::-1].copy()  # order given by the caller
    for mode in ("oc", "stream"):
        ref, _ = oracle_lib.tgv_solve(cubes, h, leaves, mode, 0.5, 0.5, 15)
        out, _ = api.tgv_solve(cubes, h, leaves, mode, api.TGVParams(0.5, 0.5, 15))
        assert_state_equal(out, ref, f"gaps {mode}")


def test_wavefront_schedules_at_scale():
    """The ordered-wavefront schedules (20: loads through L2, 21: through L1 as
    well) against band order (14, itself exact against the oracle) on a
    ray-cast torus workload of about 270 k cubes, where thousands of tiles and
    hundreds of blocks run concurrently: bit for bit in in-memory and streaming
    semantics, with and without the stopping test.  An unsorted cube order
    (dependencies pointing forwards) makes them fall back to band order."""
    from tgvreconclaude_gb300 import workloads as W
    ctx = api.context()
    w = W.build("torus16", seed=3)
    leaves = W.chunk_leaves(w.cubes, 8, np.random.default_rng(0))
    try:
        for mode, lv in (("inmem", None), ("stream", leaves)):
            for prm in (api.TGVParams(alpha0=2.0, alpha1=1.0, iters=30),
                        api.TGVParams(alpha0=2.0, alpha1=1.0, iters=200, tol=1e-3, check_every=10)):
                ctx.set_schedule(mode, -1, 14)
                ref, rst = api.tgv_solve(w.cubes, w.hists, lv, mode, prm)
                for cfg in (20, 21):
                    ctx.set_schedule(mode, -1, cfg)
                    out, st = api.tgv_solve(w.cubes, w.hists, lv, mode, prm)
                    assert set(st["schedule"]) == {cfg}
                    assert_state_equal(out, ref, f"wavefront {cfg} {mode} tol={prm.tol}")
                    assert st["iters_run"] == rst["iters_run"]
        perm = np.random.default_rng(1).permutation(len(w.cubes))
        ctx.set_schedule("inmem", -1, 20)
        out, st = api.tgv_solve(w.cubes[perm], w.hists[perm], None, "inmem", api.TGVParams(2.0, 1.0, 10))
        assert 14 in st["schedule"]
        ctx.set_schedule("inmem", -1, 14)
        ref, _ = api.tgv_solve(w.cubes[perm], w.hists[perm], None, "inmem", api.TGVParams(2.0, 1.0, 10))
        assert_state_equal(out, ref, "unsorted fallback")
    finally:
        for mode in ("inmem", "oc", "stream"):
            ctx.set_schedule(mode, -1, -1)


@pytest.mark.parametrize("mode", ["inmem", "oc"])
def test_level_energy_matches_oracle(oracle_lib, mode):
    """The FP64 per-level primal energy (tgvg_stats.energy) against the oracle's
    FP64 sum over the same bit-identical state: equal to 1e-12 relative (only
    the summation order differs)."""
    rng = np.random.default_rng(23)
    cubes = S.random_octree(rng, dmin=2, dmax=7, target=20000, shape="sphere")
    hists = S.random_histograms(rng, len(cubes), nbins=8, empty_frac=0.1)
    leaves = S.split_leaves(len(cubes), 6, rng, cubes, aligned=True)
    lv = None if mode == "inmem" else leaves
    ref, rst = oracle_lib.tgv_solve(cubes, hists, lv, mode, 2.0, 1.0, 40, nthreads=8)
    out, st = api.tgv_solve(cubes, hists, lv, mode, api.TGVParams(alpha0=2.0, alpha1=1.0, iters=40))
    assert_state_equal(out, ref, "energy case")
    want = [r["energy"] for r in rst]
    assert st["depth"] == [r["depth"] for r in rst]
    assert all(e > 0 for e in want)
    np.testing.assert_allclose(st["energy"], want, rtol=1e-12)


def test_tgv_stopping_rule(oracle_lib):
    """Per-level (per-leaf in OC and streaming) stop at relative residual <= tol.  A
    level that stops early has residual <= tol; the iteration counts and the
    final state agree with the oracle.  (Cubes without votes make the
    reference's iteration drift, so some levels may run to the cap.)"""
    rng = np.random.default_rng(4)
    cubes = S.random_octree(rng, 2, 6, 8000)
    h = S.random_histograms(rng, len(cubes), empty_frac=0.0)
    h[h.sum(1) == 0, 3] = 1
    leaves = S.split_leaves(len(cubes), 3, rng, cubes, aligned=True)
    for mode in ("inmem", "oc", "stream"):
        ref, rst = oracle_lib.tgv_solve(cubes, h, leaves, mode, 1.0, 2.0, 1500, tol=1e-4, check_every=10)
        out, st = api.tgv_solve(cubes, h, leaves, mode, api.TGVParams(1.0, 2.0, 1500, tol=1e-4, check_every=10))
        assert [r["iters_run"] for r in rst] == st["iters_run"], mode
        assert any(i < 1500 for i in st["iters_run"])
        assert all(r <= 1e-4 for r, i in zip(st["residual"], st["iters_run"]) if i < 1500)
        assert_state_equal(out, ref, f"stop {mode}")


@pytest.mark.parametrize("mode", ["inmem", "stream"])
def test_coarse_neighbour_ghosts(oracle_lib, mode):
    """Levels of at least 16,384 cubes copy the p/q values their -x/-y/-z
    coarser neighbours give into a compact table at the level's start, and the
    per-launch sweep schedules gather from it.  Every schedule that reads it
    (per-sweep launches in chunk and band order, two cubes per thread, L2
    prefetch, the L1 wavefront, the single block), fixed count and
    tolerance-stopped, must give the oracle's state bit for bit.  Some cubes
    have no votes and some vote totals are above 2^28."""
    ctx = api.context()
    rng = np.random.default_rng(77)
    cubes = S.random_octree(rng, dmin=3, dmax=8, target=150000, shape="sphere")
    depth = cubes["depth"]
    assert np.bincount(depth).max() >= 16384
    hists = S.random_histograms(rng, len(cubes), nbins=8, empty_frac=0.0)
    hists[::97, 2] = 300_000_000  # vote totals above 2^28
    hists[::89] = 0               # cubes without votes
    leaves = S.split_leaves(len(cubes), 4, rng, cubes, aligned=True)
    nb = oracle_lib.neighbour_table(cubes)
    big = np.bincount(depth).argmax()
    fine = np.where(depth == big)[0]
    minus = nb[fine][:, [1, 3, 5]]
    coarse = (minus >= 0) & (depth[np.maximum(minus, 0)] < big)
    assert coarse.mean() > 0.05  # the largest level has coarser neighbours to copy
    fixed, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 30, nthreads=8)
    stop, rst = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 200, tol=1e-3, check_every=10,
                                     nthreads=8)
    try:
        for cfg in (0, 8, 14, 15, 16, 21, 22):
            ctx.set_schedule(mode, -1, cfg)
            out, st = api.tgv_solve(cubes, hists, leaves, mode, api.TGVParams(alpha0=2.0, alpha1=1.0, iters=30))
            assert_state_equal(out, fixed, f"ghosts schedule {cfg} {mode}")
            out, st = api.tgv_solve(cubes, hists, leaves, mode,
                                    api.TGVParams(alpha0=2.0, alpha1=1.0, iters=200, tol=1e-3, check_every=10))
            assert_state_equal(out, stop, f"ghosts schedule {cfg} {mode} stopping")
            assert st["iters_run"] == [r["iters_run"] for r in rst]
    finally:
        ctx.set_schedule(mode, -1, -1)


def _refined_slab():
    """A 512 x 512 slab of depth-9 cubes (z cell 0) under a slab of depth-10
    cubes filling z cell 1: the depth-9 level (262,144 cubes) has a deeper
    neighbour across every +z face (the depth-10 octant-0 child shares the
    code), and the depth-10 level a coarser one across every -z face."""
    sh9, sh10 = F.MAX_DEPTH - 9, F.MAX_DEPTH - 10
    g9 = np.arange(512, dtype=np.uint64)
    X, Y = np.meshgrid(g9, g9, indexing="ij")
    k9 = F.morton_encode(X.ravel() << np.uint64(sh9), Y.ravel() << np.uint64(sh9), np.zeros(X.size, np.uint64))
    g10 = np.arange(1024, dtype=np.uint64)
    X, Y = np.meshgrid(g10, g10, indexing="ij")
    k10 = np.concatenate([F.morton_encode(X.ravel() << np.uint64(sh10), Y.ravel() << np.uint64(sh10),
                                          np.full(X.size, z << sh10, np.uint64)) for z in (2, 3)])
    keys = np.concatenate([k9, k10])
    depth = np.concatenate([np.full(len(k9), 9, np.int32), np.full(len(k10), 10, np.int32)])
    o = np.argsort(keys, kind="stable")
    return F.make_cubes(keys[o], depth[o], np.full(len(keys), 0.01, np.float32))


@pytest.mark.parametrize("mode", ["inmem", "stream"])
def test_dual_ghosts_on_a_refined_slab(oracle_lib, mode):
    """Levels of at least 262,144 cubes whose next level is at least twice as
    large also copy the bars of the dual sweep's +x/+y/+z neighbours on other
    levels into a compact table; per-launch schedules (and the schedules that
    share their loads) read them.  The state must equal the oracle's."""
    ctx = api.context()
    cubes = _refined_slab()
    rng = np.random.default_rng(17)
    hists = S.random_histograms(rng, len(cubes), nbins=8, empty_frac=0.05)
    leaves = S.split_leaves(len(cubes), 3, rng, cubes, aligned=True)
    ref, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 12, nthreads=8)
    try:
        for cfg in (0, 14, 16, 21):
            ctx.set_schedule(mode, -1, cfg)
            out, st = api.tgv_solve(cubes, hists, leaves, mode, api.TGVParams(alpha0=2.0, alpha1=1.0, iters=12))
            assert st["active"][:2] == [262144, 2097152]
            assert_state_equal(out, ref, f"dual ghosts schedule {cfg} {mode}")
    finally:
        ctx.set_schedule(mode, -1, -1)


def test_stream_leaves_stop_apart_within_a_level(oracle_lib):
    """Streaming semantics, per-launch schedules: within one level some leaves
    meet the tolerance while another runs to the cap (its cubes have no votes, so
    the reference iteration drifts), and on shallow levels some leaves have no
    cube at all.  The sweep kernels skip the per-cube stopping-flag reads until a
    leaf of the level has met the tolerance; states and iteration counts must
    still equal the oracle's on every level."""
    ctx = api.context()
    rng = np.random.default_rng(52)
    cubes = S.random_octree(rng, dmin=2, dmax=7, target=30000, shape="sphere")
    hists = S.random_histograms(rng, len(cubes), nbins=8, empty_frac=0.0)
    leaves = S.split_leaves(len(cubes), 6, rng, cubes, aligned=True)
    f, l = int(leaves["first_idx"][0]), int(leaves["last_idx"][0])
    hists[f:l + 1] = 0
    ref, rst = oracle_lib.tgv_solve(cubes, hists, leaves, "stream", 2.0, 1.0, 600, tol=1e-3, check_every=10,
                                    nthreads=8)
    its = [r["iters_run"] for r in rst]
    assert 600 in its and min(its) < 600
    try:
        for cfg in (0, 7, 8, 12, 14, 16, 18):
            ctx.set_schedule("stream", -1, cfg)
            out, st = api.tgv_solve(cubes, hists, leaves, "stream",
                                    api.TGVParams(alpha0=2.0, alpha1=1.0, iters=600, tol=1e-3, check_every=10))
            assert set(st["schedule"]) == {cfg}
            assert_state_equal(out, ref, f"schedule {cfg} leaves stopping apart")
            assert st["iters_run"] == its, cfg
    finally:
        ctx.set_schedule("stream", -1, -1)


@pytest.mark.parametrize("mode", ["inmem", "stream"])
def test_tgv_autotuned_stopping_solves(oracle_lib, mode):
    """Tolerance-stopped solves with a large iteration cap tune their untuned
    size classes online; levels that meet the tolerance during the trials end
    there.  States and per-level iteration counts equal the oracle's; a second
    solve reuses the tuned table."""
    ctx = api.context()
    rng = np.random.default_rng(88)
    cubes = S.random_octree(rng, dmin=1, dmax=7, target=60000, shape="sphere")
    hists = S.random_histograms(rng, len(cubes), nbins=8, empty_frac=0.0)
    leaves = S.split_leaves(len(cubes), 5, rng, cubes, aligned=True)
    ref, rst = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 2.0, 1.0, 3000, tol=2e-4, check_every=10,
                                    nthreads=8)
    ctx.set_schedule(mode, -1, -1)
    try:
        for _ in range(2):
            out, st = api.tgv_solve(cubes, hists, leaves, mode,
                                    api.TGVParams(2.0, 1.0, 3000, tol=2e-4, check_every=10))
            assert_state_equal(out, ref, f"tuned stopping {mode}")
            assert st["iters_run"] == [r["iters_run"] for r in rst]
    finally:
        ctx.set_schedule(mode, -1, -1)


def test_tgv_reference_kats():
    """tests/test_stage6.cpp:25-184 through the GPU API."""
    cubes = F.make_cubes([int(F.morton_encode(np.uint32(ix << 16), np.uint32(0), np.uint32(0))) for ix in range(3)],
                         5, 1.0)
    h = np.zeros((3, 8), np.uint32); h[0, 6] = 50; h[2, 1] = 50
    p = api.TGVParams(alpha0=0.1, alpha1=0.2, iters=50)
    s = api.tgv_minimize(cubes, h, None, 32.0, p)
    assert s["u"][0] > 0 > s["u"][2] and s["u"][2] < s["u"][1] < s["u"][0]
    one = np.zeros(1, F.LEAF_DTYPE); one["last_idx"] = 2
    two = np.zeros(2, F.LEAF_DTYPE); two["first_idx"] = [0, 2]; two["last_idx"] = [1, 2]
    assert np.abs(api.tgv_minimize_oc(cubes, h, one, None, 32.0, p)["u"] - s["u"]).max() <= 1e-5
    s2 = api.tgv_minimize_oc(cubes, h, two, None, 32.0, p)
    assert s2["u"][0] > 0 > s2["u"][2] and s2["u"][2] < s2["u"][1] < s2["u"][0]
    c4 = F.make_cubes([int(F.morton_encode(np.uint32(ix << 17), np.uint32(0), np.uint32(0))) for ix in range(4)], 4, 1.0)
    h4 = np.zeros((4, 8), np.uint32); h4[:, 6] = 10
    s4 = api.tgv_minimize(c4, h4, None, 16.0, api.TGVParams(iters=20))
    assert np.all(np.abs(s4["u"] - 0.625) <= 0.15)
    assert len(api.tgv_minimize_oc(np.zeros(0, F.CUBE_DTYPE), np.zeros((0, 8), np.uint32),
                                   np.zeros(0, F.LEAF_DTYPE), None, 1.0)) == 0


def test_tgv_streaming_files(tmp_path):
    """tgv_minimize_streaming: TGV1/TGVH/TGVT in, TGVS out (test_stage6.cpp:242-344)."""
    g = load_golden("tgv_balanced.npz")
    cp, hp, tp, sp = (tmp_path / x for x in ("c", "h", "t", "s"))
    F.save_cubes(cp, g["cubes"], 1.5)
    F.save_histograms(hp, g["hists"])
    F.save_treetop(tp, g["leaves"], 1.5)
    a0, a1 = (float(x) for x in g["params"])
    api.tgv_minimize_streaming(cp, hp, tp, None, 1.5, sp, api.TGVParams(a0, a1, int(g["iters"])))
    assert_state_equal(F.load_state(sp), g["stream"], "streaming files")
    F.save_cubes(cp, np.zeros(0, F.CUBE_DTYPE), 1.5)
    api.tgv_minimize_streaming(cp, hp, tp, None, 1.5, sp)
    assert len(F.load_state(sp)) == 0


def test_tgv_errors(tmp_path):
    rng = np.random.default_rng(1)
    cubes = S.random_octree(rng, 2, 5, 500)
    h = S.random_histograms(rng, len(cubes))
    lv = S.split_leaves(len(cubes), 2, rng, cubes)
    with pytest.raises(RuntimeError, match="sorted"):
        api.tgv_solve(cubes[::-1].copy(), h, lv, "stream")
    bad = lv.copy(); bad["last_idx"][0] = bad["first_idx"][1] + 3
    with pytest.raises(RuntimeError, match="overlap"):
        api.tgv_solve(cubes, h, bad, "oc")
    dbad = cubes.copy(); dbad["depth"][3] = 22
    with pytest.raises(RuntimeError, match="invalid"):
        api.tgv_solve(dbad, h, None, "inmem")
    (tmp_path / "x").write_bytes(b"XXXX" + bytes(20))
    with pytest.raises(RuntimeError, match="magic"):
        api.tgv_minimize_streaming(tmp_path / "x", tmp_path / "x", tmp_path / "x", None, 1.0, tmp_path / "o")


def test_constant_field_is_a_fixed_point():
    """Size-independent property: identical histograms everywhere -> u stays at
    the common median exactly and v, p, q stay 0, at any size."""
    rng = np.random.default_rng(3)
    cubes = S.random_octree(rng, 3, 7, 400000)
    h = np.zeros((len(cubes), 8), np.uint32); h[:, 5] = 7
    out, st = api.tgv_solve(cubes, h, None, "inmem", api.TGVParams(1.0, 2.0, 30))
    assert np.all(out["u"] == np.float32(0.375)) and not out["v"].any() and not out["p"].any() and not out["q"].any()


@pytest.mark.parametrize("case", TGV_CASES)
def test_tgv_error_against_fp64(case, oracle_lib):
    """The FP32 result (bit-identical to the reference) against an FP64 run of
    the same solver on the same inputs: max |du| <= 1e-4 after the same
    iteration count."""
    g = load_golden(case)
    a0, a1 = (float(x) for x in g["params"])
    for mode in ("inmem", "stream"):
        out, _ = api.tgv_solve(g["cubes"], g["hists"], g["leaves"], mode,
                               api.TGVParams(alpha0=a0, alpha1=a1, iters=int(g["iters"])))
        ref64, _ = oracle_lib.tgv_solve(g["cubes"], g["hists"], g["leaves"], mode, a0, a1, int(g["iters"]), fp64=True)
        du = np.abs(out["u"].astype(np.float64) - ref64[:, 0]).max()
        print(case, mode, "max|du| vs FP64", du)
        assert du <= 1e-4, (case, mode, du)
