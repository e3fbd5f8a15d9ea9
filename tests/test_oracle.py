"""The oracle (oracle/tgv_oracle.cpp) against the reference's own outputs.

CPU only.  Pins the restatement bit for bit: against the committed golden
fixtures (made by the unmodified reference, tests/golden/make_golden.py) and,
where the reference checkout exists, against the reference compiled here on
fresh seeded inputs.  Also restates the reference's own known-answer tests
(tests/test_stage5.cpp, tests/test_stage6.cpp) against the oracle.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_maps, load_golden
from tgvreconclaude_gb300 import formats as F, scenes as S

TGV_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "tgv_*.npz")))
HIST_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "hist_*.npz")))


@pytest.mark.parametrize("case", TGV_CASES)
@pytest.mark.parametrize("mode", ["inmem", "oc", "stream"])
def test_oracle_tgv_matches_golden(oracle_lib, case, mode):
    g = load_golden(case)
    a0, a1 = (float(x) for x in g["params"])
    out, _ = oracle_lib.tgv_solve(g["cubes"], g["hists"], g["leaves"], mode, a0, a1, int(g["iters"]))
    assert out.tobytes() == g[mode].tobytes()


@pytest.mark.parametrize("case", HIST_CASES)
def test_oracle_histograms_match_golden(oracle_lib, case):
    g = load_golden(case)
    bins = oracle_lib.compute_histograms(g["cubes"], golden_maps(g), g["origin"], float(g["r_root"]))
    assert np.array_equal(bins, g["bins"])


def test_level_thresholds_exhaustive(oracle_lib):
    """The product's pyramid-level thresholds give (int)log2f(x) for every float
    x in [1, 2^14) (and at the top of the range) on this host."""
    import ctypes as C
    from tgvreconclaude_gb300 import _native as N
    t = (C.c_float * 13)()
    N.lib().tgvg_level_thresholds(t)
    arr = np.array(t[:], np.float32)
    assert arr[0] == 1.0 and np.all(np.diff(arr) > 0)
    assert arr[1] <= 2.0 and arr[12] <= 4096.0
    oracle_lib.lib().orc_check_thresholds.restype = C.c_int64
    assert oracle_lib.lib().orc_check_thresholds(t) == 0


# --------------------------------------------------------- live reference ---

needs_ref = pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference checkout absent")


@needs_ref
@pytest.mark.parametrize("seed", range(4))
def test_oracle_tgv_matches_reference(oracle_lib, seed):
    rng = np.random.default_rng(1000 + seed)
    cubes = S.random_octree(rng, dmin=1 + seed % 3, dmax=4 + seed % 3, target=900,
                            shape=["sphere", "plane", "random"][seed % 3])
    hists = S.random_histograms(rng, len(cubes))
    leaves = S.split_leaves(len(cubes), 2 + seed, rng, cubes, aligned=bool(seed % 2))
    for mode in ("inmem", "oc", "stream"):
        ref = oracle_lib.ref_tgv(cubes, hists, leaves, mode, 0.05 * (seed + 1), 0.1 * (seed + 1), 12)
        out, _ = oracle_lib.tgv_solve(cubes, hists, leaves, mode, 0.05 * (seed + 1), 0.1 * (seed + 1), 12)
        assert out.tobytes() == ref.tobytes(), mode


@needs_ref
def test_oracle_histograms_and_pyramids_match_reference(oracle_lib):
    rng = np.random.default_rng(7)
    rig = S.sphere_rig(4, 3.0, width=50, height=37)  # odd sizes exercise the pyramid edges
    maps = []
    for i, c in enumerate(rig):
        d = S.render_depth(S.torus_scene(0.01), c, seed=i).numpy()
        d[::7, ::5] = np.nan
        d[3, :] = -1.0
        m = dict(depth=d, rt=c["rt"], fx=c["fx"], fy=c["fy"], cx=c["cx"], cy=c["cy"], lidar=i == 1)
        m["rt_inv"], tex, dims = oracle_lib.ref_mipmap(m)
        otex, odims = oracle_lib.pyramid(d)
        assert dims == odims
        assert tex.view(np.uint32).tobytes() == otex.view(np.uint32).tobytes()
        maps.append(m)
    cubes = S.random_octree(rng, dmin=2, dmax=8, target=3000, r_root=1.5)
    for nb in (8,):
        ref = oracle_lib.ref_compute_histograms(cubes, maps, (-1.5, -1.5, -1.5), 1.5)
        out = oracle_lib.compute_histograms(cubes, maps, (-1.5, -1.5, -1.5), 1.5, nbins=nb)
        assert np.array_equal(ref, out)


@needs_ref
def test_morton_helpers_match_reference(oracle_lib):
    import ctypes as C
    rng = np.random.default_rng(3)
    r = oracle_lib.ref()
    for _ in range(300):
        d = int(rng.integers(1, 22))
        x, y, z = (int(v) << (21 - d) for v in rng.integers(0, 1 << d, 3))
        k = int(F.morton_encode(np.uint32(x), np.uint32(y), np.uint32(z)))
        hi, lo = k >> 32, k & 0xffffffff
        oh, ol = C.c_uint32(), C.c_uint32()
        r.ref_parent_code(C.c_uint32(hi), C.c_uint32(lo), d, C.byref(oh), C.byref(ol))
        assert (oh.value << 32 | ol.value) == int(F.ancestor_key(np.uint64(k), d - 1))
        for f in range(6):
            r.ref_face_neighbor(C.c_uint32(hi), C.c_uint32(lo), f, d, C.byref(oh), C.byref(ol))
            step = 1 << (21 - d)
            c = [x, y, z]
            ax, sgn = f // 2, 1 if f % 2 == 0 else -1
            c[ax] += sgn * step
            if c[ax] < 0 or c[ax] >= 1 << 21:
                assert (oh.value, ol.value) == (0xffffffff, 0xffffffff)
            else:
                kk = int(F.morton_encode(np.uint32(c[0]), np.uint32(c[1]), np.uint32(c[2])))
                assert (oh.value << 32 | ol.value) == kk


# ------------------------------------- the reference's known-answer tests ---

def _chain(r_root=32.0):
    cubes = F.make_cubes([int(F.morton_encode(np.uint32(ix << 16), np.uint32(0), np.uint32(0))) for ix in range(3)],
                         5, r_root / 32)
    h = np.zeros((3, 8), np.uint32)
    h[0, 6] = 50
    h[2, 1] = 50
    return cubes, h


def test_kat_stage6_smoothing_and_chunks(oracle_lib):
    """tests/test_stage6.cpp:25-66, 133-175, 242-310: polarity and B between A and C."""
    cubes, h = _chain()
    one = np.zeros(1, F.LEAF_DTYPE); one["last_idx"] = 2
    two = np.zeros(2, F.LEAF_DTYPE); two["last_idx"] = [1, 2]; two["first_idx"] = [0, 2]
    s1, _ = oracle_lib.tgv_solve(cubes, h, None, "inmem", 0.1, 0.2, 50)
    for st in (s1,) + tuple(oracle_lib.tgv_solve(cubes, h, lv, m, 0.1, 0.2, 50)[0]
                            for m in ("oc", "stream") for lv in (one, two)):
        assert st["u"][0] > 0 and st["u"][2] < 0 and st["u"][2] < st["u"][1] < st["u"][0]
    so, _ = oracle_lib.tgv_solve(cubes, h, one, "oc", 0.1, 0.2, 50)
    ss, _ = oracle_lib.tgv_solve(cubes, h, one, "stream", 0.1, 0.2, 50)
    assert np.abs(so["u"] - s1["u"]).max() <= 1e-5
    assert np.abs(ss["u"] - s1["u"]).max() <= 1e-4


def test_kat_stage6_constant_and_empty(oracle_lib):
    """tests/test_stage6.cpp:68-94 and 178-184."""
    cubes = F.make_cubes([int(F.morton_encode(np.uint32(ix << 17), np.uint32(0), np.uint32(0))) for ix in range(4)],
                         4, 1.0)
    h = np.zeros((4, 8), np.uint32); h[:, 6] = 10
    st, _ = oracle_lib.tgv_solve(cubes, h, None, "inmem", 0.02, 0.04, 20)
    assert np.all(np.abs(st["u"] - 0.625) <= 0.15)
    e, _ = oracle_lib.tgv_solve(np.zeros(0, F.CUBE_DTYPE), np.zeros((0, 8), np.uint32), np.zeros(0, F.LEAF_DTYPE), "oc")
    assert len(e) == 0


def test_kat_stage5_stats_and_pyramid(oracle_lib):
    """tests/test_stage5.cpp:21-41 and 84-101."""
    b = np.zeros(8, np.uint32); b[4] = 10
    assert abs(oracle_lib.median_indicator(b) - 0.125) < 0.01 and abs(oracle_lib.mean_indicator(b) - 0.125) < 0.01
    b = np.zeros(8, np.uint32); b[3] = 5; b[4] = 5
    assert abs(oracle_lib.median_indicator(b) + 0.125) < 0.01
    z = np.zeros(8, np.uint32)
    assert oracle_lib.median_indicator(z) == 0.0 and oracle_lib.mean_indicator(z) == 0.0
    tex, dims = oracle_lib.pyramid(np.full((8, 8), 10.0, np.float32))
    assert len(dims) >= 4 and [d[0] for d in dims[:3]] == [8, 4, 2]
    assert np.all(tex == 10.0)


def test_kat_stage5_project_and_plane(oracle_lib):
    """tests/test_stage5.cpp:45-80 and 105-146 (identity camera at the origin)."""
    m = dict(depth=np.full((32, 32), 5.0, np.float32), rt_inv=np.eye(4, dtype=np.float32), fx=100.0, fy=100.0,
             cx=16.0, cy=16.0)
    ok, lv, u, v, z = oracle_lib.project(m, (0.0, 0.0, 5.0), 0.04)
    assert ok and abs(z - 5.0) <= 1e-4 and lv == 0
    assert not oracle_lib.project(m, (0.0, 0.0, -1.0), 0.1)[0]
    assert not oracle_lib.project(m, (1000.0, 0.0, 5.0), 0.1)[0]
    ok, lv, *_ = oracle_lib.project(m, (0.0, 0.0, 1.0), 2.0)
    assert ok and lv >= 1
    plane = dict(depth=np.full((16, 16), 5.0, np.float32), rt_inv=np.eye(4, dtype=np.float32), fx=50.0, fy=50.0,
                 cx=8.0, cy=8.0)
    c = F.make_cubes([int(F.morton_encode(np.uint32(4 << 17), np.uint32(4 << 17), np.uint32(8 << 17)))], 4, 1 / 16)
    h = oracle_lib.compute_histograms(c, [plane], (-0.5, -0.5, 4.0), 1.0)
    assert h.sum() > 0 and h[0, :4].sum() > h[0, 4:].sum()


# ---- whole-state warm start (level_init): an extension with no counterpart in the
# reference, pinned here to the reference's own level start (tgv.cpp:391-409).

def _level_start_records(cubes, hists, final):
    """The state each cube has when its level starts in the plain solve:
    u and v of the cube that the parent-code lookup returns (the largest index
    with that code; its state is final when it is coarser, initial otherwise),
    p = q = 0; the cube's own initial state where no such cube exists or on the
    coarsest level."""
    keys = F.cube_keys(cubes).astype(np.uint64)
    d = cubes["depth"].astype(np.int64)
    init = np.zeros(len(cubes), F.STATE_DTYPE)
    import oracle
    init["u"] = oracle.stream_init(cubes, hists)["u"]
    last = {}
    for i, k in enumerate(keys.tolist()):
        last[k] = i
    rec = init.copy()
    dmin = int(d.min())
    for i in range(len(cubes)):
        L = int(d[i])
        if L == dmin:
            continue
        sh = 3 * (21 - (L - 1))
        pk = int(keys[i]) >> sh << sh
        j = last.get(pk, -1)
        if j < 0:
            continue
        src = final[j] if d[j] < L else init[j]
        rec["u"][i] = src["u"]
        rec["v"][i] = src["v"]
    return rec


@pytest.mark.parametrize("seed", range(3))
def test_level_init_reproduces_the_reference_level_start(oracle_lib, seed):
    """Seeding every level with the records the reference's parent copy would
    produce gives the plain solve bit for bit, in in-memory semantics."""
    rng = np.random.default_rng(70 + seed)
    cubes = S.random_octree(rng, dmin=1 + seed, dmax=4 + seed, target=2500, shape=["sphere", "plane", "random"][seed])
    hists = S.random_histograms(rng, len(cubes), nbins=8 if seed % 2 == 0 else 10)
    plain, pst = oracle_lib.tgv_solve(cubes, hists, None, "inmem", 2.0, 1.0, 25)
    rec = _level_start_records(cubes, hists, plain)
    out, ost = oracle_lib.tgv_solve(cubes, hists, None, "inmem", 2.0, 1.0, 25, level_init=rec)
    assert out.tobytes() == plain.tobytes()
    assert [s["iters_run"] for s in ost] == [s["iters_run"] for s in pst]


def test_level_init_zero_records_on_one_level(oracle_lib):
    """All-zero records on a one-level octree are the zero initialisation."""
    rng = np.random.default_rng(3)
    cubes = S.random_octree(rng, dmin=4, dmax=4, target=1500)
    hists = S.random_histograms(rng, len(cubes))
    z = np.zeros(len(cubes), F.STATE_DTYPE)
    a, _ = oracle_lib.tgv_solve(cubes, hists, None, "inmem", 2.0, 1.0, 30, init="zero")
    b, _ = oracle_lib.tgv_solve(cubes, hists, None, "inmem", 2.0, 1.0, 30, level_init=z)
    assert a.tobytes() == b.tobytes()


def test_neighbour_table_on_a_uniform_grid(oracle_lib):
    """Every cell of a full 4^3 grid at depth 2 has its face-adjacent cells as
    neighbours and -1 across the domain boundary."""
    g = np.arange(4, dtype=np.uint32)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    sh = F.MAX_DEPTH - 2
    k = F.morton_encode(X.ravel() << sh, Y.ravel() << sh, Z.ravel() << sh)
    o = np.argsort(k)
    cubes = F.make_cubes(k[o], np.full(len(k), 2, np.int32), np.full(len(k), 0.25, np.float32))
    nb = oracle_lib.neighbour_table(cubes)
    xyz = np.stack([X.ravel()[o], Y.ravel()[o], Z.ravel()[o]], 1)
    pos = {tuple(p): i for i, p in enumerate(xyz.tolist())}
    for i, p in enumerate(xyz.tolist()):
        for f in range(6):
            q = list(p)
            q[f // 2] += 1 if f % 2 == 0 else -1
            assert nb[i, f] == pos.get(tuple(q), -1)


def test_coarser_neighbours_are_shared_within_sibling_runs(oracle_lib):
    """The ghost tables of the primal sweep store one entry per (coarser
    neighbour, face) and sibling run: a cube looks for an earlier cube with the
    same neighbour value among the previous 7 positions with the same parent.
    The cubes of a level that reach one coarser cube across a face are the
    children of at most two parents: the coarse cube's neighbour, and the coarse
    cube itself where the octree keeps a cube together with cubes inside it (the
    reference's parent-code lookup, tgv.cpp:97-109).  So each (neighbour, face)
    has at most two entries, and the dedup is complete within each run if a run
    spans at most 8 positions.  Checked on the reference-balanced octrees of the
    fixtures and on random octrees, in the solver's level-major order."""
    g = np.load(os.path.join(GOLDEN, "octree_cases.npz"))
    cases = [g[f"bal_out{k}"] for k in (0, 1, 2, 4)]
    for seed, shape in ((5, "sphere"), (6, "plane"), (7, "random")):
        cases.append(S.random_octree(np.random.default_rng(seed), dmin=2, dmax=7, target=40000, shape=shape))
    for cubes in cases:
        cubes = cubes[np.argsort(F.cube_keys(cubes), kind="stable")]
        nb = oracle_lib.neighbour_table(cubes)
        d = cubes["depth"].astype(np.int64)
        keys = F.cube_keys(cubes).astype(np.uint64)
        pos = np.empty(len(cubes), np.int64)
        pos[np.lexsort((np.arange(len(cubes)), d))] = np.arange(len(cubes))
        parent = (keys >> (np.uint64(3) * (np.uint64(F.MAX_DEPTH) - (d - 1).astype(np.uint64)))).astype(np.int64)
        checked = 0
        for f in (1, 3, 5):
            j = nb[:, f].astype(np.int64)
            idx = np.nonzero((j >= 0) & (d[np.maximum(j, 0)] < d))[0]
            if len(idx) == 0:
                continue
            _, run = np.unique(np.stack([j[idx], d[idx], parent[idx]], 1), axis=0, return_inverse=True)
            run = run.ravel()
            lo = np.full(run.max() + 1, np.iinfo(np.int64).max)
            hi = np.full(run.max() + 1, np.iinfo(np.int64).min)
            np.minimum.at(lo, run, pos[idx])
            np.maximum.at(hi, run, pos[idx])
            assert (hi - lo).max() <= 7
            _, grp = np.unique(np.stack([j[idx], d[idx]], 1), axis=0, return_inverse=True)
            pairs = np.unique(np.stack([grp.ravel(), run], 1), axis=0)
            assert np.bincount(pairs[:, 0]).max() <= 2
            checked += len(idx)
        assert checked > 500
