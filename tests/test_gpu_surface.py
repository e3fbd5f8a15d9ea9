"""Surface extraction on the GPU (tgvg_extract_surface*, tgvg_compute_normals,
tgvg_write_obj) against the oracle and the reference's mesh fixtures: vertices,
faces and normals bit for bit, .obj text byte for byte."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from test_surface_oracle import assert_mesh_equal, random_surface_case
from tgvreconclaude_gb300 import api, formats as F, scenes as S

pytestmark = pytest.mark.gpu
MESH_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "mesh_*.npz")))


@pytest.mark.parametrize("case", MESH_CASES)
def test_surface_matches_golden(case, tmp_path, oracle_lib):
    g = load_golden(case)
    o, r = g["origin"], float(g["r_root"])
    out = api.extract_surface(g["cubes"], g["state"], o, r, has_data=g["has_data"], normals=True)
    assert_mesh_equal(out, (g["verts"], g["faces"], g["normals"]), case)
    v, f = api.extract_surface_leaves(g["cubes"], g["state"], g["hists"], g["leaves"], o, r)
    assert oracle_lib.obj_text(v, f) == str(g["s_obj"])
    # files in, .obj out (the reference's extract_surface_streaming entry point)
    cp, sp, tp, hp, op = (tmp_path / x for x in ("c.bin", "s.bin", "t.bin", "h.bin", "m.obj"))
    F.save_cubes(cp, g["cubes"], r)
    F.save_state(sp, g["state"])
    F.save_treetop(tp, g["leaves"], r)
    F.save_histograms(hp, g["hists"])
    api.extract_surface_streaming(cp, sp, tp, hp, o, r, op)
    assert op.read_text() == str(g["s_obj"])
    # write_obj with normals, as the reference formats it
    api.write_obj(tmp_path / "n.obj", *out)
    assert (tmp_path / "n.obj").read_text() == oracle_lib.obj_text(*out)


@pytest.mark.parametrize("seed", range(6))
def test_surface_random_vs_oracle(seed, oracle_lib):
    cubes, state, hists, leaves, origin, r_root = random_surface_case(seed, n=6000 + 3000 * seed)
    has = (hists.sum(1) > 0).astype(np.uint8)
    for hd in (None, has):
        ref = oracle_lib.extract_surface(cubes, state, origin, r_root, has_data=hd, normals=True)
        out = api.extract_surface(cubes, state, origin, r_root, has_data=hd, normals=True)
        assert len(ref[1]) > 0
        assert_mesh_equal(out, ref, f"seed {seed}")
    if seed % 2:
        leaves = leaves[::-1].copy()
    rv, rf = oracle_lib.extract_surface_streaming(cubes, state, hists, leaves, origin, r_root)
    v, f = api.extract_surface_leaves(cubes, state, hists, leaves, origin, r_root)
    assert v.tobytes() == rv.tobytes() and f.tobytes() == rf.tobytes()
    n = api.compute_normals(ref[0], ref[1])
    assert n.tobytes() == ref[2].tobytes()


def test_surface_of_a_solved_scene(oracle_lib):
    """A ray-cast torus, its histograms and a GPU TGV solve: the iso-surface
    of the solved u, GPU against oracle."""
    rng = np.random.default_rng(3)
    cubes = S.random_octree(rng, dmin=3, dmax=7, target=60000, shape="sphere", r_root=1.5)
    hists = S.random_histograms(rng, len(cubes), nbins=10, empty_frac=0.1)
    state, _ = api.tgv_solve(cubes, hists, None, "inmem", api.TGVParams(alpha0=2.0, alpha1=1.0, iters=50))
    origin = np.float32([-1.5, -1.5, -1.5])
    has = (hists.sum(1) > 0).astype(np.uint8)
    ref = oracle_lib.extract_surface(cubes, state, origin, 1.5, has_data=has, normals=True)
    out = api.extract_surface(cubes, state, origin, 1.5, has_data=has, normals=True)
    assert len(ref[1]) > 100
    assert_mesh_equal(out, ref, "solved")


def test_surface_edge_cases(tmp_path):
    o = np.zeros(3, np.float32)
    v, f, n = api.extract_surface(np.zeros(0, F.CUBE_DTYPE), np.zeros(0, F.STATE_DTYPE), o, 1.0, normals=True)
    assert v.shape == (0, 3) and f.shape == (0, 3)
    cubes, state, hists, leaves, origin, r_root = random_surface_case(1)
    state["u"] = 1.0  # no sign change anywhere
    v, f, _ = api.extract_surface(cubes, state, origin, r_root)
    assert len(v) == 0 and len(f) == 0
    bad = cubes.copy()
    bad["depth"][5] = 22
    with pytest.raises(RuntimeError, match="invalid"):
        api.extract_surface(bad, state, origin, r_root)
    lv = leaves.copy()
    if len(lv) >= 2:
        lv["last_idx"][0] = lv["last_idx"][1]
        with pytest.raises(RuntimeError, match="overlap"):
            api.extract_surface_leaves(cubes, state, hists, lv, origin, r_root)
    with pytest.raises(RuntimeError):
        api.extract_surface_streaming(tmp_path / "missing.bin", tmp_path / "s", tmp_path / "t", tmp_path / "h",
                                      origin, r_root, tmp_path / "m.obj")


def _grid(nx, ny, nz, depth, u_of, r_root):
    """Cubes of one depth in x-fastest loop order (as the reference's tests
    build them, not Morton-sorted), with u from u_of(ix, iy, iz)."""
    sh = 21 - depth
    cubes, us = [], []
    for iz in range(nz):
        for iy in range(ny):
            for ix in range(nx):
                k = int(F.morton_encode(np.uint64(ix << sh), np.uint64(iy << sh), np.uint64(iz << sh)))
                cubes.append((k >> 32, k & 0xffffffff, r_root / (1 << depth), depth))
                us.append(u_of(ix, iy, iz))
    c = np.array(cubes, F.CUBE_DTYPE)
    st = np.zeros(len(c), F.STATE_DTYPE)
    st["u"] = us
    return c, st


def _edges(faces):
    cnt = {}
    for tri in np.asarray(faces, np.int64):
        for e in range(3):
            a, b = sorted((int(tri[e]), int(tri[(e + 1) % 3])))
            cnt[(a, b)] = cnt.get((a, b), 0) + 1
    vals = list(cnt.values())
    return vals.count(1), vals.count(2), sum(v > 2 for v in vals)


def test_surface_reference_kats(tmp_path):
    """tests/test_stage7.cpp:113-273 and 405-560 through the GPU API."""
    z = np.zeros(3, np.float32)
    # all u > 0: empty (:113-131)
    c, st = _grid(2, 2, 2, 3, lambda *a: 1.0, 8.0)
    assert len(api.extract_surface(c, st, z, 8.0)[1]) == 0
    # A(+) B(-) C(+) in a row: two quads, 8 boundary and 2 interior edges (:185-210)
    c, st = _grid(3, 1, 1, 3, lambda ix, iy, iz: [1.0, -1.0, 1.0][ix], 8.0)
    v, f, _ = api.extract_surface(c, st, z, 8.0)
    assert _edges(f) == (8, 2, 0)
    # a face across two cubes needs both (:215-241)
    c, st = _grid(2, 1, 1, 4, lambda ix, iy, iz: [1.0, -1.0][ix], 16.0)
    assert len(api.extract_surface(c, st, z, 16.0)[1]) > 0
    assert len(api.extract_surface(c[:1], st[:1], z, 16.0)[1]) == 0
    assert len(api.extract_surface(c[1:], st[1:], z, 16.0)[1]) == 0
    # the solid centre of a 3x3x3 grid: a closed box of 12 triangles (:245-273)
    c, st = _grid(3, 3, 3, 3, lambda ix, iy, iz: -1.0 if (ix, iy, iz) == (1, 1, 1) else 1.0, 24.0)
    v, f, _ = api.extract_surface(c, st, z, 24.0)
    assert len(f) == 12 and _edges(f)[0] == 0 and _edges(f)[2] == 0
    # streaming: the same box from files, one leaf (:405-460)
    h = np.zeros((len(c), 8), np.uint32)
    h[:, 0] = 1
    lv = np.zeros(1, F.LEAF_DTYPE)
    lv["hi"], lv["lo"], lv["first_idx"], lv["last_idx"] = c["hi"][0], c["lo"][0], 0, len(c) - 1
    paths = [tmp_path / x for x in ("c.bin", "s.bin", "t.bin", "h.bin", "m.obj")]
    F.save_cubes(paths[0], c, 24.0)
    F.save_state(paths[1], st)
    F.save_treetop(paths[2], lv, 24.0)
    F.save_histograms(paths[3], h)
    api.extract_surface_streaming(*paths[:4], z, 24.0, paths[4])
    lines = paths[4].read_text().splitlines()
    sf = np.array([[int(x) - 1 for x in ln.split()[1:]] for ln in lines if ln.startswith("f ")])
    assert len(sf) == 12 and _edges(sf)[0] == 0 and _edges(sf)[2] == 0
    # streaming: a face between two one-cube leaves is emitted once (:462-510)
    c, st = _grid(2, 1, 1, 4, lambda ix, iy, iz: [1.0, -1.0][ix], 16.0)
    h = np.zeros((2, 8), np.uint32)
    h[:, 0] = 1
    lv = np.zeros(2, F.LEAF_DTYPE)
    lv["first_idx"], lv["last_idx"], lv["depth"] = [0, 1], [0, 1], 4
    v, f = api.extract_surface_leaves(c, st, h, lv, z, 16.0)
    assert len(f) == 2 and len(v) == 4
    # streaming with one leaf matches the in-memory extraction with has_data (:513-560)
    c, st = _grid(2, 2, 2, 4, lambda ix, iy, iz: 1.0 if ix == 0 else -1.0, 16.0)
    h = np.zeros((len(c), 8), np.uint32)
    h[:, 0] = 1
    lv = np.zeros(1, F.LEAF_DTYPE)
    lv["last_idx"] = len(c) - 1
    sv, sf = api.extract_surface_leaves(c, st, h, lv, z, 16.0)
    rv, rf, _ = api.extract_surface(c, st, z, 16.0, has_data=np.ones(len(c), np.uint8))
    assert len(sf) == len(rf) and len(sv) == len(rv)


def test_surface_unsorted_streaming_vs_oracle(oracle_lib):
    cubes, state, hists, leaves, origin, r_root = random_surface_case(14)
    perm = np.random.default_rng(4).permutation(len(cubes))
    cubes, state, hists = cubes[perm], state[perm], hists[perm]
    rv, rf = oracle_lib.extract_surface_streaming(cubes, state, hists, leaves, origin, r_root)
    v, f = api.extract_surface_leaves(cubes, state, hists, leaves, origin, r_root)
    assert len(rf) > 0 and v.tobytes() == rv.tobytes() and f.tobytes() == rf.tobytes()
