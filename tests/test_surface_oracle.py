"""The surface-extraction oracle (oracle/tgv_oracle.cpp, extract_surface and
extract_surface_streaming) against the reference's own src/marching_cubes.cpp
compiled here, and against the committed mesh fixtures.

CPU only.  Vertices, faces and normals are compared bit for bit; the streaming
variant is compared through the .obj text the reference writes.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from tgvreconclaude_gb300 import formats as F, scenes as S

MESH_CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "mesh_*.npz")))


def needs_ref(f):
    import oracle
    return pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout absent")(f)


def random_surface_case(seed, n=3000):
    rng = np.random.default_rng(seed)
    cubes = S.random_octree(rng, dmin=2 + seed % 2, dmax=5 + seed % 3, target=n,
                            shape=["sphere", "plane", "random"][seed % 3])
    state = np.zeros(len(cubes), F.STATE_DTYPE)
    state["u"] = rng.uniform(-1, 1, len(cubes)).astype(np.float32)
    state["u"][rng.random(len(cubes)) < 0.05] = 0.0          # the u >= 0 side of the sign test
    state["u"][rng.random(len(cubes)) < 0.02] = -0.0
    hists = S.random_histograms(rng, len(cubes), empty_frac=0.15)
    leaves = S.split_leaves(len(cubes), 1 + seed % 5, rng, cubes, aligned=seed % 2 == 0)
    origin = rng.uniform(-2, 0, 3).astype(np.float32)
    r_root = float(rng.uniform(0.7, 3.0))
    return cubes, state, hists, leaves, origin, r_root


def assert_mesh_equal(a, b, what):
    for x, y, name in zip(a, b, ("verts", "faces", "normals")):
        if x is None and y is None:
            continue
        assert x.shape == y.shape, (what, name, x.shape, y.shape)
        assert x.tobytes() == y.tobytes(), (what, name)


@needs_ref
@pytest.mark.parametrize("seed", range(6))
def test_extract_surface_matches_reference(oracle_lib, seed):
    cubes, state, hists, _, origin, r_root = random_surface_case(seed)
    has = (hists.sum(1) > 0).astype(np.uint8)
    for hd in (None, has):
        ref = oracle_lib.ref_extract_surface(cubes, state, origin, r_root, has_data=hd, normals=True)
        out = oracle_lib.extract_surface(cubes, state, origin, r_root, has_data=hd, normals=True)
        assert len(ref[1]) > 0
        assert_mesh_equal(out, ref, f"seed {seed} has_data {hd is not None}")


@needs_ref
@pytest.mark.parametrize("seed", range(5))
def test_extract_surface_streaming_matches_reference(oracle_lib, tmp_path, seed):
    cubes, state, hists, leaves, origin, r_root = random_surface_case(10 + seed)
    if seed == 3:
        leaves = leaves[::-1].copy()  # treetop order is the caller's
    if seed == 4:  # an unsorted cube file (the reference's own tests write such files)
        perm = np.random.default_rng(seed).permutation(len(cubes))
        cubes, state, hists = cubes[perm], state[perm], hists[perm]
    cp, sp, tp, hp, op = (tmp_path / x for x in ("c.bin", "s.bin", "t.bin", "h.bin", "m.obj"))
    F.save_cubes(cp, cubes, r_root)
    F.save_state(sp, state)
    F.save_treetop(tp, leaves, r_root)
    F.save_histograms(hp, hists)
    oracle_lib.ref_extract_surface_streaming(cp, sp, tp, hp, origin, r_root, op)
    v, f = oracle_lib.extract_surface_streaming(cubes, state, hists, leaves, origin, r_root)
    assert len(f) > 0
    assert oracle_lib.obj_text(v, f) == op.read_text()


@pytest.mark.parametrize("case", MESH_CASES)
def test_extract_surface_matches_golden(oracle_lib, case):
    g = load_golden(case)
    out = oracle_lib.extract_surface(g["cubes"], g["state"], g["origin"], float(g["r_root"]),
                                     has_data=g["has_data"], normals=True)
    assert_mesh_equal(out, (g["verts"], g["faces"], g["normals"]), case)
    v, f = oracle_lib.extract_surface_streaming(g["cubes"], g["state"], g["hists"], g["leaves"], g["origin"],
                                                float(g["r_root"]))
    assert oracle_lib.obj_text(v, f) == str(g["s_obj"])
