"""The Stage-1 oracle (cubes from a depth map) against the reference's own
build_cubes_from_depthmap compiled here, compared as multisets (the reference
orders equal codes arbitrarily), and against the committed fixture."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from tgvreconclaude_gb300 import scenes as S


def needs_ref(f):
    import oracle
    return pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout absent")(f)


def stage1_maps(seed, n=3, w=96, h=72):
    rng = np.random.default_rng(seed)
    scene = [S.torus_scene(0.005), S.three_objects_scene(rng)][seed % 2]
    rig = S.sphere_rig(n, [3.0, 6.0][seed % 2], width=w, height=h, half_fov_deg=28)
    maps = []
    for i, c in enumerate(rig):
        d = S.render_depth(scene, c, seed=seed * 10 + i).numpy()
        d[rng.random(d.shape) < 0.03] = np.nan  # holes
        maps.append(dict(depth=d, rt=c["rt"], fx=c["fx"], fy=c["fy"], cx=c["cx"], cy=c["cy"]))
    return maps, [(-1.5, -1.5, -1.5), (-3.0, -3.0, -3.0)][seed % 2], [1.5, 3.0][seed % 2]


def edge_maps():
    """Depth maps the reference's edge handling decides: no valid pixel, zero and
    negative depths, isolated pixels, a 1x1 map, infinite depths, a ragged
    3x257 map."""
    rng = np.random.default_rng(3)
    base = dict(rt=np.eye(4, dtype=np.float32), fx=np.float32(50.0), fy=np.float32(50.0),
                cx=np.float32(15.5), cy=np.float32(11.5))
    cases = {
        "all_nan": np.full((24, 32), np.nan, np.float32),
        "zeros_and_negative": np.where(rng.random((24, 32)) < 0.5, 0.0, -1.0).astype(np.float32),
        "isolated_pixels": np.where(rng.random((24, 32)) < 0.1, 2.0, np.nan).astype(np.float32),
        "one_pixel": np.full((1, 1), 2.0, np.float32),
        "inf_depth": np.where(rng.random((24, 32)) < 0.2, np.inf, 2.0).astype(np.float32),
        "ragged_wide": (1.5 + 0.2 * rng.random((3, 257))).astype(np.float32),
    }
    return {k: dict(base, depth=d) for k, d in cases.items()}


@needs_ref
def test_build_cubes_edge_cases_match_reference(oracle_lib):
    for name, m in edge_maps().items():
        ref = oracle_lib.ref_build_cubes(m, (-3, -3, -3), 3.0)
        out = oracle_lib.build_cubes(m, (-3, -3, -3), 3.0)
        assert oracle_lib.cube_multiset(out).tobytes() == oracle_lib.cube_multiset(ref).tobytes(), name


@needs_ref
@pytest.mark.parametrize("seed", range(4))
def test_build_cubes_matches_reference(oracle_lib, seed):
    maps, origin, r_root = stage1_maps(seed)
    for m in maps:
        ref = oracle_lib.ref_build_cubes(m, origin, r_root)
        out = oracle_lib.build_cubes(m, origin, r_root)
        assert len(ref) > 100
        assert np.array_equal(out["hi"].astype(np.uint64) << 32 | out["lo"], ref["hi"].astype(np.uint64) << 32 | ref["lo"])
        assert oracle_lib.cube_multiset(out).tobytes() == oracle_lib.cube_multiset(ref).tobytes()


def test_build_cubes_matches_golden(oracle_lib):
    g = load_golden("stage1_maps.npz")
    for k in range(len(g["depths"])):
        m = dict(depth=g["depths"][k], rt=g["rt"][k], fx=g["fx"][k], fy=g["fy"][k], cx=g["cx"][k], cy=g["cy"][k])
        out = oracle_lib.build_cubes(m, g["origin"], float(g["r_root"]))
        ref = g[f"cubes{k}"]
        assert oracle_lib.cube_multiset(out).tobytes() == oracle_lib.cube_multiset(ref).tobytes()


def test_reference_build_kat(oracle_lib):
    """tests/test_stage1.cpp:84-117 on the oracle: sorted cubes whose depths
    satisfy 0.75 r_c <= r_root / 2^d < 1.5 r_c."""
    m = dict(depth=np.full((10, 10), 5.0, np.float32), rt=np.eye(4, dtype=np.float32), fx=np.float32(50),
             fy=np.float32(50), cx=np.float32(5), cy=np.float32(5))
    cubes = oracle_lib.build_cubes(m, (-1.0, -1.0, 4.0), 2.5)
    assert len(cubes) > 0
    k = (cubes["hi"].astype(np.uint64) << np.uint64(32)) | cubes["lo"]
    assert np.all(k[1:] >= k[:-1])
    cell = np.float32(2.5) / (np.uint32(1) << cubes["depth"].astype(np.uint32)).astype(np.float32)
    assert np.all(cell >= np.float32(0.75) * cubes["r_c"]) and np.all(cell < np.float32(1.5) * cubes["r_c"])
