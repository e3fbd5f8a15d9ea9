"""Stage 1 on the GPU (tgvg_build_cubes) against the oracle: bit-exact, in the
same order (both sort stably by code over pixel order)."""
import os

import numpy as np
import pytest

from conftest import load_golden
from test_stage1_oracle import edge_maps, stage1_maps
from tgvreconclaude_gb300 import api, formats as F

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", range(4))
def test_build_cubes_matches_oracle(oracle_lib, seed):
    maps, origin, r_root = stage1_maps(seed)
    for m in maps:
        ref = oracle_lib.build_cubes(m, origin, r_root)
        out = api.build_cubes(m, origin, r_root)
        assert len(out) == len(ref) > 100
        assert out.tobytes() == ref.tobytes()


def test_build_cubes_golden(oracle_lib):
    g = load_golden("stage1_maps.npz")
    for k in range(len(g["depths"])):
        m = dict(depth=g["depths"][k], rt=g["rt"][k], fx=g["fx"][k], fy=g["fy"][k], cx=g["cx"][k], cy=g["cy"][k])
        out = api.build_cubes(m, g["origin"], float(g["r_root"]))
        assert oracle_lib.cube_multiset(out).tobytes() == oracle_lib.cube_multiset(g[f"cubes{k}"]).tobytes()


def test_build_cubes_edge_cases(oracle_lib, tmp_path):
    maps = edge_maps()
    for name, m in maps.items():
        ref = oracle_lib.build_cubes(m, (-3, -3, -3), 3.0)
        out = api.build_cubes(m, (-3, -3, -3), 3.0)
        assert out.tobytes() == ref.tobytes(), name
    # the file form writes the same cubes
    m = maps["ragged_wide"]
    p = tmp_path / "c.bin"
    api.build_cubes_file(m, (-3, -3, -3), 3.0, p)
    cubes, _ = F.load_cubes(str(p))
    assert cubes.tobytes() == api.build_cubes(m, (-3, -3, -3), 3.0).tobytes()


def test_build_cubes_dataclass_form(oracle_lib):
    maps, origin, r_root = stage1_maps(1, n=1)
    m = maps[0]
    h, w = m["depth"].shape
    K = np.array([[m["fx"], 0, m["cx"]], [0, m["fy"], m["cy"]], [0, 0, 1]], np.float32)
    dm = api.DepthMap(w, h, m["depth"].reshape(-1), K, np.asarray(m["rt"], np.float32).reshape(4, 4))
    assert api.build_cubes(dm, origin, r_root).tobytes() == oracle_lib.build_cubes(m, origin, r_root).tobytes()


def test_reference_build_and_load_kat(tmp_path):
    """tests/test_stage1.cpp:84-117: a 10x10 plane at z = 5 seen head-on; the
    file round-trips r_root, the cubes are sorted, and every depth satisfies
    0.75 r_c <= r_root / 2^d < 1.5 r_c."""
    K = np.array([[50, 0, 5], [0, 50, 5], [0, 0, 1]], np.float32)
    dm = api.DepthMap(10, 10, np.full(100, 5.0, np.float32), K, np.eye(4, dtype=np.float32))
    p = tmp_path / "t.cubes"
    api.build_cubes_file(dm, (-1.0, -1.0, 4.0), 2.5, p)
    cubes, rr = F.load_cubes(str(p))
    assert abs(rr - 2.5) <= 1e-5 and len(cubes) > 0
    k = F.cube_keys(cubes)
    assert np.all(k[1:] >= k[:-1])
    cell = np.float32(2.5) / (np.uint32(1) << cubes["depth"].astype(np.uint32)).astype(np.float32)
    assert np.all(cell >= np.float32(0.75) * cubes["r_c"]) and np.all(cell < np.float32(1.5) * cubes["r_c"])
