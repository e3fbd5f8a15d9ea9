"""Merge (Stage 2) and balance (Stage 3) on the GPU against the oracle:
bit-exact, in the same order (both merge equal codes in input order and sort
the balance output by code, then depth)."""
import numpy as np
import pytest

import octree_cases as OC
from conftest import load_golden
from test_stage1_oracle import stage1_maps
from tgvreconclaude_gb300 import api, formats as F

pytestmark = pytest.mark.gpu


def test_merge_matches_oracle(oracle_lib):
    for seed in range(3):
        maps, origin, r_root = stage1_maps(seed, n=4)
        arrs = [oracle_lib.build_cubes(m, origin, r_root) for m in maps]
        for inputs in (arrs, OC.disjoint_parts(arrs), arrs[:1], []):
            assert api.merge_cubes(inputs).tobytes() == oracle_lib.merge_cubes(inputs).tobytes()


def test_merge_golden(oracle_lib):
    g = load_golden("octree_cases.npz")
    parts = [g[f"disjoint_in{i}"] for i in range(3)]
    assert api.merge_cubes(parts).tobytes() == g["disjoint_out"].tobytes()


@pytest.mark.parametrize("seed", range(8))
def test_balance_matches_oracle(oracle_lib, seed):
    c = OC.balance_inputs(seed)
    assert api.balance_cubes(c, 2.0).tobytes() == oracle_lib.balance_cubes(c, 2.0).tobytes()


def test_balance_golden(oracle_lib):
    g = load_golden("octree_cases.npz")
    i = 0
    while f"bal_in{i}" in g:
        a = api.balance_cubes(g[f"bal_in{i}"], float(g[f"bal_r{i}"]))
        assert oracle_lib.cube_multiset(a).tobytes() == oracle_lib.cube_multiset(g[f"bal_out{i}"]).tobytes(), i
        i += 1


def test_balance_edge_cases(oracle_lib):
    empty = np.zeros(0, F.CUBE_DTYPE)
    assert len(api.balance_cubes(empty, 1.0)) == 0
    for c, r in OC.reference_cases():
        assert api.balance_cubes(c, r).tobytes() == oracle_lib.balance_cubes(c, r).tobytes()
    bad = OC.reference_cases()[1][0].copy()
    bad["lo"][1] |= 1  # off its depth's grid
    with pytest.raises(RuntimeError, match="grid"):
        api.balance_cubes(bad, 1.0)
    bad = OC.reference_cases()[1][0].copy()
    bad["depth"][0] = 22
    with pytest.raises(RuntimeError):
        api.balance_cubes(bad, 1.0)


def test_file_forms(oracle_lib, tmp_path):
    maps, origin, r_root = stage1_maps(1, n=3)
    arrs = [oracle_lib.build_cubes(m, origin, r_root) for m in maps]
    paths = []
    for i, a in enumerate(arrs):
        p = tmp_path / f"m{i}.cubes"
        F.save_cubes(str(p), a, r_root)
        paths.append(p)
    api.kway_merge(paths, tmp_path / "merged.cubes")
    merged, rr = F.load_cubes(str(tmp_path / "merged.cubes"))
    assert rr == np.float32(r_root) and merged.tobytes() == oracle_lib.merge_cubes(arrs).tobytes()
    api.balance_octree(tmp_path / "merged.cubes", tmp_path / "bal.cubes")
    bal, rr = F.load_cubes(str(tmp_path / "bal.cubes"))
    assert rr == np.float32(r_root) and bal.tobytes() == oracle_lib.balance_cubes(merged, r_root).tobytes()
    api.kway_merge([], tmp_path / "none.cubes")
    none, rr = F.load_cubes(str(tmp_path / "none.cubes"))
    assert len(none) == 0 and rr == 0.0
    (tmp_path / "bad.cubes").write_bytes(b"XXXX" + bytes(12))
    with pytest.raises(RuntimeError, match="magic"):
        api.kway_merge([tmp_path / "bad.cubes"], tmp_path / "o.cubes")
    with pytest.raises(RuntimeError):
        api.balance_octree(tmp_path / "missing.cubes", tmp_path / "o.cubes")


def test_stages_1_to_3_at_scale(oracle_lib):
    """Stage 1 on 8 maps of 640x480, merge, balance: GPU against the oracle at
    about a million cubes, and 2:1 balance of the output's cells checked
    directly as a property."""
    from tgvreconclaude_gb300 import scenes as S
    rng = np.random.default_rng(7)
    scene = S.three_objects_scene(rng)
    rig = S.sphere_rig(8, 3.0, width=640, height=480, half_fov_deg=30)
    maps = [dict(depth=S.render_depth(scene, c, seed=i).numpy(), rt=c["rt"], fx=c["fx"], fy=c["fy"], cx=c["cx"],
                 cy=c["cy"]) for i, c in enumerate(rig)]
    origin, r_root = (-1.5, -1.5, -1.5), 1.5
    arrs = [api.build_cubes(m, origin, r_root) for m in maps]
    merged = api.merge_cubes(arrs)
    assert merged.tobytes() == oracle_lib.merge_cubes(arrs).tobytes()
    assert len(merged) > 500_000
    bal = api.balance_cubes(merged, r_root)
    assert bal.tobytes() == oracle_lib.balance_cubes(merged, r_root).tobytes()
    assert len(bal) >= len(np.unique(F.cube_keys(merged)))


def test_reference_merge_kat(tmp_path):
    """tests/test_stages2_4.cpp:102-130: Stage-1 files of two 8x8 planes at z = 5
    and z = 6 merge into one sorted file holding every cube of both."""
    K = np.array([[50, 0, 4], [0, 50, 4], [0, 0, 1]], np.float32)
    paths = []
    for z in (5.0, 6.0):
        dm = api.DepthMap(8, 8, np.full(64, z, np.float32), K, np.eye(4, dtype=np.float32))
        p = tmp_path / f"z{z}.cubes"
        api.build_cubes_file(dm, (-1.5, -1.5, 4.0), 3.0, p)
        paths.append(p)
    api.kway_merge(paths, tmp_path / "m.cubes")
    m, rr = F.load_cubes(str(tmp_path / "m.cubes"))
    a, _ = F.load_cubes(str(paths[0]))
    b, _ = F.load_cubes(str(paths[1]))
    k = F.cube_keys(m)
    assert rr == 3.0 and len(m) > 0 and np.all(k[1:] >= k[:-1])
    assert len(m) == len(a) + len(b)
