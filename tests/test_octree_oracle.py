"""The merge (Stage 2) and balance (Stage 3) oracles against the reference's
kway_merge and balance_octree compiled here, and against the committed
fixture made from them.

Merge: bit-exact when no code occurs in two inputs (the reference's heap
order for equal codes from different inputs is std::priority_queue's); the
same distinct (code, depth) cells otherwise.  Balance: the same multiset of
cubes (the reference leaves equal codes in hash-table order)."""
import numpy as np
import pytest

import octree_cases as OC
from conftest import load_golden
from tgvreconclaude_gb300 import formats as F


def needs_ref(f):
    import oracle
    return pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout absent")(f)


def cells(c):
    return set(zip(c["hi"].tolist(), c["lo"].tolist(), c["depth"].tolist()))


@needs_ref
def test_merge_matches_reference(oracle_lib):
    from test_stage1_oracle import stage1_maps
    for seed in range(3):
        maps, origin, r_root = stage1_maps(seed, n=4)
        arrs = [oracle_lib.build_cubes(m, origin, r_root) for m in maps]
        parts = OC.disjoint_parts(arrs)
        assert oracle_lib.merge_cubes(parts).tobytes() == oracle_lib.ref_merge_cubes(parts, r_root).tobytes()
        a, b = oracle_lib.merge_cubes(arrs), oracle_lib.ref_merge_cubes(arrs, r_root)
        assert cells(a) == cells(b)
        assert np.all(np.diff(F.cube_keys(a).astype(np.float64)) >= 0)


@needs_ref
def test_merge_edge_cases_match_reference(oracle_lib):
    rng = np.random.default_rng(5)
    c = OC.sort_by_code(OC.rand_cells(rng, 400, 3, 6))
    cases = [[], [c[:0]], [c], [c[:0], c, c[:0]],
             [c[::2], c[1::2]]]  # alternating entries of one list: equal codes split across inputs
    for arrs in cases:
        a = oracle_lib.merge_cubes(arrs)
        b = oracle_lib.ref_merge_cubes(arrs, 1.0)
        if len(arrs) <= 1 or sum(len(x) > 0 for x in arrs) <= 1:
            assert a.tobytes() == b.tobytes()
        assert cells(a) == cells(b)


@needs_ref
@pytest.mark.parametrize("seed", range(8))
def test_balance_matches_reference(oracle_lib, seed):
    c = OC.balance_inputs(seed)
    a, b = oracle_lib.balance_cubes(c, 2.0), oracle_lib.ref_balance_cubes(c, 2.0)
    assert len(a) >= len(np.unique(F.cube_keys(c)))
    assert oracle_lib.cube_multiset(a).tobytes() == oracle_lib.cube_multiset(b).tobytes()


@needs_ref
def test_balance_reference_cases(oracle_lib):
    for c, r in OC.reference_cases():
        a, b = oracle_lib.balance_cubes(c, r), oracle_lib.ref_balance_cubes(c, r)
        assert oracle_lib.cube_multiset(a).tobytes() == oracle_lib.cube_multiset(b).tobytes()
    # the two-cube case gains the depth-6 bridge (test_stages2_4.cpp:175-180)
    c, r = OC.reference_cases()[1]
    out = oracle_lib.balance_cubes(c, r)
    assert len(out) == 3 and sorted(out["depth"].tolist()) == [5, 6, 7]


def test_golden(oracle_lib):
    g = load_golden("octree_cases.npz")
    parts = [g[f"disjoint_in{i}"] for i in range(3)]
    assert oracle_lib.merge_cubes(parts).tobytes() == g["disjoint_out"].tobytes()
    arrs = [g[f"overlap_in{i}"] for i in range(4)]
    assert cells(oracle_lib.merge_cubes(arrs)) == cells(g["overlap_out"])
    i = 0
    while f"bal_in{i}" in g:
        a = oracle_lib.balance_cubes(g[f"bal_in{i}"], float(g[f"bal_r{i}"]))
        assert oracle_lib.cube_multiset(a).tobytes() == oracle_lib.cube_multiset(g[f"bal_out{i}"]).tobytes(), i
        i += 1
    assert i == 7
