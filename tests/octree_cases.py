"""Seeded inputs for the merge (Stage 2) and balance (Stage 3) tests."""
from __future__ import annotations

import numpy as np

from tgvreconclaude_gb300 import formats as F


def rand_cells(rng, n, dmin, dmax, clustered=True):
    """n valid cells with depths in [dmin, dmax]: near a sphere of radius 0.3 at
    the root's centre (so every root octant is hit), or uniform in the root."""
    d = rng.integers(dmin, dmax + 1, n)
    if clustered:
        v = rng.normal(size=(n, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        p = 0.5 + 0.3 * v
    else:
        p = rng.random((n, 3))
    ix = np.minimum((p * (1 << 21)).astype(np.uint64), (1 << 21) - 1)
    sh = (21 - d).astype(np.uint64)
    ix = (ix >> sh[:, None]) << sh[:, None]
    k = F.morton_encode(ix[:, 0], ix[:, 1], ix[:, 2])
    rc = (0.7 * 2.0 ** -d.astype(np.float64) * (1 + 0.1 * rng.random(n))).astype(np.float32)
    return F.make_cubes(k, d, rc)


def balance_inputs(seed):
    """Balance stress inputs: clustered and uniform cells over several depth
    ranges, deep cells (depths 14..19), duplicated cells, sorted or not."""
    rng = np.random.default_rng(seed)
    kind = seed % 4
    if kind == 0:
        c = rand_cells(rng, 3000, 3, 9)
    elif kind == 1:
        c = rand_cells(rng, 3000, 2, 12, clustered=False)
    elif kind == 2:
        c = rand_cells(rng, 2000, 14, 19)
    else:
        c = rand_cells(rng, 3000, 3, 10)
        c = np.concatenate([c, c[rng.integers(0, len(c), 500)]])
    if seed % 2:
        c = c[np.argsort(F.cube_keys(c), kind="stable")]
    return c


def sort_by_code(c):
    return c[np.argsort(F.cube_keys(c), kind="stable")]


def disjoint_parts(arrays, k=3):
    """The cubes of `arrays` split into k code-sorted lists whose code sets are
    disjoint (split by a hash of the code; each list keeps the stable order)."""
    one = sort_by_code(np.concatenate(arrays))
    key = F.cube_keys(one)
    grp = ((key * np.uint64(0x9E3779B97F4A7C15)) >> np.uint64(61)).astype(np.int64) % k
    return [one[grp == g] for g in range(k)]


def reference_cases():
    """The reference's own balance cases (tests/test_stages2_4.cpp:134-226): one
    cube, and a depth-5 cube with a depth-7 cube across its +x face."""
    one = F.make_cubes(np.array([0], np.uint64), np.array([5]), np.array([0.3], np.float32))
    step5 = np.uint64(1 << 16)
    k = np.array([0, F.morton_encode(step5, np.uint64(0), np.uint64(0))], np.uint64)
    two = F.make_cubes(k, np.array([5, 7]), np.array([100.0 / 32, 100.0 / 128], np.float32))
    return [(one, 10.0), (two, 100.0)]
