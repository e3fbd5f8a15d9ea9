"""Chunk partitioning of the streaming semantics across ranks.

The streaming solve (reference src/tgv.cpp:802-1070) is the reference's only
decomposition: within a level, treetop leaves ("chunks") see one another only
through the level-start snapshot of u/v and zero border p/q.  So chunks can be
spread over ranks that exchange state once per level:

* every rank holds the whole cube and histogram arrays and its own copy of the
  state;
* at level L every rank re-derives the level-start state (parent init of every
  chunk's level-L cubes, then the snapshot) and iterates only its own chunks;
* after level L, each rank publishes the final state of those of its level-L
  cubes that another rank will read later -- as a parent, as a border
  neighbour, or as the parent of a border neighbour -- and nothing else.

`assign_chunks` balances chunks over ranks by cube count (largest first onto
the least-loaded rank).  `publish_sets` derives the exchange from the same
neighbour and parent resolution the solver uses (leaf-local lookups, else the
cube file's bisection hit).  The GB300 build runs one GPU per box, so this is
exercised with CPU ranks (gloo) driving the oracle's per-level step; the GPU
solver runs replicas only.
"""
from __future__ import annotations

import numpy as np

from . import formats as F


def assign_chunks(leaves, world: int) -> np.ndarray:
    """owner[l] for each leaf: longest-processing-time greedy on cube counts."""
    sizes = np.maximum(0, leaves["last_idx"].astype(np.int64) - leaves["first_idx"].astype(np.int64) + 1)
    owner = np.zeros(len(leaves), np.int32)
    load = np.zeros(world, np.int64)
    for l in np.argsort(-sizes, kind="stable"):
        r = int(np.argmin(load))
        owner[l] = r
        load[r] += sizes[l]
    return owner


def _face_keys(keys, depth, face):
    x, y, z = (c.astype(np.int64) for c in F.morton_decode(keys))
    step = np.left_shift(np.int64(1), (21 - depth).astype(np.int64))
    c = [x, y, z]
    ax, sg = face // 2, (1 if face % 2 == 0 else -1)
    nv = c[ax] + sg * step
    ok = (nv >= 0) & (nv < (1 << 21))
    c[ax] = np.clip(nv, 0, (1 << 21) - 1)
    return F.morton_encode(c[0].astype(np.uint32), c[1].astype(np.uint32), c[2].astype(np.uint32)), ok


def _bisect_hit(n, r0, r1):
    """Index the reference's cube-file bisection (tgv.cpp:673-683) returns for
    a code whose equal-code run is [r0, r1]."""
    lo = np.zeros_like(r0)
    hi = np.full_like(r0, n)
    res = np.full_like(r0, -1)
    act = r0 <= r1
    for _ in range(64):
        if not act.any():
            break
        mid = lo + (hi - lo) // 2
        hit = act & (mid >= r0) & (mid <= r1)
        res[hit] = mid[hit]
        act &= ~hit
        lt = act & (mid < r0)
        gt = act & (mid > r1)
        lo[lt] = mid[lt] + 1
        hi[gt] = mid[gt]
        act &= lo < hi
    return res


def leaf_of(n, leaves) -> np.ndarray:
    out = np.full(n, -1, np.int64)
    for l, lv in enumerate(leaves):
        a, b = int(lv["first_idx"]), int(lv["last_idx"])
        if a < n and a <= b:
            out[a:min(b, n - 1) + 1] = l
    return out


def stream_refs(cubes, leaves, level: int):
    """Cube indices that the level-`level` cubes of each chunk read outside
    their chunk: (reader cube, referenced cube) pairs for border neighbours and
    for parents.  Cubes must be Morton-sorted."""
    keys = F.cube_keys(cubes)
    n = len(cubes)
    lo_of = leaf_of(n, leaves)
    idx = np.nonzero((cubes["depth"] == level) & (lo_of >= 0))[0]
    if len(idx) == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    f0 = leaves["first_idx"][lo_of[idx]].astype(np.int64)
    l0 = np.minimum(leaves["last_idx"][lo_of[idx]].astype(np.int64), n - 1)
    readers, refs = [], []
    d = np.full(len(idx), level, np.int64)

    def run(codes):
        r0 = np.searchsorted(keys, codes, "left").astype(np.int64)
        r1 = np.searchsorted(keys, codes, "right").astype(np.int64) - 1
        return r0, r1

    for face in range(6):
        c1, ok = _face_keys(keys[idx], d, face)
        r0, r1 = run(c1)
        ex1 = ok & (r0 <= r1)
        loc1 = ex1 & (np.maximum(r0, f0) <= np.minimum(r1, l0))
        border = ex1 & ~loc1
        g = _bisect_hit(n, r0, r1)
        readers.append(idx[border]); refs.append(g[border])
        if level > 0:
            c2 = F.ancestor_key(c1, level - 1)
            q0, q1 = run(c2)
            ex2 = ok & ~ex1 & (q0 <= q1)
            loc2 = ex2 & (np.maximum(q0, f0) <= np.minimum(q1, l0))
            b2 = ex2 & ~loc2
            g2 = _bisect_hit(n, q0, q1)
            readers.append(idx[b2]); refs.append(g2[b2])
    if level > 0:
        pk = F.ancestor_key(keys[idx], level - 1)
        p0, p1 = run(pk)
        has = p0 <= p1
        gp = _bisect_hit(n, p0, p1)
        readers.append(idx[has]); refs.append(gp[has])
    return np.concatenate(readers), np.concatenate(refs)


def publish_sets(cubes, leaves, owner, world: int):
    """publish[L][r] = sorted indices of rank r's level-L cubes whose final state
    another rank reads at a later level."""
    n = len(cubes)
    lo_of = leaf_of(n, leaves)
    own = np.where(lo_of >= 0, owner[np.maximum(lo_of, 0)], -1)
    depth = cubes["depth"].astype(np.int64)
    levels = sorted(set(int(x) for x in depth))
    needed = np.zeros(n, bool)
    for L in levels:
        rd, rf = stream_refs(cubes, leaves, L)
        # a border cube at the same level is re-derived by the reader from its parent
        same = depth[rf] == L
        if same.any():
            keys = F.cube_keys(cubes)
            pk = F.ancestor_key(keys[rf[same]], L - 1) if L > 0 else keys[rf[same]]
            p0 = np.searchsorted(keys, pk, "left")
            p1 = np.searchsorted(keys, pk, "right") - 1
            gp = _bisect_hit(n, p0.astype(np.int64), p1.astype(np.int64))
            ok = gp >= 0
            rd = np.concatenate([rd, rd[same][ok]])
            rf = np.concatenate([rf, gp[ok]])
        cross = (own[rf] >= 0) & (own[rf] != own[rd]) & (depth[rf] < L)
        needed[rf[cross]] = True
    out = {}
    for L in levels:
        out[L] = [np.nonzero(needed & (depth == L) & (own == r))[0] for r in range(world)]
    return out


def emulate_ranks(cubes, hists, leaves, params, world: int, oracle, exchange: str = "publish"):
    """All ranks of `sharded_stream_solve` stepped level by level in one
    process.  Returns the merged state (each cube from its owner) and the
    per-level exchange sizes."""
    n = len(cubes)
    owner = assign_chunks(leaves, world)
    masks = [(owner == r).astype(np.uint8) for r in range(world)]
    states = [oracle.stream_init(cubes, hists) for _ in range(world)]
    depth = cubes["depth"]
    pub = publish_sets(cubes, leaves, owner, world) if exchange == "publish" else None
    lo_of = leaf_of(n, leaves)
    own = np.where(lo_of >= 0, owner[np.maximum(lo_of, 0)], -1)
    sent = []
    for L in sorted(set(int(x) for x in depth)):
        for r in range(world):
            oracle.stream_level(cubes, hists, leaves, masks[r], L, params, states[r])
        msgs = [(pub[L][r] if pub is not None else np.nonzero((depth == L) & (own == r))[0]) for r in range(world)]
        msgs = [(ix, states[r][ix].copy()) for r, ix in enumerate(msgs)]
        sent.append(sum(len(ix) for ix, _ in msgs))
        for r in range(world):
            for q, (ix, vals) in enumerate(msgs):
                if q != r and len(ix):
                    states[r][ix] = vals
    merged = states[0].copy()
    for r in range(world):
        sel = own == r
        merged[sel] = states[r][sel]
    return merged, sent


def sharded_stream_solve(cubes, hists, leaves, params, rank: int, world: int, allgather, oracle,
                         exchange: str = "publish"):
    """Streaming solve of this rank's chunks with one exchange per level.
    `allgather(obj) -> list` gathers one Python object from every rank;
    `oracle` provides stream_level (the CPU step).  exchange = "publish" (only
    the cubes another rank reads) or "level" (every level-L cube).  Returns the
    local state (exact on this rank's own cubes) and the per-level exchange sizes."""
    n = len(cubes)
    owner = assign_chunks(leaves, world)
    mask = (owner == rank).astype(np.uint8)
    state = oracle.stream_init(cubes, hists)
    depth = cubes["depth"]
    levels = sorted(set(int(x) for x in depth))
    pub = publish_sets(cubes, leaves, owner, world) if exchange == "publish" else None
    lo_of = leaf_of(n, leaves)
    own = np.where(lo_of >= 0, owner[np.maximum(lo_of, 0)], -1)
    sent = []
    for L in levels:
        oracle.stream_level(cubes, hists, leaves, mask, L, params, state)
        idx = pub[L][rank] if pub is not None else np.nonzero((depth == L) & (own == rank))[0]
        sent.append(len(idx))
        for r, (ix, vals) in enumerate(allgather((idx, state[idx].copy()))):
            if r != rank and len(ix):
                state[ix] = vals
    return state, owner, sent
