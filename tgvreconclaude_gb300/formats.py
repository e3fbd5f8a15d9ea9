"""Record layouts and on-disk formats of the reference's Stage-5/6 boundary.

The in-memory records are byte-identical to the reference's structs, so arrays
of them can be handed to the C-ABI (include/tgvg.h) without conversion:

* ``OctreeCube``    16 B  {code.hi u32, code.lo u32, r_c f32, depth i32}
  (reference src/types.hpp:18-35)
* ``CubeHistogram`` 32 B  {bins u32[8]}  (src/histogram.hpp:10-19); the 10-bin
  extension uses 40-byte rows
* ``TGVCube``       52 B  {u, v[3], p[3], q[6] (Voigt xx yy zz xy xz yz)}
  (src/tgv.hpp:12-17)
* ``TreetopLeaf``   20 B  {code.hi, code.lo, depth i32, first_idx u32, last_idx u32}
  (src/treetop.hpp:8-13)

Files (little-endian, packed):

* ``TGV1`` cube file: magic, version u32 = 1, r_root f32, count u32, cubes
  (src/octree_builder.hpp:8-19)
* ``TGVH`` histograms: magic, version, count, rows (src/histogram.cpp:167-185)
* ``TGVT`` treetop: magic, version, r_root f32, leaf_count, leaves (src/treetop.hpp:15-20)
* ``TGVS`` TGV state: magic, version, count, TGVCube[] (src/tgv.cpp:16-33)
"""
from __future__ import annotations

import numpy as np

CUBE_DTYPE = np.dtype([("hi", "<u4"), ("lo", "<u4"), ("r_c", "<f4"), ("depth", "<i4")])
LEAF_DTYPE = np.dtype([("hi", "<u4"), ("lo", "<u4"), ("depth", "<i4"),
                       ("first_idx", "<u4"), ("last_idx", "<u4")])
STATE_DTYPE = np.dtype([("u", "<f4"), ("v", "<f4", (3,)), ("p", "<f4", (3,)), ("q", "<f4", (6,))])
assert CUBE_DTYPE.itemsize == 16 and LEAF_DTYPE.itemsize == 20 and STATE_DTYPE.itemsize == 52

MAX_DEPTH = 21  # fine-grid bits per axis (src/types.hpp:36-73)


# ---------------------------------------------------------------- Morton ---
_M = [(32, 0x001F00000000FFFF), (16, 0x001F0000FF0000FF), (8, 0x100F00F00F00F00F),
      (4, 0x10C30C30C30C30C3), (2, 0x1249249249249249)]


def spread3(v):
    """Interleave two zero bits between the 21 low bits of each element (uint64)."""
    x = np.asarray(v, np.uint64) & np.uint64(0x1FFFFF)
    for s, m in _M:
        x = (x | (x << np.uint64(s))) & np.uint64(m)
    return x


def gather3(v):
    """Inverse of spread3: collect every third bit (from bit 0) into 21 bits."""
    x = np.asarray(v, np.uint64) & np.uint64(0x1249249249249249)
    for s, m in ((2, 0x10C30C30C30C30C3), (4, 0x100F00F00F00F00F), (8, 0x001F0000FF0000FF),
                 (16, 0x001F00000000FFFF), (32, 0x00000000001FFFFF)):
        x = (x | (x >> np.uint64(s))) & np.uint64(m)
    return x.astype(np.uint32)


def morton_encode(x, y, z):
    """uint64 Z-code of fine-grid coordinates (bit 3k = x_k, 3k+1 = y_k, 3k+2 = z_k)."""
    return spread3(x) | (spread3(y) << np.uint64(1)) | (spread3(z) << np.uint64(2))


def morton_decode(k):
    k = np.asarray(k, np.uint64)
    return gather3(k), gather3(k >> np.uint64(1)), gather3(k >> np.uint64(2))


def cube_keys(cubes) -> np.ndarray:
    return (cubes["hi"].astype(np.uint64) << np.uint64(32)) | cubes["lo"].astype(np.uint64)


def make_cubes(keys, depth, r_c) -> np.ndarray:
    keys = np.asarray(keys, np.uint64)
    out = np.zeros(len(keys), CUBE_DTYPE)
    out["hi"] = (keys >> np.uint64(32)).astype(np.uint32)
    out["lo"] = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    out["depth"] = depth
    out["r_c"] = r_c
    return out


def ancestor_key(keys, depth):
    """Code of the depth-``depth`` ancestor: clear the low 3*(21-depth) bits."""
    keys = np.asarray(keys, np.uint64)
    sh = (3 * (MAX_DEPTH - np.asarray(depth, np.int64))).astype(np.uint64)
    mask = np.where(sh >= 64, np.uint64(0), ~((np.uint64(1) << np.minimum(sh, 63)) - np.uint64(1)))
    return keys & mask


# ---------------------------------------------------------------- files ---

def save_cubes(path, cubes, r_root: float) -> None:
    cubes = np.ascontiguousarray(cubes, CUBE_DTYPE)
    with open(path, "wb") as f:
        f.write(b"TGV1" + np.array([1], "<u4").tobytes() + np.array([r_root], "<f4").tobytes()
                + np.array([len(cubes)], "<u4").tobytes())
        f.write(cubes.tobytes())


def load_cubes(path):
    with open(path, "rb") as f:
        b = f.read()
    if b[:4] != b"TGV1":
        raise ValueError(f"Bad magic in cube file: {path}")
    r_root = float(np.frombuffer(b, "<f4", 1, 8)[0])
    n = int(np.frombuffer(b, "<u4", 1, 12)[0])
    return np.frombuffer(b, CUBE_DTYPE, n, 16).copy(), r_root


def save_histograms(path, hists) -> None:
    hists = np.ascontiguousarray(hists, np.uint32)
    with open(path, "wb") as f:
        f.write(b"TGVH" + np.array([1, len(hists)], "<u4").tobytes())
        f.write(hists.tobytes())


def load_histograms(path, nbins: int = 8):
    with open(path, "rb") as f:
        b = f.read()
    if b[:4] != b"TGVH":
        raise ValueError("Bad histogram magic")
    n = int(np.frombuffer(b, "<u4", 1, 8)[0])
    return np.frombuffer(b, np.uint32, n * nbins, 12).reshape(n, nbins).copy()


def save_treetop(path, leaves, r_root: float) -> None:
    leaves = np.ascontiguousarray(leaves, LEAF_DTYPE)
    with open(path, "wb") as f:
        f.write(b"TGVT" + np.array([1], "<u4").tobytes() + np.array([r_root], "<f4").tobytes()
                + np.array([len(leaves)], "<u4").tobytes())
        f.write(leaves.tobytes())


def load_treetop(path):
    with open(path, "rb") as f:
        b = f.read()
    if b[:4] != b"TGVT":
        raise ValueError(f"Bad treetop magic: {path}")
    r_root = float(np.frombuffer(b, "<f4", 1, 8)[0])
    n = int(np.frombuffer(b, "<u4", 1, 12)[0])
    return np.frombuffer(b, LEAF_DTYPE, n, 16).copy(), r_root


def save_state(path, state) -> None:
    state = np.ascontiguousarray(state, STATE_DTYPE)
    with open(path, "wb") as f:
        f.write(b"TGVS" + np.array([1, len(state)], "<u4").tobytes())
        f.write(state.tobytes())


def load_state(path):
    with open(path, "rb") as f:
        b = f.read()
    if b[:4] != b"TGVS":
        raise ValueError("Bad TGV state magic")
    n = int(np.frombuffer(b, "<u4", 1, 8)[0])
    return np.frombuffer(b, STATE_DTYPE, n, 12).copy()
