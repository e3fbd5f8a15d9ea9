"""ctypes access to the oracle libraries.

TEST INFRASTRUCTURE ONLY.  ``liboracle`` is the CPU restatement of the
reference's histogram and TGV algorithms (oracle/tgv_oracle.cpp); ``libref`` is
the reference's own src/*.cpp compiled unmodified with the project-written
Eigen/TBB shims (oracle/Makefile, built only where the reference checkout
exists).  Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, to check results or as the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from tgvreconclaude_gb300.formats import (  # noqa: E402
    CUBE_DTYPE, LEAF_DTYPE, STATE_DTYPE, cube_keys)

ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
_REF_DIR = None


def ref_dir() -> str:
    """The reference checkout: $TGV_REFERENCE_DIR, else the build recipe's
    default (oracle/Makefile REF_DIR).  It exists only where the reference was
    checked out; nothing that runs on the GPU needs it."""
    global _REF_DIR
    if _REF_DIR is None:
        d = os.environ.get("TGV_REFERENCE_DIR", "")
        if not d:
            r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref-dir"],
                               capture_output=True, text=True)
            d = r.stdout.strip()
        _REF_DIR = d
    return _REF_DIR


def build(ref: bool = False) -> None:
    """Compile the oracle (and, when asked and the reference exists, libref)."""
    targets = ["all"]
    rd = ref_dir()
    if ref and rd and os.path.isdir(os.path.join(rd, "src")):
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE, f"REF_DIR={rd}", f"-j{os.cpu_count() or 4}"]
                   + targets, check=True)


class Camera(C.Structure):
    """orc::Camera: pyramid + Rt_inv (row-major) + base intrinsics."""
    _fields_ = [("rt_inv", C.c_float * 16), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("width", C.c_int32),
                ("height", C.c_int32), ("lidar", C.c_int32), ("n_levels", C.c_int32),
                ("dims", C.c_int32 * 26), ("offs", C.c_int64 * 13),
                ("texels", C.POINTER(C.c_float))]


class Params(C.Structure):
    _fields_ = [("alpha0", C.c_float), ("alpha1", C.c_float), ("iters", C.c_int32),
                ("init", C.c_int32), ("tol", C.c_float), ("check_every", C.c_int32),
                ("keep_init_u", C.c_int32)]


class LevelStats(C.Structure):
    _fields_ = [("depth", C.c_int32), ("iters_run", C.c_int32), ("active", C.c_int64),
                ("residual", C.c_double), ("energy", C.c_double)]


class RefDepthMap(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("rt", C.c_float * 16), ("width", C.c_int32), ("height", C.c_int32),
                ("lidar", C.c_int32), ("depths", C.POINTER(C.c_float))]


def _ptr(a, t=C.c_void_p):
    return a.ctypes.data_as(t) if a is not None and a.size else None


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        _lib = C.CDLL(ORACLE_SO)
        _lib.orc_median_indicator.restype = C.c_float
        _lib.orc_mean_indicator.restype = C.c_float
    return _lib


def ref_available() -> bool:
    rd = ref_dir()
    return os.path.exists(REF_SO) or bool(rd and os.path.isdir(os.path.join(rd, "src")))


def ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            build(ref=True)
        _ref = C.CDLL(REF_SO)
        _ref.ref_mipmap_build.restype = C.c_int64
        _ref.ref_median_indicator.restype = C.c_float
        _ref.ref_mean_indicator.restype = C.c_float
    return _ref


# ---------------------------------------------------------------- pyramids ---

def pyramid_dims(w: int, h: int):
    dims = (C.c_int32 * 26)()
    n = lib().orc_pyramid_dims(w, h, dims)
    return [(dims[2 * i], dims[2 * i + 1]) for i in range(n)]


def pyramid(depth: np.ndarray):
    """Oracle pyramid of one map -> (texels concatenated, [(w, h)...])."""
    h, w = depth.shape
    dims = pyramid_dims(w, h)
    total = sum(a * b for a, b in dims)
    out = np.empty(total, np.float32)
    nl = C.c_int32()
    d = (C.c_int32 * 26)()
    base = np.ascontiguousarray(depth, np.float32)
    lib().orc_pyramid_build(_ptr(base), w, h, _ptr(out), C.byref(nl), d)
    return out, dims


def make_cameras(maps):
    """maps: list of dicts with depth (HxW f32), rt_inv (4x4), fx, fy, cx, cy, lidar.
    Returns (ctypes Camera array, keepalive list)."""
    cams = (Camera * max(1, len(maps)))()
    keep = []
    for c, m in zip(cams, maps):
        tex, dims = pyramid(m["depth"])
        keep.append(tex)
        c.rt_inv[:] = [float(x) for x in np.asarray(m["rt_inv"], np.float32).reshape(16)]
        c.fx, c.fy, c.cx, c.cy = m["fx"], m["fy"], m["cx"], m["cy"]
        c.width, c.height = dims[0]
        c.lidar = int(bool(m.get("lidar", False)))
        c.n_levels = len(dims)
        off = 0
        for i, (a, b) in enumerate(dims):
            c.dims[2 * i], c.dims[2 * i + 1] = a, b
            c.offs[i] = off
            off += a * b
        c.texels = tex.ctypes.data_as(C.POINTER(C.c_float))
    return cams, keep


def compute_histograms(cubes, maps, origin, r_root, nbins=8, nthreads=1):
    cubes = np.ascontiguousarray(cubes, CUBE_DTYPE)
    cams, keep = make_cameras(maps)
    out = np.zeros((len(cubes), nbins), np.uint32)
    o = np.asarray(origin, np.float32)
    rc = lib().orc_compute_histograms(_ptr(cubes), C.c_int64(len(cubes)), cams, len(maps),
                                      _ptr(o), C.c_float(r_root), nbins, _ptr(out), nthreads)
    assert rc == 0
    del keep
    return out


def project(m, p, r_c):
    cams, keep = make_cameras([m])
    lv, u, v, z = C.c_int32(), C.c_int32(), C.c_int32(), C.c_float()
    ok = lib().orc_project(cams, C.c_float(p[0]), C.c_float(p[1]), C.c_float(p[2]),
                           C.c_float(r_c), C.byref(lv), C.byref(u), C.byref(v), C.byref(z))
    del keep
    return bool(ok), lv.value, u.value, v.value, z.value


def median_indicator(bins):
    b = np.ascontiguousarray(bins, np.uint32)
    return lib().orc_median_indicator(_ptr(b), len(b))


def mean_indicator(bins):
    b = np.ascontiguousarray(bins, np.uint32)
    return lib().orc_mean_indicator(_ptr(b), len(b))


# ---------------------------------------------------------------------- TGV ---

MODES = {"inmem": 0, "oc": 1, "stream": 2}
INITS = {"median": 0, "zero": 1, "given": 2}


def tgv_solve(cubes, hists, leaves=None, mode="inmem", alpha0=0.02, alpha1=0.04, iters=200,
              init="median", u_init=None, tol=0.0, check_every=10, fp64=False, nthreads=1, keep_init_u=False,
              level_init=None):
    """Oracle solve.  Returns (state, level_stats).  State is a STATE_DTYPE array
    (float) or an (n, 13) float64 array when fp64.  keep_init_u: levels keep
    their initial u and copy only v from the parent (warm / zero start).
    level_init (STATE_DTYPE, float solve only): every cube starts its level from
    this whole state (u, v, p, q) instead of the parent copy; until its level
    starts it holds the state `init` gives."""
    cubes = np.ascontiguousarray(cubes, CUBE_DTYPE)
    hists = np.ascontiguousarray(hists, np.uint32)
    n = len(cubes)
    nbins = hists.shape[1] if n else 8
    if leaves is None:
        leaves = np.zeros(1, LEAF_DTYPE)
        leaves["first_idx"] = 0
        leaves["last_idx"] = max(n - 1, 0)
        if n == 0:
            leaves = np.zeros(0, LEAF_DTYPE)
    leaves = np.ascontiguousarray(leaves, LEAF_DTYPE)
    p = Params(alpha0, alpha1, iters, INITS[init], tol, check_every, int(keep_init_u))
    ui = None if u_init is None else np.ascontiguousarray(u_init, np.float32)
    ls = (LevelStats * 24)()
    nls = C.c_int()
    if level_init is not None:
        assert not fp64
        li = np.ascontiguousarray(level_init, STATE_DTYPE)
        out = np.zeros(n, STATE_DTYPE)
        rc = lib().orc_tgv_solve_level_init(_ptr(cubes), _ptr(hists), C.c_int64(n), nbins, _ptr(leaves),
                                            len(leaves), MODES[mode], C.byref(p), _ptr(ui), _ptr(li), _ptr(out),
                                            ls, C.byref(nls), nthreads)
        assert rc == 0, rc
        return out, [dict(depth=ls[i].depth, iters_run=ls[i].iters_run, active=ls[i].active,
                          residual=ls[i].residual, energy=ls[i].energy) for i in range(nls.value)]
    if fp64:
        out = np.zeros((n, 13), np.float64)
        fn = lib().orc_tgv_solve_f64
    else:
        out = np.zeros(n, STATE_DTYPE)
        fn = lib().orc_tgv_solve
    rc = fn(_ptr(cubes), _ptr(hists), C.c_int64(n), nbins, _ptr(leaves), len(leaves),
            MODES[mode], C.byref(p), _ptr(ui), _ptr(out), ls, C.byref(nls), nthreads)
    assert rc == 0, rc
    stats = [dict(depth=ls[i].depth, iters_run=ls[i].iters_run, active=ls[i].active,
                  residual=ls[i].residual, energy=ls[i].energy) for i in range(nls.value)]
    return out, stats


def neighbour_table(cubes):
    """(n, 6) int32: the in-memory neighbour of every cube per face (+x, -x, +y,
    -y, +z, -z), -1 where none (the reference's neighbor_idx_ctf)."""
    cubes = np.ascontiguousarray(cubes, CUBE_DTYPE)
    nb = np.zeros((len(cubes), 6), np.int32)
    lib().orc_neighbour_table(_ptr(cubes), C.c_int64(len(cubes)), _ptr(nb))
    return nb


def stream_init(cubes, hists):
    """Initial streaming state: u = median_indicator (float, reference order), rest 0."""
    h = np.ascontiguousarray(hists, np.uint32)
    nb = h.shape[1]
    tot = h.sum(1, dtype=np.uint32)
    cum = np.cumsum(h, 1, dtype=np.uint32)
    k = np.argmax(cum * np.uint32(2) >= tot[:, None], axis=1)
    med = np.float32(-1.0) + (k.astype(np.float32) + np.float32(0.5)) / np.float32(nb / 2.0)
    st = np.zeros(len(cubes), STATE_DTYPE)
    st["u"] = np.where(tot > 0, med, np.float32(0.0))
    return st


def stream_level(cubes, hists, leaves, mask, level, params, state, nthreads=1):
    """One rank's share of one streaming level (orc_stream_level), in place.
    params: dict(alpha0, alpha1, iters)."""
    cubes = np.ascontiguousarray(cubes, CUBE_DTYPE)
    hists = np.ascontiguousarray(hists, np.uint32)
    leaves = np.ascontiguousarray(leaves, LEAF_DTYPE)
    mask = np.ascontiguousarray(mask, np.uint8)
    p = Params(params["alpha0"], params["alpha1"], params["iters"], 0, 0.0, 1)
    assert state.flags["C_CONTIGUOUS"] and state.dtype == STATE_DTYPE
    rc = lib().orc_stream_level(_ptr(cubes), _ptr(hists), C.c_int64(len(cubes)), hists.shape[1], _ptr(leaves),
                                len(leaves), _ptr(mask), level, C.byref(p), _ptr(state), nthreads)
    assert rc == 0


# ------------------------------------------------------ reference (libref) ---

def _refmap(m):
    d = RefDepthMap()
    d.fx, d.fy, d.cx, d.cy = m["fx"], m["fy"], m["cx"], m["cy"]
    d.rt[:] = [float(x) for x in np.asarray(m["rt"], np.float32).reshape(16)]
    h, w = m["depth"].shape
    d.width, d.height = w, h
    d.lidar = int(bool(m.get("lidar", False)))
    arr = np.ascontiguousarray(m["depth"], np.float32)
    d.depths = arr.ctypes.data_as(C.POINTER(C.c_float))
    return d, arr


def ref_mipmap(m):
    """Reference DepthMipmap::build -> (rt_inv 4x4, texels, dims)."""
    d, keep = _refmap(m)
    rt_inv = np.zeros(16, np.float32)
    nl = C.c_int32()
    dims = (C.c_int32 * 26)()
    total = ref().ref_mipmap_build(C.byref(d), _ptr(rt_inv), C.byref(nl), dims, None)
    tex = np.zeros(total, np.float32)
    ref().ref_mipmap_build(C.byref(d), _ptr(rt_inv), C.byref(nl), dims, _ptr(tex))
    del keep
    return rt_inv.reshape(4, 4), tex, [(dims[2 * i], dims[2 * i + 1]) for i in range(nl.value)]


def ref_compute_histograms(cubes, maps, origin, r_root):
    cubes = np.ascontiguousarray(cubes, CUBE_DTYPE)
    arr = (RefDepthMap * max(1, len(maps)))()
    keep = []
    for i, m in enumerate(maps):
        d, k = _refmap(m)
        arr[i] = d
        keep.append(k)
    out = np.zeros((len(cubes), 8), np.uint32)
    rc = ref().ref_compute_histograms(_ptr(cubes), C.c_int64(len(cubes)), arr, len(maps),
                                      C.c_float(origin[0]), C.c_float(origin[1]),
                                      C.c_float(origin[2]), C.c_float(r_root), _ptr(out))
    assert rc == 0
    return out


def ref_project(m, p, r_c):
    d, keep = _refmap(m)
    lv, u, v, z = C.c_int32(), C.c_int32(), C.c_int32(), C.c_float()
    ok = ref().ref_project(C.byref(d), C.c_float(p[0]), C.c_float(p[1]), C.c_float(p[2]),
                           C.c_float(r_c), C.byref(lv), C.byref(u), C.byref(v), C.byref(z))
    return bool(ok), lv.value, u.value, v.value, z.value


def ref_median_indicator(bins8):
    b = np.ascontiguousarray(bins8, np.uint32)
    return ref().ref_median_indicator(_ptr(b))


def ref_mean_indicator(bins8):
    b = np.ascontiguousarray(bins8, np.uint32)
    return ref().ref_mean_indicator(_ptr(b))


def ref_tgv(cubes, hists, leaves=None, mode="inmem", alpha0=0.02, alpha1=0.04, iters=200,
            r_root=1.0, tmpdir=None):
    """The reference's tgv_minimize / tgv_minimize_oc / tgv_minimize_streaming."""
    import tempfile
    from tgvreconclaude_gb300 import formats
    cubes = np.ascontiguousarray(cubes, CUBE_DTYPE)
    hists = np.ascontiguousarray(hists, np.uint32)
    assert hists.shape[1] == 8
    n = len(cubes)
    out = np.zeros(n, STATE_DTYPE)
    if mode == "inmem":
        rc = ref().ref_tgv_minimize(_ptr(cubes), _ptr(hists), C.c_int64(n), C.c_float(alpha0),
                                    C.c_float(alpha1), iters, C.c_float(r_root), _ptr(out))
        assert rc == 0
        return out
    leaves = np.ascontiguousarray(leaves, LEAF_DTYPE)
    if mode == "oc":
        rc = ref().ref_tgv_minimize_oc(_ptr(cubes), _ptr(hists), C.c_int64(n), _ptr(leaves),
                                       len(leaves), C.c_float(alpha0), C.c_float(alpha1), iters,
                                       C.c_float(r_root), _ptr(out))
        assert rc == 0
        return out
    with tempfile.TemporaryDirectory(dir=tmpdir) as td:
        cp, hp, tp, sp = (os.path.join(td, x) for x in ("c.bin", "h.bin", "t.bin", "s.bin"))
        formats.save_cubes(cp, cubes, r_root)
        formats.save_histograms(hp, hists)
        formats.save_treetop(tp, leaves, r_root)
        rc = ref().ref_tgv_minimize_streaming(cp.encode(), hp.encode(), tp.encode(),
                                              C.c_float(r_root), sp.encode(), C.c_float(alpha0),
                                              C.c_float(alpha1), iters)
        assert rc == 0
        return formats.load_state(sp)


def ref_pipeline_cubes(maps, origin, r_root, tmpdir=None):
    """Reference Stages 1-4 on base depth maps (fixture generation only):
    build_cubes_from_depthmap per map, kway_merge, balance_octree, build_treetop.
    Returns (balanced cubes, treetop leaves)."""
    import tempfile
    from tgvreconclaude_gb300 import formats
    with tempfile.TemporaryDirectory(dir=tmpdir) as td:
        paths = []
        for i, m in enumerate(maps):
            d, keep = _refmap(m)
            p = os.path.join(td, f"m{i}.cubes")
            rc = ref().ref_build_cubes_from_depthmap(C.byref(d), C.c_float(origin[0]),
                                                     C.c_float(origin[1]), C.c_float(origin[2]),
                                                     C.c_float(r_root), p.encode())
            assert rc == 0
            paths.append(p)
        arr = (C.c_char_p * len(paths))(*[p.encode() for p in paths])
        merged, bal, tt = (os.path.join(td, x) for x in ("m.cubes", "b.cubes", "t.bin"))
        assert ref().ref_kway_merge(arr, len(paths), merged.encode()) == 0
        assert ref().ref_balance_octree(merged.encode(), bal.encode()) == 0
        assert ref().ref_build_treetop(bal.encode(), tt.encode()) == 0
        cubes, _ = formats.load_cubes(bal)
        leaves, _ = formats.load_treetop(tt)
        return cubes, leaves


__all__ = ["build", "lib", "ref", "ref_available", "compute_histograms", "pyramid",
           "pyramid_dims", "project", "median_indicator", "mean_indicator", "tgv_solve",
           "ref_mipmap", "ref_compute_histograms", "ref_project", "ref_median_indicator",
           "ref_mean_indicator", "ref_tgv", "ref_pipeline_cubes", "cube_keys"]


# ------------------------------------------------------- surface extraction ---

def _mesh_out(L, h, nv, nf, normals, prefix):
    if not h:
        raise RuntimeError(f"{prefix}extract_surface failed")
    v = np.zeros((nv, 3), np.float32)
    f = np.zeros((nf, 3), np.uint32)
    nr = np.zeros((nv, 3), np.float32) if normals else None
    getattr(L, prefix + "mesh_read")(C.c_void_p(h), _ptr(v), _ptr(f), _ptr(nr))
    getattr(L, prefix + "mesh_free")(C.c_void_p(h))
    return v, f, nr


def _surface_args(cubes, state, has_data):
    cubes = np.ascontiguousarray(cubes, CUBE_DTYPE)
    state = np.ascontiguousarray(state, STATE_DTYPE)
    hd = None if has_data is None else np.ascontiguousarray(has_data, np.uint8)
    return cubes, state, hd


def extract_surface(cubes, state, origin, r_root, has_data=None, normals=False):
    """Oracle extract_surface (+ compute_normals): (verts (nv,3), faces (nf,3), normals or None)."""
    cubes, state, hd = _surface_args(cubes, state, has_data)
    L = lib()
    L.orc_extract_surface.restype = C.c_void_p
    o = np.ascontiguousarray(origin, np.float32)
    nv, nf = C.c_int64(), C.c_int64()
    h = L.orc_extract_surface(_ptr(cubes), _ptr(state), C.c_int64(len(cubes)), _ptr(hd), _ptr(o),
                              C.c_float(r_root), int(normals), C.byref(nv), C.byref(nf))
    return _mesh_out(L, h, nv.value, nf.value, normals, "orc_")


def extract_surface_streaming(cubes, state, hists, leaves, origin, r_root):
    """Oracle extract_surface_streaming held in memory: (verts (nv,3) dequantised, faces (nf,3))."""
    cubes, state, _ = _surface_args(cubes, state, None)
    tot = np.ascontiguousarray(np.asarray(hists, np.uint32).sum(1, dtype=np.uint32))
    lv = np.ascontiguousarray(leaves, LEAF_DTYPE)
    L = lib()
    L.orc_extract_surface_streaming.restype = C.c_void_p
    o = np.ascontiguousarray(origin, np.float32)
    nv, nf = C.c_int64(), C.c_int64()
    h = L.orc_extract_surface_streaming(_ptr(cubes), _ptr(state), _ptr(tot), C.c_int64(len(cubes)), _ptr(lv),
                                        len(lv), _ptr(o), C.c_float(r_root), C.byref(nv), C.byref(nf))
    v, f, _ = _mesh_out(L, h, nv.value, nf.value, False, "orc_")
    return v, f


def ref_extract_surface(cubes, state, origin, r_root, has_data=None, normals=False):
    """The reference's extract_surface (+ compute_normals) through libref."""
    cubes, state, hd = _surface_args(cubes, state, has_data)
    R = ref()
    R.ref_extract_surface.restype = C.c_void_p
    nv, nf = C.c_int64(), C.c_int64()
    h = R.ref_extract_surface(_ptr(cubes), _ptr(state), C.c_int64(len(cubes)), _ptr(hd),
                              C.c_float(origin[0]), C.c_float(origin[1]), C.c_float(origin[2]),
                              C.c_float(r_root), int(normals), C.byref(nv), C.byref(nf))
    return _mesh_out(R, h, nv.value, nf.value, normals, "ref_")


def ref_extract_surface_streaming(cube_path, state_path, treetop_path, hist_path, origin, r_root, out_obj):
    """The reference's extract_surface_streaming (files in, .obj out)."""
    rc = ref().ref_extract_surface_streaming(str(cube_path).encode(), str(state_path).encode(),
                                              str(treetop_path).encode(), str(hist_path).encode(),
                                              C.c_float(origin[0]), C.c_float(origin[1]), C.c_float(origin[2]),
                                              C.c_float(r_root), str(out_obj).encode())
    assert rc == 0, rc


def obj_text(verts, faces, normals=None):
    """Wavefront text as the reference writes it (write_obj / the streaming
    aggregator: `v x y z` with the stream's default 6-digit %g formatting,
    `vn` lines and `f a//a b//b c//c` when there are normals, else 1-based
    `f a b c`)."""
    out = ["v %g %g %g\n" % (float(x), float(y), float(z)) for x, y, z in np.asarray(verts, np.float32)]
    if normals is not None:
        out += ["vn %g %g %g\n" % (float(x), float(y), float(z)) for x, y, z in np.asarray(normals, np.float32)]
        out += ["f %d//%d %d//%d %d//%d\n" % (a + 1, a + 1, b + 1, b + 1, c + 1, c + 1)
                for a, b, c in np.asarray(faces, np.int64)]
    else:
        out += ["f %d %d %d\n" % (a + 1, b + 1, c + 1) for a, b, c in np.asarray(faces, np.int64)]
    return "".join(out)


# ------------------------------------------------------------------ Stage 1 ---

class DepthMapO(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("rt", C.c_float * 16), ("width", C.c_int32), ("height", C.c_int32),
                ("depths", C.POINTER(C.c_float))]


def _dmo(m):
    d = DepthMapO()
    d.fx, d.fy, d.cx, d.cy = m["fx"], m["fy"], m["cx"], m["cy"]
    d.rt[:] = [float(x) for x in np.asarray(m["rt"], np.float32).reshape(16)]
    arr = np.ascontiguousarray(m["depth"], np.float32)
    d.height, d.width = arr.shape
    d.depths = arr.ctypes.data_as(C.POINTER(C.c_float))
    return d, arr


def build_cubes(m, origin, r_root):
    """Oracle build_cubes_from_depthmap: cubes in code order, ties in pixel order."""
    d, keep = _dmo(m)
    o = np.ascontiguousarray(origin, np.float32)
    L = lib()
    L.orc_build_cubes.restype = C.c_int64
    n = L.orc_build_cubes(C.byref(d), _ptr(o), C.c_float(r_root), None, C.c_int64(0))
    out = np.zeros(n, CUBE_DTYPE)
    L.orc_build_cubes(C.byref(d), _ptr(o), C.c_float(r_root), _ptr(out), C.c_int64(n))
    return out


def ref_build_cubes(m, origin, r_root, tmpdir=None):
    """The reference's build_cubes_from_depthmap (through its TGV1 file)."""
    import tempfile
    from tgvreconclaude_gb300 import formats
    d, keep = _refmap(m)
    with tempfile.TemporaryDirectory(dir=tmpdir) as td:
        p = os.path.join(td, "c.bin")
        rc = ref().ref_build_cubes_from_depthmap(C.byref(d), C.c_float(origin[0]), C.c_float(origin[1]),
                                                 C.c_float(origin[2]), C.c_float(r_root), p.encode())
        assert rc == 0
        cubes, _ = formats.load_cubes(p)
    return cubes


def cube_multiset(cubes):
    """Cubes sorted by (code, depth, r_c bits): order-free comparison key."""
    c = np.ascontiguousarray(cubes, CUBE_DTYPE)
    rc_bits = c["r_c"].view(np.uint32)
    order = np.lexsort((rc_bits, c["depth"], c["lo"], c["hi"]))
    return c[order]


# ------------------------------------------------- Stages 2 and 3 (merge, balance) ---

def merge_cubes(arrays):
    """Oracle merge of sorted cube arrays (stable in input order for equal codes)."""
    arrs = [np.ascontiguousarray(a, CUBE_DTYPE) for a in arrays]
    ptrs = (C.c_void_p * max(1, len(arrs)))(*[a.ctypes.data if len(a) else None for a in arrs])
    ns = np.array([len(a) for a in arrs] or [0], np.int64)
    L = lib()
    L.orc_merge_cubes.restype = C.c_int64
    n = L.orc_merge_cubes(ptrs, _ptr(ns), len(arrs), None, C.c_int64(0))
    out = np.zeros(n, CUBE_DTYPE)
    L.orc_merge_cubes(ptrs, _ptr(ns), len(arrs), _ptr(out), C.c_int64(n))
    return out


def ref_merge_cubes(arrays, r_root, tmpdir=None):
    """The reference's kway_merge over TGV1 files holding the arrays."""
    import tempfile
    from tgvreconclaude_gb300 import formats
    with tempfile.TemporaryDirectory(dir=tmpdir) as td:
        paths = []
        for i, a in enumerate(arrays):
            p = os.path.join(td, f"in{i}.cubes")
            formats.save_cubes(p, a, r_root)
            paths.append(p)
        out = os.path.join(td, "out.cubes")
        arr = (C.c_char_p * max(1, len(paths)))(*[p.encode() for p in paths])
        assert ref().ref_kway_merge(arr, len(paths), out.encode()) == 0
        cubes, rr = formats.load_cubes(out)
    return cubes


def balance_cubes(cubes, r_root):
    """Oracle 2:1 balance (output sorted by code, then depth)."""
    c = np.ascontiguousarray(cubes, CUBE_DTYPE)
    L = lib()
    L.orc_balance_cubes.restype = C.c_int64
    n = L.orc_balance_cubes(_ptr(c), C.c_int64(len(c)), C.c_float(r_root), None, C.c_int64(0))
    out = np.zeros(n, CUBE_DTYPE)
    L.orc_balance_cubes(_ptr(c), C.c_int64(len(c)), C.c_float(r_root), _ptr(out), C.c_int64(n))
    return out


def ref_balance_cubes(cubes, r_root, tmpdir=None):
    """The reference's balance_octree through TGV1 files."""
    import tempfile
    from tgvreconclaude_gb300 import formats
    with tempfile.TemporaryDirectory(dir=tmpdir) as td:
        p, q = os.path.join(td, "in.cubes"), os.path.join(td, "out.cubes")
        formats.save_cubes(p, cubes, r_root)
        assert ref().ref_balance_octree(p.encode(), q.encode()) == 0
        out, _ = formats.load_cubes(q)
    return out
