"""Python mirror of the reference's Stage-5/6 interface (src/histogram.hpp,
src/tgv.hpp) over the sm_103a C ABI (include/tgvg.h).

Same names, same argument meaning, same error behaviour: a failing call raises
``RuntimeError`` where the reference throws ``std::runtime_error``, and empty
inputs return empty results.  Arrays use the byte-exact record dtypes of
:mod:`tgvreconclaude_gb300.formats`.  All compute runs on the GPU; there is no
CPU path.
"""
from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from . import formats as F


# ------------------------------------------------------------------ context ---

TGVG_ERR_LIMIT = -10


class Context:
    """One CUDA stream + buffer pool on one device (tgvg_create)."""

    def __init__(self, device: int = 0):
        self.lib = N.lib()
        h = C.c_void_p()
        rc = self.lib.tgvg_create(device, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"tgvg_create: {self.lib.tgvg_strerror(rc).decode()}")
        self.h = h

    def check(self, rc: int, what: str):
        if rc < 0:
            detail = self.lib.tgvg_last_error(self.h).decode()
            raise RuntimeError(f"{what}: {self.lib.tgvg_strerror(rc).decode()}"
                               + (f" ({detail})" if detail else ""))
        return rc

    @property
    def stream(self) -> int:
        return self.lib.tgvg_stream(self.h) or 0

    def set_graphs(self, on: bool) -> None:
        """CUDA graphs for the level loop (default on; tgvg_set_graphs)."""
        self.check(self.lib.tgvg_set_graphs(self.h, int(bool(on))), "tgvg_set_graphs")

    def set_schedule(self, mode: str, cls: int, cfg: int) -> None:
        """Fix the iteration schedule of a size class (tgvg_set_schedule)."""
        self.check(self.lib.tgvg_set_schedule(self.h, MODES[mode], cls, cfg), "tgvg_set_schedule")

    def kernel_count(self) -> int:
        return self.lib.tgvg_kernel_count(self.h)

    def close(self):
        if self.h:
            self.lib.tgvg_destroy(self.h)
            self.h = None


_ctx = None
_ctx_lock = threading.Lock()


def context() -> Context:
    global _ctx
    with _ctx_lock:
        if _ctx is None:
            _ctx = Context(0)
    return _ctx


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None and a.size else None


# ------------------------------------------------------------- depth maps ---

@dataclass
class DepthMap:
    """DepthMap (reference src/depth_map.hpp:7-25): row-major depths, NaN = invalid."""
    width: int
    height: int
    depths: np.ndarray
    K: np.ndarray = field(default_factory=lambda: np.eye(3, dtype=np.float32))
    Rt: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))


# ---------------------------------------------------------------- Stage 1 ---

def _depthmap_struct(dm):
    """A DepthMap, or a dict with depth/rt/fx/fy/cx/cy, as the C struct (plus
    the array that must stay alive while it is used)."""
    if isinstance(dm, DepthMap):
        depth = np.ascontiguousarray(np.asarray(dm.depths, np.float32).reshape(dm.height, dm.width))
        K = np.asarray(dm.K, np.float32)
        fx, fy, cx, cy, rt = K[0, 0], K[1, 1], K[0, 2], K[1, 2], dm.Rt
    else:
        depth = np.ascontiguousarray(dm["depth"], np.float32)
        fx, fy, cx, cy, rt = dm["fx"], dm["fy"], dm["cx"], dm["cy"], dm["rt"]
    s = N.DepthMapS()
    s.fx, s.fy, s.cx, s.cy = float(fx), float(fy), float(cx), float(cy)
    s.rt[:] = [float(x) for x in np.asarray(rt, np.float32).reshape(16)]
    s.height, s.width = depth.shape
    s.depths = depth.ctypes.data_as(C.POINTER(C.c_float))
    return s, depth


def build_cubes(dm, scene_origin, r_root) -> np.ndarray:
    """build_cubes_from_depthmap (reference src/octree_builder.hpp:21-29) on the
    GPU: one cube per valid pixel, sorted by Morton code, equal codes in pixel
    order.  ``dm`` is a DepthMap or a dict (depth, rt, fx, fy, cx, cy)."""
    ctx = context()
    s, keep = _depthmap_struct(dm)
    o = np.ascontiguousarray(scene_origin, np.float32)
    n = C.c_int64(0)
    out = np.empty(keep.size, F.CUBE_DTYPE)  # at most one cube per pixel
    ctx.check(ctx.lib.tgvg_build_cubes(ctx.h, C.byref(s), _p(o), C.c_float(r_root), _p(out), len(out), C.byref(n)),
              "tgvg_build_cubes")
    return out[: n.value].copy()


def build_cubes_file(dm, scene_origin, r_root, out_path) -> None:
    """The same, written as a TGV1 cube file (reference src/octree_io.hpp)."""
    ctx = context()
    s, keep = _depthmap_struct(dm)
    o = np.ascontiguousarray(scene_origin, np.float32)
    ctx.check(ctx.lib.tgvg_build_cubes_file(ctx.h, C.byref(s), _p(o), C.c_float(r_root), str(out_path).encode()),
              "tgvg_build_cubes_file")


# ------------------------------------------------------- Stages 2 and 3 ---

def merge_cubes(arrays) -> np.ndarray:
    """kway_merge (reference src/merge.hpp:6-8) over code-sorted cube arrays on
    the GPU: merged by code (equal codes in array order), consecutive equal
    (code, depth) collapsed with the mean r_c."""
    ctx = context()
    arrs = [np.ascontiguousarray(a, F.CUBE_DTYPE) for a in arrays]
    ptrs = (C.c_void_p * max(1, len(arrs)))(*[a.ctypes.data if len(a) else None for a in arrs])
    ns = np.array([len(a) for a in arrs] or [0], np.int64)
    n = C.c_int64(0)
    out = np.empty(int(ns.sum()), F.CUBE_DTYPE)  # the merge never grows the list
    ctx.check(ctx.lib.tgvg_merge_cubes(ctx.h, ptrs, _p(ns), len(arrs), _p(out), len(out), C.byref(n)),
              "tgvg_merge_cubes")
    return out[: n.value].copy()


def kway_merge(in_paths, out_path) -> None:
    """The file form (reference kway_merge(in_paths, out_path))."""
    ctx = context()
    arr = (C.c_char_p * max(1, len(in_paths)))(*[str(p).encode() for p in in_paths])
    ctx.check(ctx.lib.tgvg_kway_merge(ctx.h, arr, len(in_paths), str(out_path).encode()), "tgvg_kway_merge")


def balance_cubes(cubes, r_root) -> np.ndarray:
    """balance_octree (reference src/balance.hpp:15-16) on the GPU over a cube
    array: the reference's bridge cubes and output table, sorted by code then
    depth."""
    ctx = context()
    c = np.ascontiguousarray(cubes, F.CUBE_DTYPE)
    n = C.c_int64(0)
    out = np.empty(4 * len(c) + 4096, F.CUBE_DTYPE)
    rc = ctx.lib.tgvg_balance_cubes(ctx.h, _p(c), len(c), C.c_float(r_root), _p(out), len(out), C.byref(n))
    if rc == TGVG_ERR_LIMIT:  # more bridges than the first guess: run again with the exact size
        out = np.empty(n.value, F.CUBE_DTYPE)
        rc = ctx.lib.tgvg_balance_cubes(ctx.h, _p(c), len(c), C.c_float(r_root), _p(out), len(out), C.byref(n))
    ctx.check(rc, "tgvg_balance_cubes")
    return out[: n.value].copy()


def balance_octree(in_path, out_path) -> None:
    """The file form (reference balance_octree(in_path, out_path))."""
    ctx = context()
    ctx.check(ctx.lib.tgvg_balance_octree(ctx.h, str(in_path).encode(), str(out_path).encode()),
              "tgvg_balance_octree")


# ---------------------------------------------------------------- Stage 5 ---

class DepthMipmap:
    """DepthMipmap (reference src/histogram.hpp:22-38).  ``build`` runs on the GPU."""

    def __init__(self):
        self.levels: list[np.ndarray] = []
        self.dims: list[tuple[int, int]] = []
        self.Rt_inv = np.eye(4, dtype=np.float32)
        self.K = np.eye(3, dtype=np.float32)
        self.lidar = False

    def build(self, base: DepthMap, is_lidar: bool = False) -> "DepthMipmap":
        self.lidar = bool(is_lidar)
        self.K = np.asarray(base.K, np.float32)
        # The reference inverts with Eigen; any accurate inverse serves since
        # the same matrix then feeds both the GPU and any parity check.
        self.Rt_inv = np.linalg.inv(np.asarray(base.Rt, np.float64)).astype(np.float32)
        cam = camera_struct(self)
        cam.width, cam.height = base.width, base.height
        ctx = context()
        dims = (C.c_int32 * 26)()
        nl = ctx.check(ctx.lib.tgvg_pyramid_dims(base.width, base.height, dims), "pyramid_dims")
        self.dims = [(dims[2 * i], dims[2 * i + 1]) for i in range(nl)]
        total = sum(w * h for w, h in self.dims)
        out = np.empty(total, np.float32)
        src = np.ascontiguousarray(base.depths, np.float32).reshape(-1)
        basep = (C.c_void_p * 1)(src.ctypes.data)
        outp = (C.c_void_p * 1)(out.ctypes.data)
        ctx.check(ctx.lib.tgvg_build_pyramids(ctx.h, C.byref(cam), 1, basep, outp), "DepthMipmap::build")
        self.levels, off = [], 0
        for w, h in self.dims:
            self.levels.append(out[off:off + w * h].reshape(h, w))
            off += w * h
        self._flat = out
        return self

    @property
    def width(self):
        return self.dims[0][0]

    @property
    def height(self):
        return self.dims[0][1]

    def project(self, P, r_c):
        """Host mirror of DepthMipmap::project (histogram.cpp:76-106), float32
        arithmetic in the reference's order.  Returns (ok, level, u, v, cam_z)."""
        if not self.levels:
            return False, 0, 0, 0, 0.0
        f = np.float32
        m = self.Rt_inv.astype(f)
        p = [f(P[0]), f(P[1]), f(P[2]), f(1.0)]
        cam = []
        for r in range(3):
            acc = f(m[r, 0] * p[0])
            for k in range(1, 4):
                acc = f(acc + f(m[r, k] * p[k]))
            cam.append(acc)
        z = cam[2]
        if z <= 0:
            return False, 0, 0, 0, 0.0
        fx, fy, cx, cy = f(self.K[0, 0]), f(self.K[1, 1]), f(self.K[0, 2]), f(self.K[1, 2])
        with np.errstate(all="ignore"):
            u_f = f(f(f(cam[0] / z) * fx) + cx)
            v_f = f(f(f(cam[1] / z) * fy) + cy)
        u0, v0 = _trunc(u_f), _trunc(v_f)
        if u0 < 0 or u0 >= self.width or v0 < 0 or v0 >= self.height:
            return False, 0, 0, 0, 0.0
        with np.errstate(all="ignore"):
            fp = f(f(abs(fx) * f(r_c)) / z)
            lv = max(0, _trunc(np.log2(f(fp) if f(1.0) < fp else f(1.0))))
        lv = min(lv, len(self.levels) - 1)
        w, h = self.dims[lv]
        return True, lv, min(max(u0 >> lv, 0), w - 1), min(max(v0 >> lv, 0), h - 1), float(z)

    def depth_at(self, level, u, v):
        if level < 0 or level >= len(self.levels):
            return float("nan")
        w, h = self.dims[level]
        if u < 0 or u >= w or v < 0 or v >= h:
            return float("nan")
        return float(self.levels[level][v, u])


def _trunc(x) -> int:
    x = float(x)
    if not (-2147483904.0 < x < 2147483648.0):
        return -(2 ** 31)
    return int(x)


def camera_struct(mm: DepthMipmap) -> N.Camera:
    c = N.Camera()
    c.rt_inv[:] = [float(v) for v in np.asarray(mm.Rt_inv, np.float32).reshape(16)]
    K = np.asarray(mm.K, np.float32)
    c.fx, c.fy, c.cx, c.cy = float(K[0, 0]), float(K[1, 1]), float(K[0, 2]), float(K[1, 2])
    if mm.dims:
        c.width, c.height = mm.dims[0]
    c.lidar = int(mm.lidar)
    return c


def _cams(depth_maps):
    arr = (N.Camera * max(1, len(depth_maps)))()
    for i, m in enumerate(depth_maps):
        arr[i] = camera_struct(m)
    return arr


def compute_histograms(cubes, depth_maps, scene_origin, r_root, nbins: int = 8) -> np.ndarray:
    """compute_histograms (reference src/histogram.hpp:44-48) on the GPU.
    Returns (n, nbins) uint32; bit-exact with the reference at nbins = 8."""
    ctx = context()
    cubes = np.ascontiguousarray(cubes, F.CUBE_DTYPE)
    out = np.zeros((len(cubes), nbins), np.uint32)
    if len(cubes) == 0:
        return out
    lv = (C.c_void_p * max(1, len(depth_maps)))(*[m._flat.ctypes.data for m in depth_maps])
    o = np.asarray(scene_origin, np.float32)
    ctx.check(ctx.lib.tgvg_compute_histograms_pyr(ctx.h, _p(cubes), len(cubes), _cams(depth_maps),
                                                  len(depth_maps), lv, _p(o), float(r_root), nbins, _p(out)),
              "compute_histograms")
    return out


def compute_histograms_from_maps(cubes, cams, bases, scene_origin, r_root, nbins: int = 8) -> np.ndarray:
    """Histograms straight from level-0 maps (pyramids built on the device).
    cams: sequence of N.Camera; bases: sequence of (H, W) float32 arrays."""
    ctx = context()
    cubes = np.ascontiguousarray(cubes, F.CUBE_DTYPE)
    out = np.empty((len(cubes), nbins), np.uint32)
    if len(cubes) == 0:
        return out
    bases = [np.ascontiguousarray(b, np.float32) for b in bases]
    arr = (N.Camera * max(1, len(cams)))(*cams)
    bp = (C.c_void_p * max(1, len(bases)))(*[b.ctypes.data for b in bases])
    o = np.asarray(scene_origin, np.float32)
    ctx.check(ctx.lib.tgvg_compute_histograms(ctx.h, _p(cubes), len(cubes), arr, len(cams), bp, _p(o),
                                              float(r_root), nbins, _p(out)), "compute_histograms")
    return out


def compute_histograms_oc(balanced_cube_path, leaves, depth_maps, scene_origin, r_root, out_hist_path):
    """compute_histograms_oc (reference src/histogram.hpp:55-61)."""
    ctx = context()
    leaves = np.ascontiguousarray(leaves, F.LEAF_DTYPE)
    bases = [np.ascontiguousarray(m.levels[0], np.float32) for m in depth_maps]
    bp = (C.c_void_p * max(1, len(bases)))(*[b.ctypes.data for b in bases])
    o = np.asarray(scene_origin, np.float32)
    ctx.check(ctx.lib.tgvg_compute_histograms_oc(ctx.h, str(balanced_cube_path).encode(), _p(leaves),
                                                 len(leaves), _cams(depth_maps), len(depth_maps), bp, _p(o),
                                                 float(r_root), str(out_hist_path).encode()),
              "compute_histograms_oc")


# ---------------------------------------------------------------- Stage 6 ---

@dataclass
class TGVParams:
    """TGVParams (reference src/tgv.hpp:24-28) plus the stopping extension."""
    alpha0: float = 0.02
    alpha1: float = 0.04
    iters: int = 200
    init: str = "median"       # "median" (reference), "zero", "given", "state" (whole-state start per level)
    tol: float = 0.0           # relative residual stop; 0 = fixed iteration count
    check_every: int = 10
    keep_init_u: bool = False  # True: every level keeps its initial u (warm / zero start), copies only v

    def struct(self) -> N.Params:
        return N.Params(self.alpha0, self.alpha1, self.iters,
                        {"median": 0, "zero": 1, "given": 2, "state": 3}[self.init],
                        self.tol, self.check_every, int(self.keep_init_u))


MODES = {"inmem": 0, "oc": 1, "stream": 2}


def tgv_solve(cubes, hists, leaves=None, mode="inmem", params: TGVParams | None = None, u_init=None,
              state_init=None):
    """Generic solve over host arrays -> (state (n,) STATE_DTYPE, stats dict).
    state_init (STATE_DTYPE): whole-state warm start, every cube starts its
    level from its record (params.init is taken as "state")."""
    ctx = context()
    params = params or TGVParams()
    cubes = np.ascontiguousarray(cubes, F.CUBE_DTYPE)
    hists = np.ascontiguousarray(hists, np.uint32)
    n = len(cubes)
    nbins = hists.shape[1] if hists.ndim == 2 else 8
    out = np.zeros(n, F.STATE_DTYPE)
    lv = None if leaves is None else np.ascontiguousarray(leaves, F.LEAF_DTYPE)
    ui = None if u_init is None else np.ascontiguousarray(u_init, np.float32)
    st = N.Stats()
    if state_init is not None:
        si = np.ascontiguousarray(state_init, F.STATE_DTYPE)
        prm = TGVParams(**{**params.__dict__, "init": "state"}).struct()
        ctx.check(ctx.lib.tgvg_tgv_minimize_state(ctx.h, _p(cubes), _p(hists), n, nbins, _p(lv),
                                                  0 if lv is None else len(lv), MODES[mode], C.byref(prm), _p(si),
                                                  _p(out), C.byref(st)), "tgv_minimize_state")
        return out, st.as_dict()
    prm = params.struct()
    ctx.check(ctx.lib.tgvg_tgv_minimize(ctx.h, _p(cubes), _p(hists), n, nbins, _p(lv),
                                        0 if lv is None else len(lv), MODES[mode], C.byref(prm), _p(ui), _p(out),
                                        C.byref(st)), "tgv_minimize")
    return out, st.as_dict()


def tgv_minimize(cubes, hists, origin=None, r_root=1.0, params: TGVParams | None = None):
    """tgv_minimize (reference src/tgv.hpp:31-36)."""
    return tgv_solve(cubes, hists, None, "inmem", params)[0]


def tgv_minimize_oc(cubes, hists, leaves, origin=None, r_root=1.0, params: TGVParams | None = None):
    """tgv_minimize_oc (reference src/tgv.hpp:42-48)."""
    return tgv_solve(cubes, hists, leaves, "oc", params)[0]


def tgv_minimize_streaming(balanced_cube_path, hist_path, treetop_path, origin, r_root, out_state_path,
                           params: TGVParams | None = None):
    """tgv_minimize_streaming (reference src/tgv.hpp:57-64): files in, TGVS out."""
    ctx = context()
    prm = (params or TGVParams()).struct()
    st = N.Stats()
    ctx.check(ctx.lib.tgvg_tgv_minimize_streaming(ctx.h, str(balanced_cube_path).encode(), str(hist_path).encode(),
                                                  str(treetop_path).encode(), str(out_state_path).encode(),
                                                  C.byref(prm), C.byref(st)), "tgv_minimize_streaming")
    return st.as_dict()


def tgv_solve_device(cubes_t, hists_t, out_t, leaves=None, mode="inmem", params: TGVParams | None = None,
                     u_init_t=None, state_init_t=None):
    """Device-resident solve: torch CUDA tensors in and out (cubes (n,4) int32
    view of the records, hists (n,nbins) int32/uint32, out (n,13) float32).
    state_init_t ((n,13) float32): whole-state warm start."""
    ctx = context()
    params = params or TGVParams()
    n = cubes_t.shape[0]
    nbins = hists_t.shape[1]
    lv = None if leaves is None else np.ascontiguousarray(leaves, F.LEAF_DTYPE)
    st = N.Stats()
    if state_init_t is not None:
        prm = TGVParams(**{**params.__dict__, "init": "state"}).struct()
        ctx.check(ctx.lib.tgvg_tgv_minimize_state_dev(ctx.h, cubes_t.data_ptr(), hists_t.data_ptr(), n, nbins,
                                                      _p(lv), 0 if lv is None else len(lv), MODES[mode],
                                                      C.byref(prm), state_init_t.data_ptr(), out_t.data_ptr(),
                                                      C.byref(st)), "tgv_minimize_state_dev")
        return st.as_dict()
    prm = params.struct()
    ctx.check(ctx.lib.tgvg_tgv_minimize_dev(ctx.h, cubes_t.data_ptr(), hists_t.data_ptr(), n, nbins, _p(lv),
                                            0 if lv is None else len(lv), MODES[mode], C.byref(prm),
                                            None if u_init_t is None else u_init_t.data_ptr(), out_t.data_ptr(),
                                            C.byref(st)), "tgv_minimize_dev")
    return st.as_dict()


# --------------------------------------------------------------------- I/O ---

def save_tgv(path, state):
    return F.save_state(path, state)


def load_tgv(path):
    return F.load_state(path)


def save_histograms(path, hists):
    return F.save_histograms(path, hists)


def load_histograms(path):
    return F.load_histograms(path)


def load_histograms_range(path, first_idx, last_idx):
    h = F.load_histograms(path)
    if first_idx >= len(h) or first_idx > last_idx:
        return h[:0]
    return h[first_idx:min(last_idx + 1, len(h))]


# ------------------------------------------------------ surface extraction ---

def _take_mesh(ctx, h):
    nv, nf, hn = C.c_int64(), C.c_int64(), C.c_int32()
    ctx.check(ctx.lib.tgvg_mesh_size(h, C.byref(nv), C.byref(nf), C.byref(hn)), "tgvg_mesh_size")
    v = np.zeros((nv.value, 3), np.float32)
    f = np.zeros((nf.value, 3), np.uint32)
    nrm = np.zeros((nv.value, 3), np.float32) if hn.value else None
    ctx.check(ctx.lib.tgvg_mesh_read(h, _p(v), _p(f), _p(nrm)), "tgvg_mesh_read")
    ctx.lib.tgvg_mesh_free(h)
    return v, f, nrm


def extract_surface(cubes, state, origin, r_root, has_data=None, normals=False):
    """extract_surface (reference src/marching_cubes.hpp:28-33) on the GPU,
    followed by compute_normals when normals=True.  Returns (verts (nv, 3)
    float32, faces (nf, 3) uint32, normals (nv, 3) or None)."""
    ctx = context()
    cubes = np.ascontiguousarray(cubes, F.CUBE_DTYPE)
    state = np.ascontiguousarray(state, F.STATE_DTYPE)
    hd = None if has_data is None else np.ascontiguousarray(has_data, np.uint8)
    o = np.ascontiguousarray(origin, np.float32)
    h = C.c_void_p()
    ctx.check(ctx.lib.tgvg_extract_surface(ctx.h, _p(cubes), _p(state), len(cubes), _p(hd), _p(o), C.c_float(r_root),
                                           int(bool(normals)), C.byref(h)), "tgvg_extract_surface")
    return _take_mesh(ctx, h)


def extract_surface_leaves(cubes, state, hists, leaves, origin, r_root):
    """The streaming extraction's semantics (reference marching_cubes.cpp:374-580)
    over arrays: returns (verts dequantised (nv, 3), faces (nf, 3))."""
    ctx = context()
    cubes = np.ascontiguousarray(cubes, F.CUBE_DTYPE)
    state = np.ascontiguousarray(state, F.STATE_DTYPE)
    hists = np.ascontiguousarray(hists, np.uint32)
    lv = np.ascontiguousarray(leaves, F.LEAF_DTYPE)
    o = np.ascontiguousarray(origin, np.float32)
    h = C.c_void_p()
    ctx.check(ctx.lib.tgvg_extract_surface_leaves(ctx.h, _p(cubes), _p(state), _p(hists),
                                                  hists.shape[1] if hists.ndim == 2 else 8, len(cubes), _p(lv),
                                                  len(lv), _p(o), C.c_float(r_root), C.byref(h)),
              "tgvg_extract_surface_leaves")
    v, f, _ = _take_mesh(ctx, h)
    return v, f


def extract_surface_streaming(balanced_cube_path, tgv_state_path, treetop_path, hist_path, origin, r_root,
                              out_obj_path):
    """extract_surface_streaming (reference src/marching_cubes.hpp:44-51): files in, .obj out."""
    ctx = context()
    o = np.ascontiguousarray(origin, np.float32)
    ctx.check(ctx.lib.tgvg_extract_surface_streaming(ctx.h, str(balanced_cube_path).encode(),
                                                     str(tgv_state_path).encode(), str(treetop_path).encode(),
                                                     str(hist_path).encode(), _p(o), C.c_float(r_root),
                                                     str(out_obj_path).encode()), "tgvg_extract_surface_streaming")


def compute_normals(verts, faces):
    """compute_normals (reference src/marching_cubes.hpp:55) on the GPU."""
    ctx = context()
    v = np.ascontiguousarray(verts, np.float32)
    f = np.ascontiguousarray(faces, np.uint32)
    nrm = np.zeros_like(v)
    ctx.check(ctx.lib.tgvg_compute_normals(ctx.h, _p(v), len(v), _p(f), len(f), _p(nrm)), "tgvg_compute_normals")
    return nrm


def write_obj(path, verts, faces, normals=None):
    """write_obj (reference src/marching_cubes.hpp:58)."""
    v = np.ascontiguousarray(verts, np.float32)
    f = np.ascontiguousarray(faces, np.uint32)
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
    rc = N.lib().tgvg_write_obj(str(path).encode(), _p(v), len(v), _p(f), len(f), _p(nrm))
    if rc:
        raise RuntimeError(f"write_obj: {N.lib().tgvg_strerror(rc).decode()}")
