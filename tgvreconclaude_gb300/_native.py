"""Build and load the sm_103a library (``lib/libtgvg.so``) behind include/tgvg.h.

The library is compiled in-tree with nvcc for ``sm_103a`` only (one
``-gencode``); translation units are compiled in parallel and linked into one
shared object with plain C entry points.  There is no fallback: if the library
cannot be loaded, or no sm_103 device is present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libtgvg.so")
SOURCES = ["capi.cu", "hist.cu", "tgv.cu", "mlp.cu", "surface.cu", "prep.cu", "octree.cu"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "tgvg.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.isfile(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link libtgvg.so."""
    if not force and not _stale():
        return LIB
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)

    def one(src):
        obj = os.path.join(objdir, src.replace(".cu", ".o"))
        cmd = [NVCC, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        res = list(ex.map(one, SOURCES))
    if verbose:
        for _, err in res:
            print(err)
    tmp = LIB + ".tmp"
    r = subprocess.run([NVCC, *ARCH, "-shared", "-o", tmp, *[o for o, _ in res]], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


# ------------------------------------------------------------------ ABI ---

class Cube(C.Structure):
    _fields_ = [("hi", C.c_uint32), ("lo", C.c_uint32), ("r_c", C.c_float), ("depth", C.c_int32)]


class Leaf(C.Structure):
    _fields_ = [("hi", C.c_uint32), ("lo", C.c_uint32), ("depth", C.c_int32),
                ("first_idx", C.c_uint32), ("last_idx", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("rt_inv", C.c_float * 16), ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float),
                ("cy", C.c_float), ("width", C.c_int32), ("height", C.c_int32), ("lidar", C.c_int32),
                ("reserved", C.c_int32)]


class DepthMapS(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
                ("rt", C.c_float * 16), ("width", C.c_int32), ("height", C.c_int32),
                ("depths", C.POINTER(C.c_float))]


class Params(C.Structure):
    _fields_ = [("alpha0", C.c_float), ("alpha1", C.c_float), ("iters", C.c_int32), ("init", C.c_int32),
                ("tol", C.c_float), ("check_every", C.c_int32), ("keep_init_u", C.c_int32)]


MAX_LEVELS = 22


class Stats(C.Structure):
    _fields_ = [("n_levels", C.c_int32), ("min_depth", C.c_int32), ("max_depth", C.c_int32),
                ("depth", C.c_int32 * MAX_LEVELS), ("active", C.c_int64 * MAX_LEVELS),
                ("iters_run", C.c_int32 * MAX_LEVELS), ("residual", C.c_double * MAX_LEVELS),
                ("leaf_iters", C.c_int64), ("kernel_launches", C.c_int32), ("graph", C.c_int32),
                ("setup_ms", C.c_double), ("iterate_ms", C.c_double), ("total_ms", C.c_double),
                ("kt_depth", C.c_int32), ("kt_launches", C.c_int32), ("kt_active", C.c_int64),
                ("kt_dual_ms", C.c_double), ("kt_primal_ms", C.c_double),
                ("level_ms", C.c_double * MAX_LEVELS), ("schedule", C.c_int32 * MAX_LEVELS),
                ("kt_fused", C.c_int32), ("placement", C.c_int32), ("energy", C.c_double * MAX_LEVELS)]

    def as_dict(self):
        k = self.n_levels
        return dict(n_levels=k, min_depth=self.min_depth, max_depth=self.max_depth,
                    depth=list(self.depth[:k]), active=list(self.active[:k]),
                    iters_run=list(self.iters_run[:k]), residual=list(self.residual[:k]),
                    leaf_iters=self.leaf_iters, kernel_launches=self.kernel_launches, graph=self.graph,
                    setup_ms=self.setup_ms, iterate_ms=self.iterate_ms, total_ms=self.total_ms,
                    kt_depth=self.kt_depth, kt_launches=self.kt_launches, kt_active=self.kt_active,
                    kt_dual_ms=self.kt_dual_ms, kt_primal_ms=self.kt_primal_ms,
                    level_ms=list(self.level_ms[:k]), schedule=list(self.schedule[:k]), kt_fused=self.kt_fused,
                    placement=self.placement,
                    energy=list(self.energy[:k]))


P = C.c_void_p
_SIGS = {
    "tgvg_abi_version": ([], C.c_int),
    "tgvg_create": ([C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "tgvg_destroy": ([P], C.c_int),
    "tgvg_strerror": ([C.c_int], C.c_char_p),
    "tgvg_last_error": ([P], C.c_char_p),
    "tgvg_stream": ([P], C.c_void_p),
    "tgvg_kernel_count": ([P], C.c_int64),
    "tgvg_level_thresholds": ([P], None),
    "tgvg_set_timing": ([P, C.c_int], C.c_int),
    "tgvg_set_schedule": ([P, C.c_int32, C.c_int32, C.c_int32], C.c_int),
    "tgvg_set_graphs": ([P, C.c_int], C.c_int),
    "tgvg_set_device_budget": ([P, C.c_int64], C.c_int),
    "tgvg_pyramid_dims": ([C.c_int32, C.c_int32, P], C.c_int),
    "tgvg_build_pyramids": ([P, P, C.c_int32, P, P], C.c_int),
    "tgvg_compute_histograms": ([P, P, C.c_int64, P, C.c_int32, P, P, C.c_float, C.c_int32, P], C.c_int),
    "tgvg_compute_histograms_pyr": ([P, P, C.c_int64, P, C.c_int32, P, P, C.c_float, C.c_int32, P], C.c_int),
    "tgvg_compute_histograms_dev": ([P, P, C.c_int64, P, C.c_int32, P, P, P, C.c_float, C.c_int32, P], C.c_int),
    "tgvg_compute_histograms_noalloc": ([P, C.c_int64, P, C.c_int32, P, P, C.c_float, C.c_int32, P, P],
                                        C.c_int),
    "tgvg_compute_histograms_oc":([P, C.c_char_p, P, C.c_int32, P, C.c_int32, P, P, C.c_float, C.c_char_p],
                                   C.c_int),
    "tgvg_tgv_minimize": ([P, P, P, C.c_int64, C.c_int32, P, C.c_int32, C.c_int32, P, P, P, P], C.c_int),
    "tgvg_tgv_minimize_dev": ([P, P, P, C.c_int64, C.c_int32, P, C.c_int32, C.c_int32, P, P, P, P], C.c_int),
    "tgvg_tgv_minimize_state": ([P, P, P, C.c_int64, C.c_int32, P, C.c_int32, C.c_int32, P, P, P, P], C.c_int),
    "tgvg_tgv_minimize_state_dev": ([P, P, P, C.c_int64, C.c_int32, P, C.c_int32, C.c_int32, P, P, P, P],
                                    C.c_int),
    "tgvg_tgv_minimize_streaming": ([P, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, P, P], C.c_int),
    "tgvg_mlp_create": ([P, C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)], C.c_int),
    "tgvg_mlp_destroy": ([P], C.c_int),
    "tgvg_mlp_num_params": ([], C.c_int32),
    "tgvg_mlp_params": ([P, P, P, P], C.c_int),
    "tgvg_mlp_features": ([P, P, P, C.c_int64, C.c_int32, P, C.c_int32, P], C.c_int),
    "tgvg_mlp_predict": ([P, P, P, C.c_int64, P], C.c_int),
    "tgvg_mlp_warm_start": ([P, P, P, P, C.c_int64, C.c_int32, P, C.c_int32, P], C.c_int),
    "tgvg_mlp_warm_start_dev": ([P, P, P, P, C.c_int64, C.c_int32, P, C.c_int32, P], C.c_int),
    "tgvg_mlp_grad": ([P, P, P, P, C.c_int64, P, P], C.c_int),
    "tgvg_mlp_train": ([P, P, P, P, C.c_int64, C.c_int32, C.c_int32, C.c_float, C.c_uint64, P], C.c_int),
    "tgvg_build_cubes": ([P, P, P, C.c_float, P, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
    "tgvg_build_cubes_file": ([P, P, P, C.c_float, C.c_char_p], C.c_int),
    "tgvg_merge_cubes": ([P, P, P, C.c_int32, P, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
    "tgvg_kway_merge": ([P, P, C.c_int32, C.c_char_p], C.c_int),
    "tgvg_balance_cubes": ([P, P, C.c_int64, C.c_float, P, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
    "tgvg_balance_octree": ([P, C.c_char_p, C.c_char_p], C.c_int),
    "tgvg_extract_surface": ([P, P, P, C.c_int64, P, P, C.c_float, C.c_int32, C.POINTER(C.c_void_p)], C.c_int),
    "tgvg_extract_surface_leaves": ([P, P, P, P, C.c_int32, C.c_int64, P, C.c_int32, P, C.c_float,
                                     C.POINTER(C.c_void_p)], C.c_int),
    "tgvg_extract_surface_streaming": ([P, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, P, C.c_float,
                                        C.c_char_p], C.c_int),
    "tgvg_mesh_size": ([P, P, P, P], C.c_int),
    "tgvg_mesh_read": ([P, P, P, P], C.c_int),
    "tgvg_mesh_free": ([P], None),
    "tgvg_compute_normals": ([P, P, C.c_int64, P, C.c_int64, P], C.c_int),
    "tgvg_write_obj": ([C.c_char_p, P, C.c_int64, P, C.c_int64, P], C.c_int),
    "tgvg_save_tgv": ([C.c_char_p, P, C.c_int64], C.c_int),
    "tgvg_load_tgv": ([C.c_char_p, P, C.c_int64], C.c_int64),
    "tgvg_save_histograms": ([C.c_char_p, P, C.c_int64], C.c_int),
    "tgvg_load_histograms": ([C.c_char_p, P, C.c_int64], C.c_int64),
}

_lib = None


def lib():
    """Load libtgvg.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)
