"""Named synthetic workloads with the shapes of the benchmark configurations.

Each workload is seeded and generated here (no dataset is available): analytic
scene -> camera rig -> ray-cast float32 depth maps with per-object noise ->
cube set (Stage-1 depth rule, merge, 2:1 balance, depth capped) -> histograms
computed by this package's own Stage-5 kernels -> chunk leaves.

  torus16     torus R=1 r=0.3, N(0,0.005); 16 cameras on a radius-3 sphere at 640x480;
              max depth 8; 10-bin histograms; TGV alpha1=1, alpha0=2, 300 iterations
  three64     sphere r=0.8 + box side 1.2 + torus 1.0/0.25 at seeded offsets, sigma ~ U[0.002,0.01];
              64 cameras at 1920x1080; max depth 11; 10 bins; 1000 iterations
  terrain128  8 seeded sinusoids (amplitude 0.1-0.5) + N(0,0.003) over [-4,4]^2; 128 nadir/oblique
              cameras at 1280x960; max depth 12; 64 chunks of log-uniform 50k-4M cubes
  prims256    12 seeded primitives (sphere, box, torus, cylinder in turn; size 0.55-1.1, centres in [-1.7, 1.7]^3), sigma 0.004;
              256 cameras at 2048x1536, each framing one primitive with a 16-degree field of view
              (21-22 views per primitive); max depth 13; 128 chunks
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N, formats as F, scenes as S

CONFIGS = {
    "torus16": dict(scene="torus", ncam=16, cam_radius=3.0, width=640, height=480, half_fov=25.0,
                    origin=(-1.5, -1.5, -1.5), r_root=1.5, max_depth=8, nbins=10, iters=300, chunks=1),
    "three64": dict(scene="three", ncam=64, cam_radius=4.5, width=1920, height=1080, half_fov=25.0,
                    origin=(-3.0, -3.0, -3.0), r_root=3.0, max_depth=11, nbins=10, iters=1000, chunks=1),
    "terrain128": dict(scene="terrain", ncam=128, cam_radius=4.0, width=1280, height=960, half_fov=30.0,
                       origin=(-4.0, -4.0, -4.0), r_root=4.0, max_depth=12, nbins=10, iters=1000, chunks=64),
    "prims256": dict(scene="prims", rig="objects", prim_size=(0.55, 1.1), prim_spread=1.7, ncam=256, cam_radius=7.0, width=2048,
                     height=1536, half_fov=8.0,
                     origin=(-3.0, -3.0, -3.0), r_root=3.0, max_depth=13, nbins=10, iters=1000, chunks=128),
}


@dataclass
class Workload:
    name: str
    cfg: dict
    cams: list            # N.Camera structs (rt_inv row-major)
    depths: list          # (H, W) float32 arrays (host) -- or None when kept on the GPU
    cubes: np.ndarray     # CUBE_DTYPE, Morton-sorted
    hists: np.ndarray     # (n, nbins) uint32
    leaves: np.ndarray    # LEAF_DTYPE
    timings: dict = field(default_factory=dict)


def make_scene(kind: str, rng, size=None, spread=None):
    if kind == "torus":
        return S.torus_scene(0.005)
    if kind == "three":
        return S.three_objects_scene(rng)
    if kind == "terrain":
        return S.terrain_scene(rng)
    if kind == "prims":
        return S.primitives_scene(rng, 12, 0.004, size=size or (0.25, 0.6), spread=spread or 1.8)
    raise ValueError(kind)


def make_rig(cfg, rng, scene=None):
    if cfg.get("rig") == "objects":
        return S.object_rig(scene, cfg["ncam"], cfg["width"], cfg["height"], cfg["half_fov"], cfg.get("fill", 0.8))
    if cfg["scene"] == "terrain":
        return S.terrain_rig(cfg["ncam"], 4.0, cfg["cam_radius"], cfg["width"], cfg["height"], cfg["half_fov"], rng)
    return S.sphere_rig(cfg["ncam"], cfg["cam_radius"], (0.0, 0.0, 0.0), cfg["width"], cfg["height"],
                        cfg["half_fov"])


def camera(c) -> N.Camera:
    cam = N.Camera()
    rt_inv = np.linalg.inv(np.asarray(c["rt"], np.float64)).astype(np.float32)
    cam.rt_inv[:] = [float(v) for v in rt_inv.reshape(16)]
    cam.fx, cam.fy, cam.cx, cam.cy = c["fx"], c["fy"], c["cx"], c["cy"]
    cam.width, cam.height = c["width"], c["height"]
    cam.lidar = int(bool(c.get("lidar", False)))
    return cam


def chunk_leaves(cubes, k: int, rng, lo=50_000, hi=4_000_000):
    """Split the Morton-sorted cube array into k contiguous chunks with
    log-uniform target sizes in [lo, hi] (scaled to the cube count), cutting
    only where the code changes so no code straddles two chunks."""
    n = len(cubes)
    if k <= 1 or n == 0:
        return S.split_leaves(n, 1, rng, cubes)
    w = np.exp(rng.uniform(math.log(lo), math.log(hi), k))
    bounds = np.floor(np.cumsum(w) / w.sum() * n).astype(np.int64)[:-1]
    keys = F.cube_keys(cubes)
    cuts = []
    for b in bounds:
        b = int(min(max(b, 1), n - 1))
        while b < n - 1 and keys[b] == keys[b - 1]:
            b += 1
        cuts.append(b)
    cuts = np.unique(np.array(cuts))
    edges = np.concatenate([[0], cuts, [n]])
    leaves = np.zeros(len(edges) - 1, F.LEAF_DTYPE)
    leaves["first_idx"] = edges[:-1]
    leaves["last_idx"] = edges[1:] - 1
    leaves["hi"], leaves["lo"], leaves["depth"] = (cubes["hi"][edges[:-1]], cubes["lo"][edges[:-1]],
                                                   cubes["depth"][edges[:-1]])
    return leaves


_CAM_FIELDS = ("fx", "fy", "cx", "cy", "width", "height", "lidar")


def save(w: Workload, path: str) -> None:
    """Cubes, histograms, leaves, cameras and depth maps of a workload as one .npz
    (so that a profiled run can skip the ray casting)."""
    extra = {}
    if w.cams and w.depths is not None and len({d.shape for d in w.depths}) == 1:
        extra["depths"] = np.stack([np.asarray(d, np.float32) for d in w.depths])
        extra["cam_rt_inv"] = np.array([list(c.rt_inv) for c in w.cams], np.float32)
        extra["cam_par"] = np.array([[getattr(c, f) for f in _CAM_FIELDS] for c in w.cams], np.float64)
    np.savez(path, name=w.name, cubes=w.cubes, hists=w.hists, leaves=w.leaves, **extra)


def load(path: str) -> Workload:
    d = np.load(path)
    name = str(d["name"])
    cams, depths = [], None
    if "depths" in d.files:
        depths = list(d["depths"])
        for rt, par in zip(d["cam_rt_inv"], d["cam_par"]):
            c = N.Camera()
            c.rt_inv[:] = [float(v) for v in rt]
            c.fx, c.fy, c.cx, c.cy = (float(v) for v in par[:4])
            c.width, c.height, c.lidar = (int(v) for v in par[4:])
            cams.append(c)
    return Workload(name, dict(CONFIGS[name]), cams, depths, d["cubes"], d["hists"], d["leaves"], {})


def build(name: str, seed: int = 0, device: str = "cuda", keep_depths: bool = False,
          max_cubes: int | None = None, verbose: bool = False, histograms: bool = True) -> Workload:
    """Generate workload `name` (see module docstring).  With histograms=False
    the histogram rows are left empty for the caller to fill."""
    import torch
    from . import api
    cfg = dict(CONFIGS[name])
    rng = np.random.default_rng(seed)
    t0 = time.time()
    scene = make_scene(cfg["scene"], rng, cfg.get("prim_size"), cfg.get("prim_spread"))
    rig = make_rig(cfg, rng, scene)
    dtype = torch.float32 if device != "cpu" else torch.float64
    Ps, Rs, depths, cams = [], [], [], []
    for i, c in enumerate(rig):
        seen = S.primitives_in_view(scene, c) if cfg.get("rig") == "objects" else scene
        d = S.render_depth(seen, c, seed=seed * 100003 + i, device=device, dtype=dtype)
        P, r = S.samples_from_depth_map(d, c, torch)
        Ps.append(P)
        Rs.append(r)
        depths.append(d.cpu().numpy())
        cams.append(camera(c))
    t1 = time.time()
    P = torch.cat(Ps)
    r = torch.cat(Rs)
    del Ps, Rs
    key, rc = S.cubes_from_samples(P, r, cfg["origin"], cfg["r_root"], cfg["max_depth"], torch)
    del P, r
    key, rc = S.balance_2to1(key, rc, cfg["r_root"], torch)
    cubes = S.keys_to_cubes(key, rc)
    del key, rc
    if max_cubes and len(cubes) > max_cubes:
        cubes = cubes[:max_cubes]
    t2 = time.time()
    if histograms:
        hists = api.compute_histograms_from_maps(cubes, cams, depths, cfg["origin"], cfg["r_root"], cfg["nbins"])
    else:
        hists = np.zeros((len(cubes), cfg["nbins"]), np.uint32)
    t3 = time.time()
    leaves = chunk_leaves(cubes, cfg["chunks"], rng)
    w = Workload(name, cfg, cams, depths if keep_depths else None, cubes, hists, leaves,
                 dict(render_s=t1 - t0, cubes_s=t2 - t1, hist_s=t3 - t2))
    if verbose:
        dd = np.bincount(cubes["depth"], minlength=22)
        print(f"[{name}] {len(cubes)} cubes, depths {dict((int(k), int(v)) for k, v in enumerate(dd) if v)}, "
              f"{len(leaves)} leaves, votes {int(hists.sum())}, times {w.timings}", flush=True)
    if not keep_depths:
        w.depths = depths  # kept for the histogram bench; callers may drop it
    return w
