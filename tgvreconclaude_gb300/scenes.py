"""Seeded synthetic inputs for the Stage-5/6 path: analytic scenes, camera rigs,
ray-cast depth maps, multi-level Morton cube sets and histograms.

No dataset ships with the reference's benchmarks (and none is reachable here),
so every workload is generated from a seed with the shapes and value ranges of
the configuration it stands in for.  Generation runs on the CPU with numpy for
small cases and on the GPU through torch for the large ones; it is input
preparation, never part of a timed region.
"""
from __future__ import annotations

import math

import numpy as np

from . import formats as F


# ------------------------------------------------------------ cube sets ---

def random_octree(rng: np.random.Generator, dmin: int = 2, dmax: int = 5,
                  target: int = 2000, shape: str = "sphere", dup_shuffle: bool = True,
                  r_root: float = 1.0):
    """Multi-level cube set around a surface band, Morton-sorted.

    Every depth in [dmin, dmax] holds the cells of a band around an analytic
    surface, so cubes nest across depths the way the reference's merged and
    balanced sets do (every sample spawns a cube at its own depth).  Cubes of
    different depths that share a fine-grid code (the octant-0 chain) are kept;
    with ``dup_shuffle`` their relative order is randomised, which decides the
    "largest index wins" lookups of the reference.
    """
    keys_all, dep_all = [], []
    for d in range(dmin, dmax + 1):
        g = 1 << d
        c = (np.arange(g) + 0.5) / g
        X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
        if shape == "sphere":
            f = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2) - 0.3
        elif shape == "plane":
            f = Z - (0.45 + 0.1 * X + 0.05 * Y)
        else:
            f = rng.uniform(-1, 1, X.shape)
        sel = np.abs(f) < 1.0 / g  # cells within one cell size of the surface
        ix, iy, iz = np.nonzero(sel)
        sh = F.MAX_DEPTH - d
        k = F.morton_encode(ix.astype(np.uint32) << sh, iy.astype(np.uint32) << sh,
                            iz.astype(np.uint32) << sh)
        keys_all.append(k)
        dep_all.append(np.full(len(k), d, np.int32))
    keys = np.concatenate(keys_all)
    dep = np.concatenate(dep_all)
    if len(keys) > target:
        keep = np.sort(rng.choice(len(keys), target, replace=False))
        keys, dep = keys[keep], dep[keep]
    tie = rng.random(len(keys)) if dup_shuffle else dep.astype(np.float64)
    order = np.lexsort((tie, keys))
    keys, dep = keys[order], dep[order]
    r_c = (r_root / (1 << dep.astype(np.int64))).astype(np.float32) * rng.uniform(0.7, 1.3, len(keys)).astype(np.float32)
    return F.make_cubes(keys, dep, r_c)


def random_histograms(rng: np.random.Generator, n: int, nbins: int = 8, empty_frac: float = 0.2,
                      max_count: int = 40) -> np.ndarray:
    h = rng.integers(0, max_count, (n, nbins)).astype(np.uint32)
    # concentrate mass: zero out a random subset of bins per row
    h[rng.random((n, nbins)) < 0.5] = 0
    h[rng.random(n) < empty_frac] = 0
    return h


def split_leaves(n: int, k: int, rng: np.random.Generator | None = None, cubes=None,
                 aligned: bool = False):
    """Contiguous index ranges covering [0, n).  ``aligned`` cuts only where the
    Morton code changes (so that equal codes never straddle two leaves, as in the
    reference's treetop); otherwise cuts are arbitrary (as in its tests)."""
    leaves = np.zeros(k, F.LEAF_DTYPE)
    if n == 0 or k <= 0:
        return leaves[:0]
    rng = rng or np.random.default_rng(0)
    cuts = np.sort(rng.choice(np.arange(1, n), min(k - 1, n - 1), replace=False)) if n > 1 else np.array([], int)
    if aligned and cubes is not None:
        keys = F.cube_keys(cubes)
        cuts = np.array([c for c in cuts if keys[c] != keys[c - 1]], int)
    bounds = np.concatenate([[0], cuts, [n]])
    leaves = np.zeros(len(bounds) - 1, F.LEAF_DTYPE)
    leaves["first_idx"] = bounds[:-1]
    leaves["last_idx"] = bounds[1:] - 1
    if cubes is not None:
        leaves["hi"] = cubes["hi"][bounds[:-1]]
        leaves["lo"] = cubes["lo"][bounds[:-1]]
        leaves["depth"] = cubes["depth"][bounds[:-1]]
    return leaves


# ------------------------------------------------------------ cameras ---

def look_at(eye, target, up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """World<-camera transform (the reference's DepthMap::Rt): camera +z looks at
    `target`, +x is image-right, +y image-down."""
    eye = np.asarray(eye, np.float64)
    z = np.asarray(target, np.float64) - eye
    z /= np.linalg.norm(z)
    upv = np.asarray(up, np.float64)
    if abs(np.dot(upv, z)) > 0.99:
        upv = np.array([0.0, 1.0, 0.0])
    x = np.cross(z, upv)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    rt = np.eye(4)
    rt[:3, 0], rt[:3, 1], rt[:3, 2], rt[:3, 3] = x, y, z, eye
    return rt.astype(np.float32)


def sphere_rig(n: int, radius: float, target=(0.0, 0.0, 0.0), width=640, height=480,
               half_fov_deg: float = 25.0):
    """`n` cameras evenly spread on a sphere (Fibonacci spiral) looking at `target`."""
    cams = []
    ga = math.pi * (3.0 - math.sqrt(5.0))
    fx = (width / 2.0) / math.tan(math.radians(half_fov_deg))
    for i in range(n):
        zc = 1.0 - 2.0 * (i + 0.5) / n
        rr = math.sqrt(max(0.0, 1.0 - zc * zc))
        eye = np.array([rr * math.cos(ga * i), rr * math.sin(ga * i), zc]) * radius + np.asarray(target)
        cams.append(dict(rt=look_at(eye, target), fx=fx, fy=fx, cx=width / 2.0, cy=height / 2.0,
                         width=width, height=height, lidar=False))
    return cams


def bounding_radius(prim) -> float:
    """Radius of a sphere about the primitive's centre that encloses it."""
    k = prim["kind"]
    if k == "sphere":
        return prim["r"]
    if k == "box":
        return prim["h"] * math.sqrt(3.0)
    if k == "torus":
        return prim["R"] + prim["r"]
    if k == "cylinder":
        return math.hypot(prim["r"], prim["h"])
    raise ValueError(k)


def object_rig(scene, n: int, width=2048, height=1536, half_fov_deg: float = 8.0, fill: float = 0.8):
    """A multi-object capture: camera i looks at primitive i mod P from the
    next direction of that primitive's Fibonacci sphere, at the distance where
    the primitive's bounding sphere fills `fill` of the image height.  Narrow
    fields of view put most pixels on surfaces."""
    cams = []
    P = len(scene)
    ga = math.pi * (3.0 - math.sqrt(5.0))
    fx = (width / 2.0) / math.tan(math.radians(half_fov_deg))
    tan_v = (height / 2.0) / fx
    for i in range(n):
        j, k = i % P, i // P
        m = (n - j + P - 1) // P  # cameras of primitive j
        zc = 1.0 - 2.0 * (k + 0.5) / m
        rr = math.sqrt(max(0.0, 1.0 - zc * zc))
        a = ga * k + 2.0 * math.pi * j / P
        c = np.asarray(scene[j]["c"], np.float64)
        dist = bounding_radius(scene[j]) / (tan_v * fill)
        eye = c + np.array([rr * math.cos(a), rr * math.sin(a), zc]) * dist
        cams.append(dict(rt=look_at(eye, c), fx=fx, fy=fx, cx=width / 2.0, cy=height / 2.0,
                         width=width, height=height, lidar=False))
    return cams


def primitives_in_view(scene, cam, margin_deg: float = 2.0):
    """The primitives whose bounding sphere reaches into the camera's view cone
    (the cone around the optical axis through the image corners).  Sphere
    tracing only these finds the same surfaces at a fraction of the cost when
    each camera frames one object with a narrow field of view."""
    rt = np.asarray(cam["rt"], np.float64)
    eye, axis = rt[:3, 3], rt[:3, 2]
    half_diag = math.atan(math.hypot(cam["width"] / 2.0 / cam["fx"], cam["height"] / 2.0 / cam["fy"]))
    out = []
    for p in scene:
        d = np.asarray(p["c"], np.float64) - eye
        dist = float(np.linalg.norm(d))
        rb = bounding_radius(p)
        if dist <= rb:
            out.append(p)
            continue
        ang = math.acos(max(-1.0, min(1.0, float(np.dot(d, axis)) / dist)))
        if ang - math.asin(rb / dist) <= half_diag + math.radians(margin_deg):
            out.append(p)
    return out


def terrain_rig(n: int, extent: float, height_above: float, width=1280, height=960,
                half_fov_deg: float = 30.0, rng: np.random.Generator | None = None):
    """Nadir and oblique cameras over the square [-extent, extent]^2: a grid of
    nadir views plus obliques tilted towards the centre."""
    rng = rng or np.random.default_rng(0)
    fx = (width / 2.0) / math.tan(math.radians(half_fov_deg))
    cams = []
    g = int(math.ceil(math.sqrt(n / 2)))
    for i in range(n):
        if i < n // 2:
            gx, gy = (i % g + 0.5) / g, (i // g + 0.5) / g
            eye = np.array([(2 * gx - 1) * extent * 0.85, (2 * gy - 1) * extent * 0.85, height_above])
            tgt = eye - np.array([0.0, 0.0, height_above])
            rt = look_at(eye, tgt, up=(0.0, 1.0, 0.0))
        else:
            a = 2 * math.pi * rng.random()
            rad = extent * rng.uniform(0.3, 1.1)
            eye = np.array([rad * math.cos(a), rad * math.sin(a), height_above * rng.uniform(0.6, 1.0)])
            tgt = np.array([eye[0] * 0.3, eye[1] * 0.3, 0.0])
            rt = look_at(eye, tgt)
        cams.append(dict(rt=rt, fx=fx, fy=fx, cx=width / 2.0, cy=height / 2.0, width=width,
                         height=height, lidar=False))
    return cams


# --------------------------------------------------------- analytic scenes ---
# A scene is a list of primitives; each is evaluated as a signed distance so that
# one sphere tracer renders any union.  Primitive dicts:
#   {"kind": "sphere", "c": (x,y,z), "r": r, "sigma": s}
#   {"kind": "box", "c": ..., "h": half side, "sigma": s}
#   {"kind": "torus", "c": ..., "R": R, "r": r, "sigma": s}       (axis z)
#   {"kind": "cylinder", "c": ..., "r": r, "h": half height, "sigma": s}  (axis z)
#   {"kind": "terrain", "A": [...], "k": [[kx,ky],...], "phi": [...], "sigma": s}

def _sdf(prim, px, py, pz, torch):
    k = prim["kind"]
    if k == "terrain":
        h = torch.zeros_like(px)
        for A, kk, ph in zip(prim["A"], prim["k"], prim["phi"]):
            h = h + A * torch.sin(kk[0] * px + kk[1] * py + ph)
        # vertical distance scaled by the Lipschitz bound keeps sphere tracing safe
        lip = math.sqrt(1.0 + sum(A * math.hypot(*kk) for A, kk in zip(prim["A"], prim["k"])) ** 2)
        return (pz - h) / lip
    cx, cy, cz = prim["c"]
    x, y, z = px - cx, py - cy, pz - cz
    if k == "sphere":
        return torch.sqrt(x * x + y * y + z * z) - prim["r"]
    if k == "box":
        qx, qy, qz = x.abs() - prim["h"], y.abs() - prim["h"], z.abs() - prim["h"]
        out = torch.sqrt(qx.clamp(min=0) ** 2 + qy.clamp(min=0) ** 2 + qz.clamp(min=0) ** 2)
        return out + torch.clamp(torch.maximum(qx, torch.maximum(qy, qz)), max=0)
    if k == "torus":
        q = torch.sqrt(x * x + y * y) - prim["R"]
        return torch.sqrt(q * q + z * z) - prim["r"]
    if k == "cylinder":
        dx = torch.sqrt(x * x + y * y) - prim["r"]
        dz = z.abs() - prim["h"]
        out = torch.sqrt(dx.clamp(min=0) ** 2 + dz.clamp(min=0) ** 2)
        return out + torch.clamp(torch.maximum(dx, dz), max=0)
    raise ValueError(k)


def render_depth(scene, cam, seed: int, device="cpu", steps: int = 160, max_dist: float = 50.0,
                 rows_per_chunk: int = 0, dtype=None):
    """Ray-cast one camera: camera-z depth per pixel (NaN where no surface), plus
    N(0, sigma) noise of the primitive hit.  Pixel (u, v) is traced through the
    same point the reference unprojects it from (src/depth_map.cpp:4-11)."""
    import torch
    dtype = dtype or torch.float64
    eps = 1e-6 if dtype == torch.float64 else 2e-5
    W, H = cam["width"], cam["height"]
    if not scene:
        return torch.full((H, W), float("nan"), dtype=torch.float32, device=device)
    rt = torch.tensor(np.asarray(cam["rt"], np.float64), device=device, dtype=dtype)
    gen = torch.Generator(device=device).manual_seed(int(seed))
    out = torch.empty((H, W), dtype=torch.float32, device=device)
    rows = rows_per_chunk or H
    for r0 in range(0, H, rows):
        r1 = min(H, r0 + rows)
        v, u = torch.meshgrid(torch.arange(r0, r1, device=device, dtype=dtype),
                              torch.arange(W, device=device, dtype=dtype), indexing="ij")
        dxc = (u - cam["cx"]) / cam["fx"]
        dyc = (v - cam["cy"]) / cam["fy"]
        nrm = torch.sqrt(dxc * dxc + dyc * dyc + 1.0)
        dwx = (rt[0, 0] * dxc + rt[0, 1] * dyc + rt[0, 2]) / nrm
        dwy = (rt[1, 0] * dxc + rt[1, 1] * dyc + rt[1, 2]) / nrm
        dwz = (rt[2, 0] * dxc + rt[2, 1] * dyc + rt[2, 2]) / nrm
        ox, oy, oz = rt[0, 3], rt[1, 3], rt[2, 3]
        t = torch.zeros_like(dxc)
        hit = torch.zeros_like(dxc, dtype=torch.bool)
        which = torch.zeros_like(dxc, dtype=torch.int64)
        for _ in range(steps):
            px, py, pz = ox + t * dwx, oy + t * dwy, oz + t * dwz
            ds = torch.stack([_sdf(p, px, py, pz, torch) for p in scene])
            d, which = ds.min(dim=0)
            hit = hit | (d.abs() < eps * (1.0 + t))
            t = torch.where(hit | (t > max_dist), t, t + d)
        sig = torch.tensor([p.get("sigma", 0.0) for p in scene], device=device, dtype=dtype)
        noise = torch.randn(t.shape, generator=gen, device=device, dtype=dtype) * sig[which]
        depth = (t / nrm) + noise  # camera z = distance along the ray / |dir_cam|
        depth = torch.where(hit & (t <= max_dist), depth, torch.full_like(depth, float("nan")))
        out[r0:r1] = depth.to(torch.float32)
    return out


def torus_scene(sigma=0.005):
    return [dict(kind="torus", c=(0.0, 0.0, 0.0), R=1.0, r=0.3, sigma=sigma)]


def three_objects_scene(rng: np.random.Generator):
    """Sphere r=0.8, box side 1.2 and torus 1.0/0.25 at seeded offsets, each with
    its own noise sigma ~ U[0.002, 0.01]."""
    offs = rng.uniform(-0.6, 0.6, (3, 3))
    base = np.array([[-1.4, 0.0, 0.0], [1.3, 0.2, 0.0], [0.0, 0.0, 0.0]])
    c = base + offs * np.array([0.5, 1.0, 0.5])
    s = rng.uniform(0.002, 0.01, 3)
    return [dict(kind="sphere", c=tuple(c[0]), r=0.8, sigma=float(s[0])),
            dict(kind="box", c=tuple(c[1]), h=0.6, sigma=float(s[1])),
            dict(kind="torus", c=tuple(c[2] + np.array([0.0, 1.6, 0.0])), R=1.0, r=0.25,
                 sigma=float(s[2]))]


def primitives_scene(rng: np.random.Generator, n: int = 12, sigma: float = 0.004, size=(0.25, 0.6),
                     spread: float = 1.8):
    """`n` seeded spheres, boxes, tori and cylinders (in turn) of size drawn from
    `size`, centred in [-spread, spread]^3."""
    kinds = ["sphere", "box", "torus", "cylinder"]
    out = []
    for i in range(n):
        k = kinds[i % 4]
        c = tuple(rng.uniform(-spread, spread, 3))
        s = float(rng.uniform(*size))
        if k == "sphere":
            out.append(dict(kind=k, c=c, r=s, sigma=sigma))
        elif k == "box":
            out.append(dict(kind=k, c=c, h=s * 0.8, sigma=sigma))
        elif k == "torus":
            out.append(dict(kind=k, c=c, R=s, r=s * 0.3, sigma=sigma))
        else:
            out.append(dict(kind=k, c=c, r=s * 0.6, h=s, sigma=sigma))
    return out


def terrain_scene(rng: np.random.Generator, sigma=0.003):
    A = rng.uniform(0.1, 0.5, 8)
    k = rng.uniform(0.3, 2.0, (8, 2)) * rng.choice([-1, 1], (8, 2))
    phi = rng.uniform(0, 2 * math.pi, 8)
    return [dict(kind="terrain", A=A.tolist(), k=k.tolist(), phi=phi.tolist(), sigma=sigma)]


# ------------------------------------------------- cube sets from depth maps ---
# Input preparation in the reference pipeline's shape: every valid pixel spawns
# a cube at the depth its sample radius asks for (src/octree_builder.cpp:11-97),
# equal (code, depth) cubes merge with their radii averaged (src/merge.cpp),
# and 2:1 bridge cubes are added until no face neighbour is two or more levels
# coarser (src/balance.cpp:60-150).  Written with torch so that the large
# workloads build on the GPU in seconds; not bit-identical to the reference's
# own Stage 1-3 (which the fixture script uses where exactness matters).

def _t_spread3(v, torch):
    x = v & 0x1FFFFF
    for s, m in _M_T:
        x = (x | (x << s)) & m
    return x


def _t_gather3(v, torch):
    x = v & 0x1249249249249249
    for s, m in ((2, 0x10C30C30C30C30C3), (4, 0x100F00F00F00F00F), (8, 0x001F0000FF0000FF),
                 (16, 0x001F00000000FFFF), (32, 0x00000000001FFFFF)):
        x = (x | (x >> s)) & m
    return x


_M_T = [(32, 0x001F00000000FFFF), (16, 0x001F0000FF0000FF), (8, 0x100F00F00F00F00F),
        (4, 0x10C30C30C30C30C3), (2, 0x1249249249249249)]


def _t_encode(x, y, z, torch):
    return _t_spread3(x, torch) | (_t_spread3(y, torch) << 1) | (_t_spread3(z, torch) << 2)


def cube_depth_for_radius(r_x, r_root: float, max_depth: int, torch):
    """Depth d with 0.75 r_x <= r_root / 2^d < 1.5 r_x, clamped to [0, max_depth]
    (src/octree_builder.cpp:11-28), vectorised."""
    d = torch.round(torch.log2(r_root / (r_x * 1.125))).clamp(0, max_depth)
    for _ in range(3):
        cell = r_root / torch.exp2(d)
        lo = cell < 0.75 * r_x
        hi = cell >= 1.5 * r_x
        d = torch.where(lo & (d > 0), d - 1, torch.where(hi & (d < max_depth), d + 1, d))
    return d.to(torch.int64)


def samples_from_depth_map(depth, cam, torch):
    """Unprojected points and sample radii of one map (src/depth_map.cpp:4-30):
    r_x = half the mean distance to the valid 4-neighbours."""
    H, W = depth.shape
    dev = depth.device
    ok = torch.isfinite(depth) & (depth > 0)
    v, u = torch.meshgrid(torch.arange(H, device=dev, dtype=torch.float32),
                          torch.arange(W, device=dev, dtype=torch.float32), indexing="ij")
    d = torch.where(ok, depth, torch.zeros_like(depth))
    cx = (u - cam["cx"]) * d / cam["fx"]
    cy = (v - cam["cy"]) * d / cam["fy"]
    rt = torch.tensor(np.asarray(cam["rt"], np.float32), device=dev)
    P = torch.stack([rt[i, 0] * cx + rt[i, 1] * cy + rt[i, 2] * d + rt[i, 3] for i in range(3)], -1)
    acc = torch.zeros_like(depth)
    cnt = torch.zeros_like(depth)
    for dy, dx in ((0, 1), (0, -1), (1, 0), (-1, 0)):
        nok = torch.zeros_like(ok)
        nP = torch.zeros_like(P)
        ys, ye = max(0, -dy), H - max(0, dy)
        xs, xe = max(0, -dx), W - max(0, dx)
        nok[ys:ye, xs:xe] = ok[ys + dy:ye + dy, xs + dx:xe + dx]
        nP[ys:ye, xs:xe] = P[ys + dy:ye + dy, xs + dx:xe + dx]
        dist = torch.linalg.norm(nP - P, dim=-1)
        acc += torch.where(nok, dist, torch.zeros_like(dist))
        cnt += nok.float()
    r = torch.where(cnt > 0, 0.5 * acc / cnt.clamp(min=1), torch.zeros_like(acc))
    keep = ok & (r > 0)
    return P[keep], r[keep]


def cubes_from_samples(P, r, origin, r_root: float, max_depth: int, torch):
    """Stage-1 cubes of samples + merge of equal (code, depth) with mean radius.
    Returns (key = code | depth, r_c) sorted by code, then depth."""
    n = (P - torch.tensor(origin, device=P.device, dtype=P.dtype)) / (2.0 * r_root)
    inside = ((n >= 0) & (n < 1)).all(-1)
    n, r = n[inside], r[inside]
    d = cube_depth_for_radius(r, r_root, max_depth, torch)
    g = torch.exp2(d.to(torch.float32))
    idx = (n * g[:, None]).to(torch.int64)
    idx = torch.minimum(idx, (g[:, None] - 1).to(torch.int64))
    sh = (21 - d)[:, None]
    c = _t_encode(idx[:, 0] << sh[:, 0], idx[:, 1] << sh[:, 0], idx[:, 2] << sh[:, 0], torch)
    key = c | d  # codes of depth <= 16 cubes have >= 15 zero low bits
    uk, inv = torch.unique(key, return_inverse=True)
    rs = torch.zeros(len(uk), device=P.device, dtype=torch.float64).index_add_(0, inv, r.double())
    cn = torch.zeros(len(uk), device=P.device, dtype=torch.float64).index_add_(0, inv, torch.ones_like(r, dtype=torch.float64))
    return uk, (rs / cn).to(torch.float32)


def _t_face(code, d, f, torch):
    x, y, z = _t_gather3(code, torch), _t_gather3(code >> 1, torch), _t_gather3(code >> 2, torch)
    step = torch.ones_like(d) << (21 - d)
    c = [x, y, z]
    ax, sg = f // 2, (1 if f % 2 == 0 else -1)
    nv = c[ax] + sg * step
    ok = (nv >= 0) & (nv < (1 << 21))
    c[ax] = nv.clamp(0, (1 << 21) - 1)
    return _t_encode(c[0], c[1], c[2], torch), ok


def _t_anc(code, d, torch):
    sh = 3 * (21 - d)
    return code & ~((torch.ones_like(code) << sh) - 1)


def balance_2to1(key, r_c, r_root: float, torch, max_rounds: int = 64):
    """Add bridge cubes until no cube of depth d >= 2 has a face neighbour region
    whose nearest existing cube is two or more levels coarser (the rule of
    src/balance.cpp:100-133).  key = code | depth, sorted."""
    frontier = key
    for _ in range(max_rounds):
        code, d = frontier & ~31, frontier & 31
        sel = d >= 2
        code, d = code[sel], d[sel]
        new = []
        for f in range(6):
            nb, ok = _t_face(code, d, f, torch)
            nb, dd = nb[ok], d[ok]

            def has(c, depth):
                k = c | depth
                pos = torch.searchsorted(key, k).clamp(max=len(key) - 1)
                return key[pos] == k
            sat = has(nb, dd) | has(_t_anc(nb, dd - 1, torch), dd - 1)
            nb, dd = nb[~sat], dd[~sat]
            viol = torch.zeros_like(nb, dtype=torch.bool)
            for d2 in range(int(dd.max().item()) - 2 if len(dd) else -1, -1, -1):
                m = (dd - 2 >= d2) & ~viol
                if m.any():
                    viol |= m & has(_t_anc(nb, torch.full_like(dd, d2), torch), torch.full_like(dd, d2))
            new.append(_t_anc(nb[viol], dd[viol] - 1, torch) | (dd[viol] - 1))
        cand = torch.unique(torch.cat(new)) if new else key[:0]
        if len(cand) == 0:
            break
        pos = torch.searchsorted(key, cand).clamp(max=len(key) - 1)
        cand = cand[key[pos] != cand]
        if len(cand) == 0:
            break
        bd = cand & 31
        rc = (r_root / torch.exp2(bd.to(torch.float32))).to(torch.float32)
        key, order = torch.sort(torch.cat([key, cand]))
        r_c = torch.cat([r_c, rc])[order]
        frontier = cand
    return key, r_c


def keys_to_cubes(key, r_c) -> np.ndarray:
    k = key.cpu().numpy().astype(np.uint64)
    code = k & ~np.uint64(31)
    return F.make_cubes(code, (k & np.uint64(31)).astype(np.int32), r_c.cpu().numpy())
