"""Learned warm start for the TGV solve.

A per-cube MLP (F -> 64 -> 64 -> 1, F = nbins + 5 features: the histogram
normalised by its total, depth / 21, the cube centre's position inside its
chunk's node, and the median indicator) predicts the converged u minus the
median indicator, the reference's own start; the warm start is median +
network.  It is trained on the GPU by this package's own forward/backward
kernels (include/tgvg.h, tgvg_mlp_*) on pairs that the plain solver produces
on seeded scenes, and it seeds a solve with params.init = "given" and
every level starts from the prediction (tgvg_tgv_minimize_state records with
v = p = q = 0) instead of the parent copy.  The plain primal-dual iterations
still run to the same stopping tolerance, so the prediction only changes how
many iterations that takes.
"""
from __future__ import annotations

import ctypes as C
import os
import time
from dataclasses import dataclass

import numpy as np

from . import _native as N, api, formats as F, scenes as S, workloads as W


class WarmStartMLP:
    def __init__(self, nbins: int = 10, seed: int = 0):
        self.ctx = api.context()
        self.lib = self.ctx.lib
        h = C.c_void_p()
        self.ctx.check(self.lib.tgvg_mlp_create(self.ctx.h, nbins, seed, C.byref(h)), "tgvg_mlp_create")
        self.h = h
        self.nbins = nbins
        self.n_params = self.lib.tgvg_mlp_num_params()

    def __del__(self):
        try:
            if self.h:
                self.lib.tgvg_mlp_destroy(self.h)
        except Exception:
            pass

    # -- parameters
    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        self.ctx.check(self.lib.tgvg_mlp_params(self.ctx.h, self.h, p.ctypes.data, None), "mlp params")
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        self.ctx.check(self.lib.tgvg_mlp_params(self.ctx.h, self.h, None, p.ctypes.data), "mlp params")

    def save(self, path) -> None:
        np.savez(path, params=self.get_params(), nbins=self.nbins)

    @classmethod
    def load(cls, path) -> "WarmStartMLP":
        d = np.load(path)
        m = cls(int(d["nbins"]))
        m.set_params(d["params"])
        return m

    # -- data
    def features(self, cubes, hists, leaves=None) -> np.ndarray:
        cubes = np.ascontiguousarray(cubes, F.CUBE_DTYPE)
        hists = np.ascontiguousarray(hists, np.uint32)
        X = np.zeros((len(cubes), 16), np.uint16)
        lv = None if leaves is None else np.ascontiguousarray(leaves, F.LEAF_DTYPE)
        self.ctx.check(self.lib.tgvg_mlp_features(self.ctx.h, api._p(cubes), api._p(hists), len(cubes),
                                                  hists.shape[1], api._p(lv), 0 if lv is None else len(lv),
                                                  api._p(X)), "tgvg_mlp_features")
        return X

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.uint16)
        y = np.zeros(len(X), np.float32)
        self.ctx.check(self.lib.tgvg_mlp_predict(self.ctx.h, self.h, api._p(X), len(X), api._p(y)),
                       "tgvg_mlp_predict")
        return y

    def warm_start(self, cubes, hists, leaves=None) -> np.ndarray:
        """u = median indicator + network, computed on the device."""
        cubes = np.ascontiguousarray(cubes, F.CUBE_DTYPE)
        hists = np.ascontiguousarray(hists, np.uint32)
        lv = None if leaves is None else np.ascontiguousarray(leaves, F.LEAF_DTYPE)
        u = np.zeros(len(cubes), np.float32)
        self.ctx.check(self.lib.tgvg_mlp_warm_start(self.ctx.h, self.h, api._p(cubes), api._p(hists), len(cubes),
                                                    hists.shape[1], api._p(lv), 0 if lv is None else len(lv),
                                                    api._p(u)), "tgvg_mlp_warm_start")
        return u

    def grad(self, X, t):
        X = np.ascontiguousarray(X, np.uint16)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        self.ctx.check(self.lib.tgvg_mlp_grad(self.ctx.h, self.h, api._p(X), api._p(t), len(X), api._p(g),
                                              C.byref(loss)), "tgvg_mlp_grad")
        return loss.value, g

    def train(self, X, t, epochs: int = 10, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> float:
        X = np.ascontiguousarray(X, np.uint16)
        t = np.ascontiguousarray(t, np.float32)
        loss = C.c_float()
        self.ctx.check(self.lib.tgvg_mlp_train(self.ctx.h, self.h, api._p(X), api._p(t), len(X), epochs, batch,
                                               C.c_float(lr), seed, C.byref(loss)), "tgvg_mlp_train")
        return loss.value


# ------------------------------------------------------------ scene data ---

SMALL = dict(torus=dict(scene="torus", ncam=16, cam_radius=4.0, width=320, height=240, half_fov=25.0,
                        origin=(-1.5, -1.5, -1.5), r_root=1.5, max_depth=7, nbins=10),
             three=dict(scene="three", ncam=16, cam_radius=6.5, width=320, height=240, half_fov=28.0,
                        origin=(-3.0, -3.0, -3.0), r_root=3.0, max_depth=8, nbins=10))


def small_scene(seed: int, kind: str = "torus", device: str = "cuda"):
    """A reduced scene of the torus / three-object configurations: 16 cameras at
    320x240, cubes to depth 7 (torus) or 8 (three objects).  The cameras stand
    far enough out (radius 4 / 6.5) that each sees the whole object: with closer
    or fewer cameras a quarter of the finest cubes get at most two votes, and on
    those the reference iteration is unstable (u grows by up to ~0.75 per
    iteration without bound)."""
    import torch
    cfg = SMALL[kind]
    rng = np.random.default_rng(seed)
    scene = W.make_scene(cfg["scene"], rng)
    if kind == "torus":  # vary the torus per seed
        scene[0]["R"] = float(rng.uniform(0.8, 1.1))
        scene[0]["r"] = float(rng.uniform(0.2, 0.35))
        scene[0]["sigma"] = float(rng.uniform(0.002, 0.008))
    rig = S.sphere_rig(cfg["ncam"], cfg["cam_radius"] * float(rng.uniform(0.9, 1.1)), width=cfg["width"],
                       height=cfg["height"], half_fov_deg=cfg["half_fov"])
    Ps, Rs, depths, cams = [], [], [], []
    for i, c in enumerate(rig):
        d = S.render_depth(scene, c, seed=seed * 1000 + i, device=device, dtype=torch.float32, steps=128)
        P, r = S.samples_from_depth_map(d, c, torch)
        Ps.append(P); Rs.append(r); depths.append(d.cpu().numpy()); cams.append(W.camera(c))
    key, rc = S.cubes_from_samples(torch.cat(Ps), torch.cat(Rs), cfg["origin"], cfg["r_root"], cfg["max_depth"],
                                   torch)
    key, rc = S.balance_2to1(key, rc, cfg["r_root"], torch)
    cubes = S.keys_to_cubes(key, rc)
    hists = api.compute_histograms_from_maps(cubes, cams, depths, cfg["origin"], cfg["r_root"], cfg["nbins"])
    return cubes, hists


SOLVE = dict(alpha0=2.0, alpha1=1.0)
# The shipped network, trained by train_warmstart on seeds 0-99.
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warmstart_nb10.npz")


def converged_u(cubes, hists, tol: float = 1e-6, max_iters: int = 6000):
    """Plain solver (reference initialisation) run to a tight residual."""
    prm = api.TGVParams(alpha0=SOLVE["alpha0"], alpha1=SOLVE["alpha1"], iters=max_iters, tol=tol, check_every=20)
    out, st = api.tgv_solve(cubes, hists, None, "inmem", prm)
    return out["u"].copy(), st


# Cubes whose solved |u| exceeds this have no fixed point of the reference
# iteration (weakly observed cubes on which u drifts without bound); they are
# left out of the training pairs.
U_BOUND = 1.5


def dataset(seeds, kinds=("torus", "three")):
    """Training pairs: features and converged u minus the median indicator,
    over the cubes whose converged |u| <= U_BOUND."""
    Xs, ts = [], []
    mlp = WarmStartMLP()
    for s in seeds:
        kind = kinds[s % len(kinds)]
        cubes, hists = small_scene(s, kind)
        u, _ = converged_u(cubes, hists)
        ok = np.abs(u) <= U_BOUND
        Xs.append(mlp.features(cubes, hists)[ok])
        ts.append((u - median_start(hists))[ok])
    return np.concatenate(Xs), np.concatenate(ts)


@dataclass
class SolveRecord:
    leaf_iters: int
    iters: list
    device_ms: float
    wall_ms: float
    predict_ms: float = 0.0


def start_records(n: int, u=None) -> np.ndarray:
    """Whole-state records (tgvg_tgv_minimize_state) that start every level from
    u (zero when None) with v = p = q = 0."""
    s = np.zeros(n, F.STATE_DTYPE)
    if u is not None:
        s["u"] = u
    return s


def time_to_tol(cubes, hists, start: str = "zero", u0=None, tol: float = 1e-4, max_iters: int = 6000,
                check_every: int = 10, leaves=None, mode: str = "inmem"):
    """Solve to relative residual `tol` and return (state, SolveRecord).

    All starts solve the reference's problem: cubes hold the reference's
    initial state until their level starts.  start = "reference": the
    reference's initialisation (median, then the parent's u and v at each
    level); "zero": every level from u = v = p = q = 0; "warm": every level
    from u = u0 with v = p = q = 0."""
    prm = api.TGVParams(alpha0=SOLVE["alpha0"], alpha1=SOLVE["alpha1"], iters=max_iters, tol=tol,
                        check_every=check_every)
    t0 = time.perf_counter()
    if start == "reference":
        out, st = api.tgv_solve(cubes, hists, leaves, mode, prm)
    else:
        out, st = api.tgv_solve(cubes, hists, leaves, mode, prm,
                                state_init=start_records(len(cubes), u0 if start == "warm" else None))
    wall = 1e3 * (time.perf_counter() - t0)
    return out, SolveRecord(st["leaf_iters"], st["iters_run"], st["total_ms"], wall)


def median_start(hists) -> np.ndarray:
    """The reference's initial u: the histogram's median indicator, 0 when empty
    (src/histogram.cpp:12-31)."""
    h = np.asarray(hists, np.uint32)
    nb = h.shape[1]
    tot = h.sum(1, dtype=np.uint32)
    k = np.argmax(np.cumsum(h, 1, dtype=np.uint32) * np.uint32(2) >= tot[:, None], axis=1)
    med = np.float32(-1.0) + (k.astype(np.float32) + np.float32(0.5)) / np.float32(nb / 2.0)
    return np.where(tot > 0, med, np.float32(0.0)).astype(np.float32)


def start_errors(mlp: WarmStartMLP, cubes, hists, u_conv) -> dict:
    """RMS distance to the converged u of the three starts: zero, the median
    indicator, and the network's prediction."""
    pred = mlp.warm_start(cubes, hists)
    rms = lambda a: float(np.sqrt(np.mean((np.asarray(a, np.float64) - u_conv) ** 2)))
    return dict(zero=rms(np.zeros_like(u_conv)), median=rms(median_start(hists)), network=rms(pred))


def compare(mlp: WarmStartMLP, cubes, hists, tol: float = 1e-4, leaves=None, mode: str = "inmem"):
    """The zero start, the learned warm start and the reference's initialisation
    on one problem, each to the same tolerance -> dict of SolveRecords and the
    warm solve's state.

    The solves run with direct launches: later sightings of the same problem
    would otherwise pay for, or profit from, the level-loop graph's capture."""
    ctx = api.context()
    ctx.set_graphs(False)
    try:
        _, zero = time_to_tol(cubes, hists, "zero", tol=tol, leaves=leaves, mode=mode)
        t0 = time.perf_counter()
        u0 = mlp.warm_start(cubes, hists, leaves)
        pred_ms = 1e3 * (time.perf_counter() - t0)
        out, warm = time_to_tol(cubes, hists, "warm", u0, tol, leaves=leaves, mode=mode)
        _, ref = time_to_tol(cubes, hists, "reference", tol=tol, leaves=leaves, mode=mode)
    finally:
        ctx.set_graphs(True)
    warm.predict_ms = pred_ms
    return dict(zero=zero, warm=warm, reference=ref), out


def evaluate(mlp: WarmStartMLP, seeds, tol: float = 1e-4, max_iters: int = 6000):
    """Held-out evaluation on small scenes (torus on even seeds, three objects
    on odd ones): time and leaf-iterations to relative residual `tol` from the
    zero start, from the network's prediction and from the reference's
    initialisation.  Returns (records, summary)."""
    recs = []
    for seed in seeds:
        kind = "torus" if seed % 2 == 0 else "three"
        cubes, hists = small_scene(seed, kind)
        r, _ = compare(mlp, cubes, hists, tol=tol)
        rec = dict(seed=seed, kind=kind, cubes=int(len(cubes)), predict_ms=r["warm"].predict_ms)
        for k, v in r.items():
            rec[f"{k}_ms"] = v.device_ms + (v.predict_ms if k == "warm" else 0.0)
            rec[f"{k}_leaf_iters"] = v.leaf_iters
            rec[f"{k}_iters"] = v.iters
            rec[f"{k}_capped_levels"] = sum(i >= max_iters for i in v.iters)
        recs.append(rec)
    med = lambda k: float(np.median([r[k] for r in recs]))
    ratio = lambda a, b: float(np.median([r[f"{a}_ms"] / r[f"{b}_ms"] for r in recs]))
    summary = {
        "time_ratio_zero_over_warm": ratio("zero", "warm"),
        "time_ratio_reference_over_warm": ratio("reference", "warm"),
        "leaf_iters_ratio_zero_over_warm": med("zero_leaf_iters") / med("warm_leaf_iters"),
        "leaf_iters_ratio_reference_over_warm": med("reference_leaf_iters") / med("warm_leaf_iters"),
        "median_zero_ms": med("zero_ms"), "median_warm_ms": med("warm_ms"), "median_reference_ms": med("reference_ms"),
        "median_predict_ms": med("predict_ms"),
        "scenes_with_capped_levels": int(sum(r["zero_capped_levels"] > 0 for r in recs)),
    }
    return recs, summary
