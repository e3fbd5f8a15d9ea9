"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own src/histogram.cpp, src/tgv.cpp and src/marching_cubes.cpp (compiled unmodified
into oracle/_ref/libref.so by oracle/Makefile, with the project-written
Eigen/TBB shims) on seeded synthetic inputs and stores inputs + outputs as
compressed .npz files.  Needs the reference checkout ($TGV_REFERENCE_DIR, else
the REF_DIR default of oracle/Makefile); the fixtures it writes are committed
so the tests can run where the reference is absent.

    python tests/golden/make_golden.py            # histogram and TGV fixtures, then
    python tests/golden/make_golden.py --mesh     # the surface fixtures (read tgv_balanced.npz)
    python tests/golden/make_golden.py --stage1   # the Stage-1 cube fixture
    python tests/golden/make_golden.py --octree   # the merge and balance fixture
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle as O  # noqa: E402
from tgvreconclaude_gb300 import formats as F, scenes as S  # noqa: E402


def maps_for(scene, rig, seed0=0, lidar_every=0):
    maps = []
    for i, c in enumerate(rig):
        d = S.render_depth(scene, c, seed=seed0 + i).numpy()
        m = dict(depth=d, rt=c["rt"], fx=c["fx"], fy=c["fy"], cx=c["cx"], cy=c["cy"],
                 lidar=bool(lidar_every and i % lidar_every == 0))
        m["rt_inv"], _, _ = O.ref_mipmap(m)
        maps.append(m)
    return maps


def pack_maps(maps):
    return dict(depths=np.stack([m["depth"] for m in maps]), rt=np.stack([m["rt"] for m in maps]),
                rt_inv=np.stack([m["rt_inv"] for m in maps]),
                k=np.array([[m["fx"], m["fy"], m["cx"], m["cy"]] for m in maps], np.float32),
                lidar=np.array([m["lidar"] for m in maps], bool))


def hist_case(name, rng, scene, rig, cubes, origin, r_root, lidar_every=0):
    maps = maps_for(scene, rig, int(rng.integers(1 << 30)), lidar_every)
    bins = O.ref_compute_histograms(cubes, maps, origin, r_root)
    np.savez_compressed(os.path.join(HERE, f"hist_{name}.npz"), cubes=cubes, origin=np.float32(origin),
                        r_root=np.float32(r_root), bins=bins, **pack_maps(maps))
    print(f"hist_{name}: {len(cubes)} cubes, {len(maps)} maps, votes {int(bins.sum())}")


def tgv_case(name, cubes, hists, leaves, alpha0, alpha1, iters, r_root=1.0):
    out = {}
    for mode in ("inmem", "oc", "stream"):
        out[mode] = O.ref_tgv(cubes, hists, leaves, mode, alpha0, alpha1, iters, r_root=r_root)
    np.savez_compressed(os.path.join(HERE, f"tgv_{name}.npz"), cubes=cubes, hists=hists, leaves=leaves,
                        params=np.array([alpha0, alpha1], np.float32), iters=np.int32(iters),
                        inmem=out["inmem"], oc=out["oc"], stream=out["stream"])
    d = np.bincount(cubes["depth"])
    print(f"tgv_{name}: {len(cubes)} cubes, depths {np.nonzero(d)[0].tolist()}, leaves {len(leaves)}")


def mesh_case(name, cubes, state, hists, leaves, origin, r_root):
    """The reference's extract_surface (has_data = any vote, with normals) and
    extract_surface_streaming (its .obj text) on one octree and state."""
    import tempfile
    has = (hists.sum(1) > 0).astype(np.uint8)
    v, f, nrm = O.ref_extract_surface(cubes, state, origin, r_root, has_data=has, normals=True)
    with tempfile.TemporaryDirectory() as td:
        paths = [os.path.join(td, x) for x in ("c.bin", "s.bin", "t.bin", "h.bin", "m.obj")]
        F.save_cubes(paths[0], cubes, r_root)
        F.save_state(paths[1], state)
        F.save_treetop(paths[2], leaves, r_root)
        F.save_histograms(paths[3], hists)
        O.ref_extract_surface_streaming(*paths[:4], origin, r_root, paths[4])
        obj = open(paths[4]).read()
    np.savez_compressed(os.path.join(HERE, f"mesh_{name}.npz"), cubes=cubes, state=state, hists=hists,
                        leaves=leaves, origin=np.float32(origin), r_root=np.float32(r_root), has_data=has,
                        verts=v, faces=f, normals=nrm, s_obj=np.array(obj))
    print(f"mesh_{name}: {len(cubes)} cubes, {len(v)} vertices, {len(f)} triangles, "
          f"streaming obj {obj.count(chr(10))} lines")


def mesh_cases():
    """Surface-extraction fixtures: the balanced reference octree with the
    reference's TGV state, and a random octree with random u."""
    O.build(ref=True)
    g = dict(np.load(os.path.join(HERE, "tgv_balanced.npz")))
    mesh_case("balanced", g["cubes"], g["inmem"], g["hists"], g["leaves"], (-1.5, -1.5, -1.5), 1.5)
    rng = np.random.default_rng(7)
    c = S.random_octree(rng, dmin=2, dmax=6, target=3000, shape="sphere", r_root=2.0)
    st = np.zeros(len(c), F.STATE_DTYPE)
    st["u"] = rng.uniform(-1, 1, len(c)).astype(np.float32)
    h = S.random_histograms(rng, len(c), empty_frac=0.15)
    lv = S.split_leaves(len(c), 4, rng, c, aligned=True)
    mesh_case("rand", c, st, h, lv, (-2.0, -1.5, -1.0), 2.0)


def stage1_case():
    """Stage 1: the reference's build_cubes_from_depthmap on three ray-cast maps
    of the torus (with holes)."""
    O.build(ref=True)
    rng = np.random.default_rng(11)
    rig = S.sphere_rig(3, 3.0, width=96, height=72, half_fov_deg=28)
    maps = maps_for(S.torus_scene(0.005), rig, 500)
    for m in maps:
        m["depth"][rng.random(m["depth"].shape) < 0.03] = np.nan
    out = {f"cubes{k}": O.ref_build_cubes(m, (-1.5, -1.5, -1.5), 1.5) for k, m in enumerate(maps)}
    np.savez_compressed(os.path.join(HERE, "stage1_maps.npz"), origin=np.float32([-1.5, -1.5, -1.5]),
                        r_root=np.float32(1.5), depths=np.stack([m["depth"] for m in maps]),
                        rt=np.stack([m["rt"] for m in maps]).astype(np.float32),
                        fx=np.float32([m["fx"] for m in maps]), fy=np.float32([m["fy"] for m in maps]),
                        cx=np.float32([m["cx"] for m in maps]), cy=np.float32([m["cy"] for m in maps]), **out)
    print("stage1_maps:", [len(v) for v in out.values()], "cubes")


def octree_case():
    """Stages 2 and 3: the reference's kway_merge on Stage-1 lists of four maps
    (as given, and split into code-disjoint lists), and its balance_octree on the
    merged list, on stress inputs and on its own test cases."""
    sys.path.insert(0, os.path.dirname(HERE))
    import octree_cases as OC
    from test_stage1_oracle import stage1_maps
    O.build(ref=True)
    maps, origin, r_root = stage1_maps(0, n=4)
    arrs = [O.ref_build_cubes(m, origin, r_root) for m in maps]
    parts = OC.disjoint_parts(arrs)
    out = {}
    for i, a in enumerate(arrs):
        out[f"overlap_in{i}"] = a
    for i, a in enumerate(parts):
        out[f"disjoint_in{i}"] = a
    out["overlap_out"] = O.ref_merge_cubes(arrs, r_root)
    out["disjoint_out"] = O.ref_merge_cubes(parts, r_root)
    cases = [(out["overlap_out"], r_root)] + [(OC.balance_inputs(s), 2.0) for s in range(4)] + OC.reference_cases()
    for i, (c, rr) in enumerate(cases):
        out[f"bal_in{i}"] = c
        out[f"bal_r{i}"] = np.float32(rr)
        out[f"bal_out{i}"] = O.ref_balance_cubes(c, rr)
    np.savez_compressed(os.path.join(HERE, "octree_cases.npz"), **out)
    print("octree_cases:", {k: len(v) for k, v in out.items() if v.ndim})


def main():
    if "--octree" in sys.argv:
        return octree_case()
    if "--mesh" in sys.argv:
        return mesh_cases()
    if "--stage1" in sys.argv:
        return stage1_case()
    O.build(ref=True)
    rng = np.random.default_rng(20261203)

    # Stage 5: torus seen by a sphere rig (one LIDAR map), cubes from a random band
    scene = S.torus_scene(0.005)
    rig = S.sphere_rig(6, 3.0, width=96, height=72)
    cubes = S.random_octree(rng, dmin=3, dmax=7, target=4000, shape="sphere", r_root=1.5)
    cubes["r_c"][:6] = [0.0, -1.0, np.nan, np.inf, 100.0, 1e-6]
    hist_case("torus", rng, scene, rig, cubes, (-1.5, -1.5, -1.5), 1.5, lidar_every=4)

    # Stage 5: three objects with the cubes of the reference's own Stages 1-4
    scene3 = S.three_objects_scene(rng)
    rig3 = S.sphere_rig(8, 6.0, width=80, height=60, half_fov_deg=28)
    maps3 = maps_for(scene3, rig3, 100)
    cubes3, leaves3 = O.ref_pipeline_cubes(maps3[:3], (-3.0, -3.0, -3.0), 3.0)
    if len(cubes3) > 6000:
        cubes3 = cubes3[:6000]
    hist_case("three", rng, scene3, rig3, cubes3, (-3.0, -3.0, -3.0), 3.0)

    # Stage 6: random multi-level octrees with duplicate codes, several leaf splits
    for k, (shape, dmin, dmax, nleaf, aligned, a0, a1, it) in enumerate([
            ("sphere", 2, 5, 3, True, 0.02, 0.04, 25),
            ("plane", 3, 6, 4, False, 0.1, 0.2, 30),
            ("random", 1, 4, 2, False, 1.0, 2.0, 20)]):
        c = S.random_octree(rng, dmin=dmin, dmax=dmax, target=1500, shape=shape)
        h = S.random_histograms(rng, len(c))
        lv = S.split_leaves(len(c), nleaf, rng, c, aligned=aligned)
        tgv_case(f"rand{k}", c, h, lv, a0, a1, it)

    # Stage 6: reference-built balanced octree (Stages 1-4) with reference histograms
    maps_b = maps_for(S.torus_scene(0.005), S.sphere_rig(3, 3.0, width=64, height=48), 300)
    cb, lb = O.ref_pipeline_cubes(maps_b, (-1.5, -1.5, -1.5), 1.5)
    hb = O.ref_compute_histograms(cb, maps_b, (-1.5, -1.5, -1.5), 1.5)
    lv = S.split_leaves(len(cb), 3, rng, cb, aligned=True)
    tgv_case("balanced", cb, hb, lv, 2.0, 1.0, 40, r_root=1.5)
    mesh_cases()
    stage1_case()
    octree_case()


if __name__ == "__main__":
    main()
