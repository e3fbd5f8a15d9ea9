"""The binning kernel skips, per block of 256 Morton-consecutive cubes, the
cameras that no cube centre of the block can pass project()'s tests for
(behind the camera or outside the image, src/histogram.cpp:76-106).  These
cases make that skip frequent and put cube centres right on its boundaries;
the histograms must stay bit-identical to the oracle's."""
import numpy as np
import pytest

from test_gpu_parity import cams_from, render_maps
from tgvreconclaude_gb300 import api, scenes as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nbins", [8, 10])
def test_narrow_views_of_separate_objects(oracle_lib, nbins):
    """Object rig: each camera frames one of 12 primitives with a narrow field
    of view, so most blocks are outside most cameras' images."""
    rng = np.random.default_rng(300 + nbins)
    scene = S.primitives_scene(rng, 12, 0.004)
    rig = S.object_rig(scene, 36, width=160, height=120, half_fov_deg=8.0)
    maps = render_maps(scene, rig, 7, lidar_every=7)
    cubes = S.random_octree(rng, dmin=3, dmax=9, target=120000, shape="random", r_root=3.0)
    ref = oracle_lib.compute_histograms(cubes, maps, (-3.0, -3.0, -3.0), 3.0, nbins=nbins, nthreads=8)
    gpu = api.compute_histograms_from_maps(cubes, cams_from(maps), [m["depth"] for m in maps], (-3.0, -3.0, -3.0),
                                           3.0, nbins=nbins)
    assert ref.sum() > 0
    assert np.array_equal(gpu, ref)


def test_cameras_inside_the_cube_cloud(oracle_lib):
    """Cameras inside the octree's volume: blocks straddle every camera's z = 0
    plane and the image borders in all directions; wide and very narrow views."""
    rng = np.random.default_rng(9)
    scene = S.three_objects_scene(rng)
    maps = []
    for fov, r in ((60.0, 0.4), (3.0, 0.9), (25.0, 1.7)):
        maps += render_maps(scene, S.sphere_rig(6, r, width=96, height=64, half_fov_deg=fov), 3)
    for m in maps:  # make every depth valid so that culled pairs would otherwise vote
        d = m["depth"]
        d[~np.isfinite(d)] = 2.0
    cubes = S.random_octree(rng, dmin=2, dmax=8, target=80000, shape="sphere", r_root=3.0)
    ref = oracle_lib.compute_histograms(cubes, maps, (-3.0, -3.0, -3.0), 3.0, nbins=8, nthreads=8)
    gpu = api.compute_histograms_from_maps(cubes, cams_from(maps), [m["depth"] for m in maps], (-3.0, -3.0, -3.0),
                                           3.0, nbins=8)
    assert ref.sum() > 0
    assert np.array_equal(gpu, ref)
