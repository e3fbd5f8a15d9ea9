"""The no-allocation histogram entry point (tgvg_compute_histograms_noalloc).

It exists for callers that must not allocate device memory while they run:
one that reserves all device memory up front for its own pool, a real-time
loop where an allocation's implicit synchronisation would stall other work, or
a runtime that routes every allocation through its own allocator.  These tests
call it through the C ABI with device buffers the test owns, and check it
against the regular histogram entry point on two calls in a row.  The second
call uses a different scene, so the first call's leftovers in the shared
scratch array cannot leak into the second.  Histograms are integer counts:
the tolerance is exact equality, as in the other histogram tests."""
import ctypes as C

import numpy as np
import pytest

from tgvreconclaude_gb300 import _native as N, api, scenes as S

pytestmark = pytest.mark.gpu

TGVG_ERR_LIMIT = -10


def _scene(seed, ncam, w, h, nbins, target):
    rng = np.random.default_rng(seed)
    rig = S.sphere_rig(ncam, 3.0, width=w, height=h)
    cams, depths = [], []
    for i, c in enumerate(rig):
        d = S.render_depth(S.torus_scene(0.01), c, seed=seed * 100 + i).numpy()
        rt_inv = np.linalg.inv(np.asarray(c["rt"], np.float64)).astype(np.float32)
        cam = N.Camera()
        cam.rt_inv[:] = [float(v) for v in rt_inv.reshape(16)]
        cam.fx, cam.fy, cam.cx, cam.cy = c["fx"], c["fy"], c["cx"], c["cy"]
        cam.width, cam.height, cam.lidar = w, h, int(i % 3 == 0)
        cams.append(cam)
        depths.append(d)
    cubes = S.random_octree(rng, dmin=3, dmax=8, target=target, r_root=1.5)
    return cams, depths, cubes, nbins


def _noalloc(cams, depths, cubes, nbins):
    import torch
    dev_maps = [torch.from_numpy(d).cuda() for d in depths]
    d_cubes = torch.from_numpy(cubes.view(np.int32).reshape(len(cubes), 4)).cuda()
    d_out = torch.full((len(cubes), nbins), -1, dtype=torch.int32, device="cuda")
    arr = (N.Camera * len(cams))(*cams)
    bases = (C.c_void_p * len(cams))(*[t.data_ptr() for t in dev_maps])
    origin = np.array([-1.5, -1.5, -1.5], np.float32)
    stream = torch.cuda.current_stream()
    rc = N.lib().tgvg_compute_histograms_noalloc(d_cubes.data_ptr(), len(cubes), arr, len(cams), bases,
                                                 origin.ctypes.data, C.c_float(1.5), nbins, d_out.data_ptr(),
                                                 stream.cuda_stream)
    assert rc == 0, N.lib().tgvg_strerror(rc)
    stream.synchronize()
    return d_out.cpu().numpy().view(np.uint32)


def test_noalloc_matches_regular_entry_on_two_calls_in_a_row():
    for args in (_scene(1, 5, 320, 240, 8, 30000), _scene(2, 3, 200, 150, 10, 12000)):
        cams, depths, cubes, nbins = args
        got = _noalloc(cams, depths, cubes, nbins)
        want = api.compute_histograms_from_maps(cubes, cams, depths, (-1.5, -1.5, -1.5), 1.5, nbins)
        assert want.sum() > 0
        assert np.array_equal(got, want)


def test_noalloc_call_leaves_free_device_memory_unchanged():
    """After a first call on the device (which may load the library's device
    code together with its scratch array), a call allocates nothing: the
    device's free memory is the same before and after it."""
    import torch
    cams, depths, cubes, nbins = _scene(3, 4, 256, 192, 8, 20000)
    dev_maps = [torch.from_numpy(d).cuda() for d in depths]
    d_cubes = torch.from_numpy(cubes.view(np.int32).reshape(len(cubes), 4)).cuda()
    d_out = torch.zeros((len(cubes), nbins), dtype=torch.int32, device="cuda")
    arr = (N.Camera * len(cams))(*cams)
    bases = (C.c_void_p * len(cams))(*[t.data_ptr() for t in dev_maps])
    origin = np.array([-1.5, -1.5, -1.5], np.float32)
    stream = torch.cuda.current_stream()

    def call():
        rc = N.lib().tgvg_compute_histograms_noalloc(d_cubes.data_ptr(), len(cubes), arr, len(cams), bases,
                                                     origin.ctypes.data, C.c_float(1.5), nbins, d_out.data_ptr(),
                                                     stream.cuda_stream)
        assert rc == 0, N.lib().tgvg_strerror(rc)
        stream.synchronize()

    call()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert int(d_out.sum()) > 0


def test_noalloc_rejects_requests_beyond_its_scratch():
    lib = N.lib()
    big = N.Camera()
    big.width, big.height = 2048, 1536  # 5 such pyramids exceed 16 Mi texels
    arr = (N.Camera * 5)(*([big] * 5))
    bases = (C.c_void_p * 5)()
    origin = np.zeros(3, np.float32)
    rc = lib.tgvg_compute_histograms_noalloc(None, 0, arr, 5, bases, origin.ctypes.data, C.c_float(1.0), 8, None,
                                             None)
    assert rc == TGVG_ERR_LIMIT
    small = N.Camera()
    small.width, small.height = 8, 8
    many = (N.Camera * 300)(*([small] * 300))
    rc = lib.tgvg_compute_histograms_noalloc(None, 0, many, 300, (C.c_void_p * 300)(), origin.ctypes.data,
                                             C.c_float(1.0), 8, None, None)
    assert rc == TGVG_ERR_LIMIT
    assert "no-allocation" in lib.tgvg_strerror(rc).decode()
