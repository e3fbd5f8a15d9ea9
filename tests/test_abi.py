"""The C ABI library without a GPU: it builds, loads, exports every entry point
that include/tgvg.h declares, refuses to run compute without an sm_103 device,
and its host-only file routines read and write the reference's formats."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from tgvreconclaude_gb300 import _native as N, formats as F

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "tgvg.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tgvg_\w+)\s*\(", src)))


def test_header_declarations_are_all_exported():
    lib = N.lib()
    names = declared()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(N.exported_symbols())


def test_abi_version_and_errors():
    lib = N.lib()
    assert lib.tgvg_abi_version() == 4
    assert lib.tgvg_strerror(-4).decode() == "cubes are not sorted by Morton code"
    assert lib.tgvg_strerror(-9).decode() == "treetop leaves overlap"


def test_no_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = N.lib()
    h = C.c_void_p()
    assert lib.tgvg_create(0, C.byref(h)) == -8  # TGVG_ERR_NODEVICE: no silent CPU path
    from tgvreconclaude_gb300 import api
    with pytest.raises(RuntimeError, match="sm_103"):
        api.Context(0)


def test_pyramid_dims_rule():
    lib = N.lib()
    d = (C.c_int32 * 26)()
    assert lib.tgvg_pyramid_dims(1920, 1080, d) == 11  # ... 7x4, 3x2, 1x1
    assert (d[2], d[3]) == (960, 540) and (d[18], d[19]) == (3, 2) and (d[20], d[21]) == (1, 1)
    assert lib.tgvg_pyramid_dims(8, 8, d) == 4
    assert lib.tgvg_pyramid_dims(1, 100, d) == 1
    assert lib.tgvg_pyramid_dims(0, 5, d) == -1


def test_state_and_histogram_files_roundtrip(tmp_path):
    lib = N.lib()
    rng = np.random.default_rng(0)
    st = np.zeros(7, F.STATE_DTYPE)
    st.view(np.float32)[:] = rng.standard_normal(7 * 13).astype(np.float32)
    p = str(tmp_path / "s.tgvs").encode()
    assert lib.tgvg_save_tgv(p, st.ctypes.data, 7) == 0
    assert np.array_equal(F.load_state(tmp_path / "s.tgvs"), st)
    back = np.zeros(7, F.STATE_DTYPE)
    assert lib.tgvg_load_tgv(p, back.ctypes.data, 7) == 7 and back.tobytes() == st.tobytes()
    assert lib.tgvg_load_tgv(p, None, 0) == 7
    h = rng.integers(0, 100, (5, 8)).astype(np.uint32)
    F.save_histograms(tmp_path / "h.tgvh", h)
    hb = np.zeros((5, 8), np.uint32)
    assert lib.tgvg_load_histograms(str(tmp_path / "h.tgvh").encode(), hb.ctypes.data, 5) == 5
    assert np.array_equal(hb, h)
    (tmp_path / "bad").write_bytes(b"NOPE" + bytes(40))
    assert lib.tgvg_load_tgv(str(tmp_path / "bad").encode(), None, 0) == -6
    assert lib.tgvg_load_histograms(str(tmp_path / "missing").encode(), None, 0) == -5
    (tmp_path / "short").write_bytes(b"TGVS" + np.array([1, 9], "<u4").tobytes() + bytes(52))
    assert lib.tgvg_load_tgv(str(tmp_path / "short").encode(), None, 0) == -6


def test_python_formats_roundtrip(tmp_path):
    rng = np.random.default_rng(1)
    cubes = F.make_cubes(np.sort(rng.integers(0, 1 << 62, 50).astype(np.uint64)), 9, 0.01)
    F.save_cubes(tmp_path / "c", cubes, 2.5)
    c2, r = F.load_cubes(tmp_path / "c")
    assert r == 2.5 and c2.tobytes() == cubes.tobytes()
    lv = np.zeros(3, F.LEAF_DTYPE); lv["first_idx"] = [0, 10, 20]; lv["last_idx"] = [9, 19, 49]
    F.save_treetop(tmp_path / "t", lv, 2.5)
    l2, r = F.load_treetop(tmp_path / "t")
    assert r == 2.5 and l2.tobytes() == lv.tobytes()
    with pytest.raises(ValueError):
        F.load_cubes(tmp_path / "t")
    # byte layout of the 12/16-byte headers
    b = (tmp_path / "c").read_bytes()
    assert b[:4] == b"TGV1" and len(b) == 16 + 16 * 50
