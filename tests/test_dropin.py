"""The C++ drop-in (tgvreconclaude_gb300/dropin/tgv_dropin.cpp, surface_dropin.cpp,
octree_dropin.cpp) compiles against the reference's own headers and links into the
reference's own Stage-1, 2-4, 5 and 6 test programs in place of src/histogram.cpp,
src/tgv.cpp, src/octree_builder.cpp, src/merge.cpp and src/balance.cpp; the
Stage-7 replacement of src/marching_cubes.cpp compiles against the reference's
header (its test program also needs src/qslim.cpp, hence a full Eigen).  Needs the reference
checkout; without a GPU the programs must stop at their first call with the
no-device error (there is no CPU path)."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(REPO, "tgvreconclaude_gb300", "dropin")
import oracle  # noqa: E402  (tests/conftest.py puts oracle/ on the path)

REF_DIR = oracle.ref_dir()

pytestmark = pytest.mark.skipif(not REF_DIR or not os.path.isdir(os.path.join(REF_DIR, "tests")),
                                reason="reference checkout absent (set TGV_REFERENCE_DIR)")


def test_dropin_links_reference_tests():
    from tgvreconclaude_gb300 import _native
    _native.build()
    r = subprocess.run(["make", "-s", "-C", DROPIN, f"REF_DIR={REF_DIR}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for t in ("test_stage1_dropin", "test_stages2_4_dropin", "test_stage5_dropin", "test_stage6_dropin",
              "obj/surface_dropin.o", "obj/octree_dropin.o"):
        assert os.path.exists(os.path.join(DROPIN, "_build", t))


def test_dropin_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    exe = os.path.join(DROPIN, "_build", "test_stage6_dropin")
    if not os.path.exists(exe):
        test_dropin_links_reference_tests()
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode != 0
    assert "no usable sm_103 device" in r.stderr
