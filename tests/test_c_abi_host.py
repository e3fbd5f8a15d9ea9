"""A plain C host program (tests/c_abi_host.c) drives the solver through
include/tgvg.h alone, as a C, cgo or JNI binding of the reference's
tgv_minimize / tgv_minimize_oc / tgv_minimize_streaming would (reference
src/tgv.hpp).  On the CPU it must compile and link against the library and stop
with the no-device error; on the GPU its states must equal the golden states
the reference wrote, bit for bit, in all three semantics."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from tgvreconclaude_gb300 import _native as N, formats as F

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "c_abi_host.c")


def _compile(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    lib = N.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "c_abi_host")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-O2", "-I", os.path.join(REPO, "include"),
                        SRC, "-L", libdir, "-ltgvg", f"-Wl,-rpath,{libdir}", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _write_case(d, case):
    g = load_golden(case)
    cubes, hists, leaves = g["cubes"], g["hists"], g["leaves"]
    a0, a1 = (float(x) for x in g["params"])
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "meta.txt"), "w") as f:
        f.write(f"{len(cubes)} {hists.shape[1]} {len(leaves)} {int(g['iters'])} {a0!r} {a1!r}\n")
    np.ascontiguousarray(cubes, F.CUBE_DTYPE).tofile(os.path.join(d, "cubes.bin"))
    np.ascontiguousarray(hists, np.uint32).tofile(os.path.join(d, "hists.bin"))
    np.ascontiguousarray(leaves, F.LEAF_DTYPE).tofile(os.path.join(d, "leaves.bin"))
    return g


def test_c_host_program_links_and_fails_loudly_without_a_gpu(tmp_path):
    import torch
    exe = _compile(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    _write_case(str(tmp_path / "case"), "tgv_rand0.npz")
    r = subprocess.run([exe, str(tmp_path / "case")], capture_output=True, text=True)
    assert r.returncode == 2
    assert "no usable sm_103 device" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["tgv_rand0.npz", "tgv_balanced.npz"])
def test_c_host_program_matches_golden(tmp_path, case):
    exe = _compile(tmp_path)
    d = str(tmp_path / "case")
    g = _write_case(d, case)
    r = subprocess.run([exe, d], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for mode, name in ((0, "inmem"), (1, "oc"), (2, "stream")):
        got = np.fromfile(os.path.join(d, f"state_{mode}.bin"), F.STATE_DTYPE)
        assert got.tobytes() == np.ascontiguousarray(g[name], F.STATE_DTYPE).tobytes(), (case, name)
