"""Shared test setup: the ``gpu`` marker, import paths and fixture loaders.

Tests marked ``gpu`` need an sm_103 GPU and call the CUDA path through the C
ABI; everything else runs on the CPU (oracle, host logic, library exports)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(HERE, "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU; calls the CUDA path through the C ABI")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


def golden_maps(g):
    """Fixture maps -> list of dicts for the oracle (rt_inv as the reference computed it)."""
    maps = []
    for i in range(len(g["depths"])):
        fx, fy, cx, cy = (float(x) for x in g["k"][i])
        maps.append(dict(depth=g["depths"][i], rt=g["rt"][i], rt_inv=g["rt_inv"][i], fx=fx, fy=fy, cx=cx,
                         cy=cy, lidar=bool(g["lidar"][i])))
    return maps


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle
