"""Chunk sharding of the streaming semantics (tgvreconclaude_gb300/partition.py)
on CPU ranks: the sharded solve with one exchange per level equals the
single-process streaming solve bit for bit, whether every level-L cube or only
the published border/parent set is exchanged."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from tgvreconclaude_gb300 import partition, scenes as S

HERE = os.path.dirname(os.path.abspath(__file__))


def _case(seed, n=3000, nleaf=7):
    rng = np.random.default_rng(seed)
    cubes = S.random_octree(rng, dmin=1, dmax=6, target=n, shape=["sphere", "plane"][seed % 2])
    hists = S.random_histograms(rng, len(cubes), empty_frac=0.1)
    leaves = S.split_leaves(len(cubes), nleaf, rng, cubes, aligned=seed % 2 == 0)
    return cubes, hists, leaves, dict(alpha0=1.0, alpha1=2.0, iters=12)


def test_assign_chunks_is_balanced():
    rng = np.random.default_rng(0)
    leaves = np.zeros(40, partition.F.LEAF_DTYPE)
    sizes = rng.integers(50, 4000, 40)
    edges = np.concatenate([[0], np.cumsum(sizes)])
    leaves["first_idx"], leaves["last_idx"] = edges[:-1], edges[1:] - 1
    for w in (2, 3, 8):
        owner = partition.assign_chunks(leaves, w)
        load = np.bincount(owner, weights=sizes, minlength=w)
        assert load.max() - load.min() <= sizes.max()
        assert set(owner) == set(range(w))


@pytest.mark.parametrize("seed", [1, 2])
@pytest.mark.parametrize("world", [2, 3])
def test_emulated_ranks_match_single_process(oracle_lib, seed, world):
    cubes, hists, leaves, p = _case(seed)
    ref, _ = oracle_lib.tgv_solve(cubes, hists, leaves, "stream", p["alpha0"], p["alpha1"], p["iters"])
    full, sent_full = partition.emulate_ranks(cubes, hists, leaves, p, world, oracle_lib, "level")
    pub, sent_pub = partition.emulate_ranks(cubes, hists, leaves, p, world, oracle_lib, "publish")
    assert full.tobytes() == ref.tobytes()
    assert pub.tobytes() == ref.tobytes()
    assert sum(sent_pub) < sum(sent_full)  # the border/parent exchange is smaller


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


@pytest.mark.parametrize("exchange", ["publish", "level"])
def test_gloo_world2_matches_single_process(oracle_lib, tmp_path, exchange):
    cubes, hists, leaves, p = _case(3, n=2500, nleaf=5)
    case = tmp_path / "case.npz"
    np.savez(case, cubes=cubes, hists=hists, leaves=leaves, **{k: v for k, v in p.items()})
    out = tmp_path / "out.npz"
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                   CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, os.path.join(HERE, "partition_worker.py"), str(case), str(out),
                                       exchange], env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE))
    for pr in procs:
        _, err = pr.communicate(timeout=300)
        assert pr.returncode == 0, err.decode()[-2000:]
    got = np.load(out)["state"]
    ref, _ = oracle_lib.tgv_solve(cubes, hists, leaves, "stream", p["alpha0"], p["alpha1"], p["iters"])
    assert got.tobytes() == ref.tobytes()
