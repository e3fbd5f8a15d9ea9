"""One CPU rank of the sharded streaming solve (run by tests/test_partition.py
as a gloo process group of 127.0.0.1 ranks).

usage: RANK=r WORLD_SIZE=w MASTER_ADDR=127.0.0.1 MASTER_PORT=p python partition_worker.py case.npz out.npz exchange
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import torch.distributed as dist  # noqa: E402

import oracle  # noqa: E402
from tgvreconclaude_gb300 import partition  # noqa: E402


def main():
    case, out, exchange = sys.argv[1], sys.argv[2], sys.argv[3]
    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    d = np.load(case)
    params = dict(alpha0=float(d["alpha0"]), alpha1=float(d["alpha1"]), iters=int(d["iters"]))

    def allgather(obj):
        res = [None] * world
        dist.all_gather_object(res, obj)
        return res

    state, owner, sent = partition.sharded_stream_solve(d["cubes"], d["hists"], d["leaves"], params, rank, world,
                                                        allgather, oracle, exchange)
    # gather each rank's own cubes to rank 0
    lo_of = partition.leaf_of(len(d["cubes"]), d["leaves"])
    own = np.where(lo_of >= 0, owner[np.maximum(lo_of, 0)], -1)
    mine = np.nonzero(own == rank)[0]
    parts = allgather((mine, state[mine].copy()))
    if rank == 0:
        merged = state.copy()
        for ix, vals in parts:
            merged[ix] = vals
        np.savez(out, state=merged, sent=np.array(sent))
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
