"""The multi-GPU form on CPU: world_size-2 gloo ranks, each joining its
A-shard of R with all of S (the oracle stands in for a GPU per rank).  The
shards' results are disjoint and together equal the full result (per-A-tile
summaries summed across ranks), and the bench's max-over-ranks timing
reduction picks the slowest rank.  Only the verification and the timing use
a collective; the join itself exchanges nothing."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, case, tiles, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "joinproject-dim3_gb300"), os.path.join(root, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    import dim3gpu
    from oracle import oracle_py as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    R, S = case
    Rs = dim3gpu.a_shard(R, rank, world)
    # S stays the larger side: pairs come back as (c, a)
    wp, n, _, _ = O.join_project(S, Rs)
    pairs = np.ascontiguousarray(wp.reshape(-1, 2)[:, ::-1]) if n else np.empty((0, 2), np.uint32)
    # every pair's A is in this rank's shard
    assert np.all(dim3gpu.fmix32_np(pairs[:, 0]) % np.uint64(world) == np.uint64(rank))
    summ = torch.from_numpy(O.tile_summary(pairs, None, tiles).view(np.int64).copy())
    dist.all_reduce(summ, op=dist.ReduceOp.SUM)  # int64 addition wraps like the uint64 hash sums
    t = torch.tensor([0.5 + rank], dtype=torch.float64)  # a rank's step time
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        np.save(os.path.join(out_dir, "sum.npy"), summ.numpy().view(np.uint64))
        np.save(os.path.join(out_dir, "t.npy"), t.numpy())
    dist.destroy_process_group()


@pytest.mark.parametrize("name", ["grd_small", "zipf_1m_s001"])
def test_a_sharded_replicas_cover_the_result(built, golden, name, tmp_path):
    import torch.multiprocessing as mp
    from helpers import case_inputs
    from oracle import oracle_py as O
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    tiles = 16
    mp.start_processes(_rank_main, args=(2, _free_port(), (R, S), tiles, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(str(tmp_path / "sum.npy"))
    wp, n, _, _ = O.join_project(R, S)
    want = O.tile_summary(wp.reshape(-1, 2), None, tiles)
    assert n == index[name]["n_out"]
    assert np.array_equal(got, want)
    assert float(np.load(str(tmp_path / "t.npy"))[0]) == 1.5
