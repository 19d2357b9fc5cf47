"""Parity at the benchmarked sizes, through size-independent checks.

The fixtures of test_join_gpu.py stop at 1/10 of the 1M-tuple Zipf case and
1/200 of the 20M-edge 2-hop.  Here the workloads run at the sizes the
benchmark times them at:

* the 20M-edge Chung-Lu 2-hop (10.9e9 distinct pairs): the per-A-tile
  summaries of the whole join (64 tiles) against the oracle run on the rows
  of R of three tiles with all of S (the join is row-separable in A, so a
  tile's pairs come only from its own rows); the tiles' totals against the
  pair count of the materialising entry point; the materialised output
  (87.4 GB, the benchmark's call) hashed on the device against the sum of
  the tile hashes; OUT_J against its definition;
* the 1M-tuple Zipf case (2.35e9 pairs): the materialised output's count and
  set hash against the reference itself (fixture zipf_1m_full, recorded by
  tests/golden/make_golden.py --large from the reference compiled from its
  own sources);
* the 16M x 16M Zipf-1.2 COUNT (about 9.9e11 groups, which no memory holds):
  a 1/4096 A-slice's groups, count sum and group hash against the oracle on
  that slice's rows, and the count sum of all 16 A-slices against OUT_J.

The oracle runs with every host core (its OpenMP form).  Comparisons are
exact (integer pairs, counts and 64-bit hashes).
"""
import os

import numpy as np
import pytest

from helpers import device_set_hash, exact_out_j, tile_rows

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

THREADS = os.cpu_count() or 1


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _oracle_tile_project(S, Rs, tiles, t):
    """Tile t's (groups, groups, hash) from the oracle on the tile's rows of R
    with all of S.  S is passed first so it stays the larger side (no swap of
    roles): the oracle's pairs are then (c, a), transposed back here."""
    from oracle import oracle_py as O
    pairs, n, _, _ = O.join_project(S, Rs, threads=THREADS)
    assert pairs.shape[0] == n
    return O.tile_summary(np.ascontiguousarray(pairs[:, ::-1]), None, tiles, t, t + 1)[t]


def test_chung_lu_20m_full_size(built):
    import torch

    import dim3gpu

    R, S = dim3gpu.workload("chung_lu_20m", 1.0)
    assert R.shape[0] == 19999188
    dR, dS = _dev(R), _dev(S)
    ctx = dim3gpu.Context(0)
    tiles = 64
    sm = ctx.join_project_summary(dR, R.shape[0], dS, S.shape[0], tiles)
    n = ctx.join_project_count_device(dR, R.shape[0], dS, S.shape[0])
    assert ctx.stats()["out_j"] == exact_out_j(R, S) == 16354723326
    assert int(sm[:, 0].sum()) == n == 10925644404
    assert np.array_equal(sm[:, 0], sm[:, 1])
    # the benchmark's call: every pair materialised in device memory
    out = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    assert ctx.join_project_device(dR, R.shape[0], dS, S.shape[0], out, n) == n
    torch.cuda.synchronize()
    head = out[:1 << 20].cpu().numpy().view(np.uint32)
    from oracle import oracle_py as O
    assert device_set_hash(out, 1 << 20) == O.set_hash(head)  # the device hash is the oracle's hash
    assert device_set_hash(out, n) == int(sm[:, 2].sum(dtype=np.uint64))
    del out
    ctx.close()
    torch.cuda.empty_cache()
    for t in (0, 21, 63):
        want = _oracle_tile_project(S, tile_rows(R, tiles, t), tiles, t)
        assert np.array_equal(sm[t], want), (t, sm[t], want)


def test_zipf_1m_full_size_matches_reference(built, golden):
    import torch

    import dim3gpu

    index, _ = golden
    rec = index["zipf_1m_full"]
    R, S = dim3gpu.workload("zipf_1m", 1.0)
    from helpers import input_hash
    assert str(input_hash(R, S)) == rec["input_hash"]
    dR, dS = _dev(R), _dev(S)
    ctx = dim3gpu.Context(0)
    for dense in (1, 0):  # the cost model's choice (the dense block) and the sparse kernels alone
        ctx.set_param("dense_block", dense)
        n = ctx.join_project_count_device(dR, R.shape[0], dS, S.shape[0])
        assert n == rec["n_out"]
        out = torch.empty((n, 2), dtype=torch.int32, device="cuda")
        assert ctx.join_project_device(dR, R.shape[0], dS, S.shape[0], out, n) == n
        if dense:
            assert ctx.stats()["rows_dense"] > 0
        assert str(device_set_hash(out, n)) == rec["set_hash"], dense
        del out
        torch.cuda.empty_cache()
    ctx.close()


def test_count16m_slice_and_totals(built):
    import dim3gpu
    from oracle import oracle_py as O

    R, S = dim3gpu.workload("zipf12_16m", 1.0)
    dR, dS = _dev(R), _dev(S)
    ctx = dim3gpu.Context(0)
    # a 1/4096 A-slice against the oracle on that slice's rows
    fine = 4096
    sm = ctx.join_count_summary(dR, R.shape[0], dS, S.shape[0], fine, 0, 1)
    Rs = tile_rows(R, fine, 0)
    pairs, cnt, ng, _, _ = O.join_count(S, Rs, threads=THREADS)
    want = O.tile_summary(np.ascontiguousarray(pairs[:, ::-1]), cnt, fine, 0, 1)[0]
    assert ng > 10 ** 8
    assert np.array_equal(sm[0], want), (sm[0], want)
    assert not sm[1:].any()
    # all of the join in 16 A-slices: the counts add up to OUT_J exactly
    coarse = 16
    tot = np.zeros((coarse, 3), dtype=np.uint64)
    for k in range(coarse):
        tot += ctx.join_count_summary(dR, R.shape[0], dS, S.shape[0], coarse, k, k + 1)
    assert int(tot[:, 1].sum()) == exact_out_j(R, S)
    # slice 0 of 16 contains slice 0 of 4096 (fmix32(a) & 15 == 0 there)
    assert int(tot[0, 0]) > int(sm[0, 0])
    ctx.close()
