"""GPU parity of the dense block -- the heavy rows' join through their
heaviest join values as one boolean product on the tensor cores
(csrc/dense.cuh) -- against the golden fixtures.  The block is forced on
(dense_block=2) with small hash tables so that most rows are heavy, with a
product over few join values (most candidates then go through the light
pass) and over many; single pass, ordered, and count only."""
import numpy as np
import pytest

from helpers import case_inputs, check_pairs

pytestmark = pytest.mark.gpu

CASES = ["empty_R", "empty_S", "no_match", "single", "extreme_keys", "heavy_duplicates", "one_join_value",
         "grd_tiny", "grd_swap_dense", "grd_small", "grd_classical", "grd_dense_z", "grd_swap", "grd_sparse",
         "grd_all_dense", "zipf_1m_s001", "chung_lu_s0005", "chung_lu_s005"]


def _dev(a):
    import torch
    if a.shape[0] == 0:
        return torch.zeros((1, 2), dtype=torch.int32, device="cuda")
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _ctx(params):
    import dim3gpu
    c = dim3gpu.Context(0)
    for k, v in params.items():
        c.set_param(k, v)
    return c


@pytest.mark.parametrize("kmax,mem_mb", [(32, 16384), (1024, 16384), (1024, 1)])
@pytest.mark.parametrize("ordered", [0, 1])
def test_dense_block_forced_matches_golden(built, golden, kmax, mem_mb, ordered):
    """mem_mb = 1: the bitmap budget holds only some of the heavy rows; the
    block takes the first of them and the bitmap-class kernels the rest."""
    import torch
    index, arrays = golden
    c = _ctx({"dense_block": 2, "dense_k_max": kmax, "dense_mem_mb": mem_mb, "ordered_output": ordered,
              "warp_slots_log2": 5, "block_slots_log2": 8})
    partial = 0
    used = []
    for name in CASES:
        R, S = case_inputs(name, index, arrays)
        n_need = index[name]["n_out"]
        dR, dS = _dev(R), _dev(S)
        out = torch.empty((max(n_need, 1), 2), dtype=torch.int32, device="cuda")
        n = c.join_project_device(dR, R.shape[0], dS, S.shape[0], out, n_need)
        torch.cuda.synchronize()
        got = out[:n].cpu().numpy().view(np.uint32)
        check_pairs(got, index[name], arrays, name)
        st = c.stats()
        if st["rows_dense"]:
            used.append(name)
            assert 0 < st["heavy_y"] <= kmax and st["dense_kp"] % 128 == 0
            partial += st["rows_bitmap"] > 0
        if ordered and n > 1:
            firsts = got[:, 0]
            assert np.count_nonzero(firsts[1:] != firsts[:-1]) + 1 == np.unique(firsts).shape[0]
        assert c.join_project_count_device(dR, R.shape[0], dS, S.shape[0]) == n_need, name
    assert len(used) >= 8, used
    if mem_mb == 1:
        assert partial >= 2, partial
    c.close()


def test_dense_block_larger_cases(built, golden):
    """Cases whose heavy rows fill many product tiles (grid-stride over
    tiles, both accumulators in turn), forced and by the cost model."""
    import torch
    index, arrays = golden
    small = {"warp_slots_log2": 5, "block_slots_log2": 8}
    for params in ({"dense_block": 2, **small}, {"dense_block": 2, "dense_k_max": 256, **small}, {"dense_block": 1}):
        c = _ctx(params)
        for name in ["zipf_1m_s01", "grd_all_dense"]:
            R, S = case_inputs(name, index, arrays)
            n_need = index[name]["n_out"]
            out = torch.empty((n_need, 2), dtype=torch.int32, device="cuda")
            n = c.join_project_device(_dev(R), R.shape[0], _dev(S), S.shape[0], out, n_need)
            torch.cuda.synchronize()
            check_pairs(out[:n].cpu().numpy().view(np.uint32), index[name], arrays, name)
            st = c.stats()
            if params["dense_block"] == 2:
                assert st["rows_dense"] > 0, (name, st)
        c.close()


def test_dense_block_off_and_knobs(ctx):
    import dim3gpu
    for k, bad in (("dense_block", 3), ("dense_k_max", 16), ("dense_k_max", 8192), ("dense_mem_mb", 0)):
        with pytest.raises(dim3gpu.Dim3GError):
            ctx.set_param(k, bad)
    ctx.set_param("dense_block", 0)
    assert ctx.get_param("dense_block") == 0
    ctx.set_param("dense_block", 1)


@pytest.mark.timeout(600, method="thread")
@pytest.mark.parametrize("kmax", [32, 4096])
def test_dense_block_summaries_match_oracle(built, golden, kmax):
    """Per-A-tile summaries with the dense block forced: the product's
    counts in the fused epilogue, the light candidates bucketed by tile and
    added per group, equal the oracle's tile summaries of the join-project
    and the COUNT join-aggregate, on all tiles and on a slice.  With few
    join values in the product most candidates are light and the buckets
    too large, so the sparse kernels run instead (exact either way)."""
    import torch
    from oracle import oracle_py as O
    index, arrays = golden
    c = _ctx({"dense_block": 2, "dense_k_max": kmax, "warp_slots_log2": 5, "block_slots_log2": 8})
    used = []
    for name in ["grd_small", "grd_swap", "grd_dense_z", "heavy_duplicates", "one_join_value", "zipf_1m_s001",
                 "chung_lu_s0005", "chung_lu_s005"]:
        R, S = case_inputs(name, index, arrays)
        dR, dS = _dev(R), _dev(S)
        wp, n, _, _ = O.join_project(R, S)
        wg, wc, ng, _, _ = O.join_count(R, S)
        tiles = 64
        want_p = O.tile_summary(wp.reshape(-1, 2) if n else np.empty((0, 2), np.uint32), None, tiles)
        want_c = O.tile_summary(wg.reshape(-1, 2) if ng else np.empty((0, 2), np.uint32),
                                wc if ng else np.empty(0, np.uint64), tiles)
        got_p = c.join_project_summary(dR, R.shape[0], dS, S.shape[0], tiles)
        used_p = c.stats()["rows_dense"]
        got_c = c.join_count_summary(dR, R.shape[0], dS, S.shape[0], tiles)
        used_c = c.stats()["rows_dense"]
        assert np.array_equal(got_p, want_p), name
        assert np.array_equal(got_c, want_c), name
        lo, hi = 8, 24
        sl = c.join_count_summary(dR, R.shape[0], dS, S.shape[0], tiles, lo, hi)
        assert np.array_equal(sl[lo:hi], want_c[lo:hi]) and not sl[:lo].any() and not sl[hi:].any(), name
        if used_p and used_c:
            used.append(name)
    if kmax == 4096:
        assert len(used) >= 3, used
    c.close()
