"""GPU parity: the CUDA path against the reference's golden fixtures, through
the C ABI (host and device entry points), plus the edge cases the reference
exercises (empty inputs, no matches, swap, duplicates, extreme keys)."""
import numpy as np
import pytest

from helpers import case_inputs, check_groups, check_pairs

pytestmark = pytest.mark.gpu

CASES = ["empty_R", "empty_S", "no_match", "single", "extreme_keys", "heavy_duplicates", "one_join_value",
         "grd_tiny", "grd_swap_dense", "grd_small", "grd_classical", "grd_dense_z", "grd_swap", "grd_sparse",
         "grd_all_dense", "zipf_1m_s001", "zipf_1m_s01", "chung_lu_s0005", "chung_lu_s005"]


@pytest.mark.parametrize("name", CASES)
def test_join_project_host_api(ctx, golden, name):
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    got = ctx.join_project(R, S)
    check_pairs(got, index[name], arrays, name)
    st = ctx.stats()
    assert st["n_out"] == index[name]["n_out"]
    assert st["swapped"] == (1 if R.shape[0] < S.shape[0] else 0)


@pytest.mark.parametrize("name", CASES)
def test_join_count_host_api(ctx, golden, name):
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    pairs, cnt = ctx.join_count(R, S)
    check_groups(pairs, cnt, index[name], arrays, name)


@pytest.mark.parametrize("name", ["grd_small", "grd_swap", "chung_lu_s005", "zipf_1m_s001"])
def test_join_project_device_api(ctx, golden, name):
    import torch
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    n_need = index[name]["n_out"]
    # too small a buffer: CAPACITY with the size needed
    import dim3gpu
    small = torch.full((max(1, n_need // 2), 2), -1, dtype=torch.int32, device="cuda")
    if n_need > 1:
        with pytest.raises(dim3gpu.Dim3GError) as e:
            ctx.join_project_device(dR, R.shape[0], dS, S.shape[0], small, small.shape[0])
        assert e.value.code == dim3gpu.ERR_CAPACITY
        assert ctx.stats()["n_out"] == n_need
    assert ctx.join_project_count_device(dR, R.shape[0], dS, S.shape[0]) == n_need
    out = torch.empty((n_need + 5, 2), dtype=torch.int32, device="cuda")
    n = ctx.join_project_device(dR, R.shape[0], dS, S.shape[0], out, out.shape[0])
    torch.cuda.synchronize()
    got = out[:n].cpu().numpy().view(np.uint32)
    check_pairs(got, index[name], arrays, name)


@pytest.mark.parametrize("ordered", [0, 1])
@pytest.mark.parametrize("name", CASES)
def test_join_project_device_single_and_ordered(built, golden, name, ordered):
    """Every golden case through the device entry point with an exact buffer:
    the single pass (ordered_output=0) and the two-pass x-grouped form (1)."""
    import torch
    import dim3gpu
    from oracle import oracle_py as O
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    c = dim3gpu.Context(0)
    c.set_param("ordered_output", ordered)
    n_need = index[name]["n_out"]
    dR = torch.from_numpy(R.view(np.int32)).cuda() if R.shape[0] else torch.zeros((1, 2), dtype=torch.int32, device="cuda")
    dS = torch.from_numpy(S.view(np.int32)).cuda() if S.shape[0] else torch.zeros((1, 2), dtype=torch.int32, device="cuda")
    out = torch.empty((max(n_need, 1), 2), dtype=torch.int32, device="cuda")
    for _ in range(2):
        n = c.join_project_device(dR, R.shape[0], dS, S.shape[0], out, n_need)
        torch.cuda.synchronize()
        got = out[:n].cpu().numpy().view(np.uint32)
        check_pairs(got, index[name], arrays, name)
    if ordered and n > 1:
        # pairs of one first value are contiguous
        firsts = got[:, 0]
        changes = np.count_nonzero(firsts[1:] != firsts[:-1]) + 1
        assert changes == np.unique(firsts).shape[0]
    c.close()


def test_join_count_device_api(ctx, golden):
    import torch
    index, arrays = golden
    name = "grd_dense_z"
    R, S = case_inputs(name, index, arrays)
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    n_need = index[name]["n_groups"]
    oxz = torch.empty((n_need, 2), dtype=torch.int32, device="cuda")
    oc = torch.empty((n_need,), dtype=torch.int64, device="cuda")
    n = ctx.join_count_device(dR, R.shape[0], dS, S.shape[0], oxz, oc, n_need)
    torch.cuda.synchronize()
    check_groups(oxz[:n].cpu().numpy().view(np.uint32), oc[:n].cpu().numpy().view(np.uint64), index[name],
                 arrays, name)


@pytest.mark.parametrize("params", [
    {"warp_slots_log2": 5, "block_slots_log2": 8, "tile_bits_log2": 10},
    {"warp_slots_log2": 8, "block_slots_log2": 10, "tile_bits_log2": 12},
    {"warp_slots_log2": 11, "block_slots_log2": 14, "tile_bits_log2": 20},
])
def test_kernel_classes_and_tiling_agree(built, golden, params):
    """Every row class and z tiling gives the same answer (forces rows through
    the bitmap class with many z tiles, or through the hash classes)."""
    import dim3gpu
    index, arrays = golden
    c = dim3gpu.Context(0)
    for k, v in params.items():
        c.set_param(k, v)
    for name in ["grd_small", "grd_sparse", "chung_lu_s005", "zipf_1m_s001"]:
        R, S = case_inputs(name, index, arrays)
        check_pairs(c.join_project(R, S), index[name], arrays, name)
        p, cnt = c.join_count(R, S)
        check_groups(p, cnt, index[name], arrays, name)
    c.close()


@pytest.mark.parametrize("walk", [0, 1, 2, 3])
def test_cta_walks_agree(built, golden, walk):
    """Every way a CTA row's candidates are shared among its warps gives the
    same answer; small hash sets and narrow z tiles put most rows through the
    CTA classes, with many tiles (projection, ordered projection, per-A-tile
    summaries)."""
    import torch
    import dim3gpu
    from oracle import oracle_py as O
    index, arrays = golden
    c = dim3gpu.Context(0)
    for k, v in (("cta_walk", walk), ("warp_slots_log2", 6), ("block_slots_log2", 9), ("tile_bits_log2", 12)):
        c.set_param(k, v)
    for name in ["grd_small", "grd_sparse", "chung_lu_s005", "zipf_1m_s001", "heavy_duplicates", "one_join_value"]:
        R, S = case_inputs(name, index, arrays)
        check_pairs(c.join_project(R, S), index[name], arrays, name)
        c.set_param("ordered_output", 1)
        check_pairs(c.join_project(R, S), index[name], arrays, name)
        c.set_param("ordered_output", 0)
        dR = torch.from_numpy(R.view(np.int32)).cuda()
        dS = torch.from_numpy(S.view(np.int32)).cuda()
        got = c.join_project_summary(dR, R.shape[0], dS, S.shape[0], 16)
        assert int(got[:, 0].sum()) == index[name]["n_out"]
        assert str(int(got[:, 2].sum(dtype=np.uint64))) == index[name]["set_hash"]
    c.close()


@pytest.mark.parametrize("params", [
    {"warp_slots_log2": 6, "block_slots_log2": 9, "tile_bits_log2": 10},
    {"warp_slots_log2": 6, "block_slots_log2": 9, "tile_bits_log2": 14},
    {"tile_bits_log2": 19},
    {"tile_bits_log2": 20},
])
def test_streamed_bitmap_rows_agree(built, golden, params):
    """The bitmap-class rows with their S segments streamed into shared
    memory by bulk copies (stream_rows = 1): exact on every case, with many
    narrow z tiles (segments split across stages, many tile ends) and with
    the default and widest tiles; twice in a row on one context."""
    import torch
    import dim3gpu
    index, arrays = golden
    c = dim3gpu.Context(0)
    c.set_param("stream_rows", 1)
    for k, v in params.items():
        c.set_param(k, v)
    for name in CASES:
        R, S = case_inputs(name, index, arrays)
        for _ in range(2):
            check_pairs(c.join_project(R, S), index[name], arrays, name)
        if R.shape[0] and S.shape[0]:
            dR = torch.from_numpy(R.view(np.int32)).cuda()
            dS = torch.from_numpy(S.view(np.int32)).cuda()
            n = index[name]["n_out"]
            out = torch.empty((max(n, 1), 2), dtype=torch.int32, device="cuda")
            assert c.join_project_device(dR, R.shape[0], dS, S.shape[0], out, out.shape[0]) == n
            check_pairs(out[:n].cpu().numpy().view(np.uint32), index[name], arrays, name)
    c.close()


@pytest.mark.parametrize("split,block_lg,walk", [(1, 14, 3), (0, 14, 3), (1, 9, 3), (1, 12, 1), (1, 11, 0)])
def test_block_split_launches_agree(built, golden, split, block_lg, walk):
    """Block-class rows in three launches by hash-set size (block_split = 1,
    256-thread CTAs for the two smaller sizes) or one: exact on the cases
    with most rows in the block class (small warp sets), for several set
    sizes and CTA walks, twice on one context (the launches' row counters
    restart), and on the device-resident entry point."""
    import torch
    import dim3gpu
    index, arrays = golden
    c = dim3gpu.Context(0)
    for k, v in (("block_split", split), ("warp_slots_log2", 6), ("block_slots_log2", block_lg),
                 ("cta_walk", walk)):
        c.set_param(k, v)
    assert c.get_param("block_split") == split
    for name in ["grd_small", "grd_all_dense", "grd_dense_z", "chung_lu_s005", "zipf_1m_s001", "one_join_value",
                 "heavy_duplicates", "grd_sparse"]:
        R, S = case_inputs(name, index, arrays)
        for _ in range(2):
            check_pairs(c.join_project(R, S), index[name], arrays, name)
        dR = torch.from_numpy(R.view(np.int32)).cuda()
        dS = torch.from_numpy(S.view(np.int32)).cuda()
        n = index[name]["n_out"]
        out = torch.empty((max(n, 1), 2), dtype=torch.int32, device="cuda")
        assert c.join_project_device(dR, R.shape[0], dS, S.shape[0], out, out.shape[0]) == n
        check_pairs(out[:n].cpu().numpy().view(np.uint32), index[name], arrays, name)
        assert c.stats()["rows_block"] >= 0
    c.close()


@pytest.mark.parametrize("prefetch", [1, 0])
def test_prefetched_block_rows_agree(built, golden, prefetch):
    """Block-class rows with their metadata fetched ahead by a producer warp
    (prefetch_rows = 1) or not: exact on the golden cases with most rows in
    the block class (small warp sets), on rows of more than 64 join values
    (staged by the expanding warps) and on a row of 3000 join values (staged
    in blocks of 1024), against the oracle."""
    import dim3gpu
    from oracle import oracle_py as O
    index, arrays = golden
    c = dim3gpu.Context(0)
    for k, v in (("prefetch_rows", prefetch), ("warp_slots_log2", 6), ("block_slots_log2", 14)):
        c.set_param(k, v)
    for name in ["grd_small", "grd_all_dense", "grd_dense_z", "chung_lu_s005", "zipf_1m_s001", "one_join_value"]:
        R, S = case_inputs(name, index, arrays)
        check_pairs(c.join_project(R, S), index[name], arrays, name)
    rng = np.random.default_rng(11)
    R = np.stack([np.zeros(3000, np.uint32), np.arange(3000, dtype=np.uint32)], 1)
    R = np.concatenate([R, rng.integers(1, 50, size=(2000, 2)).astype(np.uint32)])
    S = np.stack([rng.integers(0, 6000, 5000), rng.integers(0, 3000, 5000)], 1).astype(np.uint32)
    want, n, h, _ = O.join_project(R, S)
    got = c.join_project(R, S)
    assert got.shape[0] == n and O.set_hash(got) == h
    assert np.array_equal(O.sorted_pairs(got), O.sorted_pairs(want))
    c.close()


@pytest.mark.parametrize("sized,slack", [(1, 150), (0, 150), (1, 10)])
def test_mapping_tables_sized_by_sketch(built, golden, sized, slack):
    """The mapping's hash tables sized by the distinct-key sketch (far
    smaller than tuple-sized ones where keys repeat), tuple-sized, and sized
    too small on purpose (10 % of the distinct keys): the overfilled build is
    detected and redone at full size.  All exact."""
    import dim3gpu
    index, arrays = golden
    c = dim3gpu.Context(0)
    c.set_param("sized_tables", sized)
    c.set_param("table_slack_pct", slack)
    for name in ["chung_lu_s005", "grd_sparse", "zipf_1m_s001", "heavy_duplicates", "extreme_keys", "grd_classical"]:
        R, S = case_inputs(name, index, arrays)
        check_pairs(c.join_project(R, S), index[name], arrays, name)
        p, cnt = c.join_count(R, S)
        check_groups(p, cnt, index[name], arrays, name)
        st = c.stats()
        full = 2 * (1 << int(np.ceil(np.log2(max(1024, 2 * max(R.shape[0], S.shape[0]))))))
        if sized and slack == 10 and st["nx"] > 2000:
            assert st["table_rebuilds"] == 1, (name, st["table_slots"])
        if sized and slack == 150 and name == "chung_lu_s005":
            assert st["table_rebuilds"] == 0 and st["table_slots"] < full, (st["table_slots"], full)
    c.close()


def test_repeated_calls_are_stable(ctx, golden):
    index, arrays = golden
    R, S = case_inputs("chung_lu_s005", index, arrays)
    for _ in range(3):
        check_pairs(ctx.join_project(R, S), index["chung_lu_s005"], arrays, "chung_lu_s005")


def test_bad_params_rejected(ctx):
    import dim3gpu
    with pytest.raises(dim3gpu.Dim3GError):
        ctx.set_param("warp_slots_log2", 40)
    with pytest.raises(dim3gpu.Dim3GError):
        ctx.set_param("no_such_knob", 1)


def test_mapper_matches_sequential_insert_semantics(ctx):
    """GPU L+S mapper: ids equal those of a sequential LS_mapper insert loop."""
    import dim3gpu
    rng = np.random.default_rng(3)
    m = dim3gpu.Mapper(ctx, 16)
    ref = {}
    cnt = 0
    for batch in range(4):
        keys = rng.integers(0, 5000, size=20000, dtype=np.uint64).astype(np.uint32)
        if batch == 2:
            keys[:5] = [0xFFFFFFFF, 0, 0xFFFFFFFF, 7, 0]
        ids = m.insert(keys)
        want = np.empty_like(ids)
        for i, k in enumerate(keys.tolist()):
            if k not in ref:
                ref[k] = cnt
                cnt += 1
            want[i] = ref[k]
        assert np.array_equal(ids, want)
        assert m.size() == cnt
    probe = np.array([0xFFFFFFFF, 0, 123456789, 7], dtype=np.uint32)
    f = m.find(probe)
    assert f.tolist() == [ref.get(int(k), -1) for k in probe]
    m.clear()
    assert (m.find(probe) == -1).all()
    assert m.size() == cnt  # clear() keeps the counter (L+S_mapper.hpp:37-40)
    ids = m.insert(np.array([5, 6, 5], dtype=np.uint32))
    assert ids.tolist() == [cnt, cnt + 1, cnt]
    m.set_cnt(0)
    m.clear()
    assert m.insert(np.array([9], dtype=np.uint32)).tolist() == [0]
    m.close()


def test_autotune_applies_settings_and_keeps_results_exact(built, golden, tmp_path):
    """The autotuner times the join under candidate settings, applies the
    fastest (never slower than the starting settings) and the results under
    them stay exact; the cache round-trips the chosen settings."""
    import torch
    import dim3gpu
    index, arrays = golden
    c = dim3gpu.Context(0)
    name = "chung_lu_s005"
    R, S = case_inputs(name, index, arrays)
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    key = c.tuning_key(dR, R.shape[0], dS, S.shape[0])
    assert key.startswith("p")
    t = c.autotune(dR, R.shape[0], dS, S.shape[0], max_trials=8)
    assert 1 <= t["trials"] <= 8 and t["ms"] <= t["ms_default"]
    for k in ["tile_bits_log2", "block_threads", "block_slots_log2", "warp_slots_log2", "cta_walk", "dense_block",
              "dense_k_max"]:
        assert c.get_param(k) == t[k]
    check_pairs(c.join_project(R, S), index[name], arrays, name)
    path = str(tmp_path / "t.txt")
    dim3gpu.tuning_save(path, key, t)
    c2 = dim3gpu.Context(0)
    c2.apply_tuning(dim3gpu.tuning_load(path, key))
    assert c2.get_param("tile_bits_log2") == t["tile_bits_log2"]
    p, cnt = c2.join_count(R, S)
    check_groups(p, cnt, index[name], arrays, name)
    c.close()
    c2.close()


@pytest.mark.parametrize("name,dense", [("grd_all_dense", True), ("chung_lu_s005", False)])
def test_autotune_chooses_the_dense_sparse_split(built, golden, name, dense):
    """The dense/sparse split is tuned by measurement: the tuner times the
    heavy rows on the sparse kernels (dense_block 0), through the tensor-core
    product (2) and by the calibrated cost model (1), then how many join
    values the product takes (dense_k_max), and keeps the fastest.  The
    all-dense case's heavy rows are dense (every (x, z) group exists: a
    product over its heaviest join values beats expanding them); the 2-hop's
    are not (1 % output density in its heavy rows).  Results under the
    choice are exact."""
    import torch
    import dim3gpu
    index, arrays = golden
    c = dim3gpu.Context(0)
    cal = c.calibrate()
    assert cal["fp8_tflops"] > 500 and cal["hbm_gbs"] > 1000 and cal["tile_us"] > 0
    R, S = case_inputs(name, index, arrays)
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    t = c.autotune(dR, R.shape[0], dS, S.shape[0])
    assert t["ms"] <= t["ms_default"]
    assert c.get_param("dense_block") == t["dense_block"] and c.get_param("dense_k_max") == t["dense_k_max"]
    n = c.join_project_count_device(dR, R.shape[0], dS, S.shape[0])
    out = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    assert c.join_project_device(dR, R.shape[0], dS, S.shape[0], out, n) == n
    took_dense = c.stats()["rows_dense"] > 0
    assert took_dense == dense, (name, t, c.stats()["dense_skip"])
    check_pairs(out.cpu().numpy().view(np.uint32), index[name], arrays, name)
    c.close()


@pytest.mark.parametrize("name", ["grd_small", "grd_swap", "heavy_duplicates", "zipf_1m_s001", "chung_lu_s005",
                                  "empty_S", "extreme_keys"])
def test_summaries_match_oracle_per_tile(ctx, golden, name):
    """Per-A-tile summaries (nothing written) of the join-project and the
    COUNT join-aggregate equal the oracle's, on all tiles and on a slice."""
    import torch
    from oracle import oracle_py as O
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    dR = torch.from_numpy(R.view(np.int32)).cuda() if R.shape[0] else 0
    dS = torch.from_numpy(S.view(np.int32)).cuda() if S.shape[0] else 0
    wp, n, _, _ = O.join_project(R, S)
    wg, wc, ng, _, _ = O.join_count(R, S)
    tiles = 64
    want_p = O.tile_summary(wp.reshape(-1, 2) if n else np.empty((0, 2), np.uint32), None, tiles)
    want_c = O.tile_summary(wg.reshape(-1, 2) if ng else np.empty((0, 2), np.uint32),
                            wc if ng else np.empty(0, np.uint64), tiles)
    got_p = ctx.join_project_summary(dR, R.shape[0], dS, S.shape[0], tiles)
    got_c = ctx.join_count_summary(dR, R.shape[0], dS, S.shape[0], tiles)
    assert np.array_equal(got_p, want_p), name
    assert np.array_equal(got_c, want_c), name
    assert int(got_p[:, 0].sum()) == index[name]["n_out"]
    lo, hi = 8, 24
    sl = ctx.join_count_summary(dR, R.shape[0], dS, S.shape[0], tiles, lo, hi)
    assert np.array_equal(sl[lo:hi], want_c[lo:hi]) and not sl[:lo].any() and not sl[hi:].any()


@pytest.mark.parametrize("direct", [1, 0])
def test_into_pinned_host_buffer(built, golden, direct):
    """dim3g_join_project_into with a pinned (mapped) host buffer: the
    kernels store into it directly (host_direct_output = 1) or through the
    staging copy (0); both exact, and a too-small pinned buffer reports the
    size needed."""
    import torch
    import dim3gpu
    index, arrays = golden
    c = dim3gpu.Context(0)
    c.set_param("host_direct_output", direct)
    for name in ["grd_small", "grd_swap", "chung_lu_s005", "zipf_1m_s001", "empty_S"]:
        R, S = case_inputs(name, index, arrays)
        need = index[name]["n_out"]
        out = torch.empty((max(need, 1), 2), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        n = c.join_project_into(R, S, out)
        assert n == need
        check_pairs(out[:n], index[name], arrays, name)
        if need > 1:
            small = torch.empty((need // 2, 2), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
            with pytest.raises(dim3gpu.Dim3GError) as e:
                c.join_project_into(R, S, small)
            assert e.value.code == dim3gpu.ERR_CAPACITY and c.stats()["n_out"] == need
    c.close()
