"""GPU parity of the many-query paths -- resident relation sets
(dim3g_relset_join) and batches run as one CUDA graph (dim3g_batch_run) --
against the golden fixtures and, for joins across cases, the oracle.  Every
query's result must equal what it gives alone."""
import numpy as np
import pytest

from helpers import case_inputs, check_groups, check_pairs

pytestmark = pytest.mark.gpu

CASES = ["empty_R", "empty_S", "no_match", "single", "extreme_keys", "heavy_duplicates", "one_join_value",
         "grd_tiny", "grd_swap_dense", "grd_small", "grd_classical", "grd_dense_z", "grd_swap", "grd_sparse",
         "zipf_1m_s001", "chung_lu_s0005", "chung_lu_s005"]


def _dev(a):
    import torch
    if a.shape[0] == 0:
        return 0
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _inputs(golden, names):
    index, arrays = golden
    host, rels = [], []
    for name in names:
        R, S = case_inputs(name, index, arrays)
        host.append((R, S))
        rels += [(_dev(R), R.shape[0]), (_dev(S), S.shape[0])]
    return host, rels


def _specs(golden, names, ops):
    """One query per (case, op): exact-size outputs."""
    import torch
    import dim3gpu
    index, _ = golden
    specs = []
    for i, name in enumerate(names):
        for op in ops:
            n = index[name]["n_out"] if op == dim3gpu.OP_PROJECT else index[name]["n_groups"]
            s = {"r": 2 * i, "s": 2 * i + 1, "op": op, "capacity": n, "name": name,
                 "out": torch.empty((max(n, 1), 2), dtype=torch.int32, device="cuda")}
            if op == dim3gpu.OP_COUNT:
                s["cnt"] = torch.empty((max(n, 1),), dtype=torch.int64, device="cuda")
            specs.append(s)
    return specs


def _check(golden, specs, res):
    import torch
    import dim3gpu
    index, arrays = golden
    torch.cuda.synchronize()
    for s, r in zip(specs, res):
        name = s["name"]
        assert r["status"] == 0, (name, r)
        n = r["n_out"]
        pairs = s["out"][:n].cpu().numpy().view(np.uint32)
        if s["op"] == dim3gpu.OP_PROJECT:
            check_pairs(pairs, index[name], arrays, name)
        else:
            check_groups(pairs, s["cnt"][:n].cpu().numpy().view(np.uint64), index[name], arrays, name)


@pytest.mark.parametrize("params", [
    {},
    {"warp_slots_log2": 5, "block_slots_log2": 8, "tile_bits_log2": 10},
    {"warp_slots_log2": 8, "block_slots_log2": 10, "tile_bits_log2": 12},
    {"warp_slots_log2": 6, "block_slots_log2": 12, "block_split": 0},
])
def test_relset_golden_project_and_count(built, golden, params):
    """All golden cases as one relation set; every case's join-project and
    COUNT join-aggregate in one mixed pass (forced classes and z tilings in
    the parametrised runs; block-class rows in three launches by hash-set
    size unless block_split = 0)."""
    import dim3gpu
    c = dim3gpu.Context(0)
    for k, v in params.items():
        c.set_param(k, v)
    _, rels = _inputs(golden, CASES)
    rs = dim3gpu.RelSet(c, rels)
    assert rs.bytes() > 0
    specs = _specs(golden, CASES, [dim3gpu.OP_PROJECT, dim3gpu.OP_COUNT])
    res = rs.join(specs)
    _check(golden, specs, res)
    # the same set, queries in another order and one at a time
    for s in specs[::-7]:
        _check(golden, [s], rs.join([s]))
    rs.close()
    c.close()


@pytest.mark.parametrize("sized,slack", [(1, 150), (0, 150), (1, 5)])
def test_relset_tables_sized_by_sketch(built, golden, sized, slack):
    """The relation set's value -> id tables sized per relation by a
    distinct-key sketch (smaller than tuple-sized ones: fewer device bytes),
    tuple-sized, and sized far too small on purpose (5 % of the distinct
    keys): the overfilled build is detected and redone with tuple-sized
    tables.  Every query exact in each case."""
    import dim3gpu
    _, rels = _inputs(golden, CASES)
    sizes = {}
    for sz, sl in [(0, 150), (sized, slack)]:
        c = dim3gpu.Context(0)
        c.set_param("sized_tables", sz)
        c.set_param("table_slack_pct", sl)
        rs = dim3gpu.RelSet(c, rels)
        sizes[(sz, sl)] = rs.bytes()
        specs = _specs(golden, CASES, [dim3gpu.OP_PROJECT, dim3gpu.OP_COUNT])
        _check(golden, specs, rs.join(specs))
        rs.close()
        c.close()
    if sized and slack == 150:
        assert sizes[(1, 150)] < sizes[(0, 150)], sizes
    if sized and slack == 5:
        assert sizes[(1, 5)] >= sizes[(0, 150)], sizes  # rebuilt with tuple-sized tables


def test_batch_sized_tables_overflow_rebuilds(built, golden):
    """A batch whose sketch-sized tables are too small (5 % slack): its first
    run detects the overflow, re-plans with tuple-sized tables, re-captures
    the graph and returns exact results; later runs replay the new graph."""
    import dim3gpu
    c = dim3gpu.Context(0)
    c.set_param("table_slack_pct", 5)
    names = ["grd_small", "zipf_1m_s001", "chung_lu_s005", "heavy_duplicates", "grd_sparse"]
    _, rels = _inputs(golden, names)
    pairs = [(rels[2 * i], rels[2 * i + 1]) for i in range(len(names))]
    specs = _specs(golden, names, [dim3gpu.OP_PROJECT])
    b = dim3gpu.Batch(c, pairs, specs)
    small = b.info()["device_bytes"]
    for _ in range(2):
        _check(golden, specs, b.run())
    assert b.info()["device_bytes"] > small
    b.close()
    c.close()


def test_relset_cross_joins_match_oracle(ctx, golden):
    """Joins across cases (R of one, S of another, both orientations) against
    the oracle on the same relations."""
    import torch
    import dim3gpu
    from oracle import oracle_py as O
    names = ["grd_tiny", "grd_small", "grd_swap_dense", "zipf_1m_s001", "heavy_duplicates"]
    host, rels = _inputs(golden, names)
    rs = dim3gpu.RelSet(ctx, rels)
    pairs = [(0, 3), (3, 0), (2, 5), (5, 2), (6, 7), (9, 1), (8, 9)]
    specs, want = [], []
    for r, s in pairs:
        R, S = host[r // 2][r % 2], host[s // 2][s % 2]
        wp, n, h, _ = O.join_project(R, S)
        wg, wc, ng, hg, _ = O.join_count(R, S)
        want.append((wp, wg, wc))
        specs.append({"r": r, "s": s, "op": dim3gpu.OP_PROJECT, "capacity": n,
                      "out": torch.empty((max(n, 1), 2), dtype=torch.int32, device="cuda")})
        specs.append({"r": r, "s": s, "op": dim3gpu.OP_COUNT, "capacity": ng,
                      "out": torch.empty((max(ng, 1), 2), dtype=torch.int32, device="cuda"),
                      "cnt": torch.empty((max(ng, 1),), dtype=torch.int64, device="cuda")})
    res = rs.join(specs)
    torch.cuda.synchronize()
    for k, (r, s) in enumerate(pairs):
        wp, wg, wc = want[k]
        sp, sg = specs[2 * k], specs[2 * k + 1]
        rp, rg = res[2 * k], res[2 * k + 1]
        assert rp["swapped"] == (1 if host[r // 2][r % 2].shape[0] < host[s // 2][s % 2].shape[0] else 0)
        got = sp["out"][:rp["n_out"]].cpu().numpy().view(np.uint32)
        assert np.array_equal(np.sort(O.pair_keys(got)), np.sort(O.pair_keys(wp))), (r, s)
        gp = sg["out"][:rg["n_out"]].cpu().numpy().view(np.uint32)
        gc = sg["cnt"][:rg["n_out"]].cpu().numpy().view(np.uint64)
        o1, o2 = np.argsort(O.pair_keys(gp)), np.argsort(O.pair_keys(wg))
        assert np.array_equal(O.pair_keys(gp)[o1], O.pair_keys(wg)[o2]), (r, s)
        assert np.array_equal(gc[o1], np.asarray(wc, dtype=np.uint64)[o2]), (r, s)
    rs.close()


def test_relset_capacity_is_per_query(ctx, golden):
    import torch
    import dim3gpu
    names = ["grd_small", "grd_tiny"]
    _, rels = _inputs(golden, names)
    rs = dim3gpu.RelSet(ctx, rels)
    specs = _specs(golden, names, [dim3gpu.OP_PROJECT])
    need = specs[0]["capacity"]
    specs[0]["capacity"] = need // 2
    res = rs.join(specs, check=False)
    assert res[0]["status"] == dim3gpu.ERR_CAPACITY and res[0]["n_out"] == need
    specs[0]["capacity"] = need
    _check(golden, specs[1:], res[1:])
    with pytest.raises(dim3gpu.Dim3GError):
        rs.join([{"r": 9, "s": 0, "op": 0, "capacity": 0}])
    rs.close()


def test_batch_graph_matches_golden_and_replays(ctx, golden):
    """Independent joins planned once and run as one CUDA graph launch; the
    second launch (a replay) gives the same exact results."""
    import dim3gpu
    _, rels = _inputs(golden, CASES)
    pairs = [(rels[2 * i], rels[2 * i + 1]) for i in range(len(CASES))]
    specs = _specs(golden, CASES, [dim3gpu.OP_PROJECT])
    specs_c = _specs(golden, CASES, [dim3gpu.OP_COUNT])
    # project and COUNT joins of every case: 2 x |CASES| joins
    b = dim3gpu.Batch(ctx, pairs + pairs, specs + specs_c)
    for _ in range(2):
        res = b.run()
        _check(golden, specs + specs_c, res)
    info = b.info()
    assert info["launches_per_run"] > 0 and info["ms_last"] > 0
    b.close()


def test_batch_autotune_keeps_results_exact(built, golden):
    """The batch autotuner re-captures and times the graph under candidate
    settings; afterwards the graph (with the chosen settings) is exact."""
    import dim3gpu
    c = dim3gpu.Context(0)
    names = ["grd_small", "grd_swap", "zipf_1m_s001", "chung_lu_s005", "heavy_duplicates"]
    _, rels = _inputs(golden, names)
    pairs = [(rels[2 * i], rels[2 * i + 1]) for i in range(len(names))]
    specs = _specs(golden, names, [dim3gpu.OP_PROJECT])
    b = dim3gpu.Batch(c, pairs, specs)
    t = b.autotune(max_trials=6)
    assert 1 <= t["trials"] <= 6 and t["ms"] <= t["ms_default"]
    assert c.get_param("cta_walk") == t["cta_walk"]
    _check(golden, specs, b.run())
    b.close()
    c.close()


@pytest.mark.slow
def test_batch512_smallest_queries_match_oracle(built):
    """The 24 smallest queries (by |R| + |S|) of the 512-query mixed batch the
    benchmark times, from the same seeded generator, run as one CUDA-graph
    batch: every query's count, set hash and sorted pairs equal the oracle's
    (its swap rule orients the pairs the same way)."""
    import torch

    import dim3gpu
    from oracle import oracle_py as O

    params = dim3gpu.batch_queries(nq=512)
    order = sorted(range(len(params)), key=lambda i: params[i]["nR"] + params[i]["nS"])[:24]
    rels = dim3gpu.batch_relations([params[i] for i in order])
    c = dim3gpu.Context(0)
    pairs = [((_dev(R), R.shape[0]), (_dev(S), S.shape[0])) for R, S in rels]
    sizer = dim3gpu.Batch(c, pairs, [{"op": 0, "capacity": 0} for _ in rels])
    need = [r["n_out"] for r in sizer.run(check=False)]
    sizer.close()
    outs = [torch.empty((max(n, 1), 2), dtype=torch.int32, device="cuda") for n in need]
    b = dim3gpu.Batch(c, pairs, [{"op": 0, "capacity": n, "out": o} for n, o in zip(need, outs)])
    res = b.run()
    torch.cuda.synchronize()
    for (R, S), r, o in zip(rels, res, outs):
        want, n, h, _ = O.join_project(R, S)
        assert r["status"] == 0 and r["n_out"] == n
        got = o[:n].cpu().numpy().view(np.uint32)
        assert O.set_hash(got) == h
        assert np.array_equal(O.sorted_pairs(got), O.sorted_pairs(want))
    b.close()
    c.close()
