"""GPU tests of the serving loop (dim3g_server_*): requests submitted
concurrently from several threads give, each, exactly the result the same
join gives alone (a one-query pass over the set, itself checked against the
oracle on the same relations), under a budget that forces admission to
wait; the pair matrix is exact."""
import threading

import numpy as np
import pytest

from helpers import case_inputs

pytestmark = pytest.mark.gpu

NAMES = ["grd_tiny", "grd_small", "grd_swap_dense", "heavy_duplicates", "one_join_value", "zipf_1m_s001",
         "chung_lu_s0005", "grd_classical", "empty_S"]


def _set(ctx, golden):
    import torch
    import dim3gpu
    index, arrays = golden
    host, rels = [], []
    for name in NAMES:
        R, S = case_inputs(name, index, arrays)
        host += [R, S]
        for a in (R, S):
            rels.append((torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda() if a.shape[0] else 0,
                         a.shape[0]))
    return host, dim3gpu.RelSet(ctx, rels)


def _alone(rs, r, s, op):
    """The same join as a one-query pass: (pairs, counts or None)."""
    import torch
    import dim3gpu
    res = rs.join([{"r": r, "s": s, "op": op, "capacity": 0}], check=False)[0]
    n = res["n_out"]
    out = torch.empty((max(n, 1), 2), dtype=torch.int32, device="cuda")
    cnt = torch.empty((max(n, 1),), dtype=torch.int64, device="cuda") if op == dim3gpu.OP_COUNT else None
    res = rs.join([{"r": r, "s": s, "op": op, "capacity": n, "out": out, "cnt": cnt}])[0]
    torch.cuda.synchronize()
    p = out[:n].cpu().numpy().view(np.uint32)
    c = cnt[:n].cpu().numpy().view(np.uint64) if cnt is not None else None
    return p, c


def _canon(p, c):
    from oracle import oracle_py as O
    k = O.pair_keys(p)
    o = np.argsort(k)
    return k[o], (None if c is None else c[o])


def test_pair_matrix_is_exact(ctx, golden):
    import dim3gpu
    host, rs = _set(ctx, golden)
    m = rs.pair_outj()
    n = len(host)
    specs = [{"r": r, "s": s, "op": dim3gpu.OP_PROJECT, "capacity": 0} for r in range(n) for s in range(n)]
    res = rs.join(specs, check=False)
    got = np.array([x["out_j"] for x in res], dtype=np.uint64).reshape(n, n)
    assert np.array_equal(got, m)
    # and against the definition on the host for a few pairs
    for r, s in [(0, 1), (2, 3), (10, 11), (4, 9)]:
        R, S = host[r], host[s]
        yr, cr = np.unique(R[:, 1], return_counts=True)
        ys, cs = np.unique(S[:, 1], return_counts=True)
        common, ir, is_ = np.intersect1d(yr, ys, return_indices=True)
        assert int(m[r, s]) == int((cr[ir].astype(np.uint64) * cs[is_].astype(np.uint64)).sum())
    rs.close()


@pytest.mark.parametrize("lanes,budget_mb", [(2, 4096), (3, 0)])
def test_served_results_equal_alone(ctx, golden, lanes, budget_mb):
    """Many concurrent requests (every case's own join, its COUNT, and
    cross joins) through the server; each equals its one-query result, and
    the cases' own joins equal the golden fixtures.  budget_mb = 0: a budget
    just above the set and scratch, so admission has to wait for releases."""
    import dim3gpu
    index, arrays = golden
    host, rs = _set(ctx, golden)
    n = len(host)
    reqs = []
    for i in range(len(NAMES)):
        reqs.append((2 * i, 2 * i + 1, dim3gpu.OP_PROJECT))
        reqs.append((2 * i, 2 * i + 1, dim3gpu.OP_COUNT))
    rng = np.random.default_rng(5)
    for _ in range(24):
        r, s = rng.integers(0, n, size=2)
        reqs.append((int(r), int(s), int(rng.integers(0, 2))))
    want = {}
    for r, s, op in set(reqs):
        want[(r, s, op)] = _canon(*_alone(rs, r, s, op))
    # the one-query passes the served results are held to are themselves
    # checked against the oracle on the same relations (its swap rule
    # orients the pairs as the set's does)
    from oracle import oracle_py as O
    for (r, s, op), (wk, wc) in want.items():
        if op == dim3gpu.OP_PROJECT:
            wp, _, _, _ = O.join_project(host[r], host[s])
            assert np.array_equal(wk, np.sort(O.pair_keys(wp))), (r, s, op)
        else:
            wg, wcnt, _, _, _ = O.join_count(host[r], host[s])
            k = O.pair_keys(wg)
            o = np.argsort(k)
            assert np.array_equal(wk, k[o]), (r, s, op)
            assert np.array_equal(wc, np.asarray(wcnt, dtype=np.uint64)[o]), (r, s, op)
    m = rs.pair_outj()
    largest = max(((int(m[r, s]) * 8 + 255) // 256) * 256 * 2 for r, s, _ in reqs)  # a COUNT reservation bound
    if budget_mb == 0:
        probe = dim3gpu.Server(rs, lanes=lanes, max_batch=8, budget_bytes=1 << 45)
        fixed = (1 << 45) - probe.stats()["output_budget"]
        probe.close()
        budget = fixed + 2 * largest
    else:
        probe = dim3gpu.Server(rs, lanes=lanes, max_batch=8, budget_bytes=1 << 45)
        budget = (budget_mb << 20) + (1 << 45) - probe.stats()["output_budget"]
        probe.close()
    srv = dim3gpu.Server(rs, lanes=lanes, max_batch=8, budget_bytes=budget)
    errors = []
    results = {}

    def client(sub):
        try:
            for r, s, op in sub:
                t = srv.submit(r, s, op)
                res = srv.wait(t)
                assert res["status"] == 0, res
                p = dim3gpu.device_pairs(res["d_out"], res["n_out"])
                c = dim3gpu.device_u64(res["d_cnt"], res["n_out"]) if op == dim3gpu.OP_COUNT else None
                results.setdefault((r, s, op), []).append(_canon(p, c))
                srv.release(t)
        except Exception as e:  # surfaced below
            errors.append(e)

    threads = [threading.Thread(target=client, args=(reqs[k::4],)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["reserved_bytes"] == 0
    for key, got in results.items():
        wk, wc = want[key]
        for gk, gc in got:
            assert np.array_equal(gk, wk), key
            if wc is not None:
                assert np.array_equal(gc, wc), key
    for i, name in enumerate(NAMES):
        k, _ = want[(2 * i, 2 * i + 1, dim3gpu.OP_PROJECT)]
        assert k.shape[0] == index[name]["n_out"], name
    srv.close()
    rs.close()


def test_server_admission_limits_and_shutdown(ctx, golden):
    """A budget that holds one result of (0, 1) at a time: a second request
    waits for the first's release; a request larger than the whole output
    budget is refused at submit; shutdown with unreleased and queued work
    returns."""
    import dim3gpu
    host, rs = _set(ctx, golden)
    m = rs.pair_outj()
    one = ((int(m[0, 1]) * 8 + 255) // 256) * 256
    probe = dim3gpu.Server(rs, lanes=2, max_batch=4, budget_bytes=1 << 45)
    fixed = (1 << 45) - probe.stats()["output_budget"]
    probe.close()
    srv = dim3gpu.Server(rs, lanes=2, max_batch=4, budget_bytes=fixed + one + 4096)
    assert int(m[10, 11]) * 8 > one + 4096
    with pytest.raises(dim3gpu.Dim3GError) as e:
        srv.submit(10, 11, dim3gpu.OP_PROJECT)
    assert e.value.code == dim3gpu.ERR_NOMEM
    t1 = srv.submit(0, 1)
    r1 = srv.wait(t1)
    assert r1["status"] == 0
    t2 = srv.submit(0, 1)  # admitted only once t1's output is released
    srv.release(t1)
    r2 = srv.wait(t2)
    assert r2["status"] == 0 and r2["n_out"] == r1["n_out"] and r2["t_start"] >= r1["t_done"]
    srv.release(t2)
    # shutdown with an unreleased result and a request queued behind it
    t3 = srv.submit(0, 1)
    srv.wait(t3)
    srv.submit(0, 1)
    srv.close()
    rs.close()
