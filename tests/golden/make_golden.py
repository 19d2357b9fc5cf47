"""Generate the golden fixtures in this directory by running the reference.

The reference (schencoding/JoinProject-DIM3, header-only C++) is compiled
from its own sources into oracle/_ref/ by oracle/Makefile.ref and driven
through oracle/ref_driver.cpp.  This needs the reference sources and an
x86 host with AVX; the fixtures it writes are committed, so tests run
anywhere.

    python tests/golden/make_golden.py            # small cases (seconds)
    python tests/golden/make_golden.py --large    # + full-size zipf_1m (~1 min, ~25 GB RAM)

Each case records, from the reference:
  - join-project: |Result|, the order-independent set hash, and for small
    outputs the sorted (x<<32|z) keys;
  - join-aggregate COUNT: number of groups, group hash, and for small outputs
    the sorted keys with their counts.
Inputs are stored verbatim for small cases; larger ones are regenerated by
the package's seeded generators, whose output hash is recorded too.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "joinproject-dim3_gb300"))

from oracle import oracle_py as O  # noqa: E402

import dim3gpu  # noqa: E402  (generators only)

STORE_INPUT_MAX = 20000
STORE_OUTPUT_MAX = 200000


def input_hash(R, S):
    return O.set_hash(np.concatenate([R, S]).reshape(-1, 2)) ^ (R.shape[0] << 32) ^ S.shape[0]


def edge_cases():
    u = np.uint32
    cases = {}
    cases["empty_R"] = (np.zeros((0, 2), u), np.array([[1, 2], [3, 4]], u))
    cases["empty_S"] = (np.array([[1, 2], [3, 4]], u), np.zeros((0, 2), u))
    cases["no_match"] = (np.array([[1, 2], [3, 4], [5, 6]], u), np.array([[1, 7], [3, 8]], u))
    cases["single"] = (np.array([[10, 20]], u), np.array([[30, 20]], u))
    cases["extreme_keys"] = (np.array([[0xFFFFFFFF, 0xFFFFFFFF], [0, 0xFFFFFFFF], [0xFFFFFFFF, 0], [7, 0]], u),
                             np.array([[0xFFFFFFFF, 0xFFFFFFFF], [0, 0], [5, 0xFFFFFFFF], [0xFFFFFFFF, 0]], u))
    rng = np.random.default_rng(5)
    d = rng.integers(0, 4, size=(3000, 2)).astype(u)
    cases["heavy_duplicates"] = (d, d[::-1].copy())
    one_y = np.stack([np.arange(1500, dtype=u), np.full(1500, 9, u)], 1)
    cases["one_join_value"] = (one_y, one_y[:700].copy())
    return cases


def generated_cases():
    c = {}
    for name, args in {
        "grd_tiny": (1000, 1000, 100, 100, 100),
        "grd_swap_dense": (1000, 2000, 50, 20, 50),
        "grd_small": (5000, 3000, 300, 200, 400),
        "grd_classical": (20000, 20000, 10 ** 6, 10 ** 6, 10 ** 6),
        "grd_dense_z": (200000, 100000, 1000, 300, 5000),
        "grd_swap": (100000, 200000, 5000, 5000, 300),
        "grd_sparse": (500000, 500000, 100000, 20000, 100000),
        "grd_all_dense": (300000, 300000, 3000, 100, 3000),
    }.items():
        R, S = dim3gpu.gen_rand_data(*args, seed=492)
        c[name] = (R, S, {"gen": "gen_rand_data", "args": list(args)})
    for name, scale in {"zipf_1m_s001": 0.01, "zipf_1m_s01": 0.1}.items():
        R, S = dim3gpu.workload("zipf_1m", scale)
        c[name] = (R, S, {"gen": "zipf_1m", "scale": scale})
    for name, scale in {"chung_lu_s0005": 0.0005, "chung_lu_s005": 0.005}.items():
        R, S = dim3gpu.workload("chung_lu_20m", scale)
        c[name] = (R, S, {"gen": "chung_lu_20m", "scale": scale})
    return c


def record(R, S, meta, with_agg=True):
    ref = O.ref_join_project(R, S)
    keys = np.sort(O.pair_keys(ref))
    assert np.unique(keys).shape[0] == keys.shape[0], "reference output not distinct"
    rec = dict(meta)
    rec["nR"] = int(R.shape[0])
    rec["nS"] = int(S.shape[0])
    rec["input_hash"] = str(input_hash(R, S))
    rec["n_out"] = int(keys.shape[0])
    rec["set_hash"] = str(O.set_hash(ref))
    arrays = {}
    if keys.shape[0] <= STORE_OUTPUT_MAX:
        arrays["keys"] = keys
    if with_agg:
        gp, gc = O.ref_join_count(R, S)
        gk = O.pair_keys(gp)
        order = np.argsort(gk)
        rec["n_groups"] = int(gk.shape[0])
        rec["group_hash"] = str(O.group_hash(gp, gc))
        rec["count_sum"] = str(int(gc.sum(dtype=np.uint64)))
        if gk.shape[0] <= STORE_OUTPUT_MAX:
            arrays["agg_keys"] = gk[order]
            arrays["agg_counts"] = gc[order]
    if R.shape[0] <= STORE_INPUT_MAX and S.shape[0] <= STORE_INPUT_MAX:
        arrays["R"] = R
        arrays["S"] = S
    return rec, arrays


def main():
    if O.ref() is None:
        raise SystemExit("the reference could not be built here (needs its sources and an x86 host)")
    index = {}
    arrays = {}
    # The reference's join-aggregate dereferences an uninitialised domain size
    # when the semi-join leaves no tuple (dim3.hpp:1342-1350) and faults; for
    # those inputs the aggregate answer is the empty set by definition.
    agg_faults = {"empty_R", "empty_S", "no_match"}
    for name, (R, S) in edge_cases().items():
        rec, arr = record(R, S, {"gen": "inline"}, with_agg=name not in agg_faults)
        if name in agg_faults:
            rec.update(n_groups=0, group_hash="0", count_sum="0",
                       note="reference join-aggregate faults on an empty semi-join; empty by definition")
            arr["agg_keys"] = np.zeros(0, np.uint64)
            arr["agg_counts"] = np.zeros(0, np.uint64)
        index[name] = rec
        for k, v in arr.items():
            arrays[name + "/" + k] = v
    for name, (R, S, meta) in generated_cases().items():
        rec, arr = record(R, S, meta)
        index[name] = rec
        for k, v in arr.items():
            arrays[name + "/" + k] = v
        print(name, rec["n_out"], rec.get("n_groups"))
    # The reference's own default workload: gen_rand_data() with its default
    # arguments (1e7 x 1e7 tuples, domains 1e6, seed 492).
    R, S = dim3gpu.gen_rand_data()
    ref = O.ref_join_project(R, S)
    index["gen_rand_data_default"] = {"gen": "gen_rand_data", "args": [10 ** 7, 10 ** 7, 10 ** 6, 10 ** 6, 10 ** 6],
                                      "nR": 10 ** 7, "nS": 10 ** 7, "input_hash": str(input_hash(R, S)),
                                      "n_out": int(ref.shape[0]), "set_hash": str(O.set_hash(ref))}
    print("default", ref.shape[0])
    del ref
    if "--large" in sys.argv:
        # 2.35e9 pairs (18.8 GB): hashed in chunks from the reference's own
        # buffer; its uint32 result counter still holds the count
        R, S = dim3gpu.workload("zipf_1m", 1.0)
        n, h = O.ref_join_project_hash(R, S)
        index["zipf_1m_full"] = {"gen": "zipf_1m", "scale": 1.0, "nR": int(R.shape[0]), "nS": int(S.shape[0]),
                                 "input_hash": str(input_hash(R, S)), "n_out": n, "set_hash": str(h)}
        print("zipf_1m full", n)
    else:
        old = os.path.join(HERE, "golden_index.json")
        if os.path.exists(old):
            prev = json.load(open(old))
            if "zipf_1m_full" in prev:
                index["zipf_1m_full"] = prev["zipf_1m_full"]
    np.savez_compressed(os.path.join(HERE, "golden_arrays.npz"), **arrays)
    with open(os.path.join(HERE, "golden_index.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
