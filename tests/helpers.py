"""Shared helpers for the parity tests: case inputs from the golden fixtures."""
import numpy as np

import dim3gpu
from oracle import oracle_py as O


def case_inputs(name, index, arrays):
    rec = index[name]
    if name + "/R" in arrays:
        return arrays[name + "/R"], arrays[name + "/S"]
    g = rec["gen"]
    if g == "gen_rand_data":
        return dim3gpu.gen_rand_data(*rec["args"], seed=492)
    return dim3gpu.workload(g, rec["scale"])


def input_hash(R, S):
    return O.set_hash(np.concatenate([R, S]).reshape(-1, 2)) ^ (R.shape[0] << 32) ^ S.shape[0]


def check_pairs(got, rec, arrays, name):
    """got: (n, 2) uint32 pairs.  Distinct, and equal to the golden set."""
    keys = np.sort(O.pair_keys(got))
    assert keys.shape[0] == rec["n_out"], (name, keys.shape[0], rec["n_out"])
    if keys.shape[0]:
        assert np.all(keys[1:] != keys[:-1]), name + ": duplicate pairs"
    assert str(O.set_hash(got)) == rec["set_hash"], name + ": set hash differs"
    if name + "/keys" in arrays:
        assert np.array_equal(keys, arrays[name + "/keys"]), name + ": pair sets differ"


def check_groups(pairs, counts, rec, arrays, name):
    k = O.pair_keys(pairs)
    order = np.argsort(k)
    assert k.shape[0] == rec["n_groups"], (name, k.shape[0], rec["n_groups"])
    assert str(O.group_hash(pairs, counts)) == rec["group_hash"], name + ": group hash differs"
    assert str(int(np.asarray(counts, dtype=np.uint64).sum(dtype=np.uint64))) == rec["count_sum"]
    if name + "/agg_keys" in arrays:
        assert np.array_equal(k[order], arrays[name + "/agg_keys"]), name + ": group keys differ"
        assert np.array_equal(np.asarray(counts, dtype=np.uint64)[order], arrays[name + "/agg_counts"]), \
            name + ": counts differ"
