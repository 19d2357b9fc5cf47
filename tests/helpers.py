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


_M64 = (1 << 64) - 1


def _signed64(v):
    return v - (1 << 64) if v >= 1 << 63 else v


def device_set_hash(out, n, chunk=1 << 27):
    """The order-independent set hash (sum of mix64(x << 32 | z), mod 2^64)
    of the first n pairs of a device (capacity, 2) int32 tensor, computed
    on the device in chunks (results of billions of pairs never come to the
    host).  int64 arithmetic wraps mod 2^64, which is the hash's own ring;
    right shifts are made logical by masking."""
    import torch

    m1, m2 = _signed64(0xbf58476d1ce4e5b9), _signed64(0x94d049bb133111eb)

    def lshr(v, s):
        return (v >> s) & ((1 << (64 - s)) - 1)

    total = 0
    for i in range(0, n, chunk):
        p = out[i:min(n, i + chunk)].to(torch.int64) & 0xFFFFFFFF
        k = (p[:, 0] << 32) | p[:, 1]
        del p
        k = (k ^ lshr(k, 30)) * m1
        k = (k ^ lshr(k, 27)) * m2
        k = k ^ lshr(k, 31)
        total = (total + int(k.sum().item())) & _M64
    return total


def exact_out_j(R, S):
    """OUT_J = sum over join values b of deg_R(b) * deg_S(b), exactly."""
    yr, cr = np.unique(np.asarray(R)[:, 1], return_counts=True)
    ys, cs = np.unique(np.asarray(S)[:, 1], return_counts=True)
    common, ir, is_ = np.intersect1d(yr, ys, assume_unique=True, return_indices=True)
    return int(np.sum(cr[ir].astype(np.uint64) * cs[is_].astype(np.uint64), dtype=np.uint64))


def tile_rows(R, tiles, t):
    """Rows of R whose first value lies in A-tile t (fmix32(a) & (tiles - 1))."""
    sel = (dim3gpu.fmix32_np(R[:, 0]) & np.uint64(tiles - 1)) == np.uint64(t)
    return np.ascontiguousarray(R[sel])
