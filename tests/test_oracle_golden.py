"""The C oracle against the reference's golden fixtures (CPU only)."""
import numpy as np
import pytest

from helpers import case_inputs, check_groups, check_pairs, input_hash
from oracle import oracle_py as O

SMALL = ["empty_R", "empty_S", "no_match", "single", "extreme_keys", "heavy_duplicates", "one_join_value",
         "grd_tiny", "grd_swap_dense", "grd_small", "grd_classical", "grd_dense_z", "grd_swap", "grd_sparse",
         "grd_all_dense", "zipf_1m_s001", "chung_lu_s0005", "chung_lu_s005"]


@pytest.mark.parametrize("name", SMALL)
def test_oracle_join_project_matches_reference(built, golden, name):
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    assert str(input_hash(R, S)) == index[name]["input_hash"], "generator output changed"
    pairs, n, h, st = O.join_project(R, S, threads=1)
    check_pairs(pairs, index[name], arrays, name)


@pytest.mark.parametrize("name", ["grd_small", "grd_dense_z", "grd_swap", "chung_lu_s005"])
def test_oracle_parallel_matches_reference(built, golden, name):
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    pairs, n, h, st = O.join_project(R, S, threads=4)
    check_pairs(pairs, index[name], arrays, name)
    _, n2, h2, _ = O.join_project(R, S, threads=4, hash_only=True)
    assert n2 == n and str(h2) == index[name]["set_hash"]


@pytest.mark.parametrize("name", SMALL)
def test_oracle_join_count_matches_reference(built, golden, name):
    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    pairs, cnt, n, h, st = O.join_count(R, S, threads=1)
    check_groups(pairs, cnt, index[name], arrays, name)


def test_oracle_known_answer_default_workload(built, golden):
    """The reference's default gen_rand_data workload: |Result| = 98,931,829."""
    index, _ = golden
    rec = index["gen_rand_data_default"]
    assert rec["n_out"] == 98931829
    import dim3gpu
    R, S = dim3gpu.gen_rand_data()
    assert str(input_hash(R, S)) == rec["input_hash"]
    _, n, h, _ = O.join_project(R, S, threads=8, hash_only=True)
    assert n == 98931829 and str(h) == rec["set_hash"]


def test_oracle_classical_equals_hybrid(built, golden):
    index, arrays = golden
    R, S = case_inputs("grd_small", index, arrays)
    pairs, h = O.classical(R, S)
    check_pairs(pairs, index["grd_small"], arrays, "grd_small")


def test_oracle_avg_aggregate_bit_exact_against_reference(built):
    ref = O.ref()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    import dim3gpu
    R, S = dim3gpu.gen_rand_data(20000, 15000, 500, 300, 700, 492)
    Rv = np.arange(R.shape[0], dtype=np.float32)
    Sv = np.arange(S.shape[0], dtype=np.float32)
    rp, ra = O.ref_join_avg(R, Rv, S, Sv)
    op, oa = O.join_avg(R, Rv, S, Sv)
    assert np.array_equal(rp, op)
    assert np.array_equal(ra.view(np.uint32), oa.view(np.uint32))


def test_oracle_restatement_matches_reference_order(built):
    """Ids, CSR order and emission order are restated exactly: the COUNT
    output equals the reference's element for element, not only as a set."""
    ref = O.ref()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    import dim3gpu
    R, S = dim3gpu.gen_rand_data(50000, 40000, 2000, 1500, 2500, 7)
    rp, rc = O.ref_join_count(R, S)
    op, oc, n, h, st = O.join_count(R, S)
    assert np.array_equal(rp, op) and np.array_equal(rc, oc)


def test_oracle_full_size_zipf_1m_matches_reference(built, golden):
    """Config 1 at full size (1M x 1M, 2.36e9 distinct pairs): the oracle's
    OpenMP form, hashing without storing pairs, against the reference's own
    count and set hash (fixture zipf_1m_full)."""
    import os

    import dim3gpu
    index, _ = golden
    rec = index["zipf_1m_full"]
    R, S = dim3gpu.workload("zipf_1m", 1.0)
    assert str(input_hash(R, S)) == rec["input_hash"]
    _, n, h, _ = O.join_project(R, S, threads=os.cpu_count() or 1, hash_only=True)
    assert n == rec["n_out"] == 2356052933 and str(h) == rec["set_hash"]
