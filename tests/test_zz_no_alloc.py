"""The allocation-free join-project entry point (dim3g_join_project_noalloc).

It exists for callers that must not allocate device memory at the point of
the join (custom or fixed-budget allocators, hosts that preallocate at
start-up).  It is checked here through the C ABI against the regular
device entry point on the same inputs, on two calls in a row: the second
call reuses the shared scratch array and must clear it correctly.  The
comparison is exact (integer pairs).  This file is collected last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import case_inputs, check_pairs

pytestmark = pytest.mark.gpu


def _noalloc(lib, dR, nR, dS, nS, dout, cap, stream):
    n = ctypes.c_uint64()
    vp = ctypes.c_void_p
    lib.dim3g_join_project_noalloc.argtypes = [vp, ctypes.c_uint64, vp, ctypes.c_uint64, vp, ctypes.c_uint64,
                                               ctypes.POINTER(ctypes.c_uint64), vp]
    rc = lib.dim3g_join_project_noalloc(vp(dR), nR, vp(dS), nS, vp(dout), cap, ctypes.byref(n), vp(stream))
    return rc, n.value


@pytest.mark.parametrize("name", ["grd_small", "grd_swap_dense", "grd_tiny", "chung_lu_s0005", "grd_classical",
                                  "extreme_keys", "heavy_duplicates"])
def test_noalloc_matches_device_entry_two_calls(built, golden, name):
    import torch

    import dim3gpu
    from oracle import oracle_py as O

    index, arrays = golden
    R, S = case_inputs(name, index, arrays)
    lib = dim3gpu.load()
    ctx = dim3gpu.Context(0)
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    n_ref = ctx.join_project_count_device(dR, R.shape[0], dS, S.shape[0])
    ref_out = torch.empty((max(n_ref, 1), 2), dtype=torch.int32, device="cuda")
    n_ref = ctx.join_project_device(dR, R.shape[0], dS, S.shape[0], ref_out, n_ref)
    torch.cuda.synchronize()
    want = np.sort(O.pair_keys(ref_out[:n_ref].cpu().numpy().view(np.uint32)))
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out = torch.full((max(n_ref, 1), 2), -1, dtype=torch.int32, device="cuda")
        rc, n = _noalloc(lib, dR.data_ptr(), R.shape[0], dS.data_ptr(), S.shape[0], out.data_ptr(), out.shape[0],
                         stream)
        assert rc == dim3gpu.OK, (name, call, rc)
        assert n == n_ref, (name, call, n, n_ref)
        got = out[:n].cpu().numpy().view(np.uint32)
        assert np.array_equal(np.sort(O.pair_keys(got)), want), (name, call)
        check_pairs(got, index[name], arrays, name)
    ctx.close()


def test_noalloc_rejects_inputs_beyond_its_scratch(built):
    import torch

    import dim3gpu

    lib = dim3gpu.load()
    big = (1 << 18) + 1  # DIM3G_NOALLOC_MAX_TUPLES + 1
    d = torch.zeros((big, 2), dtype=torch.int32, device="cuda")
    out = torch.empty((16, 2), dtype=torch.int32, device="cuda")
    rc, n = _noalloc(lib, d.data_ptr(), big, d.data_ptr(), 10, out.data_ptr(), 16, 0)
    assert rc == dim3gpu.ERR_UNSUPPORTED and n == 0


def test_noalloc_rejects_results_beyond_its_pair_limit(built, golden):
    """grd_swap has 1,375,660 distinct pairs, above DIM3G_NOALLOC_MAX_PAIRS."""
    import torch

    import dim3gpu

    index, arrays = golden
    R, S = case_inputs("grd_swap", index, arrays)
    assert index["grd_swap"]["n_out"] > (1 << 20)
    lib = dim3gpu.load()
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    out = torch.empty((1 << 20, 2), dtype=torch.int32, device="cuda")
    rc, n = _noalloc(lib, dR.data_ptr(), R.shape[0], dS.data_ptr(), S.shape[0], out.data_ptr(), 1 << 20, 0)
    assert rc == dim3gpu.ERR_UNSUPPORTED and n == 0


@pytest.mark.parametrize("na", [1024, 1025])
def test_noalloc_pair_limit_is_exact(built, na):
    """na x 1024 distinct pairs through one join value: exactly
    DIM3G_NOALLOC_MAX_PAIRS (2^20) is accepted in full, one row more is
    refused."""
    import torch

    import dim3gpu
    from oracle import oracle_py as O

    R = np.stack([np.arange(na, dtype=np.uint32), np.full(na, 5, np.uint32)], 1)
    S = np.stack([np.arange(1024, dtype=np.uint32) + 7, np.full(1024, 5, np.uint32)], 1)
    lib = dim3gpu.load()
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    cap = na * 1024
    out = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    rc, n = _noalloc(lib, dR.data_ptr(), na, dS.data_ptr(), 1024, out.data_ptr(), cap, 0)
    if na * 1024 <= (1 << 20):
        assert rc == dim3gpu.OK and n == na * 1024
        got = np.sort(O.pair_keys(out.cpu().numpy().view(np.uint32)))
        want = np.sort((np.repeat(np.arange(na, dtype=np.uint64), 1024) << np.uint64(32))
                       | np.tile(np.arange(1024, dtype=np.uint64) + np.uint64(7), na))
        assert np.array_equal(got, want)
    else:
        assert rc == dim3gpu.ERR_UNSUPPORTED and n == 0


def test_noalloc_empty_input_is_empty_whatever_the_other_size(built):
    """An empty relation joins to nothing, even beside one above the size
    limit (the same answer as dim3g_join_project_device)."""
    import torch

    import dim3gpu

    lib = dim3gpu.load()
    big = (1 << 18) + 1
    d = torch.zeros((big, 2), dtype=torch.int32, device="cuda")
    out = torch.empty((16, 2), dtype=torch.int32, device="cuda")
    rc, n = _noalloc(lib, d.data_ptr(), big, d.data_ptr(), 0, out.data_ptr(), 16, 0)
    assert rc == dim3gpu.OK and n == 0


def test_noalloc_reports_capacity(built, golden):
    import torch

    import dim3gpu

    index, arrays = golden
    R, S = case_inputs("grd_small", index, arrays)
    lib = dim3gpu.load()
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    out = torch.empty((100, 2), dtype=torch.int32, device="cuda")
    rc, n = _noalloc(lib, dR.data_ptr(), R.shape[0], dS.data_ptr(), S.shape[0], out.data_ptr(), 100, 0)
    assert rc == dim3gpu.ERR_CAPACITY and n == index["grd_small"]["n_out"]
