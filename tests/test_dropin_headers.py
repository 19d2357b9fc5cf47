"""The C++ drop-in headers (joinproject-dim3_gb300/dim3/): code written for
the reference's dim3.hpp / dim3_parallel.hpp / L+S_mapper.hpp compiles
against them unchanged and gets the reference's answers from the GPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "joinproject-dim3_gb300")
HDR = os.path.join(PKG, "dim3")
from oracle import oracle_py

REF = oracle_py.REF_SRC  # the reference sources, where present


def _compile(src, out, extra=()):
    cmd = ["g++", "-std=c++14", "-O2", "-I", HDR, src, "-o", out, "-L", PKG, "-ldim3gpu",
           "-Wl,-rpath," + PKG] + list(extra)
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def test_dropin_driver_compiles(built, tmp_path):
    _compile(os.path.join(HDR, "examples", "dropin_main.cpp"), str(tmp_path / "dropin_main"))


@pytest.mark.parametrize("prog", ["main.cpp", "main_parallel.cpp", "join_aggregate.cpp"])
def test_reference_drivers_compile_unchanged(built, tmp_path, prog):
    """The reference's own driver sources, untouched, build on the drop-in."""
    if not os.path.exists(os.path.join(REF, prog)):
        pytest.skip("reference sources not present on this machine")
    src = tmp_path / prog
    shutil.copy(os.path.join(REF, prog), src)  # alone, so "dim3.hpp" resolves to the drop-in
    _compile(str(src), str(tmp_path / "a.out"), ["-fopenmp"])


def test_reference_avg_driver_reports_unsupported(built, tmp_path):
    """join_aggregate.cpp asks for AVG(R.v + S.v), which has no GPU kernel:
    it builds, generates its valued tuples, and stops with the reference's
    print-and-exit behaviour and the unsupported status before any GPU work."""
    if not os.path.exists(os.path.join(REF, "join_aggregate.cpp")):
        pytest.skip("reference sources not present on this machine")
    src = tmp_path / "join_aggregate.cpp"
    shutil.copy(os.path.join(REF, "join_aggregate.cpp"), src)
    exe = _compile(str(src), str(tmp_path / "a.out"), ["-fopenmp"])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 255, r.stdout + r.stderr
    assert "only the COUNT aggregate" in r.stdout and "status 6" in r.stdout, r.stdout


def test_dropin_types_behave_like_the_reference(built, tmp_path):
    """myBitVector, S_DENSE, myvector::pop_back and the valued-tuple
    generator of the drop-in headers (host-only, no GPU)."""
    src = tmp_path / "types.cpp"
    src.write_text(r'''
#include "dim3.hpp"
int main() {
    myBitVector<> bv(4);
    bv.setTrue(0); bv.setTrue(37); bv.setTrue(127);
    int bits = 0;
    for (int i = 0; i < 128; i++) bits += bv.checkIfTrue(i);
    if (bits != 3 || !bv.checkIfTrue(37) || bv.checkIfTrue(36)) return 1;
    bv.clear(4);
    if (bv.checkIfTrue(37)) return 2;
    S_DENSE sd; sd.data = &bv; sd.size = 1; sd.dense_bitvector_len = 4; (void)sd;
    myvector<pair<int, int>> v;
    v.push_back({1, 2}); v.push_back({3, 4});
    pair<int, int> b = v.pop_back();
    if (b.first != 3 || v.size() != 1) return 3;
    v.pop_back();
    if (v.size() != 0 || v.pop_back() != pair<int, int>()) return 4;
    myvector<TUPLE<int, int, float>> R, S;
    gen_rand_data(R, S, 1000, 500, 50, 20, 60, 7);
    myvector<pair<int, int>> R2, S2;
    gen_rand_data(R2, S2, 1000, 500, 50, 20, 60, 7);
    if (R.size() != 1000 || S.size() != 500) return 5;
    for (int i = 0; i < 1000; i++)
        if (R.data[i].x != R2.data[i].first || R.data[i].y != R2.data[i].second || R.data[i].v != (float)i) return 6;
    for (int i = 0; i < 500; i++)
        if (S.data[i].x != S2.data[i].first || S.data[i].y != S2.data[i].second || S.data[i].v != (float)i) return 7;
    return 0;
}
''')
    exe = _compile(str(src), str(tmp_path / "types"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.returncode


def _run(exe, *args):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = dict(line.split("=", 1) for line in r.stdout.splitlines() if "=" in line)
    return int(out["|Result|"]), int(out["hash"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["grd_tiny", "grd_swap_dense", "grd_small", "grd_dense_z", "grd_swap"])
def test_dropin_join_project_and_count(built, golden, tmp_path, name):
    index, _ = golden
    rec = index[name]
    exe = _compile(os.path.join(HDR, "examples", "dropin_main.cpp"), str(tmp_path / "dropin_main"))
    for mode in ("project", "parallel"):
        n, h = _run(exe, mode, *rec["args"])
        assert n == rec["n_out"] and str(h) == rec["set_hash"], (mode, n, rec["n_out"])
    n, h = _run(exe, "count", *rec["args"])
    assert n == rec["n_groups"] and str(h) == rec["group_hash"]


@pytest.mark.gpu
def test_dropin_default_workload_known_answer(built, golden, tmp_path):
    """main.cpp's own workload: gen_rand_data() defaults, |Result| = 98,931,829."""
    rec = golden[0]["gen_rand_data_default"]
    exe = _compile(os.path.join(HDR, "examples", "dropin_main.cpp"), str(tmp_path / "dropin_main"))
    n, h = _run(exe, "project")
    assert n == 98931829 and str(h) == rec["set_hash"]


@pytest.mark.gpu
def test_dropin_ls_mapper(built, tmp_path):
    import dim3gpu
    exe = _compile(os.path.join(HDR, "examples", "dropin_main.cpp"), str(tmp_path / "dropin_main"))
    n, h = _run(exe, "mapper", 20000, 10, 500, 3000, 500)
    R, _ = dim3gpu.gen_rand_data(20000, 10, 500, 3000, 500, 492)
    ids, seen = [], {}
    for y in R[:, 1].tolist():
        seen.setdefault(y, len(seen))
        ids.append(seen[y])
    from oracle import oracle_py as O
    want = O.set_hash(np.stack([R[:, 1], np.array(ids, dtype=np.uint32)], 1))
    assert n == len(seen) and h == want
