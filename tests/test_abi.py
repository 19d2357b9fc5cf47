"""The C ABI library: it loads and exports every symbol include/dim3gpu.h
declares (no compute calls -- this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "dim3gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dim3g_\w+)\s*\(", src)))


def test_header_declares_the_expected_api():
    names = declared_functions()
    import dim3gpu
    assert sorted(dim3gpu.EXPORTS) == names


def test_library_exports_every_declared_symbol(built):
    import dim3gpu
    lib = ctypes.CDLL(dim3gpu.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_create_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import dim3gpu
    with pytest.raises(dim3gpu.Dim3GError):
        dim3gpu.Context(0)


def test_tuning_cache_roundtrip(built, tmp_path):
    """The autotuner's cache is host-only: save / load by key, last line of
    a key wins, absent keys and files report no entry."""
    import dim3gpu
    path = str(tmp_path / "tuning.txt")
    assert dim3gpu.tuning_load(path, "p24_z20_w3") is None
    a = {"tile_bits_log2": 18, "block_threads": 256, "block_slots_log2": 13, "warp_slots_log2": 10,
         "cta_walk": 1, "dense_block": 2, "dense_k_max": 512, "ms": 12.5, "ms_default": 14.0, "trials": 9}
    b = dict(a, tile_bits_log2=19, ms=11.0)
    dim3gpu.tuning_save(path, "p24_z20_w3", a)
    dim3gpu.tuning_save(path, "p20_z16_w5", dict(a, warp_slots_log2=9))
    dim3gpu.tuning_save(path, "p24_z20_w3", b)
    got = dim3gpu.tuning_load(path, "p24_z20_w3")
    assert got["tile_bits_log2"] == 19 and abs(got["ms"] - 11.0) < 1e-3 and got["trials"] == 9
    assert got["dense_block"] == 2 and got["dense_k_max"] == 512
    assert dim3gpu.tuning_load(path, "p20_z16_w5")["warp_slots_log2"] == 9
    assert dim3gpu.tuning_load(path, "nope") is None
    with pytest.raises(dim3gpu.Dim3GError):
        dim3gpu.tuning_save(path, "has space", a)


@pytest.mark.parametrize("cname,pyname", [("dim3g_stats", "Stats"), ("dim3g_tuning", "Tuning"),
                                          ("dim3g_calibration", "Calibration")])
def test_struct_mirrors_match_header(tmp_path, cname, pyname):
    """The ctypes mirror of a header struct has its size and field offsets
    (a C probe compiled against include/dim3gpu.h)."""
    import shutil
    import subprocess
    import ctypes
    import dim3gpu
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    py = getattr(dim3gpu, pyname)
    fields = [f for f, _ in py._fields_]
    src = tmp_path / "probe.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"dim3gpu.h\"\nint main(void){\n"
                   "printf(\"%%zu\\n\", sizeof(%s));\n" % cname
                   + "".join("printf(\"%%zu\\n\", offsetof(%s, %s));\n" % (cname, f) for f in fields)
                   + "return 0;}\n")
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-I", os.path.join(root, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert got[0] == ctypes.sizeof(py)
    assert got[1:] == [getattr(py, f).offset for f in fields]


def test_noalloc_rejects_misaligned_pointers_before_any_gpu_work(built):
    """The allocation-free entry point reads and writes pairs as 8-byte
    words: a pointer off that alignment is refused with DIM3G_ERR_INVALID
    before any CUDA call (this runs without a GPU, so a call that reached
    the runtime would report DIM3G_ERR_CUDA instead)."""
    import dim3gpu
    lib = ctypes.CDLL(dim3gpu.LIB_PATH)
    vp, u64 = ctypes.c_void_p, ctypes.c_uint64
    fn = lib.dim3g_join_project_noalloc
    fn.argtypes = [vp, u64, vp, u64, vp, u64, ctypes.POINTER(u64), vp]
    n = u64(7)
    good, off = 0x10000, 0x10004  # never dereferenced: the check comes first
    for r, s, o in ((off, good, good), (good, off, good), (good, good, off)):
        n.value = 7
        assert fn(vp(r), 10, vp(s), 10, vp(o), 100, ctypes.byref(n), None) == dim3gpu.ERR_INVALID
        assert n.value == 0
