"""ctypes bindings for the CPU oracle (test infrastructure only).

Loads ``oracle/libdim3oracle.so`` (the C restatement of the reference, built
by ``oracle.build``) and, where it exists, ``oracle/_ref/libdim3ref.so`` (the
unmodified reference compiled from its own sources; x86 validation only).

Only tests, the smoke check and the CPU-baseline leg of the benchmark import
this module; the product path never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libdim3oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdim3ref.so")
# The reference sources (present only where the fixtures are made);
# DIM3_REFERENCE_SRC overrides the default location.
REF_SRC = os.environ.get("DIM3_REFERENCE_SRC", "/root/reference")

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)


class Stats(ctypes.Structure):
    _fields_ = [
        ("used_classical", ctypes.c_int32),
        ("swapped", ctypes.c_int32),
        ("nx", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("nz", ctypes.c_int32),
        ("n_dense_z", ctypes.c_int32),
        ("out_j_hat", ctypes.c_int64),
        ("out_j", ctypes.c_uint64),
        ("t_estimate", ctypes.c_double),
        ("t_mapping", ctypes.c_double),
        ("t_divide", ctypes.c_double),
        ("t_expand", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build(force=False):
    """Compile the C oracle (gcc, OpenMP, no FP contraction so x86 and Arm agree)."""
    src = os.path.join(HERE, "dim3_oracle.c")
    if not force and os.path.exists(ORACLE_SO) and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src):
        return ORACLE_SO
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           src, "-o", ORACLE_SO, "-lm"]
    subprocess.check_call(cmd)
    return ORACLE_SO


def build_ref():
    """Compile the unmodified reference into oracle/_ref (only where its
    sources are present and the host has AVX, i.e. the x86 dev container)."""
    if not os.path.isdir(REF_SRC):
        return None
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        return None
    repo = os.path.dirname(HERE)
    subprocess.check_call(["make", "-s", "-f", os.path.join("oracle", "Makefile.ref"), "REF=" + REF_SRC], cwd=repo)
    return REF_SO


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(ORACLE_SO)
        L.dim3o_join_project.argtypes = [_u32p, ctypes.c_uint64, _u32p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(_u32p), _u64p, _u64p, ctypes.POINTER(Stats)]
        L.dim3o_join_count.argtypes = [_u32p, ctypes.c_uint64, _u32p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(_u32p), ctypes.POINTER(_u64p), _u64p, _u64p,
                                       ctypes.POINTER(Stats)]
        L.dim3o_join_avg.argtypes = [_u32p, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64,
                                     _u32p, ctypes.POINTER(ctypes.c_float), ctypes.c_uint64,
                                     ctypes.POINTER(_u32p), ctypes.POINTER(ctypes.POINTER(ctypes.c_float)), _u64p,
                                     ctypes.POINTER(Stats)]
        L.dim3o_classical.argtypes = [_u32p, ctypes.c_uint64, _u32p, ctypes.c_uint64,
                                      ctypes.POINTER(_u32p), _u64p, _u64p]
        L.dim3o_estimate.argtypes = [_u32p, ctypes.c_uint64, _u32p, ctypes.c_uint64]
        L.dim3o_estimate.restype = ctypes.c_int64
        L.dim3o_pair_hash.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.dim3o_pair_hash.restype = ctypes.c_uint64
        L.dim3o_free.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def ref():
    """The reference compiled from its sources, or None where unavailable."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            try:
                build_ref()
            except Exception:
                return None
        if not os.path.exists(REF_SO):
            return None
        L = ctypes.CDLL(REF_SO)
        ip = ctypes.POINTER(ctypes.c_int)
        L.ref_gen_rand_data.argtypes = [ctypes.c_int] * 6 + [ip, ip]
        L.ref_join_project.argtypes = [ip, ctypes.c_uint, ip, ctypes.c_uint, ctypes.c_int, ctypes.POINTER(ip)]
        L.ref_join_project.restype = ctypes.c_uint
        L.ref_classical.argtypes = [ip, ctypes.c_uint, ip, ctypes.c_uint, ctypes.POINTER(ip)]
        L.ref_classical.restype = ctypes.c_uint
        L.ref_estimate.argtypes = [ip, ctypes.c_uint, ip, ctypes.c_uint]
        L.ref_estimate.restype = ctypes.c_longlong
        L.ref_join_count.argtypes = [ip, ctypes.c_uint, ip, ctypes.c_uint, ctypes.POINTER(ip),
                                     ctypes.POINTER(ctypes.POINTER(ctypes.c_longlong))]
        L.ref_join_count.restype = ctypes.c_uint
        fp = ctypes.POINTER(ctypes.c_float)
        L.ref_join_avg.argtypes = [ip, fp, ctypes.c_uint, ip, fp, ctypes.c_uint, ctypes.POINTER(ip),
                                   ctypes.POINTER(fp)]
        L.ref_join_avg.restype = ctypes.c_uint
        L.ref_free.argtypes = [ctypes.c_void_p]
        _ref = L
    return _ref


def _pairs(a):
    a = np.ascontiguousarray(a, dtype=np.uint32).reshape(-1, 2)
    return a, a.ctypes.data_as(_u32p), a.shape[0]


def _take_pairs(L, p, n):
    if n == 0 or not p:
        if p:
            L.dim3o_free(ctypes.cast(p, ctypes.c_void_p))
        return np.zeros((0, 2), dtype=np.uint32)
    out = np.ctypeslib.as_array(p, shape=(n * 2,)).copy().reshape(-1, 2)
    L.dim3o_free(ctypes.cast(p, ctypes.c_void_p))
    return out


def join_project(R, S, threads=1, hash_only=False):
    """Oracle join-project.  Returns (pairs or None, count, set_hash, stats)."""
    L = lib()
    R, rp, nr = _pairs(R)
    S, sp, ns = _pairs(S)
    out = _u32p()
    n = ctypes.c_uint64()
    h = ctypes.c_uint64()
    st = Stats()
    rc = L.dim3o_join_project(rp, nr, sp, ns, threads, int(hash_only), ctypes.byref(out), ctypes.byref(n),
                              ctypes.byref(h), ctypes.byref(st))
    if rc != 0:
        raise MemoryError("oracle join_project failed")
    pairs = None if hash_only else _take_pairs(L, out, n.value)
    return pairs, n.value, h.value, st.as_dict()


def join_count(R, S, threads=1, hash_only=False):
    """Oracle COUNT(*) join-aggregate.  Returns (pairs, counts, n, hash, stats)."""
    L = lib()
    R, rp, nr = _pairs(R)
    S, sp, ns = _pairs(S)
    oxz = _u32p()
    oc = _u64p()
    n = ctypes.c_uint64()
    h = ctypes.c_uint64()
    st = Stats()
    rc = L.dim3o_join_count(rp, nr, sp, ns, threads, int(hash_only), ctypes.byref(oxz), ctypes.byref(oc),
                            ctypes.byref(n), ctypes.byref(h), ctypes.byref(st))
    if rc != 0:
        raise MemoryError("oracle join_count failed")
    if hash_only:
        return None, None, n.value, h.value, st.as_dict()
    pairs = _take_pairs(L, oxz, n.value)
    if n.value:
        cnt = np.ctypeslib.as_array(oc, shape=(n.value,)).copy()
    else:
        cnt = np.zeros(0, dtype=np.uint64)
    if oc:
        L.dim3o_free(ctypes.cast(oc, ctypes.c_void_p))
    return pairs, cnt, n.value, h.value, st.as_dict()


def join_avg(R, Rv, S, Sv):
    L = lib()
    R, rp, nr = _pairs(R)
    S, sp, ns = _pairs(S)
    Rv = np.ascontiguousarray(Rv, dtype=np.float32)
    Sv = np.ascontiguousarray(Sv, dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    oxz = _u32p()
    oa = fp()
    n = ctypes.c_uint64()
    st = Stats()
    rc = L.dim3o_join_avg(rp, Rv.ctypes.data_as(fp), nr, sp, Sv.ctypes.data_as(fp), ns, ctypes.byref(oxz),
                          ctypes.byref(oa), ctypes.byref(n), ctypes.byref(st))
    if rc != 0:
        raise MemoryError("oracle join_avg failed")
    pairs = _take_pairs(L, oxz, n.value)
    avg = np.ctypeslib.as_array(oa, shape=(n.value,)).copy() if n.value else np.zeros(0, np.float32)
    if oa:
        L.dim3o_free(ctypes.cast(oa, ctypes.c_void_p))
    return pairs, avg


def classical(R, S):
    L = lib()
    R, rp, nr = _pairs(R)
    S, sp, ns = _pairs(S)
    out = _u32p()
    n = ctypes.c_uint64()
    h = ctypes.c_uint64()
    if L.dim3o_classical(rp, nr, sp, ns, ctypes.byref(out), ctypes.byref(n), ctypes.byref(h)) != 0:
        raise MemoryError("oracle classical failed")
    return _take_pairs(L, out, n.value), h.value


def estimate(R, S):
    L = lib()
    R, rp, nr = _pairs(R)
    S, sp, ns = _pairs(S)
    return L.dim3o_estimate(rp, nr, sp, ns)


# ---------------------------------------------------------------- hashing
def pair_keys(pairs):
    p = np.asarray(pairs, dtype=np.uint32).reshape(-1, 2)
    return (p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64)


def mix64(v):
    v = np.asarray(v, dtype=np.uint64)
    with np.errstate(over="ignore"):
        v = (v ^ (v >> np.uint64(30))) * np.uint64(0xbf58476d1ce4e5b9)
        v = (v ^ (v >> np.uint64(27))) * np.uint64(0x94d049bb133111eb)
        v = v ^ (v >> np.uint64(31))
    return v


def set_hash(pairs):
    """Order-independent hash of a set of (x, z) pairs (sum of mix64)."""
    with np.errstate(over="ignore"):
        return int(np.sum(mix64(pair_keys(pairs)), dtype=np.uint64))


def group_hash(pairs, counts):
    with np.errstate(over="ignore"):
        g = mix64(mix64(pair_keys(pairs)) + np.asarray(counts, dtype=np.uint64))
        return int(np.sum(g, dtype=np.uint64))


def fmix32(v):
    """murmur3 fmix32 (the A-tile function of the summaries)."""
    v = np.asarray(v, dtype=np.uint32).astype(np.uint64)
    with np.errstate(over="ignore"):
        v ^= v >> np.uint64(16)
        v = (v * np.uint64(0x85ebca6b)) & np.uint64(0xFFFFFFFF)
        v ^= v >> np.uint64(13)
        v = (v * np.uint64(0xc2b2ae35)) & np.uint64(0xFFFFFFFF)
        v ^= v >> np.uint64(16)
    return v


def tile_summary(pairs, counts, tiles, lo=0, hi=None):
    """Per-A-tile (groups, count sum, hash) of a result, tile = fmix32(first
    value) & (tiles - 1): the definition dim3g_join_*_summary computes, for
    tiles [lo, hi) (others zero).  counts None: join-project (count sum =
    groups, hash = pair hash)."""
    hi = tiles if hi is None else hi
    p = np.asarray(pairs, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros((tiles, 3), dtype=np.uint64)
    step = 1 << 24
    with np.errstate(over="ignore"):
        for i0 in range(0, p.shape[0], step):  # bounded temporaries
            q = p[i0:i0 + step]
            t = (fmix32(q[:, 0]) & np.uint64(tiles - 1)).astype(np.int64)
            if counts is None:
                h = mix64(pair_keys(q))
                c = np.ones(q.shape[0], dtype=np.uint64)
            else:
                c = np.asarray(counts[i0:i0 + step], dtype=np.uint64)
                h = mix64(mix64(pair_keys(q)) + c)
            if hi - lo == tiles and tiles > 1:
                order = np.argsort(t, kind="stable")
                ts, cs, hs = t[order], c[order], h[order]
                bounds = np.searchsorted(ts, np.arange(tiles + 1))
                for k in range(tiles):
                    a, b = bounds[k], bounds[k + 1]
                    out[k, 0] += np.uint64(b - a)
                    out[k, 1] += np.sum(cs[a:b], dtype=np.uint64)
                    out[k, 2] += np.sum(hs[a:b], dtype=np.uint64)
            else:
                for k in range(lo, hi):
                    sel = t == k
                    out[k, 0] += np.uint64(np.count_nonzero(sel))
                    out[k, 1] += np.sum(c[sel], dtype=np.uint64)
                    out[k, 2] += np.sum(h[sel], dtype=np.uint64)
    return out


def sorted_pairs(pairs):
    k = np.sort(pair_keys(pairs))
    return k


# ---------------------------------------------------------------- reference
def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def ref_gen_rand_data(nR, nS, modx, mody, modz, seed=492):
    L = ref()
    R = np.zeros((nR, 2), dtype=np.int32)
    S = np.zeros((nS, 2), dtype=np.int32)
    L.ref_gen_rand_data(nR, nS, modx, mody, modz, seed, _ip(R), _ip(S))
    return R.view(np.uint32), S.view(np.uint32)


def _ref_take(L, p, n, width):
    if n == 0:
        if p:
            L.ref_free(ctypes.cast(p, ctypes.c_void_p))
        return np.zeros((0, width), dtype=np.uint32)
    a = np.ctypeslib.as_array(p, shape=(n * width,)).copy().view(np.uint32).reshape(-1, width)
    L.ref_free(ctypes.cast(p, ctypes.c_void_p))
    return a


def ref_join_project(R, S, parallel=False):
    L = ref()
    R = np.ascontiguousarray(R, dtype=np.uint32).view(np.int32)
    S = np.ascontiguousarray(S, dtype=np.uint32).view(np.int32)
    out = ctypes.POINTER(ctypes.c_int)()
    n = L.ref_join_project(_ip(R), R.shape[0], _ip(S), S.shape[0], int(parallel), ctypes.byref(out))
    return _ref_take(L, out, n, 2)


def ref_join_project_hash(R, S, chunk=1 << 26):
    """The reference's join-project reduced to (|Result|, set hash), hashed in
    chunks straight from its own result buffer (no copy), so results of
    billions of pairs fit in host memory."""
    L = ref()
    R = np.ascontiguousarray(R, dtype=np.uint32).view(np.int32)
    S = np.ascontiguousarray(S, dtype=np.uint32).view(np.int32)
    out = ctypes.POINTER(ctypes.c_int)()
    n = L.ref_join_project(_ip(R), R.shape[0], _ip(S), S.shape[0], 0, ctypes.byref(out))
    h = 0
    if n:
        a = np.ctypeslib.as_array(out, shape=(n * 2,)).view(np.uint32).reshape(-1, 2)
        for i in range(0, n, chunk):
            h = (h + set_hash(a[i:i + chunk])) & 0xFFFFFFFFFFFFFFFF
    if out:
        L.ref_free(ctypes.cast(out, ctypes.c_void_p))
    return int(n), h


def ref_classical(R, S):
    L = ref()
    R = np.ascontiguousarray(R, dtype=np.uint32).view(np.int32)
    S = np.ascontiguousarray(S, dtype=np.uint32).view(np.int32)
    out = ctypes.POINTER(ctypes.c_int)()
    n = L.ref_classical(_ip(R), R.shape[0], _ip(S), S.shape[0], ctypes.byref(out))
    return _ref_take(L, out, n, 2)


def ref_estimate(R, S):
    L = ref()
    R = np.ascontiguousarray(R, dtype=np.uint32).view(np.int32)
    S = np.ascontiguousarray(S, dtype=np.uint32).view(np.int32)
    return L.ref_estimate(_ip(R), R.shape[0], _ip(S), S.shape[0])


def ref_join_count(R, S):
    L = ref()
    R = np.ascontiguousarray(R, dtype=np.uint32).view(np.int32)
    S = np.ascontiguousarray(S, dtype=np.uint32).view(np.int32)
    oxz = ctypes.POINTER(ctypes.c_int)()
    oc = ctypes.POINTER(ctypes.c_longlong)()
    n = L.ref_join_count(_ip(R), R.shape[0], _ip(S), S.shape[0], ctypes.byref(oxz), ctypes.byref(oc))
    pairs = _ref_take(L, oxz, n, 2)
    cnt = np.ctypeslib.as_array(oc, shape=(max(n, 1),)).copy()[:n].astype(np.uint64)
    L.ref_free(ctypes.cast(oc, ctypes.c_void_p))
    return pairs, cnt


def ref_join_avg(R, Rv, S, Sv):
    L = ref()
    R = np.ascontiguousarray(R, dtype=np.uint32).view(np.int32)
    S = np.ascontiguousarray(S, dtype=np.uint32).view(np.int32)
    Rv = np.ascontiguousarray(Rv, dtype=np.float32)
    Sv = np.ascontiguousarray(Sv, dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    oxz = ctypes.POINTER(ctypes.c_int)()
    oa = fp()
    n = L.ref_join_avg(_ip(R), Rv.ctypes.data_as(fp), R.shape[0], _ip(S), Sv.ctypes.data_as(fp), S.shape[0],
                       ctypes.byref(oxz), ctypes.byref(oa))
    pairs = _ref_take(L, oxz, n, 2)
    avg = np.ctypeslib.as_array(oa, shape=(max(n, 1),)).copy()[:n]
    L.ref_free(ctypes.cast(oa, ctypes.c_void_p))
    return pairs, avg
