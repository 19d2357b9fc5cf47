"""Python binding of the GB300 join-project library (ctypes over the C ABI
declared in include/dim3gpu.h).

The binding mirrors the reference's entry points:

    DIM3::doJoinProject(R, S, result)          -> Context.join_project(R, S)
    DIM3_parallel::doJoinProject_parallel(...) -> Context.join_project(R, S)
    DIM3JoinAggregate::doJoinAggregate (COUNT) -> Context.join_count(R, S)
    LS_mapper insert / find / size / clear     -> Mapper

Relations are (n, 2) uint32 arrays (x, y) / (z, y).  There is no CPU
fallback: loading fails loudly when the CUDA library is absent.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# DIM3G_LIB selects an alternative build of the same library (tuning sweeps).
LIB_PATH = os.environ.get("DIM3G_LIB") or os.path.join(HERE, "libdim3gpu.so")
GEN_PATH = os.path.join(HERE, "libdim3gen.so")

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_CAPACITY, ERR_DEVICE, ERR_UNSUPPORTED = range(7)
_NAMES = {1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "CAPACITY", 5: "DEVICE", 6: "UNSUPPORTED"}

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_i32p = ctypes.POINTER(ctypes.c_int32)


class Dim3GError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("dim3g error %s (%d): %s" % (_NAMES.get(code, "?"), code, msg))
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [
        ("n_big", ctypes.c_uint64), ("n_small", ctypes.c_uint64), ("n_small_kept", ctypes.c_uint64),
        ("out_j", ctypes.c_uint64), ("n_out", ctypes.c_uint64),
        ("swapped", ctypes.c_uint32), ("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32),
        ("rows_warp", ctypes.c_uint32), ("rows_block", ctypes.c_uint32), ("rows_bitmap", ctypes.c_uint32),
        ("rows_dense", ctypes.c_uint32), ("z_tiles", ctypes.c_uint32), ("heavy_y", ctypes.c_uint32),
        ("ms_map", ctypes.c_float), ("ms_csr", ctypes.c_float), ("ms_count", ctypes.c_float),
        ("ms_write", ctypes.c_float), ("ms_total", ctypes.c_float), ("launches", ctypes.c_uint64),
        ("ms_count_cls", ctypes.c_float * 3), ("ms_write_cls", ctypes.c_float * 3),
        ("out_j_cls", ctypes.c_uint64 * 3), ("n_out_cls", ctypes.c_uint64 * 3),
        ("ms_dense", ctypes.c_float * 3), ("dense_kp", ctypes.c_uint32),
        ("dense_light", ctypes.c_uint64), ("dense_skip", ctypes.c_uint32), ("dense_bucket_max", ctypes.c_uint32),
        ("table_slots", ctypes.c_uint64), ("table_rebuilds", ctypes.c_uint32), ("pad0", ctypes.c_uint32),
    ]

    def as_dict(self):
        d = {}
        for k, _ in self._fields_:
            v = getattr(self, k)
            if k.startswith("ms_") and (k.endswith("_cls") or k == "ms_dense"):
                v = [round(float(x), 3) for x in v]
            elif k.endswith("_cls"):
                v = [int(x) for x in v]
            d[k] = v
        return d


# Every symbol include/dim3gpu.h declares (checked by the CPU test suite).
EXPORTS = [
    "dim3g_create", "dim3g_destroy", "dim3g_set_stream", "dim3g_last_error", "dim3g_get_stats",
    "dim3g_set_param", "dim3g_get_param", "dim3g_trim",
    "dim3g_join_project", "dim3g_join_project_into", "dim3g_join_project_device",
    "dim3g_join_project_count_device", "dim3g_join_count", "dim3g_join_count_device",
    "dim3g_mapper_create", "dim3g_mapper_destroy", "dim3g_mapper_insert", "dim3g_mapper_find",
    "dim3g_mapper_size", "dim3g_mapper_clear", "dim3g_mapper_set_cnt",
    "dim3g_join_project_noalloc",
    "dim3g_relset_create", "dim3g_relset_destroy", "dim3g_relset_bytes", "dim3g_relset_join",
    "dim3g_batch_create", "dim3g_batch_run", "dim3g_batch_info", "dim3g_batch_destroy",
    "dim3g_relset_pair_outj", "dim3g_server_create", "dim3g_server_submit", "dim3g_server_wait",
    "dim3g_server_release", "dim3g_server_stats", "dim3g_server_destroy",
    "dim3g_autotune", "dim3g_tuning_apply", "dim3g_tuning_key", "dim3g_tuning_save", "dim3g_tuning_load",
    "dim3g_join_project_summary", "dim3g_join_count_summary", "dim3g_batch_autotune", "dim3g_calibrate",
]


class Tuning(ctypes.Structure):
    _fields_ = [("tile_bits_log2", ctypes.c_int32), ("block_threads", ctypes.c_int32),
                ("block_slots_log2", ctypes.c_int32), ("warp_slots_log2", ctypes.c_int32),
                ("cta_walk", ctypes.c_int32), ("dense_block", ctypes.c_int32), ("dense_k_max", ctypes.c_int32),
                ("ms", ctypes.c_float), ("ms_default", ctypes.c_float), ("trials", ctypes.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Calibration(ctypes.Structure):
    _fields_ = [("fp8_tflops", ctypes.c_float), ("tile_us", ctypes.c_float), ("hbm_gbs", ctypes.c_float),
                ("sparse_gbs", ctypes.c_float)]

    def as_dict(self):
        return {k: round(float(getattr(self, k)), 4) for k, _ in self._fields_}


class Result(ctypes.Structure):
    _fields_ = [
        ("ticket", ctypes.c_uint64), ("status", ctypes.c_int32), ("swapped", ctypes.c_uint32),
        ("n_out", ctypes.c_uint64), ("out_j", ctypes.c_uint64), ("d_out", ctypes.c_void_p), ("d_cnt", ctypes.c_void_p),
        ("t_submit", ctypes.c_double), ("t_start", ctypes.c_double), ("t_done", ctypes.c_double),
        ("pass_size", ctypes.c_uint32), ("lane", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

OP_PROJECT, OP_COUNT = 0, 1


class Relation(ctypes.Structure):
    _fields_ = [("d_pairs", ctypes.c_void_p), ("n", ctypes.c_uint64)]


class Query(ctypes.Structure):
    _fields_ = [
        ("r", ctypes.c_uint32), ("s", ctypes.c_uint32), ("op", ctypes.c_uint32), ("swapped", ctypes.c_uint32),
        ("d_out", ctypes.c_void_p), ("d_cnt", ctypes.c_void_p), ("capacity", ctypes.c_uint64),
        ("n_out", ctypes.c_uint64), ("out_j", ctypes.c_uint64), ("status", ctypes.c_int32),
        ("pad", ctypes.c_uint32),
    ]

_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError("libdim3gpu.so not built (run __graft_entry__.build()): " + path)
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.dim3g_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
    L.dim3g_destroy.argtypes = [vp]
    L.dim3g_destroy.restype = None
    L.dim3g_set_stream.argtypes = [vp, vp]
    L.dim3g_last_error.argtypes = [vp]
    L.dim3g_last_error.restype = ctypes.c_char_p
    L.dim3g_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.dim3g_set_param.argtypes = [vp, ctypes.c_char_p, ctypes.c_int64]
    L.dim3g_get_param.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]
    L.dim3g_trim.argtypes = [vp]
    L.dim3g_join_project.argtypes = [vp, _u32p, ctypes.c_uint64, _u32p, ctypes.c_uint64, ctypes.POINTER(_u32p), _u64p]
    L.dim3g_join_project_into.argtypes = [vp, _u32p, ctypes.c_uint64, _u32p, ctypes.c_uint64, _u32p,
                                          ctypes.c_uint64, _u64p]
    L.dim3g_join_project_device.argtypes = [vp, vp, ctypes.c_uint64, vp, ctypes.c_uint64, vp, ctypes.c_uint64, _u64p]
    L.dim3g_join_project_count_device.argtypes = [vp, vp, ctypes.c_uint64, vp, ctypes.c_uint64, _u64p]
    L.dim3g_join_count.argtypes = [vp, _u32p, ctypes.c_uint64, _u32p, ctypes.c_uint64, ctypes.POINTER(_u32p),
                                   ctypes.POINTER(_u64p), _u64p]
    L.dim3g_join_count_device.argtypes = [vp, vp, ctypes.c_uint64, vp, ctypes.c_uint64, vp, vp, ctypes.c_uint64,
                                          _u64p]
    L.dim3g_mapper_create.argtypes = [vp, ctypes.c_uint64, ctypes.POINTER(vp)]
    L.dim3g_mapper_destroy.argtypes = [vp]
    L.dim3g_mapper_destroy.restype = None
    L.dim3g_mapper_insert.argtypes = [vp, _u32p, ctypes.c_uint64, _i32p]
    L.dim3g_mapper_find.argtypes = [vp, _u32p, ctypes.c_uint64, _i32p]
    L.dim3g_mapper_size.argtypes = [vp]
    L.dim3g_mapper_size.restype = ctypes.c_int64
    L.dim3g_mapper_clear.argtypes = [vp]
    L.dim3g_mapper_set_cnt.argtypes = [vp, ctypes.c_int64]
    relp, qp = ctypes.POINTER(Relation), ctypes.POINTER(Query)
    L.dim3g_relset_create.argtypes = [vp, relp, ctypes.c_uint32, ctypes.POINTER(vp)]
    L.dim3g_relset_destroy.argtypes = [vp]
    L.dim3g_relset_destroy.restype = None
    L.dim3g_relset_bytes.argtypes = [vp]
    L.dim3g_relset_bytes.restype = ctypes.c_uint64
    L.dim3g_relset_join.argtypes = [vp, qp, ctypes.c_uint32]
    L.dim3g_batch_create.argtypes = [vp, relp, qp, ctypes.c_uint32, ctypes.POINTER(vp)]
    L.dim3g_batch_run.argtypes = [vp, qp]
    L.dim3g_batch_info.argtypes = [vp, ctypes.POINTER(ctypes.c_float), _u64p, _u64p]
    L.dim3g_batch_destroy.argtypes = [vp]
    L.dim3g_batch_destroy.restype = None
    L.dim3g_relset_pair_outj.argtypes = [vp, _u64p]
    L.dim3g_server_create.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(vp)]
    L.dim3g_server_submit.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _u64p]
    L.dim3g_server_wait.argtypes = [vp, ctypes.c_uint64, ctypes.POINTER(Result)]
    L.dim3g_server_release.argtypes = [vp, ctypes.c_uint64]
    L.dim3g_server_stats.argtypes = [vp, _u64p, _u64p, _u64p, _u64p]
    L.dim3g_server_destroy.argtypes = [vp]
    L.dim3g_server_destroy.restype = None
    tp = ctypes.POINTER(Tuning)
    L.dim3g_autotune.argtypes = [vp, vp, ctypes.c_uint64, vp, ctypes.c_uint64, ctypes.c_uint32, tp]
    L.dim3g_tuning_apply.argtypes = [vp, tp]
    L.dim3g_tuning_key.argtypes = [vp, vp, ctypes.c_uint64, vp, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_uint64]
    L.dim3g_tuning_save.argtypes = [ctypes.c_char_p, ctypes.c_char_p, tp]
    L.dim3g_tuning_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, tp]
    L.dim3g_batch_autotune.argtypes = [vp, ctypes.c_uint32, tp]
    L.dim3g_calibrate.argtypes = [vp, ctypes.POINTER(Calibration)]
    for f in (L.dim3g_join_project_summary, L.dim3g_join_count_summary):
        f.argtypes = [vp, vp, ctypes.c_uint64, vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                      _u64p]
    _lib = L
    return L


_libc = ctypes.CDLL(None)
_libc.free.argtypes = [ctypes.c_void_p]


def _pairs(a):
    a = np.ascontiguousarray(a, dtype=np.uint32).reshape(-1, 2)
    return a, a.ctypes.data_as(_u32p), a.shape[0]


def _ptr(t):
    """Device pointer of a torch tensor or an int."""
    return ctypes.c_void_p(t if isinstance(t, int) else t.data_ptr())


class Context:
    """One GPU context: a stream, a workspace and the last call's stats."""

    def __init__(self, device=0):
        self.L = load()
        self.h = ctypes.c_void_p()
        rc = self.L.dim3g_create(device, ctypes.byref(self.h))
        if rc != OK:
            raise Dim3GError(rc, "dim3g_create failed for device %d" % device)

    def close(self):
        if self.h:
            self.L.dim3g_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != OK:
            raise Dim3GError(rc, self.L.dim3g_last_error(self.h).decode(errors="replace"))

    def set_stream(self, stream_handle):
        self._check(self.L.dim3g_set_stream(self.h, ctypes.c_void_p(stream_handle or None)))

    def set_param(self, name, value):
        self._check(self.L.dim3g_set_param(self.h, name.encode(), int(value)))

    def get_param(self, name):
        v = ctypes.c_int64()
        self._check(self.L.dim3g_get_param(self.h, name.encode(), ctypes.byref(v)))
        return v.value

    def stats(self):
        s = Stats()
        self._check(self.L.dim3g_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def trim(self):
        self._check(self.L.dim3g_trim(self.h))

    # -------------------------------------------------------- join-project
    def join_project(self, R, S):
        """Host arrays in, (n, 2) uint32 distinct pairs out (DIM3::doJoinProject)."""
        R, rp, nr = _pairs(R)
        S, sp, ns = _pairs(S)
        out = _u32p()
        n = ctypes.c_uint64()
        self._check(self.L.dim3g_join_project(self.h, rp, nr, sp, ns, ctypes.byref(out), ctypes.byref(n)))
        try:
            if n.value == 0:
                return np.zeros((0, 2), dtype=np.uint32)
            return np.ctypeslib.as_array(out, shape=(n.value * 2,)).copy().reshape(-1, 2)
        finally:
            _libc.free(ctypes.cast(out, ctypes.c_void_p))

    def join_project_into(self, R, S, out):
        """Host arrays in; pairs into the caller's (capacity, 2) uint32 array."""
        R, rp, nr = _pairs(R)
        S, sp, ns = _pairs(S)
        assert out.dtype == np.uint32 and out.flags["C_CONTIGUOUS"]
        n = ctypes.c_uint64()
        self._check(self.L.dim3g_join_project_into(self.h, rp, nr, sp, ns, out.ctypes.data_as(_u32p),
                                                   out.size // 2, ctypes.byref(n)))
        return n.value

    def join_project_device(self, dR, nR, dS, nS, dout, capacity):
        """Device pointers (ints or torch tensors) in and out; returns the pair count."""
        n = ctypes.c_uint64()
        self._check(self.L.dim3g_join_project_device(self.h, _ptr(dR), nR, _ptr(dS), nS, _ptr(dout), capacity,
                                                     ctypes.byref(n)))
        return n.value

    def join_project_count_device(self, dR, nR, dS, nS):
        n = ctypes.c_uint64()
        self._check(self.L.dim3g_join_project_count_device(self.h, _ptr(dR), nR, _ptr(dS), nS, ctypes.byref(n)))
        return n.value

    # ------------------------------------------------------ join-aggregate
    def _summary(self, fn, dR, nR, dS, nS, tiles, lo, hi):
        hi = tiles if hi is None else hi
        out = np.zeros((tiles, 3), dtype=np.uint64)
        self._check(fn(self.h, _ptr(dR), nR, _ptr(dS), nS, tiles, lo, hi, out.ctypes.data_as(_u64p)))
        return out

    def join_project_summary(self, dR, nR, dS, nS, tiles=1, lo=0, hi=None):
        """Per-A-tile (groups, groups, hash) of the join-project, nothing
        written (see dim3g_join_project_summary): a (tiles, 3) uint64 array."""
        return self._summary(self.L.dim3g_join_project_summary, dR, nR, dS, nS, tiles, lo, hi)

    def join_count_summary(self, dR, nR, dS, nS, tiles=1, lo=0, hi=None):
        """Per-A-tile (groups, count sum, hash) of COUNT(*) GROUP BY (a, c)."""
        return self._summary(self.L.dim3g_join_count_summary, dR, nR, dS, nS, tiles, lo, hi)

    def autotune(self, dR, nR, dS, nS, max_trials=0):
        """Time the join under candidate knob settings on this input and
        apply the fastest (see dim3g_autotune); returns the tuning."""
        t = Tuning()
        self._check(self.L.dim3g_autotune(self.h, _ptr(dR), nR, _ptr(dS), nS, max_trials, ctypes.byref(t)))
        return t.as_dict()

    def calibrate(self):
        """Measure the dense block's product rates and the copy bandwidth on
        this device and use them in its cost model (see dim3g_calibrate)."""
        cal = Calibration()
        self._check(self.L.dim3g_calibrate(self.h, ctypes.byref(cal)))
        return cal.as_dict()

    def apply_tuning(self, t):
        tt = Tuning(**{k: t[k] for k, _ in Tuning._fields_})
        self._check(self.L.dim3g_tuning_apply(self.h, ctypes.byref(tt)))

    def tuning_key(self, dR, nR, dS, nS):
        buf = ctypes.create_string_buffer(64)
        self._check(self.L.dim3g_tuning_key(self.h, _ptr(dR), nR, _ptr(dS), nS, buf, 64))
        return buf.value.decode()

    def join_count(self, R, S):
        """COUNT(*) GROUP BY (x, z): returns ((n, 2) uint32 pairs, (n,) uint64 counts)."""
        R, rp, nr = _pairs(R)
        S, sp, ns = _pairs(S)
        oxz = _u32p()
        oc = _u64p()
        n = ctypes.c_uint64()
        self._check(self.L.dim3g_join_count(self.h, rp, nr, sp, ns, ctypes.byref(oxz), ctypes.byref(oc),
                                            ctypes.byref(n)))
        try:
            if n.value == 0:
                return np.zeros((0, 2), dtype=np.uint32), np.zeros(0, dtype=np.uint64)
            pairs = np.ctypeslib.as_array(oxz, shape=(n.value * 2,)).copy().reshape(-1, 2)
            cnt = np.ctypeslib.as_array(oc, shape=(n.value,)).copy()
            return pairs, cnt
        finally:
            _libc.free(ctypes.cast(oxz, ctypes.c_void_p))
            _libc.free(ctypes.cast(oc, ctypes.c_void_p))

    def join_count_device(self, dR, nR, dS, nS, dout_xz, dout_cnt, capacity):
        n = ctypes.c_uint64()
        self._check(self.L.dim3g_join_count_device(self.h, _ptr(dR), nR, _ptr(dS), nS, _ptr(dout_xz),
                                                   _ptr(dout_cnt), capacity, ctypes.byref(n)))
        return n.value


def _queries(specs):
    """Query array from dicts {r, s, op, out, cnt, capacity}; out / cnt are
    torch tensors or device addresses."""
    q = (Query * len(specs))()
    for i, d in enumerate(specs):
        q[i].r, q[i].s = d.get("r", 0), d.get("s", 0)
        q[i].op = d.get("op", OP_PROJECT)
        q[i].d_out = _ptr(d["out"]).value if d.get("out") is not None else None
        q[i].d_cnt = _ptr(d["cnt"]).value if d.get("cnt") is not None else None
        q[i].capacity = d.get("capacity", 0)
    return q


def _results(q):
    return [{"n_out": x.n_out, "out_j": x.out_j, "status": x.status, "swapped": x.swapped} for x in q]


def _relations(rels):
    """Relation array from (device tensor or address, n) pairs."""
    arr = (Relation * len(rels))()
    for i, (t, n) in enumerate(rels):
        arr[i].d_pairs = _ptr(t).value if n else None
        arr[i].n = n
    return arr


class RelSet:
    """Resident relation indexes; joins between them in many-query passes."""

    def __init__(self, ctx, rels):
        self.ctx, self.L = ctx, ctx.L
        self.h = ctypes.c_void_p()
        self._keep = rels
        arr = _relations(rels)
        ctx._check(self.L.dim3g_relset_create(ctx.h, arr, len(rels), ctypes.byref(self.h)))

    def bytes(self):
        return self.L.dim3g_relset_bytes(self.h)

    def pair_outj(self):
        n = len(self._keep)
        m = np.zeros(n * n, dtype=np.uint64)
        self.ctx._check(self.L.dim3g_relset_pair_outj(self.h, m.ctypes.data_as(_u64p)))
        return m.reshape(n, n)

    def join(self, specs, check=True):
        """Runs the queries in one pass; returns per-query results (and
        raises on the first failing status when check is set)."""
        q = _queries(specs)
        rc = self.L.dim3g_relset_join(self.h, q, len(specs))
        if check:
            self.ctx._check(rc)
        return _results(q)

    def close(self):
        if self.h:
            self.L.dim3g_relset_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching server over a RelSet (lanes run query passes on
    their own streams; outputs stay on the device until released)."""

    def __init__(self, relset, lanes=2, max_batch=64, budget_bytes=120 << 30):
        self.relset, self.ctx, self.L = relset, relset.ctx, relset.L
        self.h = ctypes.c_void_p()
        self.ctx._check(self.L.dim3g_server_create(relset.h, lanes, max_batch, budget_bytes, ctypes.byref(self.h)))

    def submit(self, r, s, op=OP_PROJECT):
        t = ctypes.c_uint64()
        self.ctx._check(self.L.dim3g_server_submit(self.h, r, s, op, ctypes.byref(t)))
        return t.value

    def wait(self, ticket):
        res = Result()
        self.ctx._check(self.L.dim3g_server_wait(self.h, ticket, ctypes.byref(res)))
        return res.as_dict()

    def release(self, ticket):
        self.ctx._check(self.L.dim3g_server_release(self.h, ticket))

    def stats(self):
        v = [ctypes.c_uint64() for _ in range(4)]
        self.ctx._check(self.L.dim3g_server_stats(self.h, *[ctypes.byref(x) for x in v]))
        return dict(zip(["completed", "passes", "reserved_bytes", "output_budget"], [x.value for x in v]))

    def close(self):
        if self.h:
            self.L.dim3g_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DeviceArray:
    """A device address viewed through __cuda_array_interface__ (zero copy)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2, "strides": None}


def device_tensor(ptr, shape, typestr="<i4"):
    """torch tensor over device memory the library owns (valid until that
    memory is released)."""
    import torch
    return torch.as_tensor(_DeviceArray(ptr, shape, typestr), device="cuda")


def device_pairs(d_out, n):
    """n pairs at a device address as a (n, 2) uint32 host array."""
    if n == 0:
        return np.empty((0, 2), dtype=np.uint32)
    return device_tensor(d_out, (n, 2), "<i4").cpu().numpy().view(np.uint32)


def device_u64(d_ptr, n):
    if n == 0:
        return np.empty(0, dtype=np.uint64)
    return device_tensor(d_ptr, (n,), "<i8").cpu().numpy().view(np.uint64)


class Batch:
    """Independent joins (R_i, S_i) planned once, each run one CUDA graph."""

    def __init__(self, ctx, pairs, specs):
        """pairs: [((dR, nR), (dS, nS)), ...]; specs: per-join dicts (op,
        out, cnt, capacity)."""
        self.ctx, self.L = ctx, ctx.L
        self.h = ctypes.c_void_p()
        self._keep = (pairs, specs)
        rels = [x for p in pairs for x in p]
        self.q = _queries(specs)
        ctx._check(self.L.dim3g_batch_create(ctx.h, _relations(rels), self.q, len(specs), ctypes.byref(self.h)))

    def run(self, check=True):
        rc = self.L.dim3g_batch_run(self.h, self.q)
        if check:
            self.ctx._check(rc)
        return _results(self.q)

    def autotune(self, max_trials=0):
        """Time the batch graph under candidate knob settings and keep the
        fastest (see dim3g_batch_autotune)."""
        t = Tuning()
        self.ctx._check(self.L.dim3g_batch_autotune(self.h, max_trials, ctypes.byref(t)))
        return t.as_dict()

    def info(self):
        ms, nl, nb = ctypes.c_float(), ctypes.c_uint64(), ctypes.c_uint64()
        self.ctx._check(self.L.dim3g_batch_info(self.h, ctypes.byref(ms), ctypes.byref(nl), ctypes.byref(nb)))
        return {"ms_last": ms.value, "launches_per_run": nl.value, "device_bytes": nb.value}

    def close(self):
        if self.h:
            self.L.dim3g_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tuning_save(path, key, t):
    """Append a tuning (dict of Tuning fields) to the cache file."""
    tt = Tuning(**{k: t[k] for k, _ in Tuning._fields_})
    rc = load().dim3g_tuning_save(path.encode(), key.encode(), ctypes.byref(tt))
    if rc != OK:
        raise Dim3GError(rc, "tuning cache write failed: " + path)


def tuning_load(path, key):
    """The cached tuning of key, or None."""
    tt = Tuning()
    if load().dim3g_tuning_load(path.encode(), key.encode(), ctypes.byref(tt)) != OK:
        return None
    return tt.as_dict()


class Mapper:
    """GPU L+S mapper: value -> dense id with the reference's insert order."""

    def __init__(self, ctx, capacity_hint=1024):
        self.ctx = ctx
        self.L = ctx.L
        self.h = ctypes.c_void_p()
        ctx._check(self.L.dim3g_mapper_create(ctx.h, capacity_hint, ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.L.dim3g_mapper_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _batch(self, fn, keys):
        k = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1)
        ids = np.empty(k.shape[0], dtype=np.int32)
        self.ctx._check(fn(self.h, k.ctypes.data_as(_u32p), k.shape[0], ids.ctypes.data_as(_i32p)))
        return ids

    def insert(self, keys):
        return self._batch(self.L.dim3g_mapper_insert, keys)

    def find(self, keys):
        return self._batch(self.L.dim3g_mapper_find, keys)

    def size(self):
        return self.L.dim3g_mapper_size(self.h)

    def clear(self):
        self.ctx._check(self.L.dim3g_mapper_clear(self.h))

    def set_cnt(self, v):
        self.ctx._check(self.L.dim3g_mapper_set_cnt(self.h, int(v)))


# ------------------------------------------------------------ generators
_gen = None


def gen():
    global _gen
    if _gen is None:
        if not os.path.exists(GEN_PATH):
            raise OSError("libdim3gen.so not built: " + GEN_PATH)
        G = ctypes.CDLL(GEN_PATH)
        G.dim3gen_minstd.argtypes = [ctypes.c_uint32] * 6 + [_u32p, _u32p]
        G.dim3gen_zipf_side.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                        ctypes.c_uint64, _u32p]
        G.dim3gen_chung_lu.argtypes = [ctypes.c_uint32, ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64, _u32p,
                                       _u32p]
        G.dim3gen_chung_lu.restype = ctypes.c_uint64
        G.dim3gen_batch_params.argtypes = [ctypes.c_uint64, ctypes.c_uint32] + [ctypes.c_double] * 6 + [
            _u64p, ctypes.POINTER(ctypes.c_double), _u32p]
        G.dim3gen_rank_value.argtypes = [ctypes.c_uint32]
        G.dim3gen_serve_relation.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                             ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, _u32p]
        G.dim3gen_rank_value.restype = ctypes.c_uint32
        _gen = G
    return _gen


def gen_rand_data(nR=10 ** 7, nS=10 ** 7, modx=10 ** 6, mody=10 ** 6, modz=10 ** 6, seed=492):
    """The reference's gen_rand_data (dim3.hpp:1556-1568), bit-identical."""
    R = np.empty((nR, 2), dtype=np.uint32)
    S = np.empty((nS, 2), dtype=np.uint32)
    gen().dim3gen_minstd(nR, nS, modx, mody, modz, seed, R.ctypes.data_as(_u32p), S.ctypes.data_as(_u32p))
    return R, S


def zipf_side(n, dom_a, dom_b, s, seed):
    out = np.empty((n, 2), dtype=np.uint32)
    if gen().dim3gen_zipf_side(n, dom_a, dom_b, s, seed, out.ctypes.data_as(_u32p)) != 0:
        raise MemoryError("zipf generator failed")
    return out


def chung_lu(n=1 << 21, beta=2.1, M=10 ** 7, seed=7):
    buf = np.empty((2 * M, 2), dtype=np.uint32)
    mw = ctypes.c_uint32()
    k = gen().dim3gen_chung_lu(n, beta, M, seed, buf.ctypes.data_as(_u32p), ctypes.byref(mw))
    return buf[:k]


def batch_params(seed, q, n_lo=1e4, n_hi=4e6, s_lo=0.5, s_hi=1.5, d_lo=1e3, d_hi=1e6):
    n = ctypes.c_uint64()
    s = ctypes.c_double()
    d = ctypes.c_uint32()
    gen().dim3gen_batch_params(seed, q, n_lo, n_hi, s_lo, s_hi, d_lo, d_hi, ctypes.byref(n), ctypes.byref(s),
                               ctypes.byref(d))
    return n.value, s.value, d.value


# Named workloads (the bench and the tests use the same shapes).
def fmix32_np(v):
    """murmur3 fmix32 over a uint32 array (the A-tile and shard function)."""
    v = np.asarray(v, dtype=np.uint32).astype(np.uint64)
    v ^= v >> np.uint64(16)
    v = (v * np.uint64(0x85ebca6b)) & np.uint64(0xFFFFFFFF)
    v ^= v >> np.uint64(13)
    v = (v * np.uint64(0xc2b2ae35)) & np.uint64(0xFFFFFFFF)
    v ^= v >> np.uint64(16)
    return v


def a_shard(R, rank, world):
    """Rows of R whose first value A falls in shard `rank` of `world`
    (fmix32(A) mod world).  The multi-GPU form of the join-project: rank r
    joins its shard of R with all of S; shards of the result are disjoint
    (they partition the pairs by A), so no data is exchanged."""
    R = np.asarray(R, dtype=np.uint32).reshape(-1, 2)
    return np.ascontiguousarray(R[(fmix32_np(R[:, 0]) % np.uint64(world)) == np.uint64(rank)])


def _zipf_sum_p2(dom, s):
    k = np.arange(1, dom + 1, dtype=np.float64)
    w = k ** -s
    return float((w * w).sum() / w.sum() ** 2)


def batch_queries(nq=512, seed=4, n_lo=1e4, n_hi=4e6, s_lo=0.5, s_hi=1.5, d_lo=1e3, d_hi=1e6,
                  cap_outj=2 ** 28, cap_out=2 ** 26):
    """Parameters of the mixed batch: per query |R| and |S| log-uniform in
    [n_lo, n_hi] (drawn separately), B Zipf exponent s uniform in
    [s_lo, s_hi], dom(A) = dom(C) = dom(B) log-uniform in [d_lo, d_hi].
    A draw whose expected join size n_R n_S sum(p_b^2) exceeds cap_outj, or
    whose expected distinct output dom^2 (1 - exp(-E[OUT_J] / dom^2))
    exceeds cap_out, is redrawn from the next seeded stream (`redraws`
    counts them), so the whole batch's output fits in device memory."""
    out = []
    for i in range(nq):
        a = 0
        while True:
            rng = np.random.default_rng([seed, i, a])
            nR = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
            nS = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
            s = float(rng.uniform(s_lo, s_hi))
            dom = int(np.exp(rng.uniform(np.log(d_lo), np.log(d_hi))))
            ej = nR * nS * _zipf_sum_p2(dom, s)
            eo = dom * dom * -np.expm1(-ej / (dom * dom))
            if ej <= cap_outj and eo <= cap_out:
                break
            a += 1
        out.append({"nR": nR, "nS": nS, "s": s, "dom": dom, "redraws": a,
                    "seed_R": (seed << 40) + 2 * i, "seed_S": (seed << 40) + 2 * i + 1})
    return out


def batch_relations(params):
    """(R, S) of every query: first column uniform in [0, dom), y Zipf(s)
    over dom ranks, the same rank -> value map on both sides."""
    return [(zipf_side(p["nR"], p["dom"], p["dom"], p["s"], p["seed_R"]),
             zipf_side(p["nS"], p["dom"], p["dom"], p["s"], p["seed_S"])) for p in params]


def serve_params(n_rel=64, seed=5, n_lo=1e6, n_hi=16e6, alpha_lo=1.8, alpha_hi=2.5, dom_b_log2=18, scale=1.0):
    """Relations of the served set: |R| log-uniform in [n_lo, n_hi] (times
    scale); B-degree power-law exponent alpha uniform in [alpha_lo,
    alpha_hi], drawn as Zipf ranks with s = 1 / (alpha - 1) over a shared
    domain of 2^dom_b_log2 B values, each relation with its own rank -> value
    bijection; dom(A) = |R| / 4."""
    out = []
    for i in range(n_rel):
        rng = np.random.default_rng([seed, i])
        n = max(1, int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))) * scale))
        alpha = float(rng.uniform(alpha_lo, alpha_hi))
        out.append({"n": n, "alpha": alpha, "s": 1.0 / (alpha - 1.0), "dom_a": max(1024, n // 4),
                    "dom_b_log2": dom_b_log2, "mul": int(rng.integers(0, 1 << 31)) * 2 + 1,
                    "add": int(rng.integers(0, 1 << 31)), "seed": (seed << 40) + i})
    return out


def serve_relation(p):
    out = np.empty((p["n"], 2), dtype=np.uint32)
    if gen().dim3gen_serve_relation(p["n"], p["dom_a"], p["dom_b_log2"], p["s"], p["mul"] & 0xFFFFFFFF,
                                    p["add"] & 0xFFFFFFFF, p["seed"], out.ctypes.data_as(_u32p)) != 0:
        raise MemoryError("serve generator failed")
    return out


def workload(name, scale=1.0):
    """Seeded synthetic relations by name; scale < 1 shrinks tuple counts."""
    if name == "zipf_1m":  # 1M tuples per side, dom(A)=dom(C)=50k, dom(B)=20k Zipf s=1.0
        n = max(1, int(10 ** 6 * scale))
        return zipf_side(n, 50000, 20000, 1.0, 101), zipf_side(n, 50000, 20000, 1.0, 202)
    if name == "chung_lu_20m":  # self join of a 2^21-vertex Chung-Lu graph, ~20M directed edges
        M = max(1, int(10 ** 7 * scale))
        nv = 1 << 21 if scale >= 1 else max(1024, int((1 << 21) * scale))
        E = chung_lu(nv, 2.1, M, 7)
        return E, E
    if name == "zipf12_16m":  # 16M tuples per side, dom(A)=dom(C)=1M, dom(B)=200k Zipf s=1.2
        n = max(1, int(16 * 10 ** 6 * scale))
        return zipf_side(n, 10 ** 6, 200000, 1.2, 303), zipf_side(n, 10 ** 6, 200000, 1.2, 404)
    if name == "gen_rand_data":
        n = max(1, int(10 ** 7 * scale))
        return gen_rand_data(n, n, 10 ** 6, 10 ** 6, 10 ** 6, 492)
    if name == "grd_all_dense":  # 3000 x 100 x 3000 domains: every (x, z) group exists
        n = max(1, int(300000 * scale))
        return gen_rand_data(n, n, 3000, 100, 3000, 492)
    raise KeyError(name)
