"""Python binding of libatc's C ABI (include/atc.h), used by the tests and bench.py.

The binding is a thin ctypes layer: it loads the in-tree libatc.so and raises
ATCError when the library is missing or a call fails — there is no Python or CPU
fallback for any entry point.  Host arrays are numpy int32 arrays of shape (m, 2).
"""
from __future__ import annotations

import ctypes as C
import enum
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libatc.so")
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "atc.h")


class ATCError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (Status(status).name if status in Status._value2member_map_ else "?", status, msg))
        self.status = status


class Status(enum.IntEnum):
    OK = 0
    ERR_INVALID = 1
    ERR_OOM = 2
    ERR_CUDA = 3
    ERR_TIMEOUT = 4
    ERR_UNSUPPORTED = 5


class Dir(enum.IntEnum):
    ID = 0
    DEGREE = 1
    DEGREE_LOWID = 2
    ADIRECTION = 3
    KCORE = 4
    ADIRECTION_PAR = 5


class Order(enum.IntEnum):
    NONE = 0
    AORDER = 1
    DEGREE_DESC = 2
    AORDER_V2 = 3
    GRO = 4
    ADIRECTION_BISSON = 5
    NAIVE_SHUFFLED = 6
    RANDOM = 7


class Relabel(enum.IntEnum):
    DEGREE_DESC = 0
    AORDER_V2 = 1
    OUTDEG_DESC = 2
    GRO = 3
    ADIRECTION_BISSON = 4
    NAIVE_SHUFFLED = 5
    OUTDEG_SHUFFLED = 6
    RANDOM = 7


class Kernel(enum.IntEnum):
    AUTO = 0
    HU = 1
    BISSON = 2
    FOX = 3
    TRICORE = 4


class Tuning(C.Structure):
    _fields_ = [
        ("prune_deg1", C.c_int32),
        ("hu_blocks", C.c_int32),
        ("hu_stage_ints", C.c_int32),
        ("bisson_cutover", C.c_int32),
        ("fox_rearrange", C.c_int32),
        ("fox_work_per_thread", C.c_int32),
        ("tricore_blocks", C.c_int32),
        ("bisson_warp_max", C.c_int32),
        ("bisson_warp_chunk", C.c_int32),
        ("bisson_block_chunk", C.c_int32),
        ("bisson_slots", C.c_int32),
        ("group_by_source", C.c_int32),
        ("kcl_dense", C.c_int32),
        ("edge_kernels", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]


class CSRStruct(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("m", C.c_int64),
        ("offsets", C.c_void_p),
        ("cols", C.c_void_p),
        ("n_input", C.c_int64),
        ("wedges", C.c_int64),
        ("dir", C.c_int32),
        ("order", C.c_int32),
        ("pruned", C.c_int32),
        ("max_outdeg", C.c_int32),
        ("wedges_min", C.c_int64),
        ("priv", C.c_void_p),
    ]


class StatsStruct(C.Structure):
    _fields_ = [
        ("kernel_ms", C.c_float),
        ("total_ms", C.c_float),
        ("alg_bytes", C.c_uint64),
        ("wedges", C.c_uint64),
        ("alg_bytes_min", C.c_uint64),
        ("kernel_used", C.c_int32),
        ("launches", C.c_int32),
    ]


class PhaseTimeStruct(C.Structure):
    _fields_ = [
        ("name", C.c_char * 40),
        ("depth", C.c_int32),
        ("ms", C.c_float),
    ]


@dataclass
class Stats:
    kernel_ms: float
    total_ms: float
    alg_bytes: int
    wedges: int
    alg_bytes_min: int
    kernel_used: int
    launches: int


_lib = None

_P = C.c_void_p
_I32P = C.POINTER(C.c_int32)
_SIGS = {
    "atc_version": (C.c_char_p, []),
    "atc_status_string": (C.c_char_p, [C.c_int]),
    "atc_last_error": (C.c_char_p, []),
    "atc_init": (C.c_int, [C.c_int]),
    "atc_set_alloc_budget": (C.c_int, [C.c_int64]),
    "atc_phase_timing": (C.c_int, [C.c_int32]),
    "atc_phase_times": (C.c_int, [C.POINTER(PhaseTimeStruct), C.c_int32, C.POINTER(C.c_int32)]),
    "atc_check_wait_timeout": (C.c_int, [_P]),
    "atc_gen_rmat_host": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, _P, C.c_int]),
    "atc_gen_rmat_device": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, _P, _P]),
    "atc_gen_rgg_host": (C.c_int, [C.c_uint32, C.c_double, C.c_uint64, _P, C.c_uint64, C.POINTER(C.c_uint64), C.c_int]),
    "atc_gen_rgg_device": (C.c_int, [C.c_uint32, C.c_double, C.c_uint64, _P, C.c_uint64, C.POINTER(C.c_uint64), _P]),
    "atc_gen_chunglu_device": (C.c_int, [C.c_uint32, C.c_double, C.c_double, C.c_uint64, _P, C.c_uint64,
                                          C.POINTER(C.c_uint64), _P]),
    "atc_simplify_host": (C.c_int, [_P, C.c_uint64, C.c_int, _P, C.POINTER(C.c_uint64)]),
    "atc_pretc": (C.c_int, [_P, C.c_uint64, C.c_int, C.c_int, C.POINTER(Tuning), C.POINTER(CSRStruct), _P, _P]),
    "atc_pretc_device": (C.c_int, [_P, C.c_uint64, C.c_int, C.c_int, C.POINTER(Tuning), C.POINTER(CSRStruct), _P, _P]),
    "atc_csr_to_host": (C.c_int, [C.POINTER(CSRStruct), _P, _P, _P]),
    "atc_csr_free": (C.c_int, [C.POINTER(CSRStruct)]),
    "atc_kcore_direction": (C.c_int, [_P, C.c_uint64, _P, _P, C.POINTER(C.c_uint64), _P]),
    "atc_adirection_par": (C.c_int, [_P, C.c_uint64, C.c_int, _P, _P, _P, C.POINTER(C.c_uint64), _P, _P]),
    "atc_read_edges": (C.c_int, [C.c_char_p, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "atc_csr_save": (C.c_int, [C.POINTER(CSRStruct), C.c_char_p, _P]),
    "atc_csr_load": (C.c_int, [C.c_char_p, C.POINTER(CSRStruct), _P]),
    "atc_csr_load_host": (C.c_int, [C.c_char_p, C.POINTER(CSRStruct), _P]),
    "atc_csr_host_resident": (C.c_int, [C.POINTER(CSRStruct), _P]),
    "atc_adirection": (C.c_int, [_P, C.c_uint64, _P, C.POINTER(C.c_uint64), _P, _P]),
    "atc_aorder": (C.c_int, [_P, C.c_uint64, _P, _P, _P, _P]),
    "atc_relabel": (C.c_int, [_P, C.c_uint64, C.c_int, _P, _P, _P, _P]),
    "atc_tc": (C.c_int, [C.POINTER(CSRStruct), C.c_int, C.POINTER(Tuning), C.POINTER(C.c_uint64), C.POINTER(StatsStruct), _P]),
    "atc_tc_noalloc": (C.c_int, [_P, _P, C.c_int64, C.c_int64, C.POINTER(C.c_uint64), _P]),
    "atc_kcl_part": (C.c_int, [C.POINTER(CSRStruct), C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64),
                               C.POINTER(C.c_int64), C.POINTER(StatsStruct), _P]),
    "atc_tc_part": (C.c_int, [C.POINTER(CSRStruct), C.c_int, C.POINTER(Tuning), C.c_uint32, C.c_uint32,
                              C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.POINTER(StatsStruct), _P]),
    "atc_kcl_part_tuned": (C.c_int, [C.POINTER(CSRStruct), C.c_uint32, C.POINTER(Tuning), C.c_uint32, C.c_uint32,
                                     C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.POINTER(StatsStruct), _P]),
    "atc_kcl": (C.c_int, [C.POINTER(CSRStruct), C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(StatsStruct), _P]),
    "atc_batch_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "atc_batch_reserve": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, _P]),
    "atc_batch_add": (C.c_int, [C.c_void_p, C.POINTER(CSRStruct), C.POINTER(C.c_int32), _P]),
    "atc_batch_run": (C.c_int, [C.c_void_p, C.POINTER(Tuning), _P, C.POINTER(StatsStruct), _P]),
    "atc_batch_tune": (C.c_int, [C.c_void_p, _P, C.c_int32, C.POINTER(C.c_int32), _P, _P]),
    "atc_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "atc_batch_destroy": (C.c_int, [C.c_void_p]),
    "atc_mlp_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "atc_mlp_destroy": (C.c_int, [C.c_void_p]),
    "atc_mlp_params": (C.c_int, [C.c_void_p, _P, _P, C.POINTER(C.c_int64)]),
    "atc_mlp_scaling": (C.c_int, [C.c_void_p, _P, _P, _P, _P]),
    "atc_mlp_forward": (C.c_int, [C.c_void_p, _P, C.c_int32, _P, _P]),
    "atc_mlp_gradients": (C.c_int, [C.c_void_p, _P, _P, _P, C.c_int32, _P, _P, _P]),
    "atc_mlp_train": (C.c_int, [C.c_void_p, _P, _P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_uint64,
                                _P, _P]),
    "atc_graph_features": (C.c_int, [_P, C.c_uint64, _P, _P]),
    "atc_select": (C.c_int, [C.c_void_p, _P, C.POINTER(C.c_int32), _P, _P]),
    "atc_costfunc": (C.c_int, [_P, C.c_uint64, C.c_int32, _P, _P]),
    "atc_verification": (C.c_int, [_P, C.c_uint64, _P, _P]),
}


def lib():
    """Loads libatc.so (built by build.py); raises ATCError when it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ATCError(Status.ERR_UNSUPPORTED, "libatc.so not built: run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status):
    if status != 0:
        raise ATCError(status, lib().atc_last_error().decode(errors="replace"))


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _pairs(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    if a.ndim == 1:
        a = a.reshape(-1, 2)
    assert a.ndim == 2 and a.shape[1] == 2
    return a


def version():
    return lib().atc_version().decode()


def init(device=0):
    """Initialises `device` and makes it current (-1: the current device, left as it is)."""
    _check(lib().atc_init(device))


def set_alloc_budget(nbytes):
    """Caps the library's device allocations at `nbytes` in total from now on (None or a
    negative value: no cap).  An allocation beyond the cap fails with ERR_OOM."""
    _check(lib().atc_set_alloc_budget(-1 if nbytes is None else int(nbytes)))


def phase_timing(enable=True):
    """Starts (or stops) recording the library's named phases on this thread."""
    _check(lib().atc_phase_timing(1 if enable else 0))


def phase_times(cap=256):
    """[(name, depth, ms)] of the phases recorded since the last read (cleared by the read)."""
    buf = (PhaseTimeStruct * cap)()
    n = C.c_int32(0)
    _check(lib().atc_phase_times(buf, cap, C.byref(n)))
    return [(buf[i].name.decode(), buf[i].depth, buf[i].ms) for i in range(min(n.value, cap))]


def check_wait_timeout(stream=None):
    """Runs the library's bounded-wait check: returns the status of a wait that cannot
    complete (Status.ERR_TIMEOUT when it gave up within its limit, as it must)."""
    return Status(lib().atc_check_wait_timeout(stream))


GRAPH500 = (570000, 190000, 190000)


def gen_rmat(scale, edge_factor=16, seed=1, abc=GRAPH500, nthreads=None):
    """Raw R-MAT samples (edge_factor * 2^scale pairs) generated on the host."""
    n = edge_factor << scale
    out = np.empty((n, 2), dtype=np.int32)
    _check(lib().atc_gen_rmat_host(scale, edge_factor, abc[0], abc[1], abc[2], seed, _ptr(out),
                                    nthreads or os.cpu_count() or 1))
    return out


def gen_rgg(n, mean_degree=32.0, seed=1, nthreads=None):
    """2-D random geometric graph on the host: edges (i, j), i < j, sorted."""
    cnt = C.c_uint64(0)
    nt = nthreads or os.cpu_count() or 1
    _check(lib().atc_gen_rgg_host(n, mean_degree, seed, None, 0, C.byref(cnt), nt))
    out = np.empty((max(cnt.value, 1), 2), dtype=np.int32)
    _check(lib().atc_gen_rgg_host(n, mean_degree, seed, _ptr(out), cnt.value, C.byref(cnt), nt))
    return out[: cnt.value]


def simplify(pairs, symmetric=True):
    """Loop-free, duplicate-free edges: (min,max) once, or both directions sorted."""
    p = _pairs(pairs)
    out = np.empty((p.shape[0] * (2 if symmetric else 1), 2), dtype=np.int32)
    n = C.c_uint64(0)
    _check(lib().atc_simplify_host(_ptr(p), p.shape[0], 1 if symmetric else 0, _ptr(out), C.byref(n)))
    return out[: n.value].copy()


def read_edges(path):
    """Edge pairs from a Galois .gr file (by suffix) or an int32 pair file (host only)."""
    n = C.c_uint64(0)
    p = os.fsencode(path)
    _check(lib().atc_read_edges(p, None, 0, C.byref(n)))
    out = np.empty((max(n.value, 1), 2), dtype=np.int32)
    _check(lib().atc_read_edges(p, _ptr(out), n.value, C.byref(n)))
    return out[: n.value]


def rmat_graph(scale, edge_factor=16, seed=1, symmetric=True):
    """The benchmarks' input: seeded R-MAT, symmetrised, loops and repeats removed."""
    return simplify(gen_rmat(scale, edge_factor, seed), symmetric=symmetric)


class CSR:
    """Device-resident oriented CSR owned by libatc; freed with free() or on GC."""

    def __init__(self, st: CSRStruct, perm=None):
        self._st = st
        self.perm = perm

    @property
    def n(self):
        return self._st.n

    @property
    def m(self):
        return self._st.m

    @property
    def wedges(self):
        return self._st.wedges

    @property
    def wedges_min(self):
        return self._st.wedges_min

    @property
    def max_outdeg(self):
        return self._st.max_outdeg

    @property
    def struct(self):
        return self._st

    def to_host(self, stream=None):
        off = np.empty(self.n + 1, dtype=np.int64)
        cols = np.empty(self.m, dtype=np.int32)
        _check(lib().atc_csr_to_host(C.byref(self._st), _ptr(off), _ptr(cols), stream))
        return off, cols

    def save(self, path, stream=None):
        _check(lib().atc_csr_save(C.byref(self._st), os.fsencode(path), stream))

    @staticmethod
    def load(path, stream=None, host_resident=False):
        """Loads a CSR cache file; host_resident: edge arrays in mapped host memory."""
        st = CSRStruct()
        f = lib().atc_csr_load_host if host_resident else lib().atc_csr_load
        _check(f(os.fsencode(path), C.byref(st), stream))
        return CSR(st)

    def to_host_resident(self, stream=None):
        """Moves the edge arrays to pinned host memory read by the kernels in place."""
        _check(lib().atc_csr_host_resident(C.byref(self._st), stream))
        return self

    def free(self):
        if self._st is not None and self._st.offsets is not None:
            lib().atc_csr_free(C.byref(self._st))
        self._st = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _tuning(t):
    if t is None:
        return None
    if isinstance(t, Tuning):
        return C.byref(t)
    tt = Tuning()
    for k, v in t.items():
        setattr(tt, k, v)
    return C.byref(tt)


def pretc(pairs, dir=Dir.DEGREE, order=Order.NONE, tuning=None, want_perm=False, stream=None):
    p = _pairs(pairs)
    st = CSRStruct()
    perm = None
    if want_perm:
        nin = int(p.max()) + 1 if p.size else 0
        perm = np.empty(max(nin, 1), dtype=np.int32)
    _check(lib().atc_pretc(_ptr(p), p.shape[0], int(dir), int(order), _tuning(tuning), C.byref(st),
                           _ptr(perm), stream))
    return CSR(st, perm)


def pretc_host_ptr(pairs_ptr, n_pairs, dir=Dir.DEGREE, order=Order.NONE, tuning=None, stream=None):
    """atc_pretc on a raw host address (e.g. a pinned torch tensor's data_ptr())."""
    st = CSRStruct()
    _check(lib().atc_pretc(C.c_void_p(pairs_ptr), n_pairs, int(dir), int(order), _tuning(tuning), C.byref(st),
                           None, stream))
    return CSR(st)


def pretc_device(pairs_dev_ptr, n_pairs, dir=Dir.DEGREE, order=Order.NONE, tuning=None, stream=None):
    st = CSRStruct()
    _check(lib().atc_pretc_device(C.c_void_p(pairs_dev_ptr), n_pairs, int(dir), int(order), _tuning(tuning),
                                  C.byref(st), None, stream))
    return CSR(st)


def _stats(s: StatsStruct):
    return Stats(s.kernel_ms, s.total_ms, s.alg_bytes, s.wedges, s.alg_bytes_min, s.kernel_used, s.launches)


def tc(csr: CSR, kernel=Kernel.AUTO, tuning=None, stream=None):
    cnt = C.c_uint64(0)
    st = StatsStruct()
    _check(lib().atc_tc(C.byref(csr.struct), int(kernel), _tuning(tuning), C.byref(cnt), C.byref(st), stream))
    return cnt.value, _stats(st)


def tc_part(csr: CSR, part, nparts, kernel=Kernel.AUTO, tuning=None, stream=None):
    """atc_tc_part: (count of part `part` of `nparts` work-balanced edge ranges, (first, last) edge, stats)."""
    cnt = C.c_uint64(0)
    rng = (C.c_int64 * 2)()
    st = StatsStruct()
    _check(lib().atc_tc_part(C.byref(csr.struct), int(kernel), _tuning(tuning), part, nparts, C.byref(cnt), rng,
                             C.byref(st), stream))
    return cnt.value, (rng[0], rng[1]), _stats(st)


def kcl_part(csr: CSR, k, part, nparts, dense=True, stream=None):
    """atc_kcl_part: (k-cliques of part `part` of `nparts` edge ranges, (first, last) edge, stats).
    dense=False puts every edge on the warp search (atc_kcl_part_tuned, kcl_dense = -1)."""
    cnt = C.c_uint64(0)
    rng = (C.c_int64 * 2)()
    st = StatsStruct()
    if dense:
        _check(lib().atc_kcl_part(C.byref(csr.struct), k, part, nparts, C.byref(cnt), rng, C.byref(st), stream))
    else:
        _check(lib().atc_kcl_part_tuned(C.byref(csr.struct), k, _tuning({"kcl_dense": -1}), part, nparts,
                                        C.byref(cnt), rng, C.byref(st), stream))
    return cnt.value, (rng[0], rng[1]), _stats(st)


def tc_noalloc(offsets_dev_ptr, cols_dev_ptr, n, m, stream=None):
    """atc_tc_noalloc on plain device arrays (no device allocation inside the call)."""
    cnt = C.c_uint64(0)
    _check(lib().atc_tc_noalloc(C.c_void_p(offsets_dev_ptr), C.c_void_p(cols_dev_ptr), n, m, C.byref(cnt), stream))
    return cnt.value


def kcl(csr: CSR, k, stream=None):
    cnt = C.c_uint64(0)
    st = StatsStruct()
    _check(lib().atc_kcl(C.byref(csr.struct), k, C.byref(cnt), C.byref(st), stream))
    return cnt.value, _stats(st)


class Batch:
    """Many graphs counted in one CUDA-graph replay (atc_batch_*)."""

    def __init__(self):
        h = C.c_void_p()
        _check(lib().atc_batch_create(C.byref(h)))
        self._h = h

    def reserve(self, n, m, stream=None):
        _check(lib().atc_batch_reserve(self._h, n, m, stream))

    def add(self, csr: CSR, stream=None):
        idx = C.c_int32(0)
        _check(lib().atc_batch_add(self._h, C.byref(csr.struct), C.byref(idx), stream))
        return idx.value

    def info(self):
        g, n, m = C.c_int32(0), C.c_int64(0), C.c_int64(0)
        _check(lib().atc_batch_info(self._h, C.byref(g), C.byref(n), C.byref(m)))
        return g.value, n.value, m.value

    def run(self, tuning=None, stream=None):
        g = self.info()[0]
        counts = np.zeros(max(g, 1), dtype=np.uint64)
        st = StatsStruct()
        _check(lib().atc_batch_run(self._h, _tuning(tuning), _ptr(counts), C.byref(st), stream))
        return counts[:g], _stats(st)

    def tune(self, candidates, stream=None):
        arr = (Tuning * len(candidates))()
        for i, c in enumerate(candidates):
            for k, v in c.items():
                setattr(arr[i], k, v)
        best = C.c_int32(0)
        ms = np.zeros(len(candidates), dtype=np.float32)
        _check(lib().atc_batch_tune(self._h, C.cast(arr, C.c_void_p), len(candidates), C.byref(best), _ptr(ms), stream))
        return best.value, ms

    def free(self):
        if self._h:
            lib().atc_batch_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class MLP:
    """The selector network (atc_mlp_*): FP32, trained and run on the GPU."""

    def __init__(self, n_in=6, hidden=64, n_out=24, seed=1):
        h = C.c_void_p()
        _check(lib().atc_mlp_create(n_in, hidden, n_out, seed, C.byref(h)))
        self._h, self.n_in, self.hidden, self.n_out = h, n_in, hidden, n_out

    def params(self, new=None):
        cnt = C.c_int64(0)
        _check(lib().atc_mlp_params(self._h, None, None, C.byref(cnt)))
        if new is not None:
            new = np.ascontiguousarray(new, dtype=np.float32)
            assert new.size == cnt.value
            _check(lib().atc_mlp_params(self._h, None, _ptr(new), C.byref(cnt)))
        out = np.empty(cnt.value, dtype=np.float32)
        _check(lib().atc_mlp_params(self._h, _ptr(out), None, C.byref(cnt)))
        return out

    def scaling(self, mean=None, std=None):
        if mean is not None:
            mean = np.ascontiguousarray(mean, dtype=np.float32)
            std = np.ascontiguousarray(std, dtype=np.float32)
            _check(lib().atc_mlp_scaling(self._h, None, None, _ptr(mean), _ptr(std)))
        m = np.empty(self.n_in, dtype=np.float32)
        s = np.empty(self.n_in, dtype=np.float32)
        _check(lib().atc_mlp_scaling(self._h, _ptr(m), _ptr(s), None, None))
        return m, s

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.n_in)
        y = np.empty((x.shape[0], self.n_out), dtype=np.float32)
        _check(lib().atc_mlp_forward(self._h, _ptr(x), x.shape[0], _ptr(y), None))
        return y

    def gradients(self, x, t, mask=None):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.n_in)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, self.n_out)
        mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        g = np.empty(self.params().size, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _check(lib().atc_mlp_gradients(self._h, _ptr(x), _ptr(t), _ptr(mask), x.shape[0], _ptr(g), _ptr(loss), None))
        return float(loss[0]), g

    def train(self, x, t, mask=None, epochs=200, batch=256, lr=3e-3, seed=1):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.n_in)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, self.n_out)
        mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _check(lib().atc_mlp_train(self._h, _ptr(x), _ptr(t), _ptr(mask), x.shape[0], epochs, batch, lr, seed,
                                   _ptr(loss), None))
        return float(loss[0])

    def select(self, features):
        f = np.ascontiguousarray(features, dtype=np.float32)
        ch = C.c_int32(0)
        y = np.empty(self.n_out, dtype=np.float32)
        _check(lib().atc_select(self._h, _ptr(f), C.byref(ch), _ptr(y), None))
        return ch.value, y

    def free(self):
        if self._h:
            lib().atc_mlp_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def graph_features(pairs_dev_ptr, n_pairs, stream=None):
    out = np.zeros(6, dtype=np.float32)
    _check(lib().atc_graph_features(C.c_void_p(pairs_dev_ptr), n_pairs, _ptr(out), stream))
    return out


def gen_chunglu_device(n, gamma, mean_degree, seed, stream=None):
    """Chung-Lu graph generated on the device; returns a torch int32 (m, 2) cuda tensor."""
    import torch
    cnt = C.c_uint64(0)
    _check(lib().atc_gen_chunglu_device(n, gamma, mean_degree, seed, None, 0, C.byref(cnt), stream))
    out = torch.empty((max(cnt.value, 1), 2), dtype=torch.int32, device="cuda")
    _check(lib().atc_gen_chunglu_device(n, gamma, mean_degree, seed, C.c_void_p(out.data_ptr()), cnt.value,
                                        C.byref(cnt), stream))
    return out[: cnt.value]


def adirection(pairs, want_prio=False, stream=None):
    p = _pairs(pairs)
    out = np.empty((max(p.shape[0], 1), 2), dtype=np.int32)
    n = C.c_uint64(0)
    prio = None
    if want_prio:
        prio = np.empty(int(p.max()) + 1 if p.size else 1, dtype=np.int32)
    _check(lib().atc_adirection(_ptr(p), p.shape[0], _ptr(out), C.byref(n), _ptr(prio), stream))
    res = out[: n.value].copy()
    return (res, prio) if want_prio else res


def kcore_direction(edges_u64, want_core=False, stream=None):
    """The kcore_direction program on packed uint64 edges (src = x >> 32): the oriented
    packed edges in input order, and optionally the core numbers."""
    e = np.ascontiguousarray(edges_u64, dtype=np.uint64)
    out = np.empty(max(e.size, 1), dtype=np.uint64)
    nv = C.c_uint64(0)
    core = None
    if want_core:
        hi = (e >> np.uint64(32)).max() if e.size else 0
        lo = (e & np.uint64(0xFFFFFFFF)).max() if e.size else 0
        core = np.empty(int(max(hi, lo)) + 1 if e.size else 1, dtype=np.int32)
    _check(lib().atc_kcore_direction(_ptr(e), e.size, _ptr(out), _ptr(core), C.byref(nv), stream))
    res = out[: e.size].copy()
    return (res, core[: nv.value]) if want_core else res


def adirection_par(edges_u64, compat=False, stream=None):
    """The Peel program on packed uint64 edges: (oriented edges, flags, minor, iterations)."""
    e = np.ascontiguousarray(edges_u64, dtype=np.uint64)
    hi = (e >> np.uint64(32)).max() if e.size else 0
    lo = (e & np.uint64(0xFFFFFFFF)).max() if e.size else 0
    n = int(max(hi, lo)) + 1 if e.size else 0
    out = np.empty(max(e.size, 1), dtype=np.uint64)
    flags = np.empty(max(n, 1), dtype=np.uint32)
    minor = np.empty(max(n, 1), dtype=np.uint32)
    nv = C.c_uint64(0)
    it = C.c_int32(0)
    _check(lib().atc_adirection_par(_ptr(e), e.size, 1 if compat else 0, _ptr(out), _ptr(flags), _ptr(minor),
                                    C.byref(nv), C.byref(it), stream))
    return out[: e.size].copy(), flags[: nv.value].copy(), minor[: nv.value].copy(), it.value


def relabel(pairs, kind, stream=None):
    """(lookup, normal, relabeled) as A-order-v2 / relabel-naive / relabel4lpOut /
    relabel-random / GRO / Bisson's A-direction compute them (atc_relabel_kind)."""
    p = _pairs(pairs)
    n_v = int(p.max()) + 1 if p.size else 1
    lookup = np.empty(n_v, dtype=np.int32)
    normal = np.empty((max(p.shape[0], 1), 2), dtype=np.int32)
    rel = np.empty_like(normal)
    _check(lib().atc_relabel(_ptr(p), p.shape[0], int(kind), _ptr(lookup), _ptr(normal), _ptr(rel), stream))
    return lookup, normal[: p.shape[0]], rel[: p.shape[0]]


def aorder(pairs, stream=None):
    """Returns (lookup, normal, reordered) exactly as the A-order program computes them."""
    p = _pairs(pairs)
    nin = int(p.max()) + 1 if p.size else 1
    lookup = np.empty(nin, dtype=np.int32)
    normal = np.empty_like(p)
    reordered = np.empty_like(p)
    _check(lib().atc_aorder(_ptr(p), p.shape[0], _ptr(lookup), _ptr(normal), _ptr(reordered), stream))
    return lookup, normal, reordered


def costfunc(pairs, k, stream=None):
    p = _pairs(pairs)
    out = np.zeros(3, dtype=np.float32)
    _check(lib().atc_costfunc(_ptr(p), p.shape[0], k, _ptr(out), stream))
    return out


def verification(pairs, stream=None):
    p = _pairs(pairs)
    out = np.zeros(2, dtype=np.float32)
    _check(lib().atc_verification(_ptr(p), p.shape[0], _ptr(out), stream))
    return out


def header_symbols():
    """Names of every function declared in include/atc.h."""
    import re
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(atc_[a-z0-9_]+)\s*\(", txt)))
