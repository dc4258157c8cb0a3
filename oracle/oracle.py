"""ctypes loader for the CPU oracle (atc_oracle.cpp) — TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU legs as the checker
or the timed CPU baseline.  The product library never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
_lib = None
_P = C.c_void_p


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_simple_stats.argtypes = [_P, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.orc_tc_count.restype = C.c_uint64
        L.orc_tc_count.argtypes = [_P, C.c_uint64, C.c_int]
        L.orc_tc_count_lower_sample.restype = C.c_uint64
        L.orc_tc_count_lower_sample.argtypes = [_P, _P, C.c_int64, C.c_int64, C.c_int64, C.c_int,
                                                C.POINTER(C.c_int64)]
        L.orc_lower_csr.argtypes = [_P, C.c_uint64, _P, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int]
        L.orc_symmetric_csr.argtypes = [_P, C.c_uint64, _P, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.orc_adirection.restype = C.c_int64
        L.orc_adirection.argtypes = [_P, C.c_uint64, _P, _P]
        L.orc_aorder.restype = C.c_int
        L.orc_aorder.argtypes = [_P, C.c_uint64, _P, _P, _P]
        L.orc_kclique.restype = C.c_uint64
        L.orc_kclique.argtypes = [_P, C.c_uint64, C.c_int, C.c_int]
        L.orc_kclique_sample.restype = C.c_uint64
        L.orc_kclique_sample.argtypes = [_P, C.c_uint64, C.c_int, C.c_int64, C.c_int64, C.c_int, C.POINTER(C.c_int64)]
        L.orc_mlp_grad.argtypes = [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_int, _P,
                                   C.POINTER(C.c_double)]
        L.orc_core_numbers.argtypes = [_P, C.c_uint64, _P]
        L.orc_relabel.argtypes = [_P, C.c_uint64, C.c_int, _P, _P]
        L.orc_gro.restype = C.c_int32
        L.orc_gro.argtypes = [_P, C.c_uint64, _P, _P]
        L.orc_adirection_par.argtypes = [_P, C.c_uint64, C.c_int, _P, _P, _P, _P]
        L.orc_costfunc.argtypes = [_P, C.c_uint64, C.c_int, _P]
        L.orc_verification.argtypes = [_P, C.c_uint64, _P]
        L.orc_hu_csr.restype = C.c_int64
        L.orc_hu_csr.argtypes = [_P, C.c_uint64, _P, _P, C.POINTER(C.c_int64)]
        L.orc_adirection_bisson.restype = C.c_int64
        L.orc_adirection_bisson.argtypes = [_P, C.c_uint64, _P, _P]
        L.orc_gen_rmat.restype = C.c_int
        L.orc_gen_rmat.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, _P,
                                   C.c_int]
        L.orc_wedges.restype = C.c_uint64
        L.orc_wedges.argtypes = [_P, _P, C.c_int64]
        _lib = L
    return _lib


def _pairs(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a.reshape(-1, 2)


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def nthreads_default():
    return os.cpu_count() or 1


def gen_rmat(scale, edge_factor=16, seed=1, abc=(570000, 190000, 190000), nthreads=None):
    """The benchmark's seeded R-MAT samples (edge_factor * 2^scale pairs), generated without
    libatc (equal to atc.gen_rmat, checked by a CPU test)."""
    out = np.empty(((edge_factor << scale), 2), dtype=np.int32)
    rc = lib().orc_gen_rmat(scale, edge_factor, abc[0], abc[1], abc[2], seed, _ptr(out), nthreads or nthreads_default())
    assert rc == 0, "bad R-MAT parameters"
    return out


def simple_stats(pairs):
    p = _pairs(pairs)
    n, m = C.c_int64(0), C.c_int64(0)
    lib().orc_simple_stats(_ptr(p), p.shape[0], C.byref(n), C.byref(m))
    return n.value, m.value


def tc_count(pairs, nthreads=None):
    p = _pairs(pairs)
    return lib().orc_tc_count(_ptr(p), p.shape[0], nthreads or nthreads_default())


def symmetric_csr(pairs):
    p = _pairs(pairs)
    n, nnz = C.c_int64(0), C.c_int64(0)
    lib().orc_symmetric_csr(_ptr(p), p.shape[0], None, None, C.byref(n), C.byref(nnz))
    off = np.empty(n.value + 1, dtype=np.int64)
    nbr = np.empty(max(nnz.value, 1), dtype=np.int32)
    lib().orc_symmetric_csr(_ptr(p), p.shape[0], _ptr(off), _ptr(nbr), C.byref(n), C.byref(nnz))
    return off, nbr


def lower_csr(pairs, nthreads=None):
    """Per-vertex sorted lists of smaller neighbours of the simple graph (int64 offsets)."""
    p = _pairs(pairs)
    n, nnz = C.c_int64(0), C.c_int64(0)
    nt = nthreads or nthreads_default()
    lib().orc_lower_csr(_ptr(p), p.shape[0], None, None, C.byref(n), C.byref(nnz), nt)
    off = np.empty(n.value + 1, dtype=np.int64)
    nbr = np.empty(max(nnz.value, 1), dtype=np.int32)
    lib().orc_lower_csr(_ptr(p), p.shape[0], _ptr(off), _ptr(nbr), C.byref(n), C.byref(nnz), nt)
    return off, nbr


def tc_count_lower_sample(off, nbr, stride, phase=0, nthreads=None):
    """(triangles, edges) over the vertices phase, phase+stride, ... of a lower CSR."""
    e = C.c_int64(0)
    c = lib().orc_tc_count_lower_sample(_ptr(off), _ptr(nbr), len(off) - 1, stride, phase,
                                        nthreads or nthreads_default(), C.byref(e))
    return c, e.value


def adirection(pairs, want_prio=False):
    p = _pairs(pairs)
    out = np.empty((max(p.shape[0], 1), 2), dtype=np.int32)
    prio = np.empty((int(p.max()) + 1) if p.size else 1, dtype=np.int32)
    k = lib().orc_adirection(_ptr(p), p.shape[0], _ptr(out), _ptr(prio))
    res = out[:k].copy()
    return (res, prio) if want_prio else res


UNSUPPORTED = 5


def adirection_bisson(pairs):
    """Bisson/A-direction.cpp: (lookup, lpBasedGraph.bin pairs), or None where the serial
    program would not terminate."""
    p = _pairs(pairs)
    n = int(p.max()) + 1 if p.size else 1
    lookup = np.empty(n, dtype=np.int32)
    out = np.empty((2 * p.shape[0] + 1, 2), dtype=np.int32)
    r = lib().orc_adirection_bisson(_ptr(p), p.shape[0], _ptr(lookup), _ptr(out))
    if r < 0:
        return None
    sym = simple_stats(p)[1] * 2 if p.size else 0
    return lookup, out[:sym].copy()


def aorder(pairs):
    """(lookup, normal, reordered), or None where the reference would read out of bounds."""
    p = _pairs(pairs)
    nin = (int(p.max()) + 1) if p.size else 1
    lookup = np.empty(nin, dtype=np.int32)
    normal = np.empty_like(p)
    reordered = np.empty_like(p)
    st = lib().orc_aorder(_ptr(p), p.shape[0], _ptr(lookup), _ptr(normal), _ptr(reordered))
    if st == UNSUPPORTED:
        return None
    return lookup, normal, reordered


def kclique(pairs, k, nthreads=None):
    p = _pairs(pairs)
    return lib().orc_kclique(_ptr(p), p.shape[0], k, nthreads or nthreads_default())


def kclique_sample(pairs, k, stride, phase=0, nthreads=None):
    """(k-cliques whose smallest vertex is phase, phase+stride, ..., edges out of those)."""
    p = _pairs(pairs)
    e = C.c_int64(0)
    c = lib().orc_kclique_sample(_ptr(p), p.shape[0], k, stride, phase, nthreads or nthreads_default(), C.byref(e))
    return c, e.value


def mlp_grad(params, I, H, O, mean, std, x, t, mask=None):
    """(loss, gradient vector) of the selector MLP in double precision."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    params, mean, std, x, t = f(params), f(mean), f(std), f(x), f(t)
    mask = None if mask is None else f(mask)
    g = np.zeros(params.size, dtype=np.float64)
    loss = C.c_double(0)
    lib().orc_mlp_grad(_ptr(params), I, H, O, _ptr(mean), _ptr(std), _ptr(x), _ptr(t), _ptr(mask), x.shape[0],
                       _ptr(g), C.byref(loss))
    return loss.value, g


def core_numbers(pairs):
    p = _pairs(pairs)
    n = (int(p.max()) + 1) if p.size else 0
    out = np.empty(max(n, 1), dtype=np.int32)
    lib().orc_core_numbers(_ptr(p), p.shape[0], _ptr(out))
    return out[:n]


def relabel(pairs, kind):
    """(lookup, normal, relabeled) of A-order-v2 / relabel-naive / relabel4lpOut /
    relabel-random (kinds as atc_relabel_kind: 0, 1, 2, 5, 6, 7)."""
    p = _pairs(pairs)
    n = int(p.max()) + 1 if p.size else 1
    lookup = np.empty(n, dtype=np.int32)
    normal = np.empty((max(p.shape[0], 1), 2), dtype=np.int32)
    lib().orc_relabel(_ptr(p), p.shape[0], int(kind), _ptr(lookup), _ptr(normal))
    normal = normal[: p.shape[0]]
    return lookup, normal, lookup[normal] if normal.size else normal.copy()


def gro(edges_u64):
    """(new_id, max_gain) of other_order's GRO order (porder.cpp:141-226) on packed
    uint64 directed edges (source in the high half)."""
    e = np.ascontiguousarray(edges_u64, dtype=np.uint64)
    vn = lib().orc_gro(_ptr(e), e.size, None, None)
    new_id = np.empty(max(vn, 1), dtype=np.int32)
    mg = C.c_int32(0)
    lib().orc_gro(_ptr(e), e.size, _ptr(new_id), C.byref(mg))
    return new_id[:vn], mg.value


def adirection_par(edges_u64, compat=False):
    """peel.cu on packed uint64 edges: (oriented edges, flags, minor, iterations)."""
    e = np.ascontiguousarray(edges_u64, dtype=np.uint64)
    hi = (e >> np.uint64(32)).max() if e.size else 0
    lo = (e & np.uint64(0xFFFFFFFF)).max() if e.size else 0
    n = int(max(hi, lo)) + 1 if e.size else 0
    out = np.empty(max(e.size, 1), dtype=np.uint64)
    flags = np.empty(max(n, 1), dtype=np.uint32)
    minor = np.empty(max(n, 1), dtype=np.uint32)
    it = np.zeros(1, dtype=np.int32)
    lib().orc_adirection_par(_ptr(e), e.size, 1 if compat else 0, _ptr(out), _ptr(flags), _ptr(minor), _ptr(it))
    return out[: e.size], flags[:n], minor[:n], int(it[0])


def costfunc(pairs, k):
    p = _pairs(pairs)
    out = np.zeros(3, dtype=np.float32)
    lib().orc_costfunc(_ptr(p), p.shape[0], k, _ptr(out))
    return out


def verification(pairs):
    p = _pairs(pairs)
    out = np.zeros(2, dtype=np.float32)
    lib().orc_verification(_ptr(p), p.shape[0], _ptr(out))
    return out


def hu_csr(pairs):
    p = _pairs(pairs)
    m = C.c_int64(0)
    n = lib().orc_hu_csr(_ptr(p), p.shape[0], None, None, C.byref(m))
    off = np.empty(n + 1, dtype=np.uint32)
    cols = np.empty(max(m.value, 1), dtype=np.int32)
    lib().orc_hu_csr(_ptr(p), p.shape[0], _ptr(off), _ptr(cols), C.byref(m))
    return off, cols[: m.value]


def wedges(off, cols):
    off = np.ascontiguousarray(off, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    return lib().orc_wedges(_ptr(off), _ptr(cols), len(off) - 1)
