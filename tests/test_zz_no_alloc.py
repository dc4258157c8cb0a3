"""atc_tc_noalloc: the triangle count for callers that cannot allocate device memory.

Such callers (a host whose device memory belongs to another allocator or runtime, a
real-time loop that must not block in the allocator) hand the library their own device
CSR arrays.  The entry point runs the Bisson-style count with all of its scratch in one
fixed array inside the library.  Here it must return exactly the count of the allocating
entry point, atc_tc, for the same CSR, and the oracle's count of the same graph, on two
calls in a row (the second call finds the first call's leftovers in the shared array),
and refuse graphs above its limits and malformed CSRs.  This file runs last so that a
failure here cannot stop other tests.
"""
import ctypes as C

import numpy as np
import pytest

import atc
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _init(gpu_ready):
    yield


def _noalloc(csr):
    st = csr.struct
    return atc.tc_noalloc(st.offsets, st.cols, st.n, st.m)


@pytest.mark.parametrize("scale,seed,d", [(10, 1, atc.Dir.ADIRECTION), (13, 2, atc.Dir.DEGREE),
                                         (14, 3, atc.Dir.ID), (15, 4, atc.Dir.ADIRECTION)])
def test_noalloc_matches_allocating_entry_point(scale, seed, d):
    g = atc.rmat_graph(scale, 16, seed)
    csr = atc.pretc(g, d)
    want, _ = atc.tc(csr, atc.Kernel.BISSON)
    assert want == oracle.tc_count(g)
    assert _noalloc(csr) == want
    assert _noalloc(csr) == want  # second call reuses the shared scratch


def test_noalloc_after_a_larger_graph():
    big = atc.pretc(atc.rmat_graph(15, 16, 9), atc.Dir.DEGREE)
    small = atc.pretc(np.array([[0, 1], [1, 2], [2, 0], [2, 3]], dtype=np.int32), atc.Dir.DEGREE)
    assert _noalloc(big) == atc.tc(big)[0]
    assert _noalloc(small) == 1
    assert _noalloc(small) == 1


def test_noalloc_rejects_oversized_and_malformed_input():
    csr = atc.pretc(atc.rmat_graph(8, 8, 1), atc.Dir.DEGREE)
    st = csr.struct
    cnt = C.c_uint64(7)
    lib = atc.lib()
    rc = lib.atc_tc_noalloc(C.c_void_p(st.offsets), C.c_void_p(st.cols), (1 << 17) + 1, st.m, C.byref(cnt), None)
    assert rc == atc.Status.ERR_INVALID
    assert b"too large" in lib.atc_last_error()
    rc = lib.atc_tc_noalloc(C.c_void_p(st.offsets), C.c_void_p(st.cols), st.n, (1 << 20) + 1, C.byref(cnt), None)
    assert rc == atc.Status.ERR_INVALID
    # an m that does not match the offsets is caught by the device-side check
    rc = lib.atc_tc_noalloc(C.c_void_p(st.offsets), C.c_void_p(st.cols), st.n, st.m - 1, C.byref(cnt), None)
    assert rc == atc.Status.ERR_INVALID
    # the library still counts correctly afterwards
    assert _noalloc(csr) == atc.tc(csr)[0]
