"""C-ABI checks that need no GPU: the library loads, exports every symbol the header
declares, rejects bad arguments before touching the device, and its host-side
generators are deterministic."""
import ctypes as C

import numpy as np
import pytest

import atc
from conftest import write_gr


def test_exports_every_declared_symbol():
    lib = atc.lib()
    names = atc.header_symbols()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_status_strings():
    assert "sm_103a" in atc.version()
    lib = atc.lib()
    for s in atc.Status:
        assert lib.atc_status_string(int(s))


def test_rmat_host_deterministic():
    a = atc.gen_rmat(10, 4, seed=9, nthreads=1)
    b = atc.gen_rmat(10, 4, seed=9, nthreads=7)
    assert np.array_equal(a, b)
    c = atc.gen_rmat(10, 4, seed=10)
    assert not np.array_equal(a, c)
    assert a.min() >= 0 and a.max() < 1024


def test_rmat_skew():
    # quadrant a = 0.57 puts most mass on low ids
    a = atc.gen_rmat(12, 16, seed=1)
    assert (a < 2048).mean() > 0.7


def test_simplify():
    p = np.array([[1, 2], [2, 1], [3, 3], [0, 5], [5, 0], [1, 2]], dtype=np.int32)
    assert atc.simplify(p, symmetric=False).tolist() == [[0, 5], [1, 2]]
    assert atc.simplify(p, symmetric=True).tolist() == [[0, 5], [1, 2], [2, 1], [5, 0]]


def test_argument_checks_without_gpu():
    lib = atc.lib()
    st = atc.CSRStruct()
    # NULL pairs with a non-zero count is rejected before any device work
    assert lib.atc_pretc(None, 5, 0, 0, None, C.byref(st), None, None) == atc.Status.ERR_INVALID
    assert lib.atc_pretc(None, 0, 9, 0, None, C.byref(st), None, None) in (atc.Status.ERR_INVALID,)
    cnt = C.c_uint64()
    assert lib.atc_tc(None, 0, None, C.byref(cnt), None, None) == atc.Status.ERR_INVALID
    assert lib.atc_kcl(C.byref(st), 2, C.byref(cnt), None, None) == atc.Status.ERR_INVALID
    buf = np.zeros(4, dtype=np.int32)
    assert lib.atc_gen_rmat_host(40, 1, 570000, 190000, 190000, 1, buf.ctypes.data, 1) == atc.Status.ERR_INVALID
    assert lib.atc_gen_rmat_host(4, 1, 900000, 190000, 190000, 1, buf.ctypes.data, 1) == atc.Status.ERR_INVALID
    with pytest.raises(atc.ATCError):
        atc.simplify(np.array([[-1, 2]], dtype=np.int32))
    # parts: a part outside [0, nparts) and zero parts are refused before any device work
    rng = (C.c_int64 * 2)()
    assert lib.atc_tc_part(C.byref(st), 0, None, 3, 3, C.byref(cnt), rng, None, None) == atc.Status.ERR_INVALID
    assert lib.atc_tc_part(C.byref(st), 0, None, 0, 0, C.byref(cnt), rng, None, None) == atc.Status.ERR_INVALID
    assert lib.atc_tc_part(None, 0, None, 0, 1, C.byref(cnt), rng, None, None) == atc.Status.ERR_INVALID
    assert lib.atc_kcl_part(C.byref(st), 4, 3, 3, C.byref(cnt), rng, None, None) == atc.Status.ERR_INVALID
    assert lib.atc_kcl_part(C.byref(st), 4, 0, 0, C.byref(cnt), rng, None, None) == atc.Status.ERR_INVALID
    assert lib.atc_kcl_part(C.byref(st), 2, 0, 1, C.byref(cnt), rng, None, None) == atc.Status.ERR_INVALID
    assert lib.atc_kcl_part(None, 4, 0, 1, C.byref(cnt), rng, None, None) == atc.Status.ERR_INVALID
    assert lib.atc_csr_host_resident(None, None) == atc.Status.ERR_INVALID
    assert lib.atc_csr_host_resident(C.byref(st), None) == atc.Status.ERR_INVALID  # not built by the library
    assert lib.atc_csr_load_host(b"/nonexistent/g.atccsr", C.byref(st), None) == atc.Status.ERR_INVALID


def test_csr_cache_forged_headers_rejected(tmp_path):
    # the cache reader checks n and m against the file before allocating or touching a device
    lib = atc.lib()
    st = atc.CSRStruct()

    def cache(n, m, body_ints):
        h = b"ATCCSR01" + np.array([n, m, n, 0, 0], dtype=np.int64).tobytes() + np.zeros(4, np.int32).tobytes()
        return h + np.array(body_ints, dtype=np.int32).tobytes()

    cases = {
        "huge_m": cache(2, 1 << 60, [0, 0, 1, 0, 1, 0, 1]),       # m far beyond the file
        "wrapping_m": cache(2, (1 << 62) + 1, [0, 0, 1, 0, 1, 0, 1]),
        "short_offsets": cache(1 << 20, 1, [0, 0]),               # n beyond the file
        "negative_n": cache(-1, 0, []),
        "bad_order": cache(2, 2, [0, 0, 2, 0, 2, 0, 1, 0]),      # offsets 0, 2, 2 but row 0 is [1, 0]
        "bad_magic": b"ATCCSR02" + cache(1, 0, [0, 0, 0, 0])[8:],
    }
    for name, data in cases.items():
        p = tmp_path / (name + ".atccsr")
        p.write_bytes(data)
        for load in (lib.atc_csr_load, lib.atc_csr_load_host):
            assert load(str(p).encode(), C.byref(st), None) == atc.Status.ERR_INVALID, name
    # unknown relabel kind
    pairs = np.array([[0, 1], [1, 2]], dtype=np.int32)
    lookup = np.zeros(3, dtype=np.int32)
    assert lib.atc_relabel(pairs.ctypes.data, 2, 9, lookup.ctypes.data, None, None, None) == atc.Status.ERR_INVALID


def test_csr_free_is_idempotent():
    st = atc.CSRStruct()
    assert atc.lib().atc_csr_free(C.byref(st)) == 0


def test_rgg_host_deterministic_and_geometric():
    a = atc.gen_rgg(4096, 16.0, seed=5, nthreads=1)
    b = atc.gen_rgg(4096, 16.0, seed=5, nthreads=5)
    assert np.array_equal(a, b)
    assert np.all(a[:, 0] < a[:, 1])
    mean_deg = 2 * a.shape[0] / 4096
    assert 13.0 < mean_deg < 17.0


@pytest.mark.parametrize("version", [1, 2])
def test_read_edges_galois_gr(tmp_path, version):
    rng = np.random.default_rng(version)
    n = 50
    pairs = atc.simplify(rng.integers(0, n, size=(300, 2)).astype(np.int32))
    adj = [sorted(int(v) for v in pairs[pairs[:, 0] == u][:, 1]) for u in range(n)]
    path = tmp_path / "g.gr"
    write_gr(path, n, adj, version)
    got = atc.read_edges(path)
    assert np.array_equal(got, pairs)


def test_read_edges_pair_file_and_errors(tmp_path):
    pairs = np.array([[0, 1], [2, 3], [5, 4]], dtype=np.int32)
    p = tmp_path / "e.bin"
    p.write_bytes(pairs.tobytes() + b"\1\2\3")          # trailing partial pair ignored
    assert np.array_equal(atc.read_edges(p), pairs)
    empty = tmp_path / "empty.bin"
    empty.write_bytes(b"")
    assert atc.read_edges(empty).shape == (0, 2)
    bad = tmp_path / "bad.gr"
    write_gr(bad, 3, [[1], [5], []], 1)                  # target beyond n
    with pytest.raises(atc.ATCError):
        atc.read_edges(bad)
    trunc = tmp_path / "trunc.gr"
    write_gr(trunc, 3, [[1, 2], [0], [0]], 2)
    trunc.write_bytes(trunc.read_bytes()[:-8])
    with pytest.raises(atc.ATCError):
        atc.read_edges(trunc)
    with pytest.raises(atc.ATCError):
        atc.read_edges(tmp_path / "missing.bin")
    # forged headers: an edge count whose byte size wraps, a node count beyond the file,
    # an unknown version, and end offsets that go down
    for hdr in ([1, 0, 2, 1 << 62], [2, 0, 1 << 30, 1], [3, 0, 2, 1]):
        forged = tmp_path / "forged.gr"
        forged.write_bytes(np.array(hdr + [0, 1, 1, 0], dtype=np.uint64).tobytes())
        with pytest.raises(atc.ATCError):
            atc.read_edges(forged)
    down = tmp_path / "down.gr"
    down.write_bytes(np.array([2, 0, 2, 1, 1, 0, 1], dtype=np.uint64).tobytes())
    with pytest.raises(atc.ATCError):
        atc.read_edges(down)


def test_struct_layouts_and_enums_match_the_header(tmp_path):
    # sizeof / offsetof of every struct of atc.h and the value of every enumerator, from a C
    # compiler, against the ctypes mirrors
    import os
    import shutil
    import subprocess
    from conftest import ROOT
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"atc_tuning": atc.Tuning, "atc_csr": atc.CSRStruct, "atc_stats": atc.StatsStruct,
               "atc_phase_time": atc.PhaseTimeStruct}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "atc.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    enums = {"ATC_": atc.Status, "ATC_DIR_": atc.Dir, "ATC_ORDER_": atc.Order, "ATC_RELABEL_": atc.Relabel,
             "ATC_KERNEL_": atc.Kernel}
    for prefix, py in enums.items():
        for e in py:
            lines.append('printf("enum %s%s %%d\\n", (int)%s%s);' % (prefix, e.name, prefix, e.name))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {(a, b): int(c) for a, b, c in (ln.split() for ln in out if ln)}
    for prefix, py in enums.items():
        for e in py:
            assert got[("enum", prefix + e.name)] == int(e), prefix + e.name
    for cname, py in mirrors.items():
        assert got[(cname, "sizeof")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_error_text_is_per_thread():
    # two threads fail different argument checks at the same time; each reads its own message
    import threading
    lib = atc.lib()
    cnt = C.c_uint64()
    barrier = threading.Barrier(2)
    seen = {}

    def fail_kcl():
        barrier.wait()
        for _ in range(200):
            assert lib.atc_kcl(None, 4, C.byref(cnt), None, None) == atc.Status.ERR_INVALID
            seen.setdefault("kcl", set()).add(lib.atc_last_error())

    def fail_relabel():
        pairs = np.array([[0, 1]], dtype=np.int32)
        lookup = np.zeros(2, dtype=np.int32)
        barrier.wait()
        for _ in range(200):
            assert lib.atc_relabel(pairs.ctypes.data, 1, 9, lookup.ctypes.data, None, None, None) == \
                atc.Status.ERR_INVALID
            seen.setdefault("relabel", set()).add(lib.atc_last_error())

    ts = [threading.Thread(target=fail_kcl), threading.Thread(target=fail_relabel)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert len(seen["kcl"]) == 1 and len(seen["relabel"]) == 1
    assert seen["kcl"] != seen["relabel"]


def test_alloc_budget_refuses_device_allocations_before_any_device_call():
    # a spent budget turns the first device allocation of a call into ATC_ERR_OOM; the call
    # returns before it touches the device, so this runs without a GPU
    pairs = np.array([[0, 1], [1, 2], [2, 0]], dtype=np.int32)
    csr = atc.CSRStruct()
    lib = atc.lib()
    try:
        atc.set_alloc_budget(0)
        rc = lib.atc_pretc(pairs.ctypes.data, 3, int(atc.Dir.DEGREE), 0, None, C.byref(csr), None, None)
        assert rc == atc.Status.ERR_OOM
        assert b"allocation budget" in lib.atc_last_error()
        with pytest.raises(atc.ATCError) as ei:
            atc.pretc(pairs, atc.Dir.DEGREE)
        assert ei.value.status == atc.Status.ERR_OOM
        b = C.c_void_p()
        assert lib.atc_batch_create(C.byref(b)) == 0
        try:
            assert lib.atc_batch_reserve(b, 1 << 20, 1 << 22, None) == atc.Status.ERR_OOM
            assert b"allocation budget" in lib.atc_last_error()
        finally:
            lib.atc_batch_destroy(b)
    finally:
        atc.set_alloc_budget(None)


def test_phase_timing_without_gpu():
    # recording on, nothing recorded by calls that fail their argument checks, then off
    atc.phase_timing(True)
    try:
        cnt = C.c_uint64()
        assert atc.lib().atc_kcl(None, 4, C.byref(cnt), None, None) == atc.Status.ERR_INVALID
        assert atc.phase_times() == []
    finally:
        atc.phase_timing(False)
    n = C.c_int32(5)
    assert atc.lib().atc_phase_times(None, 0, C.byref(n)) == 0 and n.value == 0
    assert atc.lib().atc_phase_times(None, 0, None) == atc.Status.ERR_INVALID
