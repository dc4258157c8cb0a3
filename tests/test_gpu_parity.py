"""GPU parity: libatc (through its C ABI) against the reference programs' golden outputs
and the CPU oracle, on the same seeded inputs.

Integer results must be identical: triangle / k-clique counts, the A-direction
orientation, the A-order permutation and its output files, the CSR.  The cost figures
must print identically to the reference tools.
"""
import hashlib
import json
import os
import sys
from math import comb

import numpy as np
import pytest

import atc
import oracle
from conftest import ROOT, golden_input, load_golden, write_gr

pytestmark = pytest.mark.gpu

CASES = sorted(load_golden()["cases"])
KERNELS = [atc.Kernel.HU, atc.Kernel.BISSON, atc.Kernel.FOX, atc.Kernel.TRICORE]
DIRS = [atc.Dir.ID, atc.Dir.DEGREE, atc.Dir.DEGREE_LOWID, atc.Dir.ADIRECTION, atc.Dir.KCORE,
        atc.Dir.ADIRECTION_PAR]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


def fmt6(x):
    return "%g" % np.float32(x)


@pytest.fixture(scope="module", autouse=True)
def _init(gpu_ready):
    yield


# ---- orientation / ordering: bit-exact against the reference programs -----------------
@pytest.mark.parametrize("name", CASES)
def test_adirection_matches_reference(golden, name):
    c = golden["cases"][name]
    got, prio = atc.adirection(golden_input(c), want_prio=True)
    assert got.shape[0] == c["adirection"]["count"]
    assert sha(got) == c["adirection"]["sha256"]
    _, oprio = oracle.adirection(golden_input(c), want_prio=True)
    assert np.array_equal(prio, oprio)


@pytest.mark.parametrize("name", CASES)
def test_adirection_bisson_matches_reference(golden, name):
    """Bisson/A-direction.cpp: the relabelling (lookup) and its lpBasedGraph.bin output."""
    c = golden["cases"][name]
    g = golden_input(c)
    lookup, normal, rel = atc.relabel(g, atc.Relabel.ADIRECTION_BISSON)
    olookup, oout = oracle.adirection_bisson(g)
    assert np.array_equal(lookup, olookup)
    assert np.array_equal(normal, g) and np.array_equal(rel, lookup[g])
    out = lookup[atc.simplify(g, symmetric=True)] if g.size else np.zeros((0, 2), dtype=np.int32)
    assert out.shape[0] == c["bisson_adir"]["count"] and sha(out) == c["bisson_adir"]["sha256"]


def test_adirection_bisson_order_in_pretc():
    # with the id orientation (src = larger new id) the relabelling realises A-direction:
    # every edge leaves the vertex the peel took first
    for g in (atc.rmat_graph(13, 16, 5), atc.gen_rgg(30000, 10.0, 2), atc.gen_rmat(12, 8, 3)):
        want = oracle.tc_count(g)
        csr = atc.pretc(g, atc.Dir.ID, atc.Order.ADIRECTION_BISSON, want_perm=True)
        olookup, _ = oracle.adirection_bisson(g)
        assert np.array_equal(csr.perm[: olookup.size], olookup)
        for k in KERNELS:
            assert atc.tc(csr, k)[0] == want, k.name
        csr.free()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("which", ["aorder", "aorder_raw"])
def test_aorder_matches_reference(golden, name, which):
    c = golden["cases"][name]
    g = golden_input(c)
    src = oracle.adirection(g) if which == "aorder" else g
    rec = c[which]
    if rec.get("unsupported"):
        with pytest.raises(atc.ATCError) as ei:
            atc.aorder(src)
        assert ei.value.status == atc.Status.ERR_UNSUPPORTED
        return
    lookup, normal, reordered = atc.aorder(src)
    assert sha(normal) == rec["normal"]["sha256"]
    assert sha(reordered) == rec["reordered"]["sha256"]
    olookup, _, _ = oracle.aorder(src)
    assert np.array_equal(lookup, olookup)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("which,kind", [("aorder_v2", atc.Relabel.AORDER_V2), ("relabel_good", atc.Relabel.DEGREE_DESC),
                                        ("relabel4lp", atc.Relabel.OUTDEG_DESC),
                                        ("relabel_naive", atc.Relabel.NAIVE_SHUFFLED),
                                        ("relabel4lp_bad", atc.Relabel.OUTDEG_SHUFFLED),
                                        ("relabel_random", atc.Relabel.RANDOM)])
def test_relabel_matches_reference(golden, name, which, kind):
    c = golden["cases"][name]
    src = oracle.adirection(golden_input(c))
    lookup, normal, rel = atc.relabel(src, kind)
    assert rel.shape[0] == c[which]["count"] and sha(rel) == c[which]["sha256"]
    olookup, onormal, _ = oracle.relabel(src, kind)
    assert np.array_equal(lookup, olookup) and np.array_equal(normal, onormal)


@pytest.mark.parametrize("kind", [atc.Relabel.NAIVE_SHUFFLED, atc.Relabel.OUTDEG_SHUFFLED, atc.Relabel.RANDOM])
def test_shuffled_relabellings_at_scale(kind):
    """The device's rand() stream (every thread jumping ahead to its own stretch) and its
    replay of the shuffles against the oracle, which calls the C library's rand(), on R-MAT
    scale 20 (a million ids: about 500 stretches of the stream) and on an id range with a
    ragged tail (n mod 64 and n mod 40 both non-zero)."""
    for g in (atc.rmat_graph(20, 16, 1), np.array([(0, 1), (1, 2), (2, 0), (5, 1234566)], dtype=np.int32)):
        src = oracle.adirection(g) if g.shape[0] > 4 else g
        lookup, normal, rel = atc.relabel(src, kind)
        olookup, onormal, orel = oracle.relabel(src, int(kind))
        assert np.array_equal(lookup, olookup) and np.array_equal(normal, onormal) and np.array_equal(rel, orel)
        assert np.array_equal(np.sort(lookup), np.arange(lookup.size))


@pytest.mark.parametrize("order", [atc.Order.NAIVE_SHUFFLED, atc.Order.RANDOM])
def test_pretc_shuffled_orders_count_exactly(order):
    g = atc.rmat_graph(14, 16, 3)
    csr = atc.pretc(g, atc.Dir.ADIRECTION, order)
    want = oracle.tc_count(g)
    for k in (atc.Kernel.HU, atc.Kernel.BISSON, atc.Kernel.FOX, atc.Kernel.TRICORE):
        assert atc.tc(csr, k)[0] == want, k
    csr.free()


def pack_u64(pairs):
    pairs = np.asarray(pairs, dtype=np.int32).reshape(-1, 2)
    return (pairs[:, 0].astype(np.uint64) << np.uint64(32)) | pairs[:, 1].astype(np.uint32).astype(np.uint64)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("which", ["gro_sym", "gro_lp"])
def test_gro_matches_reference(golden, name, which):
    """other_order's GRO order (the reorder program's _GRO_newID.txt)."""
    c = golden["cases"][name]
    g = golden_input(c)
    src = atc.simplify(g, symmetric=True) if which == "gro_sym" else oracle.adirection(g)
    lookup, normal, rel = atc.relabel(src, atc.Relabel.GRO)
    onew, _ = oracle.gro(pack_u64(src))
    assert np.array_equal(lookup[: onew.size], onew)
    assert np.array_equal(normal, src) and np.array_equal(rel, lookup[src])
    rec = c.get(which)
    if rec and not rec.get("unsupported"):
        got = np.ascontiguousarray(lookup[: rec["count"]], dtype=np.int32)
        assert hashlib.sha256(got.tobytes()).hexdigest() == rec["sha256"]


def test_gro_order_in_pretc():
    g = atc.rmat_graph(12, 16, 4)
    want = oracle.tc_count(g)
    sym = atc.simplify(g, symmetric=True)
    onew, _ = oracle.gro(pack_u64(sym))
    for d in (atc.Dir.ADIRECTION, atc.Dir.DEGREE, atc.Dir.ID):
        csr = atc.pretc(g, d, atc.Order.GRO, want_perm=True)
        assert np.array_equal(csr.perm[: onew.size], onew)
        for k in KERNELS:
            assert atc.tc(csr, k)[0] == want, (d.name, k.name)


@pytest.mark.parametrize("order", [atc.Order.DEGREE_DESC, atc.Order.AORDER_V2])
def test_relabel_orders_in_pretc(order):
    g = atc.rmat_graph(13, 16, 6)
    want = oracle.tc_count(g)
    kind = atc.Relabel.DEGREE_DESC if order == atc.Order.DEGREE_DESC else atc.Relabel.AORDER_V2
    once = atc.simplify(g, symmetric=False)
    olookup, _, _ = oracle.relabel(once, kind)
    for d in DIRS:
        csr = atc.pretc(g, d, order, want_perm=True)
        assert np.array_equal(csr.perm[: olookup.size], olookup)
        for k in KERNELS:
            assert atc.tc(csr, k)[0] == want, (order.name, d.name, k.name)


@pytest.mark.parametrize("name", CASES)
def test_costs_match_reference(golden, name):
    c = golden["cases"][name]
    lp = oracle.adirection(golden_input(c))
    for k, printed in c["costfunc"].items():
        assert [fmt6(x) for x in atc.costfunc(lp, int(k))] == printed
    assert [fmt6(x) for x in atc.verification(lp)] == c["verification"]


# ---- counts ------------------------------------------------------------------------------
@pytest.mark.parametrize("name", CASES)
def test_counts_all_kernels_and_directions(golden, name):
    c = golden["cases"][name]
    g = golden_input(c)
    want = oracle.tc_count(g)
    if "triangles" in c:
        assert want == c["triangles"]
    for d in DIRS:
        csr = atc.pretc(g, d)
        for k in KERNELS:
            got, st = atc.tc(csr, k)
            assert got == want, (d.name, k.name)
            assert st.kernel_used == int(k)
        for k in (atc.Kernel.FOX, atc.Kernel.TRICORE):  # the per-edge global-search kernels
            assert atc.tc(csr, k, tuning={"edge_kernels": 1})[0] == want, (d.name, k.name)
        csr.free()


@pytest.mark.parametrize("name", [n for n in CASES if n.startswith("rmat_s1")])
def test_counts_with_aorder_and_prune(golden, name):
    g = golden_input(golden["cases"][name])
    want = oracle.tc_count(g)
    for d in DIRS:
        for prune in (0, 1):
            csr = atc.pretc(g, d, atc.Order.AORDER, tuning={"prune_deg1": prune}, want_perm=True)
            assert np.array_equal(np.sort(csr.perm), np.arange(csr.perm.size))
            for k in KERNELS:
                assert atc.tc(csr, k)[0] == want, (d.name, prune, k.name)


def test_tuning_knobs_do_not_change_counts():
    g = atc.rmat_graph(12, 16, 3)
    want = oracle.tc_count(g)
    csr = atc.pretc(g, atc.Dir.ID)  # id orientation: long lists, hubs
    for t in ({"bisson_cutover": 8}, {"bisson_cutover": 64}, {"fox_rearrange": 1, "edge_kernels": 1},
              {"fox_work_per_thread": 4, "edge_kernels": 1}, {"edge_kernels": 1},
              {"hu_blocks": 7}, {"tricore_blocks": 3, "edge_kernels": 1}, {"hu_blocks": 2000}, {"bisson_slots": 1},
              {"bisson_slots": 2}, {"bisson_slots": 4}, {"bisson_slots": 2, "bisson_warp_max": 64, "bisson_cutover": 4},
              {"bisson_warp_max": 512}, {"bisson_warp_max": 384, "bisson_slots": 2},
              {"bisson_warp_max": 512, "bisson_slots": 1, "bisson_warp_chunk": 64}):
        for k in KERNELS:
            assert atc.tc(csr, k, tuning=t)[0] == want, (t, k.name)


def test_warp_tables_at_their_limits():
    """Hubs whose oriented lists are 255, 256 and 257 long (the compact 16-bit warp tables
    hold up to 256 keys; 257 takes the 32-bit table), each joined to a path of its leaves, plus
    a dense core: Bisson- and Hu-style counts with the default and the tuned item shapes."""
    e = []
    base = 0
    for k in (255, 256, 257):
        leaves = list(range(base + 1, base + 1 + k))
        e += [(base, x) for x in leaves] + list(zip(leaves[:-1], leaves[1:]))
        base += k + 1
    e += [(base + a, base + b) for a in range(40) for b in range(a + 1, 40)]
    g = np.array(e, dtype=np.int32)
    want = oracle.tc_count(g)
    assert want == 254 + 255 + 256 + 40 * 39 * 38 // 6
    csr = atc.pretc(g, atc.Dir.ID)
    for t in (None, {"bisson_cutover": 4}, {"bisson_warp_max": 512}, {"bisson_slots": 2}):
        for k in (atc.Kernel.BISSON, atc.Kernel.HU):
            assert atc.tc(csr, k, tuning=t)[0] == want, (t, k.name)


def test_bad_slot_count_rejected():
    csr = atc.pretc(atc.rmat_graph(8, 8, 1), atc.Dir.DEGREE)
    for k in (atc.Kernel.BISSON, atc.Kernel.HU):
        with pytest.raises(atc.ATCError):
            atc.tc(csr, k, tuning={"bisson_slots": 3})


# ---- CSR layout ----------------------------------------------------------------------------
def test_pretc_degree_pruned_equals_hu_csr():
    # Hu's preTC on a once-per-edge list (what A-direction-seri writes)
    g = oracle.adirection(atc.rmat_graph(12, 16, 7))
    off, cols = atc.pretc(g, atc.Dir.DEGREE, tuning={"prune_deg1": 1}).to_host()
    hoff, hcols = oracle.hu_csr(g)
    assert np.array_equal(off, hoff.astype(np.int64))
    assert np.array_equal(cols, hcols)


@pytest.mark.parametrize("d", DIRS)
def test_csr_invariants_and_wedges(d):
    g = atc.rmat_graph(11, 16, 5)
    n, m = oracle.simple_stats(g)
    csr = atc.pretc(g, d)
    off, cols = csr.to_host()
    assert csr.n == n and csr.m == m
    assert off[0] == 0 and off[-1] == m
    for u in range(n):
        lst = cols[off[u]:off[u + 1]]
        assert np.all(np.diff(lst) > 0)
    assert csr.wedges == oracle.wedges(off, cols)
    assert csr.max_outdeg == int(np.diff(off).max())


def test_adirection_csr_is_reference_orientation():
    g = atc.rmat_graph(12, 16, 7)
    off, cols = atc.pretc(g, atc.Dir.ADIRECTION).to_host()
    src = np.repeat(np.arange(off.size - 1), np.diff(off)).astype(np.int32)
    lp = np.stack([src, cols], 1)
    assert np.array_equal(lp, oracle.adirection(g))


@pytest.mark.parametrize("order", [atc.Order.AORDER, atc.Order.DEGREE_DESC, atc.Order.GRO])
def test_direction_programs_orient_before_relabelling(order):
    # the pipeline's CSR is the direction program's output relabelled by the ordering
    g = atc.rmat_graph(12, 16, 7)
    csr = atc.pretc(g, atc.Dir.ADIRECTION, order, want_perm=True)
    off, cols = csr.to_host()
    src = np.repeat(np.arange(off.size - 1), np.diff(off)).astype(np.int32)
    got = np.stack([src, cols], 1)
    lp = oracle.adirection(g)
    rel = csr.perm[lp]
    want = rel[np.lexsort((rel[:, 1], rel[:, 0]))]
    assert np.array_equal(got, want)


def test_aorder_perm_in_pipeline_matches_reference_program():
    # pipeline A-order = the A-order program run on A-direction-seri's output
    g = atc.rmat_graph(12, 16, 7)
    csr = atc.pretc(g, atc.Dir.DEGREE, atc.Order.AORDER, want_perm=True)
    lookup, _, _ = oracle.aorder(oracle.adirection(g))
    assert np.array_equal(csr.perm[: lookup.size], lookup)
    assert np.array_equal(csr.perm[lookup.size:], np.arange(lookup.size, csr.perm.size))


# ---- k-cliques --------------------------------------------------------------------------------
@pytest.mark.parametrize("k", [3, 4, 5, 6, 7])
def test_kcl_matches_oracle(k):
    g = atc.rmat_graph(10, 16, 1)
    want = oracle.kclique(g, k)
    for d in (atc.Dir.ADIRECTION, atc.Dir.DEGREE, atc.Dir.ID):
        csr = atc.pretc(g, d)
        assert atc.kcl(csr, k)[0] == want, (d.name, k)


def test_kcl_complete_graphs():
    for n in (5, 9, 17, 40):
        kn = np.array([(a, b) for a in range(n) for b in range(n) if a != b], dtype=np.int32)
        csr = atc.pretc(kn, atc.Dir.ADIRECTION)
        for k in range(3, 9):
            assert atc.kcl(csr, k)[0] == comb(n, k), (n, k)


def test_kcl_dense_candidate_sets():
    # C0 = N+(u) ∩ N+(v) above 64 members: the CTA-per-edge bitmap path
    for n, ks in ((100, range(3, 9)), (300, range(3, 6))):
        kn = np.array([(a, b) for a in range(n) for b in range(n) if a != b], dtype=np.int32)
        csr = atc.pretc(kn, atc.Dir.DEGREE)
        for k in ks:
            assert atc.kcl(csr, k)[0] == comb(n, k), (n, k)
    g = atc.rmat_graph(12, 32, 8)
    for k in (4, 5, 6):
        want = oracle.kclique(g, k)
        for d in (atc.Dir.ID, atc.Dir.ADIRECTION):
            csr = atc.pretc(g, d)
            assert csr.max_outdeg > 64
            assert atc.kcl(csr, k)[0] == want, (d.name, k)


def test_kcl_three_equals_triangles():
    g = atc.rmat_graph(13, 16, 2)
    csr = atc.pretc(g, atc.Dir.ADIRECTION)
    assert atc.kcl(csr, 3)[0] == atc.tc(csr, atc.Kernel.AUTO)[0] == oracle.tc_count(g)


# ---- edge cases --------------------------------------------------------------------------------
def test_empty_and_degenerate_inputs():
    empty = np.zeros((0, 2), dtype=np.int32)
    for k in KERNELS:
        csr = atc.pretc(empty, atc.Dir.DEGREE)
        assert csr.n == 0 and csr.m == 0
        assert atc.tc(csr, k)[0] == 0
    loops = np.array([[3, 3], [7, 7]], dtype=np.int32)
    csr = atc.pretc(loops, atc.Dir.ADIRECTION)
    assert csr.m == 0 and csr.n == 8 and atc.tc(csr)[0] == 0
    one = np.array([[0, 1]], dtype=np.int32)
    for d in DIRS:
        csr = atc.pretc(one, d)
        assert csr.m == 1 and atc.tc(csr)[0] == 0
    tri_sparse = np.array([[5, 2_000_000], [2_000_000, 77], [77, 5]], dtype=np.int32)
    for d in DIRS:
        for k in KERNELS:
            assert atc.tc(atc.pretc(tri_sparse, d), k)[0] == 1


def test_negative_id_rejected():
    with pytest.raises(atc.ATCError) as ei:
        atc.pretc(np.array([[0, 1], [-4, 2]], dtype=np.int32))
    assert ei.value.status == atc.Status.ERR_INVALID


def test_duplicates_and_reverse_pairs_counted_once():
    tri = np.array([[0, 1], [1, 2], [2, 0]], dtype=np.int32)
    noisy = np.concatenate([tri, tri[:, ::-1], tri, [[1, 1]]]).astype(np.int32)
    for d in DIRS:
        for k in KERNELS:
            assert atc.tc(atc.pretc(noisy, d), k)[0] == 1


def test_hub_heavy_graph():
    # a star of 3000 leaves plus a clique among 60 of them: long lists on both sides
    hub = [(0, i) for i in range(1, 3001)]
    cl = [(a, b) for a in range(1, 61) for b in range(a + 1, 61)]
    g = np.array(hub + cl, dtype=np.int32)
    want = oracle.tc_count(g)
    assert want == comb(60, 2) + comb(60, 3)
    for d in DIRS:
        csr = atc.pretc(g, d)
        for k in KERNELS:
            assert atc.tc(csr, k)[0] == want, (d.name, k.name)
        for t in ({"bisson_cutover": 1},):
            assert atc.tc(csr, atc.Kernel.BISSON, tuning=t)[0] == want


def test_device_generator_matches_host():
    import torch
    n = 16 << 12
    buf = torch.empty((n, 2), dtype=torch.int32, device="cuda")
    rc = atc.lib().atc_gen_rmat_device(12, 16, 570000, 190000, 190000, 5, buf.data_ptr(), None)
    assert rc == 0
    assert np.array_equal(buf.cpu().numpy(), atc.gen_rmat(12, 16, 5))


def test_pretc_device_input_matches_host_input():
    import torch
    g = atc.rmat_graph(11, 16, 4)
    d = torch.from_numpy(g).cuda()
    c1 = atc.pretc_device(d.data_ptr(), g.shape[0], atc.Dir.ADIRECTION)
    c2 = atc.pretc(g, atc.Dir.ADIRECTION)
    o1, k1 = c1.to_host()
    o2, k2 = c2.to_host()
    assert np.array_equal(o1, o2) and np.array_equal(k1, k2)


def test_rmat_s16_config_counts(golden):
    # the reference's CPU-runnable configuration: R-MAT s16 ef16, A-direction, Hu-style
    c = golden["cases"]["rmat_s16_ef16_seed1"]
    g = golden_input(c)
    csr = atc.pretc(g, atc.Dir.ADIRECTION)
    for k in KERNELS:
        assert atc.tc(csr, k)[0] == c["triangles"]


@pytest.mark.parametrize("scale", [18, 20])
def test_larger_graphs_all_kernels_agree_with_oracle(scale):
    g = atc.rmat_graph(scale, 16, 11)
    want = oracle.tc_count(g)
    for d, o in ((atc.Dir.ADIRECTION, atc.Order.AORDER), (atc.Dir.DEGREE, atc.Order.NONE), (atc.Dir.ID, atc.Order.NONE)):
        csr = atc.pretc(g, d, o)
        for k in KERNELS:
            assert atc.tc(csr, k)[0] == want, (scale, d.name, k.name)


def test_cli_dropins(tmp_path):
    import os
    import subprocess
    g = atc.rmat_graph(10, 16, 1)
    want = oracle.tc_count(g)
    e = tmp_path / "E.bin"
    g.tofile(e)
    u64 = (g[:, 0].astype(np.uint64) << np.uint64(32)) | g[:, 1].astype(np.uint32).astype(np.uint64)
    (tmp_path / "E.u64").write_bytes(u64.tobytes())
    bindir = os.path.join(os.path.dirname(atc.LIB_PATH), "bin")
    line = "There are %d triangles in the input graph." % want
    for cmd in (["tc_hu", "-f", str(e)], ["tc_bisson", "-f", str(e), "0"], ["tc_fox", "-f", str(e), "1"],
                ["tric_gpu", "-f", str(tmp_path / "E.u64")]):
        r = subprocess.run([os.path.join(bindir, cmd[0])] + cmd[1:], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert line in r.stdout
    r = subprocess.run([os.path.join(bindir, "a_direction_seri"), str(e)], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lp = np.fromfile(tmp_path / "lpBasedGraph.bin", dtype=np.int32).reshape(-1, 2)
    assert np.array_equal(lp, oracle.adirection(g))
    bdir = tmp_path / "bisson"
    bdir.mkdir()
    r = subprocess.run([os.path.join(bindir, "bisson_a_direction"), str(e)], cwd=bdir, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(bdir / "lpBasedGraph.bin", dtype=np.int32).reshape(-1, 2),
                          oracle.adirection_bisson(g)[1])
    assert (bdir / "lpBasedGraph").stat().st_size == 0
    r = subprocess.run([os.path.join(bindir, "a_order"), str(tmp_path / "lpBasedGraph.bin")], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, normal, reordered = oracle.aorder(lp)
    assert np.array_equal(np.fromfile(tmp_path / "reordered", dtype=np.int32).reshape(-1, 2), reordered)
    r = subprocess.run([os.path.join(bindir, "a_order_v2"), str(tmp_path / "lpBasedGraph.bin")], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(tmp_path / "naive", dtype=np.int32).reshape(-1, 2), oracle.relabel(lp, 1)[2])
    # the shuffled relabellings: relabel-naive, relabel4lpOut (text input), relabel-random
    def pairs_file(name):
        return np.fromfile(tmp_path / name, dtype=np.int32).reshape(-1, 2)
    r = subprocess.run([os.path.join(bindir, "relabel_naive"), str(tmp_path / "lpBasedGraph.bin")], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(pairs_file("naive"), oracle.relabel(lp, 5)[2])
    assert np.array_equal(pairs_file("degreeOrder"), oracle.relabel(lp, 0)[2])
    rt = np.bincount(oracle.relabel(lp, 0)[1][:, 0], minlength=int(lp.max()) + 1)
    assert "the max runtime degree is %d" % rt.max() in r.stdout
    r = subprocess.run([os.path.join(bindir, "relabel4lp_out"), str(tmp_path / "lpBasedGraph")], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(pairs_file("normal"), lp)
    assert np.array_equal(pairs_file("bad"), oracle.relabel(lp, 6)[2])
    assert np.array_equal(pairs_file("good"), oracle.relabel(lp, 2)[2])
    r = subprocess.run([os.path.join(bindir, "relabel_random"), str(tmp_path / "lpBasedGraph.bin")], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lookup7, normal7, bad7 = oracle.relabel(lp, 7)
    assert np.array_equal(pairs_file("normal"), normal7) and np.array_equal(pairs_file("bad"), bad7)
    assert np.array_equal(pairs_file("good"), oracle.relabel(lp, 0)[2])
    at = np.argsort(lookup7)  # the vertex at each position of the shuffle
    assert r.stdout.split("\n")[1:at.size] == [str(x) for x in rt[at[:-1]]]
    r = subprocess.run([os.path.join(bindir, "kcl"), str(e), "-k=4"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "total_num_cliques = %d" % oracle.kclique(g, 4) in r.stdout
    r = subprocess.run([os.path.join(bindir, "Peel"), str(tmp_path / "E.u64"), str(tmp_path / "P.u64")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(tmp_path / "P.u64", dtype=np.uint64), oracle.adirection_par(u64)[0])
    r = subprocess.run([os.path.join(bindir, "kcore_direction"), str(tmp_path / "E.u64"), str(tmp_path / "K.u64")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(tmp_path / "K.u64", dtype=np.uint64), atc.kcore_direction(u64))
    # other_order's reorder (GRO): <name>_GRO_newID.txt and the sorted, relabelled edges
    r = subprocess.run([os.path.join(bindir, "reorder"), str(tmp_path / "E.u64")], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ids = np.loadtxt(tmp_path / "E_GRO_newID.txt", dtype=np.int64, ndmin=2)
    e = np.fromfile(tmp_path / "E.u64", dtype=np.uint64)
    directed = np.stack([(e >> np.uint64(32)).astype(np.int32), (e & np.uint64(0xffffffff)).astype(np.int32)], 1)
    onew, _ = oracle.gro(e)
    assert np.array_equal(ids[:, 0], np.arange(onew.size)) and np.array_equal(ids[:, 1], onew)
    srt = directed[np.lexsort((directed[:, 1], directed[:, 0]))]
    assert np.array_equal(np.loadtxt(tmp_path / "E_GRO.txt", dtype=np.int64, ndmin=2), onew[srt])
    n = int(g.max()) + 1
    adj = [[] for _ in range(n)]
    for u, v in g:
        adj[u].append(int(v))
    for version in (1, 2):
        gr = tmp_path / ("G%d.gr" % version)
        write_gr(gr, n, adj, version)
        r = subprocess.run([os.path.join(bindir, "kcl"), "-symmetricGraph", "-simpleGraph", str(gr), "-k=5"],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert "total_num_cliques = %d" % oracle.kclique(g, 5) in r.stdout


@pytest.mark.parametrize("d", [atc.Dir.ADIRECTION, atc.Dir.DEGREE])
def test_csr_save_load_round_trip(tmp_path, d):
    g = atc.rmat_graph(12, 16, 5)
    csr = atc.pretc(g, d, tuning={"prune_deg1": 1 if d == atc.Dir.DEGREE else 0})
    path = tmp_path / "g.csr"
    csr.save(path)
    back = atc.CSR.load(path)
    a, b = csr.to_host(), back.to_host()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    for f in ("n", "m", "n_input", "wedges", "wedges_min", "max_outdeg", "dir", "order", "pruned"):
        assert getattr(back._st, f) == getattr(csr._st, f), f
    want = oracle.tc_count(g)
    for k in KERNELS:
        assert atc.tc(back, k)[0] == want
    assert atc.kcl(back, 4)[0] == oracle.kclique(g, 4)
    raw = path.read_bytes()
    bad = tmp_path / "bad.csr"
    bad.write_bytes(raw[:-4])
    with pytest.raises(atc.ATCError):
        atc.CSR.load(bad)


def test_rgg_device_matches_host():
    import ctypes as C
    import torch
    n = 1 << 14
    host = atc.gen_rgg(n, 32.0, 3)
    cnt = C.c_uint64(0)
    buf = torch.empty((host.shape[0] + 100, 2), dtype=torch.int32, device="cuda")
    assert atc.lib().atc_gen_rgg_device(n, 32.0, 3, buf.data_ptr(), buf.shape[0], C.byref(cnt), None) == 0
    dev = buf[: cnt.value].cpu().numpy()
    order = np.lexsort((dev[:, 1], dev[:, 0]))
    assert np.array_equal(dev[order], host)


@pytest.mark.parametrize("k", [3, 4, 5, 6, 7])
def test_kcl_rgg_matches_oracle(k):
    g = atc.gen_rgg(1 << 14, 32.0, 2)
    csr = atc.pretc(g, atc.Dir.ADIRECTION)
    assert atc.kcl(csr, k)[0] == oracle.kclique(g, k)


# ---- batched counting ---------------------------------------------------------------------------
def _batch_graphs():
    import torch
    gs = [atc.rmat_graph(10, 16, 1), atc.gen_rgg(3000, 20.0, 4), np.zeros((0, 2), dtype=np.int32),
          np.array([(a, b) for a in range(4) for b in range(4) if a != b], dtype=np.int32),
          atc.rmat_graph(12, 8, 2)]
    for n, gamma, d, seed in ((2000, 2.1, 16.0, 1), (50000, 2.5, 40.0, 2), (300, 3.0, 8.0, 3)):
        gs.append(atc.gen_chunglu_device(n, gamma, d, seed).cpu().numpy())
    hub = [(0, i) for i in range(1, 3001)] + [(a, b) for a in range(1, 61) for b in range(a + 1, 61)]
    gs.append(np.array(hub, dtype=np.int32))
    return gs


def test_batch_counts_match_per_graph():
    gs = _batch_graphs()
    want = [oracle.tc_count(g) if g.size else 0 for g in gs]
    b = atc.Batch()
    for i, g in enumerate(gs):
        d = (atc.Dir.ADIRECTION, atc.Dir.DEGREE, atc.Dir.ID)[i % 3]
        assert b.add(atc.pretc(g, d)) == i
    counts, st = b.run()
    assert counts.tolist() == want
    counts2, _ = b.run()  # a second replay of the same captured graph
    assert counts2.tolist() == want
    for t in ({"bisson_cutover": 8, "bisson_warp_max": 64}, {"bisson_warp_chunk": 32, "bisson_block_chunk": 64},
              {"bisson_warp_max": 256, "bisson_cutover": 256}, {"bisson_warp_max": 512}, {"group_by_source": 1},
              {"group_by_source": 1, "bisson_warp_max": 512},
              {"group_by_source": 1, "bisson_warp_max": 64, "bisson_warp_chunk": 32}, {"group_by_source": 2},
              {"group_by_source": 2, "bisson_warp_max": 64, "bisson_warp_chunk": 32}):
        assert b.run(tuning=t)[0].tolist() == want, t
    best, ms = b.tune([{}, {"bisson_warp_max": 128}, {"bisson_block_chunk": 256}])
    assert 0 <= best < 3 and np.all(ms > 0)
    assert b.run()[0].tolist() == want
    # graphs added after a run rebuild the pipeline
    extra = atc.rmat_graph(11, 16, 9)
    b.add(atc.pretc(extra, atc.Dir.DEGREE))
    assert b.run()[0].tolist() == want + [oracle.tc_count(extra)]


def _hub_path(k, step):
    """Vertex 0 joined to k vertices step, 2*step, ..., which form a path: k - 1 triangles."""
    leaves = [step * i for i in range(1, k + 1)]
    e = [(0, x) for x in leaves] + list(zip(leaves[:-1], leaves[1:]))
    return np.array(e, dtype=np.int32)


def test_batch_long_lists():
    """Oriented lists longer than the batch's 32 KB tables: hashed (3000), bitmap (5000) and
    searched in global memory (4200 over a span of 546 000), in the grouped and the rows items."""
    gs = [_hub_path(3000, 1), _hub_path(5000, 1), _hub_path(4200, 130), atc.rmat_graph(10, 16, 1)]
    want = [oracle.tc_count(g) for g in gs]
    assert want[:3] == [2999, 4999, 4199]
    b = atc.Batch()
    for g in gs:
        b.add(atc.pretc(g, atc.Dir.ID))
    for t in (None, {"group_by_source": 1}, {"group_by_source": 2}, {"bisson_block_chunk": 64},
              {"group_by_source": 1, "bisson_block_chunk": 64}):
        assert b.run(tuning=t)[0].tolist() == want, t
    b.free()


def test_batch_reserve_and_empty():
    b = atc.Batch()
    assert b.run()[0].tolist() == []
    b.reserve(10000, 100000)
    g = atc.rmat_graph(9, 8, 3)
    b.add(atc.pretc(g, atc.Dir.DEGREE))
    assert b.run()[0].tolist() == [oracle.tc_count(g)]


def test_chunglu_generator_shape():
    g = atc.gen_chunglu_device(100000, 2.5, 20.0, 7).cpu().numpy()
    assert np.all(g[:, 0] < g[:, 1]) and g.min() >= 0 and g.max() < 100000
    mean_deg = 2 * g.shape[0] / 100000
    assert 12.0 < mean_deg < 24.0, mean_deg
    g2 = atc.gen_chunglu_device(100000, 2.5, 20.0, 7).cpu().numpy()
    assert np.array_equal(g, g2)


def test_kcore_orientation_matches_oracle_core_numbers():
    g = atc.rmat_graph(12, 16, 4)
    core = oracle.core_numbers(g)
    off, cols = atc.pretc(g, atc.Dir.KCORE).to_host()
    src = np.repeat(np.arange(off.size - 1), np.diff(off))
    cs, cd = core[src], core[cols]
    assert np.all((cs < cd) | ((cs == cd) & (src < cols)))
    assert off[-1] == oracle.simple_stats(g)[1]


def test_kcore_direction_program_matches_oracle():
    """kcore_direction.cpp:133-141 on a simple edge list given once per undirected edge."""
    rng = np.random.default_rng(11)
    for g in (atc.simplify(atc.gen_rmat(11, 8, 3), symmetric=False),
              atc.simplify(rng.integers(0, 300, size=(3000, 2)).astype(np.int32), symmetric=False)):
        g = g[rng.permutation(g.shape[0])]
        flip = rng.random(g.shape[0]) < 0.5
        g[flip] = g[flip][:, ::-1]                        # either endpoint first
        packed = (g[:, 0].astype(np.uint64) << np.uint64(32)) | g[:, 1].astype(np.uint64)
        out, core = atc.kcore_direction(packed, want_core=True)
        want_core = oracle.core_numbers(g)
        assert np.array_equal(core, want_core)
        src = (out >> np.uint64(32)).astype(np.int64)
        dst = (out & np.uint64(0xFFFFFFFF)).astype(np.int64)
        a, b = g[:, 0].astype(np.int64), g[:, 1].astype(np.int64)
        swap = (want_core[a] > want_core[b]) | ((want_core[a] == want_core[b]) & (a > b))
        assert np.array_equal(src, np.where(swap, b, a)) and np.array_equal(dst, np.where(swap, a, b))
    assert atc.kcore_direction(np.zeros(0, dtype=np.uint64)).size == 0


sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from apeel_cases import apeel_graphs as _apeel_graphs, packed as _packed  # noqa: E402


@pytest.mark.parametrize("compat", [False, True])
def test_adirection_par_matches_oracle(compat):
    """peel.cu:130-317 bit-exact: flags, minor priorities, iterations and the output file."""
    for name, g in _apeel_graphs():
        e = _packed(g)
        got = atc.adirection_par(e, compat=compat)
        want = oracle.adirection_par(e, compat=compat)
        assert np.array_equal(got[1], want[1]), name
        assert np.array_equal(got[2], want[2]), name
        assert got[3] == want[3], name
        assert np.array_equal(got[0], want[0]), name


PEEL_GOLDEN = os.path.join(ROOT, "tests", "golden", "peel_par.json")


@pytest.mark.skipif(not os.path.exists(PEEL_GOLDEN), reason="no recorded output of the Peel program")
def test_adirection_par_matches_the_peel_program():
    """The Peel drop-in (compat comparison, peel.cu:49) against the output file the reference
    program itself wrote on the same inputs (recorded on a GB300 by make_peel_golden.py)."""
    with open(PEEL_GOLDEN) as f:
        rec = json.load(f)["cases"]
    for name, g in _apeel_graphs():
        e = _packed(g)
        assert hashlib.sha256(e.tobytes()).hexdigest() == rec[name]["input"]["sha256"], name
        got = atc.adirection_par(e, compat=True)[0]
        assert hashlib.sha256(np.ascontiguousarray(got).tobytes()).hexdigest() == rec[name]["peel_out"]["sha256"], name


def test_adirection_par_direction_in_pretc():
    for name, g in _apeel_graphs():
        _, flags, minor, _ = oracle.adirection_par(_packed(g))
        off, cols = atc.pretc(g, atc.Dir.ADIRECTION_PAR).to_host()
        src = np.repeat(np.arange(off.size - 1), np.diff(off))
        fs, fd = flags.view(np.int32)[src], flags.view(np.int32)[cols]
        ms, md = minor.astype(np.int64)[src], minor.astype(np.int64)[cols]
        assert np.all((fs < fd) | ((fs == fd) & ((ms < md) | ((ms == md) & (src < cols))))), name
        assert off[-1] == oracle.simple_stats(g)[1], name
        want = oracle.tc_count(g)
        for k in KERNELS:
            assert atc.tc(atc.pretc(g, atc.Dir.ADIRECTION_PAR), k)[0] == want, (name, k.name)
