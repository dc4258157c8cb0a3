"""The CPU oracle against the reference programs' own outputs (tests/golden).

These pin the restatement in oracle/atc_oracle.cpp: A-direction orientation and A-order
permutation byte for byte, costFuncCal / verification figures as the tools print them,
and the OrgTriangleCount triangle counts.
"""
import hashlib
import os

import numpy as np
import pytest

import oracle
from conftest import golden_input, load_golden

CASES = sorted(load_golden()["cases"])


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


def fmt6(x):
    """C++ ostream default formatting (%g, 6 significant digits)."""
    s = "%g" % np.float32(x)
    return s


def check_pairs(got, rec):
    assert got.shape[0] == rec["count"]
    assert sha(got) == rec["sha256"]


@pytest.mark.parametrize("name", CASES)
def test_input_bytes(golden, name):
    c = golden["cases"][name]
    check_pairs(golden_input(c), c["input"])


@pytest.mark.parametrize("name", CASES)
def test_adirection(golden, name):
    c = golden["cases"][name]
    check_pairs(oracle.adirection(golden_input(c)), c["adirection"])


@pytest.mark.parametrize("name", CASES)
def test_adirection_bisson(golden, name):
    # Bisson/A-direction.cpp's lpBasedGraph.bin, position-indexed degreeRecord included
    c = golden["cases"][name]
    lookup, out = oracle.adirection_bisson(golden_input(c))
    check_pairs(out, c["bisson_adir"])
    assert np.array_equal(np.sort(lookup), np.arange(lookup.size))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("which", ["aorder", "aorder_raw"])
def test_aorder(golden, name, which):
    c = golden["cases"][name]
    g = golden_input(c)
    src = oracle.adirection(g) if which == "aorder" else g
    rec = c[which]
    res = oracle.aorder(src)
    if rec.get("unsupported"):
        assert res is None
        assert rec["ref_returncode"] != 0  # the reference crashed on it
        return
    assert res is not None
    lookup, normal, reordered = res
    check_pairs(normal, rec["normal"])
    check_pairs(reordered, rec["reordered"])
    assert np.array_equal(np.sort(lookup), np.arange(lookup.size))  # a permutation


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("which,kind", [("aorder_v2", 1), ("relabel_good", 0), ("relabel4lp", 2), ("relabel_naive", 5),
                                        ("relabel4lp_bad", 6), ("relabel_random", 7)])
def test_relabel(golden, name, which, kind):
    """A-order-v2 "naive", relabel-naive "degreeOrder" and "naive", relabel4lpOut "good" and
    "bad", relabel-random "bad" on lpBasedGraph."""
    c = golden["cases"][name]
    lookup, normal, rel = oracle.relabel(oracle.adirection(golden_input(c)), kind)
    check_pairs(rel, c[which])
    assert np.array_equal(np.sort(lookup), np.arange(lookup.size))


def pack_u64(pairs):
    pairs = np.asarray(pairs, dtype=np.int32).reshape(-1, 2)
    return (pairs[:, 0].astype(np.uint64) << np.uint64(32)) | pairs[:, 1].astype(np.uint32).astype(np.uint64)


def check_ids(got, rec):
    got = np.ascontiguousarray(got, dtype=np.int32)
    assert got.size == rec["count"]
    if "ids" in rec:
        assert got.tolist() == rec["ids"]
    assert hashlib.sha256(got.tobytes()).hexdigest() == rec["sha256"]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("which", ["gro_sym", "gro_lp"])
def test_gro(golden, name, which):
    """other_order's GRO order (reorder program, _GRO_newID.txt) on the symmetrised input and on
    the A-direction output, where the program's output is defined (max gain < vertex count)."""
    c = golden["cases"][name]
    rec = c.get(which)
    if rec is None or rec.get("unsupported"):
        pytest.skip("no GRO fixture for this case")
    g = golden_input(c)
    import atc
    src = atc.simplify(g, symmetric=True) if which == "gro_sym" else oracle.adirection(g)
    new_id, max_gain = oracle.gro(pack_u64(src))
    assert max_gain < new_id.size
    check_ids(new_id, rec)
    assert np.array_equal(np.sort(new_id), np.arange(new_id.size))


@pytest.mark.parametrize("name", CASES)
def test_costfunc(golden, name):
    c = golden["cases"][name]
    lp = oracle.adirection(golden_input(c))
    for k, printed in c["costfunc"].items():
        got = oracle.costfunc(lp, int(k))
        assert [fmt6(x) for x in got] == printed


@pytest.mark.parametrize("name", CASES)
def test_verification(golden, name):
    c = golden["cases"][name]
    lp = oracle.adirection(golden_input(c))
    got = oracle.verification(lp)
    assert [fmt6(x) for x in got] == c["verification"]


@pytest.mark.parametrize("name", CASES)
def test_triangles(golden, name):
    c = golden["cases"][name]
    if "triangles" not in c:
        pytest.skip("fixture made without the x86-only OrgTriangleCount")
    assert oracle.tc_count(golden_input(c)) == c["triangles"]


def test_kclique_identities():
    # K_n has C(n,k) k-cliques; k=3 equals the triangle count.
    from math import comb
    for n in (5, 7, 9):
        kn = np.array([(a, b) for a in range(n) for b in range(n) if a != b], dtype=np.int32)
        for k in range(3, 8):
            assert oracle.kclique(kn, k) == comb(n, k)
    import atc
    g = atc.rmat_graph(10, 16, 1)
    assert oracle.kclique(g, 3) == oracle.tc_count(g)


def test_kclique_oracle_matches_networkx():
    # the oracle's DFS against an independent clique enumeration, k = 4..6
    nx = pytest.importorskip("networkx")
    import atc
    rng = np.random.default_rng(11)
    graphs = [atc.rmat_graph(9, 8, 3), atc.rmat_graph(8, 16, 4)]
    er = rng.integers(0, 120, size=(1500, 2)).astype(np.int32)
    graphs.append(atc.simplify(er, symmetric=True))
    for g in graphs:
        G = nx.Graph()
        G.add_edges_from(map(tuple, g.tolist()))
        G.remove_edges_from(nx.selfloop_edges(G))
        want = {}
        for cl in nx.enumerate_all_cliques(G):
            if len(cl) > 6:
                break
            want[len(cl)] = want.get(len(cl), 0) + 1
        for k in (4, 5, 6):
            assert oracle.kclique(g, k) == want.get(k, 0), k


def test_hu_csr_matches_reference_rules():
    # Hu's preTC CSR on a once-per-edge list: every vertex of degree >= 2 kept, lists
    # oriented low degree -> high degree (ties: larger id is the source), sorted.
    import atc
    g = atc.rmat_graph(8, 8, 2, symmetric=False)
    off, cols = oracle.hu_csr(g)
    assert off[-1] == cols.size
    for u in range(off.size - 1):
        lst = cols[off[u]:off[u + 1]]
        assert np.all(np.diff(lst) > 0)
    # orientation preserves the triangle count
    oriented = np.stack([np.repeat(np.arange(off.size - 1), np.diff(off)), cols], 1)
    assert oracle.tc_count(oriented) == oracle.tc_count(g)


def test_oracle_mlp_gradient_by_finite_differences():
    # pins the oracle's backward pass (the checker of the GPU training kernels)
    rng = np.random.default_rng(0)
    I, H, O, B = 3, 5, 4, 7
    npar = I * H + H + H * H + H + H * O + O
    p = rng.normal(size=npar).astype(np.float32) * 0.5
    x = rng.normal(size=(B, I)).astype(np.float32)
    t = rng.normal(size=(B, O)).astype(np.float32)
    mean = np.zeros(I, np.float32)
    std = np.ones(I, np.float32)
    _, g = oracle.mlp_grad(p, I, H, O, mean, std, x, t)
    h = 1e-3
    for k in range(0, npar, 7):
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        lp, _ = oracle.mlp_grad(pp, I, H, O, mean, std, x, t)
        lm, _ = oracle.mlp_grad(pm, I, H, O, mean, std, x, t)
        num = (lp - lm) / (2 * h)
        assert abs(num - g[k]) < 2e-3 * max(1.0, abs(g[k])), (k, num, g[k])


def test_oracle_core_numbers_match_networkx():
    nx = pytest.importorskip("networkx")
    import atc
    for scale, seed in ((9, 1), (11, 2)):
        g = atc.rmat_graph(scale, 8, seed, symmetric=False)
        G = nx.Graph()
        G.add_nodes_from(range(int(g.max()) + 1))
        G.add_edges_from(map(tuple, g))
        want = nx.core_number(G)
        got = oracle.core_numbers(g)
        assert all(got[v] == want[v] for v in G.nodes)


def _pack(pairs):
    p = np.asarray(pairs, dtype=np.uint64).reshape(-1, 2)
    return (p[:, 0] << np.uint64(32)) | p[:, 1]


def test_oracle_adirection_par_hand_worked():
    """peel.cu:130-317 worked by hand on a star 0-{1,2,3,4} plus edge 1-2: m/n = 1, the
    first frontier is the two leaves {3, 4}; vertex 0 drops to degree 2, the next limit 1
    finds nothing, the depth rises to 2 and {0, 1, 2} join as iteration 2."""
    e = _pack([[0, 1], [0, 2], [0, 3], [0, 4], [1, 2], [3, 0]])
    out, flags, minor, it = oracle.adirection_par(e)
    assert flags.tolist() == [2, 2, 2, 1, 1]
    assert minor.tolist() == [2, 2, 2, 1, 1]
    assert it == 2
    assert out.tolist() == _pack([[0, 1], [0, 2], [3, 0], [4, 0], [1, 2], [3, 0]]).tolist()


def test_oracle_adirection_par_compat_term():
    """The compat comparison uses minor[src] - flag[dst] (peel.cu:49).  A 4-cycle 0-1-2-3
    with chord 0-2: m/n = 1.25 -> limit 1 and no degree is <= 1, so the depth climbs to 2
    and {1, 3} (degree 2) join as iteration 2; 0 and 2 (degree 3, now 1) join as 3."""
    e = _pack([[0, 1], [1, 2], [2, 3], [3, 0], [0, 2], [2, 0]])
    out, flags, minor, it = oracle.adirection_par(e)
    assert flags.tolist() == [3, 2, 3, 2]
    assert minor.tolist() == [1, 2, 1, 2]
    assert it == 3
    # fixed rule: 1 -> 0, 1 -> 2, 3 -> 2, 3 -> 0; 0 and 2 tie on flag and minor, 0 first
    assert out.tolist() == _pack([[1, 0], [1, 2], [3, 2], [3, 0], [0, 2], [0, 2]]).tolist()
    out_c, _, _, _ = oracle.adirection_par(e, compat=True)
    # compat: minor[0] - flag[2] = 1 - 3 < 0 keeps 0 -> 2, and minor[2] - flag[0] < 0 keeps
    # 2 -> 0 as well: the program's rule is not antisymmetric
    assert out_c.tolist() == _pack([[1, 0], [1, 2], [3, 2], [3, 0], [0, 2], [2, 0]]).tolist()


def test_oracle_rmat_generator_equals_libatc():
    # the CPU arm of the benchmark generates its input with the oracle's copy of the generator
    import atc
    for scale, ef, seed in ((6, 4, 3), (10, 16, 1), (14, 8, 9)):
        assert np.array_equal(oracle.gen_rmat(scale, ef, seed, nthreads=3), atc.gen_rmat(scale, ef, seed))


REF_GPU = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_counts.json")


@pytest.mark.skipif(not os.path.exists(REF_GPU), reason="no recorded run of the reference GPU programs")
def test_reference_gpu_programs_count_what_the_oracle_counts(golden):
    """The counts the reference's own GPU programs (Hu, Bisson, Fox, TriCore, built for sm_103a,
    recorded by tests/golden/make_refgpu_golden.py) printed on the benchmark graphs equal the
    oracle's: the golden R-MAT scale 16 count, and the config pins at scales 20 and 24."""
    import json
    with open(REF_GPU) as f:
        rec = json.load(f)["graphs"]
    with open(os.path.join(os.path.dirname(REF_GPU), "config_pins.json")) as f:
        pins = json.load(f)
    want = {"rmat16": golden["cases"]["rmat_s16_ef16_seed1"]["triangles"],
            "rmat20": pins["kcl"]["rmat20"]["cliques"]["3"], "rmat24": pins["rmat24"]["triangles"]}
    seen = 0
    for gname, g in rec.items():
        for pname, p in g["programs"].items():
            if "skipped" in p:
                assert pname == "bisson" and gname == "rmat24"
                continue
            assert p["rc"] == 0 and p["count"] == want[gname], (gname, pname, p)
            seen += 1
    assert seen >= 4


def test_c_library_rand_is_the_published_generator():
    """The shuffled relabellings replay the C library's rand() on the device from its published
    description (an additive lagged-Fibonacci generator of degree 31 and separation 3 seeded
    through 16807 x mod 2^31-1; P. Selinger, "The GLIBC pseudo-random number generator").  The
    host's rand() after srand(1), the state of a program that never seeds it, is that stream."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand(1)
    want = [libc.rand() for _ in range(2000)]
    r = [1]
    for i in range(1, 31):
        r.append(16807 * r[-1] % 2147483647)
    r += r[0:3]
    while len(r) < 344 + 2000:
        r.append((r[-3] + r[-31]) & 0xFFFFFFFF)
    assert [x >> 1 for x in r[344:]] == want
    libc.srand(1)
