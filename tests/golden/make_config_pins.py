"""Regenerates tests/golden/config_pins.json: reference outputs and oracle counts at the
benchmark configurations' full sizes.

Runs only where the reference tree exists (the reference programs are compiled from their
unmodified sources by `make -C oracle ref` into oracle/_ref/).  Records:

  rmat24   R-MAT scale 24, edge factor 16, (a,b,c) = (.57,.19,.19), seed 1, symmetrised and
           simplified (the headline graph):
             adirection   A-direction-seri E.bin -> lpBasedGraph.bin (count, sha256)
             aorder       A-order lpBasedGraph.bin -> normal, reordered (sha256 each)
             csr_edges    the A-direction edges relabelled by the A-order permutation and
                          sorted by (src, dst): the edge list of the oriented CSR that
                          A-direction + A-order hand to the counting kernels (sha256).  The
                          permutation is read off the program's two outputs, which list the
                          same edges in the same order before (normal) and after (reordered)
                          relabelling; A-order's own files are degree-oriented, the counted
                          CSR keeps the A-direction orientation (all priorities distinct)
             wedges, wedges_min  W = sum_v indeg(v) outdeg(v) and sum over edges of
                          min(outdeg u, outdeg v) of that orientation
             triangles    the oracle's uint64 count (OrgTriangleCount's scalar merge,
                          other_order/set_operation.cpp:129-144, all host threads); the
                          reference's own counter returns int and overflows here
           The oracle's A-direction and A-order restatements are checked against the
           programs' outputs at this size before anything is written.
  kcl      k-clique counts of the oracle (k-clique/kcl.cu:147-215 semantics): the 2-D RGG
           with n = 2^20 and mean degree 32 (seed 1) at k = 4..7, and R-MAT scale 20 edge
           factor 16 (seed 1) at k = 4.

Usage: python tests/golden/make_config_pins.py [--skip-rmat24] [--skip-kcl]
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "accelerating-tc_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import atc  # noqa: E402
import oracle  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
OUT = os.path.join(HERE, "config_pins.json")


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


def read_pairs(path):
    return np.fromfile(path, dtype=np.int32).reshape(-1, 2)


def sorted_pairs(p):
    """Pairs sorted by (src, dst) (ids are non-negative int32)."""
    key = (p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64)
    key.sort()
    out = np.empty_like(p)
    out[:, 0] = (key >> np.uint64(32)).astype(np.int32)
    out[:, 1] = (key & np.uint64(0xFFFFFFFF)).astype(np.int32)
    return out


def wedge_stats(lp, n):
    """W and sum over edges of min(outdeg u, outdeg v) of the oriented pairs."""
    outd = np.bincount(lp[:, 0], minlength=n).astype(np.int64)
    ind = np.bincount(lp[:, 1], minlength=n).astype(np.int64)
    w = int(np.dot(ind, outd))
    wmin = int(np.minimum(outd[lp[:, 0]], outd[lp[:, 1]]).sum())
    return w, wmin


def run(args, cwd, timeout=7200):
    t0 = time.time()
    r = subprocess.run(args, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout[-2000:]
    print("  %s: %.1f s" % (os.path.basename(args[0]), time.time() - t0), flush=True)
    return r


def rmat24():
    scale, ef, seed = 24, 16, 1
    t0 = time.time()
    g = atc.rmat_graph(scale, ef, seed, symmetric=True)
    print("graph %d pairs, %.1f s" % (g.shape[0], time.time() - t0), flush=True)
    rec = {"source": {"kind": "rmat", "scale": scale, "edge_factor": ef, "seed": seed,
                      "abc_ppm": list(atc.GRAPH500), "symmetric": True},
           "input": {"count": int(g.shape[0]), "sha256": sha(g)}}
    with tempfile.TemporaryDirectory(dir=os.environ.get("ATC_PIN_TMP")) as d:
        e = os.path.join(d, "E.bin")
        g.tofile(e)
        run([os.path.join(REF, "A-direction-seri"), e], d)
        lp = read_pairs(os.path.join(d, "lpBasedGraph.bin"))
        rec["adirection"] = {"count": int(lp.shape[0]), "sha256": sha(lp)}
        olp = oracle.adirection(g)
        assert olp.shape == lp.shape and sha(olp) == rec["adirection"]["sha256"], "oracle A-direction differs"
        del olp
        os.remove(os.path.join(d, "lpBasedGraph"))  # the text copy is not needed
        run([os.path.join(REF, "A-order"), os.path.join(d, "lpBasedGraph.bin")], d)
        normal = read_pairs(os.path.join(d, "normal"))
        reordered = read_pairs(os.path.join(d, "reordered"))
        rec["aorder"] = {"normal": {"count": int(normal.shape[0]), "sha256": sha(normal)},
                         "reordered": {"count": int(reordered.shape[0]), "sha256": sha(reordered)}}
        _, onormal, oreord = oracle.aorder(lp)
        assert sha(onormal) == rec["aorder"]["normal"]["sha256"], "oracle A-order (normal) differs"
        assert sha(oreord) == rec["aorder"]["reordered"]["sha256"], "oracle A-order (reordered) differs"
        del onormal, oreord
    n = int(g.max()) + 1
    lookup = np.full(n, -1, dtype=np.int64)
    lookup[normal[:, 0]] = reordered[:, 0]
    lookup[normal[:, 1]] = reordered[:, 1]
    assert np.array_equal(lookup[normal], reordered), "normal -> reordered is not a relabelling"
    del normal
    csr_edges = sorted_pairs(lookup[lp].astype(np.int32))
    rec["csr_edges"] = {"count": int(csr_edges.shape[0]), "sha256": sha(csr_edges)}
    rec["n"] = n
    w, wmin = wedge_stats(csr_edges, n)
    rec["wedges"], rec["wedges_min"] = w, wmin
    del csr_edges, reordered, lp
    t0 = time.time()
    rec["triangles"] = int(oracle.tc_count(g))
    print("  oracle count %d: %.1f s" % (rec["triangles"], time.time() - t0), flush=True)
    return rec


def kcl_pins():
    out = {}
    t0 = time.time()
    rgg = atc.gen_rgg(1 << 20, 32.0, 1)
    print("rgg %d edges, %.1f s" % (rgg.shape[0], time.time() - t0), flush=True)
    out["rgg20"] = {"source": {"kind": "rgg", "n": 1 << 20, "mean_degree": 32.0, "seed": 1},
                    "input": {"count": int(rgg.shape[0]), "sha256": sha(rgg)}, "cliques": {}}
    for k in range(4, 8):
        t0 = time.time()
        out["rgg20"]["cliques"][str(k)] = int(oracle.kclique(rgg, k))
        print("  rgg k=%d %d: %.1f s" % (k, out["rgg20"]["cliques"][str(k)], time.time() - t0), flush=True)
    g = atc.rmat_graph(20, 16, 1, symmetric=True)
    out["rmat20"] = {"source": {"kind": "rmat", "scale": 20, "edge_factor": 16, "seed": 1,
                                "abc_ppm": list(atc.GRAPH500), "symmetric": True},
                     "input": {"count": int(g.shape[0]), "sha256": sha(g)}, "cliques": {}}
    for k in (3, 4):
        t0 = time.time()
        out["rmat20"]["cliques"][str(k)] = int(oracle.kclique(g, k))
        print("  rmat20 k=%d %d: %.1f s" % (k, out["rmat20"]["cliques"][str(k)], time.time() - t0), flush=True)
    return out


def main():
    pins = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            pins = json.load(f)
    if "--skip-rmat24" not in sys.argv:
        assert os.path.exists(os.path.join(REF, "A-direction-seri")), "run `make -C oracle ref` first"
        pins["rmat24"] = rmat24()
    if "--skip-kcl" not in sys.argv:
        pins["kcl"] = kcl_pins()
    pins["meta"] = {"generated_by": "tests/golden/make_config_pins.py", "host_machine": os.uname().machine,
                    "oracle_threads": oracle.nthreads_default()}
    with open(OUT, "w") as f:
        json.dump(pins, f, indent=1, sort_keys=True)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
