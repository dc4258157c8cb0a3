"""Regenerates tests/golden/golden.json from the reference's own CPU programs.

Runs only where the reference tree exists (it is not on the GPU hosts): the programs
are compiled from their unmodified sources by `make -C oracle ref` into oracle/_ref/.
Each case is a seeded input graph produced by libatc's generator (the input bytes'
SHA-256 is recorded so a generator change shows up as a fixture mismatch).  For each
case the script records what the reference programs output:

  adirection   A-direction-seri E.bin        -> lpBasedGraph.bin
  bisson_adir  Bisson/A-direction E.bin      -> lpBasedGraph.bin (both directions, relabelled)
  aorder       A-order lpBasedGraph.bin      -> lookup-free outputs normal / reordered
  aorder_raw   A-order E.bin                 -> normal / reordered on the raw input
  aorder_v2    A-order-v2 lpBasedGraph.bin   -> naive (the 40-column mix, relabelled)
  relabel_good relabel-naive lpBasedGraph.bin -> degreeOrder (descending runtime degree)
  relabel_naive relabel-naive lpBasedGraph.bin -> naive (64 columns, blocks of 64 shuffled)
  relabel4lp   relabel4lpOut lpBasedGraph   -> good (descending out-degree as given; text input)
  relabel4lp_bad relabel4lpOut lpBasedGraph -> bad (40 columns, blocks of 40 shuffled)
  relabel_random relabel-random lpBasedGraph.bin -> bad (every id shuffled)
  costfunc     costFuncCal lpBasedGraph.bin k -> three printed floats, k = 1, 2
  verification verification lpBasedGraph    -> two printed floats (text input)
  triangles    OrgTriangleCount on E symmetrised (x86 only; int result, small graphs)
  gro_sym      other_order reorder (GRO) on E symmetrised, packed uint64 -> _GRO_newID.txt
  gro_lp       the same on the A-direction output (directed edges)
               (x86 only; recorded only where its gain headers stay initialised:
               max gain < vertex count, see orc_gro)

Small outputs are stored in full, larger ones as (count, sha256).

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "accelerating-tc_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import atc  # noqa: E402
import oracle  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
INLINE_MAX = 600  # pairs stored in full up to this size

TINY = {
    "k4_sym": [(a, b) for a in range(4) for b in range(4) if a != b],
    "k6_once": [(a, b) for a in range(6) for b in range(a + 1, 6)],
    "dups_loops": [(0, 1), (1, 0), (1, 2), (2, 0), (2, 2), (3, 4), (4, 3), (3, 4), (0, 3), (5, 5), (1, 3), (3, 2)],
    "star_tri": [(0, i) for i in range(1, 9)] + [(1, 2), (2, 3), (3, 1), (9, 10)],
    "eleven_edges": [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5), (5, 6), (6, 7), (7, 8), (8, 9), (9, 10), (10, 0)],
}
RMAT = [  # (name, scale, edge_factor, seed)
    ("rmat_s6_ef4_seed3", 6, 4, 3),
    ("rmat_s8_ef8_seed2", 8, 8, 2),
    ("rmat_s10_ef16_seed1", 10, 16, 1),
    ("rmat_s12_ef16_seed7", 12, 16, 7),
    ("rmat_s16_ef16_seed1", 16, 16, 1),
]


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def record(arr: np.ndarray):
    arr = np.ascontiguousarray(arr, dtype=np.int32)
    d = {"count": int(arr.size // 2), "sha256": sha(arr.tobytes())}
    if arr.size // 2 <= INLINE_MAX:
        d["pairs"] = arr.reshape(-1).tolist()
    return d


def record_ids(arr: np.ndarray):
    arr = np.ascontiguousarray(arr, dtype=np.int32)
    d = {"count": int(arr.size), "sha256": sha(arr.tobytes())}
    if arr.size <= 2 * INLINE_MAX:
        d["ids"] = arr.tolist()
    return d


def gro_case(d, pairs):
    """GRO newID of the directed pairs through the reference reorder program."""
    if not pairs.size:
        return {"unsupported": True, "reason": "empty"}
    u64 = (pairs[:, 0].astype(np.uint64) << np.uint64(32)) | pairs[:, 1].astype(np.uint32).astype(np.uint64)
    new_id, max_gain = oracle.gro(u64)
    if max_gain >= new_id.size:
        return {"unsupported": True, "reason": "max gain %d >= %d vertices" % (max_gain, new_id.size)}
    u64.tofile(os.path.join(d, "G.bin"))
    r = run([os.path.join(REF, "reorder"), "G.bin"], d)
    assert r.returncode == 0, r.stdout
    ids = np.loadtxt(os.path.join(d, "G_GRO_newID.txt"), dtype=np.int64, ndmin=2)
    assert np.array_equal(ids[:, 0], np.arange(ids.shape[0]))
    return record_ids(ids[:, 1])


def run(args, cwd):
    return subprocess.run(args, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)


def read_pairs(path):
    return np.fromfile(path, dtype=np.int32).reshape(-1, 2)


def grab(stdout, prefix):
    for line in stdout.splitlines():
        if line.startswith(prefix):
            return line[len(prefix):].strip()
    raise KeyError(prefix)


def case(name, pairs):
    pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
    out = {"input": record(pairs)}
    with tempfile.TemporaryDirectory() as d:
        e = os.path.join(d, "E.bin")
        pairs.tofile(e)
        r = run([os.path.join(REF, "A-direction-seri"), e], d)
        assert r.returncode == 0, r.stdout
        lp = read_pairs(os.path.join(d, "lpBasedGraph.bin"))
        out["adirection"] = record(lp)
        with tempfile.TemporaryDirectory() as d2:
            r = run([os.path.join(REF, "Bisson-A-direction"), e], d2)
            assert r.returncode == 0, r.stdout
            out["bisson_adir"] = record(read_pairs(os.path.join(d2, "lpBasedGraph.bin")))

        for key, src in (("aorder", os.path.join(d, "lpBasedGraph.bin")), ("aorder_raw", e)):
            src_pairs = read_pairs(src)
            if oracle.aorder(src_pairs) is None:
                # The reference indexes outside its arrays on this input; record its exit
                # status only (a crash shows as a non-zero / negative return code).
                r = run([os.path.join(REF, "A-order"), src], d)
                out[key] = {"unsupported": True, "ref_returncode": r.returncode}
                continue
            r = run([os.path.join(REF, "A-order"), src], d)
            assert r.returncode == 0, r.stdout
            out[key] = {"normal": record(read_pairs(os.path.join(d, "normal"))),
                        "reordered": record(read_pairs(os.path.join(d, "reordered")))}

        lpb = os.path.join(d, "lpBasedGraph.bin")
        r = run([os.path.join(REF, "A-order-v2"), lpb], d)
        assert r.returncode == 0, r.stdout
        out["aorder_v2"] = record(read_pairs(os.path.join(d, "naive")))
        r = run([os.path.join(REF, "relabel-naive"), lpb], d)
        assert r.returncode == 0, r.stdout
        out["relabel_good"] = record(read_pairs(os.path.join(d, "degreeOrder")))
        out["relabel_naive"] = record(read_pairs(os.path.join(d, "naive")))
        r = run([os.path.join(REF, "relabel4lpOut"), os.path.join(d, "lpBasedGraph")], d)
        assert r.returncode == 0, r.stdout
        out["relabel4lp"] = record(read_pairs(os.path.join(d, "good")))
        out["relabel4lp_bad"] = record(read_pairs(os.path.join(d, "bad")))
        r = run([os.path.join(REF, "relabel-random"), lpb], d)
        assert r.returncode == 0, r.stdout
        out["relabel_random"] = record(read_pairs(os.path.join(d, "bad")))

        cf = {}
        for k in (1, 2):
            r = run([os.path.join(REF, "costFuncCal"), os.path.join(d, "lpBasedGraph.bin"), str(k)], d)
            assert r.returncode == 0, r.stdout
            cf[str(k)] = [grab(r.stdout, "idPartCost: "), grab(r.stdout, "degreePartCost: "),
                          grab(r.stdout, "lpPartCost: ")]
        out["costfunc"] = cf
        r = run([os.path.join(REF, "verification"), os.path.join(d, "lpBasedGraph")], d)
        assert r.returncode == 0, r.stdout
        out["verification"] = [grab(r.stdout, "the lp base value is "),
                               grab(r.stdout, "the degree based value is ")]
        if os.path.exists(os.path.join(REF, "orgtc")):
            # OrgTriangleCount reads packed uint64 (u = high half) and needs both directions.
            sym = atc.simplify(pairs, symmetric=True) if pairs.size else pairs
            u64 = (sym[:, 0].astype(np.uint64) << np.uint64(32)) | sym[:, 1].astype(np.uint32).astype(np.uint64)
            u64.tofile(os.path.join(d, "E.u64"))
            r = run([os.path.join(REF, "orgtc"), os.path.join(d, "E.u64")], d)
            assert r.returncode == 0, r.stdout
            out["triangles"] = int(grab(r.stdout, "triangles="))
        if os.path.exists(os.path.join(REF, "reorder")):
            sym = atc.simplify(pairs, symmetric=True) if pairs.size else pairs
            out["gro_sym"] = gro_case(d, sym)
            out["gro_lp"] = gro_case(d, lp)
    return out


def main():
    assert os.path.exists(os.path.join(REF, "A-direction-seri")), "run `make -C oracle ref` first"
    cases = {}
    for name, pairs in TINY.items():
        cases[name] = {"source": {"kind": "inline"}, **case(name, pairs)}
        print(name, "ok")
    for name, scale, ef, seed in RMAT:
        g = atc.rmat_graph(scale, ef, seed, symmetric=True)
        cases[name] = {"source": {"kind": "rmat", "scale": scale, "edge_factor": ef, "seed": seed,
                                  "abc_ppm": list(atc.GRAPH500), "symmetric": True},
                       **case(name, g)}
        print(name, "ok", cases[name].get("triangles"))
    meta = {"generated_by": "tests/golden/make_golden.py", "host_machine": os.uname().machine,
            "programs": sorted(os.listdir(REF))}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"meta": meta, "cases": cases}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
