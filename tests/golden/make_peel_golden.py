"""Records the output of the reference's approximate GPU A-direction program
(edge_directing/A-direction-parallel, binary `Peel`, built by `make -C oracle ref-gpu` from
the staged sources) on the seven cases of tests/golden/apeel_cases.py, as SHA-256 of the
oriented uint64 edge file it writes.  Runs on a machine with a GPU; each run is bounded by
a host deadline.

Usage: python tests/golden/make_peel_golden.py OUT.json
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
sys.path.insert(0, HERE)
from apeel_cases import apeel_graphs, packed  # noqa: E402

PEEL = os.path.join(ROOT, "oracle", "_ref", "Peel")


def main(out_path):
    assert os.path.exists(PEEL), "build it first: make -C oracle ref-gpu"
    cases = {}
    with tempfile.TemporaryDirectory() as d:
        for name, g in apeel_graphs():
            e = packed(g)
            fin, fout = os.path.join(d, name + ".u64"), os.path.join(d, name + ".out")
            e.tofile(fin)
            r = subprocess.run([PEEL, fin, fout], cwd=d, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                               text=True, timeout=120)
            assert r.returncode == 0, (name, r.stdout[-2000:])
            out = np.fromfile(fout, dtype=np.uint64)
            assert out.size == e.size, (name, out.size, e.size)
            cases[name] = {"input": {"count": int(e.size), "sha256": hashlib.sha256(e.tobytes()).hexdigest()},
                           "peel_out": {"sha256": hashlib.sha256(out.tobytes()).hexdigest()},
                           "itera": [ln for ln in r.stdout.splitlines() if ln.startswith("itera is")][-1:]}
            print(name, "ok", flush=True)
    meta = {"generated_by": "tests/golden/make_peel_golden.py", "program": "edge_directing/A-direction-parallel "
            "(peel.cu, buildCSR.cu), nvcc sm_103a with oracle/ref_gpu_compat.h", "host_machine": os.uname().machine}
    with open(out_path, "w") as f:
        json.dump({"meta": meta, "cases": cases}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1])
