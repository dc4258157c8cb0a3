"""Runs the reference's four GPU counting programs (Hu, Bisson, Fox: `TC -f <file> <arg>`;
TriCore: `tric_gpu -f <file> debug`), built for sm_103a by `make -C oracle ref-gpu` from the
staged sources, on the benchmark graphs, and records the count each prints and the kernel
time each reports.  Runs on a machine with a GPU; every run has a host deadline.

Graphs (int32 pair files; TriCore reads the same bytes as uint64 edges, which swaps the two
ids of every edge and leaves the count unchanged):
  rmat16   R-MAT scale 16 ef 16 seed 1, symmetrised and simplified (golden case)
  rmat20   R-MAT scale 20 ef 16 seed 1, the same
  rmat24   the headline input: A-order's `reordered` file of A-direction-seri's output on
           R-MAT scale 24 ef 16 seed 1, made by libatc's drop-ins (byte-identical to the
           programs' outputs at this size, tests/test_gpu_config_pins.py)
Bisson refuses graphs of more than 13 107 200 vertices (Bisson/tc.cu:180-183), so it is not
run on rmat24.

Usage: python tests/golden/make_refgpu_golden.py OUT.json [graph ...]
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "accelerating-tc_gb300"))
import atc  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
PROGRAMS = {  # name -> (binary, extra args, kernel-time pattern)
    "hu": ("Hu-TC", [], r"kernel use ([0-9.eE+-]+) s"),
    "bisson": ("Bisson-TC", ["0"], r"kernel use ([0-9.eE+-]+) s"),
    "fox": ("Fox-TC", ["0"], None),
    "tricore": ("tric_gpu", ["debug"], None),
}


def graph(name):
    if name == "rmat16":
        return atc.rmat_graph(16, 16, 1)
    if name == "rmat20":
        return atc.rmat_graph(20, 16, 1)
    assert name == "rmat24"
    import torch
    atc.init(0)
    raw = torch.empty((16 << 24, 2), dtype=torch.int32, device="cuda")
    assert atc.lib().atc_gen_rmat_device(24, 16, *atc.GRAPH500, 1, raw.data_ptr(), None) == 0
    csr = atc.pretc_device(raw.data_ptr(), raw.shape[0], atc.Dir.ADIRECTION)
    del raw
    off, cols = csr.to_host()
    csr.free()
    lp = np.stack([np.repeat(np.arange(off.size - 1, dtype=np.int32), np.diff(off)), cols], 1)
    _, _, reordered = atc.aorder(lp)
    return reordered


def kernel_seconds(name, out):
    if name == "fox":  # per-bin " use time X ms." lines (Fox/tc.cu:382)
        ms = [float(x) for x in re.findall(r" use time ([0-9.eE+-]+) ms", out)]
        return sum(ms) / 1e3 if ms else None
    if name == "tricore":  # the TriCount clock's log line (main.cpp:96)
        m = re.findall(r"TriCount[^\n]*?([0-9.]+)\s*(ms|s)\b", out)
        if m:
            v, unit = m[-1]
            return float(v) / (1e3 if unit == "ms" else 1.0)
        return None
    m = re.search(PROGRAMS[name][2], out)
    return float(m.group(1)) if m else None


def main(out_path, names):
    res = {}
    with tempfile.TemporaryDirectory() as d:
        for gname in names:
            g = np.ascontiguousarray(graph(gname), dtype=np.int32)
            f = os.path.join(d, gname + ".bin")
            g.tofile(f)
            rec = {"pairs": int(g.shape[0]), "programs": {}}
            for pname, (binary, extra, _) in PROGRAMS.items():
                if pname == "bisson" and int(g.max()) + 1 > 13107200:
                    rec["programs"][pname] = {"skipped": "the program refuses more than 13107200 vertices"}
                    continue
                t0 = time.perf_counter()
                try:
                    r = subprocess.run([os.path.join(REF, binary), "-f", f] + extra, cwd=d, stdout=subprocess.PIPE,
                                       stderr=subprocess.STDOUT, text=True, timeout=900)
                except subprocess.TimeoutExpired:
                    rec["programs"][pname] = {"error": "timed out after 900 s"}
                    continue
                wall = time.perf_counter() - t0
                m = re.search(r"There are (\d+) triangles in the input graph", r.stdout)
                rec["programs"][pname] = {"rc": r.returncode, "count": int(m.group(1)) if m else None,
                                          "kernel_s": kernel_seconds(pname, r.stdout), "wall_s": wall}
                if r.returncode != 0 or not m:
                    rec["programs"][pname]["tail"] = r.stdout[-1500:]
                print(gname, pname, rec["programs"][pname].get("count"), rec["programs"][pname].get("kernel_s"),
                      "%.1f s" % wall, flush=True)
            res[gname] = rec
    meta = {"generated_by": "tests/golden/make_refgpu_golden.py", "host_machine": os.uname().machine,
            "build": "oracle/Makefile ref-gpu: nvcc sm_103a with oracle/ref_gpu_compat.h, staged sources with the two "
                     "warp-barrier patches"}
    with open(out_path, "w") as fo:
        json.dump({"meta": meta, "graphs": res}, fo, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2:] or ["rmat16", "rmat20", "rmat24"])
