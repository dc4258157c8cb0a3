"""Build recipe for libatc.so (sm_103a), the CLI drop-ins and the test oracle.

Every CUDA translation unit under csrc/ is compiled by nvcc for sm_103a only, in
parallel, into _build/; the objects are linked into libatc.so next to this file.
The CLI programs under cli/ link against it.  The oracle (test infrastructure) is
built by oracle/Makefile; the reference programs too when the reference tree exists.

Usage: python accelerating-tc_gb300/build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libatc.so")
BIN = os.path.join(PKG, "bin")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
    "--expt-relaxed-constexpr", "-I", INC, "-I", CSRC,
]
CLI_PROGRAMS = {
    # binary name -> source
    "tc_hu": "tc_main.cpp",
    "tc_bisson": "tc_main.cpp",
    "tc_fox": "tc_main.cpp",
    "tric_gpu": "tc_main.cpp",
    "a_direction_seri": "order_main.cpp",
    "a_order": "order_main.cpp",
    "bisson_a_direction": "order_main.cpp",
    "a_order_v2": "order_main.cpp",
    "relabel_naive": "order_main.cpp",
    "relabel4lp_out": "order_main.cpp",
    "relabel_random": "order_main.cpp",
    "kcl": "kcl_main.cpp",
    "cost_func_cal": "order_main.cpp",
    "kcore_direction": "order_main.cpp",
    "Peel": "order_main.cpp",
    "reorder": "order_main.cpp",
}


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (r.returncode, " ".join(cmd), r.stdout))
    return r.stdout


def _digest(paths, extra=""):
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    return h.hexdigest()


def _headers():
    hs = [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def build_lib(force=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdrs = _headers()
    objs = []
    todo = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        stamp = o + ".stamp"
        d = _digest([s] + hdrs, " ".join(NVFLAGS) + NVCC)
        objs.append(o)
        if force or not (os.path.exists(o) and os.path.exists(stamp) and open(stamp).read() == d):
            todo.append((s, o, stamp, d))

    def compile_one(item):
        s, o, stamp, d = item
        _run([NVCC] + NVFLAGS + ["-c", s, "-o", o])
        with open(stamp, "w") as f:
            f.write(d)
        return s

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for _ in ex.map(compile_one, todo):
                pass
    link_stamp = os.path.join(BUILD, "libatc.stamp")
    ld = _digest(objs)
    if force or todo or not os.path.exists(LIB) or not os.path.exists(link_stamp) or open(link_stamp).read() != ld:
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"])
        with open(link_stamp, "w") as f:
            f.write(ld)
    return LIB


def build_cli(force=False):
    os.makedirs(BIN, exist_ok=True)
    for name, src in CLI_PROGRAMS.items():
        path = os.path.join(CLI, src)
        if not os.path.exists(path):
            continue
        out = os.path.join(BIN, name)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(path), os.path.getmtime(LIB)):
            continue
        define = "-DATC_PROGRAM_" + name.upper()
        _run(["g++", "-O2", "-std=c++17", define, "-I", INC, path, "-o", out,
              "-L", PKG, "-latc", "-Wl,-rpath,$ORIGIN/.."])


STAGED_REF = os.path.join(ROOT, "baseline", "_ref", "src")


def build_oracle():
    """The oracle library, and the reference's CPU programs: from the reference tree where it
    exists (oracle/Makefile's REF, or ATC_REFERENCE_TREE when set), else from the sources
    staged into baseline/_ref/src by `make -C oracle stage`."""
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"])
    ref = os.environ.get("ATC_REFERENCE_TREE")
    if not ref and os.path.isdir(STAGED_REF):
        default = _run(["make", "-s", "--no-print-directory", "-C", os.path.join(ROOT, "oracle"), "print-ref"]).strip()
        if not os.path.isdir(default):
            ref = STAGED_REF
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-if-present"] + (["REF=" + ref] if ref else []))


def build_all(force=False):
    build_lib(force)
    build_cli(force)
    build_oracle()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB)
