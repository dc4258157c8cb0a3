"""The source-level drop-in header for the reference's kcl_gpu_solver (include/atc_kcl_solver.hpp):
a program written against the reference's signature compiles, links against libatc and counts.
The CPU test covers compiling, linking and the error path (no device needed); the GPU test
checks the count on a Galois .gr file against the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import atc
import oracle
from conftest import ROOT, write_gr

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include "atc_kcl_solver.hpp"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  typedef unsigned long long AccType;  // as in the reference's kcl_gpu.cpp
  AccType total = 7;
  try {
    kcl_gpu_solver(argv[1], (unsigned)atoi(argv[2]), total);
  } catch (const std::exception& e) {
    std::cerr << e.what() << "\n";
    std::cout << "unchanged " << total << "\n";
    return 3;
  }
  std::cout << "\n\ttotal_num_cliques = " << total - 7 << "\n\n";
  return 0;
}
"""


def _build(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "kcl_prog.cpp"
    src.write_text(PROGRAM)
    libdir = os.path.dirname(atc.LIB_PATH)
    exe = tmp_path / "kcl_prog"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe),
                        "-L", libdir, "-latc", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_header_compiles_links_and_reports_errors(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), str(tmp_path / "missing.gr"), "4"], capture_output=True, text=True)
    assert r.returncode == 3
    assert "kcl_gpu_solver: reading the graph" in r.stderr
    assert "unchanged 7" in r.stdout  # the accumulator is not touched on failure


@pytest.mark.gpu
def test_header_counts_like_the_oracle(tmp_path):
    exe = _build(tmp_path)
    g = atc.rmat_graph(10, 16, 2)
    n = int(g.max()) + 1
    adj = [[] for _ in range(n)]
    for u, v in g:
        adj[u].append(int(v))
    gr = tmp_path / "g.gr"
    write_gr(gr, n, adj, 1)
    for k in (3, 4, 5):
        r = subprocess.run([str(exe), str(gr), str(k)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert "total_num_cliques = %d" % oracle.kclique(g, k) in r.stdout
