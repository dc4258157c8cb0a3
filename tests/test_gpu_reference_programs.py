"""The reference's own GPU counting programs (Hu, Bisson, Fox `TC`, TriCore `tric_gpu`), built
for sm_103a from the sources staged into baseline/_ref/src (`make -C oracle stage` where the
reference tree exists; `make -C oracle ref-gpu-tc` builds them), run on the golden R-MAT
scale 16 graph: each must print the count the oracle and libatc compute.  Skipped where the
sources were not staged.  The same programs' counts and kernel times at scales 20 and 24 are
recorded in tests/golden/ref_gpu_counts.json (tests/golden/make_refgpu_golden.py)."""
import os
import re
import subprocess

import pytest

import atc
from conftest import ROOT, golden_input, load_golden

pytestmark = pytest.mark.gpu

STAGED = os.path.join(ROOT, "baseline", "_ref", "src", "Hu", "tc.cu")
REF = os.path.join(ROOT, "oracle", "_ref")
PROGRAMS = {"hu": ("Hu-TC", []), "bisson": ("Bisson-TC", ["0"]), "fox": ("Fox-TC", ["0"]),
            "tricore": ("tric_gpu", [])}


@pytest.fixture(scope="module")
def built():
    if not all(os.path.exists(os.path.join(REF, b)) for b, _ in PROGRAMS.values()):
        if not os.path.exists(STAGED):
            pytest.skip("the reference's GPU sources are not staged here")
        r = subprocess.run(["make", "-s", "-j4", "-C", os.path.join(ROOT, "oracle"), "ref-gpu-tc"],
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=900)
        assert r.returncode == 0, r.stdout[-3000:]
    return True


@pytest.mark.parametrize("name", sorted(PROGRAMS))
def test_reference_program_counts_the_golden_graph(built, tmp_path, gpu_ready, name):
    case = load_golden()["cases"]["rmat_s16_ef16_seed1"]
    g = golden_input(case)
    f = tmp_path / "E.bin"
    g.tofile(f)
    binary, extra = PROGRAMS[name]
    r = subprocess.run([os.path.join(REF, binary), "-f", str(f)] + extra, cwd=tmp_path, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    m = re.search(r"There are (\d+) triangles in the input graph", r.stdout)
    assert m, r.stdout[-2000:]
    assert int(m.group(1)) == case["triangles"]
    csr = atc.pretc(g, atc.Dir.ADIRECTION)
    assert atc.tc(csr, atc.Kernel.AUTO)[0] == int(m.group(1))
    csr.free()
