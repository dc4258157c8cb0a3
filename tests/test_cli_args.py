"""The drop-in programs' argument handling, without a GPU: a missing argument prints the
program's usage and exits 2; an unreadable input exits 1 with the path in the message (the
file is read before the device is touched)."""
import os
import subprocess

import pytest

import atc

BIN = os.path.join(os.path.dirname(atc.LIB_PATH), "bin")

# program -> (arguments that name a missing input, where its usage is printed)
PROGRAMS = {
    "tc_hu": (["-f", "{}"], "stdout"),
    "tc_bisson": (["-f", "{}", "0"], "stdout"),
    "tc_fox": (["-f", "{}", "0"], "stdout"),
    "tric_gpu": (["-f", "{}"], "stdout"),
    "a_direction_seri": (["{}"], "stderr"),
    "a_order": (["{}"], "stderr"),
    "a_order_v2": (["{}"], "stderr"),
    "cost_func_cal": (["{}", "2"], "stderr"),
    "kcore_direction": (["{}", "{}.out"], "stderr"),
    "Peel": (["{}", "{}.out"], "stderr"),
    "reorder": (["{}"], "stderr"),
    "kcl": (["{}", "-k=4"], "stderr"),
}


@pytest.mark.parametrize("prog", sorted(PROGRAMS))
def test_usage_and_missing_input(prog, tmp_path):
    exe = os.path.join(BIN, prog)
    if not os.path.exists(exe):
        pytest.skip("programs not built")
    r = subprocess.run([exe], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 2
    assert "sage" in getattr(r, PROGRAMS[prog][1])
    missing = str(tmp_path / "missing.bin")
    r = subprocess.run([exe] + [a.format(missing) for a in PROGRAMS[prog][0]], capture_output=True, text=True,
                       cwd=tmp_path)
    assert r.returncode == 1, (r.stdout, r.stderr)
    assert missing in r.stderr
