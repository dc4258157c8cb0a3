"""The benchmark's CPU parts (no GPU needed): the reference arm's JSON line carries the
contract's keys on the GPU arm's metric, unit, config and direction (small R-MAT scale), and
the k-clique CPU baseline calibrates its sample."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "12",
                        "--steps", "2", "--warmup", "3"], cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["unit"] == "edges/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["scale"] == 12 and "workload" in d["config"]
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_kcl_cpu_sample_is_calibrated():
    # the k-clique CPU baseline lowers its stride from a sparse first sample towards the target
    import time
    sys.path.insert(0, ROOT)
    import bench
    import atc
    g = atc.rmat_graph(12, 16, 1)
    n = int(g.max()) + 1
    t0 = time.perf_counter()
    s = bench.kcl_cpu_sample(g, 4, n, 0.5)
    assert time.perf_counter() - t0 < 30
    assert set(s) == {"stride", "edges", "seconds", "edges_per_s", "cores", "kind"}
    assert 1 <= s["stride"] < n // 16 and s["edges"] > 0 and s["kind"] == "port"


def test_cpu_baseline_samples_are_bounded_by_the_clock():
    # the GPU line's CPU baseline: an all-core sample calibrated to the target and a one-thread
    # sample that stops after about a third of it, both labelled
    import time
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import oracle
    raw = oracle.gen_rmat(16, 16, 1)
    loff, lcols = oracle.lower_csr(raw)
    t0 = time.perf_counter()
    r = bench.cpu_baseline(loff, lcols, int(loff[-1]), 1.5)
    assert time.perf_counter() - t0 < 30
    assert r["kind"] == "port" and r["cores"] >= 1 and r["value"] > 0
    one = r["one_thread"]
    assert one["cores"] == 1 and one["value"] > 0 and one["unit"] == r["unit"]
    assert "phases 1.." in one["sample"]
