"""Shared test set-up: import paths, the `gpu` marker and golden-fixture helpers."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "accelerating-tc_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

GOLDEN_PATH = os.path.join(ROOT, "tests", "golden", "golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: long-running case")


def load_golden():
    with open(GOLDEN_PATH) as f:
        return json.load(f)


def golden_input(case):
    """Rebuilds a golden case's input pairs (inline, or via libatc's generator)."""
    import atc
    src = case["source"]
    if src["kind"] == "inline":
        return np.array(case["input"]["pairs"], dtype=np.int32).reshape(-1, 2)
    assert src["kind"] == "rmat"
    return atc.rmat_graph(src["scale"], src["edge_factor"], src["seed"], symmetric=src["symmetric"])


@pytest.fixture(scope="session")
def golden():
    return load_golden()


@pytest.fixture(scope="session")
def gpu_ready():
    """Initialises device 0 through libatc; the GPU tests need the CUDA path loaded."""
    import atc
    atc.init(0)
    return True


def write_gr(path, n, adj, version):
    """A Galois .gr file: header, u64 end offsets, targets (u32 padded to 8 or u64)."""
    ends = np.cumsum([len(a) for a in adj]).astype(np.uint64)
    dst = np.array([v for a in adj for v in a], dtype=np.uint32 if version == 1 else np.uint64)
    with open(path, "wb") as f:
        f.write(np.array([version, 0, n, len(dst)], dtype=np.uint64).tobytes())
        f.write(ends.tobytes())
        f.write(dst.tobytes())
        if version == 1 and len(dst) % 2:
            f.write(b"\0" * 4)

