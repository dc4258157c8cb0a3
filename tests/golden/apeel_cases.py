"""The seven seeded input graphs of the approximate A-direction parity cases (shared by
tests/test_gpu_parity.py and tests/golden/make_peel_golden.py): symmetric, once-listed and
raw R-MAT (repeats and loops kept), uniform random, geometric, sparse (m / n < 1) and a
40-clique with both directions."""
import numpy as np


def apeel_graphs():
    import atc
    rng = np.random.default_rng(21)
    yield "rmat12-sym", atc.rmat_graph(12, 16, 2)
    yield "rmat13-once", atc.simplify(atc.gen_rmat(13, 8, 9), symmetric=False)
    yield "rmat11-raw", atc.gen_rmat(11, 16, 4)                       # repeats and loops kept
    yield "uniform", rng.integers(0, 2000, size=(20000, 2)).astype(np.int32)
    yield "rgg", atc.gen_rgg(20000, 12.0, 3)
    yield "sparse", rng.integers(0, 5000, size=(2000, 2)).astype(np.int32)  # m / n < 1
    yield "clique", np.array([(i, j) for i in range(40) for j in range(40) if i != j], dtype=np.int32)


def packed(g):
    """int32 pairs as the programs' uint64 edges (FIRST = high half = the pair's first id)."""
    return (g[:, 0].astype(np.uint64) << np.uint64(32)) | g[:, 1].astype(np.uint32).astype(np.uint64)
