"""Parity at the benchmark configurations' full sizes.

The golden fixtures of test_gpu_parity.py stop at R-MAT scale 16.  Here the library's
results on the configurations the benchmark measures are compared with what the
reference's own programs and the oracle produce on the same seeded graphs
(tests/golden/config_pins.json, made by tests/golden/make_config_pins.py):

- R-MAT scale 24 (the headline): the A-direction orientation (A-direction-seri's
  lpBasedGraph.bin), the A-order outputs (normal, reordered), the oriented CSR that
  A-direction + A-order hand to the kernels, its W statistics, and the triangle count of
  every kernel family against the oracle's count;
- k-cliques: the RGG with n = 2^20 (mean degree 32) at k = 4..7 and R-MAT scale 20 at
  k = 3, 4 against the oracle; at k = 6, 7 on R-MAT scale 20 (beyond what the oracle
  enumerates in reasonable time) the dense-candidate-set kernel is checked against the
  warp search forced on the same edge ranges;
- batches: a seeded 64-graph subset of the Chung-Lu batch generator against the oracle,
  graph by graph.

Inputs are generated on the device (the generators are byte-identical to the host ones,
test_device_generator_matches_host) and reduced to the simple graph by preTC.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import atc
import oracle
from conftest import ROOT

pytestmark = pytest.mark.gpu

PINS = os.path.join(ROOT, "tests", "golden", "config_pins.json")
KERNELS = [atc.Kernel.HU, atc.Kernel.BISSON, atc.Kernel.FOX, atc.Kernel.TRICORE]


@pytest.fixture(scope="module")
def pins(gpu_ready):
    with open(PINS) as f:
        return json.load(f)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


def edge_list(csr):
    off, cols = csr.to_host()
    src = np.repeat(np.arange(off.size - 1, dtype=np.int32), np.diff(off))
    return np.stack([src, cols], 1)


def device_rmat(scale, ef, seed):
    import torch
    nraw = ef << scale
    raw = torch.empty((nraw, 2), dtype=torch.int32, device="cuda")
    assert atc.lib().atc_gen_rmat_device(scale, ef, *atc.GRAPH500, seed, raw.data_ptr(), None) == 0
    return raw


def sorted_pairs(p):
    key = (p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64)
    key.sort()
    return np.stack([(key >> np.uint64(32)).astype(np.int32), (key & np.uint64(0xFFFFFFFF)).astype(np.int32)], 1)


def device_rgg(n, mean_degree, seed):
    import ctypes as C
    import torch
    cnt = C.c_uint64(0)
    cap = n * 20
    dev = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    assert atc.lib().atc_gen_rgg_device(n, mean_degree, seed, dev.data_ptr(), cap, C.byref(cnt), None) == 0
    return dev[: cnt.value]


def test_rmat24_headline_orientation_order_and_counts(pins):
    import torch
    p = pins["rmat24"]
    src = p["source"]
    raw = device_rmat(src["scale"], src["edge_factor"], src["seed"])
    # A-direction alone: the CSR's edge list is A-direction-seri's lpBasedGraph.bin
    csr = atc.pretc_device(raw.data_ptr(), raw.shape[0], atc.Dir.ADIRECTION)
    lp = edge_list(csr)
    csr.free()
    assert lp.shape[0] == p["adirection"]["count"]
    assert sha(lp) == p["adirection"]["sha256"]
    # the A-order drop-in on that output: the program's two files
    _, normal, reordered = atc.aorder(lp)
    assert sha(normal) == p["aorder"]["normal"]["sha256"]
    assert sha(reordered) == p["aorder"]["reordered"]["sha256"]
    del normal, reordered, lp
    # the headline pipeline: A-direction + A-order in preTC
    csr = atc.pretc_device(raw.data_ptr(), raw.shape[0], atc.Dir.ADIRECTION, atc.Order.AORDER)
    del raw
    torch.cuda.empty_cache()
    assert sha(edge_list(csr)) == p["csr_edges"]["sha256"]
    assert csr.wedges == p["wedges"] and csr.wedges_min == p["wedges_min"]
    for k in KERNELS + [atc.Kernel.AUTO]:
        assert atc.tc(csr, k)[0] == p["triangles"], k.name
    csr.free()


@pytest.mark.parametrize("k", [4, 5, 6, 7])
def test_kcl_rgg20_config_counts(pins, k):
    p = pins["kcl"]["rgg20"]
    src = p["source"]
    g = device_rgg(src["n"], src["mean_degree"], src["seed"])
    # the device generator writes the same edges as the host one, in an order of its own
    assert sha(sorted_pairs(g.cpu().numpy())) == p["input"]["sha256"]
    csr = atc.pretc_device(g.data_ptr(), g.shape[0], atc.Dir.ADIRECTION)
    assert atc.kcl(csr, k)[0] == p["cliques"][str(k)]
    csr.free()


@pytest.fixture(scope="module")
def rmat20_csr(pins):
    p = pins["kcl"]["rmat20"]
    src = p["source"]
    raw = device_rmat(src["scale"], src["edge_factor"], src["seed"])
    csr = atc.pretc_device(raw.data_ptr(), raw.shape[0], atc.Dir.ADIRECTION)
    yield csr
    csr.free()


@pytest.mark.parametrize("k", [3, 4])
def test_kcl_rmat20_config_counts(pins, rmat20_csr, k):
    assert atc.kcl(rmat20_csr, k)[0] == pins["kcl"]["rmat20"]["cliques"][str(k)]
    if k == 3:
        assert atc.tc(rmat20_csr)[0] == pins["kcl"]["rmat20"]["cliques"]["3"]


@pytest.mark.parametrize("k,nparts,parts", [(5, 16, (3, 11)), (6, 256, (5, 160)), (7, 16384, (77, 11000))])
def test_kcl_dense_path_equals_warp_search_at_rmat20(rmat20_csr, k, nparts, parts):
    # the same edge ranges counted with the dense-candidate-set kernel (default) and with
    # every edge on the warp search (too slow over the whole graph at k = 6, 7)
    total = 0
    for part in parts:
        dense, rng, _ = atc.kcl_part(rmat20_csr, k, part, nparts)
        warp, rng2, _ = atc.kcl_part(rmat20_csr, k, part, nparts, dense=False)
        assert rng == rng2 and dense == warp, (k, part, dense, warp)
        total += dense
    assert total > 0


def test_batch_chunglu_subset_matches_oracle():
    """Every 64th graph of the 4096-graph Chung-Lu batch (the generator's seeded
    parameters), counted as one batch and graph by graph by the oracle."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    params = bench.batch_params(4096, 1)
    b = atc.Batch()
    want = []
    for i in range(0, 4096, 64):
        n, gamma, md = params[i]
        pairs = atc.gen_chunglu_device(n, gamma, md, 1 * 100003 + i)
        csr = atc.pretc_device(pairs.data_ptr(), pairs.shape[0], atc.Dir.ADIRECTION)
        b.add(csr)
        csr.free()
        want.append(oracle.tc_count(pairs.cpu().numpy()))
    for t in (None, {"group_by_source": 1, "bisson_cutover": 8}, {"group_by_source": 2},
              {"group_by_source": 2, "bisson_cutover": 64}):
        got, _ = b.run(tuning=t)
        assert [int(x) for x in got] == want
    b.free()
