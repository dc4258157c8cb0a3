"""Counting in parts (atc_tc_part, atc_kcl_part): the work-balanced edge ranges of a CSR tile
it, and the part counts add up to the whole count for every kernel family and for k-cliques.  This is the sharding
unit of a count spread over several GPUs; here the parts run one after another on one GPU.
"""
import pytest

import atc
import oracle

pytestmark = pytest.mark.gpu

KERNELS = [atc.Kernel.HU, atc.Kernel.BISSON, atc.Kernel.FOX, atc.Kernel.TRICORE]


@pytest.fixture(scope="module", autouse=True)
def _init(gpu_ready):
    yield


@pytest.mark.parametrize("d,o,scale", [(atc.Dir.ID, atc.Order.NONE, 12), (atc.Dir.ADIRECTION, atc.Order.AORDER, 14),
                                       (atc.Dir.DEGREE, atc.Order.NONE, 15)])
def test_parts_add_up_to_the_count(d, o, scale):
    g = atc.rmat_graph(scale, 16, 5)
    want = oracle.tc_count(g)
    csr = atc.pretc(g, d, o)
    for k in KERNELS:
        assert atc.tc(csr, k)[0] == want
        for nparts in (1, 2, 3, 7):
            total, prev = 0, 0
            for p in range(nparts):
                c, (e0, e1), _ = atc.tc_part(csr, p, nparts, k)
                assert e0 == prev and e1 >= e0, (k.name, nparts, p, e0, e1)
                prev = e1
                total += c
            assert prev == csr.m
            assert total == want, (d.name, k.name, nparts)


def test_parts_are_balanced_by_work():
    csr = atc.pretc(atc.rmat_graph(14, 16, 2), atc.Dir.ADIRECTION)
    off, cols = csr.to_host()
    deg = off[1:] - off[:-1]
    import numpy as np
    src = np.repeat(np.arange(len(deg)), deg)
    work = np.minimum(deg[src], deg[cols]) + 1
    nparts = 4
    shares = []
    for p in range(nparts):
        _, (e0, e1), _ = atc.tc_part(csr, p, nparts)
        shares.append(int(work[e0:e1].sum()))
    top = max(int(work.max()), 1)
    for sh in shares:
        assert abs(sh - work.sum() / nparts) <= top + 1, shares


def test_more_parts_than_edges_and_bad_arguments():
    g = atc.simplify([[0, 1], [1, 2], [0, 2], [2, 3], [1, 3]])
    csr = atc.pretc(g, atc.Dir.DEGREE)
    want = atc.tc(csr)[0]
    assert want == 2
    for k in KERNELS:
        assert sum(atc.tc_part(csr, p, 50, k)[0] for p in range(50)) == want
    with pytest.raises(atc.ATCError):
        atc.tc_part(csr, 3, 3)
    with pytest.raises(atc.ATCError):
        atc.tc_part(csr, 0, 0)


def test_kclique_parts_add_up():
    # R-MAT s12 with 32 edges a vertex has candidate sets above 64 (the dense path at k >= 5)
    g = atc.rmat_graph(12, 32, 8)
    csr = atc.pretc(g, atc.Dir.ADIRECTION, atc.Order.AORDER)
    tc_ranges = [atc.tc_part(csr, p, 5)[1] for p in range(5)]
    for k in (3, 4, 5):
        want = atc.kcl(csr, k)[0]
        assert want == oracle.kclique(g, k)
        for nparts in (1, 2, 5):
            total, prev = 0, 0
            for p in range(nparts):
                c, (e0, e1), _ = atc.kcl_part(csr, k, p, nparts)
                assert e0 == prev and e1 >= e0
                if nparts == 5:
                    assert (e0, e1) == tc_ranges[p]
                prev = e1
                total += c
            assert prev == csr.m
            assert total == want, (k, nparts)
    with pytest.raises(atc.ATCError):
        atc.kcl_part(csr, 4, 2, 2)
