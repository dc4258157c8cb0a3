"""CSRs whose edge arrays live in pinned host memory mapped into the device (for graphs
larger than device memory): every kernel family, the parts, k-cliques and the cache file
give the same results as the device-resident CSR."""
import numpy as np
import pytest

import atc
import oracle

pytestmark = pytest.mark.gpu

KERNELS = [atc.Kernel.HU, atc.Kernel.BISSON, atc.Kernel.FOX, atc.Kernel.TRICORE]


@pytest.fixture(scope="module", autouse=True)
def _init(gpu_ready):
    yield


@pytest.mark.parametrize("d", [atc.Dir.ADIRECTION, atc.Dir.ID])
def test_host_resident_counts_equal(d):
    g = atc.rmat_graph(13, 16, 9)
    want = oracle.tc_count(g)
    csr = atc.pretc(g, d)
    off0, cols0 = csr.to_host()
    k4 = atc.kcl(csr, 4)[0]
    csr.to_host_resident()
    csr.to_host_resident()  # a second call is a no-op
    off1, cols1 = csr.to_host()
    assert np.array_equal(off0, off1) and np.array_equal(cols0, cols1)
    for k in KERNELS:
        assert atc.tc(csr, k)[0] == want, k.name
        assert sum(atc.tc_part(csr, p, 3, k)[0] for p in range(3)) == want, k.name
    assert atc.kcl(csr, 4)[0] == k4
    csr.free()


def test_load_host_resident_cache(tmp_path):
    g = atc.rmat_graph(12, 16, 4)
    want = oracle.tc_count(g)
    csr = atc.pretc(g, atc.Dir.DEGREE)
    path = str(tmp_path / "g.atccsr")
    csr.save(path)
    h = atc.CSR.load(path, host_resident=True)
    assert h.m == csr.m and h.n == csr.n
    for k in KERNELS:
        assert atc.tc(h, k)[0] == want, k.name
    path2 = str(tmp_path / "g2.atccsr")
    h.save(path2)
    assert open(path, "rb").read() == open(path2, "rb").read()
    h.free()
    csr.free()
