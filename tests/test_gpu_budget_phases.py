"""Failure paths and instrumentation on the device.

- Device allocation budget (atc_set_alloc_budget): every allocation the budget cannot cover
  fails with ATC_ERR_OOM, wherever in the pipeline it falls, the failed call leaves nothing
  behind that breaks the next one, and the counts stay exact once the budget is lifted.
  This drives the library's out-of-memory returns without exhausting the device.
- Phase timing (atc_phase_timing / atc_phase_times): the preTC and counting phases are
  recorded, nest, and their device times add up within their parents.
"""
import numpy as np
import pytest

import atc
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _init(gpu_ready):
    yield
    atc.set_alloc_budget(None)
    atc.phase_timing(False)


SMALL = None


def _small():
    """A small graph on which A-order is defined, and its count."""
    global SMALL
    if SMALL is None:
        g = atc.rmat_graph(9, 8, 5)
        SMALL = (g, oracle.tc_count(g))
    return SMALL


def _pipeline(g, kernel):
    csr = atc.pretc(g, atc.Dir.ADIRECTION, atc.Order.AORDER)
    try:
        return atc.tc(csr, kernel)[0]
    finally:
        csr.free()


@pytest.mark.parametrize("kernel", [atc.Kernel.HU, atc.Kernel.BISSON, atc.Kernel.FOX, atc.Kernel.TRICORE])
def test_budget_oom_anywhere_then_exact(kernel):
    g = atc.rmat_graph(12, 16, 3)
    want = oracle.tc_count(g)
    failed = 0
    budget = 1 << 10
    got = None
    while got is None:
        atc.set_alloc_budget(budget)
        try:
            got = _pipeline(g, kernel)
        except atc.ATCError as e:
            assert e.status == atc.Status.ERR_OOM, str(e)
            assert "allocation budget" in str(e)
            failed += 1
        finally:
            atc.set_alloc_budget(None)
        # the failed call left the library usable: a small count right after it is exact
        sg, sc = _small()
        assert _pipeline(sg, kernel) == sc
        budget = budget * 3 // 2
        assert budget < 1 << 34
    assert failed >= 5  # the budget ran out at several different allocations
    assert got == want


def test_phase_times_nest_and_add_up():
    g = atc.rmat_graph(14, 16, 2)
    atc.phase_timing(True)
    try:
        csr = atc.pretc(g, atc.Dir.ADIRECTION, atc.Order.AORDER)
        c, _ = atc.tc(csr, atc.Kernel.BISSON)
        csr.free()
        ph = atc.phase_times()
        assert atc.phase_times() == []  # a read clears the record
    finally:
        atc.phase_timing(False)
    assert c == oracle.tc_count(g)
    names = [(d, n) for n, d, _ in ph]
    for want in [(0, "pretc"), (1, "pretc.alloc"), (1, "pretc.h2d"), (1, "pretc.dedup"), (1, "pretc.degrees"), (1, "pretc.order+peel"),
                 (1, "pretc.orient+sort"), (1, "pretc.csr"), (0, "tc"), (1, "tc.group"), (1, "tc.count"),
                 (1, "tc.readback")]:
        assert want in names, (want, names)
    assert all(ms >= 0 for _, _, ms in ph)
    # children of a depth-0 phase (the depth-1 phases that follow it) fit inside it
    i = 0
    while i < len(ph):
        name, d, ms = ph[i]
        assert d == 0, ph[i]
        j = i + 1
        child = 0.0
        while j < len(ph) and ph[j][1] > 0:
            if ph[j][1] == 1:
                child += ph[j][2]
            j += 1
        assert child <= ms * 1.05 + 0.05, (name, ms, child)
        i = j


@pytest.mark.parametrize("tuning", [None, {"group_by_source": 1}, {"group_by_source": 2}])
def test_batch_replay_stages(tuning):
    """The stages of a batch replay are timed by event nodes inside its CUDA graph and
    recorded under the call's phase; they fit inside it and the counts stay exact."""
    graphs = [atc.rmat_graph(9 + i % 4, 8, 20 + i) for i in range(8)]
    want = [oracle.tc_count(g) for g in graphs]
    b = atc.Batch()
    for g in graphs:
        csr = atc.pretc(g, atc.Dir.ADIRECTION)
        b.add(csr)
        csr.free()
    atc.phase_timing(True)
    try:
        got, st = b.run(tuning=tuning)
        ph = atc.phase_times()
    finally:
        atc.phase_timing(False)
    b.free()
    assert [int(x) for x in got] == want
    assert ph[0][0] == "batch" and ph[0][1] == 0, ph
    stages = ph[1:]
    names = [n for n, _, _ in stages]
    assert all(d == 1 for _, d, _ in stages), ph
    assert names[0] == "batch.reset" and "batch.items" in names and "batch.block" in names and "batch.warp" in names
    assert ("batch.group" in names) == (tuning is None or tuning["group_by_source"] != 1)
    assert all(ms >= 0 for _, _, ms in stages)
    assert sum(ms for _, _, ms in stages) <= ph[0][2] * 1.05 + 0.05
    assert st.launches >= 3


def test_bounded_wait_gives_up_and_leaves_the_device_usable():
    """The staged kernels' bulk-copy waits are bounded in time: a wait on a barrier that can
    never complete gives up within its limit and is reported as ERR_TIMEOUT; the context stays
    usable and the next counts are exact."""
    import time
    g, want = _small()
    for _ in range(3):
        t0 = time.perf_counter()
        assert atc.check_wait_timeout() == atc.Status.ERR_TIMEOUT
        assert time.perf_counter() - t0 < 5.0
        assert "time limit" in atc.lib().atc_last_error().decode()
        csr = atc.pretc(g, atc.Dir.ADIRECTION)
        for k in (atc.Kernel.TRICORE, atc.Kernel.FOX):
            assert atc.tc(csr, k)[0] == want
        csr.free()
