"""Benchmark: triangle-counting throughput (undirected edges per second) on one GB300.

Workload (default): seeded R-MAT scale 24, edge factor 16 (a,b,c = .57,.19,.19), raw
samples deduplicated on the device, A-order relabelling + A-direction orientation
(the reference's "A-direction + A-order then each kernel" configuration).

A step counts the triangles of the resident oriented CSR once with the headline kernel
(AUTO).  `value` = undirected simple edges / device time of a step (CSR already in HBM;
the 1+ GB CSR exceeds the 129 MB L2, so no flush is needed between steps).  `e2e` is the
same metric through the public C ABI with host buffers: every step copies the raw
int32 pairs from pinned host memory, builds the CSR (dedup, A-order, A-direction),
counts and reads the count back.  Every kernel family is also timed ("kernels").  The
single-GPU line also carries a reduced batch leg (256 of the 4096 Chung-Lu graphs, batched
against per-graph loops), the learned selector on its committed timing fixture, a k-clique
leg (the RGG configuration at k = 4..7), and the CPU baseline (all cores and one thread, and
the reference's own preprocessing programs).

With N > 1 ranks (torchrun, NCCL) every rank builds the same CSR, each step counts the rank's
work-balanced part of the edges (atc_tc_part) and sums the parts with one all_reduce: the
total work is fixed ("scaling": "strong") and `value` = edges / the slowest rank's step.

--impl reference times the reference's CPU triangle count (the oracle restatement of
OrgTriangleCount's scalar merge, all host threads) on a bounded vertex sample of the same
graph and prints the same JSON line with "impl": "reference".

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--scale S] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "accelerating-tc_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "TC edges/s (1 GB300), HBM % of roofline; batched/learned vs plain, exact counts"
UNIT = "edges/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--scale", type=int, default=24)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU work of the baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kernels", default="hu,bisson,fox,tricore,fox_edge,tricore_edge",
                    help="families timed besides the headline (suffix _edge: the per-edge global-search kernels)")
    ap.add_argument("--mode", default="tc", choices=["tc", "kcl", "batch", "select"],
                    help="tc: the headline (R-MAT scale 24, every kernel family); kcl: k-clique counts; "
                         "batch: many Chung-Lu graphs, batched vs per-graph loop; select: the learned selector")
    ap.add_argument("--batch-graphs", type=int, default=4096)
    ap.add_argument("--select-train", type=int, default=2048, help="training graphs of the selector")
    ap.add_argument("--select-eval", type=int, default=512, help="held-out graphs of the selector")
    ap.add_argument("--select-out", default="", help="write features and timings (.npz) here")
    ap.add_argument("--select-space", choices=("config", "extended"), default="config",
                    help="triples timed: the config's 24, or also k-core / approximate A-direction and the "
                         "rank relabellings (60)")
    ap.add_argument("--batch-plain-kernels", default="bisson",
                    help="fixed kernels timed in the per-graph loop (the first is the reference line)")
    ap.add_argument("--batch-select", action="store_true",
                    help="batched path picks each graph's orientation (degree or A-direction) by its work estimate")
    ap.add_argument("--kcl-graphs", default="rgg:20:4-7,rmat:20:4-6,rmat:14:6-7",
                    help="comma list of kind:log2size:kmin-kmax (kind rmat or rgg)")
    ap.add_argument("--leg-batch-graphs", type=int, default=256,
                    help="tc mode: graphs of the reduced batch leg (every (4096 / N)-th graph of the 4096-graph "
                         "batch; 0 = no batch leg)")
    ap.add_argument("--no-select-leg", action="store_true", help="tc mode: skip the selector leg")
    ap.add_argument("--no-kcl-leg", action="store_true", help="tc mode: skip the k-clique leg")
    ap.add_argument("--prep-scale", type=int, default=20,
                    help="R-MAT scale of the reference preprocessing programs' timed run (0 = skip)")
    return ap.parse_args()


def workload_config(a):
    return {
        "workload": "R-MAT scale %d edge factor %d (a,b,c=.57,.19,.19) seed %d; A-order + A-direction; int32 CSR"
        % (a.scale, a.edge_factor, a.seed),
        "scale": a.scale,
        "edge_factor": a.edge_factor,
        "seed": a.seed,
        "direction": "A-direction",
        "ordering": "A-order",
        "l2": "CSR larger than L2 (129 MB); no flush between steps",
    }


# ---------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_for(cfg, kernel_name):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    rec = d.get("%s|scale%d" % (kernel_name, cfg["scale"]))
    return rec.get("dram_bytes_per_launch") if rec else None


def sharded_throughput(units, ms, part_count, dist=None, device="cpu"):
    """Whole-job throughput of a count sharded over the ranks (each rank counts one part of
    the same graph, atc_tc_part): the units are the graph's, counted once; the time is the
    slowest rank's; the count is the sum of the parts (the one collective of the path).
    Returns (units, max ms, units per second, total count)."""
    if dist is None:
        return units, ms, units / (ms * 1e-3), int(part_count)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([int(part_count)], dtype=torch.int64, device=device)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    worst = float(t.item())
    return units, worst, units / (worst * 1e-3), int(c.item())


def count_step(atc, csr, kernel, rank, world, sp, dist=None, device="cuda"):
    """One counting step: the whole count on one GPU, or this rank's part plus the sum of
    the parts over the ranks.  Returns (total count, stats of this rank's call)."""
    if world == 1:
        return atc.tc(csr, kernel, stream=sp)
    c, _, st = atc.tc_part(csr, rank, world, kernel, stream=sp)
    import torch
    t = torch.tensor([int(c)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item()), st


# ---------------------------------------------------------------------------------------
def cpu_baseline(g_lower_off, g_lower_cols, m_total, target_s):
    """Times the oracle's scalar-merge triangle count on a strided vertex sample."""
    import oracle
    n = g_lower_off.size - 1
    nthreads = os.cpu_count() or 1
    stride = max(1, n // 1024)
    for _ in range(3):  # calibrate the stride to about target_s seconds of CPU work
        t0 = time.perf_counter()
        oracle.tc_count_lower_sample(g_lower_off, g_lower_cols, stride, 1, nthreads)
        dt = time.perf_counter() - t0
        if dt > target_s / 4 or stride == 1:
            break
        stride = max(1, int(stride * dt / target_s * 1.2)) if dt > 0 else stride // 16
    if dt > 0:
        stride = max(1, int(round(stride * dt / target_s)))
    t0 = time.perf_counter()
    cnt, e = oracle.tc_count_lower_sample(g_lower_off, g_lower_cols, stride, 0, nthreads)
    dt = time.perf_counter() - t0
    # the same count on one host thread: successive phases of a fine stride (each call a few
    # thousand vertices) until about a third of the all-core time has passed, so the sample's
    # length is bounded by the clock and not by how its edges fall on a skewed graph
    stride1 = max(2, n // 4096)
    e1, dt1, calls = 0, 0.0, 0
    for phase in range(1, stride1):
        t0 = time.perf_counter()
        _, e_p = oracle.tc_count_lower_sample(g_lower_off, g_lower_cols, stride1, phase, 1)
        dt1 += time.perf_counter() - t0
        e1 += e_p
        calls += 1
        if dt1 >= target_s / 3:
            break
    return {"value": e / dt if dt > 0 else None, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "every %d-th vertex u (%d of %d) with all its smaller-neighbour edges (%d of %d edges); %.1f s"
            % (stride, (n + stride - 1) // stride, n, e, m_total, dt),
            "one_thread": {"value": e1 / dt1 if dt1 > 0 else None, "unit": UNIT, "cores": 1,
                           "sample": "phases 1..%d of every %d-th vertex u (%d edges), %.1f s" % (calls, stride1, e1, dt1)},
            "machine": os.uname().machine}


def reference_preprocessing(scale, edge_factor, seed, sp):
    """The reference's own preprocessing programs, A-direction-seri, A-order and costFuncCal
    (compiled from their sources into oracle/_ref; single-threaded, as written), run one after
    another on seeded R-MAT raw pairs of the given scale, each timed by the host wall clock,
    next to libatc's preTC (A-direction + A-order) of the same pairs from host memory."""
    import tempfile
    import atc
    import oracle
    ref = os.path.join(ROOT, "oracle", "_ref")
    progs = ("A-direction-seri", "A-order", "costFuncCal")
    if not all(os.path.exists(os.path.join(ref, p)) for p in progs):
        return {"unavailable": "reference programs not built (no reference sources here)"}
    raw = oracle.gen_rmat(scale, edge_factor, seed)
    out = {"graph": "R-MAT scale %d edge factor %d seed %d, %d raw pairs" % (scale, edge_factor, seed, raw.shape[0]),
           "threads": 1, "machine": os.uname().machine, "nproc": os.cpu_count()}
    with tempfile.TemporaryDirectory() as d:
        e = os.path.join(d, "E.bin")
        raw.tofile(e)
        lp = os.path.join(d, "lpBasedGraph.bin")
        for name, args in (("A-direction-seri", [e]), ("A-order", [lp]), ("costFuncCal", [lp, "1"])):
            t0 = time.perf_counter()
            r = subprocess.run([os.path.join(ref, name)] + args, cwd=d, stdout=subprocess.DEVNULL,
                               stderr=subprocess.DEVNULL, timeout=1200)
            out[name + "_s"] = time.perf_counter() - t0
            if r.returncode != 0:
                out[name + "_s"] = None
        m = os.path.getsize(lp) // 8 if os.path.exists(lp) else 0
    host = np.ascontiguousarray(raw)
    atc.pretc(host, atc.Dir.ADIRECTION, atc.Order.AORDER, stream=sp).free()  # warm
    t0 = time.perf_counter()
    c = atc.pretc(host, atc.Dir.ADIRECTION, atc.Order.AORDER, stream=sp)
    gpu_s = time.perf_counter() - t0
    out["edges"] = m
    out["libatc_pretc_s"] = gpu_s
    ref_s = sum(out[p + "_s"] or 0 for p in progs)
    out["reference_s"] = ref_s
    out["reference_edges_per_s"] = m / ref_s if ref_s else None
    out["libatc_edges_per_s"] = c.m / gpu_s if gpu_s else None
    c.free()
    return out


# ---------------------------------------------------------------------------------------
def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    t0 = time.perf_counter()
    raw = oracle.gen_rmat(a.scale, a.edge_factor, a.seed)  # the same bytes as libatc's generator
    loff, lcols = oracle.lower_csr(raw)
    m = int(loff[-1])
    setup = time.perf_counter() - t0
    nthreads = os.cpu_count() or 1
    n = loff.size - 1
    # stride so one step is about a.cpu_seconds / (steps + warmup) of work
    steps, warm = max(1, a.steps), max(0, a.warmup)
    per_step = max(0.5, a.cpu_seconds * 2 / (steps + warm))
    stride = max(1, n // 1024)
    for _ in range(3):  # calibrate the stride to about per_step seconds (phase 1: vertex 0 is the top hub)
        t1 = time.perf_counter()
        oracle.tc_count_lower_sample(loff, lcols, stride, 1, nthreads)
        dt = time.perf_counter() - t1
        if dt > per_step / 4 or stride == 1:
            break
        stride = max(1, int(stride * dt / per_step * 1.2)) if dt > 0 else stride // 16
    stride = max(1, int(round(stride * dt / per_step))) if dt > 0 else stride
    for i in range(warm):
        oracle.tc_count_lower_sample(loff, lcols, stride, i % stride, nthreads)
    edges, secs = 0, 0.0
    for i in range(steps):
        t1 = time.perf_counter()
        _, e = oracle.tc_count_lower_sample(loff, lcols, stride, (warm + i) % stride, nthreads)
        secs += time.perf_counter() - t1
        edges += e
    v = edges / secs if secs > 0 else None
    # the same count on one host thread, on a sparser sample of the same kind (vertex 0, the top
    # hub, is in phase 0 of every stride and is left out of both by starting at phase 1)
    stride1 = stride * max(1, nthreads)
    t1 = time.perf_counter()
    _, e1 = oracle.tc_count_lower_sample(loff, lcols, stride1, 1, 1)
    s1 = time.perf_counter() - t1
    cfg = workload_config(a)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": steps,
        "warmup": warm, "ms_per_step": secs / steps * 1e3, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded R-MAT)", "config": cfg,
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": "per step every %d-th vertex u with all its smaller-neighbour edges "
                                   "(OrgTriangleCount scalar merge, other_order/set_operation.cpp:129-144); "
                                   "graph build %.1f s untimed" % (stride, setup),
                         "one_thread": {"value": e1 / s1 if s1 > 0 else None, "unit": UNIT, "cores": 1,
                                        "sample": "every %d-th vertex u from vertex 1 (%d edges), %.1f s"
                                                  % (stride1, e1, s1)}},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "graph": {"n": int(n), "m": m},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
def run_ours(a):
    import torch
    import atc

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    atc.init(local)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    # ---- input: raw R-MAT samples generated on the device (every rank builds the same CSR)
    nraw = a.edge_factor << a.scale
    raw = torch.empty((nraw, 2), dtype=torch.int32, device="cuda")
    rc = atc.lib().atc_gen_rmat_device(a.scale, a.edge_factor, *atc.GRAPH500, a.seed, raw.data_ptr(), sp)
    assert rc == 0, atc.lib().atc_last_error()
    host_raw = torch.empty((nraw, 2), dtype=torch.int32, pin_memory=True)
    host_raw.copy_(raw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    csr = atc.pretc_device(raw.data_ptr(), nraw, atc.Dir.ADIRECTION, atc.Order.AORDER, stream=sp)
    pretc_s = time.perf_counter() - t0
    del raw
    torch.cuda.empty_cache()
    m = csr.m

    # ---- every kernel family once (count check + per-kernel time)
    kernels = {}
    counts = {}
    wanted = [x.strip().lower() for x in a.kernels.split(",") if x.strip()]
    for name in wanted:
        k = atc.Kernel[name.split("_")[0].upper()]
        tun = {"edge_kernels": 1} if name.endswith("_edge") else None
        atc.tc(csr, k, tuning=tun, stream=sp)
        c, st = atc.tc(csr, k, tuning=tun, stream=sp)
        counts[name] = c
        kernels[name] = {"ms": st.kernel_ms, "edges_per_s": m / (st.kernel_ms * 1e-3) if st.kernel_ms else None,
                         "hbm_frac_alg": st.alg_bytes / (st.kernel_ms * 1e-3) / 1e9 / measured_peak()[0]
                         if st.kernel_ms else None,
                         "hbm_frac_min": st.alg_bytes_min / (st.kernel_ms * 1e-3) / 1e9 / measured_peak()[0]
                         if st.kernel_ms else None}
    assert len(set(counts.values())) <= 1, counts
    best = min(kernels, key=lambda k: kernels[k]["ms"]) if kernels else None

    # ---- value: K steps of the headline kernel on the resident CSR
    head = atc.Kernel.AUTO
    # (N > 1: each rank counts one work-balanced part of the edges, atc_tc_part, and the
    # parts are summed over the ranks; the CSR is built on every rank)
    for _ in range(max(3, a.warmup)):
        count_step(atc, csr, head, rank, world, sp, dist)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kms = []
    launches = 0
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(a.steps):
            c, st = count_step(atc, csr, head, rank, world, sp, dist)
            kms.append(st.kernel_ms)
            launches += st.launches
        ev1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    total_ms = ev0.elapsed_time(ev1)
    _, total_ms, value, _ = sharded_throughput(m * a.steps, total_ms, 0, dist, "cuda")
    ms_step = total_ms / a.steps
    head_count = c
    assert all(v == head_count for v in counts.values()), (head_count, counts)
    # N > 1: a rank's part holds about 1/N of the work (the parts are balanced by it)
    alg = st.alg_bytes // world
    alg_min = st.alg_bytes_min // world
    kern_ms = statistics.mean(kms)
    peak, peak_kind = measured_peak()
    achieved = alg / (kern_ms * 1e-3) / 1e9

    # ---- e2e: public C ABI from pinned host buffers; the library's phase events give the
    # stage breakdown of each step
    e2e_ms = []
    stage_ms = {}
    for i in range(a.e2e_steps + 1 if a.e2e_steps > 0 else 0):
        atc.phase_timing(i > 0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w0 = time.perf_counter()
        c2 = atc.pretc_host_ptr(host_raw.data_ptr(), nraw, atc.Dir.ADIRECTION, atc.Order.AORDER, stream=sp)
        cnt, _ = count_step(atc, c2, head, rank, world, sp, dist)
        e1.record(stream)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - w0) * 1e3
        c2.free()
        assert cnt == head_count
        if i > 0:  # first pass warms the allocator pools
            e2e_ms.append(max(wall, e0.elapsed_time(e1)))
            for name, depth, ms in atc.phase_times():
                stage_ms.setdefault((depth, name), []).append(ms)
    atc.phase_timing(False)
    e2e_step = statistics.mean(e2e_ms) if e2e_ms else None
    stages = {("  " * d) + nm: statistics.mean(v) for (d, nm), v in stage_ms.items() if len(v) == len(e2e_ms)}
    top = sum(v for k, v in stages.items() if not k.startswith(" "))
    if dist and e2e_step is not None:
        e2e_step = sharded_throughput(m, e2e_step, 0, dist, "cuda")[1]
    e2e_value = m / (e2e_step * 1e-3) if e2e_step else None

    cfg = workload_config(a)
    kname = {1: "hu", 2: "bisson", 3: "fox", 4: "tricore"}.get(st.kernel_used, "auto")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded R-MAT generated on the device)", "config": cfg,
        "graph": {"n": csr.n, "m": m, "wedges": csr.wedges, "wedges_min": csr.wedges_min,
                  "max_outdeg": csr.max_outdeg, "triangles": head_count},
        "headline_kernel": kname, "fastest_kernel": best, "kernels": kernels,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic_for(cfg, kname), "peak_source": peak_kind,
                     "alg_bytes_per_launch": alg, "kernel_ms": kern_ms,
                     "alg_bytes_min_per_launch": alg_min,
                     "achieved_min": alg_min / (kern_ms * 1e-3) / 1e9,
                     "frac_min": alg_min / (kern_ms * 1e-3) / 1e9 / peak},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nraw * 8, "d2h_bytes_per_step": 8,
                "ms_per_step": e2e_step, "steps": len(e2e_ms),
                "stages_ms": stages,
                "stages_note": "device time between each library phase's start and end events on the step's stream "
                               "(indented = nested); unattributed = step time outside the top-level phases "
                               "(host work before the first and after the last event)",
                "unattributed_ms": (e2e_step - top) if e2e_step else None},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "pretc_s_first_call": pretc_s,
    }
    csr.free()
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and a.leg_batch_graphs > 0:
        step = max(1, 4096 // a.leg_batch_graphs)
        idx = list(range(0, 4096, step))[: a.leg_batch_graphs]
        line["batch_leg"] = batch_leg(a, idx, ["bisson", "hu"], sp, stream)
    if rank == 0 and world == 1 and not a.no_select_leg:
        line["select_leg"] = select_leg()
    if rank == 0 and world == 1 and not a.no_kcl_leg:
        line["kcl_leg"] = kcl_leg(sp)
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        import oracle
        off, cols = oracle.lower_csr(host_raw.numpy())
        line["cpu_baseline"] = cpu_baseline(off, cols, m, a.cpu_seconds)
        if a.prep_scale > 0:
            line["cpu_baseline"]["preprocessing"] = reference_preprocessing(a.prep_scale, a.edge_factor, a.seed, sp)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def kcl_cpu_sample(host_pairs, k, n, target_s):
    """CPU baseline of a k-clique count: the oracle's DFS on the first vertices r = 0, stride,
    2 stride, ... (rank order), all host threads.  The stride starts sparse (16 vertices) and is
    lowered from the measured time so that the sample takes about target_s; a sample already
    above a quarter of it is kept (per-vertex work is very uneven, so a denser one could take
    many times longer)."""
    import oracle
    stride = max(1, n // 16)
    for _ in range(4):
        t0 = time.perf_counter()
        _, ce = oracle.kclique_sample(host_pairs, k, stride, 0)
        dt = time.perf_counter() - t0
        if dt >= target_s / 4 or stride == 1:
            break
        stride = max(1, int(stride * max(dt, 1e-3) / target_s))
    return {"stride": stride, "edges": ce, "seconds": dt, "edges_per_s": ce / dt if dt > 0 else None,
            "cores": oracle.nthreads_default(), "kind": "port"}


def run_kcl(a):
    """k-clique counting, k = 4..7, on R-MAT and 2-D RGG graphs, A-direction orientation."""
    import ctypes as C
    import torch
    import atc
    import oracle
    torch.cuda.set_device(0)
    atc.init(0)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    out = []
    for spec in a.kcl_graphs.split(","):
        kind, lg, kr = spec.split(":")
        lg = int(lg)
        kmin, kmax = (int(x) for x in kr.split("-"))
        if kind == "rmat":
            npairs = a.edge_factor << lg
            dev = torch.empty((npairs, 2), dtype=torch.int32, device="cuda")
            assert atc.lib().atc_gen_rmat_device(lg, a.edge_factor, *atc.GRAPH500, a.seed, dev.data_ptr(), sp) == 0
            name = "R-MAT scale %d edge factor %d" % (lg, a.edge_factor)
        else:
            n = 1 << lg
            cnt = C.c_uint64(0)
            cap = n * 20
            dev = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
            assert atc.lib().atc_gen_rgg_device(n, 32.0, a.seed, dev.data_ptr(), cap, C.byref(cnt), sp) == 0
            npairs = int(cnt.value)
            name = "RGG n=2^%d mean degree 32" % lg
        csr = atc.pretc_device(dev.data_ptr(), npairs, atc.Dir.ADIRECTION, stream=sp)
        host_pairs = dev[:npairs].cpu().numpy()
        del dev
        rec = {"graph": name, "n": csr.n, "m": csr.m, "max_outdeg": csr.max_outdeg, "k": {}}
        for k in range(kmin, kmax + 1):
            atc.kcl(csr, k, stream=sp)  # warm-up
            times = []
            for _ in range(max(1, a.steps)):
                c, st = atc.kcl(csr, k, stream=sp)
                times.append(st.kernel_ms)
            ms = statistics.mean(times)
            entry = {"cliques": c, "ms": ms, "cliques_per_s": c / (ms * 1e-3), "edges_per_s": csr.m / (ms * 1e-3),
                     "alg_bytes": st.alg_bytes, "achieved_gbs": st.alg_bytes / (ms * 1e-3) / 1e9}
            if not a.no_cpu_baseline:
                entry["cpu_sample"] = kcl_cpu_sample(host_pairs, k, csr.n, a.cpu_seconds)
            rec["k"][str(k)] = entry
            print(json.dumps({"partial": name, "k": k, **entry}), file=sys.stderr, flush=True)
        out.append(rec)
        csr.free()
    peak, kind = measured_peak()
    print(json.dumps({"mode": "kcl", "metric": "k-clique counting, edges/s and cliques/s", "unit": "edges/s",
                      "dtype": "int32", "data": "synthetic (seeded, generated on the device)", "peak_gbs": peak,
                      "peak_source": kind, "graphs": out}), flush=True)


def batch_params(count, seed):
    """Seeded Chung-Lu parameters: gamma ~ U[2,3], n log-uniform in [1e3, 2e6], mean degree ~ U[4,64]."""
    import math
    import random
    rng = random.Random(seed)
    out = []
    for _ in range(count):
        gamma = rng.uniform(2.0, 3.0)
        n = int(round(math.exp(rng.uniform(math.log(1e3), math.log(2e6)))))
        d = rng.uniform(4.0, 64.0)
        out.append((n, gamma, min(d, n / 4.0)))
    return out


BATCH_CANDIDATES = [{}, {"bisson_warp_max": 128}, {"bisson_warp_max": 64, "bisson_cutover": 16},
                    {"bisson_warp_chunk": 256, "bisson_block_chunk": 1024},
                    {"bisson_warp_chunk": 2048, "bisson_block_chunk": 8192},
                    {"bisson_cutover": 64}, {"group_by_source": 1}, {"group_by_source": 1, "bisson_cutover": 8},
                    {"group_by_source": 2}, {"group_by_source": 2, "bisson_cutover": 64}]


def batch_leg(a, indices, plain_kernels, sp, stream=None, candidates=None):
    """Graphs `indices` of the seeded Chung-Lu batch (batch_params(4096, seed)) counted in one
    CUDA-graph replay (autotuned items) and, for comparison, one atc_tc call per graph with each
    of `plain_kernels` (host-synchronised, L2 flushed before each timed call)."""
    import ctypes as C
    import torch
    import atc
    allp = batch_params(max(4096, max(indices) + 1), a.seed)
    params = [(i, allp[i]) for i in indices]
    # sizes first, so the batch's union is allocated once
    tot_n = tot_m = 0
    for i, (n, gamma, d) in params:
        cnt = C.c_uint64(0)
        assert atc.lib().atc_gen_chunglu_device(n, gamma, d, a.seed * 100003 + i, None, 0, C.byref(cnt), sp) == 0
        tot_n += n
        tot_m += int(cnt.value)
    batch = atc.Batch()
    batch.reserve(tot_n, tot_m, stream=sp)
    kfixed = [atc.Kernel[x.strip().upper()] for x in plain_kernels]
    plain_ms = [[] for _ in kfixed]
    plain_dev = [[] for _ in kfixed]  # device time of the counting kernels of each call
    plain_counts = []
    dirs = []
    gstats = []  # (m, W, sum of min) of every graph as added
    wmin_adir = wmin_sel = 0
    # the per-graph calls are timed with L2 flushed before each (a graph counted right after
    # it was built or warmed would otherwise be read from L2, which a pass over many graphs,
    # and the batch, cannot do)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    t_setup = time.perf_counter()
    for i, (n, gamma, d) in params:
        pairs = atc.gen_chunglu_device(n, gamma, d, a.seed * 100003 + i, stream=sp)
        csr = atc.pretc_device(pairs.data_ptr(), pairs.shape[0], atc.Dir.ADIRECTION, stream=sp)
        for j, kf in enumerate(kfixed):
            atc.tc(csr, kf, stream=sp)  # warm
            flush.fill_(j)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            c, st = atc.tc(csr, kf, stream=sp)
            plain_ms[j].append((time.perf_counter() - t0) * 1e3)
            plain_dev[j].append(st.kernel_ms)
            if j == 0:
                plain_counts.append(c)
            else:
                assert c == plain_counts[-1]
        wmin_adir += csr.wedges_min
        chosen = csr
        dsel = "A-direction"
        if getattr(a, "batch_select", False):
            alt = atc.pretc_device(pairs.data_ptr(), pairs.shape[0], atc.Dir.DEGREE, stream=sp)
            if alt.wedges_min < csr.wedges_min:
                chosen, dsel = alt, "degree"
        wmin_sel += chosen.wedges_min
        gstats.append((chosen.m, chosen.wedges, chosen.wedges_min))
        dirs.append(dsel)
        batch.add(chosen, stream=sp)
        csr.free()
        if chosen is not csr:
            chosen.free()
        elif getattr(a, "batch_select", False):
            alt.free()
        del pairs
    del flush
    setup_s = time.perf_counter() - t_setup
    ng, n_all, m_all = batch.info()
    cands = candidates or BATCH_CANDIDATES
    best, tune_ms = batch.tune(cands, stream=sp)
    counts, _ = batch.run(stream=sp)
    assert counts.tolist() == plain_counts, "batched and per-graph counts differ"
    times = []
    for _ in range(max(1, a.steps)):
        _, st = batch.run(stream=sp)
        times.append(st.kernel_ms)
    batch_ms = statistics.mean(times)
    # the replay's stages, from the event nodes between them
    atc.phase_timing(True)
    try:
        batch.run(stream=sp)
        stages = {name: round(ms, 3) for name, _, ms in atc.phase_times() if name.startswith("batch.")}
    finally:
        atc.phase_timing(False)
    batch.free()
    # the batch's per-graph item mode (group_by_source = 2) by the library's cost model, and the
    # per-graph device times of the matching kernels, for the stages of the replay to be read against
    split = None
    names = [kf.name.lower() for kf in kfixed]
    if "hu" in names and "bisson" in names:
        hu_dev, bi_dev = plain_dev[names.index("hu")], plain_dev[names.index("bisson")]
        rows = [1.097 * w + 103.5 * m < 1.232 * wm + 117.5 * m for m, w, wm in gstats]
        split = {"rows_graphs": int(sum(rows)), "rows_edges": int(sum(g[0] for g, r in zip(gstats, rows) if r)),
                 "hu_device_ms_rows_graphs": float(sum(t for t, r in zip(hu_dev, rows) if r)),
                 "bisson_device_ms_grouped_graphs": float(sum(t for t, r in zip(bi_dev, rows) if not r)),
                 "bisson_device_ms_rows_graphs": float(sum(t for t, r in zip(bi_dev, rows) if r)),
                 "hu_device_ms_grouped_graphs": float(sum(t for t, r in zip(hu_dev, rows) if not r))}
    return {
        "metric": "graphs/s, batched (one CUDA-graph replay, autotuned items) vs per-graph loop",
        "unit": "graphs/s", "dtype": "int32", "data": "synthetic Chung-Lu graphs generated on the device",
        "subset": "graphs %s of the %d-graph batch" % (
            "all" if len(indices) == 4096 else "every %d-th" % (indices[1] - indices[0]) if len(indices) > 1 else
            str(indices), 4096),
        "graphs": ng, "vertices": n_all, "edges": m_all, "triangles": int(sum(plain_counts)),
        "plain": {kf.name.lower(): {"ms_total": sum(ms), "graphs_per_s": ng / (sum(ms) * 1e-3),
                                    "edges_per_s": m_all / (sum(ms) * 1e-3), "device_ms_total": sum(dv)}
                  for kf, ms, dv in zip(kfixed, plain_ms, plain_dev)},
        "plain_device_best_of_kernels_ms": float(sum(min(x) for x in zip(*plain_dev))) if plain_dev else None,
        "mode_split": split,
        "plain_note": "atc_tc per graph on its resident A-direction CSR, host-synchronised per call, L2 flushed "
                      "(256 MB written) before each timed call",
        "batched": {"ms_per_replay": batch_ms, "graphs_per_s": ng / (batch_ms * 1e-3),
                    "edges_per_s": m_all / (batch_ms * 1e-3), "tuned": cands[best],
                    "tune_ms": [float(x) for x in tune_ms], "stages_ms": stages,
                    "selection": "work estimate" if getattr(a, "batch_select", False) else "none",
                    "degree_chosen": dirs.count("degree"), "wedges_min_adirection": wmin_adir,
                    "wedges_min_selected": wmin_sel},
        "speedup_vs": {kf.name.lower(): sum(ms) / batch_ms for kf, ms in zip(kfixed, plain_ms)},
        "setup_s": setup_s,
    }


def run_batch(a):
    """Batched TC of seeded Chung-Lu graphs: one CUDA-graph replay for all graphs vs a per-graph loop."""
    import torch
    import atc
    torch.cuda.set_device(0)
    atc.init(0)
    sp = torch.cuda.current_stream().cuda_stream
    idx = list(range(a.batch_graphs)) if a.batch_graphs >= 4096 else \
        list(range(0, 4096, max(1, 4096 // a.batch_graphs)))[: a.batch_graphs]
    line = {"mode": "batch", **batch_leg(a, idx, [x.strip() for x in a.batch_plain_kernels.split(",")], sp)}
    print(json.dumps(line), flush=True)


def kcl_leg(sp):
    """The k-clique configuration's RGG (n = 2^20, mean degree 32, seed 1, A-direction) at
    k = 4..7: device time of one atc_kcl call per k (after a warm-up call), each count checked
    against the oracle's count pinned in tests/golden/config_pins.json."""
    import ctypes as C
    import torch
    import atc
    with open(os.path.join(ROOT, "tests", "golden", "config_pins.json")) as f:
        pins = json.load(f)["kcl"]["rgg20"]
    src = pins["source"]
    n = int(src["n"])
    cnt = C.c_uint64(0)
    cap = n * 20
    dev = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    assert atc.lib().atc_gen_rgg_device(n, float(src["mean_degree"]), int(src["seed"]), dev.data_ptr(), cap,
                                        C.byref(cnt), sp) == 0
    csr = atc.pretc_device(dev.data_ptr(), int(cnt.value), atc.Dir.ADIRECTION, stream=sp)
    del dev
    out = {"graph": "RGG n=2^20 mean degree 32 seed 1, A-direction", "n": csr.n, "m": csr.m, "k": {}}
    for k in range(4, 8):
        atc.kcl(csr, k, stream=sp)
        c, st = atc.kcl(csr, k, stream=sp)
        out["k"][str(k)] = {"cliques": c, "ms": st.kernel_ms, "cliques_per_s": c / (st.kernel_ms * 1e-3),
                            "matches_oracle": c == int(pins["cliques"][str(k)])}
    csr.free()
    torch.cuda.empty_cache()
    return out


def select_leg():
    """The learned selector trained on the committed timings fixture (640 seeded graphs, every
    (direction, ordering, kernel) triple timed on a GB300): policies on its held-out quarter."""
    path = os.path.join(ROOT, "tests", "golden", "select_timings.npz")
    d = np.load(path)
    feats, times, costs = d["features"], d["times_ms"], d["costs"]
    ntr = int(0.75 * feats.shape[0])
    t0 = time.perf_counter()
    res = train_and_evaluate(feats, times, costs, ntr, seed=1)
    res["train_s"] = time.perf_counter() - t0
    res["data"] = "tests/golden/select_timings.npz: %d training, %d held-out graphs" % (ntr, feats.shape[0] - ntr)
    return res


SEL_DIRS = ("ID", "DEGREE", "ADIRECTION")
SEL_ORDERS = ("NONE", "AORDER")
SEL_KERNELS = ("HU", "BISSON", "FOX", "TRICORE")


def set_select_space(name):
    """The config's direction x ordering x kernel space, or the extended one."""
    global SEL_DIRS, SEL_ORDERS
    if name == "extended":
        SEL_DIRS = ("ID", "DEGREE", "ADIRECTION", "KCORE", "ADIRECTION_PAR")
        SEL_ORDERS = ("NONE", "AORDER", "DEGREE_DESC")
    else:
        SEL_DIRS = ("ID", "DEGREE", "ADIRECTION")
        SEL_ORDERS = ("NONE", "AORDER")


def triple_name(i):
    d, rest = divmod(i, len(SEL_ORDERS) * len(SEL_KERNELS))
    o, k = divmod(rest, len(SEL_KERNELS))
    return "%s/%s/%s" % (SEL_DIRS[d], SEL_ORDERS[o], SEL_KERNELS[k])


def tail_cost(off, m):
    """costFuncCal's tail cost (tools/costFuncCal.cpp:66-81, k = 1) of an orientation."""
    n = off.size - 1
    avg = m / max(n, 1)
    dout = np.diff(off).astype(np.float64)
    sel = dout - avg > avg
    return float(np.abs(dout[sel] - avg).sum())


def select_graphs(count, seed):
    import math
    import random
    rng = random.Random(seed)
    out = []
    for i in range(count):
        if i % 2 == 0:
            n = int(round(math.exp(rng.uniform(math.log(1e3), math.log(2e5)))))
            out.append(("cl", n, rng.uniform(2.0, 3.0), min(rng.uniform(4.0, 64.0), n / 4.0)))
        else:
            out.append(("rmat", rng.randint(10, 17), rng.choice((8, 16, 32)), None))
    return out


def measure_graph(spec, gseed, sp):
    """Features, preTC+count time of every triple (inf where undefined), costs, count."""
    import atc
    kind, p1, p2, p3 = spec
    if kind == "cl":
        pairs = atc.gen_chunglu_device(p1, p2, p3, gseed, stream=sp)
    else:
        import torch
        pairs = torch.empty(((p2 << p1), 2), dtype=torch.int32, device="cuda")
        assert atc.lib().atc_gen_rmat_device(p1, p2, *atc.GRAPH500, gseed, pairs.data_ptr(), sp) == 0
    npairs = pairs.shape[0]
    feats = atc.graph_features(pairs.data_ptr(), npairs, stream=sp)
    T = len(SEL_DIRS) * len(SEL_ORDERS) * len(SEL_KERNELS)
    times = np.full(T, np.inf)
    costs = np.zeros(len(SEL_DIRS))
    counts = set()
    for di, d in enumerate(SEL_DIRS):
        for oi, o in enumerate(SEL_ORDERS):
            t0 = time.perf_counter()
            try:
                csr = atc.pretc_device(pairs.data_ptr(), npairs, atc.Dir[d], atc.Order[o], stream=sp)
            except atc.ATCError as e:
                if e.status == atc.Status.ERR_UNSUPPORTED:
                    continue
                raise
            t_pre = time.perf_counter() - t0
            if o == "NONE":
                off, _ = csr.to_host()
                costs[di] = tail_cost(off, csr.m)
            for ki, k in enumerate(SEL_KERNELS):
                t0 = time.perf_counter()
                c, _ = atc.tc(csr, atc.Kernel[k], stream=sp)
                times[(di * len(SEL_ORDERS) + oi) * len(SEL_KERNELS) + ki] = (t_pre + time.perf_counter() - t0) * 1e3
                counts.add(c)
            csr.free()
    assert len(counts) == 1, ("triples disagree", spec, counts)
    return feats, times, costs, counts.pop()


def evaluate_policies(times, choices):
    """Total time of each policy (dict name -> per-graph triple index) and its regret."""
    best = times.min(axis=1)
    out = {"oracle_best": {"ms": float(best.sum())}}
    for name, ch in choices.items():
        t = times[np.arange(times.shape[0]), ch]
        out[name] = {"ms": float(t.sum()), "regret": float(t.sum() / best.sum()),
                     "picked_best": float(np.mean(t <= best * 1.0000001))}
    return out


def selector_policies(train_t, eval_t, eval_costs, preds):
    """Choices of the non-learned baselines and of the network on the held-out graphs."""
    T = train_t.shape[1]
    finite = np.where(np.isfinite(train_t), train_t, np.nan)
    best_fixed = int(np.nanargmin(np.nansum(np.log(finite), axis=0) + np.isnan(finite).sum(axis=0) * 1e9))
    default = (SEL_DIRS.index("ADIRECTION") * len(SEL_ORDERS) + SEL_ORDERS.index("NONE")) * len(SEL_KERNELS) + \
        SEL_KERNELS.index("BISSON")
    cost_dir = eval_costs.argmin(axis=1)
    cost_choice = (cost_dir * len(SEL_ORDERS) + SEL_ORDERS.index("NONE")) * len(SEL_KERNELS) + SEL_KERNELS.index("BISSON")
    learned = np.where(np.isfinite(eval_t), preds, np.inf).argmin(axis=1)
    n = eval_t.shape[0]
    return {"fixed_default": np.full(n, default), "best_fixed_on_train": np.full(n, best_fixed),
            "cost_function": cost_choice, "learned": learned}, default, best_fixed


def run_select(a):
    """Learned (direction, ordering, kernel) selection on seeded Chung-Lu / R-MAT graphs."""
    import torch
    import atc
    torch.cuda.set_device(0)
    atc.init(0)
    sp = torch.cuda.current_stream().cuda_stream
    set_select_space(a.select_space)
    specs = select_graphs(a.select_train + a.select_eval, a.seed)
    measure_graph(("rmat", 10, 8, None), 999, sp)  # warm-up: module load, pools
    feats, times, costs = [], [], []
    t0 = time.perf_counter()
    for i, spec in enumerate(specs):
        f, t, c, _ = measure_graph(spec, a.seed * 7919 + i, sp)
        feats.append(f)
        times.append(t)
        costs.append(c)
    gen_s = time.perf_counter() - t0
    feats, times, costs = np.array(feats, np.float32), np.array(times), np.array(costs)
    if a.select_out:
        np.savez_compressed(a.select_out, features=feats, times_ms=times, costs=costs,
                            triples=np.array([triple_name(i) for i in range(times.shape[1])]))
    ntr = a.select_train
    result = train_and_evaluate(feats, times, costs, ntr, seed=a.seed)
    result.update({"mode": "select", "space": a.select_space, "triples": int(times.shape[1]),
                   "graphs_train": ntr, "graphs_eval": len(specs) - ntr,
                   "measure_s": gen_s, "data": "seeded Chung-Lu (n log-uniform 1e3..2e5) and R-MAT (scale 10..17)"})
    print(json.dumps(result), flush=True)


def train_and_evaluate(feats, times, costs, ntr, seed=1, epochs=300):
    """Trains the selector on the first ntr graphs, evaluates the policies on the rest."""
    import atc
    T = times.shape[1]
    mask = np.isfinite(times).astype(np.float32)
    target = np.where(mask > 0, np.log(np.where(mask > 0, times, 1.0)), 0.0).astype(np.float32)
    net = atc.MLP(6, 64, T, seed=seed)
    loss = net.train(feats[:ntr], target[:ntr], mask[:ntr], epochs=epochs, batch=256, lr=3e-3, seed=seed)
    preds = net.forward(feats[ntr:])
    choices, default, best_fixed = selector_policies(times[:ntr], times[ntr:], costs[ntr:], preds)
    ev = evaluate_policies(times[ntr:], choices)
    return {"metric": "total preTC+count time on held-out graphs by selection policy", "unit": "ms",
            "final_train_loss": loss, "default_triple": triple_name(default),
            "best_fixed_triple": triple_name(best_fixed), "policies": ev,
            "learned_vs_cost_function": ev["cost_function"]["ms"] / ev["learned"]["ms"],
            "learned_vs_default": ev["fixed_default"]["ms"] / ev["learned"]["ms"]}


def main():
    a = parse()
    if a.mode == "select":
        run_select(a)
        return
    if a.mode == "batch":
        run_batch(a)
        return
    if a.mode == "kcl":
        run_kcl(a)
        return
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
