"""Benchmark: TEPS of the sm_103a hash triangle counter on one GB300 (replicas for N > 1).

Workload (default): R-MAT scale 26, edge factor 32, (a,b,c,d) = (0.57,0.19,0.19,0.05), seed 3 — the
skewed, largest single-GPU graph (2.15e9 generated pairs, 2.08e9 oriented arcs after dedupe;
generated on the GPU, GPU-preprocessed to an oriented int32 CSR with int64 offsets).  A step is
one counting call over the whole graph.  Metric: TEPS = m / t, printed by the reference as GTEPS
(Without-graph-partition/mpi_main.cpp:115), for the library's default (learned) schedule, with the
plain degree-threshold schedule (the reference's USE_WARP/USE_CTA split), the tuned classes and an
autotuned launch measured in the same run, and the same graph counted as a 2x2 tile loop.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Rank 0 prints one JSON line.  `value` times the device-resident call (validation, classification,
scheduling, counting); `e2e` times the same call through the C ABI with pinned host buffers (H2D
copy and the result read inside the timed region); `roofline` relates the counting kernel's
algorithmic bytes to the measured HBM copy bandwidth; `cpu_baseline` is the CPU
forward-intersection counter; `gpu_launches` is the library's own launch counter over the timed
region.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "chung_lu_3.8m": dict(kind="chung_lu", n=3_800_000, gamma=2.5, w_max=800.0, target=16_500_000,
                          npairs=16_500_000, seed=2,
                          desc="Chung-Lu n=3.8M gamma=2.5 w_max=800 ~16.5M undirected edges seed=2"),
    "rmat16": dict(kind="rmat", scale=16, ef=16, a=0.57, b=0.19, c=0.19, seed=1,
                   desc="R-MAT scale 16 edge factor 16 (0.57,0.19,0.19,0.05) seed=1"),
    "rmat20": dict(kind="rmat", scale=20, ef=16, a=0.57, b=0.19, c=0.19, seed=3,
                   desc="R-MAT scale 20 edge factor 16 (0.57,0.19,0.19,0.05) seed=3"),
    "rmat22": dict(kind="rmat", scale=22, ef=16, a=0.57, b=0.19, c=0.19, seed=3,
                   desc="R-MAT scale 22 edge factor 16 (0.57,0.19,0.19,0.05) seed=3"),
    "rmat24_a070": dict(kind="rmat", scale=24, ef=16, a=0.70, b=0.125, c=0.125, seed=3, default_steps=20,
                        desc="R-MAT scale 24 edge factor 16 (0.70,0.125,0.125,0.05) seed=3 (cost model held out)"),
    "rmat26_ef32": dict(kind="rmat", scale=26, ef=32, a=0.57, b=0.19, c=0.19, seed=3, tiles=2, default_steps=20,
                        desc="R-MAT scale 26 edge factor 32 (0.57,0.19,0.19,0.05) seed=3"),
    "grid4096": dict(kind="grid", k=4096,
                     desc="4096 x 4096 grid with one diagonal per cell (triangulated mesh; cost model held out)"),
    "batch4096": dict(kind="batch", graphs=4096, nmin=50, nmax=50_000, seed=5, default_steps=50,
                      desc="4096 graphs, vertices log-uniform 50..50,000, alternately Erdos-Renyi (avg degree "
                           "4..64) and Barabasi-Albert (2..16 edges per vertex), seed=5"),
}
DEFAULT_WORKLOAD = "rmat26_ef32"
L2_FLUSH_BYTES = 256 << 20  # > 126 MB L2: written before every timed step (small graphs fit in L2)
BIG_ARCS = 1 << 28  # graphs this large take seconds per call: fewer repeats of the comparison runs
METRIC = "TEPS on 1 GB300: learned/autotuned vs plain TRUST schedule; % HBM roofline"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, burst copy)"
    return 6800.0, "fallback 6.8 TB/s"


def _traffic(workload):
    """(DRAM bytes of the counting kernels of one call, how they were obtained) from the committed
    ncu summaries (profiles/traffic.json), or (None, reason)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        e = d.get(workload)
        if e:
            return e.get("dram_bytes_per_call"), e.get("source")
    return None, "no ncu capture of this workload"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks", suffix=".csv")
        os.close(fd)
        try:
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.15)
        return self

    def __exit__(self, *exc):
        time.sleep(0.1)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.out.close()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for ln in f:
                    parts = [x.strip() for x in ln.split(",")]
                    if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                        rows.append(parts)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def max_over_ranks(x: float, dist, device) -> float:
    """The largest of every rank's x (the job's time is its slowest replica's); x itself when not
    distributed.  `device` holds the reduction tensor: "cuda" under NCCL, "cpu" under gloo."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gteps(ranks: int, edges: int, steps: int, total_ms: float) -> float:
    """Whole-job TEPS in G: every replica counts `edges` undirected edges per step."""
    return ranks * edges * steps / (total_ms * 1e-3) / 1e9


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_graph_gpu(w):
    """Synthetic graph on the GPU: generate pairs, preprocess to the oriented CSR (timed separately)."""
    import torch
    import trust_gb300 as T
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if w["kind"] == "chung_lu":
        pairs = T.gen_chung_lu(w["n"], w["gamma"], w["w_max"], w["target"], w["npairs"], seed=w["seed"])
        bound = w["n"]
    elif w["kind"] == "grid":
        pairs, bound = grid_pairs_gpu(w["k"]), w["k"] * w["k"]
    else:
        pairs = T.gen_rmat(w["scale"], w["ef"], w["a"], w["b"], w["c"], seed=w["seed"])
        bound = 1 << w["scale"]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    beg, adj = T.build_csr(pairs, bound)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    del pairs
    return beg, adj, {"generate_ms": (t1 - t0) * 1e3, "preprocess_ms": (t2 - t1) * 1e3}


def grid_pairs_gpu(k: int):
    """The k x k grid with one diagonal per cell (right, down and down-right neighbours) as an
    (npairs, 2) int32 CUDA tensor: 2 (k-1)^2 triangles."""
    import torch
    ids = torch.arange(k * k, dtype=torch.int32, device="cuda").view(k, k)
    e = [torch.stack([ids[:, :-1].reshape(-1), ids[:, 1:].reshape(-1)], 1),
         torch.stack([ids[:-1, :].reshape(-1), ids[1:, :].reshape(-1)], 1),
         torch.stack([ids[:-1, :-1].reshape(-1), ids[1:, 1:].reshape(-1)], 1)]
    return torch.cat(e).contiguous()


def workload_npairs(w) -> int:
    if w["kind"] == "chung_lu":
        return w["npairs"]
    if w["kind"] == "grid":
        return 3 * w["k"] * (w["k"] - 1)
    return w["ef"] << w["scale"]


def workload_pairs_cpu(w, npairs: int | None = None):
    """The first `npairs` (default all) of the workload's generated pairs and the id bound, from the
    CPU oracle's generators (counter-based: a prefix is the same pairs as in the whole stream)."""
    from oracle import oracle as O
    total = workload_npairs(w)
    k = total if npairs is None else min(npairs, total)
    if w["kind"] == "chung_lu":
        cdf = O.chung_lu_cdf(w["n"], w["gamma"], w["w_max"], w["target"])
        return O.gen_weighted(cdf, k, w["seed"]), w["n"]
    if w["kind"] == "grid":
        return grid_pairs_np(w["k"])[:k], w["k"] * w["k"]
    return O.gen_rmat(w["scale"], k, w["a"], w["b"], w["c"], w["seed"]), 1 << w["scale"]


def grid_pairs_np(k: int):
    import numpy as np
    ids = np.arange(k * k, dtype=np.int32).reshape(k, k)
    e = [np.stack([ids[:, :-1].ravel(), ids[:, 1:].ravel()], 1), np.stack([ids[:-1, :].ravel(), ids[1:, :].ravel()], 1),
         np.stack([ids[:-1, :-1].ravel(), ids[1:, 1:].ravel()], 1)]
    return np.concatenate(e).astype(np.int32)


def reference_preprocess(w, budget_s: float = 8.0):
    """The reference's CPU preprocessing of this path (Preprocess/fromDirectToUndirect.cpp then
    Preprocess/preprocess_outdegree.cpp, single-threaded as the reference runs it), restated in the
    oracle, timed on growing prefixes of the workload's pairs until one run takes `budget_s` / 4."""
    from oracle import oracle as O
    total = workload_npairs(w)
    npairs = min(total, 1 << 20)
    while True:
        pairs, _ = workload_pairs_cpu(w, npairs)
        t0 = time.perf_counter()
        k, edges = O.ref_undirect(pairs)
        O.ref_outdegree_csr(k, edges)
        t = time.perf_counter() - t0
        if t >= budget_s / 4 or npairs == total:
            break
        npairs = min(total, npairs * 4)
    return {"kind": "port", "cores": 1, "pairs": int(npairs), "of_pairs": int(total), "seconds": t,
            "mpairs_per_s": npairs / t / 1e6,
            "sample": "prefix of the workload's generated pairs: undirect (compact ids, dedupe) + orient by "
                      "degree + renumber + CSR, one thread"}


def make_graph_reference(w):
    """The workload's CSR for the reference arm, whose timed part is the CPU counter alone.  Built
    by the CPU oracle pipeline where that takes seconds; R-MAT 26 (2.15e9 pairs, hours for the
    single-threaded oracle pipeline) is built by the library's GPU preprocessing, outside the timed
    region, which equals the oracle pipeline byte for byte wherever both are run (tests)."""
    if workload_npairs(w) > (1 << 28) and w["kind"] != "batch":
        import torch
        torch.cuda.set_device(0)
        beg, adj, _ = make_graph_gpu(w)
        out = beg.cpu().numpy(), adj.cpu().numpy()
        del beg, adj
        torch.cuda.empty_cache()
        return out, "library GPU preprocessing (untimed input build)"
    return make_graph_cpu(w), "CPU oracle pipeline (untimed input build)"


def make_graph_cpu(w):
    """The same graph built by the CPU oracle (no product code on it)."""
    from oracle import oracle as O
    if w["kind"] == "batch":
        # the batch's first graphs, up to ~16M pairs, preprocessed one by one and concatenated
        import numpy as np
        from trust_gb300.batch import batch_specs
        begs, adjs, base, arcs, total = [], [], 0, 0, 0
        for sp in batch_specs(w["graphs"], w["nmin"], w["nmax"], w["seed"]):
            if total >= 16_000_000:
                break
            b, a = O.build_csr(O.batch_graph_pairs(sp.kind, sp.n, sp.param, sp.npairs, sp.seed), sp.n)
            begs.append(b[:-1] + arcs)
            adjs.append(a + base)
            base += b.size - 1
            arcs += a.size
            total += sp.npairs
        return np.concatenate(begs + [np.array([arcs], dtype=np.int64)]), np.concatenate(adjs)
    pairs, bound = workload_pairs_cpu(w)
    return O.build_csr(pairs, bound)


def sample_stride(beg_np, adj_np, threads: int, target_s: float, start_stride: int = 1 << 16):
    """The smallest power-of-two row stride (from start_stride down to 1) at which one strided
    sample of the oracle counter takes at least target_s: (stride, seconds, count, arcs)."""
    from oracle import oracle as O
    stride = start_stride
    while True:
        t0 = time.perf_counter()
        c, arcs = O.count_forward_stride(beg_np, adj_np, 0, stride, 2, threads)
        t = time.perf_counter() - t0
        if t >= target_s or stride == 1:
            return stride, t, c, arcs
        stride = max(1, stride // 4 if t < target_s / 8 else stride // 2)


def cpu_baseline(beg_np, adj_np, budget_s: float = 16.0):
    """The oracle's forward-intersection counter on every host core (rows are already sorted by the
    preprocessing, so no per-row sort is timed).  Small graphs: the whole graph, repeated within the
    budget.  Large graphs: a systematic sample (every S-th source row, S a power of two chosen so a
    sample takes about a quarter of the budget), so every degree class is represented; TEPS = the
    sampled rows' arcs / time.  Returns (baseline, whole-graph count or None)."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    n = beg_np.size - 1
    m = adj_np.size
    stride, t, c, arcs = sample_stride(beg_np, adj_np, threads, budget_s / 4)
    times, count = [t], (c if stride == 1 else None)
    t_start = time.perf_counter()
    while len(times) < 5 and (time.perf_counter() - t_start) < budget_s / 2:
        t0 = time.perf_counter()
        O.count_forward_stride(beg_np, adj_np, len(times) % stride, stride, 2, threads)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    sample = (f"whole graph, {len(times)} runs (median {t * 1e3:.1f} ms)" if stride == 1 else
              f"every {stride}th source row ({arcs} of {m} arcs per sample), {len(times)} samples (median "
              f"{t:.2f} s)")
    return {"value": (m if stride == 1 else arcs) / t / 1e9, "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": sample + f", forward intersection over presorted rows, {threads} threads",
            "single_core": single_core_counter(beg_np, adj_np)}, count


def single_core_counter(beg_np, adj_np, budget_s: float = 3.0):
    """The same counter on one core over a strided row sample (GTEPS of the arcs covered)."""
    stride, t, _, arcs = sample_stride(beg_np, adj_np, 1, budget_s / 2, start_stride=1 << 20)
    n = beg_np.size - 1
    return {"gteps": arcs / t / 1e9, "cores": 1,
            "sample": f"every {stride}th source row of {n} ({arcs} arcs), {t:.2f} s"}


def pinned_count(workload):
    """A whole-graph count of the workload pinned by a CPU oracle run (tests/golden/pinned_counts.json)."""
    p = os.path.join(ROOT, "tests", "golden", "pinned_counts.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f).get(workload)


def run_ours(args, ws, rank, local):
    import torch
    import trust_gb300 as T

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = WORKLOADS[args.workload]
    beg, adj, prep = make_graph_gpu(w)
    n, m = beg.numel() - 1, adj.numel()
    stream = torch.cuda.current_stream()
    ctx = T.Context(local)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    lib = T.load()

    def call(schedule=T.SCHED_LEARNED):
        return T.count_csr(beg, adj, ctx=ctx, stream=stream.cuda_stream, schedule=schedule)

    for _ in range(args.warmup):
        r = call()
    expect_count = r.triangles
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    res = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.trust_tc_kernel_launches()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.fill_(i)
            ev[i][0].record(stream)
            res.append(call())
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    launches = lib.trust_tc_kernel_launches() - launches0
    if dist:
        dist.barrier()
    clocks = clk.summary()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    total_ms = max_over_ranks(total_ms, dist, "cuda")
    ok = all(r.triangles == expect_count for r in res)
    count_s = statistics.median(r.count_seconds for r in res)
    kernel_s = statistics.median(r.kernel_seconds for r in res)
    wedges = res[0].wedges

    # the same call under the other schedules (same flush discipline), for the learned-vs-plain ratio
    sched = {"learned": {"gteps": m / (statistics.median(step_ms) * 1e-3) / 1e9,
                         "ms": statistics.median(step_ms), "direction_split": res[0].direction_split,
                         "predicted_split_saving_ms": res[0].split_saving_ms}}
    big = m >= BIG_ARCS  # a call takes seconds: bounded comparison runs and autotuner budget
    t_tune = time.perf_counter()
    tuned_cfg, _ = T.autotune(beg, adj, ctx, repeats=1 if big else 3,
                              time_budget_s=24.0 if big else 0.0)  # outside every timed region
    autotune_s = time.perf_counter() - t_tune
    # gate_only: the tuned classes with the direction split decided by the learned schedule's gate
    # alone (at least 2^22 arcs, a row of at least 64 entries, at least 15 % of the arcs in rows
    # longer than 128), no network: no promotions, no heaviest-first order
    deg = beg[1:] - beg[:-1]
    gate = bool(m >= (1 << 22) and int(deg.max()) >= 64 and int(deg[deg > 128].sum()) >= 0.15 * m)
    runs = (("autotuned", lambda: T.count_csr(beg, adj, ctx=ctx, stream=stream.cuda_stream, **tuned_cfg)),
            ("gate_only", lambda: T.count_csr(beg, adj, ctx=ctx, stream=stream.cuda_stream, schedule=T.SCHED_TUNED,
                                              direction_split=1 if gate else 0)),
            ("tuned", lambda: call(T.SCHED_TUNED)), ("plain", lambda: call(T.SCHED_PLAIN)))
    for name, fn in runs:
        fn()
        ms = []
        for i in range(3 if big else max(5, args.steps // 10)):
            flush.fill_(i)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r3 = fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
            ok = ok and r3.triangles == expect_count
        sched[name] = {"gteps": m / (statistics.median(ms) * 1e-3) / 1e9, "ms": statistics.median(ms),
                       "count_kernel_ms": r3.count_seconds * 1e3}
        if name == "autotuned":
            sched[name]["launch"] = tuned_cfg
            sched[name]["autotune_s"] = autotune_s
        if name == "gate_only":
            sched[name]["gate_passes"] = gate

    # the n x n tile loop on the same graph (once per mode, outside the timed region): tiles in HBM
    # under the learned and the plain schedule, and streamed through a 3.5-tile device budget
    tiles = args.tiles if args.tiles is not None else w.get("tiles", 0)
    tile_loop = None
    if tiles > 1:
        tile_bytes = (8 * (n + 1) + 4 * m) // (tiles * tiles)
        tile_loop = {"parts": tiles, "jobs": tiles ** 3}
        for name, sch, budget in (("learned", T.SCHED_LEARNED, 0), ("plain", T.SCHED_PLAIN, 0),
                                  ("learned_streamed", T.SCHED_LEARNED, 3 * tile_bytes + (tile_bytes >> 1))):
            rt = T.count_tiles(beg, adj, tiles, budget_bytes=budget, schedule=sch)
            ok = ok and rt.triangles == expect_count
            tile_loop[name] = {"s": rt.call_seconds, "gteps": m / rt.call_seconds / 1e9,
                               "split_jobs": rt.direction_split, "wedges": rt.wedges, "budget_bytes": budget}
        tile_loop["learned_vs_plain"] = tile_loop["plain"]["s"] / tile_loop["learned"]["s"]

    # end to end through the C ABI: pinned host buffers, every step's H2D copy, count and result
    # read inside the timed region.  Serial: copy then count, one call per step.  Pipelined (the
    # reported e2e): step i+1's copy is staged on the context's copy stream (trust_tc_stage_csr)
    # before step i is counted, as a caller streaming graphs does; L2 flushed before every count.
    hb = beg.cpu().pin_memory()
    ha = adj.cpu().pin_memory()
    hb_np, ha_np = hb.numpy(), ha.numpy()
    e2e_ev = []
    k_e2e = 3 if big else max(3, args.steps // 4)
    warm_e2e = 1 if big else 2
    for i in range(k_e2e + warm_e2e):
        flush.fill_(i)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        r2 = T.count_csr(hb_np, ha_np, ctx=ctx, stream=stream.cuda_stream)
        b.record(stream)
        ok = ok and r2.triangles == expect_count
        e2e_ev.append((a, b))
    torch.cuda.synchronize()
    e2e_ms = [a.elapsed_time(b) for a, b in e2e_ev[warm_e2e:]]
    e2e_serial_mean = statistics.mean(e2e_ms)
    pipe_ms = []
    for rep in range(2):  # the first pass warms the staging buffers
        k_rep = (2 if big else k_e2e) if rep == 0 else k_e2e
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        t0.synchronize()  # the region starts before the first copy is issued
        T.stage_csr(hb_np, ha_np, ctx)
        for i in range(k_rep):
            if i + 1 < k_rep:
                T.stage_csr(hb_np, ha_np, ctx)
            flush.fill_(i)
            r2 = T.count_csr(hb_np, ha_np, ctx=ctx, stream=stream.cuda_stream)
            ok = ok and r2.triangles == expect_count
        t1.record(stream)
        torch.cuda.synchronize()
        pipe_ms.append(t0.elapsed_time(t1) / k_rep)
    e2e_mean = pipe_ms[-1]

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_src = _peaks()
    algo_bytes = 24 * m + 8 * (n + 1) + 4 * wedges
    achieved = algo_bytes / count_s / 1e9
    line = {
        "metric": METRIC,
        "value": job_gteps(ws, m, args.steps, total_ms),
        "unit": "GTEPS",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic (seeded generator on the GPU, GPU-preprocessed oriented CSR); no dataset download",
        "config": {"workload": w["desc"], "vertices": n, "edges": m, "wedges": wedges, "triangles": expect_count,
                   "schedule": "learned (library default)", "class_sizes": res[0].class_sizes,
                   "parallelism": f"replicas x{ws}",
                   "l2": f"{L2_FLUSH_BYTES >> 20} MiB buffer written before every timed step (graph "
                         f"{(8 * (n + 1) + 4 * m) / 1e6:.0f} MB"
                         + (", fits in L2)" if 8 * (n + 1) + 4 * m < 126e6 else ", larger than L2)")},
        "schedules": sched,
        "learned_vs_plain": sched["learned"]["gteps"] / sched["plain"]["gteps"],
        "learned_vs_gate_only": sched["learned"]["gteps"] / sched["gate_only"]["gteps"],
        "counts_consistent": ok,
        "kernel_ms": kernel_s * 1e3,
        "count_kernel_ms": count_s * 1e3,
        "gpu_launches": int(launches),
        "e2e": {"value": m / (e2e_mean * 1e-3) / 1e9, "unit": "GTEPS",
                "h2d_bytes_per_step": 8 * (n + 1) + 4 * m, "d2h_bytes_per_step": int(lib.trust_tc_readback_bytes()),
                "ms_per_step": e2e_mean, "steps": k_e2e,
                "mode": "pipelined: step i+1's H2D copy staged on the library's copy stream while step i "
                        "is counted; L2 flushed before every count; region from before the first copy "
                        "to after the last result read",
                "serial": {"value": m / (e2e_serial_mean * 1e-3) / 1e9, "ms_per_step": e2e_serial_mean}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": _traffic(args.workload)[0], "traffic_source": _traffic(args.workload)[1],
                     "peak_source": peak_src,
                     "algorithmic_bytes": algo_bytes,
                     "bytes_formula": "24 m + 8 (n+1) + 4 W (W = wedges = probes made, both passes of the "
                                      "direction split); time = the counting kernels' wall span (count_kernel_ms)"},
        "preprocess": {"gpu_generate_ms": prep["generate_ms"], "gpu_build_csr_ms": prep["preprocess_ms"]},
        "clocks": clocks,
    }
    if tile_loop:
        line["tile_loop"] = tile_loop
    if ws == 1 and not args.no_cpu_baseline:
        cb, cpu_count = cpu_baseline(hb_np, ha_np)
        line["cpu_baseline"] = cb
        if cpu_count is not None:
            line["count_matches_oracle"] = cpu_count == expect_count
    pinned = pinned_count(args.workload)
    if pinned is not None:
        line["count_matches_pinned"] = {"pinned": pinned["triangles"], "equal": pinned["triangles"] == expect_count,
                                        "source": pinned["source"]}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_batch(args, ws, rank, local):
    """The batch workload: every graph counted by one CUDA-graph launch (autotuned per size class),
    against the plain schedule called once per graph through the public API."""
    import numpy as np
    import torch
    import trust_gb300 as T
    from trust_gb300 import batch as B

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    t0 = time.perf_counter()
    specs = B.batch_specs(w["graphs"], w["nmin"], w["nmax"], w["seed"])
    pairs, vbeg = B.gen_batch_pairs(specs)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    beg, adj, gv = B.build_batch(pairs, vbeg)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    del pairs
    n, m = beg.numel() - 1, adj.numel()
    ctx = T.Context(local)
    stream = torch.cuda.current_stream()
    bt = B.Batch(beg, adj, gv, ctx=ctx)
    default_ms = statistics.median(bt.run(stream.cuda_stream)[1].call_seconds for _ in range(3)) * 1e3
    t3 = time.perf_counter()
    tuned_kernel_ms = bt.autotune(repeats=2)
    autotune_s = time.perf_counter() - t3
    lib = T.load()
    for _ in range(args.warmup):
        expect, r = bt.run(stream.cuda_stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    steps = min(args.steps, 50)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    ok = True
    torch.cuda.synchronize()
    launches0 = lib.trust_tc_kernel_launches()
    with ClockSampler(local) as clk:
        for i in range(steps):
            flush.fill_(i)
            ev[i][0].record(stream)
            c, r = bt.run(stream.cuda_stream)
            ev[i][1].record(stream)
            ok = ok and np.array_equal(c, expect)
        torch.cuda.synchronize()
    launches = lib.trust_tc_kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    # end to end: the batch CSR from pinned host memory into the batch's device buffers, the
    # captured job, the per-graph counts back on the host
    hb, ha = beg.cpu().pin_memory(), adj.cpu().pin_memory()
    e2e = []
    for i in range(7):
        flush.fill_(i)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        beg.copy_(hb, non_blocking=True)
        adj.copy_(ha, non_blocking=True)
        c, _ = bt.run(stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        ok = ok and np.array_equal(c, expect)
        e2e.append(a.elapsed_time(b))
    e2e_serial_ms = statistics.median(e2e[2:])
    # pipelined: a second batch over a second pair of device buffers (same graphs, same per-class
    # launches); the copy of step i+1 into one pair runs on a copy stream while step i counts the
    # other (each run re-validates and re-classifies what its buffers hold)
    beg2, adj2 = torch.empty_like(beg), torch.empty_like(adj)
    beg2.copy_(beg)
    adj2.copy_(adj)
    bt2 = B.Batch(beg2, adj2, gv, ctx=T.Context(local))
    for s_ in range(4):
        bt2.set_class(s_, **bt.get_class(s_))
    bufs, jobs = ((beg, adj), (beg2, adj2)), (bt, bt2)
    copy_stream = torch.cuda.Stream()
    k_pipe = 8
    copied = [torch.cuda.Event(), torch.cuda.Event()]
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    p0.synchronize()
    def stage(i):
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_stream(stream) if i >= 2 else None  # the buffers' previous run is done
            bufs[i % 2][0].copy_(hb, non_blocking=True)
            bufs[i % 2][1].copy_(ha, non_blocking=True)
            copied[i % 2].record(copy_stream)
    stage(0)
    for i in range(k_pipe):
        if i + 1 < k_pipe:
            stage(i + 1)
        stream.wait_event(copied[i % 2])
        flush.fill_(i)
        c, _ = jobs[i % 2].run(stream.cuda_stream)
        ok = ok and np.array_equal(c, expect)
    p1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = p0.elapsed_time(p1) / k_pipe
    bt2.close()
    del beg2, adj2
    # one persistent launch over the whole union (every graph's rows in one count call, tuned
    # classes, no per-graph attribution): what a single launch for all size classes would cost
    union_ms = []
    for i in range(5):
        flush.fill_(i)
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record(stream)
        ru = T.count_csr(beg, adj, ctx=ctx, stream=stream.cuda_stream, schedule=T.SCHED_TUNED)
        b_.record(stream)
        torch.cuda.synchronize()
        union_ms.append(a_.elapsed_time(b_))
        ok = ok and ru.triangles == int(expect.sum())
    # the plain schedule, one call per graph (device-resident per-graph CSRs made beforehand)
    per = [B.graph_csr(beg, adj, gv, g) for g in range(gv.size - 1)]
    torch.cuda.synchronize()
    loop_ms = []
    for _ in range(2):
        tl = time.perf_counter()
        tot = 0
        for gb, ga in per:
            if ga.numel():
                tot += T.count_csr(gb, ga, ctx=ctx, stream=stream.cuda_stream, schedule=T.SCHED_PLAIN).triangles
        torch.cuda.synchronize()
        loop_ms.append((time.perf_counter() - tl) * 1e3)
    ok = ok and tot == int(expect.sum())
    info = bt.info()
    if rank != 0:
        return
    peak, peak_src = _peaks()
    count_s = tuned_kernel_ms * 1e-3
    algo_bytes = 24 * m + 8 * (n + 1) + 4 * r.wedges
    line = {
        "metric": METRIC,
        "value": job_gteps(ws, m, steps, total_ms),
        "unit": "GTEPS",
        "n_gpus": ws,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic (counter-based generators on the GPU, GPU-preprocessed batch CSR); no dataset download",
        "config": {"workload": w["desc"], "graphs": int(gv.size - 1), "vertices": n, "edges": m,
                   "wedges": r.wedges, "triangles": int(expect.sum()),
                   "schedule": "batched: one CUDA-graph launch, per-size-class autotuned",
                   "size_classes": {"graphs": info["graphs"], "vertices": info["vertices"],
                                    "launch": [bt.get_class(s) for s in range(4)]},
                   "parallelism": f"replicas x{ws}",
                   "l2": f"{L2_FLUSH_BYTES >> 20} MiB buffer written before every timed step"},
        "schedules": {"batched_autotuned": {"gteps": m / (statistics.median(step_ms) * 1e-3) / 1e9,
                                            "ms": statistics.median(step_ms)},
                      "batched_default": {"gteps": m / (default_ms * 1e-3) / 1e9, "ms": default_ms},
                      "union_one_launch": {"gteps": m / (statistics.median(union_ms) * 1e-3) / 1e9,
                                           "ms": statistics.median(union_ms),
                                           "note": "the union CSR in one count call (tuned classes), total "
                                                   "only: no per-graph counts"},
                      "plain_loop_per_graph": {"gteps": m / (min(loop_ms) * 1e-3) / 1e9, "ms": min(loop_ms)}},
        "learned_vs_plain": min(loop_ms) / statistics.median(step_ms),
        "counts_consistent": ok,
        "autotune_s": autotune_s,
        "count_kernel_ms": tuned_kernel_ms,
        "gpu_launches": int(launches),
        "e2e": {"value": m / (e2e_ms * 1e-3) / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": 8 * (n + 1) + 4 * m,
                "d2h_bytes_per_step": 8 * int(gv.size - 1) + 4 * int(lib.trust_tc_readback_bytes()),
                "ms_per_step": e2e_ms, "steps": k_pipe,
                "mode": "pipelined: two batches over two device buffer pairs; step i+1's H2D copy on a copy "
                        "stream while step i counts; L2 flushed before every run; region from before the "
                        "first copy to after the last per-graph counts read",
                "serial": {"value": m / (e2e_serial_ms * 1e-3) / 1e9, "ms_per_step": e2e_serial_ms}},
        "roofline": {"bound": "hbm", "achieved": algo_bytes / count_s / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": algo_bytes / count_s / 1e9 / peak, "traffic": None, "peak_source": peak_src,
                     "algorithmic_bytes": algo_bytes,
                     "bytes_formula": "24 m + 8 (n+1) + 4 W over the size classes' count kernels"},
        "preprocess": {"gpu_generate_ms": (t1 - t0) * 1e3, "gpu_build_batch_ms": (t2 - t1) * 1e3},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_reference(args, ws, rank, local):
    """The reference's CPU-side counting for this path: it ships no CPU counter, so the oracle port of
    its counted quantity runs on every host core.  Each step counts a bounded systematic sample of
    the workload (every S-th source row, the offset advancing per step; S = 1 on graphs whose whole
    count takes about a second or less), so the whole run ends within minutes.  Where the reference
    kernel cubin is present (built from Without-graph-partition/TC.cu for sm_103a) its GPU time on
    the same CSR is reported beside it."""
    if rank != 0:
        return
    from oracle import oracle as O
    w = WORKLOADS[args.workload]
    if w["kind"] == "batch":
        (beg, adj), how = make_graph_cpu(w), "CPU oracle pipeline (untimed input build)"
    else:
        (beg, adj), how = make_graph_reference(w)
    n, m = beg.size - 1, adj.size
    threads = os.cpu_count() or 1
    stride, _, _, _ = sample_stride(beg, adj, threads, 1.5)
    for i in range(args.warmup):
        O.count_forward_stride(beg, adj, i % stride, stride, 2, threads)
    tot_arcs, tot_t = 0, 0.0
    for i in range(args.steps):
        t0 = time.perf_counter()
        _, arcs = O.count_forward_stride(beg, adj, (args.warmup + i) % stride, stride, 2, threads)
        tot_t += time.perf_counter() - t0
        tot_arcs += arcs
    value = tot_arcs / tot_t / 1e9
    sample = ("the whole graph per step" if stride == 1 else
              f"every {stride}th source row per step (offset advancing per step, ~{m // stride} arcs)")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value, "unit": "GTEPS", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot_t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generators); input CSR: " + how,
        "config": {"workload": w["desc"], "vertices": n, "edges": m, "schedule": "n/a: CPU forward intersection"},
        "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": sample + f", forward intersection over presorted rows, {threads} threads"},
        "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    line["cpu_baseline"]["single_core"] = single_core_counter(beg, adj)
    if w["kind"] != "batch":
        line["reference_preprocess"] = reference_preprocess(w)
    if not O.ref_kernel_available():
        line["reference_kernel_sm103a"] = {"unavailable": "reference kernel cubin not built here (oracle/build_ref.sh "
                                                          "needs the reference sources)"}
    else:
        flags, _ = O.trust_check(beg, adj)
        if flags == O.TRUST_EXACT:
            try:
                runs = [O.ref_kernel_count(beg, adj, blocks=1024, chunk=1) for _ in range(3)]
            except (OSError, RuntimeError) as e:  # no CUDA driver or no visible device on this host
                runs = None
                line["reference_kernel_sm103a"] = {"unavailable": f"reference kernel not run: {e}"}
            if runs:
                ms = statistics.median(r[1] for r in runs)
                line["reference_kernel_sm103a"] = {"gteps": m / (ms * 1e-3) / 1e9, "kernel_ms": ms,
                                                   "count": runs[0][0],
                                                   "launch": "dynamic_assign<<<1024,1024>>> chunk 1 (README example)"}
        else:
            line["reference_kernel_sm103a"] = {"unavailable": f"reference kernel not exact on this CSR (flags {flags})"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 20 for R-MAT 24/26, whose calls take 0.17-2.3 s; 50 for the "
                         "batch; 200 otherwise)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tiles", type=int, default=None,
                    help="also run the parts x parts tile loop (default: 2 for rmat26_ef32, else off)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = WORKLOADS[args.workload].get("default_steps", 200)
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = _dist()
    if args.impl == "reference":
        run_reference(args, ws, rank, local)
    elif WORKLOADS[args.workload]["kind"] == "batch":
        run_batch(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
