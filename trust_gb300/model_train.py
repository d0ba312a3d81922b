"""Train the learned schedule's cost model on the GPU and compile it into the library.

    python -m trust_gb300.model_train [--out trust_gb300/csrc/tc_model_default.inc] [--report FILE]

Training set: 16 generated graphs - R-MAT scales 18-22 with a in {0.45, 0.57, 0.70} (d = 0.05,
b = c) and Chung-Lu degree exponents 2.1-3.0 - each preprocessed on the GPU into an oriented CSR.
For every vertex with out-degree >= 2 the counting kernel records its clock64 cycles
(tuned schedule, no direction split) and trust_tc_vertex_features gives its 8 features; the
target is log2(cycles).  The MLP is trained by the library's own CUDA forward/backward/Adam
kernels.  Held out: R-MAT scale 24 with a = 0.70 and the 4096 x 4096 triangulated grid (one
diagonal per cell).  The report gives the predictor's error per graph and, for the held-out graphs,
the time and TEPS of one counting call under the learned schedule (with the trained model), the
gate alone (tuned classes, direction split exactly when the learned schedule's gate passes), the
tuned classes and TRUST's plain split.

    python -m trust_gb300.model_train --held-out-only --report FILE

times the held-out graphs with the model compiled into the library and replaces the report's
held-out entries, without training.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import trust_gb300 as T  # noqa: E402

TRAIN = [("rmat", 18, 0.45), ("rmat", 18, 0.57), ("rmat", 18, 0.70), ("rmat", 19, 0.45), ("rmat", 19, 0.57),
         ("rmat", 19, 0.70), ("rmat", 20, 0.45), ("rmat", 20, 0.57), ("rmat", 20, 0.70), ("rmat", 21, 0.57),
         ("rmat", 21, 0.70), ("rmat", 22, 0.57), ("chung_lu", 2.1, 0), ("chung_lu", 2.4, 0), ("chung_lu", 2.7, 0),
         ("chung_lu", 3.0, 0)]
HELD_OUT = [("rmat", 24, 0.70), ("grid", 4096, 0)]


def make_graph(kind, p1, p2, seed):
    import torch
    if kind == "rmat":
        a = p2
        b = c = (1.0 - a - 0.05) / 2
        pairs = T.gen_rmat(p1, 16, a, b, c, seed=seed)
        bound = 1 << p1
    elif kind == "chung_lu":
        n = 1_000_000
        pairs = T.gen_chung_lu(n, p1, 1000.0, 4_000_000, 4_000_000, seed=seed)
        bound = n
    else:  # triangulated grid: right, down and one diagonal per cell
        k = p1
        ids = torch.arange(k * k, dtype=torch.int32, device="cuda").view(k, k)
        e = [torch.stack([ids[:, :-1].reshape(-1), ids[:, 1:].reshape(-1)], 1),
             torch.stack([ids[:-1, :].reshape(-1), ids[1:, :].reshape(-1)], 1),
             torch.stack([ids[:-1, :-1].reshape(-1), ids[1:, 1:].reshape(-1)], 1)]
        pairs = torch.cat(e).contiguous()
        bound = k * k
    beg, adj = T.build_csr(pairs, bound)
    return beg, adj


def samples(beg, adj, ctx):
    import torch
    n = beg.numel() - 1
    cyc = torch.zeros(n, dtype=torch.int64, device="cuda")
    T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED, direction_split=0)  # warm
    r = T.count_csr(beg, adj, ctx=ctx, cycles=cyc, schedule=T.SCHED_TUNED, direction_split=0)
    f = T.vertex_features(beg, adj, ctx)
    deg = (beg[1:] - beg[:-1])
    sel = (deg >= 2) & (cyc > 0)
    x = f[sel].contiguous()
    y = torch.log2(cyc[sel].to(torch.float32)).contiguous()
    return x, y, r


def gate_passes(beg) -> bool:
    """The learned schedule's gate: >= 2^22 arcs, a row of >= 64 entries, >= 15 % of the arcs in
    rows longer than 128 entries."""
    deg = (beg[1:] - beg[:-1])
    m = int(deg.sum())
    return bool(m >= (1 << 22) and int(deg.max()) >= 64 and int(deg[deg > 128].sum()) >= 0.15 * m)


def time_schedules(beg, adj, ctx, model, warmup=3, reps=5):
    """Median CUDA-event time of one counting call per schedule (256 MiB written before each
    call so the graph is not served from L2), every schedule's count checked equal."""
    import torch
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    gate = gate_passes(beg)
    arms = {
        "learned": lambda: T.count_csr(beg, adj, ctx=ctx, model=model),
        "gate_only": lambda: T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED,
                                         direction_split=1 if gate else 0),
        "tuned": lambda: T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED, direction_split=0),
        "plain": lambda: T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_PLAIN),
    }
    out, counts = {"gate_passes": gate}, set()
    edges = adj.numel()
    for name, fn in arms.items():
        for _ in range(warmup):
            counts.add(fn().triangles)
        ts = []
        for _ in range(reps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            torch.cuda.synchronize()
            counts.add(r.triangles)
            ts.append(e0.elapsed_time(e1))
        ms = float(np.median(ts))
        out[name] = {"ms": ms, "gteps": edges / (ms * 1e-3) / 1e9}
    if len(counts) != 1:
        raise RuntimeError(f"schedules disagree on the count: {sorted(counts)}")
    out["triangles"] = counts.pop()
    out["learned_vs_plain"] = out["plain"]["ms"] / out["learned"]["ms"]
    out["learned_vs_gate_only"] = out["gate_only"]["ms"] / out["learned"]["ms"]
    return out


def held_out_entry(kind, p1, p2, ctx, model):
    import torch
    beg, adj = make_graph(kind, p1, p2, seed=900)
    x, y, r = samples(beg, adj, ctx)
    p = T.model_predict(x, model)
    err = (p - y).abs()
    long_rows = x[:, 0] > np.log2(33.0)
    entry = {"graph": f"{kind}-{p1}-{p2}", "vertices": r.vertices, "edges": r.edges, "rows": int(x.shape[0]),
             "mae_log2": float(err.mean()), "median_abs_log2": float(err.median()),
             "rows_over_32": int(long_rows.sum())}
    if int(long_rows.sum()) > 0:
        entry["mae_log2_rows_over_32"] = float(err[long_rows].mean())
    entry["schedules"] = time_schedules(beg, adj, ctx, model)
    entry["gpu"] = torch.cuda.get_device_name()
    del beg, adj
    return entry


def main():
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "trust_gb300", "csrc", "tc_model_default.inc"))
    ap.add_argument("--report", default=None)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--per-graph", type=int, default=150_000, help="samples kept per training graph")
    ap.add_argument("--held-out-only", action="store_true",
                    help="time and score the held-out graphs with the compiled-in model; no training")
    args = ap.parse_args()
    torch.manual_seed(0)
    ctx = T.Context()
    if args.held_out_only:
        model = T.model_default()
        if model is None:
            raise SystemExit("no model compiled into the library")
        report = {}
        if args.report and os.path.exists(args.report):
            with open(args.report) as fh:
                report = json.load(fh)
        report["held_out"] = [held_out_entry(kind, p1, p2, ctx, model) for kind, p1, p2 in HELD_OUT]
        text = json.dumps(report, indent=1)
        if args.report:
            with open(args.report, "w") as fh:
                fh.write(text + "\n")
        print(text)
        return
    xs, ys, report = [], [], {"train": [], "held_out": []}
    t0 = time.time()
    for i, (kind, p1, p2) in enumerate(TRAIN):
        beg, adj = make_graph(kind, p1, p2, seed=100 + i)
        x, y, r = samples(beg, adj, ctx)
        if x.shape[0] > args.per_graph:  # keep every long row, subsample the rest
            long_rows = x[:, 0] > np.log2(33.0)
            idx_long = torch.nonzero(long_rows).squeeze(1)
            idx_short = torch.nonzero(~long_rows).squeeze(1)
            keep = max(args.per_graph - idx_long.numel(), 0)
            perm = idx_short[torch.randperm(idx_short.numel(), device="cuda")[:keep]]
            idx = torch.cat([idx_long, perm])
            x, y = x[idx], y[idx]
        xs.append(x)
        ys.append(y)
        report["train"].append({"graph": f"{kind}-{p1}-{p2}", "vertices": r.vertices, "edges": r.edges,
                                "samples": int(x.shape[0])})
        del beg, adj
    X = torch.cat(xs).contiguous()
    Y = torch.cat(ys).contiguous()
    perm = torch.randperm(X.shape[0], device="cuda")
    X, Y = X[perm].contiguous(), Y[perm].contiguous()
    model, loss = T.model_train(X, Y, T.model_init(seed=1), epochs=args.epochs, batch=4096, lr=2e-3)
    report["train_samples"] = int(X.shape[0])
    report["train_loss_normalised"] = loss
    pred = T.model_predict(X, model)
    report["train_rmse_log2"] = float(torch.sqrt(torch.mean((pred - Y) ** 2)))
    for kind, p1, p2 in HELD_OUT:
        report["held_out"].append(held_out_entry(kind, p1, p2, ctx, model))
    report["seconds"] = time.time() - t0
    with open(args.out, "w") as fh:
        fh.write("/* cost model trained by trust_gb300/model_train.py on the GPU; %d floats */\n" % model.size)
        for i in range(0, model.size, 4):
            fh.write(", ".join("%.9ef" % v for v in model[i:i + 4]) + ",\n")
    text = json.dumps(report, indent=1)
    if args.report:
        with open(args.report, "w") as fh:
            fh.write(text + "\n")
    print(text)


if __name__ == "__main__":
    main()
