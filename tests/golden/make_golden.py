"""Generate the golden fixtures in this folder from the reference's own preprocessing binaries.

Run in a container where the reference sources are present:
    sh oracle/build_ref.sh && python tests/golden/make_golden.py
It writes one .npz per case.  Each holds the input pairs, the outputs of the reference binaries
built from source (oracle/_ref/: fromDirectToUndirect + preprocess, TransformTxt2Binary +
preprocess_out, partition) and an independent triangle count from networkx on the undirected,
self-loop-free, deduplicated input.  The fixtures are what pins the oracle; the GPU tests read
them without needing the reference.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.path.join(ROOT, "oracle", "_ref")

from oracle import oracle  # noqa: E402


def _run(cmd, cwd):
    subprocess.run(cmd, cwd=cwd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def _read_csr(folder):
    beg = np.fromfile(os.path.join(folder, "begin.bin"), dtype=np.int64)
    adj = np.fromfile(os.path.join(folder, "adjacent.bin"), dtype=np.int32)
    return beg, adj


def _nx_triangles(pairs) -> int:
    import networkx as nx
    g = nx.Graph()
    for u, v in pairs:
        if u != v:
            g.add_edge(int(u), int(v))
    return sum(nx.triangles(g).values()) // 3


def make_case(name: str, pairs: np.ndarray, text_lines: list[str] | None = None, parts=(2, 3)) -> None:
    out = {"pairs": pairs.astype(np.int32)}
    with tempfile.TemporaryDirectory() as d:
        # Preprocess/compile.sh path: text edge list -> 1.mmio -> begin.bin/adjacent.bin
        lines = text_lines if text_lines is not None else [f"{u} {v}" for u, v in pairs]
        with open(os.path.join(d, "edges.txt"), "w") as f:
            f.write("\n".join(lines) + "\n")
        _run([os.path.join(REF, "fromDirectToUndirect"), "edges.txt", "1.mmio"], d)
        with open(os.path.join(d, "1.mmio")) as f:
            rows = [ln.split() for ln in f.read().splitlines() if ln.strip()]
        out["undirect_header"] = np.array([int(x) for x in rows[0]], dtype=np.int64)
        out["undirect_edges"] = np.array([[int(a), int(b)] for a, b in rows[1:]], dtype=np.int32).reshape(-1, 2)
        _run([os.path.join(REF, "preprocess")], d)
        out["ref_beg"], out["ref_adj"] = _read_csr(d)
        # partition of that CSR (Preprocess/partition.cpp)
        for p in parts:
            pd = os.path.join(d, f"p{p}")
            os.makedirs(pd)
            for i in range(p):
                for j in range(p):
                    os.makedirs(os.path.join(pd, f"partition{i}_{j}"))
            for fn in ("begin.bin", "adjacent.bin"):
                os.link(os.path.join(d, fn), os.path.join(pd, fn))
            _run([os.path.join(REF, "partition"), str(p)], pd)
            for i in range(p):
                for j in range(p):
                    tb, ta = _read_csr(os.path.join(pd, f"partition{i}_{j}"))
                    out[f"part{p}_{i}_{j}_beg"], out[f"part{p}_{i}_{j}_adj"] = tb, ta
    with tempfile.TemporaryDirectory() as d:
        # Preprocess/speedupIO path: 0-based "u v" text -> binary edge list -> CSR
        if text_lines is None:
            with open(os.path.join(d, "edges.txt"), "w") as f:
                f.write("\n".join(f"{u} {v}" for u, v in pairs) + "\n")
            _run([os.path.join(REF, "TransformTxt2Binary"), "edges.txt", str(len(pairs))], d)
            _run([os.path.join(REF, "preprocess_out")], d)
            out["fast_beg"], out["fast_adj"] = _read_csr(d)
    out["nx_triangles"] = np.array([_nx_triangles(pairs)], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "n=%d m=%d triangles=%d" % (out["ref_beg"].size - 1, out["ref_adj"].size, out["nx_triangles"][0]))


def main() -> None:
    # toy: K4, a triangle, a pendant, a duplicate, a self-loop and a comment line
    toy_lines = ["# toy graph", "1 2", "1 3", "1 4", "2 3", "2 4", "3 4", "5 6", "6 7", "5 7", "7 8", "1 2", "9 9"]
    toy_pairs = np.array([[int(x) for x in ln.split()] for ln in toy_lines[1:]], dtype=np.int32)
    make_case("toy", toy_pairs, toy_lines, parts=(2,))
    make_case("er_200", oracle.gen_er(200, 1500, seed=7))
    make_case("rmat_s9", oracle.gen_rmat(9, 8 << 9, seed=11))
    make_case("rmat_s12", oracle.gen_rmat(12, 16 << 12, seed=1))
    kn = np.array([[i, j] for i in range(60) for j in range(i + 1, 60)], dtype=np.int32)
    make_case("k60", kn[np.random.default_rng(3).permutation(len(kn))])
    k150 = np.array([[i, j] for i in range(150) for j in range(i + 1, 150)], dtype=np.int32)
    make_case("k150", k150[np.random.default_rng(4).permutation(len(k150))], parts=(2,))
    cdf = oracle.chung_lu_cdf(3000, 2.5, 120.0, 9000)
    make_case("chung_lu_3000", oracle.gen_weighted(cdf, 9000, seed=2))


if __name__ == "__main__":
    main()
