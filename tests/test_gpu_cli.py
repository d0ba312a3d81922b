"""The CLI and the reference-signature operator on the GPU: same argv, same output line."""
import os
import subprocess

import numpy as np
import pytest

import trust_gb300 as T

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "trust_gb300", "trust_tc")
GOLD = os.path.join(ROOT, "tests", "golden")


def test_cli_line(tmp_path):
    z = np.load(os.path.join(GOLD, "rmat_s12.npz"))
    T.save_folder(str(tmp_path), z["ref_beg"], z["ref_adj"])
    r = subprocess.run([CLI, str(tmp_path), "1", "1024", "1024", "1"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    line = r.stdout.strip("\n")
    assert line.endswith(" ")  # "%s,%d,%d,%lld,%f,%f \n" (Without-graph-partition/mpi_main.cpp:115)
    folder, n, m, tri, t, teps = line.strip().split(",")
    assert folder == str(tmp_path)
    assert int(n) == z["ref_beg"].size - 1 and int(m) == z["ref_adj"].size
    assert int(tri) == int(z["nx_triangles"][0])
    # time is printed with 6 decimals, so compare GTEPS loosely against the printed time
    assert float(t) > 0 and abs(float(teps) - int(m) / float(t) / 1e9) <= 0.1 * float(teps) + 1e-6


def test_cli_default_knobs_and_ranks(tmp_path):
    z = np.load(os.path.join(GOLD, "k150.npz"))
    T.save_folder(str(tmp_path), z["ref_beg"], z["ref_adj"])
    # two logical ranks on one process: the SUM stays the whole count
    r = subprocess.run([CLI, str(tmp_path), "2", "256", "0", "4"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert int(r.stdout.split(",")[3]) == int(z["nx_triangles"][0])


def test_cli_partitioned(tmp_path):
    z = np.load(os.path.join(GOLD, "rmat_s12.npz"))
    T.partition_folder(str(tmp_path), z["ref_beg"], z["ref_adj"], 2)
    r = subprocess.run([CLI, str(tmp_path), "1", "1024", "1024", "1", "2"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    line = r.stdout.strip().splitlines()[-1]
    assert line.startswith(str(tmp_path) + ",triangle:")
    assert int(line.split("triangle:")[1].split(",")[0]) == int(z["nx_triangles"][0])


def test_python_operator(tmp_path):
    z = np.load(os.path.join(GOLD, "chung_lu_3000.npz"))
    T.save_folder(str(tmp_path), z["ref_beg"], z["ref_adj"])
    a = T.Triangle_count(0, str(tmp_path), T.arguments(), 1, 1024, 1024, 1)
    assert a.count == int(z["nx_triangles"][0])
    assert a.edge_count == z["ref_adj"].size and a.vertices == z["ref_beg"].size - 1
    assert a.degree == a.edge_count // a.vertices and a.time > 0
    b = T.Triangle_count(1, str(tmp_path), T.arguments(), 2, 1024, 1024, 1)
    assert b.count == 0 and b.edge_count == a.edge_count


def test_reference_style_caller_links(tmp_path):
    """A main program written against the reference's own TC.cuh declarations (a fixture with the
    declarations of Without-graph-partition/TC.cuh:1-10) compiles unchanged and links against
    libtrust_tc.so, the relink recipe of INTEGRATION.md section 1, then counts a golden folder."""
    fx = os.path.join(ROOT, "tests", "fixtures", "ref_caller")
    lib_dir = os.path.join(ROOT, "trust_gb300")
    exe = str(tmp_path / "trianglecounting.bin")
    obj = str(tmp_path / "main.o")
    cc = subprocess.run(["g++", "-c", "-I" + fx, os.path.join(fx, "main.cpp"), "-o", obj], capture_output=True,
                        text=True, timeout=120)
    assert cc.returncode == 0, cc.stderr
    ld = subprocess.run(["g++", obj, "-L" + lib_dir, "-ltrust_tc", "-Wl,-rpath," + lib_dir, "-o", exe],
                        capture_output=True, text=True, timeout=120)
    assert ld.returncode == 0, ld.stderr
    z = np.load(os.path.join(GOLD, "rmat_s12.npz"))
    folder = tmp_path / "graph"
    folder.mkdir()
    T.save_folder(str(folder), z["ref_beg"], z["ref_adj"])
    r = subprocess.run([exe, str(folder), "2", "1024", "1024", "1"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = r.stdout.strip().split(",")
    assert fields[0] == str(folder)
    assert int(fields[1]) == z["ref_beg"].size - 1 and int(fields[2]) == z["ref_adj"].size
    assert int(fields[3]) == int(z["nx_triangles"][0])
