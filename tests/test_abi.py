"""The C ABI without a GPU: the library loads, exports every declared symbol, and its host-side
logic (validation, folder I/O, tile split, CLI argument handling) behaves like the reference's
operator surface with the checks the reference omits."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import trust_gb300 as T
from trust_gb300 import _lib
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("trust_tc.h",)]


def _declared(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(trust_tc_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = C.CDLL(_lib.LIB_PATH)
    names = [n for h in HEADERS for n in _declared(h)]
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, f"{n} has no Python binding"


def test_shim_symbols_exported():
    lib = C.CDLL(_lib.LIB_PATH)
    # struct arguments Triangle_count(int, char*, arguments, int, int, int, int[, int])
    assert hasattr(lib, "_Z14Triangle_countiPc9argumentsiiii")
    assert hasattr(lib, "_Z14Triangle_countiPc9argumentsiiiii")


def test_opts_defaults_and_strerror():
    lib = T.load()
    o = _lib.Opts()
    lib.trust_tc_opts_init(C.byref(o))
    assert o.device == -1 and o.ptr_kind == T.HOST and o.validate == T.VALIDATE_FULL
    assert o.threads_per_block == 0 and o.blocks == 0 and o.chunk == 0
    seen = set()
    for code in range(0, 12):
        s = lib.trust_tc_strerror(code).decode()
        assert s and s != "unknown status"
        seen.add(s)
    assert len(seen) == 12
    assert lib.trust_tc_strerror(99).decode() == "unknown status"
    assert b"sm_103a" in lib.trust_tc_version()


def _validate(beg, adj):
    b = np.ascontiguousarray(beg, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    d = C.c_int64(-1)
    rc = T.load().trust_tc_validate_csr(b.ctypes.data_as(C.c_void_p), a.ctypes.data_as(C.c_void_p), b.size - 1,
                                        a.size, C.byref(d))
    return rc, d.value


def test_validate_csr():
    assert _validate([0, 2, 3, 3], [1, 2, 2]) == (_lib.OK, 2)
    assert _validate([1, 2, 3, 3], [1, 2, 2])[0] == _lib.E_OFFSETS      # begin[0] != 0
    assert _validate([0, 2, 1, 3], [1, 2, 2])[0] == _lib.E_OFFSETS      # decreasing
    assert _validate([0, 2, 3, 4], [1, 2, 2])[0] == _lib.E_OFFSETS      # begin[n] != m
    assert _validate([0, 2, 3, 3], [1, 3, 2])[0] == _lib.E_IDS          # id == n
    assert _validate([0, 2, 3, 3], [1, -1, 2])[0] == _lib.E_IDS         # negative id
    assert _validate([0], [])[0] == _lib.OK                             # empty graph


def test_count_without_a_device_fails_loudly():
    """No CPU fallback: with no GPU visible the count call returns E_NO_DEVICE."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    beg = np.array([0, 2, 3, 3], dtype=np.int64)
    with pytest.raises(T.TrustTcError) as e:
        T.count_csr(beg, np.array([1, 2, 2], dtype=np.int32))
    assert e.value.status == _lib.E_NO_DEVICE


def test_argument_errors_come_before_any_device_call():
    """Bad source-row slices and schedules are refused before the library touches a device, so the
    answer is E_ARG on any machine (the call never reaches the GPU)."""
    beg = np.array([0, 2, 3, 3], dtype=np.int64)
    adj = np.array([1, 2, 2], dtype=np.int32)
    for rr in ((2, 1), (-1, 2), (0, 4), (4, 3)):
        with pytest.raises(T.TrustTcError) as e:
            T.count_csr(beg, adj, row_range=rr)
        assert e.value.status == _lib.E_ARG, rr
    with pytest.raises(ValueError):
        T.count_csr(beg, adj, row_range=(0, 0))  # an explicit slice ends at a positive row
    with pytest.raises(T.TrustTcError) as e:
        T.count_csr(beg, adj, schedule=7)
    assert e.value.status == _lib.E_ARG


def test_folder_roundtrip_and_errors(tmp_path):
    z = np.load(os.path.join(ROOT, "tests", "golden", "rmat_s9.npz"))
    T.save_folder(str(tmp_path), z["ref_beg"], z["ref_adj"])
    beg, adj = T.load_folder(str(tmp_path))
    np.testing.assert_array_equal(beg, z["ref_beg"])
    np.testing.assert_array_equal(adj, z["ref_adj"])
    # file format is exactly the reference's (raw little-endian int64 / int32)
    np.testing.assert_array_equal(np.fromfile(tmp_path / "begin.bin", dtype=np.int64), z["ref_beg"])
    with pytest.raises(T.TrustTcError) as e:
        T.load_folder(str(tmp_path / "missing"))
    assert e.value.status == _lib.E_IO
    with open(tmp_path / "adjacent.bin", "ab") as f:
        f.write(b"\x01\x02")  # not a whole int32
    with pytest.raises(T.TrustTcError) as e:
        T.load_folder(str(tmp_path))
    assert e.value.status == _lib.E_FORMAT


@pytest.mark.parametrize("name,p", [("rmat_s12", 2), ("rmat_s12", 3), ("k60", 2), ("toy", 2), ("k150", 2)])
def test_partition_folder_matches_reference_tiles(tmp_path, name, p):
    z = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    if f"part{p}_0_0_beg" not in z:
        pytest.skip("fixture has no tiles for this split")
    T.partition_folder(str(tmp_path), z["ref_beg"], z["ref_adj"], p)
    for i in range(p):
        for j in range(p):
            tb, ta = T.load_folder(str(tmp_path / f"partition{i}_{j}"))
            np.testing.assert_array_equal(tb, z[f"part{p}_{i}_{j}_beg"])
            np.testing.assert_array_equal(ta, z[f"part{p}_{i}_{j}_adj"])


def test_chung_lu_table_matches_oracle():
    a = T.chung_lu_table(20000, 2.5, 300.0, 60000)
    b = O.chung_lu_cdf(20000, 2.5, 300.0, 60000)
    np.testing.assert_array_equal(a, b)


CLI = os.path.join(ROOT, "trust_gb300", "trust_tc")


def test_cli_usage_errors():
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([CLI, "x", "1", "1024", "10"], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([CLI, "x", "1", "1024", "10", "1", "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2


def test_cli_missing_folder_exits_like_reference(tmp_path):
    # the reference prints the error and exits with EXIT_FAILURE (Without-graph-partition/herror.h:1-8)
    r = subprocess.run([CLI, str(tmp_path / "nope"), "1", "1024", "10", "1"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "cannot read" in r.stdout
