"""Build the sm_103a library, the CLI and the test oracles in-tree.

Outputs (all git-ignored):
  trust_gb300/libtrust_tc.so   the product: C ABI of include/trust_tc.h + the C++ shim of
                               include/trust_tc_shim.h, kernels compiled for sm_103a only
  trust_gb300/trust_tc         the CLI with the reference's argv and output line
  oracle/_build/liboracle.so   CPU oracle (tests, smoke and the bench CPU legs only)
  oracle/_build/liboracle_cuda.so  oracle + the harness that runs the reference kernel cubin
  oracle/_ref/*                the reference's own code, where its sources are present (oracle/build_ref.sh)

Compiles in parallel and skips outputs newer than their sources.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "trust_gb300")
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_OBJ = os.path.join(ORACLE, "_build")
INCLUDE = os.path.join(ROOT, "include")

LIB = os.path.join(PKG, "libtrust_tc.so")
CLI = os.path.join(PKG, "trust_tc")
ORACLE_LIB = os.path.join(ORACLE_OBJ, "liboracle.so")
ORACLE_CUDA_LIB = os.path.join(ORACLE_OBJ, "liboracle_cuda.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE]
SOURCES = ["tc_count.cu", "tc_prep.cu", "tc_gen.cu", "tc_api.cpp", "tc_tiles.cpp", "tc_shim.cpp", "tc_noalloc.cu", "tc_split.cu", "tc_model.cu", "tc_batch.cu"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _arch_guard(out_dir: str, outputs: list[str]) -> None:
    """Outputs compiled on another machine type (this tree travels between x86 and Arm hosts) are
    removed so they are rebuilt, never linked."""
    import platform
    stamp = os.path.join(out_dir, ".machine")
    here = platform.machine()
    prev = open(stamp).read().strip() if os.path.exists(stamp) else None
    if prev != here:
        for d in (out_dir,):
            for f in os.listdir(d):
                if f.endswith((".o", ".so")):
                    os.remove(os.path.join(d, f))
        for o in outputs:
            if os.path.exists(o):
                os.remove(o)
        with open(stamp, "w") as f:
            f.write(here + "\n")


def _newer(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return hs


def build_library(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    _arch_guard(OBJ, [LIB, CLI])
    nvcc = shutil.which("nvcc") or os.path.join(_cuda_home(), "bin", "nvcc")
    hdrs = _headers()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.rsplit(".", 1)[0] + ".o")
        objs.append(o)
        if not _newer(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, *NVFLAGS, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    if jobs or not _newer(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC"])
    cli_src = os.path.join(CSRC, "tc_cli.cpp")
    if not _newer(CLI, [cli_src, LIB] + hdrs):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", CLI, "-L" + PKG, "-ltrust_tc",
              "-Wl,-rpath,$ORIGIN"])
    return LIB


def build_oracle() -> None:
    os.makedirs(ORACLE_OBJ, exist_ok=True)
    _arch_guard(ORACLE_OBJ, [])
    src = os.path.join(ORACLE, "tc_oracle.c")
    if not _newer(ORACLE_LIB, [src]):
        _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-o", ORACLE_LIB, src,
              "-lpthread", "-lm"])
    drv = os.path.join(ORACLE, "ref_tc_driver.c")
    cuda = _cuda_home()
    if os.path.exists(os.path.join(cuda, "include", "cuda.h")) and not _newer(ORACLE_CUDA_LIB, [src, drv]):
        _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-I" + os.path.join(cuda, "include"),
              "-o", ORACLE_CUDA_LIB, drv, src, "-L" + os.path.join(cuda, "lib64", "stubs"), "-lcuda",
              "-lpthread", "-lm"])
    # the reference's own sources: where TRUST_REFERENCE_ROOT names them, else where the recipe
    # finds them by default (it builds nothing where they are absent); a machine without them uses
    # what an earlier build left in oracle/_ref/
    ref_root = os.environ.get("TRUST_REFERENCE_ROOT")
    ref_out = os.path.join(ORACLE, "_ref", "tc_ref_w.cubin")
    if not os.path.exists(ref_out) and (not ref_root or os.path.isdir(os.path.join(ref_root, "Preprocess"))):
        _run(["sh", os.path.join(ORACLE, "build_ref.sh")] + ([ref_root] if ref_root else []))


def build_all() -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library)
        f2 = ex.submit(build_oracle)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all()
    print("built", LIB, file=sys.stderr)
