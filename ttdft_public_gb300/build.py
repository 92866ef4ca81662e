"""In-tree build of the native libraries (no cmake, no pip install).

  lib/libttg.so       CUDA kernels + the extern "C" ABI (include/ttg.h), sm_103a
  lib/libttg_host.so  host operator producer (H_loc / C_nloc assembly, OpenMP)
  lib/libttdft_cxx.so reference-shaped C++ classes (include/ttdft/*.h) over the C ABI

Translation units compile in parallel; objects go to _build/ (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJ = os.path.join(ROOT, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["spmm.cu", "spmm_tc.cu", "dense.cu", "capi.cu", "tensor.cu", "scf.cu",
              "hupdate.cu", "eig.cu", "mlp.cu", "spmm_umma.cu", "tgemm.cu",
              "ozgemm.cu"]
CXX_SOURCES = ["host/ChebyShevFilter.cc", "host/Mult.cc", "host/MultTm.cc",
               "host/EigenSolver.cc", "host/petsc_shim.cc"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {os.path.basename(cmd[-1])}")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, "ttg.h")]
    for d in (CSRC, os.path.join(INCLUDE, "ttdft")):
        if os.path.isdir(d):
            hs += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".cuh", ".h"))]
    return hs


def build_ttg(force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    out = os.path.join(LIBDIR, "libttg.so")
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
                         "-I" + INCLUDE, "-I" + CSRC, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(out, objs):
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", out, *objs, "-lgomp"])
    return out


def build_host(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    src = os.path.join(CSRC, "gen", "assemble_h.cc")
    out = os.path.join(LIBDIR, "libttg_host.so")
    if force or _stale(out, [src]):
        # no fused multiply-adds: the pattern (|h| > truncation) and the values
        # then come out the same on x86 and Arm hosts
        _run(["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
              "-o", out, src])
    return out


def build_cxx(force: bool = False) -> str:
    """Reference-shaped C++ classes, linked against libttg.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CXX_SOURCES]
    srcs = [s for s in srcs if os.path.exists(s)]
    out = os.path.join(LIBDIR, "libttdft_cxx.so")
    if not srcs:
        return out
    if force or _stale(out, srcs + _headers()):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + INCLUDE, "-o", out, *srcs,
              "-L" + LIBDIR, "-lttg", "-Wl,-rpath,$ORIGIN"])
    return out


def build_driver(force: bool = False) -> str:
    """The C++ ChFSI driver (csrc/host/chfsi_driver.cc) that exercises the classes
    the way the reference's main.cc does."""
    src = os.path.join(CSRC, "host", "chfsi_driver.cc")
    out = os.path.join(LIBDIR, "chfsi_driver")
    if not os.path.exists(src):
        return out
    if force or _stale(out, [src] + _headers()):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, "-o", out, src, "-L" + LIBDIR,
              "-lttdft_cxx", "-lttg", "-Wl,-rpath,$ORIGIN"])
    return out


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_ttg, force)
        f2 = ex.submit(build_host, force)
        f1.result()
        f2.result()
    build_cxx(force)
    build_driver(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built into", LIBDIR)
