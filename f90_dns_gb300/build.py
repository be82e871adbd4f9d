"""Build ``libdns3d_gpu.so`` in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel to an object file under
``f90_dns_gb300/_build/`` and the objects are linked into
``f90_dns_gb300/libdns3d_gpu.so``.  Objects are rebuilt when their source or
any header is newer.
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
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libdns3d_gpu.so")
RUNNER = os.path.join(PKG, "dns3d_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I", os.path.join(ROOT, "include")]

SOURCES = ["capi.cu", "fft.cu", "step.cu", "setup.cu", "host.cpp", "noalloc.cu", "server.cpp", "restart.cpp",
           "output.cpp", "fft_ct.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "dns3d_capi.h"))
    return max(os.path.getmtime(h) for h in hs if os.path.exists(h))


def _compile(src: str, nvcc: str, hdr_mtime: float) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), hdr_mtime):
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc, *ARCH, *COMMON, *lang, "-c", path, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    """Compile every translation unit for sm_103a and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hm = _headers_mtime()
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, hm), SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-Xcompiler", "-pthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    # the driver executable (host C++ over the C-ABI)
    src = os.path.join(CSRC, "dns3d_run.cpp")
    if not os.path.exists(RUNNER) or os.path.getmtime(RUNNER) < max(os.path.getmtime(src), os.path.getmtime(LIB)):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", RUNNER,
               "-L", PKG, "-ldns3d_gpu", "-Wl,-rpath,$ORIGIN"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
