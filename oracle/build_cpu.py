"""Build recipe for the C/OpenMP restatement (test infrastructure and CPU
baseline): compiles oracle/dns3d_cpu.c into oracle/_build/libdns3d_cpu.so with
the host gcc.  Portable flags only (the same source builds on x86-64 and
aarch64 hosts)."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "dns3d_cpu.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libdns3d_cpu.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-std=c99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
           "-o", LIB, SRC, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle C build failed:\n" + res.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
