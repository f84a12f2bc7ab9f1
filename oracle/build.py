"""Build recipe for the CPU oracle (test infrastructure, not product).

Compiles ``oracle/mpm_oracle.c`` twice with the host C compiler: once in
float32 (``liborc32.so``, symbols ``orc32_*``) and once in float64
(``liborc64.so``, symbols ``orc64_*``), both with OpenMP and with
floating-point contraction switched off so the float32 build rounds the same
on x86-64 and aarch64 hosts.  Outputs go to ``oracle/_build/``.

The reference itself (Python + NVIDIA Warp kernels) has no C/C++ sources to
compile, so there is no ``oracle/_ref`` build.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mpm_oracle.c")
OUT = os.path.join(HERE, "_build")

CFLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11"]


def lib_path(bits: int) -> str:
    return os.path.join(OUT, f"liborc{bits}.so")


def _compile(bits: int) -> str:
    out = lib_path(bits)
    defs = ["-DORC_F64"] if bits == 64 else []
    cmd = [os.environ.get("CC", "gcc"), *CFLAGS, *defs, SRC, "-o", out + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def needs_build() -> bool:
    src_m = os.path.getmtime(SRC)
    for bits in (32, 64):
        p = lib_path(bits)
        if not os.path.exists(p) or os.path.getmtime(p) < src_m:
            return True
    return False


def build(force: bool = False) -> None:
    os.makedirs(OUT, exist_ok=True)
    if not force and not needs_build():
        return
    with ThreadPoolExecutor(2) as ex:
        list(ex.map(_compile, (32, 64)))


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built", lib_path(32), lib_path(64))
