"""Build recipe of the oracle's C restatements (TEST INFRASTRUCTURE ONLY).

Compiles oracle/noise.c (the Fourier-space noise stream) with the host C compiler into
oracle/_build/liboracle_noise.so.  Called by __graft_entry__.build() and, on first use,
by oracle/philox.py.  Portable C (no architecture flags), so it builds the same on
x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
NOISE_LIB = os.path.join(OUT, "liboracle_noise.so")


def build():
    src = os.path.join(HERE, "noise.c")
    if os.path.exists(NOISE_LIB) and os.path.getmtime(NOISE_LIB) > os.path.getmtime(src):
        return NOISE_LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    os.makedirs(OUT, exist_ok=True)
    tmp = NOISE_LIB + ".tmp"
    subprocess.run([cc, "-O2", "-fPIC", "-shared", "-fopenmp", src, "-o", tmp, "-lm"], check=True,
                   capture_output=True)
    os.replace(tmp, NOISE_LIB)
    return NOISE_LIB


if __name__ == "__main__":
    print(build())
