#!/usr/bin/env python3
"""Build recipe for the oracle port: ``oracle/_build/libc2oracle.so`` from ``oracle/c2_oracle.cpp``.

TEST INFRASTRUCTURE ONLY (the checker of the parity tests, smoke() and the CPU baseline).
``-ffp-contract=off`` keeps the float arithmetic unfused on x86-64 and aarch64 alike.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c2_oracle.cpp")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libc2oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cxx = os.environ.get("CXX", "g++")
    tmp = LIB + ".tmp"
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr[-6000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
