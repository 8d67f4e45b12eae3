"""Compile the CPU oracle (oracle/mt_oracle.cpp) into oracle/liboracle.so.

Test infrastructure: only tests, __graft_entry__.smoke() and bench.py's CPU
baseline load the result. Plain g++, no FMA contraction, wrapping signed
arithmetic (the reference's RNG relies on it).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = [os.path.join(HERE, "mt_oracle.cpp")]
HDR = [os.path.join(HERE, "mt_oracle.h")]


def build(force: bool = False) -> str:
    newest = max(os.path.getmtime(p) for p in SRC + HDR + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > newest:
        return LIB
    cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-fwrapv", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-function", *SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
