"""Builds the CPU oracle (liboracle.so) from oracle/*.cpp — test infrastructure
only: tests/, __graft_entry__.smoke() and bench.py's cpu_baseline use it to
check the product; the product library never links it.

The reference itself is JavaScript + WGSL with no compilable source, so there
is no oracle/_ref build: this restatement is the oracle."""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = sorted(f for f in os.listdir(HERE) if f.endswith(".cpp"))


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    # -ffp-contract=off: no fused multiply-add, so x86 and Arm give the same bits.
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", *srcs, "-o", LIB]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}")
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
