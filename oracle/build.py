"""Build recipe for the CPU oracle library (test infrastructure only).

Compiles ``oracle/*.c`` with gcc into ``oracle/_build/liboracle.so``.
``-ffp-contract=off`` keeps every multiply and add separately rounded, as a
gfortran build of the reference without FMA would, and makes the x86 and Arm
builds agree.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
load the result.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = ["letkf_core.c", "obs_local.c", "sweep.c", "obs_operator.c"]


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "letkf_oracle.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-std=c99", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-o", LIB + ".tmp"] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
