"""Build recipe for the CPU oracle library (test infrastructure only).

Compiles ``oracle/*.c`` with gcc into ``oracle/_build/liboracle.so`` (the
parity build: ``-ffp-contract=off`` keeps every multiply and add separately
rounded, as a gfortran build of the reference without FMA would, and makes the
x86 and Arm builds agree) and ``oracle/_build/liboracle_timed.so`` (``-O3``
with FMA contraction: the CPU baseline's timed build).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU legs load the result.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
LIB_TIMED = os.path.join(BUILD, "liboracle_timed.so")
SOURCES = ["letkf_core.c", "obs_local.c", "sweep.c", "obs_operator.c", "obs_operator_scale.c"]
# parity build: every multiply and add rounded on its own
FLAGS = ["-std=c99", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]
# the build the CPU baseline is timed with: -O3 and FMA contraction, as the
# reference's own optimised builds are (speedy/letkf/make_letkf.sh:6 compiles
# with -fast -O3; scale/arch/configure.user.ubuntu-gnu:26-28 adds -fopenmp);
# no -march=native, so that the same flags build on the x86 and the Arm hosts
FLAGS_TIMED = ["-std=c99", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=fast", "-fno-fast-math"]


def build(force: bool = False, timed: bool = False) -> str:
    out = LIB_TIMED if timed else LIB
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "letkf_oracle.h")]
    if not force and os.path.exists(out):
        t = os.path.getmtime(out)
        if all(os.path.getmtime(d) <= t for d in deps):
            return out
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", *(FLAGS_TIMED if timed else FLAGS), "-o", out + ".tmp"] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def build_all(force: bool = False):
    return build(force), build(force, timed=True)


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
