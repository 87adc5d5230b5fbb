"""ORACLE recipe — test infrastructure only.

Builds the oracle restatement (shg_oracle.cpp, dft_ref.h) into
``oracle/_build/liboracle.so`` with g++ and -ffp-contract=off, so that the float
operation order of the reference is kept on x86 and on Arm alike.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "shg_oracle.cpp")]
    deps = srcs + [os.path.join(HERE, "shg_oracle.h"), os.path.join(HERE, "dft_ref.h")]
    if not force and os.path.isfile(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           "-o", tmp] + srcs
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
