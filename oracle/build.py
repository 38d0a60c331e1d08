"""ORACLE build recipe (test infrastructure only): compile oems_oracle.c with gcc.

Strict IEEE float semantics are required for bit-exact comparison with the reference's FP32
engine: no FMA contraction, no fast-math, no flush-to-zero, no -march=native.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboems_oracle.so")
SRC = os.path.join(HERE, "oems_oracle.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
