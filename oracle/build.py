"""Compile the C restatements under oracle/ into oracle/_build/liboracle.so.

Test infrastructure: used by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline only.  -ffp-contract=off keeps every FP64 multiply and add separately
rounded so the restatement follows the reference's generated expression order.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SOURCES = ["lj_oracle.c", "dem_oracle.c"]
LIB = os.path.join(BUILD, "liboracle.so")


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(s) for s in srcs)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
           "-Wall", "-Wno-unknown-pragmas", "-o", LIB + ".tmp"] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
