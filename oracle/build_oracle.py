"""Builds oracle/liboracle.so from oracle/game_oracle.c (test infrastructure).

gcc -O2 -ffp-contract=off: no contraction of a*b+c into FMA, so the oracle
rounds exactly like the reference built the same way, on x86_64 and aarch64.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "game_oracle.c")
HDR = os.path.join(HERE, "game_oracle.h")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                                                         os.path.getmtime(HDR)):
        return LIB
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall", "-o", LIB, SRC, "-lm"],
                   check=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
