"""Build recipe for the oracle: compiles adhoc.cpp into oracle/liboracle.so.

Plain g++ on one source file, OpenMP over rows, no FMA contraction (the
restatement follows the reference's expression trees).  Portable flags only:
the same recipe runs on x86_64 and aarch64 hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "adhoc.cpp")
LIB = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
