"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/ubs_oracle.cpp with the host C++ compiler into
oracle/_build/libubs_oracle.so.  Contraction of a*b+c into fused multiply-adds
is disabled so the oracle rounds the same way on x86 and on Arm hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ubs_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "libubs_oracle.so")


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= os.path.getmtime(SRC)
            and os.path.getmtime(OUT) >= os.path.getmtime(__file__)):
        return OUT
    cxx = os.environ.get("CXX", "g++")
    tmp = OUT + ".tmp%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", SRC, "-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
