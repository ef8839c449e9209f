"""Build recipe of the FP64 oracle (test infrastructure): g++ with OpenMP.

-ffp-contract=off keeps the FP32 parts (grid keys, vein rest lengths)
identical on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bcs_oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")
HDR = os.path.join(os.path.dirname(HERE), "include", "bcs.h")


def build(force: bool = False) -> str:
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) > os.path.getmtime(SRC)
            and os.path.getmtime(LIB) > os.path.getmtime(HDR)):
        return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB, SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("oracle build failed")
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
