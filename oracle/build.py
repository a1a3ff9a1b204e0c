"""Build recipe of the oracle (test infrastructure only): g++ on
oracle/blobs_oracle.cpp into oracle/liboracle.so, -O2 -ffp-contract=off so
every f32 product and sum rounds separately, as the Rust reference does.

The reference itself (Rust, blobs 0.2.1) cannot be compiled on these
machines (no cargo/rustc, crates not vendored), so there is no oracle/_ref.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "blobs_oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(verbose: bool = False, force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                                                          os.path.getmtime(__file__)):
        return LIB
    cmd = ["g++"] + FLAGS + [SRC, "-o", LIB]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
