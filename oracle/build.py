"""Build recipe for the CPU oracle (test infrastructure, never the product).

Compiles ``oracle/lgt_oracle.c`` into ``oracle/liblgt_oracle.so`` with gcc.
``-ffp-contract=off`` keeps multiplies and adds separately rounded, as Julia
does, so the oracle's diagonal sums round like finite_ed.jl:265-276.

The reference (NoaFeldman/LGT) is pure Julia with no C/C++ sources, so there
is nothing to compile into ``oracle/_ref``; the oracle is the restatement.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "lgt_oracle.c")
LIB = os.path.join(HERE, "liblgt_oracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle library if it is missing or older than its source."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-std=c11", "-Wall", "-shared",
           "-fPIC", "-o", tmp, SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
