"""Build recipe for the oracle (test infrastructure only).

Compiles ``oracle/oracle.cpp`` — the CPU restatement of bankai-lightgbm's tree-learner hot
path — and ``oracle/binning.cpp`` — its own restatement of the dense dataset preparation (row
sample, bin mappers, stored bins) — into ``oracle/_build/liboracle.so``. The product never loads this library; tests, the
smoke check and the CPU-baseline leg of ``bench.py`` do.

``-ffp-contract=off`` keeps every ``a * b + c`` unfused so the oracle rounds like the
reference's unfused build; the reference's deliberate fused multiply-adds (``madd``) are
selected at run time with ``fused_madd``.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRCS = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "binning.cpp")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in SRCS):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math"] + SRCS + ["-pthread", "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
