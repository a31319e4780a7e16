"""Builds the oracle's C restatement (test infrastructure) with gcc.

Output: oracle/_build/libhermes_oracle.so.  ``-ffp-contract=off`` keeps
multiply and add separate as in the reference (gcc contracts them by default
on aarch64).
"""

import os
import subprocess
import sys

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(ORACLE_DIR, "_build")
LIB = os.path.join(BUILD_DIR, "libhermes_oracle.so")
SRC = [os.path.join(ORACLE_DIR, "hermes_oracle.c")]


def build(force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(s) <= os.path.getmtime(LIB) for s in SRC):
        return LIB
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", tmp, *SRC, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
