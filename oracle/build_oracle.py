"""Compile the oracle's C port (test infrastructure) with gcc; no make needed."""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sweep_port.c")
LIB = os.path.join(HERE, "libbldfm_oracle.so")


def build_oracle(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-std=gnu11", "-shared", "-o", LIB, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB
