"""Compile the CPU oracle port (oracle/port/sphdem_oracle.cpp) into
oracle/liboracle_port.so.  Test infrastructure only.

-ffp-contract=off keeps the port's arithmetic free of fused multiply-adds on
every host (aarch64 gcc contracts by default), as the reference's own x86
build is.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "port", "sphdem_oracle.cpp")
LIB = os.path.join(HERE, "liboracle_port.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    SRC, "-o", tmp], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
