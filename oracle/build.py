"""Builds the CPU oracle (oracle/_build/liboracle.so) with g++.

Test infrastructure only: the product library never uses it. Built with
-ffp-contract=off so the FP32 transcription keeps the shaders' operation
order, and with OpenMP for the timed CPU baseline.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
SOURCES = ["tpd_oracle.cpp", "tpd_oracle_bwd.cpp", "tpd_oracle_host.cpp"]


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    srcs = [HERE / s for s in SOURCES] + [HERE / "tpd_oracle.h"]
    newest = max(s.stat().st_mtime for s in srcs)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = OUT / "liboracle.so.tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           *[str(HERE / s) for s in SOURCES], "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
