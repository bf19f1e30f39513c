"""Builds the oracle (test infrastructure): oracle/_build/liboracle.so from oracle.cpp.

-ffp-contract=off keeps every binary32 expression as written (no fused
multiply-add except the explicit fmaf calls), so results match on x86 and Arm.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    src = HERE / "oracle.cpp"
    OUT.parent.mkdir(exist_ok=True)
    if not force and OUT.exists() and OUT.stat().st_mtime >= src.stat().st_mtime:
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", str(src), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
