"""Compiles oracle/_ref/libref.so: ref_shim.cpp + rmagine's sensors.cpp, against the
reference tree's own headers (test infrastructure only; needs the reference checkout).

    python oracle/build_ref.py            # RMAGINE_REF defaults to /root/reference
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF = Path(os.environ.get("RMAGINE_REF", "/root/reference"))
OUT = HERE / "_ref" / "libref.so"


def available() -> bool:
    return (REF / "src/rmagine_core/include/rmagine/types/sensor_models.h").exists()


def build(force: bool = False) -> Path | None:
    if not available():
        return OUT if OUT.exists() else None
    src = [HERE / "ref_shim.cpp", REF / "src/rmagine_core/src/types/sensors.cpp"]
    OUT.parent.mkdir(exist_ok=True)
    if not force and OUT.exists() and OUT.stat().st_mtime >= max(s.stat().st_mtime for s in src):
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
           "-I", str(REF / "src/rmagine_core/include"), *map(str, src), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference shim build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
