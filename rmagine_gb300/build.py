"""Builds librmg_gb300.so (sm_103a) in-tree with nvcc.

Each CUDA translation unit under csrc/ is compiled in parallel to an object
file under rmagine_gb300/_build/, then linked into rmagine_gb300/lib/.
A unit is recompiled only when it or a header it may include is newer than
its object file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIBNAME = "librmg_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I", str(ROOT / "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librmg_gb300")


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h")))


def _extra_flags() -> list[str]:
    """Additional nvcc flags from RMG_NVCC_FLAGS (space separated), e.g. -DRMG_TRACE_MIN_BLOCKS=5."""
    return os.environ.get("RMG_NVCC_FLAGS", "").split()


def _build_dir() -> Path:
    extra = _extra_flags()
    if not extra:
        return BUILD
    import hashlib

    return BUILD / ("flags_" + hashlib.sha1(" ".join(extra).encode()).hexdigest()[:10])


def _compile(src: Path, extra: list[str]) -> Path:
    bdir = _build_dir()
    bdir.mkdir(parents=True, exist_ok=True)
    obj = bdir / (src.stem + ".o")
    newest_dep = max([src.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if obj.exists() and obj.stat().st_mtime >= newest_dep:
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *_extra_flags(), *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, ptxas_info: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    srcs = _sources()
    jobs = jobs or min(len(srcs), max(1, os.cpu_count() or 1))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    out = lib_path()
    newest = max(o.stat().st_mtime for o in objs)
    stamp = LIBDIR / "build_flags.txt"
    flags = " ".join(_extra_flags())
    if not out.exists() or out.stat().st_mtime < newest or (stamp.read_text() if stamp.exists() else "") != flags:
        tmp = out.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt",
               "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, out)
        stamp.write_text(flags)
    if verbose:
        print(f"built {out}")
    return out


def build_cpp_tests() -> Path:
    """Compiles the C++ API test program (tests/cpp/test_simulators.cpp) against the library."""
    lib = build()
    src = ROOT / "tests" / "cpp" / "test_simulators.cpp"
    out = BUILD / "test_simulators"
    deps = [src, ROOT / "include" / "rmagine_gb300.hpp", ROOT / "include" / "rmg.h", lib]
    if out.exists() and out.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return out
    cmd = [nvcc(), "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(src), "-L", str(LIBDIR), "-lrmg_gb300",
           "-Xlinker", f"-rpath={LIBDIR}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"C++ test build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
