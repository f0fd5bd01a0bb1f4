"""Builds the GB300 simulator library in-tree.

``build()`` compiles every translation unit of ``csrc/`` for sm_103a only
(CUDA sources with ``nvcc -gencode arch=compute_103a,code=sm_103a``, host
sources with ``g++``) in parallel and links
``toucangpurt_gb300/_lib/libtoucan_gb300.so`` with a static CUDA runtime.
Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT = PKG / "_lib"
OBJ = PKG / "_build"
LIB = OUT / "libtoucan_gb300.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc") if (CUDA_HOME / "bin" / "nvcc").exists() else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-std=c++20", "-O2", "-fPIC", "-Wall"]


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _compile(src: Path, deps: list[Path]) -> Path:
    obj = OBJ / (src.name + ".o")
    if not _stale(obj, src, deps):
        return obj
    inc = [f"-I{INCLUDE}", f"-I{CSRC}", f"-I{CUDA_HOME / 'include'}"]
    if src.suffix == ".cu":
        cmd = [NVCC, *NVCC_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [CXX, *CXX_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    """Compile and link the library; returns its path."""
    OUT.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    deps = _headers()
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, deps), srcs))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [NVCC, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(with_reference: bool = True) -> None:
    """Build the CPU oracle (test infrastructure) and, where the reference
    checkout exists, its reference-derived checkers (oracle/Makefile)."""
    make = shutil.which("make")
    if make is None:
        raise RuntimeError("make not found")
    args = [make, "-s", "-C", str(ROOT / "oracle")]
    if not with_reference:
        args.append("REF_DIR=/nonexistent")
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    build(verbose=True)
    build_oracle()
