"""Build libhella_gb300.so (sm_103a) in-tree.

Compiles every translation unit of csrc/ with nvcc in parallel and links
the shared library into casm-hella_gb300/lib/.  Rebuilds only when a source
or header is newer than the library (or when forced).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
OBJ = PKG / "_build"
LIB = OUT / "libhella_gb300.so"

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-I", str(ROOT / "include"), "-I", str(CSRC)]
# --fmad=false: no implicit multiply-add contraction; kernels spell out every
# fused multiply-add they mean, so results match the oracle bit for bit.
CUFLAGS = ARCH + COMMON + ["-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off"]
CXXFLAGS = COMMON + ["-Xcompiler", "-fPIC,-ffp-contract=off"]


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = sources() + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def _compile(src: Path) -> Path:
    obj = OBJ / (src.name + ".o")
    flags = CUFLAGS if src.suffix == ".cu" else CXXFLAGS
    cmd = [NVCC, *flags, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    OBJ.mkdir(exist_ok=True)
    OUT.mkdir(exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [NVCC, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle() -> Path:
    """Build the CPU oracle (test infrastructure) with its Makefile."""
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{r.stdout}\n{r.stderr}")
    return ROOT / "oracle" / "build" / "libhella_oracle.so"


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    build_oracle()
