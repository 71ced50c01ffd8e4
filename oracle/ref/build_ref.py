"""Build the reference's stage code for the CPU (TEST INFRASTRUCTURE ONLY).

Reads the read-only reference tree (the first argument, or $HELLA_REF),
copies the stage sources it needs into a temporary directory, rewrites each
kernel launch `k<<<grid, block>>>(args)` into a call of the emulator in
emu_cuda.h, sets NCHAN (a compile-time constant of the reference,
src/hella/definitions.h:44) to the fixture size, and compiles everything
with g++ into oracle/_ref/libhella_ref_emu.so (git-ignored).  No reference
source is written into this repository.

Kernels keep the multiply-add fusion nvcc applies to device code
(-ffp-contract=fast with FMA, per kernel); host code is compiled without
contraction, as the reference's x86 host build is.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
SOURCES = ["flagger.cu", "normalization.cu", "transpose.cu", "timeseries.cu", "convolution.cu",
           "median_filter.cpp", "alloc.cpp", "smooth.cpp", "peaks.cu"]
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _split_top(s: str) -> list[str]:
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def _kernels_needing_fibers(src: str) -> set[str]:
    """Kernels whose bodies synchronise (barriers or warp shuffles)."""
    names = set()
    for m in re.finditer(r"__global__\s+void\s+(\w+)\s*\(", src):
        i = src.index("{", m.end())
        depth, j = 0, i
        while True:
            if src[j] == "{":
                depth += 1
            elif src[j] == "}":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        body = src[i:j]
        if "__syncthreads" in body or "__shfl" in body:
            names.add(m.group(1))
    return names


def rewrite_launches(src: str, coop: set[str]) -> str:
    out, i = [], 0
    while True:
        j = src.find("<<<", i)
        if j < 0:
            out.append(src[i:])
            return "".join(out)
        k = j
        while k > 0 and (src[k - 1].isalnum() or src[k - 1] == "_"):
            k -= 1
        name = src[k:j]
        e = src.find(">>>", j)
        cfg = _split_top(src[j + 3:e])
        p = src.find("(", e)
        depth, q = 0, p
        while True:
            if src[q] == "(":
                depth += 1
            elif src[q] == ")":
                depth -= 1
                if depth == 0:
                    break
            q += 1
        args = src[p + 1:q]
        flag = "true" if name in coop else "false"
        out.append(src[i:k])
        out.append(f"emu::launch(dim3({cfg[0]}), dim3({cfg[1]}), {flag}, [&]() {{ {name}({args}); }})")
        i = q + 1


def build(ref: Path, nchan: int = 256, verbose: bool = False) -> Path:
    ref = Path(ref)
    if not (ref / "src/hella/src/flagger.cu").exists():
        raise FileNotFoundError(f"reference sources not found under {ref}")
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libhella_ref_emu.so"
    with tempfile.TemporaryDirectory(prefix="hella_ref_") as tmp:
        tmp = Path(tmp)
        (tmp / "hella").mkdir()
        for h in (ref / "src/hella").glob("*.h"):
            text = h.read_text()
            if h.name == "definitions.h":
                text = re.sub(r"#define NCHAN \d+", f"#define NCHAN {nchan}", text)
            (tmp / "hella" / h.name).write_text(text)
        all_src = "".join((ref / "src/hella/src" / s).read_text() for s in SOURCES)
        coop = _kernels_needing_fibers(all_src)
        objs = []
        common = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", str(tmp), "-I",
                  str(HERE / "shim"), "-I", f"{CUDA}/include", "-I", f"{CUDA}/include/cccl", "-include", str(HERE / "emu_cuda.h"),
                  "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", "-w"]
        for s in SOURCES:
            text = (ref / "src/hella/src" / s).read_text()
            # device code keeps nvcc's default multiply-add fusion; kernels
            # stay out of line so the host callers' setting cannot apply
            text = text.replace("__global__",
                                "__attribute__((noinline, optimize(\"fp-contract=fast\"), target(\"fma\")))")
            text = rewrite_launches(text, coop)
            dst = tmp / (Path(s).stem + "_emu.cpp")
            dst.write_text(text)
            obj = tmp / (dst.stem + ".o")
            # The .cu files carry the kernels: fuse multiply-adds as nvcc does
            # for device code (their host parts hold no fusable expression);
            # the .cpp files are host code and are built without fusion.
            fuse = (["-ffp-contract=fast", "-mfma", "--param", "avoid-fma-max-bits=0"]
                    if s.endswith(".cu") else [])
            cmd = common + fuse + ["-c", str(dst), "-o", str(obj)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{s}: {r.stderr[:4000]}")
            objs.append(obj)
        for s in ("emu_cuda.cpp", "ref_driver.cpp"):
            obj = tmp / (Path(s).stem + ".o")
            r = subprocess.run(common + ["-c", str(HERE / s), "-o", str(obj)], capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{s}: {r.stderr[:4000]}")
            objs.append(obj)
        r = subprocess.run(["g++", "-shared", "-o", str(lib), *map(str, objs)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stderr[:4000])
    if verbose:
        print(f"built {lib} (NCHAN={nchan}, fiber kernels: {sorted(coop)})")
    return lib


def reference_tree(argv: list[str]) -> Path:
    """The reference tree: argv[1], else $HELLA_REF; there is no default."""
    path = argv[1] if len(argv) > 1 else os.environ.get("HELLA_REF")
    if not path:
        raise SystemExit(f"usage: python {Path(argv[0]).name} <reference tree>  (or set HELLA_REF)")
    return Path(path)


if __name__ == "__main__":
    import sys

    build(reference_tree(sys.argv), verbose=True)
