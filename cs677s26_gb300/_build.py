"""In-tree build of libvjgb.so (CUDA kernels for sm_103a + C++ host code).

Objects go to cs677s26_gb300/_build/, the library to cs677s26_gb300/libvjgb.so.
Translation units compile in parallel; the build is incremental on source and
header modification times.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libvjgb.so"
INCLUDE = PKG.parent / "include"

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code: no FMA contraction, so float arithmetic is the same on x86 and Arm.
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
            "-Wall", "-Wno-unused-function"]
# Device code: IEEE rounding on every operation (--fmad=false); fused
# multiply-adds appear only where a kernel calls fmaf/fma explicitly.
NVCCFLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler",
             "-fPIC,-ffp-contract=off", "-Xptxas", "-warn-spills"] + ARCH


def _sources():
    return sorted(CSRC.glob("*.cpp")) + sorted(CSRC.glob("*.cu"))


def _headers():
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return t < src.stat().st_mtime or t < newest_header


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    procs = []
    objs = []
    for src in _sources():
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if not force and not _stale(obj, src, newest_header):
            continue
        if src.suffix == ".cu":
            cmd = [NVCC, *NVCCFLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        else:
            cmd = [CXX, *CXXFLAGS, "-I", str(INCLUDE), "-I", "/usr/local/cuda/include", "-c",
                   str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append((src, text))
        elif verbose and text.strip():
            print(text)
    if failed:
        msg = "\n".join(f"--- {s.name}\n{t}" for s, t in failed)
        raise RuntimeError(f"libvjgb build failed:\n{msg}")
    if force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [NVCC, "-shared", *ARCH, "-o", str(LIB), *map(str, objs), "-lcudart", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("libvjgb link failed:\n" + r.stdout.decode(errors="replace"))
    build_tools(verbose, force)
    return LIB


TOOLS = CSRC / "tools"
BIN = PKG / "bin"


def build_tools(verbose: bool = False, force: bool = False) -> list[Path]:
    """Command-line drop-ins (vj_detect ...) linked against libvjgb.so."""
    BIN.mkdir(exist_ok=True)
    cuda_lib = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "lib64"
    out = []
    procs = []
    newest = max([LIB.stat().st_mtime] + [h.stat().st_mtime for h in TOOLS.glob("*.h")] +
                 [h.stat().st_mtime for h in INCLUDE.glob("*.h")])
    for src in sorted(TOOLS.glob("*.cpp")):
        exe = BIN / src.stem
        out.append(exe)
        if not force and exe.exists() and exe.stat().st_mtime > max(src.stat().st_mtime, newest):
            continue
        cmd = [CXX, *CXXFLAGS, "-I", str(INCLUDE), "-I", "/usr/local/cuda/include", str(src), "-o", str(exe),
               "-L", str(PKG), "-lvjgb", "-L", str(cuda_lib), "-lcudart", "-Wl,-rpath,$ORIGIN/..", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for src, p in procs:
        text, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"{src.name} build failed:\n" + text.decode(errors="replace"))
    return out


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
