"""Build the in-tree shared library libngspice_gb300.so (CUDA, sm_103a).

Each translation unit under csrc/ is compiled in parallel with nvcc into
build/, then linked with -shared.  Only one -gencode target is produced:
compute_103a / sm_103a (GB300).  Re-running is incremental on timestamps.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
BUILD = os.path.join(ROOT, "build")
LIB = os.path.join(PKG, "lib", "libngspice_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Floating-point contraction is off on both sides: the reference's x86-64
# build evaluates a*b+c unfused, and the Arm host compiler would otherwise
# fuse host-side parameter arithmetic; --fmad=false keeps the device
# arithmetic of the model equations unfused as well.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off",
          "--fmad=false", f"-I{CSRC}", f"-I{INCLUDE}"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


# engine.cu is compiled in three parts (NGSF_PART 1-3: the batched
# transient kernel, the wide launch, the operator surface and probes), in
# parallel with the other translation units: ptxas spends about a minute on
# each transient kernel
ENGINE_PARTS = 3


def sources() -> list[tuple[str, int]]:
    out = []
    for f in sorted(os.listdir(CSRC)):
        if not f.endswith((".cu", ".cpp")):
            continue
        path = os.path.join(CSRC, f)
        if f == "engine.cu":
            out += [(path, k) for k in range(1, ENGINE_PARTS + 1)]
        else:
            out.append((path, 0))
    return out


def _compile(item: tuple[str, int]) -> str:
    src, part = item
    obj = os.path.join(BUILD, os.path.basename(src) + (f".{part}" if part else "") + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh", ".def"))]
    deps += [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith((".h", ".cuh", ".def"))]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + ["-c", src, "-o", obj]
    if part:
        cmd.append(f"-DNGSF_PART={part}")
    if src.endswith(".cu") and os.environ.get("NGSF_TRAN_MAXNREG"):
        cmd.append(f"-DNGSF_TRAN_MAXNREG={int(os.environ['NGSF_TRAN_MAXNREG'])}")
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if os.environ.get("NGSF_PTXAS_VERBOSE") else []
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    if os.environ.get("NGSF_PTXAS_VERBOSE") and p.stderr:
        sys.stderr.write(p.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if (not os.path.exists(LIB) or
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs)):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
