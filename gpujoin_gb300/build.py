"""Build libgpujoin.so in-tree with nvcc for sm_103a (GB300).

Every translation unit under csrc/ is compiled in parallel into _build/ and
linked into gpujoin_gb300/libgpujoin.so.  Run ``python -m gpujoin_gb300.build``
or call :func:`build`.  Set ``GJ_NVCC_EXTRA`` to add flags (for example
``-Xptxas -v`` to print register and shared-memory use).
"""
from __future__ import annotations

import concurrent.futures
import os
import shlex
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.environ.get("GJ_BUILD_DIR", os.path.join(HERE, "_build"))
LIB = os.environ.get("GJ_LIB_PATH", os.path.join(HERE, "libgpujoin.so"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    inc = os.path.join(ROOT, "include")
    found = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    for d, _, files in os.walk(inc):
        found += [os.path.join(d, f) for f in files if f.endswith((".h", ".cuh"))]
    return found


def _compile(src: str, extra) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + headers()
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", src, "-o", obj, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr}\n{shlex.join(cmd)}")
    if r.stderr.strip() and "-Xptxas" in " ".join(extra):
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    extra = shlex.split(os.environ.get("GJ_NVCC_EXTRA", ""))
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(os.cpu_count() or 8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
