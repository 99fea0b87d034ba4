"""Build libgblu.so in-tree with nvcc for sm_103a (no CMake).

Each .cu translation unit compiles in parallel to an object file under
``_build/``; they link into ``libgblu.so`` next to this file.  Rebuilds only
what changed (source or header newer than its object).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgblu.so")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--fmad=false",
    "-Xptxas", "-warn-spills", "-I", CSRC, "-I", INCLUDE,
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library needs the CUDA toolkit")


def _cuda_lib_dir(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")


def _headers_mtime() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hs += glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def build(verbose: bool = False, force: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hmt = _headers_mtime()
    todo = []
    objs = []
    for src in srcs:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hmt):
            todo.append((src, obj))

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        os.replace(obj + ".tmp", obj)
        return src, r.stderr

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for src, err in ex.map(compile_one, todo):
                if verbose and err.strip():
                    print(f"[{os.path.basename(src)}]\n{err}")
    newest = max(os.path.getmtime(o) for o in objs)
    if force or todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        libdir = _cuda_lib_dir(nvcc)
        tmp = LIB + f".{os.getpid()}.tmp"
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs,
               "-Xlinker", "-rpath", "-Xlinker", libdir, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    _build_tool(nvcc, TOOL_LIB)
    return LIB


TOOL_LIB = os.path.join(HERE, "libgblu_tools.so")


def _build_tool(nvcc: str, out: str) -> None:
    """Measurement and check helpers used by bench.py and tests (not part of the C ABI)."""
    srcs = sorted(glob.glob(os.path.join(CSRC, "tools", "*.cu")))
    newest = max([os.path.getmtime(x) for x in srcs] + [_headers_mtime()])
    if os.path.exists(out) and os.path.getmtime(out) >= newest:
        return
    tmp = out + f".{os.getpid()}.tmp"
    cmd = [nvcc, *ARCH, "-O3", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC", "-shared",
           "-cudart", "shared", "-I", CSRC, "-I", INCLUDE, "-o", tmp, *srcs,
           "-Xlinker", "-rpath", "-Xlinker", _cuda_lib_dir(nvcc)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on tools/:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv))
