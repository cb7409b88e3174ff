"""Build the CUDA library in-tree: oibvh_gb300/_lib/liboibvh_gb300.so.

Every translation unit under csrc/ is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel, then linked into
one shared library that exports the C ABI of include/oibvh_gb300.h.
Run ``python -m oibvh_gb300.build`` or call ``build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "liboibvh_gb300.so"
LIB = os.path.join(LIBDIR, LIBNAME)
OBJDIR = os.path.join(LIBDIR, "obj")
SOURCES = ["build_kernels.cu", "refit_kernels.cu", "detect_kernels.cu", "host.cu", "noalloc.cu", "serve.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"),
            os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found (set NVCC or CUDA_HOME)")


def _inputs():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    files.append(os.path.join(ROOT, "include", "oibvh_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = nvcc_path()
    os.makedirs(OBJDIR, exist_ok=True)
    common = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if ptxas_verbose:
        common += ["-Xptxas", "-v"]

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
        cmd = [*common, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, (r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose or ptxas_verbose:
        for obj, log in results:
            if log.strip():
                print(f"--- {os.path.basename(obj)}\n{log}", file=sys.stderr)
    tmp = LIB + f".{os.getpid()}.tmp"
    # --no-undefined: a symbol missing from the library fails the build here,
    # not the first load on a GPU host
    cmd = [nvcc, *ARCH, "-shared", "-Xlinker", "--no-undefined", "-o", tmp, *[o for o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas-v" in sys.argv))
