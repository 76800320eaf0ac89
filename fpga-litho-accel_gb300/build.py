"""Build liblitho_gb300.so (sm_103a) in-tree.

Each .cu / .cpp under csrc/ is compiled to an object in parallel with nvcc, then
linked into ``litho_gb300/liblitho_gb300.so`` next to the Python binding.  The
CLI ``litho_gb300_cli`` is linked against the same objects.

    python fpga-litho-accel_gb300/build.py [-v]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "litho_gb300", "liblitho_gb300.so")
CLI = os.path.join(HERE, "litho_gb300", "litho_gb300_cli")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def nvcc() -> str:
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found (CUDA toolkit required to build liblitho_gb300)")
    return p


def _flags(verbose: bool):
    f = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-O3", "-I" + os.path.join(HERE, "..", "include")] + ARCH
    if verbose:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src: str, verbose: bool):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and all(os.path.getmtime(obj) >= os.path.getmtime(os.path.join(CSRC, h))
                    for h in os.listdir(CSRC) if h.endswith((".cuh", ".h", ".hpp")))
            and os.path.getmtime(obj) >= os.path.getmtime(os.path.join(HERE, "..", "include", "litho_gb300.h"))):
        return obj, ""
    cmd = [nvcc(), "-c", src, "-o", obj] + _flags(verbose)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stdout + r.stderr


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")) and f != "cli.cpp")
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src):
        cmd = [nvcc(), "-O2", "-std=c++17", cli_src, "-o", CLI, "-I" + os.path.join(HERE, "..", "include"),
               "-L" + os.path.dirname(LIB), "-llitho_gb300", "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
