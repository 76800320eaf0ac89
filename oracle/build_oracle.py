"""Build the reference's own litho.cpp (unmodified sources) into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  Compiles validation/golden/src/litho.cpp and
litho_thread.cpp with their common/ helpers straight from the reference
checkout, against two pieces of project code:

* oracle/fftw_shim/fftw3.h + fftw_shim.c -- the FFTW-3 API subset they call,
  implemented with a project-written FP64 FFT (FFTW itself is not installed);
* oracle/fftw_shim/zheevr_fwd.c -- zheevr_ forwarded to scipy_zheevr_ in
  scipy's bundled OpenBLAS (no system LAPACK is installed).

Outputs oracle/_ref/litho and oracle/_ref/litho_thread (git-ignored).  Where the
reference checkout is absent (the GPU host) this is a no-op.

    python oracle/build_oracle.py [/path/to/reference]
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "fftw_shim")
# the reference checkout: the first argument, else $LITHO_REFERENCE_DIR, else this build's checkout
DEFAULT_REF = os.environ.get("LITHO_REFERENCE_DIR", "/root/reference")


def _openblas():
    import scipy
    libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cand = sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so")))
    if not cand:
        raise RuntimeError("scipy's bundled OpenBLAS not found")
    return cand[0]


def build(ref: str = DEFAULT_REF, verbose: bool = False) -> bool:
    src = os.path.join(ref, "validation", "golden", "src")
    if not os.path.exists(os.path.join(src, "litho.cpp")):
        return False
    os.makedirs(OUT, exist_ok=True)
    blas = _openblas()
    shim_objs = []
    for c in ("fftw_shim.c", "zheevr_fwd.c"):
        o = os.path.join(OUT, c + ".o")
        subprocess.run(["gcc", "-O2", "-fPIC", "-c", os.path.join(SHIM, c), "-o", o, "-I", SHIM], check=True)
        shim_objs.append(o)
    common = [os.path.join(src, "common", f) for f in ("file_io.cpp", "mask.cpp", "source.cpp")]
    for prog in ("litho", "litho_thread"):
        exe = os.path.join(OUT, prog)
        srcs = [os.path.join(src, prog + ".cpp")] + common
        newest = max(os.path.getmtime(p) for p in srcs + [os.path.join(SHIM, f) for f in os.listdir(SHIM)])
        if os.path.exists(exe) and os.path.getmtime(exe) >= newest:
            continue
        cmd = (["g++", "-O2", "-std=c++17", "-fopenmp", "-w", "-I", SHIM, "-I", os.path.join(src, "common")]
               + srcs + shim_objs + ["-o", exe, blas, "-Wl,-rpath," + os.path.dirname(blas), "-lm"])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{' '.join(cmd)}\n{r.stderr[-4000:]}")
        if verbose:
            print("built", exe)
    return True


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF, verbose=True))
