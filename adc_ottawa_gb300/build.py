"""Build recipe for libadcgpu.so (sm_103a).

Compiles every translation unit under csrc/ with nvcc in parallel and links
one shared library in-tree at adc_ottawa_gb300/_lib/libadcgpu.so.  Runs on a
machine without a GPU (nvcc cross-compiles for sm_103a).

Per-file flags: the matrix-element kernels (build_kernels.cu) are compiled
with --fmad=false so that every product and sum is rounded separately, as in
the reference's FP64 expressions; host files use -ffp-contract=off for the
same reason (the synthetic generator must be bit-identical across hosts).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUTDIR = os.path.join(HERE, "_lib")
BUILDDIR = os.path.join(HERE, "_build")
LIBNAME = "libadcgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
SOURCES = [
    ("synth.cpp", []),
    ("hostla.cpp", []),
    ("context.cu", []),
    ("build_kernels.cu", ["--fmad=false"]),
    ("sigma.cu", []),
    ("sigma_umma.cu", []),
    ("sigma_ab.cu", []),
    ("dense.cu", []),
    ("dense_umma.cu", []),
    ("precond_fold.cu", []),
    ("davidson.cu", []),
    ("lanczos.cu", []),
    ("sil.cu", []),
    ("chebyshev.cu", []),
    ("mlp.cu", []),
    ("fvec.cu", ["--fmad=false"]),
    ("cvs.cu", []),
]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _compile(src: str, extra: list[str]) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILDDIR, src + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(
        os.path.getmtime(path), *[os.path.getmtime(os.path.join(CSRC, h)) for h in os.listdir(CSRC) if h.endswith(".h") or h.endswith(".cuh")],
        os.path.getmtime(os.path.join(HERE, "..", "include", "adcgpu.h")),
    ):
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj, "-std=c++17", "-O3", "-lineinfo", *ARCH,
           "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off", "-I", os.path.join(HERE, "..", "include"),
           "--expt-relaxed-constexpr", *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUTDIR, exist_ok=True)
    os.makedirs(BUILDDIR, exist_ok=True)
    srcs = [(s, f) for s, f in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda sf: _compile(*sf), srcs))
    out = os.path.join(OUTDIR, LIBNAME)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(out) or os.path.getmtime(out) < newest:
        cmd = [nvcc(), "-shared", *ARCH, "-o", out, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(out)
    return out


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
