"""Build liblentils_gb300.so (the C-ABI library) in-tree for sm_103a with nvcc.

Usage: ``python -m lentils_gb300.build`` or ``lentils_gb300.build.build()``. Translation units
compile in parallel into ``lentils_gb300/_build`` and link into
``lentils_gb300/liblentils_gb300.so``; a unit is recompiled only when it or a header changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblentils_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                  "-I", CSRC, "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


# Per-unit flags: the manifold rasteriser and the direct Fourier sum reproduce the reference's
# plain-C FP64 arithmetic, so multiply-adds are not fused there.
UNIT_FLAGS = {"manifold.cu": ["-fmad=false"], "dft.cu": ["-fmad=false"]}


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and os.path.getmtime(obj) >= _newest_header() and not extra):
        return obj, ""
    cmd = [nvcc_path(), *NVFLAGS, *UNIT_FLAGS.get(os.path.basename(src), []), *extra, "-c", src,
           "-o", obj]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{out.stdout}{out.stderr}")
    return obj, out.stdout + out.stderr


def build(verbose=False, extra_flags=()):
    """Compile every CUDA translation unit and link liblentils_gb300.so. Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = list(extra_flags)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    if (not extra and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs)):
        return LIB
    cmd = [nvcc_path(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcufft",
           "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{out.stdout}{out.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
