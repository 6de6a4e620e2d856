"""Build the CUDA library ``libefs_gb300.so`` in-tree with nvcc for sm_103a.

The translation units compile in parallel, then link into one shared library next to this file.  The
simulation units use ``--fmad=false`` so every product and sum rounds separately (the reference CPU build's
float semantics); nothing else changes the compiler's IEEE defaults (no fast math).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libefs_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
UNITS = {
    "efs_api.cu": ["--fmad=false"],
    "efs_fields.cu": ["--fmad=false"],
    "efs_stages.cu": ["--fmad=false"],
    "efs_solver.cu": ["--fmad=false"],
    "efs_noalloc.cu": ["--fmad=false"],
    "efs_unet.cu": [],
    "efs_mlfcg.cu": [],
    "efs_batch.cu": ["--fmad=false"],
    "efs_scene.cu": ["--fmad=false"],
}


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libefs_gb300.so")
    return path


def _compile(src, extra, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + (["-Xptxas", "-v"] if verbose else []) + \
        ["-c", os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr}")
    return obj, res.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "efs_gb300.h"))
    deps.append(os.path.join(HERE, "..", "include", "efs_scene.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile and link; returns the library path.  Skips the work when the library is newer than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, src, extra, verbose) for src, extra in UNITS.items()]
        results = [f.result() for f in futs]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
