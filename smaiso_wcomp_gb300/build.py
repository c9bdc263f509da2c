"""In-tree build of libswc.so (the sm_103a CUDA library) with nvcc.

The four translation units compile in parallel; only one -gencode
(arch=compute_103a, code=sm_103a) is emitted. Output: _build/libswc.so.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
SOURCES = ["swc_abi.cu", "swc_plan.cu", "swc_step_fp64.cu", "swc_step_fp64_b.cu", "swc_step_fp64_c.cu",
           "swc_step_mixed.cu", "swc_step_mixed_b.cu", "swc_step_mixed_c.cu", "swc_step_mixed_adj.cu",
           "swc_noalloc.cu", "swc_ic.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    lib = os.path.join(OUT, "libswc.so")
    cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *[o for o, _ in results], "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    # C++ host driver with the reference's command line, linked against libswc.so
    exe = os.path.join(OUT, "swc_run")
    cmd = [shutil.which("g++") or "g++", "-O2", "-std=c++17", os.path.join(CSRC, "swc_run.cpp"), "-o", exe,
           f"-L{OUT}", "-lswc", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"swc_run build failed:\n{r.stderr}")
    return lib


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:]))
