"""In-tree build of libbsamg.so for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into
bsam1.2_gb300/libbsamg.so.  The plain-FP64 kernels (fp64.cu) are built with
--fmad=false so that products and sums round separately, in the reference's
order; host code is built with -ffp-contract=off for the same reason (aarch64
compilers contract by default).
"""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbsamg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = {
    "fp64.cu": ["--fmad=false"],
    "noalloc.cu": ["--fmad=false"],
    "mixed.cu": [],
    "box.cu": [],
    "hier.cu": [],
    "ghostc.cpp": [],
    "regrid.cpp": [],
    "io.cu": ["--fmad=false"],
    "frames.cpp": [],
}


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _sources_mtime():
    m = 0.0
    for root, _, files in os.walk(CSRC):
        for f in files:
            m = max(m, os.path.getmtime(os.path.join(root, f)))
    m = max(m, os.path.getmtime(os.path.join(HERE, "..", "include", "bsamg.h")))
    m = max(m, os.path.getmtime(__file__))
    return m


def build(force=False, verbose=False):
    """Compile libbsamg.so if missing or older than its sources."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I", CSRC]

    def compile_one(item):
        src, extra = item
        obj = os.path.join(BUILD, src + ".o")
        cmd = [nvcc] + common + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import time
    t = time.time()
    print(build(force=True, verbose=True), f"{time.time() - t:.1f}s")
