"""In-tree build of libbsamg.so for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into
bsam1.2_gb300/libbsamg.so.  The plain-FP64 kernels (fp64.cu) are built with
--fmad=false so that products and sums round separately, in the reference's
order; host code is built with -ffp-contract=off for the same reason (aarch64
compilers contract by default).

Every problem plugin in plugins/ (one file per problem, the device side of
PROBLEM/<name>/problem.f90) is compiled twice: its FP64 part with
-DBSAMG_PART_FP64 --fmad=false and its mixed-precision part with
-DBSAMG_PART_MIXED.  A new plugin file is picked up by the next build; no
other file changes.  build(extra_plugins=[...], lib=...) links plugin files
kept elsewhere into a separate library.
"""
import concurrent.futures as cf
import os
import subprocess
import zlib

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbsamg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

PLUGINS = os.path.join(HERE, "plugins")
UNITS = {
    "plugin.cu": [],
    "fp64.cu": ["--fmad=false"],
    "noalloc.cu": ["--fmad=false"],
    "mixed.cu": [],
    "box.cu": [],
    "tune.cu": [],
    "hier.cu": [],
    "ghostc.cpp": [],
    "pool.cpp": [],
    "regrid.cpp": [],
    "io.cu": ["--fmad=false"],
    "frames.cpp": [],
}


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _plugin_files():
    return sorted(os.path.join(PLUGINS, f) for f in os.listdir(PLUGINS) if f.endswith(".cu"))


def _sources_mtime(extra=()):
    m = 0.0
    for d in (CSRC, PLUGINS):
        for root, _, files in os.walk(d):
            for f in files:
                m = max(m, os.path.getmtime(os.path.join(root, f)))
    for f in extra:
        m = max(m, os.path.getmtime(f))
    m = max(m, os.path.getmtime(os.path.join(HERE, "..", "include", "bsamg.h")))
    m = max(m, os.path.getmtime(__file__))
    return m


def build(force=False, verbose=False, extra_plugins=(), lib=None):
    """Compile libbsamg.so if missing or older than its sources.  With
    extra_plugins (paths of plugin files outside plugins/), link them too
    into `lib` (a path), leaving the default library alone."""
    out = lib or LIB
    extra = [os.path.abspath(p) for p in extra_plugins]
    if not force and os.path.exists(out) and os.path.getmtime(out) >= _sources_mtime(extra):
        return out
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I", CSRC]
    jobs = [(os.path.join(CSRC, src), src + ".o", extra_flags) for src, extra_flags in UNITS.items()]
    for path in _plugin_files() + extra:
        tag = "plugin_" + os.path.splitext(os.path.basename(path))[0]
        if path in extra:
            tag += "_x%08x" % zlib.crc32(path.encode())
        jobs.append((path, tag + ".fp64.o", ["-DBSAMG_PART_FP64", "--fmad=false"]))
        jobs.append((path, tag + ".mixed.o", ["-DBSAMG_PART_MIXED"]))

    def compile_one(job):
        path, objname, extra_flags = job
        obj = os.path.join(BUILD, objname)
        if not force and os.path.exists(obj) and os.path.getmtime(obj) >= _sources_mtime():
            if path not in extra or os.path.getmtime(obj) >= os.path.getmtime(path):
                return obj
        cmd = [nvcc] + common + extra_flags + ["-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(path)}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(compile_one, jobs))
    tmp = out + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    import time
    t = time.time()
    print(build(force=True, verbose=True), f"{time.time() - t:.1f}s")
