"""Compile liblqmc_gpu.so in-tree for sm_103a (GB300) with nvcc.

Each CUDA translation unit under ``csrc/`` is compiled in parallel to an object file in
``_build/`` and linked into ``latticeqmc_gb300/liblqmc_gpu.so`` (static cudart, so the
library loads without a CUDA toolkit on the library path).  Objects are rebuilt only when a
source or header is newer than them, or when the extra nvcc flags differ from those they
were compiled with (``python -m latticeqmc_gb300.build -DNAME=VALUE ...``).

    python -m latticeqmc_gb300.build
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblqmc_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblqmc_gpu.so")


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(nvcc, src, obj, extra):
    cmd = [nvcc, *ARCH, *CFLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose=False, extra=()):
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_t = _newest_header()
    # the objects were compiled with these extra flags; any change rebuilds everything
    stamp = os.path.join(BUILD, "extra_flags.txt")
    flags = " ".join(extra)
    try:
        with open(stamp) as fh:
            same_flags = fh.read() == flags
    except OSError:
        same_flags = not flags
    jobs = []
    objs = []
    for src in srcs:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if (not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_t)
                or not same_flags):
            jobs.append((src, obj))
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = {ex.submit(_compile, nvcc, s, o, list(extra)): s for s, o in jobs}
            for f in concurrent.futures.as_completed(futs):
                msg = f.result()
                if verbose and msg.strip():
                    print(msg, file=sys.stderr)
        with open(stamp, "w") as fh:
            fh.write(flags)
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:]))
