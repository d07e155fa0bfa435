"""Build libpairs_gb300.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
pairs_gb300/_lib/libpairs_gb300.so.  No cmake, no torch extension machinery: the
library has a plain C ABI (include/pairs_gb300.h) and is loaded with ctypes.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libpairs_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-I", INCLUDE, "-I", CSRC]
# per-file flags: the FP64 DEM kernels follow the reference's operation order with
# every multiply and add separately rounded
FILE_FLAGS = {"dem.cu": ["-fmad=false"],
              # the DEM grid's host-side axis coordinates (ref + k * spacing) must not be
              # contracted into a fused multiply-add (the host compiler on aarch64 would)
              "demgrid.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpairs_gb300.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _digest(paths):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(p.encode() + b"\0" + f.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + sorted(str(FILE_FLAGS).split())).encode())
    return h.hexdigest()


def build(force=False, verbose=False, extra_flags=()):
    """Compile every .cu under csrc/ and link the shared library.  Returns its path."""
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    digest = _digest(srcs + sorted(headers))
    stamp = os.path.join(LIBDIR, ".digest")
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [cc, "-c", src, "-o", obj] + ARCH + NVCC_FLAGS + FILE_FLAGS.get(os.path.basename(src), []) + \
            list(extra_flags)
        if verbose:
            cmd += ["-Xptxas", "-v"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stderr}")
        return obj, res.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose:
        for obj, log in results:
            print(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
