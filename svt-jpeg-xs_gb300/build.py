"""Builds libSvtJpegxs.so (host C + sm_103a CUDA) in-tree.

    python svt-jpeg-xs_gb300/build.py [--force]

Host C files are compiled with gcc, CUDA files with nvcc for sm_103a only,
in parallel; the shared library links the CUDA runtime statically and lands
in svt-jpeg-xs_gb300/_build/.  Rebuilds only what changed.
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
INC = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libSvtJpegxs.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INC, "*.h"))


def _compile(src, force):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if not force and not _newer(obj, [src] + _headers()):
        return obj, None
    if src.endswith(".cu"):
        cmd = [_nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INC, "-c", src, "-o", obj]
    else:
        cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter", "-I", CSRC, "-I", INC,
               "-I", "/usr/local/cuda/include", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, (r.stdout + r.stderr).strip() or None


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.c")) + glob.glob(os.path.join(CSRC, "*.cu")))
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    objs = [o for o, _ in results]
    for _, msg in results:
        if msg and verbose:
            print(msg)
    if force or _newer(LIB, objs):
        cmd = [_nvcc(), "-shared", *ARCH, "-cudart", "static", "-o", LIB, *objs, "-Xlinker", "-soname,libSvtJpegxs.so.0",
               "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        link0 = os.path.join(OUT, "libSvtJpegxs.so.0")
        if os.path.lexists(link0):
            os.remove(link0)
        os.symlink("libSvtJpegxs.so", link0)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
