"""Builds libSvtJpegxs.so (host C + sm_103a CUDA) in-tree.

    python svt-jpeg-xs_gb300/build.py [--force]

Host C files are compiled with gcc, CUDA files with nvcc for sm_103a only,
in parallel; the shared library links the CUDA runtime statically and lands
in svt-jpeg-xs_gb300/_build/.  Rebuilds only what changed.

install(prefix) lays the library out the way the reference's install step
does (Source/Lib/CMakeLists.txt, Source/Lib/pkg-config.pc.in), so that a
plugin build that finds SVT-JPEG-XS through pkg-config finds this one:
  <prefix>/include/svt-jpegxs/*.h
  <prefix>/lib/libSvtJpegxs.so.0, libSvtJpegxs.so -> libSvtJpegxs.so.0
  <prefix>/lib/pkgconfig/SvtJpegxs.pc
build() installs into svt-jpeg-xs_gb300/_build/install.
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
INSTALL = os.path.join(OUT, "install")
VERSION = "0.10.0"  # the reference's project version, whose API this library implements

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
    install(INSTALL)
    return LIB


PC_TEMPLATE = """prefix={prefix}
exec_prefix=${{prefix}}
includedir=${{prefix}}/include
libdir=${{exec_prefix}}/lib

Name: SvtJpegxs
Description: JPEG XS encoder and decoder (SVT-JPEG-XS API) on one NVIDIA GB300 GPU
Version: {version}
Libs: -L${{libdir}} -lSvtJpegxs
Libs.private: -lpthread
Cflags: -I${{includedir}}/svt-jpegxs
"""


def install(prefix):
    """Copies the headers and the library into the reference's install
    layout under prefix and writes SvtJpegxs.pc; returns the .pc path."""
    inc = os.path.join(prefix, "include", "svt-jpegxs")
    lib = os.path.join(prefix, "lib")
    pcdir = os.path.join(lib, "pkgconfig")
    for d in (inc, pcdir):
        os.makedirs(d, exist_ok=True)
    for h in glob.glob(os.path.join(INC, "*.h")):
        shutil.copy2(h, os.path.join(inc, os.path.basename(h)))
    so0 = os.path.join(lib, "libSvtJpegxs.so.0")
    if not os.path.exists(so0) or os.path.getmtime(so0) < os.path.getmtime(LIB):
        shutil.copy2(LIB, so0)
    link = os.path.join(lib, "libSvtJpegxs.so")
    if not os.path.lexists(link):
        os.symlink("libSvtJpegxs.so.0", link)
    pc = os.path.join(pcdir, "SvtJpegxs.pc")
    with open(pc, "w") as fh:
        fh.write(PC_TEMPLATE.format(prefix=os.path.abspath(prefix), version=VERSION))
    return pc


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
