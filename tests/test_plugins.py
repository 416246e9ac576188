"""The reference's own plugin sources on this library.

The FFmpeg plugin (ffmpeg-plugin/libsvtjpegxs{enc,dec}.c) and the IMTL
ST 2110-22 plugin (imtl-plugin/src/st22_svt_jpeg_xs_plugin.c) are compiled
unchanged against include/ and linked against libSvtJpegxs.so with no
undefined symbol.  tests/plugin_stubs/ stands in for the FFmpeg and IMTL
declarations they use, and tests/plugin_{ffmpeg,mtl}_host.c play the host
framework: libavcodec's encode / decode calls (option defaults from the
codec's AVOption table, packets, frames from ff_get_buffer) and IMTL's
pipeline (a session whose frames the plugin's own threads take and put back).

On the GPU the plugins then encode and decode through this library, and
their output is compared bit for bit with the library's direct API (itself
pinned on the reference by the other tests).  The plugin sources are read
from the reference tree (JXS_REFERENCE) or from the copy that
__graft_entry__.build() stages under baseline/_ref/src; without either the
tests skip.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
STUBS = os.path.join(ROOT, "tests", "plugin_stubs")


def plugin_root():
    for d in (os.environ.get("JXS_REFERENCE", "/root/reference"), os.path.join(ROOT, "baseline", "_ref", "src")):
        if os.path.exists(os.path.join(d, "ffmpeg-plugin", "libsvtjpegxsenc.c")) and \
                os.path.exists(os.path.join(d, "imtl-plugin", "src", "st22_svt_jpeg_xs_plugin.c")):
            return d
    return None


@pytest.fixture(scope="session")
def plugin_libs(jxs_lib, tmp_path_factory):
    src = plugin_root()
    if src is None:
        pytest.skip("plugin sources not present (reference tree or staged copy)")
    out = tmp_path_factory.mktemp("plugins")
    lib_dir = os.path.dirname(jxs_lib.LIB_PATH)
    common = ["gcc", "-std=gnu11", "-Wall", "-Werror", "-shared", "-fPIC", "-I", STUBS, "-I", INCLUDE, "-L", lib_dir,
              "-Wl,-rpath," + lib_dir, "-Wl,--no-undefined"]
    ff = str(out / "libffplug.so")
    subprocess.check_call(common + [os.path.join(src, "ffmpeg-plugin", "libsvtjpegxsenc.c"),
                                    os.path.join(src, "ffmpeg-plugin", "libsvtjpegxsdec.c"),
                                    os.path.join(ROOT, "tests", "plugin_ffmpeg_host.c"), "-o", ff, "-lSvtJpegxs"])
    mtl = str(out / "libmtlplug.so")
    subprocess.check_call(common + [os.path.join(src, "imtl-plugin", "src", "st22_svt_jpeg_xs_plugin.c"),
                                    os.path.join(ROOT, "tests", "plugin_mtl_host.c"), "-o", mtl, "-lSvtJpegxs", "-lpthread"])
    return ctypes.CDLL(ff), ctypes.CDLL(mtl)


def test_plugin_sources_compile_and_link(plugin_libs):
    ff, mtl = plugin_libs
    for name in ("ff_libsvtjpegxs_encoder", "ff_libsvtjpegxs_decoder", "ffh_encode", "ffh_decode"):
        assert hasattr(ff, name), name
    for name in ("st_plugin_create", "st_plugin_free", "st_plugin_get_meta", "mtlh_encode", "mtlh_decode"):
        assert hasattr(mtl, name), name


def test_imtl_plugin_meta(plugin_libs):
    _, mtl = plugin_libs
    version, magic = ctypes.c_int(), ctypes.c_uint()
    assert mtl.mtlh_meta(ctypes.byref(version), ctypes.byref(magic)) == 0
    assert version.value == 1 and magic.value == 0x5650314C


# --- on the GPU ----------------------------------------------------------
AV_PIX_FMT_YUV422P, AV_PIX_FMT_YUV422P10LE = 1, 4  # plugin_stubs/ffstub.h


def _padded(planes, align):
    """Planes copied into rows of `align`-byte multiples (AVFrame line sizes)."""
    out, ls = [], []
    for p in planes:
        row = p.shape[1] * p.itemsize
        pitch = (row + align - 1) // align * align + align
        buf = np.zeros((p.shape[0], pitch), np.uint8)
        buf[:, :row] = p.view(np.uint8).reshape(p.shape[0], row)
        out.append(buf)
        ls.append(pitch)
    return out, ls


def _unpad(bufs, planes_like):
    return [b[:, :p.shape[1] * p.itemsize].copy().view(p.dtype).reshape(p.shape) for b, p in zip(bufs, planes_like)]


@pytest.mark.gpu
@pytest.mark.parametrize("depth,bpp", [(10, "3"), (8, "2.5")])
def test_ffmpeg_plugin_encode_decode(gpu, plugin_libs, depth, bpp):
    import jxs_synth

    ff, _ = plugin_libs
    w, h = 1920, 1080
    planes = jxs_synth.frame(w, h, depth, jxs_synth.FMT_YUV422, seed=11)
    bufs, ls = _padded(planes, 64)
    ptrs = (ctypes.c_void_p * 3)(*[b.ctypes.data for b in bufs])
    lsz = (ctypes.c_int * 3)(*ls)
    cap = w * h * 4
    out = np.zeros(cap, np.uint8)
    size = ctypes.c_int()
    fmt = AV_PIX_FMT_YUV422P10LE if depth == 10 else AV_PIX_FMT_YUV422P
    r = ff.ffh_encode(bpp.encode(), w, h, fmt, ptrs, lsz, out.ctypes.data_as(ctypes.c_void_p), cap, ctypes.byref(size))
    assert r == 0
    num, den = (int(bpp), 1) if "." not in bpp else (int(bpp.replace(".", "")), 10 ** len(bpp.split(".")[1]))
    enc = gpu.Encoder(w, h, depth, gpu.FMT_YUV422, num, den)
    direct = enc.encode(planes)
    enc.close()
    bs = out[:size.value]
    assert size.value == len(direct) and np.array_equal(bs, direct), "the plugin's codestream differs from the direct API's"
    dec = gpu.Decoder(direct)
    want = dec.decode(direct)
    dec.close()
    for chunks in (1, 3):
        obufs, ols = _padded(planes, 64)
        for b in obufs:
            b[:] = 0
        optrs = (ctypes.c_void_p * 3)(*[b.ctypes.data for b in obufs])
        olsz = (ctypes.c_int * 3)(*ols)
        got, pf, ow, oh = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        r = ff.ffh_decode(bs.ctypes.data_as(ctypes.c_void_p), len(bs), chunks, optrs, olsz, ctypes.byref(got), ctypes.byref(pf),
                          ctypes.byref(ow), ctypes.byref(oh))
        assert r == len(bs) - (chunks - 1) * ((len(bs) + chunks - 1) // chunks) and got.value == 1
        assert (pf.value, ow.value, oh.value) == (fmt, w, h)
        for a, b in zip(_unpad(obufs, planes), want):
            assert np.array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("depth,quality", [(10, 1), (8, 0)])
def test_imtl_plugin_encode_decode(gpu, plugin_libs, depth, quality):
    """quality 1 (QUALITY: uniform quantization, slices of 64 lines) and 0
    (SPEED: no vertical decomposition) are the plugin's two encoder modes."""
    import jxs_synth

    _, mtl = plugin_libs
    w, h, n = 1920, 1080, 4
    frames = [jxs_synth.frame(w, h, depth, jxs_synth.FMT_YUV422, seed=20 + i) for i in range(n)]
    padded = [_padded(f, 128) for f in frames]
    ls = padded[0][1]
    ptrs = (ctypes.c_void_p * (3 * n))(*[b.ctypes.data for bufs, _ in padded for b in bufs])
    lsz = (ctypes.c_size_t * 3)(*ls)
    cs_size = w * h * 3 // 8  # 3 bits per pixel
    cap = cs_size + 4096
    cs = [np.zeros(cap, np.uint8) for _ in range(n)]
    cptrs = (ctypes.c_void_p * n)(*[c.ctypes.data for c in cs])
    sizes = (ctypes.c_size_t * n)()
    done = mtl.mtlh_encode(w, h, depth, quality, n, ptrs, lsz, ctypes.c_size_t(cs_size), cptrs, ctypes.c_size_t(cap), sizes)
    assert done == n
    extra = {"quantization": 1, "slice_height": 64} if quality == 1 else {"ndecomp_v": 0}
    enc = gpu.Encoder(w, h, depth, gpu.FMT_YUV422, 3, **extra)
    direct = [enc.encode(f) for f in frames]
    enc.close()
    for i in range(n):
        assert sizes[i] == len(direct[i]) and np.array_equal(cs[i][:sizes[i]], direct[i]), i
    out = [_padded(f, 128)[0] for f in frames]
    for bufs in out:
        for b in bufs:
            b[:] = 0
    optrs = (ctypes.c_void_p * (3 * n))(*[b.ctypes.data for bufs in out for b in bufs])
    done = mtl.mtlh_decode(w, h, depth, n, cptrs, sizes, ctypes.c_size_t(cap), optrs, lsz)
    assert done == n
    dec = gpu.Decoder(direct[0])
    for i in range(n):
        want = dec.decode(direct[i])
        for a, b in zip(_unpad(out[i], frames[i]), want):
            assert np.array_equal(a, b), i
    dec.close()
