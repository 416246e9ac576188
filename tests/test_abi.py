"""The drop-in boundary: exported symbols and struct layouts.

- libSvtJpegxs.so exports every function declared in include/*.h;
- the public structs have the reference's layout (compiled against both
  header sets when the reference sources are present) and the ctypes
  bindings agree with the C layout.
No GPU is used: the library only has to load.
"""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
REF_API = os.path.join(os.environ.get("JXS_REFERENCE", "/root/reference"), "Source", "API")


def declared_functions():
    names = set()
    for fn in sorted(os.listdir(INCLUDE)):
        if fn.endswith(".h"):
            text = open(os.path.join(INCLUDE, fn)).read()
            names.update(re.findall(r"PREFIX_API\s+[\w\s\*]+?\b(svt_jpeg_xs_\w+)\s*\(", text))
    return sorted(names)


def test_all_declared_symbols_exported(jxs_lib):
    names = declared_functions()
    assert len(names) >= 29
    lib = ctypes.CDLL(jxs_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_soname_and_reference_symbol_set(jxs_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", jxs_lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (svt_jpeg_xs_\w+)", out))
    reference_api = {
        "svt_jpeg_xs_encoder_load_default_parameters", "svt_jpeg_xs_encoder_get_image_config", "svt_jpeg_xs_encoder_init",
        "svt_jpeg_xs_encoder_close", "svt_jpeg_xs_encoder_send_picture", "svt_jpeg_xs_encoder_get_packet",
        "svt_jpeg_xs_decoder_init", "svt_jpeg_xs_decoder_close", "svt_jpeg_xs_decoder_get_single_frame_size",
        "svt_jpeg_xs_decoder_get_single_frame_size_with_proxy", "svt_jpeg_xs_decoder_send_frame",
        "svt_jpeg_xs_decoder_send_packet", "svt_jpeg_xs_decoder_get_frame", "svt_jpeg_xs_decoder_send_eoc",
        "svt_jpeg_xs_image_buffer_alloc", "svt_jpeg_xs_image_buffer_free", "svt_jpeg_xs_bitstream_alloc",
        "svt_jpeg_xs_bitstream_free", "svt_jpeg_xs_frame_pool_alloc", "svt_jpeg_xs_frame_pool_free",
        "svt_jpeg_xs_frame_pool_get", "svt_jpeg_xs_frame_pool_release"}
    assert reference_api <= exported
    soname = subprocess.run(["readelf", "-d", jxs_lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "libSvtJpegxs.so.0" in soname


def _layout(include_dir, tmp_path, tag):
    exe = str(tmp_path / ("abi_" + tag))
    subprocess.check_call(["gcc", "-std=gnu11", "-I", include_dir, os.path.join(ROOT, "tests", "abi_layout.c"), "-o", exe])
    return subprocess.run([exe], capture_output=True, text=True, check=True).stdout


def test_layout_matches_reference_headers(tmp_path):
    ours = _layout(INCLUDE, tmp_path, "ours")
    if not os.path.exists(os.path.join(REF_API, "SvtJpegxs.h")):
        pytest.skip("reference headers not present")
    theirs = _layout(REF_API, tmp_path, "ref")
    assert ours == theirs


def test_ctypes_bindings_match_c_layout(jxs_lib, tmp_path):
    lines = dict(l.rsplit(" ", 1) for l in _layout(INCLUDE, tmp_path, "ours2").strip().splitlines())
    checks = {
        "svt_jpeg_xs_encoder_api_t": jxs_lib.EncoderApi, "svt_jpeg_xs_decoder_api_t": jxs_lib.DecoderApi,
        "svt_jpeg_xs_frame_t": jxs_lib.Frame, "svt_jpeg_xs_image_buffer_t": jxs_lib.ImageBuffer,
        "svt_jpeg_xs_bitstream_buffer_t": jxs_lib.BitstreamBuffer, "svt_jpeg_xs_image_config_t": jxs_lib.ImageConfig,
    }
    for cname, py in checks.items():
        assert int(lines[cname]) == ctypes.sizeof(py), cname
        for key, off in lines.items():
            if key.startswith(cname + "."):
                field = key.split(".", 1)[1]
                assert getattr(py, field).offset == int(off), key


def test_plugins_compile_and_link(jxs_lib, tmp_path):
    """The reference's FFmpeg and IMTL plugins' use of the API (types,
    constants, struct members, functions in their call forms;
    tests/plugin_api.c) compiles against include/ and links against
    libSvtJpegxs.so with no unresolved symbol."""
    lib_dir = os.path.dirname(jxs_lib.LIB_PATH)
    so = str(tmp_path / "libplugin_api.so")
    subprocess.check_call(["gcc", "-std=gnu11", "-Wall", "-Werror", "-shared", "-fPIC", "-I", INCLUDE,
                           os.path.join(ROOT, "tests", "plugin_api.c"), "-o", so, "-L", lib_dir, "-lSvtJpegxs",
                           "-Wl,--no-undefined", "-Wl,-rpath," + lib_dir])
    undefined = subprocess.run(["nm", "-D", "--undefined-only", so], capture_output=True, text=True).stdout
    used = set(re.findall(r"(svt_jpeg_xs_\w+)", undefined))
    assert used == {"svt_jpeg_xs_encoder_load_default_parameters", "svt_jpeg_xs_encoder_init", "svt_jpeg_xs_encoder_send_picture",
                    "svt_jpeg_xs_encoder_get_packet", "svt_jpeg_xs_encoder_close",
                    "svt_jpeg_xs_decoder_get_single_frame_size_with_proxy", "svt_jpeg_xs_decoder_init",
                    "svt_jpeg_xs_decoder_send_frame", "svt_jpeg_xs_decoder_get_frame", "svt_jpeg_xs_decoder_close"}
    out = subprocess.run(["nm", "-D", "--defined-only", jxs_lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (svt_jpeg_xs_\w+)", out))
    assert used <= exported


def _pkg_config(pc_path, *fields):
    """pkg-config's --cflags / --libs for one .pc file (no pkg-config tool on
    the build host): variables expanded, the requested fields joined."""
    vars_, keys = {}, {}
    for line in open(pc_path).read().splitlines():
        line = line.strip()
        m = re.match(r"^([A-Za-z_][\w.]*)=(.*)$", line)
        if m:
            vars_[m.group(1)] = m.group(2).strip()
            continue
        m = re.match(r"^([A-Za-z.]+):\s*(.*)$", line)
        if m:
            keys[m.group(1)] = m.group(2).strip()

    def expand(v):
        for _ in range(10):
            v = re.sub(r"\$\{(\w+)\}", lambda mm: vars_[mm.group(1)], v)
        return v

    for k in list(vars_):
        vars_[k] = expand(vars_[k])
    return keys.get("Version"), " ".join(expand(keys[f]) for f in fields).split()


def test_pkg_config_install_layout(jxs_lib, tmp_path):
    """build() installs the reference's layout: headers under
    include/svt-jpegxs, libSvtJpegxs.so.0 and SvtJpegxs.pc (the file FFmpeg's
    --enable-libsvtjpegxs looks up). The plugins' API use compiles and links
    with exactly the flags the .pc file gives."""
    import build as pkg_build

    pc = os.path.join(pkg_build.INSTALL, "lib", "pkgconfig", "SvtJpegxs.pc")
    assert os.path.exists(pc)
    version, flags = _pkg_config(pc, "Cflags", "Libs")
    assert version == "0.10.0"
    inc = [f[2:] for f in flags if f.startswith("-I")]
    assert len(inc) == 1 and inc[0].endswith(os.path.join("include", "svt-jpegxs"))
    for h in ("SvtJpegxs.h", "SvtJpegxsEnc.h", "SvtJpegxsDec.h", "SvtJpegxsImageBufferTools.h"):
        assert open(os.path.join(inc[0], h)).read() == open(os.path.join(INCLUDE, h)).read()
    libdir = [f[2:] for f in flags if f.startswith("-L")][0]
    assert os.path.realpath(os.path.join(libdir, "libSvtJpegxs.so")) == os.path.join(libdir, "libSvtJpegxs.so.0")
    so = str(tmp_path / "libplugin_pc.so")
    subprocess.check_call(["gcc", "-std=gnu11", "-Wall", "-Werror", "-shared", "-fPIC", os.path.join(ROOT, "tests", "plugin_api.c"),
                           "-o", so, *flags, "-Wl,--no-undefined", "-Wl,-rpath," + libdir])
    needed = subprocess.run(["readelf", "-d", so], capture_output=True, text=True).stdout
    assert "libSvtJpegxs.so.0" in needed


def test_include_guards_are_the_references():
    """Code that tests the reference headers' include-guard macros sees them
    defined by these headers too."""
    guards = {"SvtJpegxs.h": "_SVT_JPEG_XS_API_H_", "SvtJpegxsEnc.h": "_SVT_JPEG_XS_API_ENC_H_",
              "SvtJpegxsDec.h": "_SVT_JPEG_XS_API_DEC_H_",
              "SvtJpegxsImageBufferTools.h": "_SVT_JPEG_XS_API_IMAGE_BUFFER_TOOLS_H_"}
    for h, g in guards.items():
        text = open(os.path.join(INCLUDE, h)).read()
        assert "#ifndef %s\n#define %s\n" % (g, g) in text, h
        if os.path.exists(os.path.join(REF_API, h)):
            assert ("#ifndef %s" % g) in open(os.path.join(REF_API, h)).read(), h
