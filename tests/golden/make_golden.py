"""Regenerates the golden fixtures in this directory from the reference
SVT-JPEG-XS library built from its own sources (oracle/_ref, see
oracle/Makefile).  Run in a checkout where the reference is available:

    make -C oracle ref oracle && python tests/golden/make_golden.py [--vpred-only | --proxy-only | --signs-only | --cw-only |
                                                           --mct-only]

Writes
  <case>.npz            small seeded inputs, the reference's codestream and
                        the reference decoder's planes for that codestream
  vpred*.npz            the same for the reference encoder's vertical
                        prediction modes
  signs*.npz            codestreams with separate sign sub-packets
                        (coding_signs_handling 1 / 2), with inputs and the
                        reference decoder's planes
  cw*.npz               multi-column precinct codestreams (Cw > 0) from the
                        oracle's encoder (the reference encoder writes only
                        Cw = 0) and the reference decoder's planes
  mct*.npz, nlt*.npz    colour transform (Cpih = 1, Star-Tetrix Cpih = 3) and
                        output non-linearity
                        codestreams from the oracle's encoder, with the
                        reference decoder's planes (full and half resolution)
  proxy<m>_<case>.npz   the reference decoder's proxy output (m = 1 half,
                        2 quarter resolution) for a small case's codestream
  ref_sample_16x16.npz  the 16x16 4:2:2 codestream of the reference's decoder
                        unit test (tests/UnitTests/SampleFramesData.cc), its
                        frame size and the reference decoder's planes
  full_size.json        sha256 of the reference codestream and decoded
                        planes for the full-size workloads (seeded, integer-
                        only synthetic frames, reproducible on any platform)
"""
import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "svt-jpeg-xs_gb300"))

import jxs_synth as S  # noqa: E402
import oracle_lib as O  # noqa: E402

REFERENCE = os.environ.get("JXS_REFERENCE", "/root/reference")

# name: (w, h, depth, fmt, bpp_num, bpp_den, decomp_v, decomp_h, quant, slice_h, significance, rc_mode, seed)
SMALL_CASES = {
    "c1_422_8b": (64, 32, 8, S.FMT_YUV422, 5, 1, 2, 5, 0, 16, 1, 1, 1),
    "c2_422_10b": (128, 48, 10, S.FMT_YUV422, 3, 1, 2, 5, 0, 16, 1, 1, 2),
    "c3_420_8b": (96, 48, 8, S.FMT_YUV420, 2, 1, 2, 5, 0, 16, 1, 1, 3),
    "c3_444_12b": (64, 32, 12, S.FMT_YUV444, 4, 1, 2, 5, 0, 16, 1, 1, 4),
    "c3_rgb_8b": (128, 32, 8, S.FMT_PACKED_RGB, 4, 1, 2, 5, 0, 16, 1, 1, 5),
    "c4_gbrp_14b_v1": (128, 24, 14, S.FMT_YUV444, 3, 2, 1, 5, 0, 16, 1, 1, 6),
    "odd_444_10b": (53, 37, 10, S.FMT_YUV444, 4, 1, 2, 5, 0, 16, 1, 1, 7),
    "uniform_422_10b": (80, 40, 10, S.FMT_YUV422, 3, 1, 2, 5, 1, 16, 1, 1, 8),
    "nosig_rc0_422_8b": (80, 40, 8, S.FMT_YUV422, 3, 1, 2, 5, 0, 16, 0, 0, 9),
    "v0h3_444_8b": (72, 20, 8, S.FMT_YUV444, 4, 1, 0, 3, 0, 16, 1, 1, 10),
    "v2h2_422_8b": (60, 44, 8, S.FMT_YUV422, 4, 1, 2, 2, 0, 8, 1, 1, 11),
    "raw_rgb_12b_v1": (28, 84, 12, S.FMT_PACKED_RGB, 8, 1, 1, 5, 0, 16, 1, 1, 12),
    "slice_full_422_8b": (96, 40, 8, S.FMT_YUV422, 3, 1, 2, 5, 0, 1000, 1, 1, 13),
}

# Vertical prediction (coding_vertical_prediction_mode 1 and 2 of the reference
# encoder), decoded by the reference decoder; several precinct rows per
# slice so that rows predict from the row above.
# name: (w, h, depth, fmt, bpp_num, bpp_den, decomp_v, decomp_h, quant, slice_h, significance, rc_mode, seed, vpred_mode)
VPRED_CASES = {
    "vpred1_422_8b": (128, 64, 8, S.FMT_YUV422, 3, 1, 2, 5, 0, 32, 1, 1, 21, 1),
    "vpred2_422_10b": (96, 48, 10, S.FMT_YUV422, 4, 1, 2, 5, 0, 48, 1, 1, 22, 2),
    "vpred1_444_8b": (80, 40, 8, S.FMT_YUV444, 5, 1, 2, 4, 0, 40, 1, 1, 23, 1),
    "vpred2_420_8b": (64, 64, 8, S.FMT_YUV420, 4, 1, 2, 5, 0, 64, 1, 1, 24, 2),
    "vpred1_nosig_uniform_422_12b": (72, 32, 12, S.FMT_YUV422, 6, 1, 2, 3, 1, 32, 0, 1, 25, 1),
    "vpred2_rgb_8b": (64, 48, 8, S.FMT_PACKED_RGB, 4, 1, 2, 5, 0, 48, 1, 1, 26, 2),
}

# Full-size workloads: the bench's 4K 10-bit stream, the 1080p plain case,
# the three shapes of the mixed batch and the 8K large-frame stress.
FULL_CASES = {
    "c1_1080p_422_8b_bpp5": dict(w=1920, h=1080, d=8, fmt=S.FMT_YUV422, bpp=5, den=1, v=2, hh=5, seed=1, kind="frame"),
    "c2_2160p_422_10b_bpp3_f0": dict(w=3840, h=2160, d=10, fmt=S.FMT_YUV422, bpp=3, den=1, v=2, hh=5, seed=2, kind="4k", frame=0),
    "c2_2160p_422_10b_bpp3_f1": dict(w=3840, h=2160, d=10, fmt=S.FMT_YUV422, bpp=3, den=1, v=2, hh=5, seed=2, kind="4k", frame=1),
    "c3_720p_420_8b_bpp1": dict(w=1280, h=720, d=8, fmt=S.FMT_YUV420, bpp=1, den=1, v=2, hh=5, seed=31, kind="frame"),
    "c3_1080p_444_12b_bpp4": dict(w=1920, h=1080, d=12, fmt=S.FMT_YUV444, bpp=4, den=1, v=2, hh=5, seed=32, kind="frame"),
    "c3_2160p_rgb_8b_bpp2": dict(w=3840, h=2160, d=8, fmt=S.FMT_PACKED_RGB, bpp=2, den=1, v=2, hh=5, seed=33, kind="frame"),
    "c4_4320p_gbrp_14b_bpp1.5": dict(w=7680, h=4320, d=14, fmt=S.FMT_YUV444, bpp=3, den=2, v=1, hh=5, seed=4, kind="8k"),
    # the three stream types of the serving workload
    "c5_540i_422_10b_bpp5": dict(w=1920, h=540, d=10, fmt=S.FMT_YUV422, bpp=5, den=1, v=2, hh=5, seed=51, kind="frame"),
    "c5_1080p_422_8b_bpp3": dict(w=1920, h=1080, d=8, fmt=S.FMT_YUV422, bpp=3, den=1, v=2, hh=5, seed=52, kind="frame"),
    "c5_2160p_422_10b_bpp2": dict(w=3840, h=2160, d=10, fmt=S.FMT_YUV422, bpp=2, den=1, v=2, hh=5, seed=53, kind="frame"),
}


def full_case_planes(c):
    if c["kind"] == "4k":
        return S.frame_4k_10bit(c["seed"], c["frame"])
    if c["kind"] == "8k":
        return S.frame_8k_14bit(c["seed"])
    return S.frame(c["w"], c["h"], c["d"], c["fmt"], seed=c["seed"])


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def sample_codestream():
    txt = open(os.path.join(REFERENCE, "tests", "UnitTests", "SampleFramesData.cc")).read()
    body = txt[txt.index("Frame_Sample_1_16x16_8bit_422_bitstream[] = {"):]
    body = body[body.index("{") + 1: body.index("};")]
    return np.array([int(x, 16) for x in re.findall(r"0x[0-9A-Fa-f]+", body)], np.uint8)


# Proxy decoding: the reference decoder's half- and quarter-resolution
# output for codestreams of the small cases (proxy 2 needs two vertical
# levels in every component).
PROXY_CASES = [("c1_422_8b", 1), ("c1_422_8b", 2), ("c2_422_10b", 1), ("c2_422_10b", 2), ("c3_420_8b", 1),
               ("c3_444_12b", 2), ("c3_rgb_8b", 1), ("odd_444_10b", 1), ("odd_444_10b", 2), ("c4_gbrp_14b_v1", 1),
               ("uniform_422_10b", 2)]


def make_proxy():
    for name, proxy in PROXY_CASES:
        z = np.load(os.path.join(HERE, name + ".npz"))
        bs = z["bs"]
        err, dec = O.ref_decode_proxy(bs, proxy)
        assert err == 0, (name, proxy, hex(err))
        arrays = {"bs": bs, "proxy": np.array([proxy], np.uint32)}
        for i, pl in enumerate(dec):
            arrays["dec%d" % i] = pl
        np.savez_compressed(os.path.join(HERE, "proxy%d_%s.npz" % (proxy, name)), **arrays)
        print("proxy", proxy, name, [p.shape for p in dec])


# Separate sign sub-packets (coding_signs_handling 1 fast, 2 full), with
# and without vertical prediction, decoded by the reference decoder.
# name: (w, h, depth, fmt, bpp_num, bpp_den, decomp_v, decomp_h, quant, slice_h, significance, rc_mode, seed, signs, vpred_mode)
SIGN_CASES = {
    "signs1_422_8b": (64, 32, 8, S.FMT_YUV422, 5, 1, 2, 5, 0, 16, 1, 1, 31, 1, 0),
    "signs2_422_10b": (128, 48, 10, S.FMT_YUV422, 3, 1, 2, 5, 0, 16, 1, 1, 32, 2, 0),
    "signs2_444_12b_odd": (53, 37, 12, S.FMT_YUV444, 4, 1, 2, 5, 0, 16, 1, 1, 33, 2, 0),
    "signs1_rgb_8b_uniform": (96, 32, 8, S.FMT_PACKED_RGB, 4, 1, 2, 5, 1, 16, 1, 1, 34, 1, 0),
    "signs2_vpred1_422_8b": (128, 64, 8, S.FMT_YUV422, 3, 1, 2, 5, 0, 32, 1, 1, 35, 2, 1),
    "signs1_nosig_420_8b": (96, 48, 8, S.FMT_YUV420, 3, 1, 2, 5, 0, 16, 0, 1, 36, 1, 0),
}


def make_signs():
    for name, (w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc, seed, sg, vpm) in SIGN_CASES.items():
        planes = S.frame(w, h, d, fmt, seed=seed)
        p = O.make_params(w, h, d, fmt, bn, bd, v, hh, quantization=q, slice_height=sl, significance=sig, rc_mode=rc)
        p.coding_signs_handling = sg
        p.coding_vertical_prediction_mode = vpm
        err, bs = O.ref_encode(p, planes)
        assert err == 0, (name, hex(err))
        err, dec = O.ref_decode(bs)
        assert err == 0, (name, hex(err))
        arrays = {"bs": bs, "params": np.array([w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc, sg, vpm], np.uint32)}
        for i, pl in enumerate(planes):
            arrays["in%d" % i] = pl
        for i, pl in enumerate(dec):
            arrays["dec%d" % i] = pl
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, len(bs), "bytes")


def make_vpred():
    for name, (w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc, seed, vpm) in VPRED_CASES.items():
        planes = S.frame(w, h, d, fmt, seed=seed)
        p = O.make_params(w, h, d, fmt, bn, bd, v, hh, quantization=q, slice_height=sl, significance=sig, rc_mode=rc)
        p.coding_vertical_prediction_mode = vpm
        err, bs = O.ref_encode(p, planes)
        assert err == 0, (name, hex(err))
        err, dec = O.ref_decode(bs)
        assert err == 0, (name, hex(err))
        arrays = {"bs": bs, "params": np.array([w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc, vpm], np.uint32)}
        for i, pl in enumerate(planes):
            arrays["in%d" % i] = pl
        for i, pl in enumerate(dec):
            arrays["dec%d" % i] = pl
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, len(bs), "bytes")


# Multi-column precincts (Cw > 0).  The reference encoder always writes
# Cw = 0 (EncHandle.c:401), so these codestreams come from the oracle's
# encoder; the reference decoder's planes are the expected output.
# name: (w, h, depth, fmt, bpp_num, bpp_den, decomp_v, decomp_h, quant, slice_h, significance, rc_mode, seed, signs,
#        vpred_mode, cw)
CW_CASES = {
    "cw1_422_8b": (1200, 16, 8, S.FMT_YUV422, 4, 1, 2, 5, 0, 16, 1, 1, 41, 0, 0, 1),
    "cw2_444_10b_h3": (300, 40, 10, S.FMT_YUV444, 4, 1, 2, 3, 0, 16, 1, 0, 42, 0, 0, 2),
    "cw1_420_8b_signs2": (600, 32, 8, S.FMT_YUV420, 4, 1, 2, 3, 0, 16, 1, 1, 43, 2, 0, 1),
    "cw3_rgb_12b_v1_uniform": (401, 24, 12, S.FMT_PACKED_RGB, 5, 1, 1, 2, 1, 8, 0, 1, 44, 0, 0, 3),
    "cw1_422_10b_vpred1": (320, 48, 10, S.FMT_YUV422, 3, 1, 2, 3, 0, 48, 1, 1, 45, 0, 1, 1),
    "cw2_444_8b_vpred2_rc3": (400, 40, 8, S.FMT_YUV444, 5, 1, 1, 4, 0, 40, 1, 3, 46, 1, 2, 2),
    "cw1_422_8b_v0": (180, 12, 8, S.FMT_YUV422, 4, 1, 0, 3, 0, 4, 1, 2, 47, 0, 0, 1),
}


def make_cw():
    for name, (w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc, seed, sg, vpm, cw) in CW_CASES.items():
        planes = S.frame(w, h, d, fmt, seed=seed)
        p = O.make_params(w, h, d, fmt, bn, bd, v, hh, quantization=q, slice_height=sl, significance=sig, rc_mode=rc, signs=sg,
                          vpred=vpm, cw=cw)
        err, bs = O.oracle_encode(p, planes)
        assert err == 0, (name, hex(err))
        err, dec = O.ref_decode(bs)
        assert err == 0, (name, hex(err))
        arrays = {"bs": bs, "params": np.array([w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc, sg, vpm, cw], np.uint32)}
        for i, pl in enumerate(dec):
            arrays["dec%d" % i] = pl
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, len(bs), "bytes")


# Colour transform (Cpih = 1, reversible RCT) and output non-linearities
# (NLT marker: Tnlt 1 quadratic, 2 extended).  The reference encoder writes
# none of them, so the oracle's encoder writes these codestreams (the RCT
# applied forward; the NLT marker only changes the decoder's output
# scaling); the reference decoder's planes, full and at proxy 1, are the
# expected output.
# name: (w, h, depth, fmt, bpp_num, decomp_v, decomp_h, quant, slice_h, seed, cpih, tnlt, sigma, alpha, t1, t2, e)
MCT_CASES = {
    "mct_rct_444_8b": (96, 32, 8, S.FMT_YUV444, 6, 2, 5, 0, 16, 51, 1, 0, 0, 0, 0, 0, 0),
    "mct_rct_rgb_10b_quadratic": (120, 24, 10, S.FMT_PACKED_RGB, 8, 1, 3, 1, 8, 52, 1, 1, 1, 1234, 0, 0, 0),
    "mct_rct_444_12b_extended": (72, 40, 12, S.FMT_YUV444, 5, 2, 2, 0, 16, 53, 1, 2, 0, 0, 300000, 560000, 3),
    "nlt_quadratic_422_8b": (128, 32, 8, S.FMT_YUV422, 5, 2, 5, 0, 16, 54, 0, 1, 0, 777, 0, 0, 0),
    "nlt_extended_420_10b": (96, 32, 10, S.FMT_YUV420, 4, 2, 4, 0, 32, 55, 0, 2, 0, 0, 150000, 700000, 2),
}


def make_mct():
    for name, (w, h, d, fmt, bn, v, hh, q, sl, seed, cpih, tnlt, sg, al, t1, t2, e) in MCT_CASES.items():
        planes = S.frame(w, h, d, fmt, seed=seed)
        p = O.make_params(w, h, d, fmt, bn, 1, v, hh, quantization=q, slice_height=sl)
        p.cpih, p.tnlt, p.nlt_sigma, p.nlt_alpha, p.nlt_t1, p.nlt_t2, p.nlt_e = cpih, tnlt, sg, al, t1, t2, e
        err, bs = O.oracle_encode(p, planes)
        assert err == 0, (name, hex(err))
        err, dec = O.ref_decode(bs)
        assert err == 0, (name, hex(err))
        err, dec1 = O.ref_decode_proxy(bs, 1)
        assert err == 0, (name, hex(err))
        arrays = {"bs": bs, "params": np.array([w, h, d, fmt, bn, v, hh, q, sl, seed, cpih, tnlt, sg, al, t1, t2, e], np.uint32)}
        for i, pl in enumerate(dec):
            arrays["dec%d" % i] = pl
        for i, pl in enumerate(dec1):
            arrays["proxy%d" % i] = pl
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, len(bs), "bytes")


# Star-Tetrix (Cpih = 3, four components with CTS / CRG markers), written
# by the oracle's encoder without the forward transform; the reference
# decoder's planes (full and half resolution) are the expected output.
# name: (w, h, depth, bpp_num, decomp_v, decomp_h, quant, slice_h, seed, cf, e1, e2, cfa_type, tnlt)
ST_CASES = {
    "mct_st_cf0_rggb_8b": (64, 32, 8, 8, 2, 5, 0, 16, 61, 0, 1, 2, 0, 0),
    "mct_st_cf3_grbg_10b": (90, 24, 10, 6, 1, 3, 1, 8, 62, 3, 0, 1, 1, 0),
    "mct_st_cf0_grbg_12b_quadratic": (48, 40, 12, 10, 2, 2, 0, 16, 63, 0, 2, 0, 1, 1),
}


def make_st():
    for name, (w, h, d, bn, v, hh, q, sl, seed, cf, e1, e2, ct, tnlt) in ST_CASES.items():
        planes = S.frame(w, h, d, S.FMT_4COMP, seed=seed)
        p = O.make_params(w, h, d, S.FMT_4COMP, bn, 1, v, hh, quantization=q, slice_height=sl)
        p.cpih, p.cts_cf, p.cts_e1, p.cts_e2, p.cfa_type = 3, cf, e1, e2, ct
        p.tnlt, p.nlt_alpha = tnlt, 321
        err, bs = O.oracle_encode(p, planes)
        assert err == 0, (name, hex(err))
        err, dec = O.ref_decode(bs)
        assert err == 0, (name, hex(err))
        err, dec1 = O.ref_decode_proxy(bs, 1)
        assert err == 0, (name, hex(err))
        arrays = {"bs": bs, "params": np.array([w, h, d, bn, v, hh, q, sl, seed, cf, e1, e2, ct, tnlt], np.uint32)}
        for i, pl in enumerate(dec):
            arrays["dec%d" % i] = pl
        for i, pl in enumerate(dec1):
            arrays["proxy%d" % i] = pl
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, len(bs), "bytes")


def main():
    if not O.ref_available():
        raise SystemExit("build the reference first: make -C oracle ref")
    if "--cw-only" in sys.argv:
        make_cw()
        return
    if "--mct-only" in sys.argv:
        make_mct()
        make_st()
        return
    if "--vpred-only" in sys.argv:
        make_vpred()
        return
    if "--proxy-only" in sys.argv:
        make_proxy()
        return
    if "--signs-only" in sys.argv:
        make_signs()
        return
    if "--full-only" in sys.argv:
        make_full()
        return
    make_vpred()
    make_signs()
    make_cw()
    make_mct()
    make_st()
    for name, (w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc, seed) in SMALL_CASES.items():
        planes = S.frame(w, h, d, fmt, seed=seed)
        p = O.make_params(w, h, d, fmt, bn, bd, v, hh, quantization=q, slice_height=sl, significance=sig, rc_mode=rc)
        err, bs = O.ref_encode(p, planes)
        assert err == 0, (name, hex(err))
        err, dec = O.ref_decode(bs)
        assert err == 0, (name, hex(err))
        arrays = {"bs": bs, "params": np.array([w, h, d, fmt, bn, bd, v, hh, q, sl, sig, rc], np.uint32)}
        for i, pl in enumerate(planes):
            arrays["in%d" % i] = pl
        for i, pl in enumerate(dec):
            arrays["dec%d" % i] = pl
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, len(bs), "bytes")
    make_proxy()
    bs = sample_codestream()
    err, dec = O.ref_decode(bs)
    assert err == 0
    fs = np.zeros(1, np.uint32)
    import ctypes
    info = O.ImageInfo()
    size = ctypes.c_uint32()
    comp = (ctypes.c_uint32 * 12)()
    w = ctypes.c_uint32(); h = ctypes.c_uint32(); dep = ctypes.c_uint32(); f = ctypes.c_uint32(); nc = ctypes.c_uint32()
    r = O.ref().ref_probe(bs.ctypes.data_as(ctypes.c_void_p), len(bs), ctypes.byref(w), ctypes.byref(h), ctypes.byref(dep),
                          ctypes.byref(f), ctypes.byref(nc), comp, ctypes.byref(size))
    assert r == 0
    fs[0] = size.value
    arrays = {"bs": bs, "frame_size": fs}
    for i, pl in enumerate(dec):
        arrays["dec%d" % i] = pl
    np.savez_compressed(os.path.join(HERE, "ref_sample_16x16.npz"), **arrays)
    print("ref sample", len(bs), "bytes, frame size", size.value)
    make_full()


def make_full():
    """full_size.json: the reference's codestream and decode of every full-size
    case, as SHA-256 hashes."""
    full = {}
    for name, c in FULL_CASES.items():
        planes = full_case_planes(c)
        p = O.make_params(c["w"], c["h"], c["d"], c["fmt"], c["bpp"], c["den"], c["v"], c["hh"], threads=8)
        err, bs = O.ref_encode(p, planes)
        assert err == 0, (name, hex(err))
        err, dec = O.ref_decode(bs, threads=8)
        assert err == 0, (name, hex(err))
        full[name] = dict(c, input_sha256=[sha(pl) for pl in planes], codestream_bytes=int(len(bs)),
                          codestream_sha256=sha(bs), decoded_sha256=[sha(pl) for pl in dec])
        print(name, len(bs), "bytes")
    with open(os.path.join(HERE, "full_size.json"), "w") as fh:
        json.dump(full, fh, indent=1)


if __name__ == "__main__":
    main()
