"""Host-side robustness, in the spirit of the reference's fuzz harnesses
(tests/FuzzyTests/decoder.c, encoder.c): mutated codestreams through the
frame-size query and decoder initialisation (header parse and precinct
walk), and random encoder parameter sets through encoder initialisation
(parameter validation and geometry).  Every call must return a status and
never crash.  Without a GPU, initialisation ends with
SvtJxsErrorInsufficientResources after the host checks, so the host code
is exercised up to the device boundary.  Mutated streams are never
decoded on a GPU here.
"""
import ctypes

import numpy as np

import golden_cases as G

SMALL = G.small_cases()


def _mutations(rng, bs, n):
    out = []
    for _ in range(n):
        b = bs.copy()
        kind = int(rng.integers(0, 5))
        if kind == 0:  # flip bits
            for _ in range(int(rng.integers(1, 8))):
                i = int(rng.integers(0, len(b)))
                b[i] ^= np.uint8(1 << int(rng.integers(0, 8)))
        elif kind == 1:  # truncate
            b = b[: int(rng.integers(0, len(b)))]
        elif kind == 2:  # random bytes in the header
            for _ in range(int(rng.integers(1, 6))):
                i = int(rng.integers(0, min(len(b), 64)))
                b[i] = np.uint8(rng.integers(0, 256))
        elif kind == 3:  # duplicate a chunk
            i = int(rng.integers(0, len(b)))
            j = int(rng.integers(i, min(len(b), i + 64) + 1))
            b = np.concatenate([b[:j], b[i:j], b[j:]])
        else:  # zero a run
            i = int(rng.integers(0, len(b)))
            b[i: i + int(rng.integers(1, 32))] = 0
        out.append(np.ascontiguousarray(b, dtype=np.uint8))
    return out


def test_frame_size_and_decoder_init_survive_mutated_codestreams(jxs_lib):
    L = jxs_lib.lib()
    rng = np.random.default_rng(7)
    n = 0
    for name in sorted(SMALL):
        for b in _mutations(rng, SMALL[name]["bs"], 120):
            cfg = jxs_lib.ImageConfig()
            size = ctypes.c_uint32()
            for fast in (0, 1):
                L.svt_jpeg_xs_decoder_get_single_frame_size(b.ctypes.data if len(b) else None, len(b), ctypes.byref(cfg),
                                                            ctypes.byref(size), fast)
                # a walked frame lies inside the buffer; the fast search
                # reports Lcod from the header as the reference does
                # (ParseHeader.c:845-848)
                if len(b) and not fast:
                    assert size.value <= len(b)
            api = jxs_lib.DecoderApi()
            r = L.svt_jpeg_xs_decoder_init(jxs_lib.API_MAJOR, jxs_lib.API_MINOR, ctypes.byref(api),
                                           b.ctypes.data if len(b) else None, len(b), ctypes.byref(cfg))
            if r == 0:
                L.svt_jpeg_xs_decoder_close(ctypes.byref(api))
            n += 1
    assert n == 120 * len(SMALL)


def test_encoder_init_survives_random_parameters(jxs_lib):
    L = jxs_lib.lib()
    rng = np.random.default_rng(11)
    fields = [("source_width", 0, 9000), ("source_height", 0, 9000), ("input_bit_depth", 0, 20), ("colour_format", 0, 30),
              ("bpp_numerator", 0, 60), ("bpp_denominator", 0, 12), ("ndecomp_v", 0, 4), ("ndecomp_h", 0, 8),
              ("quantization", 0, 3), ("slice_height", 0, 9000), ("coding_signs_handling", 0, 4),
              ("coding_significance", 0, 3), ("rate_control_mode", 0, 6), ("coding_vertical_prediction_mode", 0, 5),
              ("slice_packetization_mode", 0, 3)]
    for _ in range(2000):
        api = jxs_lib.default_encoder_api()
        api.verbose = 0
        for f, lo, hi in fields:
            setattr(api, f, int(rng.integers(lo, hi)))
        # keep frames small enough to lay out quickly (the reference harness caps 8000 x 8000)
        if api.source_width * api.source_height > 1920 * 1080:
            api.source_height = max(1, (1920 * 1080) // max(1, api.source_width))
        r = L.svt_jpeg_xs_encoder_init(jxs_lib.API_MAJOR, jxs_lib.API_MINOR, ctypes.byref(api))
        if r == 0:
            L.svt_jpeg_xs_encoder_close(ctypes.byref(api))
