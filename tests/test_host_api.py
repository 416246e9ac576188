"""Host-side behaviour of the C API that needs no GPU: parameter defaults and
validation (EncHandle.c:128-618), frame-size parsing (ParseHeader.c:650-889),
buffer tools (ImageBuffer.c:22-318), and failing loudly - never falling back
to a CPU path - when no CUDA device is present."""
import ctypes

import numpy as np
import pytest

import golden_cases as G


def _api(jxs, **kw):
    api = jxs.default_encoder_api()
    for k, v in kw.items():
        setattr(api, k, v)
    return api


def _has_gpu(jxs):
    return ctypes.CDLL(jxs.LIB_PATH).jxs_gpu_device_count() > 0


def test_default_parameters(jxs_lib):
    api = jxs_lib.default_encoder_api()
    assert (api.ndecomp_v, api.ndecomp_h, api.slice_height, api.bpp_denominator) == (2, 5, 16, 1)
    assert (api.rate_control_mode, api.coding_significance, api.quantization) == (1, 1, 0)
    assert api.coding_signs_handling == 0 and api.coding_vertical_prediction_mode == 0
    assert api.verbose == 2 and api.private_ptr is None


def test_api_version_check(jxs_lib):
    api = jxs_lib.EncoderApi()
    L = jxs_lib.lib()
    assert L.svt_jpeg_xs_encoder_load_default_parameters(0, 11, ctypes.byref(api)) == jxs_lib.E_INVALID_API_VERSION
    assert L.svt_jpeg_xs_encoder_load_default_parameters(1, 0, ctypes.byref(api)) == jxs_lib.E_INVALID_API_VERSION
    assert L.svt_jpeg_xs_encoder_init(1, 0, ctypes.byref(api)) == jxs_lib.E_INVALID_API_VERSION


def test_image_config(jxs_lib):
    api = _api(jxs_lib, source_width=3840, source_height=2160, input_bit_depth=10, colour_format=jxs_lib.FMT_YUV422,
               bpp_numerator=3)
    cfg, nbytes = jxs_lib.image_config(api)
    assert nbytes == 3110400
    assert cfg.components_num == 3
    assert [(cfg.components[c].width, cfg.components[c].height) for c in range(3)] == [(3840, 2160), (1920, 2160),
                                                                                         (1920, 2160)]
    assert cfg.components[1].byte_size == 1920 * 2160 * 2
    api.colour_format = jxs_lib.FMT_PACKED_RGB
    api.input_bit_depth = 8
    cfg, _ = jxs_lib.image_config(api)
    assert cfg.components_num == 1 and cfg.components[0].byte_size == 3840 * 2160 * 3


@pytest.mark.parametrize("bad", [dict(input_bit_depth=7), dict(input_bit_depth=15), dict(ndecomp_v=3), dict(ndecomp_h=6),
                                 dict(ndecomp_v=2, ndecomp_h=1), dict(bpp_numerator=0), dict(bpp_denominator=0),
                                 dict(slice_height=6), dict(slice_height=0), dict(quantization=2), dict(source_width=3),
                                 dict(rate_control_mode=4), dict(colour_format=0), dict(source_width=255),
                                 dict(bpp_numerator=1, bpp_denominator=1000)])
def test_encoder_init_rejects_bad_parameters(jxs_lib, bad):
    kw = dict(source_width=256, source_height=64, input_bit_depth=10, colour_format=jxs_lib.FMT_YUV422, bpp_numerator=3,
              verbose=0)
    kw.update(bad)
    api = _api(jxs_lib, **kw)
    assert jxs_lib.lib().svt_jpeg_xs_encoder_init(0, 10, ctypes.byref(api)) == jxs_lib.E_BAD_PARAMETER
    assert not api.private_ptr


def test_encoder_init_fails_loudly_without_gpu(jxs_lib):
    if _has_gpu(jxs_lib):
        pytest.skip("a GPU is present")
    api = _api(jxs_lib, source_width=256, source_height=64, input_bit_depth=8, colour_format=jxs_lib.FMT_YUV422,
               bpp_numerator=3, verbose=0)
    assert jxs_lib.lib().svt_jpeg_xs_encoder_init(0, 10, ctypes.byref(api)) == jxs_lib.E_INSUFFICIENT_RESOURCES
    assert not api.private_ptr


def test_decoder_init_fails_loudly_without_gpu(jxs_lib):
    if _has_gpu(jxs_lib):
        pytest.skip("a GPU is present")
    bs = G.small_cases()["c1_422_8b"]["bs"]
    with pytest.raises(jxs_lib.JxsError) as ei:
        jxs_lib.Decoder(bs)
    assert ei.value.code == jxs_lib.E_INSUFFICIENT_RESOURCES


@pytest.mark.parametrize("name", sorted(G.small_cases()))
def test_frame_size_of_golden_codestreams(jxs_lib, name):
    c = G.small_cases()[name]
    for fast in (0, 1):
        r, n, cfg = jxs_lib.frame_size(c["bs"], fast)
        assert r == 0 and n == len(c["bs"])
        assert (cfg.width, cfg.height, cfg.bit_depth) == (c["w"], c["h"], c["d"])
    r, n, _ = jxs_lib.frame_size(c["bs"][: len(c["bs"]) - 3], 0)
    assert r == jxs_lib.E_DEC_TOO_SHORT


def test_frame_size_of_reference_sample(jxs_lib):
    bs, size, _ = G.ref_sample()
    r, n, cfg = jxs_lib.frame_size(bs, 0)
    assert r == 0 and n == size == 448
    assert (cfg.width, cfg.height, cfg.format, cfg.components_num) == (16, 16, jxs_lib.FMT_YUV422, 3)


def test_frame_size_rejects_garbage(jxs_lib):
    r, _, _ = jxs_lib.frame_size(np.arange(64, dtype=np.uint8), 0)
    assert r == jxs_lib.E_DEC_INVALID_BITSTREAM


def test_buffer_tools(jxs_lib):
    L = jxs_lib.lib()
    cfg = jxs_lib.ImageConfig()
    cfg.width, cfg.height, cfg.bit_depth, cfg.format, cfg.components_num = 64, 16, 10, jxs_lib.FMT_YUV422, 3
    for c, (w, h) in enumerate([(64, 16), (32, 16), (32, 16)]):
        cfg.components[c].width, cfg.components[c].height, cfg.components[c].byte_size = w, h, w * h * 2
    b = L.svt_jpeg_xs_image_buffer_alloc(ctypes.byref(cfg))
    assert b and b.contents.stride[1] == 32 and b.contents.alloc_size[0] == 64 * 16 * 2
    L.svt_jpeg_xs_image_buffer_free(b)
    bs = L.svt_jpeg_xs_bitstream_alloc(1000)
    assert bs and bs.contents.allocation_size == 1000
    L.svt_jpeg_xs_bitstream_free(bs)
    L.svt_jpeg_xs_frame_pool_alloc.restype = ctypes.c_void_p
    L.svt_jpeg_xs_frame_pool_alloc.argtypes = [ctypes.POINTER(jxs_lib.ImageConfig), ctypes.c_uint32, ctypes.c_uint32]
    L.svt_jpeg_xs_frame_pool_get.argtypes = [ctypes.c_void_p, ctypes.POINTER(jxs_lib.Frame), ctypes.c_uint8]
    L.svt_jpeg_xs_frame_pool_release.argtypes = [ctypes.c_void_p, ctypes.POINTER(jxs_lib.Frame)]
    L.svt_jpeg_xs_frame_pool_free.argtypes = [ctypes.c_void_p]
    pool = L.svt_jpeg_xs_frame_pool_alloc(ctypes.byref(cfg), 4096, 2)
    assert pool
    f1, f2, f3 = jxs_lib.Frame(), jxs_lib.Frame(), jxs_lib.Frame()
    assert L.svt_jpeg_xs_frame_pool_get(pool, ctypes.byref(f1), 0) == 0
    assert L.svt_jpeg_xs_frame_pool_get(pool, ctypes.byref(f2), 0) == 0
    assert L.svt_jpeg_xs_frame_pool_get(pool, ctypes.byref(f3), 0) == jxs_lib.E_EMPTY_QUEUE
    assert f1.bitstream.allocation_size == 4096 and f1.image.data_yuv[0] != f2.image.data_yuv[0]
    L.svt_jpeg_xs_frame_pool_release(pool, ctypes.byref(f1))
    assert L.svt_jpeg_xs_frame_pool_get(pool, ctypes.byref(f3), 0) == 0
    L.svt_jpeg_xs_frame_pool_free(pool)


def test_batch_entry_points_reject_null(jxs_lib):
    """The batch extension's entry points validate their handle before any
    CUDA call: a null batch is a bad parameter (or no stage times)."""
    L = jxs_lib.lib()
    assert L.svt_jpeg_xs_gpu_batch_set_stage_timing(None, 1) == jxs_lib.E_BAD_PARAMETER
    n = 4
    st, var, ms = (ctypes.c_int32 * n)(), (ctypes.c_int32 * n)(), (ctypes.c_float * n)()
    assert L.svt_jpeg_xs_gpu_batch_read_stage_times(None, st, var, ms, n) == 0
    assert L.svt_jpeg_xs_gpu_batch_set_options(None, 1, 0) == jxs_lib.E_BAD_PARAMETER
    t = (ctypes.c_int32 * 5)(1, 0, 0, 4, 4)
    assert L.svt_jpeg_xs_gpu_batch_set_tune(None, t) == jxs_lib.E_BAD_PARAMETER
