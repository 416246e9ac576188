"""Python bindings (ctypes) to libSvtJpegxs.so, the GPU JPEG XS codec.

The structures mirror include/SvtJpegxs*.h field for field; the classes wrap
the reference-compatible C API (svt_jpeg_xs_encoder_* / svt_jpeg_xs_decoder_*)
plus the GPU extensions of SvtJpegxsGpu.h.  Image planes and bitstreams may be
numpy arrays (host) or raw device pointers (ints, e.g. torch.Tensor.data_ptr()).

The library has no CPU fallback: loading or using it without the built
extension or without a CUDA device raises.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libSvtJpegxs.so")

API_MAJOR, API_MINOR = 0, 10
MAX_COMPONENTS = 4

# ColourFormat_t
FMT_YUV400, FMT_YUV420, FMT_YUV422, FMT_YUV444, FMT_4COMP, FMT_GRAY = 1, 2, 3, 4, 5, 6
FMT_PACKED_RGB = 21

# SvtJxsErrorType_t (as unsigned 32-bit)
E_NONE = 0
E_BAD_PARAMETER = 0x80001005
E_INSUFFICIENT_RESOURCES = 0x80001000
E_UNDEFINED = 0x80001001
E_EMPTY_QUEUE = 0x80002033
E_ENCODE_FRAME = 0x80002035
E_DEC_INVALID_POINTER = 0x80003000
E_DEC_INVALID_BITSTREAM = 0x80003001
E_DEC_INTERNAL = 0x80003002
E_DEC_TOO_SHORT = 0x80003003
E_DEC_CONFIG_CHANGE = 0x80003004
E_END_OF_CODESTREAM = 0x80003005
E_INVALID_API_VERSION = 0x40001001

_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p)


class ImageConfigComponent(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("byte_size", ctypes.c_uint32)]


class ImageConfig(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("bit_depth", ctypes.c_uint8),
                ("format", ctypes.c_int32), ("components_num", ctypes.c_uint8),
                ("components", ImageConfigComponent * MAX_COMPONENTS)]


class ImageBuffer(ctypes.Structure):
    _fields_ = [("data_yuv", ctypes.c_void_p * MAX_COMPONENTS), ("stride", ctypes.c_uint32 * MAX_COMPONENTS),
                ("alloc_size", ctypes.c_uint32 * MAX_COMPONENTS), ("release_ctx_ptr", ctypes.c_void_p),
                ("ready_to_release", ctypes.c_uint8)]


class BitstreamBuffer(ctypes.Structure):
    _fields_ = [("buffer", ctypes.c_void_p), ("allocation_size", ctypes.c_uint32), ("used_size", ctypes.c_uint32),
                ("release_ctx_ptr", ctypes.c_void_p), ("ready_to_release", ctypes.c_uint8),
                ("last_packet_in_frame", ctypes.c_uint8)]


class Frame(ctypes.Structure):
    _fields_ = [("image", ImageBuffer), ("bitstream", BitstreamBuffer), ("user_prv_ctx_ptr", ctypes.c_void_p)]


class EncoderApi(ctypes.Structure):
    _fields_ = [("source_width", ctypes.c_uint32), ("source_height", ctypes.c_uint32), ("input_bit_depth", ctypes.c_uint8),
                ("colour_format", ctypes.c_int32), ("bpp_numerator", ctypes.c_uint32), ("bpp_denominator", ctypes.c_uint32),
                ("ndecomp_v", ctypes.c_uint32), ("ndecomp_h", ctypes.c_uint32), ("quantization", ctypes.c_uint32),
                ("slice_height", ctypes.c_uint32), ("use_cpu_flags", ctypes.c_uint64), ("threads_num", ctypes.c_uint32),
                ("cpu_profile", ctypes.c_uint8), ("print_bands_info", ctypes.c_uint32),
                ("coding_signs_handling", ctypes.c_uint32), ("coding_significance", ctypes.c_uint32),
                ("rate_control_mode", ctypes.c_uint32), ("coding_vertical_prediction_mode", ctypes.c_uint32),
                ("verbose", ctypes.c_uint32), ("callback_send_data_available", _CB),
                ("callback_send_data_available_context", ctypes.c_void_p), ("callback_get_data_available", _CB),
                ("callback_get_data_available_context", ctypes.c_void_p), ("slice_packetization_mode", ctypes.c_uint8),
                ("private_ptr", ctypes.c_void_p), ("padding", ctypes.c_uint8 * 64)]


class DecoderApi(ctypes.Structure):
    _fields_ = [("use_cpu_flags", ctypes.c_uint64), ("verbose", ctypes.c_uint32), ("threads_num", ctypes.c_uint32),
                ("packetization_mode", ctypes.c_uint8), ("proxy_mode", ctypes.c_int32),
                ("callback_send_data_available", _CB), ("callback_send_data_available_context", ctypes.c_void_p),
                ("callback_get_data_available", _CB), ("callback_get_data_available_context", ctypes.c_void_p),
                ("private_ptr", ctypes.c_void_p), ("padding", ctypes.c_uint8 * 64)]


_lib = None


class BatchInfo(ctypes.Structure):
    _fields_ = [("last_gpu_ms", ctypes.c_float), ("last_launches", ctypes.c_uint32), ("graph_hits", ctypes.c_uint64),
                ("graph_builds", ctypes.c_uint64), ("graph_updates", ctypes.c_uint64), ("tune", ctypes.c_int32 * 5),
                ("device_bytes", ctypes.c_uint64), ("device_used", ctypes.c_uint64), ("device_peak", ctypes.c_uint64)]


BATCH_MAX = 64


class ServerRequest(ctypes.Structure):
    _fields_ = [("stream", ctypes.c_int32), ("tag", ctypes.c_uint64), ("planes", ctypes.c_void_p * 4),
                ("strides", ctypes.c_uint32 * 4), ("bitstream", ctypes.c_void_p), ("bitstream_size", ctypes.c_uint32)]


class ServerCompletion(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("stream", ctypes.c_int32), ("status", ctypes.c_uint32),
                ("t_arrive_ns", ctypes.c_int64), ("t_start_ns", ctypes.c_int64), ("t_done_ns", ctypes.c_int64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_uint64), ("batched_frames", ctypes.c_uint64), ("max_batch_seen", ctypes.c_uint64),
                ("deferred", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64), ("device_used", ctypes.c_uint64),
                ("device_peak", ctypes.c_uint64)]


SERVER_BATCHED = 0
SERVER_PER_FRAME = 1


def lib():
    """The loaded libSvtJpegxs.so; raises if the extension was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libSvtJpegxs.so is not built (run svt-jpeg-xs_gb300/build.py or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        u32 = ctypes.c_uint32
        for name in ("svt_jpeg_xs_encoder_load_default_parameters", "svt_jpeg_xs_encoder_get_image_config",
                     "svt_jpeg_xs_encoder_init", "svt_jpeg_xs_encoder_send_picture", "svt_jpeg_xs_encoder_get_packet",
                     "svt_jpeg_xs_decoder_init", "svt_jpeg_xs_decoder_send_frame", "svt_jpeg_xs_decoder_get_frame",
                     "svt_jpeg_xs_decoder_send_packet", "svt_jpeg_xs_decoder_send_eoc",
                     "svt_jpeg_xs_decoder_get_single_frame_size", "svt_jpeg_xs_decoder_get_single_frame_size_with_proxy",
                     "svt_jpeg_xs_gpu_encoder_set_stream", "svt_jpeg_xs_gpu_decoder_set_stream",
                     "svt_jpeg_xs_gpu_encoder_set_streams", "svt_jpeg_xs_gpu_decoder_set_streams",
                     "svt_jpeg_xs_gpu_encoder_set_timing", "svt_jpeg_xs_gpu_decoder_set_timing",
                     "svt_jpeg_xs_gpu_encoder_rc_results", "svt_jpeg_xs_frame_pool_get"):
            getattr(L, name).restype = u32
        L.svt_jpeg_xs_encoder_load_default_parameters.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(EncoderApi)]
        L.svt_jpeg_xs_encoder_get_image_config.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(EncoderApi),
                                                           ctypes.POINTER(ImageConfig), ctypes.POINTER(u32)]
        L.svt_jpeg_xs_encoder_init.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(EncoderApi)]
        L.svt_jpeg_xs_encoder_close.argtypes = [ctypes.POINTER(EncoderApi)]
        L.svt_jpeg_xs_encoder_close.restype = None
        L.svt_jpeg_xs_encoder_send_picture.argtypes = [ctypes.POINTER(EncoderApi), ctypes.POINTER(Frame), ctypes.c_uint8]
        L.svt_jpeg_xs_encoder_get_packet.argtypes = [ctypes.POINTER(EncoderApi), ctypes.POINTER(Frame), ctypes.c_uint8]
        L.svt_jpeg_xs_decoder_init.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(DecoderApi), ctypes.c_void_p,
                                               ctypes.c_size_t, ctypes.POINTER(ImageConfig)]
        L.svt_jpeg_xs_decoder_close.argtypes = [ctypes.POINTER(DecoderApi)]
        L.svt_jpeg_xs_decoder_close.restype = None
        L.svt_jpeg_xs_decoder_send_frame.argtypes = [ctypes.POINTER(DecoderApi), ctypes.POINTER(Frame), ctypes.c_uint8]
        L.svt_jpeg_xs_decoder_get_frame.argtypes = [ctypes.POINTER(DecoderApi), ctypes.POINTER(Frame), ctypes.c_uint8]
        L.svt_jpeg_xs_decoder_send_packet.argtypes = [ctypes.POINTER(DecoderApi), ctypes.POINTER(Frame), ctypes.POINTER(u32)]
        L.svt_jpeg_xs_decoder_send_eoc.argtypes = [ctypes.POINTER(DecoderApi)]
        L.svt_jpeg_xs_decoder_get_single_frame_size.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ImageConfig),
                                                                ctypes.POINTER(u32), u32]
        L.svt_jpeg_xs_decoder_get_single_frame_size_with_proxy.argtypes = [
            ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ImageConfig), ctypes.POINTER(u32), u32, ctypes.c_int32]
        L.svt_jpeg_xs_gpu_encoder_set_stream.argtypes = [ctypes.POINTER(EncoderApi), ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_decoder_set_stream.argtypes = [ctypes.POINTER(DecoderApi), ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_encoder_set_streams.argtypes = [ctypes.POINTER(EncoderApi), ctypes.c_void_p, u32]
        L.svt_jpeg_xs_gpu_decoder_set_streams.argtypes = [ctypes.POINTER(DecoderApi), ctypes.c_void_p, u32]
        L.svt_jpeg_xs_gpu_encoder_set_timing.argtypes = [ctypes.POINTER(EncoderApi), u32]
        L.svt_jpeg_xs_gpu_decoder_set_timing.argtypes = [ctypes.POINTER(DecoderApi), u32]
        L.svt_jpeg_xs_gpu_encoder_read_timing.argtypes = [ctypes.POINTER(EncoderApi), ctypes.POINTER(ctypes.c_double), u32]
        L.svt_jpeg_xs_gpu_encoder_read_timing.restype = ctypes.c_uint64
        L.svt_jpeg_xs_gpu_decoder_read_timing.argtypes = [ctypes.POINTER(DecoderApi), ctypes.POINTER(ctypes.c_double), u32]
        L.svt_jpeg_xs_gpu_decoder_read_timing.restype = ctypes.c_uint64
        L.svt_jpeg_xs_gpu_encoder_read_kernel_timing.argtypes = [ctypes.POINTER(EncoderApi), ctypes.POINTER(ctypes.c_double), u32]
        L.svt_jpeg_xs_gpu_encoder_read_kernel_timing.restype = u32
        L.svt_jpeg_xs_gpu_decoder_read_kernel_timing.argtypes = [ctypes.POINTER(DecoderApi), ctypes.POINTER(ctypes.c_double), u32]
        L.svt_jpeg_xs_gpu_decoder_read_kernel_timing.restype = u32
        L.svt_jpeg_xs_gpu_encoder_rc_results.argtypes = [ctypes.POINTER(EncoderApi), ctypes.c_void_p, ctypes.c_void_p, u32]
        L.svt_jpeg_xs_gpu_decoder_locate_frame.argtypes = [ctypes.POINTER(DecoderApi), ctypes.c_void_p, u32, ctypes.POINTER(u32),
                                                          ctypes.c_void_p, u32, ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_decoder_locate_frame.restype = u32
        L.svt_jpeg_xs_gpu_batch_create.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]
        L.svt_jpeg_xs_gpu_batch_create.restype = u32
        L.svt_jpeg_xs_gpu_batch_destroy.argtypes = [ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_batch_destroy.restype = None
        L.svt_jpeg_xs_gpu_batch_set_options.argtypes = [ctypes.c_void_p, u32, u32]
        L.svt_jpeg_xs_gpu_batch_set_options.restype = u32
        L.svt_jpeg_xs_gpu_batch_set_tune.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]
        L.svt_jpeg_xs_gpu_batch_set_tune.restype = u32
        L.svt_jpeg_xs_gpu_batch_encode.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, u32, ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_batch_encode.restype = u32
        L.svt_jpeg_xs_gpu_batch_decode.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, u32, ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_batch_decode.restype = u32
        L.svt_jpeg_xs_gpu_batch_wait.argtypes = [ctypes.c_void_p, ctypes.POINTER(u32)]
        L.svt_jpeg_xs_gpu_batch_wait.restype = u32
        L.svt_jpeg_xs_gpu_batch_ready.argtypes = [ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_batch_ready.restype = u32
        L.svt_jpeg_xs_gpu_batch_get_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(BatchInfo)]
        L.svt_jpeg_xs_gpu_batch_get_info.restype = u32
        L.svt_jpeg_xs_gpu_batch_set_stage_timing.argtypes = [ctypes.c_void_p, u32]
        L.svt_jpeg_xs_gpu_batch_set_stage_timing.restype = u32
        L.svt_jpeg_xs_gpu_batch_read_stage_times.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                                            ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float), u32]
        L.svt_jpeg_xs_gpu_batch_read_stage_times.restype = u32
        L.svt_jpeg_xs_gpu_server_create.argtypes = [ctypes.c_uint64, u32, u32, u32, ctypes.POINTER(ctypes.c_void_p)]
        L.svt_jpeg_xs_gpu_server_create.restype = u32
        L.svt_jpeg_xs_gpu_server_destroy.argtypes = [ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_server_destroy.restype = None
        L.svt_jpeg_xs_gpu_server_add_encoder.argtypes = [ctypes.c_void_p, ctypes.POINTER(EncoderApi)]
        L.svt_jpeg_xs_gpu_server_add_encoder.restype = ctypes.c_int32
        L.svt_jpeg_xs_gpu_server_add_decoder.argtypes = [ctypes.c_void_p, ctypes.POINTER(DecoderApi)]
        L.svt_jpeg_xs_gpu_server_add_decoder.restype = ctypes.c_int32
        L.svt_jpeg_xs_gpu_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServerRequest)]
        L.svt_jpeg_xs_gpu_server_submit.restype = u32
        L.svt_jpeg_xs_gpu_server_poll.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServerCompletion), u32]
        L.svt_jpeg_xs_gpu_server_poll.restype = u32
        L.svt_jpeg_xs_gpu_server_pending.argtypes = [ctypes.c_void_p]
        L.svt_jpeg_xs_gpu_server_pending.restype = ctypes.c_uint64
        L.svt_jpeg_xs_gpu_server_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServerStats)]
        L.svt_jpeg_xs_gpu_server_get_stats.restype = u32
        L.svt_jpeg_xs_image_buffer_alloc.argtypes = [ctypes.POINTER(ImageConfig)]
        L.svt_jpeg_xs_image_buffer_alloc.restype = ctypes.POINTER(ImageBuffer)
        L.svt_jpeg_xs_image_buffer_free.argtypes = [ctypes.POINTER(ImageBuffer)]
        L.svt_jpeg_xs_image_buffer_free.restype = None
        L.svt_jpeg_xs_bitstream_alloc.argtypes = [u32]
        L.svt_jpeg_xs_bitstream_alloc.restype = ctypes.POINTER(BitstreamBuffer)
        L.svt_jpeg_xs_bitstream_free.argtypes = [ctypes.POINTER(BitstreamBuffer)]
        L.svt_jpeg_xs_bitstream_free.restype = None
        _lib = L
    return _lib


class JxsError(RuntimeError):
    def __init__(self, what, code):
        super().__init__("%s failed: 0x%08x" % (what, code))
        self.code = code


def _check(what, code):
    if code != E_NONE:
        raise JxsError(what, code)


def _plane_ptr(p):
    if isinstance(p, np.ndarray):
        return p.ctypes.data
    return int(p)


def _plane_bytes(p):
    return p.nbytes if isinstance(p, np.ndarray) else 0


def default_encoder_api():
    api = EncoderApi()
    _check("load_default_parameters", lib().svt_jpeg_xs_encoder_load_default_parameters(API_MAJOR, API_MINOR, ctypes.byref(api)))
    return api


def image_config(api):
    cfg = ImageConfig()
    n = ctypes.c_uint32()
    _check("get_image_config", lib().svt_jpeg_xs_encoder_get_image_config(API_MAJOR, API_MINOR, ctypes.byref(api),
                                                                           ctypes.byref(cfg), ctypes.byref(n)))
    return cfg, n.value


class Encoder:
    """GPU encoder behind the reference C API.

    planes: list of 2-D numpy arrays (host) or of (device_ptr, stride_in_samples)
    tuples.  encode() returns the codestream as a numpy uint8 array.
    """

    def __init__(self, width, height, bit_depth, colour_format, bpp_numerator, bpp_denominator=1, ndecomp_v=2, ndecomp_h=5,
                 quantization=0, slice_height=16, rate_control_mode=1, coding_significance=1, slice_packetization_mode=0,
                 verbose=0, **extra):
        api = default_encoder_api()
        api.source_width, api.source_height = width, height
        api.input_bit_depth, api.colour_format = bit_depth, colour_format
        api.bpp_numerator, api.bpp_denominator = bpp_numerator, bpp_denominator
        api.ndecomp_v, api.ndecomp_h, api.quantization = ndecomp_v, ndecomp_h, quantization
        api.slice_height, api.rate_control_mode = slice_height, rate_control_mode
        api.coding_significance = coding_significance
        api.slice_packetization_mode = slice_packetization_mode
        api.verbose = verbose
        for k, v in extra.items():
            setattr(api, k, v)
        self.api = api
        self.config, self.frame_bytes = image_config(api)
        _check("encoder_init", lib().svt_jpeg_xs_encoder_init(API_MAJOR, API_MINOR, ctypes.byref(self.api)))
        self.width, self.height, self.bit_depth, self.format = width, height, bit_depth, colour_format
        self._keep = {}

    def close(self):
        if self.api is not None and self.api.private_ptr:
            lib().svt_jpeg_xs_encoder_close(ctypes.byref(self.api))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _frame(self, planes, out, out_cap=None, user=None):
        f = Frame()
        bps = 1 if self.bit_depth <= 8 else 2
        n = len(planes)
        for c in range(MAX_COMPONENTS):
            src = planes[0] if self.format == FMT_PACKED_RGB else (planes[c] if c < n else None)
            if src is None:
                continue
            if isinstance(src, tuple):
                ptr, stride = src[0], src[1]
                rows = self.height if (self.format == FMT_PACKED_RGB or c == 0) else self.config.components[c].height
                f.image.data_yuv[c] = ptr
                f.image.stride[c] = stride
                f.image.alloc_size[c] = min(stride * rows * bps, 0xffffffff)
            else:
                f.image.data_yuv[c] = src.ctypes.data
                f.image.stride[c] = src.shape[1]
                f.image.alloc_size[c] = src.nbytes
        if isinstance(out, np.ndarray):
            f.bitstream.buffer = out.ctypes.data
            f.bitstream.allocation_size = out.nbytes
        else:
            f.bitstream.buffer = int(out)
            f.bitstream.allocation_size = out_cap
        f.user_prv_ctx_ptr = user
        return f

    def send(self, planes, out, out_cap=None, blocking=True, user=None):
        f = self._frame(planes, out, out_cap, user)
        return lib().svt_jpeg_xs_encoder_send_picture(ctypes.byref(self.api), ctypes.byref(f), 1 if blocking else 0)

    def make_frame(self, planes, out, out_cap=None):
        """A frame structure to send repeatedly (the API copies it per call)."""
        return self._frame(planes, out, out_cap)

    def send_frame(self, frame, blocking=True):
        return lib().svt_jpeg_xs_encoder_send_picture(ctypes.byref(self.api), ctypes.byref(frame), 1 if blocking else 0)

    def get(self, blocking=True):
        f = Frame()
        r = lib().svt_jpeg_xs_encoder_get_packet(ctypes.byref(self.api), ctypes.byref(f), 1 if blocking else 0)
        return r, f

    def encode(self, planes):
        out = np.zeros(self.frame_bytes + 64, np.uint8)
        _check("send_picture", self.send(planes, out))
        r, f = self.get()
        _check("get_packet", r)
        return out[: f.bitstream.used_size].copy()

    def rc_results(self):
        rows = (self.height + (1 << self.api.ndecomp_v) - 1) >> self.api.ndecomp_v
        q = np.zeros(rows, np.uint8)
        r = np.zeros(rows, np.uint8)
        _check("rc_results", lib().svt_jpeg_xs_gpu_encoder_rc_results(ctypes.byref(self.api), q.ctypes.data, r.ctypes.data, rows))
        return q, r

    def set_stream(self, stream_handle):
        _check("set_stream", lib().svt_jpeg_xs_gpu_encoder_set_stream(ctypes.byref(self.api), stream_handle or None))

    def set_streams(self, stream_handles):
        arr = (ctypes.c_void_p * max(1, len(stream_handles)))(*stream_handles)
        _check("set_streams", lib().svt_jpeg_xs_gpu_encoder_set_streams(ctypes.byref(self.api), arr, len(stream_handles)))

    def set_timing(self, on):
        _check("set_timing", lib().svt_jpeg_xs_gpu_encoder_set_timing(ctypes.byref(self.api), 1 if on else 0))

    def read_kernel_timing(self):
        ms = (ctypes.c_double * 16)()
        n = lib().svt_jpeg_xs_gpu_encoder_read_kernel_timing(ctypes.byref(self.api), ms, 16)
        return [ms[i] for i in range(n)]

    def read_timing(self):
        ms = (ctypes.c_double * 5)()
        n = lib().svt_jpeg_xs_gpu_encoder_read_timing(ctypes.byref(self.api), ms, 5)
        return int(n), list(ms)


def frame_size(bs, fast=0):
    cfg = ImageConfig()
    n = ctypes.c_uint32()
    buf = np.ascontiguousarray(bs, dtype=np.uint8)
    r = lib().svt_jpeg_xs_decoder_get_single_frame_size(buf.ctypes.data, buf.nbytes, ctypes.byref(cfg), ctypes.byref(n), fast)
    return r, n.value, cfg


class Decoder:
    """GPU decoder behind the reference C API; initialised from a codestream."""

    def __init__(self, first_codestream, packetization_mode=0, verbose=0, proxy_mode=0):
        self.api = DecoderApi()
        self.api.verbose = verbose
        self.api.packetization_mode = packetization_mode
        self.api.proxy_mode = proxy_mode
        self.config = ImageConfig()
        buf = np.ascontiguousarray(first_codestream, dtype=np.uint8)
        _check("decoder_init", lib().svt_jpeg_xs_decoder_init(API_MAJOR, API_MINOR, ctypes.byref(self.api), buf.ctypes.data,
                                                              buf.nbytes, ctypes.byref(self.config)))

    def close(self):
        if self.api is not None and self.api.private_ptr:
            lib().svt_jpeg_xs_decoder_close(ctypes.byref(self.api))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def alloc_planes(self):
        dt = np.uint8 if self.config.bit_depth <= 8 else np.uint16
        return [np.zeros((self.config.components[c].height, self.config.components[c].width), dt)
                for c in range(self.config.components_num)]

    def _frame(self, bs, planes, bs_size=None, user=None):
        f = Frame()
        if isinstance(bs, np.ndarray):
            f.bitstream.buffer = bs.ctypes.data
            f.bitstream.allocation_size = f.bitstream.used_size = bs.nbytes
        else:
            f.bitstream.buffer = int(bs)
            f.bitstream.allocation_size = f.bitstream.used_size = bs_size
        bps = 1 if self.config.bit_depth <= 8 else 2
        for c, p in enumerate(planes):
            if isinstance(p, tuple):
                f.image.data_yuv[c] = p[0]
                f.image.stride[c] = p[1]
                f.image.alloc_size[c] = p[1] * self.config.components[c].height * bps
            else:
                f.image.data_yuv[c] = p.ctypes.data
                f.image.stride[c] = p.shape[1]
                f.image.alloc_size[c] = p.nbytes
        f.user_prv_ctx_ptr = user
        return f

    def send(self, bs, planes, bs_size=None, blocking=True, user=None):
        f = self._frame(bs, planes, bs_size, user)
        return lib().svt_jpeg_xs_decoder_send_frame(ctypes.byref(self.api), ctypes.byref(f), 1 if blocking else 0)

    def make_frame(self, bs, planes, bs_size=None):
        """A frame structure to send repeatedly (the API copies it per call)."""
        return self._frame(bs, planes, bs_size)

    def send_frame(self, frame, blocking=True):
        return lib().svt_jpeg_xs_decoder_send_frame(ctypes.byref(self.api), ctypes.byref(frame), 1 if blocking else 0)

    def get(self, blocking=True):
        f = Frame()
        r = lib().svt_jpeg_xs_decoder_get_frame(ctypes.byref(self.api), ctypes.byref(f), 1 if blocking else 0)
        return r, f

    def decode(self, bs):
        bs = np.ascontiguousarray(bs, dtype=np.uint8)
        planes = self.alloc_planes()
        _check("send_frame", self.send(bs, planes))
        r, _ = self.get()
        _check("get_frame", r)
        return planes

    def set_stream(self, stream_handle):
        _check("set_stream", lib().svt_jpeg_xs_gpu_decoder_set_stream(ctypes.byref(self.api), stream_handle or None))

    def set_streams(self, stream_handles):
        arr = (ctypes.c_void_p * max(1, len(stream_handles)))(*stream_handles)
        _check("set_streams", lib().svt_jpeg_xs_gpu_decoder_set_streams(ctypes.byref(self.api), arr, len(stream_handles)))

    def set_timing(self, on):
        _check("set_timing", lib().svt_jpeg_xs_gpu_decoder_set_timing(ctypes.byref(self.api), 1 if on else 0))

    def read_kernel_timing(self):
        ms = (ctypes.c_double * 16)()
        n = lib().svt_jpeg_xs_gpu_decoder_read_kernel_timing(ctypes.byref(self.api), ms, 16)
        return [ms[i] for i in range(n)]

    def read_timing(self):
        ms = (ctypes.c_double * 4)()
        n = lib().svt_jpeg_xs_gpu_decoder_read_timing(ctypes.byref(self.api), ms, 4)
        return int(n), list(ms)


class Batch:
    """Batched encode/decode (svt_jpeg_xs_gpu_batch_*): frame i of a call uses
    the configuration of the i-th Encoder / Decoder.  One batch in flight per
    object; encode()/decode() queue it, wait() completes it."""

    def __init__(self, device_bytes, use_graph=True, autotune=False):
        self.h = ctypes.c_void_p()
        _check("batch_create", lib().svt_jpeg_xs_gpu_batch_create(int(device_bytes), ctypes.byref(self.h)))
        self.set_options(use_graph, autotune)
        self._keep = None
        self.n = 0

    def close(self):
        if self.h:
            lib().svt_jpeg_xs_gpu_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_options(self, use_graph=True, autotune=False):
        _check("batch_set_options", lib().svt_jpeg_xs_gpu_batch_set_options(self.h, 1 if use_graph else 0, 1 if autotune else 0))

    STAGES = ("fwd_v", "fwd_h", "rc", "pack", "walk", "unpack", "inv_h", "inv_v")

    def set_stage_timing(self, on=True):
        _check("batch_set_stage_timing", lib().svt_jpeg_xs_gpu_batch_set_stage_timing(self.h, 1 if on else 0))

    def read_stage_times(self):
        """[(stage name, variant, ms)] of the launches of the last batch
        issued with stage timing on (after its wait)."""
        n = 256
        st, var, ms = (ctypes.c_int32 * n)(), (ctypes.c_int32 * n)(), (ctypes.c_float * n)()
        k = lib().svt_jpeg_xs_gpu_batch_read_stage_times(self.h, st, var, ms, n)
        return [(self.STAGES[st[i]], var[i], ms[i]) for i in range(k)]

    def set_tune(self, chains=1, heavy_first=0, grid_per_sm=0, fwd_rows=4, inv_rows=4):
        t = (ctypes.c_int32 * 5)(chains, heavy_first, grid_per_sm, fwd_rows, inv_rows)
        _check("batch_set_tune", lib().svt_jpeg_xs_gpu_batch_set_tune(self.h, t))

    def encode(self, encoders, planes_list, outs, out_caps=None, stream=None):
        """Queues encoders[i].encode(planes_list[i]) into outs[i] (numpy array
        or device pointer with out_caps[i] bytes)."""
        n = len(encoders)
        frames = [e._frame(p, o, out_caps[i] if out_caps else None) for i, (e, p, o) in enumerate(zip(encoders, planes_list, outs))]
        apis = (ctypes.c_void_p * n)(*[ctypes.addressof(e.api) for e in encoders])
        fps = (ctypes.c_void_p * n)(*[ctypes.addressof(f) for f in frames])
        self._keep = (frames, apis, fps, planes_list, outs)
        self.n = n
        return lib().svt_jpeg_xs_gpu_batch_encode(self.h, apis, fps, n, stream)

    def decode(self, decoders, bitstreams, planes_list, sizes=None, stream=None):
        """Queues decoders[i].decode(bitstreams[i]) into planes_list[i] (numpy
        arrays or (device_ptr, stride) tuples); device codestreams need sizes."""
        n = len(decoders)
        frames = [d._frame(b, p, sizes[i] if sizes else None) for i, (d, b, p) in enumerate(zip(decoders, bitstreams, planes_list))]
        apis = (ctypes.c_void_p * n)(*[ctypes.addressof(d.api) for d in decoders])
        fps = (ctypes.c_void_p * n)(*[ctypes.addressof(f) for f in frames])
        self._keep = (frames, apis, fps, bitstreams, planes_list)
        self.n = n
        return lib().svt_jpeg_xs_gpu_batch_decode(self.h, apis, fps, n, stream)

    def wait(self):
        """(first error or 0, per-frame statuses)"""
        st = (ctypes.c_uint32 * BATCH_MAX)()
        r = lib().svt_jpeg_xs_gpu_batch_wait(self.h, st)
        self._keep = None
        return r, [st[i] for i in range(self.n)]

    def ready(self):
        return bool(lib().svt_jpeg_xs_gpu_batch_ready(self.h))

    def info(self):
        i = BatchInfo()
        _check("batch_get_info", lib().svt_jpeg_xs_gpu_batch_get_info(self.h, ctypes.byref(i)))
        return {"last_gpu_ms": i.last_gpu_ms, "last_launches": i.last_launches, "graph_hits": i.graph_hits,
                "graph_builds": i.graph_builds, "graph_updates": i.graph_updates, "tune": list(i.tune),
                "device_bytes": i.device_bytes, "device_used": i.device_used, "device_peak": i.device_peak}


class Server:
    """Serving loop (svt_jpeg_xs_gpu_server_*): requests on device buffers
    from many streams, batched continuously (SERVER_BATCHED) or run frame by
    frame on each stream's handle (SERVER_PER_FRAME)."""

    def __init__(self, device_bytes, mode=SERVER_BATCHED, lanes=2, max_batch=16):
        self.h = ctypes.c_void_p()
        _check("server_create", lib().svt_jpeg_xs_gpu_server_create(int(device_bytes), mode, lanes, max_batch, ctypes.byref(self.h)))
        self._buf = (ServerCompletion * 4096)()

    def close(self):
        if self.h:
            lib().svt_jpeg_xs_gpu_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_encoder(self, enc):
        sid = lib().svt_jpeg_xs_gpu_server_add_encoder(self.h, ctypes.byref(enc.api))
        if sid < 0:
            raise JxsError("server_add_encoder", E_BAD_PARAMETER)
        return sid

    def add_decoder(self, dec):
        sid = lib().svt_jpeg_xs_gpu_server_add_decoder(self.h, ctypes.byref(dec.api))
        if sid < 0:
            raise JxsError("server_add_decoder", E_BAD_PARAMETER)
        return sid

    def submit(self, stream, tag, planes, bitstream, bitstream_size=0):
        """planes: (device_ptr, stride) tuples; bitstream: device pointer"""
        r = ServerRequest()
        r.stream, r.tag = stream, tag
        for k, (ptr, stride) in enumerate(planes):
            r.planes[k] = ptr
            r.strides[k] = stride
        r.bitstream = bitstream
        r.bitstream_size = bitstream_size
        return lib().svt_jpeg_xs_gpu_server_submit(self.h, ctypes.byref(r))

    def poll(self):
        """completed requests: (tag, stream, status, t_arrive_ns, t_start_ns, t_done_ns)"""
        n = lib().svt_jpeg_xs_gpu_server_poll(self.h, self._buf, len(self._buf))
        return [(c.tag, c.stream, c.status, c.t_arrive_ns, c.t_start_ns, c.t_done_ns) for c in self._buf[:n]]

    def pending(self):
        return int(lib().svt_jpeg_xs_gpu_server_pending(self.h))

    def stats(self):
        st = ServerStats()
        _check("server_get_stats", lib().svt_jpeg_xs_gpu_server_get_stats(self.h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}
