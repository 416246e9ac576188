"""ctypes bindings to the oracle (this project's CPU restatement) and, where it
was built, the reference library compiled from source (oracle/_ref).

Test infrastructure only: used by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "libjxsoracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libjxsref.so")

_FIELDS = ("width height bit_depth colour_format bpp_num bpp_den decomp_v decomp_h quantization slice_height "
           "rate_control_mode coding_significance coding_signs_handling coding_vertical_prediction_mode threads_num "
           "precinct_width cpih tnlt nlt_sigma nlt_alpha nlt_t1 nlt_t2 nlt_e cts_cf cts_e1 cts_e2 cfa_type").split()


class EncParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in _FIELDS]


class ImageInfo(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("bit_depth", ctypes.c_uint32),
                ("format", ctypes.c_uint32), ("comps", ctypes.c_uint32), ("comp_w", ctypes.c_uint32 * 4),
                ("comp_h", ctypes.c_uint32 * 4), ("lcod", ctypes.c_uint32)]


def make_params(width, height, depth, fmt, bpp_num, bpp_den=1, decomp_v=2, decomp_h=5, quantization=0, slice_height=16,
                rc_mode=1, significance=1, threads=1, signs=0, vpred=0, cw=0):
    """cw > 0 (precinct columns) only for the oracle's own test codestreams:
    the reference encoder always writes Cw = 0."""
    return EncParams(width, height, depth, fmt, bpp_num, bpp_den, decomp_v, decomp_h, quantization, slice_height, rc_mode,
                     significance, signs, vpred, threads, cw)


def build_oracle():
    if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max(
            os.path.getmtime(os.path.join(ORACLE_DIR, f)) for f in ("jxs_oracle.c", "jxs_oracle.h")):
        subprocess.check_call(["make", "-s", "-C", ORACLE_DIR, "oracle"])


_oracle = None
_ref = None


def oracle():
    global _oracle
    if _oracle is None:
        build_oracle()
        _oracle = ctypes.CDLL(ORACLE_SO)
        _oracle.or_forward_dwt.restype = ctypes.c_int64
    return _oracle


def ref_available():
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_SO)
    return _ref


def _plane_args(planes):
    n = len(planes)
    ptrs = (ctypes.c_void_p * 4)(*([p.ctypes.data for p in planes] + [0] * (4 - n)))
    strides = (ctypes.c_uint32 * 4)(*([p.shape[1] for p in planes] + [0] * (4 - n)))
    allocs = (ctypes.c_uint32 * 4)(*([p.nbytes for p in planes] + [0] * (4 - n)))
    return ptrs, strides, allocs


def frame_size(params):
    n = ctypes.c_uint32()
    r = oracle().or_frame_size(ctypes.byref(params), ctypes.byref(n))
    if r:
        raise RuntimeError("or_frame_size failed: 0x%x" % (r & 0xffffffff))
    return n.value


def oracle_encode(params, planes, want_qr=False):
    """Returns (err, codestream bytes[, q, r per precinct row])."""
    ptrs, strides, _ = _plane_args(planes)
    cap = max(params.width * params.height * 8, 1 << 16)
    out = np.zeros(cap, np.uint8)
    sz = ctypes.c_uint32()
    rows = (params.height + (1 << params.decomp_v) - 1) >> params.decomp_v
    q = np.zeros(rows * (130 if params.precinct_width else 1), np.uint8)  # per precinct: rows x columns (< 130)
    r = np.zeros_like(q)
    err = oracle().or_encode(ctypes.byref(params), ptrs, strides, out.ctypes.data_as(ctypes.c_void_p), cap,
                             ctypes.byref(sz), q.ctypes.data_as(ctypes.c_void_p), r.ctypes.data_as(ctypes.c_void_p))
    err &= 0xffffffff
    bs = out[:sz.value].copy()
    if want_qr:
        return err, bs, q, r
    return err, bs


def oracle_forward_dwt(params, planes):
    ptrs, strides, _ = _plane_args(planes)
    cap = params.width * params.height * 4
    out = np.zeros(cap, np.uint16)
    n = oracle().or_forward_dwt(ctypes.byref(params), ptrs, strides, out.ctypes.data_as(ctypes.c_void_p), cap)
    if n < 0:
        raise RuntimeError("or_forward_dwt failed")
    return out[:n]


def probe(bs):
    info = ImageInfo()
    buf = np.ascontiguousarray(bs, dtype=np.uint8)
    err = oracle().or_probe(buf.ctypes.data_as(ctypes.c_void_p), len(buf), ctypes.byref(info))
    return err & 0xffffffff, info


def alloc_planes(info):
    dt = np.uint8 if info.bit_depth <= 8 else np.uint16
    return [np.zeros((info.comp_h[c], info.comp_w[c]), dt) for c in range(info.comps)]


def oracle_decode(bs, threads=1):
    err, info = probe(bs)
    if err:
        return err, None
    planes = alloc_planes(info)
    ptrs, strides, _ = _plane_args(planes)
    buf = np.ascontiguousarray(bs, dtype=np.uint8)
    err = oracle().or_decode(buf.ctypes.data_as(ctypes.c_void_p), len(buf), ptrs, strides, threads, None)
    return err & 0xffffffff, planes


def ref_encode(params, planes):
    ptrs, strides, allocs = _plane_args(planes)
    cap = max(params.width * params.height * 8, 1 << 16)
    out = np.zeros(cap, np.uint8)
    sz = ctypes.c_uint32()
    err = ref().ref_encode(ctypes.byref(params), ptrs, strides, allocs, out.ctypes.data_as(ctypes.c_void_p), cap,
                           ctypes.byref(sz))
    return err & 0xffffffff, out[:sz.value].copy()


def ref_decode_proxy(bs, proxy, threads=1):
    """The reference decoder at a proxy resolution (1 half, 2 quarter)."""
    buf = np.ascontiguousarray(bs, dtype=np.uint8)
    comps = ctypes.c_uint32()
    info = (ctypes.c_uint32 * 12)()
    err = ref().ref_probe_proxy(buf.ctypes.data_as(ctypes.c_void_p), len(buf), proxy, ctypes.byref(comps), info)
    if err:
        return err & 0xffffffff, None
    e0, full = probe(bs)
    dt = np.uint8 if full.bit_depth <= 8 else np.uint16
    planes = [np.zeros((info[3 * c + 1], info[3 * c]), dt) for c in range(comps.value)]
    ptrs, _, allocs = _plane_args(planes)
    err = ref().ref_decode_proxy(buf.ctypes.data_as(ctypes.c_void_p), len(buf), ptrs, allocs, threads, proxy)
    return err & 0xffffffff, planes


def ref_decode(bs, threads=1):
    err, info = probe(bs)
    if err:
        return err, None
    planes = alloc_planes(info)
    ptrs, _, allocs = _plane_args(planes)
    buf = np.ascontiguousarray(bs, dtype=np.uint8)
    err = ref().ref_decode(buf.ctypes.data_as(ctypes.c_void_p), len(buf), ptrs, allocs, threads)
    return err & 0xffffffff, planes


class RefStream:
    """The reference codec kept open over a stream of frames and driven like
    its sample applications (a sender thread with blocking sends, results
    collected as they complete, threads_num workers): the CPU baseline that
    bench.py times.  encode(frames) returns the codestreams (views into one
    buffer that the next encode call overwrites); decode(codestreams, outs)
    fills the preallocated planes."""

    def __init__(self, params):
        r = ref()
        r.ref_stream_open.restype = ctypes.c_void_p
        err = ctypes.c_int()
        self.h = r.ref_stream_open(ctypes.byref(params), ctypes.byref(err))
        if not self.h:
            raise RuntimeError("ref_stream_open failed: 0x%x" % (err.value & 0xffffffff))
        self.params = params
        self.cap = max(params.width * params.height * 8, 1 << 16)
        self._out = None

    def encode(self, frames):
        n = len(frames)
        if self._out is None or self._out.size < n * self.cap:
            self._out = np.zeros(n * self.cap, np.uint8)
        ptrs = (ctypes.c_void_p * (4 * n))()
        for i, planes in enumerate(frames):
            for c, p in enumerate(planes):
                ptrs[4 * i + c] = p.ctypes.data
        _, strides, allocs = _plane_args(frames[0])
        sizes = (ctypes.c_uint32 * n)()
        err = ref().ref_stream_encode(ctypes.c_void_p(self.h), n, ptrs, strides, allocs,
                                      self._out.ctypes.data_as(ctypes.c_void_p), self.cap, sizes)
        if err:
            raise RuntimeError("ref_stream_encode failed: 0x%x" % (err & 0xffffffff))
        return [self._out[i * self.cap:i * self.cap + sizes[i]] for i in range(n)]

    def decode(self, codestreams, outs):
        """Decodes into the preallocated plane lists `outs` (one per codestream)."""
        n = len(codestreams)
        bufs = [np.ascontiguousarray(b, dtype=np.uint8) for b in codestreams]
        bsp = (ctypes.c_void_p * n)(*[b.ctypes.data for b in bufs])
        sizes = (ctypes.c_uint32 * n)(*[len(b) for b in bufs])
        ptrs = (ctypes.c_void_p * (4 * n))()
        for i, planes in enumerate(outs):
            for c, p in enumerate(planes):
                ptrs[4 * i + c] = p.ctypes.data
        _, _, allocs = _plane_args(outs[0])
        err = ref().ref_stream_decode(ctypes.c_void_p(self.h), n, bsp, sizes, ptrs, allocs)
        if err:
            raise RuntimeError("ref_stream_decode failed: 0x%x" % (err & 0xffffffff))
        return outs

    def close(self):
        if self.h:
            ref().ref_stream_close(ctypes.c_void_p(self.h))
            self.h = None
