"""The allocation-free entry point svt_jpeg_xs_gpu_decoder_locate_frame.

It must agree with the existing entry point that answers the same question,
svt_jpeg_xs_decoder_get_single_frame_size, on two calls in a row. Its
precinct offsets must follow the codestream's own precinct lengths. The file
name sorts last so that the suite also runs it after every other GPU test;
it sets up everything it uses and passes alone as well.
"""
import ctypes

import numpy as np
import pytest

import jxs_synth as S

pytestmark = pytest.mark.gpu

W, H = 256, 64          # 4:2:2 8-bit, V2/H5: 30 bands, 16 precinct rows, 4 slices
PREC_HDR_BYTES = (40 + 2 * 30 + 7) // 8


def _encode(jxs, seed, w=W, h=H, bpp=3, **kw):
    planes = S.frame(w, h, 8, S.FMT_YUV422, seed=seed)
    enc = jxs.Encoder(w, h, 8, S.FMT_YUV422, bpp, **kw)
    bs = enc.encode(planes)
    enc.close()
    return bs


def _host_frame_size(jxs, bs):
    size = ctypes.c_uint32()
    r = jxs.lib().svt_jpeg_xs_decoder_get_single_frame_size(bs.ctypes.data, len(bs), None, ctypes.byref(size), 0)
    assert r == 0
    return size.value


def _locate(jxs, dec, dev, nbytes, cap):
    size = ctypes.c_uint32(12345)
    offs = (ctypes.c_uint32 * max(cap, 1))()
    r = jxs.lib().svt_jpeg_xs_gpu_decoder_locate_frame(ctypes.byref(dec.api), ctypes.c_void_p(dev), nbytes, ctypes.byref(size),
                                                       offs if cap else None, cap, None)
    return r, size.value, list(offs)[:cap]


def _walk_precincts(bs):
    """Precinct offsets read from the codestream: after the header, slice
    headers (FF20) and precincts (24-bit length + header bytes) up to EOC."""
    pos = bs.tobytes().index(b"\xff\x20\x00\x04")
    offs = []
    while True:
        if bs[pos] == 0xFF and bs[pos + 1] == 0x11:
            return offs, pos + 2
        if bs[pos] == 0xFF and bs[pos + 1] == 0x20:
            pos += 6
            continue
        offs.append(pos)
        pos += PREC_HDR_BYTES + ((int(bs[pos]) << 16) | (int(bs[pos + 1]) << 8) | int(bs[pos + 2]))


def test_locate_frame_matches_existing_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    a, b = _encode(gpu, 11), _encode(gpu, 12)
    assert not np.array_equal(a, b)
    dec = gpu.Decoder(a)
    np_ = H // 4
    for bs in (a, b):  # two calls in a row
        dev = torch.from_numpy(np.concatenate([bs, np.zeros(100, np.uint8)])).cuda()
        r, size, offs = _locate(gpu, dec, dev.data_ptr(), dev.numel(), np_)
        assert r == 0, hex(r)
        assert size == _host_frame_size(gpu, bs) == len(bs)
        want, end = _walk_precincts(bs)
        assert end == size and offs == want
        # the size alone, without offsets
        r, size2, _ = _locate(gpu, dec, dev.data_ptr(), dev.numel(), 0)
        assert r == 0 and size2 == size
    dec.close()


def test_locate_frame_errors(gpu):
    torch = pytest.importorskip("torch")
    a = _encode(gpu, 11)
    dec = gpu.Decoder(a)
    dev = torch.from_numpy(a).cuda()
    # too little room for the offsets
    r, _, _ = _locate(gpu, dec, dev.data_ptr(), dev.numel(), 3)
    assert r == gpu.E_BAD_PARAMETER
    # truncated stream
    r, size, _ = _locate(gpu, dec, dev.data_ptr(), dev.numel() // 2, 0)
    assert r != 0 and size == 0
    # a stream of another configuration
    other = torch.from_numpy(_encode(gpu, 11, w=W + 64)).cuda()
    r, _, _ = _locate(gpu, dec, other.data_ptr(), other.numel(), 0)
    assert r == gpu.E_DEC_CONFIG_CHANGE
    # host memory is not accepted
    r, _, _ = _locate(gpu, dec, a.ctypes.data, len(a), 0)
    assert r == gpu.E_DEC_INVALID_POINTER
    # and a good call still works afterwards
    r, size, _ = _locate(gpu, dec, dev.data_ptr(), dev.numel(), 0)
    assert r == 0 and size == len(a)
    dec.close()


def test_locate_frame_rejects_more_precincts_than_its_scratch(gpu):
    torch = pytest.importorskip("torch")
    # decomp_v 0: one precinct per line, 4104 > 4096 precincts
    bs = _encode(gpu, 3, w=64, h=4104, ndecomp_v=0)
    dec = gpu.Decoder(bs)
    dev = torch.from_numpy(bs).cuda()
    r, size, _ = _locate(gpu, dec, dev.data_ptr(), dev.numel(), 0)
    assert r == gpu.E_BAD_PARAMETER and size == 0
    dec.close()


def test_locate_frame_walks_in_order_when_slices_are_elsewhere(gpu):
    """A stream that differs from the decoder's only in Lcod (the same
    settings at another bpp) has no slice where the decoder's constant-bit-rate
    split puts it, so the one-thread walk from the header finds the precincts
    instead; its size and offsets must still match the codestream."""
    torch = pytest.importorskip("torch")
    a, b = _encode(gpu, 11), _encode(gpu, 11, bpp=4)
    assert len(b) != len(a)
    dec = gpu.Decoder(a)
    for bs in (b, a, b):
        dev = torch.from_numpy(np.concatenate([bs, np.zeros(64, np.uint8)])).cuda()
        r, size, offs = _locate(gpu, dec, dev.data_ptr(), dev.numel(), H // 4)
        assert r == 0, hex(r)
        assert size == _host_frame_size(gpu, bs) == len(bs)
        want, end = _walk_precincts(bs)
        assert end == size and offs == want
    dec.close()


def test_locate_frame_allocates_no_device_memory(gpu):
    """After a first call (which loads the module and resolves the scratch's
    address), further calls leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    a = _encode(gpu, 11)
    dec = gpu.Decoder(a)
    dev = torch.from_numpy(a).cuda()
    r, _, _ = _locate(gpu, dec, dev.data_ptr(), dev.numel(), H // 4)
    assert r == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(8):
        r, size, _ = _locate(gpu, dec, dev.data_ptr(), dev.numel(), H // 4)
        assert r == 0 and size == len(a)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    dec.close()
