"""Batched form (svt_jpeg_xs_gpu_batch_*): one launch per stage over frames
of mixed shapes, replayed as a CUDA graph.

Every frame of a batch must come out byte-identical (codestreams) and
bit-identical (decoded planes) to the oracle, to the golden fixtures and to
the per-frame path, whatever the launch shapes the batch runs with.
"""
import hashlib

import numpy as np
import pytest

import golden_cases as G
import jxs_synth as S
from test_gpu_codec import _random_cases, make_encoder

pytestmark = pytest.mark.gpu
SMALL = G.small_cases()
GB = 1 << 30


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _encode_batch(gpu, batch, encs, planes_list):
    outs = [np.zeros(e.frame_bytes + 64, np.uint8) for e in encs]
    assert batch.encode(encs, planes_list, outs) == 0
    r, st = batch.wait()
    assert r == 0 and st == [0] * len(encs)
    return [o[: e.frame_bytes].copy() for o, e in zip(outs, encs)]


def _decode_batch(gpu, batch, decs, bss):
    planes = [d.alloc_planes() for d in decs]
    assert batch.decode(decs, bss, planes) == 0
    r, st = batch.wait()
    assert r == 0 and st == [0] * len(decs)
    return planes


def test_batch_golden_mixed_shapes(gpu):
    """All golden cases (formats 4:2:2/4:2:0/4:4:4/RGB, depths 8-14, V0-V2,
    odd sizes, uniform quantization, RC mode 0) in one batch, twice: the
    second call replays the cached graph."""
    names = sorted(SMALL)
    encs = [make_encoder(gpu, SMALL[n]) for n in names]
    decs = [gpu.Decoder(SMALL[n]["bs"]) for n in names]
    batch = gpu.Batch(2 * GB)
    for rep in range(2):
        bss = _encode_batch(gpu, batch, encs, [SMALL[n]["planes"] for n in names])
        for n, bs in zip(names, bss):
            assert np.array_equal(bs, SMALL[n]["bs"]), n
        outs = _decode_batch(gpu, batch, decs, [SMALL[n]["bs"] for n in names])
        for n, out in zip(names, outs):
            assert all(np.array_equal(a, b) for a, b in zip(out, SMALL[n]["dec"])), n
    info = batch.info()
    assert info["graph_hits"] >= 2
    assert info["last_launches"] < 3 * len(names)
    batch.close()
    for x in encs + decs:
        x.close()


@pytest.mark.parametrize("tune", [None, (1, 0, 0, 4, 4), (3, 1, 2, 1, 2), (4, 0, 1, 2, 1), "auto"])
def test_batch_random_against_oracle(gpu, oracle, tune):
    """24 seeded random configurations per batch, against the oracle, under
    several launch shapes and the autotuner: the shapes change no bit."""
    cases = []
    for c in _random_cases(60, 77):
        p = oracle.make_params(c["w"], c["h"], c["d"], c["fmt"], c["bpp_num"], c["bpp_den"], c["v"], c["hh"],
                               quantization=c["q"], slice_height=c["sl"], significance=c["sig"], rc_mode=c["rc"])
        planes = S.frame(c["w"], c["h"], c["d"], c["fmt"], seed=c["seed"])
        err, ref_bs = oracle.oracle_encode(p, planes)
        if err:
            continue
        cases.append((c, planes, ref_bs))
        if len(cases) == 24:
            break
    encs = [make_encoder(gpu, c) for c, _, _ in cases]
    batch = gpu.Batch(2 * GB, autotune=(tune == "auto"))
    if isinstance(tune, tuple):
        batch.set_tune(*tune)
    bss = _encode_batch(gpu, batch, encs, [pl for _, pl, _ in cases])
    for (c, _, ref), bs in zip(cases, bss):
        assert np.array_equal(bs, ref), c
    decs = [gpu.Decoder(ref) for _, _, ref in cases]
    outs = _decode_batch(gpu, batch, decs, [ref for _, _, ref in cases])
    for (c, _, ref), out in zip(cases, outs):
        e2, want = oracle.oracle_decode(ref)
        assert e2 == 0 and all(np.array_equal(a, b) for a, b in zip(out, want)), c
    batch.close()
    for x in encs + decs:
        x.close()


def test_batch_equals_per_frame_full_size(gpu):
    """One frame of each shape of the mixed 48-frame batch workload (720p
    4:2:0 8-bit bpp 1, 1080p 4:4:4 12-bit bpp 4, 4K packed RGB 8-bit bpp 2),
    batched, against the reference's codestream and decode hashes."""
    names = ["c3_720p_420_8b_bpp1", "c3_1080p_444_12b_bpp4", "c3_2160p_rgb_8b_bpp2"]
    full = G.full_size()
    cases = [full[n] for n in names]
    planes = [G.full_planes(c) for c in cases]
    encs = [gpu.Encoder(c["w"], c["h"], c["d"], c["fmt"], c["bpp"], c["den"], c["v"], c["hh"]) for c in cases]
    batch = gpu.Batch(4 * GB, autotune=True)
    bss = _encode_batch(gpu, batch, encs, planes)
    for c, bs in zip(cases, bss):
        assert len(bs) == c["codestream_bytes"] and sha(bs) == c["codestream_sha256"]
    decs = [gpu.Decoder(bs) for bs in bss]
    outs = _decode_batch(gpu, batch, decs, bss)
    for c, out in zip(cases, outs):
        assert [sha(p) for p in out] == c["decoded_sha256"]
    batch.close()
    for x in encs + decs:
        x.close()


def test_batch_device_buffers_and_walk(gpu):
    """Device planes and codestreams: the precincts of device codestreams are
    found on the GPU; a codestream of another configuration fails its own
    frame only."""
    torch = pytest.importorskip("torch")
    a, b = SMALL["c1_422_8b"], SMALL["c3_444_12b"]
    encs = [make_encoder(gpu, a), make_encoder(gpu, b)]
    ta = [torch.from_numpy(p).cuda() for p in a["planes"]]
    tb = [torch.from_numpy(p).cuda() for p in b["planes"]]
    dplanes = [[(t.data_ptr(), t.shape[1]) for t in ta], [(t.data_ptr(), t.shape[1]) for t in tb]]
    outs = [torch.zeros(e.frame_bytes, dtype=torch.uint8, device="cuda") for e in encs]
    batch = gpu.Batch(1 * GB)
    assert batch.encode(encs, dplanes, [o.data_ptr() for o in outs], out_caps=[e.frame_bytes for e in encs]) == 0
    r, st = batch.wait()
    assert r == 0 and st == [0, 0]
    assert np.array_equal(outs[0].cpu().numpy(), a["bs"]) and np.array_equal(outs[1].cpu().numpy(), b["bs"])
    decs = [gpu.Decoder(a["bs"]), gpu.Decoder(b["bs"])]
    dout = [[torch.zeros(p.shape, dtype=torch.uint8 if p.dtype == np.uint8 else torch.int16, device="cuda") for p in c["dec"]]
            for c in (a, b)]
    planes = [[(t.data_ptr(), t.shape[1]) for t in ts] for ts in dout]
    assert batch.decode(decs, [o.data_ptr() for o in outs], planes, sizes=[o.numel() for o in outs]) == 0
    r, st = batch.wait()
    assert r == 0 and st == [0, 0]
    for ts, c in zip(dout, (a, b)):
        for t, p in zip(ts, c["dec"]):
            assert np.array_equal(t.cpu().numpy().view(p.dtype), p)
    # frame 1 gets frame 0's codestream: a configuration change for it alone
    assert batch.decode(decs, [outs[0].data_ptr(), outs[0].data_ptr()], planes, sizes=[outs[0].numel()] * 2) == 0
    r, st = batch.wait()
    assert st[0] == 0 and st[1] != 0 and r == st[1]
    batch.close()
    for x in encs + decs:
        x.close()


def test_batch_device_budget(gpu):
    """A batch whose working sets exceed the device budget is refused, and
    the object still runs batches that fit."""
    enc = gpu.Encoder(1920, 1080, 8, S.FMT_YUV422, 3)
    planes = S.frame(1920, 1080, 8, S.FMT_YUV422, seed=5)
    batch = gpu.Batch(64 << 20)
    outs = [np.zeros(enc.frame_bytes + 64, np.uint8) for _ in range(4)]
    assert batch.encode([enc] * 4, [planes] * 4, outs) == gpu.E_INSUFFICIENT_RESOURCES
    assert batch.encode([enc], [planes], outs[:1]) == 0
    r, st = batch.wait()
    assert r == 0 and np.array_equal(outs[0][: enc.frame_bytes], enc.encode(planes))
    batch.close()
    enc.close()


def test_batch_stage_timing(gpu):
    """Stage timing: with it on, a batch runs without graphs, its outputs
    unchanged, and every launch reports its stage and a device time; the
    golden 4:2:2 and 4:4:4 cases encode in one launch per stage, so the
    stages come in pipeline order."""
    names = ["c1_422_8b", "c3_444_12b"]
    encs = [make_encoder(gpu, SMALL[n]) for n in names]
    decs = [gpu.Decoder(SMALL[n]["bs"]) for n in names]
    batch = gpu.Batch(1 * GB)
    batch.set_tune(1, 0, 0, 4, 4)
    batch.set_stage_timing(True)
    bss = _encode_batch(gpu, batch, encs, [SMALL[n]["planes"] for n in names])
    for n, bs in zip(names, bss):
        assert np.array_equal(bs, SMALL[n]["bs"]), n
    enc_t = batch.read_stage_times()
    outs = _decode_batch(gpu, batch, decs, [SMALL[n]["bs"] for n in names])
    for n, out in zip(names, outs):
        assert all(np.array_equal(a, b) for a, b in zip(out, SMALL[n]["dec"])), n
    dec_t = batch.read_stage_times()
    order = {s: i for i, s in enumerate(gpu.Batch.STAGES)}
    for times, allowed in ((enc_t, {"fwd_v", "fwd_h", "rc", "pack"}), (dec_t, {"walk", "unpack", "inv_h", "inv_v"})):
        stages = [s for s, _, _ in times]
        assert stages and set(stages) <= allowed, stages
        assert all(ms > 0 for _, _, ms in times), times
        # one chain: rate control after every transform launch, packing last
        if "rc" in stages:
            assert stages.index("rc") > max(i for i, s in enumerate(stages) if s.startswith("fwd"))
            assert stages[-1] == "pack"
        assert [order[s] for s in stages if s in ("unpack", "inv_h")] == sorted(order[s] for s in stages if s in ("unpack", "inv_h"))
    assert {"fwd_v", "rc", "pack"} <= {s for s, _, _ in enc_t}
    assert {"unpack", "inv_v"} <= {s for s, _, _ in dec_t}
    assert batch.info()["graph_hits"] == 0
    # off again: graphs resume and nothing more is recorded
    batch.set_stage_timing(False)
    _encode_batch(gpu, batch, encs, [SMALL[n]["planes"] for n in names])
    _encode_batch(gpu, batch, encs, [SMALL[n]["planes"] for n in names])
    assert batch.info()["graph_hits"] >= 1
    batch.close()
    for x in encs + decs:
        x.close()
