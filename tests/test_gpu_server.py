"""Serving loop (svt_jpeg_xs_gpu_server_*): continuous batching of encode and
decode requests from many streams under a device-memory budget.

Each request's result must be the same alone and in the mix: byte-identical
codestreams and bit-identical decodes against the golden fixtures (which the
reference produced), in both the batched and the per-frame mode.
"""
import time

import numpy as np
import pytest

import golden_cases as G
import jxs_synth as S
from test_gpu_codec import make_encoder

pytestmark = pytest.mark.gpu
SMALL = G.small_cases()
GB = 1 << 30


def _drain(server, n, timeout=120.0):
    got = []
    t0 = time.time()
    while len(got) < n:
        got.extend(server.poll())
        assert time.time() - t0 < timeout, "server did not complete its requests"
        time.sleep(0.0005)
    assert server.pending() == 0
    return got


def _dev_planes(torch, arrays):
    ts = [torch.from_numpy(a).cuda() for a in arrays]
    return ts, [(t.data_ptr(), t.shape[1]) for t in ts]


@pytest.mark.parametrize("mode", ["batched", "per_frame"])
def test_server_mixed_streams_same_alone_and_in_mix(gpu, mode):
    torch = pytest.importorskip("torch")
    names = sorted(SMALL)
    m = gpu.SERVER_BATCHED if mode == "batched" else gpu.SERVER_PER_FRAME
    server = gpu.Server(2 * GB, m, lanes=2, max_batch=8)
    encs, decs, esid, dsid = {}, {}, {}, {}
    for n in names:
        encs[n] = make_encoder(gpu, SMALL[n])
        decs[n] = gpu.Decoder(SMALL[n]["bs"])
        esid[n] = server.add_encoder(encs[n])
        dsid[n] = server.add_decoder(decs[n])
    inputs = {n: _dev_planes(torch, SMALL[n]["planes"]) for n in names}
    dev_bs = {n: torch.from_numpy(SMALL[n]["bs"]).cuda() for n in names}
    rng = np.random.default_rng(11)
    jobs = [(n, kind) for n in names for kind in ("enc", "dec") for _ in range(4)]
    order = rng.permutation(len(jobs))
    outs = {}
    for tag, j in enumerate(order):
        n, kind = jobs[j]
        if kind == "enc":
            out = torch.zeros(encs[n].frame_bytes, dtype=torch.uint8, device="cuda")
            outs[tag] = (n, kind, out)
            assert server.submit(esid[n], tag, inputs[n][1], out.data_ptr()) == 0
        else:
            planes = [torch.zeros(p.shape, dtype=torch.uint8 if p.dtype == np.uint8 else torch.int16, device="cuda")
                      for p in SMALL[n]["dec"]]
            outs[tag] = (n, kind, planes)
            assert server.submit(dsid[n], tag, [(t.data_ptr(), t.shape[1]) for t in planes], dev_bs[n].data_ptr(),
                                 dev_bs[n].numel()) == 0
        if tag % 7 == 0:
            time.sleep(0.002)  # let some requests run alone
    done = _drain(server, len(jobs))
    assert sorted(d[0] for d in done) == list(range(len(jobs)))
    for tag, stream, status, ta, ts, td in done:
        assert status == 0, (tag, hex(status))
        assert ta <= ts <= td
        n, kind, out = outs[tag]
        if kind == "enc":
            assert np.array_equal(out.cpu().numpy(), SMALL[n]["bs"]), (n, tag)
        else:
            for t, p in zip(out, SMALL[n]["dec"]):
                assert np.array_equal(t.cpu().numpy().view(p.dtype), p), (n, tag)
    st = server.stats()
    if mode == "batched":
        assert st["batched_frames"] == len(jobs) and st["max_batch_seen"] > 1 and st["batches"] < len(jobs)
        assert st["device_peak"] <= st["device_bytes"]
    server.close()
    for x in list(encs.values()) + list(decs.values()):
        x.close()


def test_server_device_budget_admission(gpu):
    """A budget that holds two 1080p working sets: the other requests wait
    for memory (deferred) and all complete bit-exact; a request that can
    never fit completes with SvtJxsErrorInsufficientResources.  One lane per
    kind: the first request runs alone in its stream's frame slot, the seven
    that arrive meanwhile then form one batch, larger than the budget."""
    torch = pytest.importorskip("torch")
    enc = gpu.Encoder(1920, 1080, 8, S.FMT_YUV422, 3)
    big = gpu.Encoder(3840, 2160, 10, S.FMT_YUV422, 3)
    planes = S.frame(1920, 1080, 8, S.FMT_YUV422, seed=9)
    want = enc.encode(planes)
    server = gpu.Server(48 << 20, gpu.SERVER_BATCHED, lanes=1, max_batch=8)
    sid = server.add_encoder(enc)
    bid = server.add_encoder(big)
    _, dp = _dev_planes(torch, planes)
    outs = [torch.zeros(enc.frame_bytes, dtype=torch.uint8, device="cuda") for _ in range(8)]
    for i, o in enumerate(outs):
        assert server.submit(sid, i, dp, o.data_ptr()) == 0
    done = _drain(server, len(outs))
    assert all(d[2] == 0 for d in done)
    for o in outs:
        assert np.array_equal(o.cpu().numpy(), want)
    st = server.stats()
    assert st["deferred"] > 0 and st["device_peak"] <= 48 << 20
    bplanes = [torch.zeros((2160, 3840), dtype=torch.int16, device="cuda")] + \
              [torch.zeros((2160, 1920), dtype=torch.int16, device="cuda") for _ in range(2)]
    bout = torch.zeros(big.frame_bytes, dtype=torch.uint8, device="cuda")
    assert server.submit(bid, 99, [(t.data_ptr(), t.shape[1]) for t in bplanes], bout.data_ptr()) == 0
    done = _drain(server, 1)
    assert done[0][0] == 99 and done[0][2] == gpu.E_INSUFFICIENT_RESOURCES
    server.close()
    enc.close()
    big.close()
