/*
 * Serving loop: encode and decode requests from many streams, admitted by a
 * device-memory budget and batched continuously.
 *
 * A caller registers streams (an encoder or decoder handle each, whose
 * configuration the stream's frames share) and submits requests whose
 * planes and codestreams are already in device memory.  A scheduler thread
 * runs the device:
 *
 *   batched mode  `lanes` encode lanes and `lanes` decode lanes, each a
 *                 CUDA stream with one batch object (jxs_batch.cu).  Whenever
 *                 a lane is idle it takes the waiting requests of its kind,
 *                 oldest first, up to max_batch and as many as the device
 *                 budget admits (each request's working set is carved from
 *                 the shared arena), and launches them as one batch.
 *                 Requests that arrive while every lane is
 *                 busy wait for the next free lane, so the batch size follows
 *                 the load: one request alone runs at once, a burst runs
 *                 together.  A lane batches only what the idle lanes of its
 *                 kind cannot take one by one, and a lane that takes a
 *                 single request runs it in a free frame slot of the
 *                 request's stream (the per-frame launch path, without batch
 *                 planning).  A lane keeps its working sets for its next batch;
 *                 when a batch does not fit, the idle lanes give theirs back
 *                 to the arena first.
 *   per-frame     the plain drop-in path: every request goes to a free frame
 *                 slot of its stream's own handle as soon as it arrives
 *                 (jxs_gpu_enc_submit / jxs_gpu_dec_submit), several frames
 *                 in flight per handle.  Its memory is the handles' slots.
 *
 * Latency of a request = its completion as seen by the scheduler minus its
 * submission, both on the host's steady clock.  The scheduler polls events
 * and sleeps only when nothing is in flight or waiting.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <sys/prctl.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "jxs_batch.h"
#include "jxs_gpu.h"
#include "jxs_kernels.cuh"
#include "jxs_server.h"

static int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct SrvReq {
    jxs_srv_request_t io;
    int64_t t_arrive, t_start;
};

struct SrvStream {
    int kind; /* 0 encode, 1 decode */
    jxs_gpu_enc_t* enc;
    jxs_gpu_dec_t* dec;
    uint64_t work_bytes;
    /* per-frame mode */
    std::deque<SrvReq> waiting;
    std::vector<SrvReq> slot_req;
    std::vector<int> slot_busy;
};

struct SrvLane {
    int kind = 0; /* 0 encode, 1 decode */
    jxs_gpu_batch_t* b = nullptr;
    cudaStream_t st = nullptr;
    std::vector<SrvReq> reqs;
    int busy = 0;
    /* a lone request runs in a frame slot of its stream's own handle (the
     * per-frame launch path, no batch planning): its stream and slot */
    int single_stream = -1, single_slot = -1;
};

struct jxs_server {
    int mode, lanes_n, max_batch;
    jxs_arena_t* arena = nullptr;
    std::vector<SrvStream> streams;
    std::vector<SrvLane> lanes;
    std::mutex mu;                 /* queue, done list, stream table */
    std::condition_variable cv;
    std::deque<SrvReq> queue[2];   /* batched mode: waiting encode / decode requests, oldest first */
    std::vector<jxs_srv_done_t> done;
    std::thread th;
    std::atomic<int> stop{0};
    std::atomic<int> started{0};
    /* statistics */
    uint64_t batches = 0, batched_frames = 0, max_seen_batch = 0, deferred = 0;
    uint64_t inflight = 0;
};

static void finish(jxs_server_t* s, const SrvReq& r, int32_t status, int64_t t_done) {
    jxs_srv_done_t d;
    d.tag = r.io.tag;
    d.stream = r.io.stream;
    d.status = status;
    d.t_arrive_ns = r.t_arrive;
    d.t_start_ns = r.t_start;
    d.t_done_ns = t_done;
    std::lock_guard<std::mutex> g(s->mu);
    s->done.push_back(d);
    s->inflight--;
}

/* ---------------------------------------------------------------- batched */
static int lane_poll(jxs_server_t* s, SrvLane& L) {
    if (!L.busy) return 0;
    if (L.single_slot >= 0) {
        SrvStream& S = s->streams[L.single_stream];
        const int k = L.single_slot;
        const int ready = S.kind == 0 ? jxs_gpu_enc_ready(S.enc, k) : jxs_gpu_dec_ready(S.dec, k);
        if (!ready) return 0;
        const int32_t st = S.kind == 0 ? jxs_gpu_enc_wait(S.enc, k) : jxs_gpu_dec_wait(S.dec, k);
        finish(s, L.reqs[0], st, now_ns());
        S.slot_busy[k] = 0;
        L.reqs.clear();
        L.single_slot = L.single_stream = -1;
        L.busy = 0;
        return 1;
    }
    if (!jxs_gpu_batch_ready(L.b)) return 0;
    int32_t st[JXS_BATCH_FRAMES];
    jxs_gpu_batch_wait(L.b, st);
    const int64_t t = now_ns();
    for (size_t i = 0; i < L.reqs.size(); i++) finish(s, L.reqs[i], st[i], t);
    L.reqs.clear();
    L.busy = 0;
    return 1;
}

/* Takes the oldest waiting requests of the lane's kind and launches them as
 * one batch.  Returns 1 if anything was launched. */
static int lane_launch(jxs_server_t* s, SrvLane& L) {
    {
        /* batch only what the idle lanes cannot take one by one: with as
         * many idle lanes of this kind as waiting requests, each lane takes
         * one (a lone request runs as soon as a lane is free) */
        int idle = 0;
        for (const SrvLane& o : s->lanes) idle += o.kind == L.kind && !o.busy;
        std::lock_guard<std::mutex> g(s->mu);
        std::deque<SrvReq>& q = s->queue[L.kind];
        const int waiting = (int)q.size();
        const int take = waiting <= idle ? 1 : std::min(s->max_batch, waiting - idle + 1);
        while (!q.empty() && (int)L.reqs.size() < take) {
            L.reqs.push_back(q.front());
            q.pop_front();
        }
    }
    if (L.reqs.empty()) return 0;
    uint64_t arena_bytes = 0, arena_used = 0, arena_peak = 0;
    jxs_arena_stats(s->arena, &arena_bytes, &arena_used, &arena_peak);
    if (L.reqs.size() == 1 && s->streams[L.reqs[0].io.stream].work_bytes <= arena_bytes) {
        /* one request: a free frame slot of its stream's handle, the same
         * launches as the per-frame path; a batch only if every slot is
         * busy.  A request whose working set exceeds the whole budget still
         * goes to the batch path, which refuses it. */
        SrvReq& r = L.reqs[0];
        SrvStream& S = s->streams[r.io.stream];
        for (size_t k = 0; k < S.slot_busy.size(); k++) {
            if (S.slot_busy[k]) continue;
            r.t_start = now_ns();
            const int32_t rc = S.kind == 0 ? jxs_gpu_enc_submit(S.enc, (int)k, r.io.planes, r.io.strides, (uint8_t*)r.io.bitstream)
                                           : jxs_gpu_dec_submit(S.dec, (int)k, (const uint8_t*)r.io.bitstream,
                                                                r.io.bitstream_size, nullptr, r.io.planes, r.io.strides);
            if (rc != JXS_OK) {
                finish(s, r, rc, now_ns());
                L.reqs.clear();
                return 1;
            }
            S.slot_busy[k] = 1;
            L.single_stream = r.io.stream;
            L.single_slot = (int)k;
            L.busy = 1;
            std::lock_guard<std::mutex> g(s->mu);
            s->batches++;
            s->batched_frames++;
            if (s->max_seen_batch < 1) s->max_seen_batch = 1;
            return 1;
        }
    }
    const uint32_t n0 = (uint32_t)L.reqs.size();
    std::vector<jxs_gpu_enc_t*> eh(n0);
    std::vector<jxs_gpu_dec_t*> dh(n0);
    for (uint32_t i = 0; i < n0; i++) {
        const SrvStream& S = s->streams[L.reqs[i].io.stream];
        eh[i] = S.enc;
        dh[i] = S.dec;
    }
    /* admission by the device budget: the leading requests whose working
     * sets fit; the others go back to the head of the queue */
    auto reserve = [&]() {
        return L.kind == 0 ? jxs_gpu_batch_reserve(L.b, eh.data(), nullptr, n0, L.st)
                           : jxs_gpu_batch_reserve(L.b, nullptr, dh.data(), n0, L.st);
    };
    uint32_t n = reserve();
    if (n < n0) {
        /* idle lanes keep their working sets for the next batch of the same
         * shapes; under memory pressure they give them back first */
        for (SrvLane& o : s->lanes)
            if (!o.busy) jxs_gpu_batch_release(o.b);
        n = reserve();
    }
    if (n < n0) {
        std::lock_guard<std::mutex> g(s->mu);
        s->deferred += n0 - n;
        for (uint32_t i = n0; i-- > n;) s->queue[L.kind].push_front(L.reqs[i]);
        L.reqs.resize(n);
    }
    if (n == 0) {
        /* nothing fits: wait for a busy lane to give its memory back, unless
         * none is busy, in which case the oldest request can never fit */
        int busy = 0;
        for (const SrvLane& o : s->lanes) busy |= o.busy;
        if (busy) return 0;
        SrvReq r;
        {
            std::lock_guard<std::mutex> g(s->mu);
            r = s->queue[L.kind].front();
            s->queue[L.kind].pop_front();
        }
        fprintf(stderr, "jxs server: a request of stream %d needs more device memory than the budget holds\n", r.io.stream);
        finish(s, r, JXS_E_RESOURCES, now_ns());
        return 1;
    }
    const int64_t t = now_ns();
    void* planes[JXS_BATCH_FRAMES][4];
    uint32_t strides[JXS_BATCH_FRAMES][4];
    const uint8_t* bs[JXS_BATCH_FRAMES];
    uint8_t* out[JXS_BATCH_FRAMES];
    uint32_t size[JXS_BATCH_FRAMES];
    for (uint32_t i = 0; i < n; i++) {
        SrvReq& r = L.reqs[i];
        r.t_start = t;
        for (int k = 0; k < 4; k++) {
            planes[i][k] = r.io.planes[k];
            strides[i][k] = r.io.strides[k];
        }
        bs[i] = (const uint8_t*)r.io.bitstream;
        out[i] = (uint8_t*)r.io.bitstream;
        size[i] = r.io.bitstream_size;
    }
    const int32_t rc = L.kind == 0 ? jxs_gpu_batch_encode(L.b, eh.data(), n, (void* const(*)[4])planes,
                                                          (const uint32_t(*)[4])strides, out, L.st)
                                   : jxs_gpu_batch_decode(L.b, dh.data(), n, bs, size, nullptr, (void* const(*)[4])planes,
                                                          (const uint32_t(*)[4])strides, L.st);
    if (rc != JXS_OK) {
        for (const SrvReq& r : L.reqs) finish(s, r, rc, now_ns());
        L.reqs.clear();
        return 1;
    }
    L.busy = 1;
    std::lock_guard<std::mutex> g(s->mu);
    s->batches++;
    s->batched_frames += n;
    if (n > s->max_seen_batch) s->max_seen_batch = n;
    return 1;
}

/* -------------------------------------------------------------- per-frame */
static int frame_poll(jxs_server_t* s) {
    int any = 0;
    for (size_t si = 0; si < s->streams.size(); si++) {
        SrvStream& S = s->streams[si];
        for (size_t k = 0; k < S.slot_busy.size(); k++) {
            if (!S.slot_busy[k]) continue;
            const int ready = S.kind == 0 ? jxs_gpu_enc_ready(S.enc, (int)k) : jxs_gpu_dec_ready(S.dec, (int)k);
            if (!ready) continue;
            const int32_t st = S.kind == 0 ? jxs_gpu_enc_wait(S.enc, (int)k) : jxs_gpu_dec_wait(S.dec, (int)k);
            finish(s, S.slot_req[k], st, now_ns());
            S.slot_busy[k] = 0;
            any = 1;
        }
    }
    return any;
}

static int frame_launch(jxs_server_t* s) {
    int any = 0;
    for (size_t si = 0; si < s->streams.size(); si++) {
        SrvStream& S = s->streams[si];
        for (size_t k = 0; k < S.slot_busy.size(); k++) {
            if (S.slot_busy[k]) continue;
            SrvReq r;
            {
                std::lock_guard<std::mutex> g(s->mu);
                if (S.waiting.empty()) break;
                r = S.waiting.front();
                S.waiting.pop_front();
            }
            r.t_start = now_ns();
            int32_t rc;
            if (S.kind == 0) {
                rc = jxs_gpu_enc_submit(S.enc, (int)k, r.io.planes, r.io.strides, (uint8_t*)r.io.bitstream);
            } else {
                rc = jxs_gpu_dec_submit(S.dec, (int)k, (const uint8_t*)r.io.bitstream, r.io.bitstream_size, nullptr, r.io.planes,
                                        r.io.strides);
            }
            if (rc != JXS_OK) {
                finish(s, r, rc, now_ns());
                continue;
            }
            S.slot_req[k] = r;
            S.slot_busy[k] = 1;
            any = 1;
        }
    }
    return any;
}

/* -------------------------------------------------------------- scheduler */
static void scheduler(jxs_server_t* s) {
    /* the short sleeps between polls last what they ask for, not the
     * default 50 us timer slack (completion seen sooner in both modes) */
    prctl(PR_SET_TIMERSLACK, 1000UL, 0, 0, 0);
    while (!s->stop.load()) {
        int work = 0;
        if (s->mode == JXS_SRV_BATCHED) {
            for (SrvLane& L : s->lanes) work |= lane_poll(s, L);
            for (SrvLane& L : s->lanes)
                if (!L.busy) work |= lane_launch(s, L);
        } else {
            work |= frame_poll(s);
            work |= frame_launch(s);
        }
        if (work) continue;
        std::unique_lock<std::mutex> g(s->mu);
        if (s->inflight == 0) {
            /* nothing submitted: sleep until a request arrives */
            s->cv.wait_for(g, std::chrono::milliseconds(20));
        } else {
            /* work on the device: poll again shortly */
            g.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(10));
        }
    }
}

extern "C" jxs_server_t* jxs_server_create(uint64_t device_bytes, int mode, int lanes, int max_batch, int32_t* err) {
    *err = JXS_OK;
    if (jxs_gpu_device_count() == 0) {
        fprintf(stderr, "jxs: no CUDA device available; this library has no CPU fallback\n");
        *err = JXS_E_RESOURCES;
        return nullptr;
    }
    jxs_server_t* s = new jxs_server_t();
    s->mode = mode;
    s->lanes_n = lanes < 1 ? 1 : (lanes > 8 ? 8 : lanes);
    s->max_batch = max_batch < 1 ? 1 : (max_batch > JXS_BATCH_FRAMES ? JXS_BATCH_FRAMES : max_batch);
    if (mode == JXS_SRV_BATCHED) {
        s->arena = jxs_arena_create(device_bytes);
        if (!s->arena) {
            delete s;
            *err = JXS_E_RESOURCES;
            return nullptr;
        }
        s->lanes.resize(2 * s->lanes_n);
        for (size_t i = 0; i < s->lanes.size(); i++) {
            SrvLane& L = s->lanes[i];
            L.kind = (int)(i & 1);
            int32_t e1 = 0;
            L.b = jxs_gpu_batch_create(0, s->arena, &e1);
            if (!L.b || cudaStreamCreateWithFlags(&L.st, cudaStreamNonBlocking) != cudaSuccess) {
                cudaGetLastError();
                jxs_server_destroy(s);
                *err = JXS_E_RESOURCES;
                return nullptr;
            }
            /* parameters change with every mix of requests: launch directly.
             * Working sets stay with their positions between batches and go
             * back to the arena when another lane needs the memory */
            jxs_gpu_batch_set_options(L.b, 0, 0);
        }
    }
    return s;
}

static void ensure_started(jxs_server_t* s) {
    int expected = 0;
    if (s->started.compare_exchange_strong(expected, 1)) s->th = std::thread(scheduler, s);
}

extern "C" int jxs_server_add_stream(jxs_server_t* s, jxs_gpu_enc_t* enc, jxs_gpu_dec_t* dec) {
    if (!s || (!enc) == (!dec) || s->started.load()) return -1;
    SrvStream S;
    S.kind = enc ? 0 : 1;
    S.enc = enc;
    S.dec = dec;
    S.work_bytes = enc ? jxs_gpu_batch_enc_work_bytes(enc) : jxs_gpu_batch_dec_work_bytes(dec);
    const int slots = enc ? jxs_gpu_enc_slots(enc) : jxs_gpu_dec_slots(dec);
    S.slot_req.resize(slots);
    S.slot_busy.assign(slots, 0);
    std::lock_guard<std::mutex> g(s->mu);
    s->streams.push_back(S);
    return (int)s->streams.size() - 1;
}

extern "C" int32_t jxs_server_submit(jxs_server_t* s, const jxs_srv_request_t* io) {
    if (!s || !io || io->stream < 0 || io->stream >= (int)s->streams.size()) return JXS_E_BAD_PARAM;
    if (!jxs_gpu_is_device_ptr(io->bitstream)) return JXS_E_BAD_PARAM;
    ensure_started(s);
    SrvReq r;
    r.io = *io;
    r.t_arrive = now_ns();
    r.t_start = 0;
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->mode == JXS_SRV_BATCHED) s->queue[s->streams[io->stream].kind].push_back(r);
        else s->streams[io->stream].waiting.push_back(r);
        s->inflight++;
    }
    s->cv.notify_one();
    return JXS_OK;
}

extern "C" int jxs_server_poll(jxs_server_t* s, jxs_srv_done_t* out, int max) {
    std::lock_guard<std::mutex> g(s->mu);
    const int n = (int)std::min<size_t>((size_t)max, s->done.size());
    for (int i = 0; i < n; i++) out[i] = s->done[i];
    s->done.erase(s->done.begin(), s->done.begin() + n);
    return n;
}

extern "C" uint64_t jxs_server_pending(jxs_server_t* s) {
    std::lock_guard<std::mutex> g(s->mu);
    return s->inflight;
}

extern "C" void jxs_server_stats(jxs_server_t* s, jxs_srv_stats_t* o) {
    memset(o, 0, sizeof(*o));
    std::lock_guard<std::mutex> g(s->mu);
    o->batches = s->batches;
    o->batched_frames = s->batched_frames;
    o->max_batch_seen = s->max_seen_batch;
    o->deferred = s->deferred;
    if (s->arena) jxs_arena_stats(s->arena, &o->device_bytes, &o->device_used, &o->device_peak);
}

extern "C" void jxs_server_destroy(jxs_server_t* s) {
    if (!s) return;
    s->stop.store(1);
    s->cv.notify_all();
    if (s->th.joinable()) s->th.join();
    for (SrvLane& L : s->lanes) {
        if (L.busy && L.single_slot >= 0) {
            SrvStream& S = s->streams[L.single_stream];
            if (S.kind == 0) jxs_gpu_enc_wait(S.enc, L.single_slot);
            else jxs_gpu_dec_wait(S.dec, L.single_slot);
            S.slot_busy[L.single_slot] = 0;
        } else if (L.busy) {
            int32_t st[JXS_BATCH_FRAMES];
            jxs_gpu_batch_wait(L.b, st);
        }
        jxs_gpu_batch_destroy(L.b);
        if (L.st) cudaStreamDestroy(L.st);
    }
    for (SrvStream& S : s->streams)
        for (size_t k = 0; k < S.slot_busy.size(); k++)
            if (S.slot_busy[k]) {
                if (S.kind == 0) jxs_gpu_enc_wait(S.enc, (int)k);
                else jxs_gpu_dec_wait(S.dec, (int)k);
            }
    jxs_arena_destroy(s->arena);
    delete s;
}
