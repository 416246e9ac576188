/*
 * Batched form: many frames, of any mix of sizes, colour formats and bit
 * depths, each with the configuration of its own encoder (or decoder)
 * handle, run as ONE launch per stage over all frames of the batch instead
 * of one launch per stage per frame:
 *
 *   encode: [status reset] fwd_v level 0 (one launch per source kind)
 *           -> fwd_v level 1 -> fwd_h -> rc_cost -> pack
 *   decode: [status reset] walk (device codestreams) -> unpack -> inv_h
 *           -> inv_v (deepest level first)
 *
 * Each launch carries a job table (transform kernels: one job per frame
 * component; per-precinct kernels: one entry per frame), and every block
 * finds its job by the first block of each entry.  The launches of a batch
 * are captured into a CUDA graph, cached by the exact launch parameters, and
 * replayed: an unchanged batch costs one graph launch.
 *
 * Launch shapes come from a small autotuner (batch_autotune): how many
 * independent chains the frames are split into (each chain is a branch of
 * the graph, so the tail of one chain's stage overlaps the next stage of
 * another), the order of frames in a launch (precinct-to-CTA order: as
 * given, or heaviest frames first), the persistent grid of the first
 * transform level (blocks per SM) and the rows per block of the horizontal-
 * only levels.  None of them changes a single output bit.
 *
 * Device memory: every frame position of a batch owns a working set (level
 * planes, coefficients, GCLIs, cost tables, staging) carved from one device
 * arena whose size the caller fixes.  A batch that does not fit fails with
 * SvtJxsErrorInsufficientResources; nothing is allocated per call once the
 * positions exist.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "jxs_batch.h"
#include "jxs_gpu.h"
#include "jxs_plan.cuh"

#define BCK(x)                                                                                      \
    do {                                                                                            \
        cudaError_t e_ = (x);                                                                       \
        if (e_ != cudaSuccess) {                                                                    \
            fprintf(stderr, "jxs batch: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            return JXS_E_RESOURCES;                                                                 \
        }                                                                                           \
    } while (0)

#define MAX_CHAINS 4
#define GRAPH_CACHE 8

/* ------------------------------------------------------------------------ */
/* device arena: first-fit over one allocation                               */
/* ------------------------------------------------------------------------ */
struct jxs_arena {
    uint8_t* base = nullptr;
    uint64_t size = 0, used = 0, peak = 0;
    std::map<uint64_t, uint64_t> free_; /* offset -> bytes, neighbours merged */
    std::mutex mu;
};

static inline uint64_t round256(uint64_t n) { return (n + 255) & ~255ull; }

extern "C" jxs_arena_t* jxs_arena_create(uint64_t bytes) {
    jxs_arena_t* a = new jxs_arena_t();
    bytes = round256(bytes);
    if (!bytes || cudaMalloc(&a->base, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete a;
        return nullptr;
    }
    a->size = bytes;
    a->free_[0] = bytes;
    return a;
}

extern "C" void jxs_arena_destroy(jxs_arena_t* a) {
    if (!a) return;
    cudaFree(a->base);
    delete a;
}

extern "C" void* jxs_arena_alloc(jxs_arena_t* a, uint64_t bytes) {
    bytes = round256(bytes);
    std::lock_guard<std::mutex> g(a->mu);
    for (auto it = a->free_.begin(); it != a->free_.end(); ++it) {
        if (it->second < bytes) continue;
        const uint64_t off = it->first, rem = it->second - bytes;
        a->free_.erase(it);
        if (rem) a->free_[off + bytes] = rem;
        a->used += bytes;
        a->peak = std::max(a->peak, a->used);
        return a->base + off;
    }
    return nullptr;
}

extern "C" void jxs_arena_free(jxs_arena_t* a, void* p, uint64_t bytes) {
    if (!a || !p) return;
    bytes = round256(bytes);
    std::lock_guard<std::mutex> g(a->mu);
    uint64_t off = (uint64_t)((uint8_t*)p - a->base), n = bytes;
    a->used -= bytes;
    auto next = a->free_.lower_bound(off);
    if (next != a->free_.end() && off + n == next->first) {
        n += next->second;
        next = a->free_.erase(next);
    }
    if (next != a->free_.begin()) {
        auto prev = std::prev(next);
        if (prev->first + prev->second == off) {
            prev->second += n;
            return;
        }
    }
    a->free_[off] = n;
}

extern "C" void jxs_arena_stats(jxs_arena_t* a, uint64_t* size, uint64_t* used, uint64_t* peak) {
    std::lock_guard<std::mutex> g(a->mu);
    if (size) *size = a->size;
    if (used) *used = a->used;
    if (peak) *peak = a->peak;
}

/* ------------------------------------------------------------------------ */
/* working sets of one frame position                                        */
/* ------------------------------------------------------------------------ */
struct EncWork {
    uint64_t serial = 0;   /* encoder handle it was laid out for */
    uint8_t* mem = nullptr;
    uint64_t bytes = 0;
    uint8_t* in_stage;
    uint64_t in_off[JXS_MAXC];
    FrameBufs fb;
    uint32_t* cost;
    uint32_t* slice_done;
    PrecRC* rc;
    uint8_t* out_stage;
};

struct DecWork {
    uint64_t serial = 0;
    uint8_t* mem = nullptr;
    uint64_t bytes = 0;
    uint8_t* bs;
    uint32_t bs_cap;
    uint32_t* prec_off;
    FrameBufs fb;
    uint8_t* out_stage;
    uint64_t out_off[JXS_MAXC];
    uint32_t* prec_off_h = nullptr; /* page-locked: precinct offsets of a host codestream */
    uint32_t prec_cap = 0;
    uint8_t* hdr_h = nullptr;       /* header of a device codestream (in the batch's page-locked pool) */
};

/* Lays out (base NULL: only sizes) the encoder working set of one frame. */
static uint64_t enc_work_layout(const jxs_cfg_t* c, uint8_t* base, EncWork* w) {
    uint64_t off = 0;
    auto take = [&](uint64_t n) -> uint8_t* {
        uint8_t* p = base ? base + off : nullptr;
        off += round256(n);
        return p;
    };
    const uint32_t bps = bytes_per_sample(c);
    uint64_t in_bytes = 0;
    memset(w->in_off, 0, sizeof(w->in_off));
    if (c->fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB) {
        in_bytes = (uint64_t)c->W * c->H * 3 * bps;
    } else {
        for (uint32_t k = 0; k < c->nc; k++) {
            w->in_off[k] = in_bytes;
            in_bytes += round256((uint64_t)stage_pitch(c->comp[k].w, bps) * c->comp[k].h * bps);
        }
    }
    memset(&w->fb, 0, sizeof(w->fb));
    w->in_stage = take(in_bytes);
    w->fb.coef = take(c->coef_total * sizeof(uint16_t) + 64);
    w->fb.gcli = take(c->gcli_total + 64);
    uint64_t llsz[2][JXS_MAXC];
    ll_layout(c, w->fb.ll_pitch, llsz);
    for (int v = 0; v < 2; v++)
        for (int k = 0; k < JXS_MAXC; k++) w->fb.ll[v][k] = llsz[v][k] ? (int32_t*)take(llsz[v][k]) : nullptr;
    w->cost = (uint32_t*)take(jxs_cost_bytes(c));
    w->slice_done = (uint32_t*)take((uint64_t)c->nslices * sizeof(uint32_t));
    w->rc = (PrecRC*)take((uint64_t)c->np * sizeof(PrecRC));
    w->out_stage = take((uint64_t)c->lcod + 64);
    return off;
}

static uint64_t dec_work_layout(const jxs_cfg_t* c, uint8_t* base, DecWork* w) {
    uint64_t off = 0;
    auto take = [&](uint64_t n) -> uint8_t* {
        uint8_t* p = base ? base + off : nullptr;
        off += round256(n);
        return p;
    };
    memset(&w->fb, 0, sizeof(w->fb));
    w->bs_cap = c->lcod + 4096;
    w->bs = take((uint64_t)w->bs_cap + 64);
    w->prec_off = (uint32_t*)take((uint64_t)c->nprec * sizeof(uint32_t));
    w->fb.coef = take(c->coef_total * sizeof(int16_t) + 64);
    uint64_t llsz[2][JXS_MAXC];
    ll_layout(c, w->fb.ll_pitch, llsz);
    for (int v = 0; v < 2; v++)
        for (int k = 0; k < JXS_MAXC; k++) w->fb.ll[v][k] = llsz[v][k] ? (int32_t*)take(llsz[v][k]) : nullptr;
    const uint32_t bps = bytes_per_sample(c);
    uint64_t ob = 0;
    memset(w->out_off, 0, sizeof(w->out_off));
    for (uint32_t k = 0; k < c->nc; k++) {
        w->out_off[k] = ob;
        ob += round256((uint64_t)stage_pitch(jxs_out_w(c, k), bps) * jxs_out_h(c, k) * bps);
    }
    w->out_stage = take(ob);
    return off;
}

/* ------------------------------------------------------------------------ */
/* plans: the launches of one batch                                          */
/* ------------------------------------------------------------------------ */
/* Ops ending in _S carry the per-frame launch structure (at most 4 jobs)
 * and those ending in 1 one frame's arguments: a stage of one or two frames
 * then launches with a few hundred bytes of parameters instead of the
 * batched tables (about 9 KB), which costs host time on every launch. */
enum {
    OP_FWD_V, OP_FWD_H, OP_RC, OP_PACK, OP_WALK, OP_UNPACK, OP_INV_H, OP_INV_V,
    OP_FWD_V_S, OP_FWD_H_S, OP_INV_H_S, OP_INV_V_S, OP_RC1, OP_PACK1, OP_WALK1, OP_UNPACK1
};

/* The per-frame launch structure holding the (at most JXS_MAXC) jobs of a
 * batched one; both have the same fields before the job table. */
template <class SMALL, class BIG>
static void shrink(SMALL* sm, const BIG* big) {
    static_assert(offsetof(SMALL, job) == offsetof(BIG, job), "launch headers differ");
    memset(sm, 0, sizeof(*sm));
    memcpy(sm, big, offsetof(BIG, job));
    memcpy(sm->job, big->job, (size_t)big->njobs * sizeof(big->job[0]));
}

struct Op {
    int type, kind, chain, nblocks;
    uint32_t a, b;
    size_t off, size;
};

struct Plan {
    std::vector<Op> ops;
    std::vector<uint8_t> bytes; /* launch structures, 16-byte aligned offsets */
    int nchains = 1;
    uint32_t nframes = 0;
    void clear() {
        ops.clear();
        bytes.clear();
        nchains = 1;
        nframes = 0;
    }
    void add(int type, int kind, int chain, int nblocks, uint32_t a, uint32_t b, const void* data, size_t size) {
        Op o;
        memset(&o, 0, sizeof(o));
        o.type = type;
        o.kind = kind;
        o.chain = chain;
        o.nblocks = nblocks;
        o.a = a;
        o.b = b;
        o.off = (bytes.size() + 15) & ~(size_t)15;
        o.size = size;
        bytes.resize(o.off + size);
        memcpy(bytes.data() + o.off, data, size);
        ops.push_back(o);
    }
};

struct Tune {
    int chains;        /* independent branches the frames are split into */
    int heavy_first;   /* frames ordered by size, largest first */
    int grid_per_sm;   /* persistent first transform level: blocks per SM (0: as many as fit) */
    int fh_rpb, ih_rpb;/* rows (warps) per block of the horizontal-only levels */
};
static const Tune kDefaultTune = {1, 0, 0, 4, 4};

struct GraphEntry {
    std::vector<uint8_t> key;
    cudaGraphExec_t exec = nullptr;
    uint64_t last = 0;
};

/* one frame of the batch being planned */
struct EncItem {
    const jxs_cfg_t* c;
    const jxs_cfg_t* dcfg;
    uint32_t cap_words;
    FramePlanes in;
    uint8_t* out;     /* device codestream destination */
    EncWork* w;
    int* status;
};

struct DecItem {
    const jxs_cfg_t* c;
    const jxs_cfg_t* dcfg;
    uint32_t cap_bytes, cap_groups, cap_seg;
    const uint8_t* bs; /* device codestream */
    uint32_t size;
    int walk;          /* precinct offsets found on the GPU */
    FramePlanes out;
    DecWork* w;
    int* status;
};

struct jxs_gpu_batch {
    jxs_arena_t* arena = nullptr;
    int own_arena = 0;
    cudaStream_t st = nullptr;
    cudaStream_t side[MAX_CHAINS] = {};
    cudaEvent_t fork = nullptr, join[MAX_CHAINS] = {}, done = nullptr, t0 = nullptr, t1 = nullptr;
    int* status_d = nullptr;
    int* status_h = nullptr;
    uint8_t* hdr_pool = nullptr; /* page-locked: one codestream header per position */
    std::vector<EncWork> enc;
    std::vector<DecWork> dec;
    /* idle working sets, kept for positions that need the same handle's
     * layout again; freed when the arena runs short */
    struct Idle {
        int kind; /* 0 encoder, 1 decoder */
        uint64_t serial;
        uint8_t* mem;
        uint64_t bytes;
    };
    std::vector<Idle> idle;
    /* the call in flight */
    int pending = 0, kind = 0;
    uint32_t n = 0;
    std::vector<int> hdr_check;
    std::vector<const jxs_cfg_t*> cfgs;
    /* graphs and tuning */
    int use_graph = 1, autotune = 0;
    int release_after_wait = 0; /* serving: working sets go back to the arena when a batch completes */
    GraphEntry cache[GRAPH_CACHE];
    uint64_t clock = 0, graph_hits = 0, graph_builds = 0, graph_updates = 0;
    std::map<std::string, Tune> tuned;
    Tune last_tune = kDefaultTune;
    float last_ms = 0.f;
    uint32_t last_launches = 0;
    /* stage timing: an event pair around every launch of the batches issued
     * while it is on (no graphs); the stage and variant of each launch */
    int stage_timing = 0;
    std::vector<cudaEvent_t> tev;
    std::vector<int> tstage, tvar;
    uint32_t tcount = 0;
};

static void order_chains(const std::vector<uint64_t>& weight, const Tune& t, std::vector<std::vector<int>>* chains) {
    const int n = (int)weight.size();
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    if (t.heavy_first) std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return weight[a] > weight[b]; });
    const int nch = std::max(1, std::min(t.chains, n));
    chains->assign(nch, std::vector<int>());
    std::vector<uint64_t> load(nch, 0);
    for (int i : ord) {
        /* longest-processing-time assignment: the least loaded chain */
        int c = 0;
        for (int k = 1; k < nch; k++)
            if (load[k] < load[c]) c = k;
        (*chains)[c].push_back(i);
        load[c] += weight[i];
    }
}

/* Appends the launches of one encode chain. */
static int32_t plan_encode_chain(const std::vector<EncItem>& it, const std::vector<int>& fr, const Tune& t, int chain, Plan* P) {
    std::vector<uint8_t> scratch(std::max({sizeof(FwdVLaunchB), sizeof(FwdHLaunchB), sizeof(EncPrecLaunch)}));
    FwdVJob vj[JXS_MAXC];
    FwdHJob hj[JXS_MAXC];
    int tiles[JXS_MAXC];
    /* vertical levels: level 0 per source kind, level 1 on int32 low bands */
    for (int v = 0; v < 2; v++) {
        const int kinds[4] = {SRC_U8, SRC_U16, SRC_PK8, SRC_PK16};
        for (int ki = 0; ki < (v == 0 ? 4 : 1); ki++) {
            const int kind = v == 0 ? kinds[ki] : SRC_I32;
            FwdVLaunchB* L = (FwdVLaunchB*)scratch.data();
            memset(L, 0, sizeof(*L));
            auto flush = [&]() {
                if (L->njobs > JXS_MAXC) {
                    P->add(OP_FWD_V, kind, chain, L->ntiles, (uint32_t)t.grid_per_sm, 0, L, sizeof(*L));
                } else if (L->njobs) {
                    FwdVLaunch sm;
                    shrink(&sm, L);
                    P->add(OP_FWD_V_S, kind, chain, L->ntiles, (uint32_t)t.grid_per_sm, 0, &sm, sizeof(sm));
                }
                memset(L, 0, sizeof(*L));
            };
            for (int f : fr) {
                const EncItem& e = it[f];
                if (v == 0 && enc_level0_kind(e.c) != kind) continue;
                const int nj = plan_fwd_v(e.c, e.dcfg, e.w->fb, e.in, v, vj, tiles);
                for (int j = 0; j < nj; j++) {
                    if (L->njobs == JXS_BATCH_JOBS) flush();
                    vj[j].first_block = L->ntiles;
                    L->job[L->njobs++] = vj[j];
                    L->ntiles += tiles[j];
                }
            }
            flush();
        }
    }
    /* horizontal-only levels: pass 0 on int32 low bands, pass 1 on samples
     * (components without vertical levels) per source kind */
    for (int pass = 0; pass < 2; pass++) {
        const int kinds[4] = {SRC_U8, SRC_U16, SRC_PK8, SRC_PK16};
        for (int ki = 0; ki < (pass == 0 ? 1 : 4); ki++) {
            const int kind = pass == 0 ? SRC_I32 : kinds[ki];
            FwdHLaunchB* L = (FwdHLaunchB*)scratch.data();
            memset(L, 0, sizeof(*L));
            int32_t err = JXS_OK;
            auto flush = [&]() {
                if (L->njobs) {
                    const int blocks = fwd_h_layout(*L, t.fh_rpb);
                    if (blocks < 0) err = JXS_E_BAD_PARAM;
                    else if (L->njobs > JXS_MAXC) P->add(OP_FWD_H, kind, chain, blocks, 0, 0, L, sizeof(*L));
                    else {
                        FwdHLaunch sm;
                        shrink(&sm, L);
                        P->add(OP_FWD_H_S, kind, chain, blocks, 0, 0, &sm, sizeof(sm));
                    }
                }
                memset(L, 0, sizeof(*L));
            };
            for (int f : fr) {
                const EncItem& e = it[f];
                if (pass == 1 && enc_level0_kind(e.c) != kind) continue;
                const int nj = plan_fwd_h(e.c, e.dcfg, e.w->fb, e.in, pass, hj);
                for (int j = 0; j < nj; j++) {
                    if (L->njobs == JXS_BATCH_JOBS) flush();
                    L->job[L->njobs++] = hj[j];
                }
            }
            flush();
            if (err) return err;
        }
    }
    /* rate control, then packing: one entry per frame */
    for (int op = 0; op < 2; op++) {
        EncPrecLaunch* L = (EncPrecLaunch*)scratch.data();
        memset(L, 0, sizeof(*L));
        uint32_t cap = 0, signs = 0; /* rate-control variant: bit 0 sign handling, bit 1 vertical prediction */
        auto flush = [&]() {
            if (L->nframes > 1) P->add(op == 0 ? OP_RC : OP_PACK, 0, chain, L->nblocks, cap, signs, L, sizeof(*L));
            else if (L->nframes)
                P->add(op == 0 ? OP_RC1 : OP_PACK1, 0, chain, L->nblocks, cap, signs, &L->job[0], sizeof(L->job[0]));
            memset(L, 0, sizeof(*L));
            cap = 0;
            signs = 0;
        };
        for (int f : fr) {
            const EncItem& e = it[f];
            if (L->nframes == JXS_BATCH_FRAMES) flush();
            EncPrecFrame& F = L->job[L->nframes++];
            F.cfg = e.dcfg;
            F.coef = (const uint16_t*)e.w->fb.coef;
            F.gcli = e.w->fb.gcli;
            F.cost = e.w->cost;
            F.slice_done = e.w->slice_done;
            F.rc = e.w->rc;
            F.out = e.out;
            F.status = e.status;
            F.first_block = L->nblocks;
            L->nblocks += (int)e.c->np;
            cap = std::max(cap, e.cap_words);
            signs |= (e.c->fs ? 1u : 0u) | (e.c->vpred ? 2u : 0u);
        }
        flush();
    }
    return JXS_OK;
}

static int32_t plan_decode_chain(const std::vector<DecItem>& it, const std::vector<int>& fr, const Tune& t, int chain, Plan* P) {
    std::vector<uint8_t> scratch(std::max({sizeof(InvVLaunchB), sizeof(InvHLaunchB), sizeof(DecPrecLaunch)}));
    /* precinct walk of device codestreams, then unpacking */
    for (int op = 0; op < 2; op++) {
        DecPrecLaunch* L = (DecPrecLaunch*)scratch.data();
        memset(L, 0, sizeof(*L));
        uint32_t cb = 0, cg = 0, cs = 0;
        auto flush = [&]() {
            if (L->nframes) {
                if (op == 0) {
                    if (L->nframes > 1) P->add(OP_WALK, 0, chain, L->nslices, 0, 0, L, sizeof(*L));
                    else P->add(OP_WALK1, 0, chain, L->nslices, 0, 0, &L->job[0], sizeof(L->job[0]));
                } else {
                    /* one shared-memory layout for the launch: the largest
                     * precinct buffer that leaves room for the rest */
                    const size_t fixed = uk_layout(0, cg, cs).end;
                    const size_t room = kSmemMax - UK_STATIC_SMEM;
                    if (cb + fixed > room) cb = room > fixed + 4096 ? (uint32_t)(room - fixed) : 4096;
                    /* the launch's segment capacity travels as the op's kind */
                    if (L->nframes > 1) P->add(OP_UNPACK, (int)cs, chain, L->nblocks, cb & ~15u, cg, L, sizeof(*L));
                    else P->add(OP_UNPACK1, (int)cs, chain, L->nblocks, cb & ~15u, cg, &L->job[0], sizeof(L->job[0]));
                }
            }
            memset(L, 0, sizeof(*L));
            cb = cg = 0;
        };
        for (int f : fr) {
            const DecItem& d = it[f];
            if (op == 0 && !d.walk) continue;
            if (L->nframes == JXS_BATCH_FRAMES) flush();
            DecPrecFrame& F = L->job[L->nframes++];
            F.cfg = d.dcfg;
            F.bs = d.bs;
            F.bs_size = d.size;
            F.prec_off = d.w->prec_off;
            F.coef = (int16_t*)d.w->fb.coef;
            F.status = d.status;
            F.first_block = L->nblocks;
            F.first_slice = L->nslices;
            L->nblocks += (int)d.c->nprec;
            L->nslices += (int)d.c->nslices;
            cb = std::max(cb, d.cap_bytes);
            cg = std::max(cg, d.cap_groups);
            cs = std::max(cs, d.cap_seg);
        }
        flush();
    }
    /* horizontal-only levels: pass 0 into int32 low bands, pass 1 straight
     * to the samples (u8, then u16 planes) */
    for (int pass = 0; pass < 2; pass++) {
        for (int ok = (pass == 0 ? 0 : 1); ok <= (pass == 0 ? 0 : 2); ok++) {
            InvHLaunchB* L = (InvHLaunchB*)scratch.data();
            memset(L, 0, sizeof(*L));
            int32_t err = JXS_OK;
            auto flush = [&]() {
                if (L->njobs) {
                    const int blocks = inv_h_layout(*L, t.ih_rpb);
                    if (blocks < 0) err = JXS_E_BAD_PARAM;
                    else if (L->njobs > JXS_MAXC) P->add(OP_INV_H, ok, chain, blocks, 0, 0, L, sizeof(*L));
                    else {
                        InvHLaunch sm;
                        shrink(&sm, L);
                        P->add(OP_INV_H_S, ok, chain, blocks, 0, 0, &sm, sizeof(sm));
                    }
                }
                memset(L, 0, sizeof(*L));
            };
            InvHJob hj[JXS_MAXC];
            for (int f : fr) {
                const DecItem& d = it[f];
                if (pass == 1 && dec_sample_kind(d.c) != ok) continue;
                const int nj = plan_inv_h(d.c, d.dcfg, d.w->fb, d.out, pass, hj);
                for (int j = 0; j < nj; j++) {
                    if (L->njobs == JXS_BATCH_JOBS) flush();
                    L->job[L->njobs++] = hj[j];
                }
            }
            flush();
            if (err) return err;
        }
    }
    /* vertical levels from the deepest up; the output level (0, or the proxy
     * level) writes the samples */
    for (int v = 1; v >= 0; v--) {
        for (int ok = 0; ok <= 2; ok++) {
            InvVLaunchB* L = (InvVLaunchB*)scratch.data();
            memset(L, 0, sizeof(*L));
            int blocks = 0;
            auto flush = [&]() {
                if (L->njobs > JXS_MAXC) {
                    P->add(OP_INV_V, ok, chain, blocks, 0, 0, L, sizeof(*L));
                } else if (L->njobs) {
                    InvVLaunch sm;
                    shrink(&sm, L);
                    P->add(OP_INV_V_S, ok, chain, blocks, 0, 0, &sm, sizeof(sm));
                }
                memset(L, 0, sizeof(*L));
                blocks = 0;
            };
            InvVJob vj[JXS_MAXC];
            int tiles[JXS_MAXC];
            for (int f : fr) {
                const DecItem& d = it[f];
                if ((v > (int)d.c->proxy ? 0 : dec_sample_kind(d.c)) != ok) continue;
                const int nj = plan_inv_v(d.c, d.dcfg, d.w->fb, d.out, v, vj, tiles);
                for (int j = 0; j < nj; j++) {
                    if (L->njobs == JXS_BATCH_JOBS) flush();
                    vj[j].first_block = blocks;
                    L->job[L->njobs++] = vj[j];
                    blocks += tiles[j];
                }
            }
            flush();
        }
    }
    return JXS_OK;
}

/* ------------------------------------------------------------------------ */
/* issuing a plan: directly, or through a cached CUDA graph                  */
/* ------------------------------------------------------------------------ */
static int32_t issue(jxs_gpu_batch_t* b, const Plan& P, cudaStream_t st) {
    BCK(cudaMemsetAsync(b->status_d, 0, 2 * (size_t)P.nframes * sizeof(int), st));
    if (P.nchains > 1) {
        BCK(cudaEventRecord(b->fork, st));
        for (int c = 1; c < P.nchains; c++) BCK(cudaStreamWaitEvent(b->side[c], b->fork, 0));
    }
    if (b->stage_timing) {
        const size_t need = 2 * P.ops.size();
        while (b->tev.size() < need) {
            cudaEvent_t ev;
            BCK(cudaEventCreate(&ev));
            b->tev.push_back(ev);
        }
        b->tstage.assign(P.ops.size(), 0);
        b->tvar.assign(P.ops.size(), 0);
        b->tcount = 0;
    }
    for (const Op& o : P.ops) {
        const cudaStream_t s = o.chain == 0 ? st : b->side[o.chain];
        const void* d = P.bytes.data() + o.off;
        cudaError_t e = cudaSuccess;
        const uint32_t ti = b->tcount;
        if (b->stage_timing) BCK(cudaEventRecord(b->tev[2 * ti], s));
        switch (o.type) {
        case OP_FWD_V: e = jxs_launch_fwd_v_batch((const FwdVLaunchB*)d, o.kind, (int)o.a, s); break;
        case OP_FWD_H: e = jxs_launch_fwd_h_batch((const FwdHLaunchB*)d, o.kind, o.nblocks, s); break;
        case OP_RC: e = jxs_launch_rc_batch((const EncPrecLaunch*)d, (int)o.b, s); break;
        case OP_PACK: e = jxs_launch_pack_batch((const EncPrecLaunch*)d, o.a, (int)o.b, s); break;
        case OP_WALK: e = jxs_launch_walk_batch((const DecPrecLaunch*)d, s); break;
        case OP_UNPACK: e = jxs_launch_unpack_batch((const DecPrecLaunch*)d, o.a, o.b, (uint32_t)o.kind, s); break;
        case OP_INV_H: e = jxs_launch_inv_h_batch((const InvHLaunchB*)d, o.kind, o.nblocks, s); break;
        case OP_INV_V: e = jxs_launch_inv_v_batch((const InvVLaunchB*)d, o.kind, o.nblocks, s); break;
        case OP_FWD_V_S: e = jxs_launch_fwd_v((const FwdVLaunch*)d, o.kind, (int)o.a, s); break;
        case OP_FWD_H_S: e = jxs_launch_fwd_h((const FwdHLaunch*)d, o.kind, o.nblocks, s); break;
        case OP_INV_H_S: e = jxs_launch_inv_h((const InvHLaunch*)d, o.kind, o.nblocks, s); break;
        case OP_INV_V_S: e = jxs_launch_inv_v((const InvVLaunch*)d, o.kind, o.nblocks, s); break;
        case OP_RC1: {
            const EncPrecFrame* F = (const EncPrecFrame*)d;
            e = jxs_launch_rc(F->cfg, (uint32_t)o.nblocks, 0, F->gcli, F->coef, F->cost, F->slice_done, F->rc, F->status, (int)o.b,
                              s);
            break;
        }
        case OP_PACK1: {
            const EncPrecFrame* F = (const EncPrecFrame*)d;
            e = jxs_launch_pack(F->cfg, (uint32_t)o.nblocks, F->coef, F->gcli, F->rc, F->cost, F->out, o.a, F->status, (int)o.b, s);
            break;
        }
        case OP_WALK1: {
            const DecPrecFrame* F = (const DecPrecFrame*)d;
            e = jxs_launch_walk(F->cfg, (uint32_t)o.nblocks, F->bs, F->bs_size, F->prec_off, F->status + 1, F->status, s);
            break;
        }
        case OP_UNPACK1: {
            const DecPrecFrame* F = (const DecPrecFrame*)d;
            e = jxs_launch_unpack(F->cfg, F->bs, F->bs_size, F->prec_off, F->coef, (uint32_t)o.nblocks, o.a, o.b, (uint32_t)o.kind,
                                  F->status, s);
            break;
        }
        }
        BCK(e);
        if (b->stage_timing) {
            BCK(cudaEventRecord(b->tev[2 * ti + 1], s));
            /* the stage of each launch: the per-frame and the batched forms of
             * a kernel report the same stage */
            static const int kStage[] = {JXS_STAGE_FWD_V, JXS_STAGE_FWD_H, JXS_STAGE_RC,    JXS_STAGE_PACK,
                                         JXS_STAGE_WALK,  JXS_STAGE_UNPACK, JXS_STAGE_INV_H, JXS_STAGE_INV_V,
                                         JXS_STAGE_FWD_V, JXS_STAGE_FWD_H, JXS_STAGE_INV_H, JXS_STAGE_INV_V,
                                         JXS_STAGE_RC,    JXS_STAGE_PACK,  JXS_STAGE_WALK,  JXS_STAGE_UNPACK};
            b->tstage[ti] = kStage[o.type];
            /* transforms: the sample kind read or written (0: the 32-bit low
             * band of the next level); rate control and packing: bit 0 sign
             * handling, bit 1 vertical prediction */
            const int st = kStage[o.type];
            b->tvar[ti] = st == JXS_STAGE_RC || st == JXS_STAGE_PACK ? (int)o.b
                          : st == JXS_STAGE_WALK || st == JXS_STAGE_UNPACK ? 0 : o.kind;
            b->tcount = ti + 1;
        }
    }
    if (P.nchains > 1) {
        for (int c = 1; c < P.nchains; c++) {
            BCK(cudaEventRecord(b->join[c], b->side[c]));
            BCK(cudaStreamWaitEvent(st, b->join[c], 0));
        }
    }
    return JXS_OK;
}

static void plan_key(const Plan& P, std::vector<uint8_t>* key) {
    key->clear();
    const size_t no = P.ops.size() * sizeof(Op);
    key->resize(16 + no + P.bytes.size());
    const uint64_t hdr[2] = {(uint64_t)P.nchains, (uint64_t)P.nframes};
    memcpy(key->data(), hdr, 16);
    if (no) memcpy(key->data() + 16, P.ops.data(), no);
    if (!P.bytes.empty()) memcpy(key->data() + 16 + no, P.bytes.data(), P.bytes.size());
}

static int32_t run_plan(jxs_gpu_batch_t* b, const Plan& P, cudaStream_t st) {
    b->last_launches = (uint32_t)P.ops.size();
    if (!b->use_graph || b->stage_timing) return issue(b, P, st);
    std::vector<uint8_t> key;
    plan_key(P, &key);
    b->clock++;
    for (int i = 0; i < GRAPH_CACHE; i++) {
        GraphEntry& g = b->cache[i];
        if (g.exec && g.key == key) {
            g.last = b->clock;
            b->graph_hits++;
            BCK(cudaGraphLaunch(g.exec, st));
            return JXS_OK;
        }
    }
    /* capture the launches, then update the least recently used entry in
     * place (same topology) or instantiate a new executable graph */
    cudaGraph_t graph = nullptr;
    BCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int32_t r = issue(b, P, st);
    const cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (r != JXS_OK || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return r != JXS_OK ? r : JXS_E_RESOURCES;
    }
    int v = 0;
    for (int i = 1; i < GRAPH_CACHE; i++)
        if (b->cache[i].last < b->cache[v].last) v = i;
    GraphEntry& g = b->cache[v];
    int updated = 0;
    if (g.exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(g.exec, graph, &info) == cudaSuccess) {
            updated = 1;
        } else {
            cudaGetLastError();
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    }
    if (!updated) {
        if (cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphDestroy(graph);
            g.exec = nullptr;
            return JXS_E_RESOURCES;
        }
        b->graph_builds++;
    } else {
        b->graph_updates++;
    }
    cudaGraphDestroy(graph);
    g.key.swap(key);
    g.last = b->clock;
    BCK(cudaGraphLaunch(g.exec, st));
    return JXS_OK;
}

/* Times a plan: one run to build its graph, then `reps` timed runs. */
static float time_plan(jxs_gpu_batch_t* b, const Plan& P, cudaStream_t st, int reps) {
    if (run_plan(b, P, st) != JXS_OK) return -1.f;
    if (cudaEventRecord(b->t0, st) != cudaSuccess) return -1.f;
    for (int i = 0; i < reps; i++)
        if (run_plan(b, P, st) != JXS_OK) return -1.f;
    float ms = -1.f;
    if (cudaEventRecord(b->t1, st) != cudaSuccess || cudaEventSynchronize(b->t1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, b->t0, b->t1) != cudaSuccess) {
        cudaGetLastError();
        return -1.f;
    }
    return ms / (float)reps;
}

/* Coordinate search over the launch shapes; `build` makes the plan of a
 * candidate.  Candidates differ only in grids, block sizes and the grouping
 * of frames, never in what is computed. */
template <class BUILD>
static Tune batch_autotune(jxs_gpu_batch_t* b, uint32_t n, cudaStream_t st, BUILD build) {
    Tune best = kDefaultTune;
    Plan P;
    if (build(best, &P) != JXS_OK) return best;
    float best_ms = time_plan(b, P, st, 3);
    if (best_ms < 0) return best;
    auto consider = [&](Tune t) {
        if (build(t, &P) != JXS_OK) return;
        const float ms = time_plan(b, P, st, 3);
        if (ms > 0 && ms < best_ms * 0.98f) {
            best_ms = ms;
            best = t;
        }
    };
    for (int c = 2; c <= MAX_CHAINS && c <= (int)n; c++) {
        Tune t = best;
        t.chains = c;
        consider(t);
    }
    {
        Tune t = best;
        t.heavy_first = !t.heavy_first;
        consider(t);
    }
    const int grids[3] = {2, 3, 4};
    for (int g : grids) {
        Tune t = best;
        t.grid_per_sm = g;
        consider(t);
    }
    const int rpbs[2] = {1, 2};
    for (int r : rpbs) {
        Tune t = best;
        t.fh_rpb = r;
        consider(t);
    }
    for (int r : rpbs) {
        Tune t = best;
        t.ih_rpb = r;
        consider(t);
    }
    return best;
}

/* ------------------------------------------------------------------------ */
/* batch object                                                              */
/* ------------------------------------------------------------------------ */
extern "C" jxs_gpu_batch_t* jxs_gpu_batch_create(uint64_t device_bytes, jxs_arena_t* shared, int32_t* err) {
    *err = JXS_OK;
    if (jxs_gpu_device_count() == 0) {
        fprintf(stderr, "jxs: no CUDA device available; this library has no CPU fallback\n");
        *err = JXS_E_RESOURCES;
        return nullptr;
    }
    jxs_gpu_batch_t* b = new jxs_gpu_batch_t();
    b->arena = shared;
    if (!b->arena) {
        b->arena = jxs_arena_create(device_bytes);
        b->own_arena = 1;
    }
    bool ok = b->arena != nullptr;
    ok = ok && cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) == cudaSuccess;
    for (int c = 0; c < MAX_CHAINS && ok; c++) {
        ok = cudaStreamCreateWithFlags(&b->side[c], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->join[c], cudaEventDisableTiming) == cudaSuccess;
    }
    ok = ok && cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreate(&b->t0) == cudaSuccess && cudaEventCreate(&b->t1) == cudaSuccess;
    ok = ok && cudaMalloc(&b->status_d, 2 * JXS_BATCH_FRAMES * sizeof(int)) == cudaSuccess;
    ok = ok && cudaMallocHost(&b->status_h, 2 * JXS_BATCH_FRAMES * sizeof(int)) == cudaSuccess;
    ok = ok && cudaMallocHost(&b->hdr_pool, (size_t)JXS_BATCH_FRAMES * sizeof(((jxs_cfg_t*)0)->hdr)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        jxs_gpu_batch_destroy(b);
        *err = JXS_E_RESOURCES;
        return nullptr;
    }
    return b;
}

static void release_idle(jxs_gpu_batch_t* b);

static void release_enc(jxs_gpu_batch_t* b, EncWork* w) {
    if (w->mem) jxs_arena_free(b->arena, w->mem, w->bytes);
    w->mem = nullptr;
    w->serial = 0;
}
static void release_dec(jxs_gpu_batch_t* b, DecWork* w) {
    if (w->mem) jxs_arena_free(b->arena, w->mem, w->bytes);
    w->mem = nullptr;
    w->serial = 0;
    if (w->prec_off_h) cudaFreeHost(w->prec_off_h);
    w->prec_off_h = nullptr;
    w->hdr_h = nullptr;
    w->prec_cap = 0;
}

extern "C" void jxs_gpu_batch_destroy(jxs_gpu_batch_t* b) {
    if (!b) return;
    if (b->st) cudaStreamSynchronize(b->st);
    for (EncWork& w : b->enc) release_enc(b, &w);
    for (DecWork& w : b->dec) release_dec(b, &w);
    release_idle(b);
    for (GraphEntry& g : b->cache)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (int c = 0; c < MAX_CHAINS; c++) {
        if (b->side[c]) cudaStreamDestroy(b->side[c]);
        if (b->join[c]) cudaEventDestroy(b->join[c]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->done) cudaEventDestroy(b->done);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    for (cudaEvent_t ev : b->tev) cudaEventDestroy(ev);
    cudaFree(b->status_d);
    if (b->status_h) cudaFreeHost(b->status_h);
    if (b->hdr_pool) cudaFreeHost(b->hdr_pool);
    if (b->st) cudaStreamDestroy(b->st);
    if (b->own_arena) jxs_arena_destroy(b->arena);
    delete b;
}

extern "C" void jxs_gpu_batch_set_options(jxs_gpu_batch_t* b, int use_graph, int autotune) {
    b->use_graph = use_graph;
    b->autotune = autotune;
}

extern "C" void jxs_gpu_batch_set_release(jxs_gpu_batch_t* b, int on) { b->release_after_wait = on; }

extern "C" void jxs_gpu_batch_set_stage_timing(jxs_gpu_batch_t* b, int on) {
    b->stage_timing = on;
    b->tcount = 0;
}

extern "C" uint32_t jxs_gpu_batch_stage_times(jxs_gpu_batch_t* b, int32_t* stage, int32_t* variant, float* ms, uint32_t max) {
    if (b->pending) return 0;
    uint32_t n = 0;
    for (uint32_t i = 0; i < b->tcount && n < max; i++) {
        float t = -1.f;
        if (cudaEventElapsedTime(&t, b->tev[2 * i], b->tev[2 * i + 1]) != cudaSuccess) {
            cudaGetLastError();
            t = -1.f;
        }
        if (stage) stage[n] = b->tstage[i];
        if (variant) variant[n] = b->tvar[i];
        if (ms) ms[n] = t;
        n++;
    }
    return n;
}

static void release_all(jxs_gpu_batch_t* b);

extern "C" int jxs_gpu_batch_release(jxs_gpu_batch_t* b) {
    if (!b || b->pending) return 0;
    release_all(b);
    return 1;
}

extern "C" uint64_t jxs_gpu_batch_enc_work_bytes(jxs_gpu_enc_t* e) {
    EncWork w;
    const jxs_cfg_t* c = jxs_gpu_enc_info(e, nullptr, nullptr);
    return c ? round256(enc_work_layout(c, nullptr, &w)) : 0;
}

extern "C" uint64_t jxs_gpu_batch_dec_work_bytes(jxs_gpu_dec_t* d) {
    DecWork w;
    const jxs_cfg_t* c = jxs_gpu_dec_info(d, nullptr, nullptr, nullptr, nullptr);
    return c ? round256(dec_work_layout(c, nullptr, &w)) : 0;
}

/* Lays out the working sets of positions 0..n-1 for the given handles
 * (exactly one of enc / dec non-NULL); returns how many leading positions
 * now hold one.  Stops at the first that does not fit in the arena. */
static int32_t ensure_enc(jxs_gpu_batch_t* b, uint32_t i, jxs_gpu_enc_t* e, cudaStream_t st);
static int32_t ensure_dec(jxs_gpu_batch_t* b, uint32_t i, jxs_gpu_dec_t* d, cudaStream_t st);

extern "C" uint32_t jxs_gpu_batch_reserve(jxs_gpu_batch_t* b, jxs_gpu_enc_t* const* enc, jxs_gpu_dec_t* const* dec, uint32_t n,
                                          void* stream) {
    if (!b || b->pending || n > JXS_BATCH_FRAMES) return 0;
    /* the stream the batch will run on: a new position's counters are reset
     * there, ahead of its kernels */
    const cudaStream_t st = stream ? (cudaStream_t)stream : b->st;
    uint32_t k = 0;
    for (; k < n; k++) {
        const int32_t r = enc ? ensure_enc(b, k, enc[k], st) : ensure_dec(b, k, dec[k], st);
        if (r != JXS_OK) break;
    }
    return k;
}

static void release_idle(jxs_gpu_batch_t* b) {
    for (const auto& x : b->idle) jxs_arena_free(b->arena, x.mem, x.bytes);
    b->idle.clear();
}

static void release_all(jxs_gpu_batch_t* b) {
    for (EncWork& w : b->enc) {
        if (w.mem) jxs_arena_free(b->arena, w.mem, w.bytes);
        w.mem = nullptr;
        w.serial = 0;
    }
    for (DecWork& w : b->dec) {
        if (w.mem) jxs_arena_free(b->arena, w.mem, w.bytes);
        w.mem = nullptr;
        w.serial = 0;
    }
    release_idle(b);
}

/* A working set for a position that needs `serial`'s layout: an idle one of
 * that layout, else a new one from the arena (idle sets of other layouts are
 * freed first when the arena is short).  No batch of this object is in flight
 * when positions change, so no set handed over here is still being read. */
static uint8_t* take_set(jxs_gpu_batch_t* b, int kind, uint64_t serial, uint64_t bytes, int* fresh) {
    *fresh = 0;
    for (size_t k = 0; k < b->idle.size(); k++) {
        if (b->idle[k].kind == kind && b->idle[k].serial == serial) {
            uint8_t* m = b->idle[k].mem;
            b->idle.erase(b->idle.begin() + (long)k);
            return m;
        }
    }
    uint8_t* m = (uint8_t*)jxs_arena_alloc(b->arena, bytes);
    if (!m && !b->idle.empty()) {
        release_idle(b);
        m = (uint8_t*)jxs_arena_alloc(b->arena, bytes);
    }
    *fresh = m != nullptr;
    return m;
}

extern "C" void jxs_gpu_batch_set_tune(jxs_gpu_batch_t* b, const int* t5) {
    /* fixes the launch shapes of every signature (autotune results dropped) */
    Tune t = {std::max(1, std::min(t5[0], MAX_CHAINS)), t5[1] != 0, std::max(0, t5[2]), std::max(1, std::min(t5[3], 4)),
              std::max(1, std::min(t5[4], 4))};
    b->tuned.clear();
    b->tuned[""] = t;
}

static Tune tune_for(jxs_gpu_batch_t* b, const std::string& sig, int* found) {
    auto it = b->tuned.find(sig);
    if (it != b->tuned.end()) {
        *found = 1;
        return it->second;
    }
    it = b->tuned.find("");
    *found = it != b->tuned.end();
    return *found ? it->second : kDefaultTune;
}

/* ------------------------------------------------------------------------ */
/* working sets of the positions                                             */
/* ------------------------------------------------------------------------ */
static int32_t ensure_enc(jxs_gpu_batch_t* b, uint32_t i, jxs_gpu_enc_t* e, cudaStream_t st) {
    if (b->enc.size() <= i) b->enc.resize(i + 1);
    const jxs_cfg_t* c = jxs_gpu_enc_info(e, nullptr, nullptr);
    if (!c) return JXS_E_BAD_PARAM;
    const uint64_t serial = jxs_gpu_enc_serial(e);
    EncWork& w = b->enc[i];
    if (w.serial == serial && w.mem) return JXS_OK;
    if (w.mem) b->idle.push_back({0, w.serial, w.mem, w.bytes});
    w.mem = nullptr;
    w.serial = 0;
    w.bytes = enc_work_layout(c, nullptr, &w);
    int fresh = 0;
    w.mem = take_set(b, 0, serial, w.bytes, &fresh);
    if (!w.mem) {
        w.bytes = 0;
        return JXS_E_RESOURCES;
    }
    enc_work_layout(c, w.mem, &w);
    /* a new set's slice counters start at zero; a reused one's were reset by
     * the kernels of its last frame */
    if (fresh) BCK(cudaMemsetAsync(w.slice_done, 0, (size_t)c->nslices * sizeof(uint32_t), st));
    w.serial = serial;
    return JXS_OK;
}

static int32_t ensure_dec(jxs_gpu_batch_t* b, uint32_t i, jxs_gpu_dec_t* d, cudaStream_t st) {
    if (b->dec.size() <= i) b->dec.resize(i + 1);
    const jxs_cfg_t* c = jxs_gpu_dec_info(d, nullptr, nullptr, nullptr, nullptr);
    if (!c) return JXS_E_DEC_PTR;
    const uint64_t serial = jxs_gpu_dec_serial(d);
    DecWork& w = b->dec[i];
    if (w.serial == serial && w.mem) return JXS_OK;
    (void)st;
    if (w.mem) b->idle.push_back({1, w.serial, w.mem, w.bytes});
    w.mem = nullptr;
    w.serial = 0;
    w.bytes = dec_work_layout(c, nullptr, &w);
    int fresh = 0;
    w.mem = take_set(b, 1, serial, w.bytes, &fresh);
    if (!w.mem) {
        w.bytes = 0;
        return JXS_E_RESOURCES;
    }
    dec_work_layout(c, w.mem, &w);
    w.serial = serial;
    return JXS_OK;
}

/* ------------------------------------------------------------------------ */
/* encode                                                                    */
/* ------------------------------------------------------------------------ */
extern "C" int32_t jxs_gpu_batch_encode(jxs_gpu_batch_t* b, jxs_gpu_enc_t* const* enc, uint32_t n, void* const (*planes)[4],
                                        const uint32_t (*strides)[4], uint8_t* const* out, void* stream) {
    if (!b || !enc || !planes || !strides || !out || n == 0 || n > JXS_BATCH_FRAMES) return JXS_E_BAD_PARAM;
    if (b->pending) return JXS_E_BAD_PARAM;
    const cudaStream_t st = stream ? (cudaStream_t)stream : b->st;
    if (b->enc.size() < n) b->enc.resize(n);
    std::vector<EncItem> items(n);
    std::vector<uint64_t> weight(n);
    std::string sig = "E";
    b->cfgs.assign(n, nullptr);
    for (uint32_t i = 0; i < n; i++) {
        const jxs_cfg_t* dcfg = nullptr;
        const jxs_cfg_t* c = jxs_gpu_enc_info(enc[i], &dcfg, &items[i].cap_words);
        if (!c) return JXS_E_BAD_PARAM;
        const uint64_t serial = jxs_gpu_enc_serial(enc[i]);
        const int32_t er = ensure_enc(b, i, enc[i], st);
        if (er != JXS_OK) {
            if (er == JXS_E_RESOURCES)
                fprintf(stderr, "jxs batch: frame %u does not fit in the batch's device budget\n", i);
            return er;
        }
        EncWork& w = b->enc[i];
        EncItem& e = items[i];
        e.c = c;
        e.dcfg = dcfg;
        e.w = &w;
        e.status = b->status_d + 2 * i;
        /* sources: device planes in place, host planes staged */
        const int packed = c->fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB;
        const uint32_t bps = bytes_per_sample(c);
        memset(&e.in, 0, sizeof(e.in));
        for (int k = 0; k < (packed ? 1 : (int)c->nc); k++) {
            const uint32_t pw = packed ? c->W * 3 : c->comp[k].w, ph = packed ? c->H : c->comp[k].h;
            if (jxs_gpu_is_device_ptr(planes[i][k])) {
                e.in.p[k] = planes[i][k];
                e.in.pitch[k] = strides[i][k];
            } else {
                uint8_t* d = w.in_stage + w.in_off[k];
                const uint32_t sp = packed ? pw : stage_pitch(pw, bps);
                BCK(cudaMemcpy2DAsync(d, (size_t)sp * bps, planes[i][k], (size_t)strides[i][k] * bps, (size_t)pw * bps, ph,
                                      cudaMemcpyHostToDevice, st));
                e.in.p[k] = d;
                e.in.pitch[k] = sp;
            }
        }
        e.out = jxs_gpu_is_device_ptr(out[i]) ? out[i] : w.out_stage;
        weight[i] = c->coef_total;
        b->cfgs[i] = c;
        sig += std::to_string(serial) + ",";
    }
    auto build = [&](const Tune& t, Plan* P) -> int32_t {
        P->clear();
        std::vector<std::vector<int>> chains;
        order_chains(weight, t, &chains);
        P->nchains = (int)chains.size();
        P->nframes = n;
        for (int c = 0; c < P->nchains; c++) {
            const int32_t r = plan_encode_chain(items, chains[c], t, c, P);
            if (r) return r;
        }
        return JXS_OK;
    };
    int found = 0;
    Tune t = tune_for(b, sig, &found);
    if (!found && b->autotune) {
        t = batch_autotune(b, n, st, build);
        b->tuned[sig] = t;
    }
    b->last_tune = t;
    Plan P;
    int32_t r = build(t, &P);
    if (r) return r;
    BCK(cudaEventRecord(b->t0, st));
    r = run_plan(b, P, st);
    if (r) return r;
    BCK(cudaEventRecord(b->t1, st));
    for (uint32_t i = 0; i < n; i++)
        if (items[i].out != out[i]) BCK(cudaMemcpyAsync(out[i], items[i].out, items[i].c->lcod, cudaMemcpyDeviceToHost, st));
    BCK(cudaMemcpyAsync(b->status_h, b->status_d, 2 * (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st));
    BCK(cudaEventRecord(b->done, st));
    b->hdr_check.assign(n, 0);
    b->pending = 1;
    b->kind = 0;
    b->n = n;
    return JXS_OK;
}

/* ------------------------------------------------------------------------ */
/* decode                                                                    */
/* ------------------------------------------------------------------------ */
extern "C" uint32_t* jxs_gpu_batch_prec_buffer(jxs_gpu_batch_t* b, uint32_t i, uint32_t np) {
    /* not while a batch is in flight: its offsets may still be on their way
     * to the device */
    if (!b || i >= JXS_BATCH_FRAMES || b->pending) return nullptr;
    if (b->dec.size() <= i) b->dec.resize(i + 1);
    DecWork& w = b->dec[i];
    if (w.prec_cap < np) {
        if (w.prec_off_h) cudaFreeHost(w.prec_off_h);
        w.prec_off_h = nullptr;
        w.prec_cap = 0;
        if (cudaMallocHost(&w.prec_off_h, (size_t)np * sizeof(uint32_t)) != cudaSuccess) {
            cudaGetLastError();
            w.prec_off_h = nullptr;
            return nullptr;
        }
        w.prec_cap = np;
    }
    return w.prec_off_h;
}

extern "C" int32_t jxs_gpu_batch_decode(jxs_gpu_batch_t* b, jxs_gpu_dec_t* const* dec, uint32_t n, const uint8_t* const* bs,
                                        const uint32_t* size, const int* host_walked, void* const (*planes)[4],
                                        const uint32_t (*strides)[4], void* stream) {
    if (!b || !dec || !bs || !size || !planes || !strides || n == 0 || n > JXS_BATCH_FRAMES) return JXS_E_BAD_PARAM;
    if (b->pending) return JXS_E_BAD_PARAM;
    const cudaStream_t st = stream ? (cudaStream_t)stream : b->st;
    if (b->dec.size() < n) b->dec.resize(n);
    std::vector<DecItem> items(n);
    std::vector<uint64_t> weight(n);
    std::string sig = "D";
    b->hdr_check.assign(n, 0);
    b->cfgs.assign(n, nullptr);
    for (uint32_t i = 0; i < n; i++) {
        const jxs_cfg_t* dcfg = nullptr;
        uint32_t cb = 0, cg = 0, cs = 0;
        const jxs_cfg_t* c = jxs_gpu_dec_info(dec[i], &dcfg, &cb, &cg, &cs);
        if (!c || !bs[i]) return JXS_E_DEC_PTR;
        /* colour transforms and non-linear outputs decode per frame only */
        if (dec_needs_nlt_pass(c)) return JXS_E_BAD_PARAM;
        const uint64_t serial = jxs_gpu_dec_serial(dec[i]);
        const int32_t er = ensure_dec(b, i, dec[i], st);
        if (er != JXS_OK) {
            if (er == JXS_E_RESOURCES)
                fprintf(stderr, "jxs batch: frame %u does not fit in the batch's device budget\n", i);
            return er;
        }
        DecWork& w = b->dec[i];
        w.hdr_h = b->hdr_pool + (size_t)i * sizeof(c->hdr);
        DecItem& d = items[i];
        d.c = c;
        d.dcfg = dcfg;
        d.cap_bytes = cb;
        d.cap_groups = cg;
        d.cap_seg = cs;
        d.w = &w;
        d.status = b->status_d + 2 * i;
        d.size = size[i];
        const int dev = jxs_gpu_is_device_ptr(bs[i]);
        if (host_walked && host_walked[i]) {
            /* precinct offsets found on the host (jxs_frame_bytes_walk) */
            if (!w.prec_off_h || w.prec_cap < c->nprec) return JXS_E_BAD_PARAM;
            BCK(cudaMemcpyAsync(w.prec_off, w.prec_off_h, (size_t)c->nprec * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
            d.walk = 0;
        } else {
            if (!dev || size[i] < c->hdr_len) return JXS_E_DEC_PTR;
            d.walk = 1;
            BCK(cudaMemcpyAsync(w.hdr_h, bs[i], c->hdr_len, cudaMemcpyDeviceToHost, st));
            b->hdr_check[i] = 1;
        }
        if (dev) {
            d.bs = bs[i];
        } else {
            if (size[i] > w.bs_cap) {
                fprintf(stderr, "jxs batch: frame %u: codestream of %u bytes exceeds the %u-byte buffer of its position\n", i,
                        size[i], w.bs_cap);
                return JXS_E_BAD_PARAM;
            }
            BCK(cudaMemcpyAsync(w.bs, bs[i], size[i], cudaMemcpyHostToDevice, st));
            d.bs = w.bs;
        }
        memset(&d.out, 0, sizeof(d.out));
        for (uint32_t k = 0; k < c->nc; k++) {
            if (jxs_gpu_is_device_ptr(planes[i][k])) {
                d.out.p[k] = planes[i][k];
                d.out.pitch[k] = strides[i][k];
            } else {
                d.out.p[k] = w.out_stage + w.out_off[k];
                d.out.pitch[k] = stage_pitch(jxs_out_w(c, k), bytes_per_sample(c));
            }
        }
        weight[i] = c->coef_total;
        b->cfgs[i] = c;
        sig += std::to_string(serial) + (d.walk ? "w," : ",");
    }
    auto build = [&](const Tune& t, Plan* P) -> int32_t {
        P->clear();
        std::vector<std::vector<int>> chains;
        order_chains(weight, t, &chains);
        P->nchains = (int)chains.size();
        P->nframes = n;
        for (int c = 0; c < P->nchains; c++) {
            const int32_t r = plan_decode_chain(items, chains[c], t, c, P);
            if (r) return r;
        }
        return JXS_OK;
    };
    int found = 0;
    Tune t = tune_for(b, sig, &found);
    if (!found && b->autotune) {
        t = batch_autotune(b, n, st, build);
        b->tuned[sig] = t;
    }
    b->last_tune = t;
    Plan P;
    int32_t r = build(t, &P);
    if (r) return r;
    BCK(cudaEventRecord(b->t0, st));
    r = run_plan(b, P, st);
    if (r) return r;
    BCK(cudaEventRecord(b->t1, st));
    for (uint32_t i = 0; i < n; i++) {
        const DecItem& d = items[i];
        const uint32_t bps = bytes_per_sample(d.c);
        for (uint32_t k = 0; k < d.c->nc; k++) {
            if (d.out.p[k] == planes[i][k]) continue;
            const uint32_t ow = jxs_out_w(d.c, k), oh = jxs_out_h(d.c, k);
            BCK(cudaMemcpy2DAsync(planes[i][k], (size_t)strides[i][k] * bps, d.out.p[k], (size_t)d.out.pitch[k] * bps, (size_t)ow * bps,
                                  oh, cudaMemcpyDeviceToHost, st));
        }
    }
    BCK(cudaMemcpyAsync(b->status_h, b->status_d, 2 * (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st));
    BCK(cudaEventRecord(b->done, st));
    b->pending = 1;
    b->kind = 1;
    b->n = n;
    return JXS_OK;
}

/* ------------------------------------------------------------------------ */
/* completion                                                                */
/* ------------------------------------------------------------------------ */
extern "C" int jxs_gpu_batch_ready(jxs_gpu_batch_t* b) {
    if (!b->pending) return 1;
    return cudaEventQuery(b->done) == cudaErrorNotReady ? 0 : 1;
}

extern "C" int32_t jxs_gpu_batch_wait(jxs_gpu_batch_t* b, int32_t* status) {
    if (!b || !b->pending) return JXS_E_BAD_PARAM;
    b->pending = 0;
    if (cudaEventSynchronize(b->done) != cudaSuccess) {
        fprintf(stderr, "jxs batch: %s\n", cudaGetErrorString(cudaGetLastError()));
        for (uint32_t i = 0; i < b->n; i++)
            if (status) status[i] = b->kind ? JXS_E_DEC_INTERNAL : JXS_E_ENC_FRAME;
        if (b->release_after_wait) release_all(b);
        return JXS_E_RESOURCES;
    }
    if (cudaEventElapsedTime(&b->last_ms, b->t0, b->t1) != cudaSuccess) {
        cudaGetLastError();
        b->last_ms = 0.f;
    }
    int32_t worst = JXS_OK;
    for (uint32_t i = 0; i < b->n; i++) {
        int32_t s = b->status_h[2 * i];
        /* vertical prediction needs slice-ordered decoding, which the batched
         * form does not run: decode such frames with send_frame */
        if (s == JXS_E_DEC_VPRED) s = JXS_E_DEC_BITSTREAM;
        if (b->kind == 0) {
            s = s ? JXS_E_ENC_FRAME : JXS_OK;
        } else if (b->hdr_check[i] && s == JXS_OK) {
            /* every header byte but Lcod (12..15) must match the stream's */
            const jxs_cfg_t* c = b->cfgs[i];
            const uint8_t* h = b->dec[i].hdr_h;
            if (memcmp(h, c->hdr, 12) != 0 || memcmp(h + 16, c->hdr + 16, c->hdr_len - 16) != 0) s = JXS_E_DEC_CONFIG;
        }
        if (status) status[i] = s;
        if (s && !worst) worst = s;
    }
    if (b->release_after_wait) release_all(b);
    return worst;
}

extern "C" void jxs_gpu_batch_info(jxs_gpu_batch_t* b, jxs_batch_info_t* o) {
    memset(o, 0, sizeof(*o));
    o->last_gpu_ms = b->last_ms;
    o->last_launches = b->last_launches;
    o->graph_hits = b->graph_hits;
    o->graph_builds = b->graph_builds;
    o->graph_updates = b->graph_updates;
    o->tune[0] = b->last_tune.chains;
    o->tune[1] = b->last_tune.heavy_first;
    o->tune[2] = b->last_tune.grid_per_sm;
    o->tune[3] = b->last_tune.fh_rpb;
    o->tune[4] = b->last_tune.ih_rpb;
    jxs_arena_stats(b->arena, &o->arena_bytes, &o->arena_used, &o->arena_peak);
}
