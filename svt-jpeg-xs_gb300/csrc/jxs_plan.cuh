/*
 * Launch planning shared by the per-frame path (jxs_gpu.cu) and the batched
 * path (jxs_batch.cu): the transform jobs of one frame, built from its
 * configuration and its device buffers.  A job is one component's share of a
 * transform launch; the per-frame path launches the jobs of one frame, the
 * batched path concatenates the jobs of many frames into one launch.
 */
#ifndef JXS_PLAN_CUH
#define JXS_PLAN_CUH

#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "SvtJpegxs.h"
#include "jxs_kernels.cuh"

/* Kernel launchers (jxs_fwd_dwt.cu, jxs_inv_dwt.cu, jxs_enc_kernels.cu,
 * jxs_dec_kernels.cu). */
extern "C" cudaError_t jxs_launch_fwd_v(const FwdVLaunch* L, int src_kind, int grid_per_sm, cudaStream_t st);
extern "C" cudaError_t jxs_launch_fwd_v_batch(const FwdVLaunchB* L, int src_kind, int grid_per_sm, cudaStream_t st);
extern "C" cudaError_t jxs_launch_fwd_h(const FwdHLaunch* L, int src_kind, int nblocks, cudaStream_t st);
extern "C" cudaError_t jxs_launch_fwd_h_batch(const FwdHLaunchB* L, int src_kind, int nblocks, cudaStream_t st);
extern "C" int jxs_fwd_v_tile_rows(void);
extern "C" int jxs_fwd_v_tile_cols(void);
extern "C" int jxs_fwd_h_max_rows_per_block(void);
extern "C" cudaError_t jxs_launch_rc(const jxs_cfg_t* dcfg, uint32_t np, uint32_t nslices, const uint8_t* gcli,
                                     const uint16_t* coef, uint32_t* cost, uint32_t* slice_done, PrecRC* rc, int* status,
                                     int modes, cudaStream_t st);
extern "C" cudaError_t jxs_launch_rc_batch(const EncPrecLaunch* L, int modes, cudaStream_t st);
extern "C" cudaError_t jxs_launch_pack(const jxs_cfg_t* dcfg, uint32_t np, const uint16_t* coef, const uint8_t* gcli,
                                       const PrecRC* rc, const uint32_t* cost, uint8_t* out, uint32_t cap_words, int* status,
                                       int modes, cudaStream_t st);
extern "C" cudaError_t jxs_launch_pack_batch(const EncPrecLaunch* L, uint32_t cap_words, int modes, cudaStream_t st);
extern "C" cudaError_t jxs_launch_unpack(const jxs_cfg_t* dcfg, const uint8_t* bs, uint32_t bs_size, const uint32_t* prec_off,
                                         int16_t* coef, uint32_t np, uint32_t cap_bytes, uint32_t cap_groups, uint32_t cap_seg,
                                         int* status, cudaStream_t st);
extern "C" cudaError_t jxs_launch_unpack_batch(const DecPrecLaunch* L, uint32_t cap_bytes, uint32_t cap_groups, uint32_t cap_seg,
                                               cudaStream_t st);
extern "C" cudaError_t jxs_launch_unpack_vpred(const jxs_cfg_t* dcfg, const uint8_t* bs, uint32_t bs_size, const uint32_t* prec_off,
                                               int16_t* coef, uint32_t nslices, uint32_t cap_bytes, uint32_t cap_groups,
                                               uint32_t cap_seg, int* status, cudaStream_t st);
extern "C" cudaError_t jxs_launch_walk(const jxs_cfg_t* dcfg, uint32_t nslices, const uint8_t* bs, uint32_t size, uint32_t* prec_off,
                                       int* walk_bad, int* status, cudaStream_t st);
extern "C" cudaError_t jxs_launch_walk_batch(const DecPrecLaunch* L, cudaStream_t st);
extern "C" cudaError_t jxs_launch_inv_v(const InvVLaunch* L, int out_kind, int nblocks, cudaStream_t st);
extern "C" cudaError_t jxs_launch_inv_v_batch(const InvVLaunchB* L, int out_kind, int nblocks, cudaStream_t st);
extern "C" cudaError_t jxs_launch_inv_h(const InvHLaunch* L, int out_kind, int nblocks, cudaStream_t st);
extern "C" cudaError_t jxs_launch_inv_h_batch(const InvHLaunchB* L, int out_kind, int nblocks, cudaStream_t st);
extern "C" cudaError_t jxs_launch_nlt_out(const NltOut* P, cudaStream_t st);
extern "C" cudaError_t jxs_launch_star_tetrix(const StParams* P, cudaStream_t st);
extern "C" int jxs_inv_v_tile_rows(void);
extern "C" int jxs_inv_v_tile_cols(void);
extern "C" int jxs_inv_h_max_rows_per_block(void);

static const size_t kSmemMax = 220 * 1024;

/* Rate-control tables of a frame: per precinct row the byte cost of every
 * (Q, R); with sign handling a second set with exact sign counts; with
 * vertical prediction the per-line tables of the ordered selection
 * (5 x 80 x 16 words per row); then the per-segment histograms the rate
 * control hands to packing (JXS_SEGHIST_WORDS per segment of every row). */
static inline size_t jxs_cost_bytes(const jxs_cfg_t* c) {
    return ((size_t)jxs_seghist_word(c) + (size_t)c->np * jxs_seg_cap(c) * JXS_SEGHIST_WORDS) * sizeof(uint32_t);
}

static inline uint32_t div_up(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

/* size of component c at vertical level v (region transformed by level v) */
static inline void level_dims(const jxs_comp_t& cp, int v, uint32_t* w, uint32_t* h) {
    uint32_t ww = cp.w, hh = cp.h;
    for (int i = 0; i < v; i++) {
        ww = (ww + 1) / 2;
        hh = (hh + 1) / 2;
    }
    *w = ww;
    *h = hh;
}

static inline uint32_t bytes_per_sample(const jxs_cfg_t* c) { return c->depth <= 8 ? 1 : 2; }

/* Row pitch (elements) of a staged input plane w elements wide: rows start
 * on 16-byte boundaries, so that the first transform level reads them with
 * vector loads. */
static inline uint32_t stage_pitch(uint32_t w, uint32_t bps) { return (uint32_t)((((uint64_t)w * bps + 15) & ~15ull) / bps); }

static inline uint32_t cfg_max_dv(const jxs_cfg_t* c) {
    uint32_t m = 0;
    for (uint32_t k = 0; k < c->nc; k++) m = c->comp[k].dv > m ? c->comp[k].dv : m;
    return m;
}

/* address of the band table inside the device copy of the configuration */
static inline const jxs_band_t* dev_bands(const jxs_cfg_t* dcfg) {
    return (const jxs_band_t*)((const char*)dcfg + offsetof(jxs_cfg_t, band));
}

/* Fills the band indices of a job for vertical level v of component c
 * (bands of level v: HH = nb-1-3v, LH = HH-1, HL = HH-2; then one high band
 * per horizontal-only level and the final low band). */
static inline void job_bands(const jxs_cfg_t* cfg, int c, int v, DwtJob* J) {
    const jxs_comp_t& cp = cfg->comp[c];
    const int b0 = cp.band0;
    if (cp.dv == 0) {
        J->last = 1;
        J->nh = cp.dh;
        for (uint32_t e = 0; e < cp.dh; e++) J->b_hf[e] = b0 + (int)cp.nb - 1 - (int)e;
        J->b_ll = b0;
        return;
    }
    const int L = (int)cp.nb - 1 - 3 * v;
    J->b_hh = b0 + L;
    J->b_lh = b0 + L - 1;
    J->b_hl = b0 + L - 2;
    J->last = (v + 1 == (int)cp.dv);
    J->nh = J->last ? (int)(cp.dh - cp.dv) : 0;
    for (int e = 0; e < J->nh; e++) J->b_hf[e] = b0 + L - 3 - e;
    J->b_ll = b0 + L - 3 - J->nh;
}

/* Sample kind of the first forward level. */
static inline int enc_level0_kind(const jxs_cfg_t* c) {
    const int packed = c->fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB;
    const uint32_t bps = bytes_per_sample(c);
    return packed ? (bps == 1 ? SRC_PK8 : SRC_PK16) : (bps == 1 ? SRC_U8 : SRC_U16);
}

/* Output kind of the last inverse level: 1 u8 plane, 2 u16 plane. */
static inline int dec_sample_kind(const jxs_cfg_t* c) { return bytes_per_sample(c) == 1 ? 1 : 2; }

/* The device planes of one frame in flight. */
struct FrameBufs {
    void* coef;                    /* encoder: u16 sign-magnitude; decoder: int16 */
    uint8_t* gcli;                 /* encoder only */
    int32_t* ll[2][JXS_MAXC];      /* int32 low band after (encoder) / below (decoder) vertical level 0 / 1 */
    int ll_pitch[2][JXS_MAXC];     /* elements, a multiple of 4 */
};

/* Planes of a frame: encoder input or decoder output, per component (packed
 * input: plane 0 only). */
struct FramePlanes {
    void* p[JXS_MAXC];
    long long pitch[JXS_MAXC];     /* elements */
};

/* Decoded frames whose last inverse level writes int32 planes for
 * nlt_out_kernel: a colour transform or a non-linear output. */
static inline int dec_needs_nlt_pass(const jxs_cfg_t* c) { return c->cpih != 0 || c->tnlt != 0; }

/* The parameters of nlt_out_kernel for a frame: int32 planes `in` (pitch
 * in elements) to the output planes `out` (NltDec.c:111-116 for the
 * extended constants). */
static inline void nlt_out_params(const jxs_cfg_t* c, const FramePlanes& in, const FramePlanes& out, NltOut* P) {
    memset(P, 0, sizeof(*P));
    P->nc = (int)c->nc;
    for (uint32_t k = 0; k < c->nc; k++) {
        P->in[k] = (const int32_t*)in.p[k];
        P->in_pitch[k] = in.pitch[k];
        P->out[k] = out.p[k];
        P->out_pitch[k] = out.pitch[k];
        P->w[k] = (int)jxs_out_w(c, k);
        P->h[k] = (int)jxs_out_h(c, k);
    }
    P->cpih = (int)c->cpih;
    P->tnlt = (int)c->tnlt;
    P->bw = (int)c->bw;
    P->depth = (int)c->depth;
    P->bps = (int)bytes_per_sample(c);
    P->dco = (int32_t)c->nlt_alpha - (int32_t)c->nlt_sigma * (1 << 15);
    const int32_t bw = (int32_t)c->bw, e = (int32_t)c->nlt_e;
    P->t1 = (int32_t)c->nlt_t1;
    P->t2 = (int32_t)c->nlt_t2;
    P->e = e;
    if (c->tnlt == 2) {
        P->b1 = (int32_t)((int64_t)P->t1 + (1 << (bw - e - 1)));
        P->b2 = (int64_t)P->t1 * P->t1;
        P->b3 = (int64_t)P->t2 - ((int64_t)1 << (bw - e - 1));
        P->a1 = P->b2 + (int64_t)P->t1 * ((int64_t)1 << (bw - e)) + ((int64_t)1 << (2 * bw - 2 - 2 * e));
        P->a3 = P->b2 + (int64_t)P->t2 * ((int64_t)1 << (bw - e)) - ((int64_t)1 << (2 * bw - 2 - 2 * e));
    }
}

/* Bytes of the int32 low bands of one frame, and their pitches. */
static inline uint64_t ll_layout(const jxs_cfg_t* c, int pitch[2][JXS_MAXC], uint64_t size[2][JXS_MAXC]) {
    uint64_t total = 0;
    for (int v = 0; v < 2; v++)
        for (int k = 0; k < JXS_MAXC; k++) {
            pitch[v][k] = 0;
            size[v][k] = 0;
        }
    for (uint32_t k = 0; k < c->nc; k++) {
        for (uint32_t v = 0; v < c->comp[k].dv && v < 2; v++) {
            uint32_t w, h;
            level_dims(c->comp[k], (int)v + 1, &w, &h);
            pitch[v][k] = (int)((w + 3) & ~3u);
            size[v][k] = (((uint64_t)pitch[v][k] * h * sizeof(int32_t) + 64) + 255) & ~255ull;
            total += size[v][k];
        }
    }
    return total;
}

/* Forward jobs of vertical level v of one frame (one per component that has
 * the level); *tiles receives each job's tile count. */
static inline int plan_fwd_v(const jxs_cfg_t* c, const jxs_cfg_t* dcfg, const FrameBufs& b, const FramePlanes& in, int v,
                             FwdVJob* jobs, int* tiles) {
    const int packed = c->fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB;
    const uint32_t bps = bytes_per_sample(c);
    const uint32_t vcols = (uint32_t)jxs_fwd_v_tile_cols(), vrows = (uint32_t)jxs_fwd_v_tile_rows();
    int n = 0;
    for (uint32_t k = 0; k < c->nc; k++) {
        const jxs_comp_t& cp = c->comp[k];
        if ((int)cp.dv <= v) continue;
        FwdVJob& J = jobs[n];
        memset(&J, 0, sizeof(J));
        uint32_t w, h;
        level_dims(cp, v, &w, &h);
        J.w = (int)w;
        J.h = (int)h;
        if (v == 0) {
            const int pk = packed ? 0 : (int)k;
            J.src = in.p[pk];
            J.src_pitch = in.pitch[pk];
            J.chan = packed ? (int)k : 0;
            /* 8 samples per vector load: 16 bytes (16-bit) or 8 bytes (8-bit) */
            J.vec = !packed && ((uintptr_t)in.p[pk] % (8 * bps)) == 0 && (in.pitch[pk] % 8) == 0;
        } else {
            J.src = b.ll[v - 1][k];
            J.src_pitch = b.ll_pitch[v - 1][k];
            J.vec = 1;
        }
        J.ll = b.ll[v][k];
        J.ll_pitch = b.ll_pitch[v][k];
        const int top = (int)cp.band0 + (int)cp.nb - 1 - 3 * v;
        J.b_hh = top;
        J.b_lh = top - 1;
        J.b_hl = top - 2;
        J.col_tiles = (int)div_up(w, vcols);
        J.depth = (int)c->depth;
        J.bands = dev_bands(dcfg);
        J.coef = (uint16_t*)b.coef;
        J.gcli = b.gcli;
        tiles[n] = J.col_tiles * (int)div_up((h + 1) / 2, vrows);
        n++;
    }
    return n;
}

/* Forward horizontal-only jobs: pass 0 the components with vertical levels
 * (input: their last int32 low band, kind SRC_I32), pass 1 those without
 * (input: the samples, kind enc_level0_kind). */
static inline int plan_fwd_h(const jxs_cfg_t* c, const jxs_cfg_t* dcfg, const FrameBufs& b, const FramePlanes& in, int pass,
                             FwdHJob* jobs) {
    const int packed = c->fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB;
    int n = 0;
    for (uint32_t k = 0; k < c->nc; k++) {
        const jxs_comp_t& cp = c->comp[k];
        if ((cp.dv > 0) != (pass == 0)) continue;
        FwdHJob& J = jobs[n++];
        memset(&J, 0, sizeof(J));
        uint32_t w, h;
        level_dims(cp, (int)cp.dv, &w, &h);
        J.w = (int)w;
        J.h = (int)h;
        if (cp.dv > 0) {
            J.src = b.ll[cp.dv - 1][k];
            J.src_pitch = b.ll_pitch[cp.dv - 1][k];
        } else {
            J.src = in.p[packed ? 0 : k];
            J.src_pitch = in.pitch[packed ? 0 : k];
            J.chan = packed ? (int)k : 0;
        }
        DwtJob bj;
        memset(&bj, 0, sizeof(bj));
        job_bands(c, (int)k, cp.dv > 0 ? (int)cp.dv - 1 : 0, &bj);
        J.nh = bj.nh;
        for (int e = 0; e < 5; e++) J.b_hf[e] = bj.b_hf[e];
        J.b_ll = bj.b_ll;
        J.depth = (int)c->depth;
        J.bands = dev_bands(dcfg);
        J.coef = (uint16_t*)b.coef;
        J.gcli = b.gcli;
    }
    return n;
}

/* Inverse horizontal-only jobs: pass 0 the components whose output comes
 * from a vertical level (output: the int32 low band of their last vertical
 * level, kind 0), pass 1 the others (output: the samples, dec_sample_kind):
 * components without vertical levels, and under proxy decoding those whose
 * output level is their last vertical level (dv == proxy). */
static inline int plan_inv_h(const jxs_cfg_t* c, const jxs_cfg_t* dcfg, const FrameBufs& b, const FramePlanes& out, int pass,
                             InvHJob* jobs) {
    int n = 0;
    for (uint32_t k = 0; k < c->nc; k++) {
        const jxs_comp_t& cp = c->comp[k];
        if ((cp.dv > c->proxy) != (pass == 0)) continue;
        InvHJob& J = jobs[n++];
        memset(&J, 0, sizeof(J));
        uint32_t w, h;
        level_dims(cp, (int)cp.dv, &w, &h);
        J.w = (int)w;
        J.h = (int)h;
        DwtJob bj;
        memset(&bj, 0, sizeof(bj));
        job_bands(c, (int)k, cp.dv > 0 ? (int)cp.dv - 1 : 0, &bj);
        J.nh = bj.nh;
        for (int e = 0; e < 5; e++) J.b_hf[e] = bj.b_hf[e];
        J.b_ll = bj.b_ll;
        if (cp.dv > c->proxy) {
            J.dst = b.ll[cp.dv - 1][k];
            J.dst_pitch = b.ll_pitch[cp.dv - 1][k];
        } else {
            J.dst = out.p[k];
            J.dst_pitch = out.pitch[k];
        }
        J.depth = (int)c->depth;
        J.bw = (int)c->bw;
        J.fq = (int)c->fq;
        J.bands = dev_bands(dcfg);
        J.coef = (const int16_t*)b.coef;
    }
    return n;
}

/* Inverse jobs of vertical level v (output: the int32 low band of level v-1,
 * or the samples for v = proxy, the output level); levels below the output
 * level have no jobs.  *tiles receives each job's block count. */
static inline int plan_inv_v(const jxs_cfg_t* c, const jxs_cfg_t* dcfg, const FrameBufs& b, const FramePlanes& out, int v,
                             InvVJob* jobs, int* tiles) {
    const uint32_t bps = bytes_per_sample(c);
    const uint32_t vcols = (uint32_t)jxs_inv_v_tile_cols(), vrows = (uint32_t)jxs_inv_v_tile_rows();
    int n = 0;
    for (uint32_t k = 0; k < c->nc; k++) {
        const jxs_comp_t& cp = c->comp[k];
        if ((int)cp.dv <= v || v < (int)c->proxy) continue;
        InvVJob& J = jobs[n];
        memset(&J, 0, sizeof(J));
        uint32_t w, h;
        level_dims(cp, v, &w, &h);
        J.w = (int)w;
        J.h = (int)h;
        J.ll = b.ll[v][k];
        J.ll_pitch = b.ll_pitch[v][k];
        const int top = (int)cp.band0 + (int)cp.nb - 1 - 3 * v;
        J.b_hh = top;
        J.b_lh = top - 1;
        J.b_hl = top - 2;
        if (v > (int)c->proxy) {
            J.dst = b.ll[v - 1][k];
            J.dst_pitch = b.ll_pitch[v - 1][k];
            J.vec = 1;
        } else {
            J.dst = out.p[k];
            J.dst_pitch = out.pitch[k];
            J.vec = ((uintptr_t)J.dst % (2 * bps)) == 0 && (J.dst_pitch % 2) == 0;
        }
        J.depth = (int)c->depth;
        J.bw = (int)c->bw;
        J.fq = (int)c->fq;
        J.bands = dev_bands(dcfg);
        J.coef = (const int16_t*)b.coef;
        J.col_tiles = (int)div_up(w, vcols);
        tiles[n] = J.col_tiles * (int)div_up((h + 1) / 2, vrows);
        n++;
    }
    return n;
}

/* Shared-memory layout and block numbering of a horizontal-only launch:
 * rows_per_block is the largest power of two <= max_rpb whose buffers fit;
 * returns the block count, or -1 when one row does not fit. */
template <class LT>
static inline int fwd_h_layout(LT& L, int max_rpb) {
    int maxw = 0;
    for (int i = 0; i < L.njobs; i++) maxw = L.job[i].w > maxw ? L.job[i].w : maxw;
    L.warp_words = 4 + ((maxw + 8 + 3) & ~3) + (((maxw + 1) / 2 + 8 + 3) & ~3) + 4;
    int rpb = max_rpb;
    while (rpb > 1 && (size_t)L.warp_words * rpb * 4 > kSmemMax) rpb >>= 1;
    if ((size_t)L.warp_words * rpb * 4 > kSmemMax) return -1;
    L.rows_per_block = rpb;
    int blocks = 0;
    for (int i = 0; i < L.njobs; i++) {
        L.job[i].first_block = blocks;
        blocks += (int)div_up((uint32_t)L.job[i].h, (uint32_t)rpb);
    }
    return blocks;
}

template <class LT>
static inline int inv_h_layout(LT& L, int max_rpb) {
    int maxw = 0;
    for (int i = 0; i < L.njobs; i++) maxw = L.job[i].w > maxw ? L.job[i].w : maxw;
    L.warp_words = 2 * ((((maxw + 1) / 2) + 8 + 3) & ~3);
    int rpb = max_rpb;
    while (rpb > 1 && (size_t)L.warp_words * rpb * 4 > kSmemMax) rpb >>= 1;
    if ((size_t)L.warp_words * rpb * 4 > kSmemMax) return -1;
    L.rows_per_block = rpb;
    int blocks = 0;
    for (int i = 0; i < L.njobs; i++) {
        L.job[i].first_block = blocks;
        blocks += (int)div_up((uint32_t)L.job[i].h, (uint32_t)rpb);
    }
    return blocks;
}

#endif
