/*
 * Launch descriptors shared by the kernels (jxs_enc_kernels.cu,
 * jxs_dec_kernels.cu) and the launcher (jxs_gpu.cu).
 */
#ifndef JXS_KERNELS_CUH
#define JXS_KERNELS_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "jxs_core.h"

/* Source sample formats of the first transform level. */
enum {
    SRC_I32 = 0,    /* int32 low-pass plane of the previous level */
    SRC_U8 = 1,     /* planar 8-bit */
    SRC_U16 = 2,    /* planar 9..16-bit little endian */
    SRC_PK8 = 3,    /* packed 3 x 8-bit */
    SRC_PK16 = 4    /* packed 3 x 16-bit */
};

/* One component's share of a transform-level launch.  Blocks
 * [first_block, first_block + nblocks) of the grid belong to it. */
struct DwtJob {
    int comp;
    int first_block, nblocks;
    int R;              /* row pairs (vertical level) or rows (horizontal only) per block */
    int w, h;           /* size of the region transformed at this level */
    int last;           /* last vertical level: continue with the horizontal-only levels */
    int nh;             /* horizontal-only levels run after this one */
    int src_kind, depth, chan;
    const void* src;    /* level input (samples or int32 low band) */
    long long src_pitch;/* elements */
    int32_t* ll;        /* int32 low band for the next vertical level (forward) or from the deeper level (inverse) */
    int ll_pitch;
    int b_hl, b_lh, b_hh;   /* flat band indices produced by this vertical level */
    int b_hf[5];            /* high band of each horizontal-only level */
    int b_ll;               /* final low band */
    int smem_pitch;         /* int32 elements per shared-memory row */
    /* inverse only: destination plane */
    void* dst;
    long long dst_pitch;
    int out_kind;           /* 0: int32 ll, 1: u8 plane, 2: u16 plane */
};

/* Job capacity of one transform launch in the per-frame form (one job per
 * component) and in the batched form (jobs of many frames). */
#define JXS_BATCH_JOBS 96
/* Frames of one per-precinct launch in the batched form. */
#define JXS_BATCH_FRAMES 64

/* Forward transform, one vertical level (jxs_fwd_dwt.cu): one component's
 * share of the launch; its tiles are blocks [first_block, first_block +
 * row_tiles * col_tiles). */
struct FwdVJob {
    const void* src;        /* level input: samples (level 0) or the int32 low band of the previous level */
    long long src_pitch;    /* elements */
    int chan;               /* packed input: channel of this component */
    int vec;                /* rows may be read 8 samples per vector load (aligned planar source) */
    int w, h;               /* level input size */
    int col_tiles, first_block;
    int32_t* ll;            /* int32 low band written for the next level */
    int ll_pitch;           /* elements, a multiple of 4 */
    int b_hl, b_lh, b_hh;   /* flat band indices */
    int depth;              /* sample bit depth of the frame */
    const jxs_band_t* bands;/* the frame's band table (device copy of its configuration) */
    uint16_t* coef;         /* the frame's coefficient and GCLI planes */
    uint8_t* gcli;
};
template <int NJ> struct FwdVLaunchN {
    int njobs;
    int ntiles;             /* tiles of all jobs; job j owns [first_block, next job's first_block) */
    FwdVJob job[NJ];
};
typedef FwdVLaunchN<JXS_MAXC> FwdVLaunch;
typedef FwdVLaunchN<JXS_BATCH_JOBS> FwdVLaunchB;

/* Forward transform, horizontal-only levels: rows [0, h) of a w-wide
 * plane, rows_per_block rows (one warp each) per block. */
struct FwdHJob {
    const void* src;
    long long src_pitch;
    int chan;
    int w, h;
    int first_block;
    int nh;                 /* levels */
    int b_hf[5];            /* high band of each level */
    int b_ll;               /* final low band */
    int depth;
    const jxs_band_t* bands;
    uint16_t* coef;
    uint8_t* gcli;
};
template <int NJ> struct FwdHLaunchN {
    int njobs;
    int rows_per_block;
    int warp_words;         /* shared-memory words per warp */
    FwdHJob job[NJ];
};
typedef FwdHLaunchN<JXS_MAXC> FwdHLaunch;
typedef FwdHLaunchN<JXS_BATCH_JOBS> FwdHLaunchB;

/* Inverse transform, one vertical level (jxs_inv_dwt.cu): rebuilds the
 * w x h level input from the int32 low band ll and the HL, LH, HH bands. */
struct InvVJob {
    int w, h;
    const int32_t* ll;
    int ll_pitch;           /* elements, a multiple of 4 */
    int b_hl, b_lh, b_hh;
    int col_tiles, first_block;
    void* dst;              /* int32 low band of the next level up, or the output plane */
    long long dst_pitch;    /* elements */
    int vec;                /* two adjacent output samples may be stored at once */
    int depth, bw, fq;
    const jxs_band_t* bands;
    const int16_t* coef;
};
template <int NJ> struct InvVLaunchN {
    int njobs;
    InvVJob job[NJ];
};
typedef InvVLaunchN<JXS_MAXC> InvVLaunch;
typedef InvVLaunchN<JXS_BATCH_JOBS> InvVLaunchB;

/* Inverse transform, horizontal-only levels: rows [0, h) of width w. */
struct InvHJob {
    int w, h;
    int first_block;
    int nh;
    int b_hf[5], b_ll;
    void* dst;
    long long dst_pitch;
    int depth, bw, fq;
    const jxs_band_t* bands;
    const int16_t* coef;
};
template <int NJ> struct InvHLaunchN {
    int njobs;
    int rows_per_block, warp_words;
    InvHJob job[NJ];
};
typedef InvHLaunchN<JXS_MAXC> InvHLaunch;
typedef InvHLaunchN<JXS_BATCH_JOBS> InvHLaunchB;

/* Job of block b: the last job whose first_block is <= b.  Linear for the
 * per-frame launches (at most 4 jobs), binary for batched ones. */
template <int NJ, class JOB>
__device__ __forceinline__ int find_job(const JOB* job, int njobs, int b) {
    if (NJ <= JXS_MAXC) {
        int jb = 0;
        while (jb + 1 < njobs && b >= job[jb + 1].first_block) jb++;
        return jb;
    }
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (b >= job[mid].first_block) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

/* The colour transform and output non-linearity of a decoded frame
 * (nlt_out_kernel): int32 planes in, samples out. */
struct NltOut {
    const int32_t* in[JXS_MAXC];
    long long in_pitch[JXS_MAXC];  /* elements */
    void* out[JXS_MAXC];
    long long out_pitch[JXS_MAXC]; /* samples */
    int w[JXS_MAXC], h[JXS_MAXC];
    int nc, cpih, tnlt, bw, depth, bps;
    /* quadratic: dco = alpha - sigma 2^15; extended: thresholds and the
     * constants of NltDec.c:111-116 */
    int32_t dco, t1, t2, e, b1;
    int64_t b2, b3, a1, a3;
};

/* The inverse Star-Tetrix transform of a decoded frame (star_tetrix_kernel):
 * four int32 planes of w x h with one pitch, updated in place. */
struct StParams {
    int32_t* c[4];
    long long pitch;
    int w, h, cf, ct, e1, e2;
};

/* Encoder rate-control outputs per precinct row. */
struct PrecRC {
    uint32_t total_bytes;  /* bytes written for the precinct (header to last data byte, incl. trailing padding) */
    uint32_t offset;       /* absolute byte offset of the precinct in the codestream */
    uint32_t data_bytes;   /* sub-packet bytes chosen by the rate control (cross-check for packing) */
    uint8_t q, r, first_in_slice, pad;
};

/* Batched per-precinct launches (rate control, packing, unpacking): one
 * entry per frame.  Blocks [first_block, next frame's first_block) are the
 * frame's precincts; the kernels find their frame with find_job. */
struct EncPrecFrame {
    const jxs_cfg_t* cfg;   /* device copy of the frame's configuration */
    const uint16_t* coef;
    const uint8_t* gcli;
    uint32_t* cost;
    uint32_t* slice_done;
    PrecRC* rc;
    uint8_t* out;           /* codestream */
    int* status;
    int first_block;
};
struct EncPrecLaunch {
    int nframes;
    int nblocks;
    EncPrecFrame job[JXS_BATCH_FRAMES];
};

struct DecPrecFrame {
    const jxs_cfg_t* cfg;
    const uint8_t* bs;      /* codestream */
    uint32_t bs_size;
    uint32_t* prec_off;     /* precinct byte offsets */
    int16_t* coef;
    int* status;            /* status[0]: frame status; status[1]: the slice walk found a mismatch */
    int first_block;        /* unpacking: first precinct block */
    int first_slice;        /* walk: first slice thread */
};
struct DecPrecLaunch {
    int nframes;
    int nblocks, nslices;
    DecPrecFrame job[JXS_BATCH_FRAMES];
};

/* Dynamic shared memory of the unpacking kernels (jxs_dec_kernels.cu), laid
 * out for the largest frame of a launch: the precinct's bytes (cap_bytes +
 * 32), a GCLI per group (cap_groups), the zero-bit table (a 16-bit offset per
 * zero: one per codeword plus up to 7 padding bits per packet), then the
 * per-segment arrays (cap_seg segments): the segment table, its work order,
 * counts, bases, block-wide sums and, for separate signs, sign counts and
 * first sign bits.  `end` is the size of one precinct's area; slice-ordered
 * decoding keeps the row above's GCLIs after it (top, cap_groups bytes). */
#define UK_ZCAP(cap_groups) ((cap_groups) + 8 * JXS_MAXPK + 32)
/* 128 list entries per warp of a 512-thread unpacking block */
#define UK_LIST_BYTES (4 * 128 * 16)
struct UkLayout {
    uint32_t gcl, zend, seg, cnt, base, ex, nz, sgb, ord, end, top, top_end;
};
static inline __host__ __device__ UkLayout uk_layout(uint32_t cap_bytes, uint32_t cap_groups, uint32_t cap_seg) {
    UkLayout L;
    uint32_t o = cap_bytes + 32;
    L.gcl = o;
    o = (o + cap_groups + 15) & ~15u;
    L.zend = o;
    /* the zero-bit table; in the data pass the same area holds each warp's
     * list of groups with data (UK_LIST_BYTES) */
    o = (o + (2 * UK_ZCAP(cap_groups) > UK_LIST_BYTES ? 2 * UK_ZCAP(cap_groups) : UK_LIST_BYTES) + 15) & ~15u;
    L.seg = o;
    o += 8 * cap_seg;
    L.cnt = o;
    o += 4 * cap_seg;
    L.base = o;
    o += 4 * cap_seg;
    L.ex = o;
    o += 4 * (cap_seg + 1);
    L.nz = o;
    o += 4 * cap_seg;
    L.sgb = o;
    o += 4 * cap_seg;
    L.ord = o;
    o = (o + 2 * cap_seg + 15) & ~15u;
    L.end = o;
    L.top = o;
    L.top_end = (o + cap_groups + 15) & ~15u;
    return L;
}
/* Static shared memory of the unpacking kernels at most (the launchers size
 * the dynamic part against what is left of an SM's shared memory). */
#define UK_STATIC_SMEM (9 * 1024)

/* Launch-time queries cached per device: a kernel's dynamic shared-memory
 * limit is raised only when a launch needs more than was set before, so the
 * steady state costs no driver call. */
#define JXS_MAX_DEV 16
template <class K>
static inline cudaError_t jxs_smem_attr(K kern, int bytes, std::atomic<int>* cache) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < JXS_MAX_DEV && cache[dev].load(std::memory_order_relaxed) >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && dev >= 0 && dev < JXS_MAX_DEV) {
        int cur = cache[dev].load(std::memory_order_relaxed);
        while (cur < bytes && !cache[dev].compare_exchange_weak(cur, bytes)) {
        }
    }
    return e;
}

#define JXS_STATUS_SET(ptr, code) atomicCAS((int*)(ptr), 0, (int)(code))

#endif
