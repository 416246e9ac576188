/*
 * Forward 5/3 wavelet transform for sm_103a.
 *
 *  fwd_v_kernel  one vertical level and the horizontal level that follows
 *                it, on a tile of FV_ROWPAIRS row pairs x FV_COLS columns of
 *                one component.  Vertical lifting runs in registers, one
 *                thread per column pair.  The resulting low and high rows go
 *                to shared memory with a 2-column halo on each side.  Each
 *                row is then lifted horizontally by one warp: lanes hold 4
 *                consecutive samples and exchange the neighbours they need
 *                with shuffles.  Outputs: the HL, LH and HH bands as 16-bit
 *                sign-magnitude coefficients with the GCLI of every
 *                4-coefficient group, and the int32 LL plane for the next
 *                level.
 *  fwd_h_kernel  the horizontal-only levels below the last vertical level
 *                (or all levels of a component without vertical
 *                decomposition): one warp per row, every level in shared
 *                memory, the high band of each level and the final LL band
 *                emitted as coefficients + GCLIs.
 *
 * Arithmetic (bit-exact with the reference):
 *  - input scaling: v = ((x & (2^d - 1)) << (20 - d)) - 2^19 (NltEnc.c:33-72);
 *  - lifting: d[i] = x[2i+1] - ((x[2i] + x[2i+2]) >> 1),
 *    s[i] = x[2i] + ((d[i-1] + d[i] + 2) >> 2), with whole-sample symmetric
 *    extension at both ends (Dwt.c:15-40 horizontally, :337-398 vertically;
 *    the reference's edge special cases are what the mirrored samples give);
 *  - vertical before horizontal at every level, the low band of a level
 *    being the next level's input (Dwt.c:550-1142, frame form);
 *  - sign-magnitude with Fq = 8: m = (|v| + 128) >> 8, no negative zero
 *    (NltEnc.c:12-31);
 *  - GCLI = bit length of the OR of a group's magnitudes
 *    (GcStageProcess.c:42-68).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "jxs_core.h"
#include "jxs_kernels.cuh"

#define DEV __device__ __forceinline__
#define FULL 0xffffffffu

/* ------------------------------------------------------------------------ */
/* helpers                                                                   */
/* ------------------------------------------------------------------------ */
/* whole-sample symmetric extension of index i into [0, n) */
DEV int mirror_idx(int i, int n) {
    if ((unsigned)i < (unsigned)n) return i;
    if (n == 1) return 0;
    const int p = 2 * (n - 1);
    i %= p;
    if (i < 0) i += p;
    return i < n ? i : p - i;
}

DEV uint32_t to_sm(int32_t v) {
    if (v >= 0) return (uint32_t)((v + 128) >> 8);
    const uint32_t m = (uint32_t)((-v + 128) >> 8);
    return m ? (m | 0x8000u) : 0u;
}

template <int SRC>
DEV int32_t scale_in(uint32_t raw, int depth) {
    if (SRC == SRC_I32) return (int32_t)raw;
    const uint32_t mask = (1u << depth) - 1u;
    return (int32_t)((raw & mask) << (20 - depth)) - (1 << 19);
}

/* one sample of the level input at (row y, column x), both in range */
template <int SRC>
DEV int32_t load1(const void* src, long long pitch, int chan, int depth, int y, int x) {
    const long long row = (long long)y * pitch;
    if (SRC == SRC_I32) return ((const int32_t*)src)[row + x];
    if (SRC == SRC_U8) return scale_in<SRC>(((const uint8_t*)src)[row + x], depth);
    if (SRC == SRC_U16) return scale_in<SRC>(((const uint16_t*)src)[row + x], depth);
    if (SRC == SRC_PK8) return scale_in<SRC>(((const uint8_t*)src)[row + 3 * x + chan], depth);
    return scale_in<SRC>(((const uint16_t*)src)[row + 3 * x + chan], depth);
}

/* two horizontally adjacent samples (x even, x + 1 < width) with one load
 * where the layout allows it */
template <int SRC>
DEV void load2(const void* src, long long pitch, int chan, int depth, int y, int x, bool vec, int32_t& a, int32_t& b) {
    const long long row = (long long)y * pitch;
    if (vec && SRC == SRC_I32) {
        const int2 v = *(const int2*)((const int32_t*)src + row + x);
        a = v.x;
        b = v.y;
    } else if (vec && SRC == SRC_U16) {
        const uint32_t v = *(const uint32_t*)((const uint16_t*)src + row + x);
        a = scale_in<SRC>(v & 0xffffu, depth);
        b = scale_in<SRC>(v >> 16, depth);
    } else if (vec && SRC == SRC_U8) {
        const uint32_t v = *(const uint16_t*)((const uint8_t*)src + row + x);
        a = scale_in<SRC>(v & 0xffu, depth);
        b = scale_in<SRC>(v >> 8, depth);
    } else {
        a = load1<SRC>(src, pitch, chan, depth, y, x);
        b = load1<SRC>(src, pitch, chan, depth, y, x + 1);
    }
}

/* One lane's 4-coefficient group of a band row: coefficients j..j+3 (j a
 * multiple of 4) as sign-magnitude plus the group's GCLI.  crow / grow are
 * the band row's coefficient and GCLI rows; w its width, gw its groups.
 * Coefficients past the width are written as zero; nothing past the last
 * group. */
struct BandRow {
    uint16_t* crow;
    uint8_t* grow;
    int w, gw;
};
DEV BandRow band_row(const jxs_band_t& bd, int row, uint16_t* coef, uint8_t* gcli) {
    BandRow r;
    r.crow = coef + bd.coef_off + (uint64_t)row * bd.pitch;
    r.grow = gcli + bd.gcli_off + (uint64_t)row * bd.gpitch;
    r.w = (int)bd.w;
    r.gw = (int)bd.gcli_w;
    return r;
}
DEV void emit4(const BandRow& b, int j, int32_t v0, int32_t v1, int32_t v2, int32_t v3) {
    if ((j >> 2) >= b.gw) return;
    const uint32_t c0 = to_sm(v0), c1 = j + 1 < b.w ? to_sm(v1) : 0u, c2 = j + 2 < b.w ? to_sm(v2) : 0u,
                   c3 = j + 3 < b.w ? to_sm(v3) : 0u;
    *(uint2*)(b.crow + j) = make_uint2(c0 | (c1 << 16), c2 | (c3 << 16));
    const uint32_t m = (c0 | c1 | c2 | c3) & 0x7fffu;
    b.grow[j >> 2] = (uint8_t)(32 - __clz(m));
}

/* One horizontal lifting pass of a row held in shared memory, by one warp.
 * x points at sample 0 of the pass; x[-2], x[-1] and the samples past the
 * last pair needed hold the (mirrored or neighbouring-tile) halo.  Output
 * pairs (s[j], d[j]) for j in [0, npairs) are produced; lane l of iteration
 * it owns j = 128*it + 4l .. +3 and passes them to out(j, s[4], d[4]).
 * Reads x[-2 .. 8 * ceil(npairs / 4) + 7] at most; outputs past the valid
 * width may depend on samples past x[2 * npairs + 1] and are discarded by
 * the caller.  x must be 16-byte aligned. */
template <typename Out>
DEV void warp_lift_fwd(const int32_t* x, int npairs, Out out) {
    const int lane = threadIdx.x & 31;
    int32_t carry = x[-1] - ((x[-2] + x[0]) >> 1); /* d[-1] */
    for (int base = 0; base < npairs; base += 128) {
        const int j = base + 4 * lane;
        int4 a = make_int4(0, 0, 0, 0), b = a;
        /* the lane just past the last pair still loads: its first sample is
         * the right neighbour of the previous lane */
        if (j <= npairs) {
            a = *(const int4*)(x + 2 * j);
            b = *(const int4*)(x + 2 * j + 4);
        }
        int32_t nxt = __shfl_down_sync(FULL, a.x, 1);
        if (lane == 31) nxt = j < npairs ? x[2 * j + 8] : 0;
        int32_t d[4], sv[4];
        d[0] = a.y - ((a.x + a.z) >> 1);
        d[1] = a.w - ((a.z + b.x) >> 1);
        d[2] = b.y - ((b.x + b.z) >> 1);
        d[3] = b.w - ((b.z + nxt) >> 1);
        int32_t dm = __shfl_up_sync(FULL, d[3], 1);
        if (lane == 0) dm = carry;
        carry = __shfl_sync(FULL, d[3], 31);
        sv[0] = a.x + ((dm + d[0] + 2) >> 2);
        sv[1] = a.z + ((d[0] + d[1] + 2) >> 2);
        sv[2] = b.x + ((d[1] + d[2] + 2) >> 2);
        sv[3] = b.z + ((d[2] + d[3] + 2) >> 2);
        if (j < npairs) out(j, sv, d);
    }
}

/* ------------------------------------------------------------------------ */
/* vertical level + one horizontal level                                     */
/* ------------------------------------------------------------------------ */
#define FV_THREADS 128
#define FV_COLS (2 * FV_THREADS - 8)      /* level-input columns per tile: tile + 4 halo columns in one pass */
#define FV_ROWPAIRS 8
#define FV_SROW (FV_COLS + 16)            /* shared row: 4 front words (2 pad, 2 halo), FV_COLS, halo, slack */

#define FV_NR (2 * FV_ROWPAIRS + 3)       /* input rows per tile: 2 above, 2 R, 1 below */

/* Raw input of one column pair in the staging buffer: the two samples as
 * read (16-bit sources: packed in one word) or the two int32 low-band
 * values. */
template <int SRC> struct FvIn { typedef uint32_t T; };
template <> struct FvIn<SRC_I32> { typedef int2 T; };

DEV void cp_async4(void* smem, const void* g) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(g));
}
DEV void cp_async8(void* smem, const void* g) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(g));
}
DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
DEV void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }

/* One tile of a vertical-level launch. */
struct FvTile {
    int jb, r0, c0, npairs, ncp, rc, hc;
};
template <int NJ>
DEV FvTile fv_tile(const FwdVLaunchN<NJ>& L, int t) {
    FvTile T;
    const int jb = find_job<NJ>(L.job, L.njobs, t);
    const FwdVJob& J = L.job[jb];
    const int u = t - J.first_block;
    const int ty = u / J.col_tiles, tx = u - ty * J.col_tiles;
    const int n1 = (J.h + 1) >> 1, n2 = J.h >> 1, w1 = (J.w + 1) >> 1;
    T.jb = jb;
    T.r0 = ty * FV_ROWPAIRS;
    T.c0 = tx * FV_COLS;
    /* output pairs j in [c0/2, c0/2 + npairs) of the level's bands; lifting
     * them reads input columns c0 - 2 .. c0 + 2 npairs + 1 */
    T.npairs = min(FV_COLS / 2, ((w1 - T.c0 / 2) + 1) & ~1);
    T.ncp = T.npairs + 2;
    T.rc = min(FV_ROWPAIRS, n1 - T.r0);
    T.hc = max(0, min(FV_ROWPAIRS, n2 - T.r0));
    return T;
}

/* Stages the input of tile t into buffer `in` (FV_NR rows x column pairs):
 * asynchronous copies where the pair is inside the plane and aligned,
 * ordinary loads (with the symmetric extension) elsewhere. */
template <int SRC, int NJ>
DEV void fv_stage(const FwdVLaunchN<NJ>& L, int t, typename FvIn<SRC>::T* in) {
    const FvTile T = fv_tile(L, t);
    const FwdVJob& J = L.job[T.jb];
    const int cp = threadIdx.x;
    if (cp >= T.ncp) return;
    const int w = J.w, h = J.h;
    const int xa = T.c0 - 2 + 2 * cp;
    const bool inside = xa >= 0 && xa + 1 < w;
    const bool async = inside && J.vec && (SRC == SRC_U16 || SRC == SRC_I32);
    const int ma = mirror_idx(xa, w), mb = mirror_idx(xa + 1, w);
#pragma unroll 4
    for (int k = 0; k < FV_NR; k++) {
        const int y = mirror_idx(2 * T.r0 - 2 + k, h);
        typename FvIn<SRC>::T* dst = in + k * FV_THREADS + cp;
        const long long row = (long long)y * J.src_pitch;
        if (SRC == SRC_I32) {
            const int32_t* src = (const int32_t*)J.src + row;
            if (async) cp_async8(dst, src + xa);
            else *(int2*)dst = make_int2(src[ma], src[mb]);
        } else if (SRC == SRC_U16) {
            const uint16_t* src = (const uint16_t*)J.src + row;
            if (async) cp_async4(dst, src + xa);
            else *(uint32_t*)dst = (uint32_t)src[ma] | ((uint32_t)src[mb] << 16);
        } else if (SRC == SRC_U8) {
            const uint8_t* src = (const uint8_t*)J.src + row;
            *(uint32_t*)dst = (uint32_t)src[ma] | ((uint32_t)src[mb] << 16);
        } else if (SRC == SRC_PK8) {
            const uint8_t* src = (const uint8_t*)J.src + row;
            *(uint32_t*)dst = (uint32_t)src[3 * ma + J.chan] | ((uint32_t)src[3 * mb + J.chan] << 16);
        } else {
            const uint16_t* src = (const uint16_t*)J.src + row;
            *(uint32_t*)dst = (uint32_t)src[3 * ma + J.chan] | ((uint32_t)src[3 * mb + J.chan] << 16);
        }
    }
}

/* Persistent: each block walks tiles t = blockIdx.x, + gridDim.x, ...; the
 * next tile's input is staged (asynchronous copies) while the current one is
 * lifted.  With `persistent` false (int32 low bands, still in L2) the grid
 * has one block per tile and a single buffer. */
template <int SRC, int NJ>
__global__ void __launch_bounds__(FV_THREADS, 6) fwd_v_kernel(const __grid_constant__ FwdVLaunchN<NJ> L) {
    typedef typename FvIn<SRC>::T InT;
    extern __shared__ __align__(16) unsigned char fv_dyn[];
    InT* inbuf = (InT*)fv_dyn; /* [2][FV_NR][FV_THREADS] */
    __shared__ __align__(16) int32_t sL[FV_ROWPAIRS][FV_SROW];
    __shared__ __align__(16) int32_t sH[FV_ROWPAIRS][FV_SROW];
    const int warp = threadIdx.x >> 5;
    const bool persistent = gridDim.x < (unsigned)L.ntiles;
    int t = blockIdx.x, buf = 0;
    if (t < L.ntiles) fv_stage<SRC, NJ>(L, t, inbuf);
    cp_async_commit();
    for (; t < L.ntiles; t += gridDim.x) {
        const int tn = t + gridDim.x;
        if (persistent && tn < L.ntiles) fv_stage<SRC, NJ>(L, tn, inbuf + (buf ^ 1) * FV_NR * FV_THREADS);
        cp_async_commit();
        cp_async_wait1();
        __syncthreads();
        const FvTile T = fv_tile(L, t);
        const FwdVJob& J = L.job[T.jb];
        const int depth = J.depth;
        const InT* in = inbuf + buf * FV_NR * FV_THREADS;
        /* vertical lifting, one column pair per thread */
        const int cp = threadIdx.x;
        if (cp < T.ncp) {
            int32_t a[FV_NR], b[FV_NR];
#pragma unroll
            for (int k = 0; k < FV_NR; k++) {
                const InT v = in[k * FV_THREADS + cp];
                if (SRC == SRC_I32) {
                    a[k] = ((const int2*)&v)->x;
                    b[k] = ((const int2*)&v)->y;
                } else {
                    const uint32_t r = *(const uint32_t*)&v;
                    a[k] = scale_in<SRC>(r & 0xffffu, depth);
                    b[k] = scale_in<SRC>(r >> 16, depth);
                }
            }
            int32_t hpa = a[1] - ((a[0] + a[2]) >> 1), hpb = b[1] - ((b[0] + b[2]) >> 1);
#pragma unroll
            for (int k = 0; k < FV_ROWPAIRS; k++) {
                const int e = 2 + 2 * k; /* x[2i] of pair r0 + k */
                const int32_t ha = a[e + 1] - ((a[e] + a[e + 2]) >> 1), hb = b[e + 1] - ((b[e] + b[e + 2]) >> 1);
                const int32_t la = a[e] + ((hpa + ha + 2) >> 2), lb = b[e] + ((hpb + hb + 2) >> 2);
                *(int2*)&sL[k][2 + 2 * cp] = make_int2(la, lb);
                *(int2*)&sH[k][2 + 2 * cp] = make_int2(ha, hb);
                hpa = ha;
                hpb = hb;
            }
        }
        __syncthreads();

        /* horizontal lifting, one warp per row; the tile's output pairs are
         * j in [c0/2, c0/2 + npairs) of the level's bands */
        const int w1 = (J.w + 1) >> 1;
        const int jc = T.c0 >> 1;
        for (int r = warp; r < T.rc + T.hc; r += FV_THREADS / 32) {
            if (r < T.rc) {
                const int row = T.r0 + r;
                const BandRow bhl = band_row(J.bands[J.b_hl], row, J.coef, J.gcli);
                int32_t* ll = J.ll + (long long)row * J.ll_pitch;
                warp_lift_fwd(&sL[r][4], T.npairs, [&](int j, const int32_t* sv, const int32_t* d) {
                    const int jj = jc + j;
                    emit4(bhl, jj, d[0], d[1], d[2], d[3]);
                    if (jj + 3 < w1) {
                        *(int4*)(ll + jj) = make_int4(sv[0], sv[1], sv[2], sv[3]);
                    } else {
                        for (int q = 0; q < 4; q++)
                            if (jj + q < w1) ll[jj + q] = sv[q];
                    }
                });
            } else {
                const int row = T.r0 + r - T.rc;
                const BandRow blh = band_row(J.bands[J.b_lh], row, J.coef, J.gcli);
                const BandRow bhh = band_row(J.bands[J.b_hh], row, J.coef, J.gcli);
                warp_lift_fwd(&sH[r - T.rc][4], T.npairs, [&](int j, const int32_t* sv, const int32_t* d) {
                    emit4(blh, jc + j, sv[0], sv[1], sv[2], sv[3]);
                    emit4(bhh, jc + j, d[0], d[1], d[2], d[3]);
                });
            }
        }
        __syncthreads();
        buf ^= 1;
    }
}

/* ------------------------------------------------------------------------ */
/* horizontal-only levels                                                    */
/* ------------------------------------------------------------------------ */
#define FH_MAX_WARPS 4

/* fills the 2-sample halo on both sides of a row of n samples at x */
DEV void fill_halo(int32_t* x, int n, int lane) {
    if (lane < 4) {
        const int i = lane < 2 ? -2 + lane : n + lane - 2;
        x[i] = x[mirror_idx(i, n)];
    }
}

template <int SRC, int NJ>
__global__ void __launch_bounds__(FH_MAX_WARPS * 32) fwd_h_kernel(const __grid_constant__ FwdHLaunchN<NJ> L) {
    extern __shared__ __align__(16) int32_t hsm[];
    const FwdHJob& J = L.job[find_job<NJ>(L.job, L.njobs, (int)blockIdx.x)];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = (blockIdx.x - J.first_block) * L.rows_per_block + warp;
    if (row >= J.h) return;
    const int n = J.w;
    /* per warp: buffer A (n + 8 words) and buffer B (n/2 + 8 words) */
    int32_t* bufA = hsm + warp * L.warp_words + 4;
    int32_t* bufB = bufA + ((n + 8 + 3) & ~3);
    for (int x = lane; x < n; x += 32) bufA[x] = load1<SRC>(J.src, J.src_pitch, J.chan, J.depth, row, x);
    __syncwarp();
    fill_halo(bufA, n, lane);
    __syncwarp();
    int32_t* cur = bufA;
    int32_t* nxt = bufB;
    int m = n;
    for (int e = 0; e < J.nh; e++) {
        if (m == 1) break; /* nothing left to split: the remaining high bands are empty */
        const BandRow bd = band_row(J.bands[J.b_hf[e]], row, J.coef, J.gcli);
        const int m1 = (m + 1) >> 1;
        int32_t* dst = nxt;
        warp_lift_fwd(cur, m1, [&](int j, const int32_t* sv, const int32_t* d) {
            emit4(bd, j, d[0], d[1], d[2], d[3]);
            if (j + 3 < m1) {
                *(int4*)(dst + j) = make_int4(sv[0], sv[1], sv[2], sv[3]);
            } else {
                for (int q = 0; q < 4; q++)
                    if (j + q < m1) dst[j + q] = sv[q];
            }
        });
        __syncwarp();
        fill_halo(dst, m1, lane);
        __syncwarp();
        nxt = cur;
        cur = dst;
        m = m1;
    }
    /* final low band */
    const BandRow bl = band_row(J.bands[J.b_ll], row, J.coef, J.gcli);
    for (int j = 4 * lane; j < m; j += 128) {
        int32_t v[4];
        for (int q = 0; q < 4; q++) v[q] = j + q < m ? cur[j + q] : 0;
        emit4(bl, j, v[0], v[1], v[2], v[3]);
    }
}

/* ------------------------------------------------------------------------ */
/* launchers                                                                 */
/* ------------------------------------------------------------------------ */
extern "C" int jxs_fwd_v_tile_rows(void) { return FV_ROWPAIRS; }
extern "C" int jxs_fwd_v_tile_cols(void) { return FV_COLS; }
extern "C" int jxs_fwd_h_max_rows_per_block(void) { return FH_MAX_WARPS; }

template <int SRC, int NJ>
static cudaError_t launch_v(const FwdVLaunchN<NJ>* L, int grid_per_sm, cudaStream_t st) {
    /* int32 inputs (the previous level's low band, in L2): one block per
     * tile, one buffer; sample planes: persistent, double-buffered, with
     * grid_per_sm blocks per SM (0: as many as fit) */
    const bool persistent = SRC != SRC_I32;
    const size_t smem = (persistent ? 2 : 1) * FV_NR * FV_THREADS * sizeof(typename FvIn<SRC>::T);
    static std::atomic<int> attr[JXS_MAX_DEV];
    cudaError_t e = jxs_smem_attr(fwd_v_kernel<SRC, NJ>, (int)smem, attr);
    if (e != cudaSuccess) return e;
    int blocks = L->ntiles;
    if (persistent) {
        /* SMs and resident blocks per SM, queried once per device */
        static std::atomic<int> q_sms[JXS_MAX_DEV], q_per_sm[JXS_MAX_DEV];
        int dev = 0, sms = 0, per_sm = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        const bool cached = dev >= 0 && dev < JXS_MAX_DEV && q_sms[dev].load() > 0;
        if (cached) {
            sms = q_sms[dev].load();
            per_sm = q_per_sm[dev].load();
        } else {
            if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fwd_v_kernel<SRC, NJ>, FV_THREADS, smem)) !=
                cudaSuccess)
                return e;
            if (dev >= 0 && dev < JXS_MAX_DEV) {
                q_per_sm[dev].store(per_sm);
                q_sms[dev].store(sms);
            }
        }
        if (per_sm < 1) per_sm = 1;
        if (grid_per_sm > 0 && grid_per_sm < per_sm) per_sm = grid_per_sm;
        blocks = sms * per_sm;
        if (blocks > L->ntiles) blocks = L->ntiles;
    }
    if (blocks <= 0) return cudaSuccess;
    fwd_v_kernel<SRC, NJ><<<blocks, FV_THREADS, smem, st>>>(*L);
    return cudaGetLastError();
}

template <int NJ>
static cudaError_t launch_v_kind(const FwdVLaunchN<NJ>* L, int src_kind, int grid_per_sm, cudaStream_t st) {
    switch (src_kind) {
    case SRC_I32: return launch_v<SRC_I32, NJ>(L, grid_per_sm, st);
    case SRC_U8: return launch_v<SRC_U8, NJ>(L, grid_per_sm, st);
    case SRC_U16: return launch_v<SRC_U16, NJ>(L, grid_per_sm, st);
    case SRC_PK8: return launch_v<SRC_PK8, NJ>(L, grid_per_sm, st);
    default: return launch_v<SRC_PK16, NJ>(L, grid_per_sm, st);
    }
}

extern "C" cudaError_t jxs_launch_fwd_v(const FwdVLaunch* L, int src_kind, int grid_per_sm, cudaStream_t st) {
    return launch_v_kind<JXS_MAXC>(L, src_kind, grid_per_sm, st);
}
extern "C" cudaError_t jxs_launch_fwd_v_batch(const FwdVLaunchB* L, int src_kind, int grid_per_sm, cudaStream_t st) {
    return launch_v_kind<JXS_BATCH_JOBS>(L, src_kind, grid_per_sm, st);
}

template <int SRC, int NJ>
static cudaError_t launch_h(const FwdHLaunchN<NJ>* L, int nblocks, cudaStream_t st) {
    const size_t smem = (size_t)L->warp_words * L->rows_per_block * sizeof(int32_t);
    static std::atomic<int> attr[JXS_MAX_DEV];
    cudaError_t e = jxs_smem_attr(fwd_h_kernel<SRC, NJ>, (int)smem, attr);
    if (e != cudaSuccess) return e;
    if (nblocks <= 0) return cudaSuccess;
    fwd_h_kernel<SRC, NJ><<<nblocks, L->rows_per_block * 32, smem, st>>>(*L);
    return cudaGetLastError();
}

template <int NJ>
static cudaError_t launch_h_kind(const FwdHLaunchN<NJ>* L, int src_kind, int nblocks, cudaStream_t st) {
    switch (src_kind) {
    case SRC_I32: return launch_h<SRC_I32, NJ>(L, nblocks, st);
    case SRC_U8: return launch_h<SRC_U8, NJ>(L, nblocks, st);
    case SRC_U16: return launch_h<SRC_U16, NJ>(L, nblocks, st);
    case SRC_PK8: return launch_h<SRC_PK8, NJ>(L, nblocks, st);
    default: return launch_h<SRC_PK16, NJ>(L, nblocks, st);
    }
}

extern "C" cudaError_t jxs_launch_fwd_h(const FwdHLaunch* L, int src_kind, int nblocks, cudaStream_t st) {
    return launch_h_kind<JXS_MAXC>(L, src_kind, nblocks, st);
}
extern "C" cudaError_t jxs_launch_fwd_h_batch(const FwdHLaunchB* L, int src_kind, int nblocks, cudaStream_t st) {
    return launch_h_kind<JXS_BATCH_JOBS>(L, src_kind, nblocks, st);
}
