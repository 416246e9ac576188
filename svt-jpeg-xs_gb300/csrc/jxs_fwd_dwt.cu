/*
 * Forward 5/3 wavelet transform for sm_103a.
 *
 *  fwd_v_kernel  one vertical level and the horizontal level that follows
 *                it.  Each warp streams down a strip of 240 columns (8 per
 *                lane, plus one halo lane on either side) for 8 row pairs:
 *                vertical lifting in registers, then horizontal lifting
 *                across the warp with shuffles.  Outputs: the HL, LH and HH
 *                bands as 16-bit sign-magnitude coefficients with the GCLI of
 *                every 4-coefficient group (one group per lane and band row),
 *                and the int32 LL plane for the next level.
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

/* The same for the indices a strip reads (-n < i < 2n - 1: one reflection)
 * without a division; other indices (levels of one or two samples) take the
 * general form out of line, so that the division is never inlined into the
 * loops. */
__device__ __noinline__ int mirror_far(int i, int n) { return mirror_idx(i, n); }
DEV int mirror1(int i, int n) {
    const int a = i < 0 ? -i : i;
    const int m = a < n ? a : 2 * (n - 1) - a;
    return (unsigned)m < (unsigned)n ? m : mirror_far(i, n);
}

DEV uint32_t to_sm(int32_t v) {
    const uint32_t m = ((uint32_t)abs(v) + 128u) >> 8;
    return m ? (m | (((uint32_t)v >> 16) & 0x8000u)) : 0u;
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
/* A tile is FV_COLS columns x FV_ROWPAIRS row pairs of the level input; its
 * warps are stacked vertically, each working alone on FV_WROWPAIRS row pairs
 * of the tile's column strip.  Lane l holds the 8 columns c0 = first - 8 +
 * 8 l .. c0 + 7: lanes 1 to 30 produce the strip, lanes 0 and 31 are the
 * halo the horizontal lifting needs on either side.  Each lane streams down
 * its 8 columns: two input rows per step, the vertical lifting in registers
 * (the previous even row and high value are kept), then the horizontal
 * lifting of the new low and high rows across the warp (the neighbours by
 * two shuffles).  Every lane's 4 output pairs are one 4-coefficient group of
 * each band.  No shared memory, no block barrier. */
#define FV_WARPS 4
#define FV_THREADS (32 * FV_WARPS)
#define FV_COLS 240          /* level-input columns of a strip: lanes 1..30, 8 each */
#define FV_WROWPAIRS 8       /* row pairs per warp */
#define FV_ROWPAIRS (FV_WROWPAIRS * FV_WARPS)

/* Raw samples of one input row for a lane's 8 columns: 16-bit sources hold
 * two samples per word (column 2k in the low half of word k), int32 sources
 * one per word. */
template <int SRC> struct FvRaw { static const int N = 4; };
template <> struct FvRaw<SRC_I32> { static const int N = 8; };

/* raw value of column x (0 <= x < w) of a row */
template <int SRC>
DEV uint32_t raw1(const void* row, int chan, int x) {
    if (SRC == SRC_I32) return (uint32_t)((const int32_t*)row)[x];
    if (SRC == SRC_U8) return ((const uint8_t*)row)[x];
    if (SRC == SRC_U16) return ((const uint16_t*)row)[x];
    if (SRC == SRC_PK8) return ((const uint8_t*)row)[3 * x + chan];
    return ((const uint16_t*)row)[3 * x + chan];
}

template <int SRC> DEV size_t src_elem() { return SRC == SRC_I32 ? 4 : (SRC == SRC_U16 || SRC == SRC_PK16) ? 2 : 1; }

/* A strip's input: base, row pitch in bytes, width and channel, held in
 * registers for the whole strip. */
struct FvSrc {
    const char* base;
    size_t pitch;
    int w, chan;
};

/* Loads row y (in range) for the lane's columns c0 .. c0 + 7: one or two
 * vector loads when the lane's 8 columns are inside and the rows aligned
 * (`fast`; always so in a FAST strip), else one load per column with the
 * symmetric extension. */
template <int SRC, bool FAST>
DEV void fv_load(const FvSrc& S, int y, int c0, bool fast, uint32_t* r) {
    const char* row = S.base + (size_t)y * S.pitch;
    if constexpr (SRC == SRC_I32) {
        if (FAST || fast) {
            const int4 a = *(const int4*)((const int32_t*)row + c0), b = *(const int4*)((const int32_t*)row + c0 + 4);
            r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
            r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
        } else {
#pragma unroll
            for (int k = 0; k < 8; k++) r[k] = raw1<SRC>(row, 0, mirror1(c0 + k, S.w));
        }
    } else if ((FAST || fast) && SRC == SRC_U16) {
        const uint4 q = *(const uint4*)((const uint16_t*)row + c0);
        r[0] = q.x; r[1] = q.y; r[2] = q.z; r[3] = q.w;
    } else if ((FAST || fast) && SRC == SRC_U8) {
        const uint2 q = *(const uint2*)((const uint8_t*)row + c0);
        r[0] = __byte_perm(q.x, 0, 0x4140);
        r[1] = __byte_perm(q.x, 0, 0x4342);
        r[2] = __byte_perm(q.y, 0, 0x4140);
        r[3] = __byte_perm(q.y, 0, 0x4342);
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++)
            r[k] = raw1<SRC>(row, S.chan, mirror1(c0 + 2 * k, S.w)) | (raw1<SRC>(row, S.chan, mirror1(c0 + 2 * k + 1, S.w)) << 16);
    }
}

/* The scaled samples of a raw row: ((x & (2^d - 1)) << (20 - d)) - 2^19 as
 * one multiply-add (mul = 2^(20 - d)). */
template <int SRC>
DEV void fv_decode(const uint32_t* r, uint32_t mask, int32_t mul, int32_t* v) {
    if constexpr (SRC == SRC_I32) {
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = (int32_t)r[k];
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            v[2 * k] = (int32_t)(r[k] & mask) * mul - (1 << 19);
            v[2 * k + 1] = (int32_t)((r[k] >> 16) & mask) * mul - (1 << 19);
        }
    }
}

/* Horizontal lifting of one row across the warp: v holds the lane's 8
 * samples x[2j0 .. 2j0 + 7]; s / d receive its 4 low / high outputs.  The
 * right neighbour's first sample and the left neighbour's last high value
 * come by shuffles (lanes 0 and 31 get values only their neighbours use). */
DEV void fv_hlift(const int32_t* v, int32_t* s, int32_t* d) {
    const int32_t nx = __shfl_down_sync(FULL, v[0], 1);
    d[0] = v[1] - ((v[0] + v[2]) >> 1);
    d[1] = v[3] - ((v[2] + v[4]) >> 1);
    d[2] = v[5] - ((v[4] + v[6]) >> 1);
    d[3] = v[7] - ((v[6] + nx) >> 1);
    const int32_t dm = __shfl_up_sync(FULL, d[3], 1);
    s[0] = v[0] + ((dm + d[0] + 2) >> 2);
    s[1] = v[2] + ((d[0] + d[1] + 2) >> 2);
    s[2] = v[4] + ((d[1] + d[2] + 2) >> 2);
    s[3] = v[6] + ((d[2] + d[3] + 2) >> 2);
}

/* One band's output of a strip: coefficient and GCLI rows advanced by one
 * band row per step. */
struct FvBand {
    uint16_t* crow;
    uint8_t* grow;
    uint32_t pitch, gpitch;
    int w, gw;
};
DEV FvBand fv_band(const jxs_band_t& bd, int row, uint16_t* coef, uint8_t* gcli) {
    FvBand b;
    b.pitch = bd.pitch;
    b.gpitch = bd.gpitch;
    b.crow = coef + bd.coef_off + (uint64_t)row * bd.pitch;
    b.grow = gcli + bd.gcli_off + (uint64_t)row * bd.gpitch;
    b.w = (int)bd.w;
    b.gw = (int)bd.gcli_w;
    return b;
}
template <bool FAST>
DEV void fv_emit(const FvBand& b, int j, const int32_t* v) {
    if constexpr (FAST) {
        /* the whole group inside the band */
        const uint32_t c0 = to_sm(v[0]), c1 = to_sm(v[1]), c2 = to_sm(v[2]), c3 = to_sm(v[3]);
        *(uint2*)(b.crow + j) = make_uint2(c0 | (c1 << 16), c2 | (c3 << 16));
        b.grow[j >> 2] = (uint8_t)(32 - __clz((c0 | c1 | c2 | c3) & 0x7fffu));
    } else {
        emit4(BandRow{b.crow, b.grow, b.w, b.gw}, j, v[0], v[1], v[2], v[3]);
    }
}
DEV void fv_next(FvBand& b) {
    b.crow += b.pitch;
    b.grow += b.gpitch;
}

/* One warp's strip: row pairs r0 .. rend - 1 of columns c0 (this lane) of
 * job J.  FAST: the strip is away from the level's left and right edges
 * (every lane's 8 columns and every output group inside), so that no load
 * or store needs a check. */
template <int SRC, bool FAST>
DEV void fv_strip(const FwdVJob& J, int r0, int rend, int c0) {
    const int lane = threadIdx.x & 31;
    const int h = J.h, n2 = h >> 1;
    const FvSrc S{(const char*)J.src, (size_t)J.src_pitch * src_elem<SRC>(), J.w, J.chan};
    const bool fast = J.vec && c0 >= 0 && c0 + 8 <= J.w;
    const uint32_t mask = (1u << J.depth) - 1u;
    const int32_t mul = 1 << (20 - J.depth);
    /* output: pairs jj .. jj + 3 of the level's bands (one group), lanes 1..30 */
    const int jj = c0 >> 1, w1 = (J.w + 1) >> 1;
    const bool out_lane = lane >= 1 && lane <= 30 && c0 < J.w;
    FvBand bhl = fv_band(J.bands[J.b_hl], r0, J.coef, J.gcli);
    FvBand blh = fv_band(J.bands[J.b_lh], r0, J.coef, J.gcli);
    FvBand bhh = fv_band(J.bands[J.b_hh], r0, J.coef, J.gcli);
    const int ll_pitch = J.ll_pitch;
    int32_t* ll = J.ll + (size_t)r0 * ll_pitch + jj;
    const int N = FvRaw<SRC>::N;

    /* x[2 r0] and d[r0 - 1] (rows 2 r0 - 2, 2 r0 - 1 mirrored at the top);
     * rows 2 r0 + 1, 2 r0 + 2 already in flight */
    int32_t xe[8], dp[8];
    uint32_t ra[N], rb[N];
    {
        uint32_t q0[N], q1[N], q2[N];
        fv_load<SRC, FAST>(S, mirror1(2 * r0 - 2, h), c0, fast, q0);
        fv_load<SRC, FAST>(S, mirror1(2 * r0 - 1, h), c0, fast, q1);
        fv_load<SRC, FAST>(S, 2 * r0, c0, fast, q2);
        fv_load<SRC, FAST>(S, mirror1(2 * r0 + 1, h), c0, fast, ra);
        fv_load<SRC, FAST>(S, mirror1(2 * r0 + 2, h), c0, fast, rb);
        int32_t xa[8], xb[8];
        fv_decode<SRC>(q0, mask, mul, xa);
        fv_decode<SRC>(q1, mask, mul, xb);
        fv_decode<SRC>(q2, mask, mul, xe);
#pragma unroll
        for (int k = 0; k < 8; k++) dp[k] = xb[k] - ((xa[k] + xe[k]) >> 1);
    }
    for (int i = r0; i < rend; i++) {
        int32_t xo[8], xn[8];
        fv_decode<SRC>(ra, mask, mul, xo);
        fv_decode<SRC>(rb, mask, mul, xn);
        if (i + 1 < rend) {
            /* rows 2i + 3, 2i + 4, mirrored past the bottom */
            const int ya = 2 * i + 3, yb = 2 * i + 4;
            fv_load<SRC, FAST>(S, ya < h ? ya : mirror1(ya, h), c0, fast, ra);
            fv_load<SRC, FAST>(S, yb < h ? yb : mirror1(yb, h), c0, fast, rb);
        }
        /* vertical lifting: high d[i], low s[i] */
        int32_t d[8], s[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            d[k] = xo[k] - ((xe[k] + xn[k]) >> 1);
            s[k] = xe[k] + ((dp[k] + d[k] + 2) >> 2);
            xe[k] = xn[k];
            dp[k] = d[k];
        }
        /* low row i: LL (int32, next level) and HL */
        int32_t hs[4], hd[4];
        fv_hlift(s, hs, hd);
        if (out_lane) {
            fv_emit<FAST>(bhl, jj, hd);
            if (FAST || jj + 3 < w1) {
                *(int4*)ll = make_int4(hs[0], hs[1], hs[2], hs[3]);
            } else {
                for (int q = 0; q < 4; q++)
                    if (jj + q < w1) ll[q] = hs[q];
            }
        }
        /* high row i: LH and HH */
        if (i < n2) {
            fv_hlift(d, hs, hd);
            if (out_lane) {
                fv_emit<FAST>(blh, jj, hs);
                fv_emit<FAST>(bhh, jj, hd);
            }
        }
        fv_next(bhl);
        fv_next(blh);
        fv_next(bhh);
        ll += ll_pitch;
    }
}

template <int SRC, int NJ>
__global__ void __launch_bounds__(FV_THREADS) fwd_v_kernel(const __grid_constant__ FwdVLaunchN<NJ> L) {
    const FwdVJob& J = L.job[find_job<NJ>(L.job, L.njobs, (int)blockIdx.x)];
    const int u = blockIdx.x - J.first_block;
    const int ty = u / J.col_tiles, tx = u - ty * J.col_tiles;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n1 = (J.h + 1) >> 1;
    const int r0 = (ty * FV_WARPS + warp) * FV_WROWPAIRS;
    if (r0 >= n1) return; /* the whole warp */
    const int rend = min(r0 + FV_WROWPAIRS, n1);
    const int first = tx * FV_COLS, c0 = first - 8 + 8 * lane;
    /* the strip's 256 columns first - 8 .. first + 247 all inside: the
     * whole warp takes the path without checks */
    if (J.vec && first >= 8 && first + FV_COLS + 8 <= J.w) fv_strip<SRC, true>(J, r0, rend, c0);
    else fv_strip<SRC, false>(J, r0, rend, c0);
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
    (void)grid_per_sm; /* one block per tile */
    if (L->ntiles <= 0) return cudaSuccess;
    fwd_v_kernel<SRC, NJ><<<L->ntiles, FV_THREADS, 0, st>>>(*L);
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
