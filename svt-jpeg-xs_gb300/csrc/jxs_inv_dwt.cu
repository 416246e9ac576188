/*
 * Inverse 5/3 wavelet transform for sm_103a.
 *
 *  inv_h_kernel  the horizontal-only levels, deepest first: one warp per row
 *                combines the final LL band with the high band of each level
 *                (in shared memory) and writes the row of the last vertical
 *                level's low band, or, for a component without vertical
 *                levels, the output samples.
 *  inv_v_kernel  one vertical level: each warp streams down a strip of 240
 *                output columns (8 per lane, plus one halo lane on either
 *                side) for 8 row pairs.  Every step rebuilds a low row (LL +
 *                HL) and a high row (LH + HH) by inverse horizontal lifting
 *                across the warp, lifts vertically in registers and writes
 *                two rows of the next level's int32 low band or, for level 0,
 *                of the output samples with the linear output scaling fused.
 *
 * Arithmetic (bit-exact with the reference): coefficients are int16 two's
 * complement scaled by << Fq (Definitions.h:128); inverse lifting
 * x[2i] = s[i] - ((d[i-1] + d[i] + 2) >> 2), x[2i+1] = d[i] + ((x[2i] +
 * x[2i+2]) >> 1) with whole-sample symmetric extension (Idwt.c:11-53,
 * :186-263); linear output scaling v += 2^(Bw-1), v = (v + 2^(zeta-1)) >>
 * zeta, clamp to [0, 2^d - 1], zeta = Bw - d (NltDec.c:242-264).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "jxs_core.h"
#include "jxs_kernels.cuh"

#define DEV __device__ __forceinline__
#define FULL 0xffffffffu

DEV int32_t dq(int16_t c, int fq) { return (int32_t)((uint32_t)(int32_t)c << fq); }

/* linear_output_scaling (NltDec.c:242-264).  The reference adds 2^(Bw-1) in
 * int32, then rounds (v + 2^(zeta-1)) >> zeta in int64 and clamps to
 * [0, 2^d - 1].  With u = q 2^zeta + r (0 <= r < 2^zeta) the rounded value is
 * q + ((r + 2^(zeta-1)) >> zeta), so everything stays in 32 bits; the
 * constants of a launch are computed once (OutScale). */
struct OutScale {
    uint32_t half_bw, mask_z, half_z;
    int zeta, m;
};
DEV OutScale out_scale(int bw, int depth) {
    OutScale s;
    s.zeta = bw - depth;
    s.half_bw = (uint32_t)((1ull << bw) >> 1);
    s.mask_z = (1u << s.zeta) - 1u;
    s.half_z = (1u << s.zeta) >> 1;
    s.m = (1 << depth) - 1;
    return s;
}
DEV uint32_t out_sample(int32_t v, const OutScale& s) {
    const int32_t u = (int32_t)((uint32_t)v + s.half_bw);
    const int32_t t = (u >> s.zeta) + (int32_t)((((uint32_t)u & s.mask_z) + s.half_z) >> s.zeta);
    return (uint32_t)min(max(t, 0), s.m);
}

/* One band row of int16 coefficients as int32 << fq; index i < width. */
struct CoefRow {
    const int16_t* row;
    int w;
};
DEV CoefRow coef_row(const jxs_band_t& bd, int r, const int16_t* coef) {
    CoefRow c;
    c.row = coef + bd.coef_off + (uint64_t)r * bd.pitch;
    c.w = (int)bd.w;
    return c;
}

/* Inverse horizontal lifting of one row by one warp, 4 pairs per lane.
 * sget(i) / dget(i) return the low / high band value i for i in [0, n1) /
 * [0, n2) (any value outside); get4(...) variants load four at once.  Pairs
 * j in [j0, j0 + npairs) are produced (j0 a multiple of 4) and passed to
 * out(j, xe[4], xo[4]): x[2j + 2q] = xe[q], x[2j + 2q + 1] = xo[q]. */
template <typename S4, typename D4, typename S1, typename D1, typename Out>
DEV void warp_lift_inv(int j0, int npairs, int n1, int n2, S4 s4, D4 d4, S1 s1, D1 d1, Out out) {
    const int lane = threadIdx.x & 31;
    /* symmetric extension of the high band: d[-1] = d[0], d[n2] = d[n2-1] */
    auto dm = [&](int i) { return n2 == 0 ? 0 : d1(i < 0 ? 0 : (i >= n2 ? n2 - 1 : i)); };
    int32_t carry = dm(j0 - 1);
    for (int base = 0; base < npairs; base += 128) {
        const int j = j0 + base + 4 * lane;
        int32_t s[4], d[4];
        s4(j, s);
        d4(j, d);
        /* high values past the band: mirrored */
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (j + q >= n2) d[q] = dm(j + q);
        int32_t dp = __shfl_up_sync(FULL, d[3], 1);
        if (lane == 0) dp = carry;
        carry = __shfl_sync(FULL, d[3], 31);
        int32_t xe[4], xo[4];
        xe[0] = s[0] - ((dp + d[0] + 2) >> 2);
        xe[1] = s[1] - ((d[0] + d[1] + 2) >> 2);
        xe[2] = s[2] - ((d[1] + d[2] + 2) >> 2);
        xe[3] = s[3] - ((d[2] + d[3] + 2) >> 2);
        int32_t xn = __shfl_down_sync(FULL, xe[0], 1);
        if (lane == 31 && j + 4 < n1) xn = s1(j + 4) - ((d[3] + dm(j + 4) + 2) >> 2);
        /* x[n] = x[n-2] for even widths: the last even sample is its own
         * right neighbour */
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int32_t nx = (j + q + 1 >= n1) ? xe[q] : (q < 3 ? xe[q + 1] : xn);
            xo[q] = d[q] + ((xe[q] + nx) >> 1);
        }
        if (j < j0 + npairs) out(j, xe, xo);
    }
}

/* ------------------------------------------------------------------------ */
/* horizontal-only levels                                                    */
/* ------------------------------------------------------------------------ */
#define IH_MAX_WARPS 4

template <int OUT>
DEV void store_row8(const InvHJob& J, int row, int x0, int w, const int32_t* v, const OutScale& os) {
    if (OUT == 0) {
        int32_t* dst = (int32_t*)J.dst + (long long)row * J.dst_pitch + x0;
        if (x0 + 7 < w) {
            *(int4*)dst = make_int4(v[0], v[1], v[2], v[3]);
            *(int4*)(dst + 4) = make_int4(v[4], v[5], v[6], v[7]);
        } else {
            for (int q = 0; q < 8; q++)
                if (x0 + q < w) dst[q] = v[q];
        }
    } else {
        for (int q = 0; q < 8; q++) {
            if (x0 + q >= w) break;
            const uint32_t o = out_sample(v[q], os);
            const long long idx = (long long)row * J.dst_pitch + x0 + q;
            if (OUT == 1) ((uint8_t*)J.dst)[idx] = (uint8_t)o;
            else ((uint16_t*)J.dst)[idx] = (uint16_t)o;
        }
    }
}

template <int OUT, int NJ>
__global__ void __launch_bounds__(IH_MAX_WARPS * 32) inv_h_kernel(const __grid_constant__ InvHLaunchN<NJ> L) {
    extern __shared__ __align__(16) int32_t ism[];
    const InvHJob& J = L.job[find_job<NJ>(L.job, L.njobs, (int)blockIdx.x)];
    const jxs_band_t* __restrict__ bands = J.bands;
    const int16_t* __restrict__ coef = J.coef;
    const int warp = threadIdx.x >> 5;
    const int row = (blockIdx.x - J.first_block) * L.rows_per_block + warp;
    if (row >= J.h) return;
    const int fq = J.fq;
    const OutScale os = out_scale(J.bw, J.depth);
    int32_t* bufA = ism + warp * L.warp_words;
    int32_t* bufB = bufA + L.warp_words / 2;
    /* widths of every level's input, m[0] = row width */
    int m[6];
    m[0] = J.w;
    for (int e = 0; e < J.nh; e++) m[e + 1] = (m[e] + 1) >> 1;
    const CoefRow llr = coef_row(bands[J.b_ll], row, coef);
    const int32_t* cur = nullptr; /* int32 low band of the level being rebuilt (null: the LL band) */
    int32_t* nxt = bufA;
    for (int e = J.nh - 1; e >= -1; e--) {
        if (e == -1) {
            /* no horizontal-only level: the LL band is the row */
            if (J.nh > 0) break;
            const int w = J.w;
            for (int x0 = 8 * (threadIdx.x & 31); x0 < w; x0 += 256) {
                int32_t v[8];
                for (int q = 0; q < 8; q++) v[q] = x0 + q < w ? dq(llr.row[x0 + q], fq) : 0;
                store_row8<OUT>(J, row, x0, w, v, os);
            }
            break;
        }
        const int n = m[e], n1 = m[e + 1], n2 = n >> 1;
        const CoefRow hr = coef_row(bands[J.b_hf[e]], row, coef);
        const int32_t* sc = cur;
        auto s4 = [&](int j, int32_t* s) {
            if (sc) {
                for (int q = 0; q < 4; q++) s[q] = j + q < n1 ? sc[j + q] : 0;
            } else {
                for (int q = 0; q < 4; q++) s[q] = j + q < n1 ? dq(llr.row[j + q], fq) : 0;
            }
        };
        auto s1 = [&](int j) { return sc ? sc[j] : dq(llr.row[j], fq); };
        auto d4 = [&](int j, int32_t* d) {
            for (int q = 0; q < 4; q++) d[q] = j + q < n2 ? dq(hr.row[j + q], fq) : 0;
        };
        auto d1 = [&](int j) { return dq(hr.row[j], fq); };
        if (e > 0) {
            int32_t* dst = nxt;
            warp_lift_inv(0, n1, n1, n2, s4, d4, s1, d1, [&](int j, const int32_t* xe, const int32_t* xo) {
                for (int q = 0; q < 4; q++) {
                    if (2 * (j + q) < n) dst[2 * (j + q)] = xe[q];
                    if (2 * (j + q) + 1 < n) dst[2 * (j + q) + 1] = xo[q];
                }
            });
            __syncwarp();
            cur = dst;
            nxt = (dst == bufA) ? bufB : bufA;
        } else {
            warp_lift_inv(0, n1, n1, n2, s4, d4, s1, d1, [&](int j, const int32_t* xe, const int32_t* xo) {
                const int32_t v[8] = {xe[0], xo[0], xe[1], xo[1], xe[2], xo[2], xe[3], xo[3]};
                store_row8<OUT>(J, row, 2 * j, n, v, os);
            });
        }
    }
}

/* ------------------------------------------------------------------------ */
/* vertical level                                                            */
/* ------------------------------------------------------------------------ */
/* A tile is IV_COLS columns x IV_ROWPAIRS row pairs of the level's output;
 * its warps are stacked vertically, each working alone on IV_WROWPAIRS row
 * pairs of the tile's column strip.  Lane l holds the 8 output columns c0 =
 * first - 8 + 8 l .. c0 + 7 (band pairs j0 = c0 / 2 .. j0 + 3, one group of
 * every band): lanes 1 to 30 produce the strip, lanes 0 and 31 are the halo
 * the lifting needs on either side.  Each step rebuilds the next low row (LL
 * + HL) and high row (LH + HH) by inverse horizontal lifting across the warp
 * (the neighbours by two shuffles), lifts vertically in registers (the last
 * even row and high row are kept) and writes two output rows.  The band rows
 * of the step after are loaded while this one computes.  No shared memory,
 * no block barrier. */
#define IV_WARPS 4
#define IV_THREADS (32 * IV_WARPS)
#define IV_COLS 240                          /* output columns of a strip: lanes 1..30, 8 each */
#define IV_WROWPAIRS 8                       /* row pairs per warp */
#define IV_ROWPAIRS (IV_WROWPAIRS * IV_WARPS)

DEV int clampi(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }

/* Raw band values of one low or high row for the lane's pairs j0 .. j0 + 3:
 * the low-pass values (int32 low band, or int16 coefficients of the LH band)
 * and the high-pass int16 coefficients (HL or HH), two per word. */
struct IvRaw {
    int4 s;     /* int32 low band values */
    uint2 sc;   /* or LH coefficients, two per word */
    uint2 d;    /* HL / HH coefficients, two per word */
};

/* int16 values j0 .. j0 + 3 of a band row of n (> 0) coefficients, two per
 * word; indices outside [0, n) read the nearest inside (FAST: all inside) */
template <bool FAST>
DEV uint2 iv_ld_coef(const int16_t* row, int j0, int n) {
    if constexpr (FAST) {
        return *(const uint2*)(row + j0);
    } else {
        if (j0 >= 0 && j0 + 4 <= n) return *(const uint2*)(row + j0);
        uint32_t v[4];
#pragma unroll
        for (int q = 0; q < 4; q++) v[q] = (uint16_t)row[clampi(j0 + q, n)];
        return make_uint2(v[0] | (v[1] << 16), v[2] | (v[3] << 16));
    }
}
template <bool FAST>
DEV int4 iv_ld_low(const int32_t* row, int j0, int n) {
    if (FAST || (j0 >= 0 && j0 + 4 <= n)) return *(const int4*)(row + j0);
    return make_int4(row[clampi(j0, n)], row[clampi(j0 + 1, n)], row[clampi(j0 + 2, n)], row[clampi(j0 + 3, n)]);
}
/* two int16 values of a word as int32 << fq */
DEV void iv_dq2(uint32_t w, int fq, int32_t& a, int32_t& b) {
    a = (int32_t)(w << 16) >> (16 - fq);
    b = (int32_t)(w & 0xffff0000u) >> (16 - fq);
}

/* Inverse horizontal lifting of one row across the warp from the lane's low
 * values s[0..3] and high values d[0..3] (pairs j0 .. j0 + 3): x[2j] = s[j] -
 * ((d[j-1] + d[j] + 2) >> 2), x[2j+1] = d[j] + ((x[2j] + x[2j+2]) >> 1), with
 * x[2j] itself in place of x[2j+2] past the row (j + 1 >= w1).  The left
 * neighbour's last high value and the right neighbour's first even sample
 * come by shuffles.  x receives the lane's 8 samples. */
template <bool FAST>
DEV void iv_hrow(const int32_t* s, const int32_t* d, int j0, int w1, int32_t* x) {
    const int32_t dm = __shfl_up_sync(FULL, d[3], 1);
    const int32_t e0 = s[0] - ((dm + d[0] + 2) >> 2);
    const int32_t e1 = s[1] - ((d[0] + d[1] + 2) >> 2);
    const int32_t e2 = s[2] - ((d[1] + d[2] + 2) >> 2);
    const int32_t e3 = s[3] - ((d[2] + d[3] + 2) >> 2);
    const int32_t en = __shfl_down_sync(FULL, e0, 1);
    x[0] = e0;
    x[1] = d[0] + ((e0 + (FAST || j0 + 1 < w1 ? e1 : e0)) >> 1);
    x[2] = e1;
    x[3] = d[1] + ((e1 + (FAST || j0 + 2 < w1 ? e2 : e1)) >> 1);
    x[4] = e2;
    x[5] = d[2] + ((e2 + (FAST || j0 + 3 < w1 ? e3 : e2)) >> 1);
    x[6] = e3;
    x[7] = d[3] + ((e3 + (FAST || j0 + 4 < w1 ? en : e3)) >> 1);
}

/* linear_output_scaling of one sample with zeta >= 2: the rounded value
 * (u + 2^(zeta-1)) >> zeta (u = v + 2^(Bw-1), wrapping like the reference's
 * int32 addition) equals ((u >> 1) + 2^(zeta-2)) >> (zeta-1), which cannot
 * overflow; then the clamp to [0, 2^d - 1] */
struct OutScale8 {
    uint32_t half_bw;
    int32_t q;
    int zm1, m, general;
    OutScale os;
};
DEV OutScale8 out_scale8(int bw, int depth) {
    OutScale8 s;
    s.os = out_scale(bw, depth);
    s.half_bw = s.os.half_bw;
    s.general = s.os.zeta < 2;
    s.zm1 = s.os.zeta - 1;
    s.q = s.general ? 0 : 1 << (s.os.zeta - 2);
    s.m = s.os.m;
    return s;
}
DEV uint32_t out_sample8(int32_t v, const OutScale8& s) {
    if (s.general) return out_sample(v, s.os);
    const int32_t u = (int32_t)((uint32_t)v + s.half_bw);
    return (uint32_t)min(max(((u >> 1) + s.q) >> s.zm1, 0), s.m);
}

/* One output row of the lane's 8 columns c0 .. c0 + 7 (c0 < w): vector
 * stores where the row is aligned and all 8 are inside. */
template <int OUT, bool FAST>
DEV void iv_store8(const InvVJob& J, int y, int c0, int w, bool vec, const int32_t* x, const OutScale8& os) {
    const bool all8 = FAST || (vec && c0 + 8 <= w);
    if constexpr (OUT == 0) {
        int32_t* d = (int32_t*)J.dst + (size_t)y * J.dst_pitch + c0;
        if (all8) {
            *(int4*)d = make_int4(x[0], x[1], x[2], x[3]);
            *(int4*)(d + 4) = make_int4(x[4], x[5], x[6], x[7]);
        } else {
            for (int q = 0; q < 8; q++)
                if (c0 + q < w) d[q] = x[q];
        }
    } else {
        uint32_t o[8];
#pragma unroll
        for (int q = 0; q < 8; q++) o[q] = out_sample8(x[q], os);
        if constexpr (OUT == 1) {
            uint8_t* d = (uint8_t*)J.dst + (size_t)y * J.dst_pitch + c0;
            if (all8) {
                *(uint2*)d = make_uint2(o[0] | (o[1] << 8) | (o[2] << 16) | (o[3] << 24),
                                        o[4] | (o[5] << 8) | (o[6] << 16) | (o[7] << 24));
            } else {
                for (int q = 0; q < 8; q++)
                    if (c0 + q < w) d[q] = (uint8_t)o[q];
            }
        } else {
            uint16_t* d = (uint16_t*)J.dst + (size_t)y * J.dst_pitch + c0;
            if (all8) {
                *(uint4*)d = make_uint4(o[0] | (o[1] << 16), o[2] | (o[3] << 16), o[4] | (o[5] << 16), o[6] | (o[7] << 16));
            } else {
                for (int q = 0; q < 8; q++)
                    if (c0 + q < w) d[q] = (uint16_t)o[q];
            }
        }
    }
}

/* One warp's strip: row pairs r0 .. rend - 1 of output columns c0 (this
 * lane) of job J.  FAST: the strip is away from the level's left and right
 * edges and its rows are aligned, so that no load or store needs a check. */
template <int OUT, bool FAST>
DEV void iv_strip(const InvVJob& J, int r0, int rend, int c0, bool vec) {
    const int lane = threadIdx.x & 31;
    const int w = J.w, h = J.h, fq = J.fq;
    const int n1 = (h + 1) >> 1, n2 = h >> 1;
    const int w1 = (w + 1) >> 1, w2 = w >> 1;
    const int j0 = c0 >> 1;
    const bool out_lane = lane >= 1 && lane <= 30 && c0 < w;
    const jxs_band_t& bHL = J.bands[J.b_hl];
    const jxs_band_t& bLH = J.bands[J.b_lh];
    const jxs_band_t& bHH = J.bands[J.b_hh];
    const int16_t* hl = J.coef + bHL.coef_off;
    const int16_t* lh = J.coef + bLH.coef_off;
    const int16_t* hh = J.coef + bHH.coef_off;
    const uint32_t hl_p = bHL.pitch, lh_p = bLH.pitch, hh_p = bHH.pitch;
    const int32_t* llb = J.ll;
    const int ll_p = J.ll_pitch;
    const OutScale8 os = out_scale8(J.bw, J.depth);
    /* raw loads of low row i (i < n1) and high row i (clamped into [0, n2),
     * n2 > 0) */
    auto ld_low = [&](int i, IvRaw& r) {
        r.s = iv_ld_low<FAST>(llb + (size_t)i * ll_p, j0, w1);
        r.d = w2 ? iv_ld_coef<FAST>(hl + (size_t)i * hl_p, j0, w2) : make_uint2(0u, 0u);
    };
    auto ld_high = [&](int i, IvRaw& r) {
        i = clampi(i, n2);
        r.sc = iv_ld_coef<FAST>(lh + (size_t)i * lh_p, j0, w1);
        r.d = w2 ? iv_ld_coef<FAST>(hh + (size_t)i * hh_p, j0, w2) : make_uint2(0u, 0u);
    };
    auto build = [&](const IvRaw& r, bool low, int32_t* x) {
        int32_t sv[4], dv[4];
        if (low) {
            sv[0] = r.s.x; sv[1] = r.s.y; sv[2] = r.s.z; sv[3] = r.s.w;
        } else {
            iv_dq2(r.sc.x, fq, sv[0], sv[1]);
            iv_dq2(r.sc.y, fq, sv[2], sv[3]);
        }
        iv_dq2(r.d.x, fq, dv[0], dv[1]);
        iv_dq2(r.d.y, fq, dv[2], dv[3]);
        iv_hrow<FAST>(sv, dv, j0, w1, x);
    };
    /* x[2 r0] = low[r0] - ((high[r0 - 1] + high[r0] + 2) >> 2) */
    int32_t xe[8], hc[8];
    IvRaw nl, nh; /* the next step's low and high rows, in flight */
    {
        IvRaw a, b, c;
        ld_low(r0, a);
        if (n2) {
            ld_high(r0 - 1, b);
            ld_high(r0, c);
        }
        if (r0 + 1 < n1 && 2 * r0 + 2 < h) {
            ld_low(r0 + 1, nl);
            if (n2) ld_high(r0 + 1, nh);
        }
        int32_t hp[8];
        build(a, true, xe);
        if (n2) {
            build(b, false, hp);
            build(c, false, hc);
        } else {
#pragma unroll
            for (int k = 0; k < 8; k++) hp[k] = hc[k] = 0;
        }
#pragma unroll
        for (int k = 0; k < 8; k++) xe[k] -= (hp[k] + hc[k] + 2) >> 2;
    }
    for (int i = r0; i < rend; i++) {
        const int y = 2 * i;
        int32_t xo[8], xn[8];
        if (y + 2 < h) {
            /* x[2i + 2] from the next low and high rows */
            int32_t hn[8];
            build(nl, true, xn);
            if (n2) {
                build(nh, false, hn);
            } else {
#pragma unroll
                for (int k = 0; k < 8; k++) hn[k] = 0;
            }
            if (i + 1 < rend && y + 4 < h) {
                ld_low(i + 2, nl);
                if (n2) ld_high(i + 2, nh);
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                xn[k] -= (hc[k] + hn[k] + 2) >> 2;
                xo[k] = hc[k] + ((xe[k] + xn[k]) >> 1);
                hc[k] = hn[k];
            }
        } else {
            /* the last even row is its own lower neighbour */
#pragma unroll
            for (int k = 0; k < 8; k++) {
                xn[k] = xe[k];
                xo[k] = hc[k] + xe[k];
            }
        }
        if (out_lane) {
            iv_store8<OUT, FAST>(J, y, c0, w, vec, xe, os);
            if (y + 1 < h) iv_store8<OUT, FAST>(J, y + 1, c0, w, vec, xo, os);
        }
#pragma unroll
        for (int k = 0; k < 8; k++) xe[k] = xn[k];
    }
}

template <int OUT, int NJ>
__global__ void __launch_bounds__(IV_THREADS) inv_v_kernel(const __grid_constant__ InvVLaunchN<NJ> L) {
    const InvVJob& J = L.job[find_job<NJ>(L.job, L.njobs, (int)blockIdx.x)];
    const int t = blockIdx.x - J.first_block;
    const int ty = t / J.col_tiles, tx = t - ty * J.col_tiles;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n1 = (J.h + 1) >> 1;
    const int r0 = (ty * IV_WARPS + warp) * IV_WROWPAIRS;
    if (r0 >= n1) return; /* the whole warp */
    const int rend = min(r0 + IV_WROWPAIRS, n1);
    const int first = tx * IV_COLS, c0 = first - 8 + 8 * lane;
    const int esz = OUT == 0 ? 4 : OUT;
    const bool vec = ((uintptr_t)J.dst & 15) == 0 && (((size_t)J.dst_pitch * esz) & 15) == 0;
    /* the strip's 256 columns first - 8 .. first + 247 (band pairs up to
     * first / 2 + 123) all inside, aligned rows: the whole warp takes the
     * path without checks */
    if (vec && first >= 8 && first + IV_COLS + 8 <= J.w) iv_strip<OUT, true>(J, r0, rend, c0, vec);
    else iv_strip<OUT, false>(J, r0, rend, c0, vec);
}

/* ------------------------------------------------------------------------ */
/* launchers                                                                 */
/* ------------------------------------------------------------------------ */
extern "C" int jxs_inv_v_tile_rows(void) { return IV_ROWPAIRS; }
extern "C" int jxs_inv_v_tile_cols(void) { return IV_COLS; }
extern "C" int jxs_inv_h_max_rows_per_block(void) { return IH_MAX_WARPS; }

template <int OUT, int NJ>
static cudaError_t launch_iv(const InvVLaunchN<NJ>* L, int nblocks, cudaStream_t st) {
    if (nblocks <= 0) return cudaSuccess;
    inv_v_kernel<OUT, NJ><<<nblocks, IV_THREADS, 0, st>>>(*L);
    return cudaGetLastError();
}

extern "C" cudaError_t jxs_launch_inv_v(const InvVLaunch* L, int out_kind, int nblocks, cudaStream_t st) {
    if (out_kind == 0) return launch_iv<0, JXS_MAXC>(L, nblocks, st);
    if (out_kind == 1) return launch_iv<1, JXS_MAXC>(L, nblocks, st);
    return launch_iv<2, JXS_MAXC>(L, nblocks, st);
}
extern "C" cudaError_t jxs_launch_inv_v_batch(const InvVLaunchB* L, int out_kind, int nblocks, cudaStream_t st) {
    if (out_kind == 0) return launch_iv<0, JXS_BATCH_JOBS>(L, nblocks, st);
    if (out_kind == 1) return launch_iv<1, JXS_BATCH_JOBS>(L, nblocks, st);
    return launch_iv<2, JXS_BATCH_JOBS>(L, nblocks, st);
}

template <int OUT, int NJ>
static cudaError_t launch_ih(const InvHLaunchN<NJ>* L, int nblocks, cudaStream_t st) {
    const size_t smem = (size_t)L->warp_words * L->rows_per_block * sizeof(int32_t);
    static std::atomic<int> attr[JXS_MAX_DEV];
    cudaError_t e = jxs_smem_attr(inv_h_kernel<OUT, NJ>, (int)smem, attr);
    if (e != cudaSuccess) return e;
    if (nblocks <= 0) return cudaSuccess;
    inv_h_kernel<OUT, NJ><<<nblocks, L->rows_per_block * 32, smem, st>>>(*L);
    return cudaGetLastError();
}

extern "C" cudaError_t jxs_launch_inv_h(const InvHLaunch* L, int out_kind, int nblocks, cudaStream_t st) {
    if (out_kind == 0) return launch_ih<0, JXS_MAXC>(L, nblocks, st);
    if (out_kind == 1) return launch_ih<1, JXS_MAXC>(L, nblocks, st);
    return launch_ih<2, JXS_MAXC>(L, nblocks, st);
}
extern "C" cudaError_t jxs_launch_inv_h_batch(const InvHLaunchB* L, int out_kind, int nblocks, cudaStream_t st) {
    if (out_kind == 0) return launch_ih<0, JXS_BATCH_JOBS>(L, nblocks, st);
    if (out_kind == 1) return launch_ih<1, JXS_BATCH_JOBS>(L, nblocks, st);
    return launch_ih<2, JXS_BATCH_JOBS>(L, nblocks, st);
}

/* ------------------------------------------------------------------------ */
/* Colour transform and output non-linearity                                 */
/* ------------------------------------------------------------------------ */
/* Streams with a colour transform (Cpih = 1) or an NLT marker: the last
 * inverse level writes int32 planes, and this kernel turns them into
 * samples.  Cpih = 1: the inverse reversible colour transform of
 * components 0-2 (inverse_rct, Mct.c:137-153); then every component's
 * output scaling (nlt_inverse_transform_line_*, NltDec.c:22-194, 366-406):
 * linear, quadratic (Tnlt = 1) or extended (Tnlt = 2), with the first
 * component's depth.  One thread per sample column x, rows over grid.y. */
DEV int32_t nlt_clamp64(int64_t v, int32_t m) { return (int32_t)(v > m ? m : v < 0 ? 0 : v); }

DEV int32_t nlt_sample(const NltOut& P, int64_t v) {
    const int32_t bw = P.bw, depth = P.depth, m = (1 << depth) - 1, clampv = (1 << bw) - 1;
    v += ((int64_t)1 << bw) >> 1;
    if (P.tnlt == 1) {
        const int32_t zeta = 2 * bw - depth;
        const int64_t q = (int64_t)nlt_clamp64(v, clampv);
        return nlt_clamp64(((q * q + (((int64_t)1 << zeta) >> 1)) >> zeta) + P.dco, m);
    }
    if (P.tnlt == 2) {
        const int32_t zeta = 2 * bw - depth;
        if (v < P.t1) {
            const int64_t q = nlt_clamp64((int64_t)P.b1 - v, clampv);
            v = P.a1 - q * q;
        } else if (v < P.t2) {
            v = v * ((int64_t)1 << (bw - P.e)) + P.b2;
        } else {
            const int64_t q = nlt_clamp64(v - P.b3, clampv);
            v = P.a3 + q * q;
        }
        return nlt_clamp64((v + (((int64_t)1 << zeta) >> 1)) >> zeta, m);
    }
    const int32_t zeta = bw - depth;
    return nlt_clamp64((v + (((int64_t)1 << zeta) >> 1)) >> zeta, m);
}

__global__ void __launch_bounds__(256) nlt_out_kernel(const __grid_constant__ NltOut P) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    int32_t v[JXS_MAXC];
#pragma unroll
    for (int k = 0; k < JXS_MAXC; k++)
        v[k] = (k < P.nc && x < P.w[k] && y < P.h[k]) ? P.in[k][(size_t)y * P.in_pitch[k] + x] : 0;
    if (P.cpih == 1 && x < P.w[0] && y < P.h[0]) {
        const int32_t o1 = v[0] - ((v[1] + v[2]) >> 2);
        const int32_t o0 = o1 + v[2], o2 = o1 + v[1];
        v[0] = o0;
        v[1] = o1;
        v[2] = o2;
    }
#pragma unroll
    for (int k = 0; k < JXS_MAXC; k++) {
        if (k >= P.nc || x >= P.w[k] || y >= P.h[k]) continue;
        const int32_t o = nlt_sample(P, v[k]);
        if (P.bps == 1) ((uint8_t*)P.out[k])[(size_t)y * P.out_pitch[k] + x] = (uint8_t)o;
        else ((uint16_t*)P.out[k])[(size_t)y * P.out_pitch[k] + x] = (uint16_t)o;
    }
}

extern "C" cudaError_t jxs_launch_nlt_out(const NltOut* P, cudaStream_t st) {
    int wmax = 1, hmax = 1;
    for (int k = 0; k < P->nc; k++) {
        wmax = max(wmax, P->w[k]);
        hmax = max(hmax, P->h[k]);
    }
    nlt_out_kernel<<<dim3((unsigned)((wmax + 255) / 256), (unsigned)hmax), 256, 0, st>>>(*P);
    return cudaGetLastError();
}

/* Inverse Star-Tetrix (Cpih = 3; ISO/IEC 21122-1 Annex F, Mct.c:14-136) on
 * the int32 planes of the four components, before nlt_out_kernel.  Each of
 * the four steps updates components that none of its reads touch (the
 * access function always lands on another component), so one launch per
 * step is exact in any thread order:
 *   step 0  average: c0 -= (four diagonal neighbours) >> 3
 *   step 1  delta:   c3 += (four diagonal neighbours) >> 2
 *   step 2  Y:       c0, c3 -= (2^e2 (horizontal pair) + 2^e1 (vertical pair)) >> 3
 *   step 3  CbCr:    c1, c2 += (four direct neighbours) >> 2
 * then components 0 <-> 2 and 1 <-> 3 (done by the caller's plane order). */
__constant__ int8_t c_st_disp[2][4][2] = {{{0, 1}, {1, 1}, {0, 0}, {1, 0}}, {{1, 1}, {0, 1}, {1, 0}, {0, 0}}}; /* Table F.10 */
__constant__ uint8_t c_st_comp[2][2][2] = {{{2, 0}, {3, 1}}, {{3, 1}, {2, 0}}};                            /* Table F.11 */

/* Table F.12: mirrored at the picture edges and, for Cf = 3, within a line
 * pair */
DEV int32_t st_access(const StParams& P, int c, int x, int y, int rx, int ry) {
    const int dx = c_st_disp[P.ct][c][0], dy = c_st_disp[P.ct][c][1];
    if (2 * x + rx + dx < 0 || 2 * x + rx + dx >= 2 * P.w) rx = -rx;
    if ((P.cf == 3 && (ry + dy < 0 || ry + dy > 1)) || 2 * y + ry + dy < 0 || 2 * y + ry + dy >= 2 * P.h) ry = -ry;
    const int xx = (2 * x + rx + dx) / 2, yy = (2 * y + ry + dy) / 2;
    return P.c[c_st_comp[P.ct][(2 + rx + dx) % 2][(2 + ry + dy) % 2]][(long long)yy * P.pitch + xx];
}

/* products in 32-bit wrap-around arithmetic like the reference's int */
DEV int32_t st_mul(int32_t k, int32_t v) { return (int32_t)((uint32_t)k * (uint32_t)v); }

__global__ void __launch_bounds__(256) star_tetrix_kernel(const __grid_constant__ StParams P, int step) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= P.w || y >= P.h) return;
    const long long i = (long long)y * P.pitch + x;
#define ACC(c, rx, ry) st_access(P, c, x, y, rx, ry)
    if (step == 0) {
        P.c[0][i] -= (ACC(0, -1, -1) + ACC(0, 1, -1) + ACC(0, -1, 1) + ACC(0, 1, 1)) >> 3;
    } else if (step == 1) {
        P.c[3][i] += (ACC(3, -1, -1) + ACC(3, 1, -1) + ACC(3, -1, 1) + ACC(3, 1, 1)) >> 2;
    } else if (step == 2) {
        const int32_t k1 = 1 << P.e1, k2 = 1 << P.e2;
        P.c[0][i] -= (st_mul(k2, ACC(0, -1, 0) + ACC(0, 1, 0)) + st_mul(k1, ACC(0, 0, -1) + ACC(0, 0, 1))) >> 3;
        P.c[3][i] -= (st_mul(k2, ACC(3, 0, -1) + ACC(3, 0, 1)) + st_mul(k1, ACC(3, -1, 0) + ACC(3, 1, 0))) >> 3;
    } else {
        P.c[1][i] += (ACC(1, -1, 0) + ACC(1, 1, 0) + ACC(1, 0, -1) + ACC(1, 0, 1)) >> 2;
        P.c[2][i] += (ACC(2, -1, 0) + ACC(2, 1, 0) + ACC(2, 0, -1) + ACC(2, 0, 1)) >> 2;
    }
#undef ACC
}

extern "C" cudaError_t jxs_launch_star_tetrix(const StParams* P, cudaStream_t st) {
    const dim3 grid((unsigned)((P->w + 255) / 256), (unsigned)P->h);
    for (int step = 0; step < 4; step++) {
        star_tetrix_kernel<<<grid, 256, 0, st>>>(*P, step);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
