/*
 * Decoder kernels for sm_103a.
 *
 *  unpack_kernel   per precinct row: copies the precinct into shared memory,
 *                  parses its header and packet headers, decodes GCLIs (raw
 *                  nibbles or unary codes found by a block-wide scan of zero
 *                  bits), then all data groups at prefix-summed bit offsets,
 *                  dequantizes and writes int16 coefficients
 *                  (unpack_precinct, Packing.c:513-868; Dequant.c:9-57;
 *                  Precinct.c:9-29).
 *  inv_dwt_kernel  one vertical 5/3 level per launch: rebuilds the rows it
 *                  needs from the bands (inverse horizontal lifting in shared
 *                  memory), lifts vertically and writes the next level's
 *                  low band or, for the first level, the output samples with
 *                  the linear output scaling fused (Idwt.c:11-287,
 *                  DwtDecoder.c:322-406, NltDec.c:242-264).
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "jxs_core.h"
#include "jxs_kernels.cuh"

#define DEV __device__ __forceinline__
#define UK_THREADS 256
#define UK_MAXBL 80

struct DecBL {
    uint16_t fb;
    uint8_t line, pk, t, mode, raw;
    uint32_t row, gcli_w, sig_w, w;
    uint32_t g0, s0;
    uint32_t sig_pos, gcli_pos; /* bit positions inside the precinct */
};

struct DecPk {
    uint32_t gcli_pos, gcli_bits, data_pos, data_bits;
    uint32_t b_beg, b_end, g_beg, g_end;
    uint32_t raw;
};

DEV uint32_t bit_at(const uint8_t* p, uint32_t pos) { return (p[pos >> 3] >> (7 - (pos & 7))) & 1u; }

/* Up to 64 bits starting at `pos` (MSB first). Reads bytes up to pos/8 + 8. */
DEV uint64_t bits64(const uint8_t* p, uint32_t pos, uint32_t n) {
    const uint32_t b = pos >> 3, sh = pos & 7;
    uint64_t v = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) v = (v << 8) | p[b + k];
    uint64_t extra = p[b + 8];
    v = (v << sh) | (extra >> (8 - sh) & ((1u << sh) - 1));
    return n == 64 ? v : (v >> (64 - n));
}

DEV int find_dbl_by_group(const DecBL* bl, int n, uint32_t g) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (bl[mid].g0 <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

DEV int find_dbl_by_sig(const DecBL* bl, int n, uint32_t s) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (bl[mid].s0 <= s) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

/* Block-wide exclusive scan of one counter; returns the block total. */
DEV uint32_t block_scan1(uint32_t a, uint32_t* ea, uint32_t* ws) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t ia = a;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, ia, o);
        if (lane >= o) ia += t;
    }
    if (lane == 31) ws[warp] = ia;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = lane < nw ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += t;
        }
        if (lane < nw) ws[lane] = v;
    }
    __syncthreads();
    *ea = (warp ? ws[warp - 1] : 0) + ia - a;
    const uint32_t total = ws[nw - 1];
    __syncthreads();
    return total;
}

/* dynamic shared memory: [precinct bytes (cap_bytes + 16)] [GCLI per group (cap_groups)]
 * [significance flag per significance group (cap_groups)] [zero positions (4 B x cap_groups)] */
__global__ void __launch_bounds__(UK_THREADS) unpack_kernel(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs,
                                                            const uint32_t* __restrict__ prec_off, int16_t* __restrict__ coef,
                                                            uint32_t cap_bytes, uint32_t cap_groups, int* status) {
    extern __shared__ __align__(16) uint8_t dsm[];
    uint8_t* pbuf = dsm;
    uint8_t* gcl = dsm + cap_bytes + 16;
    uint8_t* sflag = gcl + cap_groups;
    uint32_t* zpos = (uint32_t*)(((uintptr_t)(sflag + cap_groups) + 15) & ~(uintptr_t)15);
    __shared__ DecBL bl[UK_MAXBL];
    __shared__ DecPk pk[JXS_MAXPK];
    __shared__ uint32_t pk_pref[JXS_MAXPK];
    __shared__ uint32_t ws[UK_THREADS / 32];
    __shared__ int s_nbl, s_err;
    __shared__ uint32_t s_total, s_ng, s_ns;

    const int p = blockIdx.x;
    const int last = (p + 1 >= (int)cfg->np);
    if (threadIdx.x == 0) s_err = *(volatile int*)status;
    __syncthreads();
    if (s_err) return; /* the precinct offsets could not be found */
    const uint8_t* src = bs + prec_off[p];
    if (threadIdx.x == 0) {
        s_err = 0;
        const uint32_t lprc = ((uint32_t)src[0] << 16) | ((uint32_t)src[1] << 8) | src[2];
        s_total = cfg->prec_hdr_bytes + lprc;
        if (lprc > JXS_PREC_MAX_BYTES || s_total > cap_bytes) s_err = JXS_E_DEC_BITSTREAM;
    }
    __syncthreads();
    if (s_err) {
        if (threadIdx.x == 0) JXS_STATUS_SET(status, s_err);
        return;
    }
    const uint32_t total = s_total;
    for (uint32_t i = threadIdx.x; i < total; i += blockDim.x) pbuf[i] = src[i];
    for (uint32_t i = threadIdx.x; i < 16; i += blockDim.x) pbuf[total + i] = 0;
    __syncthreads();

    if (threadIdx.x == 0) {
        int err = 0;
        const uint8_t q = pbuf[3], r = pbuf[4];
        const uint32_t lprc = total - cfg->prec_hdr_bytes;
        /* band coding modes D[p,b], 2 bits per existing band */
        uint8_t mode[JXS_MAXBL];
        uint32_t pos = 40;
        for (uint32_t gb = 0; gb < cfg->nbands_all; gb++) {
            const int fb = cfg->g2f[gb];
            if (fb == JXS_NOBAND) continue;
            mode[fb] = (uint8_t)((pbuf[pos >> 3] >> (6 - (pos & 7))) & 3);
            pos += 2;
            if (mode[fb] & 1) err = JXS_E_DEC_BITSTREAM; /* vertical prediction is not part of this decoder */
        }
        /* band lines in packet order */
        int n = 0;
        uint32_t g0 = 0, s0 = 0;
        for (uint32_t k = 0; k < cfg->npk; k++) {
            const uint32_t l = cfg->pk[k].line;
            for (uint32_t gb = cfg->pk[k].bs; gb < cfg->pk[k].be; gb++) {
                const int fb = cfg->g2f[gb];
                const jxs_band_t& bd = cfg->band[fb];
                if (l >= (last ? bd.last_lines : bd.lines)) continue;
                DecBL& b = bl[n++];
                b.fb = (uint16_t)fb; b.line = (uint8_t)l; b.pk = (uint8_t)k;
                b.t = jxs_truncation(bd.gain, bd.prio, q, r);
                b.mode = mode[fb];
                b.row = (uint32_t)p * bd.lines + l;
                b.gcli_w = bd.gcli_w; b.sig_w = bd.sig_w; b.w = bd.w;
                b.g0 = g0; b.s0 = s0;
                g0 += bd.gcli_w;
                s0 += bd.sig_w;
            }
        }
        s_nbl = n;
        s_ng = g0;
        s_ns = s0;
        if (g0 > cap_groups) err = JXS_E_DEC_INTERNAL;
        /* packet headers and sub-packet positions */
        const int long_hdr = cfg->lh || !cfg->short_hdr;
        int64_t left = (int64_t)lprc * 8;
        uint32_t bpos = cfg->prec_hdr_bytes; /* bytes */
        int b = 0;
        for (uint32_t k = 0; k < cfg->npk && !err; k++) {
            DecPk& P = pk[k];
            P.b_beg = P.b_end = b;
            P.g_beg = P.g_end = (b < n) ? bl[b].g0 : g0;
            P.gcli_bits = P.data_bits = 0;
            P.raw = 0;
            if (b >= n || bl[b].pk != k) continue;
            int be = b;
            while (be < n && bl[be].pk == k) be++;
            const uint32_t hb = long_hdr ? 7 : 5;
            left -= hb * 8;
            if (left < 0) { err = JXS_E_DEC_BITSTREAM; break; }
            const uint8_t* h = pbuf + bpos;
            uint32_t raw, dlen, glen, slen;
            if (long_hdr) {
                raw = h[0] >> 7;
                dlen = ((uint32_t)(h[0] & 0x7f) << 13) | ((uint32_t)h[1] << 5) | (h[2] >> 3);
                glen = ((uint32_t)(h[2] & 7) << 17) | ((uint32_t)h[3] << 9) | ((uint32_t)h[4] << 1) | (h[5] >> 7);
                slen = ((uint32_t)(h[5] & 0x7f) << 8) | h[6];
            } else {
                raw = h[0] >> 7;
                dlen = ((uint32_t)(h[0] & 0x7f) << 8) | h[1];
                glen = ((uint32_t)h[2] << 5) | (h[3] >> 3);
                slen = ((uint32_t)(h[3] & 7) << 8) | h[4];
            }
            bpos += hb;
            if ((uint64_t)left < ((uint64_t)dlen + glen + slen) * 8) { err = JXS_E_DEC_BITSTREAM; break; }
            P.raw = raw;
            if (raw) {
                uint32_t gp = bpos * 8, need = 0;
                for (int x = b; x < be; x++) {
                    bl[x].raw = 1;
                    bl[x].gcli_pos = gp;
                    gp += 4 * bl[x].gcli_w;
                    need += 4 * bl[x].gcli_w;
                }
                left -= need;
                if (left < 0 || need > glen * 8) { err = JXS_E_DEC_BITSTREAM; break; }
                left -= (int64_t)glen * 8 - need; /* skipped padding inside the sub-packet */
            } else {
                uint32_t sp = bpos * 8, sbits = 0;
                for (int x = b; x < be; x++) {
                    bl[x].raw = 0;
                    bl[x].sig_pos = sp;
                    if (bl[x].mode & 2) {
                        sp += bl[x].sig_w;
                        sbits += bl[x].sig_w;
                    }
                }
                left -= sbits;
                if (left < 0) { err = JXS_E_DEC_BITSTREAM; break; }
                left -= left & 7;
                bpos += (sbits + 7) >> 3;
                left -= (int64_t)glen * 8;
            }
            P.gcli_pos = bpos * 8;
            P.gcli_bits = glen * 8;
            bpos += glen;
            P.data_pos = bpos * 8;
            P.data_bits = dlen * 8;
            bpos += dlen;
            left -= (int64_t)dlen * 8;
            bpos += cfg->fs ? slen : 0;
            if (cfg->fs) err = JXS_E_DEC_BITSTREAM; /* separate sign sub-packets are not part of this decoder */
            if (left < 0 || bpos > total) { err = JXS_E_DEC_BITSTREAM; break; }
            P.b_beg = b; P.b_end = be;
            P.g_beg = bl[b].g0;
            P.g_end = (be < n) ? bl[be].g0 : g0;
            b = be;
        }
        s_err = err;
    }
    __syncthreads();
    if (s_err) {
        if (threadIdx.x == 0) JXS_STATUS_SET(status, s_err);
        return;
    }
    const int nbl = s_nbl;
    const uint32_t G = s_ng;
    /* significance flags (1 = group insignificant) and raw GCLIs */
    for (uint32_t s = threadIdx.x; s < s_ns; s += blockDim.x) {
        const DecBL& B = bl[find_dbl_by_sig(bl, nbl, s)];
        sflag[s] = (!B.raw && (B.mode & 2)) ? (uint8_t)bit_at(pbuf, B.sig_pos + (s - B.s0)) : 0;
    }
    for (uint32_t g = threadIdx.x; g < G; g += blockDim.x) {
        const DecBL& B = bl[find_dbl_by_group(bl, nbl, g)];
        if (B.raw) {
            const uint32_t pos = B.gcli_pos + 4 * (g - B.g0);
            gcl[g] = (uint8_t)((pbuf[pos >> 3] >> (4 - (pos & 7))) & 15);
        }
    }
    __syncthreads();
    /* unary-coded GCLIs, one packet at a time: codeword j ends at the j-th
     * zero bit of the sub-packet (unpack_pred_zero_gclis_*, Packing.c:435-511) */
    for (uint32_t k = 0; k < cfg->npk; k++) {
        const DecPk P = pk[k];
        if (P.b_beg == P.b_end || P.raw) continue;
        /* codeword index of each coded group */
        const uint32_t ng = P.g_end - P.g_beg;
        const uint32_t per = (ng + blockDim.x - 1) / blockDim.x;
        const uint32_t a = min(ng, threadIdx.x * per), e = min(ng, a + per);
        uint32_t cnt = 0;
        int bidx = a < e ? find_dbl_by_group(bl, nbl, P.g_beg + a) : 0;
        for (uint32_t i = a; i < e; i++) {
            const uint32_t g = P.g_beg + i;
            while (bidx + 1 < nbl && bl[bidx + 1].g0 <= g) bidx++;
            const DecBL& B = bl[bidx];
            cnt += !((B.mode & 2) && sflag[B.s0 + ((g - B.g0) >> 3)]);
        }
        uint32_t cw0;
        const uint32_t ncw = block_scan1(cnt, &cw0, ws);
        /* zero positions */
        const uint32_t nbits = P.gcli_bits, nwords = (nbits + 31) >> 5;
        const uint32_t wper = (nwords + blockDim.x - 1) / blockDim.x;
        const uint32_t wa = min(nwords, threadIdx.x * wper), we = min(nwords, wa + wper);
        uint32_t zc = 0;
        for (uint32_t wi = wa; wi < we; wi++) {
            const uint32_t bit0 = P.gcli_pos + 32 * wi;
            uint32_t word = (uint32_t)(bits64(pbuf, bit0, 32));
            const uint32_t valid = min(32u, nbits - 32 * wi);
            uint32_t z = ~word;
            if (valid < 32) z &= ~(0xffffffffu >> valid);
            zc += __popc(z);
        }
        uint32_t z0;
        const uint32_t nz = block_scan1(zc, &z0, ws);
        for (uint32_t wi = wa; wi < we; wi++) {
            const uint32_t bit0 = P.gcli_pos + 32 * wi;
            uint32_t word = (uint32_t)(bits64(pbuf, bit0, 32));
            const uint32_t valid = min(32u, nbits - 32 * wi);
            uint32_t z = ~word;
            if (valid < 32) z &= ~(0xffffffffu >> valid);
            while (z) {
                const uint32_t lead = __clz(z);
                if (z0 < ncw) zpos[z0] = 32 * wi + lead;
                z0++;
                z &= ~(0x80000000u >> lead);
            }
        }
        if (nz < ncw) {
            if (threadIdx.x == 0) JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
            return; /* uniform across the block: nz and ncw are block totals */
        }
        __syncthreads();
        bidx = a < e ? find_dbl_by_group(bl, nbl, P.g_beg + a) : 0;
        uint32_t cw = cw0;
        int bad = 0;
        for (uint32_t i = a; i < e; i++) {
            const uint32_t g = P.g_beg + i;
            while (bidx + 1 < nbl && bl[bidx + 1].g0 <= g) bidx++;
            const DecBL& B = bl[bidx];
            if ((B.mode & 2) && sflag[B.s0 + ((g - B.g0) >> 3)]) {
                gcl[g] = B.t;
            } else {
                const uint32_t start = cw ? zpos[cw - 1] + 1 : 0;
                const uint32_t ones = zpos[cw] - start;
                if (ones > 31) bad = 1;
                gcl[g] = (uint8_t)(B.t + ones);
                cw++;
            }
        }
        /* bits used must fit the declared sub-packet length */
        if (ncw && threadIdx.x == 0 && zpos[ncw - 1] + 1 > nbits) bad = 1;
        if (__syncthreads_or(bad)) {
            if (threadIdx.x == 0) JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
            return;
        }
    }
    /* data: bit lengths, block scan, per-packet bases, decode */
    const uint32_t per = (G + blockDim.x - 1) / blockDim.x;
    const uint32_t ga = min(G, threadIdx.x * per), ge = min(G, ga + per);
    uint32_t dsum = 0;
    for (uint32_t g = ga; g < ge; g++) {
        const DecBL& B = bl[find_dbl_by_group(bl, nbl, g)];
        const int planes = (int)gcl[g] - (int)B.t;
        if (planes > 0) dsum += 4 * (planes + 1);
    }
    uint32_t d0;
    block_scan1(dsum, &d0, ws);
    {
        uint32_t run = d0;
        for (uint32_t g = ga; g < ge; g++) {
            const DecBL& B = bl[find_dbl_by_group(bl, nbl, g)];
            if (g == B.g0 && pk[B.pk].b_beg == (uint32_t)(&B - bl)) pk_pref[B.pk] = run;
            const int planes = (int)gcl[g] - (int)B.t;
            if (planes > 0) run += 4 * (planes + 1);
        }
    }
    __syncthreads();
    {
        uint32_t run = d0;
        int bidx = ga < ge ? find_dbl_by_group(bl, nbl, ga) : 0;
        int bad = 0;
        const uint32_t uniform = cfg->qpih;
        for (uint32_t g = ga; g < ge; g++) {
            while (bidx + 1 < nbl && bl[bidx + 1].g0 <= g) bidx++;
            const DecBL& B = bl[bidx];
            const DecPk& P = pk[B.pk];
            const jxs_band_t& bd = cfg->band[B.fb];
            const uint32_t x = g - B.g0;
            const uint32_t t = B.t, gv = gcl[g];
            const int planes = (int)gv - (int)t;
            int32_t out[4] = {0, 0, 0, 0};
            if (planes > 0) {
                const uint32_t nb = 4 * (planes + 1);
                const uint32_t off = run - pk_pref[B.pk];
                if (off + nb > P.data_bits) bad = 1;
                else {
                    const uint32_t pos = P.data_pos + off;
                    uint32_t m[4] = {0, 0, 0, 0}, sgn;
                    /* first nibble: signs; then planes gcli-1 .. gtli */
                    if (nb <= 64) {
                        uint64_t v = bits64(pbuf, pos, nb);
                        sgn = (uint32_t)(v >> (nb - 4)) & 15;
                        for (int pl = planes - 1; pl >= 0; pl--) {
                            const uint32_t nib = (uint32_t)(v >> (4 * pl)) & 15;
                            m[0] = (m[0] << 1) | (nib >> 3);
                            m[1] = (m[1] << 1) | ((nib >> 2) & 1);
                            m[2] = (m[2] << 1) | ((nib >> 1) & 1);
                            m[3] = (m[3] << 1) | (nib & 1);
                        }
                    } else {
                        sgn = (uint32_t)bits64(pbuf, pos, 4);
                        for (int pl = 0; pl < planes; pl++) {
                            const uint32_t nib = (uint32_t)bits64(pbuf, pos + 4 + 4 * pl, 4);
                            m[0] = (m[0] << 1) | (nib >> 3);
                            m[1] = (m[1] << 1) | ((nib >> 2) & 1);
                            m[2] = (m[2] << 1) | ((nib >> 1) & 1);
                            m[3] = (m[3] << 1) | (nib & 1);
                        }
                    }
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        uint32_t mag = (m[c] << t) & 0xffffu;
                        if (t > 0 && (mag & 0x7fffu)) {
                            if (!uniform) {
                                mag |= 1u << (t - 1);
                            } else {
                                /* inv_quant_uniform (Dequant.c:23-43) */
                                uint32_t val = mag & 0x7fffu, acc = 0;
                                const uint32_t sc = gv - t + 1;
                                for (; val > 0; val >>= sc) acc = (acc + val) & 0xffffu;
                                mag = acc;
                            }
                        }
                        const uint32_t sm = (mag | (((sgn >> (3 - c)) & 1u) << 15)) & 0xffffu;
                        out[c] = (sm & 0x8000u) ? -(int32_t)(sm & 0x7fffu) : (int32_t)sm;
                    }
                }
                run += nb;
            }
            int16_t* crow = coef + bd.coef_off + (uint64_t)B.row * bd.pitch + 4 * x;
            *(uint2*)crow = make_uint2(((uint32_t)out[0] & 0xffffu) | ((uint32_t)out[1] << 16),
                                       ((uint32_t)out[2] & 0xffffu) | ((uint32_t)out[3] << 16));
        }
        if (bad) JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
    }
}

/* ------------------------------------------------------------------------ */
/* Inverse transform                                                         */
/* ------------------------------------------------------------------------ */
/* Inverse 5/3 lifting of rows in shared memory, stride S, n elements
 * (idwt_horizontal_line_*_c, Idwt.c:11-53). */
template <typename RowFn>
DEV void inv_h_level(RowFn row, int nrows, int n, int S) {
    const int n2 = n >> 1, n1 = (n + 1) >> 1;
    for (int t = threadIdx.x; t < nrows * n1; t += blockDim.x) {
        int r = t / n1, i = t - r * n1;
        int32_t* p = row(r);
        int jp = min(max(i - 1, 0), n2 - 1), jc = min(i, n2 - 1);
        p[S * 2 * i] -= (p[S * (2 * jp + 1)] + p[S * (2 * jc + 1)] + 2) >> 2;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nrows * n2; t += blockDim.x) {
        int r = t / n2, j = t - r * n2;
        int32_t* p = row(r);
        int32_t a = p[S * 2 * j];
        int32_t c = (2 * j + 2 < n) ? p[S * (2 * j + 2)] : a;
        p[S * (2 * j + 1)] += (a + c) >> 1;
    }
    __syncthreads();
}

DEV void place_band(int32_t* p, int o, int S, int n, const jxs_band_t& bd, int brow, const int16_t* coef, int fq) {
    const int16_t* crow = coef + bd.coef_off + (uint64_t)brow * bd.pitch;
    for (int k = threadIdx.x; k < n; k += blockDim.x) p[o + S * k] = (int32_t)((uint32_t)(int32_t)crow[k] << fq);
}

/* linear_output_scaling_*_line_c (NltDec.c:242-264) */
DEV void store_out(const DwtJob& J, int y, int x, int32_t v, int bw, int depth) {
    if (J.out_kind == 0) {
        J.ll[(long long)y * J.ll_pitch + x] = v;
        return;
    }
    const int zeta = bw - depth;
    long long t = (long long)v + (1 << (bw - 1));
    t = (t + ((1ll << zeta) >> 1)) >> zeta;
    const int m = (1 << depth) - 1;
    const int o = (int)(t > m ? m : (t < 0 ? 0 : t));
    if (J.out_kind == 1) ((uint8_t*)J.dst)[(long long)y * J.dst_pitch + x] = (uint8_t)o;
    else ((uint16_t*)J.dst)[(long long)y * J.dst_pitch + x] = (uint16_t)o;
}

/* Job fields for the inverse: w, h = size of the region this level rebuilds;
 * R = output row pairs per block; last = deepest vertical level (its low
 * rows come from the bands through the horizontal-only levels); src = int32
 * low band of the deeper level otherwise (src_pitch); ll/ll_pitch = int32
 * destination (out_kind 0) or dst/dst_pitch = output plane (1: 8-bit,
 * 2: 16-bit). */
template <bool VERT>
__global__ void __launch_bounds__(512) inv_dwt_kernel(const __grid_constant__ DwtLaunch L, const jxs_band_t* __restrict__ bands,
                                                      const int16_t* __restrict__ coef, int fq, int bw, int depth) {
    extern __shared__ int32_t sm[];
    int j = 0;
    while (j + 1 < L.njobs && (int)blockIdx.x >= L.job[j + 1].first_block) j++;
    const DwtJob& J = L.job[j];
    const int rb = blockIdx.x - J.first_block;
    const int w = J.w, h = J.h, sp = J.smem_pitch;
    const int w1 = (w + 1) >> 1, w2 = w >> 1;

    if (VERT) {
        const int n1 = (h + 1) >> 1, n2 = h >> 1;
        const int r0 = rb * J.R, r1 = min(r0 + J.R, n1);
        const int lcount = min(r1 + 1, n1) - r0;
        const int jlo = min(max(r0 - 1, 0), n2 - 1), jhi = min(max(r1, 0), n2 - 1);
        const int hcount = jhi - jlo + 1;
        int32_t* Ls = sm;
        int32_t* Hs = sm + (J.R + 1) * sp;
        /* low rows */
        for (int k = 0; k < lcount; k++) {
            int32_t* p = Ls + k * sp;
            const int i = r0 + k;
            if (J.last) {
                int m = w1, S = 2;
                int Sl = 1, ml = w; /* geometry of the deepest low band */
                for (int e = 0; e < J.nh; e++) {
                    place_band(p, S, 2 * S, m >> 1, bands[J.b_hf[e]], i, coef, fq);
                    m = (m + 1) >> 1;
                    S <<= 1;
                }
                Sl = S; ml = m;
                place_band(p, 0, Sl, ml, bands[J.b_ll], i, coef, fq);
            } else {
                const int32_t* srow = (const int32_t*)J.src + (long long)i * J.src_pitch;
                for (int x = threadIdx.x; x < w1; x += blockDim.x) p[2 * x] = srow[x];
            }
            place_band(p, 1, 2, w2, bands[J.b_hl], i, coef, fq);
        }
        for (int k = 0; k < hcount; k++) {
            int32_t* p = Hs + k * sp;
            place_band(p, 0, 2, w1, bands[J.b_lh], jlo + k, coef, fq);
            place_band(p, 1, 2, w2, bands[J.b_hh], jlo + k, coef, fq);
        }
        __syncthreads();
        if (J.last && J.nh > 0) {
            auto lrows = [&](int r) { return Ls + r * sp; };
            int ms[6];
            ms[0] = w1;
            for (int e = 1; e <= J.nh; e++) ms[e] = (ms[e - 1] + 1) >> 1;
            for (int e = J.nh - 1; e >= 0; e--) inv_h_level(lrows, lcount, ms[e], 2 << e);
        }
        auto all_rows = [&](int r) { return r < lcount ? Ls + r * sp : Hs + (r - lcount) * sp; };
        inv_h_level(all_rows, lcount + hcount, w, 1);
        /* vertical lifting (idwt_vertical_line_c, Idwt.c:186-263 in frame form) */
        auto H = [&](int jj, int x) { return Hs[(min(max(jj, 0), n2 - 1) - jlo) * sp + x]; };
        for (int x = threadIdx.x; x < w; x += blockDim.x) {
            int32_t xe = Ls[x] - ((H(r0 - 1, x) + H(r0, x) + 2) >> 2);
            for (int i = r0; i < r1; i++) {
                store_out(J, 2 * i, x, xe, bw, depth);
                if (2 * i + 1 < h) {
                    int32_t xn = xe;
                    if (2 * i + 2 < h) xn = Ls[(i + 1 - r0) * sp + x] - ((H(i, x) + H(i + 1, x) + 2) >> 2);
                    store_out(J, 2 * i + 1, x, H(i, x) + ((xe + xn) >> 1), bw, depth);
                    xe = xn;
                }
            }
        }
    } else {
        const int r0 = rb * J.R, rc = min(J.R, h - r0);
        for (int k = 0; k < rc; k++) {
            int32_t* p = sm + k * sp;
            int m = w, S = 1;
            for (int e = 0; e < J.nh; e++) {
                place_band(p, S, 2 * S, m >> 1, bands[J.b_hf[e]], r0 + k, coef, fq);
                m = (m + 1) >> 1;
                S <<= 1;
            }
            place_band(p, 0, S, m, bands[J.b_ll], r0 + k, coef, fq);
        }
        __syncthreads();
        auto rows = [&](int r) { return sm + r * sp; };
        int ms[6];
        ms[0] = w;
        for (int e = 1; e <= J.nh; e++) ms[e] = (ms[e - 1] + 1) >> 1;
        for (int e = J.nh - 1; e >= 0; e--) inv_h_level(rows, rc, ms[e], 1 << e);
        for (int t = threadIdx.x; t < rc * w; t += blockDim.x) {
            const int k = t / w, x = t - k * w;
            store_out(J, r0 + k, x, sm[k * sp + x], bw, depth);
        }
    }
}


/* ------------------------------------------------------------------------ */
/* Precinct offsets of a device-resident codestream                          */
/* ------------------------------------------------------------------------ */
DEV uint32_t be24(const uint8_t* p) { return ((uint32_t)p[0] << 16) | ((uint32_t)p[1] << 8) | p[2]; }

/* One thread per slice: the slice is expected where the constant-bit-rate
 * split of Lcod puts it (EncHandle.c:760-809); its precincts are found by
 * following the 24-bit precinct lengths, and the walk must end exactly at
 * the next slice (or at EOC).  Any mismatch raises *walk_bad. */
__global__ void walk_slices_kernel(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs, uint32_t size,
                                   uint32_t* __restrict__ prec_off, int* walk_bad) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cfg->nslices) return;
    if (cfg->max_slice_budget == 0) {
        *walk_bad = 1;
        return;
    }
    uint64_t off = cfg->slice_begin[s];
    if (off + 6 > size || bs[off] != 0xff || bs[off + 1] != 0x20 || bs[off + 2] != 0 || bs[off + 3] != 4 ||
        (((uint32_t)bs[off + 4] << 8) | bs[off + 5]) != s) {
        atomicExch(walk_bad, 1);
        return;
    }
    off += 6;
    const uint32_t first = s * cfg->pps, n = (s + 1 == cfg->nslices) ? cfg->np - first : cfg->pps;
    for (uint32_t i = 0; i < n; i++) {
        if (off + cfg->prec_hdr_bytes > size) {
            atomicExch(walk_bad, 1);
            return;
        }
        const uint32_t lprc = be24(bs + off);
        if (lprc > JXS_PREC_MAX_BYTES) {
            atomicExch(walk_bad, 1);
            return;
        }
        prec_off[first + i] = (uint32_t)off;
        off += cfg->prec_hdr_bytes + lprc;
    }
    const int ok = (s + 1 < cfg->nslices) ? off == cfg->slice_begin[s + 1]
                                          : (off + 2 <= size && bs[off] == 0xff && bs[off + 1] == 0x11);
    if (!ok) atomicExch(walk_bad, 1);
}

/* Fallback when the prediction failed: one thread walks the whole codestream
 * from the header (get_slice_size, DecThreadInit.c:35-131). */
__global__ void walk_sequential_kernel(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs, uint32_t size,
                                       uint32_t* __restrict__ prec_off, const int* walk_bad, int* status) {
    if (!*walk_bad) return;
    uint64_t off = cfg->hdr_len;
    for (uint32_t s = 0; s < cfg->nslices; s++) {
        if (off + 6 > size) {
            JXS_STATUS_SET(status, JXS_E_DEC_SHORT);
            return;
        }
        if (bs[off] != 0xff || bs[off + 1] != 0x20 || bs[off + 2] != 0 || bs[off + 3] != 4 ||
            (((uint32_t)bs[off + 4] << 8) | bs[off + 5]) != s) {
            JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
            return;
        }
        off += 6;
        const uint32_t first = s * cfg->pps, n = (s + 1 == cfg->nslices) ? cfg->np - first : cfg->pps;
        for (uint32_t i = 0; i < n; i++) {
            if (off + cfg->prec_hdr_bytes > size) {
                JXS_STATUS_SET(status, JXS_E_DEC_SHORT);
                return;
            }
            const uint32_t lprc = be24(bs + off);
            if (lprc > JXS_PREC_MAX_BYTES) {
                JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
                return;
            }
            prec_off[first + i] = (uint32_t)off;
            off += cfg->prec_hdr_bytes + lprc;
        }
    }
    if (off + 2 > size) JXS_STATUS_SET(status, JXS_E_DEC_SHORT);
    else if (bs[off] != 0xff || bs[off + 1] != 0x11) JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
}

/* ------------------------------------------------------------------------ */
/* host-side launchers                                                       */
/* ------------------------------------------------------------------------ */
extern "C" cudaError_t jxs_launch_walk(const jxs_cfg_t* dcfg, uint32_t nslices, const uint8_t* bs, uint32_t size, uint32_t* prec_off,
                                       int* walk_bad, int* status, cudaStream_t st) {
    walk_slices_kernel<<<(nslices + 127) / 128, 128, 0, st>>>(dcfg, bs, size, prec_off, walk_bad);
    walk_sequential_kernel<<<1, 1, 0, st>>>(dcfg, bs, size, prec_off, walk_bad, status);
    return cudaGetLastError();
}

extern "C" cudaError_t jxs_launch_unpack(const jxs_cfg_t* dcfg, const uint8_t* bs, const uint32_t* prec_off, int16_t* coef,
                                         uint32_t np, uint32_t cap_bytes, uint32_t cap_groups, int* status, cudaStream_t st) {
    size_t smem = (size_t)cap_bytes + 16 + 2ull * cap_groups + 16 + 4ull * cap_groups;
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(unpack_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    unpack_kernel<<<np, UK_THREADS, smem, st>>>(dcfg, bs, prec_off, coef, cap_bytes, cap_groups, status);
    return cudaGetLastError();
}

extern "C" cudaError_t jxs_launch_inv_dwt(const DwtLaunch* L, int vert, int nblocks, size_t smem, const jxs_band_t* bands,
                                          const int16_t* coef, int fq, int bw, int depth, cudaStream_t st) {
    static size_t configured[2] = {0, 0};
    cudaError_t e;
    if (smem > configured[vert]) {
        e = vert ? cudaFuncSetAttribute(inv_dwt_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                 : cudaFuncSetAttribute(inv_dwt_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured[vert] = smem;
    }
    if (vert) inv_dwt_kernel<true><<<nblocks, 512, smem, st>>>(*L, bands, coef, fq, bw, depth);
    else inv_dwt_kernel<false><<<nblocks, 512, smem, st>>>(*L, bands, coef, fq, bw, depth);
    return cudaGetLastError();
}
