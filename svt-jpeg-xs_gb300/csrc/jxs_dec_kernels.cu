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
 *  walk_*_kernel   precinct offsets of a device-resident codestream.
 * The inverse transform is in jxs_inv_dwt.cu.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "jxs_core.h"
#include "jxs_kernels.cuh"

#define DEV __device__ __forceinline__

#define UK_THREADS 512
#define UK_WARPS (UK_THREADS / 32)
#define FULL 0xffffffffu
static_assert(JXS_MAXSEG <= UK_THREADS, "one thread per segment");
static_assert(UK_LIST_BYTES == 4 * 128 * UK_WARPS, "a list of 128 groups per warp");

/* Per band line of the precinct being unpacked. */
struct UkLine {
    uint32_t sig_pos;           /* bit position of its significance flags; raw packets: of its 4-bit GCLIs */
    uint8_t t, meth, raw, pk;
    uint8_t vp, pad0, pad1, pad2; /* vp: GCLIs predicted from the line above */
};
/* Per packet. */
struct UkPk {
    uint32_t spos;              /* first bit after the packet header */
    uint32_t gpos, gbits;       /* GCLI sub-packet: bit position and length */
    uint32_t dpos, dbits;       /* data sub-packet */
    uint32_t sgpos, sgbits;     /* sign sub-packet (separate signs, Fs = 1) */
    uint32_t wbase, nwords;     /* its 32-bit words in the concatenated GCLI word list (VLC packets) */
    uint32_t zbase, nzero;      /* rank of its first zero bit among all VLC zeros; zeros in its range */
    uint32_t ncoded;            /* unary codewords */
    uint32_t raw, present;
};

/* 32 bits of a big-endian bit string held in shared memory, starting at
 * bit `pos`; the buffer must be readable 8 bytes past pos / 8. */
DEV uint32_t be_word(const uint8_t* b, uint32_t wi) { return __byte_perm(((const uint32_t*)b)[wi], 0, 0x0123); }
DEV uint32_t bits32_at(const uint8_t* b, uint32_t pos) {
    const uint32_t wi = pos >> 5;
    return __funnelshift_l(be_word(b, wi + 1), be_word(b, wi), pos & 31);
}

/* Transpose of the 8 x 4 bit matrix in a word: bit 4k + j moves to bit
 * 8j + k (k: nibble = bit-plane, j: bit in the nibble), so that byte 3 - c
 * collects the 8 plane bits of coefficient c.  Four swaps of index bits
 * ((4,1), (3,0), (2,1), (1,0)) as masked delta swaps. */
DEV uint32_t dswap(uint32_t x, int d, uint32_t m) {
    const uint32_t t = ((x >> d) ^ x) & m;
    return x ^ t ^ (t << d);
}
DEV uint32_t planes_to_coefs(uint32_t x) {
    x = dswap(x, 14, 0x0000ccccu);
    x = dswap(x, 7, 0x00aa00aau);
    x = dswap(x, 2, 0x0c0c0c0cu);
    return dswap(x, 1, 0x22222222u);
}

DEV uint32_t warp_excl_scan(uint32_t x, uint32_t* total) {
    const int lane = threadIdx.x & 31;
    uint32_t inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += y;
    }
    *total = __shfl_sync(FULL, inc, 31);
    return inc - x;
}

/* Block-wide exclusive scan of one counter; returns the block total. */
DEV uint32_t block_scan1(uint32_t a, uint32_t* ea, uint32_t* ws) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t ia = a;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(FULL, ia, o);
        if (lane >= o) ia += t;
    }
    if (lane == 31) ws[warp] = ia;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = lane < nw ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(FULL, v, o);
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

/* Next segment for a warp from a shared queue (the warps balance segments
 * of different lengths between them). */
DEV uint32_t next_seg(uint32_t* ctr, int lane) {
    uint32_t v = 0;
    if (lane == 0) v = atomicAdd(ctr, 1u);
    return __shfl_sync(FULL, v, 0);
}

/* Per-packet exclusive running sums of one count per segment.  Segments
 * are numbered in packet order, so a segment's base inside its packet is the
 * block-wide exclusive sum up to it minus that of its packet's first
 * segment.  Thread i holds segment i's count (nseg <= blockDim.x); base[i]
 * receives its base, ex[0 .. nseg] the block-wide exclusive sums, and
 * threads k < npk get packet k's total (0 without segments).  Other
 * threads may read base[] and ex[] after the caller's next barrier. */
DEV uint32_t seg_bases(uint32_t cnt, uint32_t nseg, uint32_t npk, const jxs_seg_t* segs, const jxs_bline_t* bls,
                       const uint8_t* pkbl0, const uint8_t* pknbl, uint32_t* ex, uint32_t* base, uint32_t* ws) {
    const uint32_t i = threadIdx.x;
    uint32_t e;
    const uint32_t total = block_scan1(i < nseg ? cnt : 0u, &e, ws);
    if (i < nseg) ex[i] = e;
    if (i == 0) ex[nseg] = total;
    __syncthreads();
    if (i < nseg) base[i] = e - ex[bls[pkbl0[bls[segs[i].bl].pk]].seg0];
    uint32_t sum = 0;
    if (i < npk && pknbl[i]) {
        const uint32_t b0 = pkbl0[i], lb = b0 + pknbl[i] - 1;
        sum = ex[bls[lb].seg0 + bls[lb].nseg] - ex[bls[b0].seg0];
    }
    return sum;
}

/* Packet header fields (get_packet_header, ParseHeader.c:20-44): raw flag,
 * data, GCLI and sign sub-packet lengths in bytes; short (5-byte) or long
 * (7-byte) form. */
DEV void pk_header(const uint8_t* h, int long_hdr, uint32_t& raw, uint32_t& dlen, uint32_t& glen, uint32_t& slen) {
    raw = h[0] >> 7;
    if (long_hdr) {
        dlen = ((uint32_t)(h[0] & 0x7f) << 13) | ((uint32_t)h[1] << 5) | (h[2] >> 3);
        glen = ((uint32_t)(h[2] & 7) << 17) | ((uint32_t)h[3] << 9) | ((uint32_t)h[4] << 1) | (h[5] >> 7);
        slen = ((uint32_t)(h[5] & 0x7f) << 8) | h[6];
    } else {
        dlen = ((uint32_t)(h[0] & 0x7f) << 8) | h[1];
        glen = ((uint32_t)h[2] << 5) | (h[3] >> 3);
        slen = ((uint32_t)(h[3] & 7) << 8) | h[4];
    }
}

/* One group's coefficients from its data bits (unpack_data_c,
 * Packing.c:134-219): sign nibble (coefficient 0 in the most significant
 * bit), then bit-planes gcli-1 .. gtli; planes placed at << gtli
 * (Packing.c:117-132), deadzone or uniform dequantization (Dequant.c:9-57)
 * and sign-magnitude to two's complement (inv_sign_c, Precinct.c:9-14).
 * Returns the four int16 results packed two per word, coefficient 0 in the
 * low half of .x; coefficients at or past `wl` (remaining width) are 0. */
DEV uint2 group_finish(uint32_t A, uint32_t B, uint32_t sgn, uint32_t uniform, int wl);

/* The dequantized magnitudes of a group's four coefficients from its plane
 * bits, as 16-bit pairs: coefficients 0 | 1 << 16 in *A, 2 | 3 << 16 in *B.
 * The plane bits are planes v-1 .. gtli as nibbles, coefficient 0 in each
 * nibble's most significant bit (Packing.c:117-132), placed at << gtli, then
 * deadzone or uniform dequantization (Dequant.c:9-57).  Returns the mask of
 * non-zero magnitudes (bit 3 - c for coefficient c). */
DEV uint32_t group_mags(uint64_t planes, uint32_t np, uint32_t t, uint32_t gv, uint32_t uniform, uint32_t* A, uint32_t* B) {
    /* the plane bits of coefficients 0, 1 / 2, 3 as 16-bit pairs */
    const uint32_t tl = planes_to_coefs((uint32_t)planes);
    uint32_t P01 = __byte_perm(tl, 0u, 0x4243), P23 = __byte_perm(tl, 0u, 0x4041);
    if (np > 8) {
        const uint32_t th = planes_to_coefs((uint32_t)(planes >> 32));
        P01 |= __byte_perm(th, 0u, 0x4243) << 8;
        P23 |= __byte_perm(th, 0u, 0x4041) << 8;
    }
    const uint32_t nz01 = __vcmpne2(P01, 0u), nz23 = __vcmpne2(P23, 0u);
    const uint32_t nz = ((nz01 & 1u) << 3) | ((nz01 >> 16 & 1u) << 2) | ((nz23 & 1u) << 1) | (nz23 >> 16 & 1u);
    if (!uniform || t == 0) {
        /* two coefficients per word: m << t stays below 2^15 */
        uint32_t a = P01 << t, b = P23 << t;
        if (t > 0) {
            const uint32_t half = (1u << (t - 1)) * 0x00010001u;
            a |= __vcmpne2(a, 0u) & half;
            b |= __vcmpne2(b, 0u) & half;
        }
        *A = a;
        *B = b;
        return nz;
    }
    const uint32_t m[4] = {P01 & 0xffffu, P01 >> 16, P23 & 0xffffu, P23 >> 16};
    uint32_t o[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        uint32_t mag = (m[c] << t) & 0xffffu;
        if (mag & 0x7fffu) {
            /* inv_quant_uniform (Dequant.c:23-43) */
            uint32_t val = mag & 0x7fffu, acc = 0;
            const uint32_t sc = gv - t + 1;
            for (; val > 0; val >>= sc) acc = (acc + val) & 0xffffu;
            mag = acc;
        }
        o[c] = mag;
    }
    *A = o[0] | (o[1] << 16);
    *B = o[2] | (o[3] << 16);
    return nz;
}

/* Sign-magnitude to two's complement (inv_sign_c, Precinct.c:9-14): sign
 * bit 3 - c of `sgn` for coefficient c; coefficients at or past `wl`
 * (remaining width) are 0.  Returns the four int16 results packed two per
 * word, coefficient 0 in the low half of .x. */
DEV uint2 group_finish(uint32_t A, uint32_t B, uint32_t sgn, uint32_t uniform, int wl) {
    const uint32_t keepA = (wl > 1 ? 0xffff0000u : 0u) | 0xffffu, keepB = (wl > 2 ? 0xffffu : 0u) | (wl > 3 ? 0xffff0000u : 0u);
    if (!uniform) {
        /* deadzone magnitudes stay below 2^15 */
        const uint32_t nA = ((sgn & 8u) ? 0xffffu : 0u) | ((sgn & 4u) ? 0xffff0000u : 0u);
        const uint32_t nB = ((sgn & 2u) ? 0xffffu : 0u) | ((sgn & 1u) ? 0xffff0000u : 0u);
        A = (A & ~nA) | (__vsub2(0u, A) & nA);
        B = (B & ~nB) | (__vsub2(0u, B) & nB);
        return make_uint2(A & keepA, B & keepB);
    }
    const uint32_t mg[4] = {A & 0xffffu, A >> 16, B & 0xffffu, B >> 16};
    uint32_t o[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const uint32_t sm = (mg[c] | (((sgn >> (3 - c)) & 1u) << 15)) & 0xffffu;
        o[c] = (uint32_t)((sm & 0x8000u) ? -(int32_t)(sm & 0x7fffu) : (int32_t)sm) & 0xffffu;
    }
    return make_uint2((o[0] | (o[1] << 16)) & keepA, (o[2] | (o[3] << 16)) & keepB);
}

/* One group's coefficients from its data bits with the signs joined to the
 * data (unpack_data_c, Packing.c:134-219): the sign nibble (coefficient 0 in
 * its most significant bit), then the plane nibbles. */
DEV uint2 decode_group(uint64_t chunk, uint32_t np, uint32_t t, uint32_t gv, uint32_t uniform, int wl) {
    const uint32_t sgn = (uint32_t)(chunk >> (4 * np)) & 15u;
    uint32_t A, B;
    group_mags(chunk & ((1ull << (4 * np)) - 1), np, t, gv, uniform, &A, &B);
    return group_finish(A, B, sgn, uniform && t != 0, wl);
}

/* The same under deadzone quantization, for a group inside its band line or
 * at its end (`wl` remaining coefficients): the sign nibble is transposed
 * with the planes, as the plane above the np magnitude planes, so that the
 * signs arrive as bit np of each coefficient. */
DEV uint2 decode_group_dz(uint64_t chunk, uint32_t np, uint32_t t, int wl) {
    const uint32_t tl = planes_to_coefs((uint32_t)chunk);
    uint32_t P01 = __byte_perm(tl, 0u, 0x4243), P23 = __byte_perm(tl, 0u, 0x4041);
    if (np >= 8) {
        const uint32_t th = planes_to_coefs((uint32_t)(chunk >> 32));
        P01 |= __byte_perm(th, 0u, 0x4243) << 8;
        P23 |= __byte_perm(th, 0u, 0x4041) << 8;
    }
    /* signs to all-ones halves; magnitudes without them */
    const uint32_t s01 = (P01 >> np) & 0x00010001u, s23 = (P23 >> np) & 0x00010001u;
    const uint32_t n01 = s01 * 0xffffu, n23 = s23 * 0xffffu;
    uint32_t a = (P01 ^ (s01 << np)) << t, b = (P23 ^ (s23 << np)) << t;
    if (t > 0) {
        /* deadzone reconstruction (Dequant.c:9-21): half a step on non-zero magnitudes */
        const uint32_t half = (1u << (t - 1)) * 0x00010001u;
        a |= __vcmpne2(a, 0u) & half;
        b |= __vcmpne2(b, 0u) & half;
    }
    /* two's complement of the negative ones, two per word */
    a = __vsub2(a ^ n01, n01);
    b = __vsub2(b ^ n23, n23);
    const uint32_t keepA = (wl > 1 ? 0xffff0000u : 0u) | 0xffffu, keepB = (wl > 2 ? 0xffffu : 0u) | (wl > 3 ? 0xffff0000u : 0u);
    return make_uint2(a & keepA, b & keepB);
}

/* unpack_precinct (Packing.c:513-868) for one precinct row; vertical
 * prediction and separate sign sub-packets are rejected.
 *
 * Dynamic shared memory (uk_layout): [precinct bytes: cap_bytes + 32,
 * stream byte i at i + lead so that 16-byte chunks are aligned] [GCLI per
 * group: cap_groups] [every zero bit of the VLC sub-packets, as a 16-bit
 * offset in its sub-packet] [the per-segment arrays, cap_seg segments].
 *
 *   copy    the precinct's bytes into shared memory;
 *   parse   thread 0: precinct header, packet headers, sub-packet positions
 *           with the reference's length checks;
 *   pass 1  warp per segment: groups with a unary codeword (the
 *           significance flags drop the insignificant ones); raw GCLIs;
 *   zeros   block pass over the VLC sub-packets: codeword c of a packet ends
 *           at the c-th zero bit of its sub-packet (unpack_pred_zero_gclis_*,
 *           Packing.c:435-511);
 *   pass 2  warp per segment: GCLI = gtli + ones in the codeword; data bits;
 *   pass 3  warp per segment: data bits at warp-scanned offsets, decoded and
 *           written as int16 coefficients (8 bytes per lane, coalesced). */
__device__ __forceinline__ void unpack_body(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs, uint32_t bs_size,
                                            const uint32_t* __restrict__ prec_off, int16_t* __restrict__ coef,
                                            uint32_t cap_bytes, uint32_t cap_groups, uint32_t cap_seg, int* status, const int p,
                                            uint8_t* top_gcl, uint8_t* top_t, const int vp_ok) {
    extern __shared__ __align__(16) uint8_t dsm[];
    const UkLayout UL = uk_layout(cap_bytes, cap_groups, cap_seg);
    uint8_t* pbuf = dsm;
    uint8_t* gcl = dsm + UL.gcl;
    uint16_t* zend = (uint16_t*)(dsm + UL.zend);
    /* zero bits: one per codeword plus up to 7 padding bits per packet */
    const uint32_t zcap = UK_ZCAP(cap_groups);
    __shared__ UkLine ln[JXS_MAXBLINES];
    __shared__ UkPk pk[JXS_MAXPK];
    __shared__ uint8_t s_mode[JXS_MAXBL];
    __shared__ uint32_t s_pksb[JXS_MAXPK], s_pkrb[JXS_MAXPK], s_hpos[JXS_MAXPK];
    __shared__ uint32_t s_next[2]; /* segment queues of the two warp passes */
    /* this precinct kind's tables, staged from the configuration */
    /* this precinct kind's segments, their work order and per-segment sums
     * (dynamic: sized for the launch's largest segment count) */
    jxs_seg_t* s_seg = (jxs_seg_t*)(dsm + UL.seg);
    uint16_t* s_ord = (uint16_t*)(dsm + UL.ord);
    uint32_t* s_cnt = (uint32_t*)(dsm + UL.cnt);
    uint32_t* s_base = (uint32_t*)(dsm + UL.base);
    uint32_t* s_ex = (uint32_t*)(dsm + UL.ex);
    uint32_t* s_nz = (uint32_t*)(dsm + UL.nz);  /* separate signs: per segment, count */
    uint32_t* s_sgb = (uint32_t*)(dsm + UL.sgb); /* and first bit */
    __shared__ jxs_bline_t s_bl[JXS_MAXBLINES];
    __shared__ uint64_t s_crow[JXS_MAXBLINES]; /* per line: coefficient row offset */
    __shared__ uint8_t s_pkbl0[JXS_MAXPK], s_pknbl[JXS_MAXPK];
    __shared__ uint32_t ws[UK_WARPS];
    __shared__ int s_err;
    __shared__ uint32_t s_total, s_lead, s_tw, s_npk, s_off;
    __shared__ uint8_t s_g2f[JXS_MAXBL];          /* global band -> flat band */
    __shared__ uint16_t s_lgp[JXS_MAXBLINES];      /* per line: band gain | priority << 8 */
    __shared__ uint32_t s_sc[9];                   /* nbands_all, npk, long headers, separate signs, precinct header bytes,
                                                      band lines, segments, groups per segment, run mode */
    __shared__ uint8_t s_topbl[JXS_MAXBLINES], s_topprev[JXS_MAXBLINES]; /* vertical prediction: the line above */
    __shared__ uint32_t s_topg[JXS_MAXBLINES];
    __shared__ int s_hasvp;

    /* the precinct kind's tables (last row / last of several columns) */
    const int last = jxs_pkind(cfg, (uint32_t)p);
    const uint32_t prow = (uint32_t)p / cfg->ncol, pcol = (uint32_t)p - prow * cfg->ncol;
    const int one_col = cfg->ncol == 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    /* thread 0: the frame's status and the precinct's length field; every
     * thread meanwhile stages this precinct kind's tables and the scalars
     * the parse needs, so that no single-warp phase waits on device memory */
    if (threadIdx.x == 0) {
        /* the precinct's offset and length field are read in bounds before
         * the frame status, so that the three loads do not wait in turn */
        const uint32_t off = prec_off[p], phb = cfg->prec_hdr_bytes;
        s_off = off; /* read once: the offsets may be in host memory */
        const bool inb = (uint64_t)off + phb <= bs_size;
        const uint32_t lprc = inb ? ((uint32_t)bs[off] << 16) | ((uint32_t)bs[off + 1] << 8) | bs[off + 2] : 0u;
        int err = *(volatile int*)status; /* set: the precinct offsets could not be found */
        s_sc[0] = cfg->nbands_all;
        s_sc[1] = cfg->npk;
        s_sc[2] = cfg->lh || !cfg->short_hdr;
        s_sc[3] = cfg->fs;
        s_sc[4] = cfg->prec_hdr_bytes;
        s_sc[5] = cfg->nbline[last];
        s_sc[6] = cfg->nseg[last];
        s_sc[7] = cfg->seg_groups;
        s_sc[8] = cfg->rm;
        s_hasvp = 0;
        if (!err) {
            if (!inb) {
                err = JXS_E_DEC_SHORT;
            } else {
                s_total = phb + lprc;
                s_lead = (uint32_t)((uintptr_t)(bs + off) & 15);
                if (lprc > JXS_PREC_MAX_BYTES || s_total + 48 > cap_bytes) err = JXS_E_DEC_BITSTREAM;
                else if ((uint64_t)off + s_total > bs_size) err = JXS_E_DEC_SHORT;
            }
            if (err) JXS_STATUS_SET(status, err);
        } else {
            err = -1; /* already reported */
        }
        s_err = err;
    }
    if (threadIdx.x < 2) s_next[threadIdx.x] = 0;
    {
        const uint32_t ns = cfg->nseg[last], nl = cfg->nbline[last];
        for (uint32_t i = threadIdx.x; i < ns * (sizeof(jxs_seg_t) / 4); i += blockDim.x)
            ((uint32_t*)s_seg)[i] = ((const uint32_t*)cfg->seg[last])[i];
        for (uint32_t i = threadIdx.x; i < nl * (sizeof(jxs_bline_t) / 4); i += blockDim.x)
            ((uint32_t*)s_bl)[i] = ((const uint32_t*)cfg->bline[last])[i];
        for (uint32_t i = threadIdx.x; i < ns; i += blockDim.x) s_ord[i] = cfg->seg_ord[last][i];
        for (uint32_t x = threadIdx.x; x < nl; x += blockDim.x) {
            const jxs_bline_t& B = cfg->bline[last][x];
            const jxs_band_t& bd = cfg->band[B.fb];
            s_crow[x] = bd.coef_off + (uint64_t)(prow * bd.lines + B.line) * bd.pitch + (uint64_t)pcol * bd.cwn;
            s_lgp[x] = (uint16_t)(bd.gain | (bd.prio << 8));
            s_topbl[x] = cfg->top_bl[last][x];
            s_topprev[x] = cfg->top_prev[last][x];
            s_topg[x] = cfg->top_gbase[last][x];
        }
        for (uint32_t k = threadIdx.x; k < cfg->npk; k += blockDim.x) {
            s_pkbl0[k] = cfg->pk_bl0[last][k];
            s_pknbl[k] = cfg->pk_nbl[last][k];
        }
        for (uint32_t gb = threadIdx.x; gb < cfg->nbands_all; gb += blockDim.x) s_g2f[gb] = cfg->g2f[gb];
    }
    __syncthreads();
    if (s_err) return;
    const uint32_t off = s_off;
    const uint32_t total = s_total, lead = s_lead;
    {
        /* aligned 16-byte chunks inside the precinct, single bytes at its
         * ends; 32 zero bytes after it for the bit readers */
        const uint8_t* gsrc = bs + off - lead;
        const uint32_t nbytes = lead + total, nch = (nbytes + 15) >> 4;
        for (uint32_t c = threadIdx.x; c < nch + 2; c += blockDim.x) {
            const uint32_t b0 = c << 4;
            if (b0 >= lead && b0 + 16 <= nbytes) {
                *(uint4*)(pbuf + b0) = *(const uint4*)(gsrc + b0);
            } else {
                for (uint32_t i = b0; i < b0 + 16; i++) pbuf[i] = (i >= lead && i < nbytes) ? gsrc[i] : 0;
            }
        }
    }
    __syncthreads();

    const uint32_t nbl = s_sc[5], nseg = s_sc[6], SG = s_sc[7];
    const jxs_bline_t* bls = s_bl;
    const jxs_seg_t* segs = s_seg;
    /* parse, by warp 0: band modes and per-line fields in parallel, the
     * packet headers in order by lane 0, then every line's positions */
    if (warp == 0) {
        const uint8_t* h0 = pbuf + lead;
        const uint8_t q = h0[3], r = h0[4];
        int err = 0, vp_seen = 0;
        /* band coding modes D[p,b], 2 bits per existing band */
        uint32_t idx0 = 0;
        const uint32_t nbands_all = s_sc[0], npk_c = s_sc[1];
        for (uint32_t gb0 = 0; gb0 < nbands_all; gb0 += 32) {
            const uint32_t gb = gb0 + lane;
            const int fb = gb < nbands_all ? s_g2f[gb] : JXS_NOBAND;
            const bool ex = fb != JXS_NOBAND;
            const uint32_t bal = __ballot_sync(FULL, ex);
            if (ex) {
                const uint32_t pos = 40 + 2 * (idx0 + __popc(bal & ((1u << lane) - 1)));
                s_mode[fb] = (uint8_t)((h0[pos >> 3] >> (6 - (pos & 7))) & 3);
                /* vertical prediction: resolved here when the precinct row
                 * above is known (slice-ordered decoding), else the frame is
                 * decoded again that way; never in a slice's first row */
                if (s_mode[fb] & 1) vp_seen = 1;
            }
            idx0 += __popc(bal);
        }
        __syncwarp();
        for (uint32_t x = lane; x < nbl; x += 32) {
            ln[x].t = jxs_truncation((uint8_t)(s_lgp[x] & 255u), (uint8_t)(s_lgp[x] >> 8), q, r);
            ln[x].meth = (s_mode[bls[x].fb] & 2) ? 1 : 0;
            ln[x].vp = (s_mode[bls[x].fb] & 1) ? 1 : 0;
            ln[x].pk = bls[x].pk;
        }
        __syncwarp();
        /* per packet: significance bits and raw GCLI bits it must hold */
        uint32_t sb = 0, rb = 0;
        if (lane < (int)npk_c) {
            const uint32_t b0 = s_pkbl0[lane], nb = s_pknbl[lane];
            for (uint32_t x = b0; x < b0 + nb; x++) {
                if (ln[x].meth) sb += bls[x].sig_w;
                rb += 4 * bls[x].gcli_w;
            }
            s_pksb[lane] = sb;
            s_pkrb[lane] = rb;
        }
        __syncwarp();
        /* packet headers: lane 0 follows the chain of header positions
         * only; one lane per packet then reads its header again and derives
         * its sub-packet positions with the reference's checks (every check
         * bounds the running position, so testing each packet's own end
         * against the precinct's end is equivalent) */
        const int long_hdr = (int)s_sc[2];
        const uint32_t hb = long_hdr ? 7u : 5u, pend_max = lead + total;
        if (lane == 0) {
            uint32_t bpos = lead + s_sc[4]; /* bytes */
            for (uint32_t k = 0; k < npk_c; k++) {
                if (!s_pknbl[k]) continue;
                if (bpos + hb > pend_max) {
                    err = JXS_E_DEC_BITSTREAM;
                    break;
                }
                uint32_t raw, dlen, glen, slen;
                pk_header(pbuf + bpos, long_hdr, raw, dlen, glen, slen);
                s_hpos[k] = bpos;
                bpos += hb + (raw ? 0u : (s_pksb[k] + 7) >> 3) + glen + dlen + slen;
            }
        }
        err = __shfl_sync(FULL, err, 0);
        uint32_t nwords = 0;
        if (lane < (int)npk_c) {
            UkPk& P = pk[lane];
            P.present = 0;
            P.gbits = P.dbits = P.ncoded = P.nzero = 0;
            P.raw = 0;
            if (!err && s_pknbl[lane]) {
                uint32_t raw, dlen, glen, slen;
                const uint32_t b = s_hpos[lane] + hb;
                pk_header(pbuf + s_hpos[lane], long_hdr, raw, dlen, glen, slen);
                uint32_t gp = b;
                if (raw) {
                    if (s_pkrb[lane] > glen * 8) err = JXS_E_DEC_BITSTREAM;
                } else {
                    gp += (s_pksb[lane] + 7) >> 3;
                    /* codeword ends are kept as 16-bit offsets in the sub-packet */
                    if (glen * 8 > 65535u) err = JXS_E_DEC_BITSTREAM;
                }
                if ((uint64_t)gp + glen + dlen + slen > pend_max) err = JXS_E_DEC_BITSTREAM;
                P.raw = raw;
                P.spos = b * 8;
                P.gpos = gp * 8;
                P.gbits = glen * 8;
                P.dpos = (gp + glen) * 8;
                P.dbits = dlen * 8;
                P.sgpos = (gp + glen + dlen) * 8;
                P.sgbits = slen * 8;
                P.present = 1;
                if (!raw) nwords = (P.gbits + 31) >> 5;
            }
        }
        {
            uint32_t tw;
            const uint32_t wb = warp_excl_scan(nwords, &tw);
            if (lane < (int)npk_c) {
                pk[lane].wbase = wb;
                pk[lane].nwords = nwords;
            }
            if (lane == 0) {
                s_tw = tw;
                s_npk = npk_c;
            }
        }
        err = __reduce_or_sync(FULL, (uint32_t)err) ? JXS_E_DEC_BITSTREAM : 0;
        if (!err && __any_sync(FULL, vp_seen)) {
            if (!top_gcl) err = JXS_E_DEC_VPRED;
            else if (!vp_ok) err = JXS_E_DEC_BITSTREAM; /* no precinct row above to predict from */
        }
        __syncwarp();
        /* line positions: significance flags, or raw GCLIs for raw packets */
        if (!err && lane < (int)npk_c && pk[lane].present) {
            const UkPk& P = pk[lane];
            const uint32_t b0 = s_pkbl0[lane], nb = s_pknbl[lane];
            uint32_t run = P.spos;
            for (uint32_t x = b0; x < b0 + nb; x++) {
                ln[x].raw = (uint8_t)P.raw;
                if (P.raw) ln[x].vp = 0;
                ln[x].sig_pos = run;
                run += P.raw ? 4 * bls[x].gcli_w : (ln[x].meth ? bls[x].sig_w : 0u);
            }
        }
        __syncwarp();
        if (!err) {
            bool hv = false;
            for (uint32_t x = lane; x < nbl; x += 32) hv |= ln[x].vp != 0;
            if (__any_sync(FULL, hv) && lane == 0) s_hasvp = 1;
        }
        if (lane == 0) s_err = err;
    }
    __syncthreads();
    if (s_err) {
        if (threadIdx.x == 0) JXS_STATUS_SET(status, s_err);
        return;
    }

    /* codewords of every segment, one thread each: its groups minus those
     * in insignificant significance groups (flags: 1 = insignificant); then
     * the codeword base of every segment inside its packet */
    const uint32_t tw = s_tw, npk = s_npk;
    {
        uint32_t cnt = 0;
        if (threadIdx.x < nseg) {
            const jxs_seg_t sg = segs[threadIdx.x];
            const jxs_bline_t& B = bls[sg.bl];
            const UkLine& L = ln[sg.bl];
            const uint32_t gend = min(sg.g0 + SG, B.gcli_w);
            if (!L.raw) {
                cnt = gend - sg.g0;
                if (L.meth) {
                    for (uint32_t s0 = sg.g0 >> 3; s0 < ((gend + 7) >> 3); s0 += 32) {
                        const uint32_t ns = min(32u, ((gend + 7) >> 3) - s0);
                        const uint32_t fl = bits32_at(pbuf, L.sig_pos + s0) >> (32 - ns);
                        cnt -= 8 * __popc(fl);
                        /* a flagged partial last group counts its own size */
                        if ((fl & 1u) && 8 * (s0 + ns) > B.gcli_w) cnt += 8 * (s0 + ns) - B.gcli_w;
                    }
                }
            }
        }
        const uint32_t ncoded = seg_bases(cnt, nseg, npk, segs, bls, s_pkbl0, s_pknbl, s_ex, s_base, ws);
        if (threadIdx.x < npk) pk[threadIdx.x].ncoded = ncoded;
        __syncthreads();
    }

    /* zero bits of the VLC sub-packets: count, scan, record positions.  A
     * thread's first word finds its packet by binary search over the
     * packets' word ranges (contiguous, in packet order; a packet without
     * VLC words has an empty range), later words step forward. */
    const uint32_t per = (tw + blockDim.x - 1) / blockDim.x;
    const uint32_t wa = min(tw, threadIdx.x * per), we = min(tw, wa + per);
    uint32_t k0 = 0;
    if (wa < we) {
        uint32_t lo = 0, hi = npk - 1; /* the first packet whose range ends past wa */
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (pk[mid].wbase + pk[mid].nwords > wa) hi = mid;
            else lo = mid + 1;
        }
        k0 = lo;
    }
    uint32_t zc = 0;
    {
        uint32_t k = k0;
        for (uint32_t wi = wa; wi < we; wi++) {
            while (k + 1 < npk && wi >= pk[k].wbase + pk[k].nwords) k++;
            const uint32_t i = wi - pk[k].wbase;
            const uint32_t valid = min(32u, pk[k].gbits - 32 * i);
            uint32_t z = ~bits32_at(pbuf, pk[k].gpos + 32 * i);
            if (valid < 32) z &= ~(0xffffffffu >> valid);
            zc += __popc(z);
        }
    }
    uint32_t z0;
    const uint32_t ztotal = block_scan1(zc, &z0, ws);
    {
        uint32_t k = k0;
        for (uint32_t wi = wa; wi < we; wi++) {
            while (k + 1 < npk && wi >= pk[k].wbase + pk[k].nwords) k++;
            const uint32_t i = wi - pk[k].wbase;
            if (i == 0) pk[k].zbase = z0;
            const uint32_t valid = min(32u, pk[k].gbits - 32 * i);
            uint32_t z = ~bits32_at(pbuf, pk[k].gpos + 32 * i);
            if (valid < 32) z &= ~(0xffffffffu >> valid);
            while (z) {
                const uint32_t lz = __clz(z);
                if (z0 < zcap) zend[z0] = (uint16_t)(32 * i + lz);
                z0++;
                z &= ~(0x80000000u >> lz);
            }
        }
    }
    __syncthreads();
    if (warp == 0) {
        /* zeros of each VLC packet: up to the next VLC packet's first zero */
        const uint32_t k = lane;
        const bool vlc = k < npk && pk[k].present && !pk[k].raw && pk[k].nwords;
        const uint32_t zb = vlc ? pk[k].zbase : 0u;
        const uint32_t later = __ballot_sync(FULL, vlc) & ~((2u << k) - 1u);
        const uint32_t zn = __shfl_sync(FULL, zb, later ? __ffs(later) - 1 : 0);
        const uint32_t znext = later ? zn : ztotal;
        bool bad_pk = false;
        if (k < npk && pk[k].present && !pk[k].raw) {
            UkPk& P = pk[k];
            if (!P.nwords) {
                P.zbase = 0;
                P.nzero = 0;
            } else {
                P.nzero = znext - P.zbase;
            }
            bad_pk = P.ncoded > P.nzero || (P.ncoded && P.zbase + P.ncoded > zcap);
        }
        if (lane == 0) s_err = 0;
        __syncwarp();
        if (__any_sync(FULL, bad_pk) && lane == 0) s_err = JXS_E_DEC_BITSTREAM;
    }
    __syncthreads();
    if (s_err) {
        if (threadIdx.x == 0) JXS_STATUS_SET(status, s_err);
        return;
    }

    /* pass 2: GCLIs from codeword ends; data bits per segment.  Each lane
     * takes 4 consecutive groups: they share one significance flag, so
     * either all of them carry a codeword or none (only the segment's last
     * lane may hold fewer than 4 groups, and no lane after it holds any). */
    int bad = 0;
    const uint32_t lt_mask = (1u << lane) - 1u;
    /* a group's data: its sign nibble (signs with the data) and its planes */
    const uint32_t fs = s_sc[3], nib_sign = fs ? 0u : 1u;
    for (uint32_t qi = next_seg(&s_next[0], lane); qi < nseg; qi = next_seg(&s_next[0], lane)) {
        const uint32_t sidx = s_ord[qi];
        const jxs_seg_t sg = segs[sidx];
        const jxs_bline_t B = bls[sg.bl];
        const UkLine L = ln[sg.bl];
        const UkPk P = pk[L.pk];
        const uint32_t gend = min(sg.g0 + SG, B.gcli_w);
        uint32_t cw = s_base[sidx], dsum = 0;
        for (uint32_t base = sg.g0; base < gend; base += 128) {
            const uint32_t g0 = base + 4 * lane;
            const uint32_t nv = g0 < gend ? min(4u, gend - g0) : 0u;
            uint32_t v4 = 0;
            bool coded = false;
            if (nv) {
                if (L.raw) {
                    /* 4 raw 4-bit GCLIs, group g0 in the top nibble */
                    const uint32_t w = bits32_at(pbuf, L.sig_pos + 4 * g0);
                    v4 = __byte_perm(((w >> 28) & 15u) | (((w >> 24) & 15u) << 8), ((w >> 20) & 15u) | (((w >> 16) & 15u) << 8),
                                     0x5410);
                } else {
                    const uint32_t sp = L.sig_pos + (g0 >> 3);
                    coded = !(L.meth && ((pbuf[sp >> 3] >> (7 - (sp & 7))) & 1));
                    /* predicted lines keep the codeword value (0xff: no
                     * codeword) until the line above is known */
                    if (!coded) v4 = L.vp ? 0xffffffffu : L.t * 0x01010101u;
                }
            }
            const uint32_t bal = __ballot_sync(FULL, coded);
            if (coded) {
                /* codeword c + q ends at the (c + q)-th zero bit: its value
                 * is the distance to the zero before, less one; the four
                 * distances as 16-bit pairs */
                const uint32_t c = cw + 4 * __popc(bal & lt_mask);
                const uint32_t zr = P.zbase + c;
                const uint32_t zm = c ? zend[zr - 1] : 0xffffu; /* -1 */
                uint32_t z[4];
#pragma unroll
                for (int q = 0; q < 4; q++) z[q] = q < (int)nv ? zend[zr + q] : 0u;
                const uint32_t r01 = __vsub2(__vsub2(z[0] | (z[1] << 16), zm | (z[0] << 16)), 0x00010001u);
                const uint32_t r23 = __vsub2(__vsub2(z[2] | (z[3] << 16), z[1] | (z[2] << 16)), 0x00010001u);
                /* GCLI = base + r, at most 15 (31 for a predicted line's
                 * codeword value) */
                const uint32_t base = L.vp ? 0u : L.t, room = (L.vp ? 31u : 15u) - base;
                const uint32_t room2 = room * 0x00010001u, base2 = base * 0x00010001u;
                const uint32_t keep = nv >= 4 ? 0xffffffffu : (1u << (8 * nv)) - 1u;
                if (__byte_perm(__vcmpgtu2(r01, room2), __vcmpgtu2(r23, room2), 0x6420) & keep) bad = 1;
                v4 = __byte_perm(__vadd2(__vminu2(r01, room2), base2), __vadd2(__vminu2(r23, room2), base2), 0x6420) & keep;
            }
            uint8_t* gdst = gcl + B.gbase + g0;
            if (nv == 4) {
                *(uint32_t*)gdst = v4;
            } else {
                for (uint32_t q = 0; q < nv; q++) gdst[q] = (uint8_t)(v4 >> (8 * q));
            }
            cw += __reduce_add_sync(FULL, coded ? nv : 0u);
            if (!L.vp) {
                /* data bits: 4 (v - t + 1) per group above gtli (4 (v - t)
                 * with separate signs) */
                const uint32_t t4 = L.t * 0x01010101u;
                const uint32_t vm = v4 & (nv >= 4 ? 0xffffffffu : (1u << (8 * nv)) - 1u);
                dsum += 4 * (__vsadu4(__vsubus4(vm, t4), 0u) + nib_sign * __popc(__vcmpgtu4(vm, t4) & 0x01010101u));
            }
        }
        dsum = __reduce_add_sync(FULL, dsum);
        if (lane == 0) s_cnt[sidx] = dsum;
    }
    __syncthreads();
    if (s_hasvp) {
        /* vertical prediction (unpack_verical_pred_gclis_*, Packing.c:267-431):
         * GCLI = the predictor max(top, max(gtli_top, gtli)) moved by the
         * codeword value; without a codeword (insignificant group) the
         * predictor, or gtli in run mode.  Line levels in order: line l reads
         * line l - 1 of its band (line 0: the row above, top_gcl). */
        const uint32_t rm = s_sc[8];
        for (uint32_t lvl = 0; lvl < 4; lvl++) {
            for (uint32_t sidx = warp; sidx < nseg; sidx += UK_WARPS) {
                const jxs_seg_t sg = segs[sidx];
                const jxs_bline_t B = bls[sg.bl];
                const UkLine L = ln[sg.bl];
                if (!L.vp || B.line != lvl) continue;
                const uint32_t tb = s_topbl[sg.bl];
                const int from_prev = s_topprev[sg.bl];
                const uint8_t* src = (from_prev ? top_gcl : gcl) + s_topg[sg.bl];
                const uint32_t tt = max(from_prev ? (uint32_t)top_t[tb] : (uint32_t)ln[tb].t, (uint32_t)L.t);
                const uint32_t gend = min(sg.g0 + SG, B.gcli_w);
                uint32_t dsum = 0;
                for (uint32_t g = sg.g0 + lane; g < gend; g += 32) {
                    const uint32_t x = gcl[B.gbase + g];
                    const uint32_t mt = max((uint32_t)src[g], tt);
                    uint32_t v;
                    if (x == 0xffu) {
                        v = rm ? L.t : mt;
                    } else {
                        const uint32_t thr = mt > L.t ? mt - L.t : 0u;
                        int d = 0;
                        if (x > 2 * thr) d = (int)(x - thr);
                        else if (x > 0) d = (x & 1) ? -(int)((x + 1) >> 1) : (int)(x >> 1);
                        v = (uint32_t)((int)mt + d);
                    }
                    if (v > 15) {
                        bad = 1;
                        v = 15;
                    }
                    gcl[B.gbase + g] = (uint8_t)v;
                    if (v > L.t) dsum += 4 * (v - L.t + nib_sign);
                }
                dsum = __reduce_add_sync(FULL, dsum);
                if (lane == 0) s_cnt[sidx] = dsum;
            }
            __syncthreads();
        }
    }
    {
        /* data base of every segment inside its packet */
        const uint32_t dbits = seg_bases(threadIdx.x < nseg ? s_cnt[threadIdx.x] : 0u, nseg, npk, segs, bls, s_pkbl0, s_pknbl,
                                         s_ex, s_base, ws);
        const int bad_pk = threadIdx.x < npk && pk[threadIdx.x].present && dbits > pk[threadIdx.x].dbits;
        if (__syncthreads_or(bad_pk)) {
            if (threadIdx.x == 0) JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
            return;
        }
    }

    /* pass 3: data */
    const uint32_t uniform = cfg->qpih;
    if (fs) {
        /* separate signs (unpack_sign, Packing.c:221-247): a sign bit for
         * every non-zero magnitude, band lines of the packet in order and each
         * line in coefficient order (the last group's padding coefficients
         * last).  Count them per segment, give each segment its first sign
         * bit in the packet's sign sub-packet, then decode with the signs. */
        for (uint32_t qi = next_seg(&s_next[1], lane); qi < nseg; qi = next_seg(&s_next[1], lane)) {
            const uint32_t sidx = s_ord[qi];
            const jxs_seg_t sg = segs[sidx];
            const jxs_bline_t B = bls[sg.bl];
            const UkLine L = ln[sg.bl];
            const UkPk P = pk[L.pk];
            const uint32_t gend = min(sg.g0 + SG, B.gcli_w);
            uint32_t dpos = P.dpos + s_base[sidx], nzs = 0;
            for (uint32_t base = sg.g0; base < gend; base += 32) {
                const uint32_t g = base + lane;
                const uint32_t v = g < gend ? gcl[B.gbase + g] : 0u;
                const uint32_t np = v > L.t ? v - L.t : 0u;
                const uint32_t len = 4 * np;
                uint32_t tot;
                const uint32_t ex = warp_excl_scan(len, &tot);
                if (len) {
                    const uint32_t pos = dpos + ex;
                    const uint64_t win = ((uint64_t)bits32_at(pbuf, pos) << 32) | bits32_at(pbuf, pos + 32);
                    uint32_t A, B2;
                    nzs += __popc(group_mags(win >> (64 - len), np, L.t, v, uniform, &A, &B2));
                }
                dpos += tot;
            }
            nzs = __reduce_add_sync(FULL, nzs);
            if (lane == 0) s_nz[sidx] = nzs;
        }
        __syncthreads();
        /* first sign bit of every segment inside its packet */
        const uint32_t sbits = seg_bases(threadIdx.x < nseg ? s_nz[threadIdx.x] : 0u, nseg, npk, segs, bls, s_pkbl0, s_pknbl,
                                         s_ex, s_sgb, ws);
        const int bad_pk = threadIdx.x < npk && pk[threadIdx.x].present && sbits > pk[threadIdx.x].sgbits;
        if (threadIdx.x == 0) s_next[1] = 0;
        if (__syncthreads_or(bad_pk)) {
            if (threadIdx.x == 0) JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
            return;
        }
    }
    for (uint32_t qi = next_seg(&s_next[1], lane); qi < nseg; qi = next_seg(&s_next[1], lane)) {
        const uint32_t sidx = s_ord[qi];
        const jxs_seg_t sg = segs[sidx];
        const jxs_bline_t B = bls[sg.bl];
        const UkLine L = ln[sg.bl];
        const UkPk P = pk[L.pk];
        int16_t* crow = coef + s_crow[sg.bl];
        const uint32_t gend = min(sg.g0 + SG, B.gcli_w);
        uint32_t dpos = P.dpos + s_base[sidx];
        if (!fs) {
            /* signs with the data: each lane 4 consecutive groups.  The lane
             * writes zeros for its groups, then the warp lists the groups
             * with data (bit offset in the warp's data, group, GCLI) and each
             * lane decodes one listed group at a time, so that the decode
             * work follows the groups that have data */
            uint32_t* list = (uint32_t*)(dsm + UL.zend) + 128 * warp;
            const uint32_t t = L.t;
            for (uint32_t base = sg.g0; base < gend; base += 128) {
                const uint32_t g = base + 4 * lane;
                const uint32_t nv = g < gend ? min(4u, gend - g) : 0u;
                uint32_t v4 = 0;
                if (nv == 4) {
                    v4 = *(const uint32_t*)(gcl + B.gbase + g);
                } else {
                    for (uint32_t q = 0; q < nv; q++) v4 |= (uint32_t)gcl[B.gbase + g + q] << (8 * q);
                }
                /* per byte: v > t, and the data of such a group: 4 (v - t + 1)
                 * bits; one scan for the data bits / 4 and the listed groups */
                const uint32_t t4 = t * 0x01010101u;
                const uint32_t s4 = __vcmpgtu4(v4, t4), nsig = __popc(s4 & 0x01010101u);
                uint32_t tot;
                const uint32_t ex = warp_excl_scan((__vsadu4(__vsubus4(v4, t4), 0u) + nsig) | (nsig << 24), &tot);
                const uint32_t o = (ex & 0xffffffu) << 2;
                /* zeros for the lane's groups (those with data are written
                 * again below, after the warp barrier) */
                if (one_col) {
                    if (nv == 4) {
                        *(uint4*)(crow + 4 * g) = make_uint4(0u, 0u, 0u, 0u);
                        *(uint4*)(crow + 4 * g + 8) = make_uint4(0u, 0u, 0u, 0u);
                    } else {
                        for (uint32_t q = 0; q < nv; q++) *(uint2*)(crow + 4 * (g + q)) = make_uint2(0u, 0u);
                    }
                } else {
                    /* a column starts anywhere in the row and ends where the
                     * next begins: the groups' coefficients inside it only */
                    const int wl = (int)B.w - 4 * (int)g;
                    for (int c = 0; c < 4 * (int)nv && c < wl; c++)
                        if (!((s4 >> (8 * (c >> 2))) & 1u)) crow[4 * g + c] = 0;
                }
                const uint32_t cnt = tot >> 24;
                {
                    /* per byte: 1 for a listed group, and its data nibbles
                     * v - t + 1; their exclusive prefix sums over the lane's
                     * bytes give each entry's slot and offset */
                    const uint32_t one = s4 & 0x01010101u, dd = __vsubus4(v4, t4) + one;
                    const uint32_t po = dd * 0x01010100u, pi = one * 0x01010100u;
                    const uint32_t e0 = (o << 11) | ((uint32_t)lane << 6), i0 = ex >> 24;
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if ((one >> (8 * q)) & 1u)
                            list[i0 + ((pi >> (8 * q)) & 255u)] =
                                e0 + (((po >> (8 * q)) & 255u) << 13) + ((uint32_t)q << 4) + ((v4 >> (8 * q)) & 15u);
                }
                __syncwarp();
                for (uint32_t r = lane; r < cnt; r += 32) {
                    const uint32_t e = list[r];
                    const uint32_t gi = base + ((e >> 4) & 127u), v = e & 15u, np = v - t, ln = 4 * (np + 1);
                    const uint32_t pos = dpos + (e >> 11);
                    const uint32_t wi = pos >> 5, sh = pos & 31;
                    const uint32_t w0 = be_word(pbuf, wi), w1 = be_word(pbuf, wi + 1), w2 = be_word(pbuf, wi + 2);
                    const uint64_t win = ((uint64_t)__funnelshift_l(w1, w0, sh) << 32) | __funnelshift_l(w2, w1, sh);
                    const int wl = (int)B.w - 4 * (int)gi;
                    const uint2 ov = uniform ? decode_group(win >> (64 - ln), np, t, v, uniform, wl)
                                             : decode_group_dz(win >> (64 - ln), np, t, wl);
                    if (one_col) {
                        *(uint2*)(crow + 4 * gi) = ov;
                    } else {
                        const uint32_t vv[2] = {ov.x, ov.y};
#pragma unroll
                        for (int c = 0; c < 4; c++)
                            if (c < wl) crow[4 * gi + c] = (int16_t)((vv[c >> 1] >> (16 * (c & 1))) & 0xffffu);
                    }
                }
                __syncwarp();
                dpos += (tot & 0xffffffu) << 2;
            }
            continue;
        }
        uint32_t spos = P.sgpos + s_sgb[sidx];
        for (uint32_t base = sg.g0; base < gend; base += 32) {
            const uint32_t g = base + lane;
            const bool valid = g < gend;
            const uint32_t v = valid ? gcl[B.gbase + g] : 0u;
            const uint32_t np = v > L.t ? v - L.t : 0u;
            const uint32_t len = 4 * np; /* separate signs: planes only */
            uint32_t tot;
            const uint32_t ex = warp_excl_scan(len, &tot);
            uint2 o = make_uint2(0u, 0u);
            {
                uint32_t A = 0, B2 = 0, nz = 0;
                if (len) {
                    const uint32_t pos = dpos + ex;
                    const uint64_t win = ((uint64_t)bits32_at(pbuf, pos) << 32) | bits32_at(pbuf, pos + 32);
                    nz = group_mags(win >> (64 - len), np, L.t, v, uniform, &A, &B2);
                }
                /* this group's sign bits follow those of the lanes before it */
                uint32_t stot;
                const uint32_t sex = warp_excl_scan(__popc(nz), &stot);
                uint32_t sgn = 0;
                if (nz) {
                    const uint32_t sw = bits32_at(pbuf, spos + sex);
                    uint32_t k = 0;
#pragma unroll
                    for (int c = 3; c >= 0; c--) {
                        if (nz & (1u << c)) {
                            sgn |= ((sw >> (31 - k)) & 1u) << c;
                            k++;
                        }
                    }
                }
                if (len) o = group_finish(A, B2, sgn, uniform && L.t != 0, (int)B.w - 4 * (int)g);
                spos += stot;
            }
            if (valid) {
                if (one_col) {
                    *(uint2*)(crow + 4 * g) = o; /* the band row's padding takes the last group's tail */
                } else {
                    /* a column starts anywhere in the row and ends where the
                     * next begins: the group's coefficients inside it only */
                    const int wl = (int)B.w - 4 * (int)g;
                    crow[4 * g] = (int16_t)(o.x & 0xffffu);
                    if (wl > 1) crow[4 * g + 1] = (int16_t)(o.x >> 16);
                    if (wl > 2) crow[4 * g + 2] = (int16_t)(o.y & 0xffffu);
                    if (wl > 3) crow[4 * g + 3] = (int16_t)(o.y >> 16);
                }
            }
            dpos += tot;
        }
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) JXS_STATUS_SET(status, JXS_E_DEC_BITSTREAM);
    if (top_gcl) {
        /* slice-ordered decoding: this row is the next one's row above */
        for (uint32_t i = threadIdx.x; i < (cap_groups >> 2); i += blockDim.x) ((uint32_t*)top_gcl)[i] = ((const uint32_t*)gcl)[i];
        for (uint32_t x = threadIdx.x; x < nbl; x += blockDim.x) top_t[x] = ln[x].t;
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
DEV void walk_slice(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs, uint32_t size,
                    uint32_t* __restrict__ prec_off, int* walk_bad, const uint32_t s) {
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
    /* the slice's precincts: rows x columns, row after row */
    const uint32_t first = s * cfg->pps * cfg->ncol,
                   n = ((s + 1 == cfg->nslices) ? cfg->np - s * cfg->pps : cfg->pps) * cfg->ncol;
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
DEV void walk_sequential(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs, uint32_t size,
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
        const uint32_t first = s * cfg->pps * cfg->ncol,
                       n = ((s + 1 == cfg->nslices) ? cfg->np - s * cfg->pps : cfg->pps) * cfg->ncol;
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
/* kernels: one frame, or a batch of frames                                  */
/* ------------------------------------------------------------------------ */
/* 4 blocks of 512 threads per SM where the shared memory allows it (32
 * registers) */
__global__ void __launch_bounds__(UK_THREADS, 4) unpack_kernel(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs,
                                                               uint32_t bs_size, const uint32_t* __restrict__ prec_off,
                                                               int16_t* __restrict__ coef, uint32_t cap_bytes, uint32_t cap_groups,
                                                               uint32_t cap_seg, int* status) {
    unpack_body(cfg, bs, bs_size, prec_off, coef, cap_bytes, cap_groups, cap_seg, status, (int)blockIdx.x, nullptr, nullptr, 0);
}

/* cap_bytes / cap_groups / cap_seg: the largest of the batch's frames
 * (shared-memory layout of the launch) */
__global__ void __launch_bounds__(UK_THREADS, 4) unpack_batch_kernel(const __grid_constant__ DecPrecLaunch L, uint32_t cap_bytes,
                                                                     uint32_t cap_groups, uint32_t cap_seg) {
    const DecPrecFrame& F = L.job[find_job<JXS_BATCH_FRAMES>(L.job, L.nframes, (int)blockIdx.x)];
    unpack_body(F.cfg, F.bs, F.bs_size, F.prec_off, F.coef, cap_bytes, cap_groups, cap_seg, F.status,
                (int)blockIdx.x - F.first_block, nullptr, nullptr, 0);
}

/* Streams with vertical prediction: one block per slice, its precinct rows
 * in order, each predicting from the row above (kept in shared memory after
 * the zero-bit table: cap_groups bytes); with several precinct columns,
 * column after column (the precinct above is in the same column). */
__global__ void __launch_bounds__(UK_THREADS) unpack_vpred_kernel(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs,
                                                                  uint32_t bs_size, const uint32_t* __restrict__ prec_off,
                                                                  int16_t* __restrict__ coef, uint32_t cap_bytes,
                                                                  uint32_t cap_groups, uint32_t cap_seg, int* status) {
    extern __shared__ __align__(16) uint8_t dsm[];
    __shared__ uint8_t top_t[JXS_MAXBLINES];
    uint8_t* top_gcl = dsm + uk_layout(cap_bytes, cap_groups, cap_seg).top;
    const uint32_t s = blockIdx.x, ncol = cfg->ncol;
    const uint32_t first = s * cfg->pps, end = min(cfg->np, first + cfg->pps);
    for (uint32_t col = 0; col < ncol; col++) {
        for (uint32_t row = first; row < end; row++) {
            unpack_body(cfg, bs, bs_size, prec_off, coef, cap_bytes, cap_groups, cap_seg, status, (int)(row * ncol + col), top_gcl,
                        top_t, row != first);
            __syncthreads();
            if (*(volatile int*)status) return;
        }
    }
}

__global__ void walk_slices_kernel(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs, uint32_t size,
                                   uint32_t* __restrict__ prec_off, int* walk_bad) {
    walk_slice(cfg, bs, size, prec_off, walk_bad, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void walk_sequential_kernel(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ bs, uint32_t size,
                                       uint32_t* __restrict__ prec_off, const int* walk_bad, int* status) {
    walk_sequential(cfg, bs, size, prec_off, walk_bad, status);
}

/* one thread per slice of every frame of the batch */
__global__ void walk_slices_batch_kernel(const __grid_constant__ DecPrecLaunch L) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= L.nslices) return;
    int lo = 0, hi = L.nframes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (g >= L.job[mid].first_slice) lo = mid;
        else hi = mid - 1;
    }
    const DecPrecFrame& F = L.job[lo];
    walk_slice(F.cfg, F.bs, F.bs_size, F.prec_off, F.status + 1, (uint32_t)(g - F.first_slice));
}

/* one thread per frame of the batch */
__global__ void walk_sequential_batch_kernel(const __grid_constant__ DecPrecLaunch L) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= L.nframes) return;
    const DecPrecFrame& F = L.job[f];
    walk_sequential(F.cfg, F.bs, F.bs_size, F.prec_off, F.status + 1, F.status);
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

extern "C" cudaError_t jxs_launch_unpack(const jxs_cfg_t* dcfg, const uint8_t* bs, uint32_t bs_size, const uint32_t* prec_off,
                                         int16_t* coef, uint32_t np, uint32_t cap_bytes, uint32_t cap_groups, uint32_t cap_seg,
                                         int* status, cudaStream_t st) {
    const size_t smem = uk_layout(cap_bytes, cap_groups, cap_seg).end;
    static std::atomic<int> attr[JXS_MAX_DEV];
    cudaError_t e = jxs_smem_attr(unpack_kernel, (int)smem, attr);
    if (e != cudaSuccess) return e;
    unpack_kernel<<<np, UK_THREADS, smem, st>>>(dcfg, bs, bs_size, prec_off, coef, cap_bytes, cap_groups, cap_seg, status);
    return cudaGetLastError();
}


extern "C" cudaError_t jxs_launch_walk_batch(const DecPrecLaunch* L, cudaStream_t st) {
    if (L->nframes <= 0) return cudaSuccess;
    walk_slices_batch_kernel<<<(L->nslices + 127) / 128, 128, 0, st>>>(*L);
    walk_sequential_batch_kernel<<<(L->nframes + 31) / 32, 32, 0, st>>>(*L);
    return cudaGetLastError();
}

extern "C" cudaError_t jxs_launch_unpack_batch(const DecPrecLaunch* L, uint32_t cap_bytes, uint32_t cap_groups, uint32_t cap_seg,
                                               cudaStream_t st) {
    const size_t smem = uk_layout(cap_bytes, cap_groups, cap_seg).end;
    static std::atomic<int> attr[JXS_MAX_DEV];
    cudaError_t e = jxs_smem_attr(unpack_batch_kernel, (int)smem, attr);
    if (e != cudaSuccess) return e;
    if (L->nblocks <= 0) return cudaSuccess;
    unpack_batch_kernel<<<L->nblocks, UK_THREADS, smem, st>>>(*L, cap_bytes, cap_groups, cap_seg);
    return cudaGetLastError();
}

extern "C" cudaError_t jxs_launch_unpack_vpred(const jxs_cfg_t* dcfg, const uint8_t* bs, uint32_t bs_size, const uint32_t* prec_off,
                                               int16_t* coef, uint32_t nslices, uint32_t cap_bytes, uint32_t cap_groups,
                                               uint32_t cap_seg, int* status, cudaStream_t st) {
    const size_t smem = uk_layout(cap_bytes, cap_groups, cap_seg).top_end;
    static std::atomic<int> attr[JXS_MAX_DEV];
    cudaError_t e = jxs_smem_attr(unpack_vpred_kernel, (int)smem, attr);
    if (e != cudaSuccess) return e;
    unpack_vpred_kernel<<<nslices, UK_THREADS, smem, st>>>(dcfg, bs, bs_size, prec_off, coef, cap_bytes, cap_groups, cap_seg,
                                                           status);
    return cudaGetLastError();
}
