/*
 * Encoder kernels for sm_103a (the forward transform is in jxs_fwd_dwt.cu).
 *
 *  rc_cost_kernel   per precinct row: GCLI histograms and the byte cost of
 *                   every (quantization, refinement) candidate.
 *                   The block that completes a slice then replays the
 *                   reference's sequential budget carry and binary searches
 *                   for that slice over the cost tables.
 *  pack_kernel      per precinct row: quantization and bit packing at
 *                   prefix-summed bit offsets into a shared-memory copy of the
 *                   precinct, then one coalesced copy to the codestream.
 *
 * Integer arithmetic follows the reference one to one (citations inline).
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "jxs_core.h"
#include "jxs_kernels.cuh"

#define DEV __device__ __forceinline__

/* ------------------------------------------------------------------------ */
/* Rate control                                                              */
/* ------------------------------------------------------------------------ */
#define FULL 0xffffffffu
#define RC_THREADS 512
#define RC_WARPS (RC_THREADS / 32)
/* shared area of the rate control: 5 tables of 16 words per band line, 6
 * with sign handling */
#define RC_AREA_WORDS(signs) (((signs) ? 6 : 5) * JXS_MAXBLINES * 16)

/* binary_search_init / binary_search_next_step (BinarySearch.c:9-78) */
struct BSearch {
    int beg, end, step, best, last, below;
};
DEV void bs_init(BSearch& s, int beg, int end, int below, int step) {
    s.beg = beg; s.end = end; s.below = below; s.best = -1; s.last = -1;
    s.step = step ? step : (end - beg) / 2;
}
enum { BS_BEGIN = 0, BS_TOO_SMALL, BS_TOO_BIG, BS_OUT_OF_RANGE };
enum { BS_CONTINUE = 0, BS_FOUND, BS_ERROR };
DEV int bs_next(BSearch& s, int res, int* out) {
    if (res == BS_TOO_SMALL) {
        if (s.below && (s.best == -1 || s.best < s.last)) s.best = s.last;
        if (s.end >= s.last + 1) s.beg = s.last + 1;
        else {
            if (s.best == -1) return BS_ERROR;
            *out = s.best;
            return BS_FOUND;
        }
    } else if (res == BS_TOO_BIG || res == BS_OUT_OF_RANGE) {
        if (res == BS_TOO_BIG && !s.below && (s.best == -1 || s.best > s.last)) s.best = s.last;
        if (s.beg <= s.last - 1) s.end = s.last - 1;
        else {
            if (s.best == -1) return BS_ERROR;
            *out = s.best;
            return BS_FOUND;
        }
    }
    if (s.step > s.end - s.beg) s.step = (s.end - s.beg + 1) / 2;
    s.last = s.step + s.beg;
    *out = s.last;
    return BS_CONTINUE;
}

/* A slice's even split of its budget over its precincts
 * (PackStageProcess.c:600-684): mode 1 gives the first precinct 10 % more
 * (20 % with fast signs, :34-35). */
struct SliceSplit {
    uint32_t slice_budget, first_p, nprec, first_b, min_b, left;
};
DEV SliceSplit slice_split(const jxs_cfg_t* __restrict__ cfg, int s) {
    SliceSplit o;
    const int last_slice = (s + 1 == (int)cfg->nslices);
    o.slice_budget = cfg->slice_size[s] - 6 - (last_slice ? 2 : 0);
    o.first_p = cfg->pps * s;
    o.nprec = last_slice ? cfg->np - o.first_p : cfg->pps;
    o.min_b = o.slice_budget / o.nprec;
    o.left = o.slice_budget - o.min_b * o.nprec;
    o.first_b = o.min_b;
    if (cfg->rc_mode == 1) {
        o.first_b = min(o.slice_budget, o.first_b * (cfg->signs == 1 ? 120u : 110u) / 100);
        if (o.nprec > 1) {
            o.min_b = (o.slice_budget - o.first_b) / (o.nprec - 1);
            o.left = o.slice_budget - o.min_b * (o.nprec - 1) - o.first_b;
        } else {
            o.left = 0;
        }
    }
    return o;
}

/* The precinct searches of rate_control_precinct (RateControl.c:1259-1333,
 * binary searches :889-1083), by one thread on tables in shared memory
 * ([q * nr + r]): the quantization by binary
 * search on T[q * nr]; with `scan` (full signs, vertical prediction) then
 * lower quantizations while TS fits, else the first higher one that fits
 * (:936-1015); the refinement by binary search on TS.  Returns an error
 * code, 0 when q, r and data (TS at (q, r)) are set. */
DEV int prec_search(const uint32_t* T, const uint32_t* TS, int ld, int scan, int nr, int max_q, int max_r,
                    const uint32_t* __restrict__ s_empty, uint32_t avail, int& q, int& r, uint32_t& data) {
    BSearch bs;
    int step = 6;
    if (step > max_q) step = 0;
    bs_init(bs, 0, max_q, 0, step);
    int res, next = BS_BEGIN, v = 0;
    while ((res = bs_next(bs, next, &v)) == BS_CONTINUE) {
        if (s_empty[v] & 1u) next = BS_OUT_OF_RANGE;
        else next = T[v * nr] > avail ? BS_TOO_SMALL : BS_TOO_BIG;
    }
    if (res != BS_FOUND) return JXS_E_ENC_FRAME;
    q = v;
    if (scan) {
        int best = -1;
        for (int qt = q - 1; qt >= 0; qt--) {
            if ((s_empty[qt] & 1u) || TS[qt * ld] > avail) break;
            best = qt;
        }
        if (best < 0)
            for (int qt = q; qt <= max_q; qt++)
                if (!(s_empty[qt] & 1u) && TS[qt * ld] <= avail) {
                    best = qt;
                    break;
                }
        if (best < 0) return JXS_E_ENC_FRAME;
        q = best;
    }
    step = 6;
    if (step >= max_r) step = 0;
    bs_init(bs, 0, max_r, 1, step);
    next = BS_BEGIN;
    while ((res = bs_next(bs, next, &v)) == BS_CONTINUE) {
        if ((s_empty[q] >> v) & 1u) next = BS_OUT_OF_RANGE;
        else next = TS[q * ld + v] <= avail ? BS_TOO_SMALL : BS_TOO_BIG;
    }
    if (res != BS_FOUND) return JXS_E_ENC_FRAME;
    r = v;
    data = TS[q * ld + r];
    return 0;
}

/* RC modes 2 and 3, per-slice common quantization (process_slice,
 * PackStageProcess.c:339-483; RateControl.c:1086-1209, 1336-1425): the
 * (fast-sign) data bytes of every (Q, R) summed over the slice's precincts
 * into `area`, one (Q, R) for the slice by the precinct searches, then the
 * budget of each precinct, kept in rc[p].total_bytes.  Run by a whole
 * block; returns the error (every thread). */
DEV int slice_common(const jxs_cfg_t* __restrict__ cfg, int s, const SliceSplit& sp, const uint32_t* __restrict__ cost,
                     uint32_t* area, const uint32_t* __restrict__ s_empty, PrecRC* __restrict__ rc, int* __restrict__ status) {
    __shared__ int s_cerr;
    const int nq = cfg->max_q + 1, nr = cfg->max_r + 1, nt = nq * nr;
    const int max_q = cfg->max_q, max_r = cfg->max_r, rc_mode = (int)cfg->rc_mode;
    const uint32_t np_all = cfg->np, hdrs0 = cfg->hdrs_bytes[0], hdrs1 = cfg->hdrs_bytes[1];
    const uint32_t first_p = sp.first_p, nprec = sp.nprec, slice_budget = sp.slice_budget;
    __syncthreads();
    for (int e = threadIdx.x; e < nt; e += blockDim.x) {
        const int q = e / nr, r = e - q * nr;
        uint32_t sum = 0;
        for (uint32_t i = 0; i < nprec; i++) sum += __ldcg(cost + (uint64_t)(first_p + i) * 1024 + q * 32 + r);
        area[e] = sum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int err = 0;
        uint32_t headers = 0;
        for (uint32_t i = 0; i < nprec; i++) headers += first_p + i + 1 >= np_all ? hdrs1 : hdrs0;
        if ((slice_budget + nprec - 1) / nprec > JXS_PREC_MAX_BYTES) err = JXS_E_ENC_FRAME;
        else if (slice_budget <= headers) err = JXS_E_UNDEFINED;
        int q = 0, r = 0;
        uint32_t dsum = 0;
        if (!err) err = prec_search(area, area, nr, 0, nr, max_q, max_r, s_empty, slice_budget - headers, q, r, dsum);
        if (!err) {
            /* each precinct its headers and data at (Q, R); the last also
             * the slice's remaining bytes */
            uint32_t pad_last = slice_budget - headers;
            for (uint32_t i = 0; i < nprec; i++) {
                const uint32_t p = first_p + i;
                const uint32_t d = __ldcg(cost + (uint64_t)p * 1024 + q * 32 + r);
                pad_last -= d;
                rc[p].total_bytes = (p + 1 >= np_all ? hdrs1 : hdrs0) + d;
            }
            rc[first_p + nprec - 1].total_bytes += pad_last;
            if (rc_mode == 3) {
                /* RC_CBR_PER_SLICE_COMMON_QUANT_MAX_RATE: no precinct below a
                 * quarter of the largest, padding excluded */
                uint32_t max_size = 0;
                for (uint32_t i = 0; i < nprec; i++)
                    max_size = max(max_size, rc[first_p + i].total_bytes - (i + 1 == nprec ? pad_last : 0u));
                const uint32_t min_size = max_size / 4;
                uint32_t need = 0;
                for (uint32_t i = 0; i < nprec; i++) {
                    const uint32_t ds = rc[first_p + i].total_bytes - (i + 1 == nprec ? pad_last : 0u);
                    if (ds < min_size) {
                        rc[first_p + i].total_bytes += min_size - ds;
                        need += min_size - ds;
                    }
                }
                if (need) {
                    if (pad_last >= need) {
                        pad_last -= need;
                        rc[first_p + nprec - 1].total_bytes -= need;
                    } else {
                        need -= pad_last;
                        rc[first_p + nprec - 1].total_bytes -= pad_last;
                        pad_last = 0;
                        /* the rest one byte at a time, round robin */
                        const uint32_t each = need / nprec, extra = need - each * nprec;
                        for (uint32_t i = 0; i < nprec; i++) rc[first_p + i].total_bytes -= each + (i < extra ? 1u : 0u);
                    }
                }
            }
            if (pad_last > 0) {
                /* the first precinct 10 % more (20 % with fast signs), the
                 * rest of the padding shared evenly */
                uint32_t add_first = rc[first_p].total_bytes * (cfg->signs == 1 ? 20u : 10u) / 100;
                if (add_first > pad_last) add_first = pad_last;
                pad_last -= add_first;
                rc[first_p + nprec - 1].total_bytes -= add_first;
                rc[first_p].total_bytes += add_first;
                if (pad_last) {
                    rc[first_p + nprec - 1].total_bytes -= pad_last;
                    const uint32_t each = pad_last / nprec, extra = pad_last - each * nprec;
                    for (uint32_t i = 0; i < nprec; i++) rc[first_p + i].total_bytes += each + (i < extra ? 1u : 0u);
                }
            }
        }
        if (err) {
            printf("jxs rc: slice %d (common quantization): error 0x%x\n", s, (unsigned)err);
            JXS_STATUS_SET(status, err);
        }
        s_cerr = err;
    }
    __syncthreads();
    return s_cerr;
}

/* One precinct's budget, searches and padding carry; thread 0.  `T` is the
 * table of the quantization search, `F` the exact-sign table (fast signs:
 * the bytes of the signs not sent are T - F at the chosen (Q, R)), `TS` the
 * table of the scan and the refinement search (row stride `ld`); all in
 * shared memory.
 * Modes 1-3 carry the padding (and fast signs' unsent sign bytes) to the
 * next precinct of the slice; a slice's last precinct and mode 0 keep them
 * as zero bytes (PackStageProcess.c:293-333, 526-560,
 * PackPrecinct.c:513-536).  Returns an error code. */
DEV int prec_select(const jxs_cfg_t* __restrict__ cfg, int s, uint32_t i, const SliceSplit& sp, const uint32_t* T,
                    const uint32_t* F, const uint32_t* TS, int ld, int scan, const uint32_t* __restrict__ s_empty, uint32_t& carry,
                    uint32_t& run, PrecRC* __restrict__ rc, int* __restrict__ status) {
    const uint32_t p = sp.first_p + i;
    const int last = (p + 1 >= cfg->np);
    const uint32_t budget =
        (cfg->rc_mode >= 2 ? rc[p].total_bytes : (i == 0 ? sp.first_b : sp.min_b) + (i < sp.left ? 1 : 0)) + carry;
    const uint32_t hdr = cfg->hdrs_bytes[last];
    const int nr = cfg->max_r + 1;
    int err = 0;
    if (budget > JXS_PREC_MAX_BYTES) err = JXS_E_ENC_FRAME;
    else if (budget <= hdr) err = JXS_E_UNDEFINED;
    int q = 0, r = 0;
    uint32_t data = 0;
    if (!err) err = prec_search(T, TS, ld, scan, nr, cfg->max_q, cfg->max_r, s_empty, budget - hdr, q, r, data);
    if (!err) {
        const uint32_t padding = budget - hdr - data;
        uint32_t total = budget;
        const uint32_t retrieve = cfg->signs == 1 ? T[q * nr + r] - F[q * nr + r] : 0u;
        if (cfg->rc_mode >= 1 && i + 1 < sp.nprec) {
            total -= padding + retrieve;
            carry = padding + retrieve;
        } else {
            carry = 0;
        }
        PrecRC o;
        o.total_bytes = total;
        o.offset = run;
        o.data_bytes = data - retrieve; /* the sub-packet bytes packed */
        o.q = (uint8_t)q;
        o.r = (uint8_t)r;
        o.first_in_slice = (uint8_t)(i == 0);
        o.pad = 0;
        rc[p] = o;
        run += total;
    } else {
        printf("jxs rc: slice %d precinct %u budget %u: error 0x%x\n", s, p, budget, (unsigned)err);
        JXS_STATUS_SET(status, err);
    }
    return err;
}

/* One slice's selection without vertical prediction, on the slice's cost
 * tables: the tables of up to `area_words / (nq * nr * tables)` precincts
 * are read (through L2) into `area` at a time; thread 0 then runs their
 * searches in order.  With sign handling each precinct has two tables:
 * signs counted the fast way (every coefficient of a group above gtli) and
 * exactly; the quantization search runs on the fast one, the full strategy
 * then scans and searches the refinement on the exact one. */
DEV void select_slice(const jxs_cfg_t* __restrict__ cfg, int s, const uint32_t* __restrict__ cost, uint32_t* area,
                      uint32_t area_words, PrecRC* __restrict__ rc, int* __restrict__ status) {
    __shared__ uint32_t s_carry, s_run;
    __shared__ int s_err;
    __shared__ uint32_t s_empty[32];
    if (threadIdx.x < 32) s_empty[threadIdx.x] = cfg->empty[threadIdx.x];
    const SliceSplit sp = slice_split(cfg, s);
    if (threadIdx.x == 0) {
        s_carry = 0;
        s_run = cfg->slice_begin[s] + 6;
        s_err = 0;
    }
    const int nq = cfg->max_q + 1, nr = cfg->max_r + 1, nt = nq * nr;
    const uint32_t np_all = cfg->np, signs = cfg->signs;
    __syncthreads();
    if (cfg->rc_mode >= 2 && slice_common(cfg, s, sp, cost, area, s_empty, rc, status)) return;
    const int ntab = signs ? 2 : 1;
    const uint32_t chunk = area_words / (uint32_t)(nt * ntab);
    for (uint32_t c0 = 0; c0 < sp.nprec; c0 += chunk) {
        const uint32_t cnt = min(chunk, sp.nprec - c0);
        __syncthreads();
        if (s_err) break;
        for (int e = threadIdx.x; e < (int)cnt * nt * ntab; e += blockDim.x) {
            const int i = e / (nt * ntab), rest = e - i * nt * ntab, tb = rest / nt, qr = rest - tb * nt, q = qr / nr,
                      r = qr - q * nr;
            area[e] = __ldcg(cost + ((uint64_t)tb * np_all + sp.first_p + c0 + i) * 1024 + q * 32 + r);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint32_t ii = 0; ii < cnt && !s_err; ii++) {
                const uint32_t* T = area + ii * nt * ntab;
                const uint32_t* F = signs ? T + nt : T; /* exact signs */
                uint32_t carry = s_carry, run = s_run;
                s_err = prec_select(cfg, s, c0 + ii, sp, T, F, signs == 2 ? F : T, nr, signs == 2, s_empty, carry, run, rc, status);
                s_carry = carry;
                s_run = run;
            }
        }
    }
}

/* Vertical prediction (RateControl.c:586-676): line tables stored by every
 * precinct's block for the ordered selection, and the shared regions of
 * that selection */
#define RC_LT_REGION (JXS_MAXBLINES * 16)
#define RC_LT_WORDS (5 * RC_LT_REGION) /* data, GCLI bits, GCLI bits with significance, fast / full sign bits */
#define RC_VP_REGIONS 10

/* vlc_encode_get_bits (PackPrecinct.h:86-104): ones of the unary code of a
 * GCLI difference x for the vertical prediction range (r, t). */
DEV uint32_t vlc_vp_bits(int x, int r, int t) {
    const int mx = max(r - t, 0);
    if (x > mx) return (uint32_t)(x + mx);
    x *= 2;
    return (uint32_t)(x < 0 ? -x - 1 : x);
}

/* One slice's selection with vertical prediction, precinct after precinct
 * (the costs of a row depend on the gtli chosen for the row above,
 * RateControl.c:586-676), by the block that completes the slice.  Per
 * precinct:
 *   tables   its line tables and (fast-sign) cost tables from the other
 *            blocks;
 *   vpred    warp per segment: for every gtli t, the unary bits of each
 *            GCLI coded from the line above (line 0: the band's last line
 *            in the row above, with that row's gtli) and the bits the
 *            significance groups without code save (run mode Rm: groups
 *            with every GCLI <= t; else groups predicted exactly);
 *   methods  per band and t: no significance, significance, prediction,
 *            prediction with significance; a later one only if strictly
 *            cheaper;
 *   costs    as in the parallel pass, with those methods and exact signs
 *            for the full strategy;
 *   search   thread 0: quantization on the plain table, then the scan and
 *            refinement on the prediction table (:909-1083). */
template <typename Stage>
DEV void select_slice_vpred(const jxs_cfg_t* __restrict__ cfg, int s, const uint8_t* __restrict__ gcli,
                            const uint32_t* __restrict__ cost, uint32_t* area, PrecRC* __restrict__ rc,
                            int* __restrict__ status, Stage& stage_kind, const uint8_t* lgain, const uint8_t* lprio,
                            const uint8_t* lfb, const uint32_t* lsig, const uint32_t* lraw, const jxs_bline_t* bls,
                            const jxs_seg_t* segs, const uint8_t* s_pkbl0, const uint8_t* s_pknbl, const uint8_t* s_order) {
    __shared__ uint32_t s_carry, s_run;
    __shared__ int s_err;
    __shared__ uint32_t s_empty[32];
    __shared__ uint8_t s_gtop[JXS_MAXBL], s_bl0[JXS_MAXBL], s_bl1[JXS_MAXBL];
    __shared__ uint32_t s_methv[JXS_MAXBL]; /* per band: 2 bits per t */
    uint32_t(*vtfs)[16] = (uint32_t(*)[16])area;
    uint32_t(*dV)[32] = (uint32_t(*)[32])(area + RC_LT_REGION);
    uint32_t(*vtdat)[16] = (uint32_t(*)[16])(area + 2 * RC_LT_REGION);
    uint32_t(*vtnos)[16] = (uint32_t(*)[16])(area + 3 * RC_LT_REGION);
    uint32_t(*vtsig)[16] = (uint32_t(*)[16])(area + 4 * RC_LT_REGION);
    uint32_t(*vtnz)[16] = (uint32_t(*)[16])(area + 5 * RC_LT_REGION);
    uint32_t(*vnos)[16] = (uint32_t(*)[16])(area + 6 * RC_LT_REGION);
    uint32_t(*vred)[16] = (uint32_t(*)[16])(area + 7 * RC_LT_REGION);
    uint32_t* Ts = area + 8 * RC_LT_REGION;
    uint32_t* Fs = area + 9 * RC_LT_REGION;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < 32) s_empty[threadIdx.x] = cfg->empty[threadIdx.x];
    const SliceSplit sp = slice_split(cfg, s);
    if (threadIdx.x == 0) {
        s_carry = 0;
        s_run = cfg->slice_begin[s] + 6;
        s_err = 0;
    }
    const int nq = cfg->max_q + 1, nr = cfg->max_r + 1, nt = nq * nr;
    const uint32_t np_all = cfg->np, signs = cfg->signs, fs = cfg->fs, SG = cfg->seg_groups, npk = cfg->npk;
    const uint32_t nbands = cfg->nbands, sig = cfg->sig;
    const int rm = cfg->rm;
    __syncthreads();
    if (cfg->rc_mode >= 2 && slice_common(cfg, s, sp, cost, Ts, s_empty, rc, status)) return;
    int kind_staged = -1;
    for (uint32_t i = 0; i < sp.nprec; i++) {
        const uint32_t p = sp.first_p + i;
        const int kind = (p + 1 >= np_all);
        __syncthreads();
        if (s_err) break;
        if (kind != kind_staged) {
            stage_kind(kind);
            kind_staged = kind;
            __syncthreads();
        }
        const uint32_t nbl = cfg->nbline[kind], nseg = cfg->nseg[kind];
        /* the lines of each band (at most two per precinct row) */
        for (uint32_t fb = threadIdx.x; fb < nbands; fb += blockDim.x) {
            s_bl0[fb] = 0xff;
            s_bl1[fb] = 0xff;
            s_methv[fb] = 0;
        }
        __syncthreads();
        for (uint32_t x = threadIdx.x; x < nbl; x += blockDim.x) {
            if (bls[x].line == 0) s_bl0[bls[x].fb] = (uint8_t)x;
            else s_bl1[bls[x].fb] = (uint8_t)x;
        }
        /* this row's tables from the other blocks */
        const uint32_t* lt = cost + (uint64_t)np_all * 1024 * (fs ? 2 : 1) + (uint64_t)p * RC_LT_WORDS;
        for (uint32_t k = threadIdx.x; k < nbl * 16; k += blockDim.x) {
            const uint32_t x = k >> 4, t = k & 15;
            vtdat[x][t] = __ldcg(lt + k);
            vtnos[x][t] = __ldcg(lt + RC_LT_REGION + k);
            vtsig[x][t] = __ldcg(lt + 2 * RC_LT_REGION + k);
            if (fs) {
                vtfs[x][t] = __ldcg(lt + 3 * RC_LT_REGION + k);
                vtnz[x][t] = __ldcg(lt + 4 * RC_LT_REGION + k);
            }
            vnos[x][t] = 0;
            vred[x][t] = 0;
        }
        for (int e = threadIdx.x; e < nt; e += blockDim.x) {
            const int q = e / nr, r = e - q * nr;
            Ts[e] = __ldcg(cost + (uint64_t)p * 1024 + q * 32 + r);
            if (fs) Fs[e] = __ldcg(cost + ((uint64_t)np_all + p) * 1024 + q * 32 + r);
        }
        for (int e = threadIdx.x; e < nq * 32; e += blockDim.x) dV[e >> 5][e & 31] = 0;
        __syncthreads();
        /* vertical prediction costs of every line, for every t */
        if (i > 0) {
            for (uint32_t sidx = warp; sidx < nseg; sidx += RC_WARPS) {
                const jxs_seg_t sg = segs[sidx];
                const uint32_t x = sg.bl;
                const jxs_bline_t B = bls[x];
                const jxs_band_t& bd = cfg->band[B.fb];
                const uint8_t* cur = gcli + bd.gcli_off + (uint64_t)(p * bd.lines + B.line) * bd.gpitch;
                const uint8_t* top = cur - bd.gpitch; /* the row above: the previous line, for line 0 in the row above */
                const int gtt = B.line ? -1 : (int)s_gtop[B.fb];
                const uint32_t gend = min(sg.g0 + SG, B.gcli_w);
                for (uint32_t base = sg.g0; base < gend; base += 128) {
                    const uint32_t g = base + 4 * lane;
                    const uint32_t nv = g < gend ? min(4u, gend - g) : 0u;
                    const uint32_t wc = nv ? *(const uint32_t*)(cur + g) : 0u, wt = nv ? *(const uint32_t*)(top + g) : 0u;
                    for (int t = 0; t < 16; t++) {
                        const int gmax = max(t, gtt);
                        uint32_t sum = 0, flag = 1;
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            if (k < (int)nv) {
                                const int c = (int)((wc >> (8 * k)) & 255u), tp = (int)((wt >> (8 * k)) & 255u);
                                const int mt = max(tp, gmax), gv = max(c, t);
                                sum += vlc_vp_bits(gv - mt, mt, t) + 1;
                                flag &= rm ? (uint32_t)(c <= t) : (uint32_t)(mt == gv);
                            }
                        }
                        /* significance group of 8 GCLIs: lanes 2j, 2j + 1 */
                        const uint32_t f2 = flag & __shfl_xor_sync(FULL, flag, 1);
                        const uint32_t s2 = sum + __shfl_xor_sync(FULL, sum, 1);
                        const uint32_t red = (!(lane & 1) && f2) ? s2 : 0u;
                        const uint32_t tot = __reduce_add_sync(FULL, sum), rtot = __reduce_add_sync(FULL, red);
                        if (lane == 0) {
                            if (tot) atomicAdd(&vnos[x][t], tot);
                            if (rtot) atomicAdd(&vred[x][t], rtot);
                        }
                    }
                }
            }
        }
        __syncthreads();
        /* coding method per band and t (RateControl.c:526-676) */
        for (uint32_t e = threadIdx.x; e < nbands * 16; e += blockDim.x) {
            const uint32_t fb = e >> 4, t = e & 15;
            const uint32_t x0 = s_bl0[fb], x1 = s_bl1[fb];
            if (x0 == 0xff) continue;
            uint32_t cnv = vtnos[x0][t], csv = vtsig[x0][t] + lsig[x0], vn = vnos[x0][t], vs = vnos[x0][t] - vred[x0][t] + lsig[x0];
            if (x1 != 0xff) {
                cnv += vtnos[x1][t];
                csv += vtsig[x1][t] + lsig[x1];
                vn += vnos[x1][t];
                vs += vnos[x1][t] - vred[x1][t] + lsig[x1];
            }
            uint32_t m = 0, best = cnv;
            if (sig && best > csv) {
                m = 2;
                best = csv;
            }
            if (i > 0) {
                if (best > vn) {
                    m = 1;
                    best = vn;
                }
                if (sig && best > vs) m = 3;
            }
            atomicOr(&s_methv[fb], m << (2 * t));
        }
        __syncthreads();
        /* costs with those methods, per (Q, packet) as in the parallel pass */
        auto gbits = [&](uint32_t x, uint32_t m, int t) -> uint32_t {
            return m == 0 ? vtnos[x][t] : m == 2 ? vtsig[x][t] : m == 1 ? vnos[x][t] : vnos[x][t] - vred[x][t];
        };
        auto nbits = [&](uint32_t x, int t) -> uint32_t { return signs == 2 ? vtnz[x][t] : signs == 1 ? vtfs[x][t] : 0u; };
        for (uint32_t e = threadIdx.x; e < (uint32_t)nq * npk; e += blockDim.x) {
            const int q = (int)(e / npk);
            const uint32_t k = e - (uint32_t)q * npk;
            const uint32_t b0 = s_pkbl0[k], nb = s_pknbl[k];
            if (!nb) continue;
            uint32_t db = 0, gb = 0, sb = 0, zb = 0;
            for (uint32_t x = b0; x < b0 + nb; x++) {
                const int g = lgain[x];
                const int t = q < g ? 0 : min(q - g, 15);
                const uint32_t m = (s_methv[lfb[x]] >> (2 * t)) & 3u;
                db += vtdat[x][t];
                gb += gbits(x, m, t);
                sb += (m & 2u) ? lsig[x] : 0u;
                zb += nbits(x, t);
            }
            uint32_t c = ((db + 7) >> 3) + min(lraw[k], ((sb + 7) >> 3) + ((gb + 7) >> 3)) + ((zb + 7) >> 3);
            atomicAdd(&dV[q][0], c);
            for (uint32_t j = 0; j < nb; j++) {
                const uint32_t x = s_order[b0 + j];
                const int rf = lprio[x] + 1;
                if (rf >= nr) break;
                const int g = lgain[x];
                const int t0 = q < g ? 0 : min(q - g, 15), t1 = q < g + 1 ? 0 : min(q - g - 1, 15);
                const uint32_t m0 = (s_methv[lfb[x]] >> (2 * t0)) & 3u, m1 = (s_methv[lfb[x]] >> (2 * t1)) & 3u;
                db += vtdat[x][t1] - vtdat[x][t0];
                gb += gbits(x, m1, t1) - gbits(x, m0, t0);
                sb += ((m1 & 2u) ? lsig[x] : 0u) - ((m0 & 2u) ? lsig[x] : 0u);
                zb += nbits(x, t1) - nbits(x, t0);
                const uint32_t c1 = ((db + 7) >> 3) + min(lraw[k], ((sb + 7) >> 3) + ((gb + 7) >> 3)) + ((zb + 7) >> 3);
                atomicAdd(&dV[q][rf], c1 - c);
                c = c1;
            }
        }
        __syncthreads();
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            uint32_t run = 0;
            for (int r = 0; r < nr; r++) {
                run += dV[q][r];
                dV[q][r] = run;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t carry = s_carry, run = s_run;
            s_err = prec_select(cfg, s, i, sp, Ts, fs ? Fs : Ts, &dV[0][0], 32, 1, s_empty, carry, run, rc, status);
            s_carry = carry;
            s_run = run;
            if (!s_err) {
                const PrecRC o = rc[p];
                for (uint32_t fb = 0; fb < nbands; fb++) s_gtop[fb] = jxs_truncation(cfg->band[fb].gain, cfg->band[fb].prio, o.q, o.r);
            }
        }
    }
}

/* Number of gtli values t (from 0 up) at which a coefficient of magnitude m
 * in a group with GCLI g stays non-zero after quantization
 * (rate_control_lut_fill, RateControl.c:124-137, and
 * rate_control_sign_coding_get_sum_nonzero_coeff_c, :366-455): the bits of
 * m for deadzone quantization; for uniform quantization the value
 * ((m << (g - t + 1)) - m + 2^g) >> (g + 1) falls as t grows and is non-zero
 * while m (2^(g-t+1) - 1) >= 2^g. */
DEV uint32_t nz_levels(uint32_t m, uint32_t g, uint32_t uniform) {
    if (!m) return 0;
    if (!uniform) return 32 - __clz(m);
    uint32_t n = 0;
    while (n < g && m * ((2u << (g - n)) - 1u) >= (1u << g)) n++;
    return n;
}

/* Byte cost of every (quantization, refinement) candidate of one precinct
 * row: rate_control_lut_fill, rate_control_calculate_band_best_method and
 * precinct_get_budget_bytes (RateControl.c:18-154, 457-781).
 *   histograms  warp per segment: GCLI histogram of every band line
 *               (warp-aggregated shared atomics) and the line's groups by
 *               the maximum GCLI of their significance group; each segment's
 *               own two histograms also go to device memory for packing
 *               (segments of at most 128 groups);
 *   tables      thread per band line: for every gtli t, data bits, GCLI bits
 *               without significance and with it (suffix sums over the
 *               histogram); per band, significance coding at t only if
 *               strictly cheaper over all its lines;
 *   costs       per packet, data / significance / GCLI bytes rounded
 *               separately, raw fallback when cheaper; summed over packets
 *               for every (Q, R). */
template <bool SIGNS, bool VPRED>
__device__ __forceinline__ void rc_cost_body(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ gcli,
                                             const uint16_t* __restrict__ coef, uint32_t* __restrict__ cost,
                                             uint32_t* __restrict__ slice_done, PrecRC* __restrict__ rc,
                                             int* __restrict__ status, const int p) {
    /* per band line: GCLI and significance-maximum histograms (with sign
     * handling also the coefficients by non-zero levels), then per gtli data
     * / GCLI bits without and with significance and the sign bits; the area
     * is reused by the slice selection at the end (with vertical prediction
     * it is dynamic shared memory of RC_VP_REGIONS regions) */
    __shared__ __align__(16) uint32_t s_area_st[VPRED ? 4 : RC_AREA_WORDS(SIGNS)];
    extern __shared__ __align__(16) uint32_t rc_dyn[];
    uint32_t* s_area = VPRED ? rc_dyn : s_area_st;
    uint32_t(*hist)[16] = (uint32_t(*)[16])s_area;                          /* later: fast sign bits per t */
    uint32_t(*shist)[16] = (uint32_t(*)[16])(s_area + JXS_MAXBLINES * 16);  /* groups by significance-group maximum; later: full-sign cost changes */
    uint32_t(*tdat)[16] = (uint32_t(*)[16])(s_area + 2 * JXS_MAXBLINES * 16);
    uint32_t(*tnos)[16] = (uint32_t(*)[16])(s_area + 3 * JXS_MAXBLINES * 16);
    uint32_t(*tsig)[16] = (uint32_t(*)[16])(s_area + 4 * JXS_MAXBLINES * 16);
    uint32_t(*nzh)[16] = (uint32_t(*)[16])(s_area + (SIGNS ? 5 : 0) * JXS_MAXBLINES * 16); /* later: full sign bits per t */
    uint32_t(*tfs)[16] = hist;
    uint32_t(*tnz)[16] = nzh;
    uint32_t(*dF)[32] = (uint32_t(*)[32])shist;
    /* SIGNS: the launch may hold frames with sign handling; VPRED: with
     * vertical prediction (compiled out otherwise) */
    const uint32_t fs = SIGNS ? cfg->fs : 0u, uniform = cfg->qpih;
    __shared__ uint32_t cn[JXS_MAXBL][16], cs[JXS_MAXBL][16];
    __shared__ uint16_t meth[JXS_MAXBL];
    __shared__ uint8_t lgain[JXS_MAXBLINES], lprio[JXS_MAXBLINES], lfb[JXS_MAXBLINES];
    __shared__ uint32_t lsig[JXS_MAXBLINES], lraw[JXS_MAXPK];
    __shared__ uint32_t dC[32][32]; /* per Q: cost at R = 0, then its changes at each R */
    /* this precinct kind's tables, staged from the configuration */
    __shared__ jxs_seg_t s_seg[JXS_MAXSEG];
    __shared__ jxs_bline_t s_bl[JXS_MAXBLINES];
    __shared__ uint64_t s_grow[JXS_MAXBLINES];
    __shared__ uint8_t s_pkbl0[JXS_MAXPK], s_pknbl[JXS_MAXPK], s_order[JXS_MAXBLINES];

    const int last = (p + 1 >= (int)cfg->np);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nbl = cfg->nbline[last], nseg = cfg->nseg[last], SG = cfg->seg_groups;
    const jxs_bline_t* bls = s_bl;
    const jxs_seg_t* segs = s_seg;
    /* the tables of a precinct kind (normal / last row) */
    auto stage_kind = [&](int kind) {
        const uint32_t nb = cfg->nbline[kind], ns = cfg->nseg[kind];
        for (uint32_t i = threadIdx.x; i < ns * (sizeof(jxs_seg_t) / 4); i += blockDim.x)
            ((uint32_t*)s_seg)[i] = ((const uint32_t*)cfg->seg[kind])[i];
        for (uint32_t i = threadIdx.x; i < nb * (sizeof(jxs_bline_t) / 4); i += blockDim.x)
            ((uint32_t*)s_bl)[i] = ((const uint32_t*)cfg->bline[kind])[i];
        for (uint32_t k = threadIdx.x; k < cfg->npk; k += blockDim.x) {
            s_pkbl0[k] = cfg->pk_bl0[kind][k];
            s_pknbl[k] = cfg->pk_nbl[kind][k];
            lraw[k] = cfg->raw_bytes[kind][k];
        }
        for (uint32_t x = threadIdx.x; x < nb; x += blockDim.x) {
            const jxs_bline_t& B = cfg->bline[kind][x];
            const jxs_band_t& bd = cfg->band[B.fb];
            lgain[x] = bd.gain;
            lprio[x] = bd.prio;
            lfb[x] = B.fb;
            lsig[x] = B.sig_w;
            s_order[x] = cfg->pk_order[kind][x];
        }
    };
    stage_kind(last);
    for (uint32_t i = threadIdx.x; i < nbl * 16; i += blockDim.x) {
        hist[i >> 4][i & 15] = 0;
        shist[i >> 4][i & 15] = 0;
        if (SIGNS) nzh[i >> 4][i & 15] = 0;
    }
    for (uint32_t i = threadIdx.x; i < cfg->nbands * 16; i += blockDim.x) {
        cn[i >> 4][i & 15] = 0;
        cs[i >> 4][i & 15] = 0;
    }
    for (uint32_t x = threadIdx.x; x < nbl; x += blockDim.x) {
        const jxs_bline_t& B = cfg->bline[last][x];
        const jxs_band_t& bd = cfg->band[B.fb];
        s_grow[x] = bd.gcli_off + (uint64_t)(p * bd.lines + B.line) * bd.gpitch;
    }
    __syncthreads();

    /* histograms: each lane 4 consecutive groups (one 4-byte load) in 4-bit
     * counters, one per GCLI value (at most 4, or 8 for a significance
     * group's weight), widened to bytes and summed over the warp per 128
     * groups (at most 128 per bin); then lane b < 16 holds the count of
     * GCLI b and lane 16 + b that of significance-group maximum b, adds it
     * to the band line's histogram and, for a segment of at most 128
     * groups, stores it as byte b / 16 + b of the segment's histograms for
     * packing */
    uint32_t* seghist = cost + jxs_seghist_word(cfg) + (uint64_t)p * jxs_seg_cap(cfg) * JXS_SEGHIST_WORDS;
    static_assert(JXS_SEGHIST_WORDS * 4 == 32, "a segment's histograms: one byte per lane");
    const bool export_hist = SG <= 128;
    /* this lane's bin: byte (b >> 1) & 3 of word 2 (b >= 8) + (b & 1) of the
     * value (lanes 0..15) or significance (16..31) words */
    const uint32_t hb = lane & 15u, hsh = 8u * ((hb >> 1) & 3u);
    uint32_t* htab = (lane < 16 ? &hist[0][0] : &shist[0][0]) + hb;
    for (uint32_t sidx = warp; sidx < nseg; sidx += RC_WARPS) {
        const jxs_seg_t sg = segs[sidx];
        const uint32_t x = sg.bl;
        const uint8_t* grow = gcli + s_grow[x];
        const uint32_t gend = min(sg.g0 + SG, bls[x].gcli_w);
        const uint16_t* crow = nullptr;
        if (fs) {
            const jxs_band_t& bd = cfg->band[lfb[x]];
            crow = coef + bd.coef_off + (uint64_t)(p * bd.lines + bls[x].line) * bd.pitch;
        }
        for (uint32_t base = sg.g0; base < gend; base += 128) {
            const uint32_t g = base + 4 * lane;
            const uint32_t nv = g < gend ? min(4u, gend - g) : 0u;
            uint32_t w4 = nv ? *(const uint32_t*)(grow + g) : 0u;
            /* GCLIs past the line's end read as 0 and are taken off bin 0 */
            w4 &= nv >= 4 ? 0xffffffffu : (1u << (8 * nv)) - 1u;
            uint32_t lo = nv - 4u, hi = 0u; /* bin 0 starts at -(4 - nv) */
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint32_t v = (w4 >> (8 * k)) & 15u;
                const uint32_t inc = 1u << (4 * (v & 7u));
                if (v & 8u) hi += inc;
                else lo += inc;
            }
            const uint32_t m2 = __vmaxu4(w4, w4 >> 16), m = max(m2 & 255u, (m2 >> 8) & 255u);
            /* significance group: 8 groups in lanes 2i, 2i+1; its groups
             * (8, or fewer at the end of a line) counted at its maximum */
            const uint32_t mx = max(m, __shfl_xor_sync(FULL, m, 1));
            const uint32_t nvp = nv + __shfl_xor_sync(FULL, nv, 1);
            uint32_t slo = 0u, shi = 0u;
            if (!(lane & 1) && nv) {
                const uint32_t si = nvp << (4 * (mx & 7u));
                if (mx & 8u) shi = si;
                else slo = si;
            }
            /* bytes: even bins, odd bins of 0..7 and of 8..15 */
            const uint32_t M = 0x0f0f0f0fu;
            const uint32_t v0 = __reduce_add_sync(FULL, lo & M), v1 = __reduce_add_sync(FULL, (lo >> 4) & M);
            const uint32_t v2 = __reduce_add_sync(FULL, hi & M), v3 = __reduce_add_sync(FULL, (hi >> 4) & M);
            const uint32_t s0 = __reduce_add_sync(FULL, slo & M), s1 = __reduce_add_sync(FULL, (slo >> 4) & M);
            const uint32_t s2 = __reduce_add_sync(FULL, shi & M), s3 = __reduce_add_sync(FULL, (shi >> 4) & M);
            const uint32_t wv = hb >= 8 ? (hb & 1 ? v3 : v2) : (hb & 1 ? v1 : v0);
            const uint32_t ws = hb >= 8 ? (hb & 1 ? s3 : s2) : (hb & 1 ? s1 : s0);
            const uint32_t c = ((lane < 16 ? wv : ws) >> hsh) & 255u;
            if (c) atomicAdd(htab + 16 * x, c);
            if (export_hist) ((uint8_t*)(seghist + sidx * JXS_SEGHIST_WORDS))[lane] = (uint8_t)c;
            if (fs) {
                /* sign handling: the lane's 16 coefficients (inside the band
                 * width) by the number of gtli values at which they stay
                 * non-zero; 16-bit counters two to a register */
                uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0;
                if (nv) {
                    c0 = *(const uint4*)(crow + 4 * g);
                    c1 = *(const uint4*)(crow + 4 * g + 8);
                }
                const uint32_t cw[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
                const int wleft = (int)bls[x].w - 4 * (int)g;
                uint32_t zc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const uint32_t m = (cw[i >> 1] >> (16 * (i & 1))) & 0x7fffu;
                    const uint32_t v = (w4 >> (8 * (i >> 2))) & 255u;
                    const uint32_t n = i < wleft && (i >> 2) < (int)nv ? nz_levels(m, v, uniform) : 0u;
#pragma unroll
                    for (int r = 0; r < 8; r++) zc[r] += (n >> 1) == (uint32_t)r ? 1u << (16 * (n & 1)) : 0u;
                }
#pragma unroll
                for (int r = 0; r < 8; r++) {
                    const uint32_t zs = __reduce_add_sync(FULL, zc[r]);
                    if (lane < 2) {
                        const uint32_t c = (zs >> (16 * lane)) & 0xffffu;
                        if (c) atomicAdd(&nzh[x][2 * r + lane], c);
                    }
                }
            }
        }
    }
    __syncthreads();

    /* per band line and gtli t: data bits, GCLI bits without / with
     * significance coding */
    for (uint32_t x = threadIdx.x; x < nbl; x += blockDim.x) {
        const uint32_t N = bls[x].gcli_w;
        int S0 = 0, S1 = 0;
        uint32_t Z1 = 0;
        for (int t = 15; t >= 0; t--) {
            const int dsum = S1 - (t - 1) * S0; /* sum over v > t of (v - t + 1) h[v] */
            const uint32_t h = hist[x][t];
            /* with sign handling the data leave out the sign nibbles
             * (RateControl.c:156-210): fast signs count 4 per group above
             * t, full signs the coefficients that stay non-zero */
            tdat[x][t] = 4u * (uint32_t)(dsum - (fs ? S0 : 0));
            tnos[x][t] = (uint32_t)dsum + N - (uint32_t)S0;
            if (SIGNS) {
                tfs[x][t] = 4u * (uint32_t)S0;
                const uint32_t zh = nzh[x][t];
                tnz[x][t] = Z1;
                Z1 += zh;
            }
            S0 += (int)h;
            S1 += t * (int)h;
        }
        uint32_t Z = 0; /* groups in significance groups whose maximum is <= t: no GCLI codes */
        const uint32_t fb = lfb[x];
        for (int t = 0; t < 16; t++) {
            Z += shist[x][t];
            tsig[x][t] = tnos[x][t] - Z;
            atomicAdd(&cn[fb][t], tnos[x][t]);
            atomicAdd(&cs[fb][t], tsig[x][t] + lsig[x]);
        }
    }
    __syncthreads();
    if (VPRED && cfg->vpred) {
        /* the line tables, for the slice's selection in precinct order */
        uint32_t* lt = cost + (uint64_t)cfg->np * 1024 * (cfg->fs ? 2 : 1) + (uint64_t)p * RC_LT_WORDS;
        for (uint32_t i = threadIdx.x; i < nbl * 16; i += blockDim.x) {
            const uint32_t x = i >> 4, t = i & 15;
            lt[i] = tdat[x][t];
            lt[RC_LT_REGION + i] = tnos[x][t];
            lt[2 * RC_LT_REGION + i] = tsig[x][t];
            if (fs) {
                lt[3 * RC_LT_REGION + i] = tfs[x][t];
                lt[4 * RC_LT_REGION + i] = tnz[x][t];
            }
        }
    }
    /* coding method per band and t: significance only if strictly cheaper
     * (RateControl.c:528-575) */
    for (uint32_t fb = threadIdx.x; fb < cfg->nbands; fb += blockDim.x) {
        uint32_t m = 0;
        if (cfg->sig)
            for (int t = 0; t < 16; t++) m |= (cn[fb][t] > cs[fb][t] ? 1u : 0u) << t;
        meth[fb] = (uint16_t)m;
    }
    __syncthreads();

    /* costs: band priorities are distinct, so raising R by one lowers the
     * gtli of one band only; each (Q, packet) thread adds its packet's cost
     * at R = 0 and its change at every R where one of its band lines drops,
     * and the table is a prefix sum over R */
    const int nq = cfg->max_q + 1, nr = cfg->max_r + 1;
    for (int e = threadIdx.x; e < nq * 32; e += blockDim.x) {
        dC[e >> 5][e & 31] = 0;
        if (SIGNS) dF[e >> 5][e & 31] = 0;
    }
    __syncthreads();
    /* with sign handling each packet adds its sign sub-packet, rounded on
     * its own: fast signs in dC, full signs in dF (RateControl.c:745-756) */
    const uint32_t npk = cfg->npk;
    /* a warp per packet, a lane per Q (at most 32): the packet's band lines
     * are the same for the whole warp */
    for (uint32_t k = warp; k < npk; k += RC_WARPS) {
        const int q = lane;
        const uint32_t b0 = s_pkbl0[k], nb = s_pknbl[k];
        if (!nb || q >= nq) continue;
        uint32_t db = 0, gb = 0, sb = 0, fb = 0, zb = 0;
        for (uint32_t x = b0; x < b0 + nb; x++) {
            const int g = lgain[x];
            const int t = q < g ? 0 : min(q - g, 15);
            db += tdat[x][t];
            if ((meth[lfb[x]] >> t) & 1u) {
                gb += tsig[x][t];
                sb += lsig[x];
            } else {
                gb += tnos[x][t];
            }
            if (fs) {
                fb += tfs[x][t];
                zb += tnz[x][t];
            }
        }
        const uint32_t base = ((db + 7) >> 3) + min(lraw[k], ((sb + 7) >> 3) + ((gb + 7) >> 3));
        uint32_t c = base + (fs ? (fb + 7) >> 3 : 0u), cf = base + ((zb + 7) >> 3);
        atomicAdd(&dC[q][0], c);
        if (fs) atomicAdd(&dF[q][0], cf);
        for (uint32_t i = 0; i < nb; i++) {
            const uint32_t x = s_order[b0 + i];
            const int rf = lprio[x] + 1; /* the line's gtli drops by one for R >= priority + 1 */
            if (rf >= nr) break;
            const int g = lgain[x];
            const int t0 = q < g ? 0 : min(q - g, 15), t1 = q < g + 1 ? 0 : min(q - g - 1, 15);
            const uint32_t m0 = (meth[lfb[x]] >> t0) & 1u, m1 = (meth[lfb[x]] >> t1) & 1u;
            db += tdat[x][t1] - tdat[x][t0];
            gb += (m1 ? tsig[x][t1] : tnos[x][t1]) - (m0 ? tsig[x][t0] : tnos[x][t0]);
            sb += (m1 ? lsig[x] : 0u) - (m0 ? lsig[x] : 0u);
            const uint32_t base1 = ((db + 7) >> 3) + min(lraw[k], ((sb + 7) >> 3) + ((gb + 7) >> 3));
            uint32_t c1 = base1;
            if (fs) {
                fb += tfs[x][t1] - tfs[x][t0];
                zb += tnz[x][t1] - tnz[x][t0];
                c1 += (fb + 7) >> 3;
                const uint32_t cf1 = base1 + ((zb + 7) >> 3);
                atomicAdd(&dF[q][rf], cf1 - cf);
                cf = cf1;
            }
            atomicAdd(&dC[q][rf], c1 - c);
            c = c1;
        }
    }
    __syncthreads();
    uint32_t* out = cost + (uint64_t)p * 32 * 32;
    uint32_t* outf = cost + ((uint64_t)cfg->np + p) * 32 * 32;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        uint32_t run = 0, runf = 0;
        for (int r = 0; r < nr; r++) {
            run += dC[q][r];
            out[q * 32 + r] = run;
            if (fs) {
                runf += dF[q][r];
                outf[q * 32 + r] = runf;
            }
        }
    }
    /* the block that completes a slice runs the slice's selection: tables
     * published with a fence, blocks counted per slice */
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    const uint32_t s = (uint32_t)p / cfg->pps;
    const uint32_t first_p = cfg->pps * s;
    const uint32_t nprec = (s + 1 == cfg->nslices) ? cfg->np - first_p : cfg->pps;
    if (threadIdx.x == 0) s_last = atomicAdd(&slice_done[s], 1u) + 1 == nprec;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if constexpr (VPRED) {
        if (cfg->vpred) select_slice_vpred(cfg, (int)s, gcli, cost, s_area, rc, status, stage_kind, lgain, lprio, lfb, lsig,
                                           lraw, s_bl, s_seg, s_pkbl0, s_pknbl, s_order);
        else select_slice(cfg, (int)s, cost, s_area, RC_VP_REGIONS * RC_LT_REGION, rc, status);
    } else {
        select_slice(cfg, (int)s, cost, s_area, RC_AREA_WORDS(SIGNS), rc, status);
    }
    if (threadIdx.x == 0) slice_done[s] = 0; /* ready for the next frame */
}

/* ------------------------------------------------------------------------ */
/* Packing                                                                   */
/* ------------------------------------------------------------------------ */
#define PK_THREADS 512
#define PK_WARPS (PK_THREADS / 32)

/* Next entry of a block's shared work queue for a warp. */
__device__ __forceinline__ uint32_t queue_next(uint32_t* ctr, int lane) {
    uint32_t v = 0;
    if (lane == 0) v = atomicAdd(ctr, 1u);
    return __shfl_sync(0xffffffffu, v, 0);
}

/* OR the low `n` bits (1..64) of `v` into a big-endian bit string stored in
 * native byte order (byte i of the string is byte i of the buffer), at bit
 * `pos`.  Bits past the buffer's `nw` words are not written and set `ovf`
 * (the sizes would disagree with the rate control). */
DEV void put_bits(uint32_t* buf, uint32_t nw, uint32_t pos, uint64_t v, uint32_t n, int& ovf) {
    if (((pos + n - 1) >> 5) >= nw) {
        ovf = 1;
        return;
    }
    const uint64_t a = v << (64 - n); /* left-aligned */
    const uint32_t hi = (uint32_t)(a >> 32), lo = (uint32_t)a;
    const uint32_t w = pos >> 5, sh = pos & 31;
    atomicOr(&buf[w], __byte_perm(hi >> sh, 0, 0x0123));
    if (sh + n > 32) atomicOr(&buf[w + 1], __byte_perm(__funnelshift_r(lo, hi, sh), 0, 0x0123));
    if (sh + n > 64) atomicOr(&buf[w + 2], __byte_perm(lo << (32 - sh), 0, 0x0123));
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

/* Inverse of the 8 x 4 bit-matrix transpose: byte 3 - c holds the 8 plane
 * bits of coefficient c; bit k of it moves to bit 4k + 3 - c (nibble k =
 * plane k, coefficient 0 in its most significant bit).  Masked delta swaps
 * of index bits (1,0), (2,1), (3,0), (4,1). */
DEV uint32_t dswap(uint32_t x, int d, uint32_t m) {
    const uint32_t t = ((x >> d) ^ x) & m;
    return x ^ t ^ (t << d);
}
DEV uint32_t coefs_to_planes(uint32_t x) {
    x = dswap(x, 1, 0x22222222u);
    x = dswap(x, 2, 0x0c0c0c0cu);
    x = dswap(x, 7, 0x00aa00aau);
    return dswap(x, 14, 0x0000ccccu);
}

/* Data bits of one 4-coefficient group with GCLI v > gtli t
 * (pack_data_c, PackPrecinct.c:128-198): bit-planes v-1 .. t, each a
 * nibble (coefficient 0 in the most significant bit).  Quantization
 * (Quant.c:9-45) is skipped for t == 0 like the reference
 * (QuantStageProcess.c:18-31).  `signs` receives the sign nibble, which has
 * a bit only for a non-zero quantized magnitude, and `nzm` the non-zero
 * magnitudes, both with coefficient 0 in bit 3.  Without sign handling the
 * sign nibble leads the group's data; with it the signs of the non-zero
 * magnitudes go to the packet's sign sub-packet (pack_sign_c, :200-233). */
DEV uint64_t data_chunk(uint2 raw4, int wleft, uint32_t v, uint32_t t, uint32_t uniform, uint32_t& signs, uint32_t& nzm) {
    /* coefficients past the band width are zero */
    uint32_t c01 = raw4.x & ((wleft > 1 ? 0xffff0000u : 0u) | 0xffffu);
    uint32_t c23 = raw4.y & ((wleft > 2 ? 0xffffu : 0u) | (wleft > 3 ? 0xffff0000u : 0u));
    uint32_t P01, P23;
    if (t == 0) {
        P01 = c01 & 0x7fff7fffu;
        P23 = c23 & 0x7fff7fffu;
    } else if (!uniform) {
        /* deadzone: magnitude >> t, two coefficients per word */
        const uint32_t keep = (0x7fffu >> t) * 0x00010001u;
        P01 = ((c01 & 0x7fff7fffu) >> t) & keep;
        P23 = ((c23 & 0x7fff7fffu) >> t) & keep;
    } else {
        uint32_t q[4];
        const uint32_t c[4] = {c01 & 0xffffu, c01 >> 16, c23 & 0xffffu, c23 >> 16};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t m = c[k] & 0x7fffu;
            /* computed in int like the reference, truncated to 16 bits */
            const uint32_t u = (((m << (v - t + 1)) - m + (1u << v)) >> (v + 1)) & 0xffffu;
            q[k] = ((u << t) & 0xffffu) >> t;
        }
        P01 = q[0] | (q[1] << 16);
        P23 = q[2] | (q[3] << 16);
    }
    const uint32_t n01 = __vcmpne2(P01, 0u), n23 = __vcmpne2(P23, 0u);
    nzm = ((n01 << 3) & 8u) | ((n01 >> 14) & 4u) | ((n23 << 1) & 2u) | (n23 >> 31);
    const uint32_t s01 = n01 & c01 & 0x80008000u, s23 = n23 & c23 & 0x80008000u;
    signs = ((s01 >> 12) & 8u) | ((s01 >> 29) & 4u) | ((s23 >> 14) & 2u) | (s23 >> 31);
    /* byte 3 - c of the word = low 8 plane bits of coefficient c */
    uint64_t planes = coefs_to_planes(__byte_perm(P01, P23, 0x0246));
    if (v - t > 8) planes |= (uint64_t)coefs_to_planes(__byte_perm(P01, P23, 0x1357)) << 32;
    return planes;
}

/* The same with the sign nibble leading the planes (signs with the data),
 * for a group whose coefficients past the band width are stored as zero:
 * the sign of every coefficient that stays non-zero enters as plane
 * v - t of its magnitude, and one transpose gives sign and planes. */
DEV uint64_t data_chunk_signed(uint2 raw4, uint32_t v, uint32_t t, uint32_t uniform) {
    const uint32_t c01 = raw4.x, c23 = raw4.y, np = v - t;
    uint32_t P01, P23;
    if (t == 0) {
        P01 = c01 & 0x7fff7fffu;
        P23 = c23 & 0x7fff7fffu;
    } else if (!uniform) {
        const uint32_t keep = (0x7fffu >> t) * 0x00010001u;
        P01 = ((c01 & 0x7fff7fffu) >> t) & keep;
        P23 = ((c23 & 0x7fff7fffu) >> t) & keep;
    } else {
        uint32_t q[4];
        const uint32_t c[4] = {c01 & 0xffffu, c01 >> 16, c23 & 0xffffu, c23 >> 16};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t m = c[k] & 0x7fffu;
            const uint32_t u = (((m << (v - t + 1)) - m + (1u << v)) >> (v + 1)) & 0xffffu;
            q[k] = ((u << t) & 0xffffu) >> t;
        }
        P01 = q[0] | (q[1] << 16);
        P23 = q[2] | (q[3] << 16);
    }
    /* sign bits (bits 15 and 31) of the non-zero magnitudes moved to bit np
     * of each half (np <= 15) */
    P01 |= (__vcmpne2(P01, 0u) & c01 & 0x80008000u) >> (15 - np);
    P23 |= (__vcmpne2(P23, 0u) & c23 & 0x80008000u) >> (15 - np);
    uint64_t planes = coefs_to_planes(__byte_perm(P01, P23, 0x0246));
    if (np >= 8) planes |= (uint64_t)coefs_to_planes(__byte_perm(P01, P23, 0x1357)) << 32;
    return planes;
}

/* Per band line of the precinct being packed. */
struct PkLine {
    uint32_t sig_pos, gcli_pos, data_pos, sign_pos; /* bit positions in the shared-memory precinct */
    uint32_t data, vlc, zero, nz; /* data bits, VLC bits without significance, groups in insignificant significance
                                     groups, signs sent in the sign sub-packet */
    uint8_t meth, raw, pad0, pad1;
};

/* pack_precinct (PackPrecinct.c:235-572) for one precinct row.
 *
 * The precinct is assembled in shared memory, `lead` bytes into the buffer
 * so that buffer byte i lands on the 16-byte aligned address
 * out + offset - lead + i, then copied out.  Band lines are split into
 * segments of seg_groups groups, one warp per segment:
 *   pass A  each segment's data bits, VLC bits and groups lying in
 *           insignificant significance groups, at the precinct's gtli: from
 *           the segment's histograms that the rate control stored (thread
 *           per segment), or, with sign handling, vertical prediction or
 *           segments of more than 128 groups, from the GCLIs (warp per
 *           segment);
 *   layout  warp 0, lanes over band lines, bands, packets: coding method per
 *           band (significance only if strictly cheaper), packet headers, raw
 *           fallback, packet positions by a warp scan, sub-packet positions,
 *           each segment's start in its GCLI and data sub-packets;
 *   pass B  each lane 4 groups: significance flags and the unary GCLI
 *           codes at positions from a warp prefix sum; the groups above
 *           gtli listed per warp, each lane then packing one listed group's
 *           data bits; everything OR-ed into the buffer.
 * VPRED (frames with vertical prediction; compiled out otherwise): a
 * precinct row below another of its slice also sums, per segment, the
 * codes of its GCLIs predicted from the line above at its gtli (line 0:
 * from the row above, with that row's gtli) and the groups that need no
 * code; the layout chooses among the four codings per band like the rate
 * control (RateControl.c:526-676), and pass B writes the prediction codes
 * (pack_bitplane_count_vpred_*, PackPrecinct.c:47-74). */
template <bool VPRED>
__device__ __forceinline__ void pack_body(const jxs_cfg_t* __restrict__ cfg, const uint16_t* __restrict__ coef,
                                          const uint8_t* __restrict__ gcli, const PrecRC* __restrict__ rc,
                                          const uint32_t* __restrict__ cost, uint8_t* __restrict__ out, uint32_t cap_words,
                                          int* status, const int p) {
    extern __shared__ __align__(16) uint32_t buf[];
    /* per segment: data bits, VLC bits, groups without codes, signs; in pass
     * B the same words hold each warp's list of significant groups */
    __shared__ uint32_t s_segw[4][JXS_MAXSEG];
    uint32_t* s_data = s_segw[0];
    uint32_t* s_vlc = s_segw[1];
    uint32_t* s_zero = s_segw[2];
    uint32_t* s_nz = s_segw[3];
    static_assert(4 * JXS_MAXSEG >= 128 * PK_WARPS, "a list of 128 groups per warp");
    __shared__ PkLine pl[JXS_MAXBLINES];
    __shared__ uint8_t s_meth[JXS_MAXBL];
    __shared__ uint32_t s_cn[JXS_MAXBL], s_cs[JXS_MAXBL];
    __shared__ uint32_t s_vn[VPRED ? JXS_MAXSEG : 1], s_vr[VPRED ? JXS_MAXSEG : 1]; /* per segment: prediction bits */
    __shared__ uint32_t s_cv[VPRED ? JXS_MAXBL : 1], s_cvs[VPRED ? JXS_MAXBL : 1];   /* per band: prediction totals */
    __shared__ int8_t s_gtt[VPRED ? JXS_MAXBLINES : 1];                            /* per line: gtli of the line above (-1: this row's) */
    __shared__ uint32_t s_lvn[VPRED ? JXS_MAXBLINES : 1], s_lvr[VPRED ? JXS_MAXBLINES : 1]; /* per line: prediction bits */
    __shared__ uint32_t s_gp[VPRED ? JXS_MAXBLINES : 1];                           /* per line: GCLI row pitch */
    __shared__ uint32_t s_lg[JXS_MAXBLINES], s_ls[JXS_MAXBLINES];       /* per line: GCLI / significance bits */
    __shared__ uint32_t s_pks[JXS_MAXPK], s_pkg[JXS_MAXPK], s_pkd[JXS_MAXPK], s_pkn[JXS_MAXPK]; /* per packet: sub-packet starts */
    __shared__ uint8_t s_pkr[JXS_MAXPK];
    __shared__ uint32_t s_vst[JXS_MAXSEG], s_dst[JXS_MAXSEG], s_nst[JXS_MAXSEG]; /* per segment: GCLI / data / sign bit starts */
    /* this precinct kind's tables, staged from the configuration */
    __shared__ jxs_seg_t s_seg[JXS_MAXSEG];
    __shared__ uint16_t s_ord[JXS_MAXSEG];                              /* work order of the segments */
    __shared__ uint32_t s_q[2];                                         /* work queues of passes A and B */
    __shared__ jxs_bline_t s_bl[JXS_MAXBLINES];
    __shared__ uint64_t s_grow[JXS_MAXBLINES], s_crow[JXS_MAXBLINES]; /* per line: GCLI / coefficient row offsets */
    __shared__ uint8_t s_lt[JXS_MAXBLINES];                            /* per line: gtli */
    __shared__ uint8_t s_pkbl0[JXS_MAXPK], s_pknbl[JXS_MAXPK];
    __shared__ uint32_t s_praw[JXS_MAXPK];
    __shared__ uint8_t s_g2f[JXS_MAXBL];                               /* global band -> flat band */
    __shared__ uint8_t s_blines[JXS_MAXBL];                            /* lines of each band in this precinct kind */
    /* configuration scalars of the layout, loaded with the tables so that the
     * single-warp layout waits on no device-memory read */
    __shared__ uint32_t s_nbands, s_nbands_all, s_npk, s_sig, s_short, s_phb, s_hdrs, s_nbl;
    __shared__ int s_ok;

    const int last = (p + 1 >= (int)cfg->np);
    const PrecRC R = rc[p];
    /* nothing to pack once the rate control failed somewhere in the frame;
     * the flag is read once so that the whole block takes the same branch */
    if (threadIdx.x == 0) s_ok = *(volatile int*)status == 0;
    __syncthreads();
    if (!s_ok) return;
    const uint32_t total = R.total_bytes;
    const uint32_t lead = (uint32_t)((uintptr_t)(out + R.offset) & 15);
    const uint32_t words = ((lead + total + 15) >> 4) << 2;
    if (words > cap_words) {
        if (threadIdx.x == 0) {
            printf("jxs pack: precinct %d needs %u words, buffer holds %u\n", p, words, cap_words);
            JXS_STATUS_SET(status, JXS_E_ENC_FRAME);
        }
        return;
    }
    int ovf = 0;
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) buf[i] = 0;
    for (uint32_t fb = threadIdx.x; fb < cfg->nbands; fb += blockDim.x) {
        s_cn[fb] = 0;
        s_cs[fb] = 0;
        if (VPRED) {
            s_cv[fb] = 0;
            s_cvs[fb] = 0;
        }
    }
    /* vertical prediction applies below the first row of a slice */
    const int vp = VPRED && cfg->vpred && !R.first_in_slice;
    const int rmode = cfg->rm;
    {
        const uint32_t ns = cfg->nseg[last], nl = cfg->nbline[last];
        for (uint32_t i = threadIdx.x; i < ns * (sizeof(jxs_seg_t) / 4); i += blockDim.x)
            ((uint32_t*)s_seg)[i] = ((const uint32_t*)cfg->seg[last])[i];
        for (uint32_t i = threadIdx.x; i < nl * (sizeof(jxs_bline_t) / 4); i += blockDim.x)
            ((uint32_t*)s_bl)[i] = ((const uint32_t*)cfg->bline[last])[i];
        for (uint32_t i = threadIdx.x; i < ns; i += blockDim.x) s_ord[i] = cfg->seg_ord[last][i];
        if (threadIdx.x < 2) s_q[threadIdx.x] = 0;
        for (uint32_t x = threadIdx.x; x < nl; x += blockDim.x) {
            const jxs_bline_t& B = cfg->bline[last][x];
            const jxs_band_t& bd = cfg->band[B.fb];
            const uint64_t row = (uint64_t)(p * bd.lines + B.line);
            s_grow[x] = bd.gcli_off + row * bd.gpitch;
            s_crow[x] = bd.coef_off + row * bd.pitch;
            s_lt[x] = jxs_truncation(bd.gain, bd.prio, R.q, R.r);
            if (VPRED) {
                s_gp[x] = bd.gpitch;
                s_gtt[x] = (int8_t)(vp && B.line == 0 ? jxs_truncation(bd.gain, bd.prio, rc[p - 1].q, rc[p - 1].r) : -1);
            }
        }
        for (uint32_t k = threadIdx.x; k < cfg->npk; k += blockDim.x) {
            s_pkbl0[k] = cfg->pk_bl0[last][k];
            s_pknbl[k] = cfg->pk_nbl[last][k];
            s_praw[k] = cfg->raw_bytes[last][k];
        }
        for (uint32_t gb = threadIdx.x; gb < cfg->nbands_all; gb += blockDim.x) s_g2f[gb] = cfg->g2f[gb];
        for (uint32_t fb = threadIdx.x; fb < cfg->nbands; fb += blockDim.x)
            s_blines[fb] = (uint8_t)(last ? cfg->band[fb].last_lines : cfg->band[fb].lines);
    }
    if (threadIdx.x == 0) {
        s_nbands = cfg->nbands;
        s_nbands_all = cfg->nbands_all;
        s_npk = cfg->npk;
        s_sig = cfg->sig;
        s_short = cfg->short_hdr;
        s_phb = cfg->prec_hdr_bytes;
        s_hdrs = cfg->hdrs_bytes[last];
        s_nbl = cfg->nbline[last];
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nseg = cfg->nseg[last], SG = cfg->seg_groups;
    const jxs_seg_t* segs = s_seg;
    const jxs_bline_t* bls = s_bl;

    /* pass A: each lane 4 consecutive groups (one 4-byte GCLI load), a warp
     * 128 groups per step; with sign handling also the non-zero quantized
     * coefficients, whose signs go to the sign sub-packets */
    const uint32_t fs = cfg->fs, uniform = cfg->qpih;
    if (!VPRED && !fs && SG <= 128) {
        /* from the rate control's histograms: data bits 4 (v - t + 1) and
         * codes of v - t + 1 bits for groups with GCLI v > t, 1-bit codes
         * for the others; no codes for the groups of significance groups
         * whose maximum is <= t */
        const uint32_t* hist = cost + jxs_seghist_word(cfg) + (uint64_t)p * jxs_seg_cap(cfg) * JXS_SEGHIST_WORDS;
        for (uint32_t i = threadIdx.x; i < nseg; i += blockDim.x) {
            const uint4 gh = __ldcg((const uint4*)(hist + i * JXS_SEGHIST_WORDS));
            const uint4 zh = __ldcg((const uint4*)(hist + i * JXS_SEGHIST_WORDS + 4));
            const uint32_t t = s_lt[segs[i].bl];
            const uint32_t gw[4] = {gh.x, gh.y, gh.z, gh.w}, zw[4] = {zh.x, zh.y, zh.z, zh.w};
            uint32_t d = 0, v = 0, z = 0;
#pragma unroll
            for (uint32_t b = 0; b < 16; b++) {
                const uint32_t c = (gw[b >> 2] >> (8 * (b & 3))) & 255u, cz = (zw[b >> 2] >> (8 * (b & 3))) & 255u;
                if (b > t) {
                    d += (b - t + 1) * c;
                    v += (b - t + 1) * c;
                } else {
                    v += c;
                    z += cz;
                }
            }
            s_data[i] = 4 * d;
            s_vlc[i] = v;
            s_zero[i] = z;
            s_nz[i] = 0;
        }
    } else
    for (uint32_t qi = queue_next(&s_q[0], lane); qi < nseg; qi = queue_next(&s_q[0], lane)) {
        const uint32_t sidx = s_ord[qi];
        const jxs_seg_t sg = segs[sidx];
        const uint32_t t = s_lt[sg.bl];
        const uint8_t* grow = gcli + s_grow[sg.bl];
        const uint16_t* crow = coef + s_crow[sg.bl];
        const int bw = (int)bls[sg.bl].w;
        const uint32_t gend = min(sg.g0 + SG, bls[sg.bl].gcli_w);
        uint32_t dsum = 0, vsum = 0, zsum = 0, nsum = 0, pnsum = 0, prsum = 0;
        for (uint32_t base = sg.g0; base < gend; base += 128) {
            const uint32_t g = base + 4 * lane;
            const uint32_t nv = g < gend ? min(4u, gend - g) : 0u;
            const uint32_t w4 = nv ? *(const uint32_t*)(grow + g) : 0u;
            if (VPRED && vp) {
                /* GCLIs predicted from the line above: code bits, and the
                 * groups of 8 that need none (lanes 2j, 2j + 1) */
                const uint32_t wt = nv ? *(const uint32_t*)(grow - s_gp[sg.bl] + g) : 0u;
                const int gmax = max((int)t, (int)s_gtt[sg.bl]);
                uint32_t sum = 0, flag = 1;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (k < (int)nv) {
                        const int c = (int)((w4 >> (8 * k)) & 255u), tp = (int)((wt >> (8 * k)) & 255u);
                        const int mt = max(tp, gmax), gv = max(c, (int)t);
                        sum += vlc_vp_bits(gv - mt, mt, (int)t) + 1;
                        flag &= rmode ? (uint32_t)(c <= (int)t) : (uint32_t)(mt == gv);
                    }
                }
                const uint32_t f2 = flag & __shfl_xor_sync(FULL, flag, 1), s2 = sum + __shfl_xor_sync(FULL, sum, 1);
                pnsum += sum;
                prsum += (!(lane & 1) && f2) ? s2 : 0u;
            }
            uint32_t m = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) m = max(m, k < (int)nv ? (w4 >> (8 * k)) & 255u : 0u);
            const uint32_t mx = max(m, __shfl_xor_sync(FULL, m, 1)); /* significance group: 2 lanes */
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (k < (int)nv) {
                    const uint32_t v = (w4 >> (8 * k)) & 255u;
                    dsum += v > t ? 4 * (v - t + 1 - fs) : 0u;
                    vsum += v > t ? v - t + 1 : 1u;
                    zsum += mx <= t;
                }
            }
            if (fs && m > t) {
                const uint4 c0 = *(const uint4*)(crow + 4 * g), c1 = *(const uint4*)(crow + 4 * g + 8);
                const uint2 cw[4] = {make_uint2(c0.x, c0.y), make_uint2(c0.z, c0.w), make_uint2(c1.x, c1.y), make_uint2(c1.z, c1.w)};
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const uint32_t v = (w4 >> (8 * k)) & 255u;
                    if (k < (int)nv && v > t) {
                        uint32_t sgn, nzm;
                        (void)data_chunk(cw[k], bw - 4 * (int)(g + k), v, t, uniform, sgn, nzm);
                        nsum += __popc(nzm);
                    }
                }
            }
        }
        dsum = __reduce_add_sync(FULL, dsum);
        vsum = __reduce_add_sync(FULL, vsum);
        zsum = __reduce_add_sync(FULL, zsum);
        nsum = __reduce_add_sync(FULL, nsum);
        if (VPRED) {
            pnsum = __reduce_add_sync(FULL, pnsum);
            prsum = __reduce_add_sync(FULL, prsum);
        }
        if (lane == 0) {
            s_data[sidx] = dsum;
            s_vlc[sidx] = vsum;
            s_zero[sidx] = zsum;
            s_nz[sidx] = nsum;
            if (VPRED) {
                s_vn[sidx] = pnsum;
                s_vr[sidx] = prsum;
            }
        }
    }
    __syncthreads();

    /* layout, by warp 0: lanes over band lines, bands, packets, segments */
    if (warp == 0) {
        const uint32_t nbl = s_nbl;
        for (uint32_t b = lane; b < nbl; b += 32) {
            const jxs_bline_t& B = bls[b];
            uint32_t d = 0, v = 0, z = 0, n = 0;
            for (uint32_t i = B.seg0; i < B.seg0 + B.nseg; i++) {
                d += s_data[i];
                v += s_vlc[i];
                z += s_zero[i];
                n += s_nz[i];
            }
            pl[b].data = d;
            pl[b].vlc = v;
            pl[b].zero = z;
            pl[b].nz = n;
            atomicAdd(&s_cn[B.fb], v);
            atomicAdd(&s_cs[B.fb], v - z + B.sig_w);
            if (VPRED && vp) {
                uint32_t vn = 0, vr = 0;
                for (uint32_t i = B.seg0; i < B.seg0 + B.nseg; i++) {
                    vn += s_vn[i];
                    vr += s_vr[i];
                }
                s_lvn[b] = vn;
                s_lvr[b] = vr;
                atomicAdd(&s_cv[B.fb], vn);
                atomicAdd(&s_cvs[B.fb], vn - vr + B.sig_w);
            }
        }
        __syncwarp();
        /* coding method per band, D[p,b] (bit 1 significance, bit 0
         * prediction): a later one only if strictly cheaper
         * (RateControl.c:526-676) */
        for (uint32_t fb = lane; fb < s_nbands; fb += 32) {
            uint32_t m = 0, best = s_cn[fb];
            if (s_sig && best > s_cs[fb]) {
                m = 2;
                best = s_cs[fb];
            }
            if (VPRED && vp) {
                if (best > s_cv[fb]) {
                    m = 1;
                    best = s_cv[fb];
                }
                if (s_sig && best > s_cvs[fb]) m = 3;
            }
            s_meth[fb] = (uint8_t)m;
        }
        __syncwarp();
        /* per line: GCLI and significance bits with the band's method */
        for (uint32_t b = lane; b < nbl; b += 32) {
            const uint8_t m = s_meth[bls[b].fb];
            pl[b].meth = m;
            s_lg[b] = m == 0 ? pl[b].vlc : m == 2 ? pl[b].vlc - pl[b].zero : m == 1 ? s_lvn[VPRED ? b : 0] : s_lvn[VPRED ? b : 0] - s_lvr[VPRED ? b : 0];
            s_ls[b] = (m & 2) ? bls[b].sig_w : 0u;
        }
        __syncwarp();
        /* one lane per packet: sub-packet sizes, raw fallback, header */
        const uint32_t k = lane;
        const uint32_t nb = k < s_npk ? s_pknbl[k] : 0u, b0 = k < s_npk ? s_pkbl0[k] : 0u;
        uint32_t db = 0, gbits = 0, sbits = 0, nbits = 0;
        for (uint32_t x = b0; x < b0 + nb; x++) {
            db += pl[x].data;
            gbits += s_lg[x];
            sbits += s_ls[x];
            nbits += pl[x].nz;
        }
        const uint32_t dB = (db + 7) >> 3, gB = (gbits + 7) >> 3, sB = (sbits + 7) >> 3, nB = (nbits + 7) >> 3;
        const uint32_t rawB = nb ? s_praw[k] : 0u;
        const int raw = nb && sB + gB > rawB;
        const uint32_t gcl_bytes = raw ? rawB : gB;
        const uint32_t hb = nb ? (s_short ? 5u : 7u) : 0u;
        const uint32_t pk_bytes = nb ? hb + (raw ? rawB : sB + gB) + dB + nB : 0u;
        uint32_t pk_total;
        const uint32_t hdr = s_phb;
        const uint32_t start = lead + hdr + warp_excl_scan(pk_bytes, &pk_total);
        const int fits = start + hb <= words * 4;
        if (nb && fits) {
            /* packet header (PackHeaders.c:98-127) */
            uint8_t* h = (uint8_t*)buf + start;
            if (s_short) {
                h[0] = (uint8_t)((raw << 7) | ((dB >> 8) & 0x7f));
                h[1] = (uint8_t)dB;
                h[2] = (uint8_t)(gcl_bytes >> 5);
                h[3] = (uint8_t)(((gcl_bytes & 0x1f) << 3) | ((nB >> 8) & 7));
                h[4] = (uint8_t)nB;
            } else {
                h[0] = (uint8_t)((raw << 7) | ((dB >> 13) & 0x7f));
                h[1] = (uint8_t)(dB >> 5);
                h[2] = (uint8_t)(((dB & 0x1f) << 3) | ((gcl_bytes >> 17) & 7));
                h[3] = (uint8_t)(gcl_bytes >> 9);
                h[4] = (uint8_t)(gcl_bytes >> 1);
                h[5] = (uint8_t)(((gcl_bytes & 1) << 7) | ((nB >> 8) & 0x7f));
                h[6] = (uint8_t)nB;
            }
            /* sub-packet starts: significance, GCLIs, data, signs */
            const uint32_t p0 = (start + hb) * 8;
            s_pks[k] = p0;
            s_pkg[k] = raw ? p0 : p0 + sB * 8;
            s_pkd[k] = p0 + (raw ? rawB : sB + gB) * 8;
            s_pkn[k] = s_pkd[k] + dB * 8;
            s_pkr[k] = (uint8_t)raw;
        }
        __syncwarp();
        /* per line: positions inside its packet's sub-packets */
        for (uint32_t x = lane; x < nbl; x += 32) {
            const uint32_t kk = bls[x].pk, xb0 = s_pkbl0[kk];
            uint32_t sp = 0, gp = 0, dp = 0, np = 0;
            const int r = s_pkr[kk];
            for (uint32_t y = xb0; y < x; y++) {
                sp += s_ls[y];
                gp += r ? 4 * bls[y].gcli_w : s_lg[y];
                dp += pl[y].data;
                np += pl[y].nz;
            }
            pl[x].raw = (uint8_t)r;
            pl[x].sig_pos = s_pks[kk] + sp;
            pl[x].gcli_pos = s_pkg[kk] + gp;
            pl[x].data_pos = s_pkd[kk] + dp;
            pl[x].sign_pos = s_pkn[kk] + np;
        }
        __syncwarp();
        /* per segment: its start in its line's GCLI and data bits */
        for (uint32_t i = lane; i < nseg; i += 32) {
            const uint32_t x = segs[i].bl;
            const uint8_t m = pl[x].meth;
            uint32_t vp = pl[x].gcli_pos, dp = pl[x].data_pos, np = pl[x].sign_pos;
            for (uint32_t j = bls[x].seg0; j < i; j++) {
                vp += m == 0 ? s_vlc[j] : m == 2 ? s_vlc[j] - s_zero[j] : m == 1 ? s_vn[VPRED ? j : 0] : s_vn[VPRED ? j : 0] - s_vr[VPRED ? j : 0];
                dp += s_data[j];
                np += s_nz[j];
            }
            s_vst[i] = vp;
            s_dst[i] = dp;
            s_nst[i] = np;
        }
        /* precinct header: Lprc, Q, R as bytes first, then the 2-bit band
         * coding modes D[p,b] of every existing band */
        if (lane == 0) {
            uint8_t* bytes = (uint8_t*)buf + lead;
            const uint32_t lprc = total - hdr;
            bytes[0] = (uint8_t)(lprc >> 16);
            bytes[1] = (uint8_t)(lprc >> 8);
            bytes[2] = (uint8_t)lprc;
            bytes[3] = R.q;
            bytes[4] = R.r;
        }
        __syncwarp();
        uint32_t idx0 = 0;
        for (uint32_t gb0 = 0; gb0 < s_nbands_all; gb0 += 32) {
            const uint32_t gb = gb0 + lane;
            const int fb = gb < s_nbands_all ? s_g2f[gb] : JXS_NOBAND;
            const bool ex = fb != JXS_NOBAND;
            const uint32_t bal = __ballot_sync(FULL, ex);
            if (ex && s_blines[fb] > 0 && s_meth[fb])
                put_bits(buf, words, lead * 8 + 40 + 2 * (idx0 + __popc(bal & ((1u << lane) - 1))), s_meth[fb], 2, ovf);
            idx0 += __popc(bal);
        }
        /* the packed size must be what the rate control paid for */
        const int all_fit = __all_sync(FULL, fits || !nb);
        if (lane == 0) {
            const uint32_t end = hdr + pk_total;
            s_ok = all_fit && end <= total && end == s_hdrs + R.data_bytes;
            if (!s_ok) {
                printf("jxs pack: precinct %d packs to %u bytes, rate control paid %u + %u bytes (total %u)\n", p, end,
                       s_hdrs, R.data_bytes, total);
                JXS_STATUS_SET(status, JXS_E_ENC_FRAME);
            }
        }
    }
    __syncthreads();
    if (!s_ok) return;

    /* pass B: each lane 4 consecutive groups; its unary codes are joined
     * into one write, its data chunks into writes of up to 64 bits, its
     * signs (with sign handling) into one write */
    for (uint32_t qi = queue_next(&s_q[1], lane); qi < nseg; qi = queue_next(&s_q[1], lane)) {
        const uint32_t sidx = s_ord[qi];
        const jxs_seg_t sg = segs[sidx];
        const jxs_bline_t B = bls[sg.bl];
        const PkLine L = pl[sg.bl];
        const uint32_t t = s_lt[sg.bl];
        const uint8_t* grow = gcli + s_grow[sg.bl];
        const uint16_t* crow = coef + s_crow[sg.bl];
        const uint32_t gend = min(sg.g0 + SG, B.gcli_w);
        uint32_t vpos = s_vst[sidx], dpos = s_dst[sidx], npos = s_nst[sidx];
        for (uint32_t base = sg.g0; base < gend; base += 128) {
            const uint32_t g = base + 4 * lane;
            const uint32_t nv = g < gend ? min(4u, gend - g) : 0u;
            /* the lane's GCLIs, one per byte (0 past the line's end) */
            uint32_t w4 = nv ? *(const uint32_t*)(grow + g) : 0u;
            w4 &= nv >= 4 ? 0xffffffffu : (1u << (8 * nv)) - 1u;
            uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0;
            if (nv && fs) {
                c0 = *(const uint4*)(crow + 4 * g);
                c1 = *(const uint4*)(crow + 4 * g + 8);
            }
            /* per byte: planes above gtli d = max(v - t, 0), and v > t */
            const uint32_t t4 = t * 0x01010101u;
            const uint32_t d4 = __vsubus4(w4, t4), s4 = __vcmpgtu4(w4, t4);
            const uint32_t dsum = __vsadu4(d4, 0u), nsig = __popc(s4 & 0x01010101u);
            uint32_t v[4];
#pragma unroll
            for (int k = 0; k < 4; k++) v[k] = (w4 >> (8 * k)) & 255u;
            const uint32_t m2 = __vmaxu4(w4, w4 >> 16), m = max(m2 & 255u, (m2 >> 8) & 255u);
            const uint32_t mx = max(m, __shfl_xor_sync(FULL, m, 1));
            /* a significance group without codes: all GCLIs <= gtli, or with
             * prediction the group's flag */
            bool insig = mx <= t;
            uint32_t n4[4] = {0, 0, 0, 0}; /* prediction: each GCLI's code length */
            uint64_t vacc = 0;             /* otherwise: the lane's codes joined */
            uint32_t vl = 0;
            if (VPRED && (L.meth & 1) && !L.raw) {
                /* codes predicted from the line above (vlc_encode,
                 * PackPrecinct.h:41-65) */
                const uint32_t wt = nv ? *(const uint32_t*)(grow - s_gp[VPRED ? sg.bl : 0] + g) : 0u;
                const int gmax = max((int)t, (int)s_gtt[VPRED ? sg.bl : 0]);
                uint32_t flag = 1;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (k < (int)nv) {
                        const int c = (int)v[k], tp = (int)((wt >> (8 * k)) & 255u);
                        const int mt = max(tp, gmax), gv = max(c, (int)t);
                        n4[k] = vlc_vp_bits(gv - mt, mt, (int)t) + 1;
                        flag &= rmode ? (uint32_t)(c <= (int)t) : (uint32_t)(mt == gv);
                    }
                }
                insig = (flag & __shfl_xor_sync(FULL, flag, 1)) != 0;
            }
            if (L.raw) {
                /* raw GCLIs: the lane's nibbles in one write */
                if (nv) put_bits(buf, words, L.gcli_pos + 4 * g, ((v[0] << 12) | (v[1] << 8) | (v[2] << 4) | v[3]) >> (4 * (4 - nv)), 4 * nv, ovf);
            } else {
                if (L.meth & 2) {
                    /* significance flags, 1 = insignificant: even lanes lead a group of 8 */
                    const uint32_t bal = __ballot_sync(FULL, nv && !(lane & 1) && insig);
                    if (lane == 0) {
                        /* the even lanes' votes compacted (bit i: group of 8
                         * number i), then reversed: group 0 first */
                        const uint32_t nsg = min(16u, (gend - base + 7) >> 3);
                        uint32_t x = bal & 0x55555555u;
                        x = (x | (x >> 1)) & 0x33333333u;
                        x = (x | (x >> 2)) & 0x0f0f0f0fu;
                        x = (x | (x >> 4)) & 0x00ff00ffu;
                        x = (x | (x >> 8)) & 0x0000ffffu;
                        const uint32_t bits = __brev(x) >> (32 - nsg);
                        if (bits) put_bits(buf, words, L.sig_pos + (base >> 3), bits, nsg, ovf);
                    }
                }
                if (!((L.meth & 2) && insig)) {
                    if (VPRED && (L.meth & 1)) {
#pragma unroll
                        for (int k = 0; k < 4; k++) vl += n4[k];
                    } else {
                        /* unary codes: d ones then a zero for each present
                         * group (PackPrecinct.h:25-39), two groups per word */
                        uint32_t n[4], c[4];
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const uint32_t dk = (d4 >> (8 * k)) & 255u;
                            n[k] = k < (int)nv ? dk + 1 : 0u;
                            c[k] = ((1u << dk) - 1u) << 1;
                        }
                        const uint32_t l23 = n[2] + n[3];
                        vacc = ((uint64_t)((c[0] << n[1]) | c[1]) << l23) | ((c[2] << n[3]) | c[3]);
                        vl = dsum + nv;
                    }
                }
            }
            /* data bits of the groups above gtli: 4 (d + 1) each (the sign
             * nibble, unless signs go to their own sub-packet) */
            const uint32_t dl4 = dsum + (fs ? 0u : nsig);
            /* one scan for three running sums: data bits / 4 (12 bits), code
             * bits (13 bits), listed groups (the exclusive sums, at most 124,
             * in the top 7 bits) */
            uint32_t tot;
            const uint32_t ex = warp_excl_scan(dl4 | (vl << 12) | (nsig << 25), &tot);
            const uint32_t ex_d = (ex & 0xfffu) << 2, ex_v = (ex >> 12) & 0x1fffu;
            const uint32_t tot_d = (tot & 0xfffu) << 2, tot_v = (tot >> 12) & 0x1fffu;
            if (vl) {
                if (VPRED && (L.meth & 1)) {
                    /* prediction codes (up to 31 bits each): n - 1 ones then
                     * a zero, joined while they fit 64 bits */
                    uint32_t pos = vpos + ex_v, an = 0;
                    uint64_t acc = 0;
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        const uint32_t n = n4[k];
                        if (n) {
                            if (an + n > 64) {
                                put_bits(buf, words, pos, acc, an, ovf);
                                pos += an;
                                acc = 0;
                                an = 0;
                            }
                            acc = (acc << n) | (((1ull << (n - 1)) - 1) << 1);
                            an += n;
                        }
                    }
                    if (an) put_bits(buf, words, pos, acc, an, ovf);
                } else {
                    put_bits(buf, words, vpos + ex_v, vacc, vl, ovf);
                }
            }
            uint32_t sbits = 0, sn = 0;
            if (!fs) {
                /* signs with the data: the warp lists its groups with GCLI
                 * > gtli (bit offset in the warp's data, group, GCLI), then
                 * each lane packs one listed group at a time, its sign
                 * nibble and planes in one write of at most 64 bits; the
                 * coefficients of the other groups are never read */
                uint32_t* list = &s_segw[0][0] + 128 * warp;
                const uint32_t cnt = __reduce_add_sync(FULL, nsig);
                {
                    /* per byte: 1 for a listed group, and its data nibbles
                     * v - t + 1; their exclusive prefix sums over the
                     * lane's bytes give each entry's slot and offset */
                    const uint32_t one = s4 & 0x01010101u, dd = d4 + one;
                    const uint32_t po = dd * 0x01010100u, pi = one * 0x01010100u;
                    const uint32_t e0 = (ex_d << 11) | ((uint32_t)lane << 6), i0 = ex >> 25;
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        if ((one >> (8 * k)) & 1u)
                            list[i0 + ((pi >> (8 * k)) & 255u)] = e0 + (((po >> (8 * k)) & 255u) << 13) + ((uint32_t)k << 4) + v[k];
                }
                __syncwarp();
                for (uint32_t r = lane; r < cnt; r += 32) {
                    const uint32_t e = list[r];
                    const uint32_t gi = base + ((e >> 4) & 127u), vv = e & 15u, np = vv - t;
                    /* the coefficients past the band width are stored as zero */
                    const uint2 raw4 = *(const uint2*)(crow + 4 * gi);
                    put_bits(buf, words, dpos + (e >> 11), data_chunk_signed(raw4, vv, t, uniform), 4 * (np + 1), ovf);
                }
                __syncwarp();
            } else if (dl4) {
                /* data bits of the groups with gcli > gtli (pack_data_c,
                 * PackPrecinct.c:128-198), joined while they fit 64 bits */
                uint32_t pos = dpos + ex_d;
                uint64_t acc = 0;
                uint32_t an = 0;
                const uint2 cw[4] = {make_uint2(c0.x, c0.y), make_uint2(c0.z, c0.w), make_uint2(c1.x, c1.y), make_uint2(c1.z, c1.w)};
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (k < (int)nv && v[k] > t) {
                        const uint32_t np = v[k] - t, n = 4 * (np + 1 - fs);
                        uint32_t sgn, nzm;
                        uint64_t ch = data_chunk(cw[k], (int)B.w - 4 * (int)(g + k), v[k], t, uniform, sgn, nzm);
                        if (fs) {
                            /* the signs of the non-zero magnitudes, coefficient 0 first */
#pragma unroll
                            for (int j = 3; j >= 0; j--) {
                                if ((nzm >> j) & 1u) {
                                    sbits = (sbits << 1) | ((sgn >> j) & 1u);
                                    sn++;
                                }
                            }
                        } else {
                            ch |= (uint64_t)sgn << (4 * np);
                        }
                        if (an + n > 64) {
                            put_bits(buf, words, pos, acc, an, ovf);
                            pos += an;
                            acc = 0;
                            an = 0;
                        }
                        acc = n == 64 ? ch : (acc << n) | ch;
                        an += n;
                    }
                }
                if (an) put_bits(buf, words, pos, acc, an, ovf);
            }
            vpos += tot_v;
            dpos += tot_d;
            if (fs) {
                /* sign sub-packet (pack_sign_c, PackPrecinct.c:200-233) */
                uint32_t stot;
                const uint32_t sx = warp_excl_scan(sn, &stot);
                if (sn) put_bits(buf, words, npos + sx, sbits, sn, ovf);
                npos += stot;
            }
        }
    }
    if (__syncthreads_or(ovf)) {
        if (threadIdx.x == 0) {
            printf("jxs pack: precinct %d wrote past its %u words\n", p, words);
            JXS_STATUS_SET(status, JXS_E_ENC_FRAME);
        }
        return;
    }
    /* copy out: whole 16-byte chunks where the precinct covers them, single
     * bytes at its two ends; slice header, codestream header and EOC around */
    const uint8_t* bytes = (const uint8_t*)buf;
    uint8_t* gbase = out + R.offset - lead;
    const uint32_t nbytes = lead + total;
    for (uint32_t c = threadIdx.x; c < (nbytes + 15) >> 4; c += blockDim.x) {
        const uint32_t b0 = c << 4;
        if (b0 >= lead && b0 + 16 <= nbytes) {
            *(uint4*)(gbase + b0) = *(const uint4*)(bytes + b0);
        } else {
            for (uint32_t i = max(b0, lead); i < min(b0 + 16, nbytes); i++) gbase[i] = bytes[i];
        }
    }
    if (threadIdx.x == 0) {
        uint8_t* dst = out + R.offset;
        if (R.first_in_slice) {
            const uint32_t s = p / cfg->pps;
            uint8_t* sh = dst - 6;
            sh[0] = 0xff; sh[1] = 0x20; sh[2] = 0; sh[3] = 4;
            sh[4] = (uint8_t)(s >> 8); sh[5] = (uint8_t)s;
        }
        if (p + 1 == (int)cfg->np) {
            dst[total] = 0xff;
            dst[total + 1] = 0x11;
        }
    }
    if (p == 0)
        for (uint32_t i = threadIdx.x; i < cfg->hdr_len; i += blockDim.x) out[i] = cfg->hdr[i];
}

/* ------------------------------------------------------------------------ */
/* kernels: one frame, or a batch of frames (block -> frame by its first block) */
/* ------------------------------------------------------------------------ */
template <bool SIGNS, bool VPRED>
__global__ void __launch_bounds__(RC_THREADS, (SIGNS || VPRED) ? 3 : 4) rc_cost_kernel(const jxs_cfg_t* __restrict__ cfg, const uint8_t* __restrict__ gcli,
                                                           const uint16_t* __restrict__ coef, uint32_t* __restrict__ cost,
                                                           uint32_t* __restrict__ slice_done, PrecRC* __restrict__ rc,
                                                           int* __restrict__ status) {
    rc_cost_body<SIGNS, VPRED>(cfg, gcli, coef, cost, slice_done, rc, status, (int)blockIdx.x);
}

template <bool SIGNS, bool VPRED>
__global__ void __launch_bounds__(RC_THREADS, (SIGNS || VPRED) ? 3 : 4) rc_cost_batch_kernel(const __grid_constant__ EncPrecLaunch L) {
    const EncPrecFrame& F = L.job[find_job<JXS_BATCH_FRAMES>(L.job, L.nframes, (int)blockIdx.x)];
    rc_cost_body<SIGNS, VPRED>(F.cfg, F.gcli, F.coef, F.cost, F.slice_done, F.rc, F.status, (int)blockIdx.x - F.first_block);
}

template <bool VPRED>
__global__ void __launch_bounds__(PK_THREADS, 4) pack_kernel(const jxs_cfg_t* __restrict__ cfg, const uint16_t* __restrict__ coef,
                                                          const uint8_t* __restrict__ gcli, const PrecRC* __restrict__ rc,
                                                          const uint32_t* __restrict__ cost, uint8_t* __restrict__ out,
                                                          uint32_t cap_words, int* status) {
    pack_body<VPRED>(cfg, coef, gcli, rc, cost, out, cap_words, status, (int)blockIdx.x);
}

template <bool VPRED>
__global__ void __launch_bounds__(PK_THREADS, 4) pack_batch_kernel(const __grid_constant__ EncPrecLaunch L, uint32_t cap_words) {
    const EncPrecFrame& F = L.job[find_job<JXS_BATCH_FRAMES>(L.job, L.nframes, (int)blockIdx.x)];
    pack_body<VPRED>(F.cfg, F.coef, F.gcli, F.rc, F.cost, F.out, cap_words, F.status, (int)blockIdx.x - F.first_block);
}

/* ------------------------------------------------------------------------ */
/* host-side launchers                                                       */
/* ------------------------------------------------------------------------ */
/* The rate-control variants: `modes` bit 0 = a frame of the launch has
 * sign handling, bit 1 = vertical prediction (dynamic shared memory for
 * the ordered selection). */
#define RC_VP_SMEM (RC_VP_REGIONS * RC_LT_REGION * 4)
template <bool S, bool V>
static cudaError_t rc_one(const jxs_cfg_t* dcfg, uint32_t np, const uint8_t* gcli, const uint16_t* coef, uint32_t* cost,
                          uint32_t* slice_done, PrecRC* rc, int* status, cudaStream_t st) {
    if (V) {
        static std::atomic<int> attr[JXS_MAX_DEV];
        cudaError_t e = jxs_smem_attr(rc_cost_kernel<S, V>, RC_VP_SMEM, attr);
        if (e != cudaSuccess) return e;
    }
    rc_cost_kernel<S, V><<<np, RC_THREADS, V ? RC_VP_SMEM : 0, st>>>(dcfg, gcli, coef, cost, slice_done, rc, status);
    return cudaGetLastError();
}
template <bool S, bool V>
static cudaError_t rc_batch_one(const EncPrecLaunch* L, cudaStream_t st) {
    if (V) {
        static std::atomic<int> attr[JXS_MAX_DEV];
        cudaError_t e = jxs_smem_attr(rc_cost_batch_kernel<S, V>, RC_VP_SMEM, attr);
        if (e != cudaSuccess) return e;
    }
    rc_cost_batch_kernel<S, V><<<L->nblocks, RC_THREADS, V ? RC_VP_SMEM : 0, st>>>(*L);
    return cudaGetLastError();
}

extern "C" cudaError_t jxs_launch_rc(const jxs_cfg_t* dcfg, uint32_t np, uint32_t nslices, const uint8_t* gcli,
                                     const uint16_t* coef, uint32_t* cost, uint32_t* slice_done, PrecRC* rc, int* status,
                                     int modes, cudaStream_t st) {
    (void)nslices;
    switch (modes & 3) {
    case 0: return rc_one<false, false>(dcfg, np, gcli, coef, cost, slice_done, rc, status, st);
    case 1: return rc_one<true, false>(dcfg, np, gcli, coef, cost, slice_done, rc, status, st);
    case 2: return rc_one<false, true>(dcfg, np, gcli, coef, cost, slice_done, rc, status, st);
    default: return rc_one<true, true>(dcfg, np, gcli, coef, cost, slice_done, rc, status, st);
    }
}

template <bool V>
static cudaError_t pack_one(const jxs_cfg_t* dcfg, uint32_t np, const uint16_t* coef, const uint8_t* gcli, const PrecRC* rc,
                            const uint32_t* cost, uint8_t* out, uint32_t cap_words, int* status, cudaStream_t st) {
    const size_t smem = (size_t)cap_words * 4;
    static std::atomic<int> attr[JXS_MAX_DEV];
    cudaError_t e = jxs_smem_attr(pack_kernel<V>, (int)smem, attr);
    if (e != cudaSuccess) return e;
    pack_kernel<V><<<np, PK_THREADS, smem, st>>>(dcfg, coef, gcli, rc, cost, out, cap_words, status);
    return cudaGetLastError();
}

/* `modes` bit 1: a frame of the launch has vertical prediction */
extern "C" cudaError_t jxs_launch_pack(const jxs_cfg_t* dcfg, uint32_t np, const uint16_t* coef, const uint8_t* gcli,
                                       const PrecRC* rc, const uint32_t* cost, uint8_t* out, uint32_t cap_words, int* status,
                                       int modes, cudaStream_t st) {
    if (modes & 2) return pack_one<true>(dcfg, np, coef, gcli, rc, cost, out, cap_words, status, st);
    return pack_one<false>(dcfg, np, coef, gcli, rc, cost, out, cap_words, status, st);
}

extern "C" cudaError_t jxs_launch_rc_batch(const EncPrecLaunch* L, int modes, cudaStream_t st) {
    if (L->nblocks <= 0) return cudaSuccess;
    switch (modes & 3) {
    case 0: return rc_batch_one<false, false>(L, st);
    case 1: return rc_batch_one<true, false>(L, st);
    case 2: return rc_batch_one<false, true>(L, st);
    default: return rc_batch_one<true, true>(L, st);
    }
}

template <bool V>
static cudaError_t pack_batch_one(const EncPrecLaunch* L, uint32_t cap_words, cudaStream_t st) {
    const size_t smem = (size_t)cap_words * 4;
    static std::atomic<int> attr[JXS_MAX_DEV];
    cudaError_t e = jxs_smem_attr(pack_batch_kernel<V>, (int)smem, attr);
    if (e != cudaSuccess) return e;
    if (L->nblocks <= 0) return cudaSuccess;
    pack_batch_kernel<V><<<L->nblocks, PK_THREADS, smem, st>>>(*L, cap_words);
    return cudaGetLastError();
}

extern "C" cudaError_t jxs_launch_pack_batch(const EncPrecLaunch* L, uint32_t cap_words, int modes, cudaStream_t st) {
    if (modes & 2) return pack_batch_one<true>(L, cap_words, st);
    return pack_batch_one<false>(L, cap_words, st);
}
