/*
 * CPU restatement of the SVT-JPEG-XS (ISO/IEC 21122 JPEG XS) encode/decode
 * path.  TEST INFRASTRUCTURE ONLY: the oracle that the GPU product is checked
 * against, and the CPU restatement bench.py times beside the reference library.
 * It is pinned against the reference library built from the reference's own
 * sources (oracle/_ref, tests/test_oracle.py) and against tests/golden/.
 *
 * The reference pipelines its transform precinct by precinct with line
 * buffers; this restatement transforms whole components at once, which the
 * reference's own tests show to be exactly equal
 * (tests/UnitTests/TestDwtFrame.cc:378-399, TestInvDwtFrame.cc:394-415).
 * Everything else follows the reference's integer steps one to one; each
 * function names the reference lines it restates.
 *
 * Scope: every option the reference encoder emits: deadzone / uniform
 * quantisation, significance on/off, rate-control modes 0-3, sign handling
 * (fast and full), vertical prediction (modes 1 and 2), all colour formats,
 * decomp_v 0-2, decomp_h 0-5.  The decoder also reads what the reference
 * decoder reads beyond that: raw-mode packets, multi-column precincts
 * (Cw > 0), the reversible colour transform and Star-Tetrix, the NLT
 * marker's output non-linearities and proxy resolutions; the encoder writes
 * those forms too, to make test codestreams for them.
 */
#include "jxs_oracle.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* SvtJxsErrorType_t values (Source/API/SvtJpegxs.h:130-159). */
#define E_NONE 0
#define E_BAD_PARAM ((int)0x80001005)
#define E_RESOURCES ((int)0x80001000)
#define E_UNDEFINED ((int)0x80001001)
#define E_ENC_FRAME ((int)0x80002035)
#define E_DEC_PTR ((int)0x80003000)
#define E_DEC_BITSTREAM ((int)0x80003001)
#define E_DEC_SHORT ((int)0x80003003)

#define FMT_YUV420 2
#define FMT_YUV422 3
#define FMT_YUV444 4
#define FMT_4COMP 5
#define FMT_GRAY 6
#define FMT_PACKED_RGB 21

#define MAXC 4
#define MAXB 10
#define MAXGB 40
#define MAXPK 30
#define NOBAND 0xff
#define TRUNC_MAX 15
#define BW 20
#define FQ 8
#define PREC_MAX_BYTES 1048575u

#define DIV_UP(a, b) (((a) + (b)-1) / (b))
#define MIN(a, b) ((a) < (b) ? (a) : (b))
#define MAX(a, b) ((a) > (b) ? (a) : (b))

/* ------------------------------------------------------------------------ */
/* Geometry: restates pi_compute / calc_packet_inclusion /                    */
/* calc_precinct_dimension (Source/Lib/Common/Codec/Pi.c:21-406).  Cw = 0     */
/* (the only value the reference encoder writes) gives one precinct per row;  */
/* Cw > 0 splits every row into columns of 8 Cw max(Sx) 2^NLx samples.       */
/* ------------------------------------------------------------------------ */
typedef struct {
    uint32_t w, h, x, y;
    uint32_t lines;          /* lines per precinct */
    uint32_t last_lines;     /* lines in the last precinct row */
    uint32_t gcli_w, sig_w;
    uint8_t gain, prio;
    uint32_t gid;
    /* precinct columns: coefficients, groups and significance groups of a
     * normal / the last column, and the row strides of the encoder's GCLI
     * and significance-maximum planes (each column grouped on its own) */
    uint32_t wn, wl, gwn, gwl, swn, swl, gstride, sstride;
} band_t;

typedef struct {
    uint32_t w, h, sx, sy, dv, dh, prec_h, nb;
    band_t b[MAXB];
} comp_t;

typedef struct {
    uint32_t bs, be, line;
} packet_t;

typedef struct {
    uint32_t nc, W, H, dv, dh, sd, prec_h, slice_h, pps, np, nslices;
    uint32_t cw, ncol;             /* precinct width (Cw) and precincts per row; np counts rows */
    uint32_t nbands_all, nbands_exist;
    uint8_t gcomp[MAXGB], gband[MAXGB];
    uint32_t npk;
    packet_t pk[MAXPK];
    int short_hdr;
    comp_t c[MAXC];
    uint32_t pk_exist[2];          /* packets present in a normal / the last precinct row */
    uint32_t raw_bytes[4][MAXPK];  /* raw-mode GCLI sub-packet bytes per precinct kind (pkind) */
} geom_t;

/* A precinct's kind: bit 0 the last row, bit 1 the last of several columns
 * (PRECINCT_NORMAL / _LAST_NORMAL / _NORMAL_LAST / _LAST, Pi.h). */
static inline int pkind(const geom_t* g, int last_row, uint32_t col) {
    return last_row + ((g->ncol > 1 && col + 1 == g->ncol) ? 2 : 0);
}

/* A band's part in precinct column `col`: coefficients, groups and
 * significance groups, and where they start in the band's rows. */
typedef struct {
    uint32_t w, gw, sw, x0, g0, s0;
} bview_t;
static inline bview_t bview(const geom_t* g, const band_t* bd, uint32_t col) {
    const int lc = col + 1 == g->ncol;
    bview_t v = {lc ? bd->wl : bd->wn, lc ? bd->gwl : bd->gwn, lc ? bd->swl : bd->swn, col * bd->wn, col * bd->gwn,
                 col * bd->swn};
    return v;
}

static int sampling(uint32_t fmt, uint32_t* nc, uint32_t sx[MAXC], uint32_t sy[MAXC]) {
    /* format_get_sampling_factory, Pi.c:521-565 */
    for (int i = 0; i < MAXC; i++) sx[i] = sy[i] = 1;
    switch (fmt) {
    case FMT_YUV422: *nc = 3; sx[1] = sx[2] = 2; return 0;
    case FMT_YUV420: *nc = 3; sx[1] = sx[2] = 2; sy[1] = sy[2] = 2; return 0;
    case FMT_YUV444:
    case FMT_PACKED_RGB: *nc = 3; return 0;
    case FMT_4COMP: *nc = 4; return 0;
    case FMT_GRAY: *nc = 1; return 0;
    default: return E_BAD_PARAM;
    }
}

static int geom_compute(geom_t* g, int for_encoder, uint32_t nc, uint32_t W, uint32_t H, uint32_t dh, uint32_t dv, uint32_t sd,
                        const uint32_t sx[MAXC], const uint32_t sy[MAXC], uint32_t slice_h, uint32_t cw) {
    memset(g, 0, sizeof(*g));
    g->cw = cw;
    if (sd > nc || dv > dh || dh > 5 || dv > 2 || nc > MAXC || slice_h == 0) return E_BAD_PARAM;
    g->nc = nc; g->W = W; g->H = H; g->dh = dh; g->dv = dv; g->sd = sd;
    const uint32_t ncd = nc - sd;
    g->prec_h = 1u << dv;
    if (slice_h < H && (slice_h % g->prec_h)) return E_BAD_PARAM;
    g->slice_h = slice_h;
    g->pps = DIV_UP(slice_h, g->prec_h);
    g->nslices = DIV_UP(H, slice_h);
    g->nbands_exist = 0;
    for (uint32_t c = 0; c < nc; c++) {
        comp_t* cp = &g->c[c];
        if (sx[c] < 1 || sy[c] < 1) return E_BAD_PARAM;
        cp->sx = sx[c]; cp->sy = sy[c];
        cp->w = W / sx[c]; cp->h = H / sy[c];
        cp->prec_h = g->prec_h / sy[c];
        if (cp->prec_h == 0) return E_BAD_PARAM;
        if (c < ncd) {
            cp->dh = dh;
            if (dv < sy[c] / 2) return E_BAD_PARAM;
            cp->dv = dv - sy[c] / 2;
        } else {
            cp->dh = cp->dv = 0;
        }
        cp->nb = 2 * cp->dv + cp->dh + 1;
        if (cp->nb > MAXB || cp->nb < 1) return E_BAD_PARAM;
        g->nbands_exist += cp->nb;
    }
    g->nbands_all = g->c[0].nb * ncd + sd;
    memset(g->gcomp, NOBAND, sizeof(g->gcomp));
    memset(g->gband, NOBAND, sizeof(g->gband));
    const uint32_t nb_global = 2 * dv + dh + 1;
    for (uint32_t c = 0; c < ncd; c++) {
        comp_t* cp = &g->c[c];
        uint32_t ignore = nb_global - cp->nb;
        uint32_t at_end = 3 * cp->dv;
        uint32_t id = c;
        for (uint32_t i = 0; i < cp->nb; i++) {
            cp->b[i].gid = id;
            g->gcomp[id] = (uint8_t)c;
            g->gband[id] = (uint8_t)i;
            id += ncd;
            if (ignore > 0 && i == cp->nb - at_end + 1 - ignore) id += ncd * ignore;
        }
    }
    for (uint32_t c = ncd; c < nc; c++) {
        comp_t* cp = &g->c[c];
        if (cp->nb != 1) return E_BAD_PARAM;
        uint32_t id = ncd * g->c[0].nb + c - ncd;
        cp->b[0].gid = id;
        g->gcomp[id] = (uint8_t)c;
        g->gband[id] = 0;
    }
    for (uint32_t c = 0; c < nc; c++) {
        comp_t* cp = &g->c[c];
        int L = (int)cp->nb - 1;
        cp->b[L].w = cp->w; cp->b[L].h = cp->h; cp->b[L].x = 0; cp->b[L].y = 0;
        for (uint32_t v = 0; v < cp->dv; v++) {
            if (L < 3) return E_BAD_PARAM;
            band_t t = cp->b[L];
            uint32_t w2 = t.w / 2, w1 = t.w - w2, h2 = t.h / 2, h1 = t.h - h2;
            cp->b[L] = (band_t){.w = w2, .h = h2, .x = w1, .y = h1, .gid = cp->b[L].gid};
            cp->b[L - 1].w = w1; cp->b[L - 1].h = h2; cp->b[L - 1].x = 0; cp->b[L - 1].y = h1;
            cp->b[L - 2].w = w2; cp->b[L - 2].h = h1; cp->b[L - 2].x = w1; cp->b[L - 2].y = 0;
            cp->b[L - 3].w = w1; cp->b[L - 3].h = h1; cp->b[L - 3].x = 0; cp->b[L - 3].y = 0;
            L -= 3;
        }
        for (uint32_t hl = cp->dv; hl < cp->dh; hl++) {
            if (L < 1) return E_BAD_PARAM;
            band_t t = cp->b[L];
            uint32_t w2 = t.w / 2, w1 = t.w - w2;
            cp->b[L].w = w2; cp->b[L].h = t.h; cp->b[L].x = w1; cp->b[L].y = 0;
            cp->b[L - 1].w = w1; cp->b[L - 1].h = t.h; cp->b[L - 1].x = 0; cp->b[L - 1].y = 0;
            L -= 1;
        }
        for (uint32_t b = 0; b < cp->nb; b++)
            if (cp->b[b].w == 0 || cp->b[b].h == 0) return E_BAD_PARAM;
        uint32_t two = (cp->dv == 2) ? 3 : 0;
        for (uint32_t b = 0; b < cp->nb; b++) cp->b[b].lines = (b < cp->nb - two) ? 1 : 2;
    }
    for (uint32_t c = ncd; c < nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++) g->c[c].b[b].lines = MIN(((1u << dv) >> (g->c[c].sy - 1)), g->c[c].h);

    /* calc_packet_inclusion, Pi.c:131-187 */
    uint32_t n = 0;
    uint32_t stop0 = MAX(dh, dv) - MIN(dh, dv) + 1;
    g->pk[n++] = (packet_t){0, stop0 * ncd, 0};
    for (uint32_t bs = stop0; bs < g->c[0].nb; bs++) {
        packet_t p = {bs * ncd, bs * ncd, 0};
        for (uint32_t i = bs * ncd; i < (bs + 1) * ncd; i++)
            if (g->gband[i] != NOBAND) p.be++;
        g->pk[n++] = p;
    }
    for (uint32_t bs = stop0; bs < g->c[0].nb; bs++) {
        if (g->c[0].b[bs].lines == 1) continue;
        packet_t p = {bs * ncd, bs * ncd, 1};
        for (uint32_t i = bs * ncd; i < (bs + 1) * ncd; i++)
            if (g->gband[i] != NOBAND && g->c[g->gcomp[i]].b[g->gband[i]].lines > 1) p.be++;
        g->pk[n++] = p;
    }
    uint32_t nbands = ncd * g->c[0].nb;
    for (uint32_t c = ncd; c < nc; c++) {
        for (uint32_t line = 0; line < g->c[c].b[0].lines; line++) g->pk[n++] = (packet_t){nbands, nbands + 1, line};
        nbands++;
    }
    if (n >= MAXPK) return E_BAD_PARAM;
    g->npk = n;
    g->short_hdr = (W * nc) < 32752;

    /* calc_precinct_dimension, Pi.c:21-129 */
    g->np = DIV_UP(H, 1u << dv);
    g->ncol = 1;
    uint32_t cs = 0;
    if (cw) {
        uint32_t sx_max = 0;
        for (uint32_t c = 0; c < nc; c++) sx_max = MAX(sx_max, g->c[c].sx);
        cs = 8 * cw * sx_max * (1u << dh);
        g->ncol = DIV_UP(W, cs);
        if (g->ncol >= 130) return E_BAD_PARAM; /* MAX_PRECINCT_IN_LINE, Decoder.c:294 */
    }
    for (uint32_t c = 0; c < nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++) {
            band_t* bd = &g->c[c].b[b];
            bd->last_lines = bd->h - (g->np - 1) * bd->lines;
            bd->gcli_w = DIV_UP(bd->w, 4);
            bd->sig_w = DIV_UP(bd->gcli_w, 8);
            bd->wn = bd->w; /* one column: it is the last one, of the band's width */
            if (cw && g->ncol > 1) {
                const uint64_t num = (uint64_t)cs * bd->w, den = (uint64_t)g->c[c].sx * g->c[c].w;
                bd->wn = (uint32_t)((bd->w % 2) ? num / den : (num + den - 1) / den);
                /* a last column without coefficients is outside this
                 * restatement (the reference's width_last would wrap) */
                if ((uint64_t)(g->ncol - 1) * bd->wn >= bd->w) return E_BAD_PARAM;
            }
            bd->wl = bd->w - (g->ncol - 1) * bd->wn;
            bd->gwn = DIV_UP(bd->wn, 4);
            bd->gwl = DIV_UP(bd->wl, 4);
            bd->swn = DIV_UP(bd->gwn, 8);
            bd->swl = DIV_UP(bd->gwl, 8);
            bd->gstride = (g->ncol - 1) * bd->gwn + bd->gwl;
            bd->sstride = (g->ncol - 1) * bd->swn + bd->swl;
        }
    if (for_encoder) {
        g->pk_exist[0] = g->npk;
        uint32_t cnt = 0;
        for (uint32_t k = 0; k < g->npk; k++) {
            int present = 0;
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++)
                if (g->pk[k].line < g->c[g->gcomp[i]].b[g->gband[i]].last_lines) { present = 1; break; }
            cnt += present;
        }
        g->pk_exist[1] = cnt;
        for (int t = 0; t < 4; t++)
            for (uint32_t k = 0; k < g->npk; k++) {
                uint32_t bits = 0;
                for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                    band_t* bd = &g->c[g->gcomp[i]].b[g->gband[i]];
                    uint32_t lines = (t & 1) ? bd->last_lines : bd->lines;
                    if (g->pk[k].line < lines) bits += ((t & 2) ? bd->gwl : bd->gwn) * 4;
                }
                g->raw_bytes[t][k] = DIV_UP(bits, 8);
            }
    }
    return E_NONE;
}

/* ------------------------------------------------------------------------ */
/* Weight tables: gains and priorities per global band for V2/H5 from         */
/* ISO/IEC 21122-1 (and the reference's added 4:2:0 rows), plus the           */
/* reference's derivation for other H/V (WeightTable.c:18-413).               */
/* ------------------------------------------------------------------------ */
static const uint8_t wt444_g[3][30] = {
    {3, 2, 2, 2, 1, 1, 2, 1, 1, 1, 0, 0, 1, 0, 0, 1, 0, 0},
    {4, 2, 2, 3, 2, 2, 2, 1, 1, 2, 1, 1, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0},
    {4, 3, 3, 3, 2, 2, 3, 2, 2, 2, 1, 1, 2, 1, 1, 2, 1, 1, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0}};
static const uint8_t wt444_p[3][30] = {
    {6, 8, 7, 1, 4, 5, 12, 14, 15, 0, 2, 3, 9, 11, 10, 13, 16, 17},
    {21, 1, 0, 15, 19, 18, 5, 9, 8, 14, 17, 16, 2, 4, 3, 7, 13, 11, 6, 12, 10, 20, 23, 22},
    {12, 15, 14, 3, 11, 10, 24, 26, 27, 0, 4, 5, 18, 21, 20, 19, 23, 22, 13, 16, 17, 2, 9, 6, 1, 7, 8, 25, 28, 29}};
static const uint8_t wt422_g[3][30] = {
    {2, 2, 2, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {3, 3, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};
static const uint8_t wt422_p[3][30] = {
    {8, 7, 6, 5, 3, 4, 13, 12, 14, 1, 0, 2, 9, 11, 10, 16, 15, 17},
    {0, 1, 2, 18, 19, 20, 6, 7, 8, 15, 16, 17, 3, 4, 5, 10, 12, 14, 9, 11, 13, 21, 22, 23},
    {14, 13, 12, 9, 11, 10, 25, 24, 26, 0, 1, 2, 19, 20, 18, 23, 22, 21, 17, 15, 16, 4, 8, 5, 3, 6, 7, 28, 27, 29}};
static const uint8_t wt444_n[3] = {18, 24, 30};
#define NE NOBAND
/* 4:2:0 tables indexed [v-1][h-1] (v = 1..2, h = v..5). */
static const uint8_t wt420_g[2][5][30] = {
    {{1, 1, 1, 1, 0, 0, 1, NE, NE, 0, NE, NE},
     {1, 1, 1, 1, 0, 0, 1, 0, 0, 1, NE, NE, 0, NE, NE},
     {2, 1, 1, 1, 1, 1, 1, 0, 0, 1, 0, 0, 1, NE, NE, 0, NE, NE},
     {2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 0, 0, 1, 0, 0, 1, NE, NE, 0, NE, NE},
     {3, 3, 3, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 0, 0, 1, 0, 0, 1, NE, NE, 0, NE, NE}},
    {{0},
     {2, 1, 1, 1, 1, 1, 1, NE, NE, 0, NE, NE, 1, 1, 1, 1, 1, 1, 0, 0, 0},
     {2, 2, 2, 2, 1, 1, 1, 1, 1, 1, NE, NE, 0, NE, NE, 1, 1, 1, 1, 1, 1, 0, 0, 0},
     {3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, NE, NE, 0, NE, NE, 1, 1, 1, 1, 1, 1, 0, 0, 0},
     {3, 3, 3, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, NE, NE, 0, NE, NE, 1, 1, 1, 1, 1, 1, 0, 0, 0}}};
static const uint8_t wt420_p[2][5][30] = {
    {{2, 5, 4, 6, 1, 0, 7, NE, NE, 3, NE, NE},
     {4, 7, 6, 8, 1, 0, 10, 3, 2, 9, NE, NE, 5, NE, NE},
     {11, 3, 2, 6, 9, 8, 10, 1, 0, 13, 5, 4, 12, NE, NE, 7, NE, NE},
     {7, 12, 11, 14, 3, 2, 6, 10, 9, 13, 1, 0, 16, 5, 4, 15, NE, NE, 8, NE, NE},
     {9, 16, 15, 7, 13, 12, 17, 3, 2, 6, 11, 10, 14, 1, 0, 19, 5, 4, 18, NE, NE, 8, NE, NE}},
    {{0},
     {10, 4, 3, 2, 9, 8, 1, NE, NE, 0, NE, NE, 16, 14, 12, 15, 13, 11, 7, 6, 5},
     {5, 12, 11, 13, 4, 3, 2, 10, 9, 1, NE, NE, 0, NE, NE, 19, 17, 15, 18, 16, 14, 8, 7, 6},
     {22, 6, 5, 7, 14, 13, 15, 4, 3, 2, 12, 11, 1, NE, NE, 0, NE, NE, 21, 19, 17, 20, 18, 16, 10, 9, 8},
     {0, 13, 12, 25, 7, 6, 8, 17, 16, 18, 5, 4, 3, 15, 14, 2, NE, NE, 1, NE, NE, 24, 22, 20, 23, 21, 19, 11, 10, 9}}};
static const uint8_t wt420_n[2][5] = {{12, 15, 18, 21, 24}, {0, 21, 24, 27, 30}};
#undef NE

/* weight_table_recalculate_table (WeightTable.c:143-335): start from the V2/H5
 * table, drop bands for fewer vertical and horizontal levels, then renumber
 * priorities densely. */
static void wt_derive(const uint8_t* g52, const uint8_t* p52, uint32_t dv, uint32_t dh, uint8_t* gain, uint8_t* prio,
                      uint32_t* size) {
    uint8_t g[30], p[30];
    memcpy(g, g52, 30);
    memcpy(p, p52, 30);
    uint32_t n = 30;
    int v = 2, h = 5;
    while (v > (int)dv) { /* reduce_v, WeightTable.c:200-230 */
        int rm = h - 1;
        v--;
        uint32_t cnt = n - 3 * (rm + 1);
        for (uint32_t i = 0; i < cnt; i++) { g[3 * rm + i] = g[3 * (rm + 1) + i]; p[3 * rm + i] = p[3 * (rm + 1) + i]; }
        n -= 3;
        n -= 3;
        for (uint32_t i = 0; i < n; i++) { g[i] = g[i + 3]; p[i] = p[i + 3]; }
    }
    int hh = 5;
    while (hh > (int)dh) { /* reduce_h, WeightTable.c:150-175 */
        hh--;
        if (hh != 1) {
            n -= 3;
            memmove(g, g + 3, n);
            memmove(p, p + 3, n);
        } else {
            n -= 3;
        }
    }
    /* rebuild_prio, WeightTable.c:232-256 */
    for (uint32_t i = 0; i < n; i++) {
        int found;
        do {
            found = 0;
            for (uint32_t j = 0; j < n; j++)
                if (p[j] == i) { found = 1; break; }
            if (!found)
                for (uint32_t j = 0; j < n; j++)
                    if (p[j] > i) { p[j]--; break; }
        } while (!found);
    }
    memcpy(gain, g, n);
    memcpy(prio, p, n);
    *size = n;
}

static int weights_assign(geom_t* g, uint32_t fmt) {
    /* weight_table_calculate, WeightTable.c:336-413 */
    uint8_t gain[30], prio[30];
    uint32_t size = 0;
    int have = 0;
    if (g->nc == 3) {
        if (fmt == FMT_YUV422 && g->dh == 5) {
            memcpy(gain, wt422_g[g->dv], 30); memcpy(prio, wt422_p[g->dv], 30); size = wt444_n[g->dv]; have = 1;
        } else if (fmt == FMT_YUV420 && g->dv >= 1 && g->dh >= g->dv && wt420_n[g->dv - 1][g->dh - 1]) {
            memcpy(gain, wt420_g[g->dv - 1][g->dh - 1], 30); memcpy(prio, wt420_p[g->dv - 1][g->dh - 1], 30);
            size = wt420_n[g->dv - 1][g->dh - 1]; have = 1;
        } else if ((fmt == FMT_YUV444 || fmt == FMT_PACKED_RGB) && g->dh == 5) {
            memcpy(gain, wt444_g[g->dv], 30); memcpy(prio, wt444_p[g->dv], 30); size = wt444_n[g->dv]; have = 1;
        }
    }
    if (!have && g->nc == 4 && fmt == FMT_4COMP) {
        /* no weight table exists for four components; the Star-Tetrix test
         * codestreams use gain 0 and priority = codestream band index */
        for (uint32_t c = 0; c < g->nc; c++)
            for (uint32_t b = 0; b < g->c[c].nb; b++) {
                g->c[c].b[b].gain = 0;
                g->c[c].b[b].prio = (uint8_t)g->c[c].b[b].gid;
            }
        return 0;
    }
    if (!have) {
        if (g->nc != 3) return -1;
        if (fmt == FMT_YUV422) wt_derive(wt422_g[2], wt422_p[2], g->dv, g->dh, gain, prio, &size);
        else if (fmt == FMT_YUV444 || fmt == FMT_PACKED_RGB) wt_derive(wt444_g[2], wt444_p[2], g->dv, g->dh, gain, prio, &size);
        else return -1;
    }
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++) {
            band_t* bd = &g->c[c].b[b];
            if (bd->gid >= size) return -1;
            bd->gain = gain[bd->gid];
            bd->prio = prio[bd->gid];
        }
    return 0;
}

/* compute_truncation, Source/Lib/Common/Codec/EncDec.c:8-21 */
static uint8_t truncation(uint8_t gain, uint8_t prio, uint8_t q, uint8_t r) {
    uint8_t up = prio < r ? 1 : 0;
    if (q < gain + up) return 0;
    uint8_t t = q - gain - up;
    return t > TRUNC_MAX ? TRUNC_MAX : t;
}

/* precinct_compute_truncation's "all bands fully truncated" test (EncDec.c:37-52). */
static int all_truncated(const geom_t* g, uint8_t q, uint8_t r) {
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++)
            if (truncation(g->c[c].b[b].gain, g->c[c].b[b].prio, q, r) != TRUNC_MAX) return 0;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Tiny pthread parallel-for.                                                 */
/* ------------------------------------------------------------------------ */
typedef void (*pf_fn)(void* ctx, uint32_t i);
typedef struct {
    pf_fn fn;
    void* ctx;
    uint32_t n;
    atomic_uint next;
} pf_t;
static void* pf_worker(void* a) {
    pf_t* p = (pf_t*)a;
    for (;;) {
        uint32_t i = atomic_fetch_add(&p->next, 1);
        if (i >= p->n) break;
        p->fn(p->ctx, i);
    }
    return NULL;
}
static void parallel_for(uint32_t n, uint32_t threads, pf_fn fn, void* ctx) {
    pf_t p;
    p.fn = fn; p.ctx = ctx; p.n = n;
    atomic_init(&p.next, 0);
    if (threads <= 1 || n <= 1) {
        pf_worker(&p);
        return;
    }
    if (threads > 256) threads = 256;
    pthread_t th[256];
    uint32_t started = 0;
    for (uint32_t t = 1; t < threads && t < n; t++)
        if (pthread_create(&th[started], NULL, pf_worker, &p) == 0) started++;
    pf_worker(&p);
    for (uint32_t t = 0; t < started; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------ */
/* 5/3 lifting along one line with symmetric extension.                       */
/* Forward: dwt_horizontal_line_c (Dwt.c:15-40) and the vertical loops        */
/* (Dwt.c:337-398).  Inverse: idwt_horizontal_line_*_c (Idwt.c:11-53) and     */
/* idwt_vertical_line_c (Idwt.c:186-263).  Output is de-interleaved: the      */
/* ceil(n/2) low-pass values first, then the floor(n/2) high-pass values.     */
/* ------------------------------------------------------------------------ */
static void fwd_line(int32_t* x, uint32_t n, size_t stride, int32_t* tmp) {
    uint32_t n1 = (n + 1) / 2, n2 = n / 2;
    int32_t* L = tmp;
    int32_t* Hh = tmp + n1;
    for (uint32_t i = 0; i < n2; i++) {
        int32_t a = x[(size_t)(2 * i) * stride];
        int32_t c = (2 * i + 2 < n) ? x[(size_t)(2 * i + 2) * stride] : a;
        Hh[i] = x[(size_t)(2 * i + 1) * stride] - ((a + c) >> 1);
    }
    for (uint32_t i = 0; i < n1; i++) {
        int32_t hp = Hh[i == 0 ? 0 : MIN(i - 1, n2 - 1)];
        int32_t hc = Hh[MIN(i, n2 - 1)];
        L[i] = x[(size_t)(2 * i) * stride] + ((hp + hc + 2) >> 2);
    }
    for (uint32_t i = 0; i < n; i++) x[(size_t)i * stride] = tmp[i];
}

static void inv_line(int32_t* x, uint32_t n, size_t stride, int32_t* tmp) {
    uint32_t n1 = (n + 1) / 2, n2 = n / 2;
    for (uint32_t i = 0; i < n1; i++) {
        int32_t hp = x[(size_t)(n1 + (i == 0 ? 0 : MIN(i - 1, n2 - 1))) * stride];
        int32_t hc = x[(size_t)(n1 + MIN(i, n2 - 1)) * stride];
        tmp[2 * i] = x[(size_t)i * stride] - ((hp + hc + 2) >> 2);
    }
    for (uint32_t i = 0; i < n2; i++) {
        int32_t a = tmp[2 * i];
        int32_t c = (2 * i + 2 < n) ? tmp[2 * i + 2] : a;
        tmp[2 * i + 1] = x[(size_t)(n1 + i) * stride] + ((a + c) >> 1);
    }
    for (uint32_t i = 0; i < n; i++) x[(size_t)i * stride] = tmp[i];
}

/* Whole-component forward transform in the Mallat layout: for each vertical
 * level, lift all columns of the current low-pass region then all its rows;
 * then lift only rows for the remaining horizontal levels.  This is the order
 * of transform_V1_Hx_precinct / transform_V2_Hx_precinct (Dwt.c:420-1142). */
static void fwd_component(int32_t* a, uint32_t w, uint32_t h, uint32_t dv, uint32_t dh) {
    int32_t* tmp = (int32_t*)malloc(sizeof(int32_t) * (MAX(w, h) + 2));
    uint32_t cw = w, ch = h;
    for (uint32_t v = 0; v < dv; v++) {
        for (uint32_t x = 0; x < cw; x++) fwd_line(a + x, ch, w, tmp);
        for (uint32_t y = 0; y < ch; y++) fwd_line(a + (size_t)y * w, cw, 1, tmp);
        cw = (cw + 1) / 2;
        ch = (ch + 1) / 2;
    }
    for (uint32_t l = dv; l < dh; l++) {
        for (uint32_t y = 0; y < ch; y++) fwd_line(a + (size_t)y * w, cw, 1, tmp);
        cw = (cw + 1) / 2;
    }
    free(tmp);
}

static void inv_component(int32_t* a, uint32_t w, uint32_t h, uint32_t dv, uint32_t dh) {
    int32_t* tmp = (int32_t*)malloc(sizeof(int32_t) * (MAX(w, h) + 2));
    uint32_t ws[8], hs[8];
    ws[0] = w; hs[0] = h;
    for (uint32_t l = 0; l < dh; l++) {
        ws[l + 1] = (ws[l] + 1) / 2;
        hs[l + 1] = l < dv ? (hs[l] + 1) / 2 : hs[l];
    }
    for (int l = (int)dh - 1; l >= (int)dv; l--)
        for (uint32_t y = 0; y < hs[l]; y++) inv_line(a + (size_t)y * w, ws[l], 1, tmp);
    for (int l = (int)dv - 1; l >= 0; l--) {
        for (uint32_t y = 0; y < hs[l]; y++) inv_line(a + (size_t)y * w, ws[l], 1, tmp);
        for (uint32_t x = 0; x < ws[l]; x++) inv_line(a + x, hs[l], w, tmp);
    }
    free(tmp);
}

/* image_shift_c (Source/Lib/Encoder/Codec/NltEnc.c:12-31): int32 -> 16-bit
 * sign-magnitude with Fq fractional bits rounded off, no negative zero. */
static inline uint16_t to_sm(int32_t v) {
    if (v >= 0) return (uint16_t)((v + (1 << (FQ - 1))) >> FQ);
    int32_t m = ((-v) + (1 << (FQ - 1))) >> FQ;
    return (uint16_t)(m ? (m | 0x8000) : 0);
}

/* ------------------------------------------------------------------------ */
/* Encoder state                                                              */
/* ------------------------------------------------------------------------ */
typedef struct {
    or_enc_params_t prm;
    geom_t g;
    uint32_t fmt, depth, lcod;
    uint8_t hdr[512];
    uint32_t hdr_len;
    uint32_t* slice_sizes;
    uint8_t max_q, max_r;
    /* band-major coefficients and GCLIs per component/band */
    uint16_t* coef[MAXC][MAXB];
    uint8_t* gcli[MAXC][MAXB];
    uint8_t* sigmax[MAXC][MAXB];
    uint8_t* out;
    uint8_t* q_out;
    uint8_t* r_out;
    int slice_err;
    int32_t* rct[MAXC]; /* Cpih = 1: the scaled input after the forward colour transform */
} enc_t;

/* encoder_init_configuration (Source/Lib/Encoder/Codec/EncHandle.c:128-454). */
static int enc_configure(enc_t* e, const or_enc_params_t* p) {
    e->prm = *p;
    or_enc_params_t* c = &e->prm;
    uint32_t nc, sx[MAXC], sy[MAXC];
    if (c->bit_depth < 8 || c->bit_depth > 14) return E_BAD_PARAM;
    if (sampling(c->colour_format, &nc, sx, sy)) return E_BAD_PARAM;
    if (c->decomp_v == 0 && c->colour_format == FMT_YUV420) return E_BAD_PARAM;
    if (c->slice_height == 0) return E_BAD_PARAM;
    if (c->slice_height >= c->height) c->slice_height = c->height;
    else if (c->slice_height % (1u << c->decomp_v)) return E_BAD_PARAM;
    if (c->quantization > 1) return E_BAD_PARAM;
    if (c->bpp_den == 0 || c->bpp_num == 0) return E_BAD_PARAM;
    uint64_t bpf = ((uint64_t)c->width * c->height * c->bpp_num / c->bpp_den + 7) / 8;
    if (bpf >= (1ull << 32) || bpf == 0) return E_BAD_PARAM;
    if (c->rate_control_mode >= 4) return E_BAD_PARAM;
    if (c->coding_vertical_prediction_mode >= 3) return E_BAD_PARAM;
    if (c->coding_signs_handling > 2) return E_BAD_PARAM;
    if (c->width < 4) return E_BAD_PARAM;
    if ((c->cpih != 0 && c->cpih != 1 && c->cpih != 3) || c->tnlt > 2) return E_BAD_PARAM;
    if (c->cpih == 1 && c->colour_format != FMT_YUV444 && c->colour_format != FMT_PACKED_RGB) return E_BAD_PARAM;
    if ((c->cpih == 3) != (c->colour_format == FMT_4COMP)) return E_BAD_PARAM;
    if (c->cpih == 3 && (c->cts_cf > 15 || c->cts_e1 > 15 || c->cts_e2 > 15 || c->cfa_type > 1)) return E_BAD_PARAM;
    if ((c->colour_format == FMT_YUV422 || c->colour_format == FMT_YUV420) && (c->width % 2)) return E_BAD_PARAM;
    if (c->colour_format == FMT_YUV420 && (c->height % 2)) return E_BAD_PARAM;
    if (c->decomp_v > 2 || c->decomp_h > 5 || c->decomp_h < c->decomp_v) return E_BAD_PARAM;
    if (c->decomp_h == 0 && c->decomp_v == 0) return E_BAD_PARAM;
    uint32_t mw = c->width, mh = c->height, mv = c->decomp_v;
    if (c->colour_format == FMT_YUV420) { mw >>= 1; mh >>= 1; mv -= 1; }
    if (c->colour_format == FMT_YUV422) mw >>= 1;
    for (uint32_t i = 0; i < c->decomp_h; i++) {
        if (mw > 1) mw -= mw / 2;
        else { mw = 0; break; }
    }
    for (uint32_t i = 0; i < mv; i++) {
        if (mh > 1) mh -= mh / 2;
        else { mh = 0; break; }
    }
    if (mw == 0 || mh == 0) return E_BAD_PARAM;
    int r = geom_compute(&e->g, 1, nc, c->width, c->height, c->decomp_h, c->decomp_v, 0, sx, sy, c->slice_height, c->precinct_width);
    if (r) return r;
    if (weights_assign(&e->g, c->colour_format)) return E_BAD_PARAM;
    e->fmt = c->colour_format;
    e->depth = c->bit_depth;
    e->lcod = (uint32_t)bpf;
    /* pi_enc_weight_table_calc_max_quantization_refinement, PiEnc.c:11-53 */
    uint32_t mr = 0;
    for (uint32_t cc = 0; cc < e->g.nc; cc++)
        for (uint32_t b = 0; b < e->g.c[cc].nb; b++) mr = MAX(mr, e->g.c[cc].b[b].prio);
    if (mr < 255) mr += 1;
    if (mr > e->g.nbands_all - 1) mr = e->g.nbands_all - 1;
    e->max_r = (uint8_t)mr;
    e->max_q = 31;
    while (e->max_q > 0) {
        if (!all_truncated(&e->g, e->max_q, e->max_r)) break;
        e->max_q--;
    }
    return E_NONE;
}

/* Big-endian bit writer (BitstreamWriter.c:166-232 semantics; partial bytes
 * are zero-filled). */
typedef struct {
    uint8_t* mem;
    uint64_t bit;
} bw_t;
static inline void bw_put(bw_t* w, uint32_t v, uint32_t n) {
    for (int i = (int)n - 1; i >= 0; i--) {
        uint64_t byte = w->bit >> 3;
        uint32_t sh = 7 - (uint32_t)(w->bit & 7);
        if (sh == 7) w->mem[byte] = 0;
        w->mem[byte] |= (uint8_t)(((v >> i) & 1u) << sh);
        w->bit++;
    }
}
static inline void bw_align(bw_t* w) { w->bit = (w->bit + 7) & ~(uint64_t)7; }

/* write_header (Source/Lib/Encoder/Codec/PackHeaders.c:11-89, 133-140). */
static void enc_write_header(enc_t* e) {
    geom_t* g = &e->g;
    bw_t w = {e->hdr, 0};
    bw_put(&w, 0xff10, 16);                    /* SOC */
    bw_put(&w, 0xff50, 16);                    /* CAP */
    bw_put(&w, DIV_UP(16 + 9, 8), 16);
    uint8_t cap[9] = {0, (uint8_t)(e->prm.cpih == 3), (uint8_t)(e->prm.tnlt == 1), (uint8_t)(e->prm.tnlt == 2),
                      (uint8_t)(e->fmt == FMT_YUV420), 0, 0, 0, 1 /* Rl */};
    for (int i = 0; i < 9; i++) bw_put(&w, cap[i], 1);
    bw_align(&w);
    bw_put(&w, 0xff12, 16);                    /* PIH */
    bw_put(&w, 26, 16);
    bw_put(&w, e->lcod, 32);
    bw_put(&w, 0, 16);                         /* Ppih */
    bw_put(&w, 0, 16);                         /* Plev */
    bw_put(&w, g->W, 16);
    bw_put(&w, g->H, 16);
    bw_put(&w, g->cw, 16);                     /* Cw */
    bw_put(&w, g->pps, 16);                    /* Hsl */
    bw_put(&w, g->nc, 8);
    bw_put(&w, 4, 8);                          /* Ng */
    bw_put(&w, 8, 8);                          /* Ss */
    bw_put(&w, BW, 8);
    bw_put(&w, (FQ << 4) | 4, 8);              /* Fq | Br */
    bw_put(&w, e->prm.cpih, 8);                /* Fslc | Ppoc | Cpih */
    bw_put(&w, (g->dh << 4) | g->dv, 8);
    bw_put(&w, !g->short_hdr, 1);              /* Lh */
    bw_put(&w, 1, 1);                          /* Rl */
    bw_put(&w, e->prm.quantization, 2);        /* Qpih */
    bw_put(&w, e->prm.coding_signs_handling ? 1 : 0, 2); /* Fs */
    bw_put(&w, e->prm.coding_vertical_prediction_mode == 2 ? 1 : 0, 2); /* Rm (EncHandle.c:250-253) */
    bw_put(&w, 0xff13, 16);                    /* CDT */
    bw_put(&w, 2 * g->nc + 2, 16);
    for (uint32_t c = 0; c < g->nc; c++) {
        bw_put(&w, e->depth, 8);
        bw_put(&w, g->c[c].sx, 4);
        bw_put(&w, g->c[c].sy, 4);
    }
    bw_put(&w, 0xff14, 16);                    /* WGT */
    bw_put(&w, 2 * g->nbands_exist + 2, 16);
    for (uint32_t i = 0; i < g->nbands_all; i++) {
        if (g->gcomp[i] == NOBAND) continue;
        band_t* bd = &g->c[g->gcomp[i]].b[g->gband[i]];
        bw_put(&w, bd->gain, 8);
        bw_put(&w, bd->prio, 8);
    }
    if (e->prm.cpih == 3) {
        bw_put(&w, 0xff18, 16); /* CTS */
        bw_put(&w, 4, 16);
        bw_put(&w, e->prm.cts_cf, 8);
        bw_put(&w, (e->prm.cts_e1 << 4) | e->prm.cts_e2, 8);
        bw_put(&w, 0xff19, 16); /* CRG: component positions of the CFA (Table F.9) */
        bw_put(&w, 2 + 4 * g->nc, 16);
        static const uint16_t crg[2][4][2] = {{{0, 0}, {32768, 0}, {0, 32768}, {32768, 32768}},
                                              {{32768, 0}, {0, 0}, {32768, 32768}, {0, 32768}}};
        for (uint32_t c = 0; c < g->nc; c++) {
            bw_put(&w, crg[e->prm.cfa_type][c][0], 16);
            bw_put(&w, crg[e->prm.cfa_type][c][1], 16);
        }
    }
    if (e->prm.tnlt == 1) { /* NLT, quadratic */
        bw_put(&w, 0xff16, 16);
        bw_put(&w, 5, 16);
        bw_put(&w, 1, 8);
        bw_put(&w, e->prm.nlt_sigma & 1, 1);
        bw_put(&w, e->prm.nlt_alpha & 0x7fff, 15);
    } else if (e->prm.tnlt == 2) { /* NLT, extended */
        bw_put(&w, 0xff16, 16);
        bw_put(&w, 12, 16);
        bw_put(&w, 2, 8);
        bw_put(&w, e->prm.nlt_t1 >> 16, 16);
        bw_put(&w, e->prm.nlt_t1 & 0xffff, 16);
        bw_put(&w, e->prm.nlt_t2 >> 16, 16);
        bw_put(&w, e->prm.nlt_t2 & 0xffff, 16);
        bw_put(&w, e->prm.nlt_e, 8);
    }
    bw_align(&w);
    e->hdr_len = (uint32_t)(w.bit >> 3);
}

/* Slice byte budgets (EncHandle.c:760-809). */
static int enc_slice_sizes(enc_t* e) {
    geom_t* g = &e->g;
    uint32_t hdrs = e->hdr_len + 2 + 6 * g->nslices;
    if (hdrs >= e->lcod) return E_BAD_PARAM;
    e->slice_sizes = (uint32_t*)malloc(sizeof(uint32_t) * g->nslices);
    uint32_t all = e->lcod - hdrs;
    uint32_t last_prec = g->pps - (g->nslices * g->pps - g->np);
    uint32_t min_prec = all / g->np;
    uint32_t min_slice = min_prec * g->pps;
    uint32_t last_slice = min_prec * last_prec;
    uint32_t left = all - last_slice - min_slice * (g->nslices - 1);
    if (g->nslices > 1) min_slice += (uint32_t)(((uint64_t)left * (g->nslices - 1) * g->pps / g->np) / (g->nslices - 1));
    last_slice += (uint32_t)((uint64_t)left * last_prec / g->np);
    left = all - last_slice - min_slice * (g->nslices - 1);
    uint32_t bytes_left = e->lcod - e->hdr_len;
    for (uint32_t i = 0; i < g->nslices; i++) {
        if (i != g->nslices - 1) {
            uint32_t s = min_slice + (i < left ? 1 : 0) + 6;
            e->slice_sizes[i] = s;
            bytes_left -= s;
        } else {
            e->slice_sizes[i] = bytes_left;
        }
    }
    return E_NONE;
}

/* Input scaling (linear_input_scaling_line_*_c, NltEnc.c:33-45; packed RGB
 * de-interleave, GcStageProcess.c:396-425) and the forward transform of one
 * component, then the sign-magnitude conversion into band arrays. */
typedef struct {
    enc_t* e;
    void* const* planes;
    const uint32_t* strides;
} dwt_job_t;

/* linear_input_scaling_line_{8,16}bit_c (NltEnc.c:33-72) of component c */
static void enc_scale_input(const enc_t* e, void* const* planes, const uint32_t* strides, uint32_t c, int32_t* a) {
    const comp_t* cp = &e->g.c[c];
    const uint32_t w = cp->w, h = cp->h, d = e->depth;
    const int packed = e->fmt == FMT_PACKED_RGB;
    const void* src = packed ? planes[0] : planes[c];
    const uint32_t stride = packed ? strides[0] : strides[c];
    const int32_t off = 1 << (BW - 1);
    const uint32_t sh = BW - d;
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) {
            size_t idx = packed ? (size_t)y * stride + 3 * x + c : (size_t)y * stride + x;
            uint32_t s = d <= 8 ? ((const uint8_t*)src)[idx] : (((const uint16_t*)src)[idx] & ((1u << d) - 1));
            a[(size_t)y * w + x] = (int32_t)(s << sh) - off;
        }
}

/* Forward reversible colour transform (inverse of Mct.c:137-153):
 * (R, G, B) -> (G + ((B - G + R - G) >> 2), B - G, R - G). */
static int enc_forward_rct(enc_t* e, void* const* planes, const uint32_t* strides) {
    const size_t n = (size_t)e->g.c[0].w * e->g.c[0].h;
    for (uint32_t c = 0; c < 3; c++) {
        e->rct[c] = (int32_t*)malloc(sizeof(int32_t) * n);
        if (!e->rct[c]) return E_RESOURCES;
        enc_scale_input(e, planes, strides, c, e->rct[c]);
    }
    for (size_t i = 0; i < n; i++) {
        const int32_t r = e->rct[0][i], g = e->rct[1][i], b = e->rct[2][i];
        e->rct[1][i] = b - g;
        e->rct[2][i] = r - g;
        e->rct[0][i] = g + ((b - g + r - g) >> 2);
    }
    return E_NONE;
}

static void enc_dwt_one(void* ctx, uint32_t c) {
    dwt_job_t* j = (dwt_job_t*)ctx;
    enc_t* e = j->e;
    comp_t* cp = &e->g.c[c];
    uint32_t w = cp->w, h = cp->h;
    int32_t* a = (int32_t*)malloc(sizeof(int32_t) * (size_t)w * h);
    if (e->rct[c]) {
        memcpy(a, e->rct[c], sizeof(int32_t) * (size_t)w * h);
    } else {
        enc_scale_input(e, j->planes, j->strides, c, a);
    }
    fwd_component(a, w, h, cp->dv, cp->dh);
    for (uint32_t b = 0; b < cp->nb; b++) {
        band_t* bd = &cp->b[b];
        uint16_t* o = e->coef[c][b];
        for (uint32_t y = 0; y < bd->h; y++)
            for (uint32_t x = 0; x < bd->w; x++) o[(size_t)y * bd->w + x] = to_sm(a[(size_t)(bd->y + y) * w + bd->x + x]);
        /* gc_precinct_stage_scalar_c and gc_precinct_sigflags_max_c
         * (GcStageProcess.c:22-97) */
        /* each precinct column grouped from its own first coefficient */
        for (uint32_t y = 0; y < bd->h; y++)
            for (uint32_t col = 0; col < e->g.ncol; col++) {
                const bview_t v = bview(&e->g, bd, col);
                const uint16_t* row = o + (size_t)y * bd->w + v.x0;
                uint8_t* gl = e->gcli[c][b] + (size_t)y * bd->gstride + v.g0;
                for (uint32_t gi = 0; gi < v.gw; gi++) {
                    uint16_t m = 0;
                    for (uint32_t k = gi * 4; k < MIN(gi * 4 + 4, v.w); k++) m |= row[k];
                    m = (uint16_t)(m << 1);
                    uint8_t nb = 0;
                    while (m >> nb) nb++;
                    gl[gi] = m ? (uint8_t)(nb - 1) : 0;
                }
                uint8_t* sm = e->sigmax[c][b] + (size_t)y * bd->sstride + v.s0;
                for (uint32_t s = 0; s < v.sw; s++) {
                    uint8_t mx = 0;
                    for (uint32_t k = s * 8; k < MIN(s * 8 + 8, v.gw); k++) mx = MAX(mx, gl[k]);
                    sm[s] = mx;
                }
            }
    }
    free(a);
}

/* ------------------------------------------------------------------------ */
/* Rate control for one precinct (RateControl.c).                            */
/* ------------------------------------------------------------------------ */
typedef struct {
    /* per band-line histograms (rate_control_lut_fill, RateControl.c:18-154) */
    uint32_t hist[MAXC][MAXB][2][16];
    uint32_t sighist[MAXC][MAXB][2][16];
    int partial_max[MAXC][MAXB][2]; /* max of the trailing partial significance group, -1 if none */
    /* sign handling: per band line, coefficients by the number of gtli values
     * (0, 1, ...) at which their quantized value is non-zero */
    uint32_t nzhist[MAXC][MAXB][2][17];
    uint32_t lines[MAXC][MAXB];
} prec_stats_t;

/* Vertical prediction: the precinct row above in the same slice (its
 * GCLIs and final gtli per band), NULL for a slice's first row. */
typedef struct {
    uint32_t p;               /* its precinct row */
    uint8_t gtli[MAXC][MAXB]; /* its gtli per band */
} vp_top_t;

typedef struct {
    uint8_t gtli[MAXC][MAXB];
    uint8_t sig_method[MAXC][MAXB]; /* D[p,b]: bit 1 significance, bit 0 vertical prediction */
    uint32_t data_bits[MAXC][MAXB][2], gcli_bits[MAXC][MAXB][2], sig_bits[MAXC][MAXB][2];
    uint8_t raw[MAXPK];
    uint32_t pk_data[MAXPK], pk_gcli[MAXPK], pk_sig[MAXPK], pk_sign[MAXPK];
    uint32_t total;
} prec_cost_t;

enum { SIGNS_OFF = 0, SIGNS_FAST = 1, SIGNS_FULL = 2 };

/* Number of gtli values t (from 0 up) at which a coefficient of magnitude m
 * in a group with GCLI g stays non-zero after quantization: deadzone keeps
 * m >> t (rate_control_lut_fill, RateControl.c:124-137, counts bits(m));
 * uniform keeps ((m << (g - t + 1)) - m + 2^g) >> (g + 1)
 * (rate_control_sign_coding_get_sum_nonzero_coeff_c, RateControl.c:366-455),
 * which falls as t grows. */
static uint32_t nz_levels(uint32_t m, uint32_t g, uint32_t uniform) {
    if (!m) return 0;
    if (!uniform) {
        uint32_t n = 0;
        while (m >> n) n++;
        return n;
    }
    uint32_t n = 0;
    while (n < g && (((m << (g - n + 1)) - m + (1u << g)) >> (g + 1)) != 0) n++;
    return n;
}

static void prec_stats(const enc_t* e, uint32_t p, uint32_t col, int last, prec_stats_t* st) {
    const geom_t* g = &e->g;
    memset(st, 0, sizeof(*st));
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++) {
            const band_t* bd = &g->c[c].b[b];
            const bview_t v = bview(g, bd, col);
            uint32_t lines = last ? bd->last_lines : bd->lines;
            st->lines[c][b] = lines;
            for (uint32_t l = 0; l < lines; l++) {
                uint32_t row = p * bd->lines + l;
                const uint8_t* gl = e->gcli[c][b] + (size_t)row * bd->gstride + v.g0;
                for (uint32_t i = 0; i < v.gw; i++) st->hist[c][b][l][gl[i]]++;
                const uint8_t* sm = e->sigmax[c][b] + (size_t)row * bd->sstride + v.s0;
                uint32_t full = v.gw / 8;
                for (uint32_t i = 0; i < full; i++) st->sighist[c][b][l][sm[i]]++;
                st->partial_max[c][b][l] = (full < v.sw) ? sm[full] : -1;
                if (e->prm.coding_signs_handling) {
                    const uint16_t* cf = e->coef[c][b] + (size_t)row * bd->w + v.x0;
                    for (uint32_t i = 0; i < v.w; i++)
                        st->nzhist[c][b][l][nz_levels(cf[i] & 0x7fffu, gl[i / 4], e->prm.quantization)]++;
                }
            }
        }
}

/* precinct_get_budget_bytes + rate_control_calculate_band_best_method
 * (RateControl.c:457-781) for one (quantization, refinement), no vertical
 * prediction.  With sign handling the data bits leave out the sign nibbles
 * and each packet adds a sign sub-packet: SIGNS_FAST counts every
 * coefficient of a group above gtli, SIGNS_FULL only those that stay
 * non-zero (RateControl.c:505-523). */
/* vlc_encode_get_bits (PackPrecinct.h:86-104): ones of the unary code of
 * x for the vertical prediction range (r, t). */
static uint32_t vlc_vp_bits(int32_t x, int32_t r, int32_t t) {
    int32_t mx = r - t;
    if (mx < 0) mx = 0;
    if (x > mx) return (uint32_t)(x + mx);
    x *= 2;
    return (uint32_t)(x < 0 ? -x - 1 : x);
}

/* GCLI line `cur` coded from the line above `top` (rate_control_calc_vpred_
 * cost_nosigf_c / _sigf_c, RateControl.c:290-347): the unary bits of every
 * GCLI, and the significance groups that need no code (run mode Rm: groups
 * with every GCLI <= gtli; otherwise groups predicted exactly).  Returns
 * the bits without significance; `*reduction` the bits the skipped groups
 * save; `flags` (optional) one byte per significance group. */
static uint32_t vp_line_cost(const uint8_t* cur, const uint8_t* top, uint32_t gcli_w, uint32_t sig_w, int gtli, int gtli_top,
                             int rm, uint32_t* reduction, uint8_t* flags, uint8_t* bits_out) {
    const int gmax = MAX(gtli, gtli_top);
    uint32_t total = 0, red = 0;
    for (uint32_t s2 = 0; s2 < sig_w; s2++) {
        const uint32_t i0 = s2 * 8, i1 = MIN(i0 + 8, gcli_w);
        int flag = 1;
        uint32_t grp = 0;
        for (uint32_t i = i0; i < i1; i++) {
            const int m_top = MAX((int)top[i], gmax), gv = MAX((int)cur[i], gtli);
            const uint32_t b = vlc_vp_bits(gv - m_top, m_top, gtli);
            if (bits_out) bits_out[i] = (uint8_t)b;
            grp += b + 1;
            if (rm ? ((int)cur[i] > gtli) : (m_top != gv)) flag = 0;
        }
        total += grp;
        if (flag) red += grp;
        if (flags) flags[s2] = (uint8_t)flag;
    }
    *reduction = red;
    return total;
}

static uint32_t prec_cost(const enc_t* e, const prec_stats_t* st, int last, uint8_t q, uint8_t r, prec_cost_t* pc, int smode,
                          uint32_t p, uint32_t col, const vp_top_t* top) {
    const geom_t* g = &e->g;
    const int kind = pkind(g, last, col);
    uint32_t sign_bits[MAXC][MAXB][2];
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++) {
            const band_t* bd = &g->c[c].b[b];
            uint8_t t = truncation(bd->gain, bd->prio, q, r);
            pc->gtli[c][b] = t;
            uint32_t lines = st->lines[c][b];
            if (!lines) continue;
            const bview_t v = bview(g, bd, col);
            uint32_t nosig[2], total_nosig = 0, total_sig = v.sw * lines, gsig[2];
            for (uint32_t l = 0; l < lines; l++) {
                const uint32_t* h = st->hist[c][b][l];
                uint32_t data = 0, zero = 0, above = 0;
                for (uint32_t v = 0; v <= TRUNC_MAX; v++) {
                    if (v > t) {
                        data += (v - t + 1) * h[v];
                        above += h[v];
                    } else {
                        zero += h[v];
                    }
                }
                pc->data_bits[c][b][l] = (data - (smode ? above : 0)) * 4;
                sign_bits[c][b][l] = 0;
                if (smode == SIGNS_FAST) {
                    sign_bits[c][b][l] = 4 * above;
                } else if (smode == SIGNS_FULL) {
                    for (uint32_t n = t + 1; n <= 16; n++) sign_bits[c][b][l] += st->nzhist[c][b][l][n];
                }
                nosig[l] = data + zero;
                total_nosig += nosig[l];
                uint32_t zeroed = 0;
                for (uint32_t v = 0; v <= t; v++) zeroed += st->sighist[c][b][l][v];
                zeroed *= 8;
                if (st->partial_max[c][b][l] >= 0 && (uint32_t)st->partial_max[c][b][l] <= t)
                    zeroed += v.gw - (v.gw / 8) * 8;
                gsig[l] = nosig[l] - zeroed;
                total_sig += gsig[l];
            }
            /* the cheapest coding of the band's GCLIs, a later method only
             * if strictly cheaper (RateControl.c:526-676) */
            int method = 0;
            uint32_t best = total_nosig;
            if (e->prm.coding_significance && best > total_sig) {
                method = 2;
                best = total_sig;
            }
            uint32_t vnos[2] = {0, 0}, vsig[2] = {0, 0};
            if (top) {
                uint32_t tot_vn = 0, tot_vs = 0;
                for (uint32_t l = 0; l < lines; l++) {
                    const size_t row = (size_t)(p * bd->lines + l);
                    const uint8_t* cur = e->gcli[c][b] + row * bd->gstride + v.g0;
                    const uint8_t* tl = l ? cur - bd->gstride : e->gcli[c][b] + ((size_t)top->p * bd->lines + bd->lines - 1) * bd->gstride + v.g0;
                    const int tt = l ? t : top->gtli[c][b];
                    uint32_t red = 0;
                    vnos[l] = vp_line_cost(cur, tl, v.gw, v.sw, t, tt, e->prm.coding_vertical_prediction_mode == 2,
                                           &red, NULL, NULL);
                    vsig[l] = vnos[l] - red;
                    tot_vn += vnos[l];
                    tot_vs += vsig[l] + v.sw;
                }
                if (best > tot_vn) {
                    method = 1;
                    best = tot_vn;
                }
                if (e->prm.coding_significance && best > tot_vs) {
                    method = 3;
                    best = tot_vs;
                }
            }
            pc->sig_method[c][b] = (uint8_t)method;
            for (uint32_t l = 0; l < lines; l++) {
                pc->gcli_bits[c][b][l] = method == 0 ? nosig[l] : method == 2 ? gsig[l] : method == 1 ? vnos[l] : vsig[l];
                pc->sig_bits[c][b][l] = (method & 2) ? v.sw : 0;
            }
        }
    uint32_t total = 0;
    for (uint32_t k = 0; k < g->npk; k++) {
        uint32_t db = 0, gb = 0, sb = 0, nb = 0;
        for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
            uint32_t c = g->gcomp[i], b = g->gband[i], l = g->pk[k].line;
            if (l < st->lines[c][b]) {
                db += pc->data_bits[c][b][l];
                gb += pc->gcli_bits[c][b][l];
                sb += pc->sig_bits[c][b][l];
                nb += sign_bits[c][b][l];
            }
        }
        uint32_t dB = DIV_UP(db, 8), gB = DIV_UP(gb, 8), sB = DIV_UP(sb, 8);
        pc->pk_data[k] = dB;
        pc->pk_sign[k] = DIV_UP(nb, 8);
        total += dB + pc->pk_sign[k];
        if (sB + gB > g->raw_bytes[kind][k]) {
            pc->raw[k] = 1;
            pc->pk_sig[k] = 0;
            pc->pk_gcli[k] = g->raw_bytes[kind][k];
        } else {
            pc->raw[k] = 0;
            pc->pk_sig[k] = sB;
            pc->pk_gcli[k] = gB;
        }
        total += pc->pk_sig[k] + pc->pk_gcli[k];
    }
    pc->total = total;
    return total;
}

/* binary_search_init / binary_search_next_step (BinarySearch.c:9-78). */
enum { BS_BEGIN = 0, BS_TOO_SMALL, BS_TOO_BIG, BS_OUT_OF_RANGE };
enum { BS_CONTINUE = 0, BS_FOUND, BS_ERROR };
typedef struct {
    int32_t beg, end, step, best, last;
    int below;
} bsearch_t;
static void bs_init(bsearch_t* s, uint32_t beg, uint32_t end, int below, uint32_t step) {
    s->beg = (int32_t)beg; s->end = (int32_t)end; s->below = below; s->best = -1; s->last = -1;
    s->step = step ? (int32_t)step : (s->end - s->beg) / 2;
}
static int bs_next(bsearch_t* s, int res, uint32_t* out) {
    if (res == BS_TOO_SMALL) {
        if (s->below && (s->best == -1 || s->best < s->last)) s->best = s->last;
        if (s->end >= s->last + 1) s->beg = s->last + 1;
        else {
            if (s->best == -1) return BS_ERROR;
            *out = (uint32_t)s->best;
            return BS_FOUND;
        }
    } else if (res == BS_TOO_BIG || res == BS_OUT_OF_RANGE) {
        if (res == BS_TOO_BIG && !s->below && (s->best == -1 || s->best > s->last)) s->best = s->last;
        if (s->beg <= s->last - 1) s->end = s->last - 1;
        else {
            if (s->best == -1) return BS_ERROR;
            *out = (uint32_t)s->best;
            return BS_FOUND;
        }
    }
    if (s->step > s->end - s->beg) s->step = (s->end - s->beg + 1) / 2;
    s->last = s->step + s->beg;
    *out = (uint32_t)s->last;
    return BS_CONTINUE;
}

/* rate_control_precinct (RateControl.c:1259-1333) with the binary searches of
 * RateControl.c:889-1083.  Returns 0 and fills q, r, data_bytes, headers. */
static int prec_rc(const enc_t* e, const prec_stats_t* st, int last, uint32_t budget, uint8_t* q_out, uint8_t* r_out,
                   uint32_t* data_bytes, uint32_t* hdr_bytes, prec_cost_t* pc, uint32_t p, uint32_t col, const vp_top_t* top) {
    const geom_t* g = &e->g;
    if (budget > PREC_MAX_BYTES) return E_ENC_FRAME;
    uint32_t hdr = DIV_UP(5 * 8 + g->nbands_exist * 2, 8);
    uint32_t pk_bits = g->short_hdr ? 40 : 56;
    hdr += DIV_UP(pk_bits * g->pk_exist[last], 8);
    if (budget <= hdr) return E_UNDEFINED;
    uint32_t avail = budget - hdr;
    *hdr_bytes = hdr;

    /* the quantization search counts signs the fast way; SIGNS_FULL then
     * steps from its result with exact sign counts (RateControl.c:909-1015) */
    const int smode = (int)e->prm.coding_signs_handling;
    const int sfast = smode == SIGNS_FULL ? SIGNS_FAST : smode;
    bsearch_t s;
    uint32_t step = 6;
    if (step > e->max_q) step = 0;
    bs_init(&s, 0, e->max_q, 0, step);
    int res, next = BS_BEGIN;
    uint32_t qv = 0;
    while ((res = bs_next(&s, next, &qv)) == BS_CONTINUE) {
        if (all_truncated(g, (uint8_t)qv, 0)) { next = BS_OUT_OF_RANGE; continue; }
        next = prec_cost(e, st, last, (uint8_t)qv, 0, pc, sfast, p, col, NULL) > avail ? BS_TOO_SMALL : BS_TOO_BIG;
    }
    if (res != BS_FOUND) return E_ENC_FRAME;
    uint8_t q = (uint8_t)qv;
    if (smode == SIGNS_FULL || e->prm.coding_vertical_prediction_mode) {
        /* lower quantizations while they fit, else the first higher that fits */
        int best = -1;
        for (int qt = (int)q - 1; qt >= 0; qt--) {
            if (all_truncated(g, (uint8_t)qt, 0) || prec_cost(e, st, last, (uint8_t)qt, 0, pc, smode, p, col, top) > avail) break;
            best = qt;
        }
        if (best < 0)
            for (uint32_t qt = q; qt <= e->max_q; qt++)
                if (!all_truncated(g, (uint8_t)qt, 0) && prec_cost(e, st, last, (uint8_t)qt, 0, pc, smode, p, col, top) <= avail) {
                    best = (int)qt;
                    break;
                }
        if (best < 0) return E_ENC_FRAME;
        q = (uint8_t)best;
    }

    step = 6;
    if (step >= e->max_r) step = 0;
    bs_init(&s, 0, e->max_r, 1, step);
    next = BS_BEGIN;
    uint32_t rv = 0;
    int32_t last_tested = -1;
    uint32_t last_cost = 0;
    while ((res = bs_next(&s, next, &rv)) == BS_CONTINUE) {
        last_tested = -1;
        if (all_truncated(g, q, (uint8_t)rv)) { next = BS_OUT_OF_RANGE; continue; }
        uint32_t cst = prec_cost(e, st, last, q, (uint8_t)rv, pc, smode, p, col, top);
        last_tested = (int32_t)rv;
        last_cost = cst;
        next = cst <= avail ? BS_TOO_SMALL : BS_TOO_BIG;
    }
    if (res != BS_FOUND) return E_ENC_FRAME;
    (void)last_tested;
    (void)last_cost;
    /* The pack step needs the per-packet decisions of the chosen pair. */
    *data_bytes = prec_cost(e, st, last, q, (uint8_t)rv, pc, smode, p, col, top);
    *q_out = q;
    *r_out = (uint8_t)rv;
    return E_NONE;
}

/* quant_deadzone_c / quant_uniform_c (Source/Lib/Encoder/Codec/Quant.c:9-45)
 * applied to one coefficient of a group with GCLI gcli; only called with
 * gtli > 0 (QuantStageProcess.c:18-31 skips gtli == 0). */
static inline uint16_t quantize(uint16_t v, uint8_t gcli, uint8_t t, uint32_t uniform) {
    if (gcli <= t) return 0;
    uint16_t sign = v & 0x8000, m = v & 0x7fff;
    if (uniform) {
        uint8_t s = gcli - t + 1;
        m = (uint16_t)(((uint32_t)(m << s) - m + (1u << gcli)) >> (gcli + 1));
        m = (uint16_t)(m << t);
    } else {
        m = (uint16_t)((m >> t) << t);
    }
    return m ? (uint16_t)(m | sign) : 0;
}

/* pack_precinct (Source/Lib/Encoder/Codec/PackPrecinct.c:235-572).  `top`
 * is the row above for vertically predicted bands.  With sign handling the data sub-packet carries no sign
 * nibbles and a sign sub-packet follows it: one bit per non-zero quantized
 * coefficient of the groups above gtli (pack_sign_c, :200-233).  Returns
 * non-zero when a sign sub-packet differs from the size the rate control
 * computed. */
static int prec_pack(const enc_t* e, uint32_t p, uint32_t col, int last, const prec_cost_t* pc, uint8_t q, uint8_t r,
                     uint32_t total_bytes, bw_t* w, const vp_top_t* top) {
    const geom_t* g = &e->g;
    uint32_t hdr_len = DIV_UP(5 * 8 + 2 * g->nbands_exist, 8);
    bw_put(w, total_bytes - hdr_len, 24);
    bw_put(w, q, 8);
    bw_put(w, r, 8);
    for (uint32_t i = 0; i < g->nbands_all; i++) {
        if (g->gband[i] == NOBAND) continue;
        uint32_t c = g->gcomp[i], b = g->gband[i];
        uint32_t lines = last ? g->c[c].b[b].last_lines : g->c[c].b[b].lines;
        bw_put(w, lines > 0 ? pc->sig_method[c][b] : 0, 2);
    }
    bw_align(w);
    const uint32_t uniform = e->prm.quantization;
    const int signs_sep = e->prm.coding_signs_handling != 0;
    uint16_t qbuf[4];
    for (uint32_t k = 0; k < g->npk; k++) {
        const uint32_t l = g->pk[k].line;
        int present = 0;
        for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
            const band_t* bd = &g->c[g->gcomp[i]].b[g->gband[i]];
            if (l < (last ? bd->last_lines : bd->lines)) { present = 1; break; }
        }
        if (!present) continue;
        /* write_packet_header, PackHeaders.c:98-127 */
        if (g->short_hdr) {
            bw_put(w, pc->raw[k], 1);
            bw_put(w, pc->pk_data[k], 15);
            bw_put(w, pc->pk_gcli[k], 13);
            bw_put(w, pc->pk_sign[k], 11);
        } else {
            bw_put(w, pc->raw[k], 1);
            bw_put(w, pc->pk_data[k], 20);
            bw_put(w, pc->pk_gcli[k], 20);
            bw_put(w, pc->pk_sign[k], 15);
        }
        if (pc->raw[k]) {
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                uint32_t c = g->gcomp[i], b = g->gband[i];
                const band_t* bd = &g->c[c].b[b];
                if (l >= (last ? bd->last_lines : bd->lines)) continue;
                const bview_t v = bview(g, bd, col);
                const uint8_t* gl = e->gcli[c][b] + (size_t)(p * bd->lines + l) * bd->gstride + v.g0;
                for (uint32_t x = 0; x < v.gw; x++) bw_put(w, gl[x], 4);
            }
            bw_align(w);
        } else {
            /* vertical prediction of a line: its codes and flags
             * (pack_bitplane_count_vpred_*, PackPrecinct.c:47-74) */
            uint8_t vbits[MAXGB][2048], vflags[MAXGB][256];
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                uint32_t c = g->gcomp[i], b = g->gband[i];
                const band_t* bd = &g->c[c].b[b];
                if (l >= (last ? bd->last_lines : bd->lines) || !(pc->sig_method[c][b] & 1)) continue;
                const bview_t v = bview(g, bd, col);
                if (v.gw > 2048 || v.sw > 256) return E_RESOURCES;
                const size_t row = (size_t)(p * bd->lines + l);
                const uint8_t* cur = e->gcli[c][b] + row * bd->gstride + v.g0;
                const uint8_t* tl = l ? cur - bd->gstride : e->gcli[c][b] + ((size_t)top->p * bd->lines + bd->lines - 1) * bd->gstride + v.g0;
                uint32_t red;
                vp_line_cost(cur, tl, v.gw, v.sw, pc->gtli[c][b], l ? pc->gtli[c][b] : top->gtli[c][b],
                             e->prm.coding_vertical_prediction_mode == 2, &red, vflags[i - g->pk[k].bs], vbits[i - g->pk[k].bs]);
            }
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                uint32_t c = g->gcomp[i], b = g->gband[i];
                const band_t* bd = &g->c[c].b[b];
                if (l >= (last ? bd->last_lines : bd->lines) || !(pc->sig_method[c][b] & 2)) continue;
                const bview_t v = bview(g, bd, col);
                const uint8_t* sm = e->sigmax[c][b] + (size_t)(p * bd->lines + l) * bd->sstride + v.s0;
                for (uint32_t s = 0; s < v.sw; s++)
                    bw_put(w, (pc->sig_method[c][b] & 1) ? vflags[i - g->pk[k].bs][s] : sm[s] <= pc->gtli[c][b], 1);
            }
            bw_align(w);
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                uint32_t c = g->gcomp[i], b = g->gband[i];
                const band_t* bd = &g->c[c].b[b];
                if (l >= (last ? bd->last_lines : bd->lines)) continue;
                const uint8_t t = pc->gtli[c][b];
                const uint8_t meth = pc->sig_method[c][b];
                const bview_t v = bview(g, bd, col);
                const uint8_t* gl = e->gcli[c][b] + (size_t)(p * bd->lines + l) * bd->gstride + v.g0;
                const uint8_t* sm = e->sigmax[c][b] + (size_t)(p * bd->lines + l) * bd->sstride + v.s0;
                for (uint32_t x = 0; x < v.gw; x++) {
                    uint32_t n;
                    if (meth & 1) {
                        if ((meth & 2) && vflags[i - g->pk[k].bs][x / 8]) continue;
                        n = vbits[i - g->pk[k].bs][x];
                    } else {
                        if ((meth & 2) && sm[x / 8] <= t) continue;
                        n = gl[x] > t ? (uint32_t)(gl[x] - t) : 0;
                    }
                    /* unary: n ones then a zero (vlc_encode_pack_bits, PackPrecinct.h:25-39) */
                    bw_put(w, (uint32_t)(((1ull << n) - 1) << 1), n + 1);
                }
            }
            bw_align(w);
        }
        /* data sub-packet: pack_data_c (PackPrecinct.c:128-198) */
        for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
            uint32_t c = g->gcomp[i], b = g->gband[i];
            const band_t* bd = &g->c[c].b[b];
            if (l >= (last ? bd->last_lines : bd->lines)) continue;
            const uint8_t t = pc->gtli[c][b];
            const size_t row = (size_t)(p * bd->lines + l);
            const bview_t v = bview(g, bd, col);
            const uint8_t* gl = e->gcli[c][b] + row * bd->gstride + v.g0;
            const uint16_t* cf = e->coef[c][b] + row * bd->w + v.x0;
            for (uint32_t x = 0; x < v.gw; x++) {
                if (gl[x] <= t) continue;
                for (uint32_t k2 = 0; k2 < 4; k2++) {
                    uint32_t xi = x * 4 + k2;
                    uint16_t cv = xi < v.w ? cf[xi] : 0;
                    qbuf[k2] = t ? quantize(cv, gl[x], t, uniform) : cv;
                }
                uint32_t signs = 0;
                for (uint32_t k2 = 0; k2 < 4; k2++) signs = (signs << 1) | (qbuf[k2] >> 15);
                if (!signs_sep) bw_put(w, signs, 4);
                for (int bit = gl[x] - 1; bit >= t; bit--) {
                    uint32_t nib = 0;
                    for (uint32_t k2 = 0; k2 < 4; k2++) nib = (nib << 1) | ((qbuf[k2] >> bit) & 1u);
                    bw_put(w, nib, 4);
                }
            }
        }
        bw_align(w);
        if (!signs_sep) continue;
        /* sign sub-packet: pack_sign_c (PackPrecinct.c:200-233) */
        uint32_t nbits = 0;
        for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
            uint32_t c = g->gcomp[i], b = g->gband[i];
            const band_t* bd = &g->c[c].b[b];
            if (l >= (last ? bd->last_lines : bd->lines)) continue;
            const uint8_t t = pc->gtli[c][b];
            const size_t row = (size_t)(p * bd->lines + l);
            const bview_t v = bview(g, bd, col);
            const uint8_t* gl = e->gcli[c][b] + row * bd->gstride + v.g0;
            const uint16_t* cf = e->coef[c][b] + row * bd->w + v.x0;
            for (uint32_t xi = 0; xi < v.w; xi++) {
                const uint8_t gv = gl[xi / 4];
                if (gv <= t) continue;
                const uint16_t qv = t ? quantize(cf[xi], gv, t, uniform) : cf[xi];
                if (qv) {
                    bw_put(w, qv >> 15, 1);
                    nbits++;
                }
            }
        }
        bw_align(w);
        if (DIV_UP(nbits, 8) != pc->pk_sign[k]) return E_ENC_FRAME;
    }
    return E_NONE;
}

typedef struct {
    enc_t* e;
} slice_job_t;

/* Precinct header + packet header bytes (rate_control_get_headers_bytes,
 * RateControl.c:258-272). */
static uint32_t prec_hdr_bytes(const geom_t* g, int last) {
    return DIV_UP(5 * 8 + g->nbands_exist * 2, 8) + DIV_UP((g->short_hdr ? 40 : 56) * g->pk_exist[last], 8);
}

/* RC modes 2 and 3, per-slice common quantization: the budget of each
 * precinct of the slice (process_slice, PackStageProcess.c:339-483;
 * rate_control_slice_quantization_fast_no_vpred_no_sign_full,
 * RateControl.c:1336-1425, with its binary searches :1086-1209).  One
 * (Q, R) for the whole slice by the same searches as a precinct's, on the
 * summed data bytes; the last precinct takes the remaining bytes; mode 3
 * raises every precinct to a quarter of the largest; then 10 % of the first
 * precinct's budget and an even share of what is left move out of the last
 * precinct's padding. */
static int slice_common_budgets(const enc_t* e, uint32_t first_p, uint32_t nprec, uint32_t slice_budget, uint32_t* total) {
    const geom_t* g = &e->g;
    if (DIV_UP(slice_budget, nprec) > PREC_MAX_BYTES) return E_ENC_FRAME;
    prec_stats_t* st = (prec_stats_t*)malloc(sizeof(prec_stats_t) * nprec);
    prec_cost_t pc;
    /* signs counted the fast way for the whole slice (RateControl.c:1341-1343) */
    const int sfast = e->prm.coding_signs_handling ? SIGNS_FAST : SIGNS_OFF;
    if (!st) return E_RESOURCES;
    uint32_t headers = 0;
    /* precinct i of the slice: row first_p + i / ncol, column i % ncol */
#define PREC_ROW(i) (first_p + (i) / g->ncol)
#define PREC_COL(i) ((i) % g->ncol)
#define PREC_LAST(i) (PREC_ROW(i) + 1 >= g->np)
    for (uint32_t i = 0; i < nprec; i++) {
        prec_stats(e, PREC_ROW(i), PREC_COL(i), PREC_LAST(i), &st[i]);
        total[i] = prec_hdr_bytes(g, PREC_LAST(i));
        headers += total[i];
    }
    if (slice_budget <= headers) {
        free(st);
        return E_UNDEFINED;
    }
    const uint32_t avail = slice_budget - headers;
    bsearch_t s;
    uint32_t step = 6;
    if (step > e->max_q) step = 0;
    bs_init(&s, 0, e->max_q, 0, step);
    int res, next = BS_BEGIN;
    uint32_t qv = 0;
    while ((res = bs_next(&s, next, &qv)) == BS_CONTINUE) {
        if (all_truncated(g, (uint8_t)qv, 0)) { next = BS_OUT_OF_RANGE; continue; }
        uint32_t sum = 0;
        for (uint32_t i = 0; i < nprec; i++) sum += prec_cost(e, &st[i], PREC_LAST(i), (uint8_t)qv, 0, &pc, sfast, PREC_ROW(i), PREC_COL(i), NULL);
        next = sum > avail ? BS_TOO_SMALL : BS_TOO_BIG;
    }
    if (res != BS_FOUND) {
        free(st);
        return E_ENC_FRAME;
    }
    const uint8_t q = (uint8_t)qv;
    step = 6;
    if (step >= e->max_r) step = 0;
    bs_init(&s, 0, e->max_r, 1, step);
    next = BS_BEGIN;
    uint32_t rv = 0;
    while ((res = bs_next(&s, next, &rv)) == BS_CONTINUE) {
        if (all_truncated(g, q, (uint8_t)rv)) { next = BS_OUT_OF_RANGE; continue; }
        uint32_t sum = 0;
        for (uint32_t i = 0; i < nprec; i++) sum += prec_cost(e, &st[i], PREC_LAST(i), q, (uint8_t)rv, &pc, sfast, PREC_ROW(i), PREC_COL(i), NULL);
        next = sum <= avail ? BS_TOO_SMALL : BS_TOO_BIG;
    }
    if (res != BS_FOUND) {
        free(st);
        return E_ENC_FRAME;
    }
    uint32_t pad_last = avail;
    for (uint32_t i = 0; i < nprec; i++) {
        const uint32_t d = prec_cost(e, &st[i], PREC_LAST(i), q, (uint8_t)rv, &pc, sfast, PREC_ROW(i), PREC_COL(i), NULL);
        pad_last -= d;
        total[i] += d;
    }
    free(st);
    total[nprec - 1] += pad_last;
    if (e->prm.rate_control_mode == 3) {
        /* RC_CBR_PER_SLICE_COMMON_QUANT_MAX_RATE: no precinct below a quarter
         * of the largest (padding excluded) */
        uint32_t max_size = 0;
        for (uint32_t i = 0; i < nprec; i++) {
            const uint32_t ds = total[i] - (i + 1 == nprec ? pad_last : 0);
            if (ds > max_size) max_size = ds;
        }
        const uint32_t min_size = max_size / 4;
        uint32_t need = 0;
        for (uint32_t i = 0; i < nprec; i++) {
            const uint32_t ds = total[i] - (i + 1 == nprec ? pad_last : 0);
            if (ds < min_size) {
                total[i] += min_size - ds;
                need += min_size - ds;
            }
        }
        if (need) {
            if (pad_last >= need) {
                pad_last -= need;
                total[nprec - 1] -= need;
            } else {
                need -= pad_last;
                total[nprec - 1] -= pad_last;
                pad_last = 0;
                while (need)
                    for (uint32_t i = 0; i < nprec && need; i++) {
                        need--;
                        total[i]--;
                    }
            }
        }
    }
    if (pad_last > 0) {
        /* 20 % with fast signs, else 10 % (PackStageProcess.c:34-35, 432-446) */
        uint32_t add_first = total[0] * (e->prm.coding_signs_handling == SIGNS_FAST ? 20 : 10) / 100;
        if (add_first > pad_last) add_first = pad_last;
        pad_last -= add_first;
        total[nprec - 1] -= add_first;
        total[0] += add_first;
        if (pad_last) {
            total[nprec - 1] -= pad_last;
            const uint32_t each = pad_last / nprec, extra = pad_last - each * nprec;
            for (uint32_t i = 0; i < nprec; i++) total[i] += each + (i < extra ? 1 : 0);
        }
    }
    return E_NONE;
}
#undef PREC_ROW
#undef PREC_COL
#undef PREC_LAST

/* pack_stage_kernel (PackStageProcess.c:567-749): RC modes 0 and 1
 * (process_precinct :274-338) split the slice evenly (mode 1: the first
 * precinct 10 % more); modes 2 and 3 (process_slice :339-565) split it by a
 * slice-wide quantization.  Then each precinct's own search, with padding
 * moved to the next precinct in modes 1-3. */
static void enc_slice(void* ctx, uint32_t s) {
    enc_t* e = ((slice_job_t*)ctx)->e;
    const geom_t* g = &e->g;
    uint32_t begin = e->hdr_len;
    for (uint32_t i = 0; i < s; i++) begin += e->slice_sizes[i];
    const int last_slice = s == g->nslices - 1;
    uint32_t slice_budget = e->slice_sizes[s] - 6 - (last_slice ? 2 : 0);
    uint32_t first_p = g->pps * s; /* first precinct row */
    /* precincts of the slice: rows x columns, row after row */
    uint32_t nprec = (last_slice ? g->np - first_p : g->pps) * g->ncol;
    uint32_t min_b = slice_budget / nprec;
    uint32_t left = slice_budget - min_b * nprec;
    uint32_t first_b = min_b;
    if (e->prm.rate_control_mode == 1) {
        /* 20 % more with fast signs, else 10 % (PackStageProcess.c:34-35, 614-622) */
        first_b = first_b * (e->prm.coding_signs_handling == SIGNS_FAST ? 120 : 110) / 100;
        first_b = MIN(slice_budget, first_b);
        if (nprec > 1) {
            min_b = (slice_budget - first_b) / (nprec - 1);
            left = slice_budget - min_b * (nprec - 1) - first_b;
        } else {
            left = 0;
        }
    }
    uint32_t* common = NULL;
    if (e->prm.rate_control_mode >= 2) {
        common = (uint32_t*)malloc(sizeof(uint32_t) * nprec);
        int err = common ? slice_common_budgets(e, first_p, nprec, slice_budget, common) : E_RESOURCES;
        if (err) {
            free(common);
            e->slice_err = err;
            return;
        }
    }
    bw_t w = {e->out + begin, 0};
    uint32_t carry = 0;
    prec_stats_t st;
    prec_cost_t pc;
    /* vertical prediction: the precinct above in the slice (same column),
     * with its final gtli */
    vp_top_t* tops = (vp_top_t*)malloc(sizeof(vp_top_t) * g->ncol);
    if (!tops) {
        free(common);
        e->slice_err = E_RESOURCES;
        return;
    }
    for (uint32_t i = 0; i < nprec; i++) {
        const uint32_t p = first_p + i / g->ncol, col = i % g->ncol;
        int last = (p + 1 >= g->np);
        const vp_top_t* top = (e->prm.coding_vertical_prediction_mode && i >= g->ncol) ? &tops[col] : NULL;
        uint32_t budget = (common ? common[i] : (i == 0 ? first_b : min_b) + (i < left ? 1 : 0)) + carry;
        prec_stats(e, p, col, last, &st);
        uint8_t q = 0, r = 0;
        uint32_t data = 0, hdr = 0;
        int err = prec_rc(e, &st, last, budget, &q, &r, &data, &hdr, &pc, p, col, top);
        if (err) {
            free(common);
            free(tops);
            e->slice_err = err;
            return;
        }
        uint32_t padding = budget - hdr - data;
        uint32_t total = budget;
        /* fast signs: the sign sub-packets shrink to the signs actually sent;
         * the bytes they free (PackPrecinct.c:513-536) are cut from the
         * precinct with its padding, or left as padding in the slice's last
         * precinct and in mode 0 (PackStageProcess.c:293-333) */
        uint32_t retrieve = 0;
        if (e->prm.coding_signs_handling == SIGNS_FAST) {
            retrieve = data - prec_cost(e, &st, last, q, r, &pc, SIGNS_FULL, p, col, top);
        }
        /* modes 1-3 move a precinct's padding to the next one */
        if (e->prm.rate_control_mode >= 1 && i + 1 < nprec) {
            total -= padding + retrieve;
            carry = padding + retrieve;
            padding = 0;
        }
        if (e->q_out) e->q_out[p * g->ncol + col] = q;
        if (e->r_out) e->r_out[p * g->ncol + col] = r;
        if (i == 0) { /* write_slice_header, PackHeaders.c:91-96 */
            bw_put(&w, 0xff20, 16);
            bw_put(&w, 4, 16);
            bw_put(&w, s, 16);
        }
        uint64_t start = w.bit;
        if (prec_pack(e, p, col, last, &pc, q, r, total, &w, top) || ((w.bit - start) >> 3) != hdr + data - retrieve) {
            free(common);
            free(tops);
            e->slice_err = E_ENC_FRAME;
            return;
        }
        if (e->prm.coding_vertical_prediction_mode) {
            tops[col].p = p;
            memcpy(tops[col].gtli, pc.gtli, sizeof(tops[col].gtli));
        }
        uint64_t used = (w.bit - start) >> 3;
        for (uint64_t z = used; z < total; z++) bw_put(&w, 0, 8);
    }
    if (last_slice) bw_put(&w, 0xff11, 16); /* EOC */
    free(common);
    free(tops);
}

static void enc_free(enc_t* e) {
    for (int c = 0; c < MAXC; c++) {
        for (int b = 0; b < MAXB; b++) {
            free(e->coef[c][b]);
            free(e->gcli[c][b]);
            free(e->sigmax[c][b]);
        }
        free(e->rct[c]);
    }
    free(e->slice_sizes);
}

static int enc_alloc(enc_t* e) {
    for (uint32_t c = 0; c < e->g.nc; c++)
        for (uint32_t b = 0; b < e->g.c[c].nb; b++) {
            band_t* bd = &e->g.c[c].b[b];
            e->coef[c][b] = (uint16_t*)malloc(sizeof(uint16_t) * (size_t)bd->w * bd->h);
            e->gcli[c][b] = (uint8_t*)malloc((size_t)bd->gstride * bd->h);
            e->sigmax[c][b] = (uint8_t*)malloc((size_t)bd->sstride * bd->h);
            if (!e->coef[c][b] || !e->gcli[c][b] || !e->sigmax[c][b]) return E_RESOURCES;
        }
    return E_NONE;
}

int or_frame_size(const or_enc_params_t* p, uint32_t* bytes_per_frame) {
    enc_t e;
    memset(&e, 0, sizeof(e));
    int r = enc_configure(&e, p);
    if (r) return r;
    *bytes_per_frame = e.lcod;
    return 0;
}

int or_encode(const or_enc_params_t* p, void* const planes[4], const uint32_t strides[4], uint8_t* out, uint32_t out_cap,
              uint32_t* out_size, uint8_t* q_out, uint8_t* r_out) {
    enc_t e;
    memset(&e, 0, sizeof(e));
    int r = enc_configure(&e, p);
    if (r) return r;
    if (out_cap < e.lcod || !out) return E_BAD_PARAM;
    enc_write_header(&e);
    r = enc_slice_sizes(&e);
    if (r) { enc_free(&e); return r; }
    r = enc_alloc(&e);
    if (r) { enc_free(&e); return r; }
    uint32_t threads = p->threads_num ? p->threads_num : 1;
    if (e.prm.cpih == 1) {
        r = enc_forward_rct(&e, planes, strides);
        if (r) { enc_free(&e); return r; }
    }
    dwt_job_t dj = {&e, planes, strides};
    parallel_for(e.g.nc, threads, enc_dwt_one, &dj);
    memcpy(out, e.hdr, e.hdr_len);
    e.out = out;
    e.q_out = q_out;
    e.r_out = r_out;
    slice_job_t sj = {&e};
    parallel_for(e.g.nslices, threads, enc_slice, &sj);
    r = e.slice_err ? E_ENC_FRAME : E_NONE;
    *out_size = e.lcod;
    enc_free(&e);
    return r;
}

int64_t or_forward_dwt(const or_enc_params_t* p, void* const planes[4], const uint32_t strides[4], uint16_t* out,
                       uint64_t out_cap) {
    enc_t e;
    memset(&e, 0, sizeof(e));
    int r = enc_configure(&e, p);
    if (r) return r;
    r = enc_alloc(&e);
    if (r) { enc_free(&e); return -1; }
    dwt_job_t dj = {&e, planes, strides};
    parallel_for(e.g.nc, p->threads_num ? p->threads_num : 1, enc_dwt_one, &dj);
    uint64_t n = 0;
    for (uint32_t c = 0; c < e.g.nc; c++)
        for (uint32_t b = 0; b < e.g.c[c].nb; b++) {
            uint64_t cnt = (uint64_t)e.g.c[c].b[b].w * e.g.c[c].b[b].h;
            if (n + cnt > out_cap) { enc_free(&e); return -1; }
            memcpy(out + n, e.coef[c][b], cnt * sizeof(uint16_t));
            n += cnt;
        }
    enc_free(&e);
    return (int64_t)n;
}

/* ------------------------------------------------------------------------ */
/* Decoder                                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    const uint8_t* mem;
    uint32_t size;
    uint64_t bit;
} br_t;
static inline int br_enough(const br_t* r, uint32_t bytes) { return ((r->bit + 7) >> 3) + bytes <= r->size; }
static inline uint32_t br_get(br_t* r, uint32_t n) {
    uint32_t v = 0;
    for (uint32_t i = 0; i < n; i++) {
        uint64_t byte = r->bit >> 3;
        uint32_t bit = byte < r->size ? (r->mem[byte] >> (7 - (r->bit & 7))) & 1u : 0u;
        v = (v << 1) | bit;
        r->bit++;
    }
    return v;
}
static inline void br_align(br_t* r) { r->bit = (r->bit + 7) & ~(uint64_t)7; }

typedef struct {
    geom_t g;
    uint32_t lcod, depth[MAXC], qpih, fs, rm, bw, fq, lh, rl, nc, cpih, tnlt;
    uint32_t nlt_sigma, nlt_alpha, nlt_t1, nlt_t2, nlt_e; /* non-linearity parameters (NLT marker) */
    uint32_t cts, cf, e1, e2, crg, xcrg[MAXC], ycrg[MAXC]; /* Star-Tetrix: CTS and CRG markers */
    uint32_t hdr_len;
    uint8_t gain[MAXGB], prio[MAXGB];
} dec_hdr_t;

/* get_header and its marker readers (Source/Lib/Decoder/Codec/ParseHeader.c:
 * 20-617). */
static int dec_parse_header(const uint8_t* bs, uint32_t size, dec_hdr_t* h) {
    memset(h, 0, sizeof(*h));
    br_t r = {bs, size, 0};
    if (!br_enough(&r, 2)) return E_DEC_SHORT;
    if (br_get(&r, 16) != 0xff10) return E_DEC_BITSTREAM;
    if (!br_enough(&r, 4)) return E_DEC_SHORT;
    if (br_get(&r, 16) != 0xff50) return E_DEC_BITSTREAM;
    uint32_t lcap = br_get(&r, 16) - 2;
    if (lcap * 8 > 16) return E_DEC_BITSTREAM;
    if (!br_enough(&r, lcap)) return E_DEC_SHORT;
    r.bit += lcap * 8;
    if (!br_enough(&r, 28)) return E_DEC_SHORT;
    if (br_get(&r, 16) != 0xff12) return E_DEC_BITSTREAM;
    if (br_get(&r, 16) != 26) return E_DEC_BITSTREAM;
    h->lcod = br_get(&r, 32);
    br_get(&r, 16);
    br_get(&r, 16);
    uint32_t W = br_get(&r, 16), H = br_get(&r, 16), cw = br_get(&r, 16), hsl = br_get(&r, 16);
    if (hsl < 1) return E_DEC_BITSTREAM;
    uint32_t nc = br_get(&r, 8);
    if (nc < 1 || nc > 8) return E_DEC_BITSTREAM;
    if (br_get(&r, 8) != 4) return E_DEC_BITSTREAM;
    if (br_get(&r, 8) != 8) return E_DEC_BITSTREAM;
    h->bw = br_get(&r, 8);
    h->fq = br_get(&r, 4);
    uint32_t br = br_get(&r, 4);
    if (!(h->fq == 0 || (h->bw == 18 && h->fq == 6) || (h->bw == 20 && h->fq == 8))) return E_DEC_BITSTREAM;
    if (br != 4) return E_DEC_BITSTREAM;
    if (br_get(&r, 1) != 0) return E_DEC_BITSTREAM; /* Fslc */
    if (br_get(&r, 3) != 0) return E_DEC_BITSTREAM; /* Ppoc */
    h->cpih = br_get(&r, 4);
    if (h->cpih != 0 && h->cpih != 1 && h->cpih != 3) return E_DEC_BITSTREAM;
    uint32_t dh = br_get(&r, 4), dv = br_get(&r, 4);
    h->lh = br_get(&r, 1);
    h->rl = br_get(&r, 1);
    h->qpih = br_get(&r, 2);
    h->fs = br_get(&r, 2);
    h->rm = br_get(&r, 2);
    if (h->qpih > 1 || h->fs > 1 || h->rm > 1) return E_DEC_BITSTREAM;
    uint32_t sx[MAXC] = {1, 1, 1, 1}, sy[MAXC] = {1, 1, 1, 1}, sd = 0;
    int have_cdt = 0, have_wgt = 0;
    uint32_t nwgt = 0;
    for (;;) {
        if (!br_enough(&r, 2)) return E_DEC_SHORT;
        uint32_t m = br_get(&r, 16);
        if (m == 0xff13) {
            if (have_cdt) return E_DEC_BITSTREAM;
            have_cdt = 1;
            if (!br_enough(&r, nc * 2 + 2)) return E_DEC_SHORT;
            if (br_get(&r, 16) - 2 != 2 * nc) return E_DEC_BITSTREAM;
            if (nc > MAXC) return E_DEC_BITSTREAM;
            for (uint32_t c = 0; c < nc; c++) {
                h->depth[c] = br_get(&r, 8);
                if (h->depth[c] < 8 || h->depth[c] > 16) return E_DEC_BITSTREAM;
                sx[c] = br_get(&r, 4);
                sy[c] = br_get(&r, 4);
            }
        } else if (m == 0xff14) {
            if (have_wgt) return E_DEC_BITSTREAM;
            have_wgt = 1;
            if (!br_enough(&r, 2)) return E_DEC_SHORT;
            uint32_t len = (br_get(&r, 16) - 2) & 0xffff;
            if (len & 1) return E_DEC_SHORT;
            nwgt = len / 2;
            if (nwgt > MAXGB) return E_DEC_BITSTREAM;
            if (!br_enough(&r, len)) return E_DEC_SHORT;
            for (uint32_t i = 0; i < nwgt; i++) {
                h->gain[i] = (uint8_t)br_get(&r, 8);
                h->prio[i] = (uint8_t)br_get(&r, 8);
            }
        } else if (m == 0xff16) { /* NLT, get_nonlinearity (ParseHeader.c:373-405) */
            if (!br_enough(&r, 3)) return E_DEC_SHORT;
            br_get(&r, 16);
            h->tnlt = br_get(&r, 8);
            if (h->tnlt == 1) {
                if (!br_enough(&r, 2)) return E_DEC_SHORT;
                h->nlt_sigma = br_get(&r, 1);
                h->nlt_alpha = br_get(&r, 15);
            } else if (h->tnlt == 2) {
                if (!br_enough(&r, 9)) return E_DEC_SHORT;
                h->nlt_t1 = br_get(&r, 32);
                h->nlt_t2 = br_get(&r, 32);
                h->nlt_e = br_get(&r, 8);
            } else {
                return E_DEC_BITSTREAM;
            }
        } else if (m == 0xff17) { /* CWD */
            if (!br_enough(&r, 3)) return E_DEC_SHORT;
            if (br_get(&r, 16) != 3) return E_DEC_BITSTREAM;
            sd = br_get(&r, 8);
        } else if (m == 0xff18) { /* CTS, get_cts (ParseHeader.c:418-446) */
            if (h->cts) return E_DEC_BITSTREAM;
            h->cts = 1;
            if (!br_enough(&r, 4)) return E_DEC_SHORT;
            if (br_get(&r, 16) != 4) return E_DEC_BITSTREAM;
            br_get(&r, 4);
            h->cf = br_get(&r, 4);
            h->e1 = br_get(&r, 4);
            h->e2 = br_get(&r, 4);
        } else if (m == 0xff19) { /* CRG, get_crg (ParseHeader.c:448-480) */
            if (h->crg) return E_DEC_BITSTREAM;
            h->crg = 1;
            if (!br_enough(&r, 2 + nc * 4)) return E_DEC_SHORT;
            if (br_get(&r, 16) != 2 + nc * 4 || nc > MAXC) return E_DEC_BITSTREAM;
            for (uint32_t c = 0; c < nc; c++) {
                h->xcrg[c] = br_get(&r, 16);
                h->ycrg[c] = br_get(&r, 16);
            }
        } else if (m == 0xff15) { /* COM */
            if (!br_enough(&r, 4)) return E_DEC_SHORT;
            uint32_t len = br_get(&r, 16);
            br_get(&r, 16);
            len -= 4;
            if (!br_enough(&r, len)) return E_DEC_SHORT;
            r.bit += (uint64_t)len * 8;
        } else if (m == 0xff20) {
            r.bit -= 16;
            break;
        } else {
            return E_DEC_BITSTREAM;
        }
    }
    if (!have_cdt || !have_wgt) return E_DEC_BITSTREAM;
    if (h->cpih == 3 && (!h->cts || !h->crg || nc != 4)) return E_DEC_BITSTREAM;
    if (h->cpih) /* the colour transform needs equal sampling (ParseHeader.c:584-594) */
        for (uint32_t c = 1; c < nc; c++)
            if (sx[c] != sx[0] || sy[c] != sy[0]) return E_DEC_BITSTREAM;
    int e = geom_compute(&h->g, 0, nc, W, H, dh, dv, sd, sx, sy, hsl * (1u << dv), cw);
    if (e) return e;
    /* copy_weights_table, Decoder.c:35-50 */
    uint32_t k = 0;
    for (uint32_t i = 0; i < h->g.nbands_all; i++) {
        if (h->g.gband[i] == NOBAND) continue;
        band_t* bd = &h->g.c[h->g.gcomp[i]].b[h->g.gband[i]];
        bd->gain = h->gain[k];
        bd->prio = h->prio[k];
        k++;
    }
    h->nc = nc;
    h->hdr_len = (uint32_t)(r.bit >> 3);
    return E_NONE;
}

static int dec_format(const geom_t* g) {
    /* svt_jpeg_xs_get_format_from_params, Decoder.c:52-79 */
    if (g->nc == 3) {
        const comp_t* c = g->c;
        if (c[0].sx == 1 && c[1].sx == 1 && c[2].sx == 1 && c[0].sy == 1 && c[1].sy == 1 && c[2].sy == 1) return FMT_YUV444;
        if (c[0].sx == 1 && c[1].sx == 2 && c[2].sx == 2 && c[0].sy == 1 && c[1].sy == 1 && c[2].sy == 1) return FMT_YUV422;
        if (c[0].sx == 1 && c[1].sx == 2 && c[2].sx == 2 && c[0].sy == 1 && c[1].sy == 2 && c[2].sy == 2) return FMT_YUV420;
        return 0;
    }
    if (g->nc == 4) return FMT_4COMP;
    if (g->nc == 1) return FMT_GRAY;
    return 0;
}

int or_probe(const uint8_t* bs, uint32_t size, or_image_info_t* info) {
    if (!bs || !size) return E_DEC_PTR;
    dec_hdr_t h;
    int e = dec_parse_header(bs, size, &h);
    if (e) return e;
    memset(info, 0, sizeof(*info));
    info->width = h.g.W;
    info->height = h.g.H;
    info->bit_depth = h.depth[0];
    info->comps = h.g.nc;
    info->format = (uint32_t)dec_format(&h.g);
    info->lcod = h.lcod;
    for (uint32_t c = 0; c < h.g.nc; c++) {
        info->comp_w[c] = h.g.c[c].w;
        info->comp_h[c] = h.g.c[c].h;
    }
    return info->format ? 0 : E_DEC_BITSTREAM;
}

typedef struct {
    dec_hdr_t* h;
    int32_t* mct[MAXC]; /* Cpih != 0: each component after the inverse transform */
    const uint8_t* bs;
    uint32_t size;
    uint32_t* slice_off;
    int16_t* coef[MAXC][MAXB];
    int err;
} dec_t;

/* Decoded GCLIs of one precinct row: for each band, up to 4 lines of
 * gcli_w values, plus the truncation of each band.  A slice keeps two of
 * these (current row and the row above) for vertical prediction. */
typedef struct {
    uint8_t* g[MAXC][MAXB];
    uint8_t gtli[MAXC][MAXB];
} gstore_t;

static int gstore_alloc(gstore_t* s, const geom_t* g) {
    memset(s, 0, sizeof(*s));
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++) {
            s->g[c][b] = (uint8_t*)calloc((size_t)MAX(g->c[c].b[b].gwn, g->c[c].b[b].gwl) * 4 + 8, 1);
            if (!s->g[c][b]) return E_RESOURCES;
        }
    return E_NONE;
}
static void gstore_free(gstore_t* s) {
    for (int c = 0; c < MAXC; c++)
        for (int b = 0; b < MAXB; b++) free(s->g[c][b]);
}

/* vlc_reader_get_next_value (Packing.c:44-115): unary code, number of ones
 * before the terminating zero; -1 past 32 ones. */
static int vlc_next(br_t* r, int64_t* left) {
    uint32_t n = 0;
    while (n < 32 && br_get(r, 1)) n++;
    if (n >= 32) return -1;
    *left -= n + 1;
    return (int)n;
}

/* Vertical prediction of one band line (unpack_verical_pred_gclis_*,
 * Packing.c:267-431): each GCLI is coded relative to the line above (the
 * last line of the same band in the precinct above for line 0). */
static int decode_vpred_line(br_t* r, int64_t* left, uint8_t* gl, const uint8_t* top, uint8_t gtli, uint8_t gtli_top,
                             uint32_t gcli_w, const uint8_t* sig, int run_mode) {
    const int t = MAX(gtli_top, gtli);
    for (uint32_t i = 0; i < gcli_w; i++) {
        const int m_top = MAX((int)top[i], t);
        if (sig && sig[i / 8]) {
            gl[i] = run_mode ? gtli : (uint8_t)m_top;
            continue;
        }
        const int x = vlc_next(r, left);
        if (x < 0) return E_DEC_BITSTREAM;
        const int thr = MAX(m_top - (int)gtli, 0);
        int delta = 0;
        if (x > 2 * thr) delta = x - thr;
        else if (x > 0) delta = (x & 1) ? -((x + 1) / 2) : x / 2;
        gl[i] = (uint8_t)(m_top + delta);
    }
    return E_NONE;
}

/* unpack_precinct (Source/Lib/Decoder/Codec/Packing.c:513-868), then
 * dequantisation and sign conversion
 * (Dequant.c:9-57, Precinct.c:9-29).  `top` is the precinct above in the
 * same slice (NULL for the first precinct of a slice). */
static int dec_precinct(dec_t* d, br_t* r, uint32_t p, uint32_t col, int last, gstore_t* cur, const gstore_t* top) {
    dec_hdr_t* h = d->h;
    const geom_t* g = &h->g;
    if (!br_enough(r, 5 + DIV_UP(g->nbands_exist * 2, 8))) return E_DEC_SHORT;
    uint32_t lprc = br_get(r, 24);
    if (lprc > PREC_MAX_BYTES) return E_DEC_BITSTREAM;
    uint8_t q = (uint8_t)br_get(r, 8), rr = (uint8_t)br_get(r, 8);
    const int long_hdr = h->lh || !g->short_hdr;
    uint8_t mode[MAXGB];
    for (uint32_t i = 0; i < g->nbands_all; i++) {
        if (g->gband[i] == NOBAND) { mode[i] = 0xff; continue; }
        mode[i] = (uint8_t)br_get(r, 2);
        if (!top && (mode[i] & 1)) return E_DEC_BITSTREAM; /* no precinct above to predict from */
    }
    br_align(r);
    if (!br_enough(r, lprc)) return E_DEC_SHORT;
    int64_t left = (int64_t)lprc * 8;
    const uint64_t prec_start = r->bit >> 3;
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++) cur->gtli[c][b] = truncation(g->c[c].b[b].gain, g->c[c].b[b].prio, q, rr);
    for (uint32_t k = 0; k < g->npk; k++) {
        const uint32_t l = g->pk[k].line;
        int present = 0;
        for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
            const band_t* bd = &g->c[g->gcomp[i]].b[g->gband[i]];
            if (l < (last ? bd->last_lines : bd->lines)) { present = 1; break; }
        }
        if (!present) continue;
        uint32_t hb = long_hdr ? 7 : 5;
        left -= hb * 8;
        if (left < 0) return E_DEC_BITSTREAM;
        if (!br_enough(r, hb)) return E_DEC_SHORT;
        uint32_t raw = br_get(r, 1), dlen, glen, slen;
        if (long_hdr) { dlen = br_get(r, 20); glen = br_get(r, 20); slen = br_get(r, 15); }
        else { dlen = br_get(r, 15); glen = br_get(r, 13); slen = br_get(r, 11); }
        if ((uint64_t)left < ((uint64_t)dlen + glen + slen) * 8) return E_DEC_BITSTREAM;
        uint64_t sub_start;
        uint8_t* sig_store[MAXGB] = {0};
        uint8_t sbuf[MAXGB][1024];
        if (raw) {
            sub_start = r->bit >> 3;
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                const band_t* bd = &g->c[g->gcomp[i]].b[g->gband[i]];
                if (l >= (last ? bd->last_lines : bd->lines)) continue;
                const bview_t v = bview(g, bd, col);
                left -= v.gw * 4;
                if (left < 0) return E_DEC_BITSTREAM;
                uint8_t* gl = cur->g[g->gcomp[i]][g->gband[i]] + (size_t)l * v.gw;
                for (uint32_t x = 0; x < v.gw; x++) gl[x] = (uint8_t)br_get(r, 4);
            }
        } else {
            /* significance sub-packet: 1 = group insignificant */
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                const band_t* bd = &g->c[g->gcomp[i]].b[g->gband[i]];
                if (l >= (last ? bd->last_lines : bd->lines)) continue;
                if (mode[i] & 2) {
                    const bview_t v = bview(g, bd, col);
                    if (v.sw > 1024) return E_RESOURCES;
                    left -= v.sw;
                    if (left < 0) return E_DEC_BITSTREAM;
                    sig_store[i - g->pk[k].bs] = sbuf[i - g->pk[k].bs];
                    for (uint32_t s2 = 0; s2 < v.sw; s2++) sig_store[i - g->pk[k].bs][s2] = (uint8_t)br_get(r, 1);
                }
            }
            br_align(r);
            left -= left & 7;
            sub_start = r->bit >> 3;
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                uint32_t c = g->gcomp[i], b = g->gband[i];
                const band_t* bd = &g->c[c].b[b];
                if (l >= (last ? bd->last_lines : bd->lines)) continue;
                const bview_t v = bview(g, bd, col);
                uint8_t* gl = cur->g[c][b] + (size_t)l * v.gw;
                const uint8_t t = cur->gtli[c][b];
                const uint8_t* sf = sig_store[i - g->pk[k].bs];
                if (mode[i] & 1) {
                    const uint8_t* tp = l == 0 ? top->g[c][b] + (size_t)(bd->lines - 1) * v.gw : cur->g[c][b] + (size_t)(l - 1) * v.gw;
                    const uint8_t tt = l == 0 ? top->gtli[c][b] : t;
                    if (decode_vpred_line(r, &left, gl, tp, t, tt, v.gw, sf, (int)h->rm)) return E_DEC_BITSTREAM;
                } else {
                    for (uint32_t x = 0; x < v.gw; x++) {
                        if (sf && sf[x / 8]) { gl[x] = t; continue; }
                        int n = vlc_next(r, &left);
                        if (n < 0) return E_DEC_BITSTREAM;
                        gl[x] = (uint8_t)(t + n);
                    }
                }
            }
        }
        br_align(r);
        left -= left & 7;
        int64_t used = (int64_t)(r->bit >> 3) - (int64_t)sub_start;
        if (used != (int64_t)glen) {
            int64_t lo = (int64_t)glen - used;
            if (lo > 0 && br_enough(r, (uint32_t)lo)) { r->bit += (uint64_t)lo * 8; left -= lo * 8; }
            else return E_DEC_BITSTREAM;
        }
        /* data sub-packet: unpack_data_c (Packing.c:134-219).  Values are
         * kept in sign-magnitude form until the packet's signs are known. */
        uint32_t leftover_nz[MAXGB] = {0};
        sub_start = r->bit >> 3;
        for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
            uint32_t c = g->gcomp[i], b = g->gband[i];
            const band_t* bd = &g->c[c].b[b];
            if (l >= (last ? bd->last_lines : bd->lines)) continue;
            const uint8_t t = cur->gtli[c][b];
            const bview_t v = bview(g, bd, col);
            const uint8_t* gl = cur->g[c][b] + (size_t)l * v.gw;
            uint16_t* out = (uint16_t*)d->coef[c][b] + (size_t)(p * bd->lines + l) * bd->w + v.x0;
            for (uint32_t x = 0; x < v.gw; x++) {
                uint16_t vv[4] = {0, 0, 0, 0};
                int32_t planes = (int32_t)gl[x] - t;
                if (planes > 0) {
                    left -= 4 * (planes + (h->fs ? 0 : 1));
                    if (left < 0) return E_DEC_BITSTREAM;
                    uint32_t sg = h->fs ? 0 : br_get(r, 4);
                    uint32_t m[4] = {0, 0, 0, 0};
                    for (int32_t pl = 0; pl < planes; pl++) {
                        uint32_t nib = br_get(r, 4);
                        for (int k2 = 0; k2 < 4; k2++) m[k2] = (m[k2] << 1) | ((nib >> (3 - k2)) & 1u);
                    }
                    for (int k2 = 0; k2 < 4; k2++) vv[k2] = (uint16_t)((uint16_t)(m[k2] << t) | (((sg >> (3 - k2)) & 1u) << 15));
                }
                for (uint32_t k2 = 0; k2 < 4; k2++) {
                    if (x * 4 + k2 < v.w) out[x * 4 + k2] = vv[k2];
                    else leftover_nz[i - g->pk[k].bs] += vv[k2] != 0; /* its sign is sent too (Packing.c:200-215) */
                }
            }
        }
        br_align(r);
        left -= left & 7;
        used = (int64_t)(r->bit >> 3) - (int64_t)sub_start;
        if (used != (int64_t)dlen) {
            int64_t lo = (int64_t)dlen - used;
            if (lo > 0 && br_enough(r, (uint32_t)lo)) { r->bit += (uint64_t)lo * 8; left -= lo * 8; }
            else return E_DEC_BITSTREAM;
        }
        if (h->fs) {
            /* sign sub-packet: unpack_sign (Packing.c:221-247), one bit per
             * non-zero magnitude, then the signs of the padding coefficients */
            sub_start = r->bit >> 3;
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                uint32_t c = g->gcomp[i], b = g->gband[i];
                const band_t* bd = &g->c[c].b[b];
                if (l >= (last ? bd->last_lines : bd->lines)) continue;
                const bview_t v = bview(g, bd, col);
                uint16_t* out = (uint16_t*)d->coef[c][b] + (size_t)(p * bd->lines + l) * bd->w + v.x0;
                for (uint32_t x = 0; x < v.w; x++) {
                    if (!out[x]) continue;
                    if (--left < 0) return E_DEC_BITSTREAM;
                    if (!br_enough(r, 1)) return E_DEC_SHORT;
                    out[x] |= (uint16_t)(br_get(r, 1) << 15);
                }
                const uint32_t lo = leftover_nz[i - g->pk[k].bs];
                if (lo && (v.w % 4)) {
                    left -= lo;
                    if (left < 0) return E_DEC_BITSTREAM;
                    r->bit += lo;
                }
            }
            br_align(r);
            left -= left & 7;
            used = (int64_t)(r->bit >> 3) - (int64_t)sub_start;
            if (used != (int64_t)slen) {
                int64_t lo = (int64_t)slen - used;
                if (lo > 0 && br_enough(r, (uint32_t)lo)) { r->bit += (uint64_t)lo * 8; left -= lo * 8; }
                else return E_DEC_BITSTREAM;
            }
        }
        /* inv_quant_deadzone / inv_quant_uniform (Dequant.c:9-43), then
         * inv_sign_c (Precinct.c:9-14) */
        for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
            uint32_t c = g->gcomp[i], b = g->gband[i];
            const band_t* bd = &g->c[c].b[b];
            if (l >= (last ? bd->last_lines : bd->lines)) continue;
            const uint8_t t = cur->gtli[c][b];
            const bview_t v = bview(g, bd, col);
            const uint8_t* gl = cur->g[c][b] + (size_t)l * v.gw;
            int16_t* out = d->coef[c][b] + (size_t)(p * bd->lines + l) * bd->w + v.x0;
            for (uint32_t x = 0; x < v.w; x++) {
                const uint16_t raw = (uint16_t)out[x];
                uint16_t mag = raw & 0x7fff;
                if (t > 0 && mag) {
                    if (h->qpih == 0) {
                        mag |= (uint16_t)(1u << (t - 1));
                    } else {
                        uint16_t val = mag, acc = 0;
                        uint8_t sc = (uint8_t)(gl[x / 4] - t + 1);
                        for (; val > 0; val >>= sc) acc = (uint16_t)(acc + val);
                        mag = acc;
                    }
                }
                out[x] = (int16_t)((raw & 0x8000) ? -(int32_t)(mag & 0x7fff) : (int32_t)mag);
            }
        }
    }
    int64_t pad = (int64_t)lprc - ((int64_t)(r->bit >> 3) - (int64_t)prec_start);
    if (pad < 0) return E_DEC_BITSTREAM;
    r->bit += (uint64_t)pad * 8;
    return E_NONE;
}

static void dec_slice(void* ctx, uint32_t s) {
    dec_t* d = (dec_t*)ctx;
    const geom_t* g = &d->h->g;
    br_t r = {d->bs, d->size, (uint64_t)d->slice_off[s] * 8};
    if (!br_enough(&r, 6)) { d->err = E_DEC_SHORT; return; }
    if (br_get(&r, 16) != 0xff20 || br_get(&r, 16) != 4 || br_get(&r, 16) != s) { d->err = E_DEC_BITSTREAM; return; }
    /* the precincts of a row, column after column (Decoder.c:537-580);
     * each column keeps the row above's GCLIs for vertical prediction */
    const uint32_t ncol = g->ncol;
    gstore_t* st = (gstore_t*)calloc(2 * (size_t)ncol, sizeof(gstore_t));
    int err = st ? E_NONE : E_RESOURCES;
    for (uint32_t k = 0; k < 2 * ncol && !err; k++) err = gstore_alloc(&st[k], g);
    uint32_t first = s * g->pps;
    uint32_t n = (s == g->nslices - 1) ? g->np - first : g->pps;
    for (uint32_t i = 0; i < n && !err; i++) {
        uint32_t p = first + i;
        for (uint32_t col = 0; col < ncol && !err; col++)
            err = dec_precinct(d, &r, p, col, p + 1 >= g->np, &st[2 * col + (i & 1)], i ? &st[2 * col + ((i + 1) & 1)] : NULL);
    }
    if (err) d->err = err;
    for (uint32_t k = 0; st && k < 2 * ncol; k++) gstore_free(&st[k]);
    free(st);
}

typedef struct {
    dec_t* d;
    void* const* planes;
    const uint32_t* strides;
} idwt_job_t;

static inline int32_t clamp_i64(int64_t v, int32_t m) { return (int32_t)(v > m ? m : v < 0 ? 0 : v); }

/* Output scaling of one sample of the inverse transform by the NLT
 * marker's non-linearity (nlt_inverse_transform_line_*, NltDec.c:22-194,
 * 366-406): linear, quadratic (Tnlt = 1) or extended (Tnlt = 2), with the
 * first component's depth. */
static int32_t nlt_sample(const dec_hdr_t* h, int64_t v) {
    const int32_t bw = (int32_t)h->bw, depth = (int32_t)h->depth[0], m = (1 << depth) - 1, clampv = (1 << bw) - 1;
    v += ((int64_t)1 << bw) >> 1;
    if (h->tnlt == 1) {
        const int32_t zeta = 2 * bw - depth;
        const int32_t dco = (int32_t)h->nlt_alpha - (int32_t)h->nlt_sigma * (1 << 15);
        const int64_t q = (int64_t)clamp_i64(v, clampv);
        const int64_t v2 = (q * q + (((int64_t)1 << zeta) >> 1)) >> zeta;
        return clamp_i64(v2 + dco, m);
    }
    if (h->tnlt == 2) {
        const int32_t zeta = 2 * bw - depth;
        const int32_t t1 = (int32_t)h->nlt_t1, t2 = (int32_t)h->nlt_t2, e = (int32_t)h->nlt_e;
        const int32_t b1 = (int32_t)((int64_t)t1 + (1 << (bw - e - 1)));
        const int64_t b2 = (int64_t)t1 * t1, b3 = (int64_t)t2 - ((int64_t)1 << (bw - e - 1));
        const int64_t a1 = b2 + (int64_t)t1 * ((int64_t)1 << (bw - e)) + ((int64_t)1 << (2 * bw - 2 - 2 * e));
        const int64_t a3 = b2 + (int64_t)t2 * ((int64_t)1 << (bw - e)) - ((int64_t)1 << (2 * bw - 2 - 2 * e));
        if (v < t1) {
            const int64_t q = clamp_i64((int64_t)b1 - v, clampv);
            v = a1 - q * q;
        } else if (v < t2) {
            v = v * ((int64_t)1 << (bw - e)) + b2;
        } else {
            const int64_t q = clamp_i64(v - b3, clampv);
            v = a3 + q * q;
        }
        return clamp_i64((v + (((int64_t)1 << zeta) >> 1)) >> zeta, m);
    }
    const int32_t zeta = bw - depth;
    return clamp_i64((v + (((int64_t)1 << zeta) >> 1)) >> zeta, m);
}

/* Star-Tetrix (ISO/IEC 21122-1 Annex F; Mct.c:14-136): the component
 * displacement vectors (Table F.10), the component at a displacement
 * (Table F.11) and the coordinate access with mirroring at the picture
 * edges and, for Cf = 3, within a line pair (Table F.12). */
static const int8_t st_disp[2][4][2] = {{{0, 1}, {1, 1}, {0, 0}, {1, 0}}, {{1, 1}, {0, 1}, {1, 0}, {0, 0}}};
static const uint8_t st_comp[2][2][2] = {{{2, 0}, {3, 1}}, {{3, 1}, {2, 0}}};
static int32_t st_access(int32_t* const* comps, int c, int x, int y, int w, int h, int rx, int ry, int cf, int ct) {
    const int dx = st_disp[ct][c][0], dy = st_disp[ct][c][1];
    if (2 * x + rx + dx < 0 || 2 * x + rx + dx >= 2 * w) rx = -rx;
    if ((cf == 3 && (ry + dy < 0 || ry + dy > 1)) || 2 * y + ry + dy < 0 || 2 * y + ry + dy >= 2 * h) ry = -ry;
    const int xx = (2 * x + rx + dx) / 2, yy = (2 * y + ry + dy) / 2;
    return comps[st_comp[ct][(2 + rx + dx) % 2][(2 + ry + dy) % 2]][(size_t)yy * w + xx];
}

/* Inverse Star-Tetrix (Tables F.4-F.8; inverse_star_tetrix, Mct.c:120-135):
 * average, delta, Y and CbCr steps in place, then components 0 <-> 2 and
 * 1 <-> 3.  Products are taken in 32-bit wrap-around arithmetic like the
 * reference's int. */
static void inv_star_tetrix(int32_t* comps[4], int cf, int ct, int e1, int e2, int w, int h) {
#define ACC(c, rx, ry) st_access(comps, c, x, y, w, h, rx, ry, cf, ct)
#define MUL(k, v) ((int32_t)((uint32_t)(k) * (uint32_t)(v)))
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            comps[0][(size_t)y * w + x] -= (ACC(0, -1, -1) + ACC(0, 1, -1) + ACC(0, -1, 1) + ACC(0, 1, 1)) >> 3;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            comps[3][(size_t)y * w + x] += (ACC(3, -1, -1) + ACC(3, 1, -1) + ACC(3, -1, 1) + ACC(3, 1, 1)) >> 2;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            comps[0][(size_t)y * w + x] -= (MUL(1 << e2, ACC(0, -1, 0) + ACC(0, 1, 0)) + MUL(1 << e1, ACC(0, 0, -1) + ACC(0, 0, 1))) >> 3;
            comps[3][(size_t)y * w + x] -= (MUL(1 << e2, ACC(3, 0, -1) + ACC(3, 0, 1)) + MUL(1 << e1, ACC(3, -1, 0) + ACC(3, 1, 0))) >> 3;
        }
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            comps[1][(size_t)y * w + x] += (ACC(1, -1, 0) + ACC(1, 1, 0) + ACC(1, 0, -1) + ACC(1, 0, 1)) >> 2;
            comps[2][(size_t)y * w + x] += (ACC(2, -1, 0) + ACC(2, 1, 0) + ACC(2, 0, -1) + ACC(2, 0, 1)) >> 2;
        }
#undef ACC
#undef MUL
    int32_t* t = comps[0];
    comps[0] = comps[2];
    comps[2] = t;
    t = comps[1];
    comps[1] = comps[3];
    comps[3] = t;
}

/* get_cfa_pattern (Mct.c:155-178): the CFA pattern type from the CRG
 * marker. */
static int st_cfa_type(const dec_hdr_t* h) {
    return (h->xcrg[1] == 32768 && h->ycrg[1] == 0 && h->xcrg[2] == 0 && h->ycrg[2] == 32768) ? 0 : 1;
}

/* With a colour transform: Cpih = 1, the inverse reversible colour
 * transform of components 0-2 (inverse_rct, Mct.c:137-153); Cpih = 3, the
 * inverse Star-Tetrix transform; on the whole frame, then every
 * component's output scaling (svt_jpeg_xs_decode_final,
 * Decoder.c:707-798). */
static void dec_mct_nlt(dec_t* d, void* const planes[4], const uint32_t strides[4]) {
    const dec_hdr_t* h = d->h;
    const geom_t* g = &h->g;
    const uint32_t w = g->c[0].w, ht = g->c[0].h;
    const size_t n = (size_t)w * ht;
    if (h->cpih == 3) inv_star_tetrix(d->mct, (int)h->cf, st_cfa_type(h), (int)h->e1, (int)h->e2, (int)w, (int)ht);
    if (h->cpih == 1) {
        int32_t *c0 = d->mct[0], *c1 = d->mct[1], *c2 = d->mct[2];
        for (size_t i = 0; i < n; i++) {
            const int32_t i0 = c0[i], i1 = c1[i], i2 = c2[i];
            const int32_t o1 = i0 - ((i1 + i2) >> 2);
            c0[i] = o1 + i2;
            c1[i] = o1;
            c2[i] = o1 + i1;
        }
    }
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t y = 0; y < ht; y++)
            for (uint32_t x = 0; x < w; x++) {
                const int32_t o = nlt_sample(h, d->mct[c][(size_t)y * w + x]);
                if (h->depth[0] <= 8) ((uint8_t*)planes[c])[(size_t)y * strides[c] + x] = (uint8_t)o;
                else ((uint16_t*)planes[c])[(size_t)y * strides[c] + x] = (uint16_t)o;
            }
}

/* Inverse transform of one component (coefficients << Fq, DwtDecoder.c:
 * 322-406) and linear output scaling (linear_output_scaling_*_line_c,
 * NltDec.c:242-264). */
static void dec_idwt_one(void* ctx, uint32_t c) {
    idwt_job_t* j = (idwt_job_t*)ctx;
    dec_t* d = j->d;
    const geom_t* g = &d->h->g;
    const comp_t* cp = &g->c[c];
    uint32_t w = cp->w, h = cp->h;
    int32_t* a = (int32_t*)malloc(sizeof(int32_t) * (size_t)w * h);
    for (uint32_t b = 0; b < cp->nb; b++) {
        const band_t* bd = &cp->b[b];
        for (uint32_t y = 0; y < bd->h; y++)
            for (uint32_t x = 0; x < bd->w; x++)
                a[(size_t)(bd->y + y) * w + bd->x + x] = (int32_t)((uint32_t)(int32_t)d->coef[c][b][(size_t)y * bd->w + x] << d->h->fq);
    }
    inv_component(a, w, h, cp->dv, cp->dh);
    if (d->h->cpih) {
        /* kept for the colour transform and the output non-linearity
         * (svt_jpeg_xs_decode_final, Decoder.c:707-798) */
        d->mct[c] = a;
        return;
    }
    const uint32_t depth = d->h->depth[0];
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) {
            const int32_t o = nlt_sample(d->h, a[(size_t)y * w + x]);
            if (depth == 8) ((uint8_t*)j->planes[c])[(size_t)y * j->strides[c] + x] = (uint8_t)o;
            else ((uint16_t*)j->planes[c])[(size_t)y * j->strides[c] + x] = (uint16_t)o;
        }
    free(a);
}

int or_decode(const uint8_t* bs, uint32_t size, void* const planes[4], const uint32_t strides[4], uint32_t threads_num,
              or_image_info_t* info) {
    if (!bs || !size) return E_DEC_PTR;
    dec_hdr_t h;
    int e = dec_parse_header(bs, size, &h);
    if (e) return e;
    if (info) {
        e = or_probe(bs, size, info);
        if (e) return e;
    }
    dec_t d;
    memset(&d, 0, sizeof(d));
    d.h = &h;
    d.bs = bs;
    d.size = size;
    const geom_t* g = &h.g;
    /* Slice start offsets: walk precinct lengths (get_slice_size,
     * DecThreadInit.c:35-131). */
    d.slice_off = (uint32_t*)malloc(sizeof(uint32_t) * g->nslices);
    uint64_t off = h.hdr_len;
    const uint32_t bands_hdr = 5 + DIV_UP(g->nbands_exist * 2, 8);
    for (uint32_t s = 0; s < g->nslices; s++) {
        d.slice_off[s] = (uint32_t)off;
        off += 6;
        uint32_t first = s * g->pps;
        uint32_t n = ((s == g->nslices - 1) ? g->np - first : g->pps) * g->ncol;
        for (uint32_t i = 0; i < n; i++) {
            if (off + 3 > size) { free(d.slice_off); return E_DEC_SHORT; }
            uint32_t lprc = ((uint32_t)bs[off] << 16) | ((uint32_t)bs[off + 1] << 8) | bs[off + 2];
            off += bands_hdr + lprc;
        }
    }
    if (off + 2 > size) { free(d.slice_off); return E_DEC_SHORT; }
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++)
            d.coef[c][b] = (int16_t*)calloc((size_t)g->c[c].b[b].w * g->c[c].b[b].h, sizeof(int16_t));
    uint32_t threads = threads_num ? threads_num : 1;
    parallel_for(g->nslices, threads, dec_slice, &d);
    if (!d.err) {
        idwt_job_t j = {&d, planes, strides};
        parallel_for(g->nc, threads, dec_idwt_one, &j);
        if (h.cpih) dec_mct_nlt(&d, planes, strides);
    }
    for (uint32_t c = 0; c < g->nc; c++) free(d.mct[c]);
    for (uint32_t c = 0; c < g->nc; c++)
        for (uint32_t b = 0; b < g->c[c].nb; b++) free(d.coef[c][b]);
    free(d.slice_off);
    return d.err;
}
