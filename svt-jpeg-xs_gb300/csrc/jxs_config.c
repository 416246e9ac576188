/*
 * Host-side stream configuration: encoder parameter validation, picture
 * geometry, weight tables, the cached codestream header, slice byte budgets,
 * and codestream header parsing for the decoder.
 *
 * Restates, for the GPU data layout of jxs_core.h:
 *   encoder_init_configuration  Source/Lib/Encoder/Codec/EncHandle.c:128-454
 *   pi_compute & helpers         Source/Lib/Common/Codec/Pi.c:21-406
 *   weight_table_calculate       Source/Lib/Encoder/Codec/WeightTable.c:18-413
 *   max quantization/refinement  Source/Lib/Encoder/Codec/PiEnc.c:11-53
 *   write_header                 Source/Lib/Encoder/Codec/PackHeaders.c:11-140
 *   slice budgets                Source/Lib/Encoder/Codec/EncHandle.c:760-809
 *   get_header                   Source/Lib/Decoder/Codec/ParseHeader.c:20-617
 */
#include "jxs_core.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "SvtJpegxsEnc.h"

#define DIV_UP(a, b) (((a) + (b)-1) / (b))
#define MIN(a, b) ((a) < (b) ? (a) : (b))
#define MAX(a, b) ((a) > (b) ? (a) : (b))
#define ALIGN_UP(a, b) (DIV_UP(a, b) * (b))

int32_t jxs_sampling(uint32_t fmt, uint32_t* nc, uint32_t sx[JXS_MAXC], uint32_t sy[JXS_MAXC]) {
    for (int i = 0; i < JXS_MAXC; i++) sx[i] = sy[i] = 1;
    switch (fmt) {
    case COLOUR_FORMAT_PLANAR_YUV422: *nc = 3; sx[1] = sx[2] = 2; return JXS_OK;
    case COLOUR_FORMAT_PLANAR_YUV420: *nc = 3; sx[1] = sx[2] = 2; sy[1] = sy[2] = 2; return JXS_OK;
    case COLOUR_FORMAT_PLANAR_YUV444_OR_RGB:
    case COLOUR_FORMAT_PACKED_YUV444_OR_RGB: *nc = 3; return JXS_OK;
    case COLOUR_FORMAT_PLANAR_4_COMPONENTS: *nc = 4; return JXS_OK;
    case COLOUR_FORMAT_GRAY: *nc = 1; return JXS_OK;
    default: return JXS_E_BAD_PARAM;
    }
}

/* Per-component band tree, global band numbering, packets and precinct
 * lines (Pi.c:131-406 for one precinct column). */
/* Band lines of the normal and the last precinct row in codestream order,
 * and their split into segments (packet order of Pi.c:189-406). */
static int32_t cfg_blines(jxs_cfg_t* g) {
    uint32_t sg = 128;
    for (;;) {
        int fits = 1;
        for (int t = 0; t < 4; t++) {
            uint32_t n = 0, ns = 0, gsum = 0;
            for (uint32_t k = 0; k < g->npk; k++) {
                const uint32_t l = g->pk[k].line;
                g->pk_bl0[t][k] = (uint8_t)n;
                g->pk_nbl[t][k] = 0;
                for (uint32_t gb = g->pk[k].bs; gb < g->pk[k].be; gb++) {
                    const uint32_t fb = g->g2f[gb];
                    if (fb == JXS_NOBAND) continue;
                    const jxs_band_t* bd = &g->band[fb];
                    if (l >= ((t & 1) ? bd->last_lines : bd->lines)) continue;
                    if (n >= JXS_MAXBLINES) return JXS_E_BAD_PARAM;
                    const uint32_t w = (t & 2) ? bd->cwl : bd->cwn, gw = DIV_UP(w, 4);
                    g->pk_nbl[t][k]++;
                    jxs_bline_t* b = &g->bline[t][n++];
                    b->fb = (uint8_t)fb;
                    b->line = (uint8_t)l;
                    b->pk = (uint8_t)k;
                    b->pad = 0;
                    b->gcli_w = gw;
                    b->sig_w = DIV_UP(gw, 8);
                    b->w = w;
                    b->gbase = gsum;
                    gsum += (gw + 3) & ~3u; /* 4-aligned: 32-bit access to 4 groups */
                    b->seg0 = ns;
                    b->nseg = (gw + sg - 1) / sg;
                    if (b->nseg == 0) b->nseg = 1;
                    for (uint32_t i = 0; i < b->nseg; i++, ns++) {
                        if (ns < JXS_MAXSEG) {
                            g->seg[t][ns].bl = (uint16_t)(n - 1);
                            g->seg[t][ns].pad = 0;
                            g->seg[t][ns].g0 = i * sg;
                        }
                    }
                }
            }
            g->nbline[t] = n;
            g->nseg[t] = ns;
            if (ns > JXS_MAXSEG) fits = 0;
        }
        if (fits) break;
        sg *= 2;
    }
    g->seg_groups = sg;
    /* work order of the segments: most groups first, so that the warps that
     * take segments from a queue finish close together */
    for (int t = 0; t < 4; t++) {
        const uint32_t n = g->nseg[t];
        for (uint32_t i = 0; i < n; i++) {
            const jxs_seg_t* si = &g->seg[t][i];
            const uint32_t gi = g->bline[t][si->bl].gcli_w - si->g0, ni = gi < sg ? gi : sg;
            uint32_t j = i;
            while (j > 0) {
                const jxs_seg_t* sj = &g->seg[t][g->seg_ord[t][j - 1]];
                const uint32_t gj = g->bline[t][sj->bl].gcli_w - sj->g0, nj = gj < sg ? gj : sg;
                if (nj >= ni) break;
                g->seg_ord[t][j] = g->seg_ord[t][j - 1];
                j--;
            }
            g->seg_ord[t][j] = (uint16_t)i;
        }
    }
    /* the line above each band line, for vertical prediction (line 0: the
     * band's last line in the precinct above, a normal row of the same
     * column kind) */
    for (int t = 0; t < 4; t++) {
        for (uint32_t x = 0; x < g->nbline[t]; x++) {
            const jxs_bline_t* b = &g->bline[t][x];
            const int prev = b->line == 0;
            const int tt = prev ? (t & 2) : t;
            const uint32_t want = prev ? g->band[b->fb].lines - 1 : b->line - 1u;
            g->top_bl[t][x] = 0xff;
            g->top_prev[t][x] = (uint8_t)prev;
            g->top_gbase[t][x] = 0;
            for (uint32_t y = 0; y < g->nbline[tt]; y++) {
                if (g->bline[tt][y].fb == b->fb && g->bline[tt][y].line == want) {
                    g->top_bl[t][x] = (uint8_t)y;
                    g->top_gbase[t][x] = g->bline[tt][y].gbase;
                    break;
                }
            }
        }
    }
    return JXS_OK;
}

/* Each packet's band lines by ascending band priority (the order in which
 * a growing refinement R lowers their gtli); needs the weight tables. */
static void cfg_pk_order(jxs_cfg_t* g) {
    for (int t = 0; t < 4; t++)
        for (uint32_t k = 0; k < g->npk; k++) {
            const uint32_t b0 = g->pk_bl0[t][k], nb = g->pk_nbl[t][k];
            for (uint32_t i = 0; i < nb; i++) g->pk_order[t][b0 + i] = (uint8_t)(b0 + i);
            for (uint32_t i = 1; i < nb; i++) {
                const uint8_t x = g->pk_order[t][b0 + i];
                uint32_t j = i;
                while (j > 0 && g->band[g->bline[t][g->pk_order[t][b0 + j - 1]].fb].prio > g->band[g->bline[t][x].fb].prio) {
                    g->pk_order[t][b0 + j] = g->pk_order[t][b0 + j - 1];
                    j--;
                }
                g->pk_order[t][b0 + j] = x;
            }
        }
}

int32_t jxs_cfg_geometry(jxs_cfg_t* g, int for_encoder, uint32_t nc, uint32_t W, uint32_t H, uint32_t dh, uint32_t dv,
                         uint32_t sd, const uint32_t sx[JXS_MAXC], const uint32_t sy[JXS_MAXC], uint32_t slice_h, uint32_t cw) {
    if (sd > nc || dv > dh || dh > 5 || dv > 2 || nc > JXS_MAXC || nc < 1 || slice_h == 0) return JXS_E_BAD_PARAM;
    g->nc = nc; g->W = W; g->H = H; g->dh = dh; g->dv = dv; g->sd = sd;
    const uint32_t ncd = nc - sd;
    g->prec_h = 1u << dv;
    if (slice_h < H && (slice_h % g->prec_h)) return JXS_E_BAD_PARAM;
    g->slice_h = slice_h;
    g->pps = DIV_UP(slice_h, g->prec_h);
    g->nslices = DIV_UP(H, slice_h);
    if (g->nslices > 8192 || H == 0 || W == 0) return JXS_E_BAD_PARAM;

    /* per-component decomposition and band counts */
    uint32_t nb[JXS_MAXC];
    g->nbands = 0;
    for (uint32_t c = 0; c < nc; c++) {
        jxs_comp_t* cp = &g->comp[c];
        if (sx[c] < 1 || sy[c] < 1) return JXS_E_BAD_PARAM;
        cp->sx = sx[c]; cp->sy = sy[c];
        cp->w = W / sx[c]; cp->h = H / sy[c];
        if ((g->prec_h / sy[c]) == 0) return JXS_E_BAD_PARAM;
        if (c < ncd) {
            if (dv < sy[c] / 2) return JXS_E_BAD_PARAM;
            cp->dh = dh;
            cp->dv = dv - sy[c] / 2;
        } else {
            cp->dh = cp->dv = 0;
        }
        cp->nb = 2 * cp->dv + cp->dh + 1;
        if (cp->nb > JXS_MAXB) return JXS_E_BAD_PARAM;
        cp->band0 = g->nbands;
        nb[c] = cp->nb;
        g->nbands += cp->nb;
    }
    g->nbands_all = nb[0] * ncd + sd;
    if (g->nbands_all > JXS_MAXBL) return JXS_E_BAD_PARAM;
    memset(g->g2f, JXS_NOBAND, sizeof(g->g2f));

    /* global (codestream) band numbering: bands of the components interleave;
     * components with fewer vertical levels leave gaps (Pi.c:268-303). */
    const uint32_t nb_global = 2 * dv + dh + 1;
    for (uint32_t c = 0; c < ncd; c++) {
        jxs_comp_t* cp = &g->comp[c];
        uint32_t ignore = nb_global - cp->nb, at_end = 3 * cp->dv, id = c;
        for (uint32_t i = 0; i < cp->nb; i++) {
            jxs_band_t* bd = &g->band[cp->band0 + i];
            memset(bd, 0, sizeof(*bd));
            bd->gid = id;
            bd->comp = (uint8_t)c;
            bd->idx = (uint8_t)i;
            g->g2f[id] = (uint8_t)(cp->band0 + i);
            id += ncd;
            if (ignore > 0 && i == cp->nb - at_end + 1 - ignore) id += ncd * ignore;
        }
    }
    for (uint32_t c = ncd; c < nc; c++) {
        jxs_comp_t* cp = &g->comp[c];
        if (cp->nb != 1) return JXS_E_BAD_PARAM;
        jxs_band_t* bd = &g->band[cp->band0];
        memset(bd, 0, sizeof(*bd));
        bd->gid = ncd * nb[0] + c - ncd;
        bd->comp = (uint8_t)c;
        g->g2f[bd->gid] = (uint8_t)cp->band0;
    }

    /* band sizes: each vertical level splits the low band in four, each
     * further horizontal level splits it in two (Pi.c:305-368) */
    for (uint32_t c = 0; c < nc; c++) {
        jxs_comp_t* cp = &g->comp[c];
        jxs_band_t* b = &g->band[cp->band0];
        int L = (int)cp->nb - 1;
        b[L].w = cp->w; b[L].h = cp->h; b[L].x = 0; b[L].y = 0;
        for (uint32_t v = 0; v < cp->dv; v++) {
            uint32_t w = b[L].w, h = b[L].h;
            uint32_t w2 = w / 2, w1 = w - w2, h2 = h / 2, h1 = h - h2;
            b[L].w = w2; b[L].h = h2; b[L].x = w1; b[L].y = h1;
            b[L - 1].w = w1; b[L - 1].h = h2; b[L - 1].x = 0; b[L - 1].y = h1;
            b[L - 2].w = w2; b[L - 2].h = h1; b[L - 2].x = w1; b[L - 2].y = 0;
            b[L - 3].w = w1; b[L - 3].h = h1; b[L - 3].x = 0; b[L - 3].y = 0;
            L -= 3;
        }
        for (uint32_t l = cp->dv; l < cp->dh; l++) {
            uint32_t w = b[L].w, h = b[L].h;
            uint32_t w2 = w / 2, w1 = w - w2;
            b[L].w = w2; b[L].h = h; b[L].x = w1; b[L].y = 0;
            b[L - 1].w = w1; b[L - 1].h = h; b[L - 1].x = 0; b[L - 1].y = 0;
            L -= 1;
        }
        for (uint32_t i = 0; i < cp->nb; i++)
            if (b[i].w == 0 || b[i].h == 0) return JXS_E_BAD_PARAM;
        uint32_t two = cp->dv == 2 ? 3 : 0;
        for (uint32_t i = 0; i < cp->nb; i++) b[i].lines = (i < cp->nb - two) ? 1 : 2;
        if (c >= ncd) b[0].lines = MIN(((1u << dv) >> (cp->sy - 1)), cp->h);
    }

    /* packets (Pi.c:131-187) */
    uint32_t n = 0;
    uint32_t stop0 = MAX(dh, dv) - MIN(dh, dv) + 1;
    g->pk[n++] = (jxs_packet_t){0, stop0 * ncd, 0};
    for (uint32_t s = stop0; s < nb[0]; s++) {
        jxs_packet_t p = {s * ncd, s * ncd, 0};
        for (uint32_t i = s * ncd; i < (s + 1) * ncd; i++)
            if (g->g2f[i] != JXS_NOBAND) p.be++;
        g->pk[n++] = p;
    }
    for (uint32_t s = stop0; s < nb[0]; s++) {
        if (g->band[s].lines == 1) continue; /* component 0, band s */
        jxs_packet_t p = {s * ncd, s * ncd, 1};
        for (uint32_t i = s * ncd; i < (s + 1) * ncd; i++)
            if (g->g2f[i] != JXS_NOBAND && g->band[g->g2f[i]].lines > 1) p.be++;
        g->pk[n++] = p;
    }
    uint32_t nbg = ncd * nb[0];
    for (uint32_t c = ncd; c < nc; c++) {
        for (uint32_t line = 0; line < g->band[g->comp[c].band0].lines; line++) g->pk[n++] = (jxs_packet_t){nbg, nbg + 1, line};
        nbg++;
    }
    if (n >= JXS_MAXPK) return JXS_E_BAD_PARAM;
    g->npk = n;
    g->short_hdr = (W * nc) < 32752;

    /* precinct rows and columns, buffer layout (calc_precinct_dimension,
     * Pi.c:21-129): Cw > 0 splits each row into columns of
     * 8 Cw max(Sx) 2^NLx samples */
    g->np = DIV_UP(H, 1u << dv);
    g->cw = cw;
    g->ncol = 1;
    uint32_t cs = 0;
    if (cw) {
        uint32_t sx_max = 0;
        for (uint32_t c = 0; c < nc; c++) sx_max = sx[c] > sx_max ? sx[c] : sx_max;
        cs = 8 * cw * sx_max * (1u << dh);
        g->ncol = DIV_UP(W, cs);
        if (g->ncol >= 130) return JXS_E_BAD_PARAM; /* MAX_PRECINCT_IN_LINE, Decoder.c:294 */
    }
    g->nprec = g->np * g->ncol;
    uint64_t coff = 0, goff = 0;
    for (uint32_t i = 0; i < g->nbands; i++) {
        jxs_band_t* bd = &g->band[i];
        bd->last_lines = bd->h - (g->np - 1) * bd->lines;
        bd->gcli_w = DIV_UP(bd->w, 4);
        bd->sig_w = DIV_UP(bd->gcli_w, 8);
        bd->cwn = bd->w; /* one column: it is the last one, of the band's width */
        if (cw && g->ncol > 1) {
            const jxs_comp_t* cp = &g->comp[bd->comp];
            const uint64_t num = (uint64_t)cs * bd->w, den = (uint64_t)cp->sx * cp->w;
            bd->cwn = (uint32_t)((bd->w % 2) ? num / den : (num + den - 1) / den);
            /* a last column without coefficients (the reference's width_last
             * would wrap) is refused */
            if ((uint64_t)(g->ncol - 1) * bd->cwn >= bd->w) return JXS_E_BAD_PARAM;
        }
        bd->cwl = bd->w - (g->ncol - 1) * bd->cwn;
        bd->pitch = ALIGN_UP(bd->w, 8);
        bd->gpitch = ALIGN_UP(bd->gcli_w, 16);
        bd->coef_off = coff;
        bd->gcli_off = goff;
        coff += (uint64_t)bd->pitch * bd->h;
        goff += (uint64_t)bd->gpitch * bd->h;
    }
    g->coef_total = coff;
    g->gcli_total = goff;
    g->prec_hdr_bytes = DIV_UP(40 + 2 * g->nbands, 8);
    for (int t = 0; t < 4; t++) {
        uint32_t cnt = 0;
        for (uint32_t k = 0; k < g->npk; k++) {
            uint32_t bits = 0;
            int present = 0;
            for (uint32_t i = g->pk[k].bs; i < g->pk[k].be; i++) {
                const jxs_band_t* bd = &g->band[g->g2f[i]];
                uint32_t lines = (t & 1) ? bd->last_lines : bd->lines;
                if (g->pk[k].line < lines) {
                    present = 1;
                    bits += DIV_UP((t & 2) ? bd->cwl : bd->cwn, 4) * 4;
                }
            }
            g->raw_bytes[t][k] = DIV_UP(bits, 8);
            cnt += present;
        }
        if (t < 2) g->pk_exist[t] = for_encoder ? (t == 0 ? g->npk : cnt) : cnt;
    }
    return cfg_blines(g);
}

/* ---- weight tables (gains / priorities per codestream band) ---- */
/* V2/H5 tables from ISO/IEC 21122-1 for 4:4:4 and 4:2:2 (index [v]), and the
 * 4:2:0 tables of the reference (index [v-1][h-1]), WeightTable.c:18-68. */
static const uint8_t t444_g[3][30] = {
    {3, 2, 2, 2, 1, 1, 2, 1, 1, 1, 0, 0, 1, 0, 0, 1, 0, 0},
    {4, 2, 2, 3, 2, 2, 2, 1, 1, 2, 1, 1, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0},
    {4, 3, 3, 3, 2, 2, 3, 2, 2, 2, 1, 1, 2, 1, 1, 2, 1, 1, 1, 0, 0, 1, 0, 0, 1, 0, 0, 1, 0, 0}};
static const uint8_t t444_p[3][30] = {
    {6, 8, 7, 1, 4, 5, 12, 14, 15, 0, 2, 3, 9, 11, 10, 13, 16, 17},
    {21, 1, 0, 15, 19, 18, 5, 9, 8, 14, 17, 16, 2, 4, 3, 7, 13, 11, 6, 12, 10, 20, 23, 22},
    {12, 15, 14, 3, 11, 10, 24, 26, 27, 0, 4, 5, 18, 21, 20, 19, 23, 22, 13, 16, 17, 2, 9, 6, 1, 7, 8, 25, 28, 29}};
static const uint8_t t422_g[3][30] = {
    {2, 2, 2, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {3, 3, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};
static const uint8_t t422_p[3][30] = {
    {8, 7, 6, 5, 3, 4, 13, 12, 14, 1, 0, 2, 9, 11, 10, 16, 15, 17},
    {0, 1, 2, 18, 19, 20, 6, 7, 8, 15, 16, 17, 3, 4, 5, 10, 12, 14, 9, 11, 13, 21, 22, 23},
    {14, 13, 12, 9, 11, 10, 25, 24, 26, 0, 1, 2, 19, 20, 18, 23, 22, 21, 17, 15, 16, 4, 8, 5, 3, 6, 7, 28, 27, 29}};
static const uint8_t tsize_v[3] = {18, 24, 30};
#define X_ JXS_NOBAND
static const uint8_t t420_g[2][5][30] = {
    {{1, 1, 1, 1, 0, 0, 1, X_, X_, 0, X_, X_},
     {1, 1, 1, 1, 0, 0, 1, 0, 0, 1, X_, X_, 0, X_, X_},
     {2, 1, 1, 1, 1, 1, 1, 0, 0, 1, 0, 0, 1, X_, X_, 0, X_, X_},
     {2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 0, 0, 1, 0, 0, 1, X_, X_, 0, X_, X_},
     {3, 3, 3, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 0, 0, 1, 0, 0, 1, X_, X_, 0, X_, X_}},
    {{0},
     {2, 1, 1, 1, 1, 1, 1, X_, X_, 0, X_, X_, 1, 1, 1, 1, 1, 1, 0, 0, 0},
     {2, 2, 2, 2, 1, 1, 1, 1, 1, 1, X_, X_, 0, X_, X_, 1, 1, 1, 1, 1, 1, 0, 0, 0},
     {3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, X_, X_, 0, X_, X_, 1, 1, 1, 1, 1, 1, 0, 0, 0},
     {3, 3, 3, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, X_, X_, 0, X_, X_, 1, 1, 1, 1, 1, 1, 0, 0, 0}}};
static const uint8_t t420_p[2][5][30] = {
    {{2, 5, 4, 6, 1, 0, 7, X_, X_, 3, X_, X_},
     {4, 7, 6, 8, 1, 0, 10, 3, 2, 9, X_, X_, 5, X_, X_},
     {11, 3, 2, 6, 9, 8, 10, 1, 0, 13, 5, 4, 12, X_, X_, 7, X_, X_},
     {7, 12, 11, 14, 3, 2, 6, 10, 9, 13, 1, 0, 16, 5, 4, 15, X_, X_, 8, X_, X_},
     {9, 16, 15, 7, 13, 12, 17, 3, 2, 6, 11, 10, 14, 1, 0, 19, 5, 4, 18, X_, X_, 8, X_, X_}},
    {{0},
     {10, 4, 3, 2, 9, 8, 1, X_, X_, 0, X_, X_, 16, 14, 12, 15, 13, 11, 7, 6, 5},
     {5, 12, 11, 13, 4, 3, 2, 10, 9, 1, X_, X_, 0, X_, X_, 19, 17, 15, 18, 16, 14, 8, 7, 6},
     {22, 6, 5, 7, 14, 13, 15, 4, 3, 2, 12, 11, 1, X_, X_, 0, X_, X_, 21, 19, 17, 20, 18, 16, 10, 9, 8},
     {0, 13, 12, 25, 7, 6, 8, 17, 16, 18, 5, 4, 3, 15, 14, 2, X_, X_, 1, X_, X_, 24, 22, 20, 23, 21, 19, 11, 10, 9}}};
static const uint8_t t420_size[2][5] = {{12, 15, 18, 21, 24}, {0, 21, 24, 27, 30}};
#undef X_

/* Tables for 4:2:2 / 4:4:4 with fewer levels than V2/H5: drop the bands the
 * missing levels would have produced, then renumber priorities densely
 * (WeightTable.c:143-335). */
static uint32_t derive_table(const uint8_t* g52, const uint8_t* p52, uint32_t dv, uint32_t dh, uint8_t* g, uint8_t* p) {
    memcpy(g, g52, 30);
    memcpy(p, p52, 30);
    uint32_t n = 30;
    for (int v = 2, h = 5; v > (int)dv;) {
        int rm = h - 1;
        v--;
        uint32_t cnt = n - 3 * (rm + 1);
        for (uint32_t i = 0; i < cnt; i++) { g[3 * rm + i] = g[3 * (rm + 1) + i]; p[3 * rm + i] = p[3 * (rm + 1) + i]; }
        n -= 6;
        for (uint32_t i = 0; i < n; i++) { g[i] = g[i + 3]; p[i] = p[i + 3]; }
    }
    for (int h = 5; h > (int)dh;) {
        h--;
        n -= 3;
        if (h != 1) {
            memmove(g, g + 3, n);
            memmove(p, p + 3, n);
        }
    }
    for (uint32_t i = 0; i < n; i++) {
        for (;;) {
            int found = 0;
            for (uint32_t j = 0; j < n; j++)
                if (p[j] == i) { found = 1; break; }
            if (found) break;
            for (uint32_t j = 0; j < n; j++)
                if (p[j] > i) { p[j]--; break; }
        }
    }
    return n;
}

static int32_t assign_weights(jxs_cfg_t* g, uint32_t fmt) {
    uint8_t gain[30], prio[30];
    uint32_t size = 0;
    if (g->nc != 3) return JXS_E_BAD_PARAM;
    int packed_or_444 = fmt == COLOUR_FORMAT_PLANAR_YUV444_OR_RGB || fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB;
    if (fmt == COLOUR_FORMAT_PLANAR_YUV422 && g->dh == 5) {
        memcpy(gain, t422_g[g->dv], 30); memcpy(prio, t422_p[g->dv], 30); size = tsize_v[g->dv];
    } else if (packed_or_444 && g->dh == 5) {
        memcpy(gain, t444_g[g->dv], 30); memcpy(prio, t444_p[g->dv], 30); size = tsize_v[g->dv];
    } else if (fmt == COLOUR_FORMAT_PLANAR_YUV420) {
        if (g->dv < 1 || g->dh < 1 || !t420_size[g->dv - 1][g->dh - 1]) return JXS_E_BAD_PARAM;
        memcpy(gain, t420_g[g->dv - 1][g->dh - 1], 30); memcpy(prio, t420_p[g->dv - 1][g->dh - 1], 30);
        size = t420_size[g->dv - 1][g->dh - 1];
    } else if (fmt == COLOUR_FORMAT_PLANAR_YUV422) {
        size = derive_table(t422_g[2], t422_p[2], g->dv, g->dh, gain, prio);
    } else if (packed_or_444) {
        size = derive_table(t444_g[2], t444_p[2], g->dv, g->dh, gain, prio);
    } else {
        return JXS_E_BAD_PARAM;
    }
    for (uint32_t i = 0; i < g->nbands; i++) {
        if (g->band[i].gid >= size) return JXS_E_BAD_PARAM;
        g->band[i].gain = gain[g->band[i].gid];
        g->band[i].prio = prio[g->band[i].gid];
    }
    return JXS_OK;
}

static int all_truncated(const jxs_cfg_t* g, uint8_t q, uint8_t r) {
    for (uint32_t i = 0; i < g->nbands; i++)
        if (jxs_truncation(g->band[i].gain, g->band[i].prio, q, r) != JXS_TRUNC_MAX) return 0;
    return 1;
}

static void rc_limits(jxs_cfg_t* g) {
    uint32_t mr = 0;
    for (uint32_t i = 0; i < g->nbands; i++) mr = MAX(mr, g->band[i].prio);
    if (mr < 255) mr += 1;
    if (mr > g->nbands_all - 1) mr = g->nbands_all - 1;
    g->max_r = (uint8_t)mr;
    g->max_q = 31;
    while (g->max_q > 0 && all_truncated(g, g->max_q, g->max_r)) g->max_q--;
    for (uint32_t q = 0; q < 32; q++) {
        g->empty[q] = 0;
        for (uint32_t r = 0; r < 32; r++)
            if (all_truncated(g, (uint8_t)q, (uint8_t)r)) g->empty[q] |= 1u << r;
    }
    uint32_t pk_bits = g->short_hdr ? 40 : 56;
    for (int t = 0; t < 2; t++) g->hdrs_bytes[t] = g->prec_hdr_bytes + DIV_UP(pk_bits * g->pk_exist[t], 8);
}

/* ---- codestream header writer (PackHeaders.c:11-140) ---- */
typedef struct {
    uint8_t* p;
    uint32_t bit;
} hw_t;
static void hw_put(hw_t* w, uint32_t v, uint32_t n) {
    while (n--) {
        uint32_t byte = w->bit >> 3, sh = 7 - (w->bit & 7);
        if (sh == 7) w->p[byte] = 0;
        w->p[byte] |= (uint8_t)(((v >> n) & 1u) << sh);
        w->bit++;
    }
}

static void write_header(jxs_cfg_t* g) {
    hw_t w = {g->hdr, 0};
    hw_put(&w, 0xff10, 16); /* SOC */
    hw_put(&w, 0xff50, 16); /* CAP: 9 capability bits, only 4:2:0 and Rl may be set */
    hw_put(&w, 4, 16);
    hw_put(&w, 0, 4);
    hw_put(&w, g->fmt == COLOUR_FORMAT_PLANAR_YUV420, 1);
    hw_put(&w, 0, 3);
    hw_put(&w, 1, 1);
    w.bit = (w.bit + 7) & ~7u;
    hw_put(&w, 0xff12, 16); /* PIH */
    hw_put(&w, 26, 16);
    hw_put(&w, g->lcod, 32);
    hw_put(&w, 0, 32);      /* Ppih, Plev */
    hw_put(&w, g->W, 16);
    hw_put(&w, g->H, 16);
    hw_put(&w, 0, 16);      /* Cw */
    hw_put(&w, g->pps, 16); /* Hsl */
    hw_put(&w, g->nc, 8);
    hw_put(&w, 4, 8);       /* Ng */
    hw_put(&w, 8, 8);       /* Ss */
    hw_put(&w, g->bw, 8);
    hw_put(&w, g->fq, 4);
    hw_put(&w, 4, 4);       /* Br */
    hw_put(&w, 0, 8);       /* Fslc, Ppoc, Cpih */
    hw_put(&w, g->dh, 4);
    hw_put(&w, g->dv, 4);
    hw_put(&w, !g->short_hdr, 1);
    hw_put(&w, 1, 1);       /* Rl */
    hw_put(&w, g->qpih, 2);
    hw_put(&w, g->fs, 2);
    hw_put(&w, g->rm, 2);
    hw_put(&w, 0xff13, 16); /* CDT */
    hw_put(&w, 2 * g->nc + 2, 16);
    for (uint32_t c = 0; c < g->nc; c++) {
        hw_put(&w, g->depth, 8);
        hw_put(&w, g->comp[c].sx, 4);
        hw_put(&w, g->comp[c].sy, 4);
    }
    hw_put(&w, 0xff14, 16); /* WGT */
    hw_put(&w, 2 * g->nbands + 2, 16);
    for (uint32_t i = 0; i < g->nbands_all; i++) {
        if (g->g2f[i] == JXS_NOBAND) continue;
        hw_put(&w, g->band[g->g2f[i]].gain, 8);
        hw_put(&w, g->band[g->g2f[i]].prio, 8);
    }
    g->hdr_len = (w.bit + 7) >> 3;
}

/* Slice byte budgets: every slice's byte range is fixed by Lcod before any
 * pixel is seen (EncHandle.c:760-809).  The decoder uses the same split to
 * predict where slices start in constant-bit-rate codestreams. */
int32_t jxs_cfg_slices(jxs_cfg_t* g) {
    g->max_slice_budget = 0;
    uint32_t hdrs = g->hdr_len + 2 + 6 * g->nslices;
    if (g->lcod == 0 || hdrs >= g->lcod) return JXS_E_BAD_PARAM;
    uint32_t all = g->lcod - hdrs;
    uint32_t last_prec = g->pps - (g->nslices * g->pps - g->np);
    uint32_t min_prec = all / g->np;
    uint32_t min_slice = min_prec * g->pps;
    uint32_t last_slice = min_prec * last_prec;
    uint32_t left = all - last_slice - min_slice * (g->nslices - 1);
    if (g->nslices > 1) min_slice += (uint32_t)(((uint64_t)left * (g->nslices - 1) * g->pps / g->np) / (g->nslices - 1));
    last_slice += (uint32_t)((uint64_t)left * last_prec / g->np);
    left = all - last_slice - min_slice * (g->nslices - 1);
    uint32_t bytes_left = g->lcod - g->hdr_len, begin = g->hdr_len;
    for (uint32_t i = 0; i < g->nslices; i++) {
        uint32_t sz;
        if (i + 1 != g->nslices) {
            sz = min_slice + (i < left ? 1 : 0) + 6;
            bytes_left -= sz;
        } else {
            sz = bytes_left;
        }
        g->slice_size[i] = sz;
        g->slice_begin[i] = begin;
        begin += sz;
        g->max_slice_budget = MAX(g->max_slice_budget, sz);
    }
    return JXS_OK;
}

int32_t jxs_cfg_encoder(jxs_cfg_t* g, struct svt_jpeg_xs_encoder_api* api) {
    memset(g, 0, sizeof(*g));
    uint32_t nc, sx[JXS_MAXC], sy[JXS_MAXC];
    if (api->input_bit_depth < 8 || api->input_bit_depth > 14) return JXS_E_BAD_PARAM;
    if (jxs_sampling(api->colour_format, &nc, sx, sy)) return JXS_E_BAD_PARAM;
    if (api->ndecomp_v == 0 && api->colour_format == COLOUR_FORMAT_PLANAR_YUV420) return JXS_E_BAD_PARAM;
    if (api->slice_height == 0) return JXS_E_BAD_PARAM;
    if (api->slice_height >= api->source_height) api->slice_height = api->source_height;
    else if (api->ndecomp_v > 31 || api->slice_height % (1u << api->ndecomp_v)) return JXS_E_BAD_PARAM;
    if (api->quantization > 1) return JXS_E_BAD_PARAM;
    if (api->bpp_denominator == 0 || api->bpp_numerator == 0) return JXS_E_BAD_PARAM;
    uint64_t bpf = ((uint64_t)api->source_width * api->source_height * api->bpp_numerator / api->bpp_denominator + 7) / 8;
    if (bpf >= (1ull << 32) || bpf == 0) return JXS_E_BAD_PARAM;
    if (api->cpu_profile > 1) return JXS_E_BAD_PARAM;
    if (api->rate_control_mode >= 4) return JXS_E_BAD_PARAM;
    if (api->coding_vertical_prediction_mode >= 3) return JXS_E_BAD_PARAM;
    if (api->coding_signs_handling > 2) return JXS_E_BAD_PARAM;
    if (api->source_width < 4) return JXS_E_BAD_PARAM;
    if ((api->colour_format == COLOUR_FORMAT_PLANAR_YUV422 || api->colour_format == COLOUR_FORMAT_PLANAR_YUV420) &&
        (api->source_width % 2))
        return JXS_E_BAD_PARAM;
    if (api->colour_format == COLOUR_FORMAT_PLANAR_YUV420 && (api->source_height % 2)) return JXS_E_BAD_PARAM;
    if (api->ndecomp_v > 2 || api->ndecomp_h > 5 || api->ndecomp_h < api->ndecomp_v) return JXS_E_BAD_PARAM;
    if (api->ndecomp_h == 0 && api->ndecomp_v == 0) return JXS_E_BAD_PARAM;
    /* every band must keep at least one sample (EncHandle.c:375-420) */
    uint32_t mw = api->source_width, mh = api->source_height, mv = api->ndecomp_v;
    if (api->colour_format == COLOUR_FORMAT_PLANAR_YUV420) { mw >>= 1; mh >>= 1; mv -= 1; }
    if (api->colour_format == COLOUR_FORMAT_PLANAR_YUV422) mw >>= 1;
    for (uint32_t i = 0; i < api->ndecomp_h; i++) {
        if (mw > 1) mw -= mw / 2;
        else { mw = 0; break; }
    }
    for (uint32_t i = 0; i < mv; i++) {
        if (mh > 1) mh -= mh / 2;
        else { mh = 0; break; }
    }
    if (mw == 0 || mh == 0) return JXS_E_BAD_PARAM;
    if (api->rate_control_mode > 3) return JXS_E_BAD_PARAM;

    /* the reference encoder writes Cw = 0 (EncHandle.c:401) */
    int32_t r = jxs_cfg_geometry(g, 1, nc, api->source_width, api->source_height, api->ndecomp_h, api->ndecomp_v, 0, sx, sy,
                                 api->slice_height, 0);
    if (r) return r;
    g->fmt = api->colour_format;
    g->depth = api->input_bit_depth;
    g->qpih = api->quantization;
    g->sig = !!api->coding_significance;
    g->rc_mode = api->rate_control_mode;
    g->signs = api->coding_signs_handling;
    g->fs = g->signs ? 1 : 0; /* hdr_Fs (EncHandle.c:278) */
    g->vpred = api->coding_vertical_prediction_mode;
    g->rm = g->vpred == 2 ? 1 : 0; /* hdr_Rm (EncHandle.c:250-253) */
    g->bw = 20;
    g->fq = 8;
    g->lcod = (uint32_t)bpf;
    if (assign_weights(g, api->colour_format)) return JXS_E_BAD_PARAM;
    rc_limits(g);
    write_header(g);

    cfg_pk_order(g);
    return jxs_cfg_slices(g);
}

/* ---- decoder header parsing (ParseHeader.c:20-617) ---- */
typedef struct {
    const uint8_t* p;
    size_t n, pos;
} hr_t;
static int hr_has(const hr_t* r, size_t k) { return r->pos + k <= r->n; }
static uint32_t hr_u8(hr_t* r) { return r->p[r->pos++]; }
static uint32_t hr_u16(hr_t* r) { uint32_t v = ((uint32_t)r->p[r->pos] << 8) | r->p[r->pos + 1]; r->pos += 2; return v; }
static uint32_t hr_u32(hr_t* r) { uint32_t v = (hr_u16(r) << 16); return v | hr_u16(r); }

int32_t jxs_cfg_decoder(jxs_cfg_t* g, const uint8_t* bs, size_t size, jxs_hdr_info_t* info) {
    memset(g, 0, sizeof(*g));
    memset(info, 0, sizeof(*info));
    if (!bs || !size) return JXS_E_DEC_PTR;
    hr_t r = {bs, size, 0};
    if (!hr_has(&r, 2)) return JXS_E_DEC_SHORT;
    if (hr_u16(&r) != 0xff10) return JXS_E_DEC_BITSTREAM;
    if (!hr_has(&r, 4)) return JXS_E_DEC_SHORT;
    if (hr_u16(&r) != 0xff50) return JXS_E_DEC_BITSTREAM;
    uint32_t lcap = (hr_u16(&r) - 2) & 0xffff;
    if (lcap * 8 > 16) return JXS_E_DEC_BITSTREAM;
    if (!hr_has(&r, lcap)) return JXS_E_DEC_SHORT;
    r.pos += lcap;
    if (!hr_has(&r, 28)) return JXS_E_DEC_SHORT;
    if (hr_u16(&r) != 0xff12) return JXS_E_DEC_BITSTREAM;
    if (hr_u16(&r) != 26) return JXS_E_DEC_BITSTREAM;
    g->lcod = hr_u32(&r);
    hr_u32(&r); /* Ppih, Plev */
    uint32_t W = hr_u16(&r), H = hr_u16(&r), cw = hr_u16(&r), hsl = hr_u16(&r);
    if (hsl < 1) return JXS_E_DEC_BITSTREAM;
    uint32_t nc = hr_u8(&r);
    if (nc < 1 || nc > 8) return JXS_E_DEC_BITSTREAM;
    if (hr_u8(&r) != 4) return JXS_E_DEC_BITSTREAM;
    if (hr_u8(&r) != 8) return JXS_E_DEC_BITSTREAM;
    g->bw = hr_u8(&r);
    uint32_t v = hr_u8(&r);
    g->fq = v >> 4;
    if (!(g->fq == 0 || (g->bw == 18 && g->fq == 6) || (g->bw == 20 && g->fq == 8))) return JXS_E_DEC_BITSTREAM;
    if ((v & 15) != 4) return JXS_E_DEC_BITSTREAM;
    v = hr_u8(&r);
    if ((v >> 7) != 0 || ((v >> 4) & 7) != 0) return JXS_E_DEC_BITSTREAM;
    info->cpih = v & 15;
    if (info->cpih != 0 && info->cpih != 1 && info->cpih != 3) return JXS_E_DEC_BITSTREAM;
    v = hr_u8(&r);
    uint32_t dh = v >> 4, dv = v & 15;
    v = hr_u8(&r);
    g->lh = v >> 7;
    g->qpih = (v >> 4) & 3;
    g->fs = (v >> 2) & 3;
    g->rm = v & 3;
    if (g->qpih > 1 || g->fs > 1 || g->rm > 1) return JXS_E_DEC_BITSTREAM;
    uint32_t sx[JXS_MAXC] = {1, 1, 1, 1}, sy[JXS_MAXC] = {1, 1, 1, 1}, sd = 0, depth[8] = {0};
    int have_cdt = 0, have_wgt = 0, have_cts = 0, have_crg = 0;
    uint8_t gain[JXS_MAXBL], prio[JXS_MAXBL];
    uint32_t nw = 0;
    for (;;) {
        if (!hr_has(&r, 2)) return JXS_E_DEC_SHORT;
        uint32_t m = hr_u16(&r);
        if (m == 0xff13) {
            if (have_cdt) return JXS_E_DEC_BITSTREAM;
            have_cdt = 1;
            if (!hr_has(&r, nc * 2 + 2)) return JXS_E_DEC_SHORT;
            if (((hr_u16(&r) - 2) & 0xffff) != 2 * nc) return JXS_E_DEC_BITSTREAM;
            if (nc > JXS_MAXC) return JXS_E_DEC_BITSTREAM;
            for (uint32_t c = 0; c < nc; c++) {
                depth[c] = hr_u8(&r);
                if (depth[c] < 8 || depth[c] > 16) return JXS_E_DEC_BITSTREAM;
                v = hr_u8(&r);
                sx[c] = v >> 4;
                sy[c] = v & 15;
            }
        } else if (m == 0xff14) {
            if (have_wgt) return JXS_E_DEC_BITSTREAM;
            have_wgt = 1;
            if (!hr_has(&r, 2)) return JXS_E_DEC_SHORT;
            uint32_t len = (hr_u16(&r) - 2) & 0xffff;
            if (len & 1) return JXS_E_DEC_SHORT;
            nw = len / 2;
            if (nw > JXS_MAXBL) return JXS_E_DEC_BITSTREAM;
            if (!hr_has(&r, len)) return JXS_E_DEC_SHORT;
            for (uint32_t i = 0; i < nw; i++) {
                gain[i] = (uint8_t)hr_u8(&r);
                prio[i] = (uint8_t)hr_u8(&r);
            }
        } else if (m == 0xff16) {
            /* NLT: quadratic (sigma, alpha) or extended (T1, T2, E) output
             * non-linearity (get_nonlinearity, ParseHeader.c:373-405) */
            if (!hr_has(&r, 3)) return JXS_E_DEC_SHORT;
            hr_u16(&r);
            info->tnlt = hr_u8(&r);
            if (info->tnlt == 1) {
                if (!hr_has(&r, 2)) return JXS_E_DEC_SHORT;
                const uint32_t q = hr_u16(&r);
                g->nlt_sigma = q >> 15;
                g->nlt_alpha = q & 0x7fff;
            } else if (info->tnlt == 2) {
                if (!hr_has(&r, 9)) return JXS_E_DEC_SHORT;
                g->nlt_t1 = hr_u32(&r);
                g->nlt_t2 = hr_u32(&r);
                g->nlt_e = hr_u8(&r);
            } else {
                return JXS_E_DEC_BITSTREAM;
            }
            g->tnlt = info->tnlt;
        } else if (m == 0xff17) {
            if (!hr_has(&r, 3)) return JXS_E_DEC_SHORT;
            if (hr_u16(&r) != 3) return JXS_E_DEC_BITSTREAM;
            sd = hr_u8(&r);
        } else if (m == 0xff18) {
            /* CTS: Cf, e1, e2 of the Star-Tetrix transform (get_cts,
             * ParseHeader.c:418-446) */
            if (have_cts) return JXS_E_DEC_BITSTREAM;
            have_cts = 1;
            if (!hr_has(&r, 4)) return JXS_E_DEC_SHORT;
            if (hr_u16(&r) != 4) return JXS_E_DEC_BITSTREAM;
            g->cts_cf = hr_u8(&r) & 15;
            v = hr_u8(&r);
            g->cts_e1 = v >> 4;
            g->cts_e2 = v & 15;
        } else if (m == 0xff19) {
            /* CRG: component registration; the CFA pattern type of
             * get_cfa_pattern (Mct.c:155-178, ParseHeader.c:448-480) */
            if (have_crg) return JXS_E_DEC_BITSTREAM;
            have_crg = 1;
            if (!hr_has(&r, 2 + nc * 4)) return JXS_E_DEC_SHORT;
            if (hr_u16(&r) != 2 + nc * 4 || nc > JXS_MAXC) return JXS_E_DEC_BITSTREAM;
            uint32_t xc[JXS_MAXC], yc[JXS_MAXC];
            for (uint32_t c = 0; c < nc; c++) {
                xc[c] = hr_u16(&r);
                yc[c] = hr_u16(&r);
            }
            g->cfa_type = (nc >= 3 && xc[1] == 32768 && yc[1] == 0 && xc[2] == 0 && yc[2] == 32768) ? 0 : 1;
        } else if (m == 0xff15) {
            if (!hr_has(&r, 4)) return JXS_E_DEC_SHORT;
            uint32_t len = hr_u16(&r);
            hr_u16(&r);
            len = (len - 4) & 0xffff;
            if (!hr_has(&r, len)) return JXS_E_DEC_SHORT;
            r.pos += len;
        } else if (m == 0xff20) {
            r.pos -= 2;
            break;
        } else {
            return JXS_E_DEC_BITSTREAM;
        }
    }
    if (!have_cdt || !have_wgt) return JXS_E_DEC_BITSTREAM;
    if (info->cpih) {
        /* the colour transforms need three (RCT) or four (Star-Tetrix, with
         * its CTS and CRG markers) components of equal sampling
         * (ParseHeader.c:584-604, Mct.c:137-153) */
        if (nc < 3) return JXS_E_DEC_BITSTREAM;
        if (info->cpih == 3 && (nc != 4 || !have_cts || !have_crg)) return JXS_E_DEC_BITSTREAM;
        for (uint32_t c = 1; c < nc; c++)
            if (sx[c] != sx[0] || sy[c] != sy[0]) return JXS_E_DEC_BITSTREAM;
    }
    g->cpih = info->cpih;
    if (dv > 31) return JXS_E_DEC_BITSTREAM;
    int32_t e = jxs_cfg_geometry(g, 0, nc, W, H, dh, dv, sd, sx, sy, hsl * (1u << dv), cw);
    if (e) return e;
    uint32_t k = 0;
    for (uint32_t i = 0; i < g->nbands_all; i++) {
        if (g->g2f[i] == JXS_NOBAND) continue;
        if (k >= nw) return JXS_E_DEC_BITSTREAM;
        g->band[g->g2f[i]].gain = gain[k];
        g->band[g->g2f[i]].prio = prio[k];
        k++;
    }
    g->depth = depth[0];
    if (nc == 3) {
        if (sx[1] == 1 && sx[2] == 1 && sy[1] == 1 && sy[2] == 1) g->fmt = COLOUR_FORMAT_PLANAR_YUV444_OR_RGB;
        else if (sx[1] == 2 && sx[2] == 2 && sy[1] == 1 && sy[2] == 1) g->fmt = COLOUR_FORMAT_PLANAR_YUV422;
        else if (sx[1] == 2 && sx[2] == 2 && sy[1] == 2 && sy[2] == 2) g->fmt = COLOUR_FORMAT_PLANAR_YUV420;
        else return JXS_E_DEC_BITSTREAM;
        if (sx[0] != 1 || sy[0] != 1) return JXS_E_DEC_BITSTREAM;
    } else if (nc == 4) {
        g->fmt = COLOUR_FORMAT_PLANAR_4_COMPONENTS;
    } else if (nc == 1) {
        g->fmt = COLOUR_FORMAT_GRAY;
    } else {
        return JXS_E_DEC_BITSTREAM;
    }
    info->hdr_len = (uint32_t)r.pos;
    info->cw = cw;
    g->hdr_len = (uint32_t)r.pos;
    if (g->hdr_len > sizeof(g->hdr)) return JXS_E_DEC_BITSTREAM;
    memcpy(g->hdr, bs, g->hdr_len);
    /* predicted slice starts for constant-bit-rate streams (checked on use) */
    cfg_pk_order(g);
    if (jxs_cfg_slices(g) != JXS_OK) g->max_slice_budget = 0;
    return JXS_OK;
}

/* Byte offset of every precinct of one picture: walk slice headers and the
 * 24-bit precinct lengths (get_slice_size, DecThreadInit.c:35-131).  Returns
 * the picture size in bytes (through EOC) or 0 with *err set. */
uint32_t jxs_frame_bytes_walk(const jxs_cfg_t* g, const uint8_t* bs, size_t size, uint32_t hdr_len, uint32_t* prec_off,
                              int32_t* err) {
    size_t off = hdr_len;
    *err = JXS_OK;
    for (uint32_t s = 0; s < g->nslices; s++) {
        if (off + 6 > size) { *err = JXS_E_DEC_SHORT; return 0; }
        if (bs[off] != 0xff || bs[off + 1] != 0x20 || bs[off + 2] != 0 || bs[off + 3] != 4 ||
            (((uint32_t)bs[off + 4] << 8) | bs[off + 5]) != s) {
            *err = JXS_E_DEC_BITSTREAM;
            return 0;
        }
        off += 6;
        /* the slice's precincts: rows x columns, row after row */
        uint32_t first = s * g->pps * g->ncol, n = ((s + 1 == g->nslices) ? g->np - s * g->pps : g->pps) * g->ncol;
        for (uint32_t i = 0; i < n; i++) {
            if (off + g->prec_hdr_bytes > size) { *err = JXS_E_DEC_SHORT; return 0; }
            uint32_t lprc = ((uint32_t)bs[off] << 16) | ((uint32_t)bs[off + 1] << 8) | bs[off + 2];
            if (lprc > JXS_PREC_MAX_BYTES) { *err = JXS_E_DEC_BITSTREAM; return 0; }
            if (prec_off) prec_off[first + i] = (uint32_t)off;
            off += g->prec_hdr_bytes + lprc;
            if (off > size) { *err = JXS_E_DEC_SHORT; return 0; }
        }
    }
    if (off + 2 > size) { *err = JXS_E_DEC_SHORT; return 0; }
    if (bs[off] != 0xff || bs[off + 1] != 0x11) { *err = JXS_E_DEC_BITSTREAM; return 0; }
    return (uint32_t)(off + 2);
}

void jxs_print_bands(const jxs_cfg_t* g) {
    printf("bands: %u (codestream order %u)\n", g->nbands, g->nbands_all);
    for (uint32_t c = 0; c < g->nc; c++) {
        const jxs_comp_t* cp = &g->comp[c];
        printf("component %u: %ux%u V%u H%u bands %u\n", c, cp->w, cp->h, cp->dv, cp->dh, cp->nb);
        for (uint32_t i = 0; i < cp->nb; i++) {
            const jxs_band_t* b = &g->band[cp->band0 + i];
            printf("  band %u [global %2u] at %u,%u size %ux%u lines %u gain %u priority %u\n", i, b->gid, b->x, b->y, b->w, b->h,
                   b->lines, b->gain, b->prio);
        }
    }
}
