/*
 * Internal configuration shared by the host C code and the CUDA kernels.
 *
 * A jxs_cfg_t describes one stream configuration: picture geometry, the band
 * and precinct layout of ISO/IEC 21122 (restating the reference's pi_t,
 * Source/Lib/Common/Codec/Pi.h:141-180), the weight tables, rate-control
 * limits, the cached codestream header and the per-slice byte budgets.  It is
 * plain data so it can be copied to device memory as-is.
 *
 * Device data layout ("band-planar"): every band of every component is a 2-D
 * array covering the whole frame, `h` rows of `pitch` 16-bit sign-magnitude
 * coefficients (`pitch` a multiple of 8 so rows are 16-byte aligned), at
 * element offset `coef_off` of one frame buffer.  Precinct row p holds band
 * rows [p * lines, p * lines + lines_in_precinct).  GCLIs (one byte per group
 * of 4 coefficients) use the same layout with row pitch `gpitch`.
 */
#ifndef JXS_CORE_H
#define JXS_CORE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JXS_MAXC 4
#define JXS_MAXB 10   /* bands per component */
#define JXS_MAXBL 40  /* bands per picture */
#define JXS_MAXPK 30  /* packets per precinct */
#define JXS_NOBAND 0xff
#define JXS_TRUNC_MAX 15
#define JXS_PREC_MAX_BYTES 1048575u

/* error codes (SvtJxsErrorType_t values) */
#define JXS_OK 0
#define JXS_E_BAD_PARAM ((int32_t)0x80001005)
#define JXS_E_RESOURCES ((int32_t)0x80001000)
#define JXS_E_UNDEFINED ((int32_t)0x80001001)
#define JXS_E_ENC_FRAME ((int32_t)0x80002035)
#define JXS_E_DEC_PTR ((int32_t)0x80003000)
#define JXS_E_DEC_BITSTREAM ((int32_t)0x80003001)
#define JXS_E_DEC_INTERNAL ((int32_t)0x80003002)
#define JXS_E_DEC_SHORT ((int32_t)0x80003003)
#define JXS_E_DEC_CONFIG ((int32_t)0x80003004)
/* internal, never returned to a caller: a precinct uses vertical prediction,
 * which the per-precinct unpacking cannot resolve; the frame is decoded
 * again slice by slice */
#define JXS_E_DEC_VPRED ((int32_t)0x800030ff)

typedef struct jxs_band {
    uint32_t w, h;              /* band size over the whole component */
    uint32_t x, y;              /* position in the component's wavelet plane */
    uint32_t lines;             /* band lines per precinct row */
    uint32_t last_lines;        /* band lines in the last precinct row */
    uint32_t gcli_w, sig_w;     /* code groups / significance groups per line */
    uint32_t pitch, gpitch;     /* coefficient / GCLI row pitch */
    uint32_t cwn, cwl;          /* coefficients per line in a normal / the last precinct column (w when Cw = 0) */
    uint64_t coef_off, gcli_off;
    uint8_t gain, prio, comp, idx;
    uint32_t gid;               /* position in the codestream band order */
} jxs_band_t;

typedef struct jxs_comp {
    uint32_t w, h, sx, sy, dv, dh, nb;
    uint32_t band0;             /* flat index of band 0 of this component */
} jxs_comp_t;

typedef struct jxs_packet {
    uint32_t bs, be, line;      /* global band range [bs, be) and band line */
} jxs_packet_t;

/* One band line of a precinct row, in codestream order (packet order, then
 * band order inside the packet).  Its GCLI groups are split into segments
 * of jxs_cfg_t.seg_groups groups that the kernels process one warp each. */
#define JXS_MAXBLINES 80
#define JXS_MAXSEG 512
typedef struct jxs_bline {
    uint8_t fb, line, pk, pad;  /* flat band, line inside the precinct row, packet */
    uint32_t gcli_w, sig_w, w;  /* groups, significance groups, coefficients */
    uint32_t seg0, nseg;        /* its segments */
    uint32_t gbase;             /* its first group in the precinct's band-line order */
} jxs_bline_t;
typedef struct jxs_seg {
    uint16_t bl, pad;           /* band line */
    uint32_t g0;                /* first group, a multiple of seg_groups */
} jxs_seg_t;

typedef struct jxs_cfg {
    uint32_t W, H, nc, fmt, depth, sd;
    uint32_t dv, dh, prec_h, slice_h, pps, np, nslices;
    uint32_t cw, ncol, nprec;   /* precinct width Cw, precincts per row (Cw = 0: 1), precincts (np rows x ncol) */
    uint32_t nbands_all, nbands;
    uint8_t g2f[JXS_MAXBL];     /* global band -> flat band index */
    jxs_comp_t comp[JXS_MAXC];
    jxs_band_t band[JXS_MAXBL];
    uint32_t npk;
    jxs_packet_t pk[JXS_MAXPK];
    uint32_t short_hdr, lh;
    uint32_t pk_exist[2];                /* packets present: normal / last precinct row */
    uint32_t raw_bytes[4][JXS_MAXPK];    /* raw-mode GCLI sub-packet bytes per precinct kind (jxs_pkind) */
    uint32_t prec_hdr_bytes;             /* ceil((40 + 2 * nbands) / 8) */
    uint32_t hdrs_bytes[2];              /* precinct header + packet headers */
    uint32_t qpih, sig, rc_mode, fs, rm, bw, fq;
    uint32_t signs;                      /* encoder sign handling: 0 off, 1 fast, 2 full */
    uint32_t vpred;                      /* encoder vertical prediction: 0 off, 1 (Rm 0), 2 (Rm 1, zero coefficients) */
    uint8_t max_q, max_r;
    uint32_t empty[32];                  /* bit r of empty[q]: every band fully truncated */
    uint32_t lcod;
    uint8_t hdr[512];
    uint32_t hdr_len;
    uint64_t coef_total, gcli_total;     /* per-frame buffer sizes (elements / bytes) */
    /* tables per precinct kind (jxs_pkind): normal, last row, last column,
     * last row and column */
    uint32_t nbline[4];                  /* band lines */
    jxs_bline_t bline[4][JXS_MAXBLINES];
    uint8_t pk_bl0[4][JXS_MAXPK];        /* first band line of each packet (its count in pk_nbl; 0: absent) */
    uint8_t pk_nbl[4][JXS_MAXPK];
    uint8_t pk_order[4][JXS_MAXBLINES];  /* band lines of each packet (from pk_bl0) in ascending band priority */
    /* vertical prediction: the band line above each band line (same band,
     * line - 1 in the same precinct; for line 0 the band's last line in the
     * precinct row above, a normal row), and where its GCLIs start */
    uint8_t top_bl[4][JXS_MAXBLINES];    /* band line index (in the normal row's table when top_prev) */
    uint8_t top_prev[4][JXS_MAXBLINES];  /* 1: in the precinct row above */
    uint32_t top_gbase[4][JXS_MAXBLINES];
    uint32_t seg_groups;                 /* groups per segment, a multiple of 32 */
    uint32_t nseg[4];
    jxs_seg_t seg[4][JXS_MAXSEG];
    uint16_t seg_ord[4][JXS_MAXSEG];     /* segments by decreasing group count (warp work queues) */
    uint32_t max_slice_budget;           /* 0 when slice starts cannot be predicted (decoder) */
    uint32_t proxy;                      /* decoder: output at 1/2^proxy resolution (proxy modes, Pi.c:567-626) */
    /* decoder: colour transform Cpih (0 none, 1 reversible RCT) and the NLT
     * marker's output non-linearity (0 linear, 1 quadratic, 2 extended) */
    uint32_t cpih, tnlt, nlt_sigma, nlt_alpha, nlt_e;
    uint32_t nlt_t1, nlt_t2;
    uint32_t cts_cf, cts_e1, cts_e2, cfa_type; /* Star-Tetrix (Cpih = 3): CTS marker, CFA pattern type from CRG */
    uint32_t slice_size[8192];           /* bytes of each slice incl. its header (last: incl. EOC) */
    uint32_t slice_begin[8192];          /* byte offset of each slice in the codestream */
} jxs_cfg_t;

/* Decoded output size of component k: full size, or the proxy resolution
 * (Pi.c:599-615, ParseHeader.c:813-829). */
static inline uint32_t jxs_out_w(const jxs_cfg_t* c, uint32_t k) {
    return (c->comp[k].w + (1u << c->proxy) - 1) >> c->proxy;
}
static inline uint32_t jxs_out_h(const jxs_cfg_t* c, uint32_t k) {
    return (c->comp[k].h + (1u << c->proxy) - 1) >> c->proxy;
}

/* Decoder-side header fields beyond the geometry. */
typedef struct jxs_hdr_info {
    uint32_t hdr_len;
    uint32_t cw, cpih, tnlt;
} jxs_hdr_info_t;

struct svt_jpeg_xs_encoder_api;

#ifdef __CUDACC__
#define JXS_HD __host__ __device__
#else
#define JXS_HD
#endif

/* compute_truncation (Source/Lib/Common/Codec/EncDec.c:8-21) */
static inline JXS_HD uint8_t jxs_truncation(uint8_t gain, uint8_t prio, uint8_t q, uint8_t r) {
    uint8_t up = prio < r ? 1 : 0;
    if (q < gain + up) return 0;
    uint8_t t = (uint8_t)(q - gain - up);
    return t > JXS_TRUNC_MAX ? JXS_TRUNC_MAX : t;
}

int32_t jxs_cfg_encoder(jxs_cfg_t* cfg, struct svt_jpeg_xs_encoder_api* api);
int32_t jxs_cfg_slices(jxs_cfg_t* cfg);
int32_t jxs_cfg_decoder(jxs_cfg_t* cfg, const uint8_t* bs, size_t size, jxs_hdr_info_t* info);
/* A precinct's kind: bit 0 the last row, bit 1 the last of several columns
 * (PRECINCT_NORMAL / _LAST_NORMAL / _NORMAL_LAST / _LAST, Pi.h); p counts
 * precincts row after row, ncol per row. */
static inline JXS_HD int jxs_pkind(const jxs_cfg_t* c, uint32_t p) {
    const uint32_t row = p / c->ncol, col = p - row * c->ncol;
    return (row + 1 >= c->np ? 1 : 0) | (c->ncol > 1 && col + 1 == c->ncol ? 2 : 0);
}

/* The encoder's per-segment histograms, written by the rate control for
 * packing (segments of at most 128 groups, so that every count fits a byte):
 * 8 words per segment of every precinct row, after the rate-control tables
 * (cost tables, exact-sign tables, vertical-prediction line tables).  Words
 * 0-3: the segment's GCLI histogram, bin v in byte v & 3 of word v >> 2;
 * words 4-7: its groups by the maximum GCLI of their significance group,
 * same layout. */
#define JXS_SEGHIST_WORDS 8
static inline JXS_HD uint32_t jxs_seg_cap(const jxs_cfg_t* c) {
    uint32_t n = 1;
    for (int k = 0; k < 4; k++) n = c->nseg[k] > n ? c->nseg[k] : n;
    return n;
}
static inline JXS_HD uint64_t jxs_seghist_word(const jxs_cfg_t* c) {
    return (uint64_t)c->np * 1024 * (c->fs ? 2 : 1) + (c->vpred ? (uint64_t)c->np * 5 * JXS_MAXBLINES * 16 : 0);
}

int32_t jxs_cfg_geometry(jxs_cfg_t* cfg, int for_encoder, uint32_t nc, uint32_t W, uint32_t H, uint32_t dh, uint32_t dv,
                         uint32_t sd, const uint32_t sx[JXS_MAXC], const uint32_t sy[JXS_MAXC], uint32_t slice_h, uint32_t cw);
int32_t jxs_sampling(uint32_t fmt, uint32_t* nc, uint32_t sx[JXS_MAXC], uint32_t sy[JXS_MAXC]);
uint32_t jxs_frame_bytes_walk(const jxs_cfg_t* cfg, const uint8_t* bs, size_t size, uint32_t hdr_len, uint32_t* prec_off,
                              int32_t* err);
void jxs_print_bands(const jxs_cfg_t* cfg);

#ifdef __cplusplus
}
#endif

#endif /* JXS_CORE_H */
