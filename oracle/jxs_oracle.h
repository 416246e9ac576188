/*
 * CPU restatement of the SVT-JPEG-XS encode/decode path (test infrastructure).
 *
 * This is the oracle: a plain-C, frame-level restatement of the reference's
 * integer algorithm, used only by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py.  It is pinned against the reference library built
 * from source (oracle/_ref) and against the committed golden fixtures.
 * The product (svt-jpeg-xs_gb300/) never links or calls it.
 */
#ifndef JXS_ORACLE_H
#define JXS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_enc_params {
    uint32_t width, height, bit_depth, colour_format;
    uint32_t bpp_num, bpp_den, decomp_v, decomp_h;
    uint32_t quantization, slice_height, rate_control_mode;
    uint32_t coding_significance, coding_signs_handling, coding_vertical_prediction_mode;
    uint32_t threads_num;
    uint32_t precinct_width; /* Cw: 0 (the reference encoder's only value), or > 0 for
                                multi-column test codestreams */
    /* decoder test codestreams only (the reference encoder writes neither):
     * Cpih = 1 applies the reversible colour transform before the wavelet
     * transform; tnlt 1 / 2 writes an NLT marker (quadratic / extended
     * output non-linearity) with the given parameters */
    uint32_t cpih, tnlt, nlt_sigma, nlt_alpha, nlt_t1, nlt_t2, nlt_e;
    /* Cpih = 3 (Star-Tetrix, 4 components): CTS Cf / e1 / e2 and the CFA
     * pattern type of the CRG marker (0 RGGB-like, 1 GRBG-like); written
     * as is, without the forward transform */
    uint32_t cts_cf, cts_e1, cts_e2, cfa_type;
} or_enc_params_t;

typedef struct or_image_info {
    uint32_t width, height, bit_depth, format, comps;
    uint32_t comp_w[4], comp_h[4];
    uint32_t lcod;
} or_image_info_t;

/* Bytes per frame (Lcod) and the per-component geometry for a configuration. */
int or_frame_size(const or_enc_params_t* p, uint32_t* bytes_per_frame);

/* Encodes one frame.  planes/strides follow the reference image buffer
 * (strides in samples; packed RGB uses plane 0 only).  Returns 0 or an
 * SvtJxsErrorType_t code.  q_out/r_out (optional, one byte per precinct row)
 * receive the chosen quantization and refinement. */
int or_encode(const or_enc_params_t* p, void* const planes[4], const uint32_t strides[4], uint8_t* out, uint32_t out_cap,
              uint32_t* out_size, uint8_t* q_out, uint8_t* r_out);

/* Forward DWT of all components into band-major u16 sign-magnitude
 * coefficients: for each component, bands 0..nb-1, each band h_b rows of w_b
 * samples, contiguous.  Returns the number of coefficients written or <0. */
int64_t or_forward_dwt(const or_enc_params_t* p, void* const planes[4], const uint32_t strides[4], uint16_t* out,
                       uint64_t out_cap);

/* Parses the codestream header. */
int or_probe(const uint8_t* bs, uint32_t size, or_image_info_t* info);

/* Decodes one frame into planes with the given strides (in samples). */
int or_decode(const uint8_t* bs, uint32_t size, void* const planes[4], const uint32_t strides[4], uint32_t threads_num,
              or_image_info_t* info);

#ifdef __cplusplus
}
#endif
#endif
