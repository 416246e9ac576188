/*
 * SvtJpegxsEnc.h - JPEG XS encoder C API.
 *
 * Drop-in boundary for the encoder: svt_jpeg_xs_encoder_api_t and the six
 * entry points below are ABI identical to the reference's
 * Source/API/SvtJpegxsEnc.h (struct :18-93, functions :100-142).  Encoding
 * runs on the GPU; the threading, queueing and callback behaviour of the
 * reference is kept (see each function).
 */
#ifndef _SVT_JPEG_XS_API_ENC_H_
#define _SVT_JPEG_XS_API_ENC_H_

#ifdef __cplusplus
extern "C" {
#endif

#include "SvtJpegxs.h"
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

typedef struct svt_jpeg_xs_encoder_api {
    uint32_t source_width;        /* luma width in pixels (mandatory) */
    uint32_t source_height;       /* luma height in pixels (mandatory) */
    uint8_t input_bit_depth;      /* 8..14 (mandatory) */
    ColourFormat_t colour_format; /* mandatory */
    uint32_t bpp_numerator;       /* bits per pixel = numerator / denominator (mandatory) */
    uint32_t bpp_denominator;     /* default 1 */
    uint32_t ndecomp_v;           /* vertical decomposition levels 0..2, default 2 */
    uint32_t ndecomp_h;           /* horizontal decomposition levels 0..5 (>= ndecomp_v), default 5 */
    uint32_t quantization;        /* 0 deadzone (default), 1 uniform */
    uint32_t slice_height;        /* luma lines per slice, multiple of 2^ndecomp_v, default 16 */
    CPU_FLAGS use_cpu_flags;      /* accepted, ignored (GPU implementation) */
    uint32_t threads_num;         /* accepted, ignored (GPU implementation) */
    uint8_t cpu_profile;          /* 0 low latency, 1 low CPU; both map to the same GPU pipeline */
    uint32_t print_bands_info;    /* print the band layout at init when verbose */
    uint32_t coding_signs_handling;   /* 0 off (default), 1 fast, 2 full */
    uint32_t coding_significance;     /* significance coding allowed, default 1 */
    uint32_t rate_control_mode;       /* 0 CBR per precinct, 1 CBR per precinct moving padding (default),
                                         2 CBR per slice, 3 CBR per slice with max rate */
    uint32_t coding_vertical_prediction_mode; /* 0 off (default) */
    uint32_t verbose;                 /* VerboseMessages */

    /* Called from a library thread when the input queue has room; one call at a time. */
    void (*callback_send_data_available)(struct svt_jpeg_xs_encoder_api* encoder, void* context);
    void* callback_send_data_available_context;
    /* Called from a library thread when an encoded frame is ready; one call at a time. */
    void (*callback_get_data_available)(struct svt_jpeg_xs_encoder_api* encoder, void* context);
    void* callback_get_data_available_context;

    uint8_t slice_packetization_mode; /* 0 whole codestream per packet, 1 one slice per packet (RFC 9134) */

    void* private_ptr; /* owned by the library */
    uint8_t padding[64];
} svt_jpeg_xs_encoder_api_t;

/* Fills enc_api with the default parameters.  Replaces the reference's
 * svt_jpeg_xs_encoder_load_default_parameters (EncHandle.c:490-532). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_load_default_parameters(uint64_t version_api_major, uint64_t version_api_minor,
                                                                         svt_jpeg_xs_encoder_api_t* enc_api);

/* Plane sizes and Lcod (bytes per frame) for a configuration, without an
 * encoder.  Replaces svt_jpeg_xs_encoder_get_image_config (EncHandle.c:537-618). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_get_image_config(uint64_t version_api_major, uint64_t version_api_minor,
                                                                  svt_jpeg_xs_encoder_api_t* enc_api,
                                                                  svt_jpeg_xs_image_config_t* out_image_config,
                                                                  uint32_t* out_bytes_per_frame);

/* Validates the configuration and allocates the GPU resources.  Replaces
 * svt_jpeg_xs_encoder_init (EncHandle.c:623-936). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_init(uint64_t version_api_major, uint64_t version_api_minor,
                                                      svt_jpeg_xs_encoder_api_t* enc_api);

/* Releases everything.  Replaces svt_jpeg_xs_encoder_close (EncHandle.c:938-950). */
PREFIX_API void svt_jpeg_xs_encoder_close(svt_jpeg_xs_encoder_api_t* enc_api);

/* Queues one picture.  The frame struct is copied; the planes must stay
 * valid until the frame is returned by get_packet.  With blocking_flag 0 a
 * full queue returns SvtJxsErrorNoErrorEmptyQueue.  Replaces
 * svt_jpeg_xs_encoder_send_picture (EncHandle.c:955-1018). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_send_picture(svt_jpeg_xs_encoder_api_t* enc_api, svt_jpeg_xs_frame_t* enc_input,
                                                              uint8_t blocking_flag);

/* Returns the next encoded packet in submission order.  With blocking_flag 0
 * and nothing ready it returns SvtJxsErrorNoErrorEmptyQueue and sets
 * user_prv_ctx_ptr to NULL; a frame that failed to encode returns
 * SvtJxsErrorEncodeFrameError.  Replaces svt_jpeg_xs_encoder_get_packet
 * (EncHandle.c:1023-1059). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_get_packet(svt_jpeg_xs_encoder_api_t* enc_api, svt_jpeg_xs_frame_t* enc_output,
                                                            uint8_t blocking_flag);

#ifdef __cplusplus
}
#endif

#endif /* _SVT_JPEG_XS_API_ENC_H_ */
