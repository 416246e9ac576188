/*
 * SvtJpegxsDec.h - JPEG XS decoder C API.
 *
 * Drop-in boundary for the decoder: svt_jpeg_xs_decoder_api_t and the entry
 * points below are ABI identical to the reference's Source/API/SvtJpegxsDec.h
 * (struct :16-57, functions :59-148).  Decoding runs on the GPU.
 */
#ifndef _SVT_JPEG_XS_API_DEC_H_
#define _SVT_JPEG_XS_API_DEC_H_

#ifdef __cplusplus
extern "C" {
#endif

#include <stdint.h>
#include <stddef.h>
#include "SvtJpegxs.h"

typedef struct svt_jpeg_xs_decoder_api {
    uint64_t use_cpu_flags; /* accepted, ignored */
    uint32_t verbose;
    uint32_t threads_num;   /* accepted, ignored */
    /* 0: one buffer holds a whole picture (send_frame); 1: pictures arrive as
     * packets (send_packet) and are reassembled inside the library. */
    uint8_t packetization_mode;
    proxy_mode_t proxy_mode;
    void (*callback_send_data_available)(struct svt_jpeg_xs_decoder_api* decoder, void* context);
    void* callback_send_data_available_context;
    void (*callback_get_data_available)(struct svt_jpeg_xs_decoder_api* decoder, void* context);
    void* callback_get_data_available_context;
    void* private_ptr;
    uint8_t padding[64];
} svt_jpeg_xs_decoder_api_t;

/* Parses the first picture header of the codestream, fills out_image_config
 * and allocates the GPU resources.  Replaces svt_jpeg_xs_decoder_init
 * (DecHandle.c:106-361). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_init(uint64_t version_api_major, uint64_t version_api_minor,
                                                      svt_jpeg_xs_decoder_api_t* dec_api, const uint8_t* bitstream_buf,
                                                      size_t codestream_size, svt_jpeg_xs_image_config_t* out_image_config);

/* Replaces svt_jpeg_xs_decoder_close (DecHandle.c:39-104). */
PREFIX_API void svt_jpeg_xs_decoder_close(svt_jpeg_xs_decoder_api_t* dec_api);

/* Size in bytes of the first picture in the buffer.  Replaces
 * svt_jpeg_xs_decoder_get_single_frame_size (DecHandle.c:24-29). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_get_single_frame_size(const uint8_t* bitstream_buf, size_t bitstream_buf_size,
                                                                       svt_jpeg_xs_image_config_t* out_image_config,
                                                                       uint32_t* frame_size, uint32_t fast_search);

/* As above for a proxy (reduced resolution) decode.  Replaces
 * svt_jpeg_xs_decoder_get_single_frame_size_with_proxy (DecHandle.c:31-37). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_get_single_frame_size_with_proxy(const uint8_t* bitstream_buf,
                                                                                  size_t bitstream_buf_size,
                                                                                  svt_jpeg_xs_image_config_t* out_image_config,
                                                                                  uint32_t* frame_size, uint32_t fast_search,
                                                                                  proxy_mode_t proxy_mode);

/* Queues one whole picture for decoding (frame mode).  Replaces
 * svt_jpeg_xs_decoder_send_frame (DecHandle.c:363-424). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_send_frame(svt_jpeg_xs_decoder_api_t* dec_api, svt_jpeg_xs_frame_t* dec_input,
                                                            uint8_t blocking_flag);

/* Feeds part of the codestream (packet mode); bytes_used receives the
 * number of bytes consumed.  Replaces svt_jpeg_xs_decoder_send_packet
 * (DecHandle.c:426-433). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_send_packet(svt_jpeg_xs_decoder_api_t* dec_api, svt_jpeg_xs_frame_t* dec_input,
                                                             uint32_t* bytes_used);

/* Returns the next decoded picture in submission order.  Replaces
 * svt_jpeg_xs_decoder_get_frame (DecHandle.c:435-464). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_get_frame(svt_jpeg_xs_decoder_api_t* dec_api, svt_jpeg_xs_frame_t* dec_output,
                                                           uint8_t blocking_flag);

/* Marks the end of the codestream: get_frame returns
 * SvtJxsDecoderEndOfCodestream once the queue drains.  Replaces
 * svt_jpeg_xs_decoder_send_eoc (DecHandle.c:466-532). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_send_eoc(svt_jpeg_xs_decoder_api_t* dec_api);

#ifdef __cplusplus
}
#endif

#endif /* _SVT_JPEG_XS_API_DEC_H_ */
