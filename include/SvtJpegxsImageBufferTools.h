/*
 * SvtJpegxsImageBufferTools.h - helpers that allocate image and bitstream
 * buffers and pools of them.
 *
 * ABI identical to the reference's Source/API/SvtJpegxsImageBufferTools.h
 * (:20-88).  Buffers come from page-locked host memory so that the GPU copies
 * them at full PCIe/C2C speed.
 */
#ifndef _SVT_JPEG_XS_API_IMAGE_BUFFER_TOOLS_H_
#define _SVT_JPEG_XS_API_IMAGE_BUFFER_TOOLS_H_

#include "SvtJpegxs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces svt_jpeg_xs_image_buffer_alloc (ImageBuffer.c:22-91). */
PREFIX_API svt_jpeg_xs_image_buffer_t* svt_jpeg_xs_image_buffer_alloc(svt_jpeg_xs_image_config_t* image_config);

/* Replaces svt_jpeg_xs_image_buffer_free (ImageBuffer.c:93-103). */
PREFIX_API void svt_jpeg_xs_image_buffer_free(svt_jpeg_xs_image_buffer_t* image_buffer);

/* Replaces svt_jpeg_xs_bitstream_alloc (ImageBuffer.c:105-122). */
PREFIX_API svt_jpeg_xs_bitstream_buffer_t* svt_jpeg_xs_bitstream_alloc(uint32_t bitstream_size);

/* Replaces svt_jpeg_xs_bitstream_free (ImageBuffer.c:124-131). */
PREFIX_API void svt_jpeg_xs_bitstream_free(svt_jpeg_xs_bitstream_buffer_t* bitstream);

typedef struct svt_jpeg_xs_frame_pool svt_jpeg_xs_frame_pool_t;

/* Pool of `count` frames, each with image buffers (unless image_config is
 * NULL) and a bitstream buffer (unless bitstream_size is 0).  Replaces
 * svt_jpeg_xs_frame_pool_alloc (ImageBuffer.c:168-244). */
PREFIX_API svt_jpeg_xs_frame_pool_t* svt_jpeg_xs_frame_pool_alloc(const svt_jpeg_xs_image_config_t* image_config,
                                                                  uint32_t bitstream_size, uint32_t count);

/* Replaces svt_jpeg_xs_frame_pool_free (ImageBuffer.c:246-257). */
PREFIX_API void svt_jpeg_xs_frame_pool_free(svt_jpeg_xs_frame_pool_t* frame_pool);

/* Takes a frame from the pool (blocking or SvtJxsErrorNoErrorEmptyQueue).
 * Replaces svt_jpeg_xs_frame_pool_get (ImageBuffer.c:259-305). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_frame_pool_get(svt_jpeg_xs_frame_pool_t* frame_pool, svt_jpeg_xs_frame_t* frame,
                                                        uint8_t blocking_flag);

/* Returns a frame to its pool.  Replaces svt_jpeg_xs_frame_pool_release
 * (ImageBuffer.c:307-318). */
PREFIX_API void svt_jpeg_xs_frame_pool_release(svt_jpeg_xs_frame_pool_t* frame_pool, svt_jpeg_xs_frame_t* frame);

#ifdef __cplusplus
}
#endif

#endif /* _SVT_JPEG_XS_API_IMAGE_BUFFER_TOOLS_H_ */
