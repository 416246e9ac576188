/*
 * SvtJpegxsGpu.h - GPU extensions of the JPEG XS C API.
 *
 * These entry points have no counterpart in the reference API; the
 * reference-compatible entry points (SvtJpegxsEnc.h, SvtJpegxsDec.h) need
 * none of them.  They let a caller that already works on the GPU keep its
 * data there and measure the pipeline:
 *  - image planes and bitstream buffers passed to send_picture/send_frame may
 *    be device pointers of the current CUDA device (detected automatically);
 *  - set_stream binds a handle's GPU work to the caller's CUDA stream;
 *  - set_timing / read_timing accumulate per-stage GPU time measured with
 *    CUDA events on the stream the work is launched on.
 */
#ifndef SVT_JPEGXS_GPU_H
#define SVT_JPEGXS_GPU_H

#include "SvtJpegxsDec.h"
#include "SvtJpegxsEnc.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Encoder stages: 0 host-to-device copy, 1 wavelet transform, 2 rate
 * control, 3 quantization and packing, 4 device-to-host copy. */
#define SVT_JPEGXS_GPU_ENC_STAGES 5
/* Decoder stages: 0 host-to-device copy, 1 unpacking and dequantization,
 * 2 inverse wavelet transform and output scaling, 3 device-to-host copy. */
#define SVT_JPEGXS_GPU_DEC_STAGES 4

/* cuda_stream is a cudaStream_t; NULL returns to the handle's own streams
 * (several frames in flight). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_encoder_set_stream(svt_jpeg_xs_encoder_api_t* enc_api, void* cuda_stream);
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_decoder_set_stream(svt_jpeg_xs_decoder_api_t* dec_api, void* cuda_stream);

/* Frame slot i of the handle runs on cuda_streams[i % count] (count = 0:
 * back to the handle's own streams).  A handle keeps 3 frames in flight, so
 * with 3 streams consecutive frames overlap on the device; an encoder and a
 * decoder bound to the same streams put frame i of both on the same stream. */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_encoder_set_streams(svt_jpeg_xs_encoder_api_t* enc_api, void* const* cuda_streams,
                                                                 uint32_t count);
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_decoder_set_streams(svt_jpeg_xs_decoder_api_t* dec_api, void* const* cuda_streams,
                                                                 uint32_t count);

/* Enabling resets the accumulated stage times. */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_encoder_set_timing(svt_jpeg_xs_encoder_api_t* enc_api, uint32_t enable);
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_decoder_set_timing(svt_jpeg_xs_decoder_api_t* dec_api, uint32_t enable);

/* Copies up to n accumulated stage times (milliseconds) and returns the
 * number of frames they cover. */
PREFIX_API uint64_t svt_jpeg_xs_gpu_encoder_read_timing(svt_jpeg_xs_encoder_api_t* enc_api, double* stage_ms, uint32_t n);
PREFIX_API uint64_t svt_jpeg_xs_gpu_decoder_read_timing(svt_jpeg_xs_decoder_api_t* dec_api, double* stage_ms, uint32_t n);

/* Accumulated milliseconds of each kernel launch of a frame, in launch order
 * (timing mode): encoder - the vertical transform levels, the horizontal-
 * only levels, rate control, packing; decoder - the precinct walk (device
 * codestreams only), unpacking, the inverse horizontal-only levels, the
 * inverse vertical levels from the deepest up.  Returns the launches per
 * frame. */
PREFIX_API uint32_t svt_jpeg_xs_gpu_encoder_read_kernel_timing(svt_jpeg_xs_encoder_api_t* enc_api, double* kernel_ms, uint32_t n);
PREFIX_API uint32_t svt_jpeg_xs_gpu_decoder_read_kernel_timing(svt_jpeg_xs_decoder_api_t* dec_api, double* kernel_ms, uint32_t n);

/* Quantization and refinement chosen for each precinct row of the most
 * recently sent picture that has not been returned yet (count >= rows). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_encoder_rc_results(svt_jpeg_xs_encoder_api_t* enc_api, uint8_t* quantization,
                                                                uint8_t* refinement, uint32_t count);

/* Size in bytes (header through EOC) and precinct byte offsets of the frame
 * that starts at dev_bitstream, a device pointer of the current device, read
 * with the configuration the decoder was initialised with.  No counterpart in
 * the reference API: svt_jpeg_xs_decoder_get_single_frame_size answers the
 * size question for host buffers.
 *
 * This entry point allocates nothing, on the device or the host. It is for
 * callers that may not allocate while they run: a receive thread that gets
 * codestreams straight into GPU memory at line rate, or a server held to a
 * device-memory budget fixed at admission. Its scratch is a fixed
 * file-scope device array, so:
 *   - frames of more than 4096 precincts are rejected with
 *     SvtJxsErrorBadParameter (and a message on stderr);
 *   - calls are serialised process-wide, because overlapping walks would
 *     race on the shared scratch;
 *   - the first call on a device resolves the scratch's address and may load
 *     the module, so make it before any stream capture begins.
 * precinct_offsets may be NULL. Otherwise precinct_capacity must be at least
 * the frame's precinct count, and the offsets are written there. The call
 * runs on cuda_stream (NULL: the default stream) and returns when the results
 * are on the host. A header that differs from the decoder's (Lcod aside)
 * returns SvtJxsErrorDecoderConfigChange. */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_decoder_locate_frame(svt_jpeg_xs_decoder_api_t* dec_api, const void* dev_bitstream,
                                                                  uint32_t bitstream_size, uint32_t* frame_size,
                                                                  uint32_t* precinct_offsets, uint32_t precinct_capacity,
                                                                  void* cuda_stream);

/* ------------------------------------------------------------------------
 * Batched form.  A batch object encodes or decodes up to
 * SVT_JPEGXS_GPU_BATCH_MAX frames per call, of any mix of sizes, colour
 * formats and bit depths: frame i uses the configuration of the i-th handle.
 * Each stage runs as one kernel launch over all frames of the batch; the
 * launches are captured into a CUDA graph that is replayed while the batch's
 * buffers and launch parameters stay the same.  Every frame position owns a
 * working set carved from the object's device budget (device_bytes); a
 * batch that does not fit returns SvtJxsErrorInsufficientResources.
 *
 * A batch call queues the work and returns; svt_jpeg_xs_gpu_batch_wait
 * completes it (one batch in flight per object; use several objects to
 * overlap batches).  Planes and codestreams may be host or device memory of
 * the current device.  Outputs are identical, byte for byte, to those of
 * send_picture / send_frame on the same handles.  A batch object is used from
 * one thread at a time.
 * ------------------------------------------------------------------------ */
#define SVT_JPEGXS_GPU_BATCH_MAX 64

typedef struct svt_jpeg_xs_gpu_batch svt_jpeg_xs_gpu_batch_t;

typedef struct svt_jpeg_xs_gpu_batch_info {
    float last_gpu_ms;         /* device time of the last batch (CUDA events around its launches) */
    uint32_t last_launches;    /* kernel launches of the last batch */
    uint64_t graph_hits;       /* batches replayed from a cached graph */
    uint64_t graph_builds;     /* graphs instantiated */
    uint64_t graph_updates;    /* cached graphs updated in place with new parameters */
    int32_t tune[5];           /* launch shapes of the last batch, as for set_tune */
    uint64_t device_bytes, device_used, device_peak; /* device budget */
} svt_jpeg_xs_gpu_batch_info_t;

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_create(uint64_t device_bytes, svt_jpeg_xs_gpu_batch_t** batch);
PREFIX_API void svt_jpeg_xs_gpu_batch_destroy(svt_jpeg_xs_gpu_batch_t* batch);

/* use_graph (default 1): capture and replay CUDA graphs.  autotune (default
 * 0): the first batch of each new composition of handles first times a set
 * of launch shapes and keeps the fastest for that composition (blocking;
 * the outputs of every candidate are identical). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_set_options(svt_jpeg_xs_gpu_batch_t* batch, uint32_t use_graph,
                                                               uint32_t autotune);

/* Fixes the launch shapes of every batch: tune[0] independent chains the
 * frames are split into (1-4), tune[1] frames ordered largest first,
 * tune[2] blocks per SM of the first transform level (0: as many as fit),
 * tune[3] / tune[4] rows per block of the forward / inverse
 * horizontal-only levels (1-4). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_set_tune(svt_jpeg_xs_gpu_batch_t* batch, const int32_t* tune);

/* Encodes frames[i] with enc[i]'s configuration into frames[i]->bitstream
 * (used_size is set to the frame size). */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_encode(svt_jpeg_xs_gpu_batch_t* batch, svt_jpeg_xs_encoder_api_t* const* enc,
                                                          svt_jpeg_xs_frame_t* const* frames, uint32_t n, void* cuda_stream);

/* Decodes frames[i]->bitstream (used_size bytes) with dec[i]'s stream
 * configuration into frames[i]->image. */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_decode(svt_jpeg_xs_gpu_batch_t* batch, svt_jpeg_xs_decoder_api_t* const* dec,
                                                          svt_jpeg_xs_frame_t* const* frames, uint32_t n, void* cuda_stream);

/* Blocks until the batch in flight completes.  status (may be NULL) receives
 * SVT_JPEGXS_GPU_BATCH_MAX entries, the first n of them the per-frame
 * results; returns the first error, or SvtJxsErrorNone. */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_wait(svt_jpeg_xs_gpu_batch_t* batch, SvtJxsErrorType_t* status);

/* 1 when no batch is in flight or it has completed. */
PREFIX_API uint32_t svt_jpeg_xs_gpu_batch_ready(svt_jpeg_xs_gpu_batch_t* batch);

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_get_info(svt_jpeg_xs_gpu_batch_t* batch, svt_jpeg_xs_gpu_batch_info_t* info);

#ifdef __cplusplus
}
#endif

#endif /* SVT_JPEGXS_GPU_H */
