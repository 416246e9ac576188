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
 *     the module, so make it before any stream capture begins;
 *   - the decoder and dev_bitstream must be on the current device, which
 *     must be the decoder's; otherwise SvtJxsErrorDecoderInvalidPointer.
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

/* Stage timing.  While on, batches are issued without graphs, with a CUDA
 * event pair around every kernel launch on the launch's stream (set one
 * chain with set_tune to time the stages one after another).  After the
 * wait of such a batch, read_stage_times gives each launch's stage
 * (SVT_JPEGXS_GPU_STAGE_*), variant and device milliseconds, at most `max`
 * entries, and returns their number (0 while a batch is in flight).
 * Variant: for the transform stages the sample kind read or written (0: the
 * 32-bit low band of the next level, 1 / 2: 8- / 16-bit planar, 3 / 4:
 * packed); for rate control and packing bit 0 sign handling and bit 1
 * vertical prediction. */
#define SVT_JPEGXS_GPU_STAGE_FWD_V 0  /* vertical level and the horizontal level after it */
#define SVT_JPEGXS_GPU_STAGE_FWD_H 1  /* horizontal-only levels */
#define SVT_JPEGXS_GPU_STAGE_RC 2     /* rate control */
#define SVT_JPEGXS_GPU_STAGE_PACK 3
#define SVT_JPEGXS_GPU_STAGE_WALK 4   /* precinct offsets of device codestreams */
#define SVT_JPEGXS_GPU_STAGE_UNPACK 5
#define SVT_JPEGXS_GPU_STAGE_INV_H 6
#define SVT_JPEGXS_GPU_STAGE_INV_V 7
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_set_stage_timing(svt_jpeg_xs_gpu_batch_t* batch, uint32_t on);
PREFIX_API uint32_t svt_jpeg_xs_gpu_batch_read_stage_times(svt_jpeg_xs_gpu_batch_t* batch, int32_t* stage, int32_t* variant,
                                                           float* ms, uint32_t max);

/* ------------------------------------------------------------------------
 * Serving loop.  Encode and decode requests from many streams are run by a
 * scheduler thread of the library:
 *   SVT_JPEGXS_GPU_SERVER_BATCHED: continuous batching.  `lanes` encode
 *     lanes and `lanes` decode lanes (CUDA streams) each take the waiting
 *     requests of their kind, oldest first, up to max_batch and as many as
 *     the device budget (device_bytes) admits, as one batch; requests that
 *     arrive while the lanes are busy join the next batch.  A request that
 *     can never fit completes with SvtJxsErrorInsufficientResources.
 *   SVT_JPEGXS_GPU_SERVER_PER_FRAME: the plain per-frame path; each request
 *     goes to a free frame slot of its stream's handle when it arrives.
 * A stream is one encoder or decoder handle (its configuration); register
 * all streams before the first submit, and do not use those handles for
 * send_picture / send_frame while the server runs.  Planes and codestreams
 * of requests are device memory of the current device and stay untouched
 * by the caller until the request completes.  Outputs are identical to those
 * of the same handles' send_picture / send_frame.
 * ------------------------------------------------------------------------ */
#define SVT_JPEGXS_GPU_SERVER_BATCHED 0
#define SVT_JPEGXS_GPU_SERVER_PER_FRAME 1

typedef struct svt_jpeg_xs_gpu_server svt_jpeg_xs_gpu_server_t;

typedef struct svt_jpeg_xs_gpu_request {
    int32_t stream;            /* id from add_encoder / add_decoder */
    uint64_t tag;              /* returned with the completion */
    void* planes[4];           /* encode: input planes; decode: output planes */
    uint32_t strides[4];       /* samples */
    void* bitstream;           /* encode: output (Lcod bytes); decode: input */
    uint32_t bitstream_size;   /* decode: codestream bytes */
} svt_jpeg_xs_gpu_request_t;

typedef struct svt_jpeg_xs_gpu_completion {
    uint64_t tag;
    int32_t stream;
    SvtJxsErrorType_t status;
    int64_t t_arrive_ns;       /* submit, host steady clock */
    int64_t t_start_ns;        /* launched on the device */
    int64_t t_done_ns;         /* completion seen by the scheduler */
} svt_jpeg_xs_gpu_completion_t;

typedef struct svt_jpeg_xs_gpu_server_stats {
    uint64_t batches, batched_frames, max_batch_seen;
    uint64_t deferred;         /* admissions postponed for lack of device memory */
    uint64_t device_bytes, device_used, device_peak;
} svt_jpeg_xs_gpu_server_stats_t;

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_server_create(uint64_t device_bytes, uint32_t mode, uint32_t lanes,
                                                           uint32_t max_batch, svt_jpeg_xs_gpu_server_t** server);
PREFIX_API void svt_jpeg_xs_gpu_server_destroy(svt_jpeg_xs_gpu_server_t* server);
/* Return the stream id, or -1. */
PREFIX_API int32_t svt_jpeg_xs_gpu_server_add_encoder(svt_jpeg_xs_gpu_server_t* server, svt_jpeg_xs_encoder_api_t* enc_api);
PREFIX_API int32_t svt_jpeg_xs_gpu_server_add_decoder(svt_jpeg_xs_gpu_server_t* server, svt_jpeg_xs_decoder_api_t* dec_api);
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_server_submit(svt_jpeg_xs_gpu_server_t* server, const svt_jpeg_xs_gpu_request_t* req);
/* Moves up to max completions to out, oldest first; returns how many. */
PREFIX_API uint32_t svt_jpeg_xs_gpu_server_poll(svt_jpeg_xs_gpu_server_t* server, svt_jpeg_xs_gpu_completion_t* out, uint32_t max);
/* Requests submitted and not yet completed. */
PREFIX_API uint64_t svt_jpeg_xs_gpu_server_pending(svt_jpeg_xs_gpu_server_t* server);
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_server_get_stats(svt_jpeg_xs_gpu_server_t* server,
                                                              svt_jpeg_xs_gpu_server_stats_t* stats);

#ifdef __cplusplus
}
#endif

#endif /* SVT_JPEGXS_GPU_H */
