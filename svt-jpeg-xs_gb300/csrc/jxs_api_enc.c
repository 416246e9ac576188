/*
 * Encoder C API (include/SvtJpegxsEnc.h) on the GPU pipeline.
 *
 * Behaviour follows the reference's Source/Lib/Encoder/Codec/EncHandle.c:
 * parameter validation (:128-454), defaults (:490-532), image config
 * (:537-618), send_picture checks and by-value copy of the frame (:955-1018),
 * get_packet in submission order with SvtJxsErrorEncodeFrameError for failed
 * frames (:1023-1059), and slice packetization (FinalStageProcess.c:148-212).
 */
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "SvtJpegxsEnc.h"
#include "jxs_core.h"
#include "SvtJpegxsGpu.h"
#include "jxs_api_internal.h"
#include "jxs_batch.h"
#include "jxs_gpu.h"
#include "jxs_queue.h"

#define ENC_SLOTS 3

typedef struct enc_prv {
    jxs_cfg_t* cfg;
    jxs_gpu_enc_t* gpu;
    jxs_queue_t q;
    svt_jpeg_xs_frame_t frame[JXS_Q_MAX];
    svt_jpeg_xs_encoder_api_t* api;
    void (*get_cb)(struct svt_jpeg_xs_encoder_api*, void*);
    void* get_ctx;
    void (*send_cb)(struct svt_jpeg_xs_encoder_api*, void*);
    void* send_ctx;
    uint8_t pkt_mode;
    uint32_t pkt_next;    /* next packet of the oldest frame in slice packetization mode */
    uint32_t pkt_offset;
    pthread_mutex_t send_mu;
} enc_prv_t;

static int version_ok(uint64_t major, uint64_t minor) {
    return !(major > SVT_JPEGXS_API_VER_MAJOR || (major == SVT_JPEGXS_API_VER_MAJOR && minor > SVT_JPEGXS_API_VER_MINOR));
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_load_default_parameters(uint64_t version_api_major, uint64_t version_api_minor,
                                                                         svt_jpeg_xs_encoder_api_t* enc_api) {
    if (!version_ok(version_api_major, version_api_minor)) return SvtJxsErrorInvalidApiVersion;
    if (!enc_api) return SvtJxsErrorBadParameter;
    memset(enc_api, 0, sizeof(*enc_api));
    enc_api->colour_format = COLOUR_FORMAT_INVALID;
    enc_api->bpp_denominator = 1;
    enc_api->ndecomp_v = 2;
    enc_api->ndecomp_h = 5;
    enc_api->slice_height = 16;
    enc_api->use_cpu_flags = CPU_FLAGS_ALL;
    enc_api->verbose = VERBOSE_SYSTEM_INFO;
    enc_api->rate_control_mode = 1;
    enc_api->coding_significance = 1;
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_get_image_config(uint64_t version_api_major, uint64_t version_api_minor,
                                                                  svt_jpeg_xs_encoder_api_t* enc_api,
                                                                  svt_jpeg_xs_image_config_t* out, uint32_t* out_bytes_per_frame) {
    if (!version_ok(version_api_major, version_api_minor)) return SvtJxsErrorInvalidApiVersion;
    if (!enc_api || !out) return SvtJxsErrorBadParameter;
    out->width = enc_api->source_width;
    out->height = enc_api->source_height;
    out->bit_depth = enc_api->input_bit_depth;
    out->format = enc_api->colour_format;
    if (out->bit_depth < 8 || out->bit_depth > 14) return SvtJxsErrorBadParameter;
    uint32_t nc, sx[JXS_MAXC], sy[JXS_MAXC];
    if (jxs_sampling(out->format, &nc, sx, sy)) return SvtJxsErrorBadParameter;
    const uint32_t ps = out->bit_depth <= 8 ? 1 : 2;
    if (out->format == COLOUR_FORMAT_PACKED_YUV444_OR_RGB) {
        uint64_t sz = (uint64_t)enc_api->source_width * enc_api->source_height * 3 * ps;
        if (sz > UINT32_MAX) return SvtJxsErrorBadParameter;
        out->components_num = 1;
        out->components[0].width = enc_api->source_width;
        out->components[0].height = enc_api->source_height;
        out->components[0].byte_size = (uint32_t)sz;
    } else {
        out->components_num = (uint8_t)nc;
        for (uint32_t c = 0; c < nc; c++) {
            out->components[c].width = out->width >> (sx[c] - 1);
            out->components[c].height = out->height >> (sy[c] - 1);
            uint64_t sz = (uint64_t)out->components[c].width * out->components[c].height * ps;
            if (sz > UINT32_MAX) return SvtJxsErrorBadParameter;
            out->components[c].byte_size = (uint32_t)sz;
        }
    }
    if (out_bytes_per_frame) {
        if (enc_api->bpp_denominator == 0) return SvtJxsErrorBadParameter;
        *out_bytes_per_frame = (uint32_t)(((uint64_t)enc_api->source_width * enc_api->source_height * enc_api->bpp_numerator /
                                               enc_api->bpp_denominator +
                                           7) /
                                          8);
    }
    return SvtJxsErrorNone;
}

static int32_t enc_wait(void* ctx, int slot) { return jxs_gpu_enc_wait(((enc_prv_t*)ctx)->gpu, slot); }
static void enc_get_cb(void* ctx) {
    enc_prv_t* p = (enc_prv_t*)ctx;
    if (p->get_cb) p->get_cb(p->api, p->get_ctx);
}
static void enc_send_cb(void* ctx) {
    enc_prv_t* p = (enc_prv_t*)ctx;
    if (p->send_cb) p->send_cb(p->api, p->send_ctx);
}

PREFIX_API void svt_jpeg_xs_encoder_close(svt_jpeg_xs_encoder_api_t* enc_api) {
    if (!enc_api || !enc_api->private_ptr) return;
    enc_prv_t* p = (enc_prv_t*)enc_api->private_ptr;
    jxs_queue_shutdown(&p->q);
    jxs_gpu_enc_destroy(p->gpu);
    pthread_mutex_destroy(&p->send_mu);
    free(p->cfg);
    free(p);
    enc_api->private_ptr = NULL;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_init(uint64_t version_api_major, uint64_t version_api_minor,
                                                      svt_jpeg_xs_encoder_api_t* enc_api) {
    if (!version_ok(version_api_major, version_api_minor)) return SvtJxsErrorInvalidApiVersion;
    if (!enc_api) return SvtJxsErrorBadParameter;
    enc_api->private_ptr = NULL;
    if (enc_api->slice_packetization_mode > 1) return SvtJxsErrorBadParameter;
    enc_prv_t* p = (enc_prv_t*)calloc(1, sizeof(enc_prv_t));
    if (!p) return SvtJxsErrorInsufficientResources;
    p->cfg = (jxs_cfg_t*)calloc(1, sizeof(jxs_cfg_t));
    if (!p->cfg) {
        free(p);
        return SvtJxsErrorInsufficientResources;
    }
    int32_t r = jxs_cfg_encoder(p->cfg, enc_api);
    if (r) {
        if (enc_api->verbose >= VERBOSE_ERRORS) fprintf(stderr, "svt-jpeg-xs-gpu: invalid encoder configuration\n");
        free(p->cfg);
        free(p);
        return (SvtJxsErrorType_t)r;
    }
    if (enc_api->print_bands_info && enc_api->verbose > VERBOSE_NONE) jxs_print_bands(p->cfg);
    p->gpu = jxs_gpu_enc_create(p->cfg, ENC_SLOTS, &r);
    if (!p->gpu) {
        free(p->cfg);
        free(p);
        return (SvtJxsErrorType_t)(r ? r : SvtJxsErrorInsufficientResources);
    }
    p->api = enc_api;
    p->get_cb = enc_api->callback_get_data_available;
    p->get_ctx = enc_api->callback_get_data_available_context;
    p->send_cb = enc_api->callback_send_data_available;
    p->send_ctx = enc_api->callback_send_data_available_context;
    p->pkt_mode = enc_api->slice_packetization_mode;
    pthread_mutex_init(&p->send_mu, NULL);
    enc_api->private_ptr = p;
    if (jxs_queue_init(&p->q, ENC_SLOTS, enc_wait, enc_get_cb, enc_send_cb, p)) {
        svt_jpeg_xs_encoder_close(enc_api);
        return SvtJxsErrorInsufficientResources;
    }
    if (enc_api->verbose >= VERBOSE_SYSTEM_INFO) {
        fprintf(stderr, "svt-jpeg-xs-gpu: %ux%u depth %u format %d, %u bytes per frame, %u slices\n", p->cfg->W, p->cfg->H,
                p->cfg->depth, (int)p->cfg->fmt, p->cfg->lcod, p->cfg->nslices);
    }
    return SvtJxsErrorNone;
}

/* send_picture's checks of a frame (EncHandle.c:955-990) */
static SvtJxsErrorType_t check_frame(const jxs_cfg_t* c, const svt_jpeg_xs_frame_t* in) {
    if (in->bitstream.allocation_size < c->lcod || !in->bitstream.buffer) return SvtJxsErrorBadParameter;
    const uint32_t ps = c->depth <= 8 ? 1 : 2;
    for (uint32_t k = 0; k < c->nc; k++) {
        if (!in->image.data_yuv[k]) return SvtJxsErrorBadParameter;
        /* the last row may be shorter than the stride (field-interleaved input) */
        uint64_t min_size = (uint64_t)in->image.stride[k] * ps * (c->comp[k].h - 1) + (uint64_t)c->comp[k].w * ps;
        if (c->fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB)
            min_size = (uint64_t)in->image.stride[0] * ps * (c->H - 1) + (uint64_t)c->W * 3 * ps;
        if (in->image.alloc_size[k] < min_size) return SvtJxsErrorBadParameter;
    }
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_send_picture(svt_jpeg_xs_encoder_api_t* enc_api, svt_jpeg_xs_frame_t* in,
                                                              uint8_t blocking_flag) {
    if (!enc_api || !enc_api->private_ptr || !in) return SvtJxsErrorBadParameter;
    enc_prv_t* p = (enc_prv_t*)enc_api->private_ptr;
    const SvtJxsErrorType_t bad = check_frame(p->cfg, in);
    if (bad) return bad;
    const int slot = jxs_queue_acquire(&p->q, blocking_flag);
    if (slot < 0) return SvtJxsErrorNoErrorEmptyQueue;
    p->frame[slot] = *in;
    /* packed input reads plane 0 only */
    void* planes[4] = {in->image.data_yuv[0], in->image.data_yuv[1], in->image.data_yuv[2], in->image.data_yuv[3]};
    uint32_t strides[4] = {in->image.stride[0], in->image.stride[1], in->image.stride[2], in->image.stride[3]};
    pthread_mutex_lock(&p->send_mu);
    int32_t r = jxs_gpu_enc_submit(p->gpu, slot, planes, strides, in->bitstream.buffer);
    pthread_mutex_unlock(&p->send_mu);
    jxs_queue_submitted(&p->q, slot, r == 0, r ? JXS_E_ENC_FRAME : 0);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_encoder_get_packet(svt_jpeg_xs_encoder_api_t* enc_api, svt_jpeg_xs_frame_t* out,
                                                            uint8_t blocking_flag) {
    if (!enc_api || !enc_api->private_ptr || !out) return SvtJxsErrorBadParameter;
    enc_prv_t* p = (enc_prv_t*)enc_api->private_ptr;
    int32_t err = 0;
    const int slot = jxs_queue_peek_done(&p->q, blocking_flag, &err);
    if (slot < 0) {
        out->user_prv_ctx_ptr = NULL;
        return SvtJxsErrorNoErrorEmptyQueue;
    }
    const jxs_cfg_t* c = p->cfg;
    *out = p->frame[slot];
    if (!p->pkt_mode) {
        out->bitstream.used_size = c->lcod;
        out->bitstream.last_packet_in_frame = 1;
        out->bitstream.ready_to_release = 1;
        out->image.ready_to_release = 1;
        jxs_queue_pop(&p->q);
    } else {
        /* RFC 9134 slice mode: the codestream header, then one packet per
         * slice; the last slice carries the EOC marker */
        if (p->pkt_next == 0) {
            out->bitstream.used_size = c->hdr_len;
            p->pkt_offset = c->hdr_len;
        } else {
            out->bitstream.buffer += p->pkt_offset;
            out->bitstream.used_size = c->slice_size[p->pkt_next - 1];
            p->pkt_offset += out->bitstream.used_size;
        }
        const int last = p->pkt_next == c->nslices;
        out->bitstream.last_packet_in_frame = (uint8_t)last;
        out->bitstream.ready_to_release = (uint8_t)last;
        out->image.ready_to_release = (uint8_t)last;
        if (last) {
            p->pkt_next = 0;
            p->pkt_offset = 0;
            jxs_queue_pop(&p->q);
        } else {
            p->pkt_next++;
        }
    }
    return err ? SvtJxsErrorEncodeFrameError : SvtJxsErrorNone;
}

/* ---- extensions used by tests and tools (declared in SvtJpegxsGpu.h) ---- */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_encoder_rc_results(svt_jpeg_xs_encoder_api_t* enc_api, uint8_t* q, uint8_t* r,
                                                                uint32_t count) {
    if (!enc_api || !enc_api->private_ptr || !q || !r) return SvtJxsErrorBadParameter;
    enc_prv_t* p = (enc_prv_t*)enc_api->private_ptr;
    if (count < p->cfg->np) return SvtJxsErrorBadParameter;
    /* results of the most recently submitted frame */
    int last_slot = -1;
    pthread_mutex_lock(&p->q.mu);
    if (p->q.count > 0) last_slot = p->q.order[(p->q.head + p->q.count - 1) % JXS_Q_MAX];
    pthread_mutex_unlock(&p->q.mu);
    if (last_slot < 0) return SvtJxsErrorNoErrorEmptyQueue;
    return (SvtJxsErrorType_t)jxs_gpu_enc_rc_results(p->gpu, last_slot, q, r);
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_encoder_set_stream(svt_jpeg_xs_encoder_api_t* enc_api, void* cuda_stream) {
    if (!enc_api || !enc_api->private_ptr) return SvtJxsErrorBadParameter;
    jxs_gpu_enc_set_stream(((enc_prv_t*)enc_api->private_ptr)->gpu, cuda_stream);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_encoder_set_streams(svt_jpeg_xs_encoder_api_t* enc_api, void* const* cuda_streams,
                                                                 uint32_t count) {
    if (!enc_api || !enc_api->private_ptr || (count && !cuda_streams)) return SvtJxsErrorBadParameter;
    jxs_gpu_enc_set_streams(((enc_prv_t*)enc_api->private_ptr)->gpu, cuda_streams, (int)count);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_encoder_set_timing(svt_jpeg_xs_encoder_api_t* enc_api, uint32_t enable) {
    if (!enc_api || !enc_api->private_ptr) return SvtJxsErrorBadParameter;
    jxs_gpu_enc_set_timing(((enc_prv_t*)enc_api->private_ptr)->gpu, (int)enable);
    return SvtJxsErrorNone;
}

PREFIX_API uint64_t svt_jpeg_xs_gpu_encoder_read_timing(svt_jpeg_xs_encoder_api_t* enc_api, double* stage_ms, uint32_t n) {
    if (!enc_api || !enc_api->private_ptr || !stage_ms) return 0;
    return jxs_gpu_enc_read_timing(((enc_prv_t*)enc_api->private_ptr)->gpu, stage_ms, (int)n);
}

PREFIX_API uint32_t svt_jpeg_xs_gpu_encoder_read_kernel_timing(svt_jpeg_xs_encoder_api_t* enc_api, double* kernel_ms, uint32_t n) {
    if (!enc_api || !enc_api->private_ptr || !kernel_ms) return 0;
    return (uint32_t)jxs_gpu_enc_read_kernel_timing(((enc_prv_t*)enc_api->private_ptr)->gpu, kernel_ms, (int)n);
}

/* Batched encode (SvtJpegxsGpu.h): frame i with the configuration of
 * enc[i].  The frames are checked as send_picture checks them; none of them
 * goes through the handle's queue, so a handle may serve batches and
 * send_picture alike. */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_encode(svt_jpeg_xs_gpu_batch_t* batch, svt_jpeg_xs_encoder_api_t* const* enc,
                                                          svt_jpeg_xs_frame_t* const* frames, uint32_t n, void* cuda_stream) {
    if (!batch || !enc || !frames || n == 0 || n > SVT_JPEGXS_GPU_BATCH_MAX) return SvtJxsErrorBadParameter;
    jxs_gpu_enc_t* gpu[SVT_JPEGXS_GPU_BATCH_MAX];
    void* planes[SVT_JPEGXS_GPU_BATCH_MAX][4];
    uint32_t strides[SVT_JPEGXS_GPU_BATCH_MAX][4];
    uint8_t* out[SVT_JPEGXS_GPU_BATCH_MAX];
    for (uint32_t i = 0; i < n; i++) {
        if (!enc[i] || !enc[i]->private_ptr || !frames[i]) return SvtJxsErrorBadParameter;
        const enc_prv_t* p = (const enc_prv_t*)enc[i]->private_ptr;
        const SvtJxsErrorType_t bad = check_frame(p->cfg, frames[i]);
        if (bad) return bad;
        gpu[i] = p->gpu;
        for (int k = 0; k < 4; k++) {
            planes[i][k] = frames[i]->image.data_yuv[k];
            strides[i][k] = frames[i]->image.stride[k];
        }
        out[i] = frames[i]->bitstream.buffer;
        /* constant bit rate: every frame is exactly Lcod bytes */
        frames[i]->bitstream.used_size = p->cfg->lcod;
        frames[i]->bitstream.last_packet_in_frame = 1;
    }
    const int32_t r = jxs_gpu_batch_encode((jxs_gpu_batch_t*)batch, gpu, n, (void* const(*)[4])planes,
                                           (const uint32_t(*)[4])strides, out, cuda_stream);
    return (SvtJxsErrorType_t)r;
}

jxs_gpu_enc_t* jxs_api_enc_gpu(svt_jpeg_xs_encoder_api_t* enc_api) {
    if (!enc_api || !enc_api->private_ptr) return NULL;
    return ((enc_prv_t*)enc_api->private_ptr)->gpu;
}
