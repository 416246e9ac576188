/*
 * Decoder C API (include/SvtJpegxsDec.h) on the GPU pipeline.
 *
 * Behaviour follows the reference's Source/Lib/Decoder/Codec/DecHandle.c:
 * init parses the first header and reports the image configuration
 * (:106-361); send_frame checks the output planes and copies the frame struct
 * (:363-424); pictures whose constant header differs from the one the decoder
 * was initialised with fail with SvtJxsErrorDecoderConfigChange
 * (Decoder.c:377-397); results come back in submission order and
 * SvtJxsDecoderEndOfCodestream follows send_eoc (:466-532).  Packet mode
 * (send_packet) gathers bytes until a whole picture is present.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "SvtJpegxsDec.h"
#include "SvtJpegxsGpu.h"
#include "jxs_core.h"
#include "jxs_api_internal.h"
#include "jxs_batch.h"
#include "jxs_gpu.h"
#include "jxs_queue.h"

#define DEC_SLOTS 3

typedef struct dec_prv {
    jxs_cfg_t* cfg;
    jxs_hdr_info_t info;
    jxs_gpu_dec_t* gpu;
    jxs_queue_t q;
    svt_jpeg_xs_frame_t frame[JXS_Q_MAX];
    int eoc[JXS_Q_MAX];
    uint32_t* prec_off;
    jxs_cfg_t* tmp_cfg;
    svt_jpeg_xs_decoder_api_t* api;
    void (*get_cb)(struct svt_jpeg_xs_decoder_api*, void*);
    void* get_ctx;
    void (*send_cb)(struct svt_jpeg_xs_decoder_api*, void*);
    void* send_ctx;
    uint8_t packet_mode;
    uint8_t* acc;          /* packet mode: bytes of the picture being gathered */
    uint32_t acc_len, acc_cap;
    uint8_t* pkt_bs[JXS_Q_MAX];  /* packet mode: owned copy of each queued picture */
    pthread_mutex_t send_mu;
} dec_prv_t;

static int version_ok(uint64_t major, uint64_t minor) {
    return !(major > SVT_JPEGXS_API_VER_MAJOR || (major == SVT_JPEGXS_API_VER_MAJOR && minor > SVT_JPEGXS_API_VER_MINOR));
}

static void fill_image_config(const jxs_cfg_t* c, svt_jpeg_xs_image_config_t* o) {
    memset(o, 0, sizeof(*o));
    o->width = c->W;
    o->height = c->H;
    o->bit_depth = (uint8_t)c->depth;
    o->format = (ColourFormat_t)c->fmt;
    o->components_num = (uint8_t)c->nc;
    const uint32_t ps = c->depth <= 8 ? 1 : 2;
    /* proxy decoding: the reduced output (ParseHeader.c:813-829) */
    o->width = (c->W + (1u << c->proxy) - 1) >> c->proxy;
    o->height = (c->H + (1u << c->proxy) - 1) >> c->proxy;
    for (uint32_t k = 0; k < c->nc; k++) {
        o->components[k].width = jxs_out_w(c, k);
        o->components[k].height = jxs_out_h(c, k);
        o->components[k].byte_size = jxs_out_w(c, k) * jxs_out_h(c, k) * ps;
    }
}

/* Size of the first picture in the buffer: walks the markers and the
 * precinct lengths up to EOC, or trusts Lcod when fast_search is set and the
 * stream is constant bit rate (ParseHeader.c:650-889). */
static SvtJxsErrorType_t frame_size(const uint8_t* bs, size_t n, svt_jpeg_xs_image_config_t* cfg_out, uint32_t* size,
                                    uint32_t fast, proxy_mode_t proxy) {
    if (!size) return SvtJxsErrorDecoderInvalidPointer;
    if (proxy >= proxy_mode_max) return SvtJxsErrorBadParameter;
    *size = 0;
    if (cfg_out) memset(cfg_out, 0, sizeof(*cfg_out));
    if (!bs || !n) return SvtJxsErrorDecoderInvalidPointer;
    size_t off = 0;
    uint32_t lcod = 0, W = 0, H = 0, depth = 0, sd = 0;
    int nc = -1, dh = -1, dv = -1, started = 0, bands = -1;
    uint32_t sx[8] = {0}, sy[8] = {0};
#define GET16(o) (((uint32_t)bs[(o)] << 8) | bs[(o) + 1])
    for (;;) {
        if (off + 2 > n) return SvtJxsErrorDecoderBitstreamTooShort;
        const uint32_t m = GET16(off);
        if (m == 0xff10) {
            off += 2;
        } else if (m == 0xff12) {
            if (started) return SvtJxsErrorDecoderInvalidBitstream;
            if (off + 28 > n) return SvtJxsErrorDecoderBitstreamTooShort;
            const uint32_t len = GET16(off + 2);
            if (off + len + 2 > n) return SvtJxsErrorDecoderBitstreamTooShort;
            lcod = (GET16(off + 4) << 16) | GET16(off + 6);
            W = GET16(off + 12);
            H = GET16(off + 14);
            nc = bs[off + 20];
            dh = bs[off + 26] >> 4;
            dv = bs[off + 26] & 15;
            off += 2 + len;
        } else if (m == 0xff17 || m == 0xff13 || m == 0xff50 || m == 0xff14 || m == 0xff16 || m == 0xff18 || m == 0xff19 ||
                   m == 0xff15) {
            if (started) return SvtJxsErrorDecoderInvalidBitstream;
            if (off + 4 > n) return SvtJxsErrorDecoderBitstreamTooShort;
            const uint32_t len = GET16(off + 2);
            if (m == 0xff17) sd = bs[off + 4];
            if (m == 0xff13) {
                if (off + len + 2 > n) return SvtJxsErrorDecoderBitstreamTooShort;
                if (nc < 1 || nc > 8 || (uint32_t)(2 * nc + 2) > len) return SvtJxsErrorDecoderInvalidBitstream;
                for (int c = 0; c < nc; c++) {
                    if (c == 0) depth = bs[off + 4];
                    sx[c] = bs[off + 5 + 2 * c] >> 4;
                    sy[c] = bs[off + 5 + 2 * c] & 15;
                }
            }
            off += 2 + len;
        } else if (m == 0xff20) {
            if (off + 6 > n) return SvtJxsErrorDecoderBitstreamTooShort;
            off += 2 + GET16(off + 2);
            if (!started) {
                started = 1;
                if (nc < 1 || dh < 0 || dv < 0 || (int)sd >= nc) return SvtJxsErrorDecoderInvalidBitstream;
                bands = (int)sd;
                for (int c = 0; c < nc - (int)sd; c++) {
                    if (sx[c] < 1 || sy[c] < 1 || sx[c] > 2 || sy[c] > sx[c]) return SvtJxsErrorDecoderInvalidBitstream;
                    const int ny = dv - (int)(sy[c] - 1);
                    if (ny < 0 || ny > dh) return SvtJxsErrorDecoderInvalidBitstream;
                    bands += 2 * ny + dh + 1;
                }
                if (cfg_out) {
                    cfg_out->width = W;
                    cfg_out->height = H;
                    cfg_out->bit_depth = (uint8_t)depth;
                    cfg_out->components_num = (uint8_t)nc;
                    ColourFormat_t f = COLOUR_FORMAT_INVALID;
                    if (nc == 3) {
                        if (sx[1] == 1 && sx[2] == 1 && sy[1] == 1 && sy[2] == 1) f = COLOUR_FORMAT_PLANAR_YUV444_OR_RGB;
                        else if (sx[1] == 2 && sx[2] == 2 && sy[1] == 1 && sy[2] == 1) f = COLOUR_FORMAT_PLANAR_YUV422;
                        else if (sx[1] == 2 && sx[2] == 2 && sy[1] == 2 && sy[2] == 2) f = COLOUR_FORMAT_PLANAR_YUV420;
                    } else if (nc == 4) {
                        f = COLOUR_FORMAT_PLANAR_4_COMPONENTS;
                    } else if (nc == 1) {
                        f = COLOUR_FORMAT_GRAY;
                    }
                    cfg_out->format = f;
                    const uint32_t ss = proxy == proxy_mode_half ? 1 : proxy == proxy_mode_quarter ? 2 : 0;
                    cfg_out->width = (W + (1u << ss) - 1) >> ss;
                    cfg_out->height = (H + (1u << ss) - 1) >> ss;
                    for (int c = 0; c < nc && c < MAX_COMPONENTS_NUM; c++) {
                        uint32_t cw = c < nc - (int)sd ? W >> (sx[c] - 1) : W;
                        uint32_t ch = c < nc - (int)sd ? H >> (sy[c] - 1) : H;
                        cfg_out->components[c].width = (cw + (1u << ss) - 1) >> ss;
                        cfg_out->components[c].height = (ch + (1u << ss) - 1) >> ss;
                        cfg_out->components[c].byte_size =
                            cfg_out->components[c].width * cfg_out->components[c].height * (depth <= 8 ? 1 : 2);
                    }
                }
                if (fast && lcod) {
                    *size = lcod;
                    return SvtJxsErrorNone;
                }
            }
        } else if (m == 0xff11) {
            *size = (uint32_t)(off + 2);
            return SvtJxsErrorNone;
        } else {
            if (!started || bands < 0 || (m >> 12) != 0) return SvtJxsErrorDecoderInvalidBitstream;
            if (off + 3 > n) return SvtJxsErrorDecoderBitstreamTooShort;
            const uint32_t lprc = (m << 8) | bs[off + 2];
            if (lprc > JXS_PREC_MAX_BYTES) return SvtJxsErrorDecoderInvalidBitstream;
            off += lprc + 5 + (uint32_t)((bands * 2 + 7) / 8);
        }
    }
#undef GET16
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_get_single_frame_size_with_proxy(const uint8_t* bitstream_buf,
                                                                                  size_t bitstream_buf_size,
                                                                                  svt_jpeg_xs_image_config_t* out_image_config,
                                                                                  uint32_t* size, uint32_t fast_search,
                                                                                  proxy_mode_t proxy_mode) {
    return frame_size(bitstream_buf, bitstream_buf_size, out_image_config, size, fast_search, proxy_mode);
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_get_single_frame_size(const uint8_t* bitstream_buf, size_t bitstream_buf_size,
                                                                       svt_jpeg_xs_image_config_t* out_image_config,
                                                                       uint32_t* size, uint32_t fast_search) {
    return frame_size(bitstream_buf, bitstream_buf_size, out_image_config, size, fast_search, proxy_mode_full);
}

static int32_t dec_wait(void* ctx, int slot) { return jxs_gpu_dec_wait(((dec_prv_t*)ctx)->gpu, slot); }
static void dec_get_cb(void* ctx) {
    dec_prv_t* p = (dec_prv_t*)ctx;
    if (p->get_cb) p->get_cb(p->api, p->get_ctx);
}
static void dec_send_cb(void* ctx) {
    dec_prv_t* p = (dec_prv_t*)ctx;
    if (p->send_cb) p->send_cb(p->api, p->send_ctx);
}

PREFIX_API void svt_jpeg_xs_decoder_close(svt_jpeg_xs_decoder_api_t* dec_api) {
    if (!dec_api || !dec_api->private_ptr) return;
    dec_prv_t* p = (dec_prv_t*)dec_api->private_ptr;
    jxs_queue_shutdown(&p->q);
    jxs_gpu_dec_destroy(p->gpu);
    pthread_mutex_destroy(&p->send_mu);
    for (int i = 0; i < JXS_Q_MAX; i++) free(p->pkt_bs[i]);
    free(p->acc);
    free(p->prec_off);
    free(p->tmp_cfg);
    free(p->cfg);
    free(p);
    dec_api->private_ptr = NULL;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_init(uint64_t version_api_major, uint64_t version_api_minor,
                                                      svt_jpeg_xs_decoder_api_t* dec_api, const uint8_t* bitstream_buf,
                                                      size_t codestream_size, svt_jpeg_xs_image_config_t* out_image_config) {
    if (!version_ok(version_api_major, version_api_minor)) return SvtJxsErrorInvalidApiVersion;
    if (!dec_api) return SvtJxsErrorBadParameter;
    dec_api->private_ptr = NULL;
    if (!bitstream_buf || !codestream_size) return SvtJxsErrorDecoderInvalidPointer;
    if (dec_api->proxy_mode >= proxy_mode_max) return SvtJxsErrorBadParameter;
    dec_prv_t* p = (dec_prv_t*)calloc(1, sizeof(dec_prv_t));
    if (!p) return SvtJxsErrorInsufficientResources;
    p->cfg = (jxs_cfg_t*)calloc(1, sizeof(jxs_cfg_t));
    p->tmp_cfg = (jxs_cfg_t*)calloc(1, sizeof(jxs_cfg_t));
    if (!p->cfg || !p->tmp_cfg) {
        free(p->cfg);
        free(p->tmp_cfg);
        free(p);
        return SvtJxsErrorInsufficientResources;
    }
    int32_t r = jxs_cfg_decoder(p->cfg, bitstream_buf, codestream_size, &p->info);
    if (r) {
        free(p->cfg);
        free(p->tmp_cfg);
        free(p);
        return (SvtJxsErrorType_t)r;
    }
    /* proxy decoding: every component needs as many vertical and horizontal
     * levels as the output drops (pi_update_proxy_mode, Pi.c:567-626) */
    const uint32_t ss = dec_api->proxy_mode == proxy_mode_half ? 1u : dec_api->proxy_mode == proxy_mode_quarter ? 2u : 0u;
    int proxy_ok = ss <= p->cfg->dv && ss <= p->cfg->dh;
    for (uint32_t k = 0; k < p->cfg->nc; k++) proxy_ok = proxy_ok && ss <= p->cfg->comp[k].dv && ss <= p->cfg->comp[k].dh;
    if (!proxy_ok) {
        if (dec_api->verbose >= VERBOSE_ERRORS)
            fprintf(stderr, "svt-jpeg-xs-gpu: proxy mode %d needs %u decomposition levels in every component\n",
                    (int)dec_api->proxy_mode, ss);
        free(p->cfg);
        free(p->tmp_cfg);
        free(p);
        return SvtJxsErrorBadParameter;
    }
    p->cfg->proxy = ss;
    p->prec_off = (uint32_t*)malloc(sizeof(uint32_t) * p->cfg->nprec);
    p->gpu = jxs_gpu_dec_create(p->cfg, DEC_SLOTS, &r);
    if (!p->gpu || !p->prec_off) {
        jxs_gpu_dec_destroy(p->gpu);
        free(p->prec_off);
        free(p->cfg);
        free(p->tmp_cfg);
        free(p);
        return (SvtJxsErrorType_t)(r ? r : SvtJxsErrorInsufficientResources);
    }
    if (out_image_config) fill_image_config(p->cfg, out_image_config);
    p->api = dec_api;
    p->get_cb = dec_api->callback_get_data_available;
    p->get_ctx = dec_api->callback_get_data_available_context;
    p->send_cb = dec_api->callback_send_data_available;
    p->send_ctx = dec_api->callback_send_data_available_context;
    p->packet_mode = dec_api->packetization_mode;
    pthread_mutex_init(&p->send_mu, NULL);
    dec_api->private_ptr = p;
    if (jxs_queue_init(&p->q, DEC_SLOTS, dec_wait, dec_get_cb, dec_send_cb, p)) {
        svt_jpeg_xs_decoder_close(dec_api);
        return SvtJxsErrorInsufficientResources;
    }
    return SvtJxsErrorNone;
}

/* Parses the picture header, checks it against the stream configuration,
 * finds the precinct offsets and queues the GPU work for `slot`. */
static int32_t submit_picture_locked(dec_prv_t* p, int slot, const uint8_t* bs, uint32_t size, svt_jpeg_xs_frame_t* f) {
    if (!bs || !size) return JXS_E_DEC_PTR;
    if (jxs_gpu_is_device_ptr(bs)) {
        /* codestream already on the GPU: header check and precinct walk run there */
        void* planes[4] = {f->image.data_yuv[0], f->image.data_yuv[1], f->image.data_yuv[2], f->image.data_yuv[3]};
        uint32_t strides[4] = {f->image.stride[0], f->image.stride[1], f->image.stride[2], f->image.stride[3]};
        return jxs_gpu_dec_submit(p->gpu, slot, bs, size, NULL, planes, strides);
    }
    jxs_hdr_info_t info;
    int32_t r = jxs_cfg_decoder(p->tmp_cfg, bs, size, &info);
    if (r) return r;
    /* every header byte but Lcod (bytes 12..15) must match the stream's */
    if (info.hdr_len != p->info.hdr_len || memcmp(bs, p->cfg->hdr, 12) != 0 ||
        memcmp(bs + 16, p->cfg->hdr + 16, info.hdr_len - 16) != 0)
        return JXS_E_DEC_CONFIG;
    int32_t err = 0;
    jxs_frame_bytes_walk(p->cfg, bs, size, info.hdr_len, p->prec_off, &err);
    if (err) return err;
    void* planes[4] = {f->image.data_yuv[0], f->image.data_yuv[1], f->image.data_yuv[2], f->image.data_yuv[3]};
    uint32_t strides[4] = {f->image.stride[0], f->image.stride[1], f->image.stride[2], f->image.stride[3]};
    return jxs_gpu_dec_submit(p->gpu, slot, bs, size, p->prec_off, planes, strides);
}

static int32_t submit_picture(dec_prv_t* p, int slot, const uint8_t* bs, uint32_t size, svt_jpeg_xs_frame_t* f) {
    pthread_mutex_lock(&p->send_mu);
    int32_t r = submit_picture_locked(p, slot, bs, size, f);
    pthread_mutex_unlock(&p->send_mu);
    return r;
}

static SvtJxsErrorType_t check_planes(const dec_prv_t* p, const svt_jpeg_xs_frame_t* f) {
    const jxs_cfg_t* c = p->cfg;
    const uint32_t ps = c->depth <= 8 ? 1 : 2;
    for (uint32_t k = 0; k < c->nc; k++) {
        if (!f->image.data_yuv[k]) return SvtJxsErrorBadParameter;
        uint64_t min_size = (uint64_t)f->image.stride[k] * ps * (jxs_out_h(c, k) - 1) + (uint64_t)jxs_out_w(c, k) * ps;
        if (f->image.alloc_size[k] < min_size) return SvtJxsErrorBadParameter;
    }
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_send_frame(svt_jpeg_xs_decoder_api_t* dec_api, svt_jpeg_xs_frame_t* in,
                                                            uint8_t blocking_flag) {
    if (!dec_api || !dec_api->private_ptr || !in) return SvtJxsErrorDecoderInvalidPointer;
    dec_prv_t* p = (dec_prv_t*)dec_api->private_ptr;
    if (p->packet_mode) return SvtJxsErrorUndefined;
    SvtJxsErrorType_t e = check_planes(p, in);
    if (e) return e;
    const int slot = jxs_queue_acquire(&p->q, blocking_flag);
    if (slot < 0) return SvtJxsErrorNoErrorEmptyQueue;
    p->frame[slot] = *in;
    p->eoc[slot] = 0;
    int32_t r = submit_picture(p, slot, in->bitstream.buffer, in->bitstream.used_size, &p->frame[slot]);
    jxs_queue_submitted(&p->q, slot, r == 0, r);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_send_packet(svt_jpeg_xs_decoder_api_t* dec_api, svt_jpeg_xs_frame_t* in,
                                                             uint32_t* bytes_used) {
    if (!dec_api || !dec_api->private_ptr || !in || !bytes_used) return SvtJxsErrorDecoderInvalidPointer;
    dec_prv_t* p = (dec_prv_t*)dec_api->private_ptr;
    *bytes_used = 0;
    if (!p->packet_mode) return SvtJxsErrorUndefined;
    const uint32_t n = in->bitstream.used_size;
    if (p->acc_len + n > p->acc_cap) {
        uint32_t cap = (p->acc_len + n) * 2;
        uint8_t* a = (uint8_t*)realloc(p->acc, cap);
        if (!a) return SvtJxsErrorInsufficientResources;
        p->acc = a;
        p->acc_cap = cap;
    }
    memcpy(p->acc + p->acc_len, in->bitstream.buffer, n);
    p->acc_len += n;
    *bytes_used = n;
    uint32_t fsize = 0;
    SvtJxsErrorType_t e = frame_size(p->acc, p->acc_len, NULL, &fsize, 0, proxy_mode_full);
    if (e == SvtJxsErrorDecoderBitstreamTooShort) return SvtJxsErrorNone; /* wait for more packets */
    if (e) {
        p->acc_len = 0;
        return SvtJxsErrorDecoderInvalidBitstream;
    }
    e = check_planes(p, in);
    if (e) return e;
    const int slot = jxs_queue_acquire(&p->q, 1);
    if (slot < 0) return SvtJxsErrorUndefined;
    free(p->pkt_bs[slot]);
    p->pkt_bs[slot] = (uint8_t*)malloc(fsize);
    if (!p->pkt_bs[slot]) {
        jxs_queue_submitted(&p->q, slot, 0, SvtJxsErrorInsufficientResources);
        return SvtJxsErrorInsufficientResources;
    }
    memcpy(p->pkt_bs[slot], p->acc, fsize);
    memmove(p->acc, p->acc + fsize, p->acc_len - fsize);
    p->acc_len -= fsize;
    p->frame[slot] = *in;
    p->eoc[slot] = 0;
    int32_t r = submit_picture(p, slot, p->pkt_bs[slot], fsize, &p->frame[slot]);
    jxs_queue_submitted(&p->q, slot, r == 0, r);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_get_frame(svt_jpeg_xs_decoder_api_t* dec_api, svt_jpeg_xs_frame_t* out,
                                                           uint8_t blocking_flag) {
    if (!dec_api || !dec_api->private_ptr || !out) return SvtJxsErrorDecoderInvalidPointer;
    dec_prv_t* p = (dec_prv_t*)dec_api->private_ptr;
    int32_t err = 0;
    const int slot = jxs_queue_peek_done(&p->q, blocking_flag, &err);
    if (slot < 0) {
        out->user_prv_ctx_ptr = NULL;
        return SvtJxsErrorNoErrorEmptyQueue;
    }
    if (p->eoc[slot]) {
        memset(out, 0, sizeof(*out));
        jxs_queue_pop(&p->q);
        return SvtJxsDecoderEndOfCodestream;
    }
    *out = p->frame[slot];
    out->image.ready_to_release = 1;
    out->bitstream.ready_to_release = 1;
    jxs_queue_pop(&p->q);
    return (SvtJxsErrorType_t)err;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_decoder_send_eoc(svt_jpeg_xs_decoder_api_t* dec_api) {
    if (!dec_api || !dec_api->private_ptr) return SvtJxsErrorDecoderInvalidPointer;
    dec_prv_t* p = (dec_prv_t*)dec_api->private_ptr;
    const int slot = jxs_queue_acquire(&p->q, 1);
    if (slot < 0) return SvtJxsErrorUndefined;
    memset(&p->frame[slot], 0, sizeof(p->frame[slot]));
    p->eoc[slot] = 1;
    jxs_queue_submitted(&p->q, slot, 0, 0);
    return SvtJxsErrorNone;
}

/* ---- extensions (declared in SvtJpegxsGpu.h) ---- */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_decoder_set_stream(svt_jpeg_xs_decoder_api_t* dec_api, void* cuda_stream) {
    if (!dec_api || !dec_api->private_ptr) return SvtJxsErrorBadParameter;
    jxs_gpu_dec_set_stream(((dec_prv_t*)dec_api->private_ptr)->gpu, cuda_stream);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_decoder_set_streams(svt_jpeg_xs_decoder_api_t* dec_api, void* const* cuda_streams,
                                                                 uint32_t count) {
    if (!dec_api || !dec_api->private_ptr || (count && !cuda_streams)) return SvtJxsErrorBadParameter;
    jxs_gpu_dec_set_streams(((dec_prv_t*)dec_api->private_ptr)->gpu, cuda_streams, (int)count);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_decoder_set_timing(svt_jpeg_xs_decoder_api_t* dec_api, uint32_t enable) {
    if (!dec_api || !dec_api->private_ptr) return SvtJxsErrorBadParameter;
    jxs_gpu_dec_set_timing(((dec_prv_t*)dec_api->private_ptr)->gpu, (int)enable);
    return SvtJxsErrorNone;
}

PREFIX_API uint64_t svt_jpeg_xs_gpu_decoder_read_timing(svt_jpeg_xs_decoder_api_t* dec_api, double* stage_ms, uint32_t n) {
    if (!dec_api || !dec_api->private_ptr || !stage_ms) return 0;
    return jxs_gpu_dec_read_timing(((dec_prv_t*)dec_api->private_ptr)->gpu, stage_ms, (int)n);
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_decoder_locate_frame(svt_jpeg_xs_decoder_api_t* dec_api, const void* dev_bitstream,
                                                                  uint32_t bitstream_size, uint32_t* frame_size,
                                                                  uint32_t* precinct_offsets, uint32_t precinct_capacity,
                                                                  void* cuda_stream) {
    if (!dec_api || !dec_api->private_ptr || !dev_bitstream || !frame_size) return SvtJxsErrorDecoderInvalidPointer;
    dec_prv_t* p = (dec_prv_t*)dec_api->private_ptr;
    return (SvtJxsErrorType_t)jxs_gpu_dec_locate_noalloc(p->gpu, dev_bitstream, bitstream_size, frame_size, precinct_offsets,
                                                         precinct_capacity, cuda_stream);
}

PREFIX_API uint32_t svt_jpeg_xs_gpu_decoder_read_kernel_timing(svt_jpeg_xs_decoder_api_t* dec_api, double* kernel_ms, uint32_t n) {
    if (!dec_api || !dec_api->private_ptr || !kernel_ms) return 0;
    return (uint32_t)jxs_gpu_dec_read_kernel_timing(((dec_prv_t*)dec_api->private_ptr)->gpu, kernel_ms, (int)n);
}

/* Batched decode (SvtJpegxsGpu.h).  Host codestreams are parsed and walked
 * here as send_frame does (header checked against the decoder's stream,
 * precinct offsets by jxs_frame_bytes_walk); device codestreams are located
 * on the GPU and their headers checked when the batch completes. */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_decode(svt_jpeg_xs_gpu_batch_t* batch, svt_jpeg_xs_decoder_api_t* const* dec,
                                                          svt_jpeg_xs_frame_t* const* frames, uint32_t n, void* cuda_stream) {
    if (!batch || !dec || !frames || n == 0 || n > SVT_JPEGXS_GPU_BATCH_MAX) return SvtJxsErrorBadParameter;
    jxs_gpu_batch_t* b = (jxs_gpu_batch_t*)batch;
    jxs_gpu_dec_t* gpu[SVT_JPEGXS_GPU_BATCH_MAX];
    const uint8_t* bs[SVT_JPEGXS_GPU_BATCH_MAX];
    uint32_t size[SVT_JPEGXS_GPU_BATCH_MAX];
    int walked[SVT_JPEGXS_GPU_BATCH_MAX];
    void* planes[SVT_JPEGXS_GPU_BATCH_MAX][4];
    uint32_t strides[SVT_JPEGXS_GPU_BATCH_MAX][4];
    for (uint32_t i = 0; i < n; i++) {
        if (!dec[i] || !dec[i]->private_ptr || !frames[i]) return SvtJxsErrorDecoderInvalidPointer;
        dec_prv_t* p = (dec_prv_t*)dec[i]->private_ptr;
        if (p->packet_mode) return SvtJxsErrorUndefined;
        const svt_jpeg_xs_frame_t* f = frames[i];
        SvtJxsErrorType_t e = check_planes(p, f);
        if (e) return e;
        gpu[i] = p->gpu;
        bs[i] = f->bitstream.buffer;
        size[i] = f->bitstream.used_size;
        if (!bs[i] || !size[i]) return SvtJxsErrorDecoderInvalidPointer;
        walked[i] = 0;
        if (!jxs_gpu_is_device_ptr(bs[i])) {
            uint32_t* prec = jxs_gpu_batch_prec_buffer(b, i, p->cfg->nprec);
            if (!prec) return SvtJxsErrorInsufficientResources;
            jxs_hdr_info_t info;
            pthread_mutex_lock(&p->send_mu);
            int32_t r = jxs_cfg_decoder(p->tmp_cfg, bs[i], size[i], &info);
            if (!r && (info.hdr_len != p->info.hdr_len || memcmp(bs[i], p->cfg->hdr, 12) != 0 ||
                       memcmp(bs[i] + 16, p->cfg->hdr + 16, info.hdr_len - 16) != 0))
                r = JXS_E_DEC_CONFIG;
            if (!r) jxs_frame_bytes_walk(p->cfg, bs[i], size[i], info.hdr_len, prec, &r);
            pthread_mutex_unlock(&p->send_mu);
            if (r) return (SvtJxsErrorType_t)r;
            walked[i] = 1;
        }
        for (int k = 0; k < 4; k++) {
            planes[i][k] = f->image.data_yuv[k];
            strides[i][k] = f->image.stride[k];
        }
    }
    const int32_t r = jxs_gpu_batch_decode(b, gpu, n, bs, size, walked, (void* const(*)[4])planes, (const uint32_t(*)[4])strides,
                                           cuda_stream);
    return (SvtJxsErrorType_t)r;
}

jxs_gpu_dec_t* jxs_api_dec_gpu(svt_jpeg_xs_decoder_api_t* dec_api) {
    if (!dec_api || !dec_api->private_ptr) return NULL;
    dec_prv_t* p = (dec_prv_t*)dec_api->private_ptr;
    return p->packet_mode ? NULL : p->gpu;
}
