/*
 * The host side of the IMTL plugin test: the pipeline functions the plugin
 * calls (see plugin_stubs/mtl/st_pipeline_api.h), playing the library's side
 * of its plugin interface, and an entry point that runs frames through the
 * plugin's own encoder or decoder (imtl-plugin/src/st22_svt_jpeg_xs_plugin.c,
 * compiled unchanged into the same test library): st_plugin_create, one
 * session, frames handed out by st22_*_get_frame after notify_frame_available
 * and returned by st22_*_put_frame, then free_session and st_plugin_free.
 * Test infrastructure; frames are host memory, as IMTL's are.
 */
#include <errno.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "mtl/st_pipeline_api.h"

st_plugin_priv st_plugin_create(mtl_handle st);
int st_plugin_free(st_plugin_priv handle);
int st_plugin_get_meta(struct st_plugin_meta* meta);

/* the registered devices (one plugin instance at a time) */
static struct st22_encoder_dev g_edev;
static struct st22_decoder_dev g_ddev;

st22_encoder_dev_handle st22_encoder_register(mtl_handle mt, struct st22_encoder_dev* dev) {
    (void)mt;
    g_edev = *dev;
    return &g_edev;
}
int st22_encoder_unregister(st22_encoder_dev_handle handle) {
    (void)handle;
    return 0;
}
st22_decoder_dev_handle st22_decoder_register(mtl_handle mt, struct st22_decoder_dev* dev) {
    (void)mt;
    g_ddev = *dev;
    return &g_ddev;
}
int st22_decoder_unregister(st22_decoder_dev_handle handle) {
    (void)handle;
    return 0;
}

/* A session's frames: handed out in order, counted back in. */
struct host_session {
    pthread_mutex_t mu;
    pthread_cond_t cv;
    int n, next, done, failed;
    struct st22_encode_frame_meta* emeta;
    struct st22_decode_frame_meta* dmeta;
};

struct st22_encode_frame_meta* st22_encoder_get_frame(st22p_encode_session session) {
    struct host_session* h = (struct host_session*)session;
    pthread_mutex_lock(&h->mu);
    struct st22_encode_frame_meta* f = h->next < h->n ? &h->emeta[h->next++] : NULL;
    pthread_mutex_unlock(&h->mu);
    return f;
}
int st22_encoder_put_frame(st22p_encode_session session, struct st22_encode_frame_meta* frame, int result) {
    (void)frame;
    struct host_session* h = (struct host_session*)session;
    pthread_mutex_lock(&h->mu);
    h->done++;
    if (result) h->failed++;
    pthread_cond_broadcast(&h->cv);
    pthread_mutex_unlock(&h->mu);
    return 0;
}
struct st22_decode_frame_meta* st22_decoder_get_frame(st22p_decode_session session) {
    struct host_session* h = (struct host_session*)session;
    pthread_mutex_lock(&h->mu);
    struct st22_decode_frame_meta* f = h->next < h->n ? &h->dmeta[h->next++] : NULL;
    pthread_mutex_unlock(&h->mu);
    return f;
}
int st22_decoder_put_frame(st22p_decode_session session, struct st22_decode_frame_meta* frame, int result) {
    (void)frame;
    struct host_session* h = (struct host_session*)session;
    pthread_mutex_lock(&h->mu);
    h->done++;
    if (result) h->failed++;
    pthread_cond_broadcast(&h->cv);
    pthread_mutex_unlock(&h->mu);
    return 0;
}

uint8_t st_frame_fmt_planes(enum st_frame_fmt fmt) { return fmt == ST_FRAME_FMT_JPEGXS_CODESTREAM ? 1 : 3; }
size_t st_frame_plane_size(struct st_frame* frame, uint8_t plane) {
    return frame->fmt == ST_FRAME_FMT_JPEGXS_CODESTREAM ? frame->buffer_size : frame->linesize[plane] * frame->height;
}
const char* st_frame_fmt_name(enum st_frame_fmt fmt) {
    return fmt == ST_FRAME_FMT_YUV422PLANAR10LE ? "YUV422PLANAR10LE" : fmt == ST_FRAME_FMT_YUV422PLANAR8 ? "YUV422PLANAR8" : "JPEGXS";
}

/* The plugin's "frame ready" callbacks, which the library calls: the
 * plugin's get thread checks for output, then sleeps until the next call,
 * so a call that lands between the two is not seen until a later frame's.
 * In a live stream later frames come; here the host repeats the call while
 * frames are outstanding. */
struct svt_jpeg_xs_encoder_api;
struct svt_jpeg_xs_decoder_api;
void callback_jpeg_xs_encoder_frame_ready(struct svt_jpeg_xs_encoder_api* encoder, void* priv);
void callback_jpeg_xs_decoder_frame_ready(struct svt_jpeg_xs_decoder_api* decoder, void* priv);

/* waits until every frame came back or `seconds` passed, nudging the
 * plugin's get thread every 20 ms; returns the frames done */
static int wait_done(struct host_session* h, int seconds, void* session, int decoder) {
    struct timespec end;
    clock_gettime(CLOCK_REALTIME, &end);
    end.tv_sec += seconds;
    pthread_mutex_lock(&h->mu);
    while (h->done < h->n) {
        struct timespec ts;
        clock_gettime(CLOCK_REALTIME, &ts);
        if (ts.tv_sec > end.tv_sec || (ts.tv_sec == end.tv_sec && ts.tv_nsec >= end.tv_nsec)) break;
        ts.tv_nsec += 20 * 1000 * 1000;
        if (ts.tv_nsec >= 1000000000L) {
            ts.tv_sec++;
            ts.tv_nsec -= 1000000000L;
        }
        if (pthread_cond_timedwait(&h->cv, &h->mu, &ts) == ETIMEDOUT) {
            pthread_mutex_unlock(&h->mu);
            if (decoder) callback_jpeg_xs_decoder_frame_ready(NULL, session);
            else callback_jpeg_xs_encoder_frame_ready(NULL, session);
            pthread_mutex_lock(&h->mu);
        }
    }
    const int d = h->done;
    pthread_mutex_unlock(&h->mu);
    return d;
}

/* plugin metadata: version and magic */
int mtlh_meta(int* version, unsigned* magic) {
    struct st_plugin_meta m;
    memset(&m, 0, sizeof(m));
    const int r = st_plugin_get_meta(&m);
    *version = m.version;
    *magic = m.magic;
    return r;
}

/* Encodes n frames of 4:2:2 planar video (8 or 10 bit; planes[i * 3 + k],
 * line size in bytes linesize[k]) through the plugin, quality mode
 * `quality`, each into cs[i] of cs_cap bytes; sizes[i] receives its size.
 * Returns the frames completed (n on success) or a negative error. */
int mtlh_encode(int width, int height, int bit_depth, int quality, int n, uint8_t* const* planes, const size_t* linesize,
                size_t codestream_size, uint8_t* const* cs, size_t cs_cap, size_t* sizes) {
    st_plugin_priv plug = st_plugin_create(NULL);
    if (!plug) return -1;
    struct host_session h;
    memset(&h, 0, sizeof(h));
    pthread_mutex_init(&h.mu, NULL);
    pthread_cond_init(&h.cv, NULL);
    struct st_frame* src = (struct st_frame*)calloc((size_t)n, sizeof(struct st_frame));
    struct st_frame* dst = (struct st_frame*)calloc((size_t)n, sizeof(struct st_frame));
    h.emeta = (struct st22_encode_frame_meta*)calloc((size_t)n, sizeof(*h.emeta));
    const enum st_frame_fmt fmt = bit_depth > 8 ? ST_FRAME_FMT_YUV422PLANAR10LE : ST_FRAME_FMT_YUV422PLANAR8;
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < 3; k++) {
            src[i].addr[k] = planes[i * 3 + k];
            src[i].linesize[k] = linesize[k];
        }
        src[i].fmt = fmt;
        src[i].width = (uint32_t)width;
        src[i].height = (uint32_t)height;
        dst[i].addr[0] = cs[i];
        dst[i].fmt = ST_FRAME_FMT_JPEGXS_CODESTREAM;
        dst[i].buffer_size = cs_cap;
        h.emeta[i].src = &src[i];
        h.emeta[i].dst = &dst[i];
    }
    struct st22_encoder_create_req req;
    memset(&req, 0, sizeof(req));
    req.width = (uint32_t)width;
    req.height = (uint32_t)height;
    req.input_fmt = fmt;
    req.output_fmt = ST_FRAME_FMT_JPEGXS_CODESTREAM;
    req.quality = (enum st22_quality_mode)quality;
    req.codec_thread_cnt = 2;
    req.codestream_size = codestream_size;
    st22_encode_priv s = g_edev.create_session(g_edev.priv, &h, &req);
    int done = -2;
    if (s) {
        h.n = n;
        g_edev.notify_frame_available(s); /* the session's handle, as IMTL passes it */
        done = wait_done(&h, 30, s, 0);
        g_edev.free_session(g_edev.priv, s);
        for (int i = 0; i < n; i++) sizes[i] = dst[i].data_size;
        if (h.failed) done = -3;
    }
    st_plugin_free(plug);
    free(src);
    free(dst);
    free(h.emeta);
    return done;
}

/* Decodes n codestreams (cs[i], sizes[i] bytes) through the plugin into
 * 4:2:2 planar frames of the given depth (out[i * 3 + k], line size in bytes
 * linesize[k]).  Returns the frames completed or a negative error. */
int mtlh_decode(int width, int height, int bit_depth, int n, uint8_t* const* cs, const size_t* sizes, size_t cs_cap,
                uint8_t* const* out, const size_t* linesize) {
    st_plugin_priv plug = st_plugin_create(NULL);
    if (!plug) return -1;
    struct host_session h;
    memset(&h, 0, sizeof(h));
    pthread_mutex_init(&h.mu, NULL);
    pthread_cond_init(&h.cv, NULL);
    struct st_frame* src = (struct st_frame*)calloc((size_t)n, sizeof(struct st_frame));
    struct st_frame* dst = (struct st_frame*)calloc((size_t)n, sizeof(struct st_frame));
    h.dmeta = (struct st22_decode_frame_meta*)calloc((size_t)n, sizeof(*h.dmeta));
    const enum st_frame_fmt fmt = bit_depth > 8 ? ST_FRAME_FMT_YUV422PLANAR10LE : ST_FRAME_FMT_YUV422PLANAR8;
    for (int i = 0; i < n; i++) {
        src[i].addr[0] = cs[i];
        src[i].fmt = ST_FRAME_FMT_JPEGXS_CODESTREAM;
        src[i].buffer_size = cs_cap;
        src[i].data_size = sizes[i];
        for (int k = 0; k < 3; k++) {
            dst[i].addr[k] = out[i * 3 + k];
            dst[i].linesize[k] = linesize[k];
        }
        dst[i].fmt = fmt;
        dst[i].width = (uint32_t)width;
        dst[i].height = (uint32_t)height;
        h.dmeta[i].src = &src[i];
        h.dmeta[i].dst = &dst[i];
    }
    struct st22_decoder_create_req req;
    memset(&req, 0, sizeof(req));
    req.width = (uint32_t)width;
    req.height = (uint32_t)height;
    req.input_fmt = ST_FRAME_FMT_JPEGXS_CODESTREAM;
    req.output_fmt = fmt;
    req.codec_thread_cnt = 2;
    st22_decode_priv s = g_ddev.create_session(g_ddev.priv, &h, &req);
    int done = -2;
    if (s) {
        h.n = n;
        g_ddev.notify_frame_available(s);
        done = wait_done(&h, 30, s, 1);
        g_ddev.free_session(g_ddev.priv, s);
        if (h.failed) done = -3;
    }
    st_plugin_free(plug);
    free(src);
    free(dst);
    free(h.dmeta);
    return done;
}
