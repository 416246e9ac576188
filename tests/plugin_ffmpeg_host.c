/*
 * The host side of the FFmpeg plugin test: the FFmpeg functions the plugin
 * calls (see plugin_stubs/ffstub.h), and entry points that drive the
 * plugin's own encoder and decoder (ffmpeg-plugin/libsvtjpegxs{enc,dec}.c,
 * compiled unchanged into the same test library) the way libavcodec does:
 * private context from priv_data_size, options set from the codec's AVOption
 * table, init, one encode / decode call per frame, close.  Test
 * infrastructure; planes are host memory, as AVFrame buffers are.
 */
#include <stdarg.h>
#include <stdio.h>

#include "ffstub.h"

extern const FFCodec ff_libsvtjpegxs_encoder;
extern const FFCodec ff_libsvtjpegxs_decoder;

const char* av_default_item_name(void* ctx) {
    (void)ctx;
    return "libsvtjpegxs";
}
void av_log(void* avcl, int level, const char* fmt, ...) {
    (void)avcl;
    if (level > AV_LOG_ERROR) return;
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
}
int av_log_get_level(void) { return AV_LOG_INFO; }
int av_cpu_count(void) { return 4; }
void* av_malloc(size_t size) { return malloc(size); }
void av_free(void* ptr) { free(ptr); }
int ff_alloc_packet(AVCodecContext* avctx, AVPacket* avpkt, int64_t size) {
    (void)avctx;
    avpkt->data = (uint8_t*)malloc((size_t)size);
    avpkt->size = (int)size;
    return avpkt->data ? 0 : AVERROR(ENOMEM);
}
int ff_set_dimensions(AVCodecContext* avctx, int width, int height) {
    avctx->width = width;
    avctx->height = height;
    return 0;
}

/* planes of the formats the tests decode: (bytes per sample, chroma shift x,
 * chroma shift y, planes) */
static int fmt_layout(enum AVPixelFormat f, int* bps, int* sx, int* sy) {
    switch (f) {
    case AV_PIX_FMT_YUV420P: *bps = 1; *sx = 1; *sy = 1; return 3;
    case AV_PIX_FMT_YUV422P: *bps = 1; *sx = 1; *sy = 0; return 3;
    case AV_PIX_FMT_YUV444P: *bps = 1; *sx = 0; *sy = 0; return 3;
    case AV_PIX_FMT_YUV420P10LE: case AV_PIX_FMT_YUV420P12LE: case AV_PIX_FMT_YUV420P14LE:
        *bps = 2; *sx = 1; *sy = 1; return 3;
    case AV_PIX_FMT_YUV422P10LE: case AV_PIX_FMT_YUV422P12LE: case AV_PIX_FMT_YUV422P14LE:
        *bps = 2; *sx = 1; *sy = 0; return 3;
    case AV_PIX_FMT_YUV444P10LE: case AV_PIX_FMT_YUV444P12LE: case AV_PIX_FMT_YUV444P14LE:
        *bps = 2; *sx = 0; *sy = 0; return 3;
    default: return 0;
    }
}

/* ff_get_buffer: planes with a 64-byte aligned line size, as libavcodec's
 * default allocator gives */
int ff_get_buffer(AVCodecContext* avctx, AVFrame* frame, int flags) {
    (void)flags;
    int bps, sx, sy;
    const int n = fmt_layout(avctx->pix_fmt, &bps, &sx, &sy);
    if (!n) return AVERROR_INVALIDDATA;
    for (int k = 0; k < n; k++) {
        const int w = k ? (avctx->width + (1 << sx) - 1) >> sx : avctx->width;
        const int h = k ? (avctx->height + (1 << sy) - 1) >> sy : avctx->height;
        frame->linesize[k] = (w * bps + 63) & ~63;
        frame->data[k] = (uint8_t*)calloc((size_t)frame->linesize[k] * h, 1);
        if (!frame->data[k]) return AVERROR(ENOMEM);
    }
    return 0;
}

/* av_opt_set_defaults on the private context, then one string option */
static void set_options(const FFCodec* c, void* priv, const char* name, const char* value) {
    for (const AVOption* o = c->p.priv_class->option; o->name; o++) {
        if (o->type == AV_OPT_TYPE_INT || o->type == AV_OPT_TYPE_BOOL) *(int*)((char*)priv + o->offset) = (int)o->default_val.i64;
        else if (o->type == AV_OPT_TYPE_STRING) *(const char**)((char*)priv + o->offset) = o->default_val.str;
    }
    if (!name) return;
    for (const AVOption* o = c->p.priv_class->option; o->name; o++) {
        if (strcmp(o->name, name)) continue;
        if (o->type == AV_OPT_TYPE_STRING) *(const char**)((char*)priv + o->offset) = value;
        else *(int*)((char*)priv + o->offset) = atoi(value);
    }
}

/* Encodes one frame through the plugin; returns the plugin's status, the
 * codestream in out (*out_size bytes). */
int ffh_encode(const char* bpp, int width, int height, int pix_fmt, uint8_t* const* planes, const int* linesize,
               uint8_t* out, int out_cap, int* out_size) {
    const FFCodec* c = &ff_libsvtjpegxs_encoder;
    AVCodecContext ctx;
    memset(&ctx, 0, sizeof(ctx));
    ctx.av_class = c->p.priv_class;
    ctx.width = width;
    ctx.height = height;
    ctx.pix_fmt = (enum AVPixelFormat)pix_fmt;
    ctx.priv_data = calloc(1, (size_t)c->priv_data_size);
    set_options(c, ctx.priv_data, "bpp", bpp);
    int r = c->init(&ctx);
    if (r == 0) {
        AVFrame f;
        memset(&f, 0, sizeof(f));
        for (int k = 0; k < 3; k++) {
            f.data[k] = planes[k];
            f.linesize[k] = linesize[k];
        }
        AVPacket pkt = {0, 0};
        int got = 0;
        r = c->encode(&ctx, &pkt, &f, &got);
        if (r == 0 && got) {
            *out_size = pkt.size;
            memcpy(out, pkt.data, (size_t)(pkt.size < out_cap ? pkt.size : out_cap));
        }
        free(pkt.data);
    }
    c->close(&ctx);
    free(ctx.priv_data);
    return r;
}

/* Decodes a codestream through the plugin, handed over in `chunks` pieces
 * (the plugin's chunked path when chunks > 1); the planes are copied into
 * out[k] rows of out_linesize[k] bytes.  Returns the plugin's status of the
 * last call; *got_frame and the output format and size are set. */
int ffh_decode(const uint8_t* bs, int size, int chunks, uint8_t* const* out, const int* out_linesize, int* got_frame,
               int* pix_fmt, int* width, int* height) {
    const FFCodec* c = &ff_libsvtjpegxs_decoder;
    AVCodecContext ctx;
    memset(&ctx, 0, sizeof(ctx));
    ctx.av_class = c->p.priv_class;
    ctx.priv_data = calloc(1, (size_t)c->priv_data_size);
    set_options(c, ctx.priv_data, NULL, NULL);
    int r = c->init(&ctx);
    *got_frame = 0;
    AVFrame f;
    memset(&f, 0, sizeof(f));
    const int piece = (size + chunks - 1) / chunks;
    for (int off = 0; r >= 0 && off < size; off += piece) {
        AVPacket pkt = {(uint8_t*)bs + off, size - off < piece ? size - off : piece};
        int got = 0;
        r = c->decode(&ctx, &f, &got, &pkt);
        if (got) *got_frame = 1;
    }
    if (*got_frame) {
        int bps, sx, sy;
        const int n = fmt_layout(ctx.pix_fmt, &bps, &sx, &sy);
        for (int k = 0; k < n; k++) {
            const int w = k ? (ctx.width + (1 << sx) - 1) >> sx : ctx.width;
            const int h = k ? (ctx.height + (1 << sy) - 1) >> sy : ctx.height;
            for (int y = 0; y < h; y++) memcpy(out[k] + (size_t)y * out_linesize[k], f.data[k] + (size_t)y * f.linesize[k], (size_t)w * bps);
        }
    }
    for (int k = 0; k < 8; k++) free(f.data[k]);
    *pix_fmt = ctx.pix_fmt;
    *width = ctx.width;
    *height = ctx.height;
    c->close(&ctx);
    free(ctx.priv_data);
    return r;
}
