/*
 * Stand-ins for the few FFmpeg declarations that the SVT-JPEG-XS FFmpeg
 * plugin (ffmpeg-plugin/libsvtjpegxs{enc,dec}.c) uses, so that the plugin's
 * own source files compile against this library and run in the tests.  Test
 * infrastructure: only the names and members the plugin touches, with
 * values of this file's choosing; this is not FFmpeg.
 */
#ifndef JXS_TEST_FFSTUB_H
#define JXS_TEST_FFSTUB_H

#include <errno.h>
#include <limits.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define av_cold
#define FFMIN(a, b) ((a) > (b) ? (b) : (a))
#define AVERROR(e) (-(e))
#define AVERROR_UNKNOWN (-1001)
#define AVERROR_INVALIDDATA (-1002)
#define AVERROR_OPTION_NOT_FOUND (-1003)
#define AVERROR_INPUT_CHANGED (-1004)

enum { AV_LOG_QUIET = -8, AV_LOG_ERROR = 16, AV_LOG_WARNING = 24, AV_LOG_INFO = 32, AV_LOG_DEBUG = 48 };

enum AVPixelFormat {
    AV_PIX_FMT_NONE = -1,
    AV_PIX_FMT_YUV420P,
    AV_PIX_FMT_YUV422P,
    AV_PIX_FMT_YUV444P,
    AV_PIX_FMT_YUV420P10LE,
    AV_PIX_FMT_YUV422P10LE,
    AV_PIX_FMT_YUV444P10LE,
    AV_PIX_FMT_YUV420P12LE,
    AV_PIX_FMT_YUV422P12LE,
    AV_PIX_FMT_YUV444P12LE,
    AV_PIX_FMT_YUV420P14LE,
    AV_PIX_FMT_YUV422P14LE,
    AV_PIX_FMT_YUV444P14LE,
    AV_PIX_FMT_GBRP,
    AV_PIX_FMT_GBRP10LE,
    AV_PIX_FMT_GBRP12LE,
    AV_PIX_FMT_GBRP14LE,
    AV_PIX_FMT_RGB24,
    AV_PIX_FMT_BGR24
};
enum AVMediaType { AVMEDIA_TYPE_VIDEO = 0 };
enum AVCodecID { AV_CODEC_ID_JPEGXS = 1 };
enum AVOptionType { AV_OPT_TYPE_INT, AV_OPT_TYPE_STRING, AV_OPT_TYPE_CONST, AV_OPT_TYPE_BOOL };
#define AV_OPT_FLAG_ENCODING_PARAM 1
#define AV_OPT_FLAG_DECODING_PARAM 2
#define AV_OPT_FLAG_VIDEO_PARAM 16
#define LIBAVUTIL_VERSION_INT 0

typedef struct AVOption {
    const char* name;
    const char* help;
    int offset;
    enum AVOptionType type;
    union {
        int64_t i64;
        double dbl;
        const char* str;
    } default_val;
    double min, max;
    int flags;
    const char* unit;
} AVOption;

typedef struct AVClass {
    const char* class_name;
    const char* (*item_name)(void* ctx);
    const AVOption* option;
    int version;
} AVClass;

typedef struct AVCodecContext {
    const AVClass* av_class;
    void* priv_data;
    int width, height;
    enum AVPixelFormat pix_fmt;
    int thread_count;
} AVCodecContext;

typedef struct AVPacket {
    uint8_t* data;
    int size;
} AVPacket;

typedef struct AVFrame {
    uint8_t* data[8];
    int linesize[8];
} AVFrame;

typedef struct AVCodec {
    const char* name;
    const char* long_name;
    enum AVMediaType type;
    enum AVCodecID id;
    int capabilities;
    const enum AVPixelFormat* pix_fmts;
    const AVClass* priv_class;
    const char* wrapper_name;
} AVCodec;

typedef struct FFCodec {
    AVCodec p;
    int caps_internal;
    int priv_data_size;
    int (*init)(AVCodecContext*);
    int (*close)(AVCodecContext*);
    int cb_type; /* 1 encode, 2 decode */
    int (*encode)(AVCodecContext*, AVPacket*, const AVFrame*, int*);
    int (*decode)(AVCodecContext*, AVFrame*, int*, AVPacket*);
} FFCodec;

#define CODEC_LONG_NAME(s) .p.long_name = (s)
#define FF_CODEC_ENCODE_CB(f) .cb_type = 1, .encode = (f)
#define FF_CODEC_DECODE_CB(f) .cb_type = 2, .decode = (f)
#define AV_CODEC_CAP_DR1 (1 << 1)
#define AV_CODEC_CAP_OTHER_THREADS (1 << 15)
#define FF_CODEC_CAP_NOT_INIT_THREADSAFE (1 << 0)
#define FF_CODEC_CAP_AUTO_THREADS (1 << 7)

const char* av_default_item_name(void* ctx);
void av_log(void* avcl, int level, const char* fmt, ...);
int av_log_get_level(void);
int av_cpu_count(void);
void* av_malloc(size_t size);
void av_free(void* ptr);
int ff_alloc_packet(AVCodecContext* avctx, AVPacket* avpkt, int64_t size);
int ff_get_buffer(AVCodecContext* avctx, AVFrame* frame, int flags);
int ff_set_dimensions(AVCodecContext* avctx, int width, int height);

#endif
