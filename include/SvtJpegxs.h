/*
 * SvtJpegxs.h - common types of the JPEG XS encoder/decoder C API.
 *
 * Drop-in boundary: every type, enum value and struct layout here is ABI
 * identical to the reference's Source/API/SvtJpegxs.h (API v0.10, lines
 * 16-190), so code compiled against the reference headers (the FFmpeg and
 * IMTL plugins, applications) links against this library unchanged.  The
 * implementation behind it runs on one NVIDIA GB300 GPU.
 */
#ifndef _SVT_JPEG_XS_API_H_
#define _SVT_JPEG_XS_API_H_

#ifdef __cplusplus
extern "C" {
#endif

#include <stdint.h>

#define SVT_JPEGXS_API_VER_MAJOR (0)
#define SVT_JPEGXS_API_VER_MINOR (10)

#if defined(DEF_DLL) && defined(DEF_BUILDING_SHARED_LIBS) && defined(__GNUC__)
#define PREFIX_API __attribute__((visibility("default")))
#else
#define PREFIX_API
#endif

#define MAX_COMPONENTS_NUM (4)

/* Sampling layout of the picture (values fixed by the ABI). */
typedef enum ColourFormat {
    COLOUR_FORMAT_INVALID = 0,
    COLOUR_FORMAT_PLANAR_YUV400 = 1,
    COLOUR_FORMAT_PLANAR_YUV420 = 2,
    COLOUR_FORMAT_PLANAR_YUV422 = 3,
    COLOUR_FORMAT_PLANAR_YUV444_OR_RGB = 4,
    COLOUR_FORMAT_PLANAR_4_COMPONENTS = 5,
    COLOUR_FORMAT_GRAY = 6,
    COLOUR_FORMAT_PLANAR_MAX,

    COLOUR_FORMAT_PACKED_MIN = 20,
    COLOUR_FORMAT_PACKED_YUV444_OR_RGB, /* interleaved 3 x 8/16-bit samples per pixel */
    COLOUR_FORMAT_PACKED_MAX
} ColourFormat_t;

enum VerboseMessages {
    VERBOSE_NONE = 0,
    VERBOSE_ERRORS = 1,
    VERBOSE_SYSTEM_INFO = 2,
    VERBOSE_SYSTEM_INFO_ALL = 3,
    VERBOSE_WARNINGS = 4,
    VERBOSE_INFO_MULTITHREADING = 5,
    VERBOSE_INFO_FULL = 6
};

typedef struct svt_jpeg_xs_image_config {
    uint32_t width;
    uint32_t height;
    uint8_t bit_depth;
    ColourFormat_t format;
    uint8_t components_num;
    struct {
        uint32_t width;
        uint32_t height;
        uint32_t byte_size;
    } components[MAX_COMPONENTS_NUM];
} svt_jpeg_xs_image_config_t;

/* Picture planes.  Strides are in samples; samples are one byte for bit
 * depth 8 and two little-endian bytes otherwise.  Planes may live in host
 * memory or in this GPU's device memory. */
typedef struct svt_jpeg_xs_image_buffer {
    void *data_yuv[MAX_COMPONENTS_NUM];
    uint32_t stride[MAX_COMPONENTS_NUM];
    uint32_t alloc_size[MAX_COMPONENTS_NUM];
    void *release_ctx_ptr;
    uint8_t ready_to_release;
} svt_jpeg_xs_image_buffer_t;

typedef struct svt_jpeg_xs_bitstream_buffer {
    uint8_t *buffer;
    uint32_t allocation_size;
    uint32_t used_size;
    void *release_ctx_ptr;
    uint8_t ready_to_release;
    uint8_t last_packet_in_frame;
} svt_jpeg_xs_bitstream_buffer_t;

/* One unit of work: the encoder reads `image` and writes `bitstream`, the
 * decoder the other way round.  `user_prv_ctx_ptr` is handed back untouched. */
typedef struct svt_jpeg_xs_frame {
    svt_jpeg_xs_image_buffer_t image;
    svt_jpeg_xs_bitstream_buffer_t bitstream;
    void *user_prv_ctx_ptr;
} svt_jpeg_xs_frame_t;

typedef enum SvtJxsErrorType {
    SvtJxsErrorNone = 0,
    SvtJxsErrorInvalidApiVersion = (int32_t)0x40001001,
    SvtJxsErrorCorrupt_Frame = (int32_t)0x4000100C,
    SvtJxsErrorInsufficientResources = (int32_t)0x80001000,
    SvtJxsErrorUndefined = (int32_t)0x80001001,
    SvtJxsErrorInvalidComponent = (int32_t)0x80001004,
    SvtJxsErrorBadParameter = (int32_t)0x80001005,
    SvtJxsErrorDestroyThreadFailed = (int32_t)0x80002012,
    SvtJxsErrorSemaphoreUnresponsive = (int32_t)0x80002021,
    SvtJxsErrorDestroySemaphoreFailed = (int32_t)0x80002022,
    SvtJxsErrorCreateMutexFailed = (int32_t)0x80002030,
    SvtJxsErrorMutexUnresponsive = (int32_t)0x80002031,
    SvtJxsErrorDestroyMutexFailed = (int32_t)0x80002032,
    SvtJxsErrorNoErrorEmptyQueue = (int32_t)0x80002033,
    SvtJxsErrorNoErrorFifoShutdown = (int32_t)0x80002034,
    SvtJxsErrorEncodeFrameError = (int32_t)0x80002035,
    SvtJxsErrorDecoderInvalidPointer = (int32_t)0x80003000,
    SvtJxsErrorDecoderInvalidBitstream = (int32_t)0x80003001,
    SvtJxsErrorDecoderInternal = (int32_t)0x80003002,
    SvtJxsErrorDecoderBitstreamTooShort = (int32_t)0x80003003,
    SvtJxsErrorDecoderConfigChange = (int32_t)0x80003004,
    SvtJxsDecoderEndOfCodestream = (int32_t)0x80003005,
    SvtJxsErrorMax = 0x7FFFFFFF
} SvtJxsErrorType_t;

typedef enum {
    proxy_mode_full = 0,
    proxy_mode_half = 1,
    proxy_mode_quarter = 2,
    proxy_mode_max
} proxy_mode_t;

/* CPU feature flags of the reference API.  Accepted and ignored: all work
 * runs on the GPU. */
typedef uint64_t CPU_FLAGS;
#define CPU_FLAGS_C        (0)
#define CPU_FLAGS_MMX      (1 << 0)
#define CPU_FLAGS_SSE      (1 << 1)
#define CPU_FLAGS_SSE2     (1 << 2)
#define CPU_FLAGS_SSE3     (1 << 3)
#define CPU_FLAGS_SSSE3    (1 << 4)
#define CPU_FLAGS_SSE4_1   (1 << 5)
#define CPU_FLAGS_SSE4_2   (1 << 6)
#define CPU_FLAGS_AVX      (1 << 7)
#define CPU_FLAGS_AVX2     (1 << 8)
#define CPU_FLAGS_AVX512F  (1 << 9)
#define CPU_FLAGS_AVX512CD (1 << 10)
#define CPU_FLAGS_AVX512DQ (1 << 11)
#define CPU_FLAGS_AVX512ER (1 << 12)
#define CPU_FLAGS_AVX512PF (1 << 13)
#define CPU_FLAGS_AVX512BW (1 << 14)
#define CPU_FLAGS_AVX512VL (1 << 15)
#define CPU_FLAGS_ALL      ((CPU_FLAGS_AVX512VL << 1) - 1)
#define CPU_FLAGS_INVALID  (1ULL << (sizeof(CPU_FLAGS) * 8ULL - 1ULL))

#ifdef __cplusplus
}
#endif

#endif /* _SVT_JPEG_XS_API_H_ */
