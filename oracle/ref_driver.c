/*
 * Test-only driver around the reference SVT-JPEG-XS library, built from the
 * reference's own C sources by oracle/Makefile into oracle/_ref/.
 *
 * It drives the reference's public API (Source/API/SvtJpegxsEnc.h:100-142,
 * Source/API/SvtJpegxsDec.h:59-148) with in-memory frames so that tests and the
 * golden-fixture generator can compare this project's codestreams and decoded
 * planes with the reference's byte for byte.  Nothing in the product links it.
 *
 * Packed RGB input: the reference encoder app fills only data_yuv[0] for packed
 * formats and then hangs in get_packet, because send_picture rejects NULL
 * data_yuv[1..2] (Source/Lib/Encoder/Codec/EncHandle.c:974-978).  This driver
 * aliases planes 1 and 2 to plane 0, which the packed path never reads
 * (Source/Lib/Encoder/Codec/GcStageProcess.c:427-660).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "SvtJpegxsEnc.h"
#include "SvtJpegxsDec.h"

/* The reference's encoder and decoder handles call get_cpu_flags() even when
 * ARCH_X86_64 is off (EncHandle.c:664, DecHandle.c:151); with no x86 CPU
 * detection built, report "no SIMD" so the C functions stay selected. */
CPU_FLAGS get_cpu_flags(void) { return CPU_FLAGS_C; }

typedef struct ref_enc_params {
    uint32_t width, height, bit_depth, colour_format;
    uint32_t bpp_num, bpp_den, decomp_v, decomp_h;
    uint32_t quantization, slice_height, rate_control_mode;
    uint32_t coding_significance, coding_signs_handling, coding_vertical_prediction_mode;
    uint32_t threads_num;
} ref_enc_params_t;

/* Returns 0 on success, else the SvtJxsErrorType_t value (as int). */
int ref_encode(const ref_enc_params_t* p, void* const planes[4], const uint32_t strides[4], const uint32_t alloc_sizes[4],
               uint8_t* out, uint32_t out_cap, uint32_t* out_size) {
    svt_jpeg_xs_encoder_api_t enc;
    SvtJxsErrorType_t err = svt_jpeg_xs_encoder_load_default_parameters(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &enc);
    if (err) return (int)err;
    enc.source_width = p->width;
    enc.source_height = p->height;
    enc.input_bit_depth = (uint8_t)p->bit_depth;
    enc.colour_format = (ColourFormat_t)p->colour_format;
    enc.bpp_numerator = p->bpp_num;
    enc.bpp_denominator = p->bpp_den;
    enc.ndecomp_v = p->decomp_v;
    enc.ndecomp_h = p->decomp_h;
    enc.quantization = p->quantization;
    enc.slice_height = p->slice_height;
    enc.rate_control_mode = p->rate_control_mode;
    enc.coding_significance = p->coding_significance;
    enc.coding_signs_handling = p->coding_signs_handling;
    enc.coding_vertical_prediction_mode = p->coding_vertical_prediction_mode;
    enc.threads_num = p->threads_num;
    enc.verbose = 0;
    err = svt_jpeg_xs_encoder_init(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &enc);
    if (err) return (int)err;

    svt_jpeg_xs_frame_t frame;
    memset(&frame, 0, sizeof(frame));
    int packed = p->colour_format == COLOUR_FORMAT_PACKED_YUV444_OR_RGB;
    for (int c = 0; c < 4; c++) {
        int src = packed ? 0 : c;
        frame.image.data_yuv[c] = planes[src];
        frame.image.stride[c] = strides[src];
        frame.image.alloc_size[c] = alloc_sizes[src];
    }
    frame.bitstream.buffer = out;
    frame.bitstream.allocation_size = out_cap;
    err = svt_jpeg_xs_encoder_send_picture(&enc, &frame, 1);
    if (err) {
        svt_jpeg_xs_encoder_close(&enc);
        return (int)err;
    }
    svt_jpeg_xs_frame_t res;
    memset(&res, 0, sizeof(res));
    err = svt_jpeg_xs_encoder_get_packet(&enc, &res, 1);
    *out_size = res.bitstream.used_size;
    svt_jpeg_xs_encoder_close(&enc);
    return (int)err;
}

/* Parses the codestream header; fills width/height/depth/format/component sizes.
 * comp_info receives (width, height, byte_size) per component. */
int ref_probe(const uint8_t* bs, uint32_t size, uint32_t* width, uint32_t* height, uint32_t* depth, uint32_t* format,
              uint32_t* comps, uint32_t comp_info[12], uint32_t* frame_size) {
    svt_jpeg_xs_image_config_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    SvtJxsErrorType_t err = svt_jpeg_xs_decoder_get_single_frame_size(bs, size, &cfg, frame_size, 0);
    if (err) return (int)err;
    *width = cfg.width;
    *height = cfg.height;
    *depth = cfg.bit_depth;
    *format = (uint32_t)cfg.format;
    *comps = cfg.components_num;
    for (int c = 0; c < 4; c++) {
        comp_info[3 * c + 0] = cfg.components[c].width;
        comp_info[3 * c + 1] = cfg.components[c].height;
        comp_info[3 * c + 2] = cfg.components[c].byte_size;
    }
    return 0;
}

/* Image configuration of a codestream decoded at a proxy resolution
 * (proxy: 0 full, 1 half, 2 quarter). */
int ref_probe_proxy(const uint8_t* bs, uint32_t size, uint32_t proxy, uint32_t* comps, uint32_t comp_info[12]) {
    svt_jpeg_xs_image_config_t cfg;
    uint32_t frame_size = 0;
    memset(&cfg, 0, sizeof(cfg));
    SvtJxsErrorType_t err = svt_jpeg_xs_decoder_get_single_frame_size_with_proxy(bs, size, &cfg, &frame_size, 0,
                                                                                 (proxy_mode_t)proxy);
    if (err) return (int)err;
    *comps = cfg.components_num;
    for (int c = 0; c < 4; c++) {
        comp_info[3 * c + 0] = cfg.components[c].width;
        comp_info[3 * c + 1] = cfg.components[c].height;
        comp_info[3 * c + 2] = cfg.components[c].byte_size;
    }
    return 0;
}

/* Decodes one frame into caller planes (stride = component width) at a
 * proxy resolution. */
int ref_decode_proxy(const uint8_t* bs, uint32_t size, void* const planes[4], const uint32_t alloc_sizes[4], uint32_t threads_num,
                     uint32_t proxy) {
    svt_jpeg_xs_decoder_api_t dec;
    memset(&dec, 0, sizeof(dec));
    dec.use_cpu_flags = 0;
    dec.verbose = 0;
    dec.threads_num = threads_num;
    dec.packetization_mode = 0;
    dec.proxy_mode = (proxy_mode_t)proxy;
    svt_jpeg_xs_image_config_t cfg;
    SvtJxsErrorType_t err = svt_jpeg_xs_decoder_init(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &dec, bs, size, &cfg);
    if (err) return (int)err;
    svt_jpeg_xs_frame_t frame;
    memset(&frame, 0, sizeof(frame));
    for (int c = 0; c < cfg.components_num; c++) {
        frame.image.data_yuv[c] = planes[c];
        frame.image.stride[c] = cfg.components[c].width;
        frame.image.alloc_size[c] = alloc_sizes[c];
    }
    frame.bitstream.buffer = (uint8_t*)bs;
    frame.bitstream.allocation_size = size;
    frame.bitstream.used_size = size;
    err = svt_jpeg_xs_decoder_send_frame(&dec, &frame, 1);
    if (err) {
        svt_jpeg_xs_decoder_close(&dec);
        return (int)err;
    }
    svt_jpeg_xs_frame_t out;
    memset(&out, 0, sizeof(out));
    err = svt_jpeg_xs_decoder_get_frame(&dec, &out, 1);
    svt_jpeg_xs_decoder_close(&dec);
    return (int)err;
}

/* Decodes one frame into caller planes (stride = component width). */
int ref_decode(const uint8_t* bs, uint32_t size, void* const planes[4], const uint32_t alloc_sizes[4], uint32_t threads_num) {
    return ref_decode_proxy(bs, size, planes, alloc_sizes, threads_num, 0);
}

/* ------------------------------------------------------------------------
 * Streaming throughput of the reference codec, driven the way its sample
 * applications drive it (Source/App/EncApp/EncAppMain.c:97-170 and the
 * decoder app): one encoder and one decoder handle kept open across calls,
 * threads_num worker threads each (--lp), a sender thread that submits
 * frames with blocking send_picture / send_frame while the calling thread
 * collects the results with blocking get_packet / get_frame, so that several
 * frames are in the reference's pipeline at once.  bench.py times these calls
 * as the CPU baseline.
 * ------------------------------------------------------------------------ */
typedef struct ref_stream {
    svt_jpeg_xs_encoder_api_t enc;
    svt_jpeg_xs_decoder_api_t dec;
    svt_jpeg_xs_image_config_t dcfg;
    int enc_open, dec_open, packed;
} ref_stream_t;

/* Opens the encoder with the given parameters; the decoder is opened on the
 * first ref_stream_decode call, from that call's first codestream. */
void* ref_stream_open(const ref_enc_params_t* p, int* err) {
    ref_stream_t* s = (ref_stream_t*)calloc(1, sizeof(*s));
    if (!s) {
        *err = (int)SvtJxsErrorInsufficientResources;
        return NULL;
    }
    SvtJxsErrorType_t e = svt_jpeg_xs_encoder_load_default_parameters(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &s->enc);
    if (!e) {
        s->enc.source_width = p->width;
        s->enc.source_height = p->height;
        s->enc.input_bit_depth = (uint8_t)p->bit_depth;
        s->enc.colour_format = (ColourFormat_t)p->colour_format;
        s->enc.bpp_numerator = p->bpp_num;
        s->enc.bpp_denominator = p->bpp_den;
        s->enc.ndecomp_v = p->decomp_v;
        s->enc.ndecomp_h = p->decomp_h;
        s->enc.quantization = p->quantization;
        s->enc.slice_height = p->slice_height;
        s->enc.rate_control_mode = p->rate_control_mode;
        s->enc.coding_significance = p->coding_significance;
        s->enc.coding_signs_handling = p->coding_signs_handling;
        s->enc.coding_vertical_prediction_mode = p->coding_vertical_prediction_mode;
        s->enc.threads_num = p->threads_num;
        s->enc.verbose = 0;
        e = svt_jpeg_xs_encoder_init(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &s->enc);
    }
    if (e) {
        free(s);
        *err = (int)e;
        return NULL;
    }
    s->enc_open = 1;
    s->packed = p->colour_format == COLOUR_FORMAT_PACKED_YUV444_OR_RGB;
    s->dec.threads_num = p->threads_num;
    *err = 0;
    return s;
}

void ref_stream_close(void* h) {
    ref_stream_t* s = (ref_stream_t*)h;
    if (!s) return;
    if (s->enc_open) svt_jpeg_xs_encoder_close(&s->enc);
    if (s->dec_open) svt_jpeg_xs_decoder_close(&s->dec);
    free(s);
}

typedef struct stream_job {
    ref_stream_t* s;
    uint32_t n;
    svt_jpeg_xs_frame_t* frames;
    int decode;
    SvtJxsErrorType_t err;
} stream_job_t;

static void* stream_sender(void* arg) {
    stream_job_t* j = (stream_job_t*)arg;
    for (uint32_t i = 0; i < j->n && !j->err; i++) {
        j->err = j->decode ? svt_jpeg_xs_decoder_send_frame(&j->s->dec, &j->frames[i], 1)
                           : svt_jpeg_xs_encoder_send_picture(&j->s->enc, &j->frames[i], 1);
    }
    return NULL;
}

/* Runs n prepared frames through the encoder (decode = 0) or the decoder;
 * frame i carries i + 1 as its user context.  done[i] receives the output
 * size (encode: codestream bytes) or 1 (decode).  Returns 0 or the first
 * error. */
static int stream_run(ref_stream_t* s, uint32_t n, svt_jpeg_xs_frame_t* frames, int decode, uint32_t* done) {
    stream_job_t j = {s, n, frames, decode, SvtJxsErrorNone};
    pthread_t th;
    if (pthread_create(&th, NULL, stream_sender, &j)) return (int)SvtJxsErrorInsufficientResources;
    int err = 0;
    for (uint32_t got = 0; got < n;) {
        svt_jpeg_xs_frame_t res;
        memset(&res, 0, sizeof(res));
        SvtJxsErrorType_t e = decode ? svt_jpeg_xs_decoder_get_frame(&s->dec, &res, 1)
                                     : svt_jpeg_xs_encoder_get_packet(&s->enc, &res, 1);
        if (e == SvtJxsErrorNoErrorEmptyQueue) continue;
        if (e != SvtJxsErrorNone) {
            err = (int)e;
            break;
        }
        const uintptr_t idx = (uintptr_t)res.user_prv_ctx_ptr;
        if (idx >= 1 && idx <= n) done[idx - 1] = decode ? 1u : res.bitstream.used_size;
        got++;
    }
    pthread_join(th, NULL);
    if (!err && j.err) err = (int)j.err;
    return err;
}

/* Encodes n frames: planes[4 i + c] is plane c of frame i (packed formats:
 * plane 0 only), codestream i goes to out + i * out_cap; sizes[i] receives
 * its length. */
int ref_stream_encode(void* h, uint32_t n, void* const* planes, const uint32_t strides[4], const uint32_t alloc_sizes[4],
                      uint8_t* out, uint32_t out_cap, uint32_t* sizes) {
    ref_stream_t* s = (ref_stream_t*)h;
    svt_jpeg_xs_frame_t* fr = (svt_jpeg_xs_frame_t*)calloc(n ? n : 1, sizeof(*fr));
    if (!fr) return (int)SvtJxsErrorInsufficientResources;
    for (uint32_t i = 0; i < n; i++) {
        for (int c = 0; c < 4; c++) {
            const int src = s->packed ? 0 : c;
            fr[i].image.data_yuv[c] = planes[4 * i + src];
            fr[i].image.stride[c] = strides[src];
            fr[i].image.alloc_size[c] = alloc_sizes[src];
        }
        fr[i].bitstream.buffer = out + (size_t)i * out_cap;
        fr[i].bitstream.allocation_size = out_cap;
        fr[i].user_prv_ctx_ptr = (void*)(uintptr_t)(i + 1);
        sizes[i] = 0;
    }
    const int err = stream_run(s, n, fr, 0, sizes);
    free(fr);
    return err;
}

/* Decodes n codestreams (bs[i], sizes[i]) into planes[4 i + c] (stride =
 * component width, alloc_sizes[c] bytes each). */
int ref_stream_decode(void* h, uint32_t n, const uint8_t* const* bs, const uint32_t* sizes, void* const* planes,
                      const uint32_t alloc_sizes[4]) {
    ref_stream_t* s = (ref_stream_t*)h;
    if (!n) return 0;
    if (!s->dec_open) {
        s->dec.use_cpu_flags = 0;
        s->dec.verbose = 0;
        s->dec.packetization_mode = 0;
        s->dec.proxy_mode = proxy_mode_full;
        SvtJxsErrorType_t e = svt_jpeg_xs_decoder_init(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &s->dec, bs[0], sizes[0],
                                                       &s->dcfg);
        if (e) return (int)e;
        s->dec_open = 1;
    }
    svt_jpeg_xs_frame_t* fr = (svt_jpeg_xs_frame_t*)calloc(n, sizeof(*fr));
    uint32_t* done = (uint32_t*)calloc(n, sizeof(uint32_t));
    if (!fr || !done) {
        free(fr);
        free(done);
        return (int)SvtJxsErrorInsufficientResources;
    }
    for (uint32_t i = 0; i < n; i++) {
        for (int c = 0; c < s->dcfg.components_num; c++) {
            fr[i].image.data_yuv[c] = planes[4 * i + c];
            fr[i].image.stride[c] = s->dcfg.components[c].width;
            fr[i].image.alloc_size[c] = alloc_sizes[c];
        }
        fr[i].bitstream.buffer = (uint8_t*)bs[i];
        fr[i].bitstream.allocation_size = sizes[i];
        fr[i].bitstream.used_size = sizes[i];
        fr[i].user_prv_ctx_ptr = (void*)(uintptr_t)(i + 1);
    }
    int err = stream_run(s, n, fr, 1, done);
    for (uint32_t i = 0; i < n && !err; i++)
        if (!done[i]) err = (int)SvtJxsErrorUndefined;
    free(fr);
    free(done);
    return err;
}
