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
#include <stdint.h>
#include <stdio.h>
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
