/* Link-compatibility check for the reference's two plugins: every type,
 * constant, struct member and function that ffmpeg-plugin/libsvtjpegxs{enc,
 * dec}.c and imtl-plugin/src/st22_svt_jpeg_xs_plugin.c use, in the call
 * forms they use them (encoder: load_default_parameters -> init ->
 * send_picture / get_packet -> close; decoder:
 * get_single_frame_size_with_proxy -> init -> send_frame / get_frame ->
 * close).  Compiled and linked against this project's headers and
 * libSvtJpegxs.so by tests/test_abi.py; it is not run (init needs a GPU).
 * FFmpeg and MTL themselves are not part of this check. */
#include <stdint.h>
#include <string.h>

#include "SvtJpegxsDec.h"
#include "SvtJpegxsEnc.h"

static void send_cb(struct svt_jpeg_xs_encoder_api* api, void* ctx) { (void)api; (void)ctx; }
static void get_cb(struct svt_jpeg_xs_encoder_api* api, void* ctx) { (void)api; (void)ctx; }
static void dec_cb(struct svt_jpeg_xs_decoder_api* api, void* ctx) { (void)api; (void)ctx; }

int plugin_encoder(uint8_t* planes[3], uint32_t strides[3], uint8_t* out, uint32_t out_size, int blocking) {
    svt_jpeg_xs_encoder_api_t enc;
    memset(&enc, 0, sizeof(enc));
    SvtJxsErrorType_t err = svt_jpeg_xs_encoder_load_default_parameters(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &enc);
    if (err != SvtJxsErrorNone) return (int)err;
    enc.source_width = 1920;
    enc.source_height = 1080;
    enc.input_bit_depth = 10;
    enc.colour_format = COLOUR_FORMAT_PLANAR_YUV422;
    enc.bpp_numerator = 3;
    enc.bpp_denominator = 1;
    enc.ndecomp_v = 2;
    enc.ndecomp_h = 5;
    enc.quantization = 0;
    enc.slice_height = 16;
    enc.threads_num = 4;
    enc.use_cpu_flags = 0;
    enc.verbose = 0;
    enc.coding_significance = 1;
    enc.coding_signs_handling = 0;
    enc.coding_vertical_prediction_mode = 0;
    enc.callback_send_data_available = send_cb;
    enc.callback_send_data_available_context = NULL;
    enc.callback_get_data_available = get_cb;
    enc.callback_get_data_available_context = NULL;
    if (enc.colour_format == COLOUR_FORMAT_PLANAR_YUV420 || enc.colour_format == COLOUR_FORMAT_PLANAR_YUV444_OR_RGB ||
        enc.colour_format == COLOUR_FORMAT_PACKED_YUV444_OR_RGB)
        return -1;
    err = svt_jpeg_xs_encoder_init(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &enc);
    if (err != SvtJxsErrorNone) return (int)err;
    svt_jpeg_xs_frame_t in, got;
    memset(&in, 0, sizeof(in));
    for (int c = 0; c < 3; c++) {
        in.image.data_yuv[c] = planes[c];
        in.image.stride[c] = strides[c];
        in.image.alloc_size[c] = strides[c] * 2 * 1080;
    }
    in.bitstream.buffer = out;
    in.bitstream.allocation_size = out_size;
    in.bitstream.used_size = 0;
    in.user_prv_ctx_ptr = NULL;
    err = svt_jpeg_xs_encoder_send_picture(&enc, &in, (uint8_t)blocking);
    if (err == SvtJxsErrorNone) err = svt_jpeg_xs_encoder_get_packet(&enc, &got, (uint8_t)blocking);
    svt_jpeg_xs_encoder_close(&enc);
    return (int)err + (int)got.bitstream.used_size;
}

int plugin_decoder(const uint8_t* bs, uint32_t size, uint8_t* planes[3], uint32_t strides[3], int blocking) {
    svt_jpeg_xs_image_config_t cfg;
    uint32_t frame_size = 0;
    SvtJxsErrorType_t err = svt_jpeg_xs_decoder_get_single_frame_size_with_proxy(bs, size, &cfg, &frame_size, 1, proxy_mode_full);
    if (err != SvtJxsErrorNone) return (int)err;
    if (cfg.format != COLOUR_FORMAT_PLANAR_YUV422 || cfg.bit_depth != 10 || cfg.components_num != 3) return -1;
    uint32_t w = cfg.width, h = cfg.height, cw = cfg.components[1].width;
    (void)w;
    (void)h;
    (void)cw;
    svt_jpeg_xs_decoder_api_t dec;
    memset(&dec, 0, sizeof(dec));
    dec.use_cpu_flags = 0;
    dec.verbose = 0;
    dec.threads_num = 4;
    dec.packetization_mode = 0;
    dec.proxy_mode = proxy_mode_full;
    dec.callback_send_data_available = dec_cb;
    dec.callback_send_data_available_context = NULL;
    dec.callback_get_data_available = dec_cb;
    dec.callback_get_data_available_context = NULL;
    err = svt_jpeg_xs_decoder_init(SVT_JPEGXS_API_VER_MAJOR, SVT_JPEGXS_API_VER_MINOR, &dec, bs, size, &cfg);
    if (err != SvtJxsErrorNone) return (int)err;
    svt_jpeg_xs_frame_t in, got;
    memset(&in, 0, sizeof(in));
    in.bitstream.buffer = (uint8_t*)bs;
    in.bitstream.allocation_size = size;
    in.bitstream.used_size = frame_size;
    for (int c = 0; c < 3; c++) {
        in.image.data_yuv[c] = planes[c];
        in.image.stride[c] = strides[c];
        in.image.alloc_size[c] = strides[c] * 2 * cfg.components[c].height;
    }
    err = svt_jpeg_xs_decoder_send_frame(&dec, &in, (uint8_t)blocking);
    if (err == SvtJxsErrorNone) err = svt_jpeg_xs_decoder_get_frame(&dec, &got, (uint8_t)blocking);
    if (err == SvtJxsErrorDecoderConfigChange) err = SvtJxsErrorNone;
    svt_jpeg_xs_decoder_close(&dec);
    return (int)err;
}
