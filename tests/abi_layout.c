/* Prints the size and field offsets of the public API structs.  Compiled by
 * tests/test_abi.py against this project's include/ and, where available,
 * against the reference's Source/API, to show the layouts are identical. */
#include <stddef.h>
#include <stdio.h>

#include "SvtJpegxs.h"
#include "SvtJpegxsDec.h"
#include "SvtJpegxsEnc.h"
#include "SvtJpegxsImageBufferTools.h"

#define F(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(T, f))
#define S(T) printf("%s %zu\n", #T, sizeof(T))

int main(void) {
    S(svt_jpeg_xs_image_config_t);
    F(svt_jpeg_xs_image_config_t, width); F(svt_jpeg_xs_image_config_t, bit_depth); F(svt_jpeg_xs_image_config_t, format);
    F(svt_jpeg_xs_image_config_t, components_num); F(svt_jpeg_xs_image_config_t, components);
    S(svt_jpeg_xs_image_buffer_t);
    F(svt_jpeg_xs_image_buffer_t, data_yuv); F(svt_jpeg_xs_image_buffer_t, stride); F(svt_jpeg_xs_image_buffer_t, alloc_size);
    F(svt_jpeg_xs_image_buffer_t, release_ctx_ptr); F(svt_jpeg_xs_image_buffer_t, ready_to_release);
    S(svt_jpeg_xs_bitstream_buffer_t);
    F(svt_jpeg_xs_bitstream_buffer_t, buffer); F(svt_jpeg_xs_bitstream_buffer_t, allocation_size);
    F(svt_jpeg_xs_bitstream_buffer_t, used_size); F(svt_jpeg_xs_bitstream_buffer_t, release_ctx_ptr);
    F(svt_jpeg_xs_bitstream_buffer_t, ready_to_release); F(svt_jpeg_xs_bitstream_buffer_t, last_packet_in_frame);
    S(svt_jpeg_xs_frame_t);
    F(svt_jpeg_xs_frame_t, image); F(svt_jpeg_xs_frame_t, bitstream); F(svt_jpeg_xs_frame_t, user_prv_ctx_ptr);
    S(svt_jpeg_xs_encoder_api_t);
    F(svt_jpeg_xs_encoder_api_t, source_width); F(svt_jpeg_xs_encoder_api_t, input_bit_depth);
    F(svt_jpeg_xs_encoder_api_t, colour_format); F(svt_jpeg_xs_encoder_api_t, bpp_numerator);
    F(svt_jpeg_xs_encoder_api_t, slice_height); F(svt_jpeg_xs_encoder_api_t, use_cpu_flags);
    F(svt_jpeg_xs_encoder_api_t, threads_num); F(svt_jpeg_xs_encoder_api_t, cpu_profile);
    F(svt_jpeg_xs_encoder_api_t, print_bands_info); F(svt_jpeg_xs_encoder_api_t, coding_signs_handling);
    F(svt_jpeg_xs_encoder_api_t, rate_control_mode); F(svt_jpeg_xs_encoder_api_t, coding_vertical_prediction_mode);
    F(svt_jpeg_xs_encoder_api_t, verbose); F(svt_jpeg_xs_encoder_api_t, callback_send_data_available);
    F(svt_jpeg_xs_encoder_api_t, callback_get_data_available_context); F(svt_jpeg_xs_encoder_api_t, slice_packetization_mode);
    F(svt_jpeg_xs_encoder_api_t, private_ptr); F(svt_jpeg_xs_encoder_api_t, padding);
    S(svt_jpeg_xs_decoder_api_t);
    F(svt_jpeg_xs_decoder_api_t, use_cpu_flags); F(svt_jpeg_xs_decoder_api_t, verbose); F(svt_jpeg_xs_decoder_api_t, threads_num);
    F(svt_jpeg_xs_decoder_api_t, packetization_mode); F(svt_jpeg_xs_decoder_api_t, proxy_mode);
    F(svt_jpeg_xs_decoder_api_t, callback_send_data_available); F(svt_jpeg_xs_decoder_api_t, callback_get_data_available_context);
    F(svt_jpeg_xs_decoder_api_t, private_ptr); F(svt_jpeg_xs_decoder_api_t, padding);
    printf("SvtJxsErrorDecoderConfigChange %d\n", (int)SvtJxsErrorDecoderConfigChange);
    printf("SvtJxsErrorEncodeFrameError %d\n", (int)SvtJxsErrorEncodeFrameError);
    printf("COLOUR_FORMAT_PACKED_YUV444_OR_RGB %d\n", (int)COLOUR_FORMAT_PACKED_YUV444_OR_RGB);
    printf("CPU_FLAGS_ALL %llu\n", (unsigned long long)CPU_FLAGS_ALL);
    return 0;
}
