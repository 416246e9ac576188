/*
 * Host-library internals shared by the API files: the GPU handle behind a
 * public encoder or decoder handle.
 */
#ifndef JXS_API_INTERNAL_H
#define JXS_API_INTERNAL_H

#include "SvtJpegxsDec.h"
#include "SvtJpegxsEnc.h"
#include "jxs_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* NULL for a handle that was not initialised */
jxs_gpu_enc_t* jxs_api_enc_gpu(svt_jpeg_xs_encoder_api_t* enc_api);
jxs_gpu_dec_t* jxs_api_dec_gpu(svt_jpeg_xs_decoder_api_t* dec_api);

#ifdef __cplusplus
}
#endif

#endif
