/*
 * Batch objects of the GPU extension API (SvtJpegxsGpu.h): creation, options,
 * completion and statistics.  The encode and decode entry points live beside
 * the handles they read (jxs_api_enc.c, jxs_api_dec.c); the engine is
 * jxs_batch.cu.
 */
#include <string.h>

#include "SvtJpegxsGpu.h"
#include "jxs_batch.h"

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_create(uint64_t device_bytes, svt_jpeg_xs_gpu_batch_t** batch) {
    if (!batch || !device_bytes) return SvtJxsErrorBadParameter;
    int32_t err = 0;
    *batch = (svt_jpeg_xs_gpu_batch_t*)jxs_gpu_batch_create(device_bytes, NULL, &err);
    return *batch ? SvtJxsErrorNone : (SvtJxsErrorType_t)err;
}

PREFIX_API void svt_jpeg_xs_gpu_batch_destroy(svt_jpeg_xs_gpu_batch_t* batch) { jxs_gpu_batch_destroy((jxs_gpu_batch_t*)batch); }

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_set_options(svt_jpeg_xs_gpu_batch_t* batch, uint32_t use_graph,
                                                               uint32_t autotune) {
    if (!batch) return SvtJxsErrorBadParameter;
    jxs_gpu_batch_set_options((jxs_gpu_batch_t*)batch, use_graph != 0, autotune != 0);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_set_tune(svt_jpeg_xs_gpu_batch_t* batch, const int32_t* tune) {
    if (!batch || !tune) return SvtJxsErrorBadParameter;
    const int t[5] = {tune[0], tune[1], tune[2], tune[3], tune[4]};
    jxs_gpu_batch_set_tune((jxs_gpu_batch_t*)batch, t);
    return SvtJxsErrorNone;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_wait(svt_jpeg_xs_gpu_batch_t* batch, SvtJxsErrorType_t* status) {
    if (!batch) return SvtJxsErrorBadParameter;
    int32_t st[SVT_JPEGXS_GPU_BATCH_MAX];
    memset(st, 0, sizeof(st));
    const int32_t r = jxs_gpu_batch_wait((jxs_gpu_batch_t*)batch, st);
    if (status)
        for (uint32_t i = 0; i < SVT_JPEGXS_GPU_BATCH_MAX; i++) status[i] = (SvtJxsErrorType_t)st[i];
    return (SvtJxsErrorType_t)r;
}

PREFIX_API uint32_t svt_jpeg_xs_gpu_batch_ready(svt_jpeg_xs_gpu_batch_t* batch) {
    return batch ? (uint32_t)jxs_gpu_batch_ready((jxs_gpu_batch_t*)batch) : 1u;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_get_info(svt_jpeg_xs_gpu_batch_t* batch, svt_jpeg_xs_gpu_batch_info_t* info) {
    if (!batch || !info) return SvtJxsErrorBadParameter;
    jxs_batch_info_t i;
    jxs_gpu_batch_info((jxs_gpu_batch_t*)batch, &i);
    memset(info, 0, sizeof(*info));
    info->last_gpu_ms = i.last_gpu_ms;
    info->last_launches = i.last_launches;
    info->graph_hits = i.graph_hits;
    info->graph_builds = i.graph_builds;
    info->graph_updates = i.graph_updates;
    for (int k = 0; k < 5; k++) info->tune[k] = i.tune[k];
    info->device_bytes = i.arena_bytes;
    info->device_used = i.arena_used;
    info->device_peak = i.arena_peak;
    return SvtJxsErrorNone;
}
