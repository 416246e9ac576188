/*
 * Batch objects of the GPU extension API (SvtJpegxsGpu.h): creation, options,
 * completion and statistics.  The encode and decode entry points live beside
 * the handles they read (jxs_api_enc.c, jxs_api_dec.c); the engine is
 * jxs_batch.cu.
 */
#include <string.h>

#include "SvtJpegxsGpu.h"
#include "jxs_api_internal.h"
#include "jxs_batch.h"
#include "jxs_server.h"

_Static_assert(SVT_JPEGXS_GPU_STAGE_FWD_V == JXS_STAGE_FWD_V && SVT_JPEGXS_GPU_STAGE_RC == JXS_STAGE_RC &&
                   SVT_JPEGXS_GPU_STAGE_PACK == JXS_STAGE_PACK && SVT_JPEGXS_GPU_STAGE_UNPACK == JXS_STAGE_UNPACK &&
                   SVT_JPEGXS_GPU_STAGE_INV_V == JXS_STAGE_INV_V,
               "stage numbers of the public header");

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

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_batch_set_stage_timing(svt_jpeg_xs_gpu_batch_t* batch, uint32_t on) {
    if (!batch) return SvtJxsErrorBadParameter;
    jxs_gpu_batch_set_stage_timing((jxs_gpu_batch_t*)batch, on != 0);
    return SvtJxsErrorNone;
}

PREFIX_API uint32_t svt_jpeg_xs_gpu_batch_read_stage_times(svt_jpeg_xs_gpu_batch_t* batch, int32_t* stage, int32_t* variant,
                                                           float* ms, uint32_t max) {
    return batch ? jxs_gpu_batch_stage_times((jxs_gpu_batch_t*)batch, stage, variant, ms, max) : 0u;
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

/* ------------------------------------------------------------------------ */
/* serving loop                                                              */
/* ------------------------------------------------------------------------ */
PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_server_create(uint64_t device_bytes, uint32_t mode, uint32_t lanes,
                                                           uint32_t max_batch, svt_jpeg_xs_gpu_server_t** server) {
    if (!server || (mode != SVT_JPEGXS_GPU_SERVER_BATCHED && mode != SVT_JPEGXS_GPU_SERVER_PER_FRAME)) return SvtJxsErrorBadParameter;
    if (mode == SVT_JPEGXS_GPU_SERVER_BATCHED && !device_bytes) return SvtJxsErrorBadParameter;
    int32_t err = 0;
    *server = (svt_jpeg_xs_gpu_server_t*)jxs_server_create(device_bytes, (int)mode, (int)lanes, (int)max_batch, &err);
    return *server ? SvtJxsErrorNone : (SvtJxsErrorType_t)err;
}

PREFIX_API void svt_jpeg_xs_gpu_server_destroy(svt_jpeg_xs_gpu_server_t* server) { jxs_server_destroy((jxs_server_t*)server); }

PREFIX_API int32_t svt_jpeg_xs_gpu_server_add_encoder(svt_jpeg_xs_gpu_server_t* server, svt_jpeg_xs_encoder_api_t* enc_api) {
    jxs_gpu_enc_t* e = jxs_api_enc_gpu(enc_api);
    if (!server || !e) return -1;
    return jxs_server_add_stream((jxs_server_t*)server, e, NULL);
}

PREFIX_API int32_t svt_jpeg_xs_gpu_server_add_decoder(svt_jpeg_xs_gpu_server_t* server, svt_jpeg_xs_decoder_api_t* dec_api) {
    jxs_gpu_dec_t* d = jxs_api_dec_gpu(dec_api);
    if (!server || !d) return -1;
    return jxs_server_add_stream((jxs_server_t*)server, NULL, d);
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_server_submit(svt_jpeg_xs_gpu_server_t* server, const svt_jpeg_xs_gpu_request_t* req) {
    if (!server || !req) return SvtJxsErrorBadParameter;
    jxs_srv_request_t r;
    memset(&r, 0, sizeof(r));
    r.stream = req->stream;
    r.tag = req->tag;
    for (int k = 0; k < 4; k++) {
        r.planes[k] = req->planes[k];
        r.strides[k] = req->strides[k];
    }
    r.bitstream = req->bitstream;
    r.bitstream_size = req->bitstream_size;
    return (SvtJxsErrorType_t)jxs_server_submit((jxs_server_t*)server, &r);
}

PREFIX_API uint32_t svt_jpeg_xs_gpu_server_poll(svt_jpeg_xs_gpu_server_t* server, svt_jpeg_xs_gpu_completion_t* out, uint32_t max) {
    if (!server || !out) return 0;
    jxs_srv_done_t d[256];
    uint32_t total = 0;
    while (total < max) {
        const int want = (int)((max - total) < 256 ? (max - total) : 256);
        const int n = jxs_server_poll((jxs_server_t*)server, d, want);
        for (int i = 0; i < n; i++) {
            svt_jpeg_xs_gpu_completion_t* c = &out[total + i];
            c->tag = d[i].tag;
            c->stream = d[i].stream;
            c->status = (SvtJxsErrorType_t)d[i].status;
            c->t_arrive_ns = d[i].t_arrive_ns;
            c->t_start_ns = d[i].t_start_ns;
            c->t_done_ns = d[i].t_done_ns;
        }
        total += (uint32_t)n;
        if (n < want) break;
    }
    return total;
}

PREFIX_API uint64_t svt_jpeg_xs_gpu_server_pending(svt_jpeg_xs_gpu_server_t* server) {
    return server ? jxs_server_pending((jxs_server_t*)server) : 0;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_gpu_server_get_stats(svt_jpeg_xs_gpu_server_t* server, svt_jpeg_xs_gpu_server_stats_t* st) {
    if (!server || !st) return SvtJxsErrorBadParameter;
    jxs_srv_stats_t s;
    jxs_server_stats((jxs_server_t*)server, &s);
    st->batches = s.batches;
    st->batched_frames = s.batched_frames;
    st->max_batch_seen = s.max_batch_seen;
    st->deferred = s.deferred;
    st->device_bytes = s.device_bytes;
    st->device_used = s.device_used;
    st->device_peak = s.device_peak;
    return SvtJxsErrorNone;
}
