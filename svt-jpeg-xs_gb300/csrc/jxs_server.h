/*
 * Serving loop (jxs_server.cu): continuous batching of encode and decode
 * requests from many streams under a device-memory budget.
 */
#ifndef JXS_SERVER_H
#define JXS_SERVER_H

#include <stdint.h>

#include "jxs_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define JXS_SRV_BATCHED 0
#define JXS_SRV_PER_FRAME 1

typedef struct jxs_server jxs_server_t;

/* One request: planes and codestream in device memory of the current
 * device.  Encode: planes in, codestream out (bitstream, Lcod bytes).
 * Decode: codestream in (bitstream_size bytes), planes out. */
typedef struct jxs_srv_request {
    int32_t stream;
    uint64_t tag;
    void* planes[4];
    uint32_t strides[4];   /* samples */
    void* bitstream;
    uint32_t bitstream_size;
} jxs_srv_request_t;

typedef struct jxs_srv_done {
    uint64_t tag;
    int32_t stream;
    int32_t status;
    int64_t t_arrive_ns, t_start_ns, t_done_ns; /* host steady clock */
} jxs_srv_done_t;

typedef struct jxs_srv_stats {
    uint64_t batches, batched_frames, max_batch_seen, deferred;
    uint64_t device_bytes, device_used, device_peak;
} jxs_srv_stats_t;

jxs_server_t* jxs_server_create(uint64_t device_bytes, int mode, int lanes, int max_batch, int32_t* err);
void jxs_server_destroy(jxs_server_t* s);
/* registers a stream (exactly one of enc / dec); returns its id, or -1
 * once requests have been submitted */
int jxs_server_add_stream(jxs_server_t* s, jxs_gpu_enc_t* enc, jxs_gpu_dec_t* dec);
int32_t jxs_server_submit(jxs_server_t* s, const jxs_srv_request_t* r);
/* moves up to max completed requests to out; returns how many */
int jxs_server_poll(jxs_server_t* s, jxs_srv_done_t* out, int max);
/* requests submitted and not yet completed */
uint64_t jxs_server_pending(jxs_server_t* s);
void jxs_server_stats(jxs_server_t* s, jxs_srv_stats_t* out);

#ifdef __cplusplus
}
#endif

#endif
