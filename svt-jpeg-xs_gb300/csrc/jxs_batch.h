/*
 * Batched form and device arena (jxs_batch.cu): the C-ABI between the host
 * library and the batch engine.
 */
#ifndef JXS_BATCH_H
#define JXS_BATCH_H

#include <stdint.h>

#include "jxs_core.h"
#include "jxs_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* First-fit allocator over one device allocation of a fixed size. */
typedef struct jxs_arena jxs_arena_t;
jxs_arena_t* jxs_arena_create(uint64_t bytes);
void jxs_arena_destroy(jxs_arena_t* a);
/* 256-byte aligned; NULL when no free range is large enough */
void* jxs_arena_alloc(jxs_arena_t* a, uint64_t bytes);
void jxs_arena_free(jxs_arena_t* a, void* p, uint64_t bytes);
void jxs_arena_stats(jxs_arena_t* a, uint64_t* size, uint64_t* used, uint64_t* peak);

typedef struct jxs_gpu_batch jxs_gpu_batch_t;

typedef struct jxs_batch_info {
    float last_gpu_ms;        /* device time of the last batch's kernels (CUDA events on its stream) */
    uint32_t last_launches;   /* kernel launches of the last batch */
    uint64_t graph_hits, graph_builds, graph_updates;
    int32_t tune[5];          /* chains, heavy-first order, first-level blocks per SM, rows per block (forward, inverse) */
    uint64_t arena_bytes, arena_used, arena_peak;
} jxs_batch_info_t;

/* A batch engine with its own arena of device_bytes, or working sets carved
 * from `shared` when it is not NULL. */
jxs_gpu_batch_t* jxs_gpu_batch_create(uint64_t device_bytes, jxs_arena_t* shared, int32_t* err);
void jxs_gpu_batch_destroy(jxs_gpu_batch_t* b);
/* use_graph: capture and replay CUDA graphs (default 1); autotune: tune the
 * launch shapes the first time a batch signature is seen (default 0) */
void jxs_gpu_batch_set_options(jxs_gpu_batch_t* b, int use_graph, int autotune);
/* serving: the positions' working sets return to the arena when a batch
 * completes (wait), so the arena holds exactly the batches in flight */
void jxs_gpu_batch_set_release(jxs_gpu_batch_t* b, int on);
/* returns every position's working set to the arena now (nothing in
 * flight); 0 if a batch is in flight */
int jxs_gpu_batch_release(jxs_gpu_batch_t* b);
/* device bytes of one encoder / decoder position of the handle's configuration */
uint64_t jxs_gpu_batch_enc_work_bytes(jxs_gpu_enc_t* e);
uint64_t jxs_gpu_batch_dec_work_bytes(jxs_gpu_dec_t* d);
/* Lays out positions 0..n-1 for enc[i] (or dec[i]; the other NULL) ahead of
 * a batch call on `stream`; returns how many leading positions fit in the
 * arena. */
uint32_t jxs_gpu_batch_reserve(jxs_gpu_batch_t* b, jxs_gpu_enc_t* const* enc, jxs_gpu_dec_t* const* dec, uint32_t n, void* stream);
/* stages of a batch's launches (the values of SVT_JPEGXS_GPU_STAGE_*) */
enum {
    JXS_STAGE_FWD_V = 0, /* vertical level + the horizontal level after it */
    JXS_STAGE_FWD_H = 1, /* horizontal-only levels */
    JXS_STAGE_RC = 2,    /* rate control */
    JXS_STAGE_PACK = 3,
    JXS_STAGE_WALK = 4,  /* precinct offsets of device codestreams */
    JXS_STAGE_UNPACK = 5,
    JXS_STAGE_INV_H = 6,
    JXS_STAGE_INV_V = 7
};
/* stage timing (see svt_jpeg_xs_gpu_batch_set_stage_timing): on, batches
 * launch without graphs with an event pair around every launch */
void jxs_gpu_batch_set_stage_timing(jxs_gpu_batch_t* b, int on);
/* stage (JXS_STAGE_*), variant and device milliseconds of each launch of the
 * last batch issued with stage timing on, after its wait; returns the count */
uint32_t jxs_gpu_batch_stage_times(jxs_gpu_batch_t* b, int32_t* stage, int32_t* variant, float* ms, uint32_t max);
/* fixed launch shapes for every batch: chains, heavy-first, blocks per SM,
 * forward / inverse rows per block */
void jxs_gpu_batch_set_tune(jxs_gpu_batch_t* b, const int* tune5);

/* Queues the encode of n frames (n <= 64): frame i with the configuration of
 * enc[i], planes[i] / strides[i] as for jxs_gpu_enc_submit, codestream into
 * out[i] (host or device).  Returns at once; jxs_gpu_batch_wait completes it. */
int32_t jxs_gpu_batch_encode(jxs_gpu_batch_t* b, jxs_gpu_enc_t* const* enc, uint32_t n, void* const (*planes)[4],
                             const uint32_t (*strides)[4], uint8_t* const* out, void* stream);
/* Page-locked buffer for the precinct offsets of frame i of the next decode
 * batch (host codestreams, found with jxs_frame_bytes_walk). */
uint32_t* jxs_gpu_batch_prec_buffer(jxs_gpu_batch_t* b, uint32_t i, uint32_t np);
/* Queues the decode of n frames: host_walked[i] set means the precinct
 * offsets are in jxs_gpu_batch_prec_buffer(b, i); otherwise bs[i] must be a
 * device codestream, located on the GPU with its header checked at wait. */
int32_t jxs_gpu_batch_decode(jxs_gpu_batch_t* b, jxs_gpu_dec_t* const* dec, uint32_t n, const uint8_t* const* bs,
                             const uint32_t* size, const int* host_walked, void* const (*planes)[4],
                             const uint32_t (*strides)[4], void* stream);
/* Blocks until the queued batch is done; status[i] receives each frame's
 * status.  Returns the first non-zero status, or 0. */
int32_t jxs_gpu_batch_wait(jxs_gpu_batch_t* b, int32_t* status);
/* 1 when nothing is in flight or the batch has completed */
int jxs_gpu_batch_ready(jxs_gpu_batch_t* b);
void jxs_gpu_batch_info(jxs_gpu_batch_t* b, jxs_batch_info_t* info);

/* Encoder / decoder handle internals the batch engine plans with. */
const jxs_cfg_t* jxs_gpu_enc_info(jxs_gpu_enc_t* e, const jxs_cfg_t** dev_cfg, uint32_t* cap_words);
uint64_t jxs_gpu_enc_serial(jxs_gpu_enc_t* e);
const jxs_cfg_t* jxs_gpu_dec_info(jxs_gpu_dec_t* d, const jxs_cfg_t** dev_cfg, uint32_t* cap_bytes, uint32_t* cap_groups,
                                  uint32_t* cap_seg);
uint64_t jxs_gpu_dec_serial(jxs_gpu_dec_t* d);

#ifdef __cplusplus
}
#endif

#endif
