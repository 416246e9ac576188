/*
 * Thin C-ABI between the host C library and the CUDA code.
 *
 * An encoder or decoder owns `nslots` independent frame slots; each slot has
 * its own device buffers and CUDA stream, so up to `nslots` frames are in
 * flight at once (host-to-device copy of one frame overlaps the kernels of
 * another).  Planes and bitstreams passed in may be host or device pointers.
 */
#ifndef JXS_GPU_H
#define JXS_GPU_H

#include <stdint.h>

#include "jxs_core.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct jxs_gpu_enc jxs_gpu_enc_t;
typedef struct jxs_gpu_dec jxs_gpu_dec_t;

/* Encoder ---------------------------------------------------------------- */
jxs_gpu_enc_t* jxs_gpu_enc_create(const jxs_cfg_t* cfg, int nslots, int32_t* err);
void jxs_gpu_enc_destroy(jxs_gpu_enc_t* e);
/* Queues the encode of one frame on `slot`.  `out` receives cfg->lcod bytes. */
int32_t jxs_gpu_enc_submit(jxs_gpu_enc_t* e, int slot, void* const planes[4], const uint32_t strides[4], uint8_t* out);
/* Blocks until the slot's frame is done; returns its status (0 or an error code). */
int32_t jxs_gpu_enc_wait(jxs_gpu_enc_t* e, int slot);
/* 1 when the slot's frame is done, 0 while it is in flight. */
int jxs_gpu_enc_ready(jxs_gpu_enc_t* e, int slot);
/* Per-precinct quantization/refinement of the slot's last frame (host copies). */
int32_t jxs_gpu_enc_rc_results(jxs_gpu_enc_t* e, int slot, uint8_t* q, uint8_t* r);

/* Decoder ---------------------------------------------------------------- */
jxs_gpu_dec_t* jxs_gpu_dec_create(const jxs_cfg_t* cfg, int nslots, int32_t* err);
void jxs_gpu_dec_destroy(jxs_gpu_dec_t* d);
/* Queues the decode of one frame whose precincts start at prec_off (host
 * array, cfg->np entries, from jxs_frame_bytes_walk).  With prec_off NULL the
 * codestream must be in device memory: its precincts are located on the GPU
 * and its header is compared with the stream's when the frame completes. */
int32_t jxs_gpu_dec_submit(jxs_gpu_dec_t* d, int slot, const uint8_t* bs, uint32_t size, const uint32_t* prec_off,
                           void* const planes[4], const uint32_t strides[4]);
int32_t jxs_gpu_dec_wait(jxs_gpu_dec_t* d, int slot);
int jxs_gpu_dec_ready(jxs_gpu_dec_t* d, int slot);

/* Binds all work of the handle to a caller stream (cudaStream_t); NULL
 * returns to the per-slot streams. */
void jxs_gpu_enc_set_stream(jxs_gpu_enc_t* e, void* stream);
void jxs_gpu_dec_set_stream(jxs_gpu_dec_t* d, void* stream);
/* slot i runs on streams[i % n]; n = 0 returns to the slots' own streams */
void jxs_gpu_enc_set_streams(jxs_gpu_enc_t* e, void* const* streams, int n);
void jxs_gpu_dec_set_streams(jxs_gpu_dec_t* d, void* const* streams, int n);
int jxs_gpu_enc_slots(jxs_gpu_enc_t* e);
/* timing mode: accumulated milliseconds of each kernel launch of a frame in
 * launch order; returns the launches per frame */
int jxs_gpu_enc_read_kernel_timing(jxs_gpu_enc_t* e, double* ms, int n);
int jxs_gpu_dec_read_kernel_timing(jxs_gpu_dec_t* d, double* ms, int n);
int jxs_gpu_dec_slots(jxs_gpu_dec_t* d);
/* Stage timing with CUDA events on the launching stream.  Encoder stages:
 * H2D, transform, rate control, packing, D2H.  Decoder stages: H2D, unpack,
 * inverse transform, D2H.  read returns the frames timed since enabling. */
void jxs_gpu_enc_set_timing(jxs_gpu_enc_t* e, int on);
uint64_t jxs_gpu_enc_read_timing(jxs_gpu_enc_t* e, double* ms, int n);
void jxs_gpu_dec_set_timing(jxs_gpu_dec_t* d, int on);
uint64_t jxs_gpu_dec_read_timing(jxs_gpu_dec_t* d, double* ms, int n);

/* 1 if p is memory of this process's current CUDA device. */
int jxs_gpu_is_device_ptr(const void* p);
int jxs_gpu_is_page_locked(const void* p);

/* Host and device copies of a decoder's configuration. */
const jxs_cfg_t* jxs_gpu_dec_cfg(jxs_gpu_dec_t* d, const jxs_cfg_t** dev_cfg);

/* Frame size and precinct offsets of a device-resident codestream, with no
 * allocation (jxs_noalloc.cu).  prec_off may be NULL; otherwise it receives
 * cfg->np offsets and cap must be at least that. */
int32_t jxs_gpu_dec_locate_noalloc(jxs_gpu_dec_t* d, const void* dev_bs, uint32_t size, uint32_t* frame_size,
                                   uint32_t* prec_off, uint32_t cap, void* stream);
/* Page-locked host allocation (falls back to malloc without a GPU). */
void* jxs_gpu_host_alloc(size_t n);
void jxs_gpu_host_free(void* p);
/* Number of GPUs visible (0 when none). */
int jxs_gpu_device_count(void);

#ifdef __cplusplus
}
#endif

#endif
