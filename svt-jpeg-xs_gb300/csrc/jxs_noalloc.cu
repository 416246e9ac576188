/*
 * Allocation-free location of a device-resident frame's precincts.
 *
 * jxs_gpu_dec_locate_noalloc backs svt_jpeg_xs_gpu_decoder_locate_frame
 * (SvtJpegxsGpu.h; no counterpart in the reference API).  Given a codestream
 * that already sits in device memory, it returns the frame's size in bytes
 * (header through EOC) and the byte offset of every precinct, using the
 * decoder handle's configuration.
 *
 * The decoder's own path walks the same structure (walk_slices_kernel /
 * walk_sequential_kernel in jxs_dec_kernels.cu) with scratch that belongs
 * to a frame slot, allocated when the decoder was created.  This variant
 * allocates nothing: no cudaMalloc, no cudaFree, no host heap or pinned
 * memory (the header and the results come back into stack variables and
 * the caller's arrays), no library call that allocates.  Its scratch is the one
 * statically sized __device__ array below.  Callers that need this:
 *   - a receive thread that takes codestreams straight into GPU memory (a
 *     NIC writing to device buffers) and must find frame boundaries at line
 *     rate. It cannot wait on an allocator lock or on first-touch mapping of
 *     new memory while packets keep arriving;
 *   - a server that admits work against a fixed device-memory budget. It
 *     counts every byte when a stream is admitted and cannot grow the
 *     footprint per request.
 *
 * Scratch: NOALLOC_HEAD_WORDS + NOALLOC_MAX_PRECINCTS 32-bit words (16.6 KB)
 * per device, file-scope __device__ memory that the module loader maps.
 *   word 0: status of the last walk (0 or an SvtJxsErrorType_t value);
 *   word 1: frame size in bytes;
 *   words NOALLOC_HEAD_WORDS..: precinct offsets, one per precinct.
 * No word has to start at zero. Every launch writes words 0 and 1, and the
 * offsets are read back only after a walk that succeeded, which has written
 * all of them. A frame with more than NOALLOC_MAX_PRECINCTS precincts is
 * rejected before any launch, with SvtJxsErrorBadParameter and a message on
 * stderr.
 *
 * The host side takes the scratch's address with cudaGetSymbolAddress, with
 * the device current. The first call on a device may load the module, so it
 * should come before any stream capture starts. The address is looked up
 * again on every call rather than cached: after cudaDeviceReset, or once the
 * primary context has been destroyed and created again, the array lives at a
 * new address, and a cached one could point into some other allocation. The
 * lookup itself allocates nothing.
 *
 * The decoder handle's configuration and the codestream must both be in the
 * memory of the current device, which must be the decoder's device; a
 * pointer on another device is refused with SvtJxsErrorDecoderInvalidPointer
 * before anything is launched.
 *
 * Overlapping calls would race on the shared scratch: two walks in flight at
 * once would write the same words. Every call therefore holds one
 * process-wide mutex from the launch until its results are copied back, and
 * calls from several threads run one after another. Separate processes have
 * separate contexts and separate copies of the scratch.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "jxs_core.h"
#include "jxs_gpu.h"

#define NOALLOC_HEAD_WORDS 64u
#define NOALLOC_MAX_PRECINCTS 4096u
#define NOALLOC_THREADS 256

static __device__ __align__(256) uint32_t noalloc_scratch[NOALLOC_HEAD_WORDS + NOALLOC_MAX_PRECINCTS];

static __device__ __forceinline__ uint32_t rd24(const uint8_t* p) {
    return ((uint32_t)p[0] << 16) | ((uint32_t)p[1] << 8) | p[2];
}

static __device__ __forceinline__ int slice_header_at(const uint8_t* bs, uint64_t off, uint32_t size, uint32_t idx) {
    return off + 6 <= size && bs[off] == 0xff && bs[off + 1] == 0x20 && bs[off + 2] == 0 && bs[off + 3] == 4 &&
           (((uint32_t)bs[off + 4] << 8) | bs[off + 5]) == idx;
}

/* Walks the precincts of slice s starting at its header `off`; returns the
 * offset just past its last precinct, or 0 on a bad or short stream. */
static __device__ uint64_t walk_one_slice(const jxs_cfg_t* cfg, const uint8_t* bs, uint32_t size, uint32_t s, uint64_t off,
                                          uint32_t* offs) {
    if (!slice_header_at(bs, off, size, s)) return 0;
    off += 6;
    /* the slice's precincts: rows x columns, row after row */
    const uint32_t first = s * cfg->pps * cfg->ncol,
                   n = ((s + 1 == cfg->nslices) ? cfg->np - s * cfg->pps : cfg->pps) * cfg->ncol;
    for (uint32_t i = 0; i < n; i++) {
        if (off + cfg->prec_hdr_bytes > size || first + i >= NOALLOC_MAX_PRECINCTS) return 0;
        const uint32_t lprc = rd24(bs + off);
        if (lprc > JXS_PREC_MAX_BYTES) return 0;
        offs[first + i] = (uint32_t)off;
        off += cfg->prec_hdr_bytes + lprc;
    }
    return off;
}

/* One block. Each thread first walks whole slices from their
 * constant-bit-rate positions (EncHandle.c:760-809). If any slice is not
 * where the split puts it, thread 0 walks the frame from the header instead
 * (get_slice_size, DecThreadInit.c:35-131). The frame ends after EOC. */
__global__ void __launch_bounds__(NOALLOC_THREADS) locate_frame_kernel(const jxs_cfg_t* __restrict__ cfg,
                                                                       const uint8_t* __restrict__ bs, uint32_t size) {
    __shared__ int s_bad;
    __shared__ uint32_t s_end;
    uint32_t* head = noalloc_scratch;
    uint32_t* offs = noalloc_scratch + NOALLOC_HEAD_WORDS;
    if (threadIdx.x == 0) {
        s_bad = cfg->max_slice_budget == 0;
        s_end = 0;
    }
    __syncthreads();
    if (!s_bad) {
        for (uint32_t s = threadIdx.x; s < cfg->nslices; s += blockDim.x) {
            const uint64_t end = walk_one_slice(cfg, bs, size, s, cfg->slice_begin[s], offs);
            int ok = end != 0;
            if (ok && s + 1 < cfg->nslices) ok = end == cfg->slice_begin[s + 1];
            if (ok && s + 1 == cfg->nslices) {
                ok = end + 2 <= size && bs[end] == 0xff && bs[end + 1] == 0x11;
                if (ok) s_end = (uint32_t)(end + 2);
            }
            if (!ok) atomicExch(&s_bad, 1);
        }
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    int32_t status = 0;
    if (s_bad) {
        s_end = 0;
        uint64_t off = cfg->hdr_len;
        for (uint32_t s = 0; s < cfg->nslices && off; s++) off = walk_one_slice(cfg, bs, size, s, off, offs);
        if (!off) status = JXS_E_DEC_BITSTREAM;
        else if (off + 2 > size) status = JXS_E_DEC_SHORT;
        else if (bs[off] != 0xff || bs[off + 1] != 0x11) status = JXS_E_DEC_BITSTREAM;
        else s_end = (uint32_t)(off + 2);
    }
    head[0] = (uint32_t)status;
    head[1] = status ? 0u : s_end;
}

static std::mutex g_mu;

/* The device that owns device memory p, or -1 for host memory or an unknown
 * pointer. */
static int device_of(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? a.device : -1;
}

extern "C" int32_t jxs_gpu_dec_locate_noalloc(jxs_gpu_dec_t* d, const void* dev_bs, uint32_t size, uint32_t* frame_size,
                                              uint32_t* prec_off, uint32_t cap, void* stream) {
    const jxs_cfg_t* dcfg = NULL;
    const jxs_cfg_t* c = jxs_gpu_dec_cfg(d, &dcfg);
    if (!c || !dev_bs || !frame_size) return JXS_E_DEC_PTR;
    *frame_size = 0;
    if (!jxs_gpu_is_device_ptr(dev_bs)) return JXS_E_DEC_PTR;
    if (c->nprec > NOALLOC_MAX_PRECINCTS) {
        fprintf(stderr,
                "svt_jpeg_xs_gpu_decoder_locate_frame: the frame has %u precincts; this entry point holds at most %u\n",
                c->nprec, NOALLOC_MAX_PRECINCTS);
        return JXS_E_BAD_PARAM;
    }
    if (prec_off && cap < c->nprec) {
        fprintf(stderr, "svt_jpeg_xs_gpu_decoder_locate_frame: room for %u precinct offsets, the frame has %u\n", cap, c->nprec);
        return JXS_E_BAD_PARAM;
    }
    if (size < c->hdr_len) return JXS_E_DEC_SHORT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return JXS_E_UNDEFINED;
    /* the kernel reads both, so both must be on the device it runs on */
    if (device_of(dcfg) != dev || device_of(dev_bs) != dev) {
        fprintf(stderr,
                "svt_jpeg_xs_gpu_decoder_locate_frame: the decoder and the codestream must be on the current device (%d)\n",
                dev);
        return JXS_E_DEC_PTR;
    }
    const cudaStream_t st = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lock(g_mu);
    void* addr = NULL;
    if (cudaGetSymbolAddress(&addr, noalloc_scratch) != cudaSuccess || !addr) {
        cudaGetLastError();
        return JXS_E_UNDEFINED;
    }
    uint32_t* scratch = (uint32_t*)addr;
    /* the stream's constant header must be the decoder's, Lcod aside */
    uint8_t hdr[sizeof(c->hdr)];
    if (cudaMemcpyAsync(hdr, dev_bs, c->hdr_len, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return JXS_E_UNDEFINED;
    if (memcmp(hdr, c->hdr, 12) != 0 || memcmp(hdr + 16, c->hdr + 16, c->hdr_len - 16) != 0) return JXS_E_DEC_CONFIG;
    locate_frame_kernel<<<1, NOALLOC_THREADS, 0, st>>>(dcfg, (const uint8_t*)dev_bs, size);
    uint32_t res[2] = {0, 0};
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(res, scratch, sizeof(res), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return JXS_E_UNDEFINED;
    if (res[0]) return (int32_t)res[0];
    if (prec_off) {
        if (cudaMemcpyAsync(prec_off, scratch + NOALLOC_HEAD_WORDS, (size_t)c->nprec * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return JXS_E_UNDEFINED;
    }
    *frame_size = res[1];
    return 0;
}
