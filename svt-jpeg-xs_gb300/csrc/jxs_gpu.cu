/*
 * Launch orchestration: per-slot device buffers, streams and the kernel
 * sequences of one encode or decode.
 *
 * Encode of one frame on a slot's stream:
 *   [H2D planes] -> fwd_dwt (one launch per vertical level, all components)
 *   -> rc_cost (with the slices' selection) -> pack -> status to the host
 *   -> [D2H codestream]
 * Decode:
 *   [H2D codestream] -> unpack (precinct offsets read in place from
 *   page-locked host memory when walked on the host) -> inv_dwt (one launch
 *   per vertical level, deepest first; the first level writes the output
 *   samples) -> status to the host -> [D2H planes]
 * Copies into pageable host memory run on the completion thread once the
 * frame is done (DeferredCopy).
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <sys/mman.h>
#include <unistd.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "SvtJpegxs.h"
#include "jxs_batch.h"
#include "jxs_gpu.h"
#include "jxs_kernels.cuh"
#include "jxs_plan.cuh"

#define CK(x)                                                                                      \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess) {                                                                   \
            fprintf(stderr, "jxs: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            return JXS_E_RESOURCES;                                                                \
        }                                                                                          \
    } while (0)

/* timing mode: events around every kernel of a frame */
#define JXS_KEV 17
#define KMARK()                                                          \
    do {                                                                 \
        if (s->timed && s->nkev < JXS_KEV) CK(cudaEventRecord(s->kev[s->nkev++], st)); \
    } while (0)

extern "C" int jxs_gpu_is_device_ptr(const void* p) {
    if (!p) return 0;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

/* Host memory the copy engines reach asynchronously: page-locked
 * (cudaMallocHost) or registered.  Ordinary (pageable) memory is not. */
extern "C" int jxs_gpu_is_page_locked(const void* p) {
    if (!p) return 0;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return a.type == cudaMemoryTypeHost;
}

/* A frame's final status into page-locked host memory, written by the GPU
 * after the frame's last compute kernel: no 4-byte copy waits in the copy
 * engines' queues between the frames' large transfers. */
__global__ void publish_status_kernel(int* __restrict__ host, const int* __restrict__ status) {
    if (threadIdx.x == 0) *(volatile int*)host = *(const volatile int*)status;
}

/* Copies from host memory by a kernel.  On a GB300 behind NVLink-C2C with
 * the host's page tables shared with the GPU
 * (cudaDevAttrPageableMemoryAccessUsesHostPageTables), a kernel reads
 * pageable memory directly: the copy is ordered in the frame's stream like
 * any kernel and the calling thread does not wait, while the CUDA copy of
 * pageable memory stages it through the driver on the calling thread.  The
 * encoder's codestream goes to page-locked memory the same way (see
 * enc_run).  The caller's buffers are the library's until the frame is
 * returned, as with the reference (EncHandle.c:1006 keeps only the input
 * structure, and its workers read the planes later). */
__global__ void __launch_bounds__(256) host_copy16_kernel(uint8_t* dst, size_t dpitch, const uint8_t* src, size_t spitch,
                                                          uint32_t chunks) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x < chunks) *(uint4*)(dst + y * dpitch + 16 * (size_t)x) = *(const uint4*)(src + y * spitch + 16 * (size_t)x);
}
__global__ void __launch_bounds__(256) host_copy1_kernel(uint8_t* dst, size_t dpitch, const uint8_t* src, size_t spitch,
                                                         uint32_t width) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x < width) dst[y * dpitch + x] = src[y * spitch + x];
}

/* 1: kernels may access this device's pageable host memory through the
 * host's page tables (queried once per device) */
static int pageable_direct(void) {
    static std::atomic<int> q[JXS_MAX_DEV];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= JXS_MAX_DEV) {
        cudaGetLastError();
        return 0;
    }
    int v = q[dev].load();
    if (v == 0) {
        int a = 0, b = 0;
        if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
            cudaGetLastError();
            a = b = 0;
        }
        v = (a && b) ? 1 : 2;
        q[dev].store(v);
    }
    return v == 1;
}

/* 1: every page of [p, p + bytes) is resident.  A GPU access to a page
 * that is not (memory never touched since it was allocated, or swapped out)
 * is a page fault served over the link, far slower than the driver's copy,
 * which takes the faults on the CPU. */
static int host_resident(const void* p, size_t bytes) {
    static thread_local std::vector<unsigned char> vec;
    const uintptr_t pg = (uintptr_t)sysconf(_SC_PAGESIZE);
    const uintptr_t a = (uintptr_t)p & ~(pg - 1), e = ((uintptr_t)p + bytes + pg - 1) & ~(pg - 1);
    const size_t n = (e - a) / pg;
    if (vec.size() < n) vec.resize(n);
    if (mincore((void*)a, e - a, vec.data()) != 0) return 0;
    for (size_t i = 0; i < n; i++)
        if (!(vec[i] & 1)) return 0;
    return 1;
}

/* A 2-D copy with one side in host memory (`host`, pageable or page-locked)
 * by a copy kernel, when the device reaches pageable memory directly and the
 * host side's pages are resident; returns 0 otherwise (the caller then
 * copies another way). */
static int host_copy_kernel(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t rows, cudaStream_t st,
                            cudaError_t* err, const void* host, size_t host_pitch) {
    *err = cudaSuccess;
    if (!pageable_direct()) return 0;
    if (!width || !rows) return 1;
    if (!host_resident(host, (rows - 1) * host_pitch + width)) return 0;
    if (rows > 65535 || width > 0xffffffffull) return 0;
    /* a thread per 16-byte chunk (or byte), a grid row per row */
    const int v16 = (((uintptr_t)dst | (uintptr_t)src | dpitch | spitch | width) & 15) == 0;
    const size_t items = v16 ? width / 16 : width;
    const dim3 grid((unsigned)((items + 255) / 256), (unsigned)rows);
    if (v16) host_copy16_kernel<<<grid, 256, 0, st>>>((uint8_t*)dst, dpitch, (const uint8_t*)src, spitch, (uint32_t)items);
    else host_copy1_kernel<<<grid, 256, 0, st>>>((uint8_t*)dst, dpitch, (const uint8_t*)src, spitch, (uint32_t)items);
    *err = cudaGetLastError();
    return 1;
}

/* A device-to-host copy into pageable memory, left for the frame's
 * completion: cudaMemcpy*Async into pageable memory returns only once the
 * copy is done, which would make the submitting call wait for the whole
 * frame.  The completion thread copies once the frame's work has finished,
 * on the slot's own stream (idle by then): the copy engines take it, while
 * copy kernels in both directions would share the host link worse, and a
 * synchronous copy on the legacy stream would serialise the handles'
 * completion threads (4K 4:2:2 10-bit from and to pageable memory: encode
 * + decode 18.1 -> 23.9 Gpix/s, decode alone 36.5 -> 44.1). */
struct DeferredCopy {
    void* dst;
    size_t dpitch;
    const void* src;
    size_t spitch, width, height;
};
static int run_deferred(DeferredCopy* d, int* n, cudaStream_t st) {
    int ok = 1;
    for (int i = 0; i < *n; i++)
        if (cudaMemcpy2DAsync(d[i].dst, d[i].dpitch, d[i].src, d[i].spitch, d[i].width, d[i].height, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess) {
            cudaGetLastError();
            ok = 0;
        }
    if (*n && cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        ok = 0;
    }
    *n = 0;
    return ok;
}

extern "C" void* jxs_gpu_host_alloc(size_t n) {
    void* p = NULL;
    if (cudaMallocHost(&p, n) != cudaSuccess) {
        cudaGetLastError();
        return malloc(n);
    }
    return p;
}

extern "C" void jxs_gpu_host_free(void* p) {
    if (!p) return;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost) {
        cudaFreeHost(p);
    } else {
        cudaGetLastError();
        free(p);
    }
}

extern "C" int jxs_gpu_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

/* ------------------------------------------------------------------------ */
/* Encoder                                                                   */
/* ------------------------------------------------------------------------ */
struct EncSlot {
    cudaStream_t st;
    cudaEvent_t done;
    uint8_t* in_stage;      /* staging for host planes */
    uint64_t in_off[JXS_MAXC];
    uint16_t* coef;
    uint8_t* gcli;
    int32_t* ll[2][JXS_MAXC];   /* int32 low band after vertical level 0 / 1 */
    int ll_pitch[2][JXS_MAXC];
    uint32_t* cost;
    uint32_t* slice_done;   /* per slice: cost blocks finished (back to 0 after each frame) */
    PrecRC* rc;
    int* status;
    uint8_t* out_stage;
    int* status_h;
    int* status_hd;       /* status_h as the device addresses it */
    int busy;
    DeferredCopy defer[1];  /* the codestream, for a pageable destination */
    int ndefer;
    cudaEvent_t tev[6];
    cudaEvent_t kev[JXS_KEV];   /* timing mode: before the first kernel and after each */
    int nkev;
    int timed;
};

/* encoder stages timed with CUDA events: H2D, transform, rate control, packing, D2H */
#define ENC_STAGES 5

struct jxs_gpu_enc {
    jxs_cfg_t cfg;
    jxs_cfg_t* dcfg;
    int nslots;
    EncSlot slot[8];
    uint32_t cap_words;
    cudaStream_t user_stream[8]; /* per slot; null: the slot's own stream */
    int timing;
    double stage_ms[ENC_STAGES];
    double kern_ms[JXS_KEV];
    int nkern;
    uint64_t timed_frames;
    uint64_t serial;             /* process-unique: identifies the handle's layout to the batch engine */
    std::mutex mu;
};

static std::atomic<uint64_t> g_serial{1};

static inline cudaStream_t enc_stream(const jxs_gpu_enc_t* e, const EncSlot* s) {
    const cudaStream_t u = e->user_stream[s - e->slot];
    return u ? u : s->st;
}

static int32_t enc_slot_alloc(jxs_gpu_enc_t* e, EncSlot* s) {
    const jxs_cfg_t* c = &e->cfg;
    memset(s, 0, sizeof(*s));
    CK(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming));
    uint64_t in_bytes = 0;
    const uint32_t bps = bytes_per_sample(c);
    if (c->fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB) {
        s->in_off[0] = 0;
        in_bytes = (uint64_t)c->W * c->H * 3 * bps;
    } else {
        for (uint32_t k = 0; k < c->nc; k++) {
            s->in_off[k] = in_bytes;
            in_bytes += ((uint64_t)stage_pitch(c->comp[k].w, bps) * c->comp[k].h * bps + 255) & ~255ull;
        }
    }
    CK(cudaMalloc(&s->in_stage, in_bytes));
    CK(cudaMalloc(&s->coef, c->coef_total * sizeof(uint16_t) + 64));
    CK(cudaMalloc(&s->gcli, c->gcli_total + 64));
    for (uint32_t k = 0; k < c->nc; k++) {
        for (uint32_t v = 0; v < c->comp[k].dv && v < 2; v++) {
            uint32_t w, h;
            level_dims(c->comp[k], (int)v + 1, &w, &h);
            s->ll_pitch[v][k] = (int)((w + 3) & ~3u);
            CK(cudaMalloc(&s->ll[v][k], (size_t)s->ll_pitch[v][k] * h * sizeof(int32_t) + 64));
        }
    }
        CK(cudaMalloc(&s->cost, jxs_cost_bytes(c)));
    CK(cudaMalloc(&s->slice_done, (size_t)c->nslices * sizeof(uint32_t)));
    CK(cudaMemset(s->slice_done, 0, (size_t)c->nslices * sizeof(uint32_t)));
    CK(cudaMalloc(&s->rc, (size_t)c->np * sizeof(PrecRC)));
    CK(cudaMalloc(&s->status, 64));
    CK(cudaMalloc(&s->out_stage, c->lcod + 64));
    CK(cudaMallocHost(&s->status_h, 64));
    *s->status_h = 0;
    CK(cudaHostGetDevicePointer((void**)&s->status_hd, s->status_h, 0));
    for (int i = 0; i < 6; i++) CK(cudaEventCreate(&s->tev[i]));
    for (int i = 0; i < JXS_KEV; i++) CK(cudaEventCreate(&s->kev[i]));
    return JXS_OK;
}

static void enc_slot_free(EncSlot* s) {
    if (s->st) cudaStreamSynchronize(s->st);
    cudaFree(s->in_stage);
    cudaFree(s->coef);
    cudaFree(s->gcli);
    for (int v = 0; v < 2; v++)
        for (int k = 0; k < JXS_MAXC; k++) cudaFree(s->ll[v][k]);
    cudaFree(s->cost);
    cudaFree(s->slice_done);
    cudaFree(s->rc);
    cudaFree(s->status);
    cudaFree(s->out_stage);
    if (s->status_h) cudaFreeHost(s->status_h);
    for (int i = 0; i < 6; i++)
        if (s->tev[i]) cudaEventDestroy(s->tev[i]);
    for (int i = 0; i < JXS_KEV; i++)
        if (s->kev[i]) cudaEventDestroy(s->kev[i]);
    if (s->done) cudaEventDestroy(s->done);
    if (s->st) cudaStreamDestroy(s->st);
    memset(s, 0, sizeof(*s));
}

extern "C" void jxs_gpu_enc_destroy(jxs_gpu_enc_t* e) {
    if (!e) return;
    for (int i = 0; i < e->nslots; i++) enc_slot_free(&e->slot[i]);
    cudaFree(e->dcfg);
    delete e;
}

extern "C" jxs_gpu_enc_t* jxs_gpu_enc_create(const jxs_cfg_t* cfg, int nslots, int32_t* err) {
    *err = JXS_OK;
    if (jxs_gpu_device_count() == 0) {
        fprintf(stderr, "jxs: no CUDA device available; this library has no CPU fallback\n");
        *err = JXS_E_RESOURCES;
        return NULL;
    }
    if (nslots < 1) nslots = 1;
    if (nslots > 8) nslots = 8;
    jxs_gpu_enc_t* e = new jxs_gpu_enc_t();
    memset(&e->slot, 0, sizeof(e->slot));
    e->cfg = *cfg;
    e->nslots = 0;
    e->serial = g_serial++;
    /* the packing kernel stages a whole precinct in shared memory, starting
     * up to 15 bytes into the buffer for aligned stores: bound it by the
     * largest slice budget (the kernel's static shared memory, up to 34 KB,
     * comes on top) */
    e->cap_words = 4 * div_up(cfg->max_slice_budget + 15, 16) + 4;
    if ((size_t)e->cap_words * 4 > kSmemMax - 28 * 1024) {
        fprintf(stderr, "jxs: precincts of this configuration (%u bytes per slice) exceed the on-chip packing buffer\n",
                cfg->max_slice_budget);
        delete e;
        *err = JXS_E_BAD_PARAM;
        return NULL;
    }
    if (cudaMalloc(&e->dcfg, sizeof(jxs_cfg_t)) != cudaSuccess ||
        cudaMemcpy(e->dcfg, cfg, sizeof(jxs_cfg_t), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        delete e;
        *err = JXS_E_RESOURCES;
        return NULL;
    }
    for (int i = 0; i < nslots; i++) {
        if (enc_slot_alloc(e, &e->slot[i]) != JXS_OK) {
            e->nslots = i + 1;
            jxs_gpu_enc_destroy(e);
            *err = JXS_E_RESOURCES;
            return NULL;
        }
    }
    e->nslots = nslots;
    return e;
}

static int32_t enc_run(jxs_gpu_enc_t* e, EncSlot* s, void* const planes[4], const uint32_t strides[4], uint8_t* out) {
    s->ndefer = 0;
    const jxs_cfg_t* c = &e->cfg;
    const int packed = c->fmt == COLOUR_FORMAT_PACKED_YUV444_OR_RGB;
    const uint32_t bps = bytes_per_sample(c);
    const cudaStream_t st = enc_stream(e, s);
    s->timed = e->timing;
#define TMARK(i) \
    if (s->timed) CK(cudaEventRecord(s->tev[i], st))
    TMARK(0);
    CK(cudaMemsetAsync(s->status, 0, sizeof(int), st));
    /* sources of the first level: caller device planes read in place, host
     * planes staged with one 2-D copy each */
    const void* src[JXS_MAXC];
    long long pitch[JXS_MAXC];
    const int nplanes = packed ? 1 : (int)c->nc;
    for (int k = 0; k < nplanes; k++) {
        const uint32_t w = packed ? c->W * 3 : c->comp[k].w, h = packed ? c->H : c->comp[k].h;
        if (jxs_gpu_is_device_ptr(planes[k])) {
            src[k] = planes[k];
            pitch[k] = strides[k];
        } else {
            uint8_t* d = s->in_stage + s->in_off[k];
            const uint32_t sp = packed ? w : stage_pitch(w, bps);
            cudaError_t ce = cudaSuccess;
            if (!jxs_gpu_is_page_locked(planes[k]) &&
                host_copy_kernel(d, (size_t)sp * bps, planes[k], (size_t)strides[k] * bps, (size_t)w * bps, h, st, &ce, planes[k],
                                 (size_t)strides[k] * bps))
                CK(ce);
            else
                CK(cudaMemcpy2DAsync(d, (size_t)sp * bps, planes[k], (size_t)strides[k] * bps, (size_t)w * bps, h,
                                     cudaMemcpyHostToDevice, st));
            src[k] = d;
            pitch[k] = sp;
        }
    }
    TMARK(1);
    s->nkev = 0;
    KMARK();
    /* forward transform: one launch per vertical level, then the
     * horizontal-only levels of every component (one launch per source
     * kind) */
    FrameBufs fb;
    memset(&fb, 0, sizeof(fb));
    fb.coef = s->coef;
    fb.gcli = s->gcli;
    memcpy(fb.ll, s->ll, sizeof(fb.ll));
    memcpy(fb.ll_pitch, s->ll_pitch, sizeof(fb.ll_pitch));
    FramePlanes in;
    memset(&in, 0, sizeof(in));
    for (int k = 0; k < nplanes; k++) {
        in.p[k] = (void*)src[k];
        in.pitch[k] = pitch[k];
    }
    const int level0_kind = enc_level0_kind(c);
    const int max_dv = (int)cfg_max_dv(c);
    for (int v = 0; v < max_dv; v++) {
        FwdVLaunch L;
        memset(&L, 0, sizeof(L));
        int tiles[JXS_MAXC];
        L.njobs = plan_fwd_v(c, e->dcfg, fb, in, v, L.job, tiles);
        for (int i = 0; i < L.njobs; i++) {
            L.job[i].first_block = L.ntiles;
            L.ntiles += tiles[i];
        }
        CK(jxs_launch_fwd_v(&L, v == 0 ? level0_kind : SRC_I32, 0, st));
        KMARK();
    }
    for (int pass = 0; pass < 2; pass++) {
        FwdHLaunch L;
        memset(&L, 0, sizeof(L));
        L.njobs = plan_fwd_h(c, e->dcfg, fb, in, pass, L.job);
        if (!L.njobs) continue;
        const int blocks = fwd_h_layout(L, jxs_fwd_h_max_rows_per_block());
        if (blocks < 0) return JXS_E_BAD_PARAM;
        CK(jxs_launch_fwd_h(&L, pass == 0 ? SRC_I32 : level0_kind, blocks, st));
        KMARK();
    }
    TMARK(2);
    CK(jxs_launch_rc(e->dcfg, c->np, c->nslices, s->gcli, s->coef, s->cost, s->slice_done, s->rc, s->status,
                     (c->fs ? 1 : 0) | (c->vpred ? 2 : 0), st));
    KMARK();
    TMARK(3);
    const int out_dev = jxs_gpu_is_device_ptr(out);
    uint8_t* dst = out_dev ? out : s->out_stage;
    CK(jxs_launch_pack(e->dcfg, c->np, s->coef, s->gcli, s->rc, s->cost, dst, e->cap_words, s->status, c->vpred ? 2 : 0, st));
    KMARK();
    publish_status_kernel<<<1, 32, 0, st>>>(s->status_hd, s->status);
    CK(cudaGetLastError());
    TMARK(4);
    s->ndefer = 0;
    if (!out_dev) {
        cudaError_t ce = cudaSuccess;
        /* into page-locked memory the codestream (a tenth of the frame's
         * bytes) goes by a copy kernel: the copy engines then carry only the
         * planes, with no small copy queued between them (encode + decode
         * from host memory: 32.2 -> 34.1 Gpix/s, 4K 4:2:2 10-bit); into
         * pageable memory it is left to the completion thread */
        const int locked = jxs_gpu_is_page_locked(out);
        if (locked && host_copy_kernel(out, c->lcod, s->out_stage, c->lcod, c->lcod, 1, st, &ce, out, c->lcod)) CK(ce);
        else if (locked) CK(cudaMemcpyAsync(out, s->out_stage, c->lcod, cudaMemcpyDeviceToHost, st));
        else s->defer[s->ndefer++] = DeferredCopy{out, c->lcod, s->out_stage, c->lcod, c->lcod, 1};
    }
    TMARK(5);
#undef TMARK
    CK(cudaEventRecord(s->done, st));
    return JXS_OK;
}

extern "C" int32_t jxs_gpu_enc_submit(jxs_gpu_enc_t* e, int slot, void* const planes[4], const uint32_t strides[4], uint8_t* out) {
    if (!e || slot < 0 || slot >= e->nslots) return JXS_E_BAD_PARAM;
    EncSlot* s = &e->slot[slot];
    s->busy = 1;
    return enc_run(e, s, planes, strides, out);
}

extern "C" int32_t jxs_gpu_enc_wait(jxs_gpu_enc_t* e, int slot) {
    EncSlot* s = &e->slot[slot];
    if (cudaEventSynchronize(s->done) != cudaSuccess) {
        fprintf(stderr, "jxs: encode failed: %s\n", cudaGetErrorString(cudaGetLastError()));
        s->ndefer = 0;
        return JXS_E_ENC_FRAME;
    }
    if (!run_deferred(s->defer, &s->ndefer, s->st)) {
        fprintf(stderr, "jxs: copying the codestream to host memory failed\n");
        return JXS_E_ENC_FRAME;
    }
    s->busy = 0;
    if (s->timed) {
        float ms[ENC_STAGES];
        for (int i = 0; i < ENC_STAGES; i++)
            if (cudaEventElapsedTime(&ms[i], s->tev[i], s->tev[i + 1]) != cudaSuccess) ms[i] = 0.f;
        std::lock_guard<std::mutex> g(e->mu);
        for (int i = 0; i < ENC_STAGES; i++) e->stage_ms[i] += ms[i];
        for (int i = 0; i + 1 < s->nkev; i++) {
            float k = 0.f;
            if (cudaEventElapsedTime(&k, s->kev[i], s->kev[i + 1]) == cudaSuccess) e->kern_ms[i] += k;
        }
        e->nkern = s->nkev > 0 ? s->nkev - 1 : 0;
        e->timed_frames++;
        s->timed = 0;
    }
    return *s->status_h ? JXS_E_ENC_FRAME : JXS_OK;
}

extern "C" void jxs_gpu_enc_set_stream(jxs_gpu_enc_t* e, void* stream) {
    for (int i = 0; i < 8; i++) e->user_stream[i] = (cudaStream_t)stream;
}
extern "C" void jxs_gpu_enc_set_streams(jxs_gpu_enc_t* e, void* const* streams, int n) {
    for (int i = 0; i < 8; i++) e->user_stream[i] = n > 0 ? (cudaStream_t)streams[i % n] : (cudaStream_t)0;
}
extern "C" int jxs_gpu_enc_slots(jxs_gpu_enc_t* e) { return e->nslots; }

extern "C" void jxs_gpu_enc_set_timing(jxs_gpu_enc_t* e, int on) {
    std::lock_guard<std::mutex> g(e->mu);
    e->timing = on;
    for (int i = 0; i < ENC_STAGES; i++) e->stage_ms[i] = 0;
    for (int i = 0; i < JXS_KEV; i++) e->kern_ms[i] = 0;
    e->timed_frames = 0;
}

extern "C" int jxs_gpu_enc_read_kernel_timing(jxs_gpu_enc_t* e, double* ms, int n) {
    std::lock_guard<std::mutex> g(e->mu);
    for (int i = 0; i < n && i < JXS_KEV; i++) ms[i] = e->kern_ms[i];
    return e->nkern;
}

extern "C" uint64_t jxs_gpu_enc_read_timing(jxs_gpu_enc_t* e, double* ms, int n) {
    std::lock_guard<std::mutex> g(e->mu);
    for (int i = 0; i < n && i < ENC_STAGES; i++) ms[i] = e->stage_ms[i];
    return e->timed_frames;
}

extern "C" int jxs_gpu_enc_ready(jxs_gpu_enc_t* e, int slot) {
    cudaError_t r = cudaEventQuery(e->slot[slot].done);
    if (r == cudaErrorNotReady) return 0;
    return 1;
}

extern "C" int32_t jxs_gpu_enc_rc_results(jxs_gpu_enc_t* e, int slot, uint8_t* q, uint8_t* r) {
    EncSlot* s = &e->slot[slot];
    const uint32_t np = e->cfg.np;
    PrecRC* h = (PrecRC*)malloc(sizeof(PrecRC) * np);
    if (!h) return JXS_E_RESOURCES;
    cudaStreamSynchronize(enc_stream(e, s));
    if (cudaMemcpy(h, s->rc, sizeof(PrecRC) * np, cudaMemcpyDeviceToHost) != cudaSuccess) {
        free(h);
        return JXS_E_RESOURCES;
    }
    for (uint32_t i = 0; i < np; i++) {
        q[i] = h[i].q;
        r[i] = h[i].r;
    }
    free(h);
    return JXS_OK;
}

/* ------------------------------------------------------------------------ */
/* Decoder                                                                   */
/* ------------------------------------------------------------------------ */
struct DecSlot {
    cudaStream_t st;
    cudaEvent_t done;
    uint8_t* bs;
    uint32_t bs_cap;
    uint32_t* prec_off;
    int16_t* coef;
    int32_t* ll[2][JXS_MAXC];   /* int32 low band below vertical level 0 / 1 */
    int ll_pitch[2][JXS_MAXC];
    uint8_t* out_stage;
    uint64_t out_off[JXS_MAXC];
    int32_t* mct;               /* colour transform / non-linear output: the int32 planes of the last inverse level */
    uint64_t mct_off[JXS_MAXC];
    int mct_pitch[JXS_MAXC];
    int* status;
    int* status_h;
    int* status_hd;       /* status_h as the device addresses it */
    uint32_t* prec_off_h;
    const uint32_t* prec_off_hd; /* prec_off_h as the device addresses it */
    uint8_t* hdr_h;       /* header of a device-resident codestream, checked at completion */
    int hdr_check;
    /* the frame's arguments, for a second decode slice by slice when it
     * turns out to use vertical prediction */
    const uint8_t* arg_bs;  /* device codestream (the caller's or the slot's copy) */
    uint32_t arg_size;
    int arg_walked;         /* precinct offsets in prec_off_h */
    void* arg_planes[4];
    uint32_t arg_strides[4];
    DeferredCopy defer[JXS_MAXC]; /* output planes in pageable memory */
    int ndefer;
    cudaEvent_t tev[5];
    cudaEvent_t kev[JXS_KEV];
    int nkev;
    int timed;
};

/* decoder stages timed with CUDA events: H2D, unpack, inverse transform, D2H */
#define DEC_STAGES 4

struct jxs_gpu_dec {
    jxs_cfg_t cfg;
    jxs_cfg_t* dcfg;
    int nslots;
    DecSlot slot[8];
    uint32_t cap_bytes, cap_groups, cap_seg;
    cudaStream_t user_stream[8]; /* per slot; null: the slot's own stream */
    int timing;
    double stage_ms[DEC_STAGES];
    double kern_ms[JXS_KEV];
    int nkern;
    uint64_t timed_frames;
    uint64_t serial;
    int vpred;                   /* decode slice by slice: the stream uses vertical prediction */
    std::mutex mu;
};

static inline cudaStream_t dec_stream(const jxs_gpu_dec_t* d, const DecSlot* s) {
    const cudaStream_t u = d->user_stream[s - d->slot];
    return u ? u : s->st;
}

static int32_t dec_slot_alloc(jxs_gpu_dec_t* d, DecSlot* s) {
    const jxs_cfg_t* c = &d->cfg;
    memset(s, 0, sizeof(*s));
    CK(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming));
    s->bs_cap = c->lcod + 4096;
    CK(cudaMalloc(&s->bs, s->bs_cap + 64));
    CK(cudaMalloc(&s->prec_off, (size_t)c->nprec * sizeof(uint32_t)));
    CK(cudaMallocHost(&s->prec_off_h, (size_t)c->nprec * sizeof(uint32_t)));
    CK(cudaHostGetDevicePointer((void**)&s->prec_off_hd, s->prec_off_h, 0));
    CK(cudaMallocHost(&s->hdr_h, sizeof(c->hdr)));
    CK(cudaMalloc(&s->coef, c->coef_total * sizeof(int16_t) + 64));
    for (uint32_t k = 0; k < c->nc; k++) {
        for (uint32_t v = 0; v < c->comp[k].dv && v < 2; v++) {
            uint32_t w, h;
            level_dims(c->comp[k], (int)v + 1, &w, &h);
            s->ll_pitch[v][k] = (int)((w + 3) & ~3u);
            CK(cudaMalloc(&s->ll[v][k], (size_t)s->ll_pitch[v][k] * h * sizeof(int32_t) + 64));
        }
    }
    uint64_t ob = 0;
    const uint32_t bps = bytes_per_sample(c);
    for (uint32_t k = 0; k < c->nc; k++) {
        s->out_off[k] = ob;
        ob += ((uint64_t)stage_pitch(jxs_out_w(c, k), bps) * jxs_out_h(c, k) * bps + 255) & ~255ull;
    }
    CK(cudaMalloc(&s->out_stage, ob));
    if (dec_needs_nlt_pass(c)) {
        uint64_t mb = 0;
        for (uint32_t k = 0; k < c->nc; k++) {
            s->mct_off[k] = mb;
            s->mct_pitch[k] = (int)((jxs_out_w(c, k) + 3) & ~3u);
            mb += ((uint64_t)s->mct_pitch[k] * jxs_out_h(c, k) + 63) & ~63ull;
        }
        CK(cudaMalloc(&s->mct, mb * sizeof(int32_t)));
    }
    CK(cudaMalloc(&s->status, 64));
    CK(cudaMallocHost(&s->status_h, 64));
    *s->status_h = 0;
    CK(cudaHostGetDevicePointer((void**)&s->status_hd, s->status_h, 0));
    for (int i = 0; i < 5; i++) CK(cudaEventCreate(&s->tev[i]));
    for (int i = 0; i < JXS_KEV; i++) CK(cudaEventCreate(&s->kev[i]));
    return JXS_OK;
}

static void dec_slot_free(DecSlot* s) {
    if (s->st) cudaStreamSynchronize(s->st);
    cudaFree(s->bs);
    cudaFree(s->prec_off);
    if (s->prec_off_h) cudaFreeHost(s->prec_off_h);
    if (s->hdr_h) cudaFreeHost(s->hdr_h);
    cudaFree(s->coef);
    for (int v = 0; v < 2; v++)
        for (int k = 0; k < JXS_MAXC; k++) cudaFree(s->ll[v][k]);
    cudaFree(s->out_stage);
    cudaFree(s->mct);
    cudaFree(s->status);
    if (s->status_h) cudaFreeHost(s->status_h);
    for (int i = 0; i < 5; i++)
        if (s->tev[i]) cudaEventDestroy(s->tev[i]);
    for (int i = 0; i < JXS_KEV; i++)
        if (s->kev[i]) cudaEventDestroy(s->kev[i]);
    if (s->done) cudaEventDestroy(s->done);
    if (s->st) cudaStreamDestroy(s->st);
    memset(s, 0, sizeof(*s));
}

extern "C" const jxs_cfg_t* jxs_gpu_dec_cfg(jxs_gpu_dec_t* d, const jxs_cfg_t** dev_cfg) {
    if (!d) return NULL;
    if (dev_cfg) *dev_cfg = d->dcfg;
    return &d->cfg;
}

extern "C" void jxs_gpu_dec_destroy(jxs_gpu_dec_t* d) {
    if (!d) return;
    for (int i = 0; i < d->nslots; i++) dec_slot_free(&d->slot[i]);
    cudaFree(d->dcfg);
    delete d;
}

extern "C" jxs_gpu_dec_t* jxs_gpu_dec_create(const jxs_cfg_t* cfg, int nslots, int32_t* err) {
    *err = JXS_OK;
    if (jxs_gpu_device_count() == 0) {
        fprintf(stderr, "jxs: no CUDA device available; this library has no CPU fallback\n");
        *err = JXS_E_RESOURCES;
        return NULL;
    }
    if (nslots < 1) nslots = 1;
    if (nslots > 8) nslots = 8;
    jxs_gpu_dec_t* d = new jxs_gpu_dec_t();
    memset(&d->slot, 0, sizeof(d->slot));
    d->cfg = *cfg;
    d->serial = g_serial++;
    uint32_t groups = 0;
    for (uint32_t b = 0; b < cfg->nbands; b++) groups += cfg->band[b].gcli_w * cfg->band[b].lines;
    /* + up to 3 groups of alignment per band line (jxs_bline_t.gbase) */
    d->cap_groups = (groups + 3 * JXS_MAXBLINES + 64) & ~31u;
    d->cap_seg = 1;
    for (int k = 0; k < 4; k++) d->cap_seg = d->cap_seg > cfg->nseg[k] ? d->cap_seg : cfg->nseg[k];
    /* the on-chip copy of a precinct: in a constant-bit-rate stream a
     * precinct lies inside its slice, so it needs at most the largest slice
     * budget (plus the 48 bytes the bit readers may look past its end and
     * the alignment lead); without that prediction a quarter more than a
     * slice's share of Lcod.  A precinct that does not fit is reported as an
     * invalid stream. */
    uint64_t cap = (uint64_t)cfg->lcod / (cfg->nslices ? cfg->nslices : 1);
    cap = cfg->max_slice_budget ? cfg->max_slice_budget + 64ull : cap + cap / 4 + 4096;
    if (cap > cfg->lcod + 64ull) cap = cfg->lcod + 64ull;
    const size_t fixed = uk_layout(0, d->cap_groups, d->cap_seg).top_end;
    const size_t room = kSmemMax - UK_STATIC_SMEM;
    if (cap + fixed > room) cap = room > fixed + 4096 ? room - fixed : 4096;
    d->cap_bytes = (uint32_t)(cap + 15) & ~15u;
    if (cudaMalloc(&d->dcfg, sizeof(jxs_cfg_t)) != cudaSuccess ||
        cudaMemcpy(d->dcfg, cfg, sizeof(jxs_cfg_t), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        delete d;
        *err = JXS_E_RESOURCES;
        return NULL;
    }
    for (int i = 0; i < nslots; i++) {
        if (dec_slot_alloc(d, &d->slot[i]) != JXS_OK) {
            d->nslots = i + 1;
            jxs_gpu_dec_destroy(d);
            *err = JXS_E_RESOURCES;
            return NULL;
        }
    }
    d->nslots = nslots;
    return d;
}

static int32_t dec_run(jxs_gpu_dec_t* d, DecSlot* s, const uint8_t* bs, uint32_t size, const uint32_t* prec_off,
                       void* const planes[4], const uint32_t strides[4]) {
    s->ndefer = 0;
    const jxs_cfg_t* c = &d->cfg;
    const uint32_t bps = bytes_per_sample(c);
    const cudaStream_t st = dec_stream(d, s);
    s->timed = d->timing;
#define TMARK(i) \
    if (s->timed) CK(cudaEventRecord(s->tev[i], st))
    TMARK(0);
    CK(cudaMemsetAsync(s->status, 0, sizeof(int), st));
    const uint8_t* dbs = bs;
    s->hdr_check = 0;
    s->nkev = 0;
    if (!prec_off) {
        /* device-resident codestream: header compared at completion, precinct
         * offsets found on the GPU */
        if (!jxs_gpu_is_device_ptr(bs) || size < c->hdr_len) return JXS_E_DEC_PTR;
        CK(cudaMemcpyAsync(s->hdr_h, bs, c->hdr_len, cudaMemcpyDeviceToHost, st));
        s->hdr_check = 1;
        CK(cudaMemsetAsync(s->status + 1, 0, sizeof(int), st));
        KMARK();
        CK(jxs_launch_walk(d->dcfg, c->nslices, bs, size, s->prec_off, s->status + 1, s->status, st));
    } else if (!jxs_gpu_is_device_ptr(bs)) {
        if (size > s->bs_cap) {
            CK(cudaStreamSynchronize(st));
            cudaFree(s->bs);
            s->bs_cap = size + 4096;
            CK(cudaMalloc(&s->bs, s->bs_cap + 64));
        }
        cudaError_t ce = cudaSuccess;
        /* by a copy kernel also from page-locked memory, as the encoder's
         * codestream: the copy engines carry only the planes */
        if (host_copy_kernel(s->bs, size, bs, size, size, 1, st, &ce, bs, size)) CK(ce);
        else CK(cudaMemcpyAsync(s->bs, bs, size, cudaMemcpyHostToDevice, st));
        dbs = s->bs;
    }
    if (prec_off) {
        /* the previous use of prec_off_h by this slot has completed: slots are
         * reused only after their completion was observed */
        if (prec_off != s->prec_off_h) memcpy(s->prec_off_h, prec_off, sizeof(uint32_t) * c->nprec);
    }
    /* host-walked offsets are read by the unpacking blocks straight from the
     * page-locked buffer (one word per block), not copied */
    const uint32_t* doff = prec_off ? s->prec_off_hd : s->prec_off;
    s->arg_bs = dbs;
    s->arg_size = size;
    s->arg_walked = prec_off != NULL;
    for (int k = 0; k < 4; k++) {
        s->arg_planes[k] = planes[k];
        s->arg_strides[k] = strides[k];
    }
    TMARK(1);
    KMARK();
    if (d->vpred)
        CK(jxs_launch_unpack_vpred(d->dcfg, dbs, size, doff, s->coef, c->nslices, d->cap_bytes, d->cap_groups, d->cap_seg,
                                   s->status, st));
    else
        CK(jxs_launch_unpack(d->dcfg, dbs, size, doff, s->coef, c->nprec, d->cap_bytes, d->cap_groups, d->cap_seg, s->status,
                             st));
    KMARK();
    TMARK(2);

    int out_dev[JXS_MAXC];
    for (uint32_t k = 0; k < c->nc; k++) out_dev[k] = jxs_gpu_is_device_ptr(planes[k]);
    /* horizontal-only levels of every component (into the int32 low band of
     * its last vertical level, or straight to the output plane), then the
     * vertical levels from the deepest up */
    FrameBufs fb;
    memset(&fb, 0, sizeof(fb));
    fb.coef = s->coef;
    memcpy(fb.ll, s->ll, sizeof(fb.ll));
    memcpy(fb.ll_pitch, s->ll_pitch, sizeof(fb.ll_pitch));
    FramePlanes out;
    memset(&out, 0, sizeof(out));
    for (uint32_t k = 0; k < c->nc; k++) {
        if (out_dev[k]) {
            out.p[k] = planes[k];
            out.pitch[k] = strides[k];
        } else {
            out.p[k] = s->out_stage + s->out_off[k];
            out.pitch[k] = stage_pitch(jxs_out_w(c, k), bps);
        }
    }
    /* a colour transform or a non-linear output: the last inverse level
     * writes int32 planes, nlt_out_kernel writes the samples */
    const int nlt_pass = dec_needs_nlt_pass(c);
    FramePlanes lout = out;
    if (nlt_pass)
        for (uint32_t k = 0; k < c->nc; k++) {
            lout.p[k] = s->mct + s->mct_off[k];
            lout.pitch[k] = s->mct_pitch[k];
        }
    const int sample_kind = nlt_pass ? 0 : dec_sample_kind(c);
    for (int pass = 0; pass < 2; pass++) {
        InvHLaunch L;
        memset(&L, 0, sizeof(L));
        L.njobs = plan_inv_h(c, d->dcfg, fb, lout, pass, L.job);
        if (!L.njobs) continue;
        const int blocks = inv_h_layout(L, jxs_inv_h_max_rows_per_block());
        if (blocks < 0) return JXS_E_BAD_PARAM;
        CK(jxs_launch_inv_h(&L, pass == 0 ? 0 : sample_kind, blocks, st));
        KMARK();
    }
    for (int v = (int)cfg_max_dv(c) - 1; v >= (int)c->proxy; v--) {
        InvVLaunch L;
        memset(&L, 0, sizeof(L));
        int tiles[JXS_MAXC], blocks = 0;
        L.njobs = plan_inv_v(c, d->dcfg, fb, lout, v, L.job, tiles);
        for (int i = 0; i < L.njobs; i++) {
            L.job[i].first_block = blocks;
            blocks += tiles[i];
        }
        if (!L.njobs) continue;
        CK(jxs_launch_inv_v(&L, v > (int)c->proxy ? 0 : sample_kind, blocks, st));
        KMARK();
    }
    if (nlt_pass) {
        FramePlanes tin = lout;
        if (c->cpih == 3) {
            /* inverse Star-Tetrix in place, then components 0 <-> 2 and
             * 1 <-> 3 (inverse_star_tetrix, Mct.c:120-135) */
            StParams T;
            memset(&T, 0, sizeof(T));
            for (int k = 0; k < 4; k++) T.c[k] = (int32_t*)lout.p[k];
            T.pitch = lout.pitch[0];
            T.w = (int)jxs_out_w(c, 0);
            T.h = (int)jxs_out_h(c, 0);
            T.cf = (int)c->cts_cf;
            T.ct = (int)c->cfa_type;
            T.e1 = (int)c->cts_e1;
            T.e2 = (int)c->cts_e2;
            CK(jxs_launch_star_tetrix(&T, st));
            const int perm[4] = {2, 3, 0, 1};
            for (int k = 0; k < 4; k++) {
                tin.p[k] = lout.p[perm[k]];
                tin.pitch[k] = lout.pitch[perm[k]];
            }
        }
        NltOut P;
        nlt_out_params(c, tin, out, &P);
        CK(jxs_launch_nlt_out(&P, st));
    }
    publish_status_kernel<<<1, 32, 0, st>>>(s->status_hd, s->status);
    CK(cudaGetLastError());
    TMARK(3);
    s->ndefer = 0;
    for (uint32_t k = 0; k < c->nc; k++) {
        if (out_dev[k]) continue;
        const uint32_t ow = jxs_out_w(c, k), oh = jxs_out_h(c, k);
        const DeferredCopy cp{planes[k], (size_t)strides[k] * bps, s->out_stage + s->out_off[k], (size_t)stage_pitch(ow, bps) * bps,
                              (size_t)ow * bps, oh};
        /* pageable planes are left to the completion thread */
        if (jxs_gpu_is_page_locked(planes[k]))
            CK(cudaMemcpy2DAsync(cp.dst, cp.dpitch, cp.src, cp.spitch, cp.width, cp.height, cudaMemcpyDeviceToHost, st));
        else
            s->defer[s->ndefer++] = cp;
    }
    TMARK(4);
#undef TMARK
    CK(cudaEventRecord(s->done, st));
    return JXS_OK;
}

extern "C" int32_t jxs_gpu_dec_submit(jxs_gpu_dec_t* d, int slot, const uint8_t* bs, uint32_t size, const uint32_t* prec_off,
                                      void* const planes[4], const uint32_t strides[4]) {
    if (!d || slot < 0 || slot >= d->nslots) return JXS_E_BAD_PARAM;
    return dec_run(d, &d->slot[slot], bs, size, prec_off, planes, strides);
}

extern "C" int32_t jxs_gpu_dec_wait(jxs_gpu_dec_t* d, int slot) {
    DecSlot* s = &d->slot[slot];
    if (cudaEventSynchronize(s->done) != cudaSuccess) {
        fprintf(stderr, "jxs: decode failed: %s\n", cudaGetErrorString(cudaGetLastError()));
        s->ndefer = 0;
        return JXS_E_DEC_INTERNAL;
    }
    if (*s->status_h == JXS_E_DEC_VPRED) {
        /* the frame uses vertical prediction: decode it again slice by slice,
         * and the stream's later frames that way from the start */
        d->vpred = 1;
        const int32_t r = dec_run(d, s, s->arg_bs, s->arg_size, s->arg_walked ? s->prec_off_h : NULL, s->arg_planes,
                                  s->arg_strides);
        if (r != JXS_OK) return r;
        if (cudaEventSynchronize(s->done) != cudaSuccess) {
            fprintf(stderr, "jxs: decode failed: %s\n", cudaGetErrorString(cudaGetLastError()));
            s->ndefer = 0;
            return JXS_E_DEC_INTERNAL;
        }
    }
    if (!run_deferred(s->defer, &s->ndefer, s->st)) {
        fprintf(stderr, "jxs: copying the decoded planes to host memory failed\n");
        return JXS_E_DEC_INTERNAL;
    }
    if (s->timed) {
        float ms[DEC_STAGES];
        for (int i = 0; i < DEC_STAGES; i++)
            if (cudaEventElapsedTime(&ms[i], s->tev[i], s->tev[i + 1]) != cudaSuccess) ms[i] = 0.f;
        std::lock_guard<std::mutex> g(d->mu);
        for (int i = 0; i < DEC_STAGES; i++) d->stage_ms[i] += ms[i];
        /* kernels in launch order: the precinct walk (device codestreams
         * only), unpack, the inverse transform launches */
        for (int i = 0; i + 1 < s->nkev; i++) {
            float k = 0.f;
            if (cudaEventElapsedTime(&k, s->kev[i], s->kev[i + 1]) == cudaSuccess) d->kern_ms[i] += k;
        }
        d->nkern = s->nkev > 0 ? s->nkev - 1 : 0;
        d->timed_frames++;
        s->timed = 0;
    }
    if (s->hdr_check) {
        /* every header byte but Lcod (12..15) must match the stream's */
        s->hdr_check = 0;
        const jxs_cfg_t* c = &d->cfg;
        if (memcmp(s->hdr_h, c->hdr, 12) != 0 || memcmp(s->hdr_h + 16, c->hdr + 16, c->hdr_len - 16) != 0)
            return JXS_E_DEC_CONFIG;
    }
    return *s->status_h;
}

extern "C" void jxs_gpu_dec_set_stream(jxs_gpu_dec_t* d, void* stream) {
    for (int i = 0; i < 8; i++) d->user_stream[i] = (cudaStream_t)stream;
}
extern "C" void jxs_gpu_dec_set_streams(jxs_gpu_dec_t* d, void* const* streams, int n) {
    for (int i = 0; i < 8; i++) d->user_stream[i] = n > 0 ? (cudaStream_t)streams[i % n] : (cudaStream_t)0;
}
extern "C" int jxs_gpu_dec_slots(jxs_gpu_dec_t* d) { return d->nslots; }

extern "C" void jxs_gpu_dec_set_timing(jxs_gpu_dec_t* d, int on) {
    std::lock_guard<std::mutex> g(d->mu);
    d->timing = on;
    for (int i = 0; i < DEC_STAGES; i++) d->stage_ms[i] = 0;
    for (int i = 0; i < JXS_KEV; i++) d->kern_ms[i] = 0;
    d->timed_frames = 0;
}

extern "C" int jxs_gpu_dec_read_kernel_timing(jxs_gpu_dec_t* d, double* ms, int n) {
    std::lock_guard<std::mutex> g(d->mu);
    for (int i = 0; i < n && i < JXS_KEV; i++) ms[i] = d->kern_ms[i];
    return d->nkern;
}

extern "C" uint64_t jxs_gpu_dec_read_timing(jxs_gpu_dec_t* d, double* ms, int n) {
    std::lock_guard<std::mutex> g(d->mu);
    for (int i = 0; i < n && i < DEC_STAGES; i++) ms[i] = d->stage_ms[i];
    return d->timed_frames;
}

extern "C" int jxs_gpu_dec_ready(jxs_gpu_dec_t* d, int slot) {
    cudaError_t r = cudaEventQuery(d->slot[slot].done);
    return r == cudaErrorNotReady ? 0 : 1;
}

extern "C" const jxs_cfg_t* jxs_gpu_enc_info(jxs_gpu_enc_t* e, const jxs_cfg_t** dev_cfg, uint32_t* cap_words) {
    if (!e) return NULL;
    if (dev_cfg) *dev_cfg = e->dcfg;
    if (cap_words) *cap_words = e->cap_words;
    return &e->cfg;
}
extern "C" uint64_t jxs_gpu_enc_serial(jxs_gpu_enc_t* e) { return e ? e->serial : 0; }

extern "C" const jxs_cfg_t* jxs_gpu_dec_info(jxs_gpu_dec_t* d, const jxs_cfg_t** dev_cfg, uint32_t* cap_bytes,
                                             uint32_t* cap_groups, uint32_t* cap_seg) {
    if (!d) return NULL;
    if (dev_cfg) *dev_cfg = d->dcfg;
    if (cap_bytes) *cap_bytes = d->cap_bytes;
    if (cap_groups) *cap_groups = d->cap_groups;
    if (cap_seg) *cap_seg = d->cap_seg;
    return &d->cfg;
}
extern "C" uint64_t jxs_gpu_dec_serial(jxs_gpu_dec_t* d) { return d ? d->serial : 0; }
