/*
 * Image / bitstream buffer helpers and frame pools
 * (include/SvtJpegxsImageBufferTools.h), following the reference's
 * Source/Lib/Common/Codec/ImageBuffer.c:22-318.  Buffers are page-locked so
 * that the GPU copies them asynchronously at full link speed.
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "SvtJpegxsImageBufferTools.h"
#include "jxs_gpu.h"

PREFIX_API svt_jpeg_xs_image_buffer_t* svt_jpeg_xs_image_buffer_alloc(svt_jpeg_xs_image_config_t* cfg) {
    if (!cfg || cfg->components_num > MAX_COMPONENTS_NUM) return NULL;
    svt_jpeg_xs_image_buffer_t* b = (svt_jpeg_xs_image_buffer_t*)calloc(1, sizeof(*b));
    if (!b) return NULL;
    const uint32_t ps = cfg->bit_depth <= 8 ? 1 : 2;
    if (cfg->format == COLOUR_FORMAT_PACKED_YUV444_OR_RGB) {
        const uint64_t stride = (uint64_t)cfg->components[0].width * 3;
        const uint64_t bytes = stride * cfg->components[0].height * ps;
        if (stride > UINT32_MAX || bytes > UINT32_MAX) {
            free(b);
            return NULL;
        }
        b->stride[0] = (uint32_t)stride;
        b->alloc_size[0] = (uint32_t)bytes;
        b->data_yuv[0] = jxs_gpu_host_alloc(bytes);
        if (!b->data_yuv[0]) {
            svt_jpeg_xs_image_buffer_free(b);
            return NULL;
        }
    } else {
        for (uint32_t c = 0; c < cfg->components_num; c++) {
            const uint64_t bytes = (uint64_t)cfg->components[c].width * cfg->components[c].height * ps;
            if (bytes > UINT32_MAX) {
                svt_jpeg_xs_image_buffer_free(b);
                return NULL;
            }
            b->stride[c] = cfg->components[c].width;
            b->alloc_size[c] = (uint32_t)bytes;
            b->data_yuv[c] = jxs_gpu_host_alloc(bytes ? bytes : 1);
            if (!b->data_yuv[c]) {
                svt_jpeg_xs_image_buffer_free(b);
                return NULL;
            }
        }
    }
    return b;
}

PREFIX_API void svt_jpeg_xs_image_buffer_free(svt_jpeg_xs_image_buffer_t* b) {
    if (!b) return;
    for (int c = 0; c < MAX_COMPONENTS_NUM; c++) jxs_gpu_host_free(b->data_yuv[c]);
    free(b);
}

PREFIX_API svt_jpeg_xs_bitstream_buffer_t* svt_jpeg_xs_bitstream_alloc(uint32_t size) {
    svt_jpeg_xs_bitstream_buffer_t* b = (svt_jpeg_xs_bitstream_buffer_t*)calloc(1, sizeof(*b));
    if (!b) return NULL;
    b->allocation_size = size;
    b->buffer = (uint8_t*)jxs_gpu_host_alloc(size ? size : 1);
    if (!b->buffer) {
        free(b);
        return NULL;
    }
    return b;
}

PREFIX_API void svt_jpeg_xs_bitstream_free(svt_jpeg_xs_bitstream_buffer_t* b) {
    if (!b) return;
    jxs_gpu_host_free(b->buffer);
    free(b);
}

/* A pool is two stacks of pre-allocated buffers guarded by one mutex. */
struct svt_jpeg_xs_frame_pool {
    uint32_t count;
    int use_image, use_bitstream;
    svt_jpeg_xs_image_buffer_t** images;
    svt_jpeg_xs_bitstream_buffer_t** bitstreams;
    uint32_t free_images, free_bitstreams;
    svt_jpeg_xs_image_buffer_t** img_stack;
    svt_jpeg_xs_bitstream_buffer_t** bs_stack;
    pthread_mutex_t mu;
    pthread_cond_t cv;
};

PREFIX_API void svt_jpeg_xs_frame_pool_free(svt_jpeg_xs_frame_pool_t* p) {
    if (!p) return;
    for (uint32_t i = 0; i < p->count; i++) {
        if (p->images) svt_jpeg_xs_image_buffer_free(p->images[i]);
        if (p->bitstreams) svt_jpeg_xs_bitstream_free(p->bitstreams[i]);
    }
    free(p->images);
    free(p->bitstreams);
    free(p->img_stack);
    free(p->bs_stack);
    pthread_mutex_destroy(&p->mu);
    pthread_cond_destroy(&p->cv);
    free(p);
}

PREFIX_API svt_jpeg_xs_frame_pool_t* svt_jpeg_xs_frame_pool_alloc(const svt_jpeg_xs_image_config_t* cfg, uint32_t bitstream_size,
                                                                  uint32_t count) {
    if (count == 0 || (!cfg && bitstream_size == 0)) return NULL;
    if (cfg && cfg->components_num > MAX_COMPONENTS_NUM) return NULL;
    svt_jpeg_xs_frame_pool_t* p = (svt_jpeg_xs_frame_pool_t*)calloc(1, sizeof(*p));
    if (!p) return NULL;
    pthread_mutex_init(&p->mu, NULL);
    pthread_cond_init(&p->cv, NULL);
    p->count = count;
    p->use_image = cfg != NULL;
    p->use_bitstream = bitstream_size != 0;
    if (p->use_image) {
        p->images = (svt_jpeg_xs_image_buffer_t**)calloc(count, sizeof(void*));
        p->img_stack = (svt_jpeg_xs_image_buffer_t**)calloc(count, sizeof(void*));
        if (!p->images || !p->img_stack) goto fail;
        svt_jpeg_xs_image_config_t c = *cfg;
        for (uint32_t i = 0; i < count; i++) {
            p->images[i] = svt_jpeg_xs_image_buffer_alloc(&c);
            if (!p->images[i]) goto fail;
            p->images[i]->release_ctx_ptr = p->images[i];
            p->img_stack[i] = p->images[i];
        }
        p->free_images = count;
    }
    if (p->use_bitstream) {
        p->bitstreams = (svt_jpeg_xs_bitstream_buffer_t**)calloc(count, sizeof(void*));
        p->bs_stack = (svt_jpeg_xs_bitstream_buffer_t**)calloc(count, sizeof(void*));
        if (!p->bitstreams || !p->bs_stack) goto fail;
        for (uint32_t i = 0; i < count; i++) {
            p->bitstreams[i] = svt_jpeg_xs_bitstream_alloc(bitstream_size);
            if (!p->bitstreams[i]) goto fail;
            p->bitstreams[i]->release_ctx_ptr = p->bitstreams[i];
            p->bs_stack[i] = p->bitstreams[i];
        }
        p->free_bitstreams = count;
    }
    return p;
fail:
    svt_jpeg_xs_frame_pool_free(p);
    return NULL;
}

PREFIX_API SvtJxsErrorType_t svt_jpeg_xs_frame_pool_get(svt_jpeg_xs_frame_pool_t* p, svt_jpeg_xs_frame_t* f, uint8_t blocking) {
    if (!p || !f) return SvtJxsErrorBadParameter;
    pthread_mutex_lock(&p->mu);
    for (;;) {
        const int ok_img = !p->use_image || p->free_images > 0;
        const int ok_bs = !p->use_bitstream || p->free_bitstreams > 0;
        if (ok_img && ok_bs) break;
        if (!blocking) {
            pthread_mutex_unlock(&p->mu);
            return SvtJxsErrorNoErrorEmptyQueue;
        }
        pthread_cond_wait(&p->cv, &p->mu);
    }
    if (p->use_image) {
        svt_jpeg_xs_image_buffer_t* b = p->img_stack[--p->free_images];
        f->image = *b;
        f->image.release_ctx_ptr = b;
    }
    if (p->use_bitstream) {
        svt_jpeg_xs_bitstream_buffer_t* b = p->bs_stack[--p->free_bitstreams];
        f->bitstream = *b;
        f->bitstream.release_ctx_ptr = b;
    }
    pthread_mutex_unlock(&p->mu);
    return SvtJxsErrorNone;
}

PREFIX_API void svt_jpeg_xs_frame_pool_release(svt_jpeg_xs_frame_pool_t* p, svt_jpeg_xs_frame_t* f) {
    if (!p || !f) return;
    pthread_mutex_lock(&p->mu);
    if (p->use_image && f->image.release_ctx_ptr && p->free_images < p->count)
        p->img_stack[p->free_images++] = (svt_jpeg_xs_image_buffer_t*)f->image.release_ctx_ptr;
    if (p->use_bitstream && f->bitstream.release_ctx_ptr && p->free_bitstreams < p->count)
        p->bs_stack[p->free_bitstreams++] = (svt_jpeg_xs_bitstream_buffer_t*)f->bitstream.release_ctx_ptr;
    pthread_cond_broadcast(&p->cv);
    pthread_mutex_unlock(&p->mu);
}
