/*
 * Stand-in for the few Media Transport Library (IMTL) pipeline declarations
 * that the SVT-JPEG-XS IMTL plugin (imtl-plugin/src/st22_svt_jpeg_xs_plugin.c)
 * uses, so that the plugin's own source compiles against this library and
 * runs in the tests, with tests/plugin_mtl_host.c playing the library's side
 * of the plugin interface.  Test infrastructure: only the names and members
 * the plugin touches, with values of this file's choosing; this is not IMTL.
 */
#ifndef JXS_TEST_MTL_STUB_H
#define JXS_TEST_MTL_STUB_H

#include <pthread.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

typedef void* mtl_handle;
typedef void* st_plugin_priv;
typedef void* st22p_encode_session;
typedef void* st22p_decode_session;
typedef void* st22_encode_priv;
typedef void* st22_decode_priv;
typedef void* st22_encoder_dev_handle;
typedef void* st22_decoder_dev_handle;

enum st_frame_fmt {
    ST_FRAME_FMT_YUV422PLANAR10LE = 0,
    ST_FRAME_FMT_YUV422PLANAR8 = 1,
    ST_FRAME_FMT_JPEGXS_CODESTREAM = 2,
};
#define ST_FMT_CAP_YUV422PLANAR10LE (1ull << ST_FRAME_FMT_YUV422PLANAR10LE)
#define ST_FMT_CAP_YUV422PLANAR8 (1ull << ST_FRAME_FMT_YUV422PLANAR8)
#define ST_FMT_CAP_JPEGXS_CODESTREAM (1ull << ST_FRAME_FMT_JPEGXS_CODESTREAM)

enum st_plugin_device { ST_PLUGIN_DEVICE_CPU = 0 };
enum st22_quality_mode { ST22_QUALITY_MODE_SPEED = 0, ST22_QUALITY_MODE_QUALITY = 1 };

#define ST_PLUGIN_VERSION_V1 1
#define ST_PLUGIN_VERSION_V1_MAGIC 0x5650314cu

struct st_plugin_meta {
    int version;
    uint32_t magic;
};

#define ST_MAX_PLANES 4
struct st_frame {
    void* addr[ST_MAX_PLANES];
    size_t linesize[ST_MAX_PLANES];
    enum st_frame_fmt fmt;
    uint32_t width, height;
    size_t buffer_size;
    size_t data_size;
};

struct st22_encode_frame_meta {
    struct st_frame* src;
    struct st_frame* dst;
};
struct st22_decode_frame_meta {
    struct st_frame* src;
    struct st_frame* dst;
};

struct st22_encoder_create_req {
    uint32_t width, height;
    enum st_frame_fmt input_fmt, output_fmt;
    enum st22_quality_mode quality;
    int codec_thread_cnt;
    size_t codestream_size;
    size_t max_codestream_size;
};
struct st22_decoder_create_req {
    uint32_t width, height;
    enum st_frame_fmt input_fmt, output_fmt;
    int codec_thread_cnt;
    size_t max_codestream_size;
};

struct st22_encoder_dev {
    const char* name;
    void* priv;
    enum st_plugin_device target_device;
    uint64_t input_fmt_caps, output_fmt_caps;
    st22_encode_priv (*create_session)(void* priv, st22p_encode_session session_p, struct st22_encoder_create_req* req);
    int (*free_session)(void* priv, st22_encode_priv session);
    int (*notify_frame_available)(void* priv);
};
struct st22_decoder_dev {
    const char* name;
    void* priv;
    enum st_plugin_device target_device;
    uint64_t input_fmt_caps, output_fmt_caps;
    st22_decode_priv (*create_session)(void* priv, st22p_decode_session session_p, struct st22_decoder_create_req* req);
    int (*free_session)(void* priv, st22_decode_priv session);
    int (*notify_frame_available)(void* priv);
};

st22_encoder_dev_handle st22_encoder_register(mtl_handle mt, struct st22_encoder_dev* dev);
int st22_encoder_unregister(st22_encoder_dev_handle handle);
st22_decoder_dev_handle st22_decoder_register(mtl_handle mt, struct st22_decoder_dev* dev);
int st22_decoder_unregister(st22_decoder_dev_handle handle);
struct st22_encode_frame_meta* st22_encoder_get_frame(st22p_encode_session session);
int st22_encoder_put_frame(st22p_encode_session session, struct st22_encode_frame_meta* frame, int result);
struct st22_decode_frame_meta* st22_decoder_get_frame(st22p_decode_session session);
int st22_decoder_put_frame(st22p_decode_session session, struct st22_decode_frame_meta* frame, int result);
uint8_t st_frame_fmt_planes(enum st_frame_fmt fmt);
size_t st_frame_plane_size(struct st_frame* frame, uint8_t plane);
const char* st_frame_fmt_name(enum st_frame_fmt fmt);

#endif
