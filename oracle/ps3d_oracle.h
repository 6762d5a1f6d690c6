/*
 * ps3d_oracle.h -- C restatement of the reference pipeline's per-fragment
 * path (CallMeZhou/Puresoft3D), used as the oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load this library, only to check results
 * against (or as the timed CPU baseline); the product never routes through it.
 *
 * The entry points mirror the reference's PuresoftPipeline API
 * (src/puresoft3d/pipeline.h:26-69) one for one, in C, with the same status
 * codes as the product's C ABI (0 ok, -1 out of range, -2 invalid argument,
 * -3 out of memory).  Processor ids are the product's built-in processor
 * classes (include/ps3d.h, PS3D_VP_* / PS3D_IP_* / PS3D_FP_*).
 */
#ifndef PS3D_ORACLE_H
#define PS3D_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct ps3do ps3do;

ps3do* ps3do_create(int width, int height, int threads);
void ps3do_destroy(ps3do* p);
int ps3do_texture_create(ps3do* p, int width, int height, int scanline, int elemLen, const void* pixels, int wrap);
int ps3do_texture_read(ps3do* p, int idx, void* out, size_t bytes);
/* createTexture with extra layers (tex.cpp:3-25; 5 makes a cube map) and
   the per-layer access of getTexture (tex.cpp:27-37). */
int ps3do_texture_create_layers(ps3do* p, int width, int height, int scanline, int elemLen, const void* pixels,
                                int wrap, int extraLayers);
int ps3do_texture_write_layer(ps3do* p, int idx, int layer, const void* pixels, size_t bytes);
int ps3do_texture_read_layer(ps3do* p, int idx, int layer, void* out, size_t bytes);
int ps3do_processor_add(ps3do* p, int id);
int ps3do_programme_create(ps3do* p, int vid, int iid, int fid);
int ps3do_programme_use(ps3do* p, int idx);
int ps3do_vao_create(ps3do* p);
int ps3do_vbo_attach(ps3do* p, int vao, int slot, int unitBytes, int count, const void* data);
int ps3do_set_uniform(ps3do* p, int idx, const void* data, size_t len);
int ps3do_set_depth(ps3do* p, int idx);
int ps3do_set_fbo(ps3do* p, int idx, int tex);
int ps3do_set_viewport(ps3do* p, int width, int height);
int ps3do_enable(ps3do* p, int bits);
int ps3do_disable(ps3do* p, int bits);
int ps3do_clear_depth(ps3do* p, float v);
int ps3do_clear_colour(ps3do* p, uint32_t bgra);
int ps3do_draw(ps3do* p, int vao);
int ps3do_read_colour(ps3do* p, void* out);
/* postProcess with a built-in post-processor (include/ps3d.h PS3D_PP_*). */
int ps3do_post_process(ps3do* p, int id, const void* params, size_t bytes);
int ps3do_read_depth(ps3do* p, void* out);
/* Fragments that reached the depth test (the reference's per-pixel loop
   iterations, fragthrd.cpp:208) and fragments that passed it, since create. */
long long ps3do_fragments_tested(ps3do* p);
long long ps3do_fragments_passed(ps3do* p);
/* Colour error of the scene shaders (LIT1/2/3): with measurement on, every
   shaded fragment's pre-truncation FP32 colour is compared with an FP64
   re-shade of the same fragment (same varyings, texels and shadow map);
   max and mean |difference| per colour channel (in 8-bit units), the number
   of channels compared and how many differed by 1 or more. */
void ps3do_set_colour_error(ps3do* p, int on);
void ps3do_colour_error(ps3do* p, double* maxErr, double* meanErr, long long* channels, long long* over1);
/* Spans drawn since create, bucketed by floor(log2(length in pixels)). */
void ps3do_span_histogram(ps3do* p, long long* out32);

#ifdef __cplusplus
}
#endif
#endif
