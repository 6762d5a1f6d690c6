/*
 * ps3d.h -- C ABI of puresoft3d_gb300, a GB300 (sm_103a) implementation of
 * the per-fragment path of Puresoft3D (CallMeZhou/Puresoft3D): vertex
 * processing, triangle set-up, scanline rasterisation, perspective-correct
 * interpolation, depth test, fragment shading, framebuffer write and 2D
 * texture sampling.
 *
 * Every entry point replaces one method of the reference's PuresoftPipeline
 * (src/puresoft3d/pipeline.h:26-69) and is cited beside it.  Plain C types
 * only; a pipeline is an opaque handle.  All calls on one pipeline must come
 * from one host thread (the reference has the same rule: one API thread,
 * pipeline.cpp).  Rendering is asynchronous on the pipeline's CUDA stream:
 * ps3d_draw records work, ps3d_flush launches it, and ps3d_finish or any
 * read-back waits for it.
 *
 * Return values: >= 0 success (an index where the reference returns one);
 * negative status codes mirror the reference's C++ exceptions:
 *   PS3D_ERR_RANGE   std::out_of_range     (bad index)
 *   PS3D_ERR_INVALID std::invalid_argument (bad format / combination)
 *   PS3D_ERR_NOMEM   std::bad_alloc        (host or device allocation)
 * and two for the device:
 *   PS3D_ERR_DEVICE  a CUDA call failed (the message: ps3d_last_error)
 *   PS3D_ERR_TIMEOUT a bounded device wait gave up (batch/serve paths)
 * ps3d_draw on a pipeline with no usable programme, or with a bad VAO index,
 * does nothing and returns PS3D_OK, as drawVAO does (drawvao.cpp:12-15).
 */
#ifndef PS3D_H
#define PS3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PS3D_OK 0
#define PS3D_ERR_RANGE (-1)
#define PS3D_ERR_INVALID (-2)
#define PS3D_ERR_NOMEM (-3)
#define PS3D_ERR_DEVICE (-4)
#define PS3D_ERR_TIMEOUT (-5)

/* behaviour bits (reference pipeline.h:16-19) */
#define PS3D_BEHAVIOR_UPDATE_DEPTH 0x1
#define PS3D_BEHAVIOR_TEST_DEPTH 0x2
#define PS3D_BEHAVIOR_FACE_CULLING 0x4
#define PS3D_BEHAVIOR_ALPHABLEND 0x8

/* Built-in processor classes.  The reference's processors are C++ classes
 * that run on the CPU (proc.h:26-71); here each class is a device functor
 * selected by id.  Low nibble: 1 vertex, 2 interpolation, 3 fragment.
 *   DEF01  VertexProcesserDEF01 / InterpolationProcessorDEF01 /
 *          FragmentProcessorDEF01 (tex1light1.cpp): point light, nearest
 *          texture; its rcpps / rsqrtss normalisations are reproduced bit
 *          for bit (tables of the instructions as the reference's x86 host
 *          computes them), as in every reference processor here.
 *   DEF05  the depth-only shadow programme (shadow.cpp), positions x0.9.
 *   SHADOW DEF05's vertex stage without the x0.9 scale.
 *   LIT1   fragment stage over DEF01 varyings: bilinear REPEAT albedo,
 *          directional Lambert + Blinn-Phong (shininess 32).
 *   LIT3   LIT1 with a trilinear mip chain.
 *   LIT2   vertex/interpolation/fragment stages with tangent, light-space
 *          position, trilinear albedo, tangent-space normal map and 3x3 PCF.
 */
#define PS3D_VP_DEF01 0x0101
#define PS3D_IP_DEF01 0x0102
#define PS3D_FP_DEF01 0x0103
/* The reference's vertex-colour processors (colr1light1.cpp): VBO slots 0
 * position, 1 normal, 2 colour (four floats, BGRA order, 0..255); uniforms
 * 3-5 and 7-8 as DEF01; DEF01's lighting on the interpolated colour. */
#define PS3D_VP_DEF02 0x0201
#define PS3D_IP_DEF02 0x0202
#define PS3D_FP_DEF02 0x0203
/* The reference's bump-mapped processors (tex1bump1light1.cpp): VBO slots 0
 * position, 1 tangent, 2 binormal, 3 normal, 4 uv; uniform 9 the diffuse
 * texture, 10 the bump texture (tangent-space normal in r, g, b). */
#define PS3D_VP_DEF03 0x0301
#define PS3D_IP_DEF03 0x0302
#define PS3D_FP_DEF03 0x0303
/* The reference's skybox processors (skybox.cpp): VBO slot 0 holds clip-space
 * positions, passed through; uniform 1 the view matrix, uniform 2 the index
 * of a cube map (ps3d_texture_create_layers with 5 extra layers, BGRA8).
 * The fragment stage reads the face texel the view direction points at
 * (samplrcube.cpp:29-127) and writes it (blended under ALPHABLEND). */
#define PS3D_VP_DEF04 0x0401
#define PS3D_IP_DEF04 0x0402
#define PS3D_FP_DEF04 0x0403
/* The reference demo's planet processors (src/test/testproc.cpp): VBO slots
 * as DEF03; uniforms 3-5 as DEF01, 16 the shadow projection (world -> the
 * shadow map's [0, 1] texture space, z compared with the stored depth), 7
 * light, 8 camera; textures by index at 9 diffuse, 10 bump, 15 shadow map
 * (FP32) and, for Earth, 11 specular (red scales the highlight) and 12
 * night (added where lambert < 0.2).  The shadow factor is the reference's
 * 4-tap Poisson projective lookup (samplrproj.cpp:20-38). */
#define PS3D_VP_PLANET 0x0701
#define PS3D_IP_PLANET 0x0702
#define PS3D_FP_EARTH 0x0703
#define PS3D_FP_SATELLITE 0x0713
/* The reference demo's cloud processors (src/test/testproc.cpp).  Cloud:
 * VBO 0 position, 3 normal, 4 uv; uniforms as the planet's plus textures 9
 * (the cloud, alpha = its red) and 15 (shadow map); writes white times
 * 2 * lambert * shadow through write4, so it blends under ALPHABLEND.
 * CloudShadow: positions x0.95 through (3 * 4), uv from VBO 4, texture 9;
 * writes no colour and discards where the texel's red is below 150 (an
 * alpha-tested depth-only pass). */
#define PS3D_VP_CLOUD 0x0801
#define PS3D_IP_CLOUD 0x0802
#define PS3D_FP_CLOUD 0x0803
#define PS3D_VP_CLOUDSHADOW 0x0901
#define PS3D_IP_CLOUDSHADOW 0x0902
#define PS3D_FP_CLOUDSHADOW 0x0903
/* The scene viewer demo's processors (src/test2/testproc.cpp), with its
 * uniform slots: 0 model, 1 model rotation, 5 PVM, 6 shadow projection;
 * 20 light position, 21 light direction, 22 camera, 23 shadow map (texture
 * index); 30 ambient, 31 diffuse colour, 32 specular colour, 33 specular
 * exponent (one float); 40 diffuse texture (index).  VBO 0 position, 3
 * normal, 4 uv.  Lighting is a 25-degree spotlight (cos^150 fall-off
 * outside the cone) with the 4-tap projective shadow lookup.  PositionOnly +
 * Null + SingleColourNoLighting draws the flat diffuse colour; Shadow (x0.9)
 * + Null + FP Null is the depth-only shadow pass. */
#define PS3D_VP_POSITIONONLY 0x0A01
#define PS3D_IP_NULL 0x0A02
#define PS3D_FP_SINGLECOLOURNOLIGHTING 0x0A03
#define PS3D_VP_SINGLECOLOUR 0x0B01
#define PS3D_IP_SINGLECOLOUR 0x0B02
#define PS3D_FP_SINGLECOLOUR 0x0B03
#define PS3D_VP_DIFFUSEONLY 0x0C01
#define PS3D_IP_DIFFUSEONLY 0x0C02
#define PS3D_FP_DIFFUSEONLY 0x0C03
#define PS3D_VP_VIEWERSHADOW 0x0D01
#define PS3D_FP_NULL 0x0D03
#define PS3D_VP_DEF05 0x0501
#define PS3D_IP_DEF05 0x0502
#define PS3D_FP_DEF05 0x0503
#define PS3D_VP_SHADOW 0x0601
#define PS3D_FP_LIT1 0x1103
/* LIT1 with an alpha test (the albedo's alpha below 128 discards the
 * fragment: no colour, no depth write, fragthrd.cpp:233-237) and the
 * albedo's alpha as the fragment's alpha (so ALPHABLEND blends by it). */
#define PS3D_FP_LIT1A 0x1403
#define PS3D_FP_LIT3 0x1303
#define PS3D_VP_LIT2 0x1201
#define PS3D_IP_LIT2 0x1202
#define PS3D_FP_LIT2 0x1203

/* limits (reference config.h:3-9) */
#define PS3D_MAX_VBOS 16
#define PS3D_MAX_UNIFORMS 1024
#define PS3D_MAX_FBOS 16

typedef struct ps3d_pipeline ps3d_pipeline;
typedef struct ps3d_cmdbuf ps3d_cmdbuf;

/* Counters since creation (ps3d_stats). */
typedef struct {
    uint64_t draws;           /* ps3d_draw calls that drew */
    uint64_t batches;         /* device passes executed */
    uint64_t kernel_launches; /* kernels this library launched */
    uint64_t triangles;       /* triangles sent through set-up */
    uint64_t fragments;       /* fragments that reached the depth test (when counting is on) */
    uint64_t fragments_passed;/* fragments that passed it (when counting is on) */
    uint64_t replays;         /* passes re-run after a bin-list capacity miss */
    uint64_t bin_pairs;       /* (bin, triangle) pairs written by the binning passes */
    uint64_t shaded;          /* pixels shaded once: covered at the end of a colour pass (when counting is on) */
    uint64_t upload_bytes;    /* host -> device bytes of draw descriptors and uniforms uploaded for passes */
} ps3d_stats_t;

/* PuresoftPipeline::PuresoftPipeline(canvas, w, h, rndr) (pipeline.cpp:24-61).
 * Creates the default FP32 depth buffer (scanline rounded to 4 floats,
 * pipeline.cpp:31) and a BGRA8 top-down colour buffer in device memory in
 * place of the renderer's back buffer.  `stream` is a cudaStream_t, or NULL
 * for a stream the pipeline creates and owns. */
int ps3d_pipeline_create(int width, int height, void* stream, ps3d_pipeline** out);
/* PuresoftPipeline::~PuresoftPipeline (pipeline.cpp:63-116). */
int ps3d_pipeline_destroy(ps3d_pipeline* p);
/* Message of the last failing call on this thread. */
const char* ps3d_last_error(void);

/* PuresoftPipeline::createTexture (tex.cpp:3-25): copies `pixels` (host
 * memory, scanline*height bytes; NULL leaves it zeroed) into a
 * pipeline-owned device texture.  elemLen must be 1 or 4 (fbo.cpp:21-24);
 * wrap 0 = CLAMP, 1 = WRAP. */
int ps3d_texture_create(ps3d_pipeline* p, int width, int height, int scanline, int elemLen, const void* pixels,
                        int wrap);
/* Same, from device memory (cudaMemcpyDeviceToDevice). */
int ps3d_texture_create_device(ps3d_pipeline* p, int width, int height, int scanline, int elemLen,
                               const void* devPixels, int wrap);
/* PuresoftPipeline::createTexture(image, extraLayers, mode) (tex.cpp:3-25,
 * fbo.cpp:59-73): a texture with 0..5 extra layers of the same size, stored
 * after the first; `pixels` fills layer 0 and the extra layers start zeroed.
 * Five extra layers make a cube map, faces in the order +x, -x, +y, -y, +z,
 * -z (PuresoftFBO::LAYER, fbo.h:19).  More than 5 is PS3D_ERR_RANGE (the
 * reference throws out_of_range above 6, and 6 overruns its layer array). */
int ps3d_texture_create_layers(ps3d_pipeline* p, int width, int height, int scanline, int elemLen,
                               const void* pixels, int wrap, int extraLayers);
/* PuresoftPipeline::getTexture(idx, image, layer) (tex.cpp:27-37) hands the
 * caller the layer's buffer to fill or read; these copy min(bytes,
 * scanline*height) bytes into or out of layer `layer` after pending work
 * has finished. */
int ps3d_texture_write_layer(ps3d_pipeline* p, int idx, int layer, const void* pixels, size_t bytes);
int ps3d_texture_read_layer(ps3d_pipeline* p, int idx, int layer, void* out, size_t bytes);
/* PuresoftPipeline::destroyTexture (tex.cpp:39-51). */
int ps3d_texture_destroy(ps3d_pipeline* p, int idx);
/* PuresoftPipeline::getTexture (tex.cpp:27-37): waits for pending work, then
 * copies min(bytes, scanline*height) bytes of the texture to host memory. */
int ps3d_texture_read(ps3d_pipeline* p, int idx, void* out, size_t bytes);
/* Device address of a texture's first byte (rows bottom-up). */
int ps3d_texture_device_ptr(ps3d_pipeline* p, int idx, void** out);

/* PuresoftPipeline::addProcessor (prog.cpp:3-20) with a built-in class id. */
int ps3d_processor_add(ps3d_pipeline* p, int processorId);
/* PuresoftPipeline::destroyProcessor (prog.cpp:22-41). */
int ps3d_processor_destroy(ps3d_pipeline* p, int idx);
/* PuresoftPipeline::createProgramme (prog.cpp:43-108).  The reference lets
 * any three processors combine and reinterprets user-data bytes; here the
 * interpolation stage must carry the varyings its fragment stage reads
 * (DEF01 varyings for DEF01/LIT1/LIT3, LIT2 varyings for LIT2), else
 * PS3D_ERR_INVALID. */
int ps3d_programme_create(ps3d_pipeline* p, int vid, int iid, int fid);
/* PuresoftPipeline::destroyProgramme (prog.cpp:110-119). */
int ps3d_programme_destroy(ps3d_pipeline* p, int idx);
/* PuresoftPipeline::useProgramme (prog.cpp:121-131). */
int ps3d_programme_use(ps3d_pipeline* p, int idx);

/* PuresoftPipeline::createVAO (pipeline.cpp:118-136). */
int ps3d_vao_create(ps3d_pipeline* p);
/* PuresoftPipeline::destroyVAO (pipeline.cpp:183-205): frees attached VBOs. */
int ps3d_vao_destroy(ps3d_pipeline* p, int vao);
/* new PuresoftVBO(unitBytes, count) + updateContent(data) + attachVBO(vao,
 * slot, vbo) (vbo.cpp:16-31, pipeline.cpp:138-151): uploads `count` elements
 * of `unitBytes` from host memory into VBO slot `slot` of `vao`; replaces and
 * frees a VBO already there. */
int ps3d_vbo_attach(ps3d_pipeline* p, int vao, int slot, int unitBytes, int count, const void* data);
/* Same, from device memory. */
int ps3d_vbo_attach_device(ps3d_pipeline* p, int vao, int slot, int unitBytes, int count, const void* devData);
/* PuresoftPipeline::getVBO(vao, idx)->updateContent(src) (pipeline.cpp:168-181,
 * vbo.cpp:28-31): overwrites the VBO's unitBytes * count bytes with `data`
 * (host memory) in place.  Draws recorded before the call are rendered with
 * the old contents first (the reference's drawVAO is synchronous); draws
 * recorded after it, and command buffers replayed after it, read the new
 * contents.  PS3D_ERR_RANGE for a bad VAO or slot or an empty slot (where
 * the reference would dereference a null VBO), PS3D_ERR_INVALID while a
 * command buffer is being recorded. */
int ps3d_vbo_update(ps3d_pipeline* p, int vao, int slot, const void* data);
/* PuresoftPipeline::detachVBO + delete (pipeline.cpp:153-166). */
int ps3d_vbo_detach(ps3d_pipeline* p, int vao, int slot);

/* PuresoftPipeline::setUniform (pipeline.cpp:277-312): copies len bytes into
 * slot idx; data == NULL frees the slot. */
int ps3d_set_uniform(ps3d_pipeline* p, int idx, const void* data, size_t len);
/* PuresoftPipeline::setDepth (pipeline.cpp:218-239): -1 = default buffer;
 * a texture must have elemLen 4 and a scanline multiple of 4 (else
 * PS3D_ERR_INVALID).  The depth target must be CLAMP-addressed. */
int ps3d_set_depth(ps3d_pipeline* p, int idx);
/* PuresoftPipeline::setFBO(idx, fbo) (pipeline.cpp:260-275) with a texture
 * of this pipeline as the FBO (borrowed, not copied; -1 = none, and slot 0
 * back to the display).  The built-in fragment processors write FBO slot 0
 * (FBOBridge, fragthrd.cpp:55-95), so after ps3d_set_fbo(p, 0, tex) the
 * draws recorded next colour the texture (BGRA8, its rows bottom-up as the
 * reference's textures are) and ps3d_post_process works on it (post.cpp:14);
 * ps3d_clear_colour still clears the display, as clearColour does
 * (pipeline.cpp:340-343), and the read-backs read the display.  The
 * texture must have 4-byte elements (PS3D_ERR_INVALID) and cover a
 * colour-writing draw's viewport (else ps3d_draw returns PS3D_ERR_INVALID,
 * where the reference would drop the writes outside it).  A texture
 * destroyed while bound leaves its slots.  PS3D_ERR_RANGE for idx outside
 * [0, 16) or a bad texture. */
int ps3d_set_fbo(ps3d_pipeline* p, int idx, int texture);
/* PuresoftPipeline::setViewport (pipeline.cpp:207-216): rasteriser size. */
int ps3d_set_viewport(ps3d_pipeline* p, int width, int height);
/* Extension (no reference counterpart): a viewport of width x height -- the
 * rasteriser size, exactly as setViewport -- whose pixel (0, 0) is written at
 * pixel (x, y) of the colour and depth targets.  Draws into one target with
 * different rectangles run in one device pass: many small views rendered into
 * tiles of an atlas are one batched launch. */
int ps3d_set_viewport_rect(ps3d_pipeline* p, int x, int y, int width, int height);
/* PuresoftPipeline::enable / disable (pipeline.cpp:324-332). */
int ps3d_enable(ps3d_pipeline* p, int bits);
int ps3d_disable(ps3d_pipeline* p, int bits);
/* PuresoftPipeline::clearDepth (pipeline.cpp:334-338): every element of the
 * current depth target. */
int ps3d_clear_depth(ps3d_pipeline* p, float furthest);
/* PuresoftPipeline::clearColour (pipeline.cpp:340-343): every pixel of the
 * colour buffer (the reference skips the last memory row, fbo.cpp:336). */
int ps3d_clear_colour(ps3d_pipeline* p, uint32_t bgra);
/* PuresoftPipeline::drawVAO(vao, false) (drawvao.cpp:3-133): records the draw
 * with a snapshot of the programme, uniforms, behaviour, viewport and
 * targets.  Work is launched by ps3d_flush / ps3d_finish / a read-back.
 * PS3D_ERR_RANGE for a depth target wider than 65535 or taller than 32767
 * pixels. */
int ps3d_draw(ps3d_pipeline* p, int vao);
/* Launch recorded work on the stream without waiting. */
int ps3d_flush(ps3d_pipeline* p);
/* Launch recorded work and wait for it (drawVAO's synchronous return,
 * drawvao.cpp:121-132). */
int ps3d_finish(ps3d_pipeline* p);

/* Schedule knob (no reference counterpart): the width in columns (8, 16 or
 * 32) of the 32-row bins the passes launched from now on are cut into.  It
 * changes time only, never results; puresoft3d_gb300.autotune picks it per
 * workload.  Default 32 (or PS3D_BIN_W). */
int ps3d_set_bin_width(ps3d_pipeline* p, int columns);
int ps3d_get_bin_width(ps3d_pipeline* p, int* columns);
/* Raster variant: on (the default), a span whose every pixel would fail the
 * depth test against its row's current depths is dropped before its depths
 * are computed, in bins with more than 128 triangles (a conservative test,
 * so results are unchanged); off leaves the test out of the kernel.  The
 * autotuner times both. */
int ps3d_set_span_culling(ps3d_pipeline* p, int on);
/* Row split of the raster: 1 (the default: one block per bin), 2, 4 or 8.
 * With n > 1, a bin of t triangles is cut into min(n, the largest power of
 * two <= t / 128) row slices, and a persistent grid takes the slices of the
 * most-cut bins first, then the other bins, so that a few crowded bins do
 * not hold up the launch.  Time only, never results; the autotuner times 1
 * and 4. */
int ps3d_set_row_split(ps3d_pipeline* p, int blocksPerBin);
/* Second schedule knob: the raster kernel variant.  0 lets each thread use
 * the registers it wants (fewer resident blocks); 8 caps registers so that
 * 8 blocks fit per SM where shared memory allows (more warps to hide
 * latency).  Time only, never results. */
int ps3d_set_raster_occupancy(ps3d_pipeline* p, int blocksPerSM);
/* Raster shape: 0 (the default) four warps share each bin and meet at
 * block barriers; 1 each warp owns a bin of 8 or 16 columns and works
 * through it alone (no block barrier; bins of 32 columns and passes that
 * blend or discard keep the shared shape).  Time only, never results. */
int ps3d_set_raster_warp_bins(ps3d_pipeline* p, int on);
/* Span items: 1 bins each row span of a triangle up to 32 rows tall as its
 * own item, set up (row result, span set-up and the sequential steps to its
 * first pixel in the bin) in the set-up kernel, where all triangles run in
 * parallel, instead of in the raster, where a crowded bin's spans are set up
 * by one block; 0 (the default) bins whole triangles and sets their spans up
 * in the raster.  Passes that blend or discard bin whole triangles either
 * way.  Time only, never results. */
int ps3d_set_span_items(ps3d_pipeline* p, int on);
/* Deferred varyings: 1 the set-up kernel computes only positions, and the
 * shade kernel runs the vertex processor on the three vertices of each
 * pixel's winning triangle (less set-up work and traffic, more per shaded
 * pixel: pays where triangles outnumber shaded pixels); 0 (the default)
 * the set-up stores every binned triangle's vertex varyings.  Passes that
 * blend or discard keep stored varyings.  Time only, never results. */
int ps3d_set_lazy_varyings(ps3d_pipeline* p, int on);

/* ps3d_finish for callers that must not allocate device memory; it has no
 * counterpart in the reference, whose CPU pipeline allocates no device memory
 * at all.  Who needs it: a real-time render thread that may not block in
 * cudaMalloc/cudaFree (both can synchronise the whole device), a process whose
 * device memory is fully committed up front, a service that must not grow
 * after admission control has accounted for its memory.
 *
 * The recorded passes run the same kernels with the same results as
 * ps3d_finish, but take all their scratch from one fixed 16 MiB device array
 * (a file-scope __device__ array, carved afresh per pass); the call makes no
 * cudaMalloc, cudaFree or other allocating call.  Limits:
 *   - a pass needs its triangle records, varyings, descriptors and (when it
 *     writes colour) 8 bytes per target pixel to fit in 16 MiB with room for
 *     at least 4096 bin pairs, and has at most 1024 draws.  Otherwise the call
 *     returns PS3D_ERR_RANGE before anything runs and the commands stay
 *     recorded (ps3d_finish renders them);
 *   - if a pass finds more bin pairs than fit, it and the passes after it do
 *     nothing and the call returns PS3D_ERR_NOMEM; ps3d_finish then completes
 *     the frame (and may allocate).
 * First call: the array's device address is looked up once per device
 * (cudaGetSymbolAddress, with that device current); make one call with
 * nothing recorded, before any stream capture starts, to do this set-up.
 * Overlap: every pipeline of the process shares the array, so two calls
 * whose work overlapped on the device would race; calls are serialised by a
 * process-wide lock and each returns only after its work has completed (on
 * an error too: work already queued is waited for, and the frame's
 * commands are then dropped, except after PS3D_ERR_RANGE / PS3D_ERR_NOMEM
 * as above).  The device current at the call must be the one the pipeline
 * was created on (else PS3D_ERR_DEVICE).
 * Flushed work (ps3d_flush) must be finished with ps3d_finish first. */
int ps3d_finish_noalloc(ps3d_pipeline* p);

/* Read-back of the colour buffer: width*height*4 bytes, BGRA8, top-down
 * (memory row = H-1-y, the display FBO layout, pipeline.cpp:48). */
int ps3d_read_colour(ps3d_pipeline* p, void* out);
/* Read-back of the default depth buffer: scanline*height bytes. */
int ps3d_read_depth(ps3d_pipeline* p, void* out);
/* Records a copy of the colour buffer (width*height*4 bytes, BGRA8 top-down)
 * to device memory at devDst, ordered after the draws recorded before it
 * (like a read-back, but asynchronous and on the device). */
int ps3d_read_colour_device(ps3d_pipeline* p, void* devDst);
/* Records a copy of the colour rectangle (x, y, width, height; pixels from
 * the bottom-left corner, as ps3d_set_viewport_rect) to dst -- device or
 * host memory (pinned for an asynchronous copy) -- rows top-down, dstPitch
 * bytes apart, ordered after the draws recorded before it.  With
 * ps3d_set_viewport_rect this reads out one view of a batched pass. */
int ps3d_copy_colour_rect(ps3d_pipeline* p, int x, int y, int width, int height, void* dst, size_t dstPitch);

/* PuresoftPipeline::postProcess(PuresoftPostProcessor*) (post.cpp:3-19,
 * proc.h:88-94): records a post-processor pass over the whole colour buffer
 * (and the depth buffer current now), ordered after everything recorded
 * before it.  Built-in post-processors only:
 *   PS3D_PP_ADD8  wrapping per-byte add of 4 bytes (B, G, R, A addends) to
 *                 every pixel -- the reference demo's post-processor
 *                 (test2/testpost.cpp:9-43, paddb of eight bytes of 50);
 *                 params NULL = {50, 50, 50, 50}.
 *   PS3D_PP_FOG   linear depth fog, params {uint32 fog BGRA, float near,
 *                 float far}: t = clamp((depth - near) / (far - near), 0, 1),
 *                 B, G, R = (unsigned char)(c + (fog - c) * t), alpha kept;
 *                 needs a depth buffer at least the colour buffer's size.
 * Runs exactly once per recorded call, also when a bin-list overflow makes
 * the frame replay. */
#define PS3D_PP_ADD8 0x7001
#define PS3D_PP_FOG 0x7002
int ps3d_post_process(ps3d_pipeline* p, int postProcessorId, const void* params, size_t bytes);
/* 1 when all launched work of the pipeline has completed, 0 while some is
 * still running (cudaStreamQuery; no wait, no verification: ps3d_finish
 * verifies and, after a bin-list overflow, re-runs -- copies included). */
int ps3d_query(ps3d_pipeline* p);
/* Device address of the colour buffer. */
int ps3d_colour_device_ptr(ps3d_pipeline* p, void** out);
/* The pipeline's CUDA stream (cudaStream_t). */
int ps3d_get_stream(ps3d_pipeline* p, void** out);

/* Count fragments reaching / passing the depth test (off by default: it
 * adds one atomic per warp-span). */
int ps3d_set_fragment_counting(ps3d_pipeline* p, int on);
int ps3d_stats(ps3d_pipeline* p, ps3d_stats_t* out);
/* Device and pinned-host allocations (cudaMalloc / cudaMallocHost calls)
 * made so far by every pipeline of the process: a caller can check that a
 * stretch of calls allocated nothing (no counterpart in the reference). */
unsigned long long ps3d_allocation_count(void);

/* ---- command buffers (no counterpart in the reference, whose drawVAO runs
 * immediately).  Between ps3d_cmdbuf_begin and ps3d_cmdbuf_end, clears and
 * draws are recorded into a command buffer instead of the pipeline's queue.
 * ps3d_cmdbuf_submit runs it: the first submission runs it like ps3d_finish
 * and then captures its kernels into a CUDA graph; later submissions launch
 * that graph (asynchronously) after, if uploadInputs, copying the recorded
 * draw descriptors and uniforms from pinned host memory again.  A command
 * buffer refers to the textures and VBOs it was recorded with: after one of
 * them is destroyed or replaced, submitting it returns PS3D_ERR_INVALID. */
int ps3d_cmdbuf_begin(ps3d_pipeline* p);
int ps3d_cmdbuf_end(ps3d_pipeline* p, ps3d_cmdbuf** out);
int ps3d_cmdbuf_submit(ps3d_pipeline* p, ps3d_cmdbuf* cb, int uploadInputs);
int ps3d_cmdbuf_destroy(ps3d_pipeline* p, ps3d_cmdbuf* cb);
/* Bytes a submission with uploadInputs copies host -> device. */
int ps3d_cmdbuf_input_bytes(ps3d_pipeline* p, ps3d_cmdbuf* cb, size_t* out);

/* ---- OBJX mesh files (the reference's objcvt/objxio.h:42-52, objxio.cpp).
 * Little-endian, packed as the reference writes them: a file header
 * (version 0x010003, camera, four lights) and per mesh a 1627-byte header,
 * float4 positions, float4 normals, float4 tangents, float2 texture
 * coordinates (each as the header says) and int32 indices.  Host-only calls
 * (no device needed) except ps3d_objx_load_vao. */
typedef struct ps3d_objx ps3d_objx;
typedef struct {                 /* scene_desc (objxio.h:29-36) */
    float camera_pos[4], camera_ypr[4];
    float light_pos[4][4], light_dir[4][4];
    int light_types[4];          /* 0 omni (direction shorter than 1e-7), 1 directional */
} ps3d_objx_scene;
typedef struct {                 /* mesh_info (objxio.h:5-27) without the arrays */
    char name[260];
    unsigned num_vertices, num_indices;
    int has_texcoords, has_normals, has_tangents;
    float ambient[4], diffuse[4], specular[4];  /* r, g, b, a; clamped to [0, 1] when read */
    float specular_exponent;
    char diffuse_file[260], bump_file[260], spc_file[260], spe_file[260], programme[260];
} ps3d_objx_mesh_info;
/* create_objxA / write_mesh: arrays may be NULL (absent) except vertices;
 * indices iff num_indices.  close writes the mesh count. */
int ps3d_objx_create(const char* path, const ps3d_objx_scene* scene, ps3d_objx** out);
int ps3d_objx_write_mesh(ps3d_objx* h, const ps3d_objx_mesh_info* info, const float* vertices, const float* normals,
                         const float* tangents, const float* texcoords, const int* indices);
/* open_objxA / get_mesh_count / read_mesh_header / read_mesh / close_objx.
 * read_mesh fills the arrays that are not NULL (num_vertices float4 / float2
 * elements, num_indices ints) and skips the rest; tangents asked for but
 * absent are derived from the texture coordinates (the reference's
 * generate_tangents reads an uninitialised vector and, for indexed meshes,
 * clears the positions; here the evident intent: per-triangle
 * ((c-a)*dv2 - (b-a)*dv1) / (du1*dv2 - dv1*du2), summed per vertex and
 * normalised when indexed). */
int ps3d_objx_open(const char* path, ps3d_objx_scene* scene, ps3d_objx** out);
int ps3d_objx_mesh_count(ps3d_objx* h);
int ps3d_objx_read_mesh_header(ps3d_objx* h, ps3d_objx_mesh_info* info);
int ps3d_objx_read_mesh(ps3d_objx* h, float* vertices, float* normals, float* tangents, float* texcoords,
                        int* indices);
int ps3d_objx_close(ps3d_objx* h);
/* The reference demo's SceneObject::findOrCreateVao (test/scenobj.cpp:88-162)
 * for mesh `meshIndex` of an OBJX file: a new VAO with slot 0 positions
 * (w = 1), and with texture coordinates slot 1 tangents, 2 binormals =
 * normalise(cross(normal, tangent)), 4 texture coordinates, and slot 3
 * normals -- the DEF03 layout.  Non-indexed meshes only. */
int ps3d_objx_load_vao(ps3d_pipeline* p, const char* path, int meshIndex, int* vao);

/* ---- timing on the pipeline's stream (CUDA events) */
int ps3d_timer_begin(ps3d_pipeline* p);
int ps3d_timer_end(ps3d_pipeline* p, float* ms);
/* Kernel families for ps3d_profile_read. */
#define PS3D_K_SETUP 0
#define PS3D_K_SCAN 1
#define PS3D_K_EMIT 2
#define PS3D_K_BOUNDS 3  /* per-bin list starts */
#define PS3D_K_SORT 4    /* radix passes of the (bin, triangle) pairs */
#define PS3D_K_RASTER 5
#define PS3D_K_SHADE 6
#define PS3D_K_FILL 7
#define PS3D_K_POST 8    /* post-processors */
#define PS3D_K_COUNT 9
/* Checks the bounded device waits: one warp polls a flag that nothing sets,
 * sleeping between polls, and gives up after `spins` polls, marking the
 * failure as an expired look-back of the bin sort does.  Returns
 * PS3D_ERR_TIMEOUT (the expected outcome: the wait ran out and the host
 * reported it) with the kernel's time in *ms; the pipeline stays usable. */
int ps3d_selftest_wait(ps3d_pipeline* p, int spins, float* ms);
/* Checks the kernels' fast correctly rounded reciprocal and quotient
 * against CUDA's IEEE ones on the current device: every float mantissa of
 * exponents -100..100 for the reciprocal, `pairs` hashed pairs for the
 * quotient.  Both counts must be 0. */
int ps3d_selftest_division(uint64_t pairs, uint64_t* rcpMismatches, uint64_t* divMismatches);
/* Checks the raster's span occlusion test (a span is dropped before its
 * per-pixel depths are computed when no pixel can pass the depth test)
 * against the per-pixel loop it replaces, on `cases` random spans with depth
 * bounds around the pass/fail boundary: *wrong must be 0; *occluded is how
 * many spans it dropped. */
int ps3d_selftest_occlusion(uint64_t cases, uint64_t* wrong, uint64_t* occluded);
/* Overwrites `bytes` of an internal device buffer on the pipeline's stream
 * (benchmarking aid: evicts the 126 MB L2 between timed frames). */
int ps3d_l2_scrub(ps3d_pipeline* p, size_t bytes);
/* When on, each kernel launch outside graphs is bracketed by CUDA events,
 * and a launch's passes run one after another on the pipeline's stream (not
 * overlapped on two), so that each kernel's events time that kernel alone. */
int ps3d_profile_enable(ps3d_pipeline* p, int on);
/* Waits, then returns per family the launches and milliseconds since the
 * last read (arrays of PS3D_K_COUNT). */
int ps3d_profile_read(ps3d_pipeline* p, int* launches, double* ms);

#ifdef __cplusplus
}
#endif
#endif
