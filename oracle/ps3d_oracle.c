/*
 * ps3d_oracle.c -- C restatement of the reference (CallMeZhou/Puresoft3D)
 * pipeline for the per-fragment path: vertex fetch and processing, perspective
 * divide, back-face cull, z-reject, scanline rasterisation, span set-up,
 * perspective-correct interpolation, depth test, fragment shading, FBO write.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg; nothing in the
 * product calls it.
 *
 * It follows the reference operation by operation, in the same FP32 order
 * (compile with -ffp-contract=off).  Parity with the reference itself is
 * pinned by golden fixtures rendered by the reference's own sources
 * (oracle/_ref, tests/golden).  Citations are file:line in
 * src/puresoft3d/ or src/mcemath/ of the reference.
 *
 * The reference's shaders normalise and divide with the x86 approximate
 * reciprocal and reciprocal square root (rcpps / rsqrtss, vector.cpp:158-169
 * mcemaths_div_3_4, :225-250 mcemaths_norm_3_4), whose results depend on the
 * host.  Here they are the table restatement of the instructions of the host
 * the golden fixtures were made on (x86_approx.h, generated from and checked
 * against the instructions on all 2^32 inputs), so that the colour matches
 * the reference build bit for bit on every host.
 *
 * Threads: the reference hands row y to fragment thread y % (N-1)
 * (drawvao.cpp:77-83); each thread walks its rows' spans in submission order.
 * Results depend only on that per-row order, so here each draw first builds
 * the span tasks (serially, like the reference's producer thread) and then
 * `threads` workers process rows y % threads == t in task order.
 *
 * Deviations (all in cases the benchmark scenes never reach):
 *  - TEST_DEPTH without UPDATE_DEPTH: the reference never positions the depth
 *    cursor in that mode (fragthrd.cpp:184-203) and reads a stale pixel; here
 *    the pixel under the fragment is read.
 *  - Triangles with non-finite vertex coordinates make the reference index
 *    its row table out of range (rasterizer.cpp:93-118); here they draw nothing.
 */
#include <math.h>
#include <float.h>
#include <limits.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include "ps3d_oracle.h"
#include "x86_approx.h"

/* rcpps / rsqrtss of one lane on the reference's host (x86_approx.h). */
static float x86_rcp(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    u = x86a_rcp_bits(u);
    memcpy(&x, &u, 4);
    return x;
}

static float x86_rsqrt(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    u = x86a_rsqrt_bits(u);
    memcpy(&x, &u, 4);
    return x;
}

/* mcemaths_norm_3_4's scale (vector.cpp:225-250): rsqrtss of the haddps sum
   of the squares. */
static float norm_scale(const float* v) { return x86_rsqrt((v[0] * v[0] + v[1] * v[1]) + (v[2] * v[2] + v[3] * v[3])); }
#include "shade_ref.h"

#define MAX_VBOS 16      /* config.h:4 */
#define MAX_UNIFORMS 1024 /* config.h:5 */
#define MAX_FBOS 16      /* config.h:3-9 */
#define MAX_VECS 8       /* float4 varyings per vertex, enough for every built-in processor */
#define MAX_LEVELS 16

#define BEHAVIOR_UPDATE_DEPTH 1 /* pipeline.h:16-19 */
#define BEHAVIOR_TEST_DEPTH 2
#define BEHAVIOR_FACE_CULLING 4
#define BEHAVIOR_ALPHABLEND 8

/* processor ids (include/ps3d.h) */
enum {
    VP_DEF01 = 0x0101, IP_DEF01 = 0x0102, FP_DEF01 = 0x0103,
    VP_DEF02 = 0x0201, IP_DEF02 = 0x0202, FP_DEF02 = 0x0203,
    VP_DEF03 = 0x0301, IP_DEF03 = 0x0302, FP_DEF03 = 0x0303,
    VP_DEF04 = 0x0401, IP_DEF04 = 0x0402, FP_DEF04 = 0x0403,
    VP_DEF05 = 0x0501, IP_DEF05 = 0x0502, FP_DEF05 = 0x0503,
    VP_SHADOW = 0x0601,
    VP_PLANET = 0x0701, IP_PLANET = 0x0702, FP_EARTH = 0x0703, FP_SATELLITE = 0x0713,
    VP_CLOUD = 0x0801, IP_CLOUD = 0x0802, FP_CLOUD = 0x0803,
    VP_CLOUDSHADOW = 0x0901, IP_CLOUDSHADOW = 0x0902, FP_CLOUDSHADOW = 0x0903,
    /* the scene viewer demo's sets (test2/testproc.h) */
    VP_POSITIONONLY = 0x0A01, IP_NULL = 0x0A02, FP_SINGLECOLOURNL = 0x0A03,
    VP_SINGLECOLOUR = 0x0B01, IP_SINGLECOLOUR = 0x0B02, FP_SINGLECOLOUR = 0x0B03,
    VP_DIFFUSEONLY = 0x0C01, IP_DIFFUSEONLY = 0x0C02, FP_DIFFUSEONLY = 0x0C03,
    VP_SHADOW2 = 0x0D01, FP_NULL = 0x0D03,
    FP_LIT1 = 0x1103, FP_LIT1A = 0x1403, FP_LIT3 = 0x1303,
    VP_LIT2 = 0x1201, IP_LIT2 = 0x1202, FP_LIT2 = 0x1203
};

/* A texture: `layers` images of scanline*height bytes each, back to back
   (layer 0 is the FBO itself, 1.. its extra layers, fbo.cpp:59-73; a cube
   map has the six faces in LAYER order, fbo.h:19). */
typedef struct {
    int width, height, scanline, elemLen, wrap, topDown, layers;
    uint8_t* buf;
} o_fbo;

typedef struct {
    int unitBytes, count;
    uint8_t* data;
} o_vbo;

typedef struct {
    o_vbo* vbo[MAX_VBOS];
} o_vao;

typedef struct {
    size_t cap;
    void* data;
} o_uniform;

typedef struct {
    int vp, ip, fp;
} o_prog;

typedef struct {
    int x1, x2, y;
    float pzStart, pzStep, cf2Start, cf2Step;
    float user[2 * MAX_VECS * 4]; /* start vectors then step vectors */
} o_task;

typedef struct {
    o_task* items;
    size_t n, cap;
} o_tasklist;

struct ps3do {
    int devW, devH;   /* device size: display and default depth */
    int W, H;         /* rasteriser size (setViewport, pipeline.cpp:364-373) */
    o_fbo display;    /* BGRA8, topDown (pipeline.cpp:48) */
    o_fbo defDepth;   /* FP32, scanline rounded to 4 floats (pipeline.cpp:31) */
    o_fbo* depth;
    o_fbo* fbos[MAX_FBOS]; /* setFBO's slots (pipeline.cpp:260-275): 0 = the colour target, the display by default */
    o_fbo** tex;
    int ntex;
    int* procs;
    int nprocs;
    o_prog* progs;
    int nprogs;
    int vp, ip, fp; /* processor ids in use, 0 = none */
    o_vao** vaos;
    int nvao;
    o_uniform uni[MAX_UNIFORMS];
    int behavior;
    int threads;
    o_tasklist* lists; /* one per worker */
    long long tested, passed;
    long long spanHist[32]; /* spans by floor(log2(x2 - x1 + 1)) */
    int errOn;              /* measure the FP32 shading error against an FP64 re-shade */
    double errMax, errSum;
    long long errN, errOver;
    /* worker pool */
    pthread_t* th;
    pthread_mutex_t mu;
    pthread_cond_t cv, done;
    int gen, finished, quit;
    void* cur_draw; /* the draw the pool is working on (guarded by gen) */
};

/* ------------------------------------------------------------------ maths */
/* mcemaths semantics (vector.cpp, matrix.cpp): 4-wide lane-wise ops. */

static void m4v4(float* r, const float* m, const float* v) /* matrix.cpp:515-557 */
{
    float o[4];
    for (int i = 0; i < 4; i++) o[i] = ((v[0] * m[i] + v[1] * m[4 + i]) + v[2] * m[8 + i]) + v[3] * m[12 + i];
    memcpy(r, o, 16);
}

static void m4m4(float* d, const float* l, const float* r) /* matrix.cpp:588-690 */
{
    for (int c = 0; c < 4; c++) m4v4(d + 4 * c, l, r + 4 * c);
}

static float hsum4(const float* a) { return (a[0] + a[1]) + (a[2] + a[3]); } /* haddps x2 */

/* ------------------------------------------------------------ object pools */

static int grow(void** arr, int n, size_t elem)
{
    void* q = realloc(*arr, (size_t)(n + 1) * elem);
    if (!q) return -3;
    *arr = q;
    return 0;
}

static void* worker(void* arg);

ps3do* ps3do_create(int width, int height, int threads)
{
    ps3do* p = (ps3do*)calloc(1, sizeof(ps3do));
    if (!p) return NULL;
    if (threads < 1) threads = 1;
    p->devW = p->W = width;
    p->devH = p->H = height;
    p->display.width = width;
    p->display.height = height;
    p->display.scanline = width * 4;
    p->display.elemLen = 4;
    p->display.topDown = 1;
    p->display.buf = (uint8_t*)calloc((size_t)width * 4 * height, 1);
    p->fbos[0] = &p->display; /* setFBO(0, NULL) in the constructor (pipeline.cpp:49) */
    p->defDepth.width = width;
    p->defDepth.height = height;
    p->defDepth.scanline = ((int)(width / 4.0f + 0.5f) * 4) * 4;
    p->defDepth.elemLen = 4;
    p->defDepth.buf = (uint8_t*)calloc((size_t)p->defDepth.scanline * height, 1);
    p->depth = &p->defDepth;
    p->behavior = BEHAVIOR_UPDATE_DEPTH | BEHAVIOR_TEST_DEPTH | BEHAVIOR_FACE_CULLING; /* pipeline.cpp:34 */
    p->threads = threads;
    p->lists = (o_tasklist*)calloc((size_t)threads, sizeof(o_tasklist));
    pthread_mutex_init(&p->mu, NULL);
    pthread_cond_init(&p->cv, NULL);
    pthread_cond_init(&p->done, NULL);
    if (threads > 1) {
        p->th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
        for (int i = 1; i < threads; i++) {
            void** a = (void**)malloc(2 * sizeof(void*));
            a[0] = p;
            a[1] = (void*)(intptr_t)i;
            pthread_create(&p->th[i], NULL, worker, a);
        }
    }
    return p;
}

void ps3do_destroy(ps3do* p)
{
    if (!p) return;
    if (p->threads > 1) {
        pthread_mutex_lock(&p->mu);
        p->quit = 1;
        p->gen++;
        pthread_cond_broadcast(&p->cv);
        pthread_mutex_unlock(&p->mu);
        for (int i = 1; i < p->threads; i++) pthread_join(p->th[i], NULL);
        free(p->th);
    }
    for (int i = 0; i < p->ntex; i++)
        if (p->tex[i]) { free(p->tex[i]->buf); free(p->tex[i]); }
    free(p->tex);
    for (int i = 0; i < p->nvao; i++)
        if (p->vaos[i]) {
            for (int j = 0; j < MAX_VBOS; j++)
                if (p->vaos[i]->vbo[j]) { free(p->vaos[i]->vbo[j]->data); free(p->vaos[i]->vbo[j]); }
            free(p->vaos[i]);
        }
    free(p->vaos);
    for (int i = 0; i < MAX_UNIFORMS; i++) free(p->uni[i].data);
    for (int i = 0; i < p->threads; i++) free(p->lists[i].items);
    free(p->lists);
    free(p->procs);
    free(p->progs);
    free(p->display.buf);
    free(p->defDepth.buf);
    pthread_mutex_destroy(&p->mu);
    pthread_cond_destroy(&p->cv);
    pthread_cond_destroy(&p->done);
    free(p);
}

/* tex.cpp:3-25: copies pixels into a pipeline-owned FBO (topDown = false). */
int ps3do_texture_create_layers(ps3do* p, int width, int height, int scanline, int elemLen, const void* pixels,
                                int wrap, int extraLayers)
{
    o_fbo* f;
    int slot = 0;
    size_t layer;
    if (elemLen != 1 && elemLen != 4) return -2; /* fbo.cpp:21-24 */
    if (width <= 0 || height <= 0 || scanline < width * elemLen) return -2;
    /* fbo.cpp:62-72: more than LAYER_MAX - 1 extra layers is out of range */
    if (extraLayers < 0 || extraLayers > 5) return -1;
    for (; slot < p->ntex; slot++)
        if (!p->tex[slot]) break;
    if (slot == p->ntex) {
        if (grow((void**)&p->tex, p->ntex, sizeof(o_fbo*))) return -3;
        p->tex[p->ntex++] = NULL;
    }
    f = (o_fbo*)calloc(1, sizeof(o_fbo));
    if (!f) return -3;
    f->width = width;
    f->height = height;
    f->scanline = scanline;
    f->elemLen = elemLen;
    f->wrap = wrap;
    f->layers = 1 + extraLayers;
    layer = (size_t)scanline * height;
    f->buf = (uint8_t*)calloc(layer * f->layers, 1);
    if (!f->buf) { free(f); return -3; }
    if (pixels) memcpy(f->buf, pixels, layer); /* tex.cpp:18-23: the default layer */
    p->tex[slot] = f;
    return slot;
}

int ps3do_texture_create(ps3do* p, int width, int height, int scanline, int elemLen, const void* pixels, int wrap)
{
    return ps3do_texture_create_layers(p, width, height, scanline, elemLen, pixels, wrap, 0);
}

/* getTexture(idx, image, layer) (tex.cpp:27-37) hands out the layer's
   buffer; these copy into or out of it. */
int ps3do_texture_write_layer(ps3do* p, int idx, int layer, const void* pixels, size_t bytes)
{
    size_t n;
    if (idx < 0 || idx >= p->ntex || !p->tex[idx]) return -1;
    if (layer < 0 || layer >= p->tex[idx]->layers) return -1;
    n = (size_t)p->tex[idx]->scanline * p->tex[idx]->height;
    memcpy(p->tex[idx]->buf + n * layer, pixels, n < bytes ? n : bytes);
    return 0;
}

int ps3do_texture_read_layer(ps3do* p, int idx, int layer, void* out, size_t bytes)
{
    size_t n;
    if (idx < 0 || idx >= p->ntex || !p->tex[idx]) return -1;
    if (layer < 0 || layer >= p->tex[idx]->layers) return -1;
    n = (size_t)p->tex[idx]->scanline * p->tex[idx]->height;
    memcpy(out, p->tex[idx]->buf + n * layer, n < bytes ? n : bytes);
    return 0;
}

int ps3do_texture_read(ps3do* p, int idx, void* out, size_t bytes)
{
    return ps3do_texture_read_layer(p, idx, 0, out, bytes);
}

static int known_processor(int id)
{
    switch (id) {
    case VP_DEF01: case IP_DEF01: case FP_DEF01: case VP_DEF05: case IP_DEF05: case FP_DEF05:
    case VP_DEF02: case IP_DEF02: case FP_DEF02: case VP_DEF03: case IP_DEF03: case FP_DEF03:
    case VP_DEF04: case IP_DEF04: case FP_DEF04:
    case VP_PLANET: case IP_PLANET: case FP_EARTH: case FP_SATELLITE:
    case VP_CLOUD: case IP_CLOUD: case FP_CLOUD: case VP_CLOUDSHADOW: case IP_CLOUDSHADOW: case FP_CLOUDSHADOW:
    case VP_POSITIONONLY: case IP_NULL: case FP_SINGLECOLOURNL: case VP_SINGLECOLOUR: case IP_SINGLECOLOUR:
    case FP_SINGLECOLOUR: case VP_DIFFUSEONLY: case IP_DIFFUSEONLY: case FP_DIFFUSEONLY: case VP_SHADOW2: case FP_NULL:
    case VP_SHADOW: case FP_LIT1: case FP_LIT1A: case FP_LIT3: case VP_LIT2: case IP_LIT2: case FP_LIT2:
        return 1;
    }
    return 0;
}

static int proc_kind(int id) { return id & 0xf; } /* 1 = VP, 2 = IP, 3 = FP */

int ps3do_processor_add(ps3do* p, int id) /* prog.cpp:3-20 */
{
    if (!known_processor(id)) return -2;
    if (grow((void**)&p->procs, p->nprocs, sizeof(int))) return -3;
    p->procs[p->nprocs] = id;
    return p->nprocs++;
}

int ps3do_programme_create(ps3do* p, int vid, int iid, int fid) /* prog.cpp:43-108 */
{
    if (vid < 0 || vid >= p->nprocs || iid < 0 || iid >= p->nprocs || fid < 0 || fid >= p->nprocs) return -1;
    if (grow((void**)&p->progs, p->nprogs, sizeof(o_prog))) return -3;
    p->progs[p->nprogs].vp = vid;
    p->progs[p->nprogs].ip = iid;
    p->progs[p->nprogs].fp = fid;
    return p->nprogs++;
}

int ps3do_programme_use(ps3do* p, int idx) /* prog.cpp:121-131: dynamic_cast yields NULL on a kind mismatch */
{
    int v, i, f;
    if (idx < 0 || idx >= p->nprogs) return -1;
    v = p->procs[p->progs[idx].vp];
    i = p->procs[p->progs[idx].ip];
    f = p->procs[p->progs[idx].fp];
    p->vp = proc_kind(v) == 1 ? v : 0;
    p->ip = proc_kind(i) == 2 ? i : 0;
    p->fp = proc_kind(f) == 3 ? f : 0;
    return 0;
}

int ps3do_vao_create(ps3do* p) /* pipeline.cpp:118-136 */
{
    int slot = 0;
    for (; slot < p->nvao; slot++)
        if (!p->vaos[slot]) break;
    if (slot == p->nvao) {
        if (grow((void**)&p->vaos, p->nvao, sizeof(o_vao*))) return -3;
        p->vaos[p->nvao++] = NULL;
    }
    p->vaos[slot] = (o_vao*)calloc(1, sizeof(o_vao));
    return p->vaos[slot] ? slot : -3;
}

int ps3do_vbo_attach(ps3do* p, int vao, int slot, int unitBytes, int count, const void* data)
{
    o_vbo* v;
    if (vao < 0 || vao >= p->nvao || !p->vaos[vao]) return -1;
    if (slot < 0 || slot >= MAX_VBOS) return -1;
    v = (o_vbo*)calloc(1, sizeof(o_vbo));
    v->unitBytes = unitBytes;
    v->count = count;
    v->data = (uint8_t*)malloc((size_t)unitBytes * count + 16);
    if (data) memcpy(v->data, data, (size_t)unitBytes * count);
    if (p->vaos[vao]->vbo[slot]) { free(p->vaos[vao]->vbo[slot]->data); free(p->vaos[vao]->vbo[slot]); }
    p->vaos[vao]->vbo[slot] = v;
    return 0;
}

int ps3do_set_uniform(ps3do* p, int idx, const void* data, size_t len) /* pipeline.cpp:277-312 */
{
    if (idx < 0 || idx >= MAX_UNIFORMS) return -1;
    if (!data) {
        free(p->uni[idx].data);
        p->uni[idx].data = NULL;
        p->uni[idx].cap = 0;
        return 0;
    }
    if (p->uni[idx].cap < len) {
        free(p->uni[idx].data);
        p->uni[idx].data = malloc(len);
        if (!p->uni[idx].data) return -3;
        p->uni[idx].cap = len;
    }
    memcpy(p->uni[idx].data, data, len);
    return 0;
}

int ps3do_set_depth(ps3do* p, int idx) /* pipeline.cpp:218-239 */
{
    if (idx == -1) { p->depth = &p->defDepth; return 0; }
    if (idx < 0 || idx >= p->ntex || !p->tex[idx]) return -1;
    if (p->tex[idx]->elemLen != 4 || p->tex[idx]->scanline % 4) return -2;
    p->depth = p->tex[idx];
    return 0;
}

/* PuresoftPipeline::setFBO (pipeline.cpp:260-275) with a texture as the
   FBO (-1: none; slot 0 then falls back to the display).  The fragment
   processors write slot 0 (FBOBridge, fragthrd.cpp:55-95) and postProcess
   runs on it (post.cpp:14); clearColour still clears the display. */
int ps3do_set_fbo(ps3do* p, int idx, int tex)
{
    if (idx < 0 || idx >= MAX_FBOS) return -1;
    if (tex == -1) {
        p->fbos[idx] = idx == 0 ? &p->display : NULL;
        return 0;
    }
    if (tex < 0 || tex >= p->ntex || !p->tex[tex]) return -1;
    if (p->tex[tex]->elemLen != 4) return -2; /* the processors write 4-byte BGRA */
    p->fbos[idx] = p->tex[tex];
    return 0;
}

int ps3do_set_viewport(ps3do* p, int width, int height)
{
    if (width <= 0 || height <= 0) return -2;
    p->W = width;
    p->H = height;
    return 0;
}

int ps3do_enable(ps3do* p, int bits) { p->behavior |= bits; return 0; }
int ps3do_disable(ps3do* p, int bits) { p->behavior &= ~bits; return 0; }

int ps3do_clear_depth(ps3do* p, float v) /* pipeline.cpp:334-338 -> fbo.cpp clear16: every byte */
{
    size_t n = (size_t)p->depth->scanline * p->depth->height / 4;
    float* d = (float*)p->depth->buf;
    for (size_t i = 0; i < n; i++) d[i] = v;
    return 0;
}

/* pipeline.cpp:340-343.  The reference's clear4 skips the last memory row
   (fbo.cpp:336); a clear here covers every pixel, as the product's does. */
int ps3do_clear_colour(ps3do* p, uint32_t bgra)
{
    uint32_t* d = (uint32_t*)p->display.buf;
    for (size_t i = 0; i < (size_t)p->display.width * p->display.height; i++) d[i] = bgra;
    return 0;
}

/* PuresoftPipeline::postProcess (post.cpp:3-19) with the built-in
   post-processors, over FBO slot 0 (the display unless setFBO moved it):
   0x7001 the demo's per-byte wrapping add (test2/testpost.cpp:9-43) of a
   BGRA addend, 0x7002 linear depth fog.  Pixel row y of the display lives at
   memory row H-1-y, of a texture (and of the depth buffer) at row y. */
int ps3do_post_process(ps3do* p, int id, const void* params, size_t bytes)
{
    o_fbo* f = p->fbos[0];
    int W = f->width, H = f->height;
    if (id == 0x7001) {
        uint8_t add[4] = {50, 50, 50, 50};
        if (params) {
            if (bytes < 4) return -2;
            memcpy(add, params, 4);
        }
        for (int r = 0; r < H; r++) {
            uint8_t* row = f->buf + (size_t)r * f->scanline;
            for (int x = 0; x < 4 * W; x++) row[x] = (uint8_t)(row[x] + add[x & 3]);
        }
        return 0;
    }
    if (id == 0x7002) {
        uint32_t fog;
        float nearD, farD, range;
        const o_fbo* d = p->depth;
        if (!params || bytes < 12) return -2;
        if (d->width < W || d->height < H || d->scanline < 4 * W) return -2;
        memcpy(&fog, params, 4);
        memcpy(&nearD, (const uint8_t*)params + 4, 4);
        memcpy(&farD, (const uint8_t*)params + 8, 4);
        range = farD - nearD;
        for (int y = 0; y < H; y++) {
            const float* drow = (const float*)(d->buf + (size_t)y * d->scanline);
            uint8_t* crow = f->buf + (size_t)(f->topDown ? H - 1 - y : y) * f->scanline;
            for (int x = 0; x < W; x++) {
                float t = (drow[x] - nearD) / range;
                t = t > 0.0f ? t : 0.0f;
                t = t < 1.0f ? t : 1.0f;
                for (int k = 0; k < 3; k++) {
                    float c = (float)crow[4 * x + k], f = (float)((fog >> (8 * k)) & 0xff);
                    crow[4 * x + k] = (uint8_t)(int)(c + (f - c) * t);
                }
            }
        }
        return 0;
    }
    return -2;
}

int ps3do_read_colour(ps3do* p, void* out)
{
    memcpy(out, p->display.buf, (size_t)p->display.scanline * p->display.height);
    return 0;
}

int ps3do_read_depth(ps3do* p, void* out)
{
    memcpy(out, p->defDepth.buf, (size_t)p->defDepth.scanline * p->defDepth.height);
    return 0;
}

void ps3do_set_colour_error(ps3do* p, int on) { p->errOn = on != 0; }

void ps3do_colour_error(ps3do* p, double* maxErr, double* meanErr, long long* channels, long long* over1)
{
    *maxErr = p->errMax;
    *meanErr = p->errN ? p->errSum / (double)p->errN : 0.0;
    *channels = p->errN;
    *over1 = p->errOver;
}

long long ps3do_fragments_tested(ps3do* p) { return p->tested; }
void ps3do_span_histogram(ps3do* p, long long* out) { memcpy(out, p->spanHist, sizeof p->spanHist); }
long long ps3do_fragments_passed(ps3do* p) { return p->passed; }

/* ------------------------------------------------------ processors (VP/IP/FP) */

static int ip_vecs(int ip)
{
    switch (ip) {
    case IP_DEF01: return 3; /* PROCDATA_DEF01: normal, worldPos, texcoord (tex1light1.h:4-9) */
    case IP_LIT2: return 5;  /* normal, tangent, worldPos, texcoord, shadowPos */
    case IP_DEF02: return 3; /* PROCDATA_DEF02: normal, worldPos, colour (colr1light1.h:3-9) */
    case IP_DEF03: return 5; /* PROCDATA_DEF03: tangent, binormal, normal, worldPos, texcoord (tex1bump1light1.h:4-11) */
    case IP_DEF04: return 1; /* PROCDATA_DEF04: direction (skybox.h:3-7) */
    case IP_PLANET: return 6; /* PROCDATA_PLANET: tangent, binormal, normal, worldPos, texcoord, shadowcoord
                                 (test/testproc.h:5-14) */
    case IP_CLOUD: return 4;  /* PROCDATA_CLOUD: normal, worldPos, texcoord, shadowcoord (test/testproc.h:73-80) */
    case IP_CLOUDSHADOW: return 1; /* PROCDATA_CLOUDSHADOW: texcoord (test/testproc.h:120-124) */
    case IP_SINGLECOLOUR: return 3; /* PROCDATA_SINGLECOLOUR: normal, worldPos, shadowcoord (test2/testproc.h:83-90) */
    case IP_DIFFUSEONLY: return 4;  /* PROCDATA_DIFFUSEONLY: normal, worldPos, texcoord, shadowcoord
                                       (test2/testproc.h:136-144) */
    default: return 0;       /* IP_DEF05: no varyings (shadow.h) */
    }
}

static const float* ufl(const ps3do* p, int i) { return (const float*)p->uni[i].data; }
static const int* uin(const ps3do* p, int i) { return (const int*)p->uni[i].data; }

/* Vertex processors.  in[j] points at this vertex's element of VBO j. */
static void run_vp(const ps3do* p, const void* const* in, float* pos, float* user)
{
    switch (p->vp) {
    case VP_DEF01: { /* tex1light1.cpp:22-41 */
        float* nrm = user, * wp = user + 4, * tc = user + 8;
        const float* uv = (const float*)in[4];
        m4v4(wp, ufl(p, 4), (const float*)in[0]);
        memcpy(pos, wp, 16);
        wp[3] = 0;
        m4v4(pos, ufl(p, 3), pos);
        m4v4(nrm, ufl(p, 5), (const float*)in[3]);
        tc[0] = uv[0];
        tc[1] = uv[1];
        tc[2] = tc[3] = 0.0f;
        break;
    }
    case VP_DEF02: { /* colr1light1.cpp:22-40: normal in VBO 1, colour in VBO 2 */
        float* nrm = user, * wp = user + 4, * col = user + 8;
        m4v4(wp, ufl(p, 4), (const float*)in[0]);
        memcpy(pos, wp, 16);
        wp[3] = 0;
        m4v4(pos, ufl(p, 3), pos);
        m4v4(nrm, ufl(p, 5), (const float*)in[1]);
        memcpy(col, in[2], 16);
        break;
    }
    case VP_DEF04: { /* skybox.cpp:23-44: the position passes through; the
                        direction is the view's inverse rotation (the
                        transposed view matrix with its last column zeroed)
                        times the normalised vector from the observer
                        (0, 0, 1) to the vertex */
        const float* v = (const float*)in[0];
        float d[4], inv[16], r;
        d[0] = v[0] - 0.0f;
        d[1] = v[1] - 0.0f;
        d[2] = v[2] - 1.0f;
        d[3] = 0.0f;
        r = norm_scale(d);
        for (int k = 0; k < 4; k++) d[k] = d[k] * r;
        for (int c = 0; c < 4; c++)
            for (int rr = 0; rr < 4; rr++) inv[4 * c + rr] = ufl(p, 1)[4 * rr + c];
        for (int k = 12; k < 16; k++) inv[k] = 0.0f;
        m4v4(user, inv, d);
        memcpy(pos, v, 16);
        break;
    }
    case VP_PLANET: { /* test/testproc.cpp:37-71: DEF03's outputs plus the world
                         position through the shadow projection (uniform 16) */
        float* tan = user, * bin = user + 4, * nrm = user + 8, * wp = user + 12, * tc = user + 16, * sc = user + 20;
        const float* uv = (const float*)in[4];
        m4v4(wp, ufl(p, 4), (const float*)in[0]);
        m4v4(sc, ufl(p, 16), wp);
        memcpy(pos, wp, 16);
        m4v4(pos, ufl(p, 3), pos);
        wp[3] = 0;
        m4v4(tan, ufl(p, 5), (const float*)in[1]);
        m4v4(bin, ufl(p, 5), (const float*)in[2]);
        m4v4(nrm, ufl(p, 5), (const float*)in[3]);
        tc[0] = uv[0];
        tc[1] = uv[1];
        tc[2] = tc[3] = 0.0f; /* left unset by the reference; never read */
        break;
    }
    case VP_CLOUD: { /* test/testproc.cpp:392-425 */
        float* nrm = user, * wp = user + 4, * tc = user + 8, * sc = user + 12;
        const float* uv = (const float*)in[4];
        m4v4(wp, ufl(p, 4), (const float*)in[0]);
        m4v4(sc, ufl(p, 16), wp);
        memcpy(pos, wp, 16);
        m4v4(pos, ufl(p, 3), pos);
        wp[3] = 0;
        m4v4(nrm, ufl(p, 5), (const float*)in[3]);
        tc[0] = uv[0];
        tc[1] = uv[1];
        tc[2] = tc[3] = 0.0f; /* left unset by the reference; never read */
        break;
    }
    case VP_POSITIONONLY: /* test2/testproc.cpp:13-23: PVM (uniform 5) * p */
        m4v4(pos, ufl(p, 5), (const float*)in[0]);
        break;
    case VP_SHADOW2: { /* test2/testproc.cpp:507-518: positions x0.9 (mcemaths_mul_3), then PVM (5) * p */
        float adj[4];
        memcpy(adj, in[0], 16);
        adj[0] = adj[0] * 0.9f;
        adj[1] = adj[1] * 0.9f;
        adj[2] = adj[2] * 0.9f;
        m4v4(pos, ufl(p, 5), adj);
        break;
    }
    case VP_SINGLECOLOUR:   /* test2/testproc.cpp:88-116 */
    case VP_DIFFUSEONLY: {  /* test2/testproc.cpp:304-336: world position M (0) * p, its
                               shadow projection (6), PVM (5) * p, normal MR (1) * n */
        const int diffuse = p->vp == VP_DIFFUSEONLY;
        float* nrm = user, * wp = user + 4, * sc = user + (diffuse ? 12 : 8);
        m4v4(wp, ufl(p, 0), (const float*)in[0]);
        m4v4(sc, ufl(p, 6), wp);
        if (!diffuse) wp[3] = 0;
        m4v4(pos, ufl(p, 5), (const float*)in[0]);
        if (diffuse) wp[3] = 0;
        m4v4(nrm, ufl(p, 1), (const float*)in[3]);
        if (diffuse) {
            const float* uv = (const float*)in[4];
            user[8] = uv[0];
            user[9] = uv[1];
            user[10] = user[11] = 0.0f; /* left unset by the reference; never read */
        }
        break;
    }
    case VP_CLOUDSHADOW: { /* test/testproc.cpp:595-610: positions x0.95 (mcemaths_mul_3), (PV*M) * p */
        float adj[4], pvm[16];
        const float* uv = (const float*)in[4];
        memcpy(adj, in[0], 16);
        adj[0] = adj[0] * 0.95f;
        adj[1] = adj[1] * 0.95f;
        adj[2] = adj[2] * 0.95f;
        m4m4(pvm, ufl(p, 3), ufl(p, 4));
        m4v4(pos, pvm, adj);
        user[0] = uv[0];
        user[1] = uv[1];
        user[2] = user[3] = 0.0f;
        break;
    }
    case VP_DEF03: { /* tex1bump1light1.cpp:22-46 */
        float* tan = user, * bin = user + 4, * nrm = user + 8, * wp = user + 12, * tc = user + 16;
        const float* uv = (const float*)in[4];
        m4v4(wp, ufl(p, 4), (const float*)in[0]);
        memcpy(pos, wp, 16);
        wp[3] = 0;
        m4v4(pos, ufl(p, 3), pos);
        m4v4(tan, ufl(p, 5), (const float*)in[1]);
        m4v4(bin, ufl(p, 5), (const float*)in[2]);
        m4v4(nrm, ufl(p, 5), (const float*)in[3]);
        tc[0] = uv[0];
        tc[1] = uv[1];
        tc[2] = tc[3] = 0.0f;
        break;
    }
    case VP_DEF05: { /* shadow.cpp:21-29 */
        float adj[4], pvm[16];
        memcpy(adj, in[0], 16);
        adj[0] = adj[0] * 0.9f; /* mcemaths_mul_3: three lanes (vector.cpp:517-534) */
        adj[1] = adj[1] * 0.9f;
        adj[2] = adj[2] * 0.9f;
        m4m4(pvm, ufl(p, 3), ufl(p, 4));
        m4v4(pos, pvm, adj);
        break;
    }
    case VP_SHADOW: { /* DEF05 without the x0.9 scale */
        float pvm[16];
        m4m4(pvm, ufl(p, 3), ufl(p, 4));
        m4v4(pos, pvm, (const float*)in[0]);
        break;
    }
    case VP_LIT2: {
        float* nrm = user, * tan = user + 4, * wp = user + 8, * tc = user + 12, * sp = user + 16;
        const float* t = (const float*)in[1];
        const float* uv = (const float*)in[4];
        float t3[4] = {t[0], t[1], t[2], 0.0f};
        m4v4(wp, ufl(p, 4), (const float*)in[0]);
        memcpy(pos, wp, 16);
        m4v4(sp, ufl(p, 6), wp);
        wp[3] = 0;
        m4v4(pos, ufl(p, 3), pos);
        m4v4(nrm, ufl(p, 5), (const float*)in[3]);
        m4v4(tan, ufl(p, 5), t3);
        tan[3] = t[3];
        tc[0] = uv[0];
        tc[1] = uv[1];
        tc[2] = tc[3] = 0.0f;
        break;
    }
    default: break;
    }
}

/* Interpolation processors: every reference IP is 4-wide linear algebra over
   its float4 varyings (tex1light1.cpp:60-135), so one routine serves all. */
static void ip_by_contributes(int nv, float* out, const float* const* vert, const float* c)
{
    for (int k = 0; k < nv; k++)
        for (int l = 0; l < 4; l++) {
            float t0 = vert[0][4 * k + l] * c[0], t1 = vert[1][4 * k + l] * c[1], t2 = vert[2][4 * k + l] * c[2];
            out[4 * k + l] = (t0 + t1) + t2;
        }
}

static void ip_calc_step(int nv, float* step, const float* start, const float* end, int n)
{
    float r = 0 == n ? 1.0f : 1.0f / (float)n;
    for (int i = 0; i < 4 * nv; i++) step[i] = (end[i] - start[i]) * r;
}

/* The step vector stepForward adds to vector k: its own, except in the
   demo's IP_Planet, which steps the tangent and the binormal by the normal's
   step (test/testproc.cpp:171-195). */
static int step_src(int ip, int k) { return (ip == IP_PLANET && k < 2) ? 2 : k; }

static void ip_step_forward(int ip, int nv, float* start, const float* step, int n)
{
    if (1 == n) {
        for (int k = 0; k < nv; k++)
            for (int l = 0; l < 4; l++) start[4 * k + l] = start[4 * k + l] + step[4 * step_src(ip, k) + l];
    } else {
        float fn = (float)n;
        for (int k = 0; k < nv; k++)
            for (int l = 0; l < 4; l++) start[4 * k + l] = start[4 * k + l] + step[4 * step_src(ip, k) + l] * fn;
    }
}

static sr_level level_of(const o_fbo* f)
{
    sr_level l;
    l.base = f->buf;
    l.width = f->width;
    l.height = f->height;
    l.scanline = f->scanline;
    return l;
}

/* Per-draw fragment-processor state (the FP's preprocess, drawvao.cpp:18-20). */
typedef struct {
    const float* light;
    const float* cam;
    const o_fbo* tex;
    const o_fbo* tex2;  /* DEF03's bump map */
    const o_fbo* cube;  /* DEF04's cube map */
    const o_fbo* spec, * night, * proj; /* the planet set's specular, night and shadow maps */
    sr_level chainA[MAX_LEVELS], chainN[MAX_LEVELS];
    int levelsA, levelsN;
    const float* shadow;
    int shadowSize, shadowScan;
    float lodScale, bias;
    /* the scene viewer demo's lighting (test2/testproc.h:1-30: uniforms 21
       light direction, 30 ambient, 31 diffuse, 32 specular colour, 33
       specular exponent) */
    const float* ldir, * amb, * dif, * scol;
    unsigned sexp;
} fp_state;

static int fp_prepare(const ps3do* p, fp_state* s)
{
    memset(s, 0, sizeof *s);
    switch (p->fp) {
    case FP_DEF01:
    case FP_LIT1:
    case FP_LIT1A: {
        int t = *uin(p, 9);
        if (t < 0 || t >= p->ntex || !p->tex[t]) return -1;
        s->light = ufl(p, 7);
        s->cam = ufl(p, 8);
        s->tex = p->tex[t];
        break;
    }
    case FP_CLOUD: { /* test/testproc.cpp:526-532: diffuse 9, shadow 15 */
        int t = *uin(p, 9), sm = *uin(p, 15);
        if (t < 0 || t >= p->ntex || !p->tex[t] || p->tex[t]->elemLen != 4) return -1;
        if (sm < 0 || sm >= p->ntex || !p->tex[sm] || p->tex[sm]->elemLen != 4) return -1;
        s->light = ufl(p, 7);
        s->cam = ufl(p, 8);
        s->tex = p->tex[t];
        s->proj = p->tex[sm];
        break;
    }
    case FP_SINGLECOLOURNL: /* test2/testproc.cpp:49-53 */
        s->dif = ufl(p, 31);
        break;
    case FP_SINGLECOLOUR:   /* test2/testproc.cpp:199-209 */
    case FP_DIFFUSEONLY: {  /* test2/testproc.cpp:447-456: shadow map 23, diffuse texture 40 */
        int sm = *uin(p, 23);
        if (sm < 0 || sm >= p->ntex || !p->tex[sm] || p->tex[sm]->elemLen != 4) return -1;
        s->proj = p->tex[sm];
        if (p->fp == FP_DIFFUSEONLY) {
            int t = *uin(p, 40);
            if (t < 0 || t >= p->ntex || !p->tex[t] || p->tex[t]->elemLen != 4) return -1;
            s->tex = p->tex[t];
        } else {
            s->dif = ufl(p, 31);
            s->scol = ufl(p, 32);
        }
        s->light = ufl(p, 20);
        s->ldir = ufl(p, 21);
        s->cam = ufl(p, 22);
        s->amb = ufl(p, 30);
        s->sexp = (unsigned)*ufl(p, 33);
        break;
    }
    case FP_CLOUDSHADOW: { /* test/testproc.cpp:672-675: the cloud texture at 9 */
        int t = *uin(p, 9);
        if (t < 0 || t >= p->ntex || !p->tex[t] || p->tex[t]->elemLen != 4) return -1;
        s->tex = p->tex[t];
        break;
    }
    case FP_EARTH:     /* test/testproc.cpp:197-206 */
    case FP_SATELLITE: { /* test/testproc.cpp:290-297 */
        const int slots[5] = {9, 10, 11, 12, 15};
        const o_fbo* t[5];
        int n = p->fp == FP_EARTH ? 5 : 3;
        for (int i = 0; i < 5; i++) {
            int slot = (p->fp == FP_SATELLITE && i >= 2) ? 15 : slots[i];
            int k = *uin(p, slot);
            if (i >= n && p->fp == FP_SATELLITE) { t[i] = NULL; continue; }
            if (k < 0 || k >= p->ntex || !p->tex[k] || p->tex[k]->elemLen != 4) return -1;
            t[i] = p->tex[k];
        }
        s->light = ufl(p, 7);
        s->cam = ufl(p, 8);
        s->tex = t[0];
        s->tex2 = t[1];
        if (p->fp == FP_EARTH) {
            s->spec = t[2];
            s->night = t[3];
            s->proj = t[4];
        } else {
            s->proj = t[2];
        }
        break;
    }
    case FP_DEF02: /* colr1light1.cpp:144-148 */
        s->light = ufl(p, 7);
        s->cam = ufl(p, 8);
        break;
    case FP_DEF04: { /* skybox.cpp:122-125: the cube map's index at uniform 2 */
        int t = *uin(p, 2);
        /* get4 reads four bytes per texel from one of six layers
           (samplrcube.cpp:119-127) */
        if (t < 0 || t >= p->ntex || !p->tex[t] || p->tex[t]->layers < 6 || p->tex[t]->elemLen != 4) return -1;
        s->cube = p->tex[t];
        break;
    }
    case FP_DEF03: { /* tex1bump1light1.cpp:170-176: diffuse at 9, bump at 10 */
        int t = *uin(p, 9), b = *uin(p, 10);
        if (t < 0 || t >= p->ntex || !p->tex[t] || b < 0 || b >= p->ntex || !p->tex[b]) return -1;
        s->light = ufl(p, 7);
        s->cam = ufl(p, 8);
        s->tex = p->tex[t];
        s->tex2 = p->tex[b];
        break;
    }
    case FP_LIT3:
    case FP_LIT2: {
        const int* a = uin(p, 9);
        s->light = ufl(p, 7);
        s->cam = ufl(p, 8);
        s->levelsA = a[1] > MAX_LEVELS ? MAX_LEVELS : a[1];
        for (int i = 0; i < s->levelsA; i++) {
            if (a[0] + i < 0 || a[0] + i >= p->ntex || !p->tex[a[0] + i]) return -1;
            s->chainA[i] = level_of(p->tex[a[0] + i]);
        }
        s->lodScale = ufl(p, 12)[0];
        s->bias = ufl(p, 12)[1];
        if (p->fp == FP_LIT2) {
            const int* n = uin(p, 10);
            int sm = *uin(p, 11);
            s->levelsN = n[1] > MAX_LEVELS ? MAX_LEVELS : n[1];
            for (int i = 0; i < s->levelsN; i++) {
                if (n[0] + i < 0 || n[0] + i >= p->ntex || !p->tex[n[0] + i]) return -1;
                s->chainN[i] = level_of(p->tex[n[0] + i]);
                s->chainN[i].width /= 2; /* RGBA16F stored as a 4-byte-element FBO twice as wide */
            }
            if (sm < 0 || sm >= p->ntex || !p->tex[sm]) return -1;
            s->shadow = (const float*)p->tex[sm]->buf;
            s->shadowSize = p->tex[sm]->width;
            s->shadowScan = p->tex[sm]->scanline / 4;
        }
        break;
    }
    default: break;
    }
    return 0;
}

/* PuresoftSampler2D::get4 (samplr2d.cpp:19-25): nearest texel at
   (unsigned)(size * coord + 0.5f), then directRead4 -> clampCoord
   (fbo.cpp:287-291, 552-594); the texel's bytes in memory (BGRA) order. */
static void sample_nearest(const o_fbo* t, const float* tc, float c[4])
{
    int row = (int)sr_f2u((float)t->height * tc[1] + 0.5f);
    int col = (int)sr_f2u((float)t->width * tc[0] + 0.5f);
    const uint8_t* px;
    if (t->wrap) {
        int mr = t->height - 1, mc = t->width - 1;
        row = mr > 0 ? row % mr : 0;
        if (row < 0) row += mr;
        col = mc > 0 ? col % mc : 0;
        if (col < 0) col += mc;
    } else {
        row = sr_clampi(row, t->height);
        col = sr_clampi(col, t->width);
    }
    px = t->buf + (size_t)row * t->scanline + 4 * col;
    for (int k = 0; k < 4; k++) c[k] = (float)px[k];
}

/* The lighting shared by DEF01 and DEF03 (tex1light1.cpp:165-192,
   tex1bump1light1.cpp:212-237) on colour c (BGRA floats), normal n and
   world position wp (all four lanes, as the 4-wide mcemaths ops use them):
   L divided by its length with rcpps, E and H normalised with rsqrtss. */
static void def_lighting(const fp_state* s, float c[4], const float* nrm, const float* wp, uint8_t* bgra)
{
    float L[4], E[4], Hv[4], dist, lambert, spec, r;
    for (int k = 0; k < 4; k++) L[k] = s->light[k] - wp[k];
    dist = sqrtf((L[0] * L[0] + L[1] * L[1]) + (L[2] * L[2] + L[3] * L[3]));
    r = x86_rcp(dist);
    for (int k = 0; k < 4; k++) L[k] = L[k] * r;
    for (int k = 0; k < 4; k++) E[k] = s->cam[k] - wp[k];
    r = norm_scale(E);
    for (int k = 0; k < 4; k++) E[k] = E[k] * r;
    for (int k = 0; k < 4; k++) Hv[k] = E[k] + L[k];
    r = norm_scale(Hv);
    for (int k = 0; k < 4; k++) Hv[k] = Hv[k] * r;
    lambert = (L[0] * nrm[0] + L[1] * nrm[1]) + (L[2] * nrm[2] + L[3] * nrm[3]);
    spec = (Hv[0] * nrm[0] + Hv[1] * nrm[1]) + (Hv[2] * nrm[2] + Hv[3] * nrm[3]);
    spec = spec < 0 ? 0 : spec;
    { /* opt_pow(spec, 50) (proc.h:73-86) */
        float pw = 1.0f, x = spec;
        unsigned n = 50;
        while (n > 0) {
            if (n & 1) pw *= x;
            x *= x;
            n >>= 1;
        }
        spec = pw;
    }
    for (int k = 0; k < 4; k++) c[k] = c[k] + 255.0f * spec;
    for (int k = 0; k < 4; k++) c[k] = c[k] * lambert;
    for (int k = 0; k < 4; k++) { /* clamp_3_4: maxps then minps (vector.cpp:370-383) */
        float v = c[k];
        v = v > 0.0f ? v : 0.0f; /* maxps returns the second operand for NaN */
        v = v < 255.0f ? v : 255.0f;
        c[k] = v;
    }
    bgra[0] = (uint8_t)(int)c[0];
    bgra[1] = (uint8_t)(int)c[1];
    bgra[2] = (uint8_t)(int)c[2];
    bgra[3] = 0;
}

/* FragmentProcessorDEF01::process (tex1light1.cpp:152-193). */
static void fp_def01(const fp_state* s, const float* in, uint8_t* bgra)
{
    const float* nrm = in, * wp = in + 4, * tc = in + 8;
    float c[4];
    sample_nearest(s->tex, tc, c);
    def_lighting(s, c, nrm, wp, bgra);
}

/* FragmentProcessorDEF02::process (colr1light1.cpp:150-190): the
   interpolated vertex colour, then DEF01's lighting. */
static void fp_def02(const fp_state* s, const float* in, uint8_t* bgra)
{
    const float* nrm = in, * wp = in + 4, * col = in + 8;
    float c[4];
    memcpy(c, col, 16);
    def_lighting(s, c, nrm, wp, bgra);
}

/* texcoordFromDirection (samplrcube.cpp:29-97): the face of the major axis
   (ties resolved by the reference's strict comparisons) and its (s, t). */
static int cube_face(const float* d, float* st)
{
    float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    if (ax > ay) {
        if (ax > az) {
            if (d[0] > 0) { st[0] = (-d[2] / ax + 1.0f) / 2.0f; st[1] = (-d[1] / ax + 1.0f) / 2.0f; return 0; }
            st[0] = (d[2] / ax + 1.0f) / 2.0f;
            st[1] = (-d[1] / ax + 1.0f) / 2.0f;
            return 1;
        }
    } else if (!(az > ay)) { /* Y wins; the sign test is on Z (samplrcube.cpp:83) */
        if (d[2] > 0) { st[0] = (d[0] / ay + 1.0f) / 2.0f; st[1] = (d[2] / ay + 1.0f) / 2.0f; return 2; }
        st[0] = (d[0] / ay + 1.0f) / 2.0f;
        st[1] = (-d[2] / ay + 1.0f) / 2.0f;
        return 3;
    }
    /* Z wins */
    if (d[2] > 0) { st[0] = (d[0] / az + 1.0f) / 2.0f; st[1] = (-d[1] / az + 1.0f) / 2.0f; return 4; }
    st[0] = (-d[0] / az + 1.0f) / 2.0f;
    st[1] = (-d[1] / az + 1.0f) / 2.0f;
    return 5;
}

/* PuresoftSamplerCube::get4 (samplrcube.cpp:119-127): row from s times the
   height, column from t times the width (the reference passes S as the
   row), each +0.5 and truncated as unsigned, then directRead4 of the face
   (fbo.cpp:287-291, clampCoord fbo.cpp:552-594). */
static void sample_cube(const o_fbo* t, const float* d, uint8_t* bgra)
{
    float st[2];
    int layer = cube_face(d, st);
    int row = (int)sr_f2u((float)t->height * st[0] + 0.5f);
    int col = (int)sr_f2u((float)t->width * st[1] + 0.5f);
    if (t->wrap) {
        row = sr_wrap(row, t->height);
        col = sr_wrap(col, t->width);
    } else {
        row = sr_clampi(row, t->height);
        col = sr_clampi(col, t->width);
    }
    memcpy(bgra, t->buf + (size_t)t->scanline * t->height * layer + (size_t)row * t->scanline + 4 * col, 4);
}

/* PuresoftSamplerProjection::get (samplrproj.cpp:20-38): the projected
   coordinate divided by its w (mcemaths_div_3_4: times rcpps(w)), then four
   Poisson taps -- row from t plus the disk's x,
   column from s plus the disk's y, each / 500 -- each lowering the factor
   by 0.2 when the stored depth is below the coordinate's z. */
static float sample_proj(const o_fbo* t, const float* proj)
{
    static const float PX[4] = {-0.94201624f, 0.94558609f, -0.094184101f, 0.34495938f};
    static const float PY[4] = {-0.39906216f, -0.76890725f, -0.92938870f, 0.29387760f};
    float tc[4], r = x86_rcp(proj[3]), factor = 1.0f;
    for (int k = 0; k < 4; k++) tc[k] = proj[k] * r;
    for (int i = 0; i < 4; i++) {
        int y = (int)sr_f2u((float)t->height * (tc[1] + PX[i] / 500.0f));
        int x = (int)sr_f2u((float)t->width * (tc[0] + PY[i] / 500.0f));
        float depth;
        if (t->wrap) {
            y = sr_wrap(y, t->height);
            x = sr_wrap(x, t->width);
        } else {
            y = sr_clampi(y, t->height);
            x = sr_clampi(x, t->width);
        }
        memcpy(&depth, t->buf + (size_t)y * t->scanline + 4 * x, 4);
        if (depth < tc[2]) factor -= 0.2f;
    }
    return factor;
}

/* The demo's planet fragment processors (test/testproc.cpp:208-288 FP_Earth,
   299-363 FP_Satellite): DEF03's bump-mapped normal and lighting, the
   specular term scaled by the specular map's red / 255 (Earth), the night
   texel added where lambert < 0.2 (Earth), then the colour times the
   projective shadow factor. */
static void fp_planet(const ps3do* p, const fp_state* s, const float* in, uint8_t* bgra)
{
    const float* tan = in, * bin = in + 4, * nrm = in + 8, * wp = in + 12, * tc = in + 16, * sc = in + 20;
    const int earth = p->fp == FP_EARTH;
    float c[4], night[4] = {0, 0, 0, 0}, bt[4], bn[4], tbn[16], r, shadow, control = 1.0f;
    float L[4], E[4], Hv[4], dist, lambert, spec;
    sample_nearest(s->tex, tc, c);
    if (earth) sample_nearest(s->night, tc, night);
    sample_nearest(s->tex2, tc, bt);
    bn[0] = bt[2];
    bn[1] = bt[1];
    bn[2] = bt[0];
    bn[3] = 0.0f;
    shadow = sample_proj(s->proj, sc);
    if (earth) {
        float st[4];
        sample_nearest(s->spec, tc, st);
        control = st[2] / 255.0f;
    }
    r = x86_rcp(255.0f);  /* mcemaths_div_3_4(bumpNormal, 255.0f) */
    for (int k = 0; k < 4; k++) bn[k] = bn[k] * r;
    for (int k = 0; k < 4; k++) bn[k] = bn[k] * 2.0f;
    for (int k = 0; k < 4; k++) bn[k] = bn[k] - 1.0f;
    memcpy(tbn, tan, 16);
    memcpy(tbn + 4, bin, 16);
    memcpy(tbn + 8, nrm, 16);
    memset(tbn + 12, 0, 16);
    m4v4(bn, tbn, bn);
    r = norm_scale(bn);
    for (int k = 0; k < 4; k++) bn[k] = bn[k] * r;
    for (int k = 0; k < 4; k++) L[k] = s->light[k] - wp[k];
    dist = sqrtf((L[0] * L[0] + L[1] * L[1]) + (L[2] * L[2] + L[3] * L[3]));
    r = x86_rcp(dist);
    for (int k = 0; k < 4; k++) L[k] = L[k] * r;
    for (int k = 0; k < 4; k++) E[k] = s->cam[k] - wp[k];
    r = norm_scale(E);
    for (int k = 0; k < 4; k++) E[k] = E[k] * r;
    for (int k = 0; k < 4; k++) Hv[k] = E[k] + L[k];
    r = norm_scale(Hv);
    for (int k = 0; k < 4; k++) Hv[k] = Hv[k] * r;
    lambert = (L[0] * bn[0] + L[1] * bn[1]) + (L[2] * bn[2] + L[3] * bn[3]);
    spec = (Hv[0] * bn[0] + Hv[1] * bn[1]) + (Hv[2] * bn[2] + Hv[3] * bn[3]);
    spec = spec < 0 ? 0 : spec;
    { /* opt_pow(spec, 50) (proc.h:73-86) */
        float pw = 1.0f, x = spec;
        unsigned n = 50;
        while (n > 0) {
            if (n & 1) pw *= x;
            x *= x;
            n >>= 1;
        }
        spec = pw;
    }
    if (earth) spec *= control;
    for (int k = 0; k < 4; k++) c[k] = c[k] + 255.0f * spec;
    for (int k = 0; k < 4; k++) c[k] = c[k] * lambert;
    if (earth && lambert < 0.2f)
        for (int k = 0; k < 4; k++) c[k] = c[k] + night[k];
    for (int k = 0; k < 4; k++) c[k] = c[k] * shadow;
    for (int k = 0; k < 4; k++) { /* clamp_3_4: maxps then minps */
        float v = c[k];
        v = v > 0.0f ? v : 0.0f;
        v = v < 255.0f ? v : 255.0f;
        c[k] = v;
    }
    bgra[0] = (uint8_t)(int)c[0];
    bgra[1] = (uint8_t)(int)c[1];
    bgra[2] = (uint8_t)(int)c[2];
    bgra[3] = 0;
}

/* cvtps2dq (round to nearest even; NaN and |x| >= 2^31 give INT_MIN), then
   packusdw (int32 -> uint16, saturating) and packuswb (the words read as
   int16 -> uint8, saturating): the byte FP_Cloud writes for lane value x
   (test/testproc.cpp:565-571). */
static uint8_t pack_sse(float x)
{
    int i;
    int w;
    if (x >= -2147483648.0f && x < 2147483648.0f) {
        float r = nearbyintf(x); /* the default rounding mode: to nearest even */
        i = (int)r;
    } else {
        i = INT_MIN;
    }
    w = i < 0 ? 0 : (i > 65535 ? 65535 : i);
    if (w >= 32768) return 0; /* a negative int16 */
    return (uint8_t)(w > 255 ? 255 : w);
}

/* FP_Cloud::process (test/testproc.cpp:534-574): white, alpha the texel's
   red; the three colour lanes times 2 lambert x the projective shadow
   factor (mcemaths_mul_3); packed as above; written through write4. */
static void fp_cloud(const fp_state* s, const float* in, uint8_t* bgra)
{
    const float* nrm = in, * wp = in + 4, * tc = in + 8, * sc = in + 12;
    float t[4], c[4], L[4], dist, r, lambert, f;
    sample_nearest(s->tex, tc, t);
    c[0] = 255.0f;
    c[1] = 255.0f;
    c[2] = 255.0f;
    c[3] = t[2];
    f = sample_proj(s->proj, sc);
    for (int k = 0; k < 4; k++) L[k] = s->light[k] - wp[k];
    dist = sqrtf((L[0] * L[0] + L[1] * L[1]) + (L[2] * L[2] + L[3] * L[3]));
    r = x86_rcp(dist);
    for (int k = 0; k < 4; k++) L[k] = L[k] * r;
    /* E and H are computed by the reference but unused */
    lambert = 2.0f * ((L[0] * nrm[0] + L[1] * nrm[1]) + (L[2] * nrm[2] + L[3] * nrm[3]));
    f = lambert * f;
    c[0] = c[0] * f;
    c[1] = c[1] * f;
    c[2] = c[2] * f;
    for (int k = 0; k < 4; k++) bgra[k] = pack_sse(c[k]);
}

/* The scene viewer's spotlight terms (test2/testproc.cpp:220-238 and
   470-488): L, E, H normalised (rsqrtss), lambert =
   L.n scaled outside the 25-degree cone by cos(yaw - cone)^150, specular =
   (H.n)^exponent (no clamp before the power), both clamped to [0, 1] by
   clamp_3_4 (NaN -> 0).  f[0] lambert, f[1] specular. */

static float opt_powf(float x, unsigned n) /* proc.h:73-86 */
{
    float pw = 1.0f;
    while (n > 0) {
        if (n & 1) pw *= x;
        x *= x;
        n >>= 1;
    }
    return pw;
}

static float clamp01(float v)
{
    v = v > 0.0f ? v : 0.0f; /* maxps: NaN -> the bound */
    return v < 1.0f ? v : 1.0f;
}

static void spot_factors(const fp_state* s, const float* nrm, const float* wp, float f[2])
{
    const float fieldOfLight = 6.283185f * (25.0f / 360.0f); /* test2/testproc.cpp:9 */
    float L[4], E[4], Hv[4], r, yaw;
    for (int k = 0; k < 4; k++) L[k] = s->light[k] - wp[k];
    r = norm_scale(L);
    for (int k = 0; k < 4; k++) L[k] = L[k] * r;
    for (int k = 0; k < 4; k++) E[k] = s->cam[k] - wp[k];
    r = norm_scale(E);
    for (int k = 0; k < 4; k++) E[k] = E[k] * r;
    for (int k = 0; k < 4; k++) Hv[k] = E[k] + L[k];
    r = norm_scale(Hv);
    for (int k = 0; k < 4; k++) Hv[k] = Hv[k] * r;
    f[0] = (L[0] * nrm[0] + L[1] * nrm[1]) + (L[2] * nrm[2] + L[3] * nrm[3]);
    yaw = acosf((L[0] * s->ldir[0] + L[1] * s->ldir[1]) + (L[2] * s->ldir[2] + L[3] * s->ldir[3]));
    f[0] = f[0] * (yaw < fieldOfLight ? 1.0f : opt_powf(cosf(yaw - fieldOfLight), 150));
    f[1] = opt_powf((Hv[0] * nrm[0] + Hv[1] * nrm[1]) + (Hv[2] * nrm[2] + Hv[3] * nrm[3]), s->sexp);
    f[0] = clamp01(f[0]);
    f[1] = clamp01(f[1]);
}

/* FP_SingleColour::process (test2/testproc.cpp:211-261) over (normal, world
   position, shadow coordinate). */
static void fp_single_colour(const fp_state* s, const float* in, uint8_t* bgra)
{
    const float* nrm = in, * wp = in + 4, * sc = in + 8;
    const float shadow = sample_proj(s->proj, sc);
    float f[2], o[4];
    spot_factors(s, nrm, wp, f);
    for (int k = 0; k < 4; k++) {
        float sp = (s->dif[k] * s->scol[k]) * f[1];
        float am = s->dif[k] * s->amb[k];
        o[k] = ((s->dif[k] * f[0] + sp) * shadow + am);
        o[k] = clamp01(o[k]) * 255.0f;
    }
    bgra[0] = (uint8_t)(int)o[0];
    bgra[1] = (uint8_t)(int)o[1];
    bgra[2] = (uint8_t)(int)o[2];
    bgra[3] = 0;
}

/* FP_DiffuseOnly::process (test2/testproc.cpp:458-499) over (normal, world
   position, uv, shadow coordinate). */
static void fp_diffuse_only(const fp_state* s, const float* in, uint8_t* bgra)
{
    const float* nrm = in, * wp = in + 4, * tc = in + 8, * sc = in + 12;
    const float shadow = sample_proj(s->proj, sc);
    float c[4], am[4], f[2], g;
    sample_nearest(s->tex, tc, c);
    for (int k = 0; k < 4; k++) am[k] = c[k] * s->amb[k];
    spot_factors(s, nrm, wp, f);
    g = (f[0] + f[1]) * shadow;
    for (int k = 0; k < 4; k++) {
        float v = c[k] * g + am[k];
        v = v > 0.0f ? v : 0.0f;
        c[k] = v < 255.0f ? v : 255.0f;
    }
    bgra[0] = (uint8_t)(int)c[0];
    bgra[1] = (uint8_t)(int)c[1];
    bgra[2] = (uint8_t)(int)c[2];
    bgra[3] = 0;
}

/* FragmentProcessorDEF03::process (tex1bump1light1.cpp:180-239): the bump
   texel's (r, g, b, 0) / 255 * 2 - 1 on four lanes, through the matrix whose
   columns are the tangent, binormal, normal and 0 (mcemaths_make_tbn,
   matrix.cpp:992-1008), normalised; then DEF01's lighting. */
static void fp_def03(const fp_state* s, const float* in, uint8_t* bgra)
{
    const float* tan = in, * bin = in + 4, * nrm = in + 8, * wp = in + 12, * tc = in + 16;
    float c[4], bt[4], bn[4], tbn[16], r;
    sample_nearest(s->tex, tc, c);
    sample_nearest(s->tex2, tc, bt);
    bn[0] = bt[2];
    bn[1] = bt[1];
    bn[2] = bt[0];
    bn[3] = 0.0f;
    r = x86_rcp(255.0f);  /* mcemaths_div_3_4(bumpNormal, 255.0f) */
    for (int k = 0; k < 4; k++) bn[k] = bn[k] * r;
    for (int k = 0; k < 4; k++) bn[k] = bn[k] * 2.0f;
    for (int k = 0; k < 4; k++) bn[k] = bn[k] - 1.0f;
    memcpy(tbn, tan, 16);
    memcpy(tbn + 4, bin, 16);
    memcpy(tbn + 8, nrm, 16);
    memset(tbn + 12, 0, 16);
    m4v4(bn, tbn, bn);
    r = norm_scale(bn);
    for (int k = 0; k < 4; k++) bn[k] = bn[k] * r;
    def_lighting(s, c, bn, wp, bgra);
}

/* Per-thread error accumulator of the FP32 vs FP64 shading comparison. */
typedef struct {
    double max, sum;
    long long n, over;
} err_acc;

/* The scene shaders' pre-truncation FP32 colour against the FP64 re-shade of
   the same fragment; |difference| per colour channel. */
static void shade_error(const ps3do* p, const fp_state* s, const float* in, err_acc* e)
{
    float pre[3];
    double ref[3];
    uint8_t bgra[4];
    switch (p->fp) {
    case FP_LIT1: {
        sr_level t = level_of(s->tex);
        sr_shade_lit1_pre(&t, s->light, s->cam, in, in + 4, in + 8, pre, bgra);
        srd_shade_lit13(&t, 1, 0, 0.0, s->light, s->cam, in, in + 4, in + 8, ref);
        break;
    }
    case FP_LIT3:
        sr_shade_lit3_pre(s->chainA, s->levelsA, s->lodScale, s->light, s->cam, in, in + 4, in + 8, pre, bgra);
        srd_shade_lit13(s->chainA, s->levelsA, 1, s->lodScale, s->light, s->cam, in, in + 4, in + 8, ref);
        break;
    case FP_LIT2:
        sr_shade_lit2_pre(s->chainA, s->levelsA, s->chainN, s->levelsN, s->shadow, s->shadowSize, s->shadowScan,
                          s->lodScale, s->bias, s->light, s->cam, in, pre, bgra);
        srd_shade_lit2(s->chainA, s->levelsA, s->chainN, s->levelsN, s->shadow, s->shadowSize, s->shadowScan,
                       s->lodScale, s->bias, s->light, s->cam, in, ref);
        break;
    default: return;
    }
    for (int k = 0; k < 3; k++) {
        double d = fabs((double)pre[k] - ref[k]);
        if (d > e->max) e->max = d;
        e->sum += d;
        e->n++;
        if (d >= 1.0) e->over++;
    }
}

/* Returns 1 if the processor wrote colour, 2 if it discarded the fragment
   (FBOBridge::discard, fragthrd.cpp:21-24: no depth write), 0 otherwise. */
static int run_fp(const ps3do* p, const fp_state* s, const float* in, uint8_t* bgra)
{
    switch (p->fp) {
    case FP_DEF01: fp_def01(s, in, bgra); return 1;
    case FP_DEF02: fp_def02(s, in, bgra); return 1;
    case FP_DEF03: fp_def03(s, in, bgra); return 1;
    case FP_DEF04: sample_cube(s->cube, in, bgra); return 1; /* skybox.cpp:127-134 */
    case FP_EARTH:
    case FP_SATELLITE: fp_planet(p, s, in, bgra); return 1;
    case FP_CLOUD: fp_cloud(s, in, bgra); return 1;
    case FP_SINGLECOLOURNL: { /* test2/testproc.cpp:55-70: the diffuse colour x 255, truncated */
        float o[4];
        for (int k = 0; k < 4; k++) o[k] = s->dif[k] * 255.0f;
        bgra[0] = (uint8_t)(int)o[0];
        bgra[1] = (uint8_t)(int)o[1];
        bgra[2] = (uint8_t)(int)o[2];
        bgra[3] = 0;
        return 1;
    }
    case FP_SINGLECOLOUR: fp_single_colour(s, in, bgra); return 1;
    case FP_DIFFUSEONLY: fp_diffuse_only(s, in, bgra); return 1;
    case FP_CLOUDSHADOW: { /* test/testproc.cpp:677-686: discard where the texel's red is below 150 */
        float t[4];
        sample_nearest(s->tex, in, t);
        return t[2] < 150.0f ? 2 : 0;
    }
    case FP_LIT1: {
        sr_level t = level_of(s->tex);
        sr_shade_lit1(&t, s->light, s->cam, in, in + 4, in + 8, bgra);
        return 1;
    }
    case FP_LIT1A: {
        sr_level t = level_of(s->tex);
        return sr_shade_lit1a(&t, s->light, s->cam, in, in + 4, in + 8, bgra) ? 2 : 1;
    }
    case FP_LIT3:
        sr_shade_lit3(s->chainA, s->levelsA, s->lodScale, s->light, s->cam, in, in + 4, in + 8, bgra);
        return 1;
    case FP_LIT2:
        sr_shade_lit2(s->chainA, s->levelsA, s->chainN, s->levelsN, s->shadow, s->shadowSize, s->shadowScan,
                      s->lodScale, s->bias, s->light, s->cam, in, bgra);
        return 1;
    default: return 0; /* FP_DEF05 writes nothing */
    }
}

/* ------------------------------------------------------------- rasteriser */
/* PuresoftRasterizer (rasterizer.h:3-49, rasterizer.cpp). */

typedef struct { float x, y; } v2f;
typedef struct { int left, leftClamped, leftVerts[2], right, rightClamped, rightVerts[2]; } o_row;
typedef struct { float dx, dy, x0, y0; int i0, i1; } o_edge;

typedef struct {
    int W, H, halfW, halfH;
    v2f v[3];
    int firstRow, lastRow;
    o_row* rows;
} o_raster;

static o_edge edge_make(const v2f* v, int a, int b) /* LineSegment, rasterizer.cpp:46-64 */
{
    o_edge e;
    e.x0 = v[a].x;
    e.y0 = v[a].y;
    e.dx = v[b].x - e.x0;
    e.dy = v[b].y - e.y0;
    e.i0 = a;
    e.i1 = b;
    if (fabsf(e.dy) < 0.000001f) e.dy = FLT_MAX;
    return e;
}

static float edge_at(const o_edge* e, float y) { return e->dx * (y - e->y0) / e->dy + e->x0; } /* :66-69 */

static void process_triangle(o_raster* r, const o_edge* L, const o_edge* R, float yMin, float yMax) /* :93-118 */
{
    int iy = yMin < 0 ? 0 : sr_f2i(yMin);
    int last = r->H - 1;
    int iyMax = yMax > (float)last ? last : sr_f2i(yMax);
    if (iy < 0) iy = 0; /* non-finite yMin: see the header note */
    for (; iy <= iyMax; iy++) {
        o_row* row = &r->rows[iy];
        row->left = sr_f2i(edge_at(L, (float)iy) + 0.5f);
        row->leftClamped = row->left < 0 ? 0 : row->left;
        row->right = sr_f2i(edge_at(R, (float)iy) + 0.5f);
        row->rightClamped = row->right >= r->W ? r->W - 1 : row->right;
        row->leftVerts[0] = L->i0;
        row->leftVerts[1] = L->i1;
        row->rightVerts[0] = R->i0;
        row->rightVerts[1] = R->i1;
    }
}

static void push_vertex(o_raster* r, int idx, const float* v) /* :73-90 */
{
    r->v[idx].y = ((float)r->halfH * v[1]) + (float)r->halfH;
    r->v[idx].x = ((float)r->halfW * v[0]) + (float)r->halfW;
    if (0 == idx) r->firstRow = r->lastRow = sr_f2i(r->v[0].y);
    else if (r->v[idx].y > (float)r->lastRow) r->lastRow = sr_f2i(r->v[idx].y);
    else if (r->v[idx].y < (float)r->firstRow) r->firstRow = sr_f2i(r->v[idx].y);
}

static int push_triangle(o_raster* r, const float* p0, const float* p1, const float* p2) /* :142-234 */
{
    const v2f* v = r->v;
    push_vertex(r, 0, p0);
    push_vertex(r, 1, p1);
    push_vertex(r, 2, p2);
    if (!(isfinite(v[0].x) && isfinite(v[0].y) && isfinite(v[1].x) && isfinite(v[1].y) && isfinite(v[2].x) &&
          isfinite(v[2].y)))
        return 0; /* see the header note */
    if (r->firstRow >= r->H || r->lastRow < 0) { r->firstRow = 0; r->lastRow = -1; }
    if (r->firstRow < 0) r->firstRow = 0;
    if (r->lastRow >= r->H) r->lastRow = r->H - 1;
    if (r->firstRow == r->lastRow) return 0;
    if (v[0].y == v[1].y) {
        o_edge a = edge_make(v, 0, 2), b = edge_make(v, 1, 2);
        if (v[0].x < v[1].x) process_triangle(r, &a, &b, (float)r->firstRow, (float)r->lastRow);
        else process_triangle(r, &b, &a, (float)r->firstRow, (float)r->lastRow);
    } else if (v[0].y == v[2].y) {
        o_edge a = edge_make(v, 0, 1), b = edge_make(v, 2, 1);
        if (v[0].x < v[2].x) process_triangle(r, &a, &b, (float)r->firstRow, (float)r->lastRow);
        else process_triangle(r, &b, &a, (float)r->firstRow, (float)r->lastRow);
    } else if (v[1].y == v[2].y) {
        o_edge a = edge_make(v, 1, 0), b = edge_make(v, 2, 0);
        if (v[1].x < v[2].x) process_triangle(r, &a, &b, (float)r->firstRow, (float)r->lastRow);
        else process_triangle(r, &b, &a, (float)r->firstRow, (float)r->lastRow);
    } else {
        int top, bottom, third = 2, t;
        if (v[0].y > v[1].y) { top = 0; bottom = 1; }
        else { top = 1; bottom = 0; }
        if (v[top].y < v[third].y) { t = top; top = third; third = t; }
        else if (v[bottom].y > v[third].y) { t = bottom; bottom = third; third = t; }
        { /* processStandingTriangle (:121-140) */
            o_edge tt = edge_make(v, top, third), tb = edge_make(v, top, bottom), thb = edge_make(v, third, bottom);
            if (edge_at(&tb, v[third].y) > edge_at(&tt, v[third].y)) {
                process_triangle(r, &tt, &tb, v[third].y, v[top].y);
                process_triangle(r, &thb, &tb, v[bottom].y, v[third].y);
            } else {
                process_triangle(r, &tb, &tt, v[third].y, v[top].y);
                process_triangle(r, &tb, &thb, v[bottom].y, v[third].y);
            }
        }
    }
    return 1;
}

/* isBackFace (vertthrd.cpp:56-65): sign of the normalised cross product's z.
   norm_3_4 scales by rsqrtss(|c|^2); the test only depends on that factor
   being finite and positive, which holds exactly when |c|^2 is a finite
   normal number.  With an infinite factor (|c|^2 zero or denormal) the dot
   product is NaN and the face is not culled; with a zero factor (|c|^2
   infinite) it is +-0 and not culled. */
static int is_back_face(const float* v0, const float* v1, const float* v2)
{
    float a[4], b[4], c[4], s;
    for (int k = 0; k < 4; k++) {
        a[k] = v1[k] - v0[k];
        b[k] = v2[k] - v1[k];
    }
    c[0] = a[1] * b[2] - a[2] * b[1]; /* cross_3 shuffles (vector.cpp:114-144) */
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
    c[3] = a[3] * b[3] - a[3] * b[3];
    s = (c[0] * c[0] + c[1] * c[1]) + (c[2] * c[2] + c[3] * c[3]);
    if (!(s >= FLT_MIN && s <= FLT_MAX)) return 0;
    if (!isfinite(c[0]) || !isfinite(c[1]) || !isfinite(c[3])) return 0;
    return c[2] < 0.0f;
}

/* -------------------------------------------------------------- span set-up */

/* lineSegmentlinearInterpolate (interp.cpp:151-160) */
static void line_contrib(const v2f* v, int v1, int v2, float x, float y, float* c)
{
    float dx = v[v1].x - v[v2].x, dy = v[v1].y - v[v2].y;
    c[v1] = fabsf(dx) > fabsf(dy) ? ((x - v[v2].x) / dx) : ((y - v[v2].y) / dy);
    c[v2] = 1.0f - c[v1];
    c[3 - v1 - v2] = 0;
}

/* interpolateStartAndStep (interp.cpp:26-80) */
static void span_setup(const o_raster* r, const o_row* row, int y, const float* rw, const float* pz, int ip, int nv,
                       const float* const* vuser, o_task* t)
{
    float cl[4], cr[4], ccl[4], ccr[4], recip;
    float* start = t->user, * step = t->user + 4 * MAX_VECS;
    int stepCount, skip;
    cl[3] = cr[3] = 0;
    line_contrib(r->v, row->leftVerts[0], row->leftVerts[1], (float)row->left, (float)y, cl);
    line_contrib(r->v, row->rightVerts[0], row->rightVerts[1], (float)row->right, (float)y, cr);
    for (int k = 0; k < 4; k++) {
        ccl[k] = cl[k] * rw[k];
        ccr[k] = cr[k] * rw[k];
    }
    ip_by_contributes(nv, start, vuser, ccl);
    ip_by_contributes(nv, step, vuser, ccr);
    stepCount = row->right - row->left;
    ip_calc_step(nv, step, start, step, stepCount);
    recip = 1.0f / (float)stepCount;
    {
        float m[4];
        for (int k = 0; k < 4; k++) m[k] = ccl[k] * pz[k];
        t->pzStart = hsum4(m);
        for (int k = 0; k < 4; k++) m[k] = ccr[k] * pz[k];
        t->pzStep = hsum4(m);
    }
    t->pzStep = (t->pzStep - t->pzStart) * recip;
    t->cf2Start = hsum4(ccl);
    t->cf2Step = hsum4(ccr);
    t->cf2Step = (t->cf2Step - t->cf2Start) * recip;
    skip = row->leftClamped - row->left;
    if (skip > 0) {
        t->cf2Start += t->cf2Step * (float)skip;
        t->pzStart += t->pzStep * (float)skip;
        ip_step_forward(ip, nv, start, step, skip);
    }
    t->x1 = row->leftClamped;
    t->x2 = row->rightClamped;
    t->y = y;
}

static int push_task(o_tasklist* l, const o_task* t)
{
    if (l->n == l->cap) {
        size_t cap = l->cap ? 2 * l->cap : 1024;
        o_task* q = (o_task*)realloc(l->items, cap * sizeof(o_task));
        if (!q) return -3;
        l->items = q;
        l->cap = cap;
    }
    l->items[l->n++] = *t;
    return 0;
}

/* ------------------------------------------------------- per-pixel loop */

typedef struct {
    ps3do* p;
    fp_state fs;
    int nv;
} draw_ctx;

/* One FBO cursor (PuresoftFBO::WORKRANGE and setCurRow/setCurCol/nextCol,
   fbo.cpp:98-173) for a CLAMP-mode buffer. */
typedef struct {
    uint8_t* rowEntry;
    int col, maxCol, overflow, elemLen;
} o_cursor;

static void cursor_set(o_cursor* c, const o_fbo* f, int row, int col)
{
    int r = sr_clampi(row, f->height); /* the row's overflow flag is overwritten by setCurCol */
    int mem = f->topDown ? f->height - r - 1 : r;
    c->rowEntry = f->buf + (size_t)mem * f->scanline;
    c->maxCol = f->width - 1;
    c->elemLen = f->elemLen;
    c->overflow = (col > c->maxCol || col < 0);
    c->col = sr_clampi(col, f->width);
}

static void cursor_next(o_cursor* c)
{
    if (c->col >= c->maxCol) c->overflow = 1;
    else c->col++;
}

/* fragmentThread's DRAW branch (fragthrd.cpp:160-252) for one task. */
static void run_task(draw_ctx* d, const o_task* t, long long* tested, long long* passed, err_acc* e)
{
    ps3do* p = d->p;
    int nv = d->nv, behav = p->behavior;
    float start[4 * MAX_VECS], step[4 * MAX_VECS], frag[4 * MAX_VECS];
    float cf2 = t->cf2Start, pz = t->pzStart;
    o_cursor cc, dc;
    memcpy(start, t->user, sizeof(float) * 4 * nv);
    memcpy(step, t->user + 4 * MAX_VECS, sizeof(float) * 4 * nv);
    cursor_set(&cc, p->fbos[0], t->y, t->x1);
    cursor_set(&dc, p->depth, t->y, t->x1);
    for (int x = t->x1; x <= t->x2; x++) {
        /* interpolateNextStep (interp.cpp:82-92) */
        float inv = 1.0f / cf2, z, cur;
        cf2 += t->cf2Step;
        for (int i = 0; i < 4 * nv; i++) frag[i] = start[i] * inv;
        ip_step_forward(p->ip, nv, start, step, 1);
        z = pz * inv;
        pz += t->pzStep;
        (*tested)++;
        cur = (behav & BEHAVIOR_TEST_DEPTH) ? *(const float*)(dc.rowEntry + (size_t)dc.col * 4) : 1.0f;
        if (-1.0f < z && (z - cur < -0.0001f)) { /* fragthrd.cpp:227 */
            uint8_t bgra[4];
            int w;
            (*passed)++;
            w = run_fp(p, &d->fs, frag, bgra);
            if (w == 1 && !cc.overflow) {
                uint8_t* dst = cc.rowEntry + (size_t)cc.col * 4;
                /* FBOBridge::write4 blends under ALPHABLEND (fragthrd.cpp:70-81, fbo.cpp:208-229);
                   DEF01 / DEF02 / DEF03 write through FBOBridge::write, which never blends */
                if ((behav & BEHAVIOR_ALPHABLEND) && p->fp != FP_DEF01 && p->fp != FP_DEF02 && p->fp != FP_DEF03)
                    sr_blend4(dst, bgra);
                else memcpy(dst, bgra, 4);
            }
            if (p->errOn) shade_error(p, &d->fs, frag, e);
            if (w != 2 && (behav & BEHAVIOR_UPDATE_DEPTH) && !dc.overflow) memcpy(dc.rowEntry + (size_t)dc.col * 4, &z, 4);
        }
        cursor_next(&cc);
        cursor_next(&dc);
    }
}

static void run_list(draw_ctx* d, int t, long long* tested, long long* passed)
{
    o_tasklist* l = &d->p->lists[t];
    err_acc e = {0.0, 0.0, 0, 0};
    for (size_t i = 0; i < l->n; i++) run_task(d, &l->items[i], tested, passed, &e);
    if (e.n) {
        ps3do* p = d->p;
        if (p->threads > 1) pthread_mutex_lock(&p->mu);
        if (e.max > p->errMax) p->errMax = e.max;
        p->errSum += e.sum;
        p->errN += e.n;
        p->errOver += e.over;
        if (p->threads > 1) pthread_mutex_unlock(&p->mu);
    }
}

static void* worker(void* arg)
{
    ps3do* p = (ps3do*)((void**)arg)[0];
    int idx = (int)(intptr_t)((void**)arg)[1];
    int seen = 0;
    free(arg);
    for (;;) {
        long long tested = 0, passed = 0;
        draw_ctx* d;
        pthread_mutex_lock(&p->mu);
        while (p->gen == seen) pthread_cond_wait(&p->cv, &p->mu);
        seen = p->gen;
        if (p->quit) { pthread_mutex_unlock(&p->mu); return NULL; }
        d = (draw_ctx*)p->cur_draw;
        pthread_mutex_unlock(&p->mu);
        run_list(d, idx, &tested, &passed);
        pthread_mutex_lock(&p->mu);
        p->tested += tested;
        p->passed += passed;
        p->finished++;
        pthread_cond_signal(&p->done);
        pthread_mutex_unlock(&p->mu);
    }
}

/* drawVAO (drawvao.cpp:3-133) */
int ps3do_draw(ps3do* p, int vao)
{
    o_vao* va;
    draw_ctx d;
    o_raster r;
    float rw[4] = {0, 0, 0, 0}, pz[4] = {0, 0, 0, 0};
    float pos[3][4], vuser[3][4 * MAX_VECS];
    const float* vu[3] = {vuser[0], vuser[1], vuser[2]};
    size_t cursor[MAX_VBOS];
    int nv, rc = 0;

    if (!p->vp || !p->ip || !p->fp || vao < 0 || vao >= p->nvao || !p->vaos[vao]) return 0;
    va = p->vaos[vao];
    d.p = p;
    nv = d.nv = ip_vecs(p->ip);
    if (fp_prepare(p, &d.fs)) return -1;
    memset(vuser, 0, sizeof vuser);
    memset(&r, 0, sizeof r);
    r.W = p->W;
    r.H = p->H;
    r.halfW = p->W / 2;
    r.halfH = p->H / 2;
    r.rows = (o_row*)calloc((size_t)p->H, sizeof(o_row));
    if (!r.rows) return -3;
    for (int t = 0; t < p->threads; t++) p->lists[t].n = 0;
    memset(cursor, 0, sizeof cursor);

    for (;;) {
        int done = 0;
        /* processVertices (vertthrd.cpp:14-51) */
        for (int i = 0; i < 3 && !done; i++) {
            const void* in[MAX_VBOS] = {0};
            for (int j = 0; j < MAX_VBOS; j++) {
                o_vbo* b = va->vbo[j];
                if (!b) continue;
                if (cursor[j] >= (size_t)b->count) { done = 1; break; } /* vbo.cpp:69-84 */
                in[j] = b->data + cursor[j] * b->unitBytes;
                cursor[j]++;
            }
            if (done) break;
            run_vp(p, in, pos[i], vuser[i]);
            {
                float rcp = 1.0f / pos[i][3];
                for (int k = 0; k < 4; k++) pos[i][k] = pos[i][k] * rcp; /* mul_3_4 is 4-wide */
                pz[i] = pos[i][2];
                rw[i] = rcp;
            }
        }
        if (done) break;
        if ((p->behavior & BEHAVIOR_FACE_CULLING) && is_back_face(pos[0], pos[1], pos[2])) continue;
        if (pos[0][2] < -1.0f || pos[0][2] > 1.0f) continue; /* drawvao.cpp:51-56 */
        if (pos[1][2] < -1.0f || pos[1][2] > 1.0f) continue;
        if (pos[2][2] < -1.0f || pos[2][2] > 1.0f) continue;
        if (!push_triangle(&r, pos[0], pos[1], pos[2])) continue;
        for (int y = r.firstRow; y <= r.lastRow; y++) {
            const o_row* row = &r.rows[y];
            o_task t;
            if (row->left == row->right) continue; /* drawvao.cpp:72-75 */
            span_setup(&r, row, y, rw, pz, p->ip, nv, vu, &t);
            if (t.x2 >= t.x1) {
                int len = t.x2 - t.x1 + 1, b = 0;
                while (len >>= 1) b++;
                p->spanHist[b]++;
            }
            if ((rc = push_task(&p->lists[y % p->threads], &t)) != 0) goto out;
        }
    }

    if (p->threads > 1) {
        long long tested = 0, passed = 0;
        pthread_mutex_lock(&p->mu);
        p->cur_draw = &d;
        p->finished = 0;
        p->gen++;
        pthread_cond_broadcast(&p->cv);
        pthread_mutex_unlock(&p->mu);
        run_list(&d, 0, &tested, &passed);
        pthread_mutex_lock(&p->mu);
        p->tested += tested;
        p->passed += passed;
        while (p->finished < p->threads - 1) pthread_cond_wait(&p->done, &p->mu);
        pthread_mutex_unlock(&p->mu);
    } else {
        run_list(&d, 0, &p->tested, &p->passed);
    }
out:
    free(r.rows);
    return rc;
}
