// pipeline.cpp -- host runtime behind the C ABI (include/ps3d.h).
//
// The pipeline keeps the reference's object model (PuresoftPipeline,
// src/puresoft3d/pipeline.h:24-156): pools of textures, processors,
// programmes and VAOs addressed by small integer indices, 1024 uniform slots,
// a behaviour word, a depth target and a viewport.  Resources live in device
// memory.  ps3d_draw records a draw with a snapshot of everything the device
// needs; a flush groups consecutive draws into one target into a "pass" and
// launches it (set-up + binning + raster + shade kernels).  Clears that
// precede a pass on the same target are fused into it.
//
// Bin lists are written into buffers sized from the previous frames.  If a
// pass needs more room, its kernels raise a flag and every later kernel of
// the flush does nothing; at the next synchronisation point the runtime grows
// the buffers and re-runs the recorded passes from the one that overflowed.
// Targets are never touched by an aborted pass, so the re-run sees exactly
// the state the first run saw.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <new>
#include <string>
#include <vector>
#include "ps3d.h"
#include "ps3d_internal.h"

namespace ps3d {
int launch_setup(const PassParams& P, cudaStream_t s, int& launches, Prof* pr);
void launch_sort(const PassParams& P, cudaStream_t s, int& launches, Prof* pr);
int radix_passes(int nBins);
int sort_desc_offset(int nTris);
size_t radix_scratch_ints(int sortBlocks, int passes, int nTris);
int selftest_division(unsigned long long pairs, unsigned long long* rcpBad, unsigned long long* divBad);
int selftest_occlusion(unsigned long long cases, unsigned long long* wrong, unsigned long long* occluded);
void launch_raster(const PassParams& P, cudaStream_t s, int& launches, Prof* pr);
void launch_selftest_wait(int* status, const int* flag, int spins, cudaStream_t s);
void launch_shade(const PassParams& P, cudaStream_t s, int& launches, Prof* pr);
void launch_post_add8(uint32_t* row0, int pitch, int width, int height, uint32_t add, const int* status, int seq,
                      cudaStream_t s, int& launches, Prof* pr);
void launch_post_fog(uint32_t* row0, int pitch, int width, int height, const float* depth, int depthScan,
                     uint32_t fog, float nearD, float farD, const int* status, int seq, cudaStream_t s, int& launches,
                     Prof* pr);
void launch_fill_u32(void* base, int width, int height, int pitchElems, uint32_t v, const int* status, int seq,
                     cudaStream_t s, int& launches, Prof* pr);
}  // namespace ps3d

using namespace ps3d;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

}  // namespace

// The same message slot for the other translation units (objx.cpp).
int ps3d::report_error(int code, const char* msg)
{
    g_err = msg;
    return code;
}

namespace {

#define CU(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) return fail(PS3D_ERR_DEVICE, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// The sort's look-back descriptors hold prefixes in 30 bits.
constexpr int kMaxPairs = (1 << 30) - kSortChunk;

// A texture: `layers` images of scanline*height bytes back to back (layer 0
// is the texture itself, 1.. its extra layers; six make a cube map with the
// faces in the reference's LAYER order +x, -x, +y, -y, +z, -z, fbo.h:19).
struct Texture {
    uint8_t* dev = nullptr;
    int width = 0, height = 0, scanline = 0, elemLen = 0, wrap = 0, layers = 1;
    bool alive = false;
};

struct Vbo {
    uint8_t* dev = nullptr;
    int unitBytes = 0, count = 0;
};

struct Vao {
    Vbo* vbo[PS3D_MAX_VBOS] = {};
    bool alive = false;
};

struct Programme {
    int vp = -1, ip = -1, fp = -1;
};

// one recorded command
struct Command {
    enum Kind { DRAW, CLEAR_DEPTH, CLEAR_COLOUR, COPY_COLOUR, POST } kind;
    void* copyDst;    // COPY_COLOUR: destination (device or host) of a rectangle of the colour buffer
    int copyX, copyY, copyW, copyH;  // the rectangle, in pixels from the bottom-left corner
    size_t copyPitch;                // destination bytes per row (rows top-down)
    int depthTarget;  // -1 = default buffer
    int colourTarget; // DRAW, POST: FBO slot 0's texture, -1 = the display (ps3d_set_fbo)
    int vpX, vpY, vpW, vpH;
    float depthValue;
    uint32_t colourValue;
    int postId;                // POST: the post-processor (PP_*), its colour parameter and depth range
    uint32_t postColour;
    float postNear, postFar;
    DrawDesc desc;
    DrawUniforms uni;
};

struct Pass {
    size_t first, last;  // commands [first, last) are its draws
    bool clearDepth = false, clearColour = false;
    float depthValue = 1.0f;
    uint32_t colourValue = 0;
};

// Every device or pinned-host allocation this runtime makes goes through
// dev_malloc / host_malloc and is counted (ps3d_allocation_count).
std::atomic<unsigned long long> g_allocCount{0};

cudaError_t dev_malloc(void** p, size_t bytes)
{
    g_allocCount.fetch_add(1, std::memory_order_relaxed);
    return cudaMalloc(p, bytes);
}

cudaError_t host_malloc(void** p, size_t bytes)
{
    g_allocCount.fetch_add(1, std::memory_order_relaxed);
    return cudaMallocHost(p, bytes);
}

// Device buffers that grow.  While a captured graph exists its kernels hold
// the old addresses, so a buffer being replaced is retired (freed when the
// last graph goes) instead of freed.
thread_local std::vector<void*>* g_retire = nullptr;

template <class T> bool dev_alloc(T*& p, size_t& cap, size_t need)
{
    if (need <= cap && p) return true;
    size_t n = std::max(need, cap + cap / 2);
    if (p) {
        if (g_retire) g_retire->push_back(p);
        else cudaFree(p);
    }
    p = nullptr;
    cap = 0;
    if (dev_malloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return false;
    cap = n;
    return true;
}

// mcemaths_transform_m4m4 (matrix.cpp:588-690): column c of d = l * (column c of r),
// each lane ((l0*r0 + l4*r1) + l8*r2) + l12*r3.  Built with -ffp-contract=off.
void m4m4(float* d, const float* l, const float* r)
{
    for (int c = 0; c < 4; c++) {
        const float* v = r + 4 * c;
        for (int i = 0; i < 4; i++) {
            float a = v[0] * l[i];
            float b = v[1] * l[4 + i];
            float s = a + b;
            float e = v[2] * l[8 + i];
            s = s + e;
            float f = v[3] * l[12 + i];
            d[4 * c + i] = s + f;
        }
    }
}

constexpr int kSlots = 2;
constexpr int kMaxOverlapPasses = 16;  // launches with more passes run on one stream

// Device scratch of one pass.
struct Scratch {
    TriRaster* tris = nullptr; size_t trisCap = 0;
    float* vary = nullptr; size_t varyCap = 0;
    int* pairKey = nullptr; size_t pairKeyCap = 0;
    int* pairTri = nullptr; size_t pairTriCap = 0;
    int* binTri = nullptr; size_t binTriCap = 0;
    int* radix = nullptr; size_t radixCap = 0;
    int* keyB = nullptr; size_t keyBCap = 0;
    int* binStart = nullptr; size_t binStartCap = 0;
    int2* shadeList = nullptr; size_t shadeListCap = 0;
    SpanItem* spans = nullptr; size_t spansCap = 0;
    DrawDesc* draws = nullptr; size_t drawsCap = 0;
    DrawUniforms* unis = nullptr; size_t unisCap = 0;
    int* slotStatus = nullptr;  // 16 ints, allocated with the pipeline
};

// Cross-stream hazards within one launch: per buffer (colour buffer, depth
// targets, by device address) the event of its last writer and of the
// readers since; and the previous pass's emit.
struct Hazard {
    cudaEvent_t write = nullptr;
    std::vector<cudaEvent_t> reads;
};
struct Tracker {
    std::vector<std::pair<const void*, Hazard>> res;
    cudaEvent_t lastEmit = nullptr;
    Hazard& at(const void* key)
    {
        for (auto& r : res)
            if (r.first == key) return r.second;
        res.emplace_back(key, Hazard());
        return res.back().second;
    }
    void clear()
    {
        res.clear();
        lastEmit = nullptr;
    }
};

}  // namespace

struct ps3d_pipeline {
    int device = -1;     // the CUDA device current when the pipeline was created
    int devW, devH;      // device size (colour buffer, default depth)
    int W, H;            // viewport size
    int vpX = 0, vpY = 0;  // viewport origin in the targets (ps3d_set_viewport_rect)
    int behavior = B_UPDATE_DEPTH | B_TEST_DEPTH | B_FACE_CULLING;  // pipeline.cpp:34
    int depthTarget = -1;
    int fbo[PS3D_MAX_FBOS];  // setFBO's slots: a texture index, -1 = none (slot 0: the display)
    int binW = 32;
    int rasterBlocks = 0;
    int cullSpans = 1;
    int rowSplit = 1;
    int warpBins = 0;
    int spanItems = 0;
    int lazyVary = 0;
    bool countFrags = false;
    cudaStream_t stream = nullptr;
    bool ownStream = false;

    uint8_t* colour = nullptr;      // BGRA8, top-down
    float* defDepth = nullptr;
    int defDepthScan = 0;           // floats

    std::vector<Texture> tex;
    std::vector<int> procs;         // processor class ids, 0 = destroyed
    std::vector<Programme> progs;
    std::vector<Vao> vaos;
    std::vector<std::vector<uint8_t>> uni = std::vector<std::vector<uint8_t>>(PS3D_MAX_UNIFORMS);
    int vp = 0, ip = 0, fp = 0;     // processor class ids in use

    std::vector<Command> pending;   // recorded, not launched
    std::vector<Command> launched;  // launched since the last verification
    std::vector<size_t> passStart;  // per launched pass: index in `launched` to re-run it from

    // Passes alternate between two scratch slots, each with its own stream:
    // pass k uses slot k % 2, so a pass can run while the previous one does
    // (a slot is reused only by the pass two later, on the same stream).
    // Work between passes and the cross-pass hazards go through `stream`.
    Scratch scr[kSlots];
    cudaStream_t gs[kSlots] = {};
    int* status = nullptr;
    int pairCap = 1 << 18;
    bool oneStream = false;              // this launch has at most one pass: everything on `stream`
    std::vector<cudaEvent_t> evPool;     // events for cross-stream ordering, reused per launch
    size_t evUsed = 0;
    Tracker trk;
    std::vector<const void*> depthTargetPtrs;  // textures ever bound as depth targets

    ps3d_stats_t stats = {};
    Prof prof;
    cudaEvent_t timerA = nullptr, timerB = nullptr;
    void* scrub = nullptr;
    size_t scrubBytes = 0;
    ps3d_cmdbuf* recording = nullptr;   // command buffer being recorded
    int liveGraphs = 0;
    std::vector<void*> retired;          // scratch replaced while graphs hold it
    std::vector<ps3d_cmdbuf*> cmdbufs;
    ps3d_cmdbuf* graphUnverified = nullptr;  // graph launched since the last verification
    const DrawDesc* cbDraws = nullptr;   // set while a command buffer's graph is captured
    const DrawUniforms* cbUnis = nullptr;
    const std::vector<size_t>* cbOffsets = nullptr;
};

// A recorded command sequence (ps3d_cmdbuf_*): its draw descriptors live in
// its own device buffers, and after its first submission it replays as a
// CUDA graph.
struct ps3d_cmdbuf {
    std::vector<Command> cmds;
    std::vector<size_t> passOffset;      // per pass of its plan: first descriptor index
    std::vector<DrawDesc> hDraws;        // host copies (pinned) of all passes' descriptors
    std::vector<DrawUniforms> hUnis;
    DrawDesc* dDraws = nullptr;
    DrawUniforms* dUnis = nullptr;
    DrawDesc* pinDraws = nullptr;        // pinned staging for per-submission uploads
    DrawUniforms* pinUnis = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool stale = false;
};

namespace {

int required_vary(int ip)
{
    switch (ip) {
    case IP_DEF01: return 9;
    case IP_DEF02: return 11;  // normal xyzw, worldPos xyz, colour xyzw
    case IP_DEF03: return 17;
    case IP_DEF04: return 3;   // direction xyz
    case IP_PLANET: return 21; // tangent, binormal, normal xyzw, worldPos xyz, uv, shadow coordinate xyzw
    case IP_CLOUD: return 13;  // normal xyzw, worldPos xyz, uv, shadow coordinate xyzw
    case IP_CLOUDSHADOW: return 2;  // uv
    case IP_SINGLECOLOUR: return 11;  // normal xyzw, worldPos xyz, shadow coordinate xyzw
    case IP_DIFFUSEONLY: return 13;   // normal xyzw, worldPos xyz, uv, shadow coordinate xyzw
    case IP_LIT2: return 16;
    default: return 0;
    }
}

int fp_needs(int fp)
{
    switch (fp) {
    case FP_DEF01: case FP_LIT1: case FP_LIT1A: case FP_LIT3: return IP_DEF01;
    case FP_LIT2: return IP_LIT2;
    case FP_DEF02: return IP_DEF02;
    case FP_DEF03: return IP_DEF03;
    case FP_DEF04: return IP_DEF04;
    case FP_EARTH: case FP_SATELLITE: return IP_PLANET;
    case FP_CLOUD: return IP_CLOUD;
    case FP_CLOUDSHADOW: return IP_CLOUDSHADOW;
    case FP_SINGLECOLOUR: return IP_SINGLECOLOUR;
    case FP_DIFFUSEONLY: return IP_DIFFUSEONLY;
    default: return 0;
    }
}

int vp_gives(int vp)
{
    switch (vp) {
    case VP_DEF01: return IP_DEF01;
    case VP_LIT2: return IP_LIT2;
    case VP_DEF02: return IP_DEF02;
    case VP_DEF03: return IP_DEF03;
    case VP_DEF04: return IP_DEF04;
    case VP_PLANET: return IP_PLANET;
    case VP_CLOUD: return IP_CLOUD;
    case VP_CLOUDSHADOW: return IP_CLOUDSHADOW;
    case VP_SINGLECOLOUR: return IP_SINGLECOLOUR;
    case VP_DIFFUSEONLY: return IP_DIFFUSEONLY;
    default: return 0;
    }
}

bool known_processor(int id)
{
    switch (id) {
    case VP_DEF01: case IP_DEF01: case FP_DEF01: case VP_DEF05: case IP_DEF05: case FP_DEF05:
    case VP_SHADOW: case FP_LIT1: case FP_LIT1A: case FP_LIT3: case VP_LIT2: case IP_LIT2: case FP_LIT2:
    case VP_DEF02: case IP_DEF02: case FP_DEF02: case VP_DEF03: case IP_DEF03: case FP_DEF03:
    case VP_DEF04: case IP_DEF04: case FP_DEF04:
    case VP_PLANET: case IP_PLANET: case FP_EARTH: case FP_SATELLITE:
    case VP_CLOUD: case IP_CLOUD: case FP_CLOUD: case VP_CLOUDSHADOW: case IP_CLOUDSHADOW: case FP_CLOUDSHADOW:
    case VP_POSITIONONLY: case IP_NULL: case FP_SINGLECOLOURNL: case VP_SINGLECOLOUR: case IP_SINGLECOLOUR:
    case FP_SINGLECOLOUR: case VP_DIFFUSEONLY: case IP_DIFFUSEONLY: case FP_DIFFUSEONLY: case VP_SHADOW2: case FP_NULL:
        return true;
    }
    return false;
}

bool tex_ok(const ps3d_pipeline* p, int i) { return i >= 0 && i < (int)p->tex.size() && p->tex[i].alive; }

TexLevel level_of(const Texture& t)
{
    TexLevel l;
    l.base = t.dev;
    l.width = t.width;
    l.height = t.height;
    l.scanline = t.scanline;
    l.wrap = t.wrap;
    return l;
}

const float* ufl(const ps3d_pipeline* p, int slot, size_t floats)
{
    const auto& u = p->uni[slot];
    return u.size() >= floats * 4 ? (const float*)u.data() : nullptr;
}

const int* uint_(const ps3d_pipeline* p, int slot, size_t ints)
{
    const auto& u = p->uni[slot];
    return u.size() >= ints * 4 ? (const int*)u.data() : nullptr;
}

int chain_of(const ps3d_pipeline* p, int slot, TexLevel* out, int& levels, bool half)
{
    const int* c = uint_(p, slot, 2);
    if (!c) return fail(PS3D_ERR_INVALID, "uniform %d must hold {first texture, levels}", slot);
    if (c[1] < 1 || c[1] > kMaxLevels) return fail(PS3D_ERR_INVALID, "uniform %d: %d levels", slot, c[1]);
    for (int i = 0; i < c[1]; i++) {
        if (!tex_ok(p, c[0] + i)) return fail(PS3D_ERR_RANGE, "uniform %d: texture %d", slot, c[0] + i);
        out[i] = level_of(p->tex[c[0] + i]);
        if (half) out[i].width /= 2;
    }
    levels = c[1];
    return 0;
}

// Snapshot of the uniforms the programme's processors read (their
// preprocess(), reference drawvao.cpp:18-20).
int snapshot_uniforms(const ps3d_pipeline* p, DrawUniforms& U)
{
    memset(&U, 0, sizeof U);
    auto need = [&](int slot, float* dst, size_t n) -> int {
        const float* f = ufl(p, slot, n);
        if (!f) return fail(PS3D_ERR_INVALID, "uniform %d is not set (the processor reads %zu floats)", slot, n);
        memcpy(dst, f, n * 4);
        return 0;
    };
    int rc;
    switch (p->vp) {
    case VP_DEF01:  // tex1light1.cpp:15-20
    case VP_DEF02:  // colr1light1.cpp:15-20
    case VP_DEF03:  // tex1bump1light1.cpp:15-20
        if ((rc = need(3, U.PV, 16)) || (rc = need(4, U.M, 16)) || (rc = need(5, U.Mrot, 16))) return rc;
        break;
    case VP_PLANET:  // test/testproc.cpp:29-35: DEF03's matrices and the shadow projection at 16
    case VP_CLOUD:   // test/testproc.cpp:384-390: the same four
        if ((rc = need(3, U.PV, 16)) || (rc = need(4, U.M, 16)) || (rc = need(5, U.Mrot, 16)) ||
            (rc = need(16, U.LPV, 16)))
            return rc;
        break;
    case VP_DEF04: {  // skybox.cpp:17-21, 34-37: the view's inverse rotation, the
                      // transposed view matrix with its last column zeroed
        float V[16];
        if ((rc = need(1, V, 16))) return rc;
        for (int c = 0; c < 4; c++)
            for (int r = 0; r < 4; r++) U.Vrot[4 * c + r] = c < 3 ? V[4 * r + c] : 0.0f;
        break;
    }
    case VP_POSITIONONLY:  // test2/testproc.cpp:13-16: PVM at 5
    case VP_SHADOW2:       // test2/testproc.cpp:502-505
        if ((rc = need(5, U.PVM, 16))) return rc;
        break;
    case VP_SINGLECOLOUR:  // test2/testproc.cpp:80-86: M 0, MR 1, PVM 5, shadow projection 6
    case VP_DIFFUSEONLY:   // test2/testproc.cpp:294-301 (its PV at 4 is read by nothing)
        if ((rc = need(0, U.M, 16)) || (rc = need(1, U.Mrot, 16)) || (rc = need(5, U.PVM, 16)) ||
            (rc = need(6, U.LPV, 16)))
            return rc;
        break;
    case VP_DEF05:
    case VP_CLOUDSHADOW:  // test/testproc.cpp:588-593
    case VP_SHADOW:
        if ((rc = need(3, U.PV, 16)) || (rc = need(4, U.M, 16))) return rc;
        m4m4(U.PVM, U.PV, U.M);
        break;
    case VP_LIT2:
        if ((rc = need(3, U.PV, 16)) || (rc = need(4, U.M, 16)) || (rc = need(5, U.Mrot, 16)) ||
            (rc = need(6, U.LPV, 16)))
            return rc;
        break;
    }
    switch (p->fp) {
    case FP_DEF02:  // colr1light1.cpp:144-148
        if ((rc = need(7, U.light, 4)) || (rc = need(8, U.cam, 4))) return rc;
        break;
    case FP_EARTH:       // test/testproc.cpp:197-206: diffuse 9, bump 10, specular 11, night 12, shadow 15
    case FP_SATELLITE: {  // test/testproc.cpp:290-297: diffuse 9, bump 10, shadow 15
        if ((rc = need(7, U.light, 4)) || (rc = need(8, U.cam, 4))) return rc;
        const int earthSlots[5] = {9, 10, 11, 12, 15}, satSlots[3] = {9, 10, 15};
        const int* slots = p->fp == FP_EARTH ? earthSlots : satSlots;
        const int n = p->fp == FP_EARTH ? 5 : 3;
        TexLevel lv[5];
        for (int i = 0; i < n; i++) {
            const int* t = uint_(p, slots[i], 1);
            if (!t) return fail(PS3D_ERR_INVALID, "uniform %d (texture index) is not set", slots[i]);
            if (!tex_ok(p, *t)) return fail(PS3D_ERR_RANGE, "uniform %d: texture %d", slots[i], *t);
            if (p->tex[*t].elemLen != 4) return fail(PS3D_ERR_INVALID, "texture %d: 4-byte texels expected", *t);
            lv[i] = level_of(p->tex[*t]);
        }
        U.tex = lv[0];
        U.tex2 = lv[1];
        for (int i = 2; i < n; i++) U.ptex[i - 2] = lv[i];
        break;
    }
    case FP_SINGLECOLOURNL:  // test2/testproc.cpp:49-53
        if ((rc = need(31, U.dif, 4))) return rc;
        break;
    case FP_SINGLECOLOUR:  // test2/testproc.cpp:199-209: lights 20-22, shadow map 23, colours 30-33
    case FP_DIFFUSEONLY: {  // test2/testproc.cpp:447-456: the same without 31 / 32; diffuse texture 40
        float e;
        if ((rc = need(20, U.light, 4)) || (rc = need(21, U.ldir, 4)) || (rc = need(22, U.cam, 4)) ||
            (rc = need(30, U.amb, 4)) || (rc = need(33, &e, 1)))
            return rc;
        if (p->fp == FP_SINGLECOLOUR && ((rc = need(31, U.dif, 4)) || (rc = need(32, U.scol, 4)))) return rc;
        U.sexp = (unsigned)e;  // (unsigned int)*m_specularExponent
        const int slots[2] = {23, 40};
        for (int i = 0; i < (p->fp == FP_DIFFUSEONLY ? 2 : 1); i++) {
            const int* t = uint_(p, slots[i], 1);
            if (!t) return fail(PS3D_ERR_INVALID, "uniform %d (texture index) is not set", slots[i]);
            if (!tex_ok(p, *t)) return fail(PS3D_ERR_RANGE, "uniform %d: texture %d", slots[i], *t);
            if (p->tex[*t].elemLen != 4) return fail(PS3D_ERR_INVALID, "texture %d: 4-byte texels expected", *t);
            (i ? U.tex : U.ptex[0]) = level_of(p->tex[*t]);
        }
        break;
    }
    case FP_CLOUD:          // test/testproc.cpp:526-532: diffuse 9, shadow 15
    case FP_CLOUDSHADOW: {  // test/testproc.cpp:672-675: the cloud texture at 9
        if (p->fp == FP_CLOUD && ((rc = need(7, U.light, 4)) || (rc = need(8, U.cam, 4)))) return rc;
        const int slots[2] = {9, 15};
        for (int i = 0; i < (p->fp == FP_CLOUD ? 2 : 1); i++) {
            const int* t = uint_(p, slots[i], 1);
            if (!t) return fail(PS3D_ERR_INVALID, "uniform %d (texture index) is not set", slots[i]);
            if (!tex_ok(p, *t)) return fail(PS3D_ERR_RANGE, "uniform %d: texture %d", slots[i], *t);
            if (p->tex[*t].elemLen != 4) return fail(PS3D_ERR_INVALID, "texture %d: 4-byte texels expected", *t);
            (i ? U.ptex[0] : U.tex) = level_of(p->tex[*t]);
        }
        break;
    }
    case FP_DEF04: {  // skybox.cpp:122-125: the cube map's index at uniform 2
        const int* t = uint_(p, 2, 1);
        if (!t) return fail(PS3D_ERR_INVALID, "uniform 2 (cube map index) is not set");
        if (!tex_ok(p, *t)) return fail(PS3D_ERR_RANGE, "uniform 2: texture %d", *t);
        const Texture& c = p->tex[*t];
        // get4 reads a 4-byte texel from one of six layers (samplrcube.cpp:119-127)
        if (c.elemLen != 4 || c.layers < 6)
            return fail(PS3D_ERR_INVALID, "texture %d is not a BGRA8 cube map (6 layers)", *t);
        U.tex = level_of(c);
        U.layerBytes = (long long)c.scanline * c.height;
        break;
    }
    case FP_DEF01:
    case FP_DEF03:
    case FP_LIT1:
    case FP_LIT1A: {
        if ((rc = need(7, U.light, 4)) || (rc = need(8, U.cam, 4))) return rc;
        const int* t = uint_(p, 9, 1);
        if (!t) return fail(PS3D_ERR_INVALID, "uniform 9 (texture index) is not set");
        if (!tex_ok(p, *t)) return fail(PS3D_ERR_RANGE, "uniform 9: texture %d", *t);
        if (p->tex[*t].elemLen != 4) return fail(PS3D_ERR_INVALID, "texture %d is not BGRA8", *t);
        U.tex = level_of(p->tex[*t]);
        if (p->fp == FP_DEF03) {  // tex1bump1light1.cpp:170-176: the bump map at 10
            const int* b = uint_(p, 10, 1);
            if (!b) return fail(PS3D_ERR_INVALID, "uniform 10 (bump texture index) is not set");
            if (!tex_ok(p, *b)) return fail(PS3D_ERR_RANGE, "uniform 10: texture %d", *b);
            if (p->tex[*b].elemLen != 4) return fail(PS3D_ERR_INVALID, "texture %d is not BGRA8", *b);
            U.tex2 = level_of(p->tex[*b]);
        }
        break;
    }
    case FP_LIT3:
        if ((rc = need(7, U.light, 4)) || (rc = need(8, U.cam, 4)) || (rc = need(12, U.params, 4))) return rc;
        if ((rc = chain_of(p, 9, U.albedo, U.albedoLevels, false))) return rc;
        break;
    case FP_LIT2: {
        if ((rc = need(7, U.light, 4)) || (rc = need(8, U.cam, 4)) || (rc = need(12, U.params, 4))) return rc;
        if ((rc = chain_of(p, 9, U.albedo, U.albedoLevels, false))) return rc;
        if ((rc = chain_of(p, 10, U.normal, U.normalLevels, true))) return rc;
        const int* s = uint_(p, 11, 1);
        if (!s || !tex_ok(p, *s)) return fail(PS3D_ERR_RANGE, "uniform 11: shadow map");
        const Texture& t = p->tex[*s];
        if (t.elemLen != 4 || t.width != t.height) return fail(PS3D_ERR_INVALID, "shadow map must be square FP32");
        U.shadow = (const float*)t.dev;
        U.shadowSize = t.width;
        U.shadowScan = t.scanline / 4;
        break;
    }
    }
    return 0;
}

int ensure_scratch(ps3d_pipeline* p, Scratch& x, int nTris, int nvMax, int W, int H, int binsX, int binsY,
                   bool colour, bool spanItems)
{
    size_t nBins = (size_t)binsX * binsY;
    int sortBlocks = (p->pairCap + kSortChunk - 1) / kSortChunk;
    bool ok = dev_alloc(x.tris, x.trisCap, nTris) && dev_alloc(x.vary, x.varyCap, (size_t)nTris * 3 * std::max(nvMax, 1)) &&
              dev_alloc(x.pairKey, x.pairKeyCap, p->pairCap) && dev_alloc(x.pairTri, x.pairTriCap, p->pairCap) &&
              dev_alloc(x.keyB, x.keyBCap, p->pairCap) && dev_alloc(x.binTri, x.binTriCap, p->pairCap) &&
              dev_alloc(x.radix, x.radixCap, radix_scratch_ints(sortBlocks, radix_passes((int)nBins), nTris)) &&
              dev_alloc(x.binStart, x.binStartCap, (2 + (size_t)kItemsPerBin) * nBins);
    if (ok && colour) ok = dev_alloc(x.shadeList, x.shadeListCap, (size_t)W * H);
    if (ok && spanItems) ok = dev_alloc(x.spans, x.spansCap, p->pairCap);
    if (!ok) return fail(PS3D_ERR_NOMEM, "device scratch allocation failed");
    return 0;
}

struct Target {
    float* depth;
    int scan, w, h;
};

int depth_target(ps3d_pipeline* p, int idx, Target& t)
{
    if (idx == -1) {
        t.depth = p->defDepth;
        t.scan = p->defDepthScan;
        t.w = p->devW;
        t.h = p->devH;
        return 0;
    }
    if (!tex_ok(p, idx)) return fail(PS3D_ERR_RANGE, "depth target %d was destroyed", idx);
    const Texture& x = p->tex[idx];
    t.depth = (float*)x.dev;
    t.scan = x.scanline / 4;
    t.w = x.width;
    t.h = x.height;
    return 0;
}

// The colour target a command recorded (FBO slot 0): the display, rows
// top-down, or a texture, rows bottom-up; `key` is its address for the
// cross-stream hazards.
struct ColourTarget {
    uint32_t* row0;  // pixel row 0
    int pitch;       // pixels from row y to row y + 1 (negative for the display)
    int w, h;
    const void* key;
    bool display;
};

int colour_target(ps3d_pipeline* p, int idx, ColourTarget& c)
{
    if (idx < 0) {
        c.row0 = (uint32_t*)p->colour + (size_t)(p->devH - 1) * p->devW;
        c.pitch = -p->devW;
        c.w = p->devW;
        c.h = p->devH;
        c.key = p->colour;
        c.display = true;
        return 0;
    }
    if (!tex_ok(p, idx)) return fail(PS3D_ERR_RANGE, "FBO texture %d was destroyed", idx);
    const Texture& x = p->tex[idx];
    c.row0 = (uint32_t*)x.dev;
    c.pitch = x.scanline / 4;
    c.w = x.width;
    c.h = x.height;
    c.key = x.dev;
    c.display = false;
    return 0;
}

// ---- cross-stream ordering (see Tracker)
cudaEvent_t next_event(ps3d_pipeline* p)
{
    if (p->evUsed == p->evPool.size()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        p->evPool.push_back(e);
    }
    return p->evPool[p->evUsed++];
}

int mark(ps3d_pipeline* p, cudaStream_t s, cudaEvent_t& e)
{
    e = nullptr;
    if (p->oneStream) return 0;  // one stream orders everything
    e = next_event(p);
    if (!e) return fail(PS3D_ERR_DEVICE, "cudaEventCreate failed");
    CU(cudaEventRecord(e, s));
    return 0;
}

int wait_event(cudaStream_t s, cudaEvent_t e)
{
    if (e) CU(cudaStreamWaitEvent(s, e, 0));
    return 0;
}

// Before an operation on stream s writes `key`: after its last writer and readers.
int before_write(ps3d_pipeline* p, cudaStream_t s, const void* key)
{
    Hazard& h = p->trk.at(key);
    int rc = wait_event(s, h.write);
    for (cudaEvent_t e : h.reads)
        if (!rc) rc = wait_event(s, e);
    return rc;
}

int before_read(ps3d_pipeline* p, cudaStream_t s, const void* key) { return wait_event(s, p->trk.at(key).write); }

void wrote(ps3d_pipeline* p, const void* key, cudaEvent_t e)
{
    Hazard& h = p->trk.at(key);
    h.write = e;
    h.reads.clear();
}

void read_by(ps3d_pipeline* p, const void* key, cudaEvent_t e) { p->trk.at(key).reads.push_back(e); }

// The index the next pass gets.
int next_seq(const ps3d_pipeline* p) { return (int)p->passStart.size(); }
// The sequence number of a fill or post-process between passes: it is skipped
// once a pass before it has failed (the replay starts at or before that pass
// and runs it then) and runs whatever happens to the passes after it.
int gap_seq(const ps3d_pipeline* p) { return next_seq(p) - 1; }

int fill_depth(ps3d_pipeline* p, int target, float v)
{
    Target t;
    int rc = depth_target(p, target, t);
    if (rc) return rc;
    uint32_t bits;
    memcpy(&bits, &v, 4);
    if ((rc = before_write(p, p->stream, t.depth))) return rc;
    int launches = 0;
    launch_fill_u32(t.depth, t.scan, t.h, t.scan, bits, p->status, gap_seq(p), p->stream, launches, &p->prof);
    p->stats.kernel_launches += launches;
    cudaEvent_t e;
    if ((rc = mark(p, p->stream, e))) return rc;
    wrote(p, t.depth, e);
    return 0;
}

int fill_colour(ps3d_pipeline* p, uint32_t v)
{
    int rc = before_write(p, p->stream, p->colour);
    if (rc) return rc;
    int launches = 0;
    launch_fill_u32(p->colour, p->devW, p->devH, p->devW, v, p->status, gap_seq(p), p->stream, launches, &p->prof);
    p->stats.kernel_launches += launches;
    cudaEvent_t e;
    if ((rc = mark(p, p->stream, e))) return rc;
    wrote(p, p->colour, e);
    return 0;
}

// The same on the pipeline's stream alone, for the single-stream
// no-allocation path (no events).
int fill_depth_plain(ps3d_pipeline* p, int target, float v)
{
    Target t;
    int rc = depth_target(p, target, t);
    if (rc) return rc;
    uint32_t bits;
    memcpy(&bits, &v, 4);
    int launches = 0;
    launch_fill_u32(t.depth, t.scan, t.h, t.scan, bits, p->status, gap_seq(p), p->stream, launches, &p->prof);
    p->stats.kernel_launches += launches;
    return 0;
}

int fill_colour_plain(ps3d_pipeline* p, uint32_t v)
{
    int launches = 0;
    launch_fill_u32(p->colour, p->devW, p->devH, p->devW, v, p->status, gap_seq(p), p->stream, launches, &p->prof);
    p->stats.kernel_launches += launches;
    return 0;
}

int post_process(ps3d_pipeline* p, const Command& c, bool tracked);

int copy_colour_plain(ps3d_pipeline* p, const Command& c)
{
    if (c.kind == Command::POST) return post_process(p, c, false);
    const uint8_t* src = p->colour + ((size_t)(p->devH - c.copyY - c.copyH) * p->devW + c.copyX) * 4;
    CU(cudaMemcpy2DAsync(c.copyDst, c.copyPitch, src, (size_t)p->devW * 4, (size_t)c.copyW * 4, c.copyH,
                         cudaMemcpyDefault, p->stream));
    return 0;
}

// The draws of a pass as device descriptors: triangle bases are running
// sums, so a pass's triangles are numbered in submission order.
// A pass is shaded forward (every passing fragment, in order, in the raster)
// when a draw blends or its fragment processor may discard (a depth-only
// draw whose processor discards included).
bool pass_forward(const DrawDesc* dd, size_t n)
{
    for (size_t i = 0; i < n; i++)
        if (((dd[i].flags & F_COLOUR) && ((dd[i].flags & B_ALPHABLEND) || dd[i].fp == FP_LIT1A)) ||
            (dd[i].flags & F_FRAGMENT))
            return true;
    return false;
}

// The fragment processor shared by every colour-writing draw, else 0.
int pass_fp(const DrawDesc* dd, size_t n)
{
    int fp = -1;
    for (size_t i = 0; i < n; i++) {
        const DrawDesc& d = dd[i];
        if (!(d.flags & F_COLOUR)) continue;
        if (fp == -1) fp = d.fp;
        else if (fp != d.fp) return 0;
    }
    return fp < 0 ? 0 : fp;
}

int pass_vp(const DrawDesc* dd, size_t n)
{
    int vp = -1;
    for (size_t i = 0; i < n; i++) {
        const DrawDesc& d = dd[i];
        if (!(d.flags & F_COLOUR)) continue;
        if (vp == -1) vp = d.vp;
        else if (vp != d.vp) return 0;
    }
    return vp < 0 ? 0 : vp;
}

void pass_descriptors(const std::vector<Command>& cmds, const Pass& ps, std::vector<DrawDesc>& dd,
                      std::vector<DrawUniforms>& uu, int& nTris, int& nvMax, bool& anyColour)
{
    for (size_t i = ps.first; i < ps.last; i++) {
        DrawDesc d = cmds[i].desc;
        if (d.triCount == 0) continue;
        d.triBase = nTris;
        d.uni = (int)uu.size();
        nTris += d.triCount;
        nvMax = std::max(nvMax, d.nv);
        anyColour |= (d.flags & F_COLOUR) != 0;
        dd.push_back(d);
        uu.push_back(cmds[i].uni);
    }
}

// The textures a pass's shaders sample that are also depth targets (and so
// may be written by passes of the same launch).
void sampled_targets(const ps3d_pipeline* p, const std::vector<DrawUniforms>& uu, std::vector<const void*>& out)
{
    if (p->depthTargetPtrs.empty()) return;
    auto add = [&](const void* ptr) {
        if (!ptr) return;
        if (std::find(p->depthTargetPtrs.begin(), p->depthTargetPtrs.end(), ptr) == p->depthTargetPtrs.end()) return;
        if (std::find(out.begin(), out.end(), ptr) == out.end()) out.push_back(ptr);
    };
    for (const DrawUniforms& u : uu) {
        add(u.tex.base);
        add(u.tex2.base);
        for (int k = 0; k < 3; k++) add(u.ptex[k].base);
        for (int k = 0; k < u.albedoLevels && k < kMaxLevels; k++) add(u.albedo[k].base);
        for (int k = 0; k < u.normalLevels && k < kMaxLevels; k++) add(u.normal[k].base);
        add(u.shadow);
    }
}

// One pass on its slot's stream: set-up and pair counts, the emit and the
// sort; the raster, after every earlier pass has emitted (so that it sees
// their overflows) and after the last writer and readers of its depth target
// (and of the colour buffer when it clears colour); the shade,
// after the last writer and readers of the colour buffer and the last writers
// of the depth targets it samples.
int run_pass(ps3d_pipeline* p, const std::vector<Command>& cmds, const Pass& ps, size_t replayFrom)
{
    const int seq = next_seq(p);
    p->passStart.push_back(replayFrom);
    const Command& c0 = cmds[ps.first];
    Target tg;
    int rc = depth_target(p, c0.depthTarget, tg);
    if (rc) return rc;
    int W = tg.w, H = tg.h;  // bins cover the depth target; each draw has its viewport rectangle
    std::vector<DrawDesc> dd;
    std::vector<DrawUniforms> uu;
    int nTris = 0, nvMax = 0;
    bool anyColour = false;
    pass_descriptors(cmds, ps, dd, uu, nTris, nvMax, anyColour);
    if (nTris == 0) {
        if (ps.clearDepth && (rc = fill_depth(p, c0.depthTarget, ps.depthValue))) return rc;
        if (ps.clearColour && (rc = fill_colour(p, ps.colourValue))) return rc;
        return 0;
    }
    g_retire = p->liveGraphs ? &p->retired : nullptr;
    const int slot = seq % kSlots;
    Scratch& x = p->scr[slot];
    cudaStream_t s = p->oneStream ? p->stream : p->gs[slot];
    const bool forward = pass_forward(dd.data(), dd.size());
    if (forward) nvMax = forward_vary(nvMax);
    int binW = forward ? 16 : p->binW;  // forward passes run with 16-column bins
    int binsX = (W + binW - 1) / binW, binsY = (H + kBinH - 1) / kBinH;
    if (radix_passes(binsX * binsY) > kRadixMaxPasses) return fail(PS3D_ERR_RANGE, "target too large for the bin sort");
    const bool spanItems = p->spanItems && !forward;  // a forward pass shades from its triangles' records
    if ((rc = ensure_scratch(p, x, nTris, nvMax, W, H, binsX, binsY, anyColour, spanItems))) return rc;
    const DrawDesc* devDraws;
    const DrawUniforms* devUnis;
    if (p->cbOffsets) {  // capturing a command buffer: its descriptors are already on the device
        size_t off = (*p->cbOffsets)[seq];
        devDraws = p->cbDraws + off;
        devUnis = p->cbUnis + off;
    } else {
        if (!dev_alloc(x.draws, x.drawsCap, dd.size()) || !dev_alloc(x.unis, x.unisCap, uu.size()))
            return fail(PS3D_ERR_NOMEM, "device allocation for draw descriptors failed");
        // pageable sources: each copy returns once its source has been read
        CU(cudaMemcpyAsync(x.draws, dd.data(), dd.size() * sizeof(DrawDesc), cudaMemcpyHostToDevice, s));
        CU(cudaMemcpyAsync(x.unis, uu.data(), uu.size() * sizeof(DrawUniforms), cudaMemcpyHostToDevice, s));
        p->stats.upload_bytes += dd.size() * sizeof(DrawDesc) + uu.size() * sizeof(DrawUniforms);
        devDraws = x.draws;
        devUnis = x.unis;
    }

    // A clear fuses into the pass when the pass covers the whole buffer.
    bool fuseDepth = ps.clearDepth && tg.w == W && tg.h == H && tg.scan == W;
    // clearColour clears the display (pipeline.cpp:340-343): fused only into
    // a pass that draws into the display
    ColourTarget ct;
    if ((rc = colour_target(p, c0.colourTarget, ct))) return rc;
    bool fuseColour = ps.clearColour && ct.display && p->devW == W && p->devH == H;
    if (ps.clearDepth && !fuseDepth && (rc = fill_depth(p, c0.depthTarget, ps.depthValue))) return rc;
    if (ps.clearColour && !fuseColour && (rc = fill_colour(p, ps.colourValue))) return rc;

    PassParams P;
    memset(&P, 0, sizeof P);
    P.W = W;
    P.H = H;
    P.binW = binW;
    P.rasterBlocks = p->rasterBlocks;
    P.cullSpans = p->cullSpans;
    P.rowSplit = p->rowSplit;
    P.warpBins = p->warpBins;
    P.spanItems = spanItems;
    P.spans = spanItems ? x.spans : nullptr;
    P.passFp = pass_fp(dd.data(), dd.size());
    P.passVp = pass_vp(dd.data(), dd.size());
    P.forward = forward;
    P.binsX = binsX;
    P.binsY = binsY;
    P.nTris = nTris;
    P.nDraws = (int)dd.size();
    P.draws = devDraws;
    P.unis = devUnis;
    P.tris = x.tris;
    P.vary = x.vary;
    P.nvMax = std::max(nvMax, 1);
    P.anyVary = nvMax > 0;
    P.lazyVary = p->lazyVary && !forward && nvMax > 0;
    P.pairKey = x.pairKey;
    P.pairTri = x.pairTri;
    P.pairCap = p->pairCap;
    P.sortBlocks = (p->pairCap + kSortChunk - 1) / kSortChunk;
    P.radixPasses = radix_passes(binsX * binsY);
    P.radix = x.radix;
    P.sortDescOff = sort_desc_offset(nTris);
    P.keyB = x.keyB;
    P.binStart = x.binStart;
    P.binItems = x.binStart + 2 * (size_t)binsX * binsY;
    P.binTri = x.binTri;
    P.sortedTri = (P.radixPasses & 1) ? x.binTri : x.pairTri;
    P.status = p->status;
    P.slotStatus = x.slotStatus;
    P.depth = tg.depth;
    P.depthScan = tg.scan;
    P.depthW = tg.w;
    P.depthH = tg.h;
    P.shadeList = x.shadeList;
    P.colourRow0 = ct.row0;
    P.colourPitch = ct.pitch;
    P.colourW = ct.w;
    P.colourH = ct.h;
    P.clearDepth = fuseDepth;
    P.clearColour = fuseColour;
    P.anyColour = anyColour;
    P.countFrags = p->countFrags;
    P.depthClearValue = fuseDepth ? ps.depthValue : 1.0f;
    P.colourClearValue = ps.colourValue;
    P.passSeq = seq;
    int launches = 0;
    cudaEvent_t e;
    if (launch_setup(P, s, launches, &p->prof)) return fail(PS3D_ERR_DEVICE, "memset of the sort scratch failed");
    launch_sort(P, s, launches, &p->prof);
    // "this pass and every earlier one have emitted": the raster must see
    // their overflows (the mark after the wait carries the chain on)
    if ((rc = wait_event(s, p->trk.lastEmit))) return rc;
    if ((rc = mark(p, s, e))) return rc;
    p->trk.lastEmit = e;
    // a forward pass shades in the raster: it reads and writes the colour
    // buffer and samples its textures there
    const bool rasterColour = fuseColour || (forward && anyColour);
    std::vector<const void*> sampled;
    if (anyColour || forward) sampled_targets(p, uu, sampled);
    if ((rc = before_write(p, s, tg.depth))) return rc;
    if (rasterColour && (rc = before_write(p, s, ct.key))) return rc;
    if (forward)
        for (const void* t : sampled)
            if ((rc = before_read(p, s, t))) return rc;
    launch_raster(P, s, launches, &p->prof);
    if ((rc = mark(p, s, e))) return rc;
    wrote(p, tg.depth, e);
    if (rasterColour) wrote(p, ct.key, e);
    if (forward)
        for (const void* t : sampled) read_by(p, t, e);
    if (anyColour && !forward) {
        if ((rc = before_write(p, s, ct.key))) return rc;
        for (const void* t : sampled)
            if ((rc = before_read(p, s, t))) return rc;
        launch_shade(P, s, launches, &p->prof);
        if ((rc = mark(p, s, e))) return rc;
        wrote(p, ct.key, e);
        for (const void* t : sampled) read_by(p, t, e);
    }
    CU(cudaGetLastError());
    p->stats.kernel_launches += launches;
    p->stats.batches++;
    p->stats.triangles += nTris;
    return 0;
}

// Splits cmds[from..] into passes (each run of draws into one target, with
// the clears in front of it) and hands them to `onPass`; clears that cannot
// fuse go to `onFill` (target -3 = colour).
template <class PassFn, class FillFn, class CopyFn>
int plan_commands(const std::vector<Command>& cmds, size_t from, PassFn onPass, FillFn onFill, CopyFn onCopy)
{
    size_t i = from, n = cmds.size();
    int rc;
    while (i < n) {
        Pass ps;
        size_t j = i;
        int depthClearTarget = -2;
        for (; j < n && cmds[j].kind != Command::DRAW; j++) {
            if (cmds[j].kind == Command::COPY_COLOUR || cmds[j].kind == Command::POST) {
                // in order: clears gathered so far first
                if (ps.clearDepth && (rc = onFill(depthClearTarget, ps.depthValue, 0u))) return rc;
                if (ps.clearColour && (rc = onFill(-3, 0.0f, ps.colourValue))) return rc;
                ps.clearDepth = ps.clearColour = false;
                if ((rc = onCopy(cmds[j]))) return rc;
                // a post-process is not idempotent: a replay of the next pass starts after it
                if (cmds[j].kind == Command::POST) i = j + 1;
                continue;
            }
            if (cmds[j].kind == Command::CLEAR_DEPTH) {
                if (ps.clearDepth && depthClearTarget != cmds[j].depthTarget &&
                    (rc = onFill(depthClearTarget, ps.depthValue, 0u)))
                    return rc;
                ps.clearDepth = true;
                ps.depthValue = cmds[j].depthValue;
                depthClearTarget = cmds[j].depthTarget;
            } else {
                ps.clearColour = true;
                ps.colourValue = cmds[j].colourValue;
            }
        }
        if (j == n) {
            if (ps.clearDepth && (rc = onFill(depthClearTarget, ps.depthValue, 0u))) return rc;
            if (ps.clearColour && (rc = onFill(-3, 0.0f, ps.colourValue))) return rc;
            break;
        }
        size_t k = j;
        while (k < n && cmds[k].kind == Command::DRAW && cmds[k].depthTarget == cmds[j].depthTarget &&
               cmds[k].colourTarget == cmds[j].colourTarget)
            k++;
        if (ps.clearDepth && depthClearTarget != cmds[j].depthTarget) {
            if ((rc = onFill(depthClearTarget, ps.depthValue, 0u))) return rc;
            ps.clearDepth = false;
        }
        ps.first = j;
        ps.last = k;
        if ((rc = onPass(ps, i))) return rc;
        i = k;
    }
    return 0;
}

// A recorded post-process (PuresoftPipeline::postProcess, post.cpp:3-19):
// one kernel over the colour buffer (and, for PP_FOG, the depth buffer
// current when it was recorded), after the colour buffer's last writer and
// readers, the depth buffer's last writer and every earlier pass's emit (so
// that it sees whether one of them failed).  `tracked` = false on the
// single-stream no-allocation path.
int post_process(ps3d_pipeline* p, const Command& c, bool tracked)
{
    Target t = {};
    ColourTarget ct;
    int rc = colour_target(p, c.colourTarget, ct);
    if (rc) return rc;
    if (c.postId == PP_FOG) {
        if ((rc = depth_target(p, c.depthTarget, t))) return rc;
        if (t.w < ct.w || t.h < ct.h || t.scan < ct.w)
            return fail(PS3D_ERR_INVALID, "the fog post-process needs a depth buffer of at least %dx%d", ct.w, ct.h);
    }
    if (tracked) {
        if ((rc = wait_event(p->stream, p->trk.lastEmit)) || (rc = before_write(p, p->stream, ct.key))) return rc;
        if (t.depth && (rc = before_read(p, p->stream, t.depth))) return rc;
    }
    int launches = 0;
    if (c.postId == PP_ADD8)
        launch_post_add8(ct.row0, ct.pitch, ct.w, ct.h, c.postColour, p->status, gap_seq(p), p->stream, launches,
                         &p->prof);
    else
        launch_post_fog(ct.row0, ct.pitch, ct.w, ct.h, t.depth, t.scan, c.postColour, c.postNear, c.postFar,
                        p->status, gap_seq(p), p->stream, launches, &p->prof);
    CU(cudaGetLastError());
    p->stats.kernel_launches += launches;
    if (tracked) {
        cudaEvent_t e;
        if ((rc = mark(p, p->stream, e))) return rc;
        wrote(p, ct.key, e);
        if (t.depth) read_by(p, t.depth, e);
    }
    return 0;
}

// A recorded colour read-out: the rectangle's rows top-down (memory row
// H-1-y of the display layout) into dst, copyPitch bytes apart.
int copy_colour(ps3d_pipeline* p, const Command& c)
{
    if (c.kind == Command::POST) return post_process(p, c, true);
    const uint8_t* src = p->colour + ((size_t)(p->devH - c.copyY - c.copyH) * p->devW + c.copyX) * 4;
    int rc = before_read(p, p->stream, p->colour);
    if (rc) return rc;
    CU(cudaMemcpy2DAsync(c.copyDst, c.copyPitch, src, (size_t)p->devW * 4, (size_t)c.copyW * 4, c.copyH,
                         cudaMemcpyDefault, p->stream));
    cudaEvent_t e;
    if ((rc = mark(p, p->stream, e))) return rc;
    read_by(p, p->colour, e);
    return 0;
}

// A launch forks the pass streams from the pipeline's stream and joins them
// back at the end, so that everything before it precedes it and the
// pipeline's stream sees all of it complete.
int launch_cmds_inner(ps3d_pipeline* p, const std::vector<Command>& cmds, size_t from);

int launch_cmds(ps3d_pipeline* p, const std::vector<Command>& cmds, size_t from)
{
    p->evUsed = 0;
    p->trk.clear();
    int passes = 0;
    plan_commands(
        cmds, from, [&](const Pass&, size_t) { return ++passes, 0; }, [&](int, float, uint32_t) { return 0; },
        [&](const Command&) { return 0; });
    // Two streams pay off for a few large passes (a shadow pass and a lit
    // pass); for many small passes the events cost more than the overlap
    // gains, and graphs of them instantiate slowly.
    // while profiling, passes run one after another, so that each kernel's
    // events time that kernel alone
    p->oneStream = passes <= 1 || passes > kMaxOverlapPasses || p->prof.on;
    if (p->oneStream) return launch_cmds_inner(p, cmds, from);
    cudaEvent_t fork;
    int rc = mark(p, p->stream, fork);
    for (int k = 0; k < kSlots && !rc; k++) rc = wait_event(p->gs[k], fork);
    if (rc) return rc;
    int rc2 = launch_cmds_inner(p, cmds, from);
    for (int k = 0; k < kSlots; k++) {  // join even after an error, so no work is left outside the stream
        cudaEvent_t j;
        if ((rc = mark(p, p->gs[k], j)) || (rc = wait_event(p->stream, j))) return rc;
    }
    return rc2;
}

int launch_cmds_inner(ps3d_pipeline* p, const std::vector<Command>& cmds, size_t from)
{
    return plan_commands(
        cmds, from, [&](const Pass& ps, size_t start) { return run_pass(p, cmds, ps, start); },
        [&](int target, float v, uint32_t c) { return target == -3 ? fill_colour(p, c) : fill_depth(p, target, v); },
        [&](const Command& c) { return copy_colour(p, c); });
}

int launch_range(ps3d_pipeline* p, size_t from) { return launch_cmds(p, p->launched, from); }

int do_flush(ps3d_pipeline* p)
{
    if (p->pending.empty()) return 0;
    size_t from = p->launched.size();
    p->launched.insert(p->launched.end(), p->pending.begin(), p->pending.end());
    p->pending.clear();
    return launch_range(p, from);
}

// Clears the failure words: flags and most pairs needed to 0, the first
// failed pass to kNoPass.
int reset_flags(ps3d_pipeline* p)
{
    CU(cudaMemsetAsync(p->status, 0, 3 * sizeof(int), p->stream));
    CU(cudaMemsetAsync(p->status + kFirstFailed, 0x7f, sizeof(int), p->stream));
    return 0;
}

// Waits for the stream.  If a pass ran out of bin-list room it recorded
// itself as the first failed pass (the lowest such); it and every pass after
// it did nothing, while the passes before it completed.  The buffers grow and
// the commands are re-run from that pass (including the clears in front of
// it, which are idempotent).
int do_finish(ps3d_pipeline* p)
{
    int rc = do_flush(p);
    if (rc) return rc;
    for (int attempt = 0; attempt < 8; attempt++) {
        CU(cudaStreamSynchronize(p->stream));
        int st[4];
        CU(cudaMemcpy(st, p->status, sizeof st, cudaMemcpyDeviceToHost));
        if (!st[0]) {
            p->launched.clear();
            p->passStart.clear();
            p->graphUnverified = nullptr;
            return 0;
        }
        if (st[0] & 2) {
            if ((rc = reset_flags(p))) return rc;
            p->launched.clear();
            p->passStart.clear();
            p->graphUnverified = nullptr;
            return fail(PS3D_ERR_TIMEOUT, "a device-side wait of the bin sort expired; the frame is incomplete");
        }
        if (p->launched.empty() && p->graphUnverified) {
            // a graph launch outgrew the room its first submission verified
            if ((rc = reset_flags(p))) return rc;
            ps3d_cmdbuf* cb = p->graphUnverified;
            p->graphUnverified = nullptr;
            cb->stale = true;
            return fail(PS3D_ERR_NOMEM, "a command buffer outgrew its bin lists; record it again");
        }
        int seq = st[3];
        if (seq < 0 || seq >= (int)p->passStart.size()) return fail(PS3D_ERR_DEVICE, "bad overflow record");
        if (st[1] > kMaxPairs) return fail(PS3D_ERR_NOMEM, "a pass needs %d bin pairs (at most %d)", st[1], kMaxPairs);
        p->pairCap = (int)std::min<long long>(std::max<long long>((long long)p->pairCap * 2, (long long)st[1] * 5 / 4 + 1024),
                                              kMaxPairs);
        if ((rc = reset_flags(p))) return rc;
        p->stats.replays++;
        size_t from = p->passStart[seq];
        p->passStart.resize(seq);
        if ((rc = launch_range(p, from))) return rc;
    }
    return fail(PS3D_ERR_NOMEM, "bin lists did not fit after growing the buffers");
}

}  // namespace

extern "C" {

const char* ps3d_last_error(void) { return g_err.c_str(); }

int ps3d_pipeline_create(int width, int height, void* stream, ps3d_pipeline** out)
{
    if (!out || width <= 0 || height <= 0) return fail(PS3D_ERR_INVALID, "bad pipeline size");
    ps3d_pipeline* p = new (std::nothrow) ps3d_pipeline();
    if (!p) return fail(PS3D_ERR_NOMEM, "host allocation failed");
    p->devW = p->W = width;
    p->devH = p->H = height;
    for (int& f : p->fbo) f = -1;  // setFBO(0, NULL) in the constructor (pipeline.cpp:49)
    if (cudaGetDevice(&p->device) != cudaSuccess) {
        delete p;
        return fail(PS3D_ERR_DEVICE, "cudaGetDevice failed");
    }
    if (const char* cap = getenv("PS3D_PAIR_CAP")) {
        long v = atol(cap);
        if (v >= 32 && v <= kMaxPairs) p->pairCap = (int)v;
    }
    if (const char* bw = getenv("PS3D_BIN_W")) {
        int v = atoi(bw);
        if (v == 8 || v == 16 || v == 32) p->binW = v;
    }
    if (stream) p->stream = (cudaStream_t)stream;
    else {
        if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete p;
            return fail(PS3D_ERR_DEVICE, "cudaStreamCreate failed");
        }
        p->ownStream = true;
    }
    p->defDepthScan = (int)(width / 4.0f + 0.5f) * 4;  // pipeline.cpp:31
    if (p->defDepthScan < width) p->defDepthScan = (width + 3) / 4 * 4;
    bool ok = dev_malloc((void**)&p->colour, (size_t)width * 4 * height) == cudaSuccess &&
              dev_malloc((void**)&p->defDepth, (size_t)p->defDepthScan * 4 * height) == cudaSuccess &&
              dev_malloc((void**)&p->status, 64 * sizeof(int)) == cudaSuccess;
    for (int k = 0; k < kSlots && ok; k++) {
        p->scr[k].slotStatus = p->status + 16 * (k + 1);
        ok = cudaStreamCreateWithFlags(&p->gs[k], cudaStreamNonBlocking) == cudaSuccess;
    }
    if (!ok) {
        ps3d_pipeline_destroy(p);
        return fail(PS3D_ERR_NOMEM, "device allocation failed");
    }
    cudaMemsetAsync(p->colour, 0, (size_t)width * 4 * height, p->stream);
    cudaMemsetAsync(p->defDepth, 0, (size_t)p->defDepthScan * 4 * height, p->stream);
    cudaMemsetAsync(p->status, 0, 64 * sizeof(int), p->stream);
    reset_flags(p);
    *out = p;
    return 0;
}

int ps3d_pipeline_destroy(ps3d_pipeline* p)
{
    if (!p) return 0;
    if (p->stream) cudaStreamSynchronize(p->stream);
    while (!p->cmdbufs.empty()) ps3d_cmdbuf_destroy(p, p->cmdbufs.back());
    for (void* r : p->retired) cudaFree(r);
    for (auto& m : p->prof.marks) {
        cudaEventDestroy(m.a);
        cudaEventDestroy(m.b);
    }
    for (auto e : p->prof.pool) cudaEventDestroy(e);
    if (p->scrub) cudaFree(p->scrub);
    if (p->timerA) cudaEventDestroy(p->timerA);
    if (p->timerB) cudaEventDestroy(p->timerB);
    for (auto& t : p->tex)
        if (t.alive) cudaFree(t.dev);
    for (auto& v : p->vaos)
        for (auto* b : v.vbo)
            if (b) {
                cudaFree(b->dev);
                delete b;
            }
    for (int k = 0; k < kSlots; k++) {
        Scratch& x = p->scr[k];
        void* sb[] = {x.tris, x.vary, x.pairKey, x.pairTri, x.keyB, x.binTri, x.radix, x.binStart, x.shadeList,
                      x.spans, x.draws, x.unis};
        for (void* b : sb)
            if (b) cudaFree(b);
        if (p->gs[k]) {
            cudaStreamSynchronize(p->gs[k]);
            cudaStreamDestroy(p->gs[k]);
        }
    }
    for (cudaEvent_t e : p->evPool) cudaEventDestroy(e);
    void* bufs[] = {p->colour, p->defDepth, p->status};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (p->ownStream && p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return 0;
}

static int texture_create(ps3d_pipeline* p, int width, int height, int scanline, int elemLen, const void* pixels,
                          int wrap, int extraLayers, cudaMemcpyKind kind)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (elemLen != 1 && elemLen != 4) return fail(PS3D_ERR_INVALID, "elemLen must be 1 or 4 (fbo.cpp:21-24)");
    if (width <= 0 || height <= 0 || scanline < width * elemLen) return fail(PS3D_ERR_INVALID, "bad texture size");
    // fbo.cpp:62-72 throws out_of_range above LAYER_MAX; LAYER_MAX itself
    // would index one past the reference's layer array, so 5 is the most
    if (extraLayers < 0 || extraLayers > 5) return fail(PS3D_ERR_RANGE, "extraLayers %d (0..5)", extraLayers);
    size_t slot = 0;
    for (; slot < p->tex.size(); slot++)
        if (!p->tex[slot].alive) break;
    if (slot == p->tex.size()) p->tex.emplace_back();
    Texture t;
    t.width = width;
    t.height = height;
    t.scanline = scanline;
    t.elemLen = elemLen;
    t.wrap = wrap ? 1 : 0;
    t.layers = 1 + extraLayers;
    size_t bytes = (size_t)scanline * height;
    size_t all = bytes * t.layers;
    if (dev_malloc((void**)&t.dev, (all + 15) / 16 * 16) != cudaSuccess)
        return fail(PS3D_ERR_NOMEM, "texture allocation of %zu bytes failed", all);
    // tex.cpp:20-23: the pixels fill the default layer; extra layers start zeroed
    if (pixels) {
        CU(cudaMemcpyAsync(t.dev, pixels, bytes, kind, p->stream));
        if (all > bytes) CU(cudaMemsetAsync(t.dev + bytes, 0, all - bytes, p->stream));
    } else {
        CU(cudaMemsetAsync(t.dev, 0, all, p->stream));
    }
    t.alive = true;
    p->tex[slot] = t;
    return (int)slot;
}

int ps3d_texture_create(ps3d_pipeline* p, int width, int height, int scanline, int elemLen, const void* pixels,
                        int wrap)
{
    return ps3d_texture_create_layers(p, width, height, scanline, elemLen, pixels, wrap, 0);
}

int ps3d_texture_create_layers(ps3d_pipeline* p, int width, int height, int scanline, int elemLen,
                               const void* pixels, int wrap, int extraLayers)
{
    int rc = texture_create(p, width, height, scanline, elemLen, pixels, wrap, extraLayers, cudaMemcpyHostToDevice);
    if (rc >= 0 && pixels && p) cudaStreamSynchronize(p->stream);  // the caller may free its pixels on return
    return rc;
}

int ps3d_texture_create_device(ps3d_pipeline* p, int width, int height, int scanline, int elemLen,
                               const void* devPixels, int wrap)
{
    return texture_create(p, width, height, scanline, elemLen, devPixels, wrap, 0, cudaMemcpyDeviceToDevice);
}

int ps3d_texture_write_layer(ps3d_pipeline* p, int idx, int layer, const void* pixels, size_t bytes)
{
    if (!p || !pixels) return fail(PS3D_ERR_INVALID, "null argument");
    if (!tex_ok(p, idx)) return fail(PS3D_ERR_RANGE, "texture %d", idx);
    const Texture& t = p->tex[idx];
    if (layer < 0 || layer >= t.layers) return fail(PS3D_ERR_RANGE, "texture %d has no layer %d", idx, layer);
    int rc = do_finish(p);  // passes still sampling the texture finish first
    if (rc) return rc;
    size_t n = std::min(bytes, (size_t)t.scanline * t.height);
    CU(cudaMemcpyAsync(t.dev + (size_t)t.scanline * t.height * layer, pixels, n, cudaMemcpyHostToDevice, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return 0;
}

int ps3d_texture_read_layer(ps3d_pipeline* p, int idx, int layer, void* out, size_t bytes)
{
    if (!p || !out) return fail(PS3D_ERR_INVALID, "null argument");
    if (!tex_ok(p, idx)) return fail(PS3D_ERR_RANGE, "texture %d", idx);
    const Texture& t = p->tex[idx];
    if (layer < 0 || layer >= t.layers) return fail(PS3D_ERR_RANGE, "texture %d has no layer %d", idx, layer);
    int rc = do_finish(p);
    if (rc) return rc;
    size_t n = std::min(bytes, (size_t)t.scanline * t.height);
    CU(cudaMemcpyAsync(out, t.dev + (size_t)t.scanline * t.height * layer, n, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return 0;
}

int ps3d_texture_destroy(ps3d_pipeline* p, int idx)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (idx < 0 || idx >= (int)p->tex.size()) return fail(PS3D_ERR_RANGE, "texture %d", idx);
    if (!p->tex[idx].alive) return 0;
    int rc = do_finish(p);
    if (rc) return rc;
    if (p->depthTarget == idx) p->depthTarget = -1;
    for (int& f : p->fbo)
        if (f == idx) f = -1;  // slot 0 falls back to the display
    for (auto* cb : p->cmdbufs) cb->stale = true;
    cudaFree(p->tex[idx].dev);
    p->tex[idx] = Texture();
    return 0;
}

int ps3d_texture_read(ps3d_pipeline* p, int idx, void* out, size_t bytes)
{
    return ps3d_texture_read_layer(p, idx, 0, out, bytes);
}

int ps3d_texture_device_ptr(ps3d_pipeline* p, int idx, void** out)
{
    if (!p || !out) return fail(PS3D_ERR_INVALID, "null argument");
    if (!tex_ok(p, idx)) return fail(PS3D_ERR_RANGE, "texture %d", idx);
    *out = p->tex[idx].dev;
    return 0;
}

int ps3d_processor_add(ps3d_pipeline* p, int id)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (!known_processor(id)) return fail(PS3D_ERR_INVALID, "unknown processor class 0x%04x", id);
    size_t slot = 0;
    for (; slot < p->procs.size(); slot++)
        if (!p->procs[slot]) break;
    if (slot == p->procs.size()) p->procs.push_back(0);
    p->procs[slot] = id;
    return (int)slot;
}

int ps3d_processor_destroy(ps3d_pipeline* p, int idx)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (idx < 0 || idx >= (int)p->procs.size()) return fail(PS3D_ERR_RANGE, "processor %d", idx);
    int id = p->procs[idx];
    if (!id) return 0;
    // prog.cpp:32-37: a processor in use is unbound
    if (p->vp == id) p->vp = 0;
    if (p->ip == id) p->ip = 0;
    if (p->fp == id) p->fp = 0;
    p->procs[idx] = 0;
    return 0;
}

int ps3d_programme_create(ps3d_pipeline* p, int vid, int iid, int fid)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    int n = (int)p->procs.size();
    if (vid < 0 || vid >= n) return fail(PS3D_ERR_RANGE, "createProgramme, vid");
    if (iid < 0 || iid >= n) return fail(PS3D_ERR_RANGE, "createProgramme, iid");
    if (fid < 0 || fid >= n) return fail(PS3D_ERR_RANGE, "createProgramme, fid");
    int v = p->procs[vid], i = p->procs[iid], f = p->procs[fid];
    if ((i & 0xf) == 2 && (f & 0xf) == 3 && fp_needs(f)) {
        if (fp_needs(f) != i || ((v & 0xf) == 1 && vp_gives(v) != i))
            return fail(PS3D_ERR_INVALID, "processors 0x%04x/0x%04x/0x%04x do not share a varying layout", v, i, f);
    }
    size_t slot = 0;
    for (; slot < p->progs.size(); slot++)
        if (p->progs[slot].vp == -1) break;
    if (slot == p->progs.size()) p->progs.emplace_back();
    p->progs[slot].vp = vid;
    p->progs[slot].ip = iid;
    p->progs[slot].fp = fid;
    return (int)slot;
}

int ps3d_programme_destroy(ps3d_pipeline* p, int idx)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (idx < 0 || idx >= (int)p->progs.size()) return fail(PS3D_ERR_RANGE, "destroyProgramme");
    p->progs[idx] = Programme();
    return 0;
}

int ps3d_programme_use(ps3d_pipeline* p, int idx)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (idx < 0 || idx >= (int)p->progs.size()) return fail(PS3D_ERR_RANGE, "useProgramme");
    const Programme& g = p->progs[idx];
    auto pick = [&](int slot, int kind) {
        if (slot < 0 || slot >= (int)p->procs.size()) return 0;
        int id = p->procs[slot];
        return (id & 0xf) == kind ? id : 0;  // dynamic_cast yields NULL on a kind mismatch
    };
    p->vp = pick(g.vp, 1);
    p->ip = pick(g.ip, 2);
    p->fp = pick(g.fp, 3);
    return 0;
}

int ps3d_vao_create(ps3d_pipeline* p)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    size_t slot = 0;
    for (; slot < p->vaos.size(); slot++)
        if (!p->vaos[slot].alive) break;
    if (slot == p->vaos.size()) p->vaos.emplace_back();
    p->vaos[slot] = Vao();
    p->vaos[slot].alive = true;
    return (int)slot;
}

int ps3d_vao_destroy(ps3d_pipeline* p, int vao)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (vao < 0 || vao >= (int)p->vaos.size()) return fail(PS3D_ERR_RANGE, "destroyVAO");
    if (!p->vaos[vao].alive) return 0;
    int rc = do_finish(p);
    if (rc) return rc;
    for (auto* cb : p->cmdbufs) cb->stale = true;
    for (auto*& b : p->vaos[vao].vbo)
        if (b) {
            cudaFree(b->dev);
            delete b;
            b = nullptr;
        }
    p->vaos[vao].alive = false;
    return 0;
}

static int vbo_attach(ps3d_pipeline* p, int vao, int slot, int unitBytes, int count, const void* data,
                      cudaMemcpyKind kind)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (vao < 0 || vao >= (int)p->vaos.size() || !p->vaos[vao].alive) return fail(PS3D_ERR_RANGE, "attachVBO vao");
    if (slot < 0 || slot >= PS3D_MAX_VBOS) return fail(PS3D_ERR_RANGE, "attachVBO idx");
    if (unitBytes <= 0 || count < 0 || (unitBytes % 4)) return fail(PS3D_ERR_INVALID, "bad VBO layout");
    if (p->vaos[vao].vbo[slot]) {
        int rc = do_finish(p);
        if (rc) return rc;
        for (auto* cb : p->cmdbufs) cb->stale = true;
        cudaFree(p->vaos[vao].vbo[slot]->dev);
        delete p->vaos[vao].vbo[slot];
        p->vaos[vao].vbo[slot] = nullptr;
    }
    Vbo* b = new (std::nothrow) Vbo();
    if (!b) return fail(PS3D_ERR_NOMEM, "host allocation failed");
    b->unitBytes = unitBytes;
    b->count = count;
    size_t bytes = (size_t)unitBytes * count;
    if (dev_malloc((void**)&b->dev, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        delete b;
        return fail(PS3D_ERR_NOMEM, "VBO allocation failed");
    }
    if (data && bytes) CU(cudaMemcpyAsync(b->dev, data, bytes, kind, p->stream));
    if (kind == cudaMemcpyHostToDevice) CU(cudaStreamSynchronize(p->stream));
    p->vaos[vao].vbo[slot] = b;
    return 0;
}

int ps3d_vbo_attach(ps3d_pipeline* p, int vao, int slot, int unitBytes, int count, const void* data)
{
    return vbo_attach(p, vao, slot, unitBytes, count, data, cudaMemcpyHostToDevice);
}

int ps3d_vbo_attach_device(ps3d_pipeline* p, int vao, int slot, int unitBytes, int count, const void* devData)
{
    return vbo_attach(p, vao, slot, unitBytes, count, devData, cudaMemcpyDeviceToDevice);
}

int ps3d_vbo_update(ps3d_pipeline* p, int vao, int slot, const void* data)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (vao < 0 || vao >= (int)p->vaos.size() || !p->vaos[vao].alive) return fail(PS3D_ERR_RANGE, "getVBO vao");
    if (slot < 0 || slot >= PS3D_MAX_VBOS) return fail(PS3D_ERR_RANGE, "getVBO idx");
    Vbo* b = p->vaos[vao].vbo[slot];
    if (!b) return fail(PS3D_ERR_RANGE, "updateContent: no VBO in that slot");
    if (!data) return fail(PS3D_ERR_INVALID, "updateContent: null source");
    if (p->recording) return fail(PS3D_ERR_INVALID, "updateContent while a command buffer is being recorded");
    // Draws recorded before the call read the old contents, as the
    // reference's synchronous drawVAO did: they are rendered (and, after a
    // bin-list overflow, re-run) before the buffer changes.  Draws recorded
    // later, and command buffers replayed later, read the new contents.
    int rc = do_finish(p);
    if (rc) return rc;
    const size_t bytes = (size_t)b->unitBytes * b->count;
    if (bytes) {
        CU(cudaMemcpyAsync(b->dev, data, bytes, cudaMemcpyHostToDevice, p->stream));
        CU(cudaStreamSynchronize(p->stream));
    }
    return 0;
}

int ps3d_vbo_detach(ps3d_pipeline* p, int vao, int slot)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (vao < 0 || vao >= (int)p->vaos.size() || !p->vaos[vao].alive) return fail(PS3D_ERR_RANGE, "detachVBO vao");
    if (slot < 0 || slot >= PS3D_MAX_VBOS) return fail(PS3D_ERR_RANGE, "detachVBO idx");
    if (!p->vaos[vao].vbo[slot]) return 0;
    int rc = do_finish(p);
    if (rc) return rc;
    for (auto* cb : p->cmdbufs) cb->stale = true;
    cudaFree(p->vaos[vao].vbo[slot]->dev);
    delete p->vaos[vao].vbo[slot];
    p->vaos[vao].vbo[slot] = nullptr;
    return 0;
}

int ps3d_set_uniform(ps3d_pipeline* p, int idx, const void* data, size_t len)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (idx < 0 || idx >= PS3D_MAX_UNIFORMS) return fail(PS3D_ERR_RANGE, "setUniform");
    if (!data) p->uni[idx].clear();
    else p->uni[idx].assign((const uint8_t*)data, (const uint8_t*)data + len);
    return 0;
}

int ps3d_set_depth(ps3d_pipeline* p, int idx)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (idx == -1) {
        p->depthTarget = -1;
        return 0;
    }
    if (!tex_ok(p, idx)) return fail(PS3D_ERR_RANGE, "setDepth");
    const Texture& t = p->tex[idx];
    if (t.elemLen != 4 || t.scanline % 4) return fail(PS3D_ERR_INVALID, "setDepth: not an FP32 texture");
    if (t.wrap) return fail(PS3D_ERR_INVALID, "setDepth: a depth target must be CLAMP-addressed");
    p->depthTarget = idx;
    if (std::find(p->depthTargetPtrs.begin(), p->depthTargetPtrs.end(), (const void*)t.dev) == p->depthTargetPtrs.end())
        p->depthTargetPtrs.push_back(t.dev);
    return 0;
}

int ps3d_set_viewport(ps3d_pipeline* p, int width, int height) { return ps3d_set_viewport_rect(p, 0, 0, width, height); }

int ps3d_set_viewport_rect(ps3d_pipeline* p, int x, int y, int width, int height)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (width <= 0 || height <= 0 || width > 32767 || height > 32767 || x < 0 || y < 0 || x + width > 32767 ||
        y + height > 32767)
        return fail(PS3D_ERR_INVALID, "bad viewport");
    p->vpX = x;
    p->vpY = y;
    p->W = width;
    p->H = height;
    return 0;
}

int ps3d_enable(ps3d_pipeline* p, int bits)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    p->behavior |= bits;
    return 0;
}

int ps3d_disable(ps3d_pipeline* p, int bits)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    p->behavior &= ~bits;
    return 0;
}

int ps3d_clear_depth(ps3d_pipeline* p, float v)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    Command c;
    memset(&c, 0, sizeof c);
    c.kind = Command::CLEAR_DEPTH;
    c.colourTarget = -1;
    c.depthTarget = p->depthTarget;
    c.depthValue = v;
    (p->recording ? p->recording->cmds : p->pending).push_back(c);
    return 0;
}

int ps3d_clear_colour(ps3d_pipeline* p, uint32_t bgra)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    Command c;
    memset(&c, 0, sizeof c);
    c.kind = Command::CLEAR_COLOUR;
    c.colourTarget = -1;
    c.depthTarget = p->depthTarget;
    c.colourValue = bgra;
    (p->recording ? p->recording->cmds : p->pending).push_back(c);
    return 0;
}

int ps3d_draw(ps3d_pipeline* p, int vao)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    // drawvao.cpp:12-15: silently nothing without a programme or with a bad VAO
    if (!p->vp || !p->ip || !p->fp || vao < 0 || vao >= (int)p->vaos.size() || !p->vaos[vao].alive) return 0;
    const Vao& va = p->vaos[vao];
    Command c;
    memset(&c, 0, sizeof c);
    c.kind = Command::DRAW;
    c.depthTarget = p->depthTarget;
    c.colourTarget = p->fbo[0];
    c.vpX = p->vpX;
    c.vpY = p->vpY;
    c.vpW = p->W;
    c.vpH = p->H;
    DrawDesc& d = c.desc;
    d.vp = p->vp;
    d.fp = p->fp;
    int need = fp_needs(p->fp);
    d.nv = need ? required_vary(need) : 0;
    // DEF05 and FP_Null write nothing; CloudShadow only discards (its depth-only pass)
    d.flags = (p->behavior & 0xf) |
              (p->fp == FP_CLOUDSHADOW ? F_FRAGMENT : (p->fp != FP_DEF05 && p->fp != FP_NULL) ? F_COLOUR : 0);
    // processVertices stops at the first VBO that runs out (vertthrd.cpp:18-31)
    long long minCount = -1;
    for (int s = 0; s < PS3D_MAX_VBOS; s++)
        if (va.vbo[s]) minCount = minCount < 0 ? va.vbo[s]->count : std::min<long long>(minCount, va.vbo[s]->count);
    if (minCount < 0) return 0;
    int reqSlots[5] = {1, 0, 0, 0, 0};
    if (p->vp == VP_DEF01 && d.nv) reqSlots[3] = reqSlots[4] = 1;
    if (p->vp == VP_LIT2 && d.nv) reqSlots[1] = reqSlots[3] = reqSlots[4] = 1;
    if (p->vp == VP_DEF03 && d.nv) reqSlots[1] = reqSlots[2] = reqSlots[3] = reqSlots[4] = 1;
    if (p->vp == VP_DEF02 && d.nv) reqSlots[1] = reqSlots[2] = 1;
    if (p->vp == VP_PLANET && d.nv) reqSlots[1] = reqSlots[2] = reqSlots[3] = reqSlots[4] = 1;
    if (p->vp == VP_CLOUD && d.nv) reqSlots[3] = reqSlots[4] = 1;
    if (p->vp == VP_CLOUDSHADOW && d.nv) reqSlots[4] = 1;
    if (p->vp == VP_SINGLECOLOUR && d.nv) reqSlots[3] = 1;
    if (p->vp == VP_DIFFUSEONLY && d.nv) reqSlots[3] = reqSlots[4] = 1;
    for (int s = 0; s < kVboSlots; s++) {
        if (reqSlots[s] && !va.vbo[s]) return fail(PS3D_ERR_INVALID, "the vertex processor reads VBO slot %d", s);
        if (va.vbo[s]) {
            d.vbo[s] = va.vbo[s]->dev;
            d.stride[s] = va.vbo[s]->unitBytes;
            int minBytes = s == 4 ? 8 : 16;
            if (reqSlots[s] && va.vbo[s]->unitBytes < minBytes)
                return fail(PS3D_ERR_INVALID, "VBO slot %d elements are %d bytes", s, va.vbo[s]->unitBytes);
        }
    }
    d.triCount = (int)(minCount / 3);
    d.vpX = p->vpX;
    d.vpY = p->vpY;
    d.vpW = p->W;
    d.vpH = p->H;
    int rc = snapshot_uniforms(p, c.uni);
    if (rc) return rc;
    Target tg;
    if ((rc = depth_target(p, p->depthTarget, tg))) return rc;
    if (tg.w < p->vpX + p->W || tg.h < p->vpY + p->H)
        return fail(PS3D_ERR_INVALID, "the viewport rectangle is not inside the depth target");
    if (tg.w > 65535 || tg.h > 32767)  // the rasters' row numbers and shade-list pixels are 16-bit
        return fail(PS3D_ERR_RANGE, "a depth target larger than 65535 x 32767 cannot be drawn into");
    if (d.flags & F_COLOUR) {
        ColourTarget ct;
        if ((rc = colour_target(p, c.colourTarget, ct))) return rc;
        if (ct.w < p->vpX + p->W || ct.h < p->vpY + p->H)
            return fail(PS3D_ERR_INVALID, "the viewport rectangle is not inside the colour target");
    }
    (p->recording ? p->recording->cmds : p->pending).push_back(c);
    p->stats.draws++;
    return 0;
}

int ps3d_set_bin_width(ps3d_pipeline* p, int columns)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (columns != 8 && columns != 16 && columns != 32)
        return fail(PS3D_ERR_INVALID, "bin width %d: 8, 16 or 32 columns", columns);
    p->binW = columns;
    return 0;
}

int ps3d_set_row_split(ps3d_pipeline* p, int blocksPerBin)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (blocksPerBin != 1 && blocksPerBin != 2 && blocksPerBin != 4 && blocksPerBin != 8)
        return fail(PS3D_ERR_INVALID, "blocks per bin must be 1, 2, 4 or 8");
    p->rowSplit = blocksPerBin;
    return 0;
}

int ps3d_set_fbo(ps3d_pipeline* p, int idx, int texture)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (idx < 0 || idx >= PS3D_MAX_FBOS) return fail(PS3D_ERR_RANGE, "setFBO");
    if (texture != -1) {
        if (!tex_ok(p, texture)) return fail(PS3D_ERR_RANGE, "setFBO: texture %d", texture);
        const Texture& t = p->tex[texture];
        if (t.elemLen != 4 || t.scanline % 4)
            return fail(PS3D_ERR_INVALID, "setFBO: the processors write 4-byte BGRA elements");
    }
    p->fbo[idx] = texture;
    return 0;
}

int ps3d_set_lazy_varyings(ps3d_pipeline* p, int on)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    p->lazyVary = on ? 1 : 0;
    return 0;
}

int ps3d_set_span_items(ps3d_pipeline* p, int on)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    p->spanItems = on ? 1 : 0;
    return 0;
}

int ps3d_set_raster_warp_bins(ps3d_pipeline* p, int on)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    p->warpBins = on ? 1 : 0;
    return 0;
}

int ps3d_set_span_culling(ps3d_pipeline* p, int on)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    p->cullSpans = on ? 1 : 0;
    return 0;
}

int ps3d_set_raster_occupancy(ps3d_pipeline* p, int blocksPerSM)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (blocksPerSM != 0 && blocksPerSM != 8)
        return fail(PS3D_ERR_INVALID, "raster occupancy %d: 0 (default) or 8 blocks per SM", blocksPerSM);
    p->rasterBlocks = blocksPerSM;
    return 0;
}

int ps3d_get_bin_width(ps3d_pipeline* p, int* columns)
{
    if (!p || !columns) return fail(PS3D_ERR_INVALID, "null argument");
    *columns = p->binW;
    return 0;
}

int ps3d_flush(ps3d_pipeline* p)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    return do_flush(p);
}

int ps3d_finish(ps3d_pipeline* p)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    return do_finish(p);
}

int ps3d_read_colour(ps3d_pipeline* p, void* out)
{
    if (!p || !out) return fail(PS3D_ERR_INVALID, "null argument");
    int rc = do_finish(p);
    if (rc) return rc;
    CU(cudaMemcpyAsync(out, p->colour, (size_t)p->devW * 4 * p->devH, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return 0;
}

int ps3d_read_depth(ps3d_pipeline* p, void* out)
{
    if (!p || !out) return fail(PS3D_ERR_INVALID, "null argument");
    int rc = do_finish(p);
    if (rc) return rc;
    CU(cudaMemcpyAsync(out, p->defDepth, (size_t)p->defDepthScan * 4 * p->devH, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return 0;
}

int ps3d_read_colour_device(ps3d_pipeline* p, void* devDst)
{
    if (!p || !devDst) return fail(PS3D_ERR_INVALID, "null argument");
    Command c;
    memset(&c, 0, sizeof c);
    c.kind = Command::COPY_COLOUR;
    c.colourTarget = -1;
    c.depthTarget = p->depthTarget;
    c.copyDst = devDst;
    c.copyW = p->devW;
    c.copyH = p->devH;
    c.copyPitch = (size_t)p->devW * 4;
    (p->recording ? p->recording->cmds : p->pending).push_back(c);
    return 0;
}

int ps3d_copy_colour_rect(ps3d_pipeline* p, int x, int y, int width, int height, void* dst, size_t dstPitch)
{
    if (!p || !dst) return fail(PS3D_ERR_INVALID, "null argument");
    if (x < 0 || y < 0 || width <= 0 || height <= 0 || x + width > p->devW || y + height > p->devH)
        return fail(PS3D_ERR_RANGE, "rectangle %d,%d %dx%d outside the %dx%d colour buffer", x, y, width, height,
                    p->devW, p->devH);
    if (dstPitch < (size_t)width * 4) return fail(PS3D_ERR_INVALID, "destination pitch below the row size");
    Command c;
    memset(&c, 0, sizeof c);
    c.kind = Command::COPY_COLOUR;
    c.colourTarget = -1;
    c.depthTarget = p->depthTarget;
    c.copyDst = dst;
    c.copyX = x;
    c.copyY = y;
    c.copyW = width;
    c.copyH = height;
    c.copyPitch = dstPitch;
    (p->recording ? p->recording->cmds : p->pending).push_back(c);
    return 0;
}

int ps3d_post_process(ps3d_pipeline* p, int postProcessorId, const void* params, size_t bytes)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    Command c;
    memset(&c, 0, sizeof c);
    c.kind = Command::POST;
    c.depthTarget = p->depthTarget;
    c.colourTarget = p->fbo[0];
    c.postId = postProcessorId;
    switch (postProcessorId) {
    case PP_ADD8:
        c.postColour = 0x32323232u;  // the demo's eight bytes of 50 (test2/testpost.cpp:16)
        if (params) {
            if (bytes < 4) return fail(PS3D_ERR_INVALID, "PS3D_PP_ADD8 takes 4 bytes (B, G, R, A addends)");
            memcpy(&c.postColour, params, 4);
        }
        break;
    case PP_FOG: {
        if (!params || bytes < 12) return fail(PS3D_ERR_INVALID, "PS3D_PP_FOG takes {uint32 BGRA, float near, float far}");
        memcpy(&c.postColour, params, 4);
        memcpy(&c.postNear, (const uint8_t*)params + 4, 4);
        memcpy(&c.postFar, (const uint8_t*)params + 8, 4);
        Target t;
        ColourTarget ct;
        int rc = depth_target(p, c.depthTarget, t);
        if (rc || (rc = colour_target(p, c.colourTarget, ct))) return rc;
        if (t.w < ct.w || t.h < ct.h || t.scan < ct.w)
            return fail(PS3D_ERR_INVALID, "the fog post-process needs a depth buffer of at least %dx%d", ct.w, ct.h);
        break;
    }
    default: return fail(PS3D_ERR_INVALID, "unknown post-processor 0x%04x", postProcessorId);
    }
    (p->recording ? p->recording->cmds : p->pending).push_back(c);
    return 0;
}

int ps3d_query(ps3d_pipeline* p)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    cudaError_t e = cudaStreamQuery(p->stream);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return fail(PS3D_ERR_DEVICE, "cudaStreamQuery: %s", cudaGetErrorString(e));
}

int ps3d_colour_device_ptr(ps3d_pipeline* p, void** out)
{
    if (!p || !out) return fail(PS3D_ERR_INVALID, "null argument");
    *out = p->colour;
    return 0;
}

int ps3d_get_stream(ps3d_pipeline* p, void** out)
{
    if (!p || !out) return fail(PS3D_ERR_INVALID, "null argument");
    *out = (void*)p->stream;
    return 0;
}

int ps3d_set_fragment_counting(ps3d_pipeline* p, int on)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    p->countFrags = on != 0;
    return 0;
}

unsigned long long ps3d_allocation_count(void) { return g_allocCount.load(std::memory_order_relaxed); }

int ps3d_stats(ps3d_pipeline* p, ps3d_stats_t* out)
{
    if (!p || !out) return fail(PS3D_ERR_INVALID, "null argument");
    int rc = do_finish(p);
    if (rc) return rc;
    unsigned long long c[4];
    CU(cudaMemcpy(c, p->status + 4, sizeof c, cudaMemcpyDeviceToHost));
    *out = p->stats;
    out->fragments = c[0];
    out->fragments_passed = c[1];
    out->bin_pairs = c[2];
    out->shaded = c[3];
    return 0;
}

int ps3d_cmdbuf_begin(ps3d_pipeline* p)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (p->recording) return fail(PS3D_ERR_INVALID, "a command buffer is already being recorded");
    p->recording = new (std::nothrow) ps3d_cmdbuf();
    if (!p->recording) return fail(PS3D_ERR_NOMEM, "host allocation failed");
    return 0;
}

int ps3d_cmdbuf_end(ps3d_pipeline* p, ps3d_cmdbuf** out)
{
    if (!p || !out) return fail(PS3D_ERR_INVALID, "null argument");
    if (!p->recording) return fail(PS3D_ERR_INVALID, "no command buffer is being recorded");
    ps3d_cmdbuf* cb = p->recording;
    p->recording = nullptr;
    // Lay every pass's descriptors out once, in plan order.
    plan_commands(
        cb->cmds, 0,
        [&](const Pass& ps, size_t) {
            std::vector<DrawDesc> dd;
            std::vector<DrawUniforms> uu;
            int nTris = 0, nvMax = 0;
            bool anyColour = false;
            pass_descriptors(cb->cmds, ps, dd, uu, nTris, nvMax, anyColour);
            cb->passOffset.push_back(cb->hDraws.size());
            cb->hDraws.insert(cb->hDraws.end(), dd.begin(), dd.end());
            cb->hUnis.insert(cb->hUnis.end(), uu.begin(), uu.end());
            return 0;
        },
        [&](int, float, uint32_t) { return 0; }, [&](const Command&) { return 0; });
    size_t n = std::max<size_t>(cb->hDraws.size(), 1);
    bool ok = dev_malloc((void**)&cb->dDraws, n * sizeof(DrawDesc)) == cudaSuccess &&
              dev_malloc((void**)&cb->dUnis, n * sizeof(DrawUniforms)) == cudaSuccess &&
              host_malloc((void**)&cb->pinDraws, n * sizeof(DrawDesc)) == cudaSuccess &&
              host_malloc((void**)&cb->pinUnis, n * sizeof(DrawUniforms)) == cudaSuccess;
    if (!ok) {
        p->cmdbufs.push_back(cb);
        ps3d_cmdbuf_destroy(p, cb);
        return fail(PS3D_ERR_NOMEM, "command buffer allocation failed");
    }
    if (!cb->hDraws.empty()) {
        memcpy(cb->pinDraws, cb->hDraws.data(), cb->hDraws.size() * sizeof(DrawDesc));
        memcpy(cb->pinUnis, cb->hUnis.data(), cb->hUnis.size() * sizeof(DrawUniforms));
        CU(cudaMemcpyAsync(cb->dDraws, cb->pinDraws, cb->hDraws.size() * sizeof(DrawDesc), cudaMemcpyHostToDevice,
                           p->stream));
        CU(cudaMemcpyAsync(cb->dUnis, cb->pinUnis, cb->hUnis.size() * sizeof(DrawUniforms), cudaMemcpyHostToDevice,
                           p->stream));
        CU(cudaStreamSynchronize(p->stream));
    }
    p->cmdbufs.push_back(cb);
    *out = cb;
    return 0;
}

int ps3d_cmdbuf_input_bytes(ps3d_pipeline* p, ps3d_cmdbuf* cb, size_t* out)
{
    if (!p || !cb || !out) return fail(PS3D_ERR_INVALID, "null argument");
    *out = cb->hDraws.size() * (sizeof(DrawDesc) + sizeof(DrawUniforms));
    return 0;
}

int ps3d_cmdbuf_submit(ps3d_pipeline* p, ps3d_cmdbuf* cb, int uploadInputs)
{
    if (!p || !cb) return fail(PS3D_ERR_INVALID, "null argument");
    if (cb->stale) return fail(PS3D_ERR_INVALID, "a texture or VBO of this command buffer changed; record it again");
    int rc;
    if (!cb->exec) {
        // First submission: run and verify like ps3d_finish, then capture.
        p->pending.insert(p->pending.end(), cb->cmds.begin(), cb->cmds.end());
        if ((rc = do_finish(p))) return rc;
        ps3d_stats_t saved = p->stats;
        bool profOn = p->prof.on;
        p->prof.on = false;
        p->liveGraphs++;
        p->cbDraws = cb->dDraws;
        p->cbUnis = cb->dUnis;
        p->cbOffsets = &cb->passOffset;
        CU(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeRelaxed));
        rc = launch_cmds(p, cb->cmds, 0);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(p->stream, &g);
        p->cbDraws = nullptr;
        p->cbUnis = nullptr;
        p->cbOffsets = nullptr;
        p->passStart.clear();
        p->prof.on = profOn;
        p->stats = saved;
        if (rc || e != cudaSuccess || !g) {
            p->liveGraphs--;
            if (g) cudaGraphDestroy(g);
            return rc ? rc : fail(PS3D_ERR_DEVICE, "graph capture failed: %s", cudaGetErrorString(e));
        }
        cb->graph = g;
        if (cudaGraphInstantiate(&cb->exec, g, 0) != cudaSuccess) {
            p->liveGraphs--;
            cudaGraphDestroy(g);
            cb->graph = nullptr;
            cb->exec = nullptr;
            return fail(PS3D_ERR_DEVICE, "graph instantiation failed");
        }
        return 0;
    }
    if (!p->pending.empty() || !p->launched.empty())
        if ((rc = do_finish(p))) return rc;
    if (uploadInputs && !cb->hDraws.empty()) {
        CU(cudaMemcpyAsync(cb->dDraws, cb->pinDraws, cb->hDraws.size() * sizeof(DrawDesc), cudaMemcpyHostToDevice,
                           p->stream));
        CU(cudaMemcpyAsync(cb->dUnis, cb->pinUnis, cb->hUnis.size() * sizeof(DrawUniforms), cudaMemcpyHostToDevice,
                           p->stream));
        p->stats.upload_bytes += cb->hDraws.size() * sizeof(DrawDesc) + cb->hUnis.size() * sizeof(DrawUniforms);
    }
    CU(cudaGraphLaunch(cb->exec, p->stream));
    p->graphUnverified = cb;
    p->stats.batches += cb->passOffset.size();
    return 0;
}

int ps3d_cmdbuf_destroy(ps3d_pipeline* p, ps3d_cmdbuf* cb)
{
    if (!p || !cb) return fail(PS3D_ERR_INVALID, "null argument");
    if (p->stream) cudaStreamSynchronize(p->stream);
    if (p->graphUnverified == cb) p->graphUnverified = nullptr;
    if (cb->exec) {
        cudaGraphExecDestroy(cb->exec);
        cudaGraphDestroy(cb->graph);
        if (--p->liveGraphs == 0) {
            for (void* r : p->retired) cudaFree(r);
            p->retired.clear();
        }
    }
    if (cb->dDraws) cudaFree(cb->dDraws);
    if (cb->dUnis) cudaFree(cb->dUnis);
    if (cb->pinDraws) cudaFreeHost(cb->pinDraws);
    if (cb->pinUnis) cudaFreeHost(cb->pinUnis);
    p->cmdbufs.erase(std::remove(p->cmdbufs.begin(), p->cmdbufs.end(), cb), p->cmdbufs.end());
    delete cb;
    return 0;
}

int ps3d_timer_begin(ps3d_pipeline* p)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (!p->timerA) {
        CU(cudaEventCreate(&p->timerA));
        CU(cudaEventCreate(&p->timerB));
    }
    CU(cudaEventRecord(p->timerA, p->stream));
    return 0;
}

int ps3d_timer_end(ps3d_pipeline* p, float* ms)
{
    if (!p || !ms || !p->timerA) return fail(PS3D_ERR_INVALID, "timer not started");
    CU(cudaEventRecord(p->timerB, p->stream));
    CU(cudaEventSynchronize(p->timerB));
    CU(cudaEventElapsedTime(ms, p->timerA, p->timerB));
    return 0;
}

int ps3d_selftest_division(uint64_t pairs, uint64_t* rcpMismatches, uint64_t* divMismatches)
{
    if (!rcpMismatches || !divMismatches) return fail(PS3D_ERR_INVALID, "null argument");
    unsigned long long a = 0, b = 0;
    if (selftest_division(pairs, &a, &b)) return fail(PS3D_ERR_DEVICE, "self-test launch failed");
    *rcpMismatches = a;
    *divMismatches = b;
    return 0;
}

int ps3d_selftest_occlusion(uint64_t cases, uint64_t* wrong, uint64_t* occluded)
{
    if (!wrong || !occluded) return fail(PS3D_ERR_INVALID, "null argument");
    unsigned long long a = 0, b = 0;
    if (selftest_occlusion(cases, &a, &b)) return fail(PS3D_ERR_DEVICE, "self-test launch failed");
    *wrong = a;
    *occluded = b;
    return 0;
}

int ps3d_selftest_wait(ps3d_pipeline* p, int spins, float* ms)
{
    if (!p || !ms || spins < 1) return fail(PS3D_ERR_INVALID, "bad argument");
    int rc = do_finish(p);
    if (rc) return rc;
    if (!p->timerA) {
        CU(cudaEventCreate(&p->timerA));
        CU(cudaEventCreate(&p->timerB));
    }
    CU(cudaEventRecord(p->timerA, p->stream));
    // status word 15 is never written: the flag that nothing sets
    launch_selftest_wait(p->status, p->status + 15, spins, p->stream);
    CU(cudaGetLastError());
    CU(cudaEventRecord(p->timerB, p->stream));
    CU(cudaEventSynchronize(p->timerB));
    CU(cudaEventElapsedTime(ms, p->timerA, p->timerB));
    return do_finish(p);  // reads the failure words like after a pass
}

int ps3d_l2_scrub(ps3d_pipeline* p, size_t bytes)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (p->scrubBytes < bytes) {
        if (p->scrub) cudaFree(p->scrub);
        p->scrub = nullptr;
        p->scrubBytes = 0;
        CU(dev_malloc(&p->scrub, bytes));
        p->scrubBytes = bytes;
    }
    static unsigned char v = 0;
    CU(cudaMemsetAsync(p->scrub, ++v, bytes, p->stream));
    return 0;
}

int ps3d_profile_enable(ps3d_pipeline* p, int on)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    p->prof.on = on != 0;
    return 0;
}

int ps3d_profile_read(ps3d_pipeline* p, int* launches, double* ms)
{
    if (!p || !launches || !ms) return fail(PS3D_ERR_INVALID, "null argument");
    int rc = do_finish(p);
    if (rc) return rc;
    for (int k = 0; k < K_COUNT; k++) {
        launches[k] = 0;
        ms[k] = 0.0;
    }
    for (auto& m : p->prof.marks) {
        float t = 0.0f;
        CU(cudaEventElapsedTime(&t, m.a, m.b));
        launches[m.id]++;
        ms[m.id] += t;
        p->prof.pool.push_back(m.a);
        p->prof.pool.push_back(m.b);
    }
    p->prof.marks.clear();
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// ps3d_finish_noalloc: ps3d_finish for callers that must not allocate device
// memory -- a real-time render thread that may not block in cudaMalloc or
// cudaFree (both can synchronise the whole device), a process whose device
// memory is fully committed up front, or a service that must not grow after
// admission control has accounted for it.  The recorded passes take their
// scratch (descriptors, triangle records, varyings, bin lists, look-back
// descriptors, shade list) from one fixed array instead of the pipeline's growable
// buffers, and run the same kernels with the same results.

namespace {

// The fixed scratch: 16 MiB per device, carved afresh for every pass.  It
// holds, for example, a 1024x1024 colour pass of ~15k triangles and ~200k
// bin pairs, or a 2048x2048 depth-only pass of ~40k triangles.
constexpr size_t kNoAllocBytes = (size_t)16 << 20;
constexpr int kNoAllocMaxDraws = 1024;  // draws per pass (host staging below)
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocBytes];

std::mutex g_noallocLock;                       // one caller at a time: they share the array
unsigned char* g_noallocPtr[kNoAllocMaxDevices];  // its address per device, looked up once
DrawDesc g_noallocDraws[kNoAllocMaxDraws];      // a pass's descriptors, staged on the host
DrawUniforms g_noallocUnis[kNoAllocMaxDraws];

// Byte offsets of one pass's buffers in the array, each 256-byte aligned.
struct NoAllocLayout {
    size_t draws, unis, tris, vary, shadeList, binStart, radix, pairKey,
        pairTri, keyB, binTri, spans;
};

size_t noalloc_layout(NoAllocLayout& L, int nd, int nTris, int nv, int W, int H, bool colour, size_t nBins,
                      int pairCap, bool spanItems)
{
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t at = off;
        off = (off + bytes + 255) & ~(size_t)255;
        return at;
    };
    size_t sortBlocks = ((size_t)pairCap + kSortChunk - 1) / kSortChunk;
    if (nBins > 0x7fffffff) return (size_t)-1;
    L.draws = take((size_t)nd * sizeof(DrawDesc));
    L.unis = take((size_t)nd * sizeof(DrawUniforms));
    L.tris = take((size_t)nTris * sizeof(TriRaster));
    L.vary = take((size_t)nTris * 3 * std::max(nv, 1) * sizeof(float));
    L.shadeList = colour ? take((size_t)W * H * sizeof(int2)) : 0;
    L.binStart = take((2 + (size_t)kItemsPerBin) * nBins * sizeof(int));
    L.radix = take(radix_scratch_ints((int)sortBlocks, radix_passes((int)nBins), nTris) * sizeof(int));
    L.pairKey = take((size_t)pairCap * sizeof(int));
    L.pairTri = take((size_t)pairCap * sizeof(int));
    L.keyB = take((size_t)pairCap * sizeof(int));
    L.binTri = take((size_t)pairCap * sizeof(int));
    L.spans = spanItems ? take((size_t)pairCap * sizeof(SpanItem)) : 0;
    return off;
}

// A pass's shape: its draws staged in g_noallocDraws/g_noallocUnis.
struct NoAllocPass {
    Target tg;
    int nd = 0, nTris = 0, nvMax = 0;
    bool anyColour = false;
    int binsX = 0, binsY = 0;
    size_t nBins = 0;
    int pairCap = 0;  // largest multiple of the sort chunk that fits, 0 if none does
    bool forward = false;
    int binW = 0;
    bool spanItems = false;
};

int noalloc_shape(ps3d_pipeline* p, const std::vector<Command>& cmds, const Pass& ps, NoAllocPass& s, bool stage)
{
    int rc = depth_target(p, cmds[ps.first].depthTarget, s.tg);
    if (rc) return rc;
    for (size_t i = ps.first; i < ps.last; i++) {
        const DrawDesc& d = cmds[i].desc;
        if (d.triCount == 0) continue;
        if (s.nd == kNoAllocMaxDraws)
            return fail(PS3D_ERR_RANGE, "ps3d_finish_noalloc: a pass has more than %d draws", kNoAllocMaxDraws);
        if (stage) {
            g_noallocDraws[s.nd] = d;
            g_noallocDraws[s.nd].triBase = s.nTris;
            g_noallocDraws[s.nd].uni = s.nd;
            g_noallocUnis[s.nd] = cmds[i].uni;
        }
        s.nd++;
        s.nTris += d.triCount;
        s.nvMax = std::max(s.nvMax, d.nv);
        s.anyColour |= (d.flags & F_COLOUR) != 0;
        s.forward |= pass_forward(&d, 1);
    }
    if (s.nTris == 0) return 0;
    if (s.forward) s.nvMax = forward_vary(s.nvMax);
    s.binW = s.forward ? 16 : p->binW;
    s.spanItems = p->spanItems && !s.forward;
    s.binsX = (s.tg.w + s.binW - 1) / s.binW;
    s.binsY = (s.tg.h + kBinH - 1) / kBinH;
    s.nBins = (size_t)s.binsX * s.binsY;
    if (s.nBins > 0x7fffffff || radix_passes((int)s.nBins) > kRadixMaxPasses)
        return fail(PS3D_ERR_RANGE, "ps3d_finish_noalloc: a %dx%d target has too many bins to sort", s.tg.w,
                    s.tg.h);
    NoAllocLayout L;
    size_t base = noalloc_layout(L, s.nd, s.nTris, s.nvMax, s.tg.w, s.tg.h, s.anyColour, s.nBins, kSortChunk,
                                 s.spanItems);
    if (base > kNoAllocBytes) {
        if (base == (size_t)-1) base = 0;
        return fail(PS3D_ERR_RANGE,
                    "ps3d_finish_noalloc: a pass of %d triangles into a %dx%d target needs %zu bytes of scratch "
                    "before its bin lists; the fixed scratch is %zu bytes (ps3d_finish has no such limit)",
                    s.nTris, s.tg.w, s.tg.h, base, kNoAllocBytes);
    }
    // each further sort tile costs its four pair arrays (and span items) and its look-back descriptors
    size_t perChunk = (size_t)kSortChunk * (4 * sizeof(int) + (s.spanItems ? sizeof(SpanItem) : 0)) +
                      (size_t)kRadixMaxPasses * kRadixDigits * sizeof(int);
    long long chunks = 1 + (long long)((kNoAllocBytes - base) / perChunk);
    chunks = std::min<long long>(chunks, 0x7fffffff / kSortChunk);
    while (chunks > 1 &&
           noalloc_layout(L, s.nd, s.nTris, s.nvMax, s.tg.w, s.tg.h, s.anyColour, s.nBins,
                          (int)(chunks * kSortChunk), s.spanItems) > kNoAllocBytes)
        chunks--;
    s.pairCap = (int)(chunks * kSortChunk);
    return 0;
}

int noalloc_run_pass(ps3d_pipeline* p, const std::vector<Command>& cmds, const Pass& ps, size_t replayFrom,
                     unsigned char* base)
{
    int seq = (int)p->passStart.size();
    p->passStart.push_back(replayFrom);
    const Command& c0 = cmds[ps.first];
    NoAllocPass s;
    int rc = noalloc_shape(p, cmds, ps, s, true);
    if (rc) return rc;
    if (s.nTris == 0) {
        if (ps.clearDepth && (rc = fill_depth_plain(p, c0.depthTarget, ps.depthValue))) return rc;
        if (ps.clearColour && (rc = fill_colour_plain(p, ps.colourValue))) return rc;
        return 0;
    }
    int W = s.tg.w, H = s.tg.h;
    NoAllocLayout L;
    noalloc_layout(L, s.nd, s.nTris, s.nvMax, W, H, s.anyColour, s.nBins, s.pairCap, s.spanItems);
    // Pageable-source copies: each returns once the staging arrays are copied
    // out, so the next pass may overwrite them.
    CU(cudaMemcpyAsync(base + L.draws, g_noallocDraws, s.nd * sizeof(DrawDesc), cudaMemcpyHostToDevice, p->stream));
    CU(cudaMemcpyAsync(base + L.unis, g_noallocUnis, s.nd * sizeof(DrawUniforms), cudaMemcpyHostToDevice,
                       p->stream));
    p->stats.upload_bytes += s.nd * (sizeof(DrawDesc) + sizeof(DrawUniforms));

    bool fuseDepth = ps.clearDepth && s.tg.scan == W;
    ColourTarget ct;
    if ((rc = colour_target(p, c0.colourTarget, ct))) return rc;
    bool fuseColour = ps.clearColour && ct.display && p->devW == W && p->devH == H;
    if (ps.clearDepth && !fuseDepth && (rc = fill_depth_plain(p, c0.depthTarget, ps.depthValue))) return rc;
    if (ps.clearColour && !fuseColour && (rc = fill_colour_plain(p, ps.colourValue))) return rc;

    PassParams P;
    memset(&P, 0, sizeof P);
    P.W = W;
    P.H = H;
    P.binW = s.binW;
    P.rasterBlocks = p->rasterBlocks;
    P.cullSpans = p->cullSpans;
    P.rowSplit = p->rowSplit;
    P.warpBins = p->warpBins;
    P.passFp = pass_fp(g_noallocDraws, (size_t)s.nd);
    P.passVp = pass_vp(g_noallocDraws, (size_t)s.nd);
    P.spanItems = s.spanItems;
    P.spans = s.spanItems ? (SpanItem*)(base + L.spans) : nullptr;
    P.forward = s.forward;
    P.binsX = s.binsX;
    P.binsY = s.binsY;
    P.nTris = s.nTris;
    P.nDraws = s.nd;
    P.draws = (const DrawDesc*)(base + L.draws);
    P.unis = (const DrawUniforms*)(base + L.unis);
    P.tris = (TriRaster*)(base + L.tris);
    P.vary = (float*)(base + L.vary);
    P.nvMax = std::max(s.nvMax, 1);
    P.anyVary = s.nvMax > 0;
    P.lazyVary = p->lazyVary && !s.forward && s.nvMax > 0;
    P.pairKey = (int*)(base + L.pairKey);
    P.pairTri = (int*)(base + L.pairTri);
    P.pairCap = s.pairCap;
    P.sortBlocks = (s.pairCap + kSortChunk - 1) / kSortChunk;
    P.radixPasses = radix_passes((int)s.nBins);
    P.radix = (int*)(base + L.radix);
    P.sortDescOff = sort_desc_offset(s.nTris);
    P.keyB = (int*)(base + L.keyB);
    P.binStart = (int*)(base + L.binStart);
    P.binItems = P.binStart + 2 * s.nBins;
    P.binTri = (int*)(base + L.binTri);
    P.sortedTri = (P.radixPasses & 1) ? P.binTri : P.pairTri;
    P.status = p->status;
    P.slotStatus = p->scr[0].slotStatus;
    P.depth = s.tg.depth;
    P.depthScan = s.tg.scan;
    P.depthW = s.tg.w;
    P.depthH = s.tg.h;
    P.shadeList = s.anyColour ? (int2*)(base + L.shadeList) : nullptr;
    P.colourRow0 = ct.row0;
    P.colourPitch = ct.pitch;
    P.colourW = ct.w;
    P.colourH = ct.h;
    P.clearDepth = fuseDepth;
    P.clearColour = fuseColour;
    P.anyColour = s.anyColour;
    P.countFrags = p->countFrags;
    P.depthClearValue = fuseDepth ? ps.depthValue : 1.0f;
    P.colourClearValue = ps.colourValue;
    P.passSeq = seq;
    Prof off;  // never records events
    int launches = 0;
    if (launch_setup(P, p->stream, launches, &off)) return fail(PS3D_ERR_DEVICE, "memset of the sort scratch failed");
    launch_sort(P, p->stream, launches, &off);
    launch_raster(P, p->stream, launches, &off);
    launch_shade(P, p->stream, launches, &off);
    CU(cudaGetLastError());
    p->stats.kernel_launches += launches;
    p->stats.batches++;
    p->stats.triangles += s.nTris;
    return 0;
}

}  // namespace

extern "C" int ps3d_finish_noalloc(ps3d_pipeline* p)
{
    if (!p) return fail(PS3D_ERR_INVALID, "null pipeline");
    if (p->recording) return fail(PS3D_ERR_INVALID, "ps3d_finish_noalloc: a command buffer is being recorded");
    if (!p->launched.empty() || p->graphUnverified)
        return fail(PS3D_ERR_INVALID, "ps3d_finish_noalloc: flushed work is not verified yet; call ps3d_finish");
    std::lock_guard<std::mutex> lock(g_noallocLock);
    int dev = -1;
    CU(cudaGetDevice(&dev));
    // the array's address is per device: it must be the device the pipeline's streams belong to
    if (dev != p->device)
        return fail(PS3D_ERR_DEVICE, "ps3d_finish_noalloc: device %d is current, the pipeline was created on %d",
                    dev, p->device);
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(PS3D_ERR_DEVICE, "device %d out of range", dev);
    if (!g_noallocPtr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noallocScratch);
        if (e != cudaSuccess || !ptr)
            return fail(PS3D_ERR_DEVICE, "cudaGetSymbolAddress of the fixed scratch: %s", cudaGetErrorString(e));
        g_noallocPtr[dev] = (unsigned char*)ptr;
    }
    unsigned char* base = g_noallocPtr[dev];
    if (p->pending.empty()) return 0;

    // Every pass must fit before anything runs; otherwise the commands stay
    // recorded for ps3d_finish.
    const std::vector<Command>& rec = p->pending;
    int rc = plan_commands(
        rec, 0,
        [&](const Pass& ps, size_t) {
            NoAllocPass s;
            return noalloc_shape(p, rec, ps, s, false);
        },
        [&](int, float, uint32_t) { return 0; }, [&](const Command&) { return 0; });
    if (rc) return rc;

    // The failure words must start clear.
    if ((rc = reset_flags(p))) return rc;
    p->launched.swap(p->pending);
    const std::vector<Command>& cmds = p->launched;
    rc = plan_commands(
        cmds, 0, [&](const Pass& ps, size_t start) { return noalloc_run_pass(p, cmds, ps, start, base); },
        [&](int target, float v, uint32_t c) {
            return target == -3 ? fill_colour_plain(p, c) : fill_depth_plain(p, target, v);
        },
        [&](const Command& c) { return copy_colour_plain(p, c); });
    if (rc) {
        // Work already queued on the shared array must finish before the
        // lock is released; the frame's commands are dropped (incomplete).
        cudaStreamSynchronize(p->stream);
        cudaGetLastError();
        p->launched.clear();
        p->passStart.clear();
        return rc;
    }
    CU(cudaStreamSynchronize(p->stream));
    int st[4];
    CU(cudaMemcpy(st, p->status, sizeof st, cudaMemcpyDeviceToHost));
    if (st[0] & 2) {
        if ((rc = reset_flags(p))) return rc;
        p->launched.clear();
        p->passStart.clear();
        return fail(PS3D_ERR_TIMEOUT, "a device-side wait of the bin sort expired; the frame is incomplete");
    }
    if (st[0]) {
        // A pass found more bin pairs than the array holds: it and the passes
        // after it did nothing.  The commands and the overflow record stay as
        // ps3d_finish's own recovery expects them.
        return fail(PS3D_ERR_NOMEM,
                    "ps3d_finish_noalloc: pass %d needs %d bin pairs, more than the fixed scratch holds; it and "
                    "the passes after it did not run; ps3d_finish completes the frame (and may allocate)",
                    st[3], st[1]);
    }
    p->launched.clear();
    p->passStart.clear();
    return 0;
}
