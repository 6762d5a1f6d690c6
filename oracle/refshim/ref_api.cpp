/*
 * ref_api.cpp -- a C entry surface over the reference's own PuresoftPipeline
 * (compiled unmodified from the reference sources), so that Python test code
 * can replay a scene on it and read back colour and depth.  TEST
 * INFRASTRUCTURE ONLY: it builds into oracle/_ref/libps3dref.so, which exists
 * only where the reference sources are present, and is used to generate and
 * check golden fixtures.
 *
 * Every ps3dr_* call forwards to the PuresoftPipeline method of the same
 * meaning (reference pipeline.h:26-69).  C++ exceptions are turned into the
 * status codes the product's C ABI uses: -1 std::out_of_range,
 * -2 std::invalid_argument, -3 std::bad_alloc.
 *
 * Colour: the pipeline draws into a headless renderer's buffer (a stand-in for
 * the GDI back buffer, reference rndrgdi.cpp).  Its memory layout is the
 * reference display FBO's: BGRA8, top-down (memory row = H - 1 - y,
 * pipeline.cpp:48, fbo.cpp:103-106).
 */
#include <string.h>
#include <stdexcept>
#include <new>
#include "pipeline.h"
#include "defproc.h"
#include "cfgproc.h"
#include "testproc.h"
#include "../test2/testproc.h"  /* the scene viewer's processors (src/test2) */

int logicCPUs(void); /* refshim/win32_runtime.cpp */

namespace {

class HeadlessRenderer : public PuresoftRenderer
{
public:
    void startup(uintptr_t, int width, int height)
    {
        m_width = width;
        m_height = height;
        m_buffer = (uint8_t*)_aligned_malloc((size_t)width * 4 * height, 64);
        memset(m_buffer, 0, (size_t)width * 4 * height);
    }
    void shutdown(void) {}
    void setCanvas(uintptr_t) {}
    void getDesc(PURESOFTIMGBUFF32* desc)
    {
        desc->width = m_width;
        desc->scanline = m_width * 4;
        desc->height = m_height;
        desc->elemLen = 4;
        desc->pixels = m_buffer;
    }
    void* swapBuffers(void) { return m_buffer; }
    void release(void)
    {
        _aligned_free(m_buffer);
        delete this;
    }
    uint8_t* m_buffer = nullptr;
    int m_width = 0, m_height = 0;
};

struct RefCtx {
    PuresoftPipeline* pipe;
    HeadlessRenderer* rndr;
    int width, height;
    // setFBO with a texture: an FBO over the texture's own memory
    // (PuresoftFBO's external-buffer form, fbo.cpp:11-45), owned here
    PuresoftFBO* fboWrap[16] = {};
};

template <class F> int guarded(F f)
{
    try {
        return f();
    } catch (const std::out_of_range&) {
        return -1;
    } catch (const std::invalid_argument&) {
        return -2;
    } catch (const std::bad_alloc&) {
        return -3;
    }
}

PuresoftProcessor* make_processor(int id)
{
    switch (id) {
    case 0x0101: return new VertexProcesserDEF01;
    case 0x0102: return new InterpolationProcessorDEF01;
    case 0x0103: return new FragmentProcessorDEF01;
    case 0x0201: return new VertexProcesserDEF02;
    case 0x0202: return new InterpolationProcessorDEF02;
    case 0x0203: return new FragmentProcessorDEF02;
    case 0x0301: return new VertexProcesserDEF03;
    case 0x0302: return new InterpolationProcessorDEF03;
    case 0x0303: return new FragmentProcessorDEF03;
    case 0x0401: return new VertexProcesserDEF04;
    case 0x0402: return new InterpolationProcessorDEF04;
    case 0x0403: return new FragmentProcessorDEF04;
    case 0x0701: return new VP_Planet;   /* the reference demo's planet set (test/testproc.cpp) */
    case 0x0702: return new IP_Planet;
    case 0x0703: return new FP_Earth;
    case 0x0713: return new FP_Satellite;
    case 0x0801: return new VP_Cloud;   /* the demo's cloud sets (test/testproc.cpp) */
    case 0x0802: return new IP_Cloud;
    case 0x0803: return new FP_Cloud;
    case 0x0901: return new VP_CloudShadow;
    case 0x0902: return new IP_CloudShadow;
    case 0x0903: return new FP_CloudShadow;
    case 0x0A01: return new VP_PositionOnly;  /* the scene viewer's sets (test2/testproc.cpp) */
    case 0x0A02: return new IP_Null;
    case 0x0A03: return new FP_SingleColourNoLighting;
    case 0x0B01: return new VP_SingleColour;
    case 0x0B02: return new IP_SingleColour;
    case 0x0B03: return new FP_SingleColour;
    case 0x0C01: return new VP_DiffuseOnly;
    case 0x0C02: return new IP_DiffuseOnly;
    case 0x0C03: return new FP_DiffuseOnly;
    case 0x0D01: return new VP_Shadow;
    case 0x0D03: return new FP_Null;
    case 0x0501: return new VertexProcesserDEF05;
    case 0x0502: return new InterpolationProcessorDEF05;
    case 0x0503: return new FragmentProcessorDEF05;
    case 0x0601: return new VertexProcesserSHADOW;
    case 0x1103: return new FragmentProcessorLIT1;
    case 0x1403: return new FragmentProcessorLIT1A;
    case 0x1303: return new FragmentProcessorLIT3;
    case 0x1201: return new VertexProcesserLIT2;
    case 0x1202: return new InterpolationProcessorLIT2;
    case 0x1203: return new FragmentProcessorLIT2;
    default: return nullptr;
    }
}

} // namespace

extern "C" {

void* ps3dr_create(int width, int height)
{
    RefCtx* c = new RefCtx();
    c->rndr = new HeadlessRenderer();
    c->rndr->startup(0, width, height);
    c->pipe = new PuresoftPipeline(0, width, height, c->rndr);
    c->width = width;
    c->height = height;
    return c;
}

void ps3dr_destroy(void* h)
{
    RefCtx* c = (RefCtx*)h;
    delete c->pipe; /* releases the renderer */
    for (PuresoftFBO* f : c->fboWrap) delete f;
    delete c;
}

/* PuresoftPipeline::setFBO (pipeline.cpp:260-275) with texture `tex` (its
   memory, wrapped as an FBO of the texture's layout, rows bottom-up as the
   pipeline creates textures, tex.cpp:17) or -1 (slot 0: the display). */
int ps3dr_set_fbo(void* h, int idx, int tex)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] {
        PuresoftFBO* wrap = nullptr;
        if (tex >= 0) {
            PURESOFTIMGBUFF32 img;
            c->pipe->getTexture(tex, &img);
            wrap = new PuresoftFBO(img.width, img.scanline, img.height, img.elemLen, false, img.pixels);
        }
        c->pipe->setFBO(idx, wrap);
        if (idx >= 0 && idx < 16) {
            delete c->fboWrap[idx];
            c->fboWrap[idx] = wrap;
        }
        return 0;
    });
}

int ps3dr_thread_count(void) { return logicCPUs(); }

int ps3dr_texture_create_layers(void* h, int width, int height, int scanline, int elemLen, const void* pixels,
                                int wrap, int extraLayers)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] {
        PURESOFTIMGBUFF32 img;
        img.width = width;
        img.height = height;
        img.scanline = scanline;
        img.elemLen = elemLen;
        img.pixels = (void*)pixels;
        return c->pipe->createTexture(&img, extraLayers, wrap ? PuresoftFBO::WRAP : PuresoftFBO::CLAMP);
    });
}

int ps3dr_texture_create(void* h, int width, int height, int scanline, int elemLen, const void* pixels, int wrap)
{
    return ps3dr_texture_create_layers(h, width, height, scanline, elemLen, pixels, wrap, 0);
}

/* getTexture(idx, image, layer) hands out the layer's own buffer (tex.cpp:27-37);
   these copy into or out of it. */
int ps3dr_texture_write_layer(void* h, int idx, int layer, const void* pixels, size_t bytes)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] {
        PURESOFTIMGBUFF32 img;
        c->pipe->getTexture(idx, &img, (PuresoftFBO::LAYER)layer);
        size_t n = (size_t)img.scanline * img.height;
        memcpy(img.pixels, pixels, n < bytes ? n : bytes);
        return 0;
    });
}

int ps3dr_texture_read_layer(void* h, int idx, int layer, void* out, size_t bytes)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] {
        PURESOFTIMGBUFF32 img;
        c->pipe->getTexture(idx, &img, (PuresoftFBO::LAYER)layer);
        size_t n = (size_t)img.scanline * img.height;
        memcpy(out, img.pixels, n < bytes ? n : bytes);
        return 0;
    });
}

int ps3dr_texture_read(void* h, int idx, void* out, size_t bytes)
{
    return ps3dr_texture_read_layer(h, idx, 0, out, bytes);
}

int ps3dr_processor_add(void* h, int id)
{
    RefCtx* c = (RefCtx*)h;
    PuresoftProcessor* p = make_processor(id);
    if (!p) return -2;
    return c->pipe->addProcessor(p);
}

int ps3dr_programme_create(void* h, int vid, int iid, int fid)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] { return c->pipe->createProgramme(vid, iid, fid); });
}

int ps3dr_programme_use(void* h, int idx)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] {
        c->pipe->useProgramme(idx);
        return 0;
    });
}

int ps3dr_vao_create(void* h) { return ((RefCtx*)h)->pipe->createVAO(); }

int ps3dr_vbo_attach(void* h, int vao, int slot, int unitBytes, int count, const void* data)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] {
        PuresoftVBO* vbo = new PuresoftVBO(unitBytes, count);
        vbo->updateContent(data);
        PuresoftVBO* old = c->pipe->attachVBO(vao, slot, vbo);
        delete old;
        return 0;
    });
}

int ps3dr_set_uniform(void* h, int idx, const void* data, size_t len)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] {
        c->pipe->setUniform(idx, data, len);
        return 0;
    });
}

int ps3dr_set_depth(void* h, int idx)
{
    RefCtx* c = (RefCtx*)h;
    return guarded([&] {
        c->pipe->setDepth(idx);
        return 0;
    });
}

int ps3dr_set_viewport(void* h, int width, int height)
{
    ((RefCtx*)h)->pipe->setViewport(width, height);
    return 0;
}

int ps3dr_enable(void* h, int bits)
{
    ((RefCtx*)h)->pipe->enable(bits);
    return 0;
}

int ps3dr_disable(void* h, int bits)
{
    ((RefCtx*)h)->pipe->disable(bits);
    return 0;
}

int ps3dr_clear_depth(void* h, float v)
{
    ((RefCtx*)h)->pipe->clearDepth(v);
    return 0;
}

/* The reference's clearColour skips the last memory row of the display
   (fbo.cpp:332-346 loops y < m_height - 1).  The harness completes that row
   so that a clear means "every pixel", which is what the product does. */
int ps3dr_clear_colour(void* h, uint32_t bgra)
{
    RefCtx* c = (RefCtx*)h;
    PURESOFTBGRA v;
    v.i32 = bgra;
    c->pipe->clearColour(v);
    uint32_t* last = (uint32_t*)(c->rndr->m_buffer + (size_t)(c->height - 1) * c->width * 4);
    for (int x = 0; x < c->width; x++) last[x] = bgra;
    return 0;
}

int ps3dr_draw(void* h, int vao)
{
    ((RefCtx*)h)->pipe->drawVAO(vao, false);
    return 0;
}

int ps3dr_post_process(void* h, int id, const void* params, size_t bytes)
{
    RefCtx* c = (RefCtx*)h;
    if (id == 0x7001) {
        unsigned char add[4] = {50, 50, 50, 50};
        if (params) {
            if (bytes < 4) return -2;
            memcpy(add, params, 4);
        }
        PostProcessorADD8 pp(add);
        return guarded([&] { c->pipe->postProcess(&pp); return 0; });
    }
    if (id == 0x7002) {
        if (!params || bytes < 12) return -2;
        unsigned int fog;
        float nearD, farD;
        memcpy(&fog, params, 4);
        memcpy(&nearD, (const unsigned char*)params + 4, 4);
        memcpy(&farD, (const unsigned char*)params + 8, 4);
        PostProcessorFOG pp(fog, nearD, farD, c->fboWrap[0] == nullptr);
        return guarded([&] { c->pipe->postProcess(&pp); return 0; });
    }
    return -2;
}

int ps3dr_read_colour(void* h, void* out)
{
    RefCtx* c = (RefCtx*)h;
    memcpy(out, c->rndr->m_buffer, (size_t)c->width * 4 * c->height);
    return 0;
}

} /* extern "C" */
