// ps3d.hpp -- header-only C++ adapter over the C ABI (ps3d.h) with the
// reference's class and method names, so code written against
// PuresoftPipeline (src/puresoft3d/pipeline.h:24-156) can switch by changing
// the type it instantiates.  Status codes become the reference's exceptions:
// std::out_of_range, std::invalid_argument, std::bad_alloc, and
// std::runtime_error for device failures.
#pragma once
#include <new>
#include <stdexcept>
#include <string>
#include <vector>
#include "ps3d.h"

namespace ps3d_gpu {

inline int check(int rc)
{
    if (rc >= 0) return rc;
    std::string m = ps3d_last_error();
    switch (rc) {
    case PS3D_ERR_RANGE: throw std::out_of_range(m);
    case PS3D_ERR_INVALID: throw std::invalid_argument(m);
    case PS3D_ERR_NOMEM: throw std::bad_alloc();
    default: throw std::runtime_error(m);
    }
}

// The reference's PURESOFTIMGBUFF32 (defs.h).
struct ImageBuffer {
    unsigned width, scanline, height, elemLen;
    const void* pixels;
};

// A VBO of a pipeline's VAO, as getVBO returns it (pipeline.cpp:168-181):
// updateContent replaces its contents in place (vbo.cpp:28-31).
class PuresoftVBO
{
public:
    PuresoftVBO(ps3d_pipeline* p, int vao, int idx) : m_p(p), m_vao(vao), m_idx(idx) {}
    void updateContent(const void* src) { check(ps3d_vbo_update(m_p, m_vao, m_idx, src)); }

private:
    ps3d_pipeline* m_p;
    int m_vao, m_idx;
};

class PuresoftPipeline
{
public:
    PuresoftPipeline(int deviceWidth, int deviceHeight, void* cudaStream = nullptr)
        : m_w(deviceWidth), m_h(deviceHeight)
    {
        check(ps3d_pipeline_create(deviceWidth, deviceHeight, cudaStream, &m_p));
    }
    ~PuresoftPipeline() { ps3d_pipeline_destroy(m_p); }
    PuresoftPipeline(const PuresoftPipeline&) = delete;
    PuresoftPipeline& operator=(const PuresoftPipeline&) = delete;

    // texture api (createTexture(image, extraLayers, mode), tex.cpp:3-25: 5 extra layers make a cube map)
    int createTexture(const ImageBuffer* image, int extraLayers = 0, bool wrap = false)
    {
        return check(ps3d_texture_create_layers(m_p, (int)image->width, (int)image->height, (int)image->scanline,
                                                (int)image->elemLen, image->pixels, wrap ? 1 : 0, extraLayers));
    }
    void destroyTexture(int idx) { check(ps3d_texture_destroy(m_p, idx)); }
    void readTexture(int idx, void* out, size_t bytes, int layer = 0)
    {
        check(ps3d_texture_read_layer(m_p, idx, layer, out, bytes));
    }
    // getTexture(idx, image, layer) then filling image.pixels (tex.cpp:27-37)
    void writeTexture(int idx, const void* pixels, size_t bytes, int layer = 0)
    {
        check(ps3d_texture_write_layer(m_p, idx, layer, pixels, bytes));
    }

    // processor api (processor classes are ids: PS3D_VP_* / PS3D_IP_* / PS3D_FP_*)
    int addProcessor(int processorClass) { return check(ps3d_processor_add(m_p, processorClass)); }
    void destroyProcessor(int idx) { check(ps3d_processor_destroy(m_p, idx)); }
    int createProgramme(int vid, int iid, int fid) { return check(ps3d_programme_create(m_p, vid, iid, fid)); }
    void destroyProgramme(int idx) { check(ps3d_programme_destroy(m_p, idx)); }
    void useProgramme(int idx) { check(ps3d_programme_use(m_p, idx)); }

    // vao api: a VBO is attached with its contents (PuresoftVBO + updateContent)
    int createVAO(void) { return check(ps3d_vao_create(m_p)); }
    void attachVBO(int vao, int idx, int unitBytes, int unitCount, const void* data)
    {
        check(ps3d_vbo_attach(m_p, vao, idx, unitBytes, unitCount, data));
    }
    void detachVBO(int vao, int idx) { check(ps3d_vbo_detach(m_p, vao, idx)); }
    PuresoftVBO getVBO(int vao, int idx) { return PuresoftVBO(m_p, vao, idx); }
    void destroyVAO(int vao) { check(ps3d_vao_destroy(m_p, vao)); }

    // rendering api
    void setViewport(int width, int height) { check(ps3d_set_viewport(m_p, width, height)); }
    void setDepth(int idx = -1) { check(ps3d_set_depth(m_p, idx)); }
    // setFBO(idx, fbo) with a texture index as the FBO (-1: none / the display)
    void setFBO(int idx, int texture) { check(ps3d_set_fbo(m_p, idx, texture)); }
    void setUniform(int idx, const void* data, size_t len) { check(ps3d_set_uniform(m_p, idx, data, len)); }
    void drawVAO(int vao) { check(ps3d_draw(m_p, vao)); }
    void enable(int behavior) { check(ps3d_enable(m_p, behavior)); }
    void disable(int behavior) { check(ps3d_disable(m_p, behavior)); }
    void clearDepth(float furthest = 1.0f) { check(ps3d_clear_depth(m_p, furthest)); }
    void clearColour(uint32_t bgra = 0) { check(ps3d_clear_colour(m_p, bgra)); }
    void finish(void) { check(ps3d_finish(m_p)); }
    // postProcess(processor) (post.cpp:3-19) with a built-in post-processor (PS3D_PP_*)
    void postProcess(int postProcessorClass, const void* params = nullptr, size_t bytes = 0)
    {
        check(ps3d_post_process(m_p, postProcessorClass, params, bytes));
    }
    // the demo's SceneObject::findOrCreateVao(objx) (test/scenobj.cpp:88-162)
    int createVAOFromObjx(const char* path, int mesh = 0)
    {
        int vao = -1;
        check(ps3d_objx_load_vao(m_p, path, mesh, &vao));
        return vao;
    }
    // in place of swapBuffers(): the frame, BGRA8 top-down
    void readColour(void* out) { check(ps3d_read_colour(m_p, out)); }
    ps3d_pipeline* handle(void) { return m_p; }

private:
    ps3d_pipeline* m_p = nullptr;
    int m_w, m_h;
};

}  // namespace ps3d_gpu
