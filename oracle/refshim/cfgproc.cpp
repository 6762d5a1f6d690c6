/*
 * cfgproc.cpp -- the benchmark scenes' shaders written as Puresoft processors
 * against the reference's own plugin API (src/puresoft3d/proc.h:26-71), for
 * the Linux build of the reference pipeline core (oracle/_ref).
 * TEST INFRASTRUCTURE ONLY.
 *
 * The reference has no directional-light, bilinear, trilinear, normal-map or
 * PCF shaders; these are new plugins in the style of its DEF01/DEF03/DEF05
 * processors (tex1light1.cpp, tex1bump1light1.cpp, shadow.cpp).  Their maths
 * is the shared CPU definition in ../shade_ref.h.  They write colour with
 * write4 (fragthrd.cpp:70-81), so BEHAVIOR_ALPHABLEND blends (blend4).
 *
 *   VertexProcesserSHADOW   DEF05 (shadow.cpp:21-29) without the x0.9 scale
 *   FragmentProcessorLIT1   DEF01 varyings, bilinear albedo, Blinn-Phong s=32
 *   FragmentProcessorLIT1A  LIT1 with an alpha test (discard) and the texture's alpha
 *   FragmentProcessorLIT3   LIT1 with a trilinear mip chain
 *   VertexProcesserLIT2 / InterpolationProcessorLIT2 / FragmentProcessorLIT2
 *                           normal-mapped, trilinear, 3x3-PCF-shadowed shader
 *
 * Uniform slots follow the reference convention (tex1light1.cpp:15-20,
 * 145-150): 3 = PV, 4 = M, 5 = Mrot, 7 = light, 8 = camera, 9 = texture; the
 * new slots are 6 = light-space PV, 10 = normal-map chain, 11 = shadow map,
 * 12 = {lodScale, shadowBias, 0, 0}.  A mip chain is passed as int[2]
 * {first texture index, level count}; its levels are consecutive textures.
 */
#include <string.h>
#include "mcemaths.h"
#include "defproc.h"
#include "cfgproc.h"
#include "../shade_ref.h"

static sr_level level_of(const PuresoftFBO* fbo)
{
    sr_level l;
    l.base = (const uint8_t*)fbo->getBuffer();
    l.width = fbo->getWidth();
    l.height = fbo->getHeight();
    l.scanline = fbo->getScanline();
    return l;
}

/* ---- SHADOW: depth-only vertex stage --------------------------------- */
void VertexProcesserSHADOW::preprocess(const PURESOFTUNIFORM* uniforms)
{
    m_PV = (const float*)uniforms[3].data;
    m_M = (const float*)uniforms[4].data;
}

void VertexProcesserSHADOW::process(const VertexProcessorInput* input, VertexProcessorOutput* output) const
{
    ALIGN16 float pvm[16];
    mcemaths_transform_m4m4(pvm, m_PV, m_M);
    mcemaths_transform_m4v4(output->position, pvm, (const float*)input->data[0]);
}

/* ---- LIT1 ----------------------------------------------------------------- */
void FragmentProcessorLIT1::preprocess(const PURESOFTUNIFORM* uniforms, const void** textures)
{
    m_light = (const float*)uniforms[7].data;
    m_camera = (const float*)uniforms[8].data;
    m_tex = (const PuresoftFBO*)textures[*(const int*)uniforms[9].data];
}

void FragmentProcessorLIT1::process(const FragmentProcessorInput* input, FragmentProcessorOutput* output) const
{
    const PROCDATA_DEF01* in = (const PROCDATA_DEF01*)input->user;
    sr_level t = level_of(m_tex);
    uint8_t bgra[4];
    sr_shade_lit1(&t, m_light, m_camera, in->normal, in->worldPos, in->texcoord, bgra);
    output->write4(0, bgra);
}

/* ---- LIT1A: alpha test + texture alpha -------------------------------------- */
void FragmentProcessorLIT1A::preprocess(const PURESOFTUNIFORM* uniforms, const void** textures)
{
    m_light = (const float*)uniforms[7].data;
    m_camera = (const float*)uniforms[8].data;
    m_tex = (const PuresoftFBO*)textures[*(const int*)uniforms[9].data];
}

void FragmentProcessorLIT1A::process(const FragmentProcessorInput* input, FragmentProcessorOutput* output) const
{
    const PROCDATA_DEF01* in = (const PROCDATA_DEF01*)input->user;
    sr_level t = level_of(m_tex);
    uint8_t bgra[4];
    if (sr_shade_lit1a(&t, m_light, m_camera, in->normal, in->worldPos, in->texcoord, bgra)) output->discard();
    else output->write4(0, bgra);
}

/* ---- LIT3 ----------------------------------------------------------------- */
void FragmentProcessorLIT3::preprocess(const PURESOFTUNIFORM* uniforms, const void** textures)
{
    const int* chain = (const int*)uniforms[9].data;
    m_light = (const float*)uniforms[7].data;
    m_camera = (const float*)uniforms[8].data;
    m_levels = chain[1] > PS3DR_MAX_LEVELS ? PS3DR_MAX_LEVELS : chain[1];
    for (int i = 0; i < m_levels; i++) m_chain[i] = level_of((const PuresoftFBO*)textures[chain[0] + i]);
    m_lodScale = ((const float*)uniforms[12].data)[0];
}

void FragmentProcessorLIT3::process(const FragmentProcessorInput* input, FragmentProcessorOutput* output) const
{
    const PROCDATA_DEF01* in = (const PROCDATA_DEF01*)input->user;
    uint8_t bgra[4];
    sr_shade_lit3(m_chain, m_levels, m_lodScale, m_light, m_camera, in->normal, in->worldPos, in->texcoord, bgra);
    output->write4(0, bgra);
}

/* ---- LIT2 ----------------------------------------------------------------- */
void VertexProcesserLIT2::preprocess(const PURESOFTUNIFORM* uniforms)
{
    m_PV = (const float*)uniforms[3].data;
    m_M = (const float*)uniforms[4].data;
    m_Mrot = (const float*)uniforms[5].data;
    m_LPV = (const float*)uniforms[6].data;
}

/* Same structure as DEF01's vertex processor (tex1light1.cpp:22-41), plus the
   tangent and the light-space position. */
void VertexProcesserLIT2::process(const VertexProcessorInput* input, VertexProcessorOutput* output) const
{
    PROCDATA_LIT2* o = (PROCDATA_LIT2*)output->user;
    const float* position = (const float*)input->data[0];
    const float* tangent = (const float*)input->data[1];
    const float* normal = (const float*)input->data[3];
    const float* texcoord = (const float*)input->data[4];
    ALIGN16 float t3[4] = {tangent[0], tangent[1], tangent[2], 0.0f};

    mcemaths_transform_m4v4(o->worldPos, m_M, position);
    mcemaths_quatcpy(output->position, o->worldPos);
    mcemaths_transform_m4v4(o->shadowPos, m_LPV, o->worldPos);
    o->worldPos[3] = 0;
    mcemaths_transform_m4v4_ip(output->position, m_PV);
    mcemaths_transform_m4v4(o->normal, m_Mrot, normal);
    mcemaths_transform_m4v4(o->tangent, m_Mrot, t3);
    o->tangent[3] = tangent[3];
    o->texcoord[0] = texcoord[0];
    o->texcoord[1] = texcoord[1];
    o->texcoord[2] = 0;
    o->texcoord[3] = 0;
}

/* Five float4 varyings handled with the same 4-wide operation order as the
   reference DEF01 interpolation processor (tex1light1.cpp:60-135). */
static const int LIT2_VECS = sizeof(PROCDATA_LIT2) / 16;

size_t InterpolationProcessorLIT2::userDataBytes(void) const { return sizeof(PROCDATA_LIT2); }
void InterpolationProcessorLIT2::preprocess(const PURESOFTUNIFORM*) {}

void InterpolationProcessorLIT2::interpolateByContributes(void* out, const void** vert, const float* c) const
{
    ALIGN16 float t[3][4];
    float* o = (float*)out;
    for (int k = 0; k < LIT2_VECS; k++) {
        for (int v = 0; v < 3; v++) {
            mcemaths_quatcpy(t[v], (const float*)vert[v] + 4 * k);
            mcemaths_mul_3_4(t[v], c[v]);
        }
        mcemaths_quatcpy(o + 4 * k, t[0]);
        mcemaths_add_3_4_ip(o + 4 * k, t[1]);
        mcemaths_add_3_4_ip(o + 4 * k, t[2]);
    }
}

void InterpolationProcessorLIT2::calcStep(void* step, const void* start, const void* end, int stepCount) const
{
    float r = 0 == stepCount ? 1.0f : 1.0f / (float)stepCount;
    for (int k = 0; k < LIT2_VECS; k++) {
        mcemaths_sub_3_4((float*)step + 4 * k, (const float*)end + 4 * k, (const float*)start + 4 * k);
        mcemaths_mul_3_4((float*)step + 4 * k, r);
    }
}

void InterpolationProcessorLIT2::correctInterpolation(void* out, const void* start, float cf2) const
{
    memcpy(out, start, sizeof(PROCDATA_LIT2));
    for (int k = 0; k < LIT2_VECS; k++) mcemaths_mul_3_4((float*)out + 4 * k, cf2);
}

void InterpolationProcessorLIT2::stepForward(void* start, const void* step, int stepCount) const
{
    for (int k = 0; k < LIT2_VECS; k++) {
        if (1 == stepCount) mcemaths_add_3_4_ip((float*)start + 4 * k, (const float*)step + 4 * k);
        else mcemaths_step_3_4_ip((float*)start + 4 * k, (const float*)step + 4 * k, (float)stepCount);
    }
}

void FragmentProcessorLIT2::preprocess(const PURESOFTUNIFORM* uniforms, const void** textures)
{
    const int* albedo = (const int*)uniforms[9].data;
    const int* normal = (const int*)uniforms[10].data;
    const PuresoftFBO* sm = (const PuresoftFBO*)textures[*(const int*)uniforms[11].data];
    const float* params = (const float*)uniforms[12].data;
    m_light = (const float*)uniforms[7].data;
    m_camera = (const float*)uniforms[8].data;
    m_albedoLevels = albedo[1] > PS3DR_MAX_LEVELS ? PS3DR_MAX_LEVELS : albedo[1];
    m_normalLevels = normal[1] > PS3DR_MAX_LEVELS ? PS3DR_MAX_LEVELS : normal[1];
    for (int i = 0; i < m_albedoLevels; i++)
        m_albedo[i] = level_of((const PuresoftFBO*)textures[albedo[0] + i]);
    /* an RGBA16F level is stored as an elemLen-4 FBO twice as wide (the
       reference's FBO supports 1- and 4-byte elements only, fbo.cpp:21-24) */
    for (int i = 0; i < m_normalLevels; i++) {
        m_normal[i] = level_of((const PuresoftFBO*)textures[normal[0] + i]);
        m_normal[i].width /= 2;
    }
    m_shadow = (const float*)sm->getBuffer();
    m_shadowSize = sm->getWidth();
    m_shadowScanlineFloats = sm->getScanline() / 4;
    m_lodScale = params[0];
    m_bias = params[1];
}

void FragmentProcessorLIT2::process(const FragmentProcessorInput* input, FragmentProcessorOutput* output) const
{
    uint8_t bgra[4];
    sr_shade_lit2(m_albedo, m_albedoLevels, m_normal, m_normalLevels, m_shadow, m_shadowSize, m_shadowScanlineFloats,
                  m_lodScale, m_bias, m_light, m_camera, (const float*)input->user, bgra);
    output->write4(0, bgra);
}

PostProcessorADD8::PostProcessorADD8(const unsigned char add[4]) { memcpy(m_add, add, 4); }

void PostProcessorADD8::process(int threadIndex, int threadCount, PuresoftFBO* frame, PuresoftFBO* depth)
{
    (void)depth;
    unsigned char* base = (unsigned char*)frame->getBuffer();
    for (int y = threadIndex; y < frame->getHeight(); y += threadCount) {
        unsigned char* row = base + (size_t)y * frame->getScanline();
        for (int x = 0; x < 4 * frame->getWidth(); x++) row[x] = (unsigned char)(row[x] + m_add[x & 3]);
    }
}

PostProcessorFOG::PostProcessorFOG(unsigned int fog, float nearD, float farD, bool frameTopDown)
    : m_fog(fog), m_near(nearD), m_far(farD), m_topDown(frameTopDown) {}

/* The frame is the display FBO (top-down: pixel row y at memory row H-1-y)
   or, after setFBO, a texture (row y at memory row y); the depth buffer's
   pixel row y is at memory row y. */
void PostProcessorFOG::process(int threadIndex, int threadCount, PuresoftFBO* frame, PuresoftFBO* depth)
{
    unsigned char* cbase = (unsigned char*)frame->getBuffer();
    const unsigned char* dbase = (const unsigned char*)depth->getBuffer();
    const int H = frame->getHeight(), W = frame->getWidth();
    const float range = m_far - m_near;
    for (int y = threadIndex; y < H; y += threadCount) {
        const float* drow = (const float*)(dbase + (size_t)y * depth->getScanline());
        unsigned char* crow = cbase + (size_t)(m_topDown ? H - 1 - y : y) * frame->getScanline();
        for (int x = 0; x < W; x++) {
            float t = (drow[x] - m_near) / range;
            t = t > 0.0f ? t : 0.0f;
            t = t < 1.0f ? t : 1.0f;
            for (int k = 0; k < 3; k++) {
                float c = (float)crow[4 * x + k], f = (float)((m_fog >> (8 * k)) & 0xff);
                crow[4 * x + k] = (unsigned char)(int)(c + (f - c) * t);
            }
        }
    }
}
