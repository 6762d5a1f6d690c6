/* cfgproc.h -- declarations of the scene-shader processors for the Linux
   build of the reference pipeline core (oracle/_ref).  TEST INFRASTRUCTURE
   ONLY.  See cfgproc.cpp. */
#pragma once
#include "proc.h"
#include "fbo.h"
#include "../shade_ref.h"

#define PS3DR_MAX_LEVELS 16

struct PROCDATA_LIT2 {
    float normal[4];
    float tangent[4];
    float worldPos[4];
    float texcoord[4];
    float shadowPos[4];
};

class VertexProcesserSHADOW : public PuresoftVertexProcessor
{
public:
    void preprocess(const PURESOFTUNIFORM* uniforms);
    void process(const VertexProcessorInput* input, VertexProcessorOutput* output) const;

private:
    const float* m_PV;
    const float* m_M;
};

class FragmentProcessorLIT1 : public PuresoftFragmentProcessor
{
public:
    void preprocess(const PURESOFTUNIFORM* uniforms, const void** textures);
    void process(const FragmentProcessorInput* input, FragmentProcessorOutput* output) const;

private:
    const float* m_light;
    const float* m_camera;
    const PuresoftFBO* m_tex;
};

class FragmentProcessorLIT1A : public PuresoftFragmentProcessor
{
public:
    void preprocess(const PURESOFTUNIFORM* uniforms, const void** textures);
    void process(const FragmentProcessorInput* input, FragmentProcessorOutput* output) const;

private:
    const float* m_light;
    const float* m_camera;
    const PuresoftFBO* m_tex;
};

class FragmentProcessorLIT3 : public PuresoftFragmentProcessor
{
public:
    void preprocess(const PURESOFTUNIFORM* uniforms, const void** textures);
    void process(const FragmentProcessorInput* input, FragmentProcessorOutput* output) const;

private:
    const float* m_light;
    const float* m_camera;
    sr_level m_chain[PS3DR_MAX_LEVELS];
    int m_levels;
    float m_lodScale;
};

class VertexProcesserLIT2 : public PuresoftVertexProcessor
{
public:
    void preprocess(const PURESOFTUNIFORM* uniforms);
    void process(const VertexProcessorInput* input, VertexProcessorOutput* output) const;

private:
    const float* m_PV;
    const float* m_M;
    const float* m_Mrot;
    const float* m_LPV;
};

class InterpolationProcessorLIT2 : public PuresoftInterpolationProcessor
{
public:
    size_t userDataBytes(void) const;
    void preprocess(const PURESOFTUNIFORM* uniforms);
    void interpolateByContributes(void* interpolatedUserData, const void** vertexUserData,
                                  const float* correctedContributes) const;
    void calcStep(void* interpolatedUserDataStep, const void* interpolatedUserDataStart,
                  const void* interpolatedUserDataEnd, int stepCount) const;
    void correctInterpolation(void* interpolatedUserData, const void* interpolatedUserDataStart,
                              float correctionFactor2) const;
    void stepForward(void* interpolatedUserDataStart, const void* interpolatedUserDataStep, int stepCount) const;
};

class FragmentProcessorLIT2 : public PuresoftFragmentProcessor
{
public:
    void preprocess(const PURESOFTUNIFORM* uniforms, const void** textures);
    void process(const FragmentProcessorInput* input, FragmentProcessorOutput* output) const;

private:
    const float* m_light;
    const float* m_camera;
    sr_level m_albedo[PS3DR_MAX_LEVELS];
    sr_level m_normal[PS3DR_MAX_LEVELS];
    int m_albedoLevels, m_normalLevels;
    const float* m_shadow;
    int m_shadowSize, m_shadowScanlineFloats;
    float m_lodScale, m_bias;
};

/* Post-processors for PuresoftPipeline::postProcess (post.cpp, proc.h:88-94):
   the demo's per-byte add (test2/testpost.cpp:9-43, MMX paddb, restated per
   byte) and a linear depth fog; each thread takes rows threadIndex,
   threadIndex + threadCount, ... as the demo does. */
class PostProcessorADD8 : public PuresoftPostProcessor
{
public:
    explicit PostProcessorADD8(const unsigned char add[4]);
    void process(int threadIndex, int threadCount, PuresoftFBO* frame, PuresoftFBO* depth);

private:
    unsigned char m_add[4];
};

class PostProcessorFOG : public PuresoftPostProcessor
{
public:
    PostProcessorFOG(unsigned int fog, float nearD, float farD, bool frameTopDown = true);
    void process(int threadIndex, int threadCount, PuresoftFBO* frame, PuresoftFBO* depth);

private:
    unsigned int m_fog;
    float m_near, m_far;
    bool m_topDown;
};
