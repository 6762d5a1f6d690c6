// vertex_stage.cuh -- the built-in vertex processors (VBO fetch and the
// reference's VertexProcessor::process for each class), shared by the set-up
// kernel (positions, and the varyings of triangles that reach a bin) and the
// shade kernel (the varyings of a winning triangle's vertices when a pass
// defers them, PassParams::lazyVary).
#pragma once
#include "device_common.cuh"

namespace ps3d {

// ----------------------------------------------------------------- vertex stage

__device__ __forceinline__ void ld4(const uint8_t* p, float v[4])
{
    const float* f = (const float*)p;
    v[0] = __ldg(f);
    v[1] = __ldg(f + 1);
    v[2] = __ldg(f + 2);
    v[3] = __ldg(f + 3);
}

// The draw's vertex processor on vertex `idx`, in two halves: the clip
// position, needed by every triangle for its cull and set-up, and the
// varyings its interpolation stage carries, computed only for triangles that
// reach a bin (the same operations in the same order as one call would do;
// the world position both halves need is computed in each).
__device__ __forceinline__ void vp_position(const DrawDesc& d, const DrawUniforms& U, int idx, float pos[4])
{
    float p[4];
    ld4(d.vbo[0] + (size_t)idx * d.stride[0], p);
    switch (d.vp) {
    case VP_DEF01:   // tex1light1.cpp:22-41
    case VP_DEF02:   // colr1light1.cpp:22-40
    case VP_DEF03:   // tex1bump1light1.cpp:22-46
    case VP_LIT2:
    case VP_CLOUD:     // test/testproc.cpp:392-425
    case VP_PLANET: {  // test/testproc.cpp:37-71
        float wp[4];
        m4v4(wp, U.M, p);
        m4v4(pos, U.PV, wp);
        break;
    }
    case VP_DEF04:  // skybox.cpp:23-44: the position passes through
        pos[0] = p[0]; pos[1] = p[1]; pos[2] = p[2]; pos[3] = p[3];
        break;
    case VP_DEF05: {  // shadow.cpp:21-29: positions x0.9 (mcemaths_mul_3), then (PV*M) * p
        float a[4] = {fmul(p[0], 0.9f), fmul(p[1], 0.9f), fmul(p[2], 0.9f), p[3]};
        m4v4(pos, U.PVM, a);
        break;
    }
    case VP_CLOUDSHADOW: {  // test/testproc.cpp:595-610: positions x0.95, then (PV*M) * p
        float a[4] = {fmul(p[0], 0.95f), fmul(p[1], 0.95f), fmul(p[2], 0.95f), p[3]};
        m4v4(pos, U.PVM, a);
        break;
    }
    case VP_SHADOW2: {  // test2/testproc.cpp:507-518: positions x0.9, then PVM (uniform 5) * p
        float a[4] = {fmul(p[0], 0.9f), fmul(p[1], 0.9f), fmul(p[2], 0.9f), p[3]};
        m4v4(pos, U.PVM, a);
        break;
    }
    case VP_POSITIONONLY:  // test2/testproc.cpp:13-23
    case VP_SINGLECOLOUR:  // test2/testproc.cpp:88-116
    case VP_DIFFUSEONLY:   // test2/testproc.cpp:304-336: PVM (uniform 5) * the model position
    case VP_SHADOW:
        m4v4(pos, U.PVM, p);
        break;
    default:
        pos[0] = pos[1] = pos[2] = pos[3] = 0.0f;
    }
}

// VPK: the vertex processor every draw using this code runs (a kernel
// compiled for one keeps only its registers), 0 = the draw's own.
template <int VPK = 0>
__device__ __forceinline__ void vp_varyings(const DrawDesc& d, const DrawUniforms& U, int idx, float* vary)
{
    float p[4];
    ld4(d.vbo[0] + (size_t)idx * d.stride[0], p);
    switch (VPK ? VPK : d.vp) {
    case VP_DEF01: {  // tex1light1.cpp:22-41
        float wp[4], n[4], nrm[4];
        m4v4(wp, U.M, p);
        ld4(d.vbo[3] + (size_t)idx * d.stride[3], n);
        m4v4(nrm, U.Mrot, n);
        const float* uv = (const float*)(d.vbo[4] + (size_t)idx * d.stride[4]);
        vary[0] = nrm[0]; vary[1] = nrm[1]; vary[2] = nrm[2]; vary[3] = nrm[3];
        vary[4] = wp[0]; vary[5] = wp[1]; vary[6] = wp[2];
        vary[7] = __ldg(uv); vary[8] = __ldg(uv + 1);
        break;
    }
    case VP_DEF02: {  // colr1light1.cpp:22-40: normal in VBO 1, colour in VBO 2
        float wp[4], n[4], nrm[4], c[4];
        m4v4(wp, U.M, p);
        ld4(d.vbo[1] + (size_t)idx * d.stride[1], n);
        ld4(d.vbo[2] + (size_t)idx * d.stride[2], c);
        m4v4(nrm, U.Mrot, n);
        vary[0] = nrm[0]; vary[1] = nrm[1]; vary[2] = nrm[2]; vary[3] = nrm[3];
        vary[4] = wp[0]; vary[5] = wp[1]; vary[6] = wp[2];
        vary[7] = c[0]; vary[8] = c[1]; vary[9] = c[2]; vary[10] = c[3];
        break;
    }
    case VP_DEF04: {  // skybox.cpp:23-44: the direction is Vrot times the
                      // normalised vector from the observer (0, 0, 1) to the vertex
        float v[4] = {fsub(p[0], 0.0f), fsub(p[1], 0.0f), fsub(p[2], 1.0f), 0.0f}, dir[4];
        float r = norm_scale(v);  // mcemaths_norm_3_4: rsqrtss
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = fmul(v[k], r);
        m4v4(dir, U.Vrot, v);
        vary[0] = dir[0]; vary[1] = dir[1]; vary[2] = dir[2];
        break;
    }
    case VP_PLANET: {  // test/testproc.cpp:37-71: DEF03's outputs plus the world
                       // position through the shadow projection
        float wp[4], v[4], o[4], sc[4];
        m4v4(wp, U.M, p);
        m4v4(sc, U.LPV, wp);
#pragma unroll
        for (int k = 0; k < 3; k++) {  // tangent, binormal, normal: Mrot on all four lanes
            ld4(d.vbo[1 + k] + (size_t)idx * d.stride[1 + k], v);
            m4v4(o, U.Mrot, v);
            vary[4 * k] = o[0]; vary[4 * k + 1] = o[1]; vary[4 * k + 2] = o[2]; vary[4 * k + 3] = o[3];
        }
        const float* uv = (const float*)(d.vbo[4] + (size_t)idx * d.stride[4]);
        vary[12] = wp[0]; vary[13] = wp[1]; vary[14] = wp[2];
        vary[15] = __ldg(uv); vary[16] = __ldg(uv + 1);
        vary[17] = sc[0]; vary[18] = sc[1]; vary[19] = sc[2]; vary[20] = sc[3];
        break;
    }
    case VP_CLOUD: {  // test/testproc.cpp:392-425: normal (Mrot, four lanes), world
                      // position xyz, uv, the world position through the shadow projection
        float wp[4], n[4], nrm[4], sc[4];
        m4v4(wp, U.M, p);
        m4v4(sc, U.LPV, wp);
        ld4(d.vbo[3] + (size_t)idx * d.stride[3], n);
        m4v4(nrm, U.Mrot, n);
        const float* uv = (const float*)(d.vbo[4] + (size_t)idx * d.stride[4]);
        vary[0] = nrm[0]; vary[1] = nrm[1]; vary[2] = nrm[2]; vary[3] = nrm[3];
        vary[4] = wp[0]; vary[5] = wp[1]; vary[6] = wp[2];
        vary[7] = __ldg(uv); vary[8] = __ldg(uv + 1);
        vary[9] = sc[0]; vary[10] = sc[1]; vary[11] = sc[2]; vary[12] = sc[3];
        break;
    }
    case VP_SINGLECOLOUR:   // test2/testproc.cpp:88-116: normal (MR, four lanes), world
                            // position xyz, the world position through the shadow projection
    case VP_DIFFUSEONLY: {  // test2/testproc.cpp:304-336: the same with the uv before the shadow coordinate
        float wp[4], n[4], nrm[4], sc[4];
        m4v4(wp, U.M, p);
        m4v4(sc, U.LPV, wp);
        ld4(d.vbo[3] + (size_t)idx * d.stride[3], n);
        m4v4(nrm, U.Mrot, n);
        vary[0] = nrm[0]; vary[1] = nrm[1]; vary[2] = nrm[2]; vary[3] = nrm[3];
        vary[4] = wp[0]; vary[5] = wp[1]; vary[6] = wp[2];
        int o = 7;
        if (d.vp == VP_DIFFUSEONLY) {
            const float* uv = (const float*)(d.vbo[4] + (size_t)idx * d.stride[4]);
            vary[7] = __ldg(uv); vary[8] = __ldg(uv + 1);
            o = 9;
        }
        vary[o] = sc[0]; vary[o + 1] = sc[1]; vary[o + 2] = sc[2]; vary[o + 3] = sc[3];
        break;
    }
    case VP_CLOUDSHADOW: {  // test/testproc.cpp:595-610: uv only
        const float* uv = (const float*)(d.vbo[4] + (size_t)idx * d.stride[4]);
        vary[0] = __ldg(uv); vary[1] = __ldg(uv + 1);
        break;
    }
    case VP_DEF03: {  // tex1bump1light1.cpp:22-46
        float wp[4], v[4], o[4];
        m4v4(wp, U.M, p);
#pragma unroll
        for (int k = 0; k < 3; k++) {  // tangent, binormal, normal: Mrot on all four lanes
            ld4(d.vbo[1 + k] + (size_t)idx * d.stride[1 + k], v);
            m4v4(o, U.Mrot, v);
            vary[4 * k] = o[0]; vary[4 * k + 1] = o[1]; vary[4 * k + 2] = o[2]; vary[4 * k + 3] = o[3];
        }
        const float* uv = (const float*)(d.vbo[4] + (size_t)idx * d.stride[4]);
        vary[12] = wp[0]; vary[13] = wp[1]; vary[14] = wp[2];
        vary[15] = __ldg(uv); vary[16] = __ldg(uv + 1);
        break;
    }
    case VP_LIT2: {
        float wp[4], sp[4], n[4], nrm[4], t[4], tan[4];
        m4v4(wp, U.M, p);
        m4v4(sp, U.LPV, wp);
        ld4(d.vbo[3] + (size_t)idx * d.stride[3], n);
        ld4(d.vbo[1] + (size_t)idx * d.stride[1], t);
        float t3[4] = {t[0], t[1], t[2], 0.0f};
        m4v4(nrm, U.Mrot, n);
        m4v4(tan, U.Mrot, t3);
        const float* uv = (const float*)(d.vbo[4] + (size_t)idx * d.stride[4]);
        vary[0] = nrm[0]; vary[1] = nrm[1]; vary[2] = nrm[2];
        vary[3] = tan[0]; vary[4] = tan[1]; vary[5] = tan[2]; vary[6] = t[3];
        vary[7] = wp[0]; vary[8] = wp[1]; vary[9] = wp[2];
        vary[10] = __ldg(uv); vary[11] = __ldg(uv + 1);
        vary[12] = sp[0]; vary[13] = sp[1]; vary[14] = sp[2]; vary[15] = sp[3];
        break;
    }
    default:
        break;
    }
}

}  // namespace ps3d
