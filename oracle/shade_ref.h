/*
 * shade_ref.h -- CPU definition of the shading and sampling used by the
 * benchmark scenes.  TEST INFRASTRUCTURE: included only by the oracle port
 * (ps3d_oracle.c) and by the config processors of the reference build
 * (refshim/cfgproc.cpp).  The product (puresoft3d_gb300/csrc) has its own,
 * independent CUDA implementation that is checked against this one.
 *
 * The reference (CallMeZhou/Puresoft3D) samples textures nearest-only
 * (src/puresoft3d/samplr2d.cpp:19-25) and has no mipmaps, no bilinear, no
 * PCF and no directional light.  The scene shaders are therefore new plugins
 * written against the reference's processor API (src/puresoft3d/proc.h:26-71).
 * They keep the reference's texel addressing rules:
 *   - texel i is centred on coordinate i: the nearest sampler reads
 *     (unsigned)(size * t + 0.5f)  (samplr2d.cpp:19-25);
 *   - WRAP maps an index i to i % (size - 1), plus (size - 1) when negative
 *     (fbo.cpp:580-591) -- the modulus is size - 1, so texel size-1 is never
 *     read; CLAMP clamps to [0, size - 1] (fbo.cpp:556-579);
 *   - texture rows are stored bottom-up from the FBO base (topDown = false,
 *     tex.cpp:17, fbo.cpp:103-106).
 * Every float operation below is IEEE single precision, evaluated in the
 * written order with no FMA contraction (compile with -ffp-contract=off).
 */
#ifndef PS3D_SHADE_REF_H
#define PS3D_SHADE_REF_H

#include <stdint.h>
#include <string.h>
#include <math.h>
#include <limits.h>

#ifdef __cplusplus
extern "C" {
#endif

/* x86 cvttss2si: truncation toward zero; NaN and out-of-range give INT_MIN.
   The reference's (int) casts compile to this instruction on x86; spelling it
   out keeps the oracle's results identical on hosts whose float->int cast
   saturates instead (AArch64). */
static inline int sr_f2i(float x)
{
    if (x >= -2147483648.0f && x < 2147483648.0f) return (int)x;
    return INT_MIN;
}

/* GCC x86-64 (unsigned int)(float): converts through a 64-bit signed
   truncation and keeps the low 32 bits; NaN / |x| >= 2^63 give 0.  Used by
   the reference samplers (samplr2d.cpp:19-25, samplrproj.cpp:29-30). */
static inline unsigned int sr_f2u(float x)
{
    if (x >= -9223372036854775808.0f && x < 9223372036854775808.0f) return (unsigned int)(uint64_t)(int64_t)x;
    return 0u;
}

static inline float sr_u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t sr_f2bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* IEEE half -> float (exact). */
static inline float sr_half2float(uint16_t h)
{
    uint32_t s = (uint32_t)(h & 0x8000u) << 16, e = (h >> 10) & 0x1fu, m = h & 0x3ffu, bits;
    if (e == 0) {
        if (m == 0) bits = s;
        else {
            e = 113;
            while (!(m & 0x400u)) { m <<= 1; e--; }
            bits = s | (e << 23) | ((m & 0x3ffu) << 13);
        }
    } else if (e == 31) bits = s | 0x7f800000u | (m << 13);
    else bits = s | ((e + 112u) << 23) | (m << 13);
    return sr_u2f(bits);
}

/* Reference WRAP addressing (fbo.cpp:580-591) with modulus size-1; a 1-texel
   dimension (modulus 0, undefined in the reference) maps to index 0. */
static inline int sr_wrap(int i, int size)
{
    int m = size - 1, r;
    if (m <= 0) return 0;
    r = i % m;
    if (r < 0) r += m;
    return r;
}

static inline int sr_clampi(int i, int size)
{
    return i < 0 ? 0 : (i > size - 1 ? size - 1 : i);
}

static inline float sr_dot3(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

/* v /= |v| as v * (1 / sqrt(v.v)); a zero vector stays zero. */
static inline void sr_normalize3(float* v)
{
    float s = sr_dot3(v, v), r;
    if (!(s > 0.0f)) { v[0] = v[1] = v[2] = 0.0f; return; }
    r = 1.0f / sqrtf(s);
    v[0] = v[0] * r;
    v[1] = v[1] * r;
    v[2] = v[2] * r;
}

static inline float sr_pow32(float x)
{
    float x2 = x * x, x4 = x2 * x2, x8 = x4 * x4, x16 = x8 * x8;
    return x16 * x16;
}

/* Truncating 0..255 store of a shaded channel; NaN and negatives give 0. */
static inline uint8_t sr_to_u8(float v)
{
    if (!(v > 0.0f)) return 0;
    if (v > 255.0f) return 255;
    return (uint8_t)(int)v;
}

/* A 2D texture level as the FBO stores it: row r starts at base + r*scanline. */
typedef struct {
    const uint8_t* base;
    int width, height, scanline; /* scanline in bytes */
} sr_level;

/* Bilinear filter of a BGRA8 level with REPEAT (reference WRAP) addressing.
   Sample position (W*u, H*v) in texel units, texel centres on integers. */
static inline void sr_bilinear_bgra8(const sr_level* t, float u, float v, float out[4])
{
    float fx = (float)t->width * u, fy = (float)t->height * v;
    float x0f = floorf(fx), y0f = floorf(fy);
    float ax = fx - x0f, ay = fy - y0f;
    int ix = sr_f2i(x0f), iy = sr_f2i(y0f);
    int c0 = sr_wrap(ix, t->width), c1 = sr_wrap(ix + 1, t->width);
    int r0 = sr_wrap(iy, t->height), r1 = sr_wrap(iy + 1, t->height);
    const uint8_t* p00 = t->base + (size_t)r0 * t->scanline + 4 * c0;
    const uint8_t* p10 = t->base + (size_t)r0 * t->scanline + 4 * c1;
    const uint8_t* p01 = t->base + (size_t)r1 * t->scanline + 4 * c0;
    const uint8_t* p11 = t->base + (size_t)r1 * t->scanline + 4 * c1;
    for (int k = 0; k < 4; k++) {
        float a = (float)p00[k], b = (float)p10[k], c = (float)p01[k], d = (float)p11[k];
        float top = a + (b - a) * ax;
        float bot = c + (d - c) * ax;
        out[k] = top + (bot - top) * ay;
    }
}

/* Same filter for an RGBA16F level (8 bytes per texel). */
static inline void sr_bilinear_rgba16f(const sr_level* t, float u, float v, float out[4])
{
    float fx = (float)t->width * u, fy = (float)t->height * v;
    float x0f = floorf(fx), y0f = floorf(fy);
    float ax = fx - x0f, ay = fy - y0f;
    int ix = sr_f2i(x0f), iy = sr_f2i(y0f);
    int c0 = sr_wrap(ix, t->width), c1 = sr_wrap(ix + 1, t->width);
    int r0 = sr_wrap(iy, t->height), r1 = sr_wrap(iy + 1, t->height);
    const uint16_t* p00 = (const uint16_t*)(t->base + (size_t)r0 * t->scanline) + 4 * c0;
    const uint16_t* p10 = (const uint16_t*)(t->base + (size_t)r0 * t->scanline) + 4 * c1;
    const uint16_t* p01 = (const uint16_t*)(t->base + (size_t)r1 * t->scanline) + 4 * c0;
    const uint16_t* p11 = (const uint16_t*)(t->base + (size_t)r1 * t->scanline) + 4 * c1;
    for (int k = 0; k < 4; k++) {
        float a = sr_half2float(p00[k]), b = sr_half2float(p10[k]);
        float c = sr_half2float(p01[k]), d = sr_half2float(p11[k]);
        float top = a + (b - a) * ax;
        float bot = c + (d - c) * ax;
        out[k] = top + (bot - top) * ay;
    }
}

/* Mip selection from the distance footprint x = dist * lodScale:
   x <= 1 (or NaN) -> level 0, weight 0; otherwise level = floor(log2 x) taken
   from the float exponent and weight = mantissa - 1 (a piecewise-linear
   log2), so selection is exact bit arithmetic on every host. */
static inline void sr_mip_select(float x, int* level, float* weight)
{
    uint32_t bits;
    if (!(x > 1.0f)) { *level = 0; *weight = 0.0f; return; }
    bits = sr_f2bits(x);
    *level = (int)((bits >> 23) & 0xffu) - 127;
    *weight = sr_u2f((bits & 0x7fffffu) | 0x3f800000u) - 1.0f;
}

/* Trilinear blend between two bilinear taps; levels past the chain end use
   the last level alone.  Each level is a texture object of the chain. */
static inline void sr_trilinear(const sr_level* chain, int levels, int half16, int level, float w, float u, float v,
                                float out[4])
{
    float a[4], b[4];
    if (level >= levels - 1) {
        if (half16) sr_bilinear_rgba16f(&chain[levels - 1], u, v, out);
        else sr_bilinear_bgra8(&chain[levels - 1], u, v, out);
        return;
    }
    if (half16) {
        sr_bilinear_rgba16f(&chain[level], u, v, a);
        sr_bilinear_rgba16f(&chain[level + 1], u, v, b);
    } else {
        sr_bilinear_bgra8(&chain[level], u, v, a);
        sr_bilinear_bgra8(&chain[level + 1], u, v, b);
    }
    for (int k = 0; k < 4; k++) out[k] = a[k] + (b[k] - a[k]) * w;
}

/* 3x3 percentage-closer filter on an FP32 shadow map of size S x S (rows
   bottom-up, CLAMP addressing).  shadowPos is the light-space clip position.
   The map was rasterised with the reference's viewport mapping
   x = (S/2) * ndc + S/2 (rasterizer.cpp:73-77) and pixel rounding (int)(x + 0.5f)
   (rasterizer.cpp:100-111); a sample is lit when ndc.z - bias <= stored depth.
   Returns the lit fraction in [0, 1]; outside the light frustum it is 1. */
static inline float sr_pcf3x3(const float* map, int size, int scanlineFloats, const float* sp, float bias)
{
    float rw, nx, ny, nz, half, sx, sy;
    int cx, cy, cnt = 0;
    if (!(sp[3] > 0.0f)) return 1.0f;
    rw = 1.0f / sp[3];
    nx = sp[0] * rw;
    ny = sp[1] * rw;
    nz = sp[2] * rw;
    if (!(nx >= -1.0f && nx <= 1.0f && ny >= -1.0f && ny <= 1.0f)) return 1.0f;
    half = (float)(size / 2);
    sx = half * nx + half;
    sy = half * ny + half;
    cx = sr_f2i(sx + 0.5f);
    cy = sr_f2i(sy + 0.5f);
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
            int r = sr_clampi(cy + dy, size), c = sr_clampi(cx + dx, size);
            float d = map[(size_t)r * scanlineFloats + c];
            if (nz - bias <= d) cnt++;
        }
    return (float)cnt / 9.0f;
}

/* Blinn-Phong with one directional light: the colour equation shared by the
   scene shaders.  albedo is BGRA (0..255), n the unit normal, L the unit
   direction towards the light, E the unit direction towards the eye, vis the
   lit fraction.  Writes BGRA8 with alpha 255. */
static inline void sr_blinn_phong_pre(const float albedo[4], const float* n, const float* L, const float* E,
                                      float vis, float pre[3])
{
    float Hv[3], ndl, ndh, spec, diff, s255;
    Hv[0] = E[0] + L[0];
    Hv[1] = E[1] + L[1];
    Hv[2] = E[2] + L[2];
    sr_normalize3(Hv);
    ndl = sr_dot3(n, L);
    if (ndl < 0.0f) ndl = 0.0f;
    ndh = sr_dot3(n, Hv);
    if (ndh < 0.0f) ndh = 0.0f;
    spec = ndl > 0.0f ? sr_pow32(ndh) : 0.0f;
    diff = 0.15f + 0.85f * (ndl * vis);
    s255 = 127.5f * (spec * vis);
    pre[0] = albedo[0] * diff + s255;
    pre[1] = albedo[1] * diff + s255;
    pre[2] = albedo[2] * diff + s255;
}

static inline void sr_blinn_phong(const float albedo[4], const float* n, const float* L, const float* E, float vis,
                                  float pre[3], uint8_t out[4])
{
    sr_blinn_phong_pre(albedo, n, L, E, vis, pre);
    out[0] = sr_to_u8(pre[0]);
    out[1] = sr_to_u8(pre[1]);
    out[2] = sr_to_u8(pre[2]);
    out[3] = 255;
}

/* Scene shader LIT1 (configs 1 and 4): bilinear REPEAT albedo, directional
   Lambert + Blinn-Phong (shininess 32).  Inputs are the DEF01 varyings
   (reference tex1light1.h:4-9): normal[4], worldPos[4], texcoord[4]. */
static inline void sr_shade_lit1_pre(const sr_level* tex, const float* lightDir, const float* camPos,
                                     const float* normal, const float* worldPos, const float* texcoord, float pre[3],
                                     uint8_t out[4])
{
    float albedo[4], n[3], E[3];
    sr_bilinear_bgra8(tex, texcoord[0], texcoord[1], albedo);
    n[0] = normal[0]; n[1] = normal[1]; n[2] = normal[2];
    sr_normalize3(n);
    E[0] = camPos[0] - worldPos[0];
    E[1] = camPos[1] - worldPos[1];
    E[2] = camPos[2] - worldPos[2];
    sr_normalize3(E);
    sr_blinn_phong(albedo, n, lightDir, E, 1.0f, pre, out);
}

/* Scene shader LIT3 (config 3): LIT1 with a trilinear mip chain. */
static inline void sr_shade_lit3_pre(const sr_level* chain, int levels, float lodScale, const float* lightDir,
                                     const float* camPos, const float* normal, const float* worldPos,
                                     const float* texcoord, float pre[3], uint8_t out[4])
{
    float albedo[4], n[3], E[3], dist, w;
    int level;
    E[0] = camPos[0] - worldPos[0];
    E[1] = camPos[1] - worldPos[1];
    E[2] = camPos[2] - worldPos[2];
    dist = sqrtf(sr_dot3(E, E));
    sr_mip_select(dist * lodScale, &level, &w);
    sr_trilinear(chain, levels, 0, level, w, texcoord[0], texcoord[1], albedo);
    n[0] = normal[0]; n[1] = normal[1]; n[2] = normal[2];
    sr_normalize3(n);
    sr_normalize3(E);
    sr_blinn_phong(albedo, n, lightDir, E, 1.0f, pre, out);
}

/* Scene shader LIT2 (config 2): trilinear albedo, tangent-space normal map
   (RGBA16F chain, same mip selection), 3x3 PCF shadow.  Varyings: normal[4],
   tangent[4] (w = handedness), worldPos[4], texcoord[4], shadowPos[4]. */
static inline void sr_shade_lit2_pre(const sr_level* albedoChain, int albedoLevels, const sr_level* normalChain,
                                     int normalLevels, const float* shadowMap, int shadowSize,
                                     int shadowScanlineFloats, float lodScale, float shadowBias,
                                     const float* lightDir, const float* camPos, const float* varyings, float pre[3],
                                     uint8_t out[4])
{
    const float* nrm = varyings;
    const float* tan = varyings + 4;
    const float* wp = varyings + 8;
    const float* tc = varyings + 12;
    const float* sp = varyings + 16;
    float N[3], T[3], B[3], E[3], nts[4], albedo[4], n[3], dist, w, vis;
    int level;
    N[0] = nrm[0]; N[1] = nrm[1]; N[2] = nrm[2];
    sr_normalize3(N);
    T[0] = tan[0]; T[1] = tan[1]; T[2] = tan[2];
    sr_normalize3(T);
    B[0] = N[1] * T[2] - N[2] * T[1];
    B[1] = N[2] * T[0] - N[0] * T[2];
    B[2] = N[0] * T[1] - N[1] * T[0];
    if (tan[3] < 0.0f) { B[0] = -B[0]; B[1] = -B[1]; B[2] = -B[2]; }
    E[0] = camPos[0] - wp[0];
    E[1] = camPos[1] - wp[1];
    E[2] = camPos[2] - wp[2];
    dist = sqrtf(sr_dot3(E, E));
    sr_mip_select(dist * lodScale, &level, &w);
    sr_trilinear(albedoChain, albedoLevels, 0, level, w, tc[0], tc[1], albedo);
    sr_trilinear(normalChain, normalLevels, 1, level, w, tc[0], tc[1], nts);
    n[0] = (T[0] * nts[0] + B[0] * nts[1]) + N[0] * nts[2];
    n[1] = (T[1] * nts[0] + B[1] * nts[1]) + N[1] * nts[2];
    n[2] = (T[2] * nts[0] + B[2] * nts[1]) + N[2] * nts[2];
    sr_normalize3(n);
    vis = sr_pcf3x3(shadowMap, shadowSize, shadowScanlineFloats, sp, shadowBias);
    sr_normalize3(E);
    sr_blinn_phong(albedo, n, lightDir, E, vis, pre, out);
}

static inline void sr_shade_lit1(const sr_level* tex, const float* lightDir, const float* camPos, const float* normal,
                                 const float* worldPos, const float* texcoord, uint8_t out[4])
{
    float pre[3];
    sr_shade_lit1_pre(tex, lightDir, camPos, normal, worldPos, texcoord, pre, out);
}

static inline void sr_shade_lit3(const sr_level* chain, int levels, float lodScale, const float* lightDir,
                                 const float* camPos, const float* normal, const float* worldPos, const float* texcoord,
                                 uint8_t out[4])
{
    float pre[3];
    sr_shade_lit3_pre(chain, levels, lodScale, lightDir, camPos, normal, worldPos, texcoord, pre, out);
}

static inline void sr_shade_lit2(const sr_level* albedoChain, int albedoLevels, const sr_level* normalChain,
                                 int normalLevels, const float* shadowMap, int shadowSize, int shadowScanlineFloats,
                                 float lodScale, float shadowBias, const float* lightDir, const float* camPos,
                                 const float* varyings, uint8_t out[4])
{
    float pre[3];
    sr_shade_lit2_pre(albedoChain, albedoLevels, normalChain, normalLevels, shadowMap, shadowSize,
                      shadowScanlineFloats, lodScale, shadowBias, lightDir, camPos, varyings, pre, out);
}

/* Scene shader LIT1A: LIT1 with an alpha test and the texture's alpha --
   the albedo's alpha (bilinear, 0..255) below 128 discards the fragment
   (no colour, no depth write: fragthrd.cpp:233-237); otherwise the colour
   is LIT1's with alpha = the albedo's alpha, so ALPHABLEND blends by it.
   Returns 1 when the fragment is discarded. */
static inline int sr_shade_lit1a_pre(const sr_level* tex, const float* lightDir, const float* camPos,
                                     const float* normal, const float* worldPos, const float* texcoord, float pre[3],
                                     uint8_t out[4])
{
    float albedo[4], n[3], E[3];
    sr_bilinear_bgra8(tex, texcoord[0], texcoord[1], albedo);
    if (!(albedo[3] >= 128.0f)) return 1;
    n[0] = normal[0]; n[1] = normal[1]; n[2] = normal[2];
    sr_normalize3(n);
    E[0] = camPos[0] - worldPos[0];
    E[1] = camPos[1] - worldPos[1];
    E[2] = camPos[2] - worldPos[2];
    sr_normalize3(E);
    sr_blinn_phong(albedo, n, lightDir, E, 1.0f, pre, out);
    out[3] = sr_to_u8(albedo[3]);
    return 0;
}

static inline int sr_shade_lit1a(const sr_level* tex, const float* lightDir, const float* camPos, const float* normal,
                                 const float* worldPos, const float* texcoord, uint8_t out[4])
{
    float pre[3];
    return sr_shade_lit1a_pre(tex, lightDir, camPos, normal, worldPos, texcoord, pre, out);
}

/* PuresoftFBO::blend4 (fbo.cpp:208-229), the MMX sequence per channel on
   16-bit lanes: a = the source's alpha; out = sat8(dst + ((sat16(src - dst)
   * a) >> 8)) -- with the unsigned saturating subtract it can only brighten. */
static inline void sr_blend4(uint8_t dst[4], const uint8_t src[4])
{
    unsigned a = src[3];
    for (int k = 0; k < 4; k++) {
        unsigned d = dst[k], sv = src[k];
        unsigned diff = sv > d ? sv - d : 0u;
        unsigned v = (((diff * a) & 0xffffu) >> 8) + d;
        dst[k] = (uint8_t)(v > 255u ? 255u : v);
    }
}

/* ------------------------------------------------------------------------
   FP64 re-shade, for measuring the FP32 shaders' error only: the same
   equations on the same fragment inputs (the FP32 varyings, the same texels
   and shadow map), every operation in double.  Mip selection uses the same
   piecewise-linear log2 (continuous across levels); texel addressing is the
   same floor / wrap / clamp, applied to the double sample position. */

static inline double srd_dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static inline void srd_normalize3(double* v)
{
    double s = srd_dot3(v, v), r;
    if (!(s > 0.0)) { v[0] = v[1] = v[2] = 0.0; return; }
    r = 1.0 / sqrt(s);
    v[0] *= r;
    v[1] *= r;
    v[2] *= r;
}

static inline double srd_texel(const sr_level* t, int half16, int r, int c, int k)
{
    if (half16) return (double)sr_half2float(((const uint16_t*)(t->base + (size_t)r * t->scanline))[4 * c + k]);
    return (double)t->base[(size_t)r * t->scanline + 4 * c + k];
}

static inline void srd_bilinear(const sr_level* t, int half16, double u, double v, double out[4])
{
    double fx = (double)t->width * u, fy = (double)t->height * v;
    double x0f = floor(fx), y0f = floor(fy);
    double ax = fx - x0f, ay = fy - y0f;
    int ix, iy, c0, c1, r0, r1;
    if (!(x0f > -2147483648.0 && x0f < 2147483647.0)) x0f = 0.0;
    if (!(y0f > -2147483648.0 && y0f < 2147483647.0)) y0f = 0.0;
    ix = (int)x0f;
    iy = (int)y0f;
    c0 = sr_wrap(ix, t->width);
    c1 = sr_wrap(ix + 1, t->width);
    r0 = sr_wrap(iy, t->height);
    r1 = sr_wrap(iy + 1, t->height);
    for (int k = 0; k < 4; k++) {
        double a = srd_texel(t, half16, r0, c0, k), b = srd_texel(t, half16, r0, c1, k);
        double c = srd_texel(t, half16, r1, c0, k), d = srd_texel(t, half16, r1, c1, k);
        double top = a + (b - a) * ax, bot = c + (d - c) * ax;
        out[k] = top + (bot - top) * ay;
    }
}

static inline void srd_mip_select(double x, int* level, double* weight)
{
    int e;
    double m;
    if (!(x > 1.0)) { *level = 0; *weight = 0.0; return; }
    m = frexp(x, &e); /* x = m * 2^e, m in [0.5, 1) */
    *level = e - 1;
    *weight = 2.0 * m - 1.0;
}

static inline void srd_trilinear(const sr_level* chain, int levels, int half16, int level, double w, double u,
                                 double v, double out[4])
{
    double a[4], b[4];
    if (level >= levels - 1) {
        srd_bilinear(&chain[levels - 1], half16, u, v, out);
        return;
    }
    srd_bilinear(&chain[level], half16, u, v, a);
    srd_bilinear(&chain[level + 1], half16, u, v, b);
    for (int k = 0; k < 4; k++) out[k] = a[k] + (b[k] - a[k]) * w;
}

static inline double srd_pcf3x3(const float* map, int size, int scanlineFloats, const float* spf, double bias)
{
    double sp[4] = {spf[0], spf[1], spf[2], spf[3]}, rw, nx, ny, nz, half, sx, sy;
    int cx, cy, cnt = 0;
    if (!(sp[3] > 0.0)) return 1.0;
    rw = 1.0 / sp[3];
    nx = sp[0] * rw;
    ny = sp[1] * rw;
    nz = sp[2] * rw;
    if (!(nx >= -1.0 && nx <= 1.0 && ny >= -1.0 && ny <= 1.0)) return 1.0;
    half = (double)(size / 2);
    sx = half * nx + half;
    sy = half * ny + half;
    cx = (int)(sx + 0.5);
    cy = (int)(sy + 0.5);
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
            int r = sr_clampi(cy + dy, size), c = sr_clampi(cx + dx, size);
            if (nz - bias <= (double)map[(size_t)r * scanlineFloats + c]) cnt++;
        }
    return (double)cnt / 9.0;
}

static inline void srd_blinn_phong(const double albedo[4], const double* n, const double* L, const double* E,
                                   double vis, double pre[3])
{
    double Hv[3] = {E[0] + L[0], E[1] + L[1], E[2] + L[2]}, ndl, ndh, spec, diff, s255, x2, x4, x8, x16;
    srd_normalize3(Hv);
    ndl = srd_dot3(n, L);
    if (ndl < 0.0) ndl = 0.0;
    ndh = srd_dot3(n, Hv);
    if (ndh < 0.0) ndh = 0.0;
    x2 = ndh * ndh;
    x4 = x2 * x2;
    x8 = x4 * x4;
    x16 = x8 * x8;
    spec = ndl > 0.0 ? x16 * x16 : 0.0;
    diff = 0.15 + 0.85 * (ndl * vis);
    s255 = 127.5 * (spec * vis);
    for (int k = 0; k < 3; k++) pre[k] = albedo[k] * diff + s255;
}

/* lightDir/camPos/varyings as the FP32 shader receives them. */
static inline void srd_shade_lit13(const sr_level* chain, int levels, int trilinear, double lodScale,
                                   const float* lightDir, const float* camPos, const float* normal,
                                   const float* worldPos, const float* texcoord, double pre[3])
{
    double albedo[4], n[3] = {normal[0], normal[1], normal[2]}, L[3] = {lightDir[0], lightDir[1], lightDir[2]};
    double E[3] = {(double)camPos[0] - worldPos[0], (double)camPos[1] - worldPos[1], (double)camPos[2] - worldPos[2]};
    if (trilinear) {
        int level;
        double w;
        srd_mip_select(sqrt(srd_dot3(E, E)) * lodScale, &level, &w);
        srd_trilinear(chain, levels, 0, level, w, texcoord[0], texcoord[1], albedo);
    } else {
        srd_bilinear(chain, 0, texcoord[0], texcoord[1], albedo);
    }
    srd_normalize3(n);
    srd_normalize3(E);
    srd_blinn_phong(albedo, n, L, E, 1.0, pre);
}

static inline void srd_shade_lit2(const sr_level* albedoChain, int albedoLevels, const sr_level* normalChain,
                                  int normalLevels, const float* shadowMap, int shadowSize, int shadowScanlineFloats,
                                  double lodScale, double shadowBias, const float* lightDir, const float* camPos,
                                  const float* v, double pre[3])
{
    double N[3] = {v[0], v[1], v[2]}, T[3] = {v[4], v[5], v[6]}, B[3], nts[4], albedo[4], n[3], w, vis;
    double L[3] = {lightDir[0], lightDir[1], lightDir[2]};
    double E[3] = {(double)camPos[0] - v[8], (double)camPos[1] - v[9], (double)camPos[2] - v[10]};
    int level;
    srd_normalize3(N);
    srd_normalize3(T);
    B[0] = N[1] * T[2] - N[2] * T[1];
    B[1] = N[2] * T[0] - N[0] * T[2];
    B[2] = N[0] * T[1] - N[1] * T[0];
    if (v[7] < 0.0f) { B[0] = -B[0]; B[1] = -B[1]; B[2] = -B[2]; }
    srd_mip_select(sqrt(srd_dot3(E, E)) * lodScale, &level, &w);
    srd_trilinear(albedoChain, albedoLevels, 0, level, w, v[12], v[13], albedo);
    srd_trilinear(normalChain, normalLevels, 1, level, w, v[12], v[13], nts);
    for (int k = 0; k < 3; k++) n[k] = (T[k] * nts[0] + B[k] * nts[1]) + N[k] * nts[2];
    srd_normalize3(n);
    vis = srd_pcf3x3(shadowMap, shadowSize, shadowScanlineFloats, v + 16, shadowBias);
    srd_normalize3(E);
    srd_blinn_phong(albedo, n, L, E, vis, pre);
}

#ifdef __cplusplus
}
#endif
#endif
