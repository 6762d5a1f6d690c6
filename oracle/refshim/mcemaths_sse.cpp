/*
 * mcemaths_sse.cpp -- the reference's maths library (src/mcemath, MSVC 32-bit
 * inline asm) restated as SSE/SSE3 intrinsics with the same instruction
 * sequence, for the Linux build of the reference pipeline core (oracle/_ref).
 * TEST INFRASTRUCTURE ONLY.
 *
 * Each function issues the same packed operations, in the same order, as the
 * asm block it replaces (file:line in src/mcemath), so results are
 * bit-identical on an x86 host: mulps/addps/subps/haddps/sqrtss are IEEE,
 * rcpps/rsqrtss are the host's approximations exactly as in the original.
 * Only the functions reachable from the compiled pipeline core are provided.
 * Unaligned loads/stores are used; alignment never changes results.
 */
#include <pmmintrin.h>
#include <string.h>
#include "mcemaths.h"

static inline __m128 ld(const float* p) { return _mm_loadu_ps(p); }
static inline void st(float* p, __m128 v) { _mm_storeu_ps(p, v); }
static inline __m128 bc(float f) { return _mm_set1_ps(f); }
static inline float hsum2(__m128 v) /* haddps twice, lane 0: (v0+v1)+(v2+v3) */
{
    v = _mm_hadd_ps(v, v);
    v = _mm_hadd_ps(v, v);
    return _mm_cvtss_f32(v);
}

extern "C" {

/* vector.cpp:4-15 */
void mcemaths_add_3_4(float* r4, const float* a, const float* b) { st(r4, _mm_add_ps(ld(a), ld(b))); }
/* vector.cpp:17-28 */
void mcemaths_sub_3_4(float* r4, const float* a, const float* b) { st(r4, _mm_sub_ps(ld(a), ld(b))); }
/* vector.cpp:30-40 */
void mcemaths_add_3_4_ip(float* a, const float* b) { st(a, _mm_add_ps(ld(a), ld(b))); }
/* vector.cpp:42-52 */
void mcemaths_sub_3_4_ip(float* a, const float* b) { st(a, _mm_sub_ps(ld(a), ld(b))); }
/* vector.cpp:54-68: base + step * n (mulps then addps) */
void mcemaths_step_3_4(float* r4, const float* base4, const float* step4, float n)
{
    st(r4, _mm_add_ps(ld(base4), _mm_mul_ps(ld(step4), bc(n))));
}
/* vector.cpp:70-83 */
void mcemaths_step_3_4_ip(float* t4, const float* step4, float n)
{
    __m128 s = _mm_mul_ps(ld(step4), bc(n));
    st(t4, _mm_add_ps(ld(t4), s));
}
/* vector.cpp:85-112: mulps + haddps x2 */
float mcemaths_dot_3_4(const float* a, const float* b) { return hsum2(_mm_mul_ps(ld(a), ld(b))); }
/* vector.cpp:114-144: a.yzx*b.zxy - a.zxy*b.yzx with the asm's shuffles */
void mcemaths_cross_3(float* r4, const float* l, const float* r)
{
    __m128 a = ld(l), b = ld(r);
    __m128 x0 = _mm_shuffle_ps(a, a, 0xc9);
    __m128 x1 = _mm_shuffle_ps(b, b, 0xd2);
    __m128 x2 = _mm_shuffle_ps(a, a, 0xd2);
    __m128 x3 = _mm_shuffle_ps(b, b, 0xc9);
    st(r4, _mm_sub_ps(_mm_mul_ps(x0, x1), _mm_mul_ps(x2, x3)));
}
/* vector.cpp:146-156 */
void mcemaths_mul_3_4(float* r4, float f) { st(r4, _mm_mul_ps(ld(r4), bc(f))); }
/* vector.cpp:158-169: rcpps of the broadcast factor, then mulps */
void mcemaths_div_3_4(float* r4, float f) { st(r4, _mm_mul_ps(ld(r4), _mm_rcp_ps(bc(f)))); }
/* vector.cpp:171-181 */
void mcemaths_mulvec_3_4(float* r4, const float* f4) { st(r4, _mm_mul_ps(ld(r4), ld(f4))); }
/* vector.cpp:183-194 */
void mcemaths_divvec_3_4(float* r4, const float* f4) { st(r4, _mm_mul_ps(ld(r4), _mm_rcp_ps(ld(f4)))); }
/* vector.cpp:196-223: mulps, haddps x2, sqrtss */
float mcemaths_len_3_4(const float* v4)
{
    __m128 v = ld(v4);
    v = _mm_mul_ps(v, v);
    v = _mm_hadd_ps(v, v);
    v = _mm_hadd_ps(v, v);
    return _mm_cvtss_f32(_mm_sqrt_ss(v));
}
/* vector.cpp:225-250: v * broadcast(rsqrtss(hsum(v*v))) */
void mcemaths_norm_3_4(float* v4)
{
    __m128 v = ld(v4);
    __m128 s = _mm_mul_ps(v, v);
    s = _mm_hadd_ps(s, s);
    s = _mm_hadd_ps(s, s);
    s = _mm_rsqrt_ss(s);
    s = _mm_shuffle_ps(s, s, 0x00);
    st(v4, _mm_mul_ps(v, s));
}
/* vector.cpp:252-279 */
void mcemaths_set_vec_ary(float* ary4, int count, const float* v4)
{
    for (int i = 0; i < (count < 1 ? 1 : count); i++) memcpy(ary4 + 4 * i, v4, 16);
}
/* vector.cpp:281-306 (count == 1 writes one vector; the loop form is do-while) */
void mcemaths_zero_vec_ary(float* ary4, int count)
{
    for (int i = 0; i < (count < 1 ? 1 : count); i++) memset(ary4 + 4 * i, 0, 16);
}
/* vector.cpp:370-383: maxps with min, then minps with max */
void mcemaths_clamp_3_4(float* v4, float mn, float mx)
{
    st(v4, _mm_min_ps(_mm_max_ps(ld(v4), bc(mn)), bc(mx)));
}
/* vector.cpp:517-534 (plain C in the reference) */
void mcemaths_mul_3(float* r4, float fac)
{
    r4[0] *= fac;
    r4[1] *= fac;
    r4[2] *= fac;
}
/* vector.cpp:557-567 */
void mcemaths_add_1to4(float* r4, float a) { st(r4, _mm_add_ps(ld(r4), bc(a))); }
/* vector.cpp:569-579 */
void mcemaths_sub_4by1(float* r4, float a) { st(r4, _mm_sub_ps(ld(r4), bc(a))); }
/* quatern.cpp:9-17 */
void mcemaths_quatcpy(float* d, const float* s) { memcpy(d, s, 16); }
/* matrix.cpp:304-318 */
void mcemaths_mat4cpy(float* d, const float* s) { memcpy(d, s, 64); }
/* matrix.cpp:20-55 */
void mcemaths_mat4transpose(float* m)
{
    __m128 r0 = ld(m), r1 = ld(m + 4), r2 = ld(m + 8), r3 = ld(m + 12);
    _MM_TRANSPOSE4_PS(r0, r1, r2, r3);
    st(m, r0);
    st(m + 4, r1);
    st(m + 8, r2);
    st(m + 12, r3);
}
/* matrix.cpp:992-1008: columns t, b, n, 0 */
void mcemaths_make_tbn(float* m44, const float* t, const float* b, const float* n)
{
    memcpy(m44, t, 16);
    memcpy(m44 + 4, b, 16);
    memcpy(m44 + 8, n, 16);
    memset(m44 + 12, 0, 16);
}

/* matrix.cpp:515-557: ((x*c0 + y*c1) + z*c2) + w*c3, column-major */
static inline __m128 m4v4(const float* m, __m128 v)
{
    __m128 x = _mm_shuffle_ps(v, v, 0x00), y = _mm_shuffle_ps(v, v, 0x55);
    __m128 z = _mm_shuffle_ps(v, v, 0xaa), w = _mm_shuffle_ps(v, v, 0xff);
    x = _mm_mul_ps(x, ld(m));
    y = _mm_mul_ps(y, ld(m + 4));
    z = _mm_mul_ps(z, ld(m + 8));
    w = _mm_mul_ps(w, ld(m + 12));
    return _mm_add_ps(_mm_add_ps(_mm_add_ps(x, y), z), w);
}
void mcemaths_transform_m4v4(float* r4, const float* m, const float* v4) { st(r4, m4v4(m, ld(v4))); }
/* matrix.cpp:559-585 */
void mcemaths_transform_m4v4_ip(float* r4, const float* m) { st(r4, m4v4(m, ld(r4))); }
/* matrix.cpp:588-690: each column of r transformed by l */
void mcemaths_transform_m4m4(float* d, const float* l, const float* r)
{
    for (int c = 0; c < 4; c++) st(d + 4 * c, m4v4(l, ld(r + 4 * c)));
}

} /* extern "C" */
