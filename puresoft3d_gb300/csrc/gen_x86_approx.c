/*
 * gen_x86_approx.c -- writes x86_approx.h: the tables behind the x86
 * approximate reciprocal (rcpps, rcpss) and reciprocal square root
 * (rsqrtss) as the host that runs it computes them, and checks the decoder
 * in x86_approx.h against the instructions for every one of the 2^32 inputs.
 *
 * The reference's maths library normalises with these instructions
 * (src/mcemath/vector.cpp:158-169 mcemaths_div_3_4, :225-250
 * mcemaths_norm_3_4), so its shaders' colour depends on the host's
 * implementation of them.  On the host the golden fixtures were made on (an
 * Intel Xeon), probing showed that
 *   - rcpps depends only on the top 11 mantissa bits of its input and
 *     rsqrtss only on the top 10 and the parity of the exponent;
 *   - both results have 12 significant bits and scale exactly with the
 *     input's exponent over the normal range;
 *   - zero and denormal inputs give infinity, infinite inputs zero, and a
 *     result below the normal range is flushed to zero.
 * A table of 2048 entries for each therefore reproduces them bit for bit.
 * Other x86 implementations (other vendors' cores) can give other values;
 * regenerate the tables on the host whose reference output is the target.
 *
 * Build and run on an x86-64 host (from the repository root):
 *   gcc -O2 -msse2 -o /tmp/gen puresoft3d_gb300/csrc/gen_x86_approx.c
 *   /tmp/gen > /tmp/x86_approx.h
 *   gcc -O2 -msse2 -DX86_APPROX_HEADER='"/tmp/x86_approx.h"' -o /tmp/check \
 *       puresoft3d_gb300/csrc/gen_x86_approx.c && /tmp/check --check
 * then move /tmp/x86_approx.h to puresoft3d_gb300/csrc/x86_approx.h.  The
 * check includes the generated decoder and compares it with the
 * instructions on all 2^32 inputs of each (about 20 s).
 */
#include <immintrin.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static float f_of(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static uint32_t u_of(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static uint32_t hw_rcp(uint32_t u) { return u_of(_mm_cvtss_f32(_mm_rcp_ss(_mm_set_ss(f_of(u))))); }
static uint32_t hw_rsqrt(uint32_t u) { return u_of(_mm_cvtss_f32(_mm_rsqrt_ss(_mm_set_ss(f_of(u))))); }

/* Entry: the result's 12 significant mantissa bits (bits 0-11) and how many
   binades its exponent lies below 1.0's (bits 12 and up). */
static unsigned entry(uint32_t r, int top)
{
    const int e = (int)((r >> 23) & 0xff);
    return ((unsigned)(top - e) << 12) | ((r >> 11) & 0xfffu);
}

#ifdef X86_APPROX_HEADER
#include X86_APPROX_HEADER
static int check(void)
{
    unsigned long long bad = 0;
    for (uint64_t i = 0; i < (1ull << 32); i++) {
        const uint32_t u = (uint32_t)i;
        const uint32_t a = hw_rcp(u), b = x86a_rcp_bits(u);
        const uint32_t c = hw_rsqrt(u), d = x86a_rsqrt_bits(u);
        if (a != b) {
            if (bad < 8) fprintf(stderr, "rcp %08x: hw %08x table %08x\n", u, a, b);
            bad++;
        }
        if (c != d) {
            if (bad < 8) fprintf(stderr, "rsqrt %08x: hw %08x table %08x\n", u, c, d);
            bad++;
        }
    }
    printf("%llu mismatches over 2^32 inputs of each\n", bad);
    return bad != 0;
}
#endif

int main(int argc, char** argv)
{
    if (argc > 1 && !strcmp(argv[1], "--check")) {
#ifdef X86_APPROX_HEADER
        return check();
#else
        fprintf(stderr, "rebuild with -DX86_APPROX_HEADER='\"path\"' to check a table header\n");
        return 2;
#endif
    }
    unsigned rcp[2048], rsq[2048];
    for (unsigned i = 0; i < 2048; i++) {  /* inputs 1.m, m = i << 12: results in (0.5, 1] */
        rcp[i] = entry(hw_rcp((127u << 23) | (i << 12)), 127);
    }
    for (unsigned p = 0; p < 2; p++)  /* inputs 1.m x 2^p, m = i << 13: results in (0.5, 1] */
        for (unsigned i = 0; i < 1024; i++) rsq[p * 1024 + i] = entry(hw_rsqrt(((127u + p) << 23) | (i << 13)), 127);
    printf("/* x86_approx.h -- generated by gen_x86_approx.c on an x86-64 host; do not edit.\n"
           " *\n"
           " * The host's rcpps / rcpss and rsqrtss, bit for bit: x86a_rcp_bits and\n"
           " * x86a_rsqrt_bits map the bits of a float to the bits of the instruction's\n"
           " * result.  Table entries, for input 1.m (the reciprocal, m = index << 12)\n"
           " * or 1.m x 2^p (the square root, p = index / 1024, m = (index %% 1024) << 13):\n"
           " * bits 0-11 the result's top 12 mantissa bits, bits 12 and up how many\n"
           " * binades its exponent lies below 1.0's.  Checked against the instructions on\n"
           " * all 2^32 inputs of each.  Usable from C and from CUDA device code. */\n");
    printf("#pragma once\n#include <stdint.h>\n\n");
    printf("#if defined(__CUDACC__)\n#define X86A_FN __device__ __forceinline__\n"
           "#define X86A_TABLE static __device__ const\n#else\n#define X86A_FN static inline\n"
           "#define X86A_TABLE static const\n#endif\n\n");
    printf("X86A_TABLE uint16_t x86a_rcp_tab[2048] = {");
    for (unsigned i = 0; i < 2048; i++) printf("%s0x%04x", i % 12 ? ", " : (i ? ",\n    " : "\n    "), rcp[i]);
    printf("};\n\n");
    printf("X86A_TABLE uint16_t x86a_rsq_tab[2048] = {");
    for (unsigned i = 0; i < 2048; i++) printf("%s0x%04x", i % 12 ? ", " : (i ? ",\n    " : "\n    "), rsq[i]);
    printf("};\n\n");
    printf("#if defined(__CUDACC__)\n#define X86A_LD(t, i) __ldg(&(t)[i])\n#else\n#define X86A_LD(t, i) ((t)[i])\n"
           "#endif\n\n");
    printf("/* rcpps of one lane */\n"
           "X86A_FN uint32_t x86a_rcp_bits(uint32_t u)\n{\n"
           "    const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;\n"
           "    if (e == 0xffu) return m ? (u | 0x400000u) : sign;  /* NaN stays (quiet); 1/inf = 0 */\n"
           "    if (e == 0u) return sign | 0x7f800000u;            /* zero and denormals: infinity */\n"
           "    const uint32_t t = X86A_LD(x86a_rcp_tab, m >> 12);\n"
           "    const int re = 127 - (int)(t >> 12) + 127 - (int)e;\n"
           "    if (re <= 0) return sign;                          /* below the normal range: zero */\n"
           "    return sign | ((uint32_t)re << 23) | ((t & 0xfffu) << 11);\n}\n\n");
    printf("/* rsqrtss */\n"
           "X86A_FN uint32_t x86a_rsqrt_bits(uint32_t u)\n{\n"
           "    const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;\n"
           "    if (e == 0xffu) return m ? (u | 0x400000u) : (sign ? 0xffc00000u : 0u);\n"
           "    if (e == 0u) return sign | 0x7f800000u;            /* zero and denormals: infinity */\n"
           "    if (sign) return 0xffc00000u;                      /* negative: the default NaN */\n"
           "    const int E = (int)e - 127, par = E & 1;\n"
           "    const uint32_t t = X86A_LD(x86a_rsq_tab, (uint32_t)par * 1024u + (m >> 13));\n"
           "    const int re = 127 - (int)(t >> 12) - (E - par) / 2;\n"
           "    return ((uint32_t)re << 23) | ((t & 0xfffu) << 11);\n}\n");
    return 0;
}
