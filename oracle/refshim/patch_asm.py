"""Generate asm-free copies of four reference translation units for the
Linux build of the reference pipeline core (oracle/_ref).  TEST
INFRASTRUCTURE ONLY.

The reference's interp.cpp and fbo.cpp, and its demo's processors
(src/test/testproc.cpp), contain MSVC 32-bit ``__asm{}`` blocks, which GCC
cannot compile.  This script reads the files from the read-only reference
tree and writes copies into the build output directory (never into the
repository) in which each ``__asm{...}`` block is replaced by SSE
intrinsics (or a plain copy) issuing the same operations:

* interp.cpp ``interpolateStartAndStep`` (reference interp.cpp:55-66): two
  haddps reductions of the left/right corrected contributions; lane 0 of the
  left and lane 2 of the right are stored to ``temp``.
* fbo.cpp ``clear16`` / ``clearToZero`` (reference fbo.cpp:348-393): fill
  m_bytes/16 16-byte slots of m_buffer with the given vector / zero.
* test/testproc.cpp: the three ``copyUserData`` helpers (6, 4 and 1 aligned
  16-byte moves, testproc.cpp:8-27, 367-381, 578-587) become memcpy of the
  same bytes; FP_Cloud's colour packing (testproc.cpp:565-571: cvtps2dq,
  packusdw, packuswb, movss) becomes the same four intrinsics.
* test2/testproc.cpp (the scene viewer's processors, written as
  testproc2.cpp): ``copyUserDataSingleColour`` and ``copyUserDataDiffuseOnly``
  (3 and 4 aligned 16-byte moves, testproc.cpp:73-86, 287-300) become memcpy.

Everything else in both files is left byte-for-byte unchanged.  Each block is
matched by its own instruction text so that a different reference revision
fails loudly instead of silently compiling something else.

Usage: python patch_asm.py <reference src/puresoft3d dir> <output dir> [<reference src/test dir>
       [<reference src/test2 dir>]]
"""
import os
import re
import sys

INTERP_REPL = """{
\t\t__m128 l = _mm_loadu_ps(correctedContributesForLeft);
\t\tl = _mm_hadd_ps(l, l);
\t\tl = _mm_hadd_ps(l, l);
\t\t__m128 r = _mm_loadu_ps(correctedContributesForLeft + 4);
\t\tr = _mm_hadd_ps(r, r);
\t\tr = _mm_hadd_ps(r, r);
\t\t_mm_storeu_ps(temp, _mm_move_ss(r, l));
\t}"""

CLEAR16_REPL = """{
\t\t__m128 v = _mm_loadu_ps((const float*)dataAligned16Bytes);
\t\tchar* d = (char*)m_buffer;
\t\tfor(size_t i = 0; i < m_bytes / 16; i++) _mm_storeu_ps((float*)(d + 16 * i), v);
\t}"""

CLEARZERO_REPL = """{
\t\t__m128 v = _mm_setzero_ps();
\t\tchar* d = (char*)m_buffer;
\t\tfor(size_t i = 0; i < m_bytes / 16; i++) _mm_storeu_ps((float*)(d + 16 * i), v);
\t}"""


def _asm_blocks(text):
    """Yield (start, end) spans of every ``__asm{ ... }`` block (no nesting)."""
    for m in re.finditer(r"__asm\s*\{", text):
        end = text.index("}", m.end())
        yield m.start(), end + 1


def _patch(text, expect):
    """Replace asm blocks in order; ``expect`` is a list of (needles, repl)."""
    spans = list(_asm_blocks(text))
    if len(spans) != len(expect):
        raise SystemExit("unexpected number of __asm blocks: %d" % len(spans))
    out, pos = [], 0
    for (s, e), (needles, repl) in zip(spans, expect):
        body = text[s:e]
        for n in needles:
            if n not in body:
                raise SystemExit("asm block does not contain %r" % n)
        out.append(text[pos:s])
        out.append(repl)
        pos = e
    out.append(text[pos:])
    return "".join(out)


COPY_REPL = """{
\t\tmemcpy(dest, src, %d);
\t}"""

PACK_REPL = """{
\t\t__m128i v_ = _mm_cvtps_epi32(_mm_load_ps(cloudColour));
\t\tv_ = _mm_packus_epi32(v_, v_);
\t\tv_ = _mm_packus_epi16(v_, v_);
\t\t_mm_store_ss(cloudColour, _mm_castsi128_ps(v_));
\t}"""


def main(src_dir, out_dir, test_dir=None, test2_dir=None):
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(src_dir, "interp.cpp"), encoding="latin-1") as f:
        interp = f.read()
    interp = _patch(interp, [(["haddps", "movss\txmm1,\txmm0", "[eax + 16]"], INTERP_REPL)])
    interp = "#include <pmmintrin.h>\n" + interp
    with open(os.path.join(out_dir, "interp.cpp"), "w", encoding="latin-1") as f:
        f.write(interp)

    with open(os.path.join(src_dir, "fbo.cpp"), encoding="latin-1") as f:
        fbo = f.read()
    fbo = _patch(fbo, [(["movaps\txmm0,\t[eax]", "loop\tlup"], CLEAR16_REPL),
                       (["xorps\txmm0, xmm0", "loop\tlup"], CLEARZERO_REPL)])
    fbo = "#include <pmmintrin.h>\n" + fbo
    with open(os.path.join(out_dir, "fbo.cpp"), "w", encoding="latin-1") as f:
        f.write(fbo)

    if test_dir:
        with open(os.path.join(test_dir, "testproc.cpp"), encoding="latin-1") as f:
            tp = f.read()
        tp = _patch(tp, [(["[eax + 80]", "movaps\t[eax + 80]"], COPY_REPL % 96),
                         (["[eax + 48]", "movaps\t[eax + 48],\txmm3"], COPY_REPL % 64),
                         (["cvtps2dq", "packusdw", "packuswb", "movss"], PACK_REPL),
                         (["movaps\txmm0,\t\t[eax]", "movaps\t[eax],\t\txmm0"], COPY_REPL % 16)])
        tp = "#include <smmintrin.h>\n#include <string.h>\n" + tp
        with open(os.path.join(out_dir, "testproc.cpp"), "w", encoding="latin-1") as f:
            f.write(tp)

    if test2_dir:
        with open(os.path.join(test2_dir, "testproc.cpp"), encoding="latin-1") as f:
            tp = f.read()
        tp = _patch(tp, [(["[eax + 32]", "movaps\t[eax + 32],\txmm2"], COPY_REPL % 48),
                         (["[eax + 48]", "movaps\t[eax + 48],\txmm3"], COPY_REPL % 64)])
        tp = "#include <string.h>\n" + tp
        with open(os.path.join(out_dir, "testproc2.cpp"), "w", encoding="latin-1") as f:
            f.write(tp)


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2], sys.argv[3] if len(sys.argv) > 3 else None,
         sys.argv[4] if len(sys.argv) > 4 else None)
