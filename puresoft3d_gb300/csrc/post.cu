// post.cu -- the post-processing hook on the device.
//
// PuresoftPipeline::postProcess (post.cpp:3-19) runs a post-processor's
// process(threadIndex, threadCount, frame, depth) on every fragment thread,
// after all fragment work queued before it, over the display colour buffer
// and the current depth buffer (proc.h:88-94).  Here a post-processor is a
// built-in class (PS3D_PP_*), and the hook is one full-frame kernel launched
// in command order after the passes before it; like every recorded command
// it does nothing once an earlier pass of its launch has failed (the
// failed frame is replayed whole).
//
// Layout: the colour target (FBO slot 0: the display, whose memory row
// H-1-y holds pixel row y, or a texture, row y at y) as its first pixel
// row and a signed row pitch; depth FP32 with row y at y * depthScan.
#include "ps3d_internal.h"
#include "device_common.cuh"

namespace ps3d {

// PS3D_PP_ADD8: a wrapping per-byte add of one BGRA addend to every pixel
// (the paddb of the reference demo's post-processor, test2/testpost.cpp:9-43).
// 16 bytes per thread (4 pixels, SIMD within a register); the ragged end of a
// row, when the width is not a multiple of 4, by single pixels.
__global__ void k_post_add8(uint32_t* row0, int pitch, int width, int height, uint32_t add, const int* status,
                            int seq)
{
    if (pass_failed(status, seq)) return;
    const int y = blockIdx.y;
    const int quads = width >> 2;
    uint32_t* row = row0 + (ptrdiff_t)y * pitch;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < quads + (width & 3); q += gridDim.x * blockDim.x) {
        if (q < quads && (((uintptr_t)row & 15) == 0)) {
            uint4 v = ((uint4*)row)[q];
            v.x = __vadd4(v.x, add);
            v.y = __vadd4(v.y, add);
            v.z = __vadd4(v.z, add);
            v.w = __vadd4(v.w, add);
            ((uint4*)row)[q] = v;
        } else if (q < quads) {
#pragma unroll
            for (int k = 0; k < 4; k++) row[4 * q + k] = __vadd4(row[4 * q + k], add);
        } else {
            int x = 4 * quads + (q - quads);
            row[x] = __vadd4(row[x], add);
        }
    }
}

// PS3D_PP_FOG: linear depth fog.  t = (d - near) / (far - near) clamped to
// [0, 1]; each of B, G, R becomes (unsigned char)(c + (f - c) * t) with the
// fog colour f; alpha is kept.  IEEE operations in this order.
__global__ void k_post_fog(uint32_t* row0, int pitch, int width, int height, const float* depth, int depthScan,
                           uint32_t fog, float nearD, float farD, const int* status, int seq)
{
    if (pass_failed(status, seq)) return;
    const int y = blockIdx.y;
    const float range = fsub(farD, nearD);
    const float* drow = depth + (size_t)y * depthScan;
    uint32_t* crow = row0 + (ptrdiff_t)y * pitch;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < width; x += gridDim.x * blockDim.x) {
        float t = fdiv(fsub(drow[x], nearD), range);
        t = t > 0.0f ? t : 0.0f;  // NaN -> 0
        t = t < 1.0f ? t : 1.0f;
        uint32_t c = crow[x], o = c & 0xff000000u;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float cc = (float)((c >> (8 * k)) & 0xff), ff = (float)((fog >> (8 * k)) & 0xff);
            float v = fadd(cc, fmul(fsub(ff, cc), t));
            o |= ((uint32_t)__float2int_rz(v) & 0xffu) << (8 * k);
        }
        crow[x] = o;
    }
}

static inline int ceil_div_post(int a, int b) { return (a + b - 1) / b; }

void launch_post_add8(uint32_t* row0, int pitch, int width, int height, uint32_t add, const int* status, int seq,
                      cudaStream_t s, int& launches, Prof* pr)
{
    pr->begin(K_POST, s);
    const int items = (width >> 2) + (width & 3);
    k_post_add8<<<dim3(ceil_div_post(items, 128), height), 128, 0, s>>>(row0, pitch, width, height, add, status, seq);
    pr->end(s);
    launches++;
}

void launch_post_fog(uint32_t* row0, int pitch, int width, int height, const float* depth, int depthScan,
                     uint32_t fog, float nearD, float farD, const int* status, int seq, cudaStream_t s, int& launches,
                     Prof* pr)
{
    pr->begin(K_POST, s);
    k_post_fog<<<dim3(ceil_div_post(width, 256), height), 256, 0, s>>>(row0, pitch, width, height, depth, depthScan,
                                                                       fog, nearD, farD, status, seq);
    pr->end(s);
    launches++;
}

}  // namespace ps3d
