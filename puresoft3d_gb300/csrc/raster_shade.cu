// raster_shade.cu -- visibility and shading passes.
//
// k_raster  one warp per bin of 32 rows x binW columns.  Lane r owns row r of
//           the bin, so every row is walked by exactly one thread, in
//           triangle order -- the reference's guarantee that a row's spans
//           are processed FIFO by one fragment thread (drawvao.cpp:77-109).
//           The bin's depth and "winner" (last colour-writing fragment that
//           passed) live in shared memory; each span is set up by the lane
//           that owns its row (interp.cpp:26-80) and walked pixel by pixel
//           with the reference's sequential accumulation (interp.cpp:82-92)
//           and epsilon depth test (fragthrd.cpp:227).
// k_shade   one thread per pixel: re-derives the winning fragment's
//           varyings (same span set-up and sequential steps) and runs the
//           draw's fragment stage once.  With no discard and no blending the
//           colour of a pixel is the colour of the last fragment that passed
//           the depth test, so shading only that fragment gives the
//           reference's framebuffer bit for bit.
#include <cuda_runtime.h>
#include "device_common.cuh"

namespace ps3d {

__device__ __forceinline__ void bin_range(const PassParams& P, int bin, int& start, int& end)
{
    int nHist = P.status[2];
    int nBins = P.binsX * P.binsY;
    int nb = nHist / nBins;
    if (nb == 0) {
        start = end = 0;
        return;
    }
    start = P.binHist[(size_t)bin * nb];
    end = bin + 1 < nBins ? P.binHist[(size_t)(bin + 1) * nb] : P.pairOffset[P.nTris];
}

template <int BW>
__global__ void __launch_bounds__(32) k_raster(PassParams P)
{
    constexpr int S = BW + 1;  // padded row stride: lanes at one column hit distinct banks
    __shared__ float sDepth[kBinH * S];
    __shared__ int sWin[kBinH * S];
    __shared__ __align__(16) TriRaster sTri[32];
    if (P.status[0]) return;

    const int bin = blockIdx.x;
    const int bx = bin % P.binsX, by = bin / P.binsX;
    const int x0 = bx * BW, y0 = by * kBinH;
    const int lane = threadIdx.x;
    const int cols = min(BW, P.W - x0);
    const int rows = min(kBinH, P.H - y0);
    int start, end;
    bin_range(P, bin, start, end);

    if (start == end) {
        if (P.clearDepth)
            for (int r = 0; r < rows; r++)
                for (int c = lane; c < cols; c += 32)
                    P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c] = P.depthClearValue;
        return;
    }
    for (int r = 0; r < kBinH; r++)
        for (int c = lane; c < BW; c += 32) {
            float d = P.depthClearValue;
            if (!P.clearDepth && r < rows && c < cols) d = P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c];
            sDepth[r * S + c] = d;
            sWin[r * S + c] = -1;
        }
    __syncwarp();

    const int y = y0 + lane;
    const int xLast = x0 + cols - 1;
    unsigned long long tested = 0, passed = 0;
    for (int chunk = start; chunk < end; chunk += 32) {
        int n = min(32, end - chunk);
        int tid = -1;
        unsigned mask = 0;
        if (lane < n) {
            tid = P.binTri[chunk + lane];
            const float4* src = (const float4*)(P.tris + tid);
            float4* dst = (float4*)(sTri + lane);
#pragma unroll
            for (int k = 0; k < 4; k++) dst[k] = src[k];
            int r0 = max((int)sTri[lane].firstRow - y0, 0), r1 = min((int)sTri[lane].lastRow - y0, kBinH - 1);
            if (r0 <= r1) mask = (r1 == 31 ? 0xffffffffu : ((1u << (r1 + 1)) - 1u)) & ~((1u << r0) - 1u);
        }
        // transpose: lane r collects the chunk's triangles that cover row r
        unsigned mine = 0;
#pragma unroll
        for (int r = 0; r < 32; r++) {
            unsigned w = __ballot_sync(0xffffffffu, (mask >> r) & 1u);
            if (lane == r) mine = w;
        }
        __syncwarp();
        if (y < P.H) {
            while (mine) {
                int j = __ffs(mine) - 1;
                mine &= mine - 1;
                const TriRaster& t = sTri[j];
                Span s;
                if (!span_row(t, y, P.W, s)) continue;
                int xs = max(s.leftClamped, x0), xe = min(s.rightClamped, xLast);
                if (xs > xe) continue;
                SpanZ z;
                span_z(t, s, y, z);
                int flags = t.edges >> 16;
                float cf2 = z.cf2, pz = z.pz;
                for (int x = s.leftClamped; x < xs; x++) {  // the steps taken left of this bin
                    cf2 = fadd(cf2, z.cf2Step);
                    pz = fadd(pz, z.pzStep);
                }
                int triId = P.binTri[chunk + j];
                float* dRow = sDepth + lane * S - x0;
                int* wRow = sWin + lane * S - x0;
                for (int x = xs; x <= xe; x++) {
                    float inv = frcp(cf2);
                    cf2 = fadd(cf2, z.cf2Step);
                    float zz = fmul(pz, inv);
                    pz = fadd(pz, z.pzStep);
                    float cur = (flags & B_TEST_DEPTH) ? dRow[x] : 1.0f;
                    if (-1.0f < zz && fsub(zz, cur) < -0.0001f) {
                        if (flags & B_UPDATE_DEPTH) dRow[x] = zz;
                        if (flags & F_COLOUR) wRow[x] = triId;
                        passed++;
                    }
                }
                tested += (unsigned long long)(xe - xs + 1);
            }
        }
        __syncwarp();
    }
    __syncwarp();
    for (int r = 0; r < rows; r++)
        for (int c = lane; c < cols; c += 32) {
            P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c] = sDepth[r * S + c];
            if (P.anyColour) P.winner[(size_t)(y0 + r) * P.W + x0 + c] = sWin[r * S + c];
        }
    if (P.countFrags) {
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            tested += __shfl_xor_sync(0xffffffffu, tested, o);
            passed += __shfl_xor_sync(0xffffffffu, passed, o);
        }
        if (lane == 0) {
            atomicAdd((unsigned long long*)(P.status + 4), tested);
            atomicAdd((unsigned long long*)(P.status + 6), passed);
        }
    }
}

// Varyings of the fragment at x on row y of triangle t (interp.cpp:26-92
// with the draw's interpolation stage): start/step from the corrected
// contributions, the left-clamp skip, then one step per pixel from
// leftClamped; returns start * (1 / cf2).
template <int NV>
__device__ __forceinline__ void fragment_varyings(const TriRaster& t, const float* vary, int nvMax, const Span& s,
                                                  const SpanZ& z, int x, float out[NV])
{
    float st[NV], sp[NV];
    const float* a = vary;
    const float* b = vary + nvMax;
    const float* c = vary + 2 * nvMax;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        float va = __ldg(a + k), vb = __ldg(b + k), vc = __ldg(c + k);
        float s0 = fadd(fadd(fmul(va, z.cl[0]), fmul(vb, z.cl[1])), fmul(vc, z.cl[2]));
        float e0 = fadd(fadd(fmul(va, z.cr[0]), fmul(vb, z.cr[1])), fmul(vc, z.cr[2]));
        st[k] = s0;
        sp[k] = fmul(fsub(e0, s0), z.recip);  // calcStep: stepCount != 0 here
    }
    if (z.skip == 1) {
#pragma unroll
        for (int k = 0; k < NV; k++) st[k] = fadd(st[k], sp[k]);
    } else if (z.skip > 1) {
        float fs = (float)z.skip;
#pragma unroll
        for (int k = 0; k < NV; k++) st[k] = fadd(st[k], fmul(sp[k], fs));
    }
    float cf2 = z.cf2;
    for (int i = s.leftClamped; i < x; i++) {
        cf2 = fadd(cf2, z.cf2Step);
#pragma unroll
        for (int k = 0; k < NV; k++) st[k] = fadd(st[k], sp[k]);
    }
    float inv = frcp(cf2);
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = fmul(st[k], inv);
}

__global__ void __launch_bounds__(256) k_shade(PassParams P)
{
    if (P.status[0]) return;
    int x = blockIdx.x * 32 + threadIdx.x;
    int y = blockIdx.y * 8 + threadIdx.y;
    if (x >= P.W || y >= P.H || x >= P.colourW || y >= P.colourH) return;
    int bin = (y / kBinH) * P.binsX + x / P.binW;
    int start, end;
    bin_range(P, bin, start, end);
    int w = -1;
    if (start != end && P.anyColour) w = P.winner[(size_t)y * P.W + x];
    uint32_t* dst = (uint32_t*)P.colour + (size_t)(P.colourH - 1 - y) * P.colourW + x;
    if (w < 0) {
        if (P.clearColour) *dst = P.colourClearValue;
        return;
    }
    TriRaster t;
    {
        const float4* src = (const float4*)(P.tris + w);
        float4* d4 = (float4*)&t;
#pragma unroll
        for (int k = 0; k < 4; k++) d4[k] = __ldg(src + k);
    }
    const DrawDesc& d = P.draws[t.draw];
    const DrawUniforms& U = P.unis[d.uni];
    Span s;
    span_row(t, y, P.W, s);
    SpanZ z;
    span_z(t, s, y, z);
    const float* vary = P.vary + (size_t)w * 3 * P.nvMax;
    uint32_t bgra;
    switch (d.fp) {
    case FP_LIT2: {
        float in[16];
        fragment_varyings<16>(t, vary, P.nvMax, s, z, x, in);
        bgra = shade_lit2(U, in);
        break;
    }
    case FP_LIT1: {
        float in[9];
        fragment_varyings<9>(t, vary, P.nvMax, s, z, x, in);
        bgra = shade_lit1(U, in);
        break;
    }
    case FP_LIT3: {
        float in[9];
        fragment_varyings<9>(t, vary, P.nvMax, s, z, x, in);
        bgra = shade_lit3(U, in);
        break;
    }
    default: {  // FP_DEF01
        float in[9];
        fragment_varyings<9>(t, vary, P.nvMax, s, z, x, in);
        bgra = shade_def01(U, in);
        break;
    }
    }
    *dst = bgra;
}

__global__ void k_fill_u32(uint32_t* base, int width, int height, int pitchElems, uint32_t v, const int* status)
{
    if (status && status[0]) return;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x < width && y < height) base[(size_t)y * pitchElems + x] = v;
}

static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

void launch_raster_shade(const PassParams& P, cudaStream_t s, int& launches, Prof* pr)
{
    int nBins = P.binsX * P.binsY;
    pr->begin(K_RASTER, s);
    switch (P.binW) {
    case 16: k_raster<16><<<nBins, 32, 0, s>>>(P); break;
    case 32: k_raster<32><<<nBins, 32, 0, s>>>(P); break;
    default: k_raster<64><<<nBins, 32, 0, s>>>(P); break;
    }
    pr->end(s);
    launches++;
    if (P.anyColour || P.clearColour) {
        dim3 g(ceil_div(P.W, 32), ceil_div(P.H, 8));
        pr->begin(K_SHADE, s);
        k_shade<<<g, dim3(32, 8), 0, s>>>(P);
        pr->end(s);
        launches++;
    }
}

void launch_fill_u32(void* base, int width, int height, int pitchElems, uint32_t v, const int* status,
                     cudaStream_t s, int& launches, Prof* pr)
{
    pr->begin(K_FILL, s);
    k_fill_u32<<<dim3(ceil_div(width, 256), height), 256, 0, s>>>((uint32_t*)base, width, height, pitchElems, v, status);
    pr->end(s);
    launches++;
}

}  // namespace ps3d
