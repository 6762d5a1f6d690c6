// raster_shade.cu -- visibility and shading passes.
//
// k_raster  one 128-thread block per bin of 32 rows x binW columns.  The
//           bin's depth and "winner" (last colour-writing fragment that
//           passed) live in shared memory.  Triangles arrive in submission
//           order, 128 at a time, and their (triangle, row) spans are handled
//           128 at a time.  Set-up: one thread per span computes the
//           reference's row result and span set-up (rasterizer.cpp:93-118,
//           interp.cpp:26-80) and the exact z of each of its pixels with the
//           reference's sequential accumulation (interp.cpp:82-92).  Walk:
//           thread (warp w, lane r) owns row r, columns
//           [w*binW/4, (w+1)*binW/4), and applies that row's spans in
//           triangle order with the epsilon depth test (fragthrd.cpp:227) --
//           every pixel has exactly one owner, so the per-pixel order is the
//           reference's per-row FIFO order (drawvao.cpp:77-109).
//           At the end the block writes the bin's depth back, appends one
//           (pixel, winner) entry per covered pixel to the pass's shade list
//           and, when the pass clears colour, writes the clear colour to the
//           pixels no fragment reached.
// k_shade   one thread per shade-list entry: re-derives the winning
//           fragment's varyings (same span set-up and sequential steps) and
//           runs the draw's fragment stage once.  With no discard and no
//           blending the colour of a pixel is the colour of the last fragment
//           that passed the depth test, so shading only that fragment gives
//           the reference's framebuffer bit for bit.
#include <cuda_runtime.h>
#include <algorithm>
#include <vector>
#include "raster_common.cuh"
#include "vertex_stage.cuh"

namespace ps3d {

// Per span of a round: its columns in the bin, its triangle slot and flags.
struct SpanRec {
    short xs, xe;   // bin-relative, inclusive
    short j;        // triangle slot in the chunk
    short flags;
};

// The interpolation stage's state along one span (interp.cpp:26-92 with the
// draw's interpolation processor): start/step from the corrected
// contributions, the left-clamp skip, then one step per pixel from
// leftClamped -- sequential adds, so pixel k needs k steps.
template <int NV> struct VaryState {
    float st[NV], sp[NV];
    float cf2, cf2Step;
    int x;  // the pixel the state is at
};

// The span's interpolation state from the varyings' values at its two ends
// (s0, e0: interpolateByContributes at left and right): calcStep, the
// interpolation stage's step rule, the left-clamp skip.  nstep: the
// interpolation stage steps the first two float4 varyings by the third's
// step (the reference demo's IP_Planet, test/testproc.cpp:171-195, adds the
// normal's step to the tangent and the binormal).
template <int NV>
__device__ __forceinline__ void vary_steps(const float* s0, const float* e0, const Span& s, const SpanZ& z,
                                           VaryState<NV>& v, bool nstep)
{
#pragma unroll
    for (int k = 0; k < NV; k++) {
        v.st[k] = s0[k];
        v.sp[k] = fmul(fsub(e0[k], s0[k]), z.recip);  // calcStep: stepCount != 0 here
    }
    if constexpr (NV >= 12) {
        if (nstep) {
#pragma unroll
            for (int k = 0; k < 8; k++) v.sp[k] = v.sp[8 + (k & 3)];
        }
    }
    if (z.skip == 1) {
#pragma unroll
        for (int k = 0; k < NV; k++) v.st[k] = fadd(v.st[k], v.sp[k]);
    } else if (z.skip > 1) {
        float fs = (float)z.skip;
#pragma unroll
        for (int k = 0; k < NV; k++) v.st[k] = fadd(v.st[k], fmul(v.sp[k], fs));
    }
    v.cf2 = z.cf2;
    v.cf2Step = z.cf2Step;
    v.x = s.leftClamped;
}

// Set-up from the triangle's vertex varyings as the set-up kernel stored them.
template <int NV>
__device__ __forceinline__ void vary_begin(const TriRaster& t, const float* vary, int nvMax, const Span& s,
                                           const SpanZ& z, VaryState<NV>& v, bool nstep = false)
{
    const float* a = vary;
    const float* b = vary + nvMax;
    const float* c = vary + 2 * nvMax;
    float s0[NV], e0[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
        float va = __ldg(a + k), vb = __ldg(b + k), vc = __ldg(c + k);
        s0[k] = fadd(fadd(fmul(va, z.cl[0]), fmul(vb, z.cl[1])), fmul(vc, z.cl[2]));
        e0[k] = fadd(fadd(fmul(va, z.cr[0]), fmul(vb, z.cr[1])), fmul(vc, z.cr[2]));
    }
    vary_steps<NV>(s0, e0, s, z, v, nstep);
}

// Set-up with the vertex varyings computed here (a pass whose set-up
// deferred them): the draw's vertex processor on the triangle's three
// vertices, each product added in vertex order as above.
template <int NV, int VPK>
__device__ __forceinline__ void vary_begin_lazy(const DrawDesc& d, const DrawUniforms& U, int lt, const Span& s,
                                                const SpanZ& z, VaryState<NV>& v, bool nstep = false)
{
    float s0[NV], e0[NV];
#pragma unroll 1
    for (int vtx = 0; vtx < 3; vtx++) {
        float a[kMaxVary];
        vp_varyings<VPK>(d, U, 3 * lt + vtx, a);
        const float cl = vtx == 0 ? z.cl[0] : (vtx == 1 ? z.cl[1] : z.cl[2]);
        const float cr = vtx == 0 ? z.cr[0] : (vtx == 1 ? z.cr[1] : z.cr[2]);
#pragma unroll
        for (int k = 0; k < NV; k++) {
            const float ps = fmul(a[k], cl), pe = fmul(a[k], cr);
            if (vtx == 0) {
                s0[k] = ps;
                e0[k] = pe;
            } else {
                s0[k] = fadd(s0[k], ps);
                e0[k] = fadd(e0[k], pe);
            }
        }
    }
    vary_steps<NV>(s0, e0, s, z, v, nstep);
}

template <int NV> __device__ __forceinline__ void vary_advance(VaryState<NV>& v, int x)
{
    for (; v.x < x; v.x++) {
        v.cf2 = fadd(v.cf2, v.cf2Step);
#pragma unroll
        for (int k = 0; k < NV; k++) v.st[k] = fadd(v.st[k], v.sp[k]);
    }
}

template <int NV> __device__ __forceinline__ void vary_out(const VaryState<NV>& v, float out[NV])
{
    float inv = frcp(v.cf2);
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = fmul(v.st[k], inv);
}

// Varyings of the shade-list fragment at x of triangle w (its record t):
// from the stored vertex varyings (LAZY = 0), or computed from the vertices
// (a pass whose set-up deferred them; LAZY = the pass's vertex processor, -1
// any).  Separate kernels, so that the stored-varyings ones keep their
// registers.
template <int NV, int LAZY>
__device__ __forceinline__ void shade_varyings(const PassParams& P, const DrawDesc& d, const DrawUniforms& U, int w,
                                               const TriRaster& t, const Span& s, const SpanZ& z, int x, float out[NV],
                                               bool nstep = false)
{
    VaryState<NV> v;
    if constexpr (LAZY != 0) vary_begin_lazy<NV, (LAZY > 0 ? LAZY : 0)>(d, U, w - d.triBase, s, z, v, nstep);
    else vary_begin<NV>(t, P.vary + (size_t)w * 3 * P.nvMax, P.nvMax, s, z, v, nstep);
    vary_advance<NV>(v, x);
    vary_out<NV>(v, out);
}

// The fragment processor of draw d on one fragment: 1 = colour written to
// bgra, 2 = discarded (no colour, no depth write), 0 = no colour (depth only).
template <int NV>
__device__ __forceinline__ int shade_fragment(const DrawDesc& d, const DrawUniforms& U, const float* in,
                                              uint32_t& bgra)
{
    switch (d.fp) {
    case FP_LIT1: bgra = shade_lit1(U, in); return 1;
    case FP_LIT1A: return shade_lit1a(U, in, bgra) ? 1 : 2;
    case FP_LIT3: bgra = shade_lit3(U, in); return 1;
    case FP_DEF01: bgra = shade_def01(U, in); return 1;
    case FP_DEF04: bgra = shade_def04(U, in); return 1;
    case FP_DEF02:
        if constexpr (NV >= 11) {
            bgra = shade_def02(U, in);
            return 1;
        }
        return 0;
    case FP_LIT2:
        if constexpr (NV >= 16) {
            bgra = shade_lit2(U, in);
            return 1;
        }
        return 0;
    case FP_DEF03:
        if constexpr (NV >= 17) {
            bgra = shade_def03(U, in);
            return 1;
        }
        return 0;
    case FP_CLOUD:
        if constexpr (NV >= 13) {
            bgra = shade_cloud(U, in);
            return 1;
        }
        return 0;
    case FP_SINGLECOLOURNL: bgra = shade_single_colour_nl(U); return 1;
    case FP_SINGLECOLOUR:
        if constexpr (NV >= 11) {
            bgra = shade_single_colour(U, in);
            return 1;
        }
        return 0;
    case FP_DIFFUSEONLY:
        if constexpr (NV >= 13) {
            bgra = shade_diffuse_only(U, in);
            return 1;
        }
        return 0;
    case FP_CLOUDSHADOW:  // test/testproc.cpp:677-686: discards where the texel's red is below 150
        return ((nearest_texel(U.tex, in[0], in[1]) >> 16) & 0xff) < 150u ? 2 : 0;
    case FP_EARTH:
    case FP_SATELLITE:
        if constexpr (NV >= 21) {
            bgra = shade_planet(U, in, d.fp == FP_EARTH);
            return 1;
        }
        return 0;
    default: return 0;
    }
}

constexpr int kRasterThreads = 128;  // 4 warps: warp = column quarter, lane = bin row
constexpr int kChunk = 128;          // triangles per chunk (one per thread)
constexpr int kSlots = 128;          // (triangle, row) spans per round (one per thread)

// FWD (forward mode, 9 or 16 varyings): for passes that blend or may
// discard, every fragment that passes the depth test is shaded in the walk,
// in order, into the bin's colour tile (blend4 under ALPHABLEND; a discard
// skips the colour and the depth write) -- the reference's per-fragment
// order (fragthrd.cpp:208-252); no shade list.
// CULL: spans are tested for occlusion before their depths are computed
// (span_occluded) in crowded bins; the variant without it keeps the
// registers and instructions of the test out of passes that gain nothing.
template <int BW, int MINB, int FWD = 0, bool CULL = true>
__global__ void __launch_bounds__(kRasterThreads, MINB) k_raster(PassParams P)
{
    constexpr int S = BW + 1;   // padded strides: threads at one column hit distinct banks
    constexpr int Q = BW / 4;   // columns per quarter
    __shared__ float sDepth[kBinH * S];
    __shared__ int sWin[kBinH * S];
    __shared__ uint32_t sCol[FWD ? kBinH * S : 1];  // forward mode: the bin's colour
    __shared__ float sZ[kSlots * S];             // exact z of every pixel of each span
    __shared__ float sZmin[4][kSlots];           // per span and quarter: min z over its pixels
    __shared__ __align__(16) TriRaster sTri[kChunk];
    __shared__ int sTid[kChunk];
    __shared__ short sOx[kChunk], sOy[kChunk], sLw[kChunk];  // each triangle's viewport origin and width
    __shared__ int sBase[kChunk];                // first span (in chunk order) of each triangle
    __shared__ unsigned char sR0[kChunk];        // first bin row of each triangle
    __shared__ SpanRec sRec[kSlots];
    __shared__ unsigned sMask[2][4][kBinH][kSlots / 32];  // by round parity: rounds alternate buffers
    __shared__ int sWarpSum[kRasterThreads / 32];
    __shared__ float sQMax[4][kBinH];            // per quarter and row: an upper bound of its depths
    __shared__ int sListBase;
    __shared__ int sItem;
    __shared__ int sItemEnd[kItemBuckets];
    if (P.rowSplit > 1) load_item_buckets(P, sItemEnd);
    __syncthreads();  // before any early return: every thread reaches it
    if (pass_failed(P.status, P.passSeq)) return;

    // One block per bin (P.rowSplit == 1), or a persistent grid whose blocks
    // take work items from the pass's list (k_bin_bounds: crowded bins first,
    // each as 1 << log2 row slices of 32 >> log2 rows -- fewer spans per
    // block, so a crowded bin no longer holds up the launch alone -- then the
    // other bins, the empty ones last) until it is exhausted.  An item is
    // taken only when the block is free for it (taking the next one early
    // would hold a crowded slice back behind the current item).
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool listed = P.rowSplit > 1;
    unsigned long long tested = 0, passed = 0, coveredAll = 0;
    for (int iter = 0;; iter++) {
    if (listed && tid == 0) sItem = next_bin_item(P, sItemEnd);
    __syncthreads();  // sItem is ready; the previous item's shared data are no longer read
    const int item = listed ? sItem : (iter ? -1 : (int)blockIdx.x);
    __syncthreads();  // sItem is written again only after every thread has read it
    if (item < 0) break;
    const int bin = item & kItemBinMask, slice = (item >> kItemSliceShift) & 15;
    const int nSlices = 1 << (item >> kItemLog2Shift);
    const int bx = bin % P.binsX, by = bin / P.binsX;
    const int x0 = bx * BW, y0 = by * kBinH;
    const int cols = min(BW, P.W - x0);
    const int rows = min(kBinH, P.H - y0);
    int start, end;
    bin_range(P, bin, start, end);
    int rowBeg = 0, rowEnd = rows;
    if (nSlices > 1) {
        const int R = kBinH / nSlices;
        rowBeg = slice * R;
        rowEnd = min(rowBeg + R, rows);
        if (rowBeg >= rowEnd) continue;
    }

    if (start == end) {
        if (P.clearDepth || P.clearColour)
            for (int i = tid; i < rows * cols; i += kRasterThreads) {
                int r = i / cols, c = i - r * cols;
                if (P.clearDepth) P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c] = P.depthClearValue;
                if (P.clearColour) clear_colour_px(P, x0 + c, y0 + r);
            }
        continue;
    }
    // prefetch (record of the first chunk, index of the second), in flight
    // while the bin's depth is loaded; an item is a triangle (its index) or
    // a span item (~its index)
    float4 rec[4];
    bool have = start + tid < end, haveNext = start + kChunk + tid < end;
    int recTid = 0, nextIdx = 0;
    if (have) {
        recTid = P.sortedTri[start + tid];
        load_item(P, recTid, rec);
    }
    if (haveNext) nextIdx = P.sortedTri[start + kChunk + tid];
    for (int i = tid; i < kBinH * BW; i += kRasterThreads) {
        int r = i / BW, c = i - r * BW;
        float d = P.depthClearValue;
        if (!P.clearDepth && r >= rowBeg && r < rowEnd && c < cols) d = P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c];
        sDepth[r * S + c] = d;
        sWin[r * S + c] = -1;
        if constexpr (FWD > 0) {
            uint32_t col = P.colourClearValue;
            int x = x0 + c, y = y0 + r;
            if (!P.clearColour && r >= rowBeg && r < rowEnd && c < cols && x < P.colourW && y < P.colourH)
                col = *colour_px(P, x, y);
            sCol[r * S + c] = col;
        }
    }
    for (int i = tid; i < 2 * 4 * kBinH * (kSlots / 32); i += kRasterThreads) (&sMask[0][0][0][0])[i] = 0u;
    // Spans are tested for occlusion (span_occluded) in bins of more than
    // one chunk of triangles, where layers overlap; each thread keeps an
    // upper bound of its quarter of its row in sQMax.
    const bool cull = CULL && end - start > kChunk;
    if (cull) {
        if (P.clearDepth) {
            sQMax[warp][lane] = P.depthClearValue;
        } else {
            __syncthreads();  // the depth tile is complete
            const float* dr = sDepth + lane * S + warp * (BW / 4);
            float m = dr[0];
#pragma unroll
            for (int c = 1; c < BW / 4; c++) m = fmaxf(m, dr[c]);
            sQMax[warp][lane] = m;
        }
    }
    int par = 0;  // mask buffer of the current round

    const int qs = warp * Q, qe = qs + Q - 1;  // this thread's columns (bin-relative)
    float* dRow = sDepth + lane * S;
    int* wRow = sWin + lane * S;
    for (int chunk = start; chunk < end; chunk += kChunk) {
        // ---- stage the chunk's triangles, count their rows in the bin
        int cnt = 0, r0 = 0;
        if (have) {
            float4* dst = (float4*)(sTri + tid);
            if (recTid >= 0) {
#pragma unroll
                for (int k = 0; k < 4; k++) dst[k] = rec[k];
                sTid[tid] = recTid;
                const DrawDesc& dd = P.draws[sTri[tid].draw];
                int oy = dd.vpY;
                sOx[tid] = (short)dd.vpX;
                sOy[tid] = (short)oy;
                sLw[tid] = (short)dd.vpW;
                r0 = max((int)sTri[tid].firstRow + oy - y0, rowBeg);
                int r1 = min((int)sTri[tid].lastRow + oy - y0, rowEnd - 1);
                if (r0 <= r1) cnt = r1 - r0 + 1;
            } else {  // a span item: one row, set up already
                dst[0] = rec[0];
                dst[1] = rec[1];
                const SpanItem& si = *(const SpanItem*)(sTri + tid);
                sTid[tid] = si.tri;
                sLw[tid] = -1;  // marks the slot as a span item
                r0 = si.y - y0;
                if (r0 >= rowBeg && r0 < rowEnd) cnt = 1;
            }
        }
        have = haveNext;  // prefetch the next chunk while this one is processed
        recTid = nextIdx;
        if (have) load_item(P, recTid, rec);
        haveNext = chunk + 2 * kChunk + tid < end;
        if (haveNext) nextIdx = P.sortedTri[chunk + 2 * kChunk + tid];
        int inc = cnt;  // block-wide exclusive scan of the row counts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) sWarpSum[warp] = inc;
        __syncthreads();
        int wbase = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kRasterThreads / 32; w++) {
            int v = sWarpSum[w];
            if (w < warp) wbase += v;
            total += v;
        }
        sBase[tid] = wbase + inc - cnt;  // triangles with no rows get the next one's base
        sR0[tid] = (unsigned char)r0;
        __syncthreads();

        for (int round = 0; round < total; round += kSlots) {
            unsigned (*mask)[kBinH][kSlots / 32] = sMask[par];
            // the other buffer was last read by the previous round's walk: clear it for the next round
            for (int i = tid; i < 4 * kBinH * (kSlots / 32); i += kRasterThreads) (&sMask[par ^ 1][0][0][0])[i] = 0u;
            // ---- set-up: thread s2 takes span s2 of the round -- the reference's
            // row result and span set-up (rasterizer.cpp:93-118, interp.cpp:26-80),
            // then the sequential per-pixel steps (interp.cpp:82-92) through the
            // bin's columns, storing each pixel's exact z
            const int nSlots = min(kSlots, total - round);
            if (tid < nSlots) {
                const int s2 = tid, g = round + s2;
                int j = 0;  // the triangle of span g: the last one whose first span is <= g
#pragma unroll
                for (int step = kChunk / 2; step; step >>= 1)
                    if (sBase[j + step] <= g) j += step;
                const int r = sR0[j] + (g - sBase[j]);
                // the span's columns in the bin and its interpolation state
                // at pixel k0: from a span item as set up, or from the
                // triangle (the row result and span set-up)
                bool live;
                int xs, xe, k0, sflags;
                SpanZ z;
                if constexpr (FWD == 0) {
                    if (sLw[j] < 0) {
                        const SpanItem& si = *(const SpanItem*)(sTri + j);
                        live = true;
                        xs = si.xs;
                        xe = si.xe;
                        k0 = xs;
                        sflags = si.flags;
                        z.cf2 = si.cf2;
                        z.pz = si.pz;
                        z.cf2Step = si.cf2Step;
                        z.pzStep = si.pzStep;
                    } else {
                        live = triangle_span(sTri[j], y0 + r - sOy[j], sLw[j], sOx[j], x0, cols, xs, xe, k0, sflags, z);
                    }
                } else {
                    live = triangle_span(sTri[j], y0 + r - sOy[j], sLw[j], sOx[j], x0, cols, xs, xe, k0, sflags, z);
                }
                if (live) {
                    // a span that no depth test can pass is dropped here: no
                    // per-pixel z, no walk (counted as tested, as the walk would)
                    if (cull && xs <= xe && (sflags & B_TEST_DEPTH)) {
                        const int qa = (xs - x0) / Q, qb = (xe - x0) / Q;
                        float bound = sQMax[qa][r];
                        for (int q = qa + 1; q <= qb; q++) bound = fmaxf(bound, sQMax[q][r]);
                        if (span_occluded(z, xs - k0, xe - k0, bound)) {
                            tested += (unsigned long long)(xe - xs + 1);
                            xe = xs - 1;
                        }
                    }
                    if (xs <= xe) {
                        float cf2 = z.cf2, pz = z.pz;
                        for (int x = k0; x < xs; x++) {
                            cf2 = fadd(cf2, z.cf2Step);
                            pz = fadd(pz, z.pzStep);
                        }
                        float* zrow = sZ + s2 * S - x0;
                        float zmin = 0.0f;
                        int q = (xs - x0) / Q;
                        for (int x = xs; x <= xe; x++) {
                            float zz = fmul(pz, frcp(cf2));
                            cf2 = fadd(cf2, z.cf2Step);
                            pz = fadd(pz, z.pzStep);
                            zrow[x] = zz;
                            int qx = (x - x0) / Q;
                            if (qx != q || x == xs) {
                                if (x != xs) {
                                    sZmin[q][s2] = zmin;
                                    atomicOr(&mask[q][r][s2 >> 5], 1u << (s2 & 31));
                                }
                                q = qx;
                                zmin = zz;
                            } else {
                                zmin = fminf(zmin, zz);
                            }
                        }
                        sZmin[q][s2] = zmin;
                        atomicOr(&mask[q][r][s2 >> 5], 1u << (s2 & 31));
                        SpanRec& R = sRec[s2];
                        R.xs = (short)(xs - x0);
                        R.xe = (short)(xe - x0);
                        R.j = (short)j;
                        R.flags = (short)sflags;
                    }
                }
            }
            __syncthreads();
            // ---- walk: thread (quarter w, row r) applies row r's spans in
            // triangle order to its columns -- the reference's depth test and
            // writes (fragthrd.cpp:208-252).  A span none of whose pixels can
            // pass (z >= zmin >= every current depth here + epsilon) is skipped:
            // with TEST_DEPTH on, depth only decreases, so curMax stays an
            // upper bound and the skip never changes a result.
            if (lane >= rowBeg && lane < rowEnd) {
                float curMax = dRow[qs];
#pragma unroll
                for (int c = 1; c < Q; c++) curMax = fmaxf(curMax, dRow[qs + c]);
                for (int w = 0; w < (nSlots + 31) / 32; w++) {
                    unsigned bits = mask[warp][lane][w];
                    while (bits) {
                        int k = __ffs(bits) - 1;
                        bits &= bits - 1;
                        const int s2 = w * 32 + k;
                        const SpanRec R = sRec[s2];
                        const int a = max((int)R.xs, qs), b = min((int)R.xe, qe);
                        const int flags = R.flags;
                        tested += (unsigned long long)(b - a + 1);
                        if ((flags & B_TEST_DEPTH) && fsub(sZmin[warp][s2], curMax) >= -0.0001f) continue;
                        const float* zrow = sZ + s2 * S;
                        const int triId = sTid[R.j];
                        if constexpr (FWD > 0) {
                            // shade each passing fragment in order; the span's
                            // interpolation state is set up at the first one
                            VaryState<FWD> vs;
                            bool begun = false;
                            const int j = R.j, ox = sOx[j], yl = y0 + lane - sOy[j];
                            const DrawDesc& dd = P.draws[sTri[j].draw];
                            for (int x = a; x <= b; x++) {
                                float zz = zrow[x];
                                float cur = (flags & B_TEST_DEPTH) ? dRow[x] : 1.0f;
                                if (!(-1.0f < zz && fsub(zz, cur) < -0.0001f)) continue;
                                passed++;
                                int w = 0;
                                uint32_t bgra = 0;
                                if (flags & (F_COLOUR | F_FRAGMENT)) {
                                    const TriRaster& t = sTri[j];
                                    if (!begun) {
                                        Span sp;
                                        span_row(t, yl, sLw[j], sp);
                                        SpanZ zs;
                                        span_z(t, sp, yl, zs);
                                        vary_begin<FWD>(t, P.vary + (size_t)triId * 3 * P.nvMax, P.nvMax, sp, zs, vs,
                                                        dd.fp == FP_EARTH || dd.fp == FP_SATELLITE);
                                        begun = true;
                                    }
                                    vary_advance<FWD>(vs, x0 + x - ox);
                                    float in[FWD];
                                    vary_out<FWD>(vs, in);
                                    w = shade_fragment<FWD>(dd, P.unis[dd.uni], in, bgra);
                                }
                                if (w == 1) {
                                    uint32_t* cp = sCol + lane * S + x;
                                    // FBOBridge::write4 blends under ALPHABLEND; DEF01 / DEF02 /
                                    // DEF03 write through FBOBridge::write, which never blends
                                    *cp = ((flags & B_ALPHABLEND) && dd.fp != FP_DEF01 && dd.fp != FP_DEF02 &&
                                           dd.fp != FP_DEF03)
                                              ? blend4(*cp, bgra)
                                              : bgra;
                                }
                                if (w != 2 && (flags & B_UPDATE_DEPTH)) dRow[x] = zz;
                            }
                        } else {
                            for (int x = a; x <= b; x++) {
                                float zz = zrow[x];
                                float cur = (flags & B_TEST_DEPTH) ? dRow[x] : 1.0f;
                                if (-1.0f < zz && fsub(zz, cur) < -0.0001f) {
                                    if (flags & B_UPDATE_DEPTH) dRow[x] = zz;
                                    if (flags & F_COLOUR) wRow[x] = triId;
                                    passed++;
                                }
                            }
                        }
                        if (!(flags & B_TEST_DEPTH)) {  // depth may have risen: recompute the bound
                            curMax = dRow[qs];
#pragma unroll
                            for (int c = 1; c < Q; c++) curMax = fmaxf(curMax, dRow[qs + c]);
                        }
                    }
                }
                if (cull) sQMax[warp][lane] = curMax;  // for the next round's set-up
            }
            __syncthreads();
            par ^= 1;
        }
    }
    // depth write-back; count of covered pixels per thread
    int covered = 0;
    const int nr = rowEnd - rowBeg;
    for (int i = tid; i < nr * cols; i += kRasterThreads) {
        int r = rowBeg + i / cols, c = i - (r - rowBeg) * cols;
        P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c] = sDepth[r * S + c];
        covered += sWin[r * S + c] >= 0;
    }
    if constexpr (FWD > 0) {
        if (P.anyColour || P.clearColour)
            for (int i = tid; i < nr * cols; i += kRasterThreads) {
                int r = rowBeg + i / cols, c = i - (r - rowBeg) * cols, x = x0 + c, y = y0 + r;
                if (x < P.colourW && y < P.colourH)
                    *colour_px(P, x, y) = sCol[r * S + c];
            }
        covered = 0;  // nothing is left to shade
    } else if (P.anyColour || P.clearColour) {
        // one block-wide reservation in the shade list, then each thread's
        // covered pixels in order; uncovered pixels get the clear colour
        int inc = covered;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        __syncthreads();  // sWarpSum was last read before the final round's barrier
        if (lane == 31) sWarpSum[warp] = inc;
        __syncthreads();
        if (tid == 0) {
            int run = 0;
            for (int w = 0; w < kRasterThreads / 32; w++) {
                int v = sWarpSum[w];
                sWarpSum[w] = run;
                run += v;
            }
            sListBase = (P.anyColour && run) ? atomicAdd(P.slotStatus + kSlotShade, run) : 0;
        }
        __syncthreads();
        int pos = sListBase + sWarpSum[warp] + inc - covered;
        for (int i = tid; i < nr * cols; i += kRasterThreads) {
            int r = rowBeg + i / cols, c = i - (r - rowBeg) * cols;
            int w = sWin[r * S + c];
            if (w >= 0) {
                if (P.anyColour) P.shadeList[pos++] = make_int2(shade_pixel(x0 + c, y0 + r), w);
            } else if (P.clearColour) {
                clear_colour_px(P, x0 + c, y0 + r);
            }
        }
    }
    coveredAll += (unsigned long long)covered;
    }
    if (P.countFrags) {
        unsigned long long cov = P.anyColour ? coveredAll : 0ull;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            tested += __shfl_xor_sync(0xffffffffu, tested, o);
            passed += __shfl_xor_sync(0xffffffffu, passed, o);
            cov += __shfl_xor_sync(0xffffffffu, cov, o);
        }
        if (lane == 0) {
            atomicAdd((unsigned long long*)(P.status + 4), tested);
            atomicAdd((unsigned long long*)(P.status + 6), passed);
            atomicAdd((unsigned long long*)(P.status + 10), cov);
        }
    }
}

// Varyings of the fragment at x on row y of triangle t (interp.cpp:26-92
// with the draw's interpolation stage): start/step from the corrected
// contributions, the left-clamp skip, then one step per pixel from
// leftClamped; returns start * (1 / cf2).

// FPK: the fragment processor when every draw of the pass uses the same
// one (a kernel with only that shader's registers), else 0 (any).
template <int FPK, int LAZY>
__device__ __forceinline__ void shade_entry(const PassParams& P, int2 e)
{
    const int y = e.x >> 16, x = e.x & 0xffff, w = e.y;
    uint32_t* dst = colour_px(P, x, y);
    TriRaster t;
    {
        const float4* src = (const float4*)(P.tris + w);
        float4* d4 = (float4*)&t;
#pragma unroll
        for (int k = 0; k < 4; k++) d4[k] = __ldg(src + k);
    }
    const DrawDesc& d = P.draws[t.draw];
    const DrawUniforms& U = P.unis[d.uni];
    const int xl = x - d.vpX, yl = y - d.vpY;  // the draw's rasteriser coordinates
    Span s;
    span_row<true>(t, yl, d.vpW, s);
    SpanZ z;
    span_z(t, s, yl, z);
    uint32_t bgra;
    switch (FPK ? FPK : d.fp) {
    case FP_EARTH:
    case FP_SATELLITE: {
        float in[21];
        shade_varyings<21, LAZY>(P, d, U, w, t, s, z, xl, in, true);
        bgra = shade_planet(U, in, (FPK ? FPK : d.fp) == FP_EARTH);
        break;
    }
    case FP_CLOUD: {
        float in[13];
        shade_varyings<13, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_cloud(U, in);
        break;
    }
    case FP_DIFFUSEONLY: {
        float in[13];
        shade_varyings<13, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_diffuse_only(U, in);
        break;
    }
    case FP_SINGLECOLOUR: {
        float in[11];
        shade_varyings<11, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_single_colour(U, in);
        break;
    }
    case FP_SINGLECOLOURNL:
        bgra = shade_single_colour_nl(U);
        break;
    case FP_DEF03: {
        float in[17];
        shade_varyings<17, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_def03(U, in);
        break;
    }
    case FP_LIT2: {
        float in[16];
        shade_varyings<16, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_lit2(U, in);
        break;
    }
    case FP_LIT1: {
        float in[9];
        shade_varyings<9, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_lit1(U, in);
        break;
    }
    case FP_DEF02: {
        float in[11];
        shade_varyings<11, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_def02(U, in);
        break;
    }
    case FP_DEF04: {
        float in[3];
        shade_varyings<3, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_def04(U, in);
        break;
    }
    case FP_LIT3: {
        float in[9];
        shade_varyings<9, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_lit3(U, in);
        break;
    }
    default: {  // FP_DEF01
        float in[9];
        shade_varyings<9, LAZY>(P, d, U, w, t, s, z, xl, in);
        bgra = shade_def01(U, in);
        break;
    }
    }
    *dst = bgra;
}

// One thread per shade-list entry; the grid strides over the list, whose
// length the raster kernel left in the slot status.
template <int FPK, int LAZY>
__global__ void __launch_bounds__(256, (LAZY != 0 && FPK != 0) ? 2 : 1) k_shade(PassParams P)
{
    if (pass_failed(P.status, P.passSeq)) return;
    const int n = P.slotStatus[kSlotShade];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        shade_entry<FPK, LAZY>(P, P.shadeList[i]);
}

__global__ void k_fill_u32(uint32_t* base, int width, int height, int pitchElems, uint32_t v, const int* status,
                           int seq)
{
    if (status && pass_failed(status, seq)) return;
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x < width && y < height) base[(size_t)y * pitchElems + x] = v;
}

static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Blocks of `threads` threads of kernel `kern` resident on the current
// device at once (queried once per kernel and device).
static int resident_blocks(const void* kern, int threads)
{
    thread_local std::vector<std::pair<std::pair<const void*, int>, int>> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    for (const auto& e : cache)
        if (e.first.first == kern && e.first.second == dev) return e.second;
    int sms = 0, perSM = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, threads, 0);
    const int resident = std::max(sms, 1) * std::max(perSM, 1);
    cache.push_back({{kern, dev}, resident});
    return resident;
}

// The persistent raster grid: as many blocks as fit on the device at once
// (more would only find the list empty), at most one per work item.
static int raster_grid(const void* kern, int nBins, int rowSplit)
{
    if (rowSplit <= 1) return nBins;  // one block per bin
    long long items = (long long)nBins * rowSplit;
    return (int)std::max<long long>(1, std::min<long long>(items, resident_blocks(kern, kRasterThreads)));
}

template <int BW> void launch_raster(const PassParams& P, int nBins, cudaStream_t s)
{
    if (P.rasterBlocks == 8) {
        if (P.cullSpans) { auto* k_ = k_raster<BW, 8, 0, true>; k_<<<raster_grid((const void*)k_, nBins, P.rowSplit), kRasterThreads, 0, s>>>(P); }
        else { auto* k_ = k_raster<BW, 8, 0, false>; k_<<<raster_grid((const void*)k_, nBins, P.rowSplit), kRasterThreads, 0, s>>>(P); }
    } else {
        if (P.cullSpans) { auto* k_ = k_raster<BW, 5, 0, true>; k_<<<raster_grid((const void*)k_, nBins, P.rowSplit), kRasterThreads, 0, s>>>(P); }
        else { auto* k_ = k_raster<BW, 5, 0, false>; k_<<<raster_grid((const void*)k_, nBins, P.rowSplit), kRasterThreads, 0, s>>>(P); }
    }
}

// Forward passes (blending or discarding draws) run with 16-column bins.
void launch_raster_forward(const PassParams& P, int nBins, cudaStream_t s)
{
    // the host lays a forward pass's varyings out with stride forward_vary()
    if (P.nvMax == forward_vary(9)) {
        if (P.cullSpans) { auto* k_ = k_raster<16, 1, 9, true>; k_<<<raster_grid((const void*)k_, nBins, P.rowSplit), kRasterThreads, 0, s>>>(P); }
        else { auto* k_ = k_raster<16, 1, 9, false>; k_<<<raster_grid((const void*)k_, nBins, P.rowSplit), kRasterThreads, 0, s>>>(P); }
    } else {
        if (P.cullSpans) { auto* k_ = k_raster<16, 1, kMaxVary, true>; k_<<<raster_grid((const void*)k_, nBins, P.rowSplit), kRasterThreads, 0, s>>>(P); }
        else { auto* k_ = k_raster<16, 1, kMaxVary, false>; k_<<<raster_grid((const void*)k_, nBins, P.rowSplit), kRasterThreads, 0, s>>>(P); }
    }
}

void launch_raster_warp(const PassParams& P, int nBins, cudaStream_t s);  // raster_warp.cu

void launch_raster(const PassParams& P, cudaStream_t s, int& launches, Prof* pr)
{
    int nBins = P.binsX * P.binsY;
    pr->begin(K_RASTER, s);
    if (P.forward) launch_raster_forward(P, nBins, s);
    else if (P.warpBins && P.binW <= 16) launch_raster_warp(P, nBins, s);
    else switch (P.binW) {
    case 8: launch_raster<8>(P, nBins, s); break;
    case 16: launch_raster<16>(P, nBins, s); break;
    default: launch_raster<32>(P, nBins, s); break;
    }
    pr->end(s);
    launches++;
}

// The shade kernel for the pass's fragment processor (0: any) and its
// varyings: stored by the set-up (LAZY = 0) or computed here (LAZY = the
// vertex processor, for the pairs the built-in programmes use, else -1).
template <int LAZY> static void (*shade_kernel(int fp))(PassParams)
{
    switch (fp) {
    case FP_LIT1: return k_shade<FP_LIT1, LAZY>;
    case FP_LIT2: return k_shade<FP_LIT2, LAZY>;
    case FP_LIT3: return k_shade<FP_LIT3, LAZY>;
    case FP_DEF01: return k_shade<FP_DEF01, LAZY>;
    case FP_DEF03: return k_shade<FP_DEF03, LAZY>;
    case FP_DEF02: return k_shade<FP_DEF02, LAZY>;
    case FP_DEF04: return k_shade<FP_DEF04, LAZY>;
    case FP_EARTH: return k_shade<FP_EARTH, LAZY>;
    case FP_SATELLITE: return k_shade<FP_SATELLITE, LAZY>;
    case FP_CLOUD: return k_shade<FP_CLOUD, LAZY>;
    case FP_SINGLECOLOUR: return k_shade<FP_SINGLECOLOUR, LAZY>;
    case FP_DIFFUSEONLY: return k_shade<FP_DIFFUSEONLY, LAZY>;
    default: return k_shade<0, LAZY>;
    }
}

static void (*lazy_shade_kernel(int fp, int vp))(PassParams)
{
    if (vp == VP_LIT2 && fp == FP_LIT2) return k_shade<FP_LIT2, VP_LIT2>;
    if (vp == VP_DEF01 && fp == FP_LIT1) return k_shade<FP_LIT1, VP_DEF01>;
    if (vp == VP_DEF01 && fp == FP_LIT3) return k_shade<FP_LIT3, VP_DEF01>;
    if (vp == VP_DEF01 && fp == FP_DEF01) return k_shade<FP_DEF01, VP_DEF01>;
    if (vp == VP_DEF03 && fp == FP_DEF03) return k_shade<FP_DEF03, VP_DEF03>;
    return shade_kernel<-1>(fp);
}

void launch_shade(const PassParams& P, cudaStream_t s, int& launches, Prof* pr)
{
    if (!P.anyColour || P.forward) return;  // a forward pass shaded in the raster
    // a grid that fills the GPU, striding over the shade list
    void (*kern)(PassParams) = P.lazyVary ? lazy_shade_kernel(P.passFp, P.passVp) : shade_kernel<0>(P.passFp);
    long long need = ((long long)P.W * P.H + 255) / 256;
    int grid = (int)std::min<long long>(need, resident_blocks((const void*)kern, 256));
    pr->begin(K_SHADE, s);
    kern<<<std::max(grid, 1), 256, 0, s>>>(P);
    pr->end(s);
    launches++;
}

void launch_fill_u32(void* base, int width, int height, int pitchElems, uint32_t v, const int* status, int seq,
                     cudaStream_t s, int& launches, Prof* pr)
{
    pr->begin(K_FILL, s);
    k_fill_u32<<<dim3(ceil_div(width, 256), height), 256, 0, s>>>((uint32_t*)base, width, height, pitchElems, v, status, seq);
    pr->end(s);
    launches++;
}

}  // namespace ps3d

namespace ps3d {

// Self-test of the fast correctly rounded reciprocal and quotient against
// the CUDA intrinsics: every mantissa of biased exponents [27, 227] (both
// signs) for the reciprocal, and `pairs` hashed operand pairs with exponents
// in [-60, 60) for the quotient.
__device__ __forceinline__ unsigned st_hash(unsigned x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__global__ void k_selftest_rcp(int biasedExp, unsigned long long* bad)
{
    unsigned m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= (1u << 23)) return;
    float b = __uint_as_float(((unsigned)biasedExp << 23) | m);
    if (__float_as_uint(frcp(b)) != __float_as_uint(__frcp_rn(b))) atomicAdd(bad, 1ull);
    if (__float_as_uint(frcp(-b)) != __float_as_uint(__frcp_rn(-b))) atomicAdd(bad, 1ull);
}

__global__ void k_selftest_div(unsigned seed, unsigned long long n, unsigned long long* bad)
{
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned h1 = st_hash((unsigned)i * 2654435761u ^ seed), h2 = st_hash(h1 + 0x9e3779b9u), h3 = st_hash(h2 ^ 0x85ebca6bu);
    int ea = -60 + (int)(h3 % 120u), eb = -60 + (int)((h3 >> 10) % 120u);
    float a = __uint_as_float(((unsigned)(ea + 127) << 23) | (h1 & 0x7fffffu) | ((h3 >> 31) << 31));
    float b = __uint_as_float(((unsigned)(eb + 127) << 23) | (h2 & 0x7fffffu) | (((h3 >> 30) & 1u) << 31));
    if (__float_as_uint(fdiv(a, b)) != __float_as_uint(__fdiv_rn(a, b))) atomicAdd(bad, 1ull);
}

// Self-test of the bounded device waits: one warp waits, the way the sort's
// look-backs do (volatile poll, short sleep, a limit on the polls), for a
// flag that nothing sets; when the limit runs out it marks the failure words
// as an expired look-back does and returns.
__global__ void k_selftest_wait(int* status, const int* flag, int spins)
{
    int n = 0;
    while (*(volatile const int*)flag == 0) {
        if (++n > spins) {
            if (threadIdx.x == 0) {
                atomicMin(status + kFirstFailed, 0);
                atomicOr(status, 2);
            }
            return;
        }
        __nanosleep(64);
    }
}

// Self-test of span_occluded against the per-pixel loop it stands in for:
// random spans (1/w in [1e-3, 10], z in [-1.2, 1.2] at both ends, up to 4095
// steps, sometimes a 1/w that crosses zero) and depth bounds placed around
// the exact pass/fail boundary.  bad[0] counts spans declared occluded that
// have a pixel passing the depth test (must be 0), bad[1] the spans
// declared occluded.
__global__ void k_selftest_occlusion(unsigned seed, unsigned long long n, unsigned long long* bad)
{
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned h = st_hash((unsigned)i * 2654435761u ^ seed);
    auto uni = [&]() {  // [0, 1)
        h = st_hash(h + 0x9e3779b9u);
        return (float)(h >> 8) * 0x1p-24f;
    };
    const int kB = 1 + (int)(uni() * uni() * 4094.0f);
    const int kA = (int)(uni() * (float)(kB + 1)) % (kB + 1);
    const float C0 = exp2f(-10.0f + 13.3f * uni());
    float C1 = exp2f(-10.0f + 13.3f * uni());
    if (uni() < 0.05f) C1 = -C1;  // 1/w through zero: must never be declared occluded wrongly
    const float z0 = -1.2f + 2.4f * uni(), z1 = uni() < 0.3f ? z0 + (uni() - 0.5f) * 1e-3f : -1.2f + 2.4f * uni();
    SpanZ z;
    z.cf2 = C0;
    z.pz = fmul(z0, C0);
    z.cf2Step = fdiv(fsub(C1, C0), (float)kB);
    z.pzStep = fdiv(fsub(fmul(z1, C1), z.pz), (float)kB);
    // the loop's z values and their minimum over kA..kB
    float cf2 = z.cf2, pz = z.pz, zmin = INFINITY;
    for (int k = 0; k <= kB; k++) {
        float zz = fmul(pz, frcp(cf2));
        if (k >= kA) zmin = fminf(zmin, zz);
        cf2 = fadd(cf2, z.cf2Step);
        pz = fadd(pz, z.pzStep);
    }
    if (!isfinite(zmin)) return;
    // a bound at the boundary (zmin + 1e-4) moved by up to 1e-3 relative, or anywhere
    float curMax = uni() < 0.7f ? zmin + 0.0001f * (1.0f + (uni() - 0.5f) * 0.002f) : -1.0f + 2.0f * uni();
    if (!span_occluded(z, kA, kB, curMax)) return;
    atomicAdd(bad + 1, 1ull);
    cf2 = z.cf2;
    pz = z.pz;
    for (int k = 0; k <= kB; k++) {
        float zz = fmul(pz, frcp(cf2));
        if (k >= kA && fsub(zz, curMax) < -0.0001f) {
            atomicAdd(bad, 1ull);
            return;
        }
        cf2 = fadd(cf2, z.cf2Step);
        pz = fadd(pz, z.pzStep);
    }
}

int selftest_occlusion(unsigned long long cases, unsigned long long* wrong, unsigned long long* occluded)
{
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) return -1;
    cudaMemset(d, 0, 16);
    if (cases) k_selftest_occlusion<<<(unsigned)((cases + 255) / 256), 256>>>(777u, cases, d);
    unsigned long long h[2];
    cudaError_t e = cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return -1;
    *wrong = h[0];
    *occluded = h[1];
    return 0;
}

void launch_selftest_wait(int* status, const int* flag, int spins, cudaStream_t s)
{
    k_selftest_wait<<<1, 32, 0, s>>>(status, flag, spins);
}

int selftest_division(unsigned long long pairs, unsigned long long* rcpBad, unsigned long long* divBad)
{
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) return -1;
    cudaMemset(d, 0, 16);
    for (int e = 27; e <= 227; e++) k_selftest_rcp<<<(1 << 23) / 256, 256>>>(e, d);
    if (pairs) k_selftest_div<<<(unsigned)((pairs + 255) / 256), 256>>>(12345u, pairs, d + 1);
    unsigned long long h[2];
    cudaError_t e = cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return -1;
    *rcpBad = h[0];
    *divBad = h[1];
    return 0;
}

}  // namespace ps3d
