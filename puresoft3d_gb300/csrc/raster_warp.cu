// raster_warp.cu -- k_raster_warp: the visibility pass with one warp per bin.
//
// The same work as k_raster (raster_shade.cu) in a different shape.  There,
// four warps share a bin of 32 rows and meet at block-wide barriers twice per
// round of 128 spans (after the span set-up, after the walk), so every round
// waits for the slowest set-up thread of the block.  Here each warp owns a
// whole bin of 32 rows x BW (8 or 16) columns and works through it alone:
// its rounds are 32 spans (lane = span in the set-up, lane = row in the
// walk) separated by __syncwarp only, and the warps of a block never wait for
// one another.  A bin's depth and winner tiles and the round's span data sit
// in the warp's own slice of shared memory (about 6.5 KB at 8 columns), so
// that 8 blocks of 4 warps are resident per SM.  Warps take bins from the
// pass's work list (k_bin_bounds: the crowded bins' row slices first, then
// the other bins, the empty ones last) until it is exhausted.
//
// The arithmetic is the reference's and the same device functions as
// k_raster's: the row result (rasterizer.cpp:93-118), the span set-up
// (interp.cpp:26-80), the per-pixel sequential steps (interp.cpp:82-92) and
// the epsilon depth test (fragthrd.cpp:217-238).  Each pixel has one owner
// lane (its row), which applies the row's spans in triangle order: the
// per-row FIFO order of the reference (drawvao.cpp:77-109).
#include <cuda_runtime.h>
#include <algorithm>
#include <vector>
#include "raster_common.cuh"

namespace ps3d {

constexpr int kWarpRasterWarps = 4;  // warps per block, each on its own bins
constexpr int kWarpRasterThreads = 32 * kWarpRasterWarps;

// One warp's shared memory.
template <int BW> struct __align__(16) WarpTile {
    int item[32];                    // the chunk's items (triangle, or ~index of a span item); their
                                     // records are read back from L1 where the set-up needs them
    float depth[kBinH * (BW + 1)];   // the bin's depth (odd row stride: lanes = rows hit distinct banks)
    int win[kBinH * (BW + 1)];       // last colour-writing fragment that passed, -1 none
    float z[32 * (BW + 1)];          // per span of the round: exact z at each of its bin columns
    int tid[32];                     // triangle id of each chunk slot
    int base[32];                    // first span (chunk order) of each triangle
    short ox[32], oy[32], lw[32];    // each triangle's viewport origin and width
    short xs[32], xe[32];            // per span: bin columns, inclusive
    short flags[32];
    unsigned char r0[32];            // first bin row of each triangle
    unsigned char j[32];             // per span: its triangle's chunk slot
    float zmin[32];                  // per span: min z over its pixels
    unsigned mask[32];               // per row: the round's spans on it
    float rowMax[32];                // per row: an upper bound of its depths
};

template <int BW, int MINB, bool CULL>
__global__ void __launch_bounds__(kWarpRasterThreads, MINB) k_raster_warp(PassParams P)
{
    constexpr int S = BW + 1;
    __shared__ WarpTile<BW> tiles[kWarpRasterWarps];
    __shared__ int sItemEnd[kItemBuckets];
    load_item_buckets(P, sItemEnd);
    __syncthreads();  // before any early return: every thread reaches it
    if (pass_failed(P.status, P.passSeq)) return;
    const int lane = threadIdx.x & 31;
    WarpTile<BW>& T = tiles[threadIdx.x >> 5];
    float* dRow = T.depth + lane * S;  // walk: lane = bin row
    int* wRow = T.win + lane * S;
    unsigned long long tested = 0, passed = 0, coveredAll = 0;
    const bool vecDepth = (P.depthScan & 3) == 0 && ((size_t)P.depth & 15) == 0;

    for (;;) {
        int item = 0;
        if (lane == 0) item = next_bin_item(P, sItemEnd);
        item = __shfl_sync(0xffffffffu, item, 0);
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
        }
        if (rowBeg >= rowEnd) continue;
        const bool myRow = lane >= rowBeg && lane < rowEnd;
        const bool vec = vecDepth && cols == BW;

        // Tile loads and stores run with the lanes along the bin's rows in
        // row-major order (whole row segments per instruction, 16-byte
        // accesses where the rows allow), not lane = row.
        const int nPx = (rowEnd - rowBeg) * BW;
        if (start == end) {  // no triangle: the bin's clears only
            if (P.clearDepth) {
                if (vec) {
                    const float v = P.depthClearValue;
                    for (int i = lane; i < nPx / 4; i += 32) {
                        const int r = rowBeg + (4 * i) / BW, c = (4 * i) % BW;
                        *(float4*)(P.depth + (size_t)(y0 + r) * P.depthScan + x0 + c) = make_float4(v, v, v, v);
                    }
                } else {
                    for (int i = lane; i < nPx; i += 32) {
                        const int r = rowBeg + i / BW, c = i % BW;
                        if (c < cols) P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c] = P.depthClearValue;
                    }
                }
            }
            if (P.clearColour)
                for (int i = lane; i < nPx; i += 32) {
                    const int r = rowBeg + i / BW, c = i % BW;
                    if (c < cols) clear_colour_px(P, x0 + c, y0 + r);
                }
            continue;
        }

        // the bin's depth: the slice's rows from the target (none when the
        // pass clears depth), the clear value elsewhere
        if (!P.clearDepth && vec) {
            for (int i = lane; i < kBinH * BW / 4; i += 32) {
                const int r = (4 * i) / BW, c = (4 * i) % BW;
                float4 d = make_float4(P.depthClearValue, P.depthClearValue, P.depthClearValue, P.depthClearValue);
                if (r >= rowBeg && r < rowEnd) d = *(const float4*)(P.depth + (size_t)(y0 + r) * P.depthScan + x0 + c);
                float* t = T.depth + r * S + c;
                t[0] = d.x;
                t[1] = d.y;
                t[2] = d.z;
                t[3] = d.w;
            }
        } else {
            for (int i = lane; i < kBinH * BW; i += 32) {
                const int r = i / BW, c = i % BW;
                T.depth[r * S + c] = (!P.clearDepth && r >= rowBeg && r < rowEnd && c < cols)
                                         ? P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c]
                                         : P.depthClearValue;
            }
        }
        __syncwarp();
        float rmax = -INFINITY;
#pragma unroll
        for (int c = 0; c < BW; c++) {
            wRow[c] = -1;
            if (c < cols) rmax = fmaxf(rmax, dRow[c]);
        }
        T.rowMax[lane] = rmax;
        // spans are tested for occlusion (span_occluded) in bins of more than one chunk
        const bool cull = CULL && end - start > 32;

        for (int chunk = start; chunk < end; chunk += 32) {
            __syncwarp();  // the previous chunk's triangles are no longer read
            // ---- stage the chunk's triangles, count their rows in the slice
            int cnt = 0, r0 = 0;
            if (chunk + lane < end) {
                const int v = P.sortedTri[chunk + lane];  // a triangle, or ~index of a span item
                float4 rec[4];
                load_item(P, v, rec);
                T.item[lane] = v;
                if (v >= 0) {
                    T.tid[lane] = v;
                    const TriRaster& tr = *reinterpret_cast<const TriRaster*>(rec);
                    const DrawDesc& dd = P.draws[tr.draw];
                    const int oy = dd.vpY;
                    T.ox[lane] = (short)dd.vpX;
                    T.oy[lane] = (short)oy;
                    T.lw[lane] = (short)dd.vpW;
                    r0 = max((int)tr.firstRow + oy - y0, rowBeg);
                    const int r1 = min((int)tr.lastRow + oy - y0, rowEnd - 1);
                    if (r0 <= r1) cnt = r1 - r0 + 1;
                } else {  // a span item: one row, set up already
                    const SpanItem& si = *reinterpret_cast<const SpanItem*>(rec);
                    T.tid[lane] = si.tri;
                    T.lw[lane] = -1;
                    r0 = si.y - y0;
                    if (r0 >= rowBeg && r0 < rowEnd) cnt = 1;
                }
            }
            int inc = cnt;  // warp scan of the row counts
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            T.base[lane] = inc - cnt;  // triangles with no rows get the next one's base
            T.r0[lane] = (unsigned char)r0;
            const int total = __shfl_sync(0xffffffffu, inc, 31);

            for (int round = 0; round < total; round += 32) {
                T.mask[lane] = 0u;
                __syncwarp();  // staging, bases and cleared masks are visible; the last walk is done
                // ---- set-up: lane = span g of the round -- the row result and
                // span set-up, then the exact z of each of its bin columns by
                // the sequential steps from leftClamped
                const int g = round + lane;
                if (g < total) {
                    int j = 0;  // the triangle of span g: the last one whose first span is <= g
#pragma unroll
                    for (int step = 16; step; step >>= 1)
                        if (T.base[j + step] <= g) j += step;
                    const int r = T.r0[j] + (g - T.base[j]);
                    // the span's columns in the bin and its interpolation
                    // state at pixel k0: from a span item as set up, or from
                    // the triangle (the row result and span set-up)
                    bool live;
                    int xs, xe, k0, sflags;
                    SpanZ z;
                    float4 rec[4];  // the item's record, staged by this chunk: an L1 hit
                    load_item(P, T.item[j], rec);
                    if (T.lw[j] < 0) {
                        const SpanItem& si = *reinterpret_cast<const SpanItem*>(rec);
                        live = true;
                        xs = k0 = si.xs;
                        xe = si.xe;
                        sflags = si.flags;
                        z.cf2 = si.cf2;
                        z.pz = si.pz;
                        z.cf2Step = si.cf2Step;
                        z.pzStep = si.pzStep;
                    } else {
                        live = triangle_span<true>(*reinterpret_cast<const TriRaster*>(rec), y0 + r - T.oy[j], T.lw[j],
                                                   T.ox[j], x0, cols, xs, xe, k0, sflags, z);
                    }
                    if (live) {
                        if (xs <= xe) {
                            // a span no depth test can pass is dropped here
                            // (counted as tested, as the walk would)
                            if (cull && (sflags & B_TEST_DEPTH) && span_occluded(z, xs - k0, xe - k0, T.rowMax[r])) {
                                tested += (unsigned long long)(xe - xs + 1);
                                xe = xs - 1;
                            }
                            if (xs <= xe) {
                                float cf2 = z.cf2, pz = z.pz;
                                for (int x = k0; x < xs; x++) {
                                    cf2 = fadd(cf2, z.cf2Step);
                                    pz = fadd(pz, z.pzStep);
                                }
                                float* zr = T.z + lane * S - x0;
                                float zmin = INFINITY;
                                for (int x = xs; x <= xe; x++) {
                                    const float zz = fmul(pz, frcp(cf2));
                                    cf2 = fadd(cf2, z.cf2Step);
                                    pz = fadd(pz, z.pzStep);
                                    zr[x] = zz;
                                    zmin = fminf(zmin, zz);
                                }
                                T.xs[lane] = (short)(xs - x0);
                                T.xe[lane] = (short)(xe - x0);
                                T.flags[lane] = (short)sflags;
                                T.j[lane] = (unsigned char)j;
                                T.zmin[lane] = zmin;
                                atomicOr(&T.mask[r], 1u << lane);
                            }
                        }
                    }
                }
                __syncwarp();
                // ---- walk: lane = row, its spans in triangle order -- the
                // reference's depth test and writes (fragthrd.cpp:208-252).  A
                // span whose min z fails against the row's maximum depth is
                // skipped: under TEST_DEPTH depths only decrease, so the
                // maximum stays an upper bound and the skip changes nothing.
                if (myRow) {
                    unsigned bits = T.mask[lane];
                    if (bits) {
                        float curMax = -INFINITY;
                        for (int c = 0; c < cols; c++) curMax = fmaxf(curMax, dRow[c]);
                        while (bits) {
                            const int s = __ffs(bits) - 1;
                            bits &= bits - 1;
                            const int a = T.xs[s], b = T.xe[s], flags = T.flags[s];
                            tested += (unsigned long long)(b - a + 1);
                            if ((flags & B_TEST_DEPTH) && fsub(T.zmin[s], curMax) >= -0.0001f) continue;
                            const float* zr = T.z + s * S;
                            const int triId = T.tid[T.j[s]];
                            for (int x = a; x <= b; x++) {
                                const float zz = zr[x];
                                const float cur = (flags & B_TEST_DEPTH) ? dRow[x] : 1.0f;
                                if (-1.0f < zz && fsub(zz, cur) < -0.0001f) {
                                    if (flags & B_UPDATE_DEPTH) dRow[x] = zz;
                                    if (flags & F_COLOUR) wRow[x] = triId;
                                    passed++;
                                }
                            }
                            if (!(flags & B_TEST_DEPTH)) {  // depth may have risen: recompute the bound
                                curMax = -INFINITY;
                                for (int c = 0; c < cols; c++) curMax = fmaxf(curMax, dRow[c]);
                            }
                        }
                        T.rowMax[lane] = curMax;  // for the next round's occlusion test
                    }
                }
            }
        }
        __syncwarp();

        // ---- depth write-back, then the shade list: row by row, each row's
        // covered pixels left to right (one reservation per warp), and the
        // clear colour of the uncovered pixels
        if (vec) {
            for (int i = lane; i < nPx / 4; i += 32) {
                const int r = rowBeg + (4 * i) / BW, c = (4 * i) % BW;
                const float* t = T.depth + r * S + c;
                *(float4*)(P.depth + (size_t)(y0 + r) * P.depthScan + x0 + c) = make_float4(t[0], t[1], t[2], t[3]);
            }
        } else {
            for (int i = lane; i < nPx; i += 32) {
                const int r = rowBeg + i / BW, c = i % BW;
                if (c < cols) P.depth[(size_t)(y0 + r) * P.depthScan + x0 + c] = T.depth[r * S + c];
            }
        }
        int covered = 0;
        if (P.anyColour || P.clearColour) {
            int listBase = 0;
            if (P.anyColour) {
                int total = 0;
                for (int i = 0; i < nPx; i += 32) {
                    const int q = i + lane, r = rowBeg + q / BW, c = q % BW;
                    total += __popc(__ballot_sync(0xffffffffu, q < nPx && c < cols && T.win[r * S + c] >= 0));
                }
                if (lane == 0 && total) listBase = atomicAdd(P.slotStatus + kSlotShade, total);
                listBase = __shfl_sync(0xffffffffu, listBase, 0);
            }
            const unsigned below = (1u << lane) - 1u;
            for (int i = 0; i < nPx; i += 32) {
                const int q = i + lane, r = rowBeg + q / BW, c = q % BW;
                const bool in = q < nPx && c < cols;
                const int w = in ? T.win[r * S + c] : -1;
                const unsigned b = __ballot_sync(0xffffffffu, w >= 0);
                if (w >= 0) {
                    if (P.anyColour) P.shadeList[listBase + __popc(b & below)] = make_int2(shade_pixel(x0 + c, y0 + r), w);
                    covered++;
                } else if (in && P.clearColour) {
                    clear_colour_px(P, x0 + c, y0 + r);
                }
                listBase += __popc(b);
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

// Blocks of kern resident on the current device at once (cached per kernel
// and device).
static int warp_raster_resident(const void* kern)
{
    thread_local std::vector<std::pair<std::pair<const void*, int>, int>> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    for (const auto& e : cache)
        if (e.first.first == kern && e.first.second == dev) return e.second;
    int sms = 0, perSM = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, kWarpRasterThreads, 0);
    const int resident = std::max(sms, 1) * std::max(perSM, 1);
    cache.push_back({{kern, dev}, resident});
    return resident;
}

template <int BW, int MINB, bool CULL> static void launch_one(const PassParams& P, int nBins, cudaStream_t s)
{
    auto* kern = k_raster_warp<BW, MINB, CULL>;
    // a persistent grid: as many blocks as fit at once, no more warps than work items
    const long long items = (long long)nBins * std::max(P.rowSplit, 1);
    const long long want = (items + kWarpRasterWarps - 1) / kWarpRasterWarps;
    const int grid = (int)std::max<long long>(1, std::min<long long>(want, warp_raster_resident((const void*)kern)));
    kern<<<grid, kWarpRasterThreads, 0, s>>>(P);
}

// The warp raster for bins of 8 or 16 columns (the host falls back to
// k_raster for wider bins and for forward passes).
void launch_raster_warp(const PassParams& P, int nBins, cudaStream_t s)
{
    if (P.binW == 8) {
        if (P.cullSpans) launch_one<8, 8, true>(P, nBins, s);
        else launch_one<8, 8, false>(P, nBins, s);
    } else {
        if (P.cullSpans) launch_one<16, 7, true>(P, nBins, s);
        else launch_one<16, 7, false>(P, nBins, s);
    }
}

}  // namespace ps3d
