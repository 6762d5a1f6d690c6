// setup_bin.cu -- vertex stage, triangle set-up and ordered tile binning.
//
//   k_setup_emit  one thread per triangle: VBO fetch, vertex processor,
//                 perspective divide, back-face cull, z-reject and the
//                 rasteriser's triangle set-up (reference drawvao.cpp:36-63,
//                 vertthrd.cpp:14-65, rasterizer.cpp:73-234), the bin
//                 rectangle the triangle's spans can touch, and -- after a
//                 scan of the pair counts across groups of triangles by
//                 decoupled look-back -- its (bin, triangle) pairs in
//                 triangle order.
//   k_onesweep    stable LSD radix passes over the pairs by bin, so that
//                 each bin lists its triangles in submission order -- per
//                 pixel the reference applies fragments in that order (its
//                 per-row FIFO queues, drawvao.cpp:77-109), and the depth
//                 test's epsilon makes the order observable
//                 (fragthrd.cpp:227).
//   k_bin_bounds  the raster's work list from each bin's range in the
//                 sorted list (the last radix pass writes the ranges).
#include <cuda_runtime.h>
#include "vertex_stage.cuh"

namespace ps3d {

// Triangles of at most this many rows get exact bin bounds and row range from
// their spans in the set-up (and none when no row has a pixel).
constexpr int kExactRows = 32;

// isBackFace (vertthrd.cpp:56-65): the z of cross(v1 - v0, v2 - v1) scaled by
// rsqrtss(|c|^2), compared with 0.  The scale factor is finite and positive
// exactly when |c|^2 (haddps order) is a finite normal number; otherwise the
// reference's dot product is NaN or +-0 and the face is kept.
__device__ __forceinline__ bool back_face(const float p[3][4])
{
    float a[4], b[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        a[k] = fsub(p[1][k], p[0][k]);
        b[k] = fsub(p[2][k], p[1][k]);
    }
    float c0 = fsub(fmul(a[1], b[2]), fmul(a[2], b[1]));
    float c1 = fsub(fmul(a[2], b[0]), fmul(a[0], b[2]));
    float c2 = fsub(fmul(a[0], b[1]), fmul(a[1], b[0]));
    float c3 = fsub(fmul(a[3], b[3]), fmul(a[3], b[3]));
    float s = fadd(fadd(fmul(c0, c0), fmul(c1, c1)), fadd(fmul(c2, c2), fmul(c3, c3)));
    if (!(s >= FLT_MIN && s <= FLT_MAX)) return false;
    if (!isfinite(c0) || !isfinite(c1) || !isfinite(c3)) return false;
    return c2 < 0.0f;
}

__device__ __forceinline__ int edge_code(int a, int b) { return a | (b << 2); }

constexpr int kSetupThreads = 128;
constexpr int kSetupDrawCache = 512;  // draws whose first triangles the set-up keeps in shared memory

// itemized: the triangle's pairs are span items (one per row span and bin),
// emitted by emit_span_items after the look-back; otherwise one pair per bin
// of `rect`.
// The draw of triangle t (the last draw whose first triangle is <= t), for
// every lane of a warp whose triangles are consecutive from `first` (t <
// nTris for the lanes that use it).  sBase: the draws' first triangles in
// shared memory -- a binary search there; null: the warp finds the draw of
// `first` by a 32-way search over the draw table (probe loads per round, 3
// rounds for 4096 draws), then each lane steps forward over the draws that
// start at or before its triangle.
__device__ __forceinline__ int draw_of(const PassParams& P, int t, int first, const int* sBase)
{
    const int lane = threadIdx.x & 31;
    int lo = 0, hi = P.nDraws - 1;
    if (sBase) {
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (sBase[mid] <= t) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    }
    while (lo < hi) {  // warp-uniform; draws[lo].triBase <= first throughout
        const int n = hi - lo;
        const int c = lo + (int)(((long long)n * (lane + 1) + 31) / 32);  // lo < c <= hi, nondecreasing in lane
        const unsigned m = __ballot_sync(0xffffffffu, __ldg(&P.draws[c].triBase) <= first);
        const int L = __popc(m);  // the candidates at or before `first` are lanes 0 .. L-1
        const int cHi = __shfl_sync(0xffffffffu, c, L < 32 ? L : 31);
        lo = L ? __shfl_sync(0xffffffffu, c, L - 1) : lo;
        hi = L < 32 ? cHi - 1 : hi;
        if (L == 32) lo = hi;
    }
    while (lo + 1 < P.nDraws && __ldg(&P.draws[lo + 1].triBase) <= t) lo++;
    return lo;
}

__device__ __forceinline__ void setup_triangle(const PassParams& P, int t, int drawIdx, float* sVary, int& pairs,
                                               int4& rect, bool& itemized)
{
    const int lo = drawIdx;
    const DrawDesc& d = P.draws[lo];
    const DrawUniforms& U = P.unis[d.uni];
    int lt = t - d.triBase;

    float pos[3][4], rw[3], pz[3];
#pragma unroll
    for (int v = 0; v < 3; v++) {
        vp_position(d, U, 3 * lt + v, pos[v]);
        float r = frcp(pos[v][3]);  // vertthrd.cpp:37-47: 1/w, then a 4-wide multiply
#pragma unroll
        for (int k = 0; k < 4; k++) pos[v][k] = fmul(pos[v][k], r);
        pz[v] = pos[v][2];
        rw[v] = r;
    }

    TriRaster tr;
    tr.draw = lo;
    tr.split = INT_MAX;
    tr.edges = (d.flags & 0xff) << 16;
    tr.firstRow = 1;
    tr.lastRow = 0;
    int count = 0;
    bool keep = true;
    if ((d.flags & B_FACE_CULLING) && back_face(pos)) keep = false;
#pragma unroll
    for (int v = 0; v < 3; v++)
        if (pos[v][2] < -1.0f || pos[v][2] > 1.0f) keep = false;  // drawvao.cpp:51-56

    const int W = d.vpW, H = d.vpH, halfW = W / 2, halfH = H / 2;  // the draw's rasteriser size
#pragma unroll
    for (int v = 0; v < 3; v++) {
        tr.vx[v] = fadd(fmul((float)halfW, pos[v][0]), (float)halfW);  // rasterizer.cpp:73-77
        tr.vy[v] = fadd(fmul((float)halfH, pos[v][1]), (float)halfH);
        tr.rw[v] = rw[v];
        tr.pz[v] = pz[v];
    }
    int bx0 = 0, bx1 = -1, by0 = 0, by1 = -1;
    if (keep) {
        const float* vx = tr.vx;
        const float* vy = tr.vy;
        // pushVertex's running min / max of (int)y (rasterizer.cpp:78-89)
        int firstRow = f2i(vy[0]), lastRow = firstRow;
#pragma unroll
        for (int v = 1; v < 3; v++) {
            if (vy[v] > (float)lastRow) lastRow = f2i(vy[v]);
            else if (vy[v] < (float)firstRow) firstRow = f2i(vy[v]);
        }
        bool finite = isfinite(vx[0]) && isfinite(vx[1]) && isfinite(vx[2]) && isfinite(vy[0]) && isfinite(vy[1]) &&
                      isfinite(vy[2]);
        if (firstRow >= H || lastRow < 0) {  // rasterizer.cpp:149-168
            firstRow = 0;
            lastRow = -1;
        }
        if (firstRow < 0) firstRow = 0;
        if (lastRow >= H) lastRow = H - 1;
        if (finite && firstRow != lastRow && firstRow <= lastRow) {
            int lower, upper = 0, split = INT_MAX;
            if (vy[0] == vy[1]) {  // flat cases (rasterizer.cpp:171-203)
                lower = vx[0] < vx[1] ? edge_code(0, 2) | (edge_code(1, 2) << 4) : edge_code(1, 2) | (edge_code(0, 2) << 4);
            } else if (vy[0] == vy[2]) {
                lower = vx[0] < vx[2] ? edge_code(0, 1) | (edge_code(2, 1) << 4) : edge_code(2, 1) | (edge_code(0, 1) << 4);
            } else if (vy[1] == vy[2]) {
                lower = vx[1] < vx[2] ? edge_code(1, 0) | (edge_code(2, 0) << 4) : edge_code(2, 0) | (edge_code(1, 0) << 4);
            } else {  // sort by y, then split at the middle vertex (rasterizer.cpp:205-233, 121-140)
                int top, bottom, third = 2, tmp;
                if (vy[0] > vy[1]) { top = 0; bottom = 1; }
                else { top = 1; bottom = 0; }
                if (sel3(vy, top) < vy[2]) { tmp = top; top = third; third = tmp; }
                else if (sel3(vy, bottom) > vy[2]) { tmp = bottom; bottom = third; third = tmp; }
                Edge tt = mk_edge<true>(vx, vy, top, third), tb = mk_edge<true>(vx, vy, top, bottom);
                float yt = sel3(vy, third);
                if (edge_at(tb, yt) > edge_at(tt, yt)) {  // pointing left
                    upper = edge_code(top, third) | (edge_code(top, bottom) << 4);
                    lower = edge_code(third, bottom) | (edge_code(top, bottom) << 4);
                } else {
                    upper = edge_code(top, bottom) | (edge_code(top, third) << 4);
                    lower = edge_code(top, bottom) | (edge_code(third, bottom) << 4);
                }
                // the lower half is processed second, so it owns the shared row
                split = yt > (float)(H - 1) ? H - 1 : f2i(yt);
            }
            tr.edges |= lower | (upper << 8);
            tr.split = split;
            tr.firstRow = (short)firstRow;
            tr.lastRow = (short)lastRow;
            // Column bounds (conservative; only used for binning).  Each edge
            // is evaluated at rows within (its lowest y - 1, its highest y]
            // (row numbers are truncations), so a span end lies within the
            // triangle's x range widened by one row of the steepest edge's
            // run |dx/dy|, plus the +0.5 rounding and a pixel of margin.
            float ext = 0.0f;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                int b2 = a == 2 ? 0 : a + 1;
                float dy = fabsf(vy[b2] - vy[a]), dx = fabsf(vx[b2] - vx[a]);
                if (dy >= 0.000001f) ext = fmaxf(ext, __fdividef(dx, dy) * 1.0001f);
            }
            float xmin = fminf(vx[0], fminf(vx[1], vx[2])) - ext - 2.0f;
            float xmax = fmaxf(vx[0], fmaxf(vx[1], vx[2])) + ext + 2.0f;
            int colLo = xmin < 0.0f ? 0 : (xmin > (float)W ? W : (int)xmin);
            int colHi = xmax > (float)(W - 1) ? W - 1 : (xmax < 0.0f ? -1 : (int)xmax);
            int rowLo = firstRow, rowHi = lastRow;
            if (lastRow - firstRow < kExactRows) {
                // a short triangle: its rows' spans exactly, as the raster will
                // find them (drawvao.cpp:72-75 skips left == right; the fragment
                // loop covers [leftClamped, rightClamped]); one with no pixel
                // reaches no bin, the others only the bins their spans touch
                int lo = W, hi = -1, yLo = lastRow, yHi = firstRow, items = 0;
#pragma unroll 1
                for (int y = firstRow; y <= lastRow; y++) {
                    Span sp;
                    if (span_row<true>(tr, y, W, sp) && sp.leftClamped <= sp.rightClamped) {
                        lo = min(lo, sp.leftClamped);
                        hi = max(hi, sp.rightClamped);
                        yLo = min(yLo, y);
                        yHi = max(yHi, y);
                        // span items: one per bin the row's span touches
                        items += (sp.rightClamped + d.vpX) / P.binW - (sp.leftClamped + d.vpX) / P.binW + 1;
                    }
                }
                itemized = P.spanItems && lo <= hi;
                if (itemized) count = items;
                colLo = lo;
                colHi = hi;
                rowLo = yLo;
                rowHi = yHi;
                if (lo <= hi) {  // the raster's row range: only rows with pixels
                    tr.firstRow = (short)yLo;
                    tr.lastRow = (short)yHi;
                }
            }
            if (colLo <= colHi && !itemized) {  // bins are in target pixels: offset by the viewport origin
                bx0 = (colLo + d.vpX) / P.binW;
                bx1 = (colHi + d.vpX) / P.binW;
                by0 = (rowLo + d.vpY) / kBinH;
                by1 = (rowHi + d.vpY) / kBinH;
                count = (bx1 - bx0 + 1) * (by1 - by0 + 1);
            }
        }
    }
    if (count == 0) {
        tr.firstRow = 1;
        tr.lastRow = 0;
        itemized = false;
    }
    float4* dst = (float4*)(P.tris + t);
    const float4* src = (const float4*)&tr;
#pragma unroll
    for (int k = 0; k < 4; k++) dst[k] = src[k];
    pairs = count;
    rect = make_int4(bx0, bx1, by0, by1);
    if (count > 0 && d.nv && !P.lazyVary) {
        // the varyings of a triangle that reaches a bin (no other is ever read)
        float* vout = sVary + threadIdx.x * 3 * P.nvMax;
#pragma unroll 1
        for (int v = 0; v < 3; v++) {
            float vary[kMaxVary];
            vp_varyings(d, U, 3 * lt + v, vary);
            // constant trip counts keep `vary` in registers
            switch (d.nv) {
            case 2:
                vout[v * P.nvMax] = vary[0];
                vout[v * P.nvMax + 1] = vary[1];
                break;
            case 3:
#pragma unroll
                for (int k = 0; k < 3; k++) vout[v * P.nvMax + k] = vary[k];
                break;
            case 9:
#pragma unroll
                for (int k = 0; k < 9; k++) vout[v * P.nvMax + k] = vary[k];
                break;
            case 11:
#pragma unroll
                for (int k = 0; k < 11; k++) vout[v * P.nvMax + k] = vary[k];
                break;
            case 13:
#pragma unroll
                for (int k = 0; k < 13; k++) vout[v * P.nvMax + k] = vary[k];
                break;
            case 16:
#pragma unroll
                for (int k = 0; k < 16; k++) vout[v * P.nvMax + k] = vary[k];
                break;
            case 17:
#pragma unroll
                for (int k = 0; k < 17; k++) vout[v * P.nvMax + k] = vary[k];
                break;
            case 21:
#pragma unroll
                for (int k = 0; k < 21; k++) vout[v * P.nvMax + k] = vary[k];
                break;
            }
        }
    }
}

// The span items of an itemized triangle, from pair offset o on, in
// (row, bin) order: each row's span set-up (interp.cpp:26-80) and, bin by
// bin, the sequential steps (interp.cpp:82-92) to the span's first pixel in
// the bin, so that the raster starts there.  The radix digit histograms of
// the items' bins are counted here too.  Items past the pair capacity are
// not written (the pass has failed and will be re-run).
__device__ __forceinline__ void emit_span_items(const PassParams& P, int t, long long o,
                                                int (*hist)[kRadixDigits])
{
    TriRaster tr;
    {
        const float4* src = (const float4*)(P.tris + t);
        float4* d4 = (float4*)&tr;
#pragma unroll
        for (int k = 0; k < 4; k++) d4[k] = src[k];
    }
    const DrawDesc& d = P.draws[tr.draw];
    const int W = d.vpW, ox = d.vpX, oy = d.vpY, flags = tr.edges >> 16;
#pragma unroll 1
    for (int y = tr.firstRow; y <= tr.lastRow; y++) {
        Span sp;
        if (!span_row<true>(tr, y, W, sp) || sp.leftClamped > sp.rightClamped) continue;
        SpanZ z;
        span_z(tr, sp, y, z);
        const int ty = y + oy, by = ty / kBinH;
        const int xa = sp.leftClamped + ox, xb = sp.rightClamped + ox;
        float cf2 = z.cf2, pz = z.pz;
        int x = xa;  // the pixel the state is at
        for (int bx = xa / P.binW; bx <= xb / P.binW; bx++, o++) {
            const int a = max(xa, bx * P.binW), b = min(xb, bx * P.binW + P.binW - 1);
            for (; x < a; x++) {
                cf2 = fadd(cf2, z.cf2Step);
                pz = fadd(pz, z.pzStep);
            }
            const int key = by * P.binsX + bx;
            for (int ps = 0; ps < P.radixPasses; ps++) atomicAdd(&hist[ps][(key >> (8 * ps)) & 255], 1);
            if (o >= P.pairCap) continue;
            P.pairKey[o] = key;
            P.pairTri[o] = ~(int)o;
            SpanItem si;
            si.cf2 = cf2;
            si.pz = pz;
            si.cf2Step = z.cf2Step;
            si.pzStep = z.pzStep;
            si.tri = t;
            si.xs = (short)a;
            si.xe = (short)b;
            si.y = ty;
            si.flags = flags;
            float4* dst = (float4*)(P.spans + o);
            const float4* s4 = (const float4*)&si;
            dst[0] = s4[0];
            dst[1] = s4[1];
        }
    }
}

// Set-up, pair offsets and pair emission in one kernel, over groups of
// kSetupThreads triangles numbered by an atomic ticket (so a group's
// predecessors are always held by running blocks).  A group is set up by one
// block, a thread per triangle (vertex processor, divide, cull, z-reject,
// row range, bin rectangle); its varyings go out through shared memory so
// that the stores are contiguous; its pair counts are scanned in the block
// and its total published as a look-back descriptor.  Its global offset is
// then found by decoupled look-back over the earlier groups (64-bit
// descriptors: flag << 62 | value; each wait bounded) and every triangle
// writes its (bin, triangle) pairs in triangle order; the radix sort's digit
// histograms are counted in shared memory.  The grid is persistent and
// software-pipelined: a block looks back for its group and emits its pairs
// only after it has set up its next group, so that the earlier groups have
// had a group's set-up time to publish and the block's warps do not idle at
// the look-back.  The holder of the last group records the pass's pair
// count and sort tiles, or the overflow when the pairs do not fit (pairs past
// the capacity are never written).  The header (tickets, histograms) and
// all descriptors are zeroed by a memset before the kernel.
constexpr int kLookbackSpins = 1 << 22;  // bounded waits: ~0.1 s and more, then the pass fails
constexpr unsigned long long kDescAgg = 1ull << 62, kDescPrefix = 2ull << 62, kDescValue = (1ull << 62) - 1;

__global__ void __launch_bounds__(kSetupThreads, 8) k_setup_emit(PassParams P)
{
    extern __shared__ float sVary[];  // kSetupThreads * 3 * nvMax floats (dynamic: sized by the pass)
    __shared__ int sHist[kRadixMaxPasses][kRadixDigits];
    __shared__ int sWarp[kSetupThreads / 32];
    __shared__ int sTicket, sPrefix, sPendTotal;
    __shared__ int sDrawBase[kSetupDrawCache];  // the draws' first triangles, for the draw search
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nGroups = (P.nTris + kSetupThreads - 1) / kSetupThreads;
    for (int i = tid; i < kRadixMaxPasses * kRadixDigits; i += kSetupThreads) (&sHist[0][0])[i] = 0;
    const int* drawBase = P.nDraws <= kSetupDrawCache ? sDrawBase : nullptr;
    if (drawBase)
        for (int i = tid; i < P.nDraws; i += kSetupThreads) sDrawBase[i] = P.draws[i].triBase;
    if (P.radixPasses > 0) {  // every bin's (start, end) starts empty: the last radix pass fills them in
        const int nBins = P.binsX * P.binsY;
        for (int i = blockIdx.x * kSetupThreads + tid; i < nBins; i += gridDim.x * kSetupThreads)
            ((int2*)P.binStart)[i] = make_int2(INT_MAX, 0);
    }
    volatile unsigned long long* desc = (volatile unsigned long long*)(P.radix + kRadixHdr);

    // the group set up but not yet emitted: its number (-1 none; its total in
    // sPendTotal) and this thread's offset in the group and bin rectangle
    // (columns and rows as two 16-bit halves each)
    int pend = -1, pendOff = 0, pendCols = -65536, pendRows = -65536;  // empty: 0 .. -1
    bool pendItem = false;
    for (;;) {
        if (tid == 0) sTicket = atomicAdd(P.radix + kTicketSetup, 1);
        __syncthreads();  // the ticket is ready; the previous group's shared data are no longer read
        const int g = sTicket < nGroups ? sTicket : -1;
        int count = 0, off = 0, total = 0;
        int4 rect = make_int4(0, -1, 0, -1);
        bool itemized = false;
        const int first = g * kSetupThreads, t = first + tid;
        if (g >= 0) {
            const int drawIdx = draw_of(P, min(t, P.nTris - 1), first + 32 * warp, drawBase);
            if (t < P.nTris) setup_triangle(P, t, drawIdx, sVary, count, rect, itemized);
            if (g == 0 && tid == 0) P.slotStatus[kSlotShade] = 0;  // the shade list starts empty
            if (g == 0 && tid < kItemBuckets + 1) P.slotStatus[kSlotBucket + tid] = 0;  // the work list too
            // block scan of the pair counts
            int inc = count;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            if (lane == 31) sWarp[warp] = inc;
        }
        __syncthreads();  // sWarp and the staged varyings are complete (and sTicket read)
        if (g >= 0) {
            if (P.anyVary && !P.lazyVary) {
                int n = min(kSetupThreads, P.nTris - first), nf = n * 3 * P.nvMax;
                float* dst = P.vary + (size_t)first * 3 * P.nvMax;
                for (int i = tid; i < nf; i += kSetupThreads) dst[i] = sVary[i];
            }
            int wbase = 0;
#pragma unroll
            for (int w = 0; w < kSetupThreads / 32; w++) {
                int v = sWarp[w];
                if (w < warp) wbase += v;
                total += v;
            }
            off = wbase;
            {
                int inc = count;  // this thread's exclusive offset in the group
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    int v = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += v;
                }
                off += inc - count;
            }
            if (tid == 0)  // publish the group's total: later groups' look-backs wait on it
                desc[g] = (g == 0 ? kDescPrefix : kDescAgg) | (unsigned long long)total;
            // the radix passes' digit histograms of the group's pairs: they
            // need no offsets (when the pairs overflow the room the pass
            // fails and the counts go unused)
            const int passes = P.radixPasses;
            for (int by = rect.z; by <= rect.w; by++)
                for (int bx = rect.x; bx <= rect.y; bx++) {
                    const int key = by * P.binsX + bx;
                    for (int ps = 0; ps < passes; ps++) atomicAdd(&sHist[ps][(key >> (8 * ps)) & 255], 1);
                }
        }
        if (pend >= 0) {
            // the pending group: its offset by look-back, then its pairs
            if (warp == 0) {
                // warp-wide look-back: 32 earlier groups' descriptors per
                // step, up to and including the nearest one that holds an
                // inclusive prefix
                long long prefix = 0;
                if (pend != 0) {
                    int top = pend - 1, spins = 0;
                    while (true) {
                        const int idx = top - lane;
                        unsigned long long v = kDescPrefix | 0ull;  // before group 0: an empty prefix
                        if (idx >= 0) v = desc[idx];
                        const unsigned long long f = v & ~kDescValue;
                        const unsigned withPrefix = __ballot_sync(0xffffffffu, f == kDescPrefix);
                        const unsigned notReady = __ballot_sync(0xffffffffu, f == 0ull);
                        const int stop = withPrefix ? __ffs(withPrefix) - 1 : 31;  // lanes 0..stop are needed
                        const unsigned need = stop == 31 ? 0xffffffffu : ((2u << stop) - 1u);
                        if (notReady & need) {
                            if (++spins > kLookbackSpins) {
                                if (lane == 0) {
                                    atomicMin(P.status + kFirstFailed, P.passSeq);
                                    atomicOr(P.status, 2);
                                }
                                break;
                            }
                            __nanosleep(32);
                            continue;
                        }
                        long long val = lane <= stop ? (long long)(v & kDescValue) : 0;
#pragma unroll
                        for (int o = 16; o; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
                        prefix += val;
                        if (withPrefix) break;
                        top -= 32;
                    }
                    if (lane == 0) desc[pend] = kDescPrefix | (unsigned long long)(prefix + sPendTotal);
                }
                if (lane == 0) {
                    sPrefix = (int)min(prefix, (long long)INT_MAX);
                    if (pend == nGroups - 1) {  // the last group: the pass's total
                        long long all = prefix + sPendTotal;
                        if (all > P.pairCap) {
                            P.slotStatus[kSlotTiles] = 0;
                            P.slotStatus[kSlotTotal] = 0;
                            atomicMax(P.status + 1, (int)min(all, (long long)INT_MAX));
                            atomicMin(P.status + kFirstFailed, P.passSeq);
                            atomicOr(P.status, 1);
                        } else {
                            P.slotStatus[kSlotTotal] = (int)all;
                            P.slotStatus[kSlotTiles] = (int)((all + kSortChunk - 1) / kSortChunk);
                            atomicAdd((unsigned long long*)(P.status + 8), (unsigned long long)all);
                            // one bin, no radix pass: its list is the pairs in emission order
                            if (P.radixPasses == 0) ((int2*)P.binStart)[0] = make_int2(0, (int)all);
                        }
                    }
                }
            }
            __syncthreads();  // sPrefix is ready
            const int pt = pend * kSetupThreads + tid;
            long long o = (long long)sPrefix + pendOff;
            if (pendItem) emit_span_items(P, pt, o, sHist);
            const int bx0 = (short)(pendCols & 0xffff), bx1 = pendCols >> 16;
            const int by0 = (short)(pendRows & 0xffff), by1 = pendRows >> 16;
            for (int by = by0; by <= by1; by++)
                for (int bx = bx0; bx <= bx1; bx++, o++) {
                    if (o >= P.pairCap) continue;
                    int key = by * P.binsX + bx;
                    P.pairKey[o] = key;
                    P.pairTri[o] = pt;
                }
        }
        if (g < 0) break;  // block-uniform: nothing is pending now
        __syncthreads();  // sPendTotal and sPrefix were last read above
        if (tid == 0) sPendTotal = total;
        pend = g;
        pendOff = off;
        pendCols = (int)(((unsigned)rect.x & 0xffffu) | ((unsigned)rect.y << 16));
        pendRows = (int)(((unsigned)rect.z & 0xffffu) | ((unsigned)rect.w << 16));
        pendItem = itemized;
    }
    __syncthreads();
    for (int i = tid; i < P.radixPasses * kRadixDigits; i += kSetupThreads) {
        int v = (&sHist[0][0])[i];
        if (v) atomicAdd(P.radix + i, v);
    }
}

// Stable LSD radix sort of the pairs by bin, 8 bits per pass, one kernel per
// pass ("one sweep": each tile ranks its keys, publishes its per-digit counts
// and finds its per-digit prefix over earlier tiles by decoupled look-back).
//
// A tile is kSortChunk consecutive pairs; warp w of the block takes pairs
// [w*256, (w+1)*256) of it in 8 groups of 32 and ranks each key among the
// equal digits before it (__match_any_sync per group, a running per-warp
// count per digit), so ranks follow input order and the sort is stable.
// Tiles are numbered by an atomic ticket taken when the block starts, so a
// tile only waits for tiles whose blocks are already running; each wait is
// bounded (on expiry the pass raises status[0] = 2 and stops).
//
// Descriptor word: flag (bits 30-31: 0 not ready, 1 tile count, 2 inclusive
// prefix) | value (bits 0-29).
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortGroups = kSortChunk / kSortThreads;  // 32-key groups per warp
constexpr unsigned kFlagCount = 1u << 30, kFlagPrefix = 2u << 30, kValueMask = (1u << 30) - 1;
constexpr int kSortLookahead = 16;  // descriptors read per look-back round trip

__global__ void __launch_bounds__(kSortThreads) k_onesweep(PassParams P, int pass, const int* __restrict__ inKey,
                                                           const int* __restrict__ inTri, int* __restrict__ outKey,
                                                           int* __restrict__ outTri)
{
    __shared__ int sTicket;
    __shared__ int sWarpCnt[kSortWarps][kRadixDigits];
    __shared__ int sBase[kRadixDigits];
    __shared__ int sScan[kSortWarps];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0)  // one read of the flag for the whole block (it may change while the pass runs)
        sTicket = pass_failed(P.status, P.passSeq) ? -1 : atomicAdd(P.radix + kRadixMaxPasses * kRadixDigits + pass, 1);
    for (int i = tid; i < kSortWarps * kRadixDigits; i += kSortThreads) (&sWarpCnt[0][0])[i] = 0;
    __syncthreads();
    const int tile = sTicket;
    if (tile < 0) return;
    const int total = P.slotStatus[kSlotTotal];
    if (tile * kSortChunk >= total) return;
    const int shift = 8 * pass;
    const unsigned lt = (1u << lane) - 1u;
    const int w0 = tile * kSortChunk + warp * (kSortChunk / kSortWarps);

    int key[kSortGroups], tri[kSortGroups], rank[kSortGroups];
#pragma unroll
    for (int g = 0; g < kSortGroups; g++) {
        int i = w0 + g * 32 + lane;
        key[g] = i < total ? __ldg(inKey + i) : -1;
        tri[g] = i < total ? __ldg(inTri + i) : 0;
    }
#pragma unroll
    for (int g = 0; g < kSortGroups; g++) {
        bool valid = key[g] >= 0;
        int d = valid ? (key[g] >> shift) & 255 : -1 - lane;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int base = valid ? sWarpCnt[warp][d] : 0;
        rank[g] = base + __popc(peers & lt);
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) sWarpCnt[warp][d] = base + __popc(peers);
        __syncwarp();
    }
    __syncthreads();

    // thread = digit: offsets of the warps within the tile, the tile's count
    const int d = tid;
    int count = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; w++) {
        int v = sWarpCnt[w][d];
        sWarpCnt[w][d] = count;
        count += v;
    }
    unsigned* desc = (unsigned*)P.radix + P.sortDescOff + ((size_t)pass * P.sortBlocks) * kRadixDigits;
    volatile unsigned* mine = desc + (size_t)tile * kRadixDigits + d;
    int prefix = 0;
    if (tile == 0) {
        *mine = kFlagPrefix | (unsigned)count;
    } else {
        *mine = kFlagCount | (unsigned)count;
        int j = tile - 1, spins = 0;
        while (j >= 0) {
            // kSortLookahead predecessors' descriptors per round trip,
            // nearest first: counts are added until an inclusive prefix ends
            // the walk; a descriptor not yet published is waited for
            // (bounded).  The tiles of a pass are few and run together, so
            // the walk's round trips set the pass's length.
            unsigned v[kSortLookahead];
#pragma unroll
            for (int k = 0; k < kSortLookahead; k++)
                v[k] = j - k >= 0 ? *(volatile unsigned*)(desc + (size_t)(j - k) * kRadixDigits + d) : (unsigned)kFlagPrefix;
            int k = 0;
            bool stop = false, wait = false;
#pragma unroll
            for (; k < kSortLookahead; k++) {
                const unsigned f = v[k] & ~kValueMask;
                if (f == 0u) {
                    wait = true;
                    break;
                }
                prefix += (int)(v[k] & kValueMask);
                if (f == kFlagPrefix) {
                    stop = true;
                    break;
                }
            }
            if (stop) break;
            j -= k;  // the counts taken
            if (wait) {
                if (++spins > kLookbackSpins) {
                    atomicMin(P.status + kFirstFailed, P.passSeq);
                    atomicOr(P.status, 2);
                    __threadfence();  // the failure is visible before the prefix below
                    break;
                }
                __nanosleep(32);
            }
        }
        *mine = kFlagPrefix | (unsigned)(prefix + count);
    }
    // global start of digit d: exclusive scan of the digit counts
    int g = P.radix[pass * kRadixDigits + d];
    int inc = g;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int n = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += n;
    }
    if (lane == 31) sScan[warp] = inc;
    __syncthreads();
    int wsum = 0;
    for (int w = 0; w < warp; w++) wsum += sScan[w];
    sBase[d] = wsum + inc - g + prefix;
    __threadfence();
    __syncthreads();
    // a wait expired: prefixes may be wrong (one read per warp, so that the
    // whole warp leaves or stays for the collective below)
    if (__shfl_sync(0xffffffffu, (int)pass_failed(P.status, P.passSeq), 0)) return;
    const bool last = pass == P.radixPasses - 1;
#pragma unroll
    for (int gi = 0; gi < kSortGroups; gi++) {
        const bool valid = key[gi] >= 0;
        const int dg = (key[gi] >> shift) & 255;
        const int pos = valid ? sBase[dg] + sWarpCnt[warp][dg] + rank[gi] : 0;
        const bool put = valid && (unsigned)pos < (unsigned)total;  // false only after an expired wait
        if (put) {
            outKey[pos] = key[gi];
            outTri[pos] = tri[gi];
        }
        if (last) {
            // each bin's (start, end) in the sorted list: the group's lanes
            // with one key hold consecutive positions (ranks follow lane
            // order), so its lowest lane gives the start and its highest the end
            const unsigned peers = __match_any_sync(0xffffffffu, put ? key[gi] : -1 - lane);
            if (put && lane == __ffs(peers) - 1) atomicMin(P.binStart + 2 * key[gi], pos);
            if (put && lane == 31 - __clz(peers)) atomicMax(P.binStart + 2 * key[gi] + 1, pos + 1);
        }
    }
}

// The raster's work list, from each bin's (start, end) in the sorted list
// (written by the last radix pass): a bin with n triangles becomes s =
// min(rowSplit, the largest power of two <= n / kSliceTris) items (row
// slices when s > 1), in buckets by s, crowded first (unsliced bins by their
// triangle count); empty bins last (they still clear their pixels).  Launched only for rasters that take work items
// (row split or one warp per bin); a raster with one block per bin reads the
// ranges directly.
__global__ void k_bin_bounds(PassParams P)
{
    if (pass_failed(P.status, P.passSeq)) return;  // one load per warp: the warp leaves or stays whole
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int nBins = P.binsX * P.binsY;
    const bool valid = b < nBins;
    const int lane = threadIdx.x & 31;
    int n = 0;
    if (valid) {
        const int2 r = P.slotStatus[kSlotTiles] ? ((const int2*)P.binStart)[b] : make_int2(0, 0);
        n = r.x < r.y ? r.y - r.x : 0;
    }
    int lg = 0;
    while (lg < 3 && (1 << (lg + 1)) <= P.rowSplit && n >= (kSliceTris << (lg + 1))) lg++;
    // sliced bins by their slice count; unsliced ones with many triangles
    // ahead of the rest (their buckets have room: one item per bin), so that
    // the long items start first
    const int bucket = n == 0 ? 4 : lg > 0 ? 3 - lg : (n >= 4 * kSliceTris ? 1 : (n >= kSliceTris ? 2 : 3));
    const int k = 1 << lg;
    // one reservation per warp and bucket (thousands of bins on five
    // counters would queue at them): the lanes' items in lane order
    int at = 0;
#pragma unroll
    for (int bk = 0; bk < kItemBuckets; bk++) {
        const bool mine = valid && bucket == bk;
        const unsigned m = __ballot_sync(0xffffffffu, mine);
        if (!m) continue;
        const int v = mine ? k : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(P.slotStatus + kSlotBucket + bk, total);
        base = __shfl_sync(0xffffffffu, base, leader);
        if (mine) at = base + incl - v;
    }
    if (!valid) return;
    int* out = P.binItems + bucket_base(bucket, nBins) + at;
    for (int s = 0; s < k; s++) out[s] = b | (s << kItemSliceShift) | (lg << kItemLog2Shift);
}

// ------------------------------------------------------------------ launches

static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

int radix_passes(int nBins)
{
    int bits = 0;
    while (bits < 31 && (1 << bits) < nBins) bits++;
    return (bits + 7) / 8;
}

// The sort scratch of a pass: header (histograms, tickets), the set-up
// blocks' look-back descriptors (two ints each), the radix passes'.
int sort_desc_offset(int nTris) { return kRadixHdr + (2 * ceil_div(nTris > 0 ? nTris : 1, kSetupThreads) + 63) / 64 * 64; }

size_t radix_scratch_ints(int sortBlocks, int passes, int nTris)
{
    return (size_t)sort_desc_offset(nTris) + (size_t)passes * sortBlocks * kRadixDigits;
}

// A pass's set-up and binning in two parts (the host orders passes on
// different streams in between): the set-up with the pair emission (after
// the memset of the sort scratch it uses), then the radix passes and the bin
// starts.
int launch_setup(const PassParams& P, cudaStream_t s, int& launches, Prof* pr)
{
    size_t ints = radix_scratch_ints(P.sortBlocks, P.radixPasses, P.nTris);
    if (cudaMemsetAsync(P.radix, 0, ints * sizeof(int), s) != cudaSuccess) return -1;
    pr->begin(K_SETUP, s);
    // nvMax <= kMaxVary: < 48 KB; none when the shade computes the varyings
    const size_t varyBytes = P.lazyVary ? 0 : (size_t)kSetupThreads * 3 * P.nvMax * sizeof(float);
    // a persistent grid: at most the blocks that fit on the device at once
    // (by the pass's own staging size: resident blocks per SM cached per
    // varying count)
    static int perSm[kMaxVary + 1] = {}, sms = 0;
    const int nvKey = P.lazyVary ? 0 : std::min(std::max(P.nvMax, 0), kMaxVary);
    if (perSm[nvKey] <= 0) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_setup_emit, kSetupThreads, varyBytes);
        perSm[nvKey] = n < 1 ? 1 : n;
    }
    const int groups = ceil_div(P.nTris, kSetupThreads);
    k_setup_emit<<<std::max(1, std::min(groups, perSm[nvKey] * sms)), kSetupThreads, varyBytes, s>>>(P);
    pr->end(s);
    launches++;
    return 0;
}

void launch_sort(const PassParams& P, cudaStream_t s, int& launches, Prof* pr)
{
    int nBins = P.binsX * P.binsY;
    const int* key = P.pairKey;
    const int* tri = P.pairTri;
    pr->begin(K_SORT, s);
    for (int ps = 0; ps < P.radixPasses; ps++) {
        int* oKey = (ps & 1) ? P.pairKey : P.keyB;
        int* oTri = (ps & 1) ? P.pairTri : P.binTri;
        k_onesweep<<<P.sortBlocks, kSortThreads, 0, s>>>(P, ps, key, tri, oKey, oTri);
        key = oKey;
        tri = oTri;
        launches++;
    }
    pr->end(s);
    if (raster_uses_items(P)) {
        pr->begin(K_BOUNDS, s);
        k_bin_bounds<<<ceil_div(nBins, 256), 256, 0, s>>>(P);
        pr->end(s);
        launches++;
    }
}

}  // namespace ps3d
