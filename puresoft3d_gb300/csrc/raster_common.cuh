// raster_common.cuh -- device helpers shared by the two raster kernels
// (k_raster: four warps share a bin; k_raster_warp: each warp owns a bin).
#pragma once
#include "device_common.cuh"

namespace ps3d {

__device__ __forceinline__ void bin_range(const PassParams& P, int bin, int& start, int& end)
{
    if (P.slotStatus[kSlotTiles] == 0) {  // no pairs
        start = end = 0;
        return;
    }
    const int2 r = ((const int2*)P.binStart)[bin];  // (start, end) in the sorted list; start >= end: empty
    start = r.x < r.y ? r.x : 0;
    end = r.x < r.y ? r.y : 0;
}

// The colour target's pixel (x, y).
__device__ __forceinline__ uint32_t* colour_px(const PassParams& P, int x, int y)
{
    return P.colourRow0 + (ptrdiff_t)y * P.colourPitch + x;
}

// A shade-list entry's pixel: y in the high and x in the low 16 bits
// (targets are at most 32767 pixels a side), so that the shade needs no
// division to find them.
__device__ __forceinline__ int shade_pixel(int x, int y) { return (y << 16) | x; }

// The pass's clear colour at target pixel (x, y).
__device__ __forceinline__ void clear_colour_px(const PassParams& P, int x, int y)
{
    *colour_px(P, x, y) = P.colourClearValue;
}

// True when no pixel kA..kB (steps from leftClamped) of a span can pass a
// depth test against depths <= curMax -- i.e. every z the per-pixel loop
// would compute satisfies z - cur >= -0.0001f -- decided without running the
// loop.  The loop's values are z_k = fl(S_k * rcp(C_k)) with S_k, C_k the
// sequential float sums S0 + dS + ... and C0 + dC + ...  Against the exact
// T(k) = S0 + k dS and U(k) = C0 + k dC: each of the k additions errs by at
// most 2^-24 |S_i| <= 2^-23 max|T| (likewise C), so |S_k - T(k)| <= eS =
// k 2^-23 AS; with U > 0 on the span, T/U is monotonic, so its minimum is at
// an end point, and |z_k - T/U| <= (eS + Tmax eC / Umin) / Umin plus two
// roundings.  Every bound below is taken at least twice as loose as this
// derivation needs (evaluation errors of the bounds themselves included),
// and anything non-finite or a U near zero keeps the span.
__device__ __forceinline__ bool span_occluded(const SpanZ& z, int kA, int kB, float curMax)
{
    const float S0 = z.pz, C0 = z.cf2, dS = z.pzStep, dC = z.cf2Step;
    const float fA = (float)kA, fB = (float)kB;
    const float TA = S0 + fA * dS, TB = S0 + fB * dS, UA = C0 + fA * dC, UB = C0 + fB * dC;
    const float evT = 0x1p-21f * (fabsf(S0) + fB * fabsf(dS)), evU = 0x1p-21f * (fabsf(C0) + fB * fabsf(dC));
    const float AS = fmaxf(fabsf(S0), fabsf(TB)) + evT, AC = fmaxf(fabsf(C0), fabsf(UB)) + evU;
    const float eS = fB * 0x1p-22f * AS + 1e-37f, eC = fB * 0x1p-22f * AC + 1e-37f;
    const float Umin = fminf(UA, UB) - evU - eC;
    if (!(Umin > 1e-30f) || !(Umin < 1e30f)) return false;
    const float Tmax = fmaxf(fabsf(TA), fabsf(TB)) + evT + eS;
    // fast quotients (2 ulp for divisors in [2^-126, 2^126]): the bound's slack covers them
    const float fmin = fminf(__fdividef(TA, UA), __fdividef(TB, UB));
    const float rU = __fdividef(1.0f, Umin);
    const float delta = 2.0f * ((eS + evT + Tmax * (eC + evU) * rU) * rU) + (Tmax * rU) * 0x1p-19f;
    const float lhs = fmin - delta - curMax;
    const float slack = (fabsf(fmin) + fabsf(curMax) + delta) * 1e-6f;
    return lhs - slack >= -0.0001f;  // false for NaN
}

// The work list's bucket ends (running sums of the counts k_bin_bounds left
// in the slot status; fixed while the raster runs), written to sEnd by
// thread 0 of the block; the caller synchronises before next_bin_item.
__device__ __forceinline__ void load_item_buckets(const PassParams& P, int* sEnd)
{
    if (threadIdx.x == 0) {
        int n[kItemBuckets];
#pragma unroll
        for (int b = 0; b < kItemBuckets; b++) n[b] = __ldcg(P.slotStatus + kSlotBucket + b);
        int run = 0;
#pragma unroll
        for (int b = 0; b < kItemBuckets; b++) {
            run += n[b];
            sEnd[b] = run;
        }
    }
}

// The next work item of the pass's list (k_bin_bounds): the crowded bins'
// row slices, then the other bins by size, then the empty ones; -1 when done.
// sEnd: the bucket ends from load_item_buckets.
__device__ __forceinline__ int next_bin_item(const PassParams& P, const int* sEnd)
{
    const int i = atomicAdd(P.slotStatus + kSlotCursor, 1);
    const int nBins = P.binsX * P.binsY;
    int start = 0;
#pragma unroll
    for (int b = 0; b < kItemBuckets; b++) {
        if (i < sEnd[b]) return __ldcg(P.binItems + bucket_base(b, nBins) + (i - start));
        start = sEnd[b];
    }
    return -1;
}

// The record of a bin list item: a triangle's (64 bytes) or a span item's
// (32 bytes, in rec[0..1]).
__device__ __forceinline__ void load_item(const PassParams& P, int v, float4 rec[4])
{
    if (v >= 0) {
        const float4* src = (const float4*)(P.tris + v);
#pragma unroll
        for (int k = 0; k < 4; k++) rec[k] = __ldg(src + k);
    } else {
        const float4* src = (const float4*)(P.spans + ~v);
        rec[0] = __ldg(src);
        rec[1] = __ldg(src + 1);
    }
}

// The span of triangle t on its rasteriser row yl, clipped to the bin's
// columns [x0, x0 + cols): the row result (rasterizer.cpp:93-118) and the
// span set-up (interp.cpp:26-80), whose state is at pixel k0 = leftClamped
// (in target columns).  False when the row has no span.
// kRegs: t is held in registers (vertex selects instead of indexed loads).
template <bool kRegs = false>
__device__ __forceinline__ bool triangle_span(const TriRaster& t, int yl, int lw, int ox, int x0, int cols, int& xs,
                                              int& xe, int& k0, int& sflags, SpanZ& z)
{
    Span sp;
    if (!span_row<kRegs>(t, yl, lw, sp)) return false;
    xs = max(sp.leftClamped + ox, x0);
    xe = min(sp.rightClamped + ox, x0 + cols - 1);
    k0 = sp.leftClamped + ox;
    sflags = t.edges >> 16;
    if (xs <= xe) span_z(t, sp, yl, z);
    return true;
}

}  // namespace ps3d
