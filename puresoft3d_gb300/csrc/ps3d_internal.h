// ps3d_internal.h -- data shared between the host runtime (pipeline.cpp) and
// the device kernels (raster.cu, shade.cu, bin.cu).  Not part of the C ABI.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include <vector>

namespace ps3d {

constexpr int kMaxLevels = 16;
constexpr int kMaxVary = 21;   // varying floats per vertex (the planet set: tangent, binormal, normal xyzw,
                               // worldPos xyz, uv, shadow coordinate xyzw)
// Varyings per vertex of the forward raster variant that serves a pass
// whose draws carry at most nv (the variants are compiled for 9 and 17); a
// forward pass lays its varyings out with this stride, so that the variant's
// reads stay inside each vertex's record.
constexpr int forward_vary(int nv) { return nv <= 9 ? 9 : kMaxVary; }
constexpr int kVboSlots = 5;     // VBO slots the built-in vertex stages read (0..4)
constexpr int kBinH = 32;        // bin height in rows: one warp lane per row
constexpr int kMaxBinW = 32;

// processor ids (include/ps3d.h)
enum : int {
    VP_DEF01 = 0x0101, IP_DEF01 = 0x0102, FP_DEF01 = 0x0103,
    VP_DEF02 = 0x0201, IP_DEF02 = 0x0202, FP_DEF02 = 0x0203,
    VP_DEF03 = 0x0301, IP_DEF03 = 0x0302, FP_DEF03 = 0x0303,
    VP_DEF04 = 0x0401, IP_DEF04 = 0x0402, FP_DEF04 = 0x0403,
    VP_DEF05 = 0x0501, IP_DEF05 = 0x0502, FP_DEF05 = 0x0503,
    VP_SHADOW = 0x0601,
    VP_PLANET = 0x0701, IP_PLANET = 0x0702, FP_EARTH = 0x0703, FP_SATELLITE = 0x0713,
    VP_CLOUD = 0x0801, IP_CLOUD = 0x0802, FP_CLOUD = 0x0803,
    VP_CLOUDSHADOW = 0x0901, IP_CLOUDSHADOW = 0x0902, FP_CLOUDSHADOW = 0x0903,
    // the scene viewer demo's sets (test2/testproc.h)
    VP_POSITIONONLY = 0x0A01, IP_NULL = 0x0A02, FP_SINGLECOLOURNL = 0x0A03,
    VP_SINGLECOLOUR = 0x0B01, IP_SINGLECOLOUR = 0x0B02, FP_SINGLECOLOUR = 0x0B03,
    VP_DIFFUSEONLY = 0x0C01, IP_DIFFUSEONLY = 0x0C02, FP_DIFFUSEONLY = 0x0C03,
    VP_SHADOW2 = 0x0D01, FP_NULL = 0x0D03,
    FP_LIT1 = 0x1103, FP_LIT1A = 0x1403, FP_LIT3 = 0x1303,
    VP_LIT2 = 0x1201, IP_LIT2 = 0x1202, FP_LIT2 = 0x1203,
};

// Sets the calling thread's last-error message (ps3d_last_error); returns code.
int report_error(int code, const char* msg);

// built-in post-processors (include/ps3d.h)
enum : int { PP_ADD8 = 0x7001, PP_FOG = 0x7002 };

// behaviour bits (reference pipeline.h:16-19) and per-draw flags
enum : int {
    B_UPDATE_DEPTH = 1, B_TEST_DEPTH = 2, B_FACE_CULLING = 4, B_ALPHABLEND = 8,
    F_COLOUR = 16,   // the fragment stage writes colour
    F_FRAGMENT = 32, // the fragment stage runs without writing colour (it may discard)
};

// One 2D texture level in device memory; row r starts at base + r*scanline
// (rows bottom-up, reference tex.cpp:17).
struct TexLevel {
    const uint8_t* base;
    int width, height, scanline, wrap;
};

// Per-draw snapshot of the uniforms and textures the built-in processors
// read (uniform slot convention of the reference, tex1light1.cpp:15-20).
struct DrawUniforms {
    float PV[16], M[16], Mrot[16], LPV[16], PVM[16];
    float light[4], cam[4], params[4];
    float Vrot[16];                 // DEF04: transposed view matrix, last column zeroed
    TexLevel tex;                   // DEF01 / DEF03 / LIT1 texture; DEF04 cube map face 0
    long long layerBytes;           // DEF04: bytes from one cube face to the next
    TexLevel tex2;                  // DEF03 / planet bump map
    TexLevel ptex[3];               // planet set: specular, night and shadow maps
    TexLevel albedo[kMaxLevels];    // LIT2 / LIT3 albedo chain
    TexLevel normal[kMaxLevels];    // LIT2 normal-map chain (RGBA16F)
    int albedoLevels, normalLevels;
    const float* shadow;            // LIT2 shadow map (FP32, CLAMP)
    int shadowSize, shadowScan;     // size and scanline in floats
    // scene viewer lighting (test2/testproc.h:4-30): light direction (21),
    // ambient (30), diffuse (31), specular colour (32), specular exponent (33)
    float ldir[4], amb[4], dif[4], scol[4];
    unsigned sexp;
};

struct DrawDesc {
    int triBase, triCount;
    int vp, fp;
    int nv;      // varying floats per vertex carried by this draw's interpolation stage
    int flags;   // behaviour bits | F_COLOUR
    int uni;     // index into the batch's DrawUniforms
    int vpX, vpY, vpW, vpH;  // viewport: rasteriser size vpW x vpH, its pixel (0,0) at target pixel (vpX, vpY)
    const uint8_t* vbo[kVboSlots];
    int stride[kVboSlots];
};

// Triangle after set-up (64 bytes).  vx/vy are the rasteriser's pixel-space
// vertices (rasterizer.h:7-28), rw = 1/w, pz = NDC z per vertex.
struct TriRaster {
    float vx[3], vy[3], rw[3], pz[3];
    short firstRow, lastRow;  // after clamping; firstRow > lastRow: nothing to draw
    int split;                // rows <= split use the lower edge pair
    int edges;                // 4 edges x (i0,i1) x 2 bits | flags << 16
    int draw;
};
static_assert(sizeof(TriRaster) == 64, "TriRaster must be 64 bytes");

// A span item: one row span of a short triangle, the part of it that lies in
// one bin, set up by k_setup_emit so that the raster reads it instead of
// deriving it (32 bytes).  cf2 / pz are the interpolation state at pixel xs
// -- the reference's span set-up (interp.cpp:26-80) followed by the
// sequential per-pixel steps from leftClamped (interp.cpp:82-92) -- and the
// steps continue it.  In the sorted bin lists a span item appears as ~index
// (negative); a triangle (non-negative index) is set up by the raster.
struct SpanItem {
    float cf2, pz, cf2Step, pzStep;
    int tri;          // the triangle (the winner id a covered pixel records)
    short xs, xe;     // target columns, inclusive, inside one bin
    int y;            // target row
    int flags;        // the draw's flags (behaviour bits | F_COLOUR | F_FRAGMENT)
};
static_assert(sizeof(SpanItem) == 32, "SpanItem must be 32 bytes");

// Kernel parameters of one device pass (a run of draws into one target).
struct PassParams {
    int W, H;                 // target (depth buffer) size; each draw has its own viewport rectangle
    int binW, binsX, binsY;   // bins of kBinH x binW pixels
    int rasterBlocks;         // raster variant: 0 = registers as needed, 8 = capped for 8 blocks per SM
    int cullSpans;            // raster variant: 1 = occluded spans dropped in crowded bins
    int rowSplit;             // raster blocks per bin (1, 2, 4 or 8): crowded bins shared out by rows
    int warpBins;             // raster shape: 1 = one warp per bin (k_raster_warp, 8- or 16-column bins)
    int spanItems;            // 1 = short triangles are binned as set-up span items (no forward passes)
    SpanItem* spans;          // span items, by emission index (capacity pairCap)
    int passFp;               // the fragment processor every colour draw of the pass uses, else 0
    int passVp;               // the vertex processor every colour draw of the pass uses, else 0
    int forward;              // some draw blends or may discard: shade every passing fragment in order
    int nTris, nDraws;
    const DrawDesc* draws;
    const DrawUniforms* unis;
    TriRaster* tris;
    float* vary;              // [tri][3][nvMax]
    int nvMax;
    int anyVary;              // some draw of the pass carries varyings
    int lazyVary;             // 1 = the set-up writes no varyings: the shade computes its winners' vertices'
                              // (passes shaded after the raster only)
    int* pairKey;             // bin of each (tri, bin) pair, in triangle order
    int* pairTri;
    int pairCap;              // capacity of pairKey / pairTri / keyB / binTri
    int sortBlocks;           // sort tiles that fit pairCap: ceil(pairCap / kSortChunk)
    int radixPasses;          // 8-bit digit passes the bin numbers need (0 for one bin)
    int* radix;               // [pass][256] digit counts, tickets; at kRadixHdr the set-up blocks'
                              // look-back descriptors (u64), at sortDescOff the radix passes'
                              // [pass][tile][256]; zeroed before each pass
    int sortDescOff;
    int* keyB;                // the sort's second key buffer
    int* binStart;            // per bin (start, end) of its list in the sorted pairs (int2; empty: start >= end)
    int* binItems;            // the raster's work list (kItemsPerBin x nBins ints)
    int* binTri;              // the sort's second triangle buffer
    const int* sortedTri;     // triangles of each bin, in submission order (binTri or pairTri)
    int* status;              // the pipeline's: [0] bit 1 = a pass overflowed, bit 2 = a wait
                              // expired; [1] most pairs a pass needed; [3] first pass that failed
                              // (kNoPass when none); [4..5] fragments tested, [6..7] passed,
                              // [8..9] pairs binned, [10..11] pixels shaded (u64)
    int* slotStatus;          // this pass's scratch slot: [0] sort tiles in use, [1] shade-list length
    float* depth;             // depth target (rows bottom-up)
    int depthScan;            // in floats
    int depthW, depthH;
    int2* shadeList;          // per covered pixel: (y << 16 | x, last colour-writing fragment that passed)
    uint32_t* colourRow0;     // the colour target (FBO slot 0), BGRA8: pixel (x, y) at colourRow0[y * colourPitch + x]
    int colourPitch;          // in pixels; negative for the display, whose rows run top-down
    int colourW, colourH;
    int clearDepth, clearColour, anyColour, countFrags;
    float depthClearValue;
    uint32_t colourClearValue;
    int passSeq;              // recorded in status[3] when this pass overflows
};

constexpr int kSortChunk = 2048;   // pairs per sort tile
constexpr int kFirstFailed = 3;    // status word: the first pass that overflowed or timed out
constexpr int kNoPass = 0x7f7f7f7f; // its value when none did (a byte-wise memset)
constexpr int kSlotTiles = 0, kSlotShade = 1, kSlotTotal = 2;  // slot status words: sort tiles, shade list, pairs
// The raster's work list (k_bin_bounds -> k_raster): items in five buckets,
// bins cut into 8, 4, 2 row slices, whole bins with triangles, empty bins;
// bucket b's count in slot status word kSlotBucket + b, the raster's cursor
// in kSlotCursor.  An item is bin | slice << 24 | log2(slices) << 28.
constexpr int kItemBuckets = 5;
constexpr int kSlotBucket = 3, kSlotCursor = kSlotBucket + kItemBuckets;
constexpr int kItemSliceShift = 24, kItemLog2Shift = 28, kItemBinMask = (1 << kItemSliceShift) - 1;
constexpr int kSliceTris = 128;  // a bin gets the most slices (up to rowSplit) that leave this many triangles each
// First item of bucket b in a list for nBins bins (capacities 8, 4, 2, 1, 1 x nBins).
__host__ __device__ constexpr long long bucket_base(int b, int nBins)
{
    return b == 0 ? 0 : b == 1 ? 8LL * nBins : b == 2 ? 12LL * nBins : b == 3 ? 14LL * nBins : 15LL * nBins;
}
constexpr int kItemsPerBin = 16;

// Whether a pass's raster takes its bins from the work list (row slices, or
// one warp per bin) rather than one block per bin.
__host__ __device__ inline bool raster_uses_items(const PassParams& P)
{
    return P.rowSplit > 1 || (P.warpBins && !P.forward && P.binW <= 16);
}

// A pass's kernels do nothing once this pass or an earlier one has failed;
// the host then re-runs the commands from the first failed pass.  Passes run
// on two streams, so the word is read volatile: it can change while they run.
#ifdef __CUDACC__
__device__ __forceinline__ bool pass_failed(const int* status, int seq)
{
    return *(volatile const int*)(status + kFirstFailed) <= seq;
}
#endif
constexpr int kRadixDigits = 256;
constexpr int kRadixMaxPasses = 3;  // bin numbers below 2^24
constexpr int kRadixHdr = 1024;     // ints before the descriptors (counts + tickets, padded)
constexpr int kTicketSetup = kRadixMaxPasses * kRadixDigits + kRadixMaxPasses;  // after the sort's tickets

// Kernel families timed by the profiler (ps3d_profile_*).
enum KernelId { K_SETUP, K_SCAN, K_EMIT, K_BOUNDS, K_SORT, K_RASTER, K_SHADE, K_FILL, K_POST, K_COUNT };

// CUDA-event brackets around kernel launches, on the launching stream.
struct Prof {
    bool on = false;
    struct Mark {
        int id;
        cudaEvent_t a, b;
    };
    std::vector<Mark> marks;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t take()
    {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    void begin(int id, cudaStream_t s)
    {
        if (!on) return;
        Mark m{id, take(), take()};
        cudaEventRecord(m.a, s);
        marks.push_back(m);
    }
    void end(cudaStream_t s)
    {
        if (on && !marks.empty()) cudaEventRecord(marks.back().b, s);
    }
};

}  // namespace ps3d
