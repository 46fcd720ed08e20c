// Device code of the tile interpolation (the hierarchical midpoint fill of one tile in shared memory and
// its finest level written to HBM), kept apart from the kernels (interp.cu) so that another kernel can run
// tiles too.  See interp.cu for the algorithm and its reference.
#pragma once

#include "s3r_internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

namespace s3r {
namespace {

constexpr float kHalf = 0.5f;
constexpr float kQuarter = 0.25f;
constexpr float kSixth = (float)(1.0 / 6.0);

__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

// put(): v may be +inf (internal no-field) or NaN; put_nan(): v is already NaN
// wherever it is masked (see inf_to_nan), so the float store needs no test.
template <typename OutT> struct Store;
template <> struct Store<float> {
    __device__ static void put(float* out, uint64_t i, float v, float, float)
    {
        out[i] = isinf(v) ? qnan() : v;
    }
    __device__ static void put_nan(float* out, uint64_t i, float v, float, float) { out[i] = v; }
};
template <> struct Store<__half> {
    __device__ static void put(__half* out, uint64_t i, float v, float inv_scale, float offset)
    {
        out[i] = (isinf(v) || isnan(v)) ? __ushort_as_half((unsigned short)0x7e00)
                                             : __float2half_rn((v - offset) * inv_scale);
    }
    __device__ static void put_nan(__half* out, uint64_t i, float v, float inv_scale, float offset)
    {
        out[i] = isnan(v) ? __ushort_as_half((unsigned short)0x7e00) : __float2half_rn((v - offset) * inv_scale);
    }
};
template <> struct Store<__nv_bfloat16> {
    __device__ static void put(__nv_bfloat16* out, uint64_t i, float v, float inv_scale, float offset)
    {
        out[i] = (isinf(v) || isnan(v)) ? __ushort_as_bfloat16((unsigned short)0x7fc0)
                                             : __float2bfloat16_rn((v - offset) * inv_scale);
    }
    __device__ static void put_nan(__nv_bfloat16* out, uint64_t i, float v, float inv_scale, float offset)
    {
        out[i] = isnan(v) ? __ushort_as_bfloat16((unsigned short)0x7fc0)
                          : __float2bfloat16_rn((v - offset) * inv_scale);
    }
};

// Two vertices adjacent along x, already NaN where masked, in one aligned store
// (the pair starts at an even x of a row whose pitch keeps it aligned).
template <typename OutT> struct Store2;
template <> struct Store2<float> {
    __device__ static void put_nan(float* out, float v0, float v1, float, float)
    {
        *reinterpret_cast<float2*>(out) = make_float2(v0, v1);
    }
};
// 16-bit pairs: (v - offset) / scale as one FMA per value and one paired conversion;
// a NaN stays NaN through both.
template <> struct Store2<__half> {
    __device__ static void put_nan(__half* out, float v0, float v1, float inv_scale, float offset)
    {
        const float c = -offset * inv_scale;
        *reinterpret_cast<__half2*>(out) = __floats2half2_rn(__fmaf_rn(v0, inv_scale, c), __fmaf_rn(v1, inv_scale, c));
    }
};
template <> struct Store2<__nv_bfloat16> {
    __device__ static void put_nan(__nv_bfloat16* out, float v0, float v1, float inv_scale, float offset)
    {
        const float c = -offset * inv_scale;
        *reinterpret_cast<__nv_bfloat162*>(out) =
            __floats2bfloat162_rn(__fmaf_rn(v0, inv_scale, c), __fmaf_rn(v1, inv_scale, c));
    }
};

// +inf -> NaN in one FFMA, every other value (-0 included) unchanged:
// 0 * v is +-0 for finite v (the sign of v, so v + 0 * v == v exactly) and NaN
// for infinite v.
__device__ __forceinline__ float inf_to_nan(float v) { return __fmaf_rn(0.f, v, v); }

// Internally a masked value is +inf: every stencil sum that touches it is
// +inf, which reproduces the reference's rule "any no-field value in the
// stencil gives the no-field value" without tests, and finite sums round as
// before.  NaN keeps its meaning "not computed yet".
__device__ __forceinline__ float to_internal(float v) { return v == kNoField ? __int_as_float(0x7f800000) : v; }

// Descent slots: 27 points (3x3x3, x fastest) per coarse level.
constexpr int kMaxDescentLevels = S3R_MAX_DEPTH;

// The threads that run one tile: a CTA of kInterpThreads (kN = kInterpThreads, CTA barriers) or one warp
// (kN = 32, warp barriers; the warp-per-tile kernel for tiles of up to 8 cells).  tid is the thread's
// index among them.
template <uint32_t kN> struct Crew {
    uint32_t tid;
    __device__ __forceinline__ void sync() const
    {
        if constexpr (kN == 32) __syncwarp();
        else __syncthreads();
    }
};

// One 27-point level held in registers: lane p < 27 holds point p (x fastest)
// of a cube -- the 8 corners known, each midpoint its sparse value or NaN --
// and gets it filled: edges from their two ends, faces from their four edges,
// the centre from its six faces, the stencil sums in the reference's order.
// Neighbours come by shuffle, so no shared memory and no __syncwarp.
__device__ __forceinline__ float level27(float v, uint32_t lane)
{
    const uint32_t px = lane % 3, py = (lane / 3) % 3, pz = lane / 9;
    const uint32_t nodd = lane < 27 ? (px & 1) + (py & 1) + (pz & 1) : 3u;
    {
        const bool mine = nodd == 1;
        const uint32_t st = (px & 1) ? 1 : ((py & 1) ? 3 : 9);
        const float lo = __shfl_sync(0xffffffffu, v, mine ? lane - st : lane);
        const float hi = __shfl_sync(0xffffffffu, v, mine ? lane + st : lane);
        if (mine && isnan(v)) v = kHalf * (lo + hi);
    }
    {
        const bool mine = nodd == 2;
        const uint32_t s1 = (px & 1) ? 1 : 3; // the two odd axes, ascending
        const uint32_t s2 = (pz & 1) ? 9 : 3;
        const float a = __shfl_sync(0xffffffffu, v, mine ? lane - s1 : lane);
        const float b = __shfl_sync(0xffffffffu, v, mine ? lane + s1 : lane);
        const float c = __shfl_sync(0xffffffffu, v, mine ? lane - s2 : lane);
        const float d = __shfl_sync(0xffffffffu, v, mine ? lane + s2 : lane);
        if (mine && isnan(v)) v = kQuarter * (a + b + c + d);
    }
    {
        const float f12 = __shfl_sync(0xffffffffu, v, 12), f14 = __shfl_sync(0xffffffffu, v, 14);
        const float f10 = __shfl_sync(0xffffffffu, v, 10), f16 = __shfl_sync(0xffffffffu, v, 16);
        const float f4 = __shfl_sync(0xffffffffu, v, 4), f22 = __shfl_sync(0xffffffffu, v, 22);
        if (lane == 13 && isnan(v)) v = kSixth * (f12 + f14 + f10 + f16 + f4 + f22);
    }
    return v;
}

// One warp, all lanes: walk from the block's root corners down L levels to the
// tile's cube, each level's 27 points in registers (level27) with the sparse
// values found in desc[27*l + p] (NaN where no node; at levels below the root
// the corner points come from the level above).  Lanes 0-7 return the tile's 8
// corners (lane & 1, lane >> 1 & 1, lane >> 2).
__device__ __forceinline__ float descend_regs(const float* desc, uint32_t d, uint32_t L, uint32_t ox, uint32_t oy,
                                              uint32_t oz, uint32_t lane)
{
    const uint32_t px = lane % 3, py = (lane / 3) % 3, pz = lane / 9;
    const bool is_corner = lane < 27 && !((px | py | pz) & 1);
    const uint32_t from = is_corner ? (px >> 1) + 2 * (py >> 1) + 4 * (pz >> 1) : lane;
    uint32_t size = 1u << d, gx0 = 0, gy0 = 0, gz0 = 0;
    float corner = 0.f;
    for (uint32_t l = 0; l < L; ++l) {
        float v = lane < 27 ? desc[27 * l + lane] : 0.f;
        if (l > 0) {
            const float cv = __shfl_sync(0xffffffffu, corner, from);
            if (is_corner) v = cv;
        }
        v = level27(v, lane);
        const uint32_t hs = size >> 1;
        const uint32_t qx = (ox - gx0) >= hs ? 1u : 0u;
        const uint32_t qy = (oy - gy0) >= hs ? 1u : 0u;
        const uint32_t qz = (oz - gz0) >= hs ? 1u : 0u;
        const uint32_t pick =
            lane < 8 ? (qx + (lane & 1)) + 3 * (qy + ((lane >> 1) & 1)) + 9 * (qz + (lane >> 2)) : lane;
        corner = __shfl_sync(0xffffffffu, v, pick);
        gx0 += qx * hs;
        gy0 += qy * hs;
        gz0 += qz * hs;
        size = hs;
    }
    return corner;
}

// One level of one tile: every cube of the level (2^j per axis) is handled by
// one thread, which reads its 27 points (8 corners known from the coarser
// levels, 19 midpoints holding a sparse value or NaN), fills the NaN midpoints
// in registers (edges, then faces, then the centre) and writes back the
// midpoints it owns: those with every coordinate on the cube's low side or
// middle, plus the far side where the cube is the last along that axis.
// Midpoints shared with a neighbour are computed by both from the same values,
// so a neighbour reading one while it is written reads the same number.
__device__ __forceinline__ void cube_level(float* s, uint32_t E, uint32_t T, uint32_t j)
{
    const uint32_t m = 1u << j, sz = T >> j, hs = sz >> 1;
    const uint32_t st0 = hs, st1 = E * hs, st2 = E * E * hs;
    const uint32_t ncubes = 1u << (3 * j);
#pragma unroll 1
    for (uint32_t c = threadIdx.x; c < ncubes; c += kInterpThreads) {
        const uint32_t ci = c & (m - 1), cj = (c >> j) & (m - 1), ck = c >> (2 * j);
        const uint32_t base = ci * sz + E * (cj * sz + E * (ck * sz));
        float v[27];
#pragma unroll
        for (int p = 0; p < 27; ++p) v[p] = s[base + (p % 3) * st0 + ((p / 3) % 3) * st1 + (p / 9) * st2];
#pragma unroll
        for (int p = 0; p < 27; ++p) {
            const int a = p % 3, b = (p / 3) % 3, cc = p / 9;
            if ((a & 1) + (b & 1) + (cc & 1) == 1 && isnan(v[p])) {
                const int st = (a & 1) ? 1 : ((b & 1) ? 3 : 9);
                v[p] = kHalf * (v[p - st] + v[p + st]);
            }
        }
#pragma unroll
        for (int p = 0; p < 27; ++p) {
            const int a = p % 3, b = (p / 3) % 3, cc = p / 9;
            if ((a & 1) + (b & 1) + (cc & 1) == 2 && isnan(v[p])) {
                const int s1 = (a & 1) ? 1 : 3;
                const int s2 = (cc & 1) ? 9 : 3;
                v[p] = kQuarter * (v[p - s1] + v[p + s1] + v[p - s2] + v[p + s2]);
            }
        }
        if (isnan(v[13])) v[13] = kSixth * (v[12] + v[14] + v[10] + v[16] + v[4] + v[22]);
        const bool lx = ci == m - 1, ly = cj == m - 1, lz = ck == m - 1;
#pragma unroll
        for (int p = 0; p < 27; ++p) {
            const int a = p % 3, b = (p / 3) % 3, cc = p / 9;
            if ((a & 1) + (b & 1) + (cc & 1) == 0) continue;
            if ((a < 2 || lx) && (b < 2 || ly) && (cc < 2 || lz))
                s[base + a * st0 + b * st1 + cc * st2] = v[p];
        }
    }
}

// Shared tile of (2^k+1)^3 floats, rounded up to whole float4s for the vector fill.
inline size_t tile_smem_bytes(uint32_t tile_log2)
{
    const size_t E = (1u << tile_log2) + 1u;
    return ((E * E * E + 3) / 4) * 16;
}

// Parity-split layout of a tile of T cells (T even): vertex (x, y, z) lives in
// sub-array c = (x&1) | (y&1)<<1 | (z&1)<<2 at (x>>1) + nx*((y>>1) + ny*(z>>1)),
// with nx = T/2 along an odd axis and T/2+1 along an even one.  At the finest
// level every class of midpoints then sits in its own dense array, so a warp
// walking one class touches consecutive words (no bank conflicts), and the
// even sub-array is the same problem at half resolution for the coarser levels.
template <uint32_t T> struct SplitTile {
    static constexpr uint32_t H = T / 2, G = T / 2 + 1;
    __host__ __device__ static constexpr uint32_t n(uint32_t odd) { return odd ? H : G; }
    __host__ __device__ static constexpr uint32_t size(uint32_t c) { return n(c & 1) * n((c >> 1) & 1) * n((c >> 2) & 1); }
    // sum of the sizes of classes 0 .. c-1 (sizes G^3, HG^2, HG^2, H^2G, HG^2, H^2G, H^2G, H^3)
    __host__ __device__ static constexpr uint32_t base(uint32_t c)
    {
        constexpr uint32_t G3 = G * G * G, HG2 = H * G * G, H2G = H * H * G;
        return (c >= 1 ? G3 : 0) + (c >= 2 ? HG2 : 0) + (c >= 3 ? HG2 : 0) + (c >= 4 ? H2G : 0) +
               (c >= 5 ? HG2 : 0) + (c >= 6 ? H2G : 0) + (c >= 7 ? H2G : 0);
    }
    // element (i, j, k) of class c
    __host__ __device__ static constexpr uint32_t idx(uint32_t c, uint32_t i, uint32_t j, uint32_t k)
    {
        return base(c) + i + n(c & 1) * (j + n((c >> 1) & 1) * k);
    }
    __host__ __device__ static constexpr uint32_t at(uint32_t x, uint32_t y, uint32_t z)
    {
        return idx((x & 1) | ((y & 1) << 1) | ((z & 1) << 2), x >> 1, y >> 1, z >> 1);
    }
};

// The first warp of the tile's threads, T >= 4: the tile cube's 27 points (corners at 0 and T, midpoints at
// T/2) from its corners and the sparse values already in the tile -- the
// tile's first level, cube_level on its single cube, in registers.
template <uint32_t T> __device__ __forceinline__ void tile_top(float* s, uint32_t lane)
{
    using S = SplitTile<T>;
    const uint32_t px = lane % 3, py = (lane / 3) % 3, pz = lane / 9;
    constexpr uint32_t h = T / 2;
    const uint32_t off = lane < 27 ? S::at(px * h, py * h, pz * h) : 0;
    float v = lane < 27 ? s[off] : 0.f;
    v = level27(v, lane);
    if (lane < 27 && ((px | py | pz) & 1)) s[off] = v;
}

// Marks the finest-level cubes holding a sparse value at one of their
// midpoints (tile position (x, y, z), at least one coordinate odd): the cube
// along each odd axis, both neighbours along each even one.
__device__ __forceinline__ void flag_cubes(uint32_t* flags, uint32_t H, uint32_t x, uint32_t y, uint32_t z)
{
    if (!((x | y | z) & 1)) return;
    const uint32_t x0 = (x & 1) ? x >> 1 : (x ? (x >> 1) - 1 : 0), x1 = (x & 1) ? x >> 1 : min(x >> 1, H - 1);
    const uint32_t y0 = (y & 1) ? y >> 1 : (y ? (y >> 1) - 1 : 0), y1 = (y & 1) ? y >> 1 : min(y >> 1, H - 1);
    const uint32_t z0 = (z & 1) ? z >> 1 : (z ? (z >> 1) - 1 : 0), z1 = (z & 1) ? z >> 1 : min(z >> 1, H - 1);
    for (uint32_t k = z0; k <= z1; ++k)
        for (uint32_t j = y0; j <= y1; ++j)
            for (uint32_t i = x0; i <= x1; ++i) {
                const uint32_t c = i + H * (j + H * k);
                atomicOr(&flags[c >> 5], 1u << (c & 31));
            }
}

// The 19 midpoints of one 2x2x2 cube from its 8 corners (v[p], p = a + 3b + 9c,
// a, b, c in {0, 1, 2}); kSlots: v also holds sparse values (or NaN) at the
// midpoints, which are kept.  Edges, then faces, then the centre, stencil sums
// in the reference's order.  kLowZDone: the cube's z = 0 face is final already
// (the z = 2 face of the cube below it), only the points above it are filled.
template <bool kSlots, bool kLowZDone = false> __device__ __forceinline__ void fill_cube(float v[27])
{
#pragma unroll
    for (int p = 0; p < 27; ++p) {
        const int a = p % 3, b = (p / 3) % 3, cc = p / 9;
        if (kLowZDone && cc == 0) continue;
        if ((a & 1) + (b & 1) + (cc & 1) == 1 && (!kSlots || isnan(v[p]))) {
            const int st = (a & 1) ? 1 : ((b & 1) ? 3 : 9);
            v[p] = kHalf * (v[p - st] + v[p + st]);
        }
    }
#pragma unroll
    for (int p = 0; p < 27; ++p) {
        const int a = p % 3, b = (p / 3) % 3, cc = p / 9;
        if (kLowZDone && cc == 0) continue;
        if ((a & 1) + (b & 1) + (cc & 1) == 2 && (!kSlots || isnan(v[p]))) {
            const int s1 = (a & 1) ? 1 : 3;
            const int s2 = (cc & 1) ? 9 : 3;
            v[p] = kQuarter * (v[p - s1] + v[p + s1] + v[p - s2] + v[p + s2]);
        }
    }
    if (!kSlots || isnan(v[13])) v[13] = kSixth * (v[12] + v[14] + v[10] + v[16] + v[4] + v[22]);
}

// cube_level with the grid stride, tile size and level known at compile time (the coarse levels
// inside a tile): the 27 point offsets become immediates and the cube loop is unrolled.
template <uint32_t E, uint32_t T, uint32_t J, uint32_t kN>
__device__ __forceinline__ void cube_level_ct(float* s, uint32_t tid)
{
    constexpr uint32_t m = 1u << J, sz = T >> J, hs = sz >> 1;
    constexpr uint32_t st0 = hs, st1 = E * hs, st2 = E * E * hs;
    constexpr uint32_t ncubes = 1u << (3 * J);
#pragma unroll
    for (uint32_t c0 = 0; c0 < ncubes; c0 += kN) {
        const uint32_t c = c0 + tid;
        if (ncubes % kN != 0 && c >= ncubes) break;
        const uint32_t ci = c & (m - 1), cj = (c >> J) & (m - 1), ck = c >> (2 * J);
        const uint32_t base = ci * sz + E * (cj * sz + E * (ck * sz));
        float v[27];
#pragma unroll
        for (int p = 0; p < 27; ++p) v[p] = s[base + (p % 3) * st0 + ((p / 3) % 3) * st1 + (p / 9) * st2];
        fill_cube<true>(v);
        const bool lx = ci == m - 1, ly = cj == m - 1, lz = ck == m - 1;
#pragma unroll
        for (int p = 0; p < 27; ++p) {
            const int a = p % 3, b = (p / 3) % 3, cc = p / 9;
            if ((a & 1) + (b & 1) + (cc & 1) == 0) continue;
            if ((a < 2 || lx) && (b < 2 || ly) && (cc < 2 || lz)) s[base + a * st0 + b * st1 + cc * st2] = v[p];
        }
    }
}

// The coarse levels 1 .. K-2 of a tile of T = 2^K cells on its even sub-array (G^3, a tile of T/2 cells).
template <uint32_t G, uint32_t H, uint32_t J, uint32_t K, uint32_t kN>
__device__ __forceinline__ void tile_levels(float* s, Crew<kN> cw)
{
    if constexpr (J + 1 < K) {
        cube_level_ct<G, H, J, kN>(s, cw.tid);
        cw.sync();
        tile_levels<G, H, J + 1, K, kN>(s, cw);
    }
}

// One finest-level cube (ci, cj, ck) of a tile: reads its corners from the even
// sub-array -- kFirst: all 8; else the upper 4, its z = 0 face being the z = 2
// face of the cube below it, already in v -- and, when flagged as holding a
// sparse midpoint, its midpoint slots (above the z = 0 face unless kFirst);
// computes its midpoints in registers and stores the vertices it owns: its low
// octant, plus the far side where it is the last cube of the block along an
// axis, with the 16-bit encoding fused into the store.  Masked corners become
// NaN as they are loaded, so unflagged cubes produce NaN directly (a NaN in a
// stencil sum gives NaN as +inf gives +inf); flagged cubes test their slots for
// NaN ("no sparse value") before any slot is overwritten, then turn masked
// sparse values to NaN.  A reused face went through the same steps in the cube
// below, so every vertex gets the value a fresh cube would give it.
// kPairs: plan bricks, whose rows are padded to whole sectors (aligned rows, even pitch): a row's two
// vertices of a cube go out as one store.  A plain (2^d+1)^3 grid (odd pitch) stores them one by one.
template <uint32_t T, typename OutT, bool kPairs, bool kFirst>
__device__ __forceinline__ void finest_cube(const float* s, bool has, uint32_t ci, uint32_t cj, uint32_t ck, float v[27],
                                            OutT* base, uint32_t pitch, uint32_t e, uint32_t e2, bool lx, bool ly,
                                            bool lz, float inv_scale, float offset)
{
    using S = SplitTile<T>;
#pragma unroll
    for (int p = 0; p < 27; ++p) {
        const uint32_t a = p % 3, b = (p / 3) % 3, cc = p / 9;
        if (!kFirst && cc < 2) continue;
        if (!((a | b | cc) & 1)) v[p] = inf_to_nan(s[S::idx(0, ci + (a >> 1), cj + (b >> 1), ck + (cc >> 1))]);
    }
    if (has) {
#pragma unroll
        for (int p = 0; p < 27; ++p) {
            const uint32_t a = p % 3, b = (p / 3) % 3, cc = p / 9;
            if (!kFirst && cc == 0) continue;
            const uint32_t cls = (a & 1) | ((b & 1) << 1) | ((cc & 1) << 2);
            if (cls) v[p] = s[S::idx(cls, ci + (a >> 1), cj + (b >> 1), ck + (cc >> 1))];
        }
        fill_cube<true, !kFirst>(v);
#pragma unroll
        for (int p = 0; p < 27; ++p) {
            if (!kFirst && p / 9 == 0) continue;
            if ((p % 3) & 1 || ((p / 3) % 3) & 1 || (p / 9) & 1) v[p] = inf_to_nan(v[p]);
        }
    } else {
        fill_cube<false, !kFirst>(v);
    }
    if constexpr (kPairs) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t b = r & 1, cc = r >> 1;
            Store2<OutT>::put_nan(base + b * pitch + cc * e2, v[3 * b + 9 * cc], v[1 + 3 * b + 9 * cc], inv_scale,
                                  offset);
        }
    } else {
#pragma unroll
        for (int p = 0; p < 27; ++p) {
            const uint32_t a = p % 3, b = (p / 3) % 3, cc = p / 9;
            if (a < 2 && b < 2 && cc < 2) Store<OutT>::put_nan(base, a + b * pitch + cc * e2, v[p], inv_scale, offset);
        }
    }
    // the far side where this is the block's last cube along an axis: the x = 2 face (with its
    // y = 2 / z = 2 edges where those are far too), then y = 2 (x < 2), then z = 2 (x, y < 2)
    auto far_put = [&](int p) {
        const uint32_t a = p % 3, b = (p / 3) % 3, cc = p / 9;
        if constexpr (std::is_same<OutT, float>::value && T >= 8) {
            if (a == 2 && pitch >= e + 7) {
                // a padded brick (plan layout, d >= 3): x = 2^d starts a sector of its own
                // (rows are 32-byte aligned, 2^d is a multiple of 8, the pitch is 2^d + 8):
                // write the whole sector, the padding as NaN
                float4* q = reinterpret_cast<float4*>(base + a + b * pitch + cc * e2);
                q[0] = make_float4(v[p], qnan(), qnan(), qnan());
                q[1] = make_float4(qnan(), qnan(), qnan(), qnan());
                return;
            }
        }
        Store<OutT>::put_nan(base, a + b * pitch + cc * e2, v[p], inv_scale, offset);
    };
    if (lx) {
#pragma unroll
        for (int bb = 0; bb < 3; ++bb)
#pragma unroll
            for (int c2 = 0; c2 < 3; ++c2)
                if ((bb < 2 || ly) && (c2 < 2 || lz)) far_put(2 + 3 * bb + 9 * c2);
    }
    if (ly) {
#pragma unroll
        for (int c2 = 0; c2 < 3; ++c2) {
            if (c2 == 2 && !lz) continue;
            if constexpr (kPairs) {
                Store2<OutT>::put_nan(base + 2 * pitch + c2 * e2, v[6 + 9 * c2], v[7 + 9 * c2], inv_scale, offset);
            } else {
                far_put(6 + 9 * c2);
                far_put(7 + 9 * c2);
            }
        }
    }
    if (lz) {
#pragma unroll
        for (int b2 = 0; b2 < 2; ++b2) {
            if constexpr (kPairs) {
                Store2<OutT>::put_nan(base + b2 * pitch + 2 * e2, v[3 * b2 + 18], v[1 + 3 * b2 + 18], inv_scale,
                                      offset);
            } else {
                far_put(3 * b2 + 18);
                far_put(1 + 3 * b2 + 18);
            }
        }
    }
}

// The finest level of a tile, written straight to HBM: its H^3 2x2x2 cubes in
// runs of Z along z, one run per thread (runs consecutive along x within a
// warp), so that each cube after the first of a run takes its z = 0 face from
// the one below; Z makes the runs about as many as the tile's threads (kN).
template <uint32_t T, typename OutT, bool kPairs, uint32_t kN>
__device__ __forceinline__ void finest_store(const float* s, const uint32_t* flags, OutT* out, uint32_t e,
                                             uint32_t pitch, uint32_t ox, uint32_t oy, uint32_t oz, bool far_x,
                                             bool far_y, bool far_z, float inv_scale, float offset, uint32_t tid)
{
    using S = SplitTile<T>;
    constexpr uint32_t H = S::H;
    constexpr uint32_t lh = (H >= 2) ? (31 - __builtin_clz(H)) : 0;
    constexpr uint32_t per = H * H * H / kN;
    constexpr uint32_t Z = per >= H ? H : (per >= 1 ? per : 1);
    constexpr uint32_t lzr = 31 - __builtin_clz(Z);
    constexpr uint32_t nruns = H * H * H / Z;
    const uint32_t e2 = e * pitch; // slab stride (a brick holds fewer than 2^32 elements)
#pragma unroll 1
    for (uint32_t rr = tid; rr < nruns; rr += kN) {
        const uint32_t ci = rr & (H - 1), cj = (rr >> lh) & (H - 1), ck0 = (rr >> (2 * lh)) << lzr;
        const bool lx = far_x && ci == H - 1, ly = far_y && cj == H - 1;
        float v[27];
        OutT* base = out + (((oz + 2 * ck0) * e + (oy + 2 * cj)) * pitch + (ox + 2 * ci));
        {
            const uint32_t c = ci + H * (cj + H * ck0);
            const bool has = (flags[c >> 5] >> (c & 31)) & 1u;
            finest_cube<T, OutT, kPairs, true>(s, has, ci, cj, ck0, v, base, pitch, e, e2, lx, ly,
                                               far_z && ck0 == H - 1, inv_scale, offset);
        }
#pragma unroll 1
        for (uint32_t z = 1; z < Z; ++z) {
            const uint32_t ck = ck0 + z;
            const uint32_t c = ci + H * (cj + H * ck);
            const bool has = (flags[c >> 5] >> (c & 31)) & 1u;
#pragma unroll
            for (int p = 0; p < 9; ++p) v[p] = v[p + 18];
            base += 2 * e2;
            finest_cube<T, OutT, kPairs, false>(s, has, ci, cj, ck, v, base, pitch, e, e2, lx, ly,
                                                far_z && ck == H - 1, inv_scale, offset);
        }
    }
}

// Entries of the next work item, loaded into registers in three stages, each
// issued one phase of the current tile ahead of its use, so that the chain of
// dependent global loads -- item and block, then entry positions and node
// indices, then node values -- completes behind the current tile's work
// instead of stalling the tile's threads at every tile.
constexpr uint32_t kPrefetch = 2; // entries per thread held in registers
struct Prefetch {
    uint32_t item;
    uint32_t flag; // word tid of the item's cube flags
    uint32_t cidx; // threads 0-7: the coarse-grid index of tile corner tid (0xffffffff: none)
    float corner;
    uint32_t node_base, e0, e1; // a plan holds fewer than 2^32 nodes and entries
    uint32_t loc[kPrefetch];
    uint32_t node[kPrefetch];
    float val[kPrefetch];
};

// stage 1: the item's block, entry range, flag word and corner positions in the coarse grid
template <uint32_t kN>
__device__ __forceinline__ void prefetch_head(Prefetch& pf, const TileArgs& a, uint32_t item, uint32_t tid)
{
    pf.item = item;
    pf.e0 = pf.e1 = 0;
    pf.cidx = 0xffffffffu;
    if (item >= a.nitems) return;
    const uint2 it = a.items[item];
    const PlanBlock* B = &a.blocks[it.x];
    pf.node_base = (uint32_t)B->node_base;
    pf.e0 = (uint32_t)a.entry_off[item];
    pf.e1 = (uint32_t)a.entry_off[item + 1];
    if (tid < a.flag_words) pf.flag = a.flags[(uint64_t)item * a.flag_words + tid];
    if (tid < 8) {
        const uint32_t L = B->coarse_log2;
        if (L > 0) {
            const uint32_t tile = it.y & 0x7fffffffu, mL = 1u << L, E = mL + 1;
            const uint32_t cx = (tile & (mL - 1)) + (tid & 1);
            const uint32_t cy = ((tile >> L) & (mL - 1)) + ((tid >> 1) & 1);
            const uint32_t cz = (tile >> (2 * L)) + (tid >> 2);
            pf.cidx = B->coarse_off + cx + E * (cy + E * cz);
        }
    }
}

// stage 2: positions and node indices of the first kPrefetch * kN entries, and the corners
template <uint32_t kN> __device__ __forceinline__ void prefetch_index(Prefetch& pf, const TileArgs& a, uint32_t tid)
{
    if (pf.cidx != 0xffffffffu) pf.corner = a.coarse[pf.cidx];
#pragma unroll
    for (uint32_t q = 0; q < kPrefetch; ++q) {
        const uint32_t i = pf.e0 + tid + q * kN;
        if (i < pf.e1) {
            pf.loc[q] = a.entry_local[i];
            pf.node[q] = a.entry_node[i];
        }
    }
}

// stage 3: their node values
template <uint32_t kN> __device__ __forceinline__ void prefetch_values(Prefetch& pf, const TileArgs& a, uint32_t tid)
{
#pragma unroll
    for (uint32_t q = 0; q < kPrefetch; ++q)
        if (pf.e0 + tid + q * kN < pf.e1) pf.val[q] = a.sparse[pf.node_base + pf.node[q]];
}

struct TileItem {
    uint32_t d, k, L, tx, ty, tz, blk, pitch;
    uint32_t slots; // the tile has flagged cubes, which read its midpoint slots
    uint64_t node_base, dense_off;
    uint32_t item;
};

// One tile of T = 2^k cells.  Tiles of T >= 2 use the split layout; T = 1
// (depth-0 blocks) is a plain 2x2x2 copy of the root corners.
// cw: the CTA or the warp running the tile; next_item(): the next work item's number (read once the current
// item's entries are placed, so that its first prefetch stage goes out behind this tile's work).
template <uint32_t T, bool kGrid, typename OutT, uint32_t kN, class NextFn>
__device__ __forceinline__ void run_tile(const TileArgs& a, float* s, float* desc, uint32_t* flags, const TileItem& t,
                                         Prefetch& pf, Crew<kN> cw, NextFn next_item)
{
    constexpr uint32_t E = T + 1, E3 = E * E * E;
    using S = SplitTile<T < 2 ? 2 : T>;
    auto at = [](uint32_t x, uint32_t y, uint32_t z) -> uint32_t {
        if constexpr (T < 2) return x + 2 * (y + 2 * z);
        else return S::at(x, y, z);
    };
    const uint32_t d = t.d, L = t.L;
    const uint32_t ox = t.tx * T, oy = t.ty * T, oz = t.tz * T;
    const uint32_t e = (1u << d) + 1u;
    constexpr uint32_t nflags = T >= 2 ? (S::H * S::H * S::H + 31) / 32 : 0;
    if constexpr (kGrid) {
        for (uint32_t q = cw.tid; q < nflags; q += kN) flags[q] = 0u;
    } else {
        if (cw.tid < nflags) flags[cw.tid] = pf.flag; // the plan's flags, prefetched
    }
    // 1. the tile's sparse values (NaN elsewhere) and the descent's
    if constexpr (kGrid) {
        cw.sync(); // flags cleared
#pragma unroll 1
        for (uint32_t p = cw.tid; p < E3; p += kN) {
            const uint32_t lx = p % E, r = p / E, ly = r % E, lz = r / E;
            const float v = to_internal(a.grid[((uint64_t)(oz + lz) * e + (oy + ly)) * e + (ox + lx)]);
            s[at(lx, ly, lz)] = v;
            if constexpr (T >= 2)
                if (!isnan(v)) flag_cubes(flags, S::H, lx, ly, lz);
        }
        for (uint32_t q = cw.tid; q < 27 * L; q += kN) {
            const uint32_t l = q / 27, p = q % 27;
            const uint32_t size = 1u << (d - l), hs = size >> 1;
            const uint32_t bx = ox & ~(size - 1), by = oy & ~(size - 1), bz = oz & ~(size - 1);
            const uint32_t gx = bx + hs * (p % 3), gy = by + hs * ((p / 3) % 3), gz = bz + hs * (p / 9);
            desc[q] = to_internal(a.grid[((uint64_t)gz * e + gy) * e + gx]);
        }
    } else {
        {
            const float4 nan4 = make_float4(qnan(), qnan(), qnan(), qnan());
            float4* s4 = reinterpret_cast<float4*>(s);
            // the even sub-array always (the coarse levels test it for NaN); the midpoint slots only
            // where a flagged cube will read them
            uint32_t n4 = (E3 + 3) / 4;
            if constexpr (T >= 2) {
                constexpr uint32_t G3 = S::G * S::G * S::G;
                if (!t.slots) n4 = (G3 + 3) / 4;
            }
#pragma unroll 1
            for (uint32_t p = cw.tid; p < n4; p += kN) s4[p] = nan4;
        }
        cw.sync();
        auto place = [&](uint32_t loc, float v) {
            if (loc < E3) s[loc] = v;
        };
        // the prefetched entries, then any beyond what the registers held
#pragma unroll
        for (uint32_t q = 0; q < kPrefetch; ++q)
            if (pf.e0 + cw.tid + q * kN < pf.e1) place(pf.loc[q], to_internal(pf.val[q]));
        for (uint32_t i = pf.e0 + cw.tid + kPrefetch * kN; i < pf.e1; i += kN)
            place(a.entry_local[i], to_internal(a.sparse[t.node_base + a.entry_node[i]]));
        // a tile of a block with coarse levels: its corners from the block's coarse grid
        if (pf.cidx != 0xffffffffu)
            s[at((cw.tid & 1) * T, ((cw.tid >> 1) & 1) * T, (cw.tid >> 2) * T)] = pf.corner;
        prefetch_head<kN>(pf, a, next_item(), cw.tid); // the current item's entries are placed
    }
    cw.sync();
    // 2. single-grid form: tile corners from the coarse levels; then the tile cube's own
    //    midpoints (its first level): the first warp, each level's 27 points in registers
    if ((kGrid && L > 0) || T >= 4) {
        if (kN == 32 || cw.tid < 32) {
            const uint32_t lane = cw.tid & 31;
            if (kGrid && L > 0) {
                const float corner = descend_regs(desc, d, L, ox, oy, oz, lane);
                if (lane < 8) s[at((lane & 1) * T, ((lane >> 1) & 1) * T, (lane >> 2) * T)] = corner;
                __syncwarp();
            }
            if constexpr (T >= 4) tile_top<T>(s, lane);
        }
        cw.sync();
    }
    if constexpr (!kGrid) prefetch_index<kN>(pf, a, cw.tid);
    // 3. the remaining coarser levels on the even sub-array (a tile of T/2 cells)
    if constexpr (T >= 8) tile_levels<S::G, S::H, 1, 31 - __builtin_clz(T), kN>(s, cw);
    // 4. the finest level, straight to HBM, while the next item's entries load
    if constexpr (!kGrid) prefetch_values<kN>(pf, a, cw.tid);
    float inv_scale = 1.f, offset = 0.f;
    if constexpr (!kGrid) {
        if (a.scale_offset) {
            const float2 so = a.scale_offset[t.blk];
            inv_scale = 1.f / so.x;
            offset = so.y;
        }
    }
    const uint32_t mL = 1u << L;
    OutT* out = reinterpret_cast<OutT*>(a.out) + t.dense_off;
    const bool far_x = t.tx == mL - 1, far_y = t.ty == mL - 1, far_z = t.tz == mL - 1;
    if constexpr (T >= 2) {
        finest_store<T, OutT, !kGrid, kN>(s, flags, out, e, t.pitch, ox, oy, oz, far_x, far_y, far_z, inv_scale,
                                          offset, cw.tid);
    } else {
        // depth-0 block: its 8 root corners
        for (uint32_t q = cw.tid; q < 8; q += kN) {
            const uint32_t x = q & 1, y = (q >> 1) & 1, z = q >> 2;
            Store<OutT>::put(out, ((uint64_t)(oz + z) * e + (oy + y)) * t.pitch + ox + x, s[at(x, y, z)],
                             inv_scale, offset);
        }
    }
}

} // namespace
} // namespace s3r
