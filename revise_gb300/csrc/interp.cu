// Sparse-octree -> dense-grid interpolation for sm_103a.
//
// Restates the hierarchical midpoint fill of the reference
// (include/s3dmm/DenseFieldInterpolator.hpp:198-419; GPU form
// src/s3dmm_cuda/DenseFieldInterpolatorArr_cu_3.cu:69-188 and :197-257):
// level by level, every cube's edge midpoints take 1/2 of their two ends,
// face midpoints 1/4 of their four edge midpoints, the cell centre 1/6 of its
// six face centres, unless a sparse node already defines the vertex; any
// stencil value equal to the no-field value makes the result the no-field
// value, which becomes NaN on output.
//
// GB300 form: a cube at level L is self-contained -- every vertex inside it
// (faces and edges included) depends only on the cube's 8 corners and on the
// sparse nodes inside it -- so the grid is cut into tiles of 2^k cells, each
// computed by one CTA (one warp, for plans of tiles up to 8 cells) in shared
// memory in a single launch:
//   1. the tile's sparse nodes are placed into a NaN-filled shared tile;
//   2. one warp walks the L = d - k coarse levels down from the block's root
//      corners to the tile's 8 corners (27 points per level);
//   3. the k fine levels run over the shared tile (edges, faces, cells);
//   4. the tile's owned vertices go to HBM once, coalesced along x, with
//      no-field -> NaN and optional FP16/BF16 encoding fused into the store.
// The reference instead makes d full-grid passes through global memory.
// Sums run in the reference CPU interpolator's order, so results are
// bit-identical to it.
#include "interp_tile.cuh"
#include "s3r_internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

namespace s3r {
namespace {

__global__ void fill_f32_kernel(float* p, uint64_t n, float v)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void fill_u32_kernel(uint32_t* p, uint64_t n, uint32_t v)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// dense[ord(n2i[i])] = sparse[i]  (scatterSparseFieldKernel, DenseFieldInterpolatorArr_cu_3.cu:38-51)
__global__ void scatter_kernel(float* grid, uint32_t e, const uint16_t* n2i, const float* sparse, uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t x = n2i[3 * i], y = n2i[3 * i + 1], z = n2i[3 * i + 2];
    if (x >= e || y >= e || z >= e) return; // out-of-range node: ignored (the reference asserts)
    grid[((uint64_t)z * e + y) * e + x] = sparse[i];
}

// Work item `item` of the batched plan (kGrid: tile `item` of the single grid) as the tile it names.
template <bool kGrid> __device__ __forceinline__ TileItem decode_item(const TileArgs& a, uint32_t item)
{
    TileItem t;
    uint32_t tile;
    t.item = item;
    t.blk = 0;
    t.slots = 1;
    t.node_base = 0;
    t.dense_off = 0;
    if constexpr (kGrid) {
        t.d = a.grid_depth;
        t.k = a.grid_tile_log2 < t.d ? a.grid_tile_log2 : t.d;
        t.L = t.d - t.k;
        t.pitch = (1u << t.d) + 1u;
        tile = item;
    } else {
        const uint2 it = a.items[item];
        t.blk = it.x;
        tile = it.y & 0x7fffffffu;
        t.slots = it.y >> 31;
        const PlanBlock b = a.blocks[t.blk];
        t.d = b.depth;
        t.k = b.tile_log2;
        t.L = b.coarse_log2;
        t.node_base = b.node_base;
        t.dense_off = b.dense_off;
        t.pitch = b.pitch;
    }
    const uint32_t mL = 1u << t.L;
    t.tx = tile & (mL - 1);
    t.ty = (tile >> t.L) & (mL - 1);
    t.tz = tile >> (2 * t.L);
    return t;
}

template <bool kGrid, typename OutT>
__global__ void __launch_bounds__(kInterpThreads, 8) interp_tiles_kernel(TileArgs a)
{
    extern __shared__ float4 s_tile[]; // tile_smem_bytes(): (2^k+1)^3 floats rounded up to whole float4s
    float* s = reinterpret_cast<float*>(s_tile);
    __shared__ float desc[27 * kMaxDescentLevels];
    __shared__ uint32_t flags[(16 * 16 * 16) / 32]; // one bit per finest cube, tiles up to 32 cells
    __shared__ uint32_t item_s, next_s[2];
    const uint32_t nitems = a.nitems;
    const Crew<kInterpThreads> cw{threadIdx.x};
    // Work items come from the queue counter when there is one (zeroed before
    // the launch), else item blockIdx.x once per CTA.  The next item is taken
    // at the start of the current one so its entries can be prefetched.  The
    // slot it goes to alternates: a warp still reading slot i & 1 after the
    // loop's closing barrier must not see thread 0 refill it for item i + 2
    // (the barriers inside the tile keep thread 0 from getting that far).
    if (threadIdx.x == 0) item_s = a.queue ? atomicAdd(a.queue, 1u) : blockIdx.x;
    __syncthreads();
    uint32_t item = item_s;
    Prefetch pf;
    if constexpr (!kGrid) {
        prefetch_head<kInterpThreads>(pf, a, item, threadIdx.x);
        prefetch_index<kInterpThreads>(pf, a, threadIdx.x);
        prefetch_values<kInterpThreads>(pf, a, threadIdx.x);
    }
    for (uint32_t iter = 0;; ++iter) {
        if (item >= nitems) break;
        uint32_t* next_p = &next_s[iter & 1];
        if (threadIdx.x == 0) *next_p = a.queue ? atomicAdd(a.queue, 1u) : nitems;
        const TileItem t = decode_item<kGrid>(a, item);
        auto next = [next_p] { return *next_p; };
        switch (t.k) {
        case 0: run_tile<1, kGrid, OutT>(a, s, desc, flags, t, pf, cw, next); break;
        case 1: run_tile<2, kGrid, OutT>(a, s, desc, flags, t, pf, cw, next); break;
        case 2: run_tile<4, kGrid, OutT>(a, s, desc, flags, t, pf, cw, next); break;
        case 3: run_tile<8, kGrid, OutT>(a, s, desc, flags, t, pf, cw, next); break;
        case 4: run_tile<16, kGrid, OutT>(a, s, desc, flags, t, pf, cw, next); break;
        default: run_tile<32, kGrid, OutT>(a, s, desc, flags, t, pf, cw, next); break;
        }
        __syncthreads();
        item = *next_p;
    }
}

// Plans whose tiles are all of 8 cells or fewer: one warp per tile.  Each warp holds its own split tile
// (9^3 floats) and flag words in shared memory, takes its own items from the queue and synchronizes only
// with itself, so an SM keeps 32 tiles in flight instead of 8 CTAs' worth: a tile is a chain of short
// dependent phases (fill, placement, tile cube, coarse level, finest level), and more chains per SM hide
// more of their latency.  Same tile code, same results as the CTA kernel.
constexpr uint32_t kWarpTileFloats = ((9 * 9 * 9 + 3) / 4) * 4; // tile_smem_bytes(3) / 4
template <typename OutT> __global__ void __launch_bounds__(kInterpThreads, 8) interp_warp_tiles_kernel(TileArgs a)
{
    constexpr uint32_t kWarps = kInterpThreads / 32;
    __shared__ float4 s_all[kWarps][kWarpTileFloats / 4];
    __shared__ uint32_t flags_all[kWarps][2]; // 8-cell tiles: 64 finest cubes
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* s = reinterpret_cast<float*>(s_all[w]);
    uint32_t* flags = flags_all[w];
    const Crew<32> cw{lane};
    const uint32_t nitems = a.nitems;
    uint32_t item = lane == 0 ? atomicAdd(a.queue, 1u) : 0u;
    item = __shfl_sync(0xffffffffu, item, 0);
    Prefetch pf;
    prefetch_head<32>(pf, a, item, lane);
    prefetch_index<32>(pf, a, lane);
    prefetch_values<32>(pf, a, lane);
    while (item < nitems) {
        const uint32_t nxt = lane == 0 ? atomicAdd(a.queue, 1u) : 0u; // read by the warp once placed
        const TileItem t = decode_item<false>(a, item);
        auto next = [nxt] { return __shfl_sync(0xffffffffu, nxt, 0); };
        switch (t.k) {
        case 0: run_tile<1, false, OutT>(a, s, nullptr, flags, t, pf, cw, next); break;
        case 1: run_tile<2, false, OutT>(a, s, nullptr, flags, t, pf, cw, next); break;
        case 2: run_tile<4, false, OutT>(a, s, nullptr, flags, t, pf, cw, next); break;
        default: run_tile<8, false, OutT>(a, s, nullptr, flags, t, pf, cw, next); break;
        }
        __syncwarp();
        item = __shfl_sync(0xffffffffu, nxt, 0);
    }
}

// Per block {scale, offset} of its valid sparse values (16-bit bricks). All
// dense values are means of sparse values, so they stay inside this range.
__global__ void block_range_kernel(const PlanBlock* blocks, const uint64_t* node_off, const float* sparse,
                                   float2* so)
{
    const uint32_t b = blockIdx.x;
    const uint64_t n0 = node_off[b], n1 = node_off[b + 1];
    float lo = INFINITY, hi = -INFINITY;
    for (uint64_t i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
        const float v = sparse[i];
        if (v != kNoField && !isnan(v)) {
            lo = fminf(lo, v);
            hi = fmaxf(hi, v);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ float slo[32], shi[32];
    const uint32_t w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        slo[w] = lo;
        shi[w] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (uint32_t i = 1; i < blockDim.x / 32; ++i) {
            lo = fminf(lo, slo[i]);
            hi = fmaxf(hi, shi[i]);
        }
        float scale = hi - lo;
        if (!(scale > 0.f) || !isfinite(scale)) scale = 1.f;
        if (!isfinite(lo)) lo = 0.f;
        so[b] = make_float2(scale, lo);
    }
}

// Per-block preparation of a plan frame, one CTA of kInterpThreads per block:
//  * 16-bit bricks: the {scale, offset} of the block's valid sparse values (as block_range_kernel);
//  * a block cut into 2^L > 1 tiles per axis: its coarse grid, the (2^L+1)^3 vertices at multiples of
//    the tile edge, from the sparse nodes on it, filled level by level exactly as cube_level fills a
//    tile (the reference's midpoint rules, sums in its order).  A midpoint of a coarse level depends
//    only on the points of that level's cube, so the full grid holds the values a descent from the
//    block's root along any one tile's path computes -- each tile then reads its 8 corners from it
//    instead of descending itself, and the plan carries the coarse nodes once per block instead of
//    once per tile.
__global__ void __launch_bounds__(kInterpThreads) block_prep_kernel(PrepArgs a)
{
    const uint32_t b = blockIdx.x;
    const PlanBlock B = a.blocks[b];
    if (a.scale_offset) {
        const uint64_t n0 = a.node_off[b], n1 = a.node_off[b + 1];
        float lo = INFINITY, hi = -INFINITY;
        for (uint64_t i = n0 + threadIdx.x; i < n1; i += kInterpThreads) {
            const float v = a.sparse[i];
            if (v != kNoField && !isnan(v)) {
                lo = fminf(lo, v);
                hi = fmaxf(hi, v);
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        __shared__ float slo[kInterpThreads / 32], shi[kInterpThreads / 32];
        if ((threadIdx.x & 31) == 0) {
            slo[threadIdx.x >> 5] = lo;
            shi[threadIdx.x >> 5] = hi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint32_t i = 1; i < kInterpThreads / 32; ++i) {
                lo = fminf(lo, slo[i]);
                hi = fmaxf(hi, shi[i]);
            }
            float scale = hi - lo;
            if (!(scale > 0.f) || !isfinite(scale)) scale = 1.f;
            if (!isfinite(lo)) lo = 0.f;
            a.scale_offset[b] = make_float2(scale, lo);
        }
    }
    const uint32_t L = B.coarse_log2;
    if (L == 0) return;
    const uint32_t T = 1u << L, E = T + 1, E3 = E * E * E;
    float* g = a.coarse + B.coarse_off;
    for (uint32_t p = threadIdx.x; p < E3; p += kInterpThreads) g[p] = qnan();
    __syncthreads();
    for (uint32_t i = a.centry_off[b] + threadIdx.x; i < a.centry_off[b + 1]; i += kInterpThreads) {
        const uint2 ce = a.centry[i];
        if (ce.x < E3) g[ce.x] = to_internal(a.sparse[B.node_base + ce.y]);
    }
    __syncthreads();
    for (uint32_t j = 0; j < L; ++j) {
        cube_level(g, E, T, j);
        __syncthreads();
    }
}

inline uint32_t ctas_for(uint64_t n, uint32_t threads)
{
    uint64_t c = (n + threads - 1) / threads;
    if (c > 152ull * 64) c = 152ull * 64;
    return c ? (uint32_t)c : 1u;
}

template <bool kGrid, typename OutT>
cudaError_t launch_tiles(const TileArgs& a, uint32_t tile_log2_max, uint32_t grid_ctas, cudaStream_t s)
{
    if constexpr (!kGrid) {
        if (tile_log2_max <= 3 && a.queue) {
            interp_warp_tiles_kernel<OutT><<<grid_ctas, kInterpThreads, 0, s>>>(a);
            return cudaGetLastError();
        }
    }
    const size_t smem = tile_smem_bytes(tile_log2_max);
    auto kern = interp_tiles_kernel<kGrid, OutT>;
    if (smem > 48 * 1024) {
        cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    kern<<<grid_ctas, kInterpThreads, smem, s>>>(a);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_fill_f32(float* p, uint64_t n, float v, cudaStream_t s)
{
    fill_f32_kernel<<<ctas_for(n, 256), 256, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_fill_u32(uint32_t* p, uint64_t n, uint32_t v, cudaStream_t s)
{
    fill_u32_kernel<<<ctas_for(n, 256), 256, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

cudaError_t launch_scatter_nodes(float* grid, uint32_t depth, const uint16_t* n2i, const float* sparse, uint32_t n,
                                 cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    scatter_kernel<<<(n + 255) / 256, 256, 0, s>>>(grid, (1u << depth) + 1u, n2i, sparse, n);
    return cudaGetLastError();
}

cudaError_t launch_interp_grid(const float* grid, uint32_t depth, float* dense, cudaStream_t s, uint32_t* launches)
{
    TileArgs a{};
    a.grid = grid;
    a.grid_depth = depth;
    a.grid_tile_log2 = depth < 4 ? depth : 4;
    const uint32_t L = depth - a.grid_tile_log2;
    a.nitems = 1u << (3 * L);
    a.out = dense;
    if (launches) ++*launches;
    return launch_tiles<true, float>(a, a.grid_tile_log2, a.nitems, s);
}

uint32_t interp_plan_ctas_per_sm(uint32_t fmt, uint32_t tile_log2)
{
    const bool warp = tile_log2 <= 3; // the warp-per-tile kernel (static shared memory only)
    const size_t smem = warp ? 0 : tile_smem_bytes(tile_log2);
    int n = 0;
    cudaError_t e = cudaErrorInvalidValue;
    auto occ = [&](auto kern) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, kInterpThreads, smem);
    };
    switch (fmt) {
    case S3R_BRICK_F32: warp ? occ(interp_warp_tiles_kernel<float>) : occ(interp_tiles_kernel<false, float>); break;
    case S3R_BRICK_F16: warp ? occ(interp_warp_tiles_kernel<__half>) : occ(interp_tiles_kernel<false, __half>); break;
    case S3R_BRICK_BF16:
        warp ? occ(interp_warp_tiles_kernel<__nv_bfloat16>) : occ(interp_tiles_kernel<false, __nv_bfloat16>);
        break;
    default: break;
    }
    return (e == cudaSuccess && n > 0) ? (uint32_t)n : 1u;
}

cudaError_t launch_interp_plan(const TileArgs& a, uint32_t fmt, uint32_t tile_log2_max, uint32_t grid_ctas,
                               cudaStream_t s)
{
    if (a.nitems == 0) return cudaSuccess;
    switch (fmt) {
    case S3R_BRICK_F32: return launch_tiles<false, float>(a, tile_log2_max, grid_ctas, s);
    case S3R_BRICK_F16: return launch_tiles<false, __half>(a, tile_log2_max, grid_ctas, s);
    case S3R_BRICK_BF16: return launch_tiles<false, __nv_bfloat16>(a, tile_log2_max, grid_ctas, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_block_prep(const PrepArgs& a, uint32_t nblocks, cudaStream_t s)
{
    if (nblocks == 0) return cudaSuccess;
    block_prep_kernel<<<nblocks, kInterpThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_block_ranges(const PlanBlock* blocks, uint32_t nblocks, const float* sparse,
                                const uint64_t* node_off_dev, float2* scale_offset, cudaStream_t s)
{
    if (nblocks == 0) return cudaSuccess;
    block_range_kernel<<<nblocks, 256, 0, s>>>(blocks, node_off_dev, sparse, scale_offset);
    return cudaGetLastError();
}

} // namespace s3r
