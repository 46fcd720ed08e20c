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
// computed by one CTA in shared memory in a single launch:
//   1. the tile's sparse nodes are placed into a NaN-filled shared tile;
//   2. one warp walks the L = d - k coarse levels down from the block's root
//      corners to the tile's 8 corners (27 points per level);
//   3. the k fine levels run over the shared tile (edges, faces, cells);
//   4. the tile's owned vertices go to HBM once, coalesced along x, with
//      no-field -> NaN and optional FP16/BF16 encoding fused into the store.
// The reference instead makes d full-grid passes through global memory.
// Sums run in the reference CPU interpolator's order, so results are
// bit-identical to it.
#include "s3r_internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace s3r {
namespace {

constexpr float kHalf = 0.5f;
constexpr float kQuarter = 0.25f;
constexpr float kSixth = (float)(1.0 / 6.0);

__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

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

template <typename OutT> struct Store;
template <> struct Store<float> {
    __device__ static void put(float* out, uint64_t i, float v, float, float)
    {
        out[i] = v == kNoField ? qnan() : v;
    }
};
template <> struct Store<__half> {
    __device__ static void put(__half* out, uint64_t i, float v, float inv_scale, float offset)
    {
        out[i] = (v == kNoField || isnan(v)) ? __ushort_as_half((unsigned short)0x7e00)
                                             : __float2half_rn((v - offset) * inv_scale);
    }
};
template <> struct Store<__nv_bfloat16> {
    __device__ static void put(__nv_bfloat16* out, uint64_t i, float v, float inv_scale, float offset)
    {
        out[i] = (v == kNoField || isnan(v)) ? __ushort_as_bfloat16((unsigned short)0x7fc0)
                                             : __float2bfloat16_rn((v - offset) * inv_scale);
    }
};

// Value of a coarse-lattice vertex for the descent: the sparse value there, or NaN.
template <bool kGrid>
__device__ __forceinline__ float coarse_value(const TileArgs& a, uint32_t gx, uint32_t gy, uint32_t gz, uint32_t e,
                                              uint32_t k, uint32_t L, uint32_t coarse_off, uint64_t node_base)
{
    if constexpr (kGrid) {
        return a.grid[((uint64_t)gz * e + gy) * e + gx];
    } else {
        uint32_t m1 = (1u << L) + 1u;
        int32_t idx = a.coarse_idx[coarse_off + (gx >> k) + m1 * ((gy >> k) + m1 * (gz >> k))];
        return idx < 0 ? qnan() : a.sparse[node_base + (uint32_t)idx];
    }
}

__device__ __forceinline__ float mid2(float lo, float hi)
{
    return (lo == kNoField || hi == kNoField) ? kNoField : kHalf * (lo + hi);
}
__device__ __forceinline__ float mid4(float l1, float h1, float l2, float h2)
{
    return (l1 == kNoField || h1 == kNoField || l2 == kNoField || h2 == kNoField) ? kNoField
                                                                                  : kQuarter * (l1 + h1 + l2 + h2);
}
__device__ __forceinline__ float mid6(float l1, float h1, float l2, float h2, float l3, float h3)
{
    return (l1 == kNoField || h1 == kNoField || l2 == kNoField || h2 == kNoField || l3 == kNoField ||
            h3 == kNoField)
               ? kNoField
               : kSixth * (l1 + h1 + l2 + h2 + l3 + h3);
}

// Warp 0: walk from the block's root corners down L levels to the 8 corners of
// the tile at (ox, oy, oz) (vertex coordinates), writing them into the tile.
template <bool kGrid>
__device__ void descend(const TileArgs& a, float* s, float* c27, uint32_t d, uint32_t k, uint32_t L,
                        uint32_t coarse_off, uint64_t node_base, uint32_t ox, uint32_t oy, uint32_t oz)
{
    const uint32_t lane = threadIdx.x;
    const uint32_t e = (1u << d) + 1u;
    const uint32_t T = 1u << k, E = T + 1u;
    uint32_t size = 1u << d;
    uint32_t gx0 = 0, gy0 = 0, gz0 = 0;
    float corner = 0.f;
    if (lane < 8)
        corner = coarse_value<kGrid>(a, (lane & 1) ? size : 0, (lane & 2) ? size : 0, (lane & 4) ? size : 0, e, k, L,
                                     coarse_off, node_base);
    const uint32_t px = lane % 3, py = (lane / 3) % 3, pz = lane / 9;
    const uint32_t nodd = (px & 1) + (py & 1) + (pz & 1);
    for (uint32_t l = 0; l < L; ++l) {
        const uint32_t hs = size >> 1;
        const uint32_t src = lane < 27 ? (px >> 1) + 2 * (py >> 1) + 4 * (pz >> 1) : 0;
        const float cv = __shfl_sync(0xffffffffu, corner, (int)src);
        if (lane < 27)
            c27[lane] = nodd == 0 ? cv
                                  : coarse_value<kGrid>(a, gx0 + hs * px, gy0 + hs * py, gz0 + hs * pz, e, k, L,
                                                        coarse_off, node_base);
        __syncwarp();
        if (lane < 27 && nodd == 1 && isnan(c27[lane])) {
            const uint32_t st = (px & 1) ? 1 : ((py & 1) ? 3 : 9);
            c27[lane] = mid2(c27[lane - st], c27[lane + st]);
        }
        __syncwarp();
        if (lane < 27 && nodd == 2 && isnan(c27[lane])) {
            // the two odd axes, ascending
            const uint32_t s1 = (px & 1) ? 1 : 3;
            const uint32_t s2 = (pz & 1) ? 9 : 3;
            c27[lane] = mid4(c27[lane - s1], c27[lane + s1], c27[lane - s2], c27[lane + s2]);
        }
        __syncwarp();
        if (lane == 13 && isnan(c27[13]))
            c27[13] = mid6(c27[12], c27[14], c27[10], c27[16], c27[4], c27[22]);
        __syncwarp();
        const uint32_t qx = (ox - gx0) >= hs ? 1u : 0u;
        const uint32_t qy = (oy - gy0) >= hs ? 1u : 0u;
        const uint32_t qz = (oz - gz0) >= hs ? 1u : 0u;
        if (lane < 8)
            corner = c27[(qx + (lane & 1)) + 3 * (qy + ((lane >> 1) & 1)) + 9 * (qz + (lane >> 2))];
        gx0 += qx * hs;
        gy0 += qy * hs;
        gz0 += qz * hs;
        size = hs;
        __syncwarp();
    }
    if (lane < 8)
        s[(lane & 1) * T + E * (((lane >> 1) & 1) * T + E * ((lane >> 2) * T))] = corner;
}

// The k fine levels of one tile of 2^k cells held in shared memory (edge E = 2^k+1).
__device__ void fine_levels(float* s, uint32_t k)
{
    const uint32_t T = 1u << k, E = T + 1u;
    const uint32_t stride[3] = {1u, E, E * E};
    for (uint32_t j = 0; j < k; ++j) {
        const uint32_t m = 1u << j, sz = T >> j, hs = sz >> 1;
        const uint32_t m1 = m + 1;
        // edges: odd along axis a only
        {
            const uint32_t per = m * m1 * m1, cnt = 3 * per;
            for (uint32_t idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
                const uint32_t a = idx / per;
                uint32_t r = idx - a * per;
                const uint32_t i = r & (m - 1);
                r >>= j;
                const uint32_t jb = r % m1, jc = r / m1;
                uint32_t c[3];
                c[a] = hs + sz * i;
                c[(a + 1) % 3] = sz * jb;
                c[(a + 2) % 3] = sz * jc;
                const uint32_t p = c[0] + E * (c[1] + E * c[2]);
                if (isnan(s[p])) {
                    const uint32_t st = hs * stride[a];
                    s[p] = mid2(s[p - st], s[p + st]);
                }
            }
        }
        __syncthreads();
        // faces: even along axis a, odd along the other two
        {
            const uint32_t per = m1 * m * m, cnt = 3 * per;
            for (uint32_t idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
                const uint32_t a = idx / per;
                uint32_t r = idx - a * per;
                const uint32_t ia = r % m1;
                r /= m1;
                const uint32_t ib = r & (m - 1), ic = r >> j;
                const uint32_t b = a == 0 ? 1u : 0u, cax = a == 2 ? 1u : 2u;
                uint32_t c[3];
                c[a] = sz * ia;
                c[b] = hs + sz * ib;
                c[cax] = hs + sz * ic;
                const uint32_t p = c[0] + E * (c[1] + E * c[2]);
                if (isnan(s[p])) {
                    const uint32_t sb = hs * stride[b], sc = hs * stride[cax];
                    s[p] = mid4(s[p - sb], s[p + sb], s[p - sc], s[p + sc]);
                }
            }
        }
        __syncthreads();
        // cells
        {
            const uint32_t cnt = m * m * m;
            for (uint32_t idx = threadIdx.x; idx < cnt; idx += blockDim.x) {
                const uint32_t x = hs + sz * (idx & (m - 1));
                const uint32_t y = hs + sz * ((idx >> j) & (m - 1));
                const uint32_t z = hs + sz * (idx >> (2 * j));
                const uint32_t p = x + E * (y + E * z);
                if (isnan(s[p])) {
                    const uint32_t s0 = hs, s1 = hs * E, s2 = hs * E * E;
                    s[p] = mid6(s[p - s0], s[p + s0], s[p - s1], s[p + s1], s[p - s2], s[p + s2]);
                }
            }
        }
        __syncthreads();
    }
}

template <bool kGrid, typename OutT>
__global__ void __launch_bounds__(kInterpThreads) interp_tiles_kernel(TileArgs a)
{
    extern __shared__ float s[];
    __shared__ float c27[32];
    const uint32_t nitems = a.nitems;
    for (uint32_t item = blockIdx.x; item < nitems; item += gridDim.x) {
        uint32_t d, k, L, tile, coarse_off = 0;
        uint64_t node_base = 0, dense_off = 0;
        uint32_t blk = 0;
        if constexpr (kGrid) {
            d = a.grid_depth;
            k = a.grid_tile_log2 < d ? a.grid_tile_log2 : d;
            L = d - k;
            tile = item;
        } else {
            const uint2 it = a.items[item];
            blk = it.x;
            tile = it.y;
            const PlanBlock b = a.blocks[blk];
            d = b.depth;
            k = b.tile_log2;
            L = b.coarse_log2;
            coarse_off = b.coarse_off;
            node_base = b.node_base;
            dense_off = b.dense_off;
        }
        const uint32_t T = 1u << k, E = T + 1u, E3 = E * E * E;
        const uint32_t mL = 1u << L;
        const uint32_t tx = tile & (mL - 1), ty = (tile >> L) & (mL - 1), tz = tile >> (2 * L);
        const uint32_t ox = tx * T, oy = ty * T, oz = tz * T;
        const uint32_t e = (1u << d) + 1u;

        // 1. nodes into the shared tile
        if constexpr (kGrid) {
            for (uint32_t p = threadIdx.x; p < E3; p += blockDim.x) {
                const uint32_t lx = p % E, r = p / E, ly = r % E, lz = r / E;
                s[p] = a.grid[((uint64_t)(oz + lz) * e + (oy + ly)) * e + (ox + lx)];
            }
        } else {
            for (uint32_t p = threadIdx.x; p < E3; p += blockDim.x)
                s[p] = qnan();
            __syncthreads();
            const uint64_t b0 = a.entry_off[item], b1 = a.entry_off[item + 1];
            for (uint64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x)
                s[a.entry_local[i]] = a.sparse[node_base + a.entry_node[i]];
        }
        __syncthreads();

        // 2. tile corners from the coarse levels
        if (L > 0) {
            if (threadIdx.x < 32)
                descend<kGrid>(a, s, c27, d, k, L, coarse_off, node_base, ox, oy, oz);
            __syncthreads();
        }

        // 3. fine levels
        fine_levels(s, k);

        // 4. owned vertices to HBM: [0, T) per axis, plus the far face on the last tile
        float inv_scale = 1.f, offset = 0.f;
        if constexpr (!kGrid) {
            if (a.scale_offset) {
                const float2 so = a.scale_offset[blk];
                inv_scale = 1.f / so.x;
                offset = so.y;
            }
        }
        OutT* out = reinterpret_cast<OutT*>(a.out) + dense_off;
        const uint32_t OX = T + (tx == mL - 1 ? 1u : 0u);
        const uint32_t OY = T + (ty == mL - 1 ? 1u : 0u);
        const uint32_t OZ = T + (tz == mL - 1 ? 1u : 0u);
        const uint32_t rows = OY * OZ;
        const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
        for (uint32_t row = warp; row < rows; row += nwarps) {
            const uint32_t ly = row % OY, lz = row / OY;
            const uint64_t g = ((uint64_t)(oz + lz) * e + (oy + ly)) * e + ox;
            const uint32_t sp = E * (ly + E * lz);
            for (uint32_t lx = lane; lx < OX; lx += 32)
                Store<OutT>::put(out, g + lx, s[sp + lx], inv_scale, offset);
        }
        __syncthreads();
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

inline uint32_t ctas_for(uint64_t n, uint32_t threads)
{
    uint64_t c = (n + threads - 1) / threads;
    if (c > 152ull * 64) c = 152ull * 64;
    return c ? (uint32_t)c : 1u;
}

template <bool kGrid, typename OutT>
cudaError_t launch_tiles(const TileArgs& a, uint32_t tile_log2_max, uint32_t grid_ctas, cudaStream_t s)
{
    const uint32_t E = (1u << tile_log2_max) + 1u;
    const size_t smem = (size_t)E * E * E * sizeof(float);
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

cudaError_t launch_block_ranges(const PlanBlock* blocks, uint32_t nblocks, const float* sparse,
                                const uint64_t* node_off_dev, float2* scale_offset, cudaStream_t s)
{
    if (nblocks == 0) return cudaSuccess;
    block_range_kernel<<<nblocks, 256, 0, s>>>(blocks, node_off_dev, sparse, scale_offset);
    return cudaGetLastError();
}

} // namespace s3r
