// Child -> parent field propagation of one metadata level: the data-parallel
// part of BlockTreeFieldProvider<3>::generatePropagatedField
// (include/s3dmm/BlockTreeFieldProvider.hpp:270-389, lines 305-350 for the
// propagation proper).
//
// A parent subtree of depth D gets, at each of its nodes, the values of the
// nodes of its (up to 8) child subtrees that land there: a child of depth Dc in
// local position c = x + 2y + 4z maps its node n to
//     signed_shift_right(n, Dc + 1 - D) + (c bits) << (D - 1)
// taking only nodes with all coordinates even when the shift is positive.  A
// parent node receives at most one node per child.  That correspondence is
// fixed by the tree, so it is computed once per level (prop_map_kernel fills a
// dense vertex -> node map per parent, prop_index_kernel resolves every child
// node through it) into 8 child-node indices per parent node, -1 where that
// child has none.  Each field and time frame is then one gather
// (prop_gather_kernel): per parent node its up-to-8 child values summed in the
// reference's child order from 0 -- the same float additions, in the same
// order, as its per-child accumulation loop, skipping the no-field value as
// it does.

#include "s3r_internal.h"

namespace s3r {

namespace {

__device__ __forceinline__ uint32_t find_owner(const uint64_t* off, uint32_t n, uint64_t i)
{
    // largest k with off[k] <= i (off has n+1 entries, off[0] = 0)
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// One thread per parent node: its dense map entry and its 8 empty sources.
__global__ void prop_map_kernel(PropArgs a)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.parent_nodes) return;
    const uint32_t p = find_owner(a.parent_node_off, a.nparents, i);
    const PropParent P = a.parents[p];
    const uint64_t e = (1ull << P.depth) + 1;
    const uint16_t* c = a.parent_n2i + 3 * i;
    a.map[P.map_off + ((uint64_t)c[2] * e + c[1]) * e + c[0]] = (int32_t)(i - a.parent_node_off[p]);
    int4* s = reinterpret_cast<int4*>(a.src + 8 * i);
    const int4 none = make_int4(-1, -1, -1, -1);
    s[0] = none;
    s[1] = none;
}

// One thread per child node: its index into source c of the parent node it lands on.
__global__ void prop_index_kernel(PropArgs a)
{
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.child_nodes) return;
    const uint32_t k = find_owner(a.child_node_off, a.nchildren, j);
    const PropChild C = a.children[k];
    const uint16_t* cn = a.child_n2i + 3 * j;
    uint32_t x = cn[0], y = cn[1], z = cn[2];
    if (C.shift >= 1) {
        if ((x | y | z) & 1u) return;
        x >>= C.shift;
        y >>= C.shift;
        z >>= C.shift;
    } else {
        x <<= -C.shift;
        y <<= -C.shift;
        z <<= -C.shift;
    }
    const PropParent P = a.parents[C.parent];
    const uint32_t half = 1u << (P.depth - 1);
    x += (C.c & 1u) * half;
    y += ((C.c >> 1) & 1u) * half;
    z += (C.c >> 2) * half;
    const uint32_t e = (1u << P.depth) + 1;
    const uint64_t pcount = a.parent_node_off[C.parent + 1] - a.parent_node_off[C.parent];
    if (x >= e || y >= e || z >= e) {
        atomicOr(a.error, 1u);
        return;
    }
    // the map is not cleared between uses: an entry counts only when it names a node of this
    // parent whose coordinates are these
    const int32_t m = a.map[P.map_off + ((uint64_t)z * e + y) * e + x];
    const uint64_t g = a.parent_node_off[C.parent] + (uint64_t)m;
    if (m < 0 || (uint64_t)m >= pcount || a.parent_n2i[3 * g] != x || a.parent_n2i[3 * g + 1] != y ||
        a.parent_n2i[3 * g + 2] != z) {
        atomicOr(a.error, 2u); // the parent has no node there (the reference's i2n.at() throws)
        return;
    }
    a.src[8 * g + C.c] = (int32_t)j;
}

// One thread per parent node: sum and count of its children's values in child order.
__global__ void prop_gather_kernel(const int32_t* __restrict__ src, const float* __restrict__ child_values, uint64_t n,
                                   float* __restrict__ sums, float* __restrict__ weights)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4* s = reinterpret_cast<const int4*>(src + 8 * i);
    const int4 lo = __ldg(s), hi = __ldg(s + 1);
    const int32_t j[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
    float v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = j[c] >= 0 ? __ldg(child_values + j[c]) : kNoField;
    float sum = 0.f, w = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c)
        if (v[c] != kNoField) {
            sum = __fadd_rn(sum, v[c]);
            w = __fadd_rn(w, 1.f);
        }
    sums[i] = sum;
    weights[i] = w;
}

__global__ void divide_kernel(const float* sums, const float* weights, uint64_t n, float* values)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float w = weights[i];
    values[i] = w > 0.f ? __fdiv_rn(sums[i], w) : kNoField;
}

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

} // namespace

cudaError_t launch_prop_index(const PropArgs& a, cudaStream_t s, uint32_t* launches)
{
    constexpr unsigned T = 256;
    *launches = 0;
    if (a.parent_nodes == 0) return cudaSuccess;
    prop_map_kernel<<<blocks_for(a.parent_nodes, T), T, 0, s>>>(a);
    ++*launches;
    if (a.child_nodes) {
        prop_index_kernel<<<blocks_for(a.child_nodes, T), T, 0, s>>>(a);
        ++*launches;
    }
    return cudaGetLastError();
}

cudaError_t launch_prop_gather(const int32_t* src, const float* child_values, uint64_t n, float* sums, float* weights,
                               cudaStream_t s)
{
    if (!n) return cudaSuccess;
    prop_gather_kernel<<<blocks_for(n, 256), 256, 0, s>>>(src, child_values, n, sums, weights);
    return cudaGetLastError();
}

cudaError_t launch_divide(const float* sums, const float* weights, uint64_t n, float* values, cudaStream_t s)
{
    if (!n) return cudaSuccess;
    divide_kernel<<<blocks_for(n, 256), 256, 0, s>>>(sums, weights, n, values);
    return cudaGetLastError();
}

} // namespace s3r
