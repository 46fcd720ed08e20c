// Internal types shared by the s3r CUDA kernels and the host side of the C ABI.
#pragma once

#include "s3r.h"

#include <cstdint>
#include <cuda_runtime.h>

namespace s3r {

// Sets the message s3r_last_error(NULL) returns on this thread (host.cpp).
void set_thread_error(const char* msg);

constexpr float kNoField = S3R_NO_FIELD_VALUE;
constexpr int kInterpThreads = 128;

// One block of a batched plan, as the interpolation kernel reads it.
struct PlanBlock {
    uint32_t depth;       // subtree depth d: (2^d+1)^3 vertices
    uint32_t tile_log2;   // k: tile edge 2^k cells (k <= d)
    uint32_t coarse_log2; // L = d - k: tiles per axis 2^L
    uint32_t coarse_off;  // first vertex of this block's coarse grid ((2^L+1)^3 values)
    uint64_t node_base;   // first node of this block in the sparse value array
    uint64_t dense_off;   // first element of this block's brick
    uint32_t pitch;       // brick row pitch in elements (>= 2^d+1): vertex (x, y, z) at (z (2^d+1) + y) pitch + x
    uint32_t pad;
};

// Row pitch of a batched plan's brick of depth d: 2^d+1 rounded up to whole
// 32-byte sectors, so that every row -- and with it every block, whose size is
// a whole number of rows times 2^d+1 -- starts on a sector boundary and tiles
// that split a row never share a sector.
inline __host__ __device__ uint32_t plan_brick_pitch(uint32_t depth, uint32_t elem_bytes)
{
    const uint32_t per = 32u / elem_bytes;
    return (((1u << depth) + 1u + per - 1u) / per) * per;
}

// Arguments of the tile interpolation kernel.  Two node sources:
//   grid   != nullptr: one block whose sparse values were scattered into a
//                      NaN-filled (2^d+1)^3 grid (blocks/items unused);
//   grid   == nullptr: a batched plan whose nodes are binned per tile.
struct TileArgs {
    const PlanBlock* blocks;
    const uint2* items;           // {block, tile} per work item
    uint32_t nitems;
    const uint64_t* entry_off;    // nitems+1 prefix offsets into local/node
    const uint16_t* entry_local;  // node position inside its tile (tile_offset)
    const uint32_t* entry_node;   // node index within its block
    // entry_local >= (2^k+1)^3 addresses descent slot 27*level + point instead of the tile
    const uint32_t* flags;        // per item flag_words words: bit c set when finest cube c of the tile
    uint32_t flag_words;          // holds a sparse value at one of its midpoints (plan form only)
    const float* sparse;          // node values
    const float2* scale_offset;   // per block {scale, offset} for 16-bit bricks
    void* out;                    // brick store
    uint32_t* queue;              // work-queue counter, zeroed before the launch (nullptr: one item per CTA)
    const float* coarse;          // plan form: per block cut into 2^L > 1 tiles per axis its coarse grid (the
                                  // (2^L+1)^3 vertices at multiples of the tile edge, internal values), from
                                  // block_prep_kernel: a tile reads its 8 corners there
    // single-block form
    const float* grid;
    uint32_t grid_depth;
    uint32_t grid_tile_log2;
};

// Position of vertex (x, y, z) inside the shared tile of T cells, as the
// interpolation kernel lays it out: for T >= 2 the parity-split layout (eight
// sub-arrays by the parities of x, y, z, each x fastest; see interp.cu), for
// T = 1 plain x + 2(y + 2z).  The plan stores node positions in this form.
inline __host__ __device__ uint32_t tile_offset(uint32_t T, uint32_t x, uint32_t y, uint32_t z)
{
    if (T < 2) return x + 2 * (y + 2 * z);
    const uint32_t H = T / 2, G = H + 1;
    const uint32_t c = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
    uint32_t base = 0;
    for (uint32_t i = 0; i < c; ++i) base += ((i & 1) ? H : G) * (((i >> 1) & 1) ? H : G) * (((i >> 2) & 1) ? H : G);
    const uint32_t nx = (x & 1) ? H : G, ny = (y & 1) ? H : G;
    return base + (x >> 1) + nx * ((y >> 1) + ny * (z >> 1));
}

// Per-block entry of the render block table (dense over the (2^level)^3 block grid).
struct RenderBlock {
    uint32_t depth;    // 0xffffffff: no block here
    uint32_t fmt;      // S3R_BRICK_*
    uint64_t brick_off;
    int32_t rect[4];   // view rectangle {x, y, w, h}
    float center[3];   // cube centre and half size (DenseFieldRenderer_cu.cu:337-350)
    float half;
    float origin[3];   // texture-space origin: centre - (half + texel/2)  (:176-180)
    float factor;      // world -> texel scale n / (2 (half + texel/2))     (:181)
    float texel;       // 2 half / n                                         (:169)
    uint32_t block;    // index into the plan's block list (per-brick scale/offset)
    uint32_t pitch;    // brick row pitch in elements; 0: 2^depth+1 (a plain dense grid)
    uint32_t pad;
};

// Per-block sampling constants of DenseFieldRenderer_cu.cu:168-181, with the
// reference's mix of float and double arithmetic (host.cpp).
void block_sampling(uint32_t level, const uint32_t idx[3], uint32_t depth, RenderBlock& rb);

struct FrameArgs {
    const s3r_view* view;          // device copy
    const RenderBlock* table;      // (2^level)^3 entries
    const void* bricks;
    const float* tf;               // tf_n RGBA
    float* rgba;                   // optional
    uint32_t* argb;                // optional
    unsigned long long* samples;   // optional
    const float2* scale_offset;    // per block {scale, offset} (16-bit bricks)
    const int32_t* cover;          // device {x0, y0, x1, y1}: union of the blocks' view rectangles
    // adjoint
    const float* fwd_rgba;
    const float* dl_drgba;
    float* dtf;
    float* ddense;
    float* dtf_part;      // kDtfParts zeroed copies of dtf (tf_n RGBA float4 each), summed into dtf afterwards
};

// The block-major frame render (render tile ids kRenderWalkTiles and up): its work
// items and per-pixel block results.
constexpr uint32_t kSegMaskWords = 6; // rank masks of up to 384 ranks: levels <= 7
struct SegArgs {
    const uint2* items;         // {block cell, tile} per warp work item: the footprint-sized tiles of every
                                // block's view rectangle, deepest blocks first
    const uint32_t* count;      // items
    uint32_t words;             // mask words per pixel: ceil((3m - 2) / 64)
    float4* seg;                // [rank][pixel] premultiplied block results
    unsigned long long* mask;   // [word][pixel] ranks holding a result
    uint32_t* queue;            // work-queue counter: 0 before the segment launch, zeroed again by the composite
};

// The adjoint spreads its transfer-function gradient over kDtfParts copies
// (CTA index modulo kDtfCtaGroups, lane modulo kDtfLaneGroups) so that global
// reductions to one table entry rarely meet; a last kernel sums the copies.
constexpr uint32_t kDtfCtaGroups = 64, kDtfLaneGroups = 8;
constexpr uint32_t kDtfParts = kDtfCtaGroups * kDtfLaneGroups;

// Records a failure for s3r_last_error(NULL) and returns code (host.cpp).
int record_error(int code, const char* msg);
int record_cuda_error(cudaError_t e, const char* what);

// Kernel launchers (defined in the .cu files); all return cudaGetLastError().
// Child -> parent propagation of one metadata level (propagate.cu).
struct PropParent {
    uint32_t depth;   // parent subtree depth D
    uint32_t pad;
    uint64_t map_off; // start of its (2^D+1)^3 dense map
};
struct PropChild {
    uint32_t parent;  // index of its parent subtree
    uint32_t c;       // local position x + 2y + 4z in the parent
    int32_t shift;    // child depth + 1 - parent depth
    uint32_t pad;
};
struct PropArgs {
    const PropParent* parents;
    const uint64_t* parent_node_off; // nparents+1
    const uint16_t* parent_n2i;
    const PropChild* children;
    const uint64_t* child_node_off;  // nchildren+1
    const uint16_t* child_n2i;
    int32_t* map;                    // dense vertex -> node maps (uninitialized; entries are verified)
    int32_t* src;                    // out: 8 child-node indices per parent node, -1 = none
    uint32_t* error;                 // bit 0: node outside the parent; bit 1: no parent node there
    uint64_t parent_nodes, child_nodes;
    uint32_t nparents, nchildren;
};
cudaError_t launch_prop_index(const PropArgs& a, cudaStream_t s, uint32_t* launches);
cudaError_t launch_prop_gather(const int32_t* src, const float* child_values, uint64_t n, float* sums, float* weights,
                               cudaStream_t s);
cudaError_t launch_divide(const float* sums, const float* weights, uint64_t n, float* values, cudaStream_t s);
// Adds n to the context's launch counter (host.cpp).
void count_launches(s3r_ctx* ctx, uint32_t n);

cudaError_t launch_fill_f32(float* p, uint64_t n, float v, cudaStream_t s);
cudaError_t launch_fill_u32(uint32_t* p, uint64_t n, uint32_t v, cudaStream_t s);
cudaError_t launch_scatter_nodes(float* grid, uint32_t depth, const uint16_t* n2i, const float* sparse, uint32_t n,
                                 cudaStream_t s);
cudaError_t launch_interp_grid(const float* grid, uint32_t depth, float* dense, cudaStream_t s, uint32_t* launches);
cudaError_t launch_interp_plan(const TileArgs& a, uint32_t fmt, uint32_t tile_log2_max, uint32_t grid_ctas,
                               cudaStream_t s);
uint32_t interp_plan_ctas_per_sm(uint32_t fmt, uint32_t tile_log2);
// Per-block preparation of a plan frame (interp.cu), one CTA per block: the 16-bit {scale, offset} when
// scale_offset is set, and the coarse grid of every block with coarse levels.
struct PrepArgs {
    const PlanBlock* blocks;
    const uint64_t* node_off;     // nblocks + 1
    const float* sparse;
    float2* scale_offset;         // nullptr: F32 bricks
    float* coarse;                // coarse grids, at PlanBlock::coarse_off
    const uint32_t* centry_off;   // nblocks + 1: the sparse nodes on each block's coarse grid
    const uint2* centry;          // {coarse grid index, node index within the block}
};
cudaError_t launch_block_prep(const PrepArgs& a, uint32_t nblocks, cudaStream_t s);
cudaError_t launch_block_ranges(const PlanBlock* blocks, uint32_t nblocks, const float* sparse,
                                const uint64_t* node_off_dev, float2* scale_offset, cudaStream_t s);

// One block in any field mode (pres) sampled through the texture unit: field / field2 / tf_tex are
// cudaTextureObject_t handles (3-D float field arrays, 1-D RGBA transfer-function array).
cudaError_t launch_render_block_texture(const s3r_view* view_host, const s3r_presentation* pres, uint64_t field,
                                       uint64_t field2, uint64_t tf_tex, const RenderBlock& rb, uint32_t* viewport,
                                       cudaStream_t s);
cudaError_t launch_render_block_mode(const s3r_view* view_host, const s3r_presentation* pres, const float* brick,
                                     const float* brick2, const RenderBlock& rb, const float* tf, uint32_t* viewport,
                                     cudaStream_t s);
cudaError_t launch_render_block_argb(const s3r_view* view_host, const float* brick, const RenderBlock& rb,
                                     const float* tf, uint32_t* viewport, cudaStream_t s);
cudaError_t launch_frame_render(const FrameArgs& a, uint32_t W, uint32_t H, uint32_t tf_n, uint32_t fmt,
                                uint32_t tile_shape, uint32_t filter, cudaStream_t s);
// The block-major form: segment kernel (persistent grid of ctas CTAs, 0: as many as fit on sms SMs) over
// the work items of footprint `shape`, then the composite kernel over all W x H pixels.
cudaError_t launch_frame_segments(const FrameArgs& a, const SegArgs& sa, uint32_t W, uint32_t H, uint32_t tf_n,
                                  uint32_t fmt, uint32_t shape, uint32_t filter, uint32_t sms, cudaStream_t s);
cudaError_t launch_frame_render_mode(const FrameArgs& a, const s3r_presentation& pres, const float* bricks2,
                                     uint32_t W, uint32_t H, uint32_t tf_n, uint32_t filter, cudaStream_t s);
cudaError_t launch_frame_backward(const FrameArgs& a, uint32_t W, uint32_t H, uint32_t tf_n, cudaStream_t s);
// dtf[i] += sum over the kDtfParts copies of part[. * n + i], n = 4 * tf_n
cudaError_t launch_dtf_reduce(const float* part, float* dtf, uint32_t n, cudaStream_t s);

cudaError_t launch_bound_rect(const uint32_t* img, uint32_t W, uint32_t H, int32_t* rect_dev, cudaStream_t s);
cudaError_t launch_crop(const uint32_t* img, uint32_t W, const int32_t rect[4], uint32_t* dst, cudaStream_t s);
cudaError_t launch_compose(const s3r_image_part* parts_dev, uint32_t nparts, int32_t just_copy_first, uint32_t* dst,
                           int32_t dw, int32_t dh, int32_t offx, int32_t offy, cudaStream_t s);

// Render CTA pixel shapes the autotuner chooses from: {x, y} pixels.  A render
// tile id below kRenderWalkTiles is a per-ray walk (frame_render_kernel), shape +
// kRenderShapes * log2(lanes per ray), lanes per ray 1..8; the kSegShapes ids
// from kRenderWalkTiles up are the block-major form with item footprint
// kSegShapeX x kSegShapeY pixels.
constexpr int kRenderShapes = 4;
constexpr int kRenderWalkTiles = kRenderShapes * 4;
constexpr int kSegShapes = 3;
constexpr int kRenderTiles = kRenderWalkTiles + kSegShapes;
constexpr int kRenderShapeX[kRenderShapes] = {16, 32, 8, 16};
constexpr int kRenderShapeY[kRenderShapes] = {8, 4, 8, 16};
static_assert(kRenderWalkTiles == S3R_RENDER_TILES_WALK && kRenderTiles == S3R_RENDER_TILES, "render tile ids");
constexpr int kSegShapeX[kSegShapes] = {8, 16, 4}; // one warp's pixels
constexpr int kSegShapeY[kSegShapes] = {4, 2, 8};

} // namespace s3r
