// Host side of the s3r C ABI (include/s3r.h): contexts, argument checks,
// parameter set-up restated from the reference's host code, the batched
// plan (tile binning of the octree nodes), CUDA-graph capture of a frame and
// the tile-size / CTA-shape autotuner.  Built with -ffp-contract=off so that
// float set-up code rounds as written.
#include "s3r_internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace s3r;

namespace {

thread_local std::string g_last_error;

} // namespace

struct s3r_ctx {
    int device = 0;
    std::string err;
    float* grid = nullptr; // single-block interpolation scratch
    size_t grid_cap = 0;   // floats
    int32_t* rect_dev = nullptr;
    int32_t* rect_host = nullptr; // pinned
    s3r_image_part* parts_dev = nullptr;
    size_t parts_cap = 0;
    cudaStream_t capture = nullptr;
    float* worker_dense[2] = {nullptr, nullptr}; // s3r_render_scene_part: primary / secondary dense field
    size_t worker_cap[2] = {0, 0};
    // s3r_render_scene_part with the texture filter: per depth a primary / secondary field texture, the
    // transfer-function texture, and the linear grid s3r_interp_dense_texture interpolates into
    s3r_texture* worker_tex[2][S3R_MAX_DEPTH + 1] = {};
    s3r_tf_texture* worker_tf = nullptr;
    float* tex_stage = nullptr;
    size_t tex_stage_cap = 0;
    uint64_t launches = 0;
    int sms = 152;
};

// One captured frame (interpolation + render) and the arguments it was captured for.
struct FrameGraph {
    cudaGraphExec_t exec = nullptr;
    const void* key[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    uint32_t dims[4] = {0, 0, 0, 0}; // W, H, tf_n, filter the launches were sized for
    uint32_t kernels = 0;
};

struct s3r_plan {
    s3r_ctx* ctx = nullptr;
    s3r_frame_desc desc{};
    uint32_t nblocks = 0, level = 0, fmt = 0;
    uint32_t tile_log2 = 4;             // the largest tile edge (log2 cells) over the blocks
    uint8_t tile_by_depth[S3R_MAX_DEPTH + 1] = {}; // per block depth: its tile edge (log2), capped by the depth
    uint32_t render_tile = 0;
    std::vector<uint32_t> blocks;      // 4 per block
    std::vector<uint64_t> node_off;    // nblocks+1
    std::vector<uint16_t> n2i;         // host copy (re-binning by the autotuner)
    std::vector<uint64_t> vertex_off;  // nblocks+1
    uint64_t vertices = 0, nodes = 0, tiles = 0, entries = 0;
    uint64_t brick_elems = 0;          // elements of the brick store (rows padded to the pitch)
    std::vector<uint32_t> pitch;       // per block: brick row pitch in elements
    // device
    PlanBlock* blocks_dev = nullptr;
    uint2* items_dev = nullptr;
    uint64_t* entry_off_dev = nullptr;
    uint16_t* entry_local_dev = nullptr;
    uint32_t* entry_node_dev = nullptr;
    uint32_t* flags_dev = nullptr;
    uint32_t flag_words = 1;
    uint32_t* centry_off_dev = nullptr; // per block the sparse nodes on its coarse grid
    uint2* centry_dev = nullptr;
    float* coarse_dev[2] = {nullptr, nullptr}; // per data slot: the blocks' coarse grids of the frame
    bool any_coarse = false;
    uint32_t* queue_dev = nullptr;
    uint64_t* node_off_dev = nullptr;
    float2* scale_offset_dev = nullptr;
    // the second data slot of s3r_frame_run_host (slot 0 is the brick store above): its own bricks and
    // per-brick 16-bit scales, so that two frames can be on the GPU at once
    void* bricks_1 = nullptr;
    float2* scale_offset_1 = nullptr;
    void* bricks = nullptr;
    RenderBlock* table_dev = nullptr;
    s3r_view* view_dev = nullptr;
    int32_t* cover_dev = nullptr;    // union of the present blocks' view rectangles {x0, y0, x1, y1}
    int32_t* cover_pinned = nullptr;
    uint32_t grid_ctas = 0;
    // host render table (rects depend on the view)
    std::vector<RenderBlock> table_host;
    RenderBlock* table_pinned = nullptr;
    s3r_view* view_pinned = nullptr;
    cudaEvent_t staged = nullptr;
    bool have_view = false;
    s3r_view last_view{};
    // frame graphs: slot 0 for s3r_frame_run, slots 1 and 2 for the two buffers of s3r_frame_run_host
    FrameGraph graphs[3];
    float* dtf_part = nullptr; // adjoint: kDtfParts copies of the transfer-function gradient
    size_t dtf_part_floats = 0;
    // block-major render: the block cells deepest first, per item footprint the running tile counts over
    // them (staged with the view), per data slot the per-rank block results and rank masks, and one
    // work-queue counter per data slot
    std::vector<uint32_t> seg_order;
    uint2* seg_items_pinned = nullptr;  // {cell, tile} per warp work item, staged with the view
    uint2* seg_items_dev = nullptr;
    uint64_t seg_items_cap = 0, seg_items_dev_cap = 0;
    uint32_t* seg_count_pinned = nullptr;
    uint32_t* seg_count_dev = nullptr;  // items staged
    int seg_staged_shape = -1;          // the footprint the staged items are cut for
    uint32_t* seg_queue = nullptr;      // 2 counters
    float4* seg_buf[2] = {nullptr, nullptr};
    unsigned long long* seg_mask[2] = {nullptr, nullptr};
    uint64_t seg_pixels = 0;            // pixels the buffers hold
    uint32_t seg_words = 0;
    // s3r_frame_run_host: per slot a device copy of the frame's sparse values and its image, and the
    // streams and events that overlap frame k's copies with frames k-1 and k+1
    float* hs_sparse[2] = {nullptr, nullptr};
    uint32_t* hs_argb[2] = {nullptr, nullptr};
    float* hs_tf[2] = {nullptr, nullptr}; // per slot: the frame's transfer function, copied on the caller's stream
    uint32_t hs_tf_n = 0;
    uint64_t hs_pixels = 0;
    uint64_t hs_frames = 0;
    cudaStream_t hs_h2d = nullptr, hs_d2h = nullptr;
    cudaStream_t hs_comp[2] = {nullptr, nullptr}; // one compute stream per slot: frames k and k+1 overlap
    cudaEvent_t hs_copied[2] = {nullptr, nullptr}, hs_rendered[2] = {nullptr, nullptr}, hs_read[2] = {nullptr, nullptr};
    cudaEvent_t hs_entry = nullptr; // work queued on the caller's stream before a frame
};

// A block's dense field as the reference holds it for rendering (DeviceField, DenseFieldRenderer_cu.cu:503-560):
// a 3-D float array with a texture object over it (unnormalized coordinates, linear filtering, clamp).
struct s3r_texture {
    s3r_ctx* ctx = nullptr;
    uint32_t depth = 0, n = 0;
    cudaArray_t array = nullptr;
    cudaTextureObject_t tex = 0;
};

// The transfer function as the reference's colour texture (makeColorTransferTexture,
// DenseFieldRenderer_cu.cu:566-586): one row of RGBA floats, normalized coordinates, linear filtering,
// clamp along x.
struct s3r_tf_texture {
    s3r_ctx* ctx = nullptr;
    uint32_t n = 0;
    cudaArray_t array = nullptr;
    cudaTextureObject_t tex = 0;
};

void s3r::set_thread_error(const char* msg) { g_last_error = msg; }
void s3r::count_launches(s3r_ctx* ctx, uint32_t n)
{
    if (ctx) ctx->launches += n;
}

namespace {

int fail(s3r_ctx* ctx, int code, const std::string& msg)
{
    g_last_error = msg;
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_fail(s3r_ctx* ctx, cudaError_t e, const char* what)
{
    return fail(ctx, S3R_ERR_CUDA, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

#define S3R_CUDA(ctx, call)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int set_device(s3r_ctx* ctx)
{
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e == cudaSuccess && cur == ctx->device) return S3R_OK;
    e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
    return S3R_OK;
}

// ---------------------------------------------------------------- geometry

void block_cube_f(uint32_t level, const uint32_t idx[3], float c[3], float& h)
{
    const float top = 5.f;
    h = top / (float)(1u << level);
    for (int d = 0; d < 3; ++d)
        c[d] = -top + h * (float)(1u + (idx[d] << 1));
}

int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// DenseFieldRenderer_cu.cu:374-409: bounding box of the projected cube corners,
// truncated toward zero, clamped to the viewport; {x, y, w, h} with w = max - min.
void view_rect(const s3r_view& v, const uint32_t idx[3], int32_t rect[4])
{
    float c[3], h;
    block_cube_f(v.level, idx, c, h);
    const float lcam = 0.01f * 2 * 5.f;
    const float pixel = v.cam.h / (float)v.H;
    const float* r = v.cam.view_r;
    const float* t = v.cam.view_t;
    bool have = false, full = false;
    int xmin = 0, xmax = 0, ymin = 0, ymax = 0;
    for (int i = 0; i < 8; ++i) {
        float p[3];
        for (int d = 0; d < 3; ++d)
            p[d] = c[d] + (float)((int)(((i >> d) & 1) << 1) - 1) * h;
        float q[3];
        for (int a = 0; a < 3; ++a)
            q[a] = r[3 * a] * p[0] + r[3 * a + 1] * p[1] + r[3 * a + 2] * p[2] + t[a];
        int sx, sy;
        if (v.cam.ortho) {
            sx = clampi((int)(q[0] / pixel) + (int)(v.W >> 1), 0, (int)v.W - 1);
            sy = clampi((int)(q[1] / pixel) + (int)(v.H >> 1), 0, (int)v.H - 1);
        } else {
            if (q[2] >= 0) {
                full = true;
                break;
            }
            sx = clampi((int)(-q[0] / q[2] * lcam / pixel) + (int)(v.W >> 1), 0, (int)v.W - 1);
            sy = clampi((int)(-q[1] / q[2] * lcam / pixel) + (int)(v.H >> 1), 0, (int)v.H - 1);
        }
        if (!have) {
            xmin = xmax = sx;
            ymin = ymax = sy;
            have = true;
        } else {
            xmin = std::min(xmin, sx);
            xmax = std::max(xmax, sx);
            ymin = std::min(ymin, sy);
            ymax = std::max(ymax, sy);
        }
    }
    if (full) {
        // a corner behind the eye: the whole viewport (bb << {0,0} << viewportSize)
        xmin = ymin = 0;
        xmax = (int)v.W;
        ymax = (int)v.H;
    }
    rect[0] = xmin;
    rect[1] = ymin;
    rect[2] = xmax - xmin;
    rect[3] = ymax - ymin;
}

int check_view(s3r_ctx* ctx, const s3r_view* v)
{
    if (!v) return fail(ctx, S3R_ERR_INVALID, "view is null");
    if (v->W == 0 || v->H == 0 || v->W > 32768 || v->H > 32768)
        return fail(ctx, S3R_ERR_INVALID, "viewport size out of range");
    if (v->tf_n < 2 || v->tf_n > 4096) return fail(ctx, S3R_ERR_INVALID, "tf_n must be in [2, 4096]");
    if (v->level > 12) return fail(ctx, S3R_ERR_INVALID, "level out of range");
    if (!(v->field_max > v->field_min)) return fail(ctx, S3R_ERR_INVALID, "field range is empty");
    if (!(v->quality > 0.f)) return fail(ctx, S3R_ERR_INVALID, "quality must be positive");
    if (v->filter != S3R_FILTER_EXACT && v->filter != S3R_FILTER_TEXTURE)
        return fail(ctx, S3R_ERR_INVALID, "unknown filter");
    return S3R_OK;
}

// ---------------------------------------------------------------- ordering

// Split of one index range by one eye coordinate (UniformIndexRangeSplitter,
// include/UniformIndexRangeSplitter.hpp:27-57), in the reference's float type.
struct Split {
    uint32_t before[2];
    uint32_t at; // ~0u: none
    uint32_t after[2];
};

Split split_range(uint32_t lo, uint32_t hi, float c0, float c1, float x)
{
    Split s;
    if (x <= c0) {
        s.before[0] = s.before[1] = 0;
        s.at = ~0u;
        s.after[0] = lo;
        s.after[1] = hi;
        return s;
    }
    if (x >= c1) {
        s.before[0] = lo;
        s.before[1] = hi;
        s.at = ~0u;
        s.after[0] = s.after[1] = 0;
        return s;
    }
    const float factor = (float)(hi - lo) / (c1 - c0);
    const uint32_t at = (uint32_t)((x - c0) * factor) + lo;
    s.before[0] = lo;
    s.before[1] = at;
    s.at = at;
    s.after[0] = at + 1;
    s.after[1] = hi;
    return s;
}

// Split of the box index range [0, n) by one eye coordinate when the boxes' boundaries sit at coords[0..n]
// (NonUniformIndexRangeSplitter, include/NonUniformIndexRangeSplitter.hpp:27-56): the first boundary not below
// x decides, so an eye exactly on a boundary belongs to the box before it.
Split split_boundaries(const float* coords, uint32_t n, float x)
{
    const float* it = std::lower_bound(coords, coords + n + 1, x);
    Split s;
    if (it == coords) {
        s.before[0] = s.before[1] = 0;
        s.at = ~0u;
        s.after[0] = 0;
        s.after[1] = n;
    } else if (it == coords + n + 1) {
        s.before[0] = 0;
        s.before[1] = n;
        s.at = ~0u;
        s.after[0] = s.after[1] = 0;
    } else {
        const uint32_t at = (uint32_t)(it - coords) - 1;
        s.before[0] = 0;
        s.before[1] = at;
        s.at = at;
        s.after[0] = at + 1;
        s.after[1] = n;
    }
    return s;
}

// Macro-block visiting order: the 27 cells of the 3x3x3 split (0 = before the
// eye, 1 = at it, 2 = beyond it per axis) taken corners first, then edges,
// faces and the eye's own cell (include/BackToFrontOrder.hpp:182-209).
constexpr uint8_t kMacroOrder[27] = {0, 2, 6, 8, 18, 20, 24, 26, 1, 3, 5, 7, 9, 11,
                                     15, 17, 19, 21, 23, 25, 4, 10, 12, 14, 16, 22, 13};

// Inside one macro block: anti-diagonal sweeps of increasing coordinate sum,
// the same successor rule as include/BackToFrontOrder.hpp:246-307 (unsigned
// arithmetic kept), mirrored on axes beyond the eye.
bool next_in_box(uint32_t p[3], const uint32_t mn[3], const uint32_t mx[3])
{
    uint32_t s = p[0] + p[1] + p[2];
    if (s + 3 == mx[0] + mx[1] + mx[2]) return false;
    if (p[0] > mn[0] && p[1] + 1 < mx[1]) {
        --p[0];
        ++p[1];
    } else if (p[0] + p[1] > mn[0] + mn[1] && p[2] + 1 < mx[2]) {
        if (s - mn[1] - p[2] < mx[0] + 1) {
            p[0] = s - mn[1] - p[2] - 1;
            p[1] = mn[1];
            p[2] = p[2] + 1;
        } else {
            p[0] = mx[0] - 1;
            p[1] = s - mx[0] - p[2];
            p[2] = p[2] + 1;
        }
    } else {
        ++s;
        const uint32_t x0 = s - mn[1] - mn[2];
        if (x0 < mx[0]) {
            p[0] = x0;
            p[1] = mn[1];
            p[2] = mn[2];
        } else {
            const uint32_t x1 = s - mx[0] + 1 - mn[2];
            if (x1 < mx[1]) {
                p[0] = mx[0] - 1;
                p[1] = x1;
                p[2] = mn[2];
            } else {
                p[0] = mx[0] - 1;
                p[1] = mx[1] - 1;
                p[2] = s + 2 - mx[0] - mx[1];
            }
        }
    }
    return true;
}

// Visits a 3-D index grid in back-to-front order for the per-axis splits of
// the eye (BackToFrontOrder::iterator, include/BackToFrontOrder.hpp:79-320):
// macro blocks in kMacroOrder, inside each the anti-diagonal sweep, mirrored on
// axes beyond the eye.  f(pos) gets each index triple.
template <class F> void b2f_traverse(const Split sp[3], F&& f)
{
    for (uint8_t ord : kMacroOrder) {
        const uint32_t mp[3] = {ord % 3u, (ord / 3u) % 3u, ord / 9u};
        uint32_t mn[3], mx[3];
        bool valid = true;
        for (int a = 0; a < 3; ++a) {
            const Split& s = sp[a];
            if (mp[a] == 0) {
                mn[a] = s.before[0];
                mx[a] = s.before[1];
                valid &= s.before[0] != s.before[1];
            } else if (mp[a] == 1) {
                mn[a] = s.at;
                mx[a] = s.at + 1;
                valid &= s.at != ~0u;
            } else {
                mn[a] = s.after[0];
                mx[a] = s.after[1];
                valid &= s.after[0] != s.after[1];
            }
        }
        if (!valid) continue;
        uint32_t p[3] = {mn[0], mn[1], mn[2]};
        do {
            uint32_t q[3];
            for (int a = 0; a < 3; ++a) q[a] = mp[a] == 2 ? mx[a] - 1 + mn[a] - p[a] : p[a];
            f(q);
        } while (next_in_box(p, mn, mx));
    }
}

// IndexCubeSplitter<3> (include/IndexCubeSplitter.hpp:36-196) over the world cube [-5, 5]^3: per axis the
// number of slabs (split_count taken greedily along x, then y, then z, each at most 2^level) and their
// index boundaries i*size/slabs and world boundaries (the float formula of init_axis_split).
struct CubeSplit {
    uint32_t n[3];
    std::vector<uint32_t> idx[3];
    std::vector<float> coord[3];
};

CubeSplit cube_split(uint32_t level, uint32_t split_count)
{
    CubeSplit cs;
    const uint32_t size = 1u << level;
    const uint64_t max_split = 1ull << (3 * level);
    uint32_t count = (uint32_t)std::min<uint64_t>(max_split, split_count);
    for (int a = 0; a < 3; ++a) {
        if (count <= size) {
            cs.n[a] = count;
            count = 1;
        } else {
            cs.n[a] = size;
            count = std::max(1u, count / size);
        }
    }
    const float origin = -5.f, length = 10.f;
    for (int a = 0; a < 3; ++a) {
        const uint32_t k = cs.n[a];
        cs.idx[a].assign(k + 1, 0);
        cs.coord[a].assign(k + 1, 0.f);
        cs.idx[a][k] = size;
        cs.coord[a][0] = origin;
        cs.coord[a][k] = origin + length;
        for (uint32_t i = 1; i < k; ++i) {
            const uint32_t si = (uint32_t)((uint64_t)i * size / k);
            cs.idx[a][i] = si;
            cs.coord[a][i] = origin + length * (float)si / (float)size;
        }
    }
    return cs;
}

void put_box(const CubeSplit& cs, const uint32_t q[3], uint32_t* out)
{
    for (int a = 0; a < 3; ++a) {
        out[a] = cs.idx[a][q[a]];
        out[3 + a] = cs.idx[a][q[a] + 1];
    }
}

// ---------------------------------------------------------------- plan

void plan_free_device(s3r_plan* p)
{
    auto f = [](void* q) {
        if (q) cudaFree(q);
    };
    f(p->blocks_dev);
    f(p->items_dev);
    f(p->entry_off_dev);
    f(p->entry_local_dev);
    f(p->entry_node_dev);
    f(p->flags_dev);
    f(p->centry_off_dev);
    f(p->centry_dev);
    f(p->coarse_dev[0]);
    f(p->coarse_dev[1]);
    p->centry_off_dev = nullptr;
    p->centry_dev = nullptr;
    p->coarse_dev[0] = p->coarse_dev[1] = nullptr;
    p->blocks_dev = nullptr;
    p->items_dev = nullptr;
    p->entry_off_dev = nullptr;
    p->entry_local_dev = nullptr;
    p->entry_node_dev = nullptr;
    p->flags_dev = nullptr;
}

void plan_drop_graph(s3r_plan* p)
{
    for (auto& g : p->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = FrameGraph{};
    }
}

template <class T> int upload(s3r_ctx* ctx, T** dst, const std::vector<T>& src)
{
    const size_t bytes = std::max<size_t>(src.size(), 1) * sizeof(T);
    cudaError_t e = cudaMalloc(dst, bytes);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(plan)");
    if (!src.empty()) {
        e = cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpy(plan)");
    }
    return S3R_OK;
}

// Bins every block's nodes by tile of 2^tile_log2 cells (closed tiles: nodes on
// shared faces, edges and corners go to every tile containing them; in a block
// of several tiles the lattice points of the tile grid go to the block's coarse
// grid instead, whose values every frame computes once per block), lists the
// coarse-grid nodes and the work items (largest tiles first), and uploads them.
// by_depth: per block depth the tile edge (log2 cells) of that depth's blocks; NULL: tile_log2 for all.
int plan_bin(s3r_plan* p, uint32_t tile_log2, const uint8_t* by_depth = nullptr)
{
    s3r_ctx* ctx = p->ctx;
    const uint32_t nb = p->nblocks;
    std::vector<PlanBlock> pb(nb);
    std::vector<uint64_t> tiles_off(nb + 1, 0), coarse_off(nb + 1, 0);
    uint8_t tl_of[S3R_MAX_DEPTH + 1];
    for (uint32_t d = 0; d <= S3R_MAX_DEPTH; ++d)
        tl_of[d] = (uint8_t)std::min<uint32_t>(by_depth ? by_depth[d] : tile_log2, d);
    tile_log2 = 0;
    for (uint32_t b = 0; b < nb; ++b) tile_log2 = std::max<uint32_t>(tile_log2, tl_of[p->blocks[4 * b + 3]]);
    for (uint32_t b = 0; b < nb; ++b) {
        const uint32_t d = p->blocks[4 * b + 3];
        const uint32_t k = tl_of[d];
        const uint32_t L = d - k;
        pb[b].depth = d;
        pb[b].tile_log2 = k;
        pb[b].coarse_log2 = L;
        pb[b].node_base = p->node_off[b];
        pb[b].dense_off = p->vertex_off[b];
        pb[b].pitch = p->pitch[b];
        const uint64_t m = 1ull << L;
        tiles_off[b + 1] = tiles_off[b] + m * m * m;
        coarse_off[b + 1] = coarse_off[b] + (m + 1) * (m + 1) * (m + 1);
    }
    if (coarse_off[nb] > 0xffffffffull) return fail(ctx, S3R_ERR_INVALID, "coarse grids too large");
    for (uint32_t b = 0; b < nb; ++b) pb[b].coarse_off = (uint32_t)coarse_off[b];
    const uint64_t ntiles = tiles_off[nb];
    std::vector<int32_t> coarse(coarse_off[nb], -1);
    std::vector<uint64_t> count(ntiles + 1, 0);

    const unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    auto parallel = [&](auto&& fn) {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nthreads; ++t)
            th.emplace_back([&, t] {
                for (uint32_t b = t; b < nb; b += nthreads) fn(b);
            });
        for (auto& x : th) x.join();
    };
    auto tile_span = [](uint32_t x, uint32_t T, uint32_t m, uint32_t& lo, uint32_t& hi) {
        lo = x == 0 ? 0 : (x - 1) / T;
        hi = std::min(x / T, m - 1);
    };
    // pass 1: counts and coarse grids
    parallel([&](uint32_t b) {
        const PlanBlock& B = pb[b];
        const uint32_t T = 1u << B.tile_log2, m = 1u << B.coarse_log2, m1 = m + 1;
        for (uint64_t i = p->node_off[b]; i < p->node_off[b + 1]; ++i) {
            const uint32_t x = p->n2i[3 * i], y = p->n2i[3 * i + 1], z = p->n2i[3 * i + 2];
            const bool lattice = (x % T == 0) && (y % T == 0) && (z % T == 0);
            if (lattice) coarse[B.coarse_off + (x / T) + m1 * ((y / T) + m1 * (z / T))] = (int32_t)(i - p->node_off[b]);
            if (lattice && B.coarse_log2 > 0) continue;
            uint32_t xl, xh, yl, yh, zl, zh;
            tile_span(x, T, m, xl, xh);
            tile_span(y, T, m, yl, yh);
            tile_span(z, T, m, zl, zh);
            for (uint32_t tz = zl; tz <= zh; ++tz)
                for (uint32_t ty = yl; ty <= yh; ++ty)
                    for (uint32_t tx = xl; tx <= xh; ++tx)
                        ++count[tiles_off[b] + tx + m * (ty + m * tz)];
        }
    });
    // items: largest tiles first, then block order
    std::vector<uint64_t> order(ntiles);
    {
        std::vector<uint32_t> bord(nb);
        for (uint32_t b = 0; b < nb; ++b) bord[b] = b;
        std::stable_sort(bord.begin(), bord.end(),
                         [&](uint32_t a, uint32_t c) { return pb[a].tile_log2 > pb[c].tile_log2; });
        uint64_t o = 0;
        for (uint32_t b : bord)
            for (uint64_t t = tiles_off[b]; t < tiles_off[b + 1]; ++t) order[o++] = t;
    }
    std::vector<uint2> items(ntiles);
    std::vector<uint64_t> entry_off(ntiles + 1, 0);
    std::vector<uint64_t> slot(ntiles); // tile (block-major) -> item position
    std::vector<uint32_t> tile_block(ntiles);
    for (uint32_t b = 0; b < nb; ++b)
        for (uint64_t t = tiles_off[b]; t < tiles_off[b + 1]; ++t) tile_block[t] = b;
    for (uint64_t it = 0; it < ntiles; ++it) {
        const uint64_t t = order[it];
        slot[t] = it;
        const uint32_t b = tile_block[t];
        items[it] = make_uint2(b, (uint32_t)(t - tiles_off[b]));
        entry_off[it + 1] = entry_off[it] + count[t];
    }
    const uint64_t nentries = entry_off[ntiles];
    if (nentries > 0xffffffffull) return fail(ctx, S3R_ERR_INVALID, "too many tile entries (2^32 or more)");
    std::vector<uint16_t> local(nentries);
    std::vector<uint32_t> node(nentries);
    // per item: one bit per finest 2x2x2 cube of the tile, set when one of the cube's midpoints holds
    // a node (the cube along each odd axis of the node, both neighbours along each even one)
    const uint32_t hmax = std::max(1u, (1u << tile_log2) / 2);
    const uint32_t fwords = std::max(1u, (hmax * hmax * hmax + 31) / 32);
    std::vector<uint32_t> flags(ntiles * fwords, 0u);
    auto flag_node = [&](uint32_t* f, uint32_t H, uint32_t x, uint32_t y, uint32_t z) {
        if (!((x | y | z) & 1)) return;
        auto span = [H](uint32_t v, uint32_t& lo, uint32_t& hi) {
            if (v & 1) {
                lo = hi = v >> 1;
            } else {
                lo = v ? (v >> 1) - 1 : 0;
                hi = std::min(v >> 1, H - 1);
            }
        };
        uint32_t x0, x1, y0, y1, z0, z1;
        span(x, x0, x1);
        span(y, y0, y1);
        span(z, z0, z1);
        for (uint32_t k = z0; k <= z1; ++k)
            for (uint32_t j = y0; j <= y1; ++j)
                for (uint32_t i = x0; i <= x1; ++i) {
                    const uint32_t c = i + H * (j + H * k);
                    f[c >> 5] |= 1u << (c & 31);
                }
    };
    std::vector<uint64_t> cursor(ntiles);
    for (uint64_t t = 0; t < ntiles; ++t) cursor[t] = entry_off[slot[t]];
    // pass 2: fill (tiles of one block are only touched by that block's thread)
    parallel([&](uint32_t b) {
        const PlanBlock& B = pb[b];
        const uint32_t T = 1u << B.tile_log2, m = 1u << B.coarse_log2, E = T + 1;
        for (uint64_t i = p->node_off[b]; i < p->node_off[b + 1]; ++i) {
            const uint32_t x = p->n2i[3 * i], y = p->n2i[3 * i + 1], z = p->n2i[3 * i + 2];
            const bool lattice = (x % T == 0) && (y % T == 0) && (z % T == 0);
            if (lattice && B.coarse_log2 > 0) continue;
            uint32_t xl, xh, yl, yh, zl, zh;
            tile_span(x, T, m, xl, xh);
            tile_span(y, T, m, yl, yh);
            tile_span(z, T, m, zl, zh);
            for (uint32_t tz = zl; tz <= zh; ++tz)
                for (uint32_t ty = yl; ty <= yh; ++ty)
                    for (uint32_t tx = xl; tx <= xh; ++tx) {
                        const uint64_t t = tiles_off[b] + tx + m * (ty + m * tz);
                        const uint64_t e = cursor[t]++;
                        local[e] = (uint16_t)tile_offset(T, x - tx * T, y - ty * T, z - tz * T);
                        node[e] = (uint32_t)(i - p->node_off[b]);
                        if (T >= 2)
                            flag_node(&flags[slot[t] * fwords], T / 2, x - tx * T, y - ty * T, z - tz * T);
                    }
        }
        (void)E;
    });
    // the nodes on every block's coarse grid (the lattice of tile corners), once per block: the frame's
    // block_prep_kernel fills the coarse grids from them
    std::vector<uint32_t> centry_off(nb + 1, 0);
    std::vector<uint2> centry;
    for (uint32_t b = 0; b < nb; ++b) {
        if (pb[b].coarse_log2 > 0) {
            const uint64_t n = coarse_off[b + 1] - coarse_off[b];
            for (uint64_t q = 0; q < n; ++q) {
                const int32_t nd = coarse[coarse_off[b] + q];
                if (nd >= 0) centry.push_back(make_uint2((uint32_t)q, (uint32_t)nd));
            }
        }
        if (centry.size() > 0xffffffffull) return fail(ctx, S3R_ERR_INVALID, "too many coarse-grid nodes");
        centry_off[b + 1] = (uint32_t)centry.size();
    }
    // items whose tile holds no node at an odd position have no flagged cube, so nothing reads their
    // midpoint slots: the top bit of the tile field says "fill the slots"
    for (uint64_t it = 0; it < ntiles; ++it)
        for (uint32_t w = 0; w < fwords; ++w)
            if (flags[it * fwords + w]) {
                items[it].y |= 0x80000000u;
                break;
            }
    plan_free_device(p);
    int rc;
    if ((rc = upload(ctx, &p->blocks_dev, pb))) return rc;
    if ((rc = upload(ctx, &p->items_dev, items))) return rc;
    if ((rc = upload(ctx, &p->entry_off_dev, entry_off))) return rc;
    if ((rc = upload(ctx, &p->entry_local_dev, local))) return rc;
    if ((rc = upload(ctx, &p->entry_node_dev, node))) return rc;
    if ((rc = upload(ctx, &p->flags_dev, flags))) return rc;
    if ((rc = upload(ctx, &p->centry_off_dev, centry_off))) return rc;
    if ((rc = upload(ctx, &p->centry_dev, centry))) return rc;
    p->any_coarse = false;
    for (uint32_t b = 0; b < nb; ++b) p->any_coarse |= pb[b].coarse_log2 > 0;
    for (int q = 0; q < 2; ++q) {
        cudaError_t e = cudaMalloc(&p->coarse_dev[q], std::max<uint64_t>(coarse_off[nb], 1) * sizeof(float));
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(coarse grids)");
    }
    p->flag_words = fwords;
    p->tile_log2 = tile_log2;
    std::memcpy(p->tile_by_depth, tl_of, sizeof(tl_of));
    p->tiles = ntiles;
    p->entries = nentries;
    // persistent grid: the CTAs that fit on every SM at once, fed by the work queue
    const uint32_t per_sm = interp_plan_ctas_per_sm(p->fmt, tile_log2);
    p->grid_ctas = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(ntiles, (uint64_t)ctx->sms * per_sm));
    plan_drop_graph(p);
    return S3R_OK;
}

// The block-major render's per-rank results and rank masks for W x H pixels, in both data slots; called
// before a frame is launched (or captured) with a block-major render tile.  Reallocation drops the captured
// frames (they hold the old buffers).
void plan_free_segments(s3r_plan* p)
{
    for (int b = 0; b < 2; ++b) {
        if (p->seg_buf[b]) cudaFree(p->seg_buf[b]);
        if (p->seg_mask[b]) cudaFree(p->seg_mask[b]);
        p->seg_buf[b] = nullptr;
        p->seg_mask[b] = nullptr;
    }
    p->seg_pixels = 0;
}

int plan_ensure_segments(s3r_plan* p, uint32_t W, uint32_t H)
{
    if (p->render_tile < (uint32_t)kRenderWalkTiles) return S3R_OK;
    s3r_ctx* ctx = p->ctx;
    const uint64_t npix = (uint64_t)W * H;
    const uint32_t m = 1u << p->level;
    const uint32_t words = (3 * m - 2 + 63) / 64;
    if (words > kSegMaskWords)
        return fail(ctx, S3R_ERR_UNSUPPORTED, "the block-major render covers levels up to 7");
    if (p->seg_buf[0] && p->seg_pixels >= npix && p->seg_words == words) return S3R_OK;
    S3R_CUDA(ctx, cudaDeviceSynchronize());
    plan_free_segments(p);
    plan_drop_graph(p);
    for (int b = 0; b < 2; ++b) {
        cudaError_t e;
        if ((e = cudaMalloc(&p->seg_buf[b], (size_t)(3 * m - 2) * npix * sizeof(float4))) != cudaSuccess ||
            (e = cudaMalloc(&p->seg_mask[b], (size_t)words * npix * sizeof(unsigned long long))) != cudaSuccess ||
            (e = cudaMemset(p->seg_mask[b], 0, (size_t)words * npix * sizeof(unsigned long long))) != cudaSuccess) {
            plan_free_segments(p);
            (void)cudaGetLastError(); // an allocation failure leaves no error behind for later launches
            return cuda_fail(ctx, e, "cudaMalloc(block-major render buffers)");
        }
    }
    S3R_CUDA(ctx, cudaDeviceSynchronize());
    p->seg_pixels = npix;
    p->seg_words = words;
    return S3R_OK;
}

int plan_stage_view(s3r_plan* p, const s3r_view* view, cudaStream_t s)
{
    s3r_ctx* ctx = p->ctx;
    if (int rc = plan_ensure_segments(p, view->W, view->H)) return rc;
    const bool seg = p->render_tile >= (uint32_t)kRenderWalkTiles;
    const bool same = p->have_view && std::memcmp(&p->last_view, view, sizeof(s3r_view)) == 0 &&
                      (!seg || p->seg_staged_shape == (int)(p->render_tile - (uint32_t)kRenderWalkTiles));
    if (same) return S3R_OK;
    // the staging buffers may still feed an earlier copy
    S3R_CUDA(ctx, cudaEventSynchronize(p->staged));
    const uint32_t m = 1u << p->level;
    RenderBlock* tb = p->table_pinned;
    std::memcpy(tb, p->table_host.data(), sizeof(RenderBlock) * p->table_host.size());
    int32_t cover[4] = {INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN};
    for (uint32_t b = 0; b < p->nblocks; ++b) {
        const uint32_t* bl = &p->blocks[4 * b];
        const uint32_t cell = bl[0] + m * (bl[1] + m * bl[2]);
        int32_t* r = tb[cell].rect;
        view_rect(*view, bl, r);
        if (r[2] > 0 && r[3] > 0) {
            cover[0] = std::min(cover[0], r[0]);
            cover[1] = std::min(cover[1], r[1]);
            cover[2] = std::max(cover[2], r[0] + r[2]);
            cover[3] = std::max(cover[3], r[1] + r[3]);
        }
    }
    if (cover[0] > cover[2]) cover[0] = cover[1] = cover[2] = cover[3] = 0;
    // block-major render: the warp-sized tiles of every block's view rectangle, deepest blocks first
    if (p->render_tile >= (uint32_t)kRenderWalkTiles) {
        const int f = (int)(p->render_tile - (uint32_t)kRenderWalkTiles);
        const int fx = kSegShapeX[f], fy = kSegShapeY[f];
        uint64_t n = 0;
        for (uint32_t i = 0; i < p->nblocks; ++i) {
            const int32_t* r = tb[p->seg_order[i]].rect;
            if (r[2] > 0 && r[3] > 0) n += (uint64_t)((r[2] + fx - 1) / fx) * ((r[3] + fy - 1) / fy);
        }
        if (n > 0xffffffffull) return fail(ctx, S3R_ERR_INVALID, "too many block-major render items");
        cudaError_t e;
        if (n > p->seg_items_cap) {
            if (p->seg_items_pinned) cudaFreeHost(p->seg_items_pinned);
            p->seg_items_pinned = nullptr;
            p->seg_items_cap = 0;
            if ((e = cudaMallocHost(&p->seg_items_pinned, n * sizeof(uint2))) != cudaSuccess)
                return cuda_fail(ctx, e, "cudaMallocHost(block-major items)");
            p->seg_items_cap = n;
        }
        if (n > p->seg_items_dev_cap) {
            // frames in flight or captured may hold the old list
            S3R_CUDA(ctx, cudaDeviceSynchronize());
            plan_drop_graph(p);
            if (p->seg_items_dev) cudaFree(p->seg_items_dev);
            p->seg_items_dev = nullptr;
            p->seg_items_dev_cap = 0;
            if ((e = cudaMalloc(&p->seg_items_dev, n * sizeof(uint2))) != cudaSuccess)
                return cuda_fail(ctx, e, "cudaMalloc(block-major items)");
            p->seg_items_dev_cap = n;
        }
        uint2* it = p->seg_items_pinned;
        for (uint32_t i = 0; i < p->nblocks; ++i) {
            const uint32_t cell = p->seg_order[i];
            const int32_t* r = tb[cell].rect;
            if (r[2] <= 0 || r[3] <= 0) continue;
            const uint32_t tiles = (uint32_t)(((r[2] + fx - 1) / fx) * ((r[3] + fy - 1) / fy));
            for (uint32_t t = 0; t < tiles; ++t) *it++ = make_uint2(cell, t);
        }
        *p->seg_count_pinned = (uint32_t)n;
        if (n) S3R_CUDA(ctx, cudaMemcpyAsync(p->seg_items_dev, p->seg_items_pinned, n * sizeof(uint2),
                                             cudaMemcpyHostToDevice, s));
        S3R_CUDA(ctx, cudaMemcpyAsync(p->seg_count_dev, p->seg_count_pinned, sizeof(uint32_t), cudaMemcpyHostToDevice,
                                      s));
        p->seg_staged_shape = f;
    }
    std::memcpy(p->cover_pinned, cover, sizeof(cover));
    S3R_CUDA(ctx, cudaMemcpyAsync(p->cover_dev, p->cover_pinned, sizeof(cover), cudaMemcpyHostToDevice, s));
    *p->view_pinned = *view;
    S3R_CUDA(ctx, cudaMemcpyAsync(p->table_dev, tb, sizeof(RenderBlock) * p->table_host.size(),
                                  cudaMemcpyHostToDevice, s));
    S3R_CUDA(ctx, cudaMemcpyAsync(p->view_dev, p->view_pinned, sizeof(s3r_view), cudaMemcpyHostToDevice, s));
    S3R_CUDA(ctx, cudaEventRecord(p->staged, s));
    p->last_view = *view;
    p->have_view = true;
    return S3R_OK;
}

// slot 1: the second data slot of the host-buffer pipeline (its bricks, scales and work-queue counter)
int plan_launch_interp(s3r_plan* p, const float* sparse, cudaStream_t s, uint32_t* kernels, int slot = 0)
{
    s3r_ctx* ctx = p->ctx;
    float2* so = slot ? p->scale_offset_1 : p->scale_offset_dev;
    if (p->fmt != S3R_BRICK_F32 || p->any_coarse) {
        // 16-bit scales and coarse grids
        PrepArgs pa{};
        pa.blocks = p->blocks_dev;
        pa.node_off = p->node_off_dev;
        pa.sparse = sparse;
        pa.scale_offset = p->fmt != S3R_BRICK_F32 ? so : nullptr;
        pa.coarse = p->coarse_dev[slot ? 1 : 0];
        pa.centry_off = p->centry_off_dev;
        pa.centry = p->centry_dev;
        S3R_CUDA(ctx, launch_block_prep(pa, p->nblocks, s));
        ++*kernels;
    }
    TileArgs a{};
    a.blocks = p->blocks_dev;
    a.items = p->items_dev;
    a.nitems = (uint32_t)p->tiles;
    a.entry_off = p->entry_off_dev;
    a.entry_local = p->entry_local_dev;
    a.entry_node = p->entry_node_dev;
    a.flags = p->flags_dev;
    a.flag_words = p->flag_words;
    a.sparse = sparse;
    a.queue = p->queue_dev + slot;
    a.scale_offset = p->fmt == S3R_BRICK_F32 ? nullptr : so;
    a.coarse = p->coarse_dev[slot ? 1 : 0];
    a.out = slot ? p->bricks_1 : p->bricks;
    S3R_CUDA(ctx, cudaMemsetAsync(a.queue, 0, sizeof(uint32_t), s));
    S3R_CUDA(ctx, launch_interp_plan(a, p->fmt, p->tile_log2, p->grid_ctas, s));
    ++*kernels;
    return S3R_OK;
}

int plan_launch_render(s3r_plan* p, const float* tf, float* rgba, uint32_t* argb, unsigned long long* samples,
                       cudaStream_t s, uint32_t* kernels, int slot = 0)
{
    FrameArgs fa{};
    fa.view = p->view_dev;
    fa.table = p->table_dev;
    fa.bricks = slot ? p->bricks_1 : p->bricks;
    fa.tf = tf;
    fa.rgba = rgba;
    fa.argb = argb;
    fa.samples = samples;
    fa.scale_offset = p->fmt == S3R_BRICK_F32 ? nullptr : (slot ? p->scale_offset_1 : p->scale_offset_dev);
    fa.cover = p->cover_dev;
    if (p->render_tile >= (uint32_t)kRenderWalkTiles) {
        const int data = slot ? 1 : 0;
        if (!p->seg_buf[data] || p->seg_pixels < (uint64_t)p->last_view.W * p->last_view.H)
            return fail(p->ctx, S3R_ERR_INVALID, "block-major render buffers not allocated for this view");
        const uint32_t shape = p->render_tile - (uint32_t)kRenderWalkTiles;
        SegArgs sa{};
        if (p->seg_staged_shape != (int)shape || !p->seg_items_dev)
            return fail(p->ctx, S3R_ERR_INVALID, "block-major render items not staged for this render tile");
        sa.items = p->seg_items_dev;
        sa.count = p->seg_count_dev;
        sa.words = p->seg_words;
        sa.seg = p->seg_buf[data];
        sa.mask = p->seg_mask[data];
        sa.queue = p->seg_queue + data;
        S3R_CUDA(p->ctx, launch_frame_segments(fa, sa, p->last_view.W, p->last_view.H, p->last_view.tf_n, p->fmt, shape,
                                               p->last_view.filter, (uint32_t)p->ctx->sms, s));
        *kernels += 2;
        return S3R_OK;
    }
    S3R_CUDA(p->ctx, launch_frame_render(fa, p->last_view.W, p->last_view.H, p->last_view.tf_n, p->fmt,
                                         p->render_tile, p->last_view.filter, s));
    ++*kernels;
    return S3R_OK;
}

} // namespace

void s3r::block_sampling(uint32_t level, const uint32_t idx[3], uint32_t depth, RenderBlock& rb)
{
    block_cube_f(level, idx, rb.center, rb.half);
    const uint32_t n = (1u << depth) + 1u;
    rb.depth = depth;
    rb.texel = 2 * rb.half / (float)n;
    const double thalf = (double)rb.half + 0.5 * (double)rb.texel;
    for (int d = 0; d < 3; ++d) rb.origin[d] = rb.center[d] - (float)thalf;
    rb.factor = (float)((double)n / (2 * thalf));
}

int s3r::record_error(int code, const char* msg) { return fail(nullptr, code, msg); }

int s3r::record_cuda_error(cudaError_t e, const char* what) { return cuda_fail(nullptr, e, what); }

// ==================================================================== C ABI

extern "C" {

int s3r_abi_version(void) { return S3R_ABI_VERSION; }

const char* s3r_last_error(const s3r_ctx* ctx) { return ctx ? ctx->err.c_str() : g_last_error.c_str(); }

uint64_t s3r_ctx_launch_count(const s3r_ctx* ctx) { return ctx ? ctx->launches : 0; }

int s3r_ctx_create(int device, s3r_ctx** out)
{
    if (!out) return fail(nullptr, S3R_ERR_INVALID, "out is null");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDeviceCount");
    if (device < 0 || device >= n) return fail(nullptr, S3R_ERR_INVALID, "no such device");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
    s3r_ctx* c = new (std::nothrow) s3r_ctx;
    if (!c) return fail(nullptr, S3R_ERR_NOMEM, "out of host memory");
    c->device = device;
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if ((e = cudaMalloc(&c->rect_dev, 4 * sizeof(int32_t))) != cudaSuccess ||
        (e = cudaMallocHost(&c->rect_host, 4 * sizeof(int32_t))) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&c->capture, cudaStreamNonBlocking)) != cudaSuccess) {
        s3r_ctx_destroy(c);
        return cuda_fail(nullptr, e, "context allocation");
    }
    *out = c;
    return S3R_OK;
}

int s3r_ctx_destroy(s3r_ctx* ctx)
{
    if (!ctx) return S3R_OK;
    cudaSetDevice(ctx->device);
    if (ctx->grid) cudaFree(ctx->grid);
    if (ctx->rect_dev) cudaFree(ctx->rect_dev);
    if (ctx->rect_host) cudaFreeHost(ctx->rect_host);
    if (ctx->parts_dev) cudaFree(ctx->parts_dev);
    if (ctx->capture) cudaStreamDestroy(ctx->capture);
    for (float* d : ctx->worker_dense)
        if (d) cudaFree(d);
    for (auto& per_field : ctx->worker_tex)
        for (s3r_texture* t : per_field) s3r_texture_destroy(t);
    s3r_tf_texture_destroy(ctx->worker_tf);
    if (ctx->tex_stage) cudaFree(ctx->tex_stage);
    delete ctx;
    return S3R_OK;
}

int s3r_interp_dense(s3r_ctx* ctx, const uint16_t* n2i_xyz, const float* sparse, uint32_t n, uint32_t depth,
                     float* dense, void* stream)
{
    if (!ctx) return fail(nullptr, S3R_ERR_INVALID, "ctx is null");
    if (depth > S3R_MAX_DEPTH) return fail(ctx, S3R_ERR_INVALID, "depth exceeds S3R_MAX_DEPTH");
    if (!dense || (n > 0 && (!n2i_xyz || !sparse))) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    int rc = set_device(ctx);
    if (rc) return rc;
    const uint64_t e = (1ull << depth) + 1ull;
    const uint64_t count = e * e * e;
    if (ctx->grid_cap < count) {
        if (ctx->grid) cudaFree(ctx->grid);
        ctx->grid = nullptr;
        ctx->grid_cap = 0;
        S3R_CUDA(ctx, cudaMalloc(&ctx->grid, count * sizeof(float)));
        ctx->grid_cap = count;
    }
    cudaStream_t s = as_stream(stream);
    S3R_CUDA(ctx, launch_fill_f32(ctx->grid, count, __builtin_nanf(""), s));
    S3R_CUDA(ctx, launch_scatter_nodes(ctx->grid, depth, n2i_xyz, sparse, n, s));
    uint32_t launches = 0;
    S3R_CUDA(ctx, launch_interp_grid(ctx->grid, depth, dense, s, &launches));
    ctx->launches += 1 + (n > 0 ? 1 : 0) + launches;
    return S3R_OK;
}

int s3r_camera_look_at(const double eye[3], const double center[3], const double up[3], double fovy_deg, uint32_t W,
                       uint32_t H, int32_t ortho, double ortho_height, s3r_camera* out)
{
    if (!eye || !center || !up || !out || W == 0 || H == 0) return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    double z[3] = {eye[0] - center[0], eye[1] - center[1], eye[2] - center[2]};
    double zl = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
    if (!(zl > 0)) return fail(nullptr, S3R_ERR_INVALID, "eye equals center");
    for (double& c : z) c /= zl;
    double x[3] = {up[1] * z[2] - up[2] * z[1], up[2] * z[0] - up[0] * z[2], up[0] * z[1] - up[1] * z[0]};
    double xl = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    if (!(xl > 0)) return fail(nullptr, S3R_ERR_INVALID, "up is parallel to the view direction");
    for (double& c : x) c /= xl;
    double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
    const float lcam = 0.01f * 2 * 5.f;
    std::memset(out, 0, sizeof(*out));
    for (int d = 0; d < 3; ++d) {
        out->eye[d] = (float)eye[d];
        out->e1[d] = (float)x[d];
        out->e2[d] = (float)y[d];
        out->n[d] = (float)z[d] * (-lcam);
        out->view_r[d] = (float)x[d];
        out->view_r[3 + d] = (float)y[d];
        out->view_r[6 + d] = (float)z[d];
    }
    const double* rows[3] = {x, y, z};
    for (int a = 0; a < 3; ++a)
        out->view_t[a] = (float)-(rows[a][0] * eye[0] + rows[a][1] * eye[1] + rows[a][2] * eye[2]);
    out->ortho = ortho ? 1 : 0;
    if (ortho) {
        out->h = (float)ortho_height;
    } else {
        out->h = (float)(2 * lcam * std::tan(0.5 * fovy_deg * M_PI / 180));
    }
    const float pixel = out->h / (float)H;
    out->w = pixel * (float)W;
    return S3R_OK;
}

int s3r_camera_from_view(const float m[16], float fovy_deg, uint32_t W, uint32_t H, s3r_camera* out)
{
    if (!m || !out || W == 0 || H == 0) return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    // m: the world -> eye transform, column-major (element (row r, column c) at m[4 c + r]): rotation R and
    // translation T.  Its inverse (a rigid motion) has rotation R^T and translation -R^T T; the eye set-up of
    // DenseFieldRenderer_cu.cu:353-372 reads the eye position -(R^T) T, the screen axes (columns of R^T,
    // normalized) and the view direction (third column of R^T) from it, in float.
    float R[3][3], T[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) R[r][c] = m[4 * c + r];
        T[r] = m[12 + r];
    }
    auto normalized = [](float v[3]) {
        const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (l > 0) {
            v[0] /= l;
            v[1] /= l;
            v[2] /= l;
        }
    };
    std::memset(out, 0, sizeof(*out));
    const float lcam = 0.01f * 2 * 5.f;
    for (int r = 0; r < 3; ++r) // (-R^T) T, summed over the columns of -R^T in order
        out->eye[r] = -R[0][r] * T[0] + -R[1][r] * T[1] + -R[2][r] * T[2];
    float x[3] = {R[0][0], R[0][1], R[0][2]}, y[3] = {R[1][0], R[1][1], R[1][2]}, z[3] = {R[2][0], R[2][1], R[2][2]};
    normalized(x);
    normalized(y);
    normalized(z);
    for (int d = 0; d < 3; ++d) {
        out->e1[d] = x[d];
        out->e2[d] = y[d];
        out->n[d] = z[d] * (-lcam);
        out->view_r[d] = R[0][d];
        out->view_r[3 + d] = R[1][d];
        out->view_r[6 + d] = R[2][d];
        out->view_t[d] = T[d];
    }
    out->h = (float)(2 * lcam * std::tan(0.5 * (double)fovy_deg * M_PI / 180));
    const float pixel = out->h / (float)H;
    out->w = pixel * (float)W;
    return S3R_OK;
}

int s3r_block_cube(uint32_t level, const uint32_t idx[3], float center[3], float* half_size)
{
    if (!idx || !center || !half_size || level > 12) return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    block_cube_f(level, idx, center, *half_size);
    return S3R_OK;
}

int s3r_block_view_rect(const s3r_view* view, const uint32_t idx[3], int32_t rect[4])
{
    if (!idx || !rect) return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    int rc = check_view(nullptr, view);
    if (rc) return rc;
    view_rect(*view, idx, rect);
    return S3R_OK;
}

int s3r_clear_viewport(s3r_ctx* ctx, uint32_t* viewport, uint32_t W, uint32_t H, uint32_t value, void* stream)
{
    if (!ctx || !viewport) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    int rc = set_device(ctx);
    if (rc) return rc;
    S3R_CUDA(ctx, launch_fill_u32(viewport, (uint64_t)W * H, value, as_stream(stream)));
    ++ctx->launches;
    return S3R_OK;
}

// pitch: the brick's row pitch in elements (0: a plain (2^depth+1)^3 grid)
static int render_block_argb_pitched(s3r_ctx* ctx, const s3r_view* view, const float* brick, uint32_t depth,
                                     uint32_t pitch, const uint32_t idx[3], const int32_t rect[4], const float* tf,
                                     uint32_t* viewport, void* stream)
{
    if (!ctx) return fail(nullptr, S3R_ERR_INVALID, "ctx is null");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (!brick || !idx || !rect || !tf || !viewport) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (depth > S3R_MAX_DEPTH) return fail(ctx, S3R_ERR_INVALID, "depth exceeds S3R_MAX_DEPTH");
    const uint32_t m = 1u << view->level;
    if (idx[0] >= m || idx[1] >= m || idx[2] >= m) return fail(ctx, S3R_ERR_INVALID, "block index outside level");
    if (rect[2] < 0 || rect[3] < 0) return fail(ctx, S3R_ERR_INVALID, "negative view rectangle");
    if ((rc = set_device(ctx))) return rc;
    RenderBlock rb{};
    block_sampling(view->level, idx, depth, rb);
    rb.pitch = pitch;
    for (int i = 0; i < 4; ++i) rb.rect[i] = rect[i];
    S3R_CUDA(ctx, launch_render_block_argb(view, brick, rb, tf, viewport, as_stream(stream)));
    if (rect[2] > 0 && rect[3] > 0) ++ctx->launches;
    return S3R_OK;
}

int s3r_render_block_argb(s3r_ctx* ctx, const s3r_view* view, const float* brick, uint32_t depth,
                          const uint32_t idx[3], const int32_t rect[4], const float* tf, uint32_t* viewport,
                          void* stream)
{
    return render_block_argb_pitched(ctx, view, brick, depth, 0, idx, rect, tf, viewport, stream);
}

int s3r_index_box_world(uint32_t level, const uint32_t bmin[3], const uint32_t bmax[3], double cmin[3], double cmax[3])
{
    if (!bmin || !bmax || !cmin || !cmax || level > 12) return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    // s3vs::boundingBoxOfIndexBox (src/s3vs_worker/BlockOrderUtil.hpp:29-52), float arithmetic
    const float top = 5.f;
    const float h = top / (float)(1u << level);
    for (int d = 0; d < 3; ++d) {
        if (bmax[d] <= bmin[d]) return fail(nullptr, S3R_ERR_INVALID, "empty index box");
        const float c0 = -top + h * (float)(1u + (bmin[d] << 1));
        const float c1 = -top + h * (float)(1u + ((bmax[d] - 1) << 1));
        cmin[d] = (double)c0 - (double)h;
        cmax[d] = (double)c1 + (double)h;
    }
    return S3R_OK;
}

int s3r_b2f_order(const uint32_t bmin[3], const uint32_t bmax[3], const double cmin[3], const double cmax[3],
                  const double eye[3], uint32_t* out, uint32_t capacity, uint32_t* count)
{
    if (!bmin || !bmax || !cmin || !cmax || !eye || !count || (capacity && !out))
        return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    Split sp[3];
    for (int a = 0; a < 3; ++a) {
        if (bmax[a] <= bmin[a] || !((float)cmax[a] > (float)cmin[a]))
            return fail(nullptr, S3R_ERR_INVALID, "index box or world box is empty");
        sp[a] = split_range(bmin[a], bmax[a], (float)cmin[a], (float)cmax[a], (float)eye[a]);
    }
    uint32_t n = 0;
    b2f_traverse(sp, [&](const uint32_t q[3]) {
        if (n < capacity)
            for (int a = 0; a < 3; ++a) out[3 * n + a] = q[a];
        ++n;
    });
    *count = n;
    return S3R_OK;
}

int s3r_split_index_cube(uint32_t level, uint32_t split_count, int32_t add_trailing_empty, uint32_t* boxes,
                         uint32_t capacity, uint32_t* count)
{
    if (!count || (capacity && !boxes) || split_count == 0 || level > 20)
        return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    const CubeSplit cs = cube_split(level, split_count);
    uint32_t n = 0;
    for (uint32_t z = 0; z < cs.n[2]; ++z)
        for (uint32_t y = 0; y < cs.n[1]; ++y)
            for (uint32_t x = 0; x < cs.n[0]; ++x) {
                const uint32_t q[3] = {x, y, z};
                if (n < capacity) put_box(cs, q, boxes + 6 * n);
                ++n;
            }
    if (add_trailing_empty)
        for (; n < split_count; ++n)
            if (n < capacity) std::fill(boxes + 6 * n, boxes + 6 * n + 6, 0u);
    *count = n;
    return S3R_OK;
}

int s3r_split_b2f(uint32_t level, uint32_t split_count, const double eye[3], uint32_t* boxes, uint32_t capacity,
                  uint32_t* count)
{
    if (!eye || !count || (capacity && !boxes) || split_count == 0 || level > 20)
        return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    const CubeSplit cs = cube_split(level, split_count);
    Split sp[3];
    for (int a = 0; a < 3; ++a) sp[a] = split_boundaries(cs.coord[a].data(), cs.n[a], (float)eye[a]);
    uint32_t n = 0;
    b2f_traverse(sp, [&](const uint32_t q[3]) {
        if (n < capacity) put_box(cs, q, boxes + 6 * n);
        ++n;
    });
    *count = n;
    return S3R_OK;
}

int s3r_bound_rect(s3r_ctx* ctx, const uint32_t* viewport, uint32_t W, uint32_t H, int32_t rect[4], void* stream)
{
    if (!ctx || !viewport || !rect) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    int rc = set_device(ctx);
    if (rc) return rc;
    cudaStream_t s = as_stream(stream);
    int32_t init[4] = {(int32_t)W, (int32_t)H, -1, -1};
    std::memcpy(ctx->rect_host, init, sizeof(init));
    S3R_CUDA(ctx, cudaMemcpyAsync(ctx->rect_dev, ctx->rect_host, sizeof(init), cudaMemcpyHostToDevice, s));
    S3R_CUDA(ctx, launch_bound_rect(viewport, W, H, ctx->rect_dev, s));
    ++ctx->launches;
    S3R_CUDA(ctx, cudaMemcpyAsync(ctx->rect_host, ctx->rect_dev, sizeof(init), cudaMemcpyDeviceToHost, s));
    S3R_CUDA(ctx, cudaStreamSynchronize(s));
    const int32_t* r = ctx->rect_host;
    if (r[2] < r[0] || r[3] < r[1]) {
        rect[0] = rect[1] = rect[2] = rect[3] = 0;
    } else {
        rect[0] = r[0];
        rect[1] = r[1];
        rect[2] = r[2] - r[0] + 1;
        rect[3] = r[3] - r[1] + 1;
    }
    return S3R_OK;
}

int s3r_crop(s3r_ctx* ctx, const uint32_t* image, uint32_t W, const int32_t rect[4], uint32_t* dst, void* stream)
{
    if (!ctx || !image || !rect || !dst) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (rect[0] < 0 || rect[1] < 0 || rect[2] < 0 || rect[3] < 0 || (uint32_t)(rect[0] + rect[2]) > W)
        return fail(ctx, S3R_ERR_INVALID, "crop rectangle outside the image");
    int rc = set_device(ctx);
    if (rc) return rc;
    S3R_CUDA(ctx, launch_crop(image, W, rect, dst, as_stream(stream)));
    if (rect[2] > 0 && rect[3] > 0) ++ctx->launches;
    return S3R_OK;
}

int s3r_default_light(const s3r_view* view, s3r_light* out)
{
    if (!view || !out) return fail(nullptr, S3R_ERR_INVALID, "null pointer");
    const s3r_camera& c = view->cam;
    for (int d = 0; d < 3; ++d) {
        out->pos[d] = (c.eye[d] + c.n[d]) + c.e2[d] * c.h; // DenseFieldRenderer_cu.cu:442
        out->ambient[d] = 0.f;
        out->diffuse[d] = 1.f;
        out->specular[d] = 0.1f;
    }
    return S3R_OK;
}

static int render_block_pitched(s3r_ctx* ctx, const s3r_view* view, const s3r_presentation* pres,
                                const float* brick, const float* brick2, uint32_t depth, uint32_t pitch,
                                const uint32_t idx[3], const int32_t rect[4], const float* tf, uint32_t* viewport,
                                void* stream)
{
    if (!ctx) return fail(nullptr, S3R_ERR_INVALID, "ctx is null");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (!pres || !brick || !idx || !rect || !tf || !viewport) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (pres->mode > S3R_MODE_VALUE_ON_ISOSURFACES) return fail(ctx, S3R_ERR_INVALID, "unknown field mode");
    if (pres->level_count > S3R_MAX_LEVELS) return fail(ctx, S3R_ERR_INVALID, "more than S3R_MAX_LEVELS levels");
    if (pres->light_count > S3R_MAX_LIGHTS) return fail(ctx, S3R_ERR_INVALID, "more than S3R_MAX_LIGHTS lights");
    for (uint32_t i = 1; i < pres->level_count; ++i)
        if (!(pres->levels[i] > pres->levels[i - 1]))
            return fail(ctx, S3R_ERR_INVALID, "levels must ascend strictly");
    const bool secondary = pres->mode == S3R_MODE_VALUE_ON_ISOSURFACE || pres->mode == S3R_MODE_VALUE_ON_ISOSURFACES;
    if (secondary && !brick2) return fail(ctx, S3R_ERR_INVALID, "this mode needs the secondary field's brick");
    if (secondary && !(pres->secondary_max > pres->secondary_min))
        return fail(ctx, S3R_ERR_INVALID, "secondary field range is empty");
    if (depth > S3R_MAX_DEPTH) return fail(ctx, S3R_ERR_INVALID, "depth exceeds S3R_MAX_DEPTH");
    const uint32_t m = 1u << view->level;
    if (idx[0] >= m || idx[1] >= m || idx[2] >= m) return fail(ctx, S3R_ERR_INVALID, "block index outside level");
    if (rect[2] < 0 || rect[3] < 0) return fail(ctx, S3R_ERR_INVALID, "negative view rectangle");
    if ((rc = set_device(ctx))) return rc;
    RenderBlock rb{};
    block_sampling(view->level, idx, depth, rb);
    rb.pitch = pitch;
    for (int i = 0; i < 4; ++i) rb.rect[i] = rect[i];
    S3R_CUDA(ctx, launch_render_block_mode(view, pres, brick, brick2, rb, tf, viewport, as_stream(stream)));
    if (rect[2] > 0 && rect[3] > 0) ++ctx->launches;
    return S3R_OK;
}

int s3r_render_block(s3r_ctx* ctx, const s3r_view* view, const s3r_presentation* pres, const float* brick,
                     const float* brick2, uint32_t depth, const uint32_t idx[3], const int32_t rect[4],
                     const float* tf, uint32_t* viewport, void* stream)
{
    return render_block_pitched(ctx, view, pres, brick, brick2, depth, 0, idx, rect, tf, viewport, stream);
}

// ------------------------------------------------------------------ texture-unit path

int s3r_texture_create(s3r_ctx* ctx, uint32_t depth, s3r_texture** out)
{
    if (!ctx || !out) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (depth > S3R_MAX_DEPTH) return fail(ctx, S3R_ERR_INVALID, "depth exceeds S3R_MAX_DEPTH");
    int rc = set_device(ctx);
    if (rc) return rc;
    auto* t = new (std::nothrow) s3r_texture;
    if (!t) return fail(ctx, S3R_ERR_NOMEM, "out of host memory");
    t->ctx = ctx;
    t->depth = depth;
    t->n = (1u << depth) + 1u;
    const cudaChannelFormatDesc desc = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
    cudaError_t e = cudaMalloc3DArray(&t->array, &desc, make_cudaExtent(t->n, t->n, t->n), cudaArraySurfaceLoadStore);
    if (e == cudaSuccess) {
        cudaResourceDesc res;
        std::memset(&res, 0, sizeof(res));
        res.resType = cudaResourceTypeArray;
        res.res.array.array = t->array;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.normalizedCoords = 0;
        td.filterMode = cudaFilterModeLinear;
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.readMode = cudaReadModeElementType;
        e = cudaCreateTextureObject(&t->tex, &res, &td, nullptr);
    }
    if (e != cudaSuccess) {
        s3r_texture_destroy(t);
        return cuda_fail(ctx, e, "field texture");
    }
    *out = t;
    return S3R_OK;
}

int s3r_texture_destroy(s3r_texture* t)
{
    if (!t) return S3R_OK;
    if (t->ctx) cudaSetDevice(t->ctx->device);
    if (t->tex) cudaDestroyTextureObject(t->tex);
    if (t->array) cudaFreeArray(t->array);
    delete t;
    return S3R_OK;
}

int s3r_texture_fill(s3r_ctx* ctx, s3r_texture* t, const float* dense, void* stream)
{
    if (!ctx || !t || !dense) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (t->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "texture belongs to another context");
    int rc = set_device(ctx);
    if (rc) return rc;
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof(p));
    p.srcPtr = make_cudaPitchedPtr(const_cast<float*>(dense), t->n * sizeof(float), t->n, t->n);
    p.dstArray = t->array;
    p.extent = make_cudaExtent(t->n, t->n, t->n);
    p.kind = cudaMemcpyDeviceToDevice;
    S3R_CUDA(ctx, cudaMemcpy3DAsync(&p, as_stream(stream)));
    return S3R_OK;
}

int s3r_interp_dense_texture(s3r_ctx* ctx, const uint16_t* n2i_xyz, const float* sparse, uint32_t n, s3r_texture* t,
                             void* stream)
{
    if (!ctx || !t) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (t->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "texture belongs to another context");
    int rc = set_device(ctx);
    if (rc) return rc;
    const uint64_t count = (uint64_t)t->n * t->n * t->n;
    if (ctx->tex_stage_cap < count) {
        if (ctx->tex_stage) cudaFree(ctx->tex_stage);
        ctx->tex_stage = nullptr;
        ctx->tex_stage_cap = 0;
        S3R_CUDA(ctx, cudaMalloc(&ctx->tex_stage, count * sizeof(float)));
        ctx->tex_stage_cap = count;
    }
    if ((rc = s3r_interp_dense(ctx, n2i_xyz, sparse, n, t->depth, ctx->tex_stage, stream))) return rc;
    return s3r_texture_fill(ctx, t, ctx->tex_stage, stream);
}

int s3r_tf_texture_create(s3r_ctx* ctx, uint32_t tf_n, s3r_tf_texture** out)
{
    if (!ctx || !out) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (tf_n < 2 || tf_n > 4096) return fail(ctx, S3R_ERR_INVALID, "tf_n must be in [2, 4096]");
    int rc = set_device(ctx);
    if (rc) return rc;
    auto* t = new (std::nothrow) s3r_tf_texture;
    if (!t) return fail(ctx, S3R_ERR_NOMEM, "out of host memory");
    t->ctx = ctx;
    t->n = tf_n;
    const cudaChannelFormatDesc desc = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindFloat);
    cudaError_t e = cudaMallocArray(&t->array, &desc, tf_n, 1, cudaArrayTextureGather);
    if (e == cudaSuccess) {
        cudaResourceDesc res;
        std::memset(&res, 0, sizeof(res));
        res.resType = cudaResourceTypeArray;
        res.res.array.array = t->array;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.normalizedCoords = 1;
        td.filterMode = cudaFilterModeLinear;
        td.addressMode[0] = cudaAddressModeClamp;
        td.readMode = cudaReadModeElementType;
        e = cudaCreateTextureObject(&t->tex, &res, &td, nullptr);
    }
    if (e != cudaSuccess) {
        s3r_tf_texture_destroy(t);
        return cuda_fail(ctx, e, "transfer-function texture");
    }
    *out = t;
    return S3R_OK;
}

int s3r_tf_texture_set(s3r_ctx* ctx, s3r_tf_texture* t, const float* tf, void* stream)
{
    if (!ctx || !t || !tf) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (t->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "texture belongs to another context");
    int rc = set_device(ctx);
    if (rc) return rc;
    const size_t row = (size_t)t->n * 4 * sizeof(float);
    S3R_CUDA(ctx, cudaMemcpy2DToArrayAsync(t->array, 0, 0, tf, row, row, 1, cudaMemcpyDeviceToDevice,
                                           as_stream(stream)));
    return S3R_OK;
}

int s3r_tf_texture_destroy(s3r_tf_texture* t)
{
    if (!t) return S3R_OK;
    if (t->ctx) cudaSetDevice(t->ctx->device);
    if (t->tex) cudaDestroyTextureObject(t->tex);
    if (t->array) cudaFreeArray(t->array);
    delete t;
    return S3R_OK;
}

int s3r_render_block_texture(s3r_ctx* ctx, const s3r_view* view, const s3r_presentation* pres,
                             const s3r_texture* field, const s3r_texture* field2, const uint32_t idx[3],
                             const int32_t rect[4], const s3r_tf_texture* tf, uint32_t* viewport, void* stream)
{
    if (!ctx) return fail(nullptr, S3R_ERR_INVALID, "ctx is null");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (!field || !idx || !rect || !tf || !viewport) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (field->ctx != ctx || tf->ctx != ctx || (field2 && field2->ctx != ctx))
        return fail(ctx, S3R_ERR_INVALID, "texture belongs to another context");
    if (tf->n != view->tf_n) return fail(ctx, S3R_ERR_INVALID, "transfer-function texture size differs from tf_n");
    s3r_presentation argb{};
    argb.mode = S3R_MODE_ARGB;
    const s3r_presentation* pr = pres ? pres : &argb;
    if (pr->mode > S3R_MODE_VALUE_ON_ISOSURFACES) return fail(ctx, S3R_ERR_INVALID, "unknown field mode");
    if (pr->level_count > S3R_MAX_LEVELS) return fail(ctx, S3R_ERR_INVALID, "more than S3R_MAX_LEVELS levels");
    if (pr->light_count > S3R_MAX_LIGHTS) return fail(ctx, S3R_ERR_INVALID, "more than S3R_MAX_LIGHTS lights");
    for (uint32_t i = 1; i < pr->level_count; ++i)
        if (!(pr->levels[i] > pr->levels[i - 1])) return fail(ctx, S3R_ERR_INVALID, "levels must ascend strictly");
    const bool secondary = pr->mode == S3R_MODE_VALUE_ON_ISOSURFACE || pr->mode == S3R_MODE_VALUE_ON_ISOSURFACES;
    if (secondary && (!field2 || field2->depth != field->depth))
        return fail(ctx, S3R_ERR_INVALID, "this mode needs the secondary field's texture, of the same depth");
    if (secondary && !(pr->secondary_max > pr->secondary_min))
        return fail(ctx, S3R_ERR_INVALID, "secondary field range is empty");
    const uint32_t m = 1u << view->level;
    if (idx[0] >= m || idx[1] >= m || idx[2] >= m) return fail(ctx, S3R_ERR_INVALID, "block index outside level");
    if (rect[2] < 0 || rect[3] < 0) return fail(ctx, S3R_ERR_INVALID, "negative view rectangle");
    if ((rc = set_device(ctx))) return rc;
    RenderBlock rb{};
    block_sampling(view->level, idx, field->depth, rb);
    for (int i = 0; i < 4; ++i) rb.rect[i] = rect[i];
    S3R_CUDA(ctx, launch_render_block_texture(view, pr, (uint64_t)field->tex, field2 ? (uint64_t)field2->tex : 0,
                                              (uint64_t)tf->tex, rb, viewport, as_stream(stream)));
    if (rect[2] > 0 && rect[3] > 0) ++ctx->launches;
    return S3R_OK;
}

int s3r_blend_image_part_mip_host(float* dst, int32_t dw, int32_t dh, const float* src, int32_t sw, int32_t sh,
                                  int32_t ox, int32_t oy, int32_t just_copy, int32_t offx, int32_t offy)
{
    if (!dst || (!src && sw * sh > 0)) return fail(nullptr, S3R_ERR_INVALID, "null pointer");
    const int32_t dx = ox - offx, dy = oy - offy;
    if (dx < 0 || dy < 0 || dx + sw > dw || dy + sh > dh)
        return fail(nullptr, S3R_ERR_INVALID, "image part does not fit the destination");
    for (int32_t y = 0; y < sh; ++y) {
        const float* srow = src + (size_t)y * sw;
        float* drow = dst + (size_t)dw * (dy + y) + dx;
        if (just_copy) {
            std::memcpy(drow, srow, sizeof(float) * sw);
            continue;
        }
        for (int32_t i = 0; i < sw; ++i) {
            const float sv = srow[i];
            if (std::isnan(sv)) continue;
            if (std::isnan(drow[i]) || drow[i] < sv) drow[i] = sv;
        }
    }
    return S3R_OK;
}

int s3r_blend_image_part_host(uint32_t* dst, int32_t dw, int32_t dh, const uint32_t* src, int32_t sw, int32_t sh,
                              int32_t ox, int32_t oy, int32_t just_copy, int32_t offx, int32_t offy)
{
    if (!dst || (!src && sw * sh > 0)) return fail(nullptr, S3R_ERR_INVALID, "null pointer");
    const int32_t dx = ox - offx, dy = oy - offy;
    if (dx < 0 || dy < 0 || dx + sw > dw || dy + sh > dh)
        return fail(nullptr, S3R_ERR_INVALID, "image part does not fit the destination");
    for (int32_t y = 0; y < sh; ++y) {
        const uint32_t* srow = src + (size_t)y * sw;
        uint32_t* drow = dst + (size_t)dw * (dy + y) + dx;
        if (just_copy) {
            std::memcpy(drow, srow, sizeof(uint32_t) * sw);
            continue;
        }
        for (int32_t i = 0; i < sw; ++i) {
            const uint32_t s = srow[i], as = s >> 24;
            if (as == 0) continue;
            const uint32_t d = drow[i], ad = d >> 24;
            if (as == 255u || ad == 0) {
                drow[i] = s;
                continue;
            }
            const uint32_t a = as + ad * (255u - as) / 255u;
            uint32_t o = (a & 0xffu) << 24;
            for (int b = 0; b < 3; ++b) {
                const uint32_t cs = (s >> (8 * b)) & 0xffu, cd = (d >> (8 * b)) & 0xffu;
                o |= (((cs * as + cd * (a - as)) / a) & 0xffu) << (8 * b);
            }
            drow[i] = o;
        }
    }
    return S3R_OK;
}

int s3r_compose_parts(s3r_ctx* ctx, const s3r_image_part* parts, uint32_t nparts, int32_t just_copy_first,
                      uint32_t* dst, int32_t dw, int32_t dh, int32_t offx, int32_t offy, void* stream)
{
    if (!ctx || !dst || (nparts && !parts)) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    int rc = set_device(ctx);
    if (rc) return rc;
    if (nparts == 0) return S3R_OK;
    if (ctx->parts_cap < nparts) {
        if (ctx->parts_dev) cudaFree(ctx->parts_dev);
        ctx->parts_dev = nullptr;
        ctx->parts_cap = 0;
        S3R_CUDA(ctx, cudaMalloc(&ctx->parts_dev, sizeof(s3r_image_part) * nparts));
        ctx->parts_cap = nparts;
    }
    cudaStream_t s = as_stream(stream);
    S3R_CUDA(ctx, cudaMemcpyAsync(ctx->parts_dev, parts, sizeof(s3r_image_part) * nparts, cudaMemcpyHostToDevice, s));
    S3R_CUDA(ctx, launch_compose(ctx->parts_dev, nparts, just_copy_first, dst, dw, dh, offx, offy, s));
    // the parts array is pageable host memory copied asynchronously: finish before returning
    S3R_CUDA(ctx, cudaStreamSynchronize(s));
    ++ctx->launches;
    return S3R_OK;
}

int s3r_make_color_transfer(const double* xs, const double* rgba, uint32_t npoints, uint32_t color_count, float* out)
{
    if (!out || color_count == 0 || (npoints && (!xs || !rgba))) return fail(nullptr, S3R_ERR_INVALID, "bad argument");
    // makeColorTransferVector (include/s3vs/ColorTransferFunction.hpp:27-69); real_type is float
    if (npoints == 0) {
        for (uint32_t i = 0; i < 4 * color_count; ++i) out[i] = 1.f;
        return S3R_OK;
    }
    if (npoints == 1) {
        for (uint32_t i = 0; i < color_count; ++i)
            for (int c = 0; c < 4; ++c) out[4 * i + c] = (float)rgba[c];
        return S3R_OK;
    }
    for (uint32_t i = 1; i < npoints; ++i)
        if (!((float)xs[i] > (float)xs[i - 1])) return fail(nullptr, S3R_ERR_INVALID, "control points not increasing");
    std::fill(out, out + 4 * color_count, 0.f);
    const float xmin = (float)xs[0], xmax = (float)xs[npoints - 1];
    float c1[4];
    for (int c = 0; c < 4; ++c) out[c] = c1[c] = (float)rgba[c];
    uint32_t i1 = 0;
    for (uint32_t ip = 1; ip < npoints; ++ip) {
        float c2[4];
        for (int c = 0; c < 4; ++c) c2[c] = (float)rgba[4 * ip + c];
        const uint32_t i2 = ip + 1 == npoints ? color_count - 1u
                                              : (uint32_t)(((float)xs[ip] - xmin) / (xmax - xmin) * (float)color_count);
        for (uint32_t i = i1 + 1; i2 > i1 && i <= i2 && i < color_count; ++i) {
            const float t = (float)(i - i1) / (float)(i2 - i1);
            for (int c = 0; c < 4; ++c) out[4 * i + c] = c1[c] * (1 - t) + c2[c] * t;
        }
        for (int c = 0; c < 4; ++c) c1[c] = c2[c];
        i1 = i2;
    }
    return S3R_OK;
}

// ------------------------------------------------------------------ plans

int s3r_frame_plan(s3r_ctx* ctx, const s3r_frame_desc* desc, s3r_plan** out)
{
    if (!ctx || !desc || !out) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    *out = nullptr;
    if (desc->level > 8) return fail(ctx, S3R_ERR_INVALID, "level out of range (max 8)");
    if (desc->nblocks == 0 || !desc->blocks || !desc->node_off || (!desc->n2i && desc->node_off[desc->nblocks]))
        return fail(ctx, S3R_ERR_INVALID, "empty or null block description");
    if (desc->brick_format > S3R_BRICK_BF16) return fail(ctx, S3R_ERR_INVALID, "unknown brick format");
    uint32_t tl = 4;
    if (desc->tile_cells) {
        if (desc->tile_cells == 8) tl = 3;
        else if (desc->tile_cells == 16) tl = 4;
        else if (desc->tile_cells == 32) tl = 5;
        else return fail(ctx, S3R_ERR_INVALID, "tile_cells must be 0, 8, 16 or 32");
    }
    int rc = set_device(ctx);
    if (rc) return rc;
    const uint32_t m = 1u << desc->level;
    auto p = new (std::nothrow) s3r_plan;
    if (!p) return fail(ctx, S3R_ERR_NOMEM, "out of host memory");
    p->ctx = ctx;
    p->desc = *desc;
    p->nblocks = desc->nblocks;
    p->level = desc->level;
    p->fmt = desc->brick_format;
    p->render_tile = desc->render_tile % kRenderTiles;
    p->blocks.assign(desc->blocks, desc->blocks + 4 * (size_t)desc->nblocks);
    p->node_off.assign(desc->node_off, desc->node_off + desc->nblocks + 1);
    p->nodes = p->node_off[desc->nblocks];
    if (p->nodes > 0xffffffffull) {
        s3r_plan_destroy(p);
        return fail(ctx, S3R_ERR_INVALID, "a plan holds fewer than 2^32 nodes");
    }
    p->n2i.assign(desc->n2i, desc->n2i + 3 * p->nodes);
    p->vertex_off.assign(desc->nblocks + 1, 0);
    p->pitch.assign(desc->nblocks, 0);
    p->vertices = 0;
    const uint32_t elem_bytes = p->fmt == S3R_BRICK_F32 ? 4u : 2u;
    p->table_host.assign((size_t)m * m * m, RenderBlock{});
    for (auto& t : p->table_host) {
        t.depth = 0xffffffffu;
        t.fmt = p->fmt;
    }
    auto bail = [&](int code) {
        s3r_plan_destroy(p);
        return code;
    };
    for (uint32_t b = 0; b < desc->nblocks; ++b) {
        const uint32_t* bl = &p->blocks[4 * b];
        if (bl[0] >= m || bl[1] >= m || bl[2] >= m)
            return bail(fail(ctx, S3R_ERR_INVALID, "block index outside the level"));
        if (bl[3] > S3R_MAX_DEPTH) return bail(fail(ctx, S3R_ERR_INVALID, "block depth exceeds S3R_MAX_DEPTH"));
        if (p->node_off[b + 1] < p->node_off[b]) return bail(fail(ctx, S3R_ERR_INVALID, "node offsets decrease"));
        if (p->node_off[b + 1] - p->node_off[b] > 0xffffffffull)
            return bail(fail(ctx, S3R_ERR_INVALID, "too many nodes in one block"));
        const uint64_t e = (1ull << bl[3]) + 1;
        const uint32_t pitch = plan_brick_pitch(bl[3], elem_bytes);
        p->pitch[b] = pitch;
        p->vertex_off[b + 1] = p->vertex_off[b] + e * e * pitch;
        p->vertices += e * e * e;
        RenderBlock& t = p->table_host[bl[0] + m * (bl[1] + m * bl[2])];
        if (t.depth != 0xffffffffu) return bail(fail(ctx, S3R_ERR_INVALID, "duplicate block index"));
        block_sampling(p->level, bl, bl[3], t);
        t.brick_off = p->vertex_off[b];
        t.pitch = pitch;
        t.block = b;
        const uint32_t lim = (uint32_t)(e - 1);
        for (uint64_t i = p->node_off[b]; i < p->node_off[b + 1]; ++i)
            if (p->n2i[3 * i] > lim || p->n2i[3 * i + 1] > lim || p->n2i[3 * i + 2] > lim)
                return bail(fail(ctx, S3R_ERR_INVALID, "node index outside its block"));
    }
    p->brick_elems = p->vertex_off[desc->nblocks];
    const size_t esz = elem_bytes;
    cudaError_t e;
    if ((e = cudaMalloc(&p->bricks, std::max<uint64_t>(p->brick_elems, 1) * esz)) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMalloc(bricks)"));
    if ((rc = upload(ctx, &p->node_off_dev, p->node_off))) return bail(rc);
    if ((e = cudaMalloc(&p->queue_dev, 2 * sizeof(uint32_t))) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMalloc(queue)"));
    if ((e = cudaMalloc(&p->scale_offset_dev, sizeof(float2) * p->nblocks)) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMalloc(scales)"));
    if ((e = cudaMalloc(&p->table_dev, sizeof(RenderBlock) * p->table_host.size())) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMalloc(table)"));
    if ((e = cudaMalloc(&p->view_dev, sizeof(s3r_view))) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMalloc(view)"));
    if ((e = cudaMallocHost(&p->table_pinned, sizeof(RenderBlock) * p->table_host.size())) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMallocHost(table)"));
    if ((e = cudaMallocHost(&p->view_pinned, sizeof(s3r_view))) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMallocHost(view)"));
    if ((e = cudaMalloc(&p->cover_dev, 4 * sizeof(int32_t))) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMalloc(cover)"));
    if ((e = cudaMallocHost(&p->cover_pinned, 4 * sizeof(int32_t))) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaMallocHost(cover)"));
    if ((e = cudaEventCreateWithFlags(&p->staged, cudaEventDisableTiming)) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaEventCreate"));
    // block-major render: blocks deepest first (most samples per ray), so that the longest work items start first
    {
        std::vector<uint32_t> idx(desc->nblocks);
        for (uint32_t b = 0; b < desc->nblocks; ++b) idx[b] = b;
        std::stable_sort(idx.begin(), idx.end(),
                         [&](uint32_t a, uint32_t b) { return p->blocks[4 * a + 3] > p->blocks[4 * b + 3]; });
        p->seg_order.resize(desc->nblocks);
        for (uint32_t i = 0; i < desc->nblocks; ++i) {
            const uint32_t* bl = &p->blocks[4 * idx[i]];
            p->seg_order[i] = bl[0] + m * (bl[1] + m * bl[2]);
        }
        if ((e = cudaMalloc(&p->seg_count_dev, sizeof(uint32_t))) != cudaSuccess ||
            (e = cudaMallocHost(&p->seg_count_pinned, sizeof(uint32_t))) != cudaSuccess ||
            (e = cudaMalloc(&p->seg_queue, 2 * sizeof(uint32_t))) != cudaSuccess ||
            (e = cudaMemset(p->seg_queue, 0, 2 * sizeof(uint32_t))) != cudaSuccess)
            return bail(cuda_fail(ctx, e, "cudaMalloc(block-major render)"));
    }
    if ((rc = plan_bin(p, tl))) return bail(rc);
    *out = p;
    return S3R_OK;
}

static void plan_destroy_host_pipeline(s3r_plan* p);

int s3r_plan_destroy(s3r_plan* p)
{
    if (!p) return S3R_OK;
    if (p->ctx) cudaSetDevice(p->ctx->device);
    plan_destroy_host_pipeline(p);
    plan_drop_graph(p);
    plan_free_device(p);
    auto f = [](void* q) {
        if (q) cudaFree(q);
    };
    f(p->bricks);
    f(p->node_off_dev);
    f(p->queue_dev);
    f(p->scale_offset_dev);
    f(p->table_dev);
    f(p->view_dev);
    if (p->table_pinned) cudaFreeHost(p->table_pinned);
    if (p->view_pinned) cudaFreeHost(p->view_pinned);
    if (p->cover_pinned) cudaFreeHost(p->cover_pinned);
    f(p->cover_dev);
    f(p->dtf_part);
    f(p->seg_items_dev);
    f(p->seg_count_dev);
    f(p->seg_queue);
    if (p->seg_items_pinned) cudaFreeHost(p->seg_items_pinned);
    if (p->seg_count_pinned) cudaFreeHost(p->seg_count_pinned);
    plan_free_segments(p);
    if (p->staged) cudaEventDestroy(p->staged);
    delete p;
    return S3R_OK;
}

int s3r_plan_info_get(const s3r_plan* p, s3r_plan_info* out)
{
    if (!p || !out) return fail(nullptr, S3R_ERR_INVALID, "null pointer");
    out->nodes = p->nodes;
    out->vertices = p->vertices;
    out->brick_bytes = p->brick_elems * (p->fmt == S3R_BRICK_F32 ? 4 : 2);
    out->tiles = p->tiles;
    out->tile_entries = p->entries;
    out->tile_cells = 1u << p->tile_log2;
    out->render_tile = p->render_tile;
    out->brick_format = p->fmt;
    out->nblocks = p->nblocks;
    return S3R_OK;
}

int s3r_plan_tile_cells(const s3r_plan* p, uint32_t depth, uint32_t* cells)
{
    if (!p || !cells) return fail(nullptr, S3R_ERR_INVALID, "null pointer");
    if (depth > S3R_MAX_DEPTH) return fail(nullptr, S3R_ERR_INVALID, "depth exceeds S3R_MAX_DEPTH");
    *cells = 1u << p->tile_by_depth[depth];
    return S3R_OK;
}

int s3r_plan_bricks(const s3r_plan* p, void** bricks, const uint64_t** vertex_off)
{
    if (!p || !bricks || !vertex_off) return fail(nullptr, S3R_ERR_INVALID, "null pointer");
    *bricks = p->bricks;
    *vertex_off = p->vertex_off.data();
    return S3R_OK;
}

int s3r_plan_brick_pitches(const s3r_plan* p, const uint32_t** pitch)
{
    if (!p || !pitch) return fail(nullptr, S3R_ERR_INVALID, "null pointer");
    *pitch = p->pitch.data();
    return S3R_OK;
}

int s3r_plan_brick_scales(const s3r_plan* p, const float** scale_offset)
{
    if (!p || !scale_offset) return fail(nullptr, S3R_ERR_INVALID, "null pointer");
    *scale_offset = p->fmt == S3R_BRICK_F32 ? nullptr : reinterpret_cast<const float*>(p->scale_offset_dev);
    return S3R_OK;
}

int s3r_frame_interp(s3r_ctx* ctx, s3r_plan* plan, const float* sparse, void* stream)
{
    if (!ctx || !plan || (!sparse && plan->nodes)) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "plan belongs to another context");
    int rc = set_device(ctx);
    if (rc) return rc;
    uint32_t k = 0;
    rc = plan_launch_interp(plan, sparse, as_stream(stream), &k);
    ctx->launches += k;
    return rc;
}

int s3r_frame_render(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* tf, float* rgba, uint32_t* argb,
                     unsigned long long* samples, void* stream)
{
    if (!ctx || !plan || !tf) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "plan belongs to another context");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (view->level != plan->level) return fail(ctx, S3R_ERR_INVALID, "view level differs from the plan level");
    if ((rc = set_device(ctx))) return rc;
    cudaStream_t s = as_stream(stream);
    if ((rc = plan_stage_view(plan, view, s))) return rc;
    uint32_t k = 0;
    rc = plan_launch_render(plan, tf, rgba, argb, samples, s, &k);
    ctx->launches += k;
    return rc;
}

int s3r_frame_render_mode(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const s3r_presentation* pres,
                          const float* tf, const void* bricks2, float* rgba, uint32_t* argb, void* stream)
{
    if (!ctx || !plan || !tf || !pres) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "plan belongs to another context");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (view->level != plan->level) return fail(ctx, S3R_ERR_INVALID, "view level differs from the plan level");
    if (pres->mode > S3R_MODE_VALUE_ON_ISOSURFACES) return fail(ctx, S3R_ERR_INVALID, "unknown field mode");
    if (pres->level_count > S3R_MAX_LEVELS || pres->light_count > S3R_MAX_LIGHTS)
        return fail(ctx, S3R_ERR_INVALID, "too many levels or lights");
    if ((pres->mode == S3R_MODE_VALUE_ON_ISOSURFACE || pres->mode == S3R_MODE_VALUE_ON_ISOSURFACES) && !bricks2)
        return fail(ctx, S3R_ERR_INVALID, "the value-on-isosurface modes need the secondary bricks");
    if (plan->fmt != S3R_BRICK_F32) return fail(ctx, S3R_ERR_UNSUPPORTED, "field modes need F32 bricks");
    if ((rc = set_device(ctx))) return rc;
    cudaStream_t s = as_stream(stream);
    if ((rc = plan_stage_view(plan, view, s))) return rc;
    FrameArgs fa{};
    fa.view = plan->view_dev;
    fa.table = plan->table_dev;
    fa.bricks = plan->bricks;
    fa.tf = tf;
    fa.rgba = rgba;
    fa.argb = argb;
    fa.cover = plan->cover_dev;
    S3R_CUDA(ctx, launch_frame_render_mode(fa, *pres, static_cast<const float*>(bricks2), view->W, view->H, view->tf_n,
                                           view->filter, s));
    ++ctx->launches;
    return S3R_OK;
}

static int plan_launch_frame(s3r_plan* plan, int slot, const s3r_view* view, const float* sparse, const float* tf,
                             float* rgba, uint32_t* argb, unsigned long long* samples, cudaStream_t s);

int s3r_frame_run(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* sparse, const float* tf,
                  float* rgba, uint32_t* argb, unsigned long long* samples, void* stream)
{
    if (!ctx || !plan || !tf || (!sparse && plan->nodes)) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "plan belongs to another context");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (view->level != plan->level) return fail(ctx, S3R_ERR_INVALID, "view level differs from the plan level");
    if ((rc = set_device(ctx))) return rc;
    cudaStream_t s = as_stream(stream);
    if ((rc = plan_stage_view(plan, view, s))) return rc;
    return plan_launch_frame(plan, 0, view, sparse, tf, rgba, argb, samples, s);
}

// The frame as a CUDA graph in cache slot `slot`, captured again when its arguments change.
static int plan_launch_frame(s3r_plan* plan, int slot, const s3r_view* view, const float* sparse, const float* tf,
                      float* rgba, uint32_t* argb, unsigned long long* samples, cudaStream_t s)
{
    s3r_ctx* ctx = plan->ctx;
    FrameGraph& G = plan->graphs[slot];
    const void* key[5] = {sparse, tf, rgba, argb, samples};
    const uint32_t dims[4] = {view->W, view->H, view->tf_n, view->filter};
    const bool same = G.exec && std::memcmp(key, G.key, sizeof(key)) == 0 && std::memcmp(dims, G.dims, sizeof(dims)) == 0;
    if (!same) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        G = FrameGraph{};
        cudaStream_t cs = ctx->capture;
        S3R_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        uint32_t k = 0;
        const int data = slot == 2 ? 1 : 0; // the host pipeline's second slot has its own bricks
        int r1 = plan_launch_interp(plan, sparse, cs, &k, data);
        int r3 = r1 ? r1 : plan_launch_render(plan, tf, rgba, argb, samples, cs, &k, data);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(cs, &graph);
        if (r3) {
            if (graph) cudaGraphDestroy(graph);
            return r3;
        }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&G.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            G.exec = nullptr;
            return cuda_fail(ctx, e, "cudaGraphInstantiate");
        }
        std::memcpy(G.key, key, sizeof(key));
        std::memcpy(G.dims, dims, sizeof(dims));
        G.kernels = k;
    }
    S3R_CUDA(ctx, cudaGraphLaunch(G.exec, s));
    ctx->launches += G.kernels;
    return S3R_OK;
}

// Releases the host-buffer pipeline's device buffers (after its copies have finished).
static void plan_free_host_slots(s3r_plan* p)
{
    if (p->hs_h2d) cudaStreamSynchronize(p->hs_h2d);
    if (p->hs_d2h) cudaStreamSynchronize(p->hs_d2h);
    for (int b = 0; b < 2; ++b)
        if (p->hs_comp[b]) cudaStreamSynchronize(p->hs_comp[b]);
    for (int b = 0; b < 2; ++b) {
        if (p->hs_sparse[b]) cudaFree(p->hs_sparse[b]);
        if (p->hs_argb[b]) cudaFree(p->hs_argb[b]);
        if (p->hs_tf[b]) cudaFree(p->hs_tf[b]);
        p->hs_sparse[b] = nullptr;
        p->hs_argb[b] = nullptr;
        p->hs_tf[b] = nullptr;
    }
    p->hs_pixels = 0;
    p->hs_tf_n = 0;
}

static void plan_destroy_host_pipeline(s3r_plan* p)
{
    plan_free_host_slots(p);
    for (int b = 0; b < 2; ++b) {
        for (cudaEvent_t* ev : {&p->hs_copied[b], &p->hs_rendered[b], &p->hs_read[b]}) {
            if (*ev) cudaEventDestroy(*ev);
            *ev = nullptr;
        }
    }
    if (p->hs_entry) cudaEventDestroy(p->hs_entry);
    p->hs_entry = nullptr;
    for (int b = 0; b < 2; ++b) {
        if (p->hs_comp[b]) cudaStreamDestroy(p->hs_comp[b]);
        p->hs_comp[b] = nullptr;
    }
    if (p->hs_h2d) cudaStreamDestroy(p->hs_h2d);
    if (p->hs_d2h) cudaStreamDestroy(p->hs_d2h);
    p->hs_h2d = p->hs_d2h = nullptr;
    if (p->bricks_1) cudaFree(p->bricks_1);
    if (p->scale_offset_1) cudaFree(p->scale_offset_1);
    p->bricks_1 = nullptr;
    p->scale_offset_1 = nullptr;
}

// The GPU work of one s3r_frame_run_host call on slot b: the copies and the frame, with the events that
// order them against the neighbouring frames.
static int frame_host_submit(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* sparse_host,
                             const float* tf, uint32_t* argb_host, cudaStream_t s, int b)
{
    int rc;
    cudaStream_t cb = plan->hs_comp[b];
    const uint64_t pixels = (uint64_t)view->W * view->H;
    // the caller's transfer function is copied on the caller's own stream into slot b's table, once the frame
    // two back (the table's last reader) has finished: work the caller queues on `stream` after this call may
    // then change or free tf
    S3R_CUDA(ctx, cudaStreamWaitEvent(s, plan->hs_rendered[b], 0));
    S3R_CUDA(ctx, cudaMemcpyAsync(plan->hs_tf[b], tf, (size_t)view->tf_n * 4 * sizeof(float), cudaMemcpyDeviceToDevice,
                                  s));
    S3R_CUDA(ctx, cudaEventRecord(plan->hs_entry, s)); // what the caller queued before comes first
    // H2D into slot b once the frame two back no longer reads it
    S3R_CUDA(ctx, cudaStreamWaitEvent(plan->hs_h2d, plan->hs_rendered[b], 0));
    if (plan->nodes)
        S3R_CUDA(ctx, cudaMemcpyAsync(plan->hs_sparse[b], sparse_host, plan->nodes * sizeof(float),
                                      cudaMemcpyHostToDevice, plan->hs_h2d));
    S3R_CUDA(ctx, cudaEventRecord(plan->hs_copied[b], plan->hs_h2d));
    // the frame on slot b's stream -- so that it overlaps the other slot's frame on the GPU -- once its
    // input has landed and the image two frames back has been read out
    S3R_CUDA(ctx, cudaStreamWaitEvent(cb, plan->hs_entry, 0));
    S3R_CUDA(ctx, cudaStreamWaitEvent(cb, plan->hs_copied[b], 0));
    S3R_CUDA(ctx, cudaStreamWaitEvent(cb, plan->hs_read[b], 0));
    if (!plan->have_view || std::memcmp(&plan->last_view, view, sizeof(s3r_view)) != 0) {
        // the render table both slots read changes: let the frames in flight finish first
        for (int q = 0; q < 2; ++q) S3R_CUDA(ctx, cudaStreamSynchronize(plan->hs_comp[q]));
    }
    if ((rc = plan_stage_view(plan, view, cb))) return rc;
    // the table upload may have been queued on the other slot's stream
    S3R_CUDA(ctx, cudaStreamWaitEvent(cb, plan->staged, 0));
    if ((rc = plan_launch_frame(plan, 1 + b, view, plan->hs_sparse[b], plan->hs_tf[b], nullptr, plan->hs_argb[b],
                                nullptr, cb)))
        return rc;
    S3R_CUDA(ctx, cudaEventRecord(plan->hs_rendered[b], cb));
    // D2H of the image while the next frame runs
    S3R_CUDA(ctx, cudaStreamWaitEvent(plan->hs_d2h, plan->hs_rendered[b], 0));
    S3R_CUDA(ctx, cudaMemcpyAsync(argb_host, plan->hs_argb[b], pixels * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                  plan->hs_d2h));
    S3R_CUDA(ctx, cudaEventRecord(plan->hs_read[b], plan->hs_d2h));
    return S3R_OK;
}

int s3r_frame_run_host(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* sparse_host, const float* tf,
                       uint32_t* argb_host, void* stream)
{
    if (!ctx || !plan || !tf || !argb_host || (!sparse_host && plan->nodes))
        return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "plan belongs to another context");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (view->level != plan->level) return fail(ctx, S3R_ERR_INVALID, "view level differs from the plan level");
    if ((rc = set_device(ctx))) return rc;
    cudaError_t e;
    if (!plan->hs_h2d) {
        if ((e = cudaStreamCreateWithFlags(&plan->hs_h2d, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaStreamCreateWithFlags(&plan->hs_d2h, cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_fail(ctx, e, "cudaStreamCreate(host frames)");
        for (int b = 0; b < 2; ++b) {
            if ((e = cudaStreamCreateWithFlags(&plan->hs_comp[b], cudaStreamNonBlocking)) != cudaSuccess)
                return cuda_fail(ctx, e, "cudaStreamCreate(host frames)");
            for (cudaEvent_t* ev : {&plan->hs_copied[b], &plan->hs_rendered[b], &plan->hs_read[b]})
                if ((e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess)
                    return cuda_fail(ctx, e, "cudaEventCreate(host frames)");
        }
        if ((e = cudaEventCreateWithFlags(&plan->hs_entry, cudaEventDisableTiming)) != cudaSuccess)
            return cuda_fail(ctx, e, "cudaEventCreate(host frames)");
    }
    if (!plan->bricks_1) {
        const size_t esz = plan->fmt == S3R_BRICK_F32 ? 4 : 2;
        if ((e = cudaMalloc(&plan->bricks_1, std::max<uint64_t>(plan->brick_elems, 1) * esz)) != cudaSuccess ||
            (e = cudaMalloc(&plan->scale_offset_1, sizeof(float2) * std::max<uint32_t>(plan->nblocks, 1))) != cudaSuccess)
            return cuda_fail(ctx, e, "cudaMalloc(second frame slot)");
    }
    const uint64_t pixels = (uint64_t)view->W * view->H;
    if (pixels != plan->hs_pixels || view->tf_n != plan->hs_tf_n || !plan->hs_sparse[0]) {
        plan_free_host_slots(plan);
        for (int b = 0; b < 2; ++b) {
            if ((e = cudaMalloc(&plan->hs_sparse[b], std::max<uint64_t>(plan->nodes, 1) * sizeof(float))) != cudaSuccess ||
                (e = cudaMalloc(&plan->hs_argb[b], pixels * sizeof(uint32_t))) != cudaSuccess ||
                (e = cudaMalloc(&plan->hs_tf[b], (size_t)view->tf_n * 4 * sizeof(float))) != cudaSuccess) {
                plan_free_host_slots(plan);
                return cuda_fail(ctx, e, "cudaMalloc(host frames)");
            }
        }
        plan->hs_pixels = pixels;
        plan->hs_tf_n = view->tf_n;
    }
    const int b = (int)(plan->hs_frames & 1);
    if ((rc = frame_host_submit(ctx, plan, view, sparse_host, tf, argb_host, as_stream(stream), b))) {
        // a step failed part way: let everything already queued finish, so that the next call starts from
        // a pipeline whose events all stand for completed work
        cudaStreamSynchronize(plan->hs_h2d);
        for (int q = 0; q < 2; ++q) cudaStreamSynchronize(plan->hs_comp[q]);
        cudaStreamSynchronize(plan->hs_d2h);
        return rc;
    }
    ++plan->hs_frames;
    // on return this frame's input buffer is free and the previous frame's image is in host memory; the GPU
    // meanwhile renders the previous frame and then this one
    S3R_CUDA(ctx, cudaEventSynchronize(plan->hs_copied[b]));
    if (plan->hs_frames > 1) S3R_CUDA(ctx, cudaEventSynchronize(plan->hs_read[b ^ 1]));
    return S3R_OK;
}

int s3r_frame_host_sync(s3r_ctx* ctx, s3r_plan* plan)
{
    if (!ctx || !plan) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (!plan->hs_d2h) return S3R_OK;
    int rc = set_device(ctx);
    if (rc) return rc;
    S3R_CUDA(ctx, cudaStreamSynchronize(plan->hs_h2d));
    for (int b = 0; b < 2; ++b) S3R_CUDA(ctx, cudaStreamSynchronize(plan->hs_comp[b]));
    S3R_CUDA(ctx, cudaStreamSynchronize(plan->hs_d2h));
    return S3R_OK;
}

int s3r_plan_autotune(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* sparse, const float* tf,
                      uint32_t reps, void* stream)
{
    if (!ctx || !plan || !tf || (!sparse && plan->nodes)) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "plan belongs to another context");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (view->level != plan->level) return fail(ctx, S3R_ERR_INVALID, "view level differs from the plan level");
    if ((rc = set_device(ctx))) return rc;
    if (reps == 0) reps = 3;
    cudaStream_t s = as_stream(stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float* img = nullptr;
    auto cleanup = [&](int code) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (img) cudaFree(img);
        return code;
    };
    cudaError_t e;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess ||
        (e = cudaMalloc(&img, sizeof(float) * 4 * (size_t)view->W * view->H)) != cudaSuccess)
        return cleanup(cuda_fail(ctx, e, "autotune set-up"));
    auto timed = [&](auto&& body, float& ms) -> int {
        uint32_t k = 0;
        int r = body(&k); // warm-up
        if (r) return r;
        if ((e = cudaEventRecord(e0, s)) != cudaSuccess) return cuda_fail(ctx, e, "cudaEventRecord");
        for (uint32_t i = 0; i < reps; ++i)
            if ((r = body(&k))) return r;
        if ((e = cudaEventRecord(e1, s)) != cudaSuccess) return cuda_fail(ctx, e, "cudaEventRecord");
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return cuda_fail(ctx, e, "cudaEventSynchronize");
        cudaEventElapsedTime(&ms, e0, e1);
        ctx->launches += k;
        return S3R_OK;
    };
    uint32_t best_tl = plan->tile_log2;
    float best = 3.4e38f;
    for (uint32_t tl = 3; tl <= 5; ++tl) {
        if ((rc = plan_bin(plan, tl))) return cleanup(rc);
        float ms = 0;
        rc = timed([&](uint32_t* k) { return plan_launch_interp(plan, sparse, s, k); }, ms);
        if (rc) return cleanup(rc);
        if (ms < best) {
            best = ms;
            best_tl = tl;
        }
    }
    // then per block depth (deepest first): a smaller tile for that depth's blocks alone, kept when faster
    // (never a larger one: the largest tile sets every CTA's shared memory)
    uint8_t by_depth[S3R_MAX_DEPTH + 1];
    for (uint32_t d = 0; d <= S3R_MAX_DEPTH; ++d) by_depth[d] = (uint8_t)std::min(best_tl, d);
    bool present[S3R_MAX_DEPTH + 1] = {};
    for (uint32_t b = 0; b < plan->nblocks; ++b) present[plan->blocks[4 * b + 3]] = true;
    for (int d = S3R_MAX_DEPTH; d >= 4; --d) {
        if (!present[d] || by_depth[d] <= 3) continue;
        const uint8_t keep = by_depth[d];
        by_depth[d] = (uint8_t)(keep - 1);
        if ((rc = plan_bin(plan, best_tl, by_depth))) return cleanup(rc);
        float ms = 0;
        rc = timed([&](uint32_t* k) { return plan_launch_interp(plan, sparse, s, k); }, ms);
        if (rc) return cleanup(rc);
        if (ms < best) best = ms;
        else by_depth[d] = keep;
    }
    if ((rc = plan_bin(plan, best_tl, by_depth))) return cleanup(rc);
    uint32_t k = 0;
    if ((rc = plan_launch_interp(plan, sparse, s, &k))) return cleanup(rc);
    ctx->launches += k;
    if ((rc = plan_stage_view(plan, view, s))) return cleanup(rc);
    uint32_t best_shape = plan->render_tile;
    best = 3.4e38f;
    for (uint32_t shape = 0; shape < (uint32_t)kRenderTiles; ++shape) {
        // several lanes per ray only where rays composite every block (alpha_stop >= 1)
        if (shape >= (uint32_t)kRenderShapes && shape < (uint32_t)kRenderWalkTiles && view->alpha_stop < 1.f) continue;
        plan->render_tile = shape;
        // the block-major forms' buffers and their footprint's work items
        if (shape >= (uint32_t)kRenderWalkTiles && plan_stage_view(plan, view, s) != S3R_OK) {
            // no room for the block-major buffers: keep to the per-ray walk
            ctx->err.clear();
            set_thread_error("");
            continue;
        }
        float ms = 0;
        rc = timed([&](uint32_t* kk) { return plan_launch_render(plan, tf, img, nullptr, nullptr, s, kk); }, ms);
        if (rc) return cleanup(rc);
        if (ms < best) {
            best = ms;
            best_shape = shape;
        }
    }
    plan->render_tile = best_shape;
    plan_drop_graph(plan);
    if (best_shape < (uint32_t)kRenderWalkTiles) {
        // the per-ray walk won: release the block-major buffers
        cudaStreamSynchronize(s);
        plan_free_segments(plan);
    }
    return cleanup(S3R_OK);
}

int s3r_render_argb_backward(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* tf, const float* rgba,
                             const float* dl_drgba, float* dtf, float* ddense, void* stream)
{
    if (!ctx || !plan || !tf || !rgba || !dl_drgba || !dtf || !ddense)
        return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->fmt != S3R_BRICK_F32) return fail(ctx, S3R_ERR_UNSUPPORTED, "the adjoint needs FP32 bricks");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (view->filter != S3R_FILTER_EXACT)
        return fail(ctx, S3R_ERR_UNSUPPORTED, "the adjoint needs S3R_FILTER_EXACT (texture weights are piecewise constant)");
    if (view->level != plan->level) return fail(ctx, S3R_ERR_INVALID, "view level differs from the plan level");
    if ((rc = set_device(ctx))) return rc;
    cudaStream_t s = as_stream(stream);
    if ((rc = plan_stage_view(plan, view, s))) return rc;
    FrameArgs fa{};
    fa.view = plan->view_dev;
    fa.table = plan->table_dev;
    fa.bricks = plan->bricks;
    fa.tf = tf;
    fa.fwd_rgba = rgba;
    fa.dl_drgba = dl_drgba;
    fa.dtf = dtf;
    fa.ddense = ddense;
    const size_t nparts = (size_t)kDtfParts * 4 * view->tf_n;
    if (plan->dtf_part_floats < nparts) {
        // allocation: synchronizes the device once, on the first adjoint call (or a larger table)
        if (plan->dtf_part) cudaFree(plan->dtf_part);
        plan->dtf_part = nullptr;
        plan->dtf_part_floats = 0;
        cudaError_t e = cudaMalloc(&plan->dtf_part, nparts * sizeof(float));
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(transfer-function gradient copies)");
        plan->dtf_part_floats = nparts;
    }
    fa.dtf_part = plan->dtf_part;
    S3R_CUDA(ctx, cudaMemsetAsync(plan->dtf_part, 0, nparts * sizeof(float), s));
    S3R_CUDA(ctx, launch_frame_backward(fa, view->W, view->H, view->tf_n, s));
    S3R_CUDA(ctx, launch_dtf_reduce(plan->dtf_part, dtf, 4 * view->tf_n, s));
    ctx->launches += 2;
    return S3R_OK;
}

} // extern "C"

extern "C" {

int s3r_render_scene_part(s3r_ctx* ctx, const s3r_view* view, const s3r_presentation* pres,
                          const s3r_worker_blocks* wb, const uint32_t box_min[3], const uint32_t box_max[3],
                          const float* tf, uint32_t* viewport, int32_t rect[4], void* stream)
{
    if (!ctx) return fail(nullptr, S3R_ERR_INVALID, "ctx is null");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (!wb || !box_min || !box_max || !tf || !viewport || !rect) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (wb->nblocks && (!wb->blocks || !wb->node_off || !wb->n2i || !wb->sparse))
        return fail(ctx, S3R_ERR_INVALID, "null block data");
    const bool secondary = pres && (pres->mode == S3R_MODE_VALUE_ON_ISOSURFACE ||
                                    pres->mode == S3R_MODE_VALUE_ON_ISOSURFACES);
    if (secondary && !wb->sparse2) return fail(ctx, S3R_ERR_INVALID, "this mode needs the secondary field");
    if ((rc = set_device(ctx))) return rc;
    const cudaStream_t s = as_stream(stream);
    const uint32_t clear = pres && pres->mode == S3R_MODE_MAX_INTENSITY ? 0x7fc00000u : 0u;
    if ((rc = s3r_clear_viewport(ctx, viewport, view->W, view->H, clear, stream))) return rc;
    // the box's blocks back to front (MacroBlock over the box, the view's eye)
    double cmin[3], cmax[3];
    if ((rc = s3r_index_box_world(view->level, box_min, box_max, cmin, cmax))) return rc;
    Split sp[3];
    for (int a = 0; a < 3; ++a)
        sp[a] = split_range(box_min[a], box_max[a], (float)cmin[a], (float)cmax[a], view->cam.eye[a]);
    // the texture filter samples through the texture unit, as the reference's renderer does: the transfer
    // function goes into the context's colour texture first
    const bool tex = view->filter == S3R_FILTER_TEXTURE;
    if (tex) {
        if (ctx->worker_tf && ctx->worker_tf->n != view->tf_n) {
            s3r_tf_texture_destroy(ctx->worker_tf);
            ctx->worker_tf = nullptr;
        }
        if (!ctx->worker_tf && (rc = s3r_tf_texture_create(ctx, view->tf_n, &ctx->worker_tf))) return rc;
        if ((rc = s3r_tf_texture_set(ctx, ctx->worker_tf, tf, stream))) return rc;
    }
    std::unordered_map<uint64_t, uint32_t> where;
    where.reserve(wb->nblocks * 2 + 1);
    for (uint32_t b = 0; b < wb->nblocks; ++b) {
        const uint32_t* bl = wb->blocks + 4 * b;
        where[(uint64_t)bl[0] | ((uint64_t)bl[1] << 21) | ((uint64_t)bl[2] << 42)] = b;
    }
    b2f_traverse(sp, [&](const uint32_t q[3]) {
        if (rc) return;
        auto it = where.find((uint64_t)q[0] | ((uint64_t)q[1] << 21) | ((uint64_t)q[2] << 42));
        if (it == where.end()) return; // not a block of this set
        const uint32_t b = it->second;
        const uint32_t depth = wb->blocks[4 * b + 3];
        if (depth > S3R_MAX_DEPTH) {
            rc = fail(ctx, S3R_ERR_INVALID, "depth exceeds S3R_MAX_DEPTH");
            return;
        }
        const uint64_t o = wb->node_off[b], n = wb->node_off[b + 1] - o;
        if (tex) {
            // DeviceField::makeField: the block's dense field interpolated into the depth's field texture
            for (int f = 0; f < (secondary ? 2 : 1); ++f) {
                if (!ctx->worker_tex[f][depth] && (rc = s3r_texture_create(ctx, depth, &ctx->worker_tex[f][depth])))
                    return;
                if ((rc = s3r_interp_dense_texture(ctx, wb->n2i + 3 * o, (f ? wb->sparse2 : wb->sparse) + o,
                                                   (uint32_t)n, ctx->worker_tex[f][depth], stream)))
                    return;
            }
            int32_t r[4];
            view_rect(*view, wb->blocks + 4 * b, r);
            if (r[2] <= 0 || r[3] <= 0) return;
            rc = s3r_render_block_texture(ctx, view, pres, ctx->worker_tex[0][depth],
                                          secondary ? ctx->worker_tex[1][depth] : nullptr, wb->blocks + 4 * b, r,
                                          ctx->worker_tf, viewport, stream);
            return;
        }
        const uint64_t e = (1ull << depth) + 1, count = e * e * e;
        for (int f = 0; f < (secondary ? 2 : 1); ++f)
            if (ctx->worker_cap[f] < count) {
                if (ctx->worker_dense[f]) cudaFree(ctx->worker_dense[f]);
                ctx->worker_dense[f] = nullptr;
                ctx->worker_cap[f] = 0;
                const cudaError_t err = cudaMalloc(&ctx->worker_dense[f], count * sizeof(float));
                if (err != cudaSuccess) {
                    rc = cuda_fail(ctx, err, "cudaMalloc(worker dense field)");
                    return;
                }
                ctx->worker_cap[f] = count;
            }
        // DeviceField::makeField: the block's dense field from its nodes
        if ((rc = s3r_interp_dense(ctx, wb->n2i + 3 * o, wb->sparse + o, (uint32_t)n, depth, ctx->worker_dense[0],
                                   stream)))
            return;
        if (secondary && (rc = s3r_interp_dense(ctx, wb->n2i + 3 * o, wb->sparse2 + o, (uint32_t)n, depth,
                                                ctx->worker_dense[1], stream)))
            return;
        int32_t r[4];
        view_rect(*view, wb->blocks + 4 * b, r);
        if (r[2] <= 0 || r[3] <= 0) return;
        rc = pres ? s3r_render_block(ctx, view, pres, ctx->worker_dense[0], secondary ? ctx->worker_dense[1] : nullptr,
                                     depth, wb->blocks + 4 * b, r, tf, viewport, stream)
                  : s3r_render_block_argb(ctx, view, ctx->worker_dense[0], depth, wb->blocks + 4 * b, r, tf, viewport,
                                          stream);
    });
    if (rc) return rc;
    (void)s;
    return s3r_bound_rect(ctx, viewport, view->W, view->H, rect, stream);
}

} // extern "C"

extern "C" {

int s3r_render_scene_part_bricks(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const s3r_presentation* pres,
                                 const void* bricks2, const uint32_t box_min[3], const uint32_t box_max[3],
                                 const float* tf, uint32_t* viewport, int32_t rect[4], void* stream)
{
    if (!ctx || !plan) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->ctx != ctx) return fail(ctx, S3R_ERR_INVALID, "plan belongs to another context");
    int rc = check_view(ctx, view);
    if (rc) return rc;
    if (view->level != plan->level) return fail(ctx, S3R_ERR_INVALID, "view level differs from the plan level");
    if (!box_min || !box_max || !tf || !viewport || !rect) return fail(ctx, S3R_ERR_INVALID, "null pointer");
    if (plan->fmt != S3R_BRICK_F32) return fail(ctx, S3R_ERR_UNSUPPORTED, "the per-block renderer reads F32 bricks");
    const bool secondary = pres && (pres->mode == S3R_MODE_VALUE_ON_ISOSURFACE ||
                                    pres->mode == S3R_MODE_VALUE_ON_ISOSURFACES);
    if (secondary && !bricks2) return fail(ctx, S3R_ERR_INVALID, "this mode needs the secondary bricks");
    if ((rc = set_device(ctx))) return rc;
    const uint32_t clear = pres && pres->mode == S3R_MODE_MAX_INTENSITY ? 0x7fc00000u : 0u;
    if ((rc = s3r_clear_viewport(ctx, viewport, view->W, view->H, clear, stream))) return rc;
    double cmin[3], cmax[3];
    if ((rc = s3r_index_box_world(view->level, box_min, box_max, cmin, cmax))) return rc;
    Split sp[3];
    for (int a = 0; a < 3; ++a)
        sp[a] = split_range(box_min[a], box_max[a], (float)cmin[a], (float)cmax[a], view->cam.eye[a]);
    const uint32_t m = 1u << plan->level;
    std::vector<int32_t> where((size_t)m * m * m, -1);
    for (uint32_t b = 0; b < plan->nblocks; ++b) {
        const uint32_t* bl = &plan->blocks[4 * b];
        where[bl[0] + m * (bl[1] + (size_t)m * bl[2])] = (int32_t)b;
    }
    const float* bricks = static_cast<const float*>(plan->bricks);
    const float* b2 = static_cast<const float*>(bricks2);
    b2f_traverse(sp, [&](const uint32_t q[3]) {
        if (rc) return;
        if (q[0] >= m || q[1] >= m || q[2] >= m) return;
        const int32_t b = where[q[0] + m * (q[1] + (size_t)m * q[2])];
        if (b < 0) return;
        const uint32_t* bl = &plan->blocks[4 * b];
        int32_t r[4];
        view_rect(*view, bl, r);
        if (r[2] <= 0 || r[3] <= 0) return;
        const uint64_t o = plan->vertex_off[b];
        const uint32_t pitch = plan->pitch[b];
        rc = pres ? render_block_pitched(ctx, view, pres, bricks + o, secondary ? b2 + o : nullptr, bl[3], pitch, bl,
                                         r, tf, viewport, stream)
                  : render_block_argb_pitched(ctx, view, bricks + o, bl[3], pitch, bl, r, tf, viewport, stream);
    });
    if (rc) return rc;
    return s3r_bound_rect(ctx, viewport, view->W, view->H, rect, stream);
}

} // extern "C"
