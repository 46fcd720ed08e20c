// Block ray casting for sm_103a.
//
// Restates renderKernel<FieldMode::Argb> + renderArgb of the reference
// (src/s3dmm_cuda/DenseFieldRenderer_cu.cu:62-215, src/s3dmm_cuda/renderArgb.hpp:30-55,
// cuda_blend.hpp:24-44, cuda_argb_transform.hpp:26-43) without texture
// hardware: bricks are linear arrays in HBM read through the read-only path,
// filtered in FP32 by software trilinear interpolation with clamp addressing
// (a sample whose 8 texels hold a NaN is skipped, as the texture unit's
// weighted sum would be NaN); the transfer function sits in shared memory.
//
// Ray set-up (per-pixel ray, per-block slab test, sample count and positions)
// is written with explicitly rounded operations (__fadd_rn, __fmul_rn, ...)
// so that it cannot be contracted and the CPU oracle reproduces the same
// sample positions bit for bit.  The sample loop keeps the reference's
// indexing: sample k = i-1 for i = 1 .. sampleCount-1, at entry + k*step,
// computed directly (fma) rather than by accumulation.
//
// Kernels:
//   render_block_argb_kernel  one block into an ARGB8 viewport (drop-in form):
//                             reference non-premultiplied blending, ARGB8
//                             read-modify-write per block;
//   frame_render_kernel       batched form: each ray walks the block grid front
//                             to back (3D DDA), marches every block it enters
//                             exactly as above, composites block results with
//                             the over operator in FP32 (premultiplied), and
//                             stops once alpha passes view.alpha_stop;
//   frame_backward_kernel     adjoint of frame_render_kernel w.r.t. the
//                             transfer function and the dense values; re-walks
//                             each ray instead of storing samples.
#include "s3r_internal.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace s3r {
namespace {

constexpr float kAlphaThreshold = 0.996f; // renderArgb.hpp:47
constexpr float kTopHalf = 5.f;           // DenseFieldRenderer_cu.cu:339

struct BlockRay {
    float tau_enter;
    float tau_exit;
    int samples;
    float p0[3];
    float step[3];
    float origin[3];
    float factor;
    uint32_t n;     // vertices per axis, 2^depth+1
    uint32_t pitch; // row pitch of the brick in elements (>= n)
};

// A brick's extent and row pitch: vertex (x, y, z) is element (z n + y) pitch + x.
struct Dim {
    uint32_t n, pitch;
};
__device__ __forceinline__ Dim dim_of(const BlockRay& r) { return Dim{r.n, r.pitch}; }

__device__ __forceinline__ void pixel_ray(const s3r_view& v, uint32_t vx, uint32_t vy, float org[3], float dir[3])
{
    const float x = __fmul_rn(__fadd_rn(-0.5f, __fdiv_rn(__fadd_rn((float)vx, 0.5f), (float)v.W)), v.cam.w);
    const float y = __fmul_rn(__fadd_rn(-0.5f, __fdiv_rn(__fadd_rn((float)vy, 0.5f), (float)v.H)), v.cam.h);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float ex = __fmul_rn(v.cam.e1[d], x);
        const float ey = __fmul_rn(v.cam.e2[d], y);
        if (v.cam.ortho) {
            org[d] = __fadd_rn(__fadd_rn(v.cam.eye[d], ex), ey);
            dir[d] = v.cam.n[d];
        } else {
            org[d] = v.cam.eye[d];
            dir[d] = __fadd_rn(__fadd_rn(v.cam.n[d], ex), ey);
        }
    }
}

// Slab test and sample set-up (DenseFieldRenderer_cu.cu:81-181). Returns true
// when the block is rendered for this ray.
__device__ __forceinline__ bool block_ray(const s3r_view& v, const float org[3], const float dir[3],
                                          const RenderBlock& rb, BlockRay& r)
{
    const float* c = rb.center;
    const float h = rb.half;
    float te = 1.f, tx = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!(fabsf(dir[a]) > 1e-10f)) continue;
        const int b1 = a == 0 ? 1 : 0;
        const int b2 = a == 2 ? 1 : 2;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const float face = side ? __fadd_rn(c[a], h) : __fsub_rn(c[a], h);
            const float tau = __fdiv_rn(__fsub_rn(face, org[a]), dir[a]);
            const float p1 = __fadd_rn(org[b1], __fmul_rn(dir[b1], tau));
            const float p2 = __fadd_rn(org[b2], __fmul_rn(dir[b2], tau));
            if (fabsf(__fsub_rn(p1, c[b1])) <= h && fabsf(__fsub_rn(p2, c[b2])) <= h) {
                const bool enter = (dir[a] > 0.f) == (side == 0);
                if (enter) te = tau;
                else tx = tau;
            }
        }
    }
    if (te < 1.f) te = 1.f;
    r.tau_enter = te;
    r.tau_exit = tx;
    if (!(tx > te)) return false;
    const uint32_t n = (1u << rb.depth) + 1u;
    const float texel = rb.texel;
    const float span = __fsub_rn(tx, te);
    const float dotr = __fadd_rn(__fadd_rn(__fmul_rn(dir[0], dir[0]), __fmul_rn(dir[1], dir[1])),
                                 __fmul_rn(dir[2], dir[2]));
    const float l1 = __fadd_rn(__fadd_rn(fabsf(dir[0]), fabsf(dir[1])), fabsf(dir[2]));
    const float num = __fmul_rn(__fmul_rn(v.quality, span), dotr);
    const float den = __fmul_rn(texel, l1);
    const int s = __float2int_rz(__fdiv_rn(num, den));
    const float dtau = __fdiv_rn(span, (float)s);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        r.step[d] = __fmul_rn(dir[d], dtau);
        r.p0[d] = __fadd_rn(org[d], __fmul_rn(dir[d], te));
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) r.origin[d] = rb.origin[d];
    r.factor = rb.factor;
    r.n = n;
    r.pitch = rb.pitch ? rb.pitch : n;
    r.samples = s;
    return true;
}

struct Cell {
    uint32_t i0[3], i1[3];
    float f[3];
};

__device__ __forceinline__ void sample_cell(const BlockRay& r, int k, Cell& c)
{
    const int hi = (int)r.n - 1;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float p = __fmaf_rn(r.step[d], (float)k, r.p0[d]);
        const float tc = __fmul_rn(__fsub_rn(p, r.origin[d]), r.factor);
        const float xb = __fsub_rn(tc, 0.5f);
        const float fl = floorf(xb);
        c.f[d] = __fsub_rn(xb, fl);
        const int a = (int)fl, b = a + 1;
        c.i0[d] = (uint32_t)min(max(a, 0), hi);
        c.i1[d] = (uint32_t)min(max(b, 0), hi);
    }
}

// 8 texels of a cell from a brick of format Fmt, decoded to float.
template <int Fmt> struct Brick;
template <> struct Brick<S3R_BRICK_F32> {
    __device__ static float get(const void* b, uint64_t i) { return __ldg(reinterpret_cast<const float*>(b) + i); }
};
template <> struct Brick<S3R_BRICK_F16> {
    __device__ static float get(const void* b, uint64_t i)
    {
        return __half2float(__ldg(reinterpret_cast<const __half*>(b) + i));
    }
};
template <> struct Brick<S3R_BRICK_BF16> {
    __device__ static float get(const void* b, uint64_t i)
    {
        return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(b) + i));
    }
};

template <int Fmt>
__device__ __forceinline__ bool trilinear(const void* brick, const Cell& c, Dim g, float& val, float t[8],
                                          uint64_t off[8])
{
    const uint64_t n64 = g.n, p64 = g.pitch;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint64_t x = (q & 1) ? c.i1[0] : c.i0[0];
        const uint64_t y = (q & 2) ? c.i1[1] : c.i0[1];
        const uint64_t z = (q & 4) ? c.i1[2] : c.i0[2];
        off[q] = (z * n64 + y) * p64 + x;
        t[q] = Brick<Fmt>::get(brick, off[q]);
    }
    bool bad = false;
#pragma unroll
    for (int q = 0; q < 8; ++q) bad |= isnan(t[q]);
    if (bad) return false;
    const float x00 = __fmaf_rn(c.f[0], t[1] - t[0], t[0]);
    const float x10 = __fmaf_rn(c.f[0], t[3] - t[2], t[2]);
    const float x01 = __fmaf_rn(c.f[0], t[5] - t[4], t[4]);
    const float x11 = __fmaf_rn(c.f[0], t[7] - t[6], t[6]);
    const float y0 = __fmaf_rn(c.f[1], x10 - x00, x00);
    const float y1 = __fmaf_rn(c.f[1], x11 - x01, x01);
    val = __fmaf_rn(c.f[2], y1 - y0, y0);
    return true;
}

// ---------------------------------------------------------------- texture-unit filtering
//
// S3R_FILTER_TEXTURE: the linear filtering the GPU texture unit applies to the
// reference's clamped float textures (measured on this GPU with one-hot
// textures over a lattice of coordinates).  Per axis xb = coordinate - 0.5,
// texels floor(xb) and floor(xb)+1 (clamped), fraction a = floor(frac * 256 +
// 1/2) in 0..256.  1D: weights (256 - a, a) / 256.  3D: the z split is exact
// (zt = 256 - c | c); in each z half xh = rn(a * zt), xl = zt - xh; the y split
// rounds the y-high part under xh (rn(xh * b)) and the y-low part under xl
// (rn(xl * (256 - b))), the rest going to the other side, rn(p) = (p + 128) >> 8.
// A NaN texel makes the sample NaN when its per-axis factors are all nonzero.

struct TexAxis {
    uint32_t i0, i1;
    int32_t a; // 0..256
};

__device__ __forceinline__ TexAxis tex_axis(float tc, int hi)
{
    const float xb = __fsub_rn(tc, 0.5f);
    // xb * 256 is exact, so the one rounding of the fma cannot carry floor() past an integer
    const float q = floorf(__fmaf_rn(xb, 256.f, 0.5f));
    const float fl = floorf(__fmul_rn(q, 0.00390625f));
    TexAxis t;
    t.a = (int32_t)__fmaf_rn(fl, -256.f, q);
    const int lo = (int)fmaxf(fminf(fl, 1e9f), -1e9f);
    t.i0 = (uint32_t)min(max(lo, 0), hi);
    t.i1 = (uint32_t)min(max(lo + 1, 0), hi);
    return t;
}

__device__ __forceinline__ int32_t rn8(int32_t x, int32_t y) { return (x * y + 128) >> 8; }

// Texel coordinate of sample k along axis d (the fetch coordinate of the reference).
__device__ __forceinline__ float sample_tc(const BlockRay& r, int k, int d)
{
    const float p = __fmaf_rn(r.step[d], (float)k, r.p0[d]);
    return __fmul_rn(__fsub_rn(p, r.origin[d]), r.factor);
}

template <int Fmt> struct Brick;

template <int Fmt>
__device__ __forceinline__ bool tex_trilinear_at(const void* brick, Dim g, float tcx, float tcy, float tcz,
                                                 float& val)
{
    const int hi = (int)g.n - 1;
    const TexAxis x = tex_axis(tcx, hi);
    const TexAxis y = tex_axis(tcy, hi);
    const TexAxis z = tex_axis(tcz, hi);
    int32_t w[8];
#pragma unroll
    for (int hz = 0; hz < 2; ++hz) {
        const int32_t zt = hz ? z.a : 256 - z.a;
        const int32_t xh = rn8(x.a, zt), xl = zt - xh;
        const int32_t yhh = rn8(xh, y.a), yll = rn8(xl, 256 - y.a);
        w[3 | (hz << 2)] = yhh;
        w[1 | (hz << 2)] = xh - yhh;
        w[hz << 2] = yll;
        w[2 | (hz << 2)] = xl - yll;
    }
    const uint64_t n64 = g.n, p64 = g.pitch;
    float t[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint64_t xi = (q & 1) ? x.i1 : x.i0;
        const uint64_t yi = (q & 2) ? y.i1 : y.i0;
        const uint64_t zi = (q & 4) ? z.i1 : z.i0;
        t[q] = Brick<Fmt>::get(brick, (zi * n64 + yi) * p64 + xi);
    }
    // per-axis factor nonzero: the low texel needs a < 256, the high one a > 0
    const bool lx = x.a < 256, hx = x.a > 0, ly = y.a < 256, hy = y.a > 0, lz = z.a < 256, hz = z.a > 0;
    bool bad = false;
    float acc = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const bool inx = (q & 1) ? hx : lx, iny = (q & 2) ? hy : ly, inz = (q & 4) ? hz : lz;
        if (isnan(t[q])) bad |= inx && iny && inz;
        else acc = __fmaf_rn((float)w[q], t[q], acc);
    }
    if (bad) return false;
    val = __fmul_rn(acc, 0.00390625f);
    return true;
}

template <int Fmt>
__device__ __forceinline__ bool tex_trilinear(const void* brick, const BlockRay& r, int k, float& val)
{
    return tex_trilinear_at<Fmt>(brick, dim_of(r), sample_tc(r, k, 0), sample_tc(r, k, 1), sample_tc(r, k, 2), val);
}

struct TfSample {
    float4 c;
    uint32_t i0, i1;
    float f;
    bool clamped;
};

__device__ __forceinline__ float4 tex_tf_lookup(const float4* tf, uint32_t tfn, float v01)
{
    const TexAxis u = tex_axis(__fmul_rn(v01, (float)tfn), (int)tfn - 1);
    const float4 p = tf[u.i0], q = tf[u.i1];
    const float wl = (float)(256 - u.a), wh = (float)u.a;
    float4 c;
    c.x = __fmul_rn(__fmaf_rn(wh, q.x, __fmul_rn(wl, p.x)), 0.00390625f);
    c.y = __fmul_rn(__fmaf_rn(wh, q.y, __fmul_rn(wl, p.y)), 0.00390625f);
    c.z = __fmul_rn(__fmaf_rn(wh, q.z, __fmul_rn(wl, p.z)), 0.00390625f);
    c.w = __fmul_rn(__fmaf_rn(wh, q.w, __fmul_rn(wl, p.w)), 0.00390625f);
    return c;
}

// tex1D with normalized coordinates, linear filtering, clamp addressing.
__device__ __forceinline__ TfSample tf_lookup(const float4* tf, uint32_t tfn, float v01)
{
    TfSample s;
    const float u = __fmaf_rn(v01, (float)tfn, -0.5f);
    const float fl = floorf(u);
    s.f = u - fl;
    const int hi = (int)tfn - 1;
    const int a = (int)fmaxf(fminf(fl, 1e9f), -1e9f), b = a + 1;
    s.clamped = a < 0 || b > hi;
    s.i0 = (uint32_t)min(max(a, 0), hi);
    s.i1 = (uint32_t)min(max(b, 0), hi);
    const float4 p = tf[s.i0], q = tf[s.i1];
    s.c.x = __fmaf_rn(s.f, q.x - p.x, p.x);
    s.c.y = __fmaf_rn(s.f, q.y - p.y, p.y);
    s.c.z = __fmaf_rn(s.f, q.z - p.z, p.z);
    s.c.w = __fmaf_rn(s.f, q.w - p.w, p.w);
    return s;
}

__device__ __forceinline__ float layer_exponent(uint32_t depth, uint32_t level, float quality)
{
    return __fmul_rn(__fdiv_rn(1.f, __fmul_rn((float)(1u << (depth + level)), quality)), 100.f);
}

__device__ __forceinline__ float4 argb_to_rgba(uint32_t p)
{
    return make_float4((float)((p >> 16) & 0xffu) / 255.f, (float)((p >> 8) & 0xffu) / 255.f,
                       (float)(p & 0xffu) / 255.f, (float)((p >> 24) & 0xffu) / 255.f);
}

__device__ __forceinline__ uint32_t rgba_to_argb(float4 c)
{
    return ((uint32_t)(c.w * 255.999f) << 24) + ((uint32_t)(c.x * 255.999f) << 16) +
           ((uint32_t)(c.y * 255.999f) << 8) + (uint32_t)(c.z * 255.999f);
}

// ---------------------------------------------------------------- plain form

__global__ void render_block_argb_kernel(const s3r_view v, const float* __restrict__ brick, const RenderBlock rb,
                                         const float4* __restrict__ tf_g, uint32_t* __restrict__ viewport)
{
    const uint32_t depth = rb.depth;
    const int32_t rx = rb.rect[0], ry = rb.rect[1], rw = rb.rect[2], rh = rb.rect[3];
    extern __shared__ float4 tf[];
    for (uint32_t i = threadIdx.y * blockDim.x + threadIdx.x; i < v.tf_n; i += blockDim.x * blockDim.y)
        tf[i] = tf_g[i];
    __syncthreads();
    const int32_t xx = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t yy = blockIdx.y * blockDim.y + threadIdx.y;
    if (xx >= rw || yy >= rh) return;
    const uint32_t vx = (uint32_t)(rx + xx), vy = (uint32_t)(ry + yy);
    if (vx >= v.W || vy >= v.H) return;
    float org[3], dir[3];
    pixel_ray(v, vx, vy, org, dir);
    BlockRay r;
    if (!block_ray(v, org, dir, rb, r)) return;
    const float span = v.field_max - v.field_min;
    const float of = (v.threshold - v.field_min) / span;
    const float il = layer_exponent(depth, v.level, v.quality);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool tex = v.filter == S3R_FILTER_TEXTURE;
    float tp[3] = {r.p0[0], r.p0[1], r.p0[2]}; // texture filter: accumulated position (increase(pos, step))
    for (int i = 1; i < r.samples; ++i) {
        float val;
        if (tex) {
            const float tcx = __fmul_rn(__fsub_rn(tp[0], r.origin[0]), r.factor);
            const float tcy = __fmul_rn(__fsub_rn(tp[1], r.origin[1]), r.factor);
            const float tcz = __fmul_rn(__fsub_rn(tp[2], r.origin[2]), r.factor);
#pragma unroll
            for (int d = 0; d < 3; ++d) tp[d] = __fadd_rn(tp[d], r.step[d]);
            if (!tex_trilinear_at<S3R_BRICK_F32>(brick, dim_of(r), tcx, tcy, tcz, val)) continue;
        } else {
            Cell cell;
            sample_cell(r, i - 1, cell);
            float t[8];
            uint64_t off[8];
            if (!trilinear<S3R_BRICK_F32>(brick, cell, dim_of(r), val, t, off)) continue;
        }
        const float v01 = (val - v.field_min) / span;
        float4 col = tex ? tex_tf_lookup(tf, v.tf_n, v01) : tf_lookup(tf, v.tf_n, v01).c;
        col.w = 1.f - powf(1.f - col.w * of, il); // the reference's pow on floats
        // blendBehind (cuda_blend.hpp:24-33)
        const float da = col.w * (1.f - acc.w);
        const float a = acc.w + da;
        if (a > 0.f) {
            const float ka = acc.w / a, kd = da / a;
            acc.x = acc.x * ka + col.x * kd;
            acc.y = acc.y * ka + col.y * kd;
            acc.z = acc.z * ka + col.z * kd;
        }
        acc.w = a;
        if (acc.w > kAlphaThreshold) break;
    }
    uint32_t* px = &viewport[(size_t)(v.H - 1 - vy) * v.W + vx];
    float4 ex = argb_to_rgba(*px);
    // blendAbove (cuda_blend.hpp:35-44)
    const float da = ex.w * (1.f - acc.w);
    const float a = acc.w + da;
    if (a > 0.f) {
        const float kd = da / a, ki = acc.w / a;
        ex.x = ex.x * kd + acc.x * ki;
        ex.y = ex.y * kd + acc.y * ki;
        ex.z = ex.z * kd + acc.z * ki;
    }
    ex.w = a;
    *px = rgba_to_argb(ex);
}

// ---------------------------------------------------------------- field modes (plain form)
//
// renderKernel<mode> with the reference's render functions (render*.hpp) and
// lighting (cuda_lighting.hpp), on the plain form's ray set-up and sampling.

// Field value at texel coordinate (x, y, z) -- the reference's fetch
// coordinate -- filtered as kTex says; NaN where the filter gives NaN.
template <bool kTex>
__device__ __forceinline__ float field_at(const float* brick, Dim n, float x, float y, float z)
{
    float val;
    if constexpr (kTex) {
        if (!tex_trilinear_at<S3R_BRICK_F32>(brick, n, x, y, z, val)) return __int_as_float(0x7fc00000);
        return val;
    } else {
        Cell c;
        const int hi = (int)n.n - 1;
        const float tc[3] = {x, y, z};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float xb = __fsub_rn(tc[d], 0.5f);
            const float fl = floorf(xb);
            c.f[d] = __fsub_rn(xb, fl);
            const int a = (int)fmaxf(fminf(fl, 1e9f), -1e9f), b = a + 1;
            c.i0[d] = (uint32_t)min(max(a, 0), hi);
            c.i1[d] = (uint32_t)min(max(b, 0), hi);
        }
        float t[8];
        uint64_t off[8];
        if (!trilinear<S3R_BRICK_F32>(brick, c, n, val, t, off)) return __int_as_float(0x7fc00000);
        return val;
    }
}

template <bool kTex> __device__ __forceinline__ float4 tf_rgba(const float4* tf, uint32_t tfn, float v01)
{
    if constexpr (kTex) return tex_tf_lookup(tf, tfn, v01);
    else return tf_lookup(tf, tfn, v01).c;
}

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(const float* p) { return F3{p[0], p[1], p[2]}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ F3 operator*(F3 a, F3 b) { return F3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 normalize3(F3 a) { return a * (1.f / sqrtf(dot3(a, a))); }
__device__ __forceinline__ float clamp01(float x) { return fmaxf(0.f, fminf(1.f, x)); }

// x^100 in double by squaring (x^64 x^32 x^4): eight multiplications, whose
// few-ulp double error almost never reaches the float the result is rounded to;
// a general double pow costs several times that on this GPU's FP64 units.
__device__ __forceinline__ double pow100(double x)
{
    const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4, x16 = x8 * x8, x32 = x16 * x16, x64 = x32 * x32;
    return x64 * x32 * x4;
}

// Blinn-Phong term of one light (cuda_lighting.hpp:26-50): material ambient 1,
// diffuse = the transfer-function colour, specular 0.5, shininess 100; the
// reference's max(., 0.0) and pow promote to double (the max is exact in float,
// the power is formed in double as above).
__device__ __forceinline__ F3 blinn(F3 N, F3 V, F3 L, const s3r_light& light, F3 kd)
{
    const float diff = fmaxf(dot3(L, N), 0.f);
    const F3 H = normalize3(L + V);
    const float spec = diff > 0.f ? (float)pow100(fmax((double)dot3(H, N), 0.0)) : 0.f;
    return f3(light.ambient) + kd * f3(light.diffuse) * diff + F3{0.5f, 0.5f, 0.5f} * f3(light.specular) * spec;
}

// Where a field-mode march takes its samples from.
//   BrickSampler<kTex>: linear bricks in HBM, filtered in software (kTex: the
//     texture unit's rule, else exact trilinear); the table in shared memory.
//   TextureSampler: the GPU's texture unit itself, as the reference samples --
//     tex3D on a 3-D float array (unnormalized coordinates, linear filtering,
//     clamp) and tex1D on the transfer-function array (normalized, linear,
//     clamp).
// kStepwise: sample positions accumulated step by step from the entry point
// (pos += step), as the reference forms them, because texture filtering's
// 8-bit fractions are sensitive to the last ulp of a position; else entry +
// k * step (one fma), as the oracle and the batched path form them.
// kContracted: the crossing positions of the isosurface modes written as the
// reference writes them (pos + step * t, which nvcc fuses into one fma), else
// rounded twice as the oracle rounds them.
template <bool kTex> struct BrickSampler {
    const float* b1;
    const float* b2;
    Dim n;
    const float4* tf;
    uint32_t tfn;
    static constexpr bool kStepwise = kTex, kContracted = false;
    __device__ float field(int second, float x, float y, float z) const
    {
        return field_at<kTex>(second ? b2 : b1, n, x, y, z);
    }
    __device__ float4 colour(float v01) const { return tf_rgba<kTex>(tf, tfn, v01); }
};

struct TextureSampler {
    cudaTextureObject_t t1, t2, tf;
    static constexpr bool kStepwise = true, kContracted = true;
    __device__ float field(int second, float x, float y, float z) const
    {
        return tex3D<float>(second ? t2 : t1, x, y, z);
    }
    __device__ float4 colour(float v01) const { return tex1D<float4>(tf, v01); }
};

// computeFragColor (cuda_lighting.hpp:52-95): normal from central differences
// of the field at +-0.1 texel, double-sided lighting, colour clamped to [0, 1].
template <class S>
__device__ __forceinline__ float4 frag_color(const S& smp, float4 diffuse, F3 eye, F3 surf, F3 tc,
                                             const s3r_presentation& pr)
{
    constexpr float d = 0.1f;
    const F3 a{smp.field(0, tc.x - d, tc.y, tc.z), smp.field(0, tc.x, tc.y - d, tc.z),
               smp.field(0, tc.x, tc.y, tc.z - d)};
    const F3 b{smp.field(0, tc.x + d, tc.y, tc.z), smp.field(0, tc.x, tc.y + d, tc.z),
               smp.field(0, tc.x, tc.y, tc.z + d)};
    F3 N = normalize3(a - b);
    const F3 V = normalize3(eye - surf);
    F3 c{0.f, 0.f, 0.f};
    const F3 kd{diffuse.x, diffuse.y, diffuse.z};
    for (uint32_t i = 0; i < pr.light_count; ++i) {
        const F3 L = normalize3(f3(pr.lights[i].pos) - surf);
        if (dot3(L, N) < 0.f) N = F3{-N.x, -N.y, -N.z};
        c = c + blinn(N, V, L, pr.lights[i], kd);
    }
    return make_float4(clamp01(c.x), clamp01(c.y), clamp01(c.z), diffuse.w);
}

// blendBehind / blendAbove (cuda_blend.hpp:24-44), non-premultiplied
__device__ __forceinline__ void blend_behind(float4& acc, float4 col)
{
    const float da = col.w * (1.f - acc.w);
    const float a = acc.w + da;
    if (a > 0.f) {
        const float ka = acc.w / a, kd = da / a;
        acc.x = acc.x * ka + col.x * kd;
        acc.y = acc.y * ka + col.y * kd;
        acc.z = acc.z * ka + col.z * kd;
    }
    acc.w = a;
}

__device__ __forceinline__ uint32_t blend_above_argb(uint32_t pix, float4 acc)
{
    float4 ex = argb_to_rgba(pix);
    const float da = ex.w * (1.f - acc.w);
    const float a = acc.w + da;
    if (a > 0.f) {
        const float kd = da / a, ki = acc.w / a;
        ex.x = ex.x * kd + acc.x * ki;
        ex.y = ex.y * kd + acc.y * ki;
        ex.z = ex.z * kd + acc.z * ki;
    }
    ex.w = a;
    return rgba_to_argb(ex);
}

// findInterval (cuda_findInterval.hpp:26-43): i with levels[i-1] <= v < levels[i]
__device__ __forceinline__ int find_interval(float v, const float* levels, uint32_t count)
{
    if (v < levels[0]) return 0;
    if (v >= levels[count - 1]) return (int)count;
    int i1 = 0, i2 = (int)count;
    while (i2 - i1 > 1) {
        const int i = (i1 + i2) >> 1;
        if (v < levels[i]) i2 = i;
        else i1 = i;
    }
    return i2;
}

// What one block contributes to one pixel in a field mode.
struct ModeOut {
    enum : uint32_t { kNone, kBlend, kMax, kClear } kind;
    float4 acc; // kBlend: non-premultiplied colour and alpha gathered front to back in the block
    float t;    // kMax: (max value - field min) / span
};

// The per-pixel march of one block in a field mode (renderKernel<mode>,
// DenseFieldRenderer_cu.cu:62-215 and render*.hpp): max intensity gives the
// block's maximum above the threshold; the colour modes (Argb, ArgbLight,
// DomainVoxels) and the isosurface modes the colour gathered with blendBehind;
// multi-level modes with no level clear the pixel.
template <class S, int kMode = -1>
__device__ __forceinline__ ModeOut march_block_mode(const s3r_view& v, const s3r_presentation& pr, const S& smp,
                                                    const BlockRay& r, uint32_t depth)
{
    ModeOut out{ModeOut::kNone, make_float4(0.f, 0.f, 0.f, 0.f), 0.f};
    const float span = v.field_max - v.field_min;
    const F3 eye = f3(v.cam.eye);
    const F3 step{r.step[0], r.step[1], r.step[2]};
    // sample k's position: with the texture filter accumulated step by step from
    // the entry point as the reference does (increase(pos, step)), because the
    // texture unit's 8-bit fractions make it sensitive to the last ulp of the
    // position; with the exact filter entry + k * step (one fma), as the oracle
    // and the batched path form it.  Every loop below visits k = 0, 1, 2, ... in
    // order, carrying the accumulated position from one iteration to the next
    // (advance), so that consecutive samples' fetches are independent of one
    // another and can be in flight together.
    F3 seq{r.p0[0], r.p0[1], r.p0[2]};
    auto advance = [&]() {
        if constexpr (S::kStepwise)
            seq = F3{__fadd_rn(seq.x, r.step[0]), __fadd_rn(seq.y, r.step[1]), __fadd_rn(seq.z, r.step[2])};
    };
    auto pos_of = [&](int k) {
        if constexpr (S::kStepwise) {
            return seq; // the caller has advanced to sample k
        } else {
            return F3{__fmaf_rn(r.step[0], (float)k, r.p0[0]), __fmaf_rn(r.step[1], (float)k, r.p0[1]),
                      __fmaf_rn(r.step[2], (float)k, r.p0[2])};
        }
    };
    auto tc_of = [&](F3 p) {
        return F3{__fmul_rn(__fsub_rn(p.x, r.origin[0]), r.factor), __fmul_rn(__fsub_rn(p.y, r.origin[1]), r.factor),
                  __fmul_rn(__fsub_rn(p.z, r.origin[2]), r.factor)};
    };
    auto value = [&](int second, F3 p) {
        const F3 tc = tc_of(p);
        return smp.field(second, tc.x, tc.y, tc.z);
    };
    constexpr float kMax = 0.996f; // AlphaThreshold / AlphaMaxThreshold
    // kMode >= 0: the mode is fixed at compile time (one kernel per mode, as renderKernel<mode> is), so
    // only its branch is compiled in and the registers are that mode's
    const uint32_t mode = kMode >= 0 ? (uint32_t)kMode : pr.mode;
    if (mode == S3R_MODE_MAX_INTENSITY) {
        // renderMaxIntensityProjection.hpp:30-50; the pixel holds float bits
        float maxv = v.field_min - span;
        for (int i = 1; i < r.samples; ++i, advance()) {
            const float val = value(0, pos_of(i - 1));
            if (val >= v.threshold && maxv < val) maxv = val;
        }
        if (maxv < v.field_min) return out;
        out.kind = ModeOut::kMax;
        out.t = (maxv - v.field_min) / span;
        return out;
    }
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (mode == S3R_MODE_ARGB || mode == S3R_MODE_ARGB_LIGHT || mode == S3R_MODE_DOMAIN_VOXELS) {
        const float of = (v.threshold - v.field_min) / span;
        const float il = layer_exponent(depth, v.level, v.quality);
        float4 dom = make_float4(0.f, 0.f, 0.f, 0.f);
        if (mode == S3R_MODE_DOMAIN_VOXELS) {
            // renderDomainVoxels.hpp:41-42: one colour, the table's middle
            dom = smp.colour(0.5f);
            dom.w = 1.f - powf(1.f - dom.w * of, il);
        }
        for (int i = 1; i < r.samples; ++i, advance()) {
            const F3 p = pos_of(i - 1);
            const float val = value(0, p);
            if (isnan(val)) continue;
            float4 col;
            if (mode == S3R_MODE_DOMAIN_VOXELS) {
                col = dom;
            } else {
                col = smp.colour((val - v.field_min) / span);
                col.w = 1.f - powf(1.f - col.w * of, il);
                if (mode == S3R_MODE_ARGB_LIGHT) {
                    // renderArgbLight.hpp:44-56: only visible enough samples are lit
                    if (!(col.w >= 0.00001f)) continue;
                    col = frag_color(smp, col, eye, p, tc_of(p), pr);
                }
            }
            blend_behind(acc, col);
            if (acc.w > kMax) break;
        }
        out.kind = ModeOut::kBlend;
        out.acc = acc;
        return out;
    }
    // isosurface modes: v1 at the entry point, v2 at samples 1 .. sampleCount-1; the
    // crossing is placed at pos + step * t from the later sample, as the reference does
    const bool multi = mode == S3R_MODE_ISOSURFACES || mode == S3R_MODE_VALUE_ON_ISOSURFACES;
    const bool secondary = mode == S3R_MODE_VALUE_ON_ISOSURFACE || mode == S3R_MODE_VALUE_ON_ISOSURFACES;
    const uint32_t nl = pr.level_count;
    if (multi && nl < 1) {
        out.kind = ModeOut::kClear; // renderIsosurfaces.hpp:36-38
        return out;
    }
    auto surface_colour = [&](float level, F3 xpos) {
        float4 dif;
        if (secondary) {
            const float vs = value(1, xpos);
            dif = smp.colour((vs - pr.secondary_min) / (pr.secondary_max - pr.secondary_min));
        } else {
            dif = smp.colour((level - v.field_min) / span);
        }
        dif.w *= pr.isosurface_opacity;
        return frag_color(smp, dif, eye, xpos, tc_of(xpos), pr);
    };
    auto xpos_of = [&](F3 p, float t) {
        if constexpr (S::kContracted) return F3{p.x + step.x * t, p.y + step.y * t, p.z + step.z * t};
        else
            return F3{__fadd_rn(p.x, __fmul_rn(step.x, t)), __fadd_rn(p.y, __fmul_rn(step.y, t)),
                      __fadd_rn(p.z, __fmul_rn(step.z, t))};
    };
    float v1 = value(0, pos_of(0));
    if (!multi) {
        const float thr = v.threshold;
        for (int i = 1; i < r.samples; ++i) {
            advance();
            const F3 p = pos_of(i);
            const float v2 = value(0, p);
            if (!isnan(v1) && !isnan(v2) && (v1 - thr) * (v2 - thr) < 0.f) {
                const float t = (thr - v1) / (v2 - v1);
                blend_behind(acc, surface_colour(thr, xpos_of(p, t)));
                if (acc.w > kMax) break;
            }
            v1 = v2;
        }
    } else {
        // renderIsosurfaces.hpp:34-106 / renderValueOnIsosurfaces.hpp
        int iint = isnan(v1) ? -1 : find_interval(v1, pr.levels, nl);
        for (int i = 1; i < r.samples; ++i) {
            advance();
            const F3 p = pos_of(i);
            const float v2 = value(0, p);
            if (isnan(v2)) {
                iint = -1;
                v1 = __int_as_float(0x7fc00000);
                continue;
            }
            if (isnan(v1)) {
                v1 = v2;
                iint = find_interval(v1, pr.levels, nl);
                continue;
            }
            int il, dl;
            if (v2 < v1) {
                if (iint == 0) {
                    v1 = v2;
                    continue;
                }
                il = iint - 1;
                dl = -1;
            } else {
                if (iint == (int)nl) {
                    v1 = v2;
                    continue;
                }
                il = iint;
                dl = 1;
            }
            while (il >= 0 && il < (int)nl) {
                const float level = pr.levels[il];
                if ((v1 - level) * (v2 - level) < 0.f) {
                    const float t = (level - v1) / (v2 - v1);
                    blend_behind(acc, surface_colour(level, xpos_of(p, t)));
                    iint += dl;
                    il += dl;
                } else {
                    break;
                }
            }
            if (acc.w > kMax) break;
            v1 = v2;
        }
    }
    out.kind = ModeOut::kBlend;
    out.acc = acc;
    return out;
}

// A block's contribution to one pixel of the ARGB8 viewport, as renderKernel<mode> stores it.
__device__ __forceinline__ void store_mode_pixel(uint32_t* px, const ModeOut& o)
{
    if (o.kind == ModeOut::kMax) {
        // renderMaxIntensityProjection.hpp:30-50; the pixel holds float bits
        const float prev = __uint_as_float(*px);
        if (!isnan(prev) && prev > o.t) return;
        *px = __float_as_uint(o.t);
    } else if (o.kind == ModeOut::kBlend) {
        *px = blend_above_argb(*px, o.acc);
    } else if (o.kind == ModeOut::kClear) {
        *px = 0u;
    }
}

template <bool kTex>
__global__ void render_block_mode_kernel(const s3r_view v, const s3r_presentation pr, const float* __restrict__ brick,
                                         const float* __restrict__ brick2, const RenderBlock rb,
                                         const float4* __restrict__ tf_g, uint32_t* __restrict__ viewport)
{
    extern __shared__ float4 tf[];
    for (uint32_t i = threadIdx.y * blockDim.x + threadIdx.x; i < v.tf_n; i += blockDim.x * blockDim.y)
        tf[i] = tf_g[i];
    __syncthreads();
    const int32_t xx = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t yy = blockIdx.y * blockDim.y + threadIdx.y;
    if (xx >= rb.rect[2] || yy >= rb.rect[3]) return;
    const uint32_t vx = (uint32_t)(rb.rect[0] + xx), vy = (uint32_t)(rb.rect[1] + yy);
    if (vx >= v.W || vy >= v.H) return;
    float org[3], dir[3];
    pixel_ray(v, vx, vy, org, dir);
    BlockRay r;
    if (!block_ray(v, org, dir, rb, r)) return;
    const BrickSampler<kTex> smp{brick, brick2, dim_of(r), tf, v.tf_n};
    store_mode_pixel(&viewport[(size_t)(v.H - 1 - vy) * v.W + vx], march_block_mode(v, pr, smp, r, rb.depth));
}

// The per-pixel ray and the block's sampling set-up written with plain float
// operators in the order of DenseFieldRenderer_cu.cu:72-181 (ray = n + e1 x +
// e2 y, face points eye + ray tau, the dot product of the sample count), so
// that nvcc fuses the same products into the same fmas as in the reference's
// kernel and the samples land where the reference's land.  The texture-unit
// path uses them; the other kernels round every step explicitly, as the
// oracle does.
__device__ __forceinline__ void pixel_ray_fused(const s3r_view& v, uint32_t vx, uint32_t vy, float org[3],
                                                float dir[3])
{
    const float x = (-0.5f + ((float)vx + 0.5f) / (float)v.W) * v.cam.w;
    const float y = (-0.5f + ((float)vy + 0.5f) / (float)v.H) * v.cam.h;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (v.cam.ortho) {
            org[d] = v.cam.eye[d] + v.cam.e1[d] * x + v.cam.e2[d] * y;
            dir[d] = v.cam.n[d];
        } else {
            org[d] = v.cam.eye[d];
            dir[d] = v.cam.n[d] + v.cam.e1[d] * x + v.cam.e2[d] * y;
        }
    }
}

__device__ __forceinline__ bool block_ray_fused(const s3r_view& v, const float org[3], const float dir[3],
                                                const RenderBlock& rb, BlockRay& r)
{
    const float* c = rb.center;
    const float h = rb.half;
    float te = 1.f, tx = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!(fabsf(dir[a]) > 1e-10f)) continue;
        const int b1 = a == 0 ? 1 : 0;
        const int b2 = a == 2 ? 1 : 2;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const float face = side ? c[a] + h : c[a] - h;
            const float tau = (face - org[a]) / dir[a];
            const float p1 = org[b1] + dir[b1] * tau;
            const float p2 = org[b2] + dir[b2] * tau;
            if (fabsf(p1 - c[b1]) <= h && fabsf(p2 - c[b2]) <= h) {
                const bool enter = (dir[a] > 0.f) == (side == 0);
                if (enter) te = tau;
                else tx = tau;
            }
        }
    }
    if (te < 1.f) te = 1.f;
    r.tau_enter = te;
    r.tau_exit = tx;
    if (!(tx > te)) return false;
    const uint32_t n = (1u << rb.depth) + 1u;
    const float dotr = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
    const int s = (int)(v.quality * (tx - te) * dotr / (rb.texel * (fabsf(dir[0]) + fabsf(dir[1]) + fabsf(dir[2]))));
    const float dtau = (tx - te) / (float)s;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        r.step[d] = dir[d] * dtau;
        r.p0[d] = org[d] + dir[d] * te;
        r.origin[d] = rb.origin[d];
    }
    r.factor = rb.factor;
    r.n = n;
    r.pitch = n;
    r.samples = s;
    return true;
}

// Pixel tile of one CTA of the texture-unit kernel, per field mode: the fastest of 8x4 .. 64x1 and 16x16
// tiles measured on the 64-block depth-6 workload at 1920x1080 (the texture fetches dominate; 8x8 tiles
// keep a CTA's rays close together, the single-isosurface modes do best with 32x2).
__host__ __device__ constexpr uint32_t tex_tile_x(uint32_t mode)
{
    return (mode == S3R_MODE_ISOSURFACE || mode == S3R_MODE_VALUE_ON_ISOSURFACE) ? 32u : 8u;
}
__host__ __device__ constexpr uint32_t tex_tile_y(uint32_t mode)
{
    return (mode == S3R_MODE_ISOSURFACE || mode == S3R_MODE_VALUE_ON_ISOSURFACE) ? 2u : 8u;
}

// One block in any field mode sampled through the texture unit (the field and
// the transfer function as texture objects), on the fused ray set-up above.
template <int kMode>
__global__ void render_block_texture_kernel(const s3r_view v, const s3r_presentation pr, const TextureSampler smp,
                                            const RenderBlock rb, uint32_t* __restrict__ viewport)
{
    const int32_t xx = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t yy = blockIdx.y * blockDim.y + threadIdx.y;
    if (xx >= rb.rect[2] || yy >= rb.rect[3]) return;
    const uint32_t vx = (uint32_t)(rb.rect[0] + xx), vy = (uint32_t)(rb.rect[1] + yy);
    if (vx >= v.W || vy >= v.H) return;
    float org[3], dir[3];
    pixel_ray_fused(v, vx, vy, org, dir);
    BlockRay r;
    if (!block_ray_fused(v, org, dir, rb, r)) return;
    store_mode_pixel(&viewport[(size_t)(v.H - 1 - vy) * v.W + vx], march_block_mode<TextureSampler, kMode>(v, pr, smp, r,
                                                                                                       rb.depth));
}

// ---------------------------------------------------------------- batched form

// Front-to-back walk of the (2^level)^3 block grid along one ray
// (Amanatides-Woo); calls f(block_index, ix, iy, iz) for every block the ray
// passes, in order; f returns false to stop.
template <class F>
__device__ __forceinline__ void walk_blocks(const float org[3], const float dir[3], uint32_t level, F&& f)
{
    const int m = 1 << level;
    const float cell = (2.f * kTopHalf) / (float)m;
    // entry/exit of the whole cube [-5, 5]^3, restricted to tau >= 1 (the screen plane)
    float t0 = 1.f, t1 = 3.4e38f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (fabsf(dir[a]) > 1e-10f) {
            const float inv = 1.f / dir[a];
            float ta = (-kTopHalf - org[a]) * inv, tb = (kTopHalf - org[a]) * inv;
            if (ta > tb) { const float t = ta; ta = tb; tb = t; }
            t0 = fmaxf(t0, ta);
            t1 = fminf(t1, tb);
        } else if (org[a] < -kTopHalf || org[a] > kTopHalf) {
            return;
        }
    }
    if (!(t1 > t0)) return;
    // start cell: the one holding the entry point itself (clamped onto the grid);
    // starting any distance inside would skip the first block's segment on rays
    // that enter close to a block boundary
    const float tm = t0;
    // start cell, step direction, next boundary crossing and crossing period per axis
    int c0, c1, c2, s0, s1, s2;
    float tx0, tx1, tx2, td0, td1, td2;
    auto setup = [&](int a, int& c, int& st, float& tmax, float& tdel) {
        const float pm = __fmaf_rn(dir[a], tm, org[a]);
        c = min(max((int)floorf((pm + kTopHalf) / cell), 0), m - 1);
        if (dir[a] > 1e-10f) {
            st = 1;
            tmax = ((-kTopHalf + cell * (float)(c + 1)) - org[a]) / dir[a];
            tdel = cell / dir[a];
        } else if (dir[a] < -1e-10f) {
            st = -1;
            tmax = ((-kTopHalf + cell * (float)c) - org[a]) / dir[a];
            tdel = -cell / dir[a];
        } else {
            st = 0;
            tmax = 3.4e38f;
            tdel = 3.4e38f;
        }
    };
    setup(0, c0, s0, tx0, td0);
    setup(1, c1, s1, tx1, td1);
    setup(2, c2, s2, tx2, td2);
    for (int guard = 0; guard < 3 * m + 3; ++guard) {
        const uint32_t b = (uint32_t)c0 + (uint32_t)m * ((uint32_t)c1 + (uint32_t)m * (uint32_t)c2);
        if (!f(b, (uint32_t)c0, (uint32_t)c1, (uint32_t)c2)) return;
        if (tx0 <= tx1 && tx0 <= tx2) {
            if (tx0 >= t1) return;
            c0 += s0;
            if (c0 < 0 || c0 >= m) return;
            tx0 += td0;
        } else if (tx1 <= tx2) {
            if (tx1 >= t1) return;
            c1 += s1;
            if (c1 < 0 || c1 >= m) return;
            tx1 += td1;
        } else {
            if (tx2 >= t1) return;
            c2 += s2;
            if (c2 < 0 || c2 >= m) return;
            tx2 += td2;
        }
    }
}

__device__ __forceinline__ bool pixel_in_rect(const int32_t* rc, uint32_t vx, uint32_t vy)
{
    return (int32_t)vx >= rc[0] && (int32_t)vx < rc[0] + rc[2] && (int32_t)vy >= rc[1] && (int32_t)vy < rc[1] + rc[3];
}

struct Premul {
    float r, g, b, a;
};

// The 8 texels of sample k issued as independent loads (32-bit offsets: a brick
// holds at most 513^3 vertices) with the cell's fractions.
template <int Fmt> struct Texels {
    float t[8];
    float f[3];
};

template <int Fmt>
__device__ __forceinline__ void fetch_texels(const void* brick, const BlockRay& r, int k, Texels<Fmt>& x)
{
    Cell c;
    sample_cell(r, k, c);
    const uint32_t n = r.n;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint32_t xi = (q & 1) ? c.i1[0] : c.i0[0];
        const uint32_t yi = (q & 2) ? c.i1[1] : c.i0[1];
        const uint32_t zi = (q & 4) ? c.i1[2] : c.i0[2];
        x.t[q] = Brick<Fmt>::get(brick, (zi * n + yi) * r.pitch + xi);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) x.f[d] = c.f[d];
}

// Trilinear value of fetched texels; false when one of them is NaN (outside the domain).
template <int Fmt> __device__ __forceinline__ bool filter_texels(const Texels<Fmt>& x, float& val)
{
    bool bad = false;
#pragma unroll
    for (int q = 0; q < 8; ++q) bad |= isnan(x.t[q]);
    if (bad) return false;
    const float* t = x.t;
    const float x00 = __fmaf_rn(x.f[0], t[1] - t[0], t[0]);
    const float x10 = __fmaf_rn(x.f[0], t[3] - t[2], t[2]);
    const float x01 = __fmaf_rn(x.f[0], t[5] - t[4], t[4]);
    const float x11 = __fmaf_rn(x.f[0], t[7] - t[6], t[6]);
    const float y0 = __fmaf_rn(x.f[1], x10 - x00, x00);
    const float y1 = __fmaf_rn(x.f[1], x11 - x01, x01);
    val = __fmaf_rn(x.f[2], y1 - y0, y0);
    return true;
}

// March one block along a ray (premultiplied, block-local early termination).
// Exact filter: software-pipelined -- sample k+1's texel loads are issued
// before sample k is filtered, looked up and composited, so a ray keeps two
// samples' loads in flight; the arithmetic and its order are unchanged.
template <int Fmt, bool kTex>
__device__ __forceinline__ Premul march_block(const s3r_view& v, const BlockRay& r, const void* brick, float scale,
                                              float offset, uint32_t depth, const float4* tf, float of,
                                              uint32_t& taken)
{
    const float span = v.field_max - v.field_min;
    const float il = layer_exponent(depth, v.level, v.quality);
    Premul acc{0.f, 0.f, 0.f, 0.f};
    if constexpr (!kTex) {
        if (r.samples < 2) return acc;
        Texels<Fmt> cur, nxt;
        fetch_texels<Fmt>(brick, r, 0, cur);
        for (int i = 1; i < r.samples; ++i) {
            ++taken;
            if (i + 1 < r.samples) fetch_texels<Fmt>(brick, r, i, nxt);
            float val;
            if (filter_texels<Fmt>(cur, val)) {
                if (Fmt != S3R_BRICK_F32) val = __fmaf_rn(scale, val, offset);
                const float v01 = __fdiv_rn(__fsub_rn(val, v.field_min), span);
                const float4 col = tf_lookup(tf, v.tf_n, v01).c;
                const float a = __fsub_rn(1.f, __powf(__fmaf_rn(-col.w, of, 1.f), il));
                const float w = __fmul_rn(__fsub_rn(1.f, acc.a), a);
                acc.r = __fmaf_rn(w, col.x, acc.r);
                acc.g = __fmaf_rn(w, col.y, acc.g);
                acc.b = __fmaf_rn(w, col.z, acc.b);
                acc.a = __fadd_rn(acc.a, w);
                if (acc.a > kAlphaThreshold) break;
            }
            cur = nxt;
        }
        return acc;
    } else {
        for (int i = 1; i < r.samples; ++i) {
            ++taken;
            float val;
            if (!tex_trilinear<Fmt>(brick, r, i - 1, val)) continue;
            if (Fmt != S3R_BRICK_F32) val = __fmaf_rn(scale, val, offset);
            const float v01 = __fdiv_rn(__fsub_rn(val, v.field_min), span);
            const float4 col = tex_tf_lookup(tf, v.tf_n, v01);
            const float a = __fsub_rn(1.f, __powf(__fmaf_rn(-col.w, of, 1.f), il));
            const float w = __fmul_rn(__fsub_rn(1.f, acc.a), a);
            acc.r = __fmaf_rn(w, col.x, acc.r);
            acc.g = __fmaf_rn(w, col.y, acc.g);
            acc.b = __fmaf_rn(w, col.z, acc.b);
            acc.a = __fadd_rn(acc.a, w);
            if (acc.a > kAlphaThreshold) break;
        }
        return acc;
    }
}

// One pixel ray per R consecutive lanes: the ray's block sequence (the DDA
// order) is cut into R contiguous runs, lane r composites run r, and the R
// premultiplied partial results are merged front to back with shuffles (the
// over operator is associative).  With R > 1 a ray stops early only inside its
// run, so R = 1 is used when view.alpha_stop < 1.
template <int Fmt, int R, bool kTex>
__global__ void frame_render_kernel(FrameArgs fa)
{
    extern __shared__ float4 tf[];
    const s3r_view v = *fa.view;
    const uint32_t nthreads = blockDim.x * blockDim.y;
    const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x;
    const uint32_t seg = threadIdx.x % R;
    const uint32_t px_per_row = blockDim.x / R;
    const uint32_t vx = blockIdx.x * px_per_row + threadIdx.x / R;
    const uint32_t vy = blockIdx.y * blockDim.y + threadIdx.y;
    {
        // CTAs whose pixels no block covers only clear their pixels
        const int4 cv = *reinterpret_cast<const int4*>(fa.cover);
        const int32_t x0 = blockIdx.x * px_per_row, y0 = blockIdx.y * blockDim.y;
        if (x0 >= cv.z || x0 + (int32_t)px_per_row <= cv.x || y0 >= cv.w || y0 + (int32_t)blockDim.y <= cv.y) {
            if (seg == 0 && vx < v.W && vy < v.H) {
                const size_t o = (size_t)(v.H - 1 - vy) * v.W + vx;
                if (fa.rgba) reinterpret_cast<float4*>(fa.rgba)[o] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (fa.argb) fa.argb[o] = 0u;
            }
            return;
        }
    }
    for (uint32_t i = tid; i < v.tf_n; i += nthreads) tf[i] = reinterpret_cast<const float4*>(fa.tf)[i];
    __syncthreads();
    uint32_t taken = 0;
    Premul acc{0.f, 0.f, 0.f, 0.f};
    const bool inside = vx < v.W && vy < v.H;
    if (inside) {
        float org[3], dir[3];
        pixel_ray(v, vx, vy, org, dir);
        const float of = (v.threshold - v.field_min) / (v.field_max - v.field_min);
        int lo = 0, hi = 1 << 30;
        if (R > 1) {
            int n = 0;
            walk_blocks(org, dir, v.level, [&](uint32_t, uint32_t, uint32_t, uint32_t) {
                ++n;
                return true;
            });
            const int chunk = (n + R - 1) / R;
            lo = (int)seg * chunk;
            hi = lo + chunk;
        }
        int idx = 0;
        walk_blocks(org, dir, v.level, [&](uint32_t b, uint32_t, uint32_t, uint32_t) {
            if (idx >= hi) return false;
            if (idx++ < lo) return true;
            const RenderBlock* rb = &fa.table[b];
            const uint32_t depth = rb->depth;
            if (depth == 0xffffffffu) return true;
            const int4 rc = *reinterpret_cast<const int4*>(rb->rect);
            const int32_t rca[4] = {rc.x, rc.y, rc.z, rc.w};
            if (!pixel_in_rect(rca, vx, vy)) return true;
            BlockRay r;
            if (!block_ray(v, org, dir, *rb, r)) return true;
            const char* base = reinterpret_cast<const char*>(fa.bricks);
            const size_t esz = Fmt == S3R_BRICK_F32 ? 4 : 2;
            float scale = 1.f, offset = 0.f;
            if (Fmt != S3R_BRICK_F32) {
                const float2 so = fa.scale_offset[rb->block];
                scale = so.x;
                offset = so.y;
            }
            const Premul p =
                march_block<Fmt, kTex>(v, r, base + rb->brick_off * esz, scale, offset, depth, tf, of, taken);
            const float T = __fsub_rn(1.f, acc.a);
            acc.r = __fmaf_rn(T, p.r, acc.r);
            acc.g = __fmaf_rn(T, p.g, acc.g);
            acc.b = __fmaf_rn(T, p.b, acc.b);
            acc.a = __fmaf_rn(T, p.a, acc.a);
            return !(acc.a > v.alpha_stop);
        });
    }
    // merge the runs front to back: lane seg (a multiple of 2*off) takes lane seg+off behind it
#pragma unroll
    for (int off = 1; off < R; off <<= 1) {
        const float br = __shfl_down_sync(0xffffffffu, acc.r, off, R);
        const float bg = __shfl_down_sync(0xffffffffu, acc.g, off, R);
        const float bb = __shfl_down_sync(0xffffffffu, acc.b, off, R);
        const float ba = __shfl_down_sync(0xffffffffu, acc.a, off, R);
        if ((seg & (2 * off - 1)) == 0) {
            const float T = __fsub_rn(1.f, acc.a);
            acc.r = __fmaf_rn(T, br, acc.r);
            acc.g = __fmaf_rn(T, bg, acc.g);
            acc.b = __fmaf_rn(T, bb, acc.b);
            acc.a = __fmaf_rn(T, ba, acc.a);
        }
    }
    if (inside && seg == 0) {
        const size_t o = (size_t)(v.H - 1 - vy) * v.W + vx;
        float4 out = make_float4(0.f, 0.f, 0.f, acc.a);
        if (acc.a > 0.f) {
            const float inv = 1.f / acc.a;
            out.x = acc.r * inv;
            out.y = acc.g * inv;
            out.z = acc.b * inv;
        }
        if (fa.rgba) reinterpret_cast<float4*>(fa.rgba)[o] = out;
        if (fa.argb) fa.argb[o] = rgba_to_argb(out);
    }
    if (fa.samples) {
        unsigned long long t = taken;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if ((tid & 31) == 0 && t) atomicAdd(fa.samples, t);
    }
}

// Non-premultiplied RGBA and ARGB32 of a composited ray, row-flipped as the reference stores pixels.
__device__ __forceinline__ void write_pixel(const FrameArgs& fa, const s3r_view& v, uint32_t vx, uint32_t vy,
                                            const Premul& acc)
{
    const size_t o = (size_t)(v.H - 1 - vy) * v.W + vx;
    float4 out = make_float4(0.f, 0.f, 0.f, acc.a);
    if (acc.a > 0.f) {
        const float inv = 1.f / acc.a;
        out.x = acc.r * inv;
        out.y = acc.g * inv;
        out.z = acc.b * inv;
    }
    if (fa.rgba) reinterpret_cast<float4*>(fa.rgba)[o] = out;
    if (fa.argb) fa.argb[o] = rgba_to_argb(out);
}

// ---------------------------------------------------------------- block-major form

// Front-to-back rank of block (ix, iy, iz) on a ray of direction dir.  Along a
// ray every block index moves monotonically in the direction of its component's
// sign, one step at a time, so this sum grows by exactly one per block the ray
// passes: the blocks of a ray sort front to back by it, and a ray meets at most
// 3m - 2 ranks (m blocks per axis).
__device__ __forceinline__ uint32_t ray_rank(const float dir[3], uint32_t ix, uint32_t iy, uint32_t iz, uint32_t m)
{
    return (dir[0] < 0.f ? m - 1 - ix : ix) + (dir[1] < 0.f ? m - 1 - iy : iy) + (dir[2] < 0.f ? m - 1 - iz : iz);
}

// Block-major ray cast: the work items are the warp-sized pixel tiles of every
// block's view rectangle, blocks in decreasing depth (most samples per ray
// first); each warp of a persistent grid takes items from a work-queue counter on
// its own, fetching the next item while it marches the current one.  A lane
// marches its pixel's ray through the item's block exactly as frame_render_kernel
// does (pixel_ray, block_ray, march_block) and stores the premultiplied result at
// the block's front-to-back rank on that ray, marking the rank in the pixel's
// mask; a zero result changes no composite and is not stored.  The lanes of an
// item read one brick, their rays cross it side by side (similar sample counts),
// and the deep blocks' items spread over every SM -- the per-ray walk's lanes
// instead each hold their own block sequence.  frame_composite_kernel then blends
// every pixel's results in rank order with frame_render_kernel's arithmetic.
template <int Fmt, bool kTex>
__global__ void __launch_bounds__(128, 8) frame_segments_kernel(FrameArgs fa, SegArgs sa, uint32_t fx)
{
    extern __shared__ float4 tf[];
    const s3r_view v = *fa.view;
    const uint32_t nthreads = blockDim.x * blockDim.y;
    const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (uint32_t i = tid; i < v.tf_n; i += nthreads) tf[i] = reinterpret_cast<const float4*>(fa.tf)[i];
    __syncthreads();
    const uint32_t lane = tid & 31u;
    const uint32_t fy = 32u / fx;
    const uint32_t total = *sa.count;
    const uint32_t m = 1u << v.level;
    const uint64_t npix = (uint64_t)v.W * v.H;
    const float of = (v.threshold - v.field_min) / (v.field_max - v.field_min);
    uint32_t taken = 0;
    auto take = [&](uint32_t& item, uint2& desc) {
        item = 0xffffffffu;
        desc = make_uint2(0u, 0u);
        if (lane == 0) {
            item = atomicAdd(sa.queue, 1u);
            if (item < total) desc = sa.items[item];
        }
    };
    uint32_t item;
    uint2 desc;
    take(item, desc);
    item = __shfl_sync(0xffffffffu, item, 0);
    desc.x = __shfl_sync(0xffffffffu, desc.x, 0);
    desc.y = __shfl_sync(0xffffffffu, desc.y, 0);
    while (item < total) {
        uint32_t next;
        uint2 ndesc;
        take(next, ndesc); // in flight while this item is marched
        const uint32_t cell = desc.x, tile = desc.y;
        const RenderBlock* rb = &fa.table[cell];
        const int4 rc = *reinterpret_cast<const int4*>(rb->rect);
        const uint32_t tiles_x = ((uint32_t)rc.z + fx - 1) / fx;
        const int32_t x = rc.x + (int32_t)((tile % tiles_x) * fx + lane % fx);
        const int32_t y = rc.y + (int32_t)((tile / tiles_x) * fy + lane / fx);
        if (x < rc.x + rc.z && y < rc.y + rc.w && x >= 0 && y >= 0 && x < (int32_t)v.W && y < (int32_t)v.H) {
            float org[3], dir[3];
            pixel_ray(v, (uint32_t)x, (uint32_t)y, org, dir);
            BlockRay r;
            if (block_ray(v, org, dir, *rb, r)) {
                const char* base = reinterpret_cast<const char*>(fa.bricks);
                const size_t esz = Fmt == S3R_BRICK_F32 ? 4 : 2;
                float scale = 1.f, offset = 0.f;
                if (Fmt != S3R_BRICK_F32) {
                    const float2 so = fa.scale_offset[rb->block];
                    scale = so.x;
                    offset = so.y;
                }
                const Premul p = march_block<Fmt, kTex>(v, r, base + rb->brick_off * esz, scale, offset, rb->depth,
                                                        tf, of, taken);
                if (!(p.r == 0.f && p.g == 0.f && p.b == 0.f && p.a == 0.f)) {
                    const uint32_t ix = cell % m, iy = (cell / m) % m, iz = cell / (m * m);
                    const uint32_t k = ray_rank(dir, ix, iy, iz, m);
                    const uint64_t pix = (uint64_t)y * v.W + (uint32_t)x;
                    sa.seg[(uint64_t)k * npix + pix] = make_float4(p.r, p.g, p.b, p.a);
                    atomicOr(&sa.mask[(uint64_t)(k >> 6) * npix + pix], 1ull << (k & 63));
                }
            }
        }
        item = __shfl_sync(0xffffffffu, next, 0);
        desc.x = __shfl_sync(0xffffffffu, ndesc.x, 0);
        desc.y = __shfl_sync(0xffffffffu, ndesc.y, 0);
    }
    if (fa.samples) {
        unsigned long long t = taken;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0 && t) atomicAdd(fa.samples, t);
    }
}

// Front-to-back blend of every pixel's block results in rank order -- the
// order frame_render_kernel's walk meets the blocks in -- with its arithmetic
// and its alpha_stop rule; clears the masks and the work-queue counter for the
// next frame.
__global__ void frame_composite_kernel(FrameArgs fa, SegArgs sa)
{
    const s3r_view v = *fa.view;
    const uint64_t npix = (uint64_t)v.W * v.H;
    const uint64_t pix = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pix == 0) *sa.queue = 0u;
    if (pix >= npix) return;
    unsigned long long bits[kSegMaskWords];
#pragma unroll
    for (uint32_t w = 0; w < kSegMaskWords; ++w) {
        bits[w] = 0ull;
        if (w < sa.words) {
            bits[w] = sa.mask[w * npix + pix];
            if (bits[w]) sa.mask[w * npix + pix] = 0ull;
        }
    }
    Premul acc{0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (uint32_t w = 0; w < kSegMaskWords; ++w) {
        while (bits[w] && !(acc.a > v.alpha_stop)) {
            const uint32_t k = 64 * w + (uint32_t)(__ffsll((long long)bits[w]) - 1);
            bits[w] &= bits[w] - 1;
            const float4 p = sa.seg[(uint64_t)k * npix + pix];
            const float T = __fsub_rn(1.f, acc.a);
            acc.r = __fmaf_rn(T, p.x, acc.r);
            acc.g = __fmaf_rn(T, p.y, acc.g);
            acc.b = __fmaf_rn(T, p.z, acc.b);
            acc.a = __fmaf_rn(T, p.w, acc.a);
        }
    }
    write_pixel(fa, v, (uint32_t)(pix % v.W), (uint32_t)(pix / v.W), acc);
}

// Batched field modes (F32 bricks): one lane per ray walks the blocks front
// to back, each block marched as render_block_mode_kernel marches it
// (march_block_mode), and the blocks' contributions are combined in float: the
// colour modes' block results composited front to back (premultiplied) with
// no ARGB8 rounding between blocks, max intensity the maximum over the
// blocks, and a multi-level mode without levels clears the pixel (what lies
// behind the first block it meets is erased, as the per-block path erases it).
template <bool kTex>
__global__ void frame_render_mode_kernel(FrameArgs fa, const s3r_presentation pr, const float* __restrict__ bricks2)
{
    extern __shared__ float4 tf[];
    const s3r_view v = *fa.view;
    const uint32_t nthreads = blockDim.x * blockDim.y;
    const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (uint32_t i = tid; i < v.tf_n; i += nthreads) tf[i] = reinterpret_cast<const float4*>(fa.tf)[i];
    __syncthreads();
    const uint32_t vx = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t vy = blockIdx.y * blockDim.y + threadIdx.y;
    if (vx >= v.W || vy >= v.H) return;
    const bool mip = pr.mode == S3R_MODE_MAX_INTENSITY;
    Premul acc{0.f, 0.f, 0.f, 0.f};
    bool have_max = false;
    float best = 0.f;
    const int4 cv = *reinterpret_cast<const int4*>(fa.cover);
    if ((int32_t)vx >= cv.x && (int32_t)vx < cv.z && (int32_t)vy >= cv.y && (int32_t)vy < cv.w) {
        float org[3], dir[3];
        pixel_ray(v, vx, vy, org, dir);
        const float* bricks = reinterpret_cast<const float*>(fa.bricks);
        walk_blocks(org, dir, v.level, [&](uint32_t b, uint32_t, uint32_t, uint32_t) {
            const RenderBlock* rb = &fa.table[b];
            const uint32_t depth = rb->depth;
            if (depth == 0xffffffffu) return true;
            const int4 rc = *reinterpret_cast<const int4*>(rb->rect);
            const int32_t rca[4] = {rc.x, rc.y, rc.z, rc.w};
            if (!pixel_in_rect(rca, vx, vy)) return true;
            BlockRay r;
            if (!block_ray(v, org, dir, *rb, r)) return true;
            const BrickSampler<kTex> smp{bricks + rb->brick_off, bricks2 ? bricks2 + rb->brick_off : nullptr, dim_of(r),
                                         tf, v.tf_n};
            const ModeOut o = march_block_mode(v, pr, smp, r, depth);
            if (o.kind == ModeOut::kMax) {
                if (!have_max || o.t > best) best = o.t;
                have_max = true;
            } else if (o.kind == ModeOut::kBlend) {
                const float T = __fsub_rn(1.f, acc.a);
                acc.r = __fmaf_rn(T, __fmul_rn(o.acc.x, o.acc.w), acc.r);
                acc.g = __fmaf_rn(T, __fmul_rn(o.acc.y, o.acc.w), acc.g);
                acc.b = __fmaf_rn(T, __fmul_rn(o.acc.z, o.acc.w), acc.b);
                acc.a = __fmaf_rn(T, o.acc.w, acc.a);
            } else if (o.kind == ModeOut::kClear) {
                return false;
            }
            return mip || !(acc.a > v.alpha_stop);
        });
    }
    const size_t o = (size_t)(v.H - 1 - vy) * v.W + vx;
    if (mip) {
        if (fa.rgba)
            reinterpret_cast<float4*>(fa.rgba)[o] =
                have_max ? make_float4(best, best, best, 1.f) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (fa.argb) fa.argb[o] = have_max ? __float_as_uint(best) : 0x7fc00000u;
        return;
    }
    write_pixel(fa, v, vx, vy, acc);
}

// ---------------------------------------------------------------- adjoint

// The 8 texels of a cell (F32 brick, 32-bit offsets), their offsets, and the trilinear value (false on a NaN).
__device__ __forceinline__ void cell_offsets(const Cell& c, Dim g, uint32_t off[8])
{
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint32_t x = (q & 1) ? c.i1[0] : c.i0[0];
        const uint32_t y = (q & 2) ? c.i1[1] : c.i0[1];
        const uint32_t z = (q & 4) ? c.i1[2] : c.i0[2];
        off[q] = (z * g.n + y) * g.pitch + x;
    }
}

__device__ __forceinline__ void fetch_cell(const float* brick, const Cell& c, Dim g, float t[8])
{
    uint32_t off[8];
    cell_offsets(c, g, off);
#pragma unroll
    for (int q = 0; q < 8; ++q) t[q] = __ldg(brick + off[q]);
}

__device__ __forceinline__ bool filter_cell(const Cell& c, const float t[8], float& val)
{
    bool bad = false;
#pragma unroll
    for (int q = 0; q < 8; ++q) bad |= isnan(t[q]);
    if (bad) return false;
    const float x00 = __fmaf_rn(c.f[0], t[1] - t[0], t[0]);
    const float x10 = __fmaf_rn(c.f[0], t[3] - t[2], t[2]);
    const float x01 = __fmaf_rn(c.f[0], t[5] - t[4], t[4]);
    const float x11 = __fmaf_rn(c.f[0], t[7] - t[6], t[6]);
    const float y0 = __fmaf_rn(c.f[1], x10 - x00, x00);
    const float y1 = __fmaf_rn(c.f[1], x11 - x01, x01);
    val = __fmaf_rn(c.f[2], y1 - y0, y0);
    return true;
}

// For L = 1/2 sum (I - target)^2 with I = (C/A, A) the premultiplied composite
// of the kept samples (front to back, T_k = prod_{j<k} (1 - a_k)):
//   dC/dc_k = T_k a_k,  dC/da_k = T_k c_k - (C - C_{<=k}) / (1 - a_k),
//   dA/da_k = (1 - A) / (1 - a_k),
// a_k = 1 - (1 - alpha_tf * of)^il, c_k / alpha_tf linear in the table
// entries around v01, v01 linear in the trilinear value.
__global__ void __launch_bounds__(128, 4) frame_backward_kernel(FrameArgs fa)
{
    extern __shared__ float4 sm[];
    const s3r_view v = *fa.view;
    float4* tf = sm;
    const uint32_t nthreads = blockDim.x * blockDim.y;
    const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (uint32_t i = tid; i < v.tf_n; i += nthreads) tf[i] = reinterpret_cast<const float4*>(fa.tf)[i];
    __syncthreads();
    // The transfer-function gradient goes to one of kDtfParts copies in global
    // memory, an RGBA float4 reduction per table entry (fire and forget).  The copy
    // is picked by CTA (modulo kDtfCtaGroups) and by lane (modulo kDtfLaneGroups):
    // neighbouring rays -- neighbouring lanes -- add to the same entry at the same
    // time, and reductions on one address serialize.  (Shared-memory atomics
    // stalled the warps on exactly those collisions.)
    float4* dtf4 = reinterpret_cast<float4*>(fa.dtf_part) +
                   (size_t)(((blockIdx.y * gridDim.x + blockIdx.x) % kDtfCtaGroups) * kDtfLaneGroups +
                            (tid & 31) % kDtfLaneGroups) * v.tf_n;
    const uint32_t vx = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t vy = blockIdx.y * blockDim.y + threadIdx.y;
    if (vx < v.W && vy < v.H) {
        const size_t o = (size_t)(v.H - 1 - vy) * v.W + vx;
        const float4 I = reinterpret_cast<const float4*>(fa.fwd_rgba)[o];
        const float4 gI = reinterpret_cast<const float4*>(fa.dl_drgba)[o];
        const float A = I.w;
        float gC[3] = {0.f, 0.f, 0.f};
        float gA = gI.w;
        const float Ct[3] = {I.x * A, I.y * A, I.z * A};
        if (A > 0.f) {
            const float inv = 1.f / A;
            gC[0] = gI.x * inv;
            gC[1] = gI.y * inv;
            gC[2] = gI.z * inv;
            gA -= (gI.x * I.x + gI.y * I.y + gI.z * I.z) * inv;
        }
        const bool active = (gC[0] != 0.f || gC[1] != 0.f || gC[2] != 0.f || gA != 0.f);
        if (active) {
            float org[3], dir[3];
            pixel_ray(v, vx, vy, org, dir);
            const float span = v.field_max - v.field_min;
            const float inv_span = 1.f / span;
            const float of = (v.threshold - v.field_min) / span;
            float T = 1.f, Cpre[3] = {0.f, 0.f, 0.f};
            float accA = 0.f;
            uint32_t tf_i0 = 0xffffffffu, tf_i1 = 0xffffffffu;
            float tf_a[4] = {0.f, 0.f, 0.f, 0.f}, tf_b[4] = {0.f, 0.f, 0.f, 0.f};
            auto flush_tf = [&]() {
                if (tf_i0 == 0xffffffffu) return;
                atomicAdd(&dtf4[tf_i0], make_float4(tf_a[0], tf_a[1], tf_a[2], tf_a[3]));
                atomicAdd(&dtf4[tf_i1], make_float4(tf_b[0], tf_b[1], tf_b[2], tf_b[3]));
#pragma unroll
                for (int ch = 0; ch < 4; ++ch) {
                    tf_a[ch] = 0.f;
                    tf_b[ch] = 0.f;
                }
            };
            walk_blocks(org, dir, v.level, [&](uint32_t b, uint32_t ix, uint32_t iy, uint32_t iz) {
                const RenderBlock* rb = &fa.table[b];
                const uint32_t depth = rb->depth;
                if (depth == 0xffffffffu) return true;
                const int4 rc = *reinterpret_cast<const int4*>(rb->rect);
                const int32_t rca[4] = {rc.x, rc.y, rc.z, rc.w};
                if (!pixel_in_rect(rca, vx, vy)) return true;
                BlockRay r;
                if (!block_ray(v, org, dir, *rb, r)) return true;
                const float* brick = reinterpret_cast<const float*>(fa.bricks) + rb->brick_off;
                float* gdense = fa.ddense + rb->brick_off;
                const float il = layer_exponent(depth, v.level, v.quality);
                float Ab = 0.f;
                // one sample's gradients from its cell and texels; false once the block is opaque
                auto step_sample = [&](const Cell& cell, const float* tcur) -> bool {
                    float val;
                    if (!filter_cell(cell, tcur, val)) return true;
                    uint32_t off[8];
                    cell_offsets(cell, dim_of(r), off);
                    const float fx = cell.f[0], fy = cell.f[1], fz = cell.f[2];
                    // the forward's v01 up to the last ulp (a reciprocal instead of the division)
                    const float v01 = __fmul_rn(__fsub_rn(val, v.field_min), inv_span);
                    const TfSample ts = tf_lookup(tf, v.tf_n, v01);
                    const float base = __fmaf_rn(-ts.c.w, of, 1.f);
                    const float pw = __powf(base, il);
                    const float a = __fsub_rn(1.f, pw);
                    // derivatives need no correctly rounded divisions: fast reciprocals
                    const float dadc = base > 0.f ? __fdividef(il * pw, base) * of : 0.f;
                    const float wa = T * a;
                    const float col[3] = {ts.c.x, ts.c.y, ts.c.z};
                    float g_col[4];
                    float g_a = 0.f;
                    const float om = 1.f - a;
                    const float inv_om = om > 1e-12f ? __fdividef(1.f, om) : 0.f;
#pragma unroll
                    for (int ch = 0; ch < 3; ++ch) {
                        const float cpost = __fmaf_rn(wa, col[ch], Cpre[ch]);
                        g_col[ch] = gC[ch] * wa;
                        g_a += gC[ch] * (T * col[ch] - (Ct[ch] - cpost) * inv_om);
                        Cpre[ch] = cpost;
                    }
                    g_a += gA * (1.f - A) * inv_om;
                    g_col[3] = g_a * dadc;
                    // transfer-function table: accumulate the two entries of the current
                    // pair in registers; when the pair changes, an entry the new pair
                    // shares (a ray moving to the next interval) keeps its sum and only
                    // the other one goes to shared memory
                    const float f = ts.f;
                    if (ts.i0 != tf_i0 || ts.i1 != tf_i1) {
                        if (tf_i0 != 0xffffffffu && ts.i0 == tf_i1 && ts.i0 != ts.i1) {
                            // moving up: old i1 becomes new i0
                            atomicAdd(&dtf4[tf_i0], make_float4(tf_a[0], tf_a[1], tf_a[2], tf_a[3]));
#pragma unroll
                            for (int ch = 0; ch < 4; ++ch) {
                                tf_a[ch] = tf_b[ch];
                                tf_b[ch] = 0.f;
                            }
                        } else if (tf_i0 != 0xffffffffu && ts.i1 == tf_i0 && ts.i0 != ts.i1) {
                            // moving down: old i0 becomes new i1
                            atomicAdd(&dtf4[tf_i1], make_float4(tf_b[0], tf_b[1], tf_b[2], tf_b[3]));
#pragma unroll
                            for (int ch = 0; ch < 4; ++ch) {
                                tf_b[ch] = tf_a[ch];
                                tf_a[ch] = 0.f;
                            }
                        } else {
                            flush_tf();
                        }
                        tf_i0 = ts.i0;
                        tf_i1 = ts.i1;
                    }
#pragma unroll
                    for (int ch = 0; ch < 4; ++ch) {
                        tf_a[ch] = __fmaf_rn(g_col[ch], 1.f - f, tf_a[ch]);
                        tf_b[ch] = __fmaf_rn(g_col[ch], f, tf_b[ch]);
                    }
                    // dense values
                    if (!ts.clamped) {
                        const float4 p = tf[ts.i0], q = tf[ts.i1];
                        const float g_v01 = (g_col[0] * (q.x - p.x) + g_col[1] * (q.y - p.y) +
                                             g_col[2] * (q.z - p.z) + g_col[3] * (q.w - p.w)) *
                                            (float)v.tf_n;
                        const float g_val = g_v01 * inv_span;
                        if (g_val != 0.f) {
#pragma unroll
                            for (int qn = 0; qn < 8; ++qn) {
                                const float w = ((qn & 1) ? fx : 1.f - fx) * ((qn & 2) ? fy : 1.f - fy) *
                                                ((qn & 4) ? fz : 1.f - fz);
                                atomicAdd(&gdense[off[qn]], g_val * w);
                            }
                        }
                    }
                    T *= om;
                    Ab = __fadd_rn(Ab, __fmul_rn(__fsub_rn(1.f, Ab), a));
                    return !(Ab > kAlphaThreshold);
                };
                // software-pipelined as the forward march, unrolled by two with two
                // buffers: sample i's texels load while sample i-1's gradients form
                Cell ca, cb;
                float ta[8], tb[8];
                if (r.samples > 1) {
                    sample_cell(r, 0, ca);
                    fetch_cell(brick, ca, dim_of(r), ta);
                }
                for (int i = 1; i < r.samples; i += 2) {
                    if (i + 1 < r.samples) {
                        sample_cell(r, i, cb);
                        fetch_cell(brick, cb, dim_of(r), tb);
                    }
                    if (!step_sample(ca, ta)) break;
                    if (i + 1 >= r.samples) break;
                    if (i + 2 < r.samples) {
                        sample_cell(r, i + 1, ca);
                        fetch_cell(brick, ca, dim_of(r), ta);
                    }
                    if (!step_sample(cb, tb)) break;
                }
                // block composite exactly as the forward kernel forms it
                accA = __fmaf_rn(__fsub_rn(1.f, accA), Ab, accA);
                return !(accA > v.alpha_stop);
            });
            flush_tf();
        }
    }
}

__global__ void dtf_reduce_kernel(const float* __restrict__ part, float* __restrict__ dtf, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = 0.f;
    for (uint32_t p = 0; p < kDtfParts; ++p) g += part[(size_t)p * n + i];
    dtf[i] += g;
}

} // namespace

cudaError_t launch_render_block_mode(const s3r_view* view_host, const s3r_presentation* pres, const float* brick,
                                     const float* brick2, const RenderBlock& rb, const float* tf, uint32_t* viewport,
                                     cudaStream_t s)
{
    if (rb.rect[2] <= 0 || rb.rect[3] <= 0) return cudaSuccess;
    dim3 block(16, 8);
    dim3 grid((rb.rect[2] + 15) / 16, (rb.rect[3] + 7) / 8);
    const size_t smem = view_host->tf_n * sizeof(float4);
    if (view_host->filter == S3R_FILTER_TEXTURE)
        render_block_mode_kernel<true><<<grid, block, smem, s>>>(*view_host, *pres, brick, brick2, rb,
                                                                 reinterpret_cast<const float4*>(tf), viewport);
    else
        render_block_mode_kernel<false><<<grid, block, smem, s>>>(*view_host, *pres, brick, brick2, rb,
                                                                  reinterpret_cast<const float4*>(tf), viewport);
    return cudaGetLastError();
}

cudaError_t launch_render_block_texture(const s3r_view* view_host, const s3r_presentation* pres, uint64_t field,
                                       uint64_t field2, uint64_t tf_tex, const RenderBlock& rb, uint32_t* viewport,
                                       cudaStream_t s)
{
    if (rb.rect[2] <= 0 || rb.rect[3] <= 0) return cudaSuccess;
    const uint32_t tx = tex_tile_x(pres->mode), ty = tex_tile_y(pres->mode);
    dim3 block(tx, ty);
    dim3 grid((rb.rect[2] + tx - 1) / tx, (rb.rect[3] + ty - 1) / ty);
    const TextureSampler smp{(cudaTextureObject_t)field, (cudaTextureObject_t)field2, (cudaTextureObject_t)tf_tex};
    switch (pres->mode) {
    case S3R_MODE_ISOSURFACE:
        render_block_texture_kernel<S3R_MODE_ISOSURFACE><<<grid, block, 0, s>>>(*view_host, *pres, smp, rb, viewport);
        break;
    case S3R_MODE_ISOSURFACES:
        render_block_texture_kernel<S3R_MODE_ISOSURFACES><<<grid, block, 0, s>>>(*view_host, *pres, smp, rb, viewport);
        break;
    case S3R_MODE_MAX_INTENSITY:
        render_block_texture_kernel<S3R_MODE_MAX_INTENSITY><<<grid, block, 0, s>>>(*view_host, *pres, smp, rb,
                                                                                   viewport);
        break;
    case S3R_MODE_ARGB:
        render_block_texture_kernel<S3R_MODE_ARGB><<<grid, block, 0, s>>>(*view_host, *pres, smp, rb, viewport);
        break;
    case S3R_MODE_ARGB_LIGHT:
        render_block_texture_kernel<S3R_MODE_ARGB_LIGHT><<<grid, block, 0, s>>>(*view_host, *pres, smp, rb, viewport);
        break;
    case S3R_MODE_DOMAIN_VOXELS:
        render_block_texture_kernel<S3R_MODE_DOMAIN_VOXELS><<<grid, block, 0, s>>>(*view_host, *pres, smp, rb,
                                                                                   viewport);
        break;
    case S3R_MODE_VALUE_ON_ISOSURFACE:
        render_block_texture_kernel<S3R_MODE_VALUE_ON_ISOSURFACE><<<grid, block, 0, s>>>(*view_host, *pres, smp, rb,
                                                                                         viewport);
        break;
    default:
        render_block_texture_kernel<S3R_MODE_VALUE_ON_ISOSURFACES><<<grid, block, 0, s>>>(*view_host, *pres, smp, rb,
                                                                                          viewport);
        break;
    }
    return cudaGetLastError();
}

cudaError_t launch_render_block_argb(const s3r_view* view_host, const float* brick, const RenderBlock& rb,
                                     const float* tf, uint32_t* viewport, cudaStream_t s)
{
    if (rb.rect[2] <= 0 || rb.rect[3] <= 0) return cudaSuccess;
    dim3 block(16, 8);
    dim3 grid((rb.rect[2] + 15) / 16, (rb.rect[3] + 7) / 8);
    render_block_argb_kernel<<<grid, block, view_host->tf_n * sizeof(float4), s>>>(
        *view_host, brick, rb, reinterpret_cast<const float4*>(tf), viewport);
    return cudaGetLastError();
}

template <int Fmt, bool kTex>
cudaError_t launch_frame_render_fmt(const FrameArgs& a, dim3 grid, dim3 block, size_t smem, uint32_t R, cudaStream_t s)
{
    switch (R) {
    case 1: frame_render_kernel<Fmt, 1, kTex><<<grid, block, smem, s>>>(a); break;
    case 2: frame_render_kernel<Fmt, 2, kTex><<<grid, block, smem, s>>>(a); break;
    case 4: frame_render_kernel<Fmt, 4, kTex><<<grid, block, smem, s>>>(a); break;
    default: frame_render_kernel<Fmt, 8, kTex><<<grid, block, smem, s>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_frame_render(const FrameArgs& a, uint32_t W, uint32_t H, uint32_t tf_n, uint32_t fmt,
                                uint32_t tile_shape, uint32_t filter, cudaStream_t s)
{
    // tile_shape: CTA pixel shape (low 2 bits) and lanes per ray R = 2^(bits 2-3)
    const uint32_t shape = tile_shape % kRenderShapes;
    const uint32_t R = 1u << ((tile_shape / kRenderShapes) % 4);
    const int sx = kRenderShapeX[shape], sy = kRenderShapeY[shape];
    // R lanes per pixel: keep 128-ish threads per CTA by narrowing the pixel tile
    const int px = sx / (int)R > 0 ? sx / (int)R : 1;
    dim3 block(px * R, sy);
    dim3 grid((W + px - 1) / px, (H + sy - 1) / sy);
    const size_t smem = tf_n * sizeof(float4);
    const bool tex = filter == S3R_FILTER_TEXTURE;
    switch (fmt) {
    case S3R_BRICK_F32:
        return tex ? launch_frame_render_fmt<S3R_BRICK_F32, true>(a, grid, block, smem, R, s)
                   : launch_frame_render_fmt<S3R_BRICK_F32, false>(a, grid, block, smem, R, s);
    case S3R_BRICK_F16:
        return tex ? launch_frame_render_fmt<S3R_BRICK_F16, true>(a, grid, block, smem, R, s)
                   : launch_frame_render_fmt<S3R_BRICK_F16, false>(a, grid, block, smem, R, s);
    case S3R_BRICK_BF16:
        return tex ? launch_frame_render_fmt<S3R_BRICK_BF16, true>(a, grid, block, smem, R, s)
                   : launch_frame_render_fmt<S3R_BRICK_BF16, false>(a, grid, block, smem, R, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int Fmt, bool kTex>
cudaError_t launch_frame_segments_fmt(const FrameArgs& a, const SegArgs& sa, uint32_t fx, dim3 block, size_t smem,
                                      uint32_t sms, cudaStream_t s)
{
    auto kernel = frame_segments_kernel<Fmt, kTex>;
    if (smem > 48 * 1024) {
        cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, (int)(block.x * block.y), smem);
    if (err != cudaSuccess) return err;
    kernel<<<sms * (uint32_t)(per_sm > 0 ? per_sm : 1), block, smem, s>>>(a, sa, fx);
    return cudaGetLastError();
}

cudaError_t launch_frame_segments(const FrameArgs& a, const SegArgs& sa, uint32_t W, uint32_t H, uint32_t tf_n,
                                  uint32_t fmt, uint32_t shape, uint32_t filter, uint32_t sms, cudaStream_t s)
{
    if (sa.words > kSegMaskWords) return cudaErrorInvalidValue;
    shape %= kSegShapes;
    const uint32_t fx = (uint32_t)kSegShapeX[shape];
    const dim3 block(128); // four warps, each on its own items
    const size_t smem = tf_n * sizeof(float4);
    const bool tex = filter == S3R_FILTER_TEXTURE;
    cudaError_t err;
    switch (fmt) {
    case S3R_BRICK_F32:
        err = tex ? launch_frame_segments_fmt<S3R_BRICK_F32, true>(a, sa, fx, block, smem, sms, s)
                  : launch_frame_segments_fmt<S3R_BRICK_F32, false>(a, sa, fx, block, smem, sms, s);
        break;
    case S3R_BRICK_F16:
        err = tex ? launch_frame_segments_fmt<S3R_BRICK_F16, true>(a, sa, fx, block, smem, sms, s)
                  : launch_frame_segments_fmt<S3R_BRICK_F16, false>(a, sa, fx, block, smem, sms, s);
        break;
    case S3R_BRICK_BF16:
        err = tex ? launch_frame_segments_fmt<S3R_BRICK_BF16, true>(a, sa, fx, block, smem, sms, s)
                  : launch_frame_segments_fmt<S3R_BRICK_BF16, false>(a, sa, fx, block, smem, sms, s);
        break;
    default: return cudaErrorInvalidValue;
    }
    if (err != cudaSuccess) return err;
    const uint64_t npix = (uint64_t)W * H;
    frame_composite_kernel<<<(uint32_t)((npix + 255) / 256), 256, 0, s>>>(a, sa);
    return cudaGetLastError();
}

cudaError_t launch_frame_render_mode(const FrameArgs& a, const s3r_presentation& pres, const float* bricks2,
                                     uint32_t W, uint32_t H, uint32_t tf_n, uint32_t filter, cudaStream_t s)
{
    dim3 block(16, 8);
    dim3 grid((W + 15) / 16, (H + 7) / 8);
    const size_t smem = tf_n * sizeof(float4);
    if (filter == S3R_FILTER_TEXTURE) frame_render_mode_kernel<true><<<grid, block, smem, s>>>(a, pres, bricks2);
    else frame_render_mode_kernel<false><<<grid, block, smem, s>>>(a, pres, bricks2);
    return cudaGetLastError();
}

cudaError_t launch_frame_backward(const FrameArgs& a, uint32_t W, uint32_t H, uint32_t tf_n, cudaStream_t s)
{
    // 32x2-pixel CTAs: measured 2-3 % faster than 32x4 on cfg5 (the rays' work is uneven; smaller CTAs
    // leave less idle at the end)
    dim3 block(32, 2);
    dim3 grid((W + 31) / 32, (H + 1) / 2);
    const size_t smem = tf_n * sizeof(float4);
    if (smem > 48 * 1024) {
        cudaError_t err =
            cudaFuncSetAttribute(frame_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    frame_backward_kernel<<<grid, block, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_dtf_reduce(const float* part, float* dtf, uint32_t n, cudaStream_t s)
{
    dtf_reduce_kernel<<<(n + 255) / 256, 256, 0, s>>>(part, dtf, n);
    return cudaGetLastError();
}

} // namespace s3r
