/*
 * s3r oracle — TEST INFRASTRUCTURE ONLY (see s3r_oracle.h).
 * Plain-C restatement of the reference's hot path; compiled with -ffp-contract=off.
 */
#define _POSIX_C_SOURCE 200809L /* fseeko */
#include "s3r_oracle.h"

#include <stdio.h>
#include <sys/types.h>

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================
 * Dense interpolation
 * include/s3dmm/DenseFieldInterpolator.hpp:198-419 (static interpolate).
 * Level by level (:243), every cube of the level (:256-410) gets its
 * edge, face and cell midpoints, in that order (HypercubeWalker.hpp:71-127,
 * NestedHypercubeWalker walks lower dimensions first); a midpoint that is
 * still NaN becomes the mean of its stencil (1/2, 1/4, 1/6 weights, summed
 * in the reference's order :277, :318-320, :374-377), or the no-field value
 * when any stencil value is the no-field value.  Finally the no-field value
 * becomes NaN (:416-418).  Midpoints shared between cubes get the same value
 * from every cube, so visiting each level's edges, then faces, then cells
 * over the whole grid yields the reference's result exactly.
 * ====================================================================== */

#define ORC_DEFINE_INTERP(NAME, T, NOFIELD, HALF, QUARTER, SIXTH)                                     \
    int NAME(const uint16_t* n2i, const float* sparse, uint32_t n, uint32_t depth, T* dense)          \
    {                                                                                                 \
        const uint32_t e = (1u << depth) + 1u;                                                         \
        const uint64_t count = (uint64_t)e * e * e;                                                   \
        const T nofield = (NOFIELD);                                                                  \
        for (uint64_t i = 0; i < count; ++i)                                                          \
            dense[i] = (T)NAN;                                                                        \
        for (uint32_t i = 0; i < n; ++i) {                                                            \
            uint64_t o = ((uint64_t)n2i[3 * i + 2] * e + n2i[3 * i + 1]) * e + n2i[3 * i];            \
            dense[o] = (T)sparse[i];                                                                  \
        }                                                                                             \
        const uint64_t stride[3] = {1, e, (uint64_t)e * e};                                           \
        for (uint32_t level = 0; level < depth; ++level) {                                            \
            const uint32_t shift = depth - level; /* cube size 2^shift */                             \
            const uint32_t half = 1u << (shift - 1);                                                  \
            const uint32_t cubes = 1u << level;                                                       \
            /* kind 1: edges, 2: faces, 3: cells */                                                   \
            for (int kind = 1; kind <= 3; ++kind) {                                                   \
                for (uint32_t cz = 0; cz < cubes; ++cz)                                               \
                for (uint32_t cy = 0; cy < cubes; ++cy)                                               \
                for (uint32_t cx = 0; cx < cubes; ++cx) {                                             \
                    const uint32_t base[3] = {cx << shift, cy << shift, cz << shift};                 \
                    /* every midpoint of this cube with `kind` odd axes: choose the odd axes,        \
                       and 0 or 1 (low/high side) for each even axis */                               \
                    for (uint32_t mask = 1; mask < 8; ++mask) {                                       \
                        int nodd = (mask & 1) + ((mask >> 1) & 1) + ((mask >> 2) & 1);                \
                        if (nodd != kind) continue;                                                   \
                        for (uint32_t side = 0; side < 8; ++side) {                                   \
                            if (side & mask) continue; /* side bits only on even axes */              \
                            uint32_t p[3];                                                            \
                            for (int d = 0; d < 3; ++d)                                               \
                                p[d] = base[d] + (((mask >> d) & 1) ? half                            \
                                                                    : (((side >> d) & 1) << shift));  \
                            uint64_t o = (p[2] * (uint64_t)e + p[1]) * e + p[0];                      \
                            if (!isnan((double)dense[o])) continue;                                   \
                            T v[6];                                                                   \
                            int k = 0, masked = 0;                                                    \
                            for (int d = 0; d < 3; ++d) {                                             \
                                if (!((mask >> d) & 1)) continue;                                     \
                                v[k] = dense[o - (uint64_t)half * stride[d]];                         \
                                v[k + 1] = dense[o + (uint64_t)half * stride[d]];                     \
                                masked |= (v[k] == nofield) | (v[k + 1] == nofield);                  \
                                k += 2;                                                               \
                            }                                                                         \
                            if (masked)                                                               \
                                dense[o] = nofield;                                                   \
                            else if (kind == 1)                                                       \
                                dense[o] = (HALF) * (v[0] + v[1]);                                    \
                            else if (kind == 2)                                                       \
                                dense[o] = (QUARTER) * (v[0] + v[1] + v[2] + v[3]);                   \
                            else                                                                      \
                                dense[o] = (SIXTH) * (v[0] + v[1] + v[2] + v[3] + v[4] + v[5]);       \
                        }                                                                             \
                    }                                                                                 \
                }                                                                                     \
            }                                                                                         \
        }                                                                                             \
        for (uint64_t i = 0; i < count; ++i)                                                          \
            if (dense[i] == nofield) dense[i] = (T)NAN;                                               \
        return (int)count;                                                                            \
    }

ORC_DEFINE_INTERP(orc_interp_dense_f32, float, ORC_NO_FIELD_VALUE, 0.5f, 0.25f, (float)(1. / 6))
ORC_DEFINE_INTERP(orc_interp_dense_f64, double, (double)ORC_NO_FIELD_VALUE, 0.5, 0.25, 1. / 6)

/* ======================================================================
 * Block geometry — DenseFieldRenderer_cu.cu:337-350 (cube) and :374-409 (view rect).
 * ====================================================================== */

void orc_block_cube(uint32_t level, const uint32_t idx[3], float center[3], float* half_size)
{
    const float top = 5.f;
    const float h = top / (float)(1u << level);
    for (int d = 0; d < 3; ++d)
        center[d] = -top + h * (float)(1u + (idx[d] << 1));
    *half_size = h;
}

static int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

void orc_block_view_rect(const orc_view* v, const float r[9], const float t[3], const uint32_t idx[3],
                         int32_t rect[4])
{
    float c[3], h;
    orc_block_cube(v->level, idx, c, &h);
    const float lcam = 0.01f * 2 * 5.f;
    const float pixel = v->cam.h / (float)v->H;
    int have = 0, full = 0;
    int xmin = 0, xmax = 0, ymin = 0, ymax = 0;
    for (int i = 0; i < 8; ++i) {
        float p[3];
        for (int d = 0; d < 3; ++d)
            p[d] = c[d] + (float)((int)(((i >> d) & 1) << 1) - 1) * h;
        float q[3];
        for (int a = 0; a < 3; ++a)
            q[a] = r[3 * a] * p[0] + r[3 * a + 1] * p[1] + r[3 * a + 2] * p[2] + t[a];
        int sx, sy;
        if (v->cam.ortho) {
            sx = clampi((int)(q[0] / pixel) + (int)(v->W >> 1), 0, (int)v->W - 1);
            sy = clampi((int)(q[1] / pixel) + (int)(v->H >> 1), 0, (int)v->H - 1);
        } else {
            if (q[2] >= 0) { full = 1; break; }
            sx = clampi((int)(-q[0] / q[2] * lcam / pixel) + (int)(v->W >> 1), 0, (int)v->W - 1);
            sy = clampi((int)(-q[1] / q[2] * lcam / pixel) + (int)(v->H >> 1), 0, (int)v->H - 1);
        }
        if (!have) { xmin = xmax = sx; ymin = ymax = sy; have = 1; }
        else {
            if (sx < xmin) xmin = sx;
            if (sx > xmax) xmax = sx;
            if (sy < ymin) ymin = sy;
            if (sy > ymax) ymax = sy;
        }
    }
    if (full) {
        /* bb << {0,0} << viewportSize on top of the corners seen so far */
        if (!have) { xmin = ymin = 0; xmax = (int)v->W; ymax = (int)v->H; }
        else {
            if (0 < xmin) xmin = 0;
            if (0 < ymin) ymin = 0;
            if ((int)v->W > xmax) xmax = (int)v->W;
            if ((int)v->H > ymax) ymax = (int)v->H;
        }
    }
    rect[0] = xmin;
    rect[1] = ymin;
    rect[2] = xmax - xmin;
    rect[3] = ymax - ymin;
}

/* ======================================================================
 * Ray set-up — DenseFieldRenderer_cu.cu:72-181.  Every float operation is
 * written out in the order the GPU kernels use (no contraction), so both
 * sides take the same samples; the reference itself leaves rounding to its
 * compiler.
 * ====================================================================== */

typedef struct orc_ray {
    float org[3];
    float dir[3];
    float tau_enter_raw; /* before the clamp to the screen plane */
    float tau_enter;
    float tau_exit;
    int sample_count;
    float p0[3];
    float step[3];
    float origin[3]; /* texture-space origin (cube corner minus half a texel) */
    float factor;    /* world -> texel scale */
    uint32_t n;      /* texels per edge */
} orc_ray;

static void ray_for_pixel(const orc_view* v, uint32_t vx, uint32_t vy, float org[3], float dir[3])
{
    const orc_camera* c = &v->cam;
    float x = (-0.5f + ((float)vx + 0.5f) / (float)v->W) * c->w;
    float y = (-0.5f + ((float)vy + 0.5f) / (float)v->H) * c->h;
    for (int d = 0; d < 3; ++d) {
        float ex = c->e1[d] * x;
        float ey = c->e2[d] * y;
        if (c->ortho) {
            org[d] = (c->eye[d] + ex) + ey;
            dir[d] = c->n[d];
        } else {
            org[d] = c->eye[d];
            dir[d] = (c->n[d] + ex) + ey;
        }
    }
}

/* Slab test against one cube (:81-166); returns 1 when the ray renders it. */
static int ray_block(const orc_view* v, const float org[3], const float dir[3], const float c[3], float h,
                     uint32_t depth, orc_ray* out)
{
    float te = 1.f, tx = 0.f;
    const float tol = 1e-10f;
    for (int a = 0; a < 3; ++a) {
        if (!(fabsf(dir[a]) > tol)) continue;
        int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        if (b1 > b2) { int s = b1; b1 = b2; b2 = s; }
        for (int side = 0; side < 2; ++side) {
            float face = side ? c[a] + h : c[a] - h;
            float tau = (face - org[a]) / dir[a];
            float p1 = org[b1] + dir[b1] * tau;
            float p2 = org[b2] + dir[b2] * tau;
            if (fabsf(p1 - c[b1]) <= h && fabsf(p2 - c[b2]) <= h) {
                int enter = (dir[a] > 0) == (side == 0);
                if (enter) te = tau; else tx = tau;
            }
        }
    }
    out->tau_enter_raw = te;
    if (te < 1) te = 1;
    out->tau_enter = te;
    out->tau_exit = tx;
    if (!(tx > te)) return 0;
    const uint32_t n = (1u << depth) + 1u;
    const float texel = 2 * h / (float)n;
    float span = tx - te;
    float dotr = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
    float l1 = fabsf(dir[0]) + fabsf(dir[1]) + fabsf(dir[2]);
    float num = v->quality * span * dotr;
    float den = texel * l1;
    int s = (int)(num / den);
    float dtau = span / (float)s;
    for (int d = 0; d < 3; ++d) {
        out->step[d] = dir[d] * dtau;
        out->p0[d] = org[d] + dir[d] * te;
    }
    double thalf = (double)h + 0.5 * (double)texel;
    for (int d = 0; d < 3; ++d)
        out->origin[d] = c[d] - (float)thalf;
    out->factor = (float)((double)n / (2 * thalf));
    out->n = n;
    out->sample_count = s;
    for (int d = 0; d < 3; ++d) { out->org[d] = org[d]; out->dir[d] = dir[d]; }
    return 1;
}

/* Sample k of the march (k = 0 is the entry point): texel-space coordinate. */
static void sample_coord(const orc_ray* r, int k, float tc[3])
{
    for (int d = 0; d < 3; ++d) {
        float p = fmaf(r->step[d], (float)k, r->p0[d]);
        tc[d] = (p - r->origin[d]) * r->factor;
    }
}

/* Linear filtering with clamp addressing on unnormalized coordinates: cell corner
 * indices and fractions for one axis. */
static void filter_axis(float tc, uint32_t n, uint32_t* i0, uint32_t* i1, float* f)
{
    float xb = tc - 0.5f;
    float fl = floorf(xb);
    *f = xb - fl;
    long a = (long)fl, b = a + 1;
    long hi = (long)n - 1;
    *i0 = (uint32_t)(a < 0 ? 0 : (a > hi ? hi : a));
    *i1 = (uint32_t)(b < 0 ? 0 : (b > hi ? hi : b));
}

typedef struct corner8 {
    uint64_t off[8];
    float f[3];
} corner8;

static void corners(const orc_ray* r, const float tc[3], corner8* c)
{
    uint32_t i0[3], i1[3];
    for (int d = 0; d < 3; ++d)
        filter_axis(tc[d], r->n, &i0[d], &i1[d], &c->f[d]);
    const uint64_t n = r->n;
    for (int k = 0; k < 8; ++k) {
        uint64_t x = (k & 1) ? i1[0] : i0[0];
        uint64_t y = (k & 2) ? i1[1] : i0[1];
        uint64_t z = (k & 4) ? i1[2] : i0[2];
        c->off[k] = (z * n + y) * n + x;
    }
}

/* ======================================================================
 * Plain per-block render, FP32, reference semantics.
 * renderArgb.hpp:30-55 with blendBehind/blendAbove (cuda_blend.hpp:24-44)
 * and ARGB8 conversion (cuda_argb_transform.hpp:26-43).
 * ====================================================================== */

static float tf_lookup_f32(const float* tf, uint32_t tfn, float v01, int ch)
{
    uint32_t i0, i1;
    float f;
    filter_axis(v01 * (float)tfn, tfn, &i0, &i1, &f);
    float a = tf[4 * i0 + ch], b = tf[4 * i1 + ch];
    return a + f * (b - a);
}

static void blend_behind(float e[4], const float in[4])
{
    float da = in[3] * (1.f - e[3]);
    float a = e[3] + da;
    if (a > 0.f) {
        float ka = e[3] / a, kd = da / a;
        for (int ch = 0; ch < 3; ++ch)
            e[ch] = e[ch] * ka + in[ch] * kd;
    }
    e[3] = a;
}

static void blend_above(float e[4], const float in[4])
{
    float da = e[3] * (1.f - in[3]);
    float a = in[3] + da;
    if (a > 0.f) {
        float kd = da / a, ki = in[3] / a;
        for (int ch = 0; ch < 3; ++ch)
            e[ch] = e[ch] * kd + in[ch] * ki;
    }
    e[3] = a;
}

static void argb_to_rgba(uint32_t p, float o[4])
{
    o[0] = (float)((p >> 16) & 0xffu) / 255.f;
    o[1] = (float)((p >> 8) & 0xffu) / 255.f;
    o[2] = (float)(p & 0xffu) / 255.f;
    o[3] = (float)((p >> 24) & 0xffu) / 255.f;
}

static uint32_t rgba_to_argb(const float c[4])
{
    return ((uint32_t)(c[3] * 255.999f) << 24) + ((uint32_t)(c[0] * 255.999f) << 16) +
           ((uint32_t)(c[1] * 255.999f) << 8) + (uint32_t)(c[2] * 255.999f);
}

static float layer_exponent(const orc_view* v, uint32_t depth)
{
    float il = 1.f / ((float)(1u << (depth + v->level)) * v->quality);
    return il * 100.f;
}

static float opacity_factor(const orc_view* v)
{
    return (v->threshold - v->field_min) / (v->field_max - v->field_min);
}

/* ======================================================================
 * Texture-unit filtering (cudaFilterModeLinear, cudaAddressModeClamp, float
 * texels), as the reference's tex3D / tex1D fetches (RenderFuncInput.hpp:42-50,
 * renderArgb.hpp:44) return it on this GPU.  Measured with one-hot 2x2x2
 * textures over a lattice of coordinates and restated here:
 *  - per axis, xb = coordinate - 0.5, texels floor(xb) and floor(xb) + 1
 *    (clamped), fraction held as an integer a = floor(frac(xb) * 256 + 1/2)
 *    in 0..256 (CUDA documents 8 fractional bits);
 *  - 1D: weights (256 - a, a) / 256;
 *  - 3D: the z split is exact (zt = 256 - c or c); within each z half the
 *    x-high weight is xh = round(a * zt / 256) (halves up) and x-low is
 *    xl = zt - xh; the y split rounds the y-high part under xh,
 *    yh = round(xh * b / 256), and the y-low part under xl,
 *    yl = round(xl * (256 - b) / 256), the other part being the rest, so the
 *    eight weights always sum to 256;
 *  - a NaN texel makes the result NaN when its per-axis factors (a or 256 - a,
 *    ...) are all nonzero, even where its rounded weight is 0; a NaN texel
 *    whose factor on some axis is 0 is ignored.
 * The weighted sum is formed in double and rounded to float once.
 * ====================================================================== */

static int32_t rn8(int32_t x, int32_t y) { return (x * y + 128) >> 8; }

static void tex_axis(float tc, uint32_t n, uint32_t* i0, uint32_t* i1, int32_t* a)
{
    double xb = (double)(tc - 0.5f);
    double q = floor(xb * 256.0 + 0.5);
    double fl = floor(q / 256.0);
    *a = (int32_t)(q - 256.0 * fl);
    long lo = (long)fl, hi = lo + 1, top = (long)n - 1;
    *i0 = (uint32_t)(lo < 0 ? 0 : (lo > top ? top : lo));
    *i1 = (uint32_t)(hi < 0 ? 0 : (hi > top ? top : hi));
}

/* returns 0 for NaN */
static int tex3d_sample(const orc_ray* r, const float tc[3], const float* brick, float* out)
{
    uint32_t i0[3], i1[3];
    int32_t a[3];
    for (int d = 0; d < 3; ++d)
        tex_axis(tc[d], r->n, &i0[d], &i1[d], &a[d]);
    int32_t w[8];
    for (int hz = 0; hz < 2; ++hz) {
        const int32_t zt = hz ? a[2] : 256 - a[2];
        const int32_t xh = rn8(a[0], zt), xl = zt - xh;
        const int32_t yhh = rn8(xh, a[1]);
        const int32_t yll = rn8(xl, 256 - a[1]);
        w[1 | 2 | (hz << 2)] = yhh;
        w[1 | (hz << 2)] = xh - yhh;
        w[(hz << 2)] = yll;
        w[2 | (hz << 2)] = xl - yll;
    }
    const uint64_t n = r->n;
    double acc = 0.0;
    for (int t = 0; t < 8; ++t) {
        const int hx = t & 1, hy = (t >> 1) & 1, hz = (t >> 2) & 1;
        const int32_t fx = hx ? a[0] : 256 - a[0], fy = hy ? a[1] : 256 - a[1], fz = hz ? a[2] : 256 - a[2];
        const uint64_t x = hx ? i1[0] : i0[0], y = hy ? i1[1] : i0[1], z = hz ? i1[2] : i0[2];
        const float val = brick[(z * n + y) * n + x];
        if (isnan(val)) {
            if (fx && fy && fz) return 0;
            continue;
        }
        acc += (double)w[t] * (double)val;
    }
    *out = (float)(acc / 256.0);
    return 1;
}

void orc_tex3d_weights(const float tc[3], uint32_t n, int32_t w[8], uint8_t footprint[8], uint32_t texel[8])
{
    uint32_t i0[3], i1[3];
    int32_t a[3];
    for (int d = 0; d < 3; ++d)
        tex_axis(tc[d], n, &i0[d], &i1[d], &a[d]);
    for (int hz = 0; hz < 2; ++hz) {
        const int32_t zt = hz ? a[2] : 256 - a[2];
        const int32_t xh = rn8(a[0], zt), xl = zt - xh;
        const int32_t yhh = rn8(xh, a[1]), yll = rn8(xl, 256 - a[1]);
        w[3 | (hz << 2)] = yhh;
        w[1 | (hz << 2)] = xh - yhh;
        w[hz << 2] = yll;
        w[2 | (hz << 2)] = xl - yll;
    }
    for (int t = 0; t < 8; ++t) {
        const int hx = t & 1, hy = (t >> 1) & 1, hz = (t >> 2) & 1;
        footprint[t] = (uint8_t)((hx ? a[0] : 256 - a[0]) && (hy ? a[1] : 256 - a[1]) && (hz ? a[2] : 256 - a[2]));
        const uint32_t x = hx ? i1[0] : i0[0], y = hy ? i1[1] : i0[1], z = hz ? i1[2] : i0[2];
        texel[t] = (z * n + y) * n + x;
    }
}

static float tex1d_tf(const float* tf, uint32_t tfn, float v01, int ch)
{
    uint32_t i0, i1;
    int32_t a;
    tex_axis(v01 * (float)tfn, tfn, &i0, &i1, &a);
    return (float)(((double)(256 - a) * tf[4 * i0 + ch] + (double)a * tf[4 * i1 + ch]) / 256.0);
}

/* One block's float RGBA along one ray (non-premultiplied, reference order). */
static void march_block_f32(const orc_view* v, const orc_ray* r, const float* brick, uint32_t depth,
                            const float* tf, float rgba[4], int tex)
{
    const float span = v->field_max - v->field_min;
    const float of = opacity_factor(v);
    const float il = layer_exponent(v, depth);
    rgba[0] = rgba[1] = rgba[2] = rgba[3] = 0.f;
    float tp[3] = {r->p0[0], r->p0[1], r->p0[2]}; /* texture filter: accumulated position */
    for (int i = 1; i < r->sample_count; ++i) {
        float tc[3];
        float val;
        if (tex) {
            for (int d = 0; d < 3; ++d) {
                tc[d] = (tp[d] - r->origin[d]) * r->factor;
                tp[d] += r->step[d];
            }
        } else {
            sample_coord(r, i - 1, tc);
        }
        if (tex) {
            if (!tex3d_sample(r, tc, brick, &val)) continue;
        } else {
            corner8 c;
            corners(r, tc, &c);
            float t[8];
            int nan = 0;
            for (int k = 0; k < 8; ++k) {
                t[k] = brick[c.off[k]];
                nan |= isnan(t[k]);
            }
            if (nan) continue;
            float x00 = t[0] + c.f[0] * (t[1] - t[0]);
            float x10 = t[2] + c.f[0] * (t[3] - t[2]);
            float x01 = t[4] + c.f[0] * (t[5] - t[4]);
            float x11 = t[6] + c.f[0] * (t[7] - t[6]);
            float y0 = x00 + c.f[1] * (x10 - x00);
            float y1 = x01 + c.f[1] * (x11 - x01);
            val = y0 + c.f[2] * (y1 - y0);
        }
        float v01 = (val - v->field_min) / span;
        float col[4];
        for (int ch = 0; ch < 4; ++ch)
            col[ch] = tex ? tex1d_tf(tf, v->tf_n, v01, ch) : tf_lookup_f32(tf, v->tf_n, v01, ch);
        col[3] = 1.f - powf(1.f - col[3] * of, il);
        blend_behind(rgba, col);
        if (rgba[3] > 0.996f) break;
    }
}

void orc_render_block_argb8(const orc_view* v, const float* brick, uint32_t depth, const uint32_t idx[3],
                            const int32_t rect[4], const float* tf, uint32_t* viewport)
{
    float c[3], h;
    orc_block_cube(v->level, idx, c, &h);
    for (int32_t yy = 0; yy < rect[3]; ++yy) {
        for (int32_t xx = 0; xx < rect[2]; ++xx) {
            uint32_t vx = (uint32_t)(rect[0] + xx), vy = (uint32_t)(rect[1] + yy);
            if (vx >= v->W || vy >= v->H) continue;
            float org[3], dir[3];
            orc_ray r;
            ray_for_pixel(v, vx, vy, org, dir);
            if (!ray_block(v, org, dir, c, h, depth, &r)) continue;
            float rgba[4], ex[4];
            march_block_f32(v, &r, brick, depth, tf, rgba, v->filter == 1);
            uint32_t* px = &viewport[(size_t)(v->H - 1 - vy) * v->W + vx];
            argb_to_rgba(*px, ex);
            blend_above(ex, rgba);
            *px = rgba_to_argb(ex);
        }
    }
}

/* ======================================================================
 * Plain per-block render in every field mode: renderKernel<mode>
 * (DenseFieldRenderer_cu.cu:62-215) with renderIsosurface.hpp:34-66,
 * renderIsosurfaces.hpp:34-106, renderMaxIntensityProjection.hpp:30-50,
 * renderArgb.hpp:30-55, renderArgbLight.hpp:30-66, renderDomainVoxels.hpp:30-55,
 * renderValueOnIsosurface.hpp:30-68, renderValueOnIsosurfaces.hpp, lighting
 * cuda_lighting.hpp:26-95, findInterval cuda_findInterval.hpp:26-43.
 * Sample positions entry + k*step (one fma), as the GPU kernel forms them;
 * filtered values in float with single-rounding fmas as the kernel does.
 * ====================================================================== */

static float field_at(const orc_view* v, const float* brick, uint32_t n, const float tc[3])
{
    if (v->filter == 1) {
        orc_ray rr;
        float val;
        rr.n = n;
        if (!tex3d_sample(&rr, tc, brick, &val)) return NAN;
        return val;
    }
    uint32_t i0[3], i1[3];
    float f[3];
    for (int d = 0; d < 3; ++d) filter_axis(tc[d], n, &i0[d], &i1[d], &f[d]);
    float t[8];
    for (int k = 0; k < 8; ++k) {
        const uint64_t x = (k & 1) ? i1[0] : i0[0], y = (k & 2) ? i1[1] : i0[1], z = (k & 4) ? i1[2] : i0[2];
        t[k] = brick[(z * n + y) * n + x];
        if (isnan(t[k])) return NAN;
    }
    const float x00 = fmaf(f[0], t[1] - t[0], t[0]), x10 = fmaf(f[0], t[3] - t[2], t[2]);
    const float x01 = fmaf(f[0], t[5] - t[4], t[4]), x11 = fmaf(f[0], t[7] - t[6], t[6]);
    const float y0 = fmaf(f[1], x10 - x00, x00), y1 = fmaf(f[1], x11 - x01, x01);
    return fmaf(f[2], y1 - y0, y0);
}

static void tf_rgba(const orc_view* v, const float* tf, float v01, float out[4])
{
    if (v->filter == 1) {
        for (int ch = 0; ch < 4; ++ch) out[ch] = tex1d_tf(tf, v->tf_n, v01, ch);
        return;
    }
    uint32_t i0, i1;
    float f;
    filter_axis(v01 * (float)v->tf_n, v->tf_n, &i0, &i1, &f);
    for (int ch = 0; ch < 4; ++ch) out[ch] = fmaf(f, tf[4 * i1 + ch] - tf[4 * i0 + ch], tf[4 * i0 + ch]);
}

static float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void normalize3(float a[3])
{
    const float il = 1.f / sqrtf(dot3(a, a));
    for (int d = 0; d < 3; ++d) a[d] *= il;
}
static float clamp01f(float x) { return fmaxf(0.f, fminf(1.f, x)); }

static void frag_color(const orc_view* v, const orc_presentation* pr, const float* brick, uint32_t n,
                       const float diffuse[4], const float surf[3], const float tc[3], float out[4])
{
    const float dl = 0.1f;
    float a[3], b[3], N[3], V[3], c[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < 3; ++d) {
        float tm[3] = {tc[0], tc[1], tc[2]}, tp[3] = {tc[0], tc[1], tc[2]};
        tm[d] = tc[d] - dl;
        tp[d] = tc[d] + dl;
        a[d] = field_at(v, brick, n, tm);
        b[d] = field_at(v, brick, n, tp);
    }
    for (int d = 0; d < 3; ++d) N[d] = a[d] - b[d];
    normalize3(N);
    for (int d = 0; d < 3; ++d) V[d] = v->cam.eye[d] - surf[d];
    normalize3(V);
    for (uint32_t i = 0; i < pr->light_count; ++i) {
        const orc_light* L0 = &pr->lights[i];
        float L[3], H[3];
        for (int d = 0; d < 3; ++d) L[d] = L0->pos[d] - surf[d];
        normalize3(L);
        if (dot3(L, N) < 0.f)
            for (int d = 0; d < 3; ++d) N[d] = -N[d];
        const float diff = (float)fmax((double)dot3(L, N), 0.0);
        for (int d = 0; d < 3; ++d) H[d] = L[d] + V[d];
        normalize3(H);
        const float spec = diff > 0.f ? (float)pow(fmax((double)dot3(H, N), 0.0), 100.0) : 0.f;
        for (int d = 0; d < 3; ++d)
            c[d] += L0->ambient[d] + diffuse[d] * L0->diffuse[d] * diff + 0.5f * L0->specular[d] * spec;
    }
    for (int d = 0; d < 3; ++d) out[d] = clamp01f(c[d]);
    out[3] = diffuse[3];
}

static int find_interval(float val, const float* levels, uint32_t count)
{
    if (val < levels[0]) return 0;
    if (val >= levels[count - 1]) return (int)count;
    int i1 = 0, i2 = (int)count;
    while (i2 - i1 > 1) {
        const int i = (i1 + i2) >> 1;
        if (val < levels[i]) i2 = i;
        else i1 = i;
    }
    return i2;
}

/* What one block contributes to one pixel in a field mode: *kind 0 nothing, 1 the colour gathered front to
 * back in the block (acc, non-premultiplied), 2 the relative maximum (*t, max intensity), 3 clear. */
static void mode_block(const orc_view* v, const orc_presentation* pr, const orc_ray* r, const float* brick,
                       const float* brick2, uint32_t depth, const float* tf, int* kind, float acc[4], float* t_out)
{
    const uint32_t n = r->n;
    const float span = v->field_max - v->field_min;
    const uint32_t mode = pr->mode;
    float pos[3], tc[3];
    /* texture filter: positions accumulated step by step (increase(pos, step));
       exact filter: entry + k * step (one fma) */
    float seq[3] = {r->p0[0], r->p0[1], r->p0[2]};
    int seq_k = 0;
#define ORC_POS(k)                                                                                  \
    do {                                                                                            \
        if (v->filter == 1) {                                                                       \
            for (; seq_k < (k); ++seq_k)                                                            \
                for (int d_ = 0; d_ < 3; ++d_) seq[d_] += r->step[d_];                              \
        }                                                                                           \
        for (int d_ = 0; d_ < 3; ++d_) {                                                            \
            pos[d_] = v->filter == 1 ? seq[d_] : fmaf(r->step[d_], (float)(k), r->p0[d_]);          \
            tc[d_] = (pos[d_] - r->origin[d_]) * r->factor;                                         \
        }                                                                                           \
    } while (0)
    if (mode == 2) { /* max intensity */
        float maxv = v->field_min - span;
        for (int i = 1; i < r->sample_count; ++i) {
            ORC_POS(i - 1);
            const float val = field_at(v, brick, n, tc);
            if (val >= v->threshold && maxv < val) maxv = val;
        }
        *kind = 0;
        if (maxv < v->field_min) return;
        *t_out = (maxv - v->field_min) / span;
        *kind = 2;
        return;
    }
    acc[0] = acc[1] = acc[2] = acc[3] = 0.f;
    *kind = 1;
    if (mode == 3 || mode == 4 || mode == 5) {
        const float of = opacity_factor(v), il = layer_exponent(v, depth);
        float dom[4] = {0, 0, 0, 0};
        if (mode == 5) {
            tf_rgba(v, tf, 0.5f, dom);
            dom[3] = 1.f - powf(1.f - dom[3] * of, il);
        }
        for (int i = 1; i < r->sample_count; ++i) {
            ORC_POS(i - 1);
            const float val = field_at(v, brick, n, tc);
            if (isnan(val)) continue;
            float col[4];
            if (mode == 5) {
                memcpy(col, dom, sizeof(col));
            } else {
                tf_rgba(v, tf, (val - v->field_min) / span, col);
                col[3] = 1.f - powf(1.f - col[3] * of, il);
                if (mode == 4) {
                    if (!(col[3] >= 0.00001f)) continue;
                    float lit[4];
                    frag_color(v, pr, brick, n, col, pos, tc, lit);
                    memcpy(col, lit, sizeof(col));
                }
            }
            blend_behind(acc, col);
            if (acc[3] > 0.996f) break;
        }
        return;
    }
    const int multi = mode == 1 || mode == 7, secondary = mode == 6 || mode == 7;
    const uint32_t nl = pr->level_count;
    if (multi && nl < 1) {
        *kind = 3;
        return;
    }
    ORC_POS(0);
    float v1 = field_at(v, brick, n, tc);
    int iint = multi ? (isnan(v1) ? -1 : find_interval(v1, pr->levels, nl)) : 0;
    for (int i = 1; i < r->sample_count; ++i) {
        ORC_POS(i);
        const float v2 = field_at(v, brick, n, tc);
        int nlev = 0, il = 0, dl = 0;
        float levs[1] = {v->threshold};
        if (!multi) {
            if (!(!isnan(v1) && !isnan(v2) && (v1 - v->threshold) * (v2 - v->threshold) < 0.f)) {
                v1 = v2;
                continue;
            }
            nlev = 1;
        } else {
            if (isnan(v2)) {
                iint = -1;
                v1 = NAN;
                continue;
            }
            if (isnan(v1)) {
                v1 = v2;
                iint = find_interval(v1, pr->levels, nl);
                continue;
            }
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
        }
        for (;;) {
            float level;
            if (!multi) {
                if (nlev-- <= 0) break;
                level = levs[0];
            } else {
                if (!(il >= 0 && il < (int)nl)) break;
                level = pr->levels[il];
                if (!((v1 - level) * (v2 - level) < 0.f)) break;
            }
            const float t = (level - v1) / (v2 - v1);
            float xpos[3], xtc[3], dif[4], col[4];
            for (int d = 0; d < 3; ++d) {
                xpos[d] = pos[d] + r->step[d] * t;
                xtc[d] = (xpos[d] - r->origin[d]) * r->factor;
            }
            if (secondary) {
                const float vs = field_at(v, brick2, n, xtc);
                tf_rgba(v, tf, (vs - pr->secondary_min) / (pr->secondary_max - pr->secondary_min), dif);
            } else {
                tf_rgba(v, tf, (level - v->field_min) / span, dif);
            }
            dif[3] *= pr->isosurface_opacity;
            frag_color(v, pr, brick, n, dif, xpos, xtc, col);
            blend_behind(acc, col);
            if (multi) {
                iint += dl;
                il += dl;
            } else if (acc[3] > 0.996f) {
                goto done;
            }
        }
        if (multi && acc[3] > 0.996f) break;
        v1 = v2;
    }
done:
    return;
#undef ORC_POS
}

static void mode_pixel(const orc_view* v, const orc_presentation* pr, const orc_ray* r, const float* brick,
                       const float* brick2, uint32_t depth, const float* tf, uint32_t* px)
{
    int kind = 0;
    float acc[4], t = 0.f, ex[4];
    mode_block(v, pr, r, brick, brick2, depth, tf, &kind, acc, &t);
    if (kind == 2) {
        float prev;
        memcpy(&prev, px, 4);
        if (!isnan(prev) && prev > t) return;
        memcpy(px, &t, 4);
    } else if (kind == 1) {
        argb_to_rgba(*px, ex);
        blend_above(ex, acc);
        *px = rgba_to_argb(ex);
    } else if (kind == 3) {
        *px = 0u;
    }
}


void orc_render_block_mode(const orc_view* v, const orc_presentation* pr, const float* brick, const float* brick2,
                           uint32_t depth, const uint32_t idx[3], const int32_t rect[4], const float* tf,
                           uint32_t* viewport)
{
    float c[3], h;
    orc_block_cube(v->level, idx, c, &h);
    for (int32_t yy = 0; yy < rect[3]; ++yy) {
        for (int32_t xx = 0; xx < rect[2]; ++xx) {
            uint32_t vx = (uint32_t)(rect[0] + xx), vy = (uint32_t)(rect[1] + yy);
            if (vx >= v->W || vy >= v->H) continue;
            float org[3], dir[3];
            orc_ray r;
            ray_for_pixel(v, vx, vy, org, dir);
            if (!ray_block(v, org, dir, c, h, depth, &r)) continue;
            mode_pixel(v, pr, &r, brick, brick2, depth, tf, &viewport[(size_t)(v->H - 1 - vy) * v->W + vx]);
        }
    }
}

/* ======================================================================
 * Frame render: per ray, every block it enters, in ray order.
 * ====================================================================== */

typedef struct hit {
    float tau;
    uint32_t block;
    orc_ray r;
} hit;

static int hit_cmp_far_first(const void* a, const void* b)
{
    const hit* x = (const hit*)a;
    const hit* y = (const hit*)b;
    if (x->tau != y->tau) return x->tau < y->tau ? 1 : -1;
    return x->block < y->block ? 1 : (x->block > y->block ? -1 : 0);
}

static int in_rect(const int32_t* rect, uint32_t vx, uint32_t vy)
{
    return (int64_t)vx >= rect[0] && (int64_t)vx < (int64_t)rect[0] + rect[2] && (int64_t)vy >= rect[1] &&
           (int64_t)vy < (int64_t)rect[1] + rect[3];
}

static int collect_hits(const orc_view* v, uint32_t nb, const uint32_t* blocks, const int32_t* rects,
                        uint32_t vx, uint32_t vy, hit* hits)
{
    float org[3], dir[3];
    ray_for_pixel(v, vx, vy, org, dir);
    int nh = 0;
    for (uint32_t b = 0; b < nb; ++b) {
        if (rects && !in_rect(rects + 4 * b, vx, vy)) continue;
        float c[3], h;
        orc_block_cube(v->level, blocks + 4 * b, c, &h);
        orc_ray r;
        if (!ray_block(v, org, dir, c, h, blocks[4 * b + 3], &r)) continue;
        hits[nh].tau = r.tau_enter_raw;
        hits[nh].block = b;
        hits[nh].r = r;
        ++nh;
    }
    qsort(hits, (size_t)nh, sizeof(hit), hit_cmp_far_first);
    return nh;
}

/* FP64 sample: returns 0 when the sample is skipped (a NaN corner). */
typedef struct sample64 {
    double val;
    double w[8];
    uint64_t off[8];
    double col[4];  /* transfer-function RGBA before opacity correction */
    double dcol[4]; /* d col / d v01 */
    uint32_t ti0, ti1;
    double tf_f;
    double v01;
} sample64;

static int sample_f64(const orc_view* v, const orc_ray* r, int k, const float* brick, const float* tf,
                      sample64* s)
{
    float tc[3];
    sample_coord(r, k, tc);
    double val = 0;
    if (v->filter == 1) {
        /* texture-unit weights (integers / 256, see tex3d_sample), summed exactly in double */
        uint32_t i0[3], i1[3];
        int32_t a3[3];
        for (int d = 0; d < 3; ++d)
            tex_axis(tc[d], r->n, &i0[d], &i1[d], &a3[d]);
        int32_t w[8];
        for (int hz = 0; hz < 2; ++hz) {
            const int32_t zt = hz ? a3[2] : 256 - a3[2];
            const int32_t xh = rn8(a3[0], zt), xl = zt - xh;
            const int32_t yhh = rn8(xh, a3[1]), yll = rn8(xl, 256 - a3[1]);
            w[3 | (hz << 2)] = yhh;
            w[1 | (hz << 2)] = xh - yhh;
            w[(hz << 2)] = yll;
            w[2 | (hz << 2)] = xl - yll;
        }
        const uint64_t n = r->n;
        for (int i = 0; i < 8; ++i) {
            const int hx = i & 1, hy = (i >> 1) & 1, hz = (i >> 2) & 1;
            const uint64_t x = hx ? i1[0] : i0[0], y = hy ? i1[1] : i0[1], z = hz ? i1[2] : i0[2];
            s->off[i] = (z * n + y) * n + x;
            const float xv = brick[s->off[i]];
            const int32_t fx = hx ? a3[0] : 256 - a3[0], fy = hy ? a3[1] : 256 - a3[1], fz = hz ? a3[2] : 256 - a3[2];
            if (isnan(xv)) {
                if (fx && fy && fz) return 0;
                s->w[i] = 0;
                continue;
            }
            s->w[i] = w[i] / 256.0;
            val += s->w[i] * (double)xv;
        }
    } else {
        corner8 c;
        corners(r, tc, &c);
        double t[8];
        for (int i = 0; i < 8; ++i) {
            float x = brick[c.off[i]];
            if (isnan(x)) return 0;
            t[i] = x;
            s->off[i] = c.off[i];
        }
        double fx = c.f[0], fy = c.f[1], fz = c.f[2];
        for (int i = 0; i < 8; ++i)
            s->w[i] = ((i & 1) ? fx : 1 - fx) * ((i & 2) ? fy : 1 - fy) * ((i & 4) ? fz : 1 - fz);
        for (int i = 0; i < 8; ++i) val += s->w[i] * t[i];
    }
    s->val = val;
    double span = (double)v->field_max - (double)v->field_min;
    double v01 = (val - (double)v->field_min) / span;
    s->v01 = v01;
    /* normalized-coordinate linear filtering with clamp addressing */
    double u = v01 * (double)v->tf_n - 0.5;
    if (v->filter == 1) {
        /* 8-bit weight, coordinate formed in float as the fetch receives it */
        uint32_t j0, j1;
        int32_t aq;
        tex_axis((float)v01 * (float)v->tf_n, v->tf_n, &j0, &j1, &aq);
        s->ti0 = j0;
        s->ti1 = j1;
        s->tf_f = aq / 256.0;
        for (int ch = 0; ch < 4; ++ch) {
            double ta = tf[4 * j0 + ch], tb = tf[4 * j1 + ch];
            s->col[ch] = ta + s->tf_f * (tb - ta);
            s->dcol[ch] = 0.0;
        }
        return 1;
    }
    double fl = floor(u);
    double f = u - fl;
    long a = (long)fl, b = a + 1, hi = (long)v->tf_n - 1;
    int clamped_lo = a < 0, clamped_hi = b > hi;
    uint32_t i0 = (uint32_t)(a < 0 ? 0 : (a > hi ? hi : a));
    uint32_t i1 = (uint32_t)(b < 0 ? 0 : (b > hi ? hi : b));
    s->ti0 = i0;
    s->ti1 = i1;
    s->tf_f = f;
    for (int ch = 0; ch < 4; ++ch) {
        double ta = tf[4 * i0 + ch], tb = tf[4 * i1 + ch];
        s->col[ch] = ta + f * (tb - ta);
        s->dcol[ch] = (clamped_lo || clamped_hi) ? 0.0 : (tb - ta) * (double)v->tf_n;
    }
    return 1;
}

typedef struct acc64 {
    double C[3]; /* premultiplied colour */
    double A;
} acc64;

/* March one block in FP64; composites into the block-local accumulator.
 * Sets *near when the early-termination test came within 1e-5 of its threshold. */
static void march_block_f64(const orc_view* v, const orc_ray* r, const float* brick, uint32_t depth,
                            const float* tf, acc64* blk, int* near)
{
    const double of = ((double)v->threshold - v->field_min) / ((double)v->field_max - v->field_min);
    const double il = (double)layer_exponent(v, depth);
    blk->C[0] = blk->C[1] = blk->C[2] = blk->A = 0;
    for (int i = 1; i < r->sample_count; ++i) {
        sample64 s;
        if (!sample_f64(v, r, i - 1, brick, tf, &s)) continue;
        double a = 1.0 - pow(1.0 - s.col[3] * of, il);
        double wgt = (1.0 - blk->A) * a;
        for (int ch = 0; ch < 3; ++ch) blk->C[ch] += wgt * s.col[ch];
        blk->A += wgt;
        if (fabs(blk->A - 0.996) < 1e-5) *near = 1;
        if (blk->A > 0.996) break;
    }
}

/* The FP64 frame, per pixel non-premultiplied RGBA; rgba_out (float) and/or rgba64_out (double) receive it. */
static void render_frame_f64_any(const orc_view* v, uint32_t nb, const uint32_t* blocks, const uint64_t* dense_off,
                                 const float* dense, const int32_t* rects, const float* tf, uint32_t np,
                                 const uint32_t* pixels, float* rgba_out, double* rgba64_out, uint8_t* flags_out)
{
    hit* hits = (hit*)malloc(sizeof(hit) * (nb ? nb : 1));
    uint64_t total = pixels ? np : (uint64_t)v->W * v->H;
    for (uint64_t p = 0; p < total; ++p) {
        uint32_t vx = pixels ? pixels[2 * p] : (uint32_t)(p % v->W);
        uint32_t vy = pixels ? pixels[2 * p + 1] : (uint32_t)(v->H - 1 - p / v->W);
        int nh = collect_hits(v, nb, blocks, rects, vx, vy, hits);
        acc64 acc = {{0, 0, 0}, 0};
        int near = 0;
        /* hits are sorted far first; composite front to back */
        for (int j = nh - 1; j >= 0; --j) {
            uint32_t b = hits[j].block;
            acc64 blk;
            march_block_f64(v, &hits[j].r, dense + dense_off[b], blocks[4 * b + 3], tf, &blk, &near);
            double T = 1.0 - acc.A;
            for (int ch = 0; ch < 3; ++ch) acc.C[ch] += T * blk.C[ch];
            acc.A += T * blk.A;
        }
        double o[4];
        for (int ch = 0; ch < 3; ++ch) o[ch] = acc.A > 0 ? acc.C[ch] / acc.A : 0.0;
        o[3] = acc.A;
        for (int ch = 0; ch < 4; ++ch) {
            if (rgba_out) rgba_out[4 * p + ch] = (float)o[ch];
            if (rgba64_out) rgba64_out[4 * p + ch] = o[ch];
        }
        if (flags_out) flags_out[p] = (uint8_t)near;
    }
    free(hits);
}

void orc_render_frame_f64(const orc_view* v, uint32_t nb, const uint32_t* blocks, const uint64_t* dense_off,
                          const float* dense, const int32_t* rects, const float* tf, uint32_t np,
                          const uint32_t* pixels, float* rgba_out, uint8_t* flags_out)
{
    render_frame_f64_any(v, nb, blocks, dense_off, dense, rects, tf, np, pixels, rgba_out, NULL, flags_out);
}

void orc_render_frame_f64d(const orc_view* v, uint32_t nb, const uint32_t* blocks, const uint64_t* dense_off,
                           const float* dense, const int32_t* rects, const float* tf, uint32_t np,
                           const uint32_t* pixels, double* rgba_out, uint8_t* flags_out)
{
    render_frame_f64_any(v, nb, blocks, dense_off, dense, rects, tf, np, pixels, NULL, rgba_out, flags_out);
}

void orc_render_frame_argb8(const orc_view* v, uint32_t nb, const uint32_t* blocks, const uint64_t* dense_off,
                            const float* dense, const int32_t* rects, const float* tf, uint32_t* viewport)
{
    hit* hits = (hit*)malloc(sizeof(hit) * (nb ? nb : 1));
    for (uint32_t vy = 0; vy < v->H; ++vy) {
        for (uint32_t vx = 0; vx < v->W; ++vx) {
            int nh = collect_hits(v, nb, blocks, rects, vx, vy, hits);
            uint32_t* px = &viewport[(size_t)(v->H - 1 - vy) * v->W + vx];
            for (int j = 0; j < nh; ++j) { /* far first */
                uint32_t b = hits[j].block;
                float rgba[4], ex[4];
                march_block_f32(v, &hits[j].r, dense + dense_off[b], blocks[4 * b + 3], tf, rgba, v->filter == 1);
                argb_to_rgba(*px, ex);
                blend_above(ex, rgba);
                *px = rgba_to_argb(ex);
            }
        }
    }
    free(hits);
}

void orc_render_frame_mode(const orc_view* v, const orc_presentation* pr, uint32_t nb, const uint32_t* blocks,
                           const uint64_t* dense_off, const float* dense, const float* dense2, const int32_t* rects,
                           const float* tf, float alpha_stop, float* rgba)
{
    hit* hits = (hit*)malloc(sizeof(hit) * (nb ? nb : 1));
    const int mip = pr->mode == 2;
    for (uint32_t vy = 0; vy < v->H; ++vy) {
        for (uint32_t vx = 0; vx < v->W; ++vx) {
            int nh = collect_hits(v, nb, blocks, rects, vx, vy, hits);
            float F[4] = {0.f, 0.f, 0.f, 0.f}, best = 0.f;
            int have = 0;
            for (int j = nh - 1; j >= 0; --j) { /* near first */
                const uint32_t b = hits[j].block;
                int kind = 0;
                float acc[4], t = 0.f;
                mode_block(v, pr, &hits[j].r, dense + dense_off[b], dense2 ? dense2 + dense_off[b] : NULL,
                           blocks[4 * b + 3], tf, &kind, acc, &t);
                if (kind == 2) {
                    if (!have || t > best) best = t;
                    have = 1;
                } else if (kind == 1) {
                    const float T = 1.f - F[3];
                    for (int c = 0; c < 3; ++c) F[c] = fmaf(T, acc[c] * acc[3], F[c]);
                    F[3] = fmaf(T, acc[3], F[3]);
                } else if (kind == 3) {
                    break;
                }
                if (!mip && F[3] > alpha_stop) break;
            }
            float* o = rgba + 4 * ((size_t)(v->H - 1 - vy) * v->W + vx);
            if (mip) {
                o[0] = o[1] = o[2] = have ? best : 0.f;
                o[3] = have ? 1.f : 0.f;
            } else {
                o[3] = F[3];
                for (int c = 0; c < 3; ++c) o[c] = F[3] > 0.f ? F[c] / F[3] : 0.f;
            }
        }
    }
    free(hits);
}

/* ======================================================================
 * Image-part blend — src/s3vs_lib/BlendImagePart.hpp:61-145 (integer src-over-dst).
 * ====================================================================== */

void orc_blend_image_part(uint32_t* dst, int32_t dw, int32_t dh, const uint32_t* src, int32_t sw, int32_t sh,
                          int32_t ox, int32_t oy, int32_t just_copy, int32_t offx, int32_t offy)
{
    (void)dh;
    int32_t dx = ox - offx, dy = oy - offy;
    for (int32_t sy = 0; sy < sh; ++sy) {
        const uint32_t* srow = src + (size_t)sy * sw;
        uint32_t* drow = dst + (size_t)dw * (dy + sy) + dx;
        for (int32_t i = 0; i < sw; ++i) {
            uint32_t s = srow[i];
            if (just_copy) { drow[i] = s; continue; }
            uint32_t as = (s >> 24) & 0xffu;
            if (as == 0) continue;
            if (as == 255u) { drow[i] = s; continue; }
            uint32_t d = drow[i];
            uint32_t ad = (d >> 24) & 0xffu;
            if (ad == 0) { drow[i] = s; continue; }
            uint32_t a = as + ad * (255u - as) / 255u;
            uint32_t out = (a & 0xffu) << 24;
            for (int b = 0; b < 3; ++b) {
                uint32_t cs = (s >> (8 * b)) & 0xffu, cd = (d >> (8 * b)) & 0xffu;
                uint32_t cc = (cs * as + cd * (a - as)) / a;
                out |= (cc & 0xffu) << (8 * b);
            }
            drow[i] = out;
        }
    }
}

/* ======================================================================
 * Transfer-function table — include/s3vs/ColorTransferFunction.hpp:27-69.
 * Control points arrive sorted by x (the reference keeps them in a std::map).
 * ====================================================================== */

void orc_make_ctf(const double* xs, const double* rgba, uint32_t npoints, uint32_t color_count, float* out)
{
    if (npoints == 0) {
        for (uint32_t i = 0; i < 4 * color_count; ++i) out[i] = 1.f;
        return;
    }
    if (npoints == 1) {
        for (uint32_t i = 0; i < color_count; ++i)
            for (int ch = 0; ch < 4; ++ch) out[4 * i + ch] = (float)rgba[ch];
        return;
    }
    for (uint32_t i = 0; i < 4 * color_count; ++i) out[i] = 0.f;
    /* real_type is float in the reference build */
    float xmin = (float)xs[0], xmax = (float)xs[npoints - 1];
    float c1[4];
    for (int ch = 0; ch < 4; ++ch) { c1[ch] = (float)rgba[ch]; out[ch] = c1[ch]; }
    uint32_t i1 = 0;
    for (uint32_t ip = 1; ip < npoints; ++ip) {
        float x2 = (float)xs[ip];
        float c2[4];
        for (int ch = 0; ch < 4; ++ch) c2[ch] = (float)rgba[4 * ip + ch];
        uint32_t i2 = ip + 1 == npoints ? color_count - 1u
                                        : (uint32_t)((x2 - xmin) / (xmax - xmin) * (float)color_count);
        if (i2 > i1) {
            for (uint32_t i = i1 + 1; i <= i2; ++i) {
                float t = (float)(i - i1) / (float)(i2 - i1);
                for (int ch = 0; ch < 4; ++ch) out[4 * i + ch] = c1[ch] * (1 - t) + c2[ch] * t;
            }
        }
        for (int ch = 0; ch < 4; ++ch) c1[ch] = c2[ch];
        i1 = i2;
    }
}

/* ======================================================================
 * Adjoint in FP64 (no reference counterpart): d L / d tf, d L / d dense for
 * L = 1/2 sum (I - target)^2 with I = (C/A, A) over the frame render above.
 * The sample set (positions, NaN skips, early terminations) is held fixed;
 * the compositing is differentiated as one front-to-back sequence of the
 * kept samples, which is what block-local compositing followed by the
 * over-operator between blocks amounts to.
 * ====================================================================== */

typedef struct kept {
    uint32_t block;
    sample64 s;
    double a;     /* corrected alpha */
    double dadc;  /* d a / d col[3] */
} kept;

double orc_render_frame_grad_f64(const orc_view* v, uint32_t nb, const uint32_t* blocks,
                                 const uint64_t* dense_off, const float* dense, const int32_t* rects,
                                 const float* tf, uint32_t np, const uint32_t* pixels, const float* target,
                                 double* dtf, double* ddense)
{
    hit* hits = (hit*)malloc(sizeof(hit) * (nb ? nb : 1));
    size_t cap = 1024;
    kept* ks = (kept*)malloc(sizeof(kept) * cap);
    double loss = 0;
    const double of = ((double)v->threshold - v->field_min) / ((double)v->field_max - v->field_min);
    const double span = (double)v->field_max - (double)v->field_min;
    uint64_t total = pixels ? np : (uint64_t)v->W * v->H;
    for (uint64_t p = 0; p < total; ++p) {
        uint32_t vx = pixels ? pixels[2 * p] : (uint32_t)(p % v->W);
        uint32_t vy = pixels ? pixels[2 * p + 1] : (uint32_t)(v->H - 1 - p / v->W);
        int nh = collect_hits(v, nb, blocks, rects, vx, vy, hits);
        /* forward: collect kept samples with their global transmittance */
        size_t nk = 0;
        acc64 acc = {{0, 0, 0}, 0};
        for (int j = nh - 1; j >= 0; --j) {
            uint32_t b = hits[j].block;
            const orc_ray* r = &hits[j].r;
            const float* brick = dense + dense_off[b];
            const double il = (double)layer_exponent(v, blocks[4 * b + 3]);
            double Ab = 0;
            double T0 = 1.0 - acc.A;
            for (int i = 1; i < r->sample_count; ++i) {
                sample64 s;
                if (!sample_f64(v, r, i - 1, brick, tf, &s)) continue;
                double base = 1.0 - s.col[3] * of;
                double a = 1.0 - pow(base, il);
                double dadc = il * pow(base, il - 1.0) * of;
                if (nk == cap) { cap *= 2; ks = (kept*)realloc(ks, sizeof(kept) * cap); }
                ks[nk].block = b;
                ks[nk].s = s;
                ks[nk].a = a;
                ks[nk].dadc = dadc;
                ++nk;
                double wgt = T0 * (1.0 - Ab) * a;
                for (int ch = 0; ch < 3; ++ch) acc.C[ch] += wgt * s.col[ch];
                Ab += (1.0 - Ab) * a;
                if (Ab > 0.996) break;
            }
            acc.A = 1.0 - T0 * (1.0 - Ab);
        }
        const float* tg = target + 4 * p;
        double I[4], gI[4];
        for (int ch = 0; ch < 3; ++ch) I[ch] = acc.A > 0 ? acc.C[ch] / acc.A : 0.0;
        I[3] = acc.A;
        for (int ch = 0; ch < 4; ++ch) {
            double d = I[ch] - (double)tg[ch];
            loss += 0.5 * d * d;
            gI[ch] = d;
        }
        /* I_c = C_c / A (A > 0), I_a = A */
        double gC[3], gA = gI[3];
        if (acc.A > 0) {
            for (int ch = 0; ch < 3; ++ch) {
                gC[ch] = gI[ch] / acc.A;
                gA -= gI[ch] * acc.C[ch] / (acc.A * acc.A);
            }
        } else {
            gC[0] = gC[1] = gC[2] = 0;
        }
        /* backward over the flat front-to-back sequence:
         * C = sum_k T_k a_k c_k, A = 1 - prod (1 - a_k), T_k = prod_{j<k} (1 - a_j).
         * dC/dc_k = T_k a_k; dC/da_k = T_k c_k - (C - C_<=k) / (1 - a_k); dA/da_k = T_k (1-A_after)... */
        double T = 1.0, Cpre[3] = {0, 0, 0};
        for (size_t k = 0; k < nk; ++k) {
            kept* q = &ks[k];
            double a = q->a;
            double Cpost[3];
            for (int ch = 0; ch < 3; ++ch) Cpost[ch] = Cpre[ch] + T * a * q->s.col[ch];
            /* colour part */
            double g_col[4] = {0, 0, 0, 0};
            for (int ch = 0; ch < 3; ++ch) g_col[ch] = gC[ch] * T * a;
            /* alpha part: contributions behind sample k scale with (1 - a_k) */
            double g_a = 0;
            for (int ch = 0; ch < 3; ++ch) {
                double behind = acc.C[ch] - Cpost[ch];
                g_a += gC[ch] * (T * q->s.col[ch] - behind / (1.0 - a));
            }
            /* A = 1 - T * (1 - a_k) * rest  =>  dA/da_k = T * rest = (1 - A) / (1 - a_k) */
            g_a += gA * (1.0 - acc.A) / (1.0 - a);
            g_col[3] = g_a * q->dadc;
            /* transfer-function table */
            double f = q->s.tf_f;
            for (int ch = 0; ch < 4; ++ch) {
                dtf[4 * q->s.ti0 + ch] += g_col[ch] * (1.0 - f);
                dtf[4 * q->s.ti1 + ch] += g_col[ch] * f;
            }
            /* dense values through v01 */
            double g_v01 = 0;
            for (int ch = 0; ch < 4; ++ch) g_v01 += g_col[ch] * q->s.dcol[ch];
            double g_val = g_v01 / span;
            const uint64_t base = dense_off[q->block];
            for (int i = 0; i < 8; ++i) ddense[base + q->s.off[i]] += g_val * q->s.w[i];
            for (int ch = 0; ch < 3; ++ch) Cpre[ch] = Cpost[ch];
            T *= 1.0 - a;
        }
    }
    free(ks);
    free(hits);
    return loss;
}

/* ---------------------------------------------------------------- per-block field read */

int orc_read_blocks_per_call(const char* path, const uint64_t* offsets, const uint64_t* counts, uint32_t nb,
                             float* out, float* ranges)
{
    uint64_t at = 0;
    for (uint32_t b = 0; b < nb; ++b) {
        FILE* f = fopen(path, "rb");
        if (!f) return -1;
        float r[2];
        int ok = fseeko(f, (off_t)offsets[b], SEEK_SET) == 0 && fread(r, sizeof(float), 2, f) == 2 &&
                 fread(out + at, sizeof(float), counts[b], f) == counts[b];
        fclose(f);
        if (!ok) return -1;
        if (ranges) {
            ranges[2 * b] = r[0];
            ranges[2 * b + 1] = r[1];
        }
        at += counts[b];
    }
    return 0;
}
