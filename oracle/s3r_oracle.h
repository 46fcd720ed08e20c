/*
 * s3r oracle — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's hot path, used as the checker by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The
 * product never links, loads or calls it.  Every function cites the reference
 * code it restates (paths relative to the reference project root).
 *
 * Pinning: the interpolation restatement is checked bit-for-bit against the
 * reference's own DenseFieldInterpolator<3> (compiled in place by
 * oracle/Makefile into oracle/_ref/) through committed golden fixtures; the
 * image-part blend and the transfer-function table likewise.  The ray caster
 * has no CPU implementation in the reference and its CUDA renderer cannot run
 * without a GPU here, so the renderer restatement is pinned only by reading
 * (src/s3dmm_cuda/DenseFieldRenderer_cu.cu:62-215, renderArgb.hpp:30-55,
 * cuda_blend.hpp:24-44, cuda_argb_transform.hpp:26-43): parity unpinned for the
 * renderer.
 *
 * Build with -ffp-contract=off: the float ray set-up below must round exactly
 * as written on every host architecture.
 */
#ifndef S3R_ORACLE_H
#define S3R_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Field value that marks "outside the domain" in sparse input
 * (include/s3dmm/BlockTreeFieldProvider.hpp:137-139). */
#define ORC_NO_FIELD_VALUE 1e30f

/* Camera, in the terms of RenderKernelEyeParam (src/s3dmm_cuda/RenderKernelParam.hpp:56-65).
 * ortho != 0 is an extension: rays start at eye + e1*x + e2*y and run along n. */
typedef struct orc_camera {
    float eye[3];
    float e1[3];
    float e2[3];
    float n[3];
    float w;
    float h;
    int32_t ortho;
    int32_t pad_;
} orc_camera;

/* Everything one frame's ray casting needs besides the bricks. */
typedef struct orc_view {
    orc_camera cam;
    uint32_t W, H;          /* viewport size, pixels */
    uint32_t level;         /* block level: cube half size 5/2^level */
    float field_min, field_max;
    float threshold;        /* absolute threshold; opacity factor = (threshold-min)/(max-min) */
    float quality;
    uint32_t tf_n;          /* transfer-function entries (RGBA float each) */
    uint32_t filter;        /* 0: exact trilinear / linear filtering; 1: the GPU texture unit's
                               linear filtering of the reference's textures (s3r_oracle.c) */
} orc_view;

/* ---- dense interpolation (include/s3dmm/DenseFieldInterpolator.hpp:198-419) ---- */
int orc_interp_dense_f32(const uint16_t* n2i_xyz, const float* sparse, uint32_t n, uint32_t depth,
                         float* dense);
int orc_interp_dense_f64(const uint16_t* n2i_xyz, const float* sparse, uint32_t n, uint32_t depth,
                         double* dense);

/* ---- block geometry (DenseFieldRenderer_cu.cu:337-409) ---- */
void orc_block_cube(uint32_t level, const uint32_t idx[3], float center[3], float* half_size);
/* View rectangle {x, y, W, H} of a block; needs the world->eye rotation rows r[9] and translation t[3]. */
void orc_block_view_rect(const orc_view* v, const float r[9], const float t[3], const uint32_t idx[3],
                         int32_t rect[4]);

/* ---- plain per-block render, reference semantics (FP32, ARGB8 read-modify-write) ----
 * renderKernel<FieldMode::Argb> + renderArgb (DenseFieldRenderer_cu.cu:62-215, renderArgb.hpp:30-55).
 * brick: (2^depth+1)^3 floats, x fastest; tf: tf_n RGBA floats; viewport: W*H ARGB32, top row first. */
void orc_render_block_argb8(const orc_view* v, const float* brick, uint32_t depth, const uint32_t idx[3],
                            const int32_t rect[4], const float* tf, uint32_t* viewport);

/* Texture-unit weights (units of 1/256) of the 8 texels around texel coordinate tc in an
 * n^3 clamped texture, whether each texel is in the NaN footprint, and its linear index. */
void orc_tex3d_weights(const float tc[3], uint32_t n, int32_t w[8], uint8_t footprint[8], uint32_t texel[8]);

/* ---- plain per-block render in every field mode (s3vs::FieldMode) ----
 * renderKernel<mode> with render*.hpp and cuda_lighting.hpp (see s3r_oracle.c);
 * same conventions as orc_render_block_argb8, sampling per v->filter.  Modes are
 * numbered as s3vs::FieldMode; MAX_INTENSITY (2) stores float bits. */
typedef struct orc_light {
    float pos[3], ambient[3], diffuse[3], specular[3];
} orc_light;
typedef struct orc_presentation {
    uint32_t mode;
    float isosurface_opacity;
    uint32_t level_count;
    float levels[50];
    uint32_t light_count;
    orc_light lights[10];
    float secondary_min, secondary_max;
} orc_presentation;
void orc_render_block_mode(const orc_view* v, const orc_presentation* pr, const float* brick, const float* brick2,
                           uint32_t depth, const uint32_t idx[3], const int32_t rect[4], const float* tf,
                           uint32_t* viewport);

/* ---- frame render in FP64, float RGBA out (batched-path semantics) ----
 * For each listed pixel: every block the ray enters, in ray order, is marched exactly as the
 * per-block kernel marches it (same float sample positions), with FP64 trilinear filtering,
 * transfer-function lookup, opacity correction and compositing; no ARGB8 quantization.
 * blocks: nb entries of {ix, iy, iz, depth}; dense_off: vertex offset of each block's brick;
 * rects: nb view rectangles (NULL: no clipping); pixels: np (vx, vy) pairs (NULL: all W*H in viewport order, pixel (vx, vy) at (H-1-vy)*W+vx).
 * rgba_out: 4 floats per pixel (non-premultiplied colour, alpha);
 * flags_out (optional): bit 0 set where a block-local early-termination test landed within
 * 1e-5 of its threshold (a decision float and double arithmetic may take differently). */
void orc_render_frame_f64(const orc_view* v, uint32_t nb, const uint32_t* blocks, const uint64_t* dense_off,
                          const float* dense, const int32_t* rects, const float* tf, uint32_t np,
                          const uint32_t* pixels, float* rgba_out, uint8_t* flags_out);
/* orc_render_frame_f64 with the colours kept in double (for finite differences of image losses). */
void orc_render_frame_f64d(const orc_view* v, uint32_t nb, const uint32_t* blocks, const uint64_t* dense_off,
                           const float* dense, const int32_t* rects, const float* tf, uint32_t np,
                           const uint32_t* pixels, double* rgba_out, uint8_t* flags_out);

/* Same march in FP32 with the reference's non-premultiplied per-block compositing followed by
 * ARGB8 read-modify-write per block in back-to-front order: the plain worker path for a whole
 * frame (VsWorker_cu.cpp:225-313 with a visibility order).  viewport must be cleared by the caller. */
void orc_render_frame_argb8(const orc_view* v, uint32_t nb, const uint32_t* blocks, const uint64_t* dense_off,
                            const float* dense, const int32_t* rects, const float* tf, uint32_t* viewport);

/* ---- batched field modes: per pixel the blocks front to back, each marched as orc_render_block_mode marches
 * it, their colours composited in FP32 (premultiplied, stop once alpha exceeds alpha_stop), max intensity the
 * maximum over the blocks, a cleared pixel (multi-level mode without levels) ending the walk.  rgba: W*H*4
 * floats, non-premultiplied (max intensity: t, t, t, 1, zero where no block gave a maximum). ---- */
void orc_render_frame_mode(const orc_view* v, const orc_presentation* pr, uint32_t nb, const uint32_t* blocks,
                           const uint64_t* dense_off, const float* dense, const float* dense2, const int32_t* rects,
                           const float* tf, float alpha_stop, float* rgba);

/* ---- image-part blend (src/s3vs_lib/BlendImagePart.hpp:61-145) ---- */
void orc_blend_image_part(uint32_t* dst, int32_t dw, int32_t dh, const uint32_t* src, int32_t sw, int32_t sh,
                          int32_t ox, int32_t oy, int32_t just_copy, int32_t offx, int32_t offy);

/* ---- transfer-function table (include/s3vs/ColorTransferFunction.hpp:27-69) ---- */
void orc_make_ctf(const double* xs, const double* rgba, uint32_t npoints, uint32_t color_count, float* out);

/* ---- adjoint, FP64 (no reference counterpart) ----
 * Gradient of L = 1/2 sum over listed pixels and channels of (I - target)^2 through
 * orc_render_frame_f64 (same sample set), w.r.t. the tf_n*4 table and the dense values.
 * Returns L.  dtf: tf_n*4 doubles; ddense: total vertex count doubles (both accumulated into). */
double orc_render_frame_grad_f64(const orc_view* v, uint32_t nb, const uint32_t* blocks,
                                 const uint64_t* dense_off, const float* dense, const int32_t* rects,
                                 const float* tf, uint32_t np, const uint32_t* pixels, const float* target,
                                 double* dtf, double* ddense);

/* ---- per-block field read, as the reference's worker does it ----
 * BlockTreeFieldService::interpolateWith constructs a BlockTreeFieldProvider per call, which opens the
 * field file (include/s3dmm/BlockTreeFieldService.hpp:118-145, BlockTreeFieldProvider.hpp:93-106), and
 * fieldValuesPriv seeks to the subtree and reads its range and values (:157-168).  For each of nb blocks:
 * open `path`, seek to offsets[b], read 2 + counts[b] floats, close; values to out at the prefix sum of
 * counts, ranges (optional) to ranges[2b].  Returns 0, or -1 on an I/O failure. */
int orc_read_blocks_per_call(const char* path, const uint64_t* offsets, const uint64_t* counts, uint32_t nb,
                             float* out, float* ranges);

#ifdef __cplusplus
}
#endif

#endif /* S3R_ORACLE_H */
