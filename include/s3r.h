/*
 * s3r — GB300-native (sm_103a) implementation of the ReVisE block hot path:
 * sparse-octree -> dense-grid interpolation, the block ray caster and the
 * blend of per-block image parts.
 *
 * C ABI.  Every entry point is extern "C", never throws, and returns an int
 * status (S3R_OK == 0).  The message of the last failure on a context comes
 * from s3r_last_error(ctx) (ctx may be NULL for failures before a context
 * exists).  Pointers documented "device" are device pointers owned by the
 * caller; pointers documented "host" are host memory.  Each call that touches
 * the GPU takes the stream to order its work on (a cudaStream_t passed as
 * void*; NULL = the legacy default stream) and returns without synchronizing
 * unless documented otherwise.  One context per host thread, as the
 * reference keeps one renderer per worker thread.
 *
 * Reference interfaces replaced (paths relative to the reference project root):
 *   s3r_interp_dense           DenseFieldInterpolatorArr_cu_3::interpolate
 *                              (src/s3dmm_cuda/DenseFieldInterpolatorArr_cu_3.cu:197-257) and the static
 *                              DenseFieldInterpolator<3>::interpolate(dense, sparse, nodes)
 *                              (include/s3dmm/DenseFieldInterpolator.hpp:198-419)
 *   s3r_clear_viewport         DenseFieldRenderer_cu::clearViewport (src/s3dmm_cuda/DenseFieldRenderer_cu.cu:268-277)
 *   s3r_render_block_argb      DenseFieldRenderer_cu::renderDenseField, Argb mode
 *                              (src/s3dmm_cuda/DenseFieldRenderer_cu.cu:279-486, renderArgb.hpp:30-55)
 *   s3r_render_block           renderDenseField in every field mode (s3vs::FieldMode,
 *                              include/s3vs/FieldMode.hpp:26-54; render*.hpp, cuda_lighting.hpp)
 *   s3r_default_light          the renderer's single light source (DenseFieldRenderer_cu.cu:440-445)
 *   s3r_block_cube,
 *   s3r_block_view_rect,
 *   s3r_camera_from_view,
 *   s3r_camera_look_at         the host-side parameter set-up of renderDenseField (:317-409, :353-372)
 *   s3r_b2f_order              BackToFrontOrder<MacroBlock<3>>::range(eye) (include/BackToFrontOrder.hpp:61-359)
 *   s3r_split_index_cube,
 *   s3r_split_b2f              IndexCubeSplitter<3> (include/IndexCubeSplitter.hpp) and
 *                              IndexCubeSplitStorage::getBoxesSorted (src/s3vs_lib/IndexCubeSplitStorage.hpp)
 *   s3r_bound_rect             getBoundRect (src/s3vs_worker/cuda/VsWorker_cu.cpp:51-88)
 *   s3r_render_scene_part      VsWorker_cu::renderScenePart (src/s3vs_worker/cuda/VsWorker_cu.cpp:225-313)
 *   s3r_blend_image_part_host,
 *   s3r_compose_parts          blendImagePart (src/s3vs_lib/BlendImagePart.hpp:61-145)
 *   s3r_blend_image_part_mip_host  blendImagePartMaxIntensity (src/s3vs_lib/BlendImagePart.hpp:148-191)
 *   s3r_make_color_transfer    makeColorTransferVector (include/s3vs/ColorTransferFunction.hpp:27-69)
 *   s3r_frame_*                no single counterpart: the batched form of VsWorker_cu::renderScenePart
 *                              (src/s3vs_worker/cuda/VsWorker_cu.cpp:225-313) over a whole block cube
 *   s3r_render_argb_backward   none (the reference has no adjoint)
 *   s3r_dataset_*              BlockTreeFieldService<3> (include/s3dmm/BlockTreeFieldService.hpp:31-262),
 *                              Metadata<3> (include/s3dmm/Metadata.hpp:119-499),
 *                              BlockTreeFieldProvider<3>::fieldValues (include/s3dmm/BlockTreeFieldProvider.hpp:111-168),
 *                              BlockTreeNodes<3> (include/s3dmm/BlockTreeNodes.hpp:51-183)
 *   s3r_dataset_propagate,
 *   s3r_field_divide           BlockTreeFieldProvider<3>::generatePropagatedField's child -> parent step
 *                              (include/s3dmm/BlockTreeFieldProvider.hpp:270-389)
 */
#ifndef S3R_H
#define S3R_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define S3R_ABI_VERSION 7

/* status codes */
#define S3R_OK 0
#define S3R_ERR_INVALID 1     /* bad argument (null pointer, size out of range, ...) */
#define S3R_ERR_CUDA 2        /* a CUDA runtime call failed; see s3r_last_error */
#define S3R_ERR_NOMEM 3       /* device or host allocation failed */
#define S3R_ERR_CANCELLED 4   /* the cancel flag was set between blocks */
#define S3R_ERR_UNSUPPORTED 5 /* valid request this build does not handle */

/* Field value that marks "outside the domain" in sparse input
 * (BlockTreeFieldProvider<N>::noFieldValue(), include/s3dmm/BlockTreeFieldProvider.hpp:137-139).
 * Masked sparse nodes must carry this value, never NaN: NaN in a dense grid
 * means "not computed yet" while the interpolation runs. */
#define S3R_NO_FIELD_VALUE 1e30f

/* Deepest subtree the kernels accept: 2^9+1 = 513 vertices per edge. */
#define S3R_MAX_DEPTH 9

typedef struct s3r_ctx s3r_ctx;
typedef struct s3r_plan s3r_plan;

/* ------------------------------------------------------------------ context */

int s3r_abi_version(void);
/* Binds the calling thread to `device` (cudaSetDevice, as selectGpu does,
 * src/s3dmm_cuda/selectGpu.cu:6-9) and creates a context there. */
int s3r_ctx_create(int device, s3r_ctx** out);
int s3r_ctx_destroy(s3r_ctx* ctx);
const char* s3r_last_error(const s3r_ctx* ctx);
/* Kernel launches this context has issued so far (for launch accounting). */
uint64_t s3r_ctx_launch_count(const s3r_ctx* ctx);

/* ---------------------------------------------------- dense interpolation */

/* Dense (2^depth+1)^3 float grid of one block-tree subtree from its n sparse
 * nodes.  n2i_xyz (device): n vertex indices (x, y, z as uint16, 6 bytes per
 * node, the BlockTreeNodes<3> n2i layout); sparse (device): n values aligned
 * with n2i, S3R_NO_FIELD_VALUE where masked; dense (device): receives the grid,
 * x fastest (ordinal (z*e + y)*e + x with e = 2^depth+1), NaN outside the
 * domain.  Scratch: a (2^depth+1)^3 float grid owned by the context, grown on
 * demand (the call may allocate device memory the first time it sees a
 * larger depth).  Bit-identical to the reference CPU interpolator. */
int s3r_interp_dense(s3r_ctx* ctx, const uint16_t* n2i_xyz, const float* sparse, uint32_t n, uint32_t depth,
                     float* dense, void* stream);

/* Deepest subtree s3r_interp_dense_noalloc accepts: its scratch holds 129^3 floats (8.6 MB). */
#define S3R_NOALLOC_MAX_DEPTH 7

/* No counterpart in the reference.  The same interpolation as s3r_interp_dense
 * (same arguments, bit-identical output) for callers that cannot call
 * cudaMalloc -- applications whose device memory belongs to their own pool
 * allocator or is reserved up front, and loops that must not stall on the
 * device-wide synchronization of cudaMalloc/cudaFree.  It takes no context and
 * allocates nothing: its scratch is a fixed 8.6 MB __device__ array that every
 * GPU loading the library holds until exit.  depth > S3R_NOALLOC_MAX_DEPTH is
 * rejected with S3R_ERR_INVALID.  All calls share the array: calls that overlap
 * on the GPU race and must be ordered on one stream.  The first call on a device
 * looks up the array's address there (make it before any stream capture).
 * Errors: s3r_last_error(NULL). */
int s3r_interp_dense_noalloc(const uint16_t* n2i_xyz, const float* sparse, uint32_t n, uint32_t depth, float* dense,
                             void* stream);

/* --------------------------------------------------------- camera / view */

/* Renderer eye parameters (RenderKernelEyeParam, src/s3dmm_cuda/RenderKernelParam.hpp:56-65)
 * plus the world-to-eye rotation rows and translation the view rectangle needs.
 * ortho != 0 (no reference counterpart): rays start at eye + e1*x + e2*y and run along n. */
typedef struct s3r_camera {
    float eye[3];
    float e1[3];
    float e2[3];
    float n[3];
    float w;
    float h;
    int32_t ortho;
    int32_t reserved;
    float view_r[9];
    float view_t[3];
} s3r_camera;

/* Everything one render needs besides bricks and the transfer function. */
typedef struct s3r_view {
    s3r_camera cam;
    uint32_t W, H;         /* viewport, pixels */
    uint32_t level;        /* block level: cube half size 5/2^level, world cube [-5,5]^3 */
    float field_min;       /* global field range (BlockTreeFieldService::fieldRange) */
    float field_max;
    float threshold;       /* absolute threshold; opacity factor = (threshold-min)/(max-min) */
    float quality;         /* sampling quality (renderQuality) */
    uint32_t tf_n;         /* transfer-function entries, RGBA float each, 2..4096 */
    float alpha_stop;      /* batched path: stop a ray once its alpha exceeds this (>= 1: never) */
    uint32_t filter;       /* S3R_FILTER_EXACT or S3R_FILTER_TEXTURE */
    uint32_t reserved[2];
} s3r_view;

/* How a sample is filtered from a brick and from the transfer function.
 * EXACT: FP32 trilinear / linear interpolation with the exact fractions; a
 *   sample whose 8 texels hold a NaN is skipped.
 * TEXTURE: the linear filtering the GPU texture unit applies to the
 *   reference's tex3D / tex1D fetches (RenderFuncInput.hpp:42-50,
 *   renderArgb.hpp:44): 8-bit fractions, weights rounded to 1/256 in the
 *   unit's own order, and a NaN texel skipping the sample only when all its
 *   per-axis weights are nonzero -- results match the reference's renderer.
 *   No adjoint (the weights are piecewise constant). */
#define S3R_FILTER_EXACT 0u
#define S3R_FILTER_TEXTURE 1u

/* getLookAt(eye, center, up) + the eye set-up of DenseFieldRenderer_cu.cu:353-372.
 * Perspective: fovy_deg is the vertical field of view.  Orthographic (ortho != 0):
 * ortho_height is the world height the viewport covers. */
int s3r_camera_look_at(const double eye[3], const double center[3], const double up[3], double fovy_deg,
                       uint32_t W, uint32_t H, int32_t ortho, double ortho_height, s3r_camera* out);

/* The camera the reference's renderer derives from VsRenderSharedState::cameraTransform
 * (DenseFieldRenderer_cu.cu:353-372): view = the world -> eye transform of a rigid camera, column-major
 * 4x4 floats; its inverse is taken as a rigid motion (rotation transposed), the screen axes normalized in
 * float; h = 2 Lcam tan(fovY/2) with Lcam = 0.1, w = (h/H) W.  view_r / view_t keep the transform for the
 * view rectangles. */
int s3r_camera_from_view(const float view[16], float fovy_deg, uint32_t W, uint32_t H, s3r_camera* out);

/* Cube of block idx at level (DenseFieldRenderer_cu.cu:337-350). */
int s3r_block_cube(uint32_t level, const uint32_t idx[3], float center[3], float* half_size);

/* View rectangle {x, y, W, H} (pixels) the reference launches a block's rays over
 * (DenseFieldRenderer_cu.cu:374-409). */
int s3r_block_view_rect(const s3r_view* view, const uint32_t idx[3], int32_t rect[4]);

/* ------------------------------------------------------ plain block render */

/* Fills W*H pixels with value (0; NaN bits for the MIP mode). */
int s3r_clear_viewport(s3r_ctx* ctx, uint32_t* viewport, uint32_t W, uint32_t H, uint32_t value, void* stream);

/* Ray-casts one block into an ARGB32 viewport (device, W*H, top row first) with
 * the reference's Argb-mode arithmetic: exact FP32 trilinear filtering, linear
 * transfer-function lookup, opacity correction, front-to-back compositing with
 * early termination at alpha > 0.996, then blend-above into the pixel with
 * ARGB8 quantization.  brick (device): (2^depth+1)^3 floats; tf (device): tf_n
 * RGBA floats; rect: the block's view rectangle (s3r_block_view_rect). */
int s3r_render_block_argb(s3r_ctx* ctx, const s3r_view* view, const float* brick, uint32_t depth,
                          const uint32_t idx[3], const int32_t rect[4], const float* tf, uint32_t* viewport,
                          void* stream);

/* Field modes, numbered as s3vs::FieldMode (include/s3vs/FieldMode.hpp:26-54). */
#define S3R_MODE_ISOSURFACE 0u            /* one isosurface at view.threshold, lit */
#define S3R_MODE_ISOSURFACES 1u           /* isosurfaces at presentation.levels, lit */
#define S3R_MODE_MAX_INTENSITY 2u         /* maximum value above view.threshold; the pixel holds float bits */
#define S3R_MODE_ARGB 3u                  /* volume rendering (s3r_render_block_argb) */
#define S3R_MODE_ARGB_LIGHT 4u            /* volume rendering, every sample lit */
#define S3R_MODE_DOMAIN_VOXELS 5u         /* constant colour where the field is defined */
#define S3R_MODE_VALUE_ON_ISOSURFACE 6u   /* secondary field's colour on one isosurface of the primary */
#define S3R_MODE_VALUE_ON_ISOSURFACES 7u  /* secondary field's colour on several isosurfaces */

#define S3R_MAX_LEVELS 50u                /* RenderKernelPresentationParam::MaxLevels */
#define S3R_MAX_LIGHTS 10u                /* RenderKernelLightsParam::MaxSources */

/* A light source (LightSource, RenderKernelParam.hpp:68-74), world coordinates. */
typedef struct s3r_light {
    float pos[3];
    float ambient[3];
    float diffuse[3];
    float specular[3];
} s3r_light;

/* What a field mode needs beyond s3r_view (RenderKernelPresentationParam and
 * RenderKernelLightsParam): view.threshold is the isosurface level (absolute)
 * in the single-isosurface modes and the opacity threshold otherwise, as the
 * reference sets it (DenseFieldRenderer_cu.cu:418-434). */
typedef struct s3r_presentation {
    uint32_t mode;                   /* S3R_MODE_* */
    float isosurface_opacity;        /* multiplies the transfer-function alpha on isosurfaces */
    uint32_t level_count;            /* isosurface levels, absolute, ascending and distinct, <= S3R_MAX_LEVELS */
    float levels[50];
    uint32_t light_count;            /* <= S3R_MAX_LIGHTS */
    s3r_light lights[10];
    float secondary_min;             /* secondary field range (value-on-isosurface modes) */
    float secondary_max;
} s3r_presentation;

/* The renderer's light: at eye + n + e2 * h, no ambient, diffuse 1, specular 0.1. */
int s3r_default_light(const s3r_view* view, s3r_light* out);

/* Ray-casts one block in any field mode into the viewport, as renderKernel<mode>
 * does (DenseFieldRenderer_cu.cu:62-215 with render*.hpp): the same ray set-up,
 * sampling (view.filter) and compositing as s3r_render_block_argb; lit modes
 * shade with a central-difference gradient of the field (+-0.1 texel) and the
 * Blinn model of cuda_lighting.hpp.  brick2: the secondary field's brick on the
 * same block (value-on-isosurface modes, else NULL).  S3R_MODE_MAX_INTENSITY
 * writes float bits (field value mapped to [0, 1], or the previous pixel) that
 * s3r_blend_image_part_mip_host composes. */
int s3r_render_block(s3r_ctx* ctx, const s3r_view* view, const s3r_presentation* pres, const float* brick,
                     const float* brick2, uint32_t depth, const uint32_t idx[3], const int32_t rect[4],
                     const float* tf, uint32_t* viewport, void* stream);

/* ------------------------------------------------- texture-unit block render
 *
 * The reference samples a block's dense field and the transfer function through the GPU's texture unit
 * (tex3D on a 3-D float array with linear filtering and clamp addressing, tex1D on a one-row RGBA array;
 * DenseFieldRenderer_cu.cu:503-586, RenderFuncInput.hpp:42-50, renderArgb.hpp:44).  These calls do the
 * same, so that their images are the reference's: the per-block drop-in for renderDenseField and the
 * worker loop (s3r_render_scene_part with S3R_FILTER_TEXTURE). */

typedef struct s3r_texture s3r_texture;       /* a block's dense field, (2^depth+1)^3 texels */
typedef struct s3r_tf_texture s3r_tf_texture; /* a transfer function, tf_n RGBA texels */

/* A field texture for blocks of this depth (Device3DArray + DeviceTextureObject; allocates). */
int s3r_texture_create(s3r_ctx* ctx, uint32_t depth, s3r_texture** out);
int s3r_texture_destroy(s3r_texture* tex);
/* Copies a dense grid (device, (2^depth+1)^3 floats in the s3r_interp_dense layout) into the texture. */
int s3r_texture_fill(s3r_ctx* ctx, s3r_texture* tex, const float* dense, void* stream);
/* s3r_interp_dense into the texture (DeviceField::makeField, DenseFieldRenderer_cu.cu:505-546): the grid
 * is interpolated into a context-owned linear grid (grown on demand) and copied into the array. */
int s3r_interp_dense_texture(s3r_ctx* ctx, const uint16_t* n2i_xyz, const float* sparse, uint32_t n,
                             s3r_texture* tex, void* stream);
/* A transfer-function texture of tf_n entries (makeColorTransferTexture, DenseFieldRenderer_cu.cu:566-586:
 * one row of RGBA floats, normalized coordinates, linear filtering, clamp; allocates). */
int s3r_tf_texture_create(s3r_ctx* ctx, uint32_t tf_n, s3r_tf_texture** out);
/* Copies tf (device, tf_n RGBA floats) into the texture. */
int s3r_tf_texture_set(s3r_ctx* ctx, s3r_tf_texture* tex, const float* tf, void* stream);
int s3r_tf_texture_destroy(s3r_tf_texture* tex);
/* renderDenseField's kernel launch (renderKernel<mode>, DenseFieldRenderer_cu.cu:62-215, 447-483) for one
 * block sampled through the texture unit: s3r_render_block's arithmetic with tex3D / tex1D fetches and the
 * reference's ray set-up.  pres NULL: Argb.  field2: the secondary field (value-on-isosurface modes), same
 * depth.  tf->tf_n must equal view->tf_n; view->filter is not consulted. */
int s3r_render_block_texture(s3r_ctx* ctx, const s3r_view* view, const s3r_presentation* pres,
                             const s3r_texture* field, const s3r_texture* field2, const uint32_t idx[3],
                             const int32_t rect[4], const s3r_tf_texture* tf, uint32_t* viewport, void* stream);

/* ----------------------------------------------------------- ordering */

/* Back-to-front order of the blocks of index box [bmin, bmax) whose world box
 * is [cmin, cmax], for the eye point.  out (host): capacity*3 uint32; *count
 * receives the block count (the full count even when capacity is smaller). */
int s3r_b2f_order(const uint32_t bmin[3], const uint32_t bmax[3], const double cmin[3], const double cmax[3],
                  const double eye[3], uint32_t* out, uint32_t capacity, uint32_t* count);

/* World box of an index box at level (s3vs::boundingBoxOfIndexBox, src/s3vs_worker/BlockOrderUtil.hpp:29-52). */
/* IndexCubeSplitter<3>(level, split_count, [-5,5]^3).all_blocks(add_trailing_empty)
 * (include/IndexCubeSplitter.hpp:36-196): the (2^level)^3 block cube cut into axis-aligned index boxes for
 * split_count workers -- slabs along x first, then y, then z, each axis into at most 2^level slabs at
 * i*size/slabs.  boxes: count x {min x, y, z, max x, y, z} (max exclusive), x fastest; with
 * add_trailing_empty, empty boxes (all zero) up to split_count. */
int s3r_split_index_cube(uint32_t level, uint32_t split_count, int32_t add_trailing_empty, uint32_t* boxes,
                         uint32_t capacity, uint32_t* count);
/* The same boxes in back-to-front order for the eye (IndexCubeSplitStorage::getBoxesSorted,
 * src/s3vs_lib/IndexCubeSplitStorage.hpp:54-74: BackToFrontOrder over the splitter, whose boundaries are
 * split at the eye coordinate by NonUniformIndexRangeSplitter). */
int s3r_split_b2f(uint32_t level, uint32_t split_count, const double eye[3], uint32_t* boxes, uint32_t capacity,
                  uint32_t* count);
int s3r_index_box_world(uint32_t level, const uint32_t bmin[3], const uint32_t bmax[3], double cmin[3],
                        double cmax[3]);

/* ------------------------------------------------------ image parts, blend */

/* Bounding rectangle {x, y, w, h} of the pixels with nonzero alpha byte, in
 * image rows as stored (getBoundRect).  w == h == 0 when there are none.
 * Synchronizes the stream (the result lands in host memory). */
int s3r_bound_rect(s3r_ctx* ctx, const uint32_t* viewport, uint32_t W, uint32_t H, int32_t rect[4], void* stream);

/* Copies the w x h sub-image at (x, y) of a W-wide image into dst (w*h pixels); device pointers. */
int s3r_crop(s3r_ctx* ctx, const uint32_t* image, uint32_t W, const int32_t rect[4], uint32_t* dst, void* stream);

/* Host restatement of blendImagePart: src (sw x sh at origin ox, oy) over dst (dw x dh). */
int s3r_blend_image_part_host(uint32_t* dst, int32_t dw, int32_t dh, const uint32_t* src, int32_t sw, int32_t sh,
                              int32_t ox, int32_t oy, int32_t just_copy, int32_t offx, int32_t offy);

/* Host restatement of blendImagePartMaxIntensity: pixels hold floats; a non-NaN
 * source replaces a NaN or smaller destination. */
int s3r_blend_image_part_mip_host(float* dst, int32_t dw, int32_t dh, const float* src, int32_t sw, int32_t sh,
                                  int32_t ox, int32_t oy, int32_t just_copy, int32_t offx, int32_t offy);

/* One image part for s3r_compose_parts: a device ARGB32 image at an origin. */
typedef struct s3r_image_part {
    const uint32_t* pixels;
    int32_t origin[2];
    int32_t size[2];
} s3r_image_part;

/* Blends the parts into dst (device, dw x dh, origin offx, offy) in array order,
 * each exactly as blendImagePart would (parts[0] first; just_copy_first copies it). */
int s3r_compose_parts(s3r_ctx* ctx, const s3r_image_part* parts, uint32_t nparts, int32_t just_copy_first,
                      uint32_t* dst, int32_t dw, int32_t dh, int32_t offx, int32_t offy, void* stream);

/* ------------------------------------------------------------- worker loop */

/* The blocks of one level a worker renders: per block {ix, iy, iz, depth} and its nodes. */
typedef struct s3r_worker_blocks {
    uint32_t nblocks;
    const uint32_t* blocks;    /* host: nblocks x {ix, iy, iz, depth} */
    const uint64_t* node_off;  /* host: nblocks+1 prefix offsets into n2i / sparse */
    const uint16_t* n2i;       /* device: node_off[nblocks] x {x, y, z} */
    const float* sparse;       /* device: node_off[nblocks] values (S3R_NO_FIELD_VALUE where masked) */
    const float* sparse2;      /* device, optional: the secondary field on the same nodes */
} s3r_worker_blocks;

/* VsWorker_cu::renderScenePart (src/s3vs_worker/cuda/VsWorker_cu.cpp:225-313) natively, for the index box
 * [box_min, box_max) of view->level: the viewport (device, W*H ARGB32) cleared as clearViewport clears it,
 * the box's blocks visited back to front for the view's eye (BackToFrontOrder over the box, blocks missing
 * from wb skipped), each block's dense field interpolated from its nodes into the context's scratch
 * (s3r_interp_dense; the secondary field too for the value-on-isosurface modes) and ray-cast into the
 * viewport (s3r_render_block, or s3r_render_block_argb when pres is NULL) -- with S3R_FILTER_TEXTURE into
 * context-owned field textures per depth and a transfer-function texture filled from tf at the start of the
 * call (s3r_interp_dense_texture, s3r_render_block_texture), as the reference samples; then rect = the bounding
 * rectangle of the non-transparent pixels (s3r_bound_rect; {0,0,0,0} when empty) -- the part s3r_crop
 * cuts out.  Allocates the scratch on the first call for a depth; synchronizes the stream at the end. */
int s3r_render_scene_part(s3r_ctx* ctx, const s3r_view* view, const s3r_presentation* pres,
                          const s3r_worker_blocks* wb, const uint32_t box_min[3], const uint32_t box_max[3],
                          const float* tf, uint32_t* viewport, int32_t rect[4], void* stream);

/* s3r_render_scene_part with the blocks' dense fields taken from a plan's brick store (F32; interpolated
 * for all of the plan's blocks at once by s3r_frame_interp) instead of interpolated block by block:
 * per block of the box (back to front) only the render launch.  bricks2: the secondary field's brick
 * store in the plan's layout (value-on-isosurface modes). */
int s3r_render_scene_part_bricks(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const s3r_presentation* pres,
                                 const void* bricks2, const uint32_t box_min[3], const uint32_t box_max[3],
                                 const float* tf, uint32_t* viewport, int32_t rect[4], void* stream);

/* ------------------------------------------------ transfer-function table */

/* npoints control points sorted by x: xs (host) and rgba (host, 4 per point). */
int s3r_make_color_transfer(const double* xs, const double* rgba, uint32_t npoints, uint32_t color_count,
                            float* out);

/* --------------------------------------------------- batched frame (plan) */

#define S3R_BRICK_F32 0
#define S3R_BRICK_F16 1  /* value = offset + scale * half, per-brick FP32 scale/offset */
#define S3R_BRICK_BF16 2 /* value = offset + scale * bfloat16 */

/* Frame render forms (s3r_frame_desc.render_tile):
 *   ids below S3R_RENDER_TILES_WALK: one thread (or 2, 4, 8 lanes) per pixel ray walks the block grid
 *     front to back and composites every block it passes (4 CTA pixel shapes x 4 lane counts; several
 *     lanes per ray merge partial composites in another association order, within 1e-5);
 *   ids S3R_RENDER_TILES_WALK .. S3R_RENDER_TILES-1: block-major -- CTAs take pixel tiles of the
 *     blocks' view rectangles (deepest blocks first) and march one block each, the per-block results
 *     are blended per pixel in front-to-back order afterwards; the same image bit for bit as id 0, for
 *     levels up to 7, at the cost of (3 * 2^level - 2) x W x H x 16 bytes of device memory per data slot.
 * The autotuner times every form. */
#define S3R_RENDER_TILES_WALK 16u
#define S3R_RENDER_TILES 19u

/* Static description of a block set: the topology part of a block tree level
 * (one BlockTreeNodes n2i list per block), fixed across time frames. */
typedef struct s3r_frame_desc {
    uint32_t level;            /* blocks are cubes of this level */
    uint32_t nblocks;
    const uint32_t* blocks;    /* host: nblocks x {ix, iy, iz, depth} */
    const uint64_t* node_off;  /* host: nblocks+1 prefix offsets into n2i / sparse values */
    const uint16_t* n2i;       /* host: node_off[nblocks] x {x, y, z} */
    uint32_t brick_format;     /* S3R_BRICK_* */
    uint32_t tile_cells;       /* interpolation tile edge in cells: 8, 16 or 32; 0 = autotuned */
    uint32_t render_tile;      /* render form and CTA shape id (< S3R_RENDER_TILES); 0 = autotuned */
    uint32_t reserved;
} s3r_frame_desc;

typedef struct s3r_plan_info {
    uint64_t nodes;          /* sparse nodes over all blocks */
    uint64_t vertices;       /* dense vertices over all blocks */
    uint64_t brick_bytes;    /* bytes of the brick store (rows padded to the brick pitch) */
    uint64_t tiles;          /* interpolation work items */
    uint64_t tile_entries;   /* binned node entries (nodes on tile boundaries repeat) */
    uint32_t tile_cells;
    uint32_t render_tile;
    uint32_t brick_format;
    uint32_t nblocks;
} s3r_plan_info;

/* Bins the nodes by interpolation tile, uploads the plan and allocates the
 * brick store (device).  Allocates; call before any stream capture. */
int s3r_frame_plan(s3r_ctx* ctx, const s3r_frame_desc* desc, s3r_plan** out);
int s3r_plan_destroy(s3r_plan* plan);
int s3r_plan_info_get(const s3r_plan* plan, s3r_plan_info* out);
/* Device pointer to the brick store and, per block, the offset of its first element (host, nblocks+1
 * entries).  Block b's vertex (x, y, z) is element vertex_off[b] + (z (2^d+1) + y) pitch[b] + x, with the
 * row pitch from s3r_plan_brick_pitches: 2^d+1 rounded up to whole 32-byte sectors (elements between
 * 2^d+1 and the pitch are never written nor read). */
int s3r_plan_bricks(const s3r_plan* plan, void** bricks, const uint64_t** vertex_off);
/* Per block: the brick row pitch in elements (host, nblocks entries). */
int s3r_plan_brick_pitches(const s3r_plan* plan, const uint32_t** pitch);
/* Per-brick {scale, offset} pairs (device, 2 floats per block; F16/BF16 only, else NULL). */
int s3r_plan_brick_scales(const s3r_plan* plan, const float** scale_offset);

/* The interpolation tile edge (cells) of the plan's blocks of depth `depth`: the
 * plan's tile_cells capped by the depth, or the autotuner's choice for that depth. */
int s3r_plan_tile_cells(const s3r_plan* plan, uint32_t depth, uint32_t* cells);

/* Project-written autotuner: times the interpolation of `sparse` with tiles of
 * 8, 16 and 32 cells, then per block depth (deepest first) a tile one step
 * smaller for that depth's blocks alone, and the frame render with each render form and CTA shape
 * (S3R_RENDER_TILES), `reps` runs each after one warm-up, keeps the fastest of
 * both and re-bins the plan for the chosen tile.  Several lanes per ray are
 * skipped when view->alpha_stop < 1; a block-major form whose buffers do not fit
 * is skipped.  Synchronizes the stream; allocates; drops captured graphs. */
int s3r_plan_autotune(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* sparse, const float* tf,
                      uint32_t reps, void* stream);

/* Interpolates every block of the plan from sparse (device, node_off[nblocks]
 * values aligned with n2i) into the brick store, in one launch of tile work items. */
int s3r_frame_interp(s3r_ctx* ctx, s3r_plan* plan, const float* sparse, void* stream);

/* Ray-casts the brick store front to back, block after block along each ray,
 * each block sampled exactly as s3r_render_block_argb samples it, composited
 * in FP32 without ARGB8 quantization.  rgba (device, optional): W*H float RGBA,
 * non-premultiplied colour and alpha, pixel (vx, vy) at (H-1-vy)*W+vx as in the
 * ARGB viewport; argb (device, optional): the same pixels as ARGB32;
 * samples (device, optional): one uint64 counter incremented by the samples taken. */
int s3r_frame_render(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* tf, float* rgba,
                     uint32_t* argb, unsigned long long* samples, void* stream);

/* The batched frame in any field mode (pres, as for s3r_render_block): every ray walks the plan's blocks
 * front to back, each block marched exactly as s3r_render_block marches it, the blocks' colours
 * composited in FP32 (no ARGB8 rounding between blocks), for max intensity the maximum over the blocks.
 * bricks2 (device): the secondary field's brick store in this plan's layout (s3r_plan_bricks of a second
 * plan over the same block set), needed by the value-on-isosurface modes, else may be NULL.
 * rgba (optional): W*H float RGBA, non-premultiplied (max intensity: t, t, t, 1 with t the relative
 * maximum, zero where no block gave one); argb (optional): ARGB32 (max intensity: the float bits of t,
 * NaN bits where none, as the reference's viewport holds them).  F32 plans only (else
 * S3R_ERR_UNSUPPORTED). */
int s3r_frame_render_mode(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const s3r_presentation* pres,
                          const float* tf, const void* bricks2, float* rgba, uint32_t* argb, void* stream);

/* s3r_frame_interp + s3r_frame_render as one CUDA graph, captured on the first
 * call for this (plan, pointers, viewport size, tf_n, filter) and replayed
 * afterwards; the view is copied to the device before each replay.  Allocates
 * on the first call. */
int s3r_frame_run(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* sparse, const float* tf,
                  float* rgba, uint32_t* argb, unsigned long long* samples, void* stream);

/* s3r_frame_run from host buffers, pipelined across frames: sparse_host (pinned, one float per node) is
 * copied to the device on a copy stream while the previous frame renders, and the frame's ARGB8 image goes
 * to argb_host (pinned, W*H) on a second copy stream while the next frame renders.  Two device slots
 * alternate, each with its own captured graph, brick store and compute stream, so that frame k and frame
 * k+1 overlap on the GPU; slot 0 is the plan's brick store, so s3r_frame_run and friends on the same plan
 * wait for s3r_frame_host_sync.
 * Ordering against `stream`: the frame starts after the work queued on `stream` before the call.  tf
 * (device) is copied into the slot's own table by a copy queued on `stream` during the call, so work the
 * caller queues on `stream` afterwards may change or free tf; the frame itself runs on the slot's
 * stream, which `stream` does not wait for.
 * On return sparse_host may be refilled, and the image of the previous call is complete in its
 * argb_host; this call's image is complete after the next call or s3r_frame_host_sync, so argb_host must
 * stay allocated until then (two host image buffers used alternately let the caller read each frame
 * while the next one renders).  A failing call first waits for the work already queued by earlier calls. */
int s3r_frame_run_host(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* sparse_host,
                       const float* tf, uint32_t* argb_host, void* stream);
/* Waits until every frame submitted with s3r_frame_run_host has been copied back. */
int s3r_frame_host_sync(s3r_ctx* ctx, s3r_plan* plan);

/* Adjoint of s3r_frame_render (F32 bricks) for L = 1/2 sum (I - target)^2:
 * given the forward image rgba (device) and dl_drgba = I - target (device,
 * W*H*4), accumulates dL/dtf (device, tf_n*4 floats) and dL/ddense (device,
 * one float per brick-store element, in the store's layout; padding elements
 * stay untouched).  Sample positions are recomputed per ray.
 * view->filter must be S3R_FILTER_EXACT (else S3R_ERR_UNSUPPORTED).
 * Allocates its scratch (512 copies of the table gradient) on the first call. */
int s3r_render_argb_backward(s3r_ctx* ctx, s3r_plan* plan, const s3r_view* view, const float* tf,
                             const float* rgba, const float* dl_drgba, float* dtf, float* ddense, void* stream);

/* ------------------------------------------------------ on-disk sparse fields
 *
 * Reader of the reference's dataset files, written by its preprocessing tools:
 *   <base>.s3dmm-fields           text: time step count, then per field "name min max animated"
 *                                 (BlockTreeFieldService::readFieldInfoFile, include/s3dmm/BlockTreeFieldService.hpp:178-262)
 *   <frame>.s3dmm-meta            binary metadata: header, compressed block tree, per level a map
 *                                 subtree root -> {tree position, field file offset, depth}, field file size
 *                                 (Metadata<3>, include/s3dmm/Metadata.hpp:182-214, 401-443; v0 files without header too)
 *   <frame>.s3dmm-field#<name>    per subtree at its offset: float min, max, then one float per node
 *                                 (BlockTreeFieldProvider<3>::fieldValuesPriv, include/s3dmm/BlockTreeFieldProvider.hpp:157-168)
 * <frame> is <base> for a single-frame dataset, <dir>/<stem>/<stem>_tNNNNNN<ext> when <dir>/<stem> is a
 * directory (frameOutputFileName, include/filename_util.hpp:34-46).  A subtree's node order is the
 * BlockTreeNodes<3> order (include/s3dmm/BlockTreeNodes.hpp:60-74): blocks in depth-first pre-order down to
 * the subtree depth, per block its 8 corners (x fastest), each node where it first appears.  Files with
 * real_type = float (the reference's default) are read.
 *
 * Host-only except s3r_dataset_frame_upload.  Failures set s3r_last_error(NULL).  A dataset handle may be
 * used from one thread at a time. */

typedef struct s3r_dataset s3r_dataset;

typedef struct s3r_dataset_info {
    uint32_t format_version;    /* metadata format: 0 (no header) or 1 */
    uint32_t time_steps;        /* time frame count (.s3dmm-fields line 2) */
    uint32_t field_count;
    uint32_t max_subtree_depth;
    uint32_t max_full_level;
    uint32_t level_count;       /* levels holding subtree roots: 0 .. level_count-1 */
    uint32_t subtree_count;     /* metadataBlockCount() */
    uint32_t has_time_steps;    /* 1: per-frame files in <dir>/<stem>/ */
    uint64_t tree_blocks;       /* blocks of the whole block tree */
    uint64_t field_file_size;   /* bytes of each field file */
    float bc_min[3];            /* block tree bounding cube */
    float bc_size;
} s3r_dataset_info;

typedef struct s3r_subtree_info {
    uint32_t level, x, y, z;    /* subtree root block: level and index at that level */
    uint32_t depth;             /* subtree depth d: (2^d+1)^3 dense vertices */
    uint32_t tree_index;        /* position of the root in the compressed block tree */
    uint64_t values_offset;     /* byte offset of its {min, max, values...} in each field file */
    uint64_t node_count;        /* BlockTreeNodes<3>::nodeCount() */
} s3r_subtree_info;

/* Opens a dataset by the base name the reference's BlockTreeFieldService takes
 * (the preprocessed mesh file name; <base>.s3dmm-meta beside it is enough). */
int s3r_dataset_open(const char* base_name, s3r_dataset** out);
int s3r_dataset_close(s3r_dataset* ds);
int s3r_dataset_info_get(const s3r_dataset* ds, s3r_dataset_info* out);
/* Field `index`: its name (NUL-terminated, truncated to name_cap), global [min, max] (NaN where the file
 * has "-") and animated flag. */
int s3r_dataset_field(const s3r_dataset* ds, uint32_t index, char* name, size_t name_cap, float range[2],
                      int32_t* animated);
/* Index of the field called `name`, or S3R_ERR_INVALID (BlockTreeFieldService::fieldIndex). */
int s3r_dataset_field_index(const s3r_dataset* ds, const char* name, uint32_t* index);
/* The blocks of the whole block tree at `level` (Metadata::blockTree(), CompressedBlockTree<3>), in the
 * tree's breadth-first order: idx triples to xyz (min(cap, count) of them), the level's count to *count. */
int s3r_dataset_tree_blocks(const s3r_dataset* ds, uint32_t level, uint32_t* xyz, uint64_t cap, uint64_t* count);
/* The subtree roots of one level (Metadata::levels()[level]), sorted by z, then y, then x.  Writes
 * min(cap, count) records to out (may be NULL with cap 0) and the level's count to *count.  Computes and
 * caches node counts. */
int s3r_dataset_subtrees(s3r_dataset* ds, uint32_t level, s3r_subtree_info* out, uint32_t cap, uint32_t* count);
/* The subtree rooted at block idx of `level` (Metadata::subtreeData + its node count); S3R_ERR_INVALID if
 * that block is no subtree root. */
int s3r_dataset_subtree(s3r_dataset* ds, uint32_t level, const uint32_t idx[3], s3r_subtree_info* out);
/* BlockTreeNodes<3>(blockTree, root, depth).data().n2i of one subtree: node_count x {x, y, z} (host). */
int s3r_dataset_subtree_nodes(s3r_dataset* ds, uint32_t level, const uint32_t idx[3], uint16_t* n2i,
                              uint64_t cap_nodes, uint64_t* count);
/* BlockTreeFieldProvider<3>::fieldValues of one subtree for field `field` at time frame `frame`: its
 * stored [min, max] and node_count values (host), S3R_NO_FIELD_VALUE where masked. */
int s3r_dataset_subtree_values(s3r_dataset* ds, uint32_t field, uint32_t frame, uint32_t level,
                               const uint32_t idx[3], float range[2], float* values, uint64_t cap_nodes,
                               uint64_t* count);

/* A block set of one level for s3r_frame_plan: blocks idx[nb][3] (subtree roots of `level`).  Fills
 * blocks[nb][4] = {ix, iy, iz, depth} and node_off[nb+1]; when n2i is not NULL also the concatenated node
 * lists (node_off[nb] x 3 uint16, n2i_cap_nodes at least that).  Subtrees are walked on `threads` host
 * threads (0 = all cores). */
int s3r_dataset_frame_topology(s3r_dataset* ds, uint32_t level, const uint32_t* idx, uint32_t nb,
                               uint32_t* blocks, uint64_t* node_off, uint16_t* n2i, uint64_t n2i_cap_nodes,
                               uint32_t threads);
/* The field values of those blocks at node_off (host; node_off[nb] floats), their stored ranges to
 * ranges[nb][2] (optional), read on `threads` host threads (0 = all cores), one positioned read per block. */
int s3r_dataset_frame_values(s3r_dataset* ds, uint32_t field, uint32_t frame, uint32_t level,
                             const uint32_t* idx, uint32_t nb, const uint64_t* node_off, float* values,
                             float* ranges, uint32_t threads);
/* s3r_dataset_frame_values into one of two pinned staging buffers the dataset owns, then one
 * cudaMemcpyAsync of all node_off[nb] values to sparse (device) on `stream`: the per-block file read and
 * two host-to-device copies of the reference's worker loop become one read pass and one copy per frame.
 * The buffer used by the call before the previous one is waited for before it is refilled, so reading
 * frame t+1 overlaps the copy of frame t.  Allocates pinned memory when a larger frame arrives. */
int s3r_dataset_frame_upload(s3r_ctx* ctx, s3r_dataset* ds, uint32_t field, uint32_t frame, uint32_t level,
                             const uint32_t* idx, uint32_t nb, const uint64_t* node_off, float* sparse,
                             float* ranges, uint32_t threads, void* stream);

/* ---------------------------------------------------- upstream field generation
 *
 * The propagation step of BlockTreeFieldProvider<3>::generatePropagatedField
 * (include/s3dmm/BlockTreeFieldProvider.hpp:270-389), one level at a time on the GPU.  child_values (device):
 * the field on every subtree of level+1, concatenated in s3r_dataset_subtrees order, each subtree's
 * node_count values in its node order (S3R_NO_FIELD_VALUE where masked; may be NULL when level+1 has no
 * subtrees).  sums, weights (device): one float per node of every subtree of `level`, in the same order:
 * the sum, in child order (c = x + 2y + 4z), of the child values that land on the node and their count --
 * the reference's fieldValues / weightValues after its child loop.  child_count (host, optional): per parent
 * subtree how many child subtrees it has.  With all 8 the reference's value is s3r_field_divide of the
 * two; with fewer it first adds its generator's contributions (BlockTreeFieldFromFunc adds the function at
 * every block corner of the subtree) to both arrays, then divides the same way.  The first call for a
 * level works out, on the device, which child nodes land on which parent nodes (uploads both levels' node
 * lists, fills a (2^D+1)^3 vertex map per parent, checks that every child node finds its parent node,
 * keeps 32 bytes per parent node and frees the rest; allocates and synchronizes the device); every call
 * then runs one gather kernel on `stream` without synchronizing. */
int s3r_dataset_propagate(s3r_ctx* ctx, s3r_dataset* ds, uint32_t level, const float* child_values, float* sums,
                          float* weights, uint8_t* child_count, void* stream);
/* values[i] = weights[i] > 0 ? sums[i] / weights[i] : S3R_NO_FIELD_VALUE for n floats (device), the
 * final transform of generatePropagatedField and of BlockTreeFieldFromFunc::generate. */
int s3r_field_divide(s3r_ctx* ctx, const float* sums, const float* weights, uint64_t n, float* values, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* S3R_H */
