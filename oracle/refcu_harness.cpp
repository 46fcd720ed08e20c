// Test infrastructure only: runs the reference's own CUDA kernels on the GPU.
//
// oracle/Makefile target `refcu` compiles the reference's CUDA translation
// units src/s3dmm_cuda/DenseFieldInterpolatorArr_cu_3.cu and
// src/s3dmm_cuda/DenseFieldRenderer_cu.cu, in place and for their device code
// only, into oracle/_ref/ref_interp.cubin and oracle/_ref/ref_render.cubin.
// This harness (built on the GPU host, target `refcu-harness`) loads them with
// the CUDA driver API, finds the kernels by name, and drives them the way the
// reference's host code does:
//   ref_interp      DenseFieldInterpolatorArr_cu_3::interpolate
//                   (DenseFieldInterpolatorArr_cu_3.cu:197-257): NaN fill of a
//                   surface-capable 3D array, per-call device vectors for n2i and
//                   values, scatter, one interpolateDense3dFieldKernel launch per
//                   level, no-field -> NaN transform;
//   ref_render      DenseFieldRenderer_cu::renderDenseField, Argb mode
//                   (DenseFieldRenderer_cu.cu:279-486): linear-filtered clamped 3D
//                   texture on that array, 1D TF texture (normalized coordinates),
//                   RenderKernelParam filled as :317-445, renderKernel<Argb> over
//                   the view rectangle with 32x1 thread blocks;
//   ref_worker      VsWorker_cu::renderScenePart (VsWorker_cu.cpp:225-313) over a
//                   block list in the given back-to-front order: clear, per block
//                   interpolate + render, read the whole viewport back, host scan
//                   for the non-transparent rectangle.  Sparse values come from
//                   host memory (the reference reads each block's values from its
//                   field file, which is left out).
// The product never links, loads or calls this.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

int fail(const std::string& m)
{
    g_err = m;
    return 1;
}

#define CKR(x)                                                                                         \
    do {                                                                                               \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess) return fail(std::string(#x) + ": " + cudaGetErrorString(e_));          \
    } while (0)
#define CKD(x)                                                                                         \
    do {                                                                                               \
        CUresult r_ = (x);                                                                             \
        if (r_ != CUDA_SUCCESS) {                                                                      \
            const char* s_ = nullptr;                                                                  \
            cuGetErrorString(r_, &s_);                                                                 \
            return fail(std::string(#x) + ": " + (s_ ? s_ : "?"));                                      \
        }                                                                                              \
    } while (0)

// RenderKernelParam and its members, field for field (src/s3dmm_cuda/RenderKernelParam.hpp:26-116).
struct RKViewport { uint32_t* pixels; unsigned W, H; };
struct RKView { unsigned x, y, W, H; };
struct RKField { cudaTextureObject_t tex; unsigned texDepth; float minValue, maxValue; };
struct RKCube { float3 center; float halfSize; unsigned level; };
struct RKEye { float3 pos, e1, e2, n; float w, h, pixelSize; };
struct RKLight { float3 pos, ambient, diffuse, specular; };
struct RKPresentation {
    float threshold;
    float isosurfaceOpacity;
    cudaTextureObject_t colorTex;
    float quality;
    float levels[50];
    unsigned levelCount;
};
struct RKLights { RKLight sources[10]; unsigned sourceCount; };
struct RenderKernelParam {
    RKViewport viewport;
    RKView view;
    RKField primaryField;
    RKField secondaryField;
    RKCube cube;
    RKEye eye;
    RKPresentation presentation;
    RKLights lights;
};

struct Kernels {
    CUmodule interp = nullptr, render = nullptr;
    CUfunction fill = nullptr, scatter = nullptr, level = nullptr, nan = nullptr, argb = nullptr;
    CUfunction mode[8] = {};  // renderKernel<FieldMode(m)>
} K;

// The product's s3r_presentation (include/s3r.h), field for field.
struct Pres {
    uint32_t mode;
    float isosurface_opacity;
    uint32_t level_count;
    float levels[50];
    uint32_t light_count;
    struct { float pos[3], ambient[3], diffuse[3], specular[3]; } lights[10];
    float secondary_min, secondary_max;
};

// View of the camera, as the product's s3r_view lays it out (include/s3r.h).
struct View {
    float eye[3], e1[3], e2[3], n[3];
    float w, h;
    int32_t ortho, reserved;
    float view_r[9], view_t[3];
    uint32_t W, H, level;
    float field_min, field_max, threshold, quality;
    uint32_t tf_n;
    float alpha_stop;
    uint32_t reserved2[3];
};

int find(CUmodule m, const char* a, const char* b, CUfunction* out)
{
    unsigned cnt = 0;
    CKD(cuModuleGetFunctionCount(&cnt, m));
    std::vector<CUfunction> fns(cnt);
    CKD(cuModuleEnumerateFunctions(fns.data(), cnt, m));
    for (CUfunction f : fns) {
        const char* name = nullptr;
        CKD(cuFuncGetName(&name, f));
        if (name && std::strstr(name, a) && (!b || std::strstr(name, b))) {
            *out = f;
            return 0;
        }
    }
    return fail(std::string("kernel not found: ") + a + (b ? std::string(" / ") + b : ""));
}

unsigned blocks_for(unsigned n, unsigned b) { return (n + b - 1) / b; }

// A surface-capable float 3D array with its surface and (linear, clamped) texture.
struct Array3 {
    cudaArray_t a = nullptr;
    cudaSurfaceObject_t surf = 0;
    cudaTextureObject_t tex = 0;
    unsigned edge = 0;
    int resize(unsigned e)
    {
        if (a && edge == e) return 0;
        release();
        cudaChannelFormatDesc d = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
        CKR(cudaMalloc3DArray(&a, &d, make_cudaExtent(e, e, e), cudaArraySurfaceLoadStore));
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = a;
        CKR(cudaCreateSurfaceObject(&surf, &rd));
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.normalizedCoords = 0;
        td.filterMode = cudaFilterModeLinear;
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.readMode = cudaReadModeElementType;
        CKR(cudaCreateTextureObject(&tex, &rd, &td, nullptr));
        edge = e;
        return 0;
    }
    void release()
    {
        if (tex) cudaDestroyTextureObject(tex);
        if (surf) cudaDestroySurfaceObject(surf);
        if (a) cudaFreeArray(a);
        tex = 0;
        surf = 0;
        a = nullptr;
        edge = 0;
    }
} g_field, g_field2;

struct TfTexture {
    cudaArray_t a = nullptr;
    cudaTextureObject_t tex = 0;
    int make(const float* rgba, unsigned n)
    {
        release();
        cudaChannelFormatDesc d = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindFloat);
        CKR(cudaMallocArray(&a, &d, n, 1, cudaArrayTextureGather));
        CKR(cudaMemcpy2DToArray(a, 0, 0, rgba, n * 16, n * 16, 1, cudaMemcpyHostToDevice));
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = a;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.normalizedCoords = 1;
        td.filterMode = cudaFilterModeLinear;
        td.addressMode[0] = cudaAddressModeClamp;
        td.readMode = cudaReadModeElementType;
        CKR(cudaCreateTextureObject(&tex, &rd, &td, nullptr));
        return 0;
    }
    void release()
    {
        if (tex) cudaDestroyTextureObject(tex);
        if (a) cudaFreeArray(a);
        tex = 0;
        a = nullptr;
    }
} g_tf;

// Kernel-only timing of the worker loop (ref_cuda_worker_kernel_ms): when g_timed is set, every launch is
// bracketed by CUDA events and its time added to g_kernel_ms[g_phase] (0: interpolation, 1: render).
bool g_timed = false;
int g_phase = 0;
double g_kernel_ms[2] = {0.0, 0.0};

int launch(CUfunction f, dim3 g, dim3 b, void** args, CUstream stream = nullptr)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (g_timed) {
        CKR(cudaEventCreate(&e0));
        CKR(cudaEventCreate(&e1));
        CKR(cudaEventRecord(e0, (cudaStream_t)stream));
    }
    CKD(cuLaunchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, 0, stream, args, nullptr));
    if (g_timed) {
        CKR(cudaEventRecord(e1, (cudaStream_t)stream));
        CKR(cudaEventSynchronize(e1));
        float t = 0.f;
        CKR(cudaEventElapsedTime(&t, e0, e1));
        g_kernel_ms[g_phase] += t;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    return 0;
}

// DenseFieldInterpolatorArr_cu_3::interpolate into dst (g_field: primary, g_field2: secondary).
int interp_into(Array3& dst, const uint16_t* n2i, const float* sparse, uint32_t n, uint32_t depth)
{
    Array3& g_field = dst;
    const unsigned e = (1u << depth) + 1u;
    if (g_field.resize(e)) return 1;
    // fill(verticesPerEdge, array, NAN): 8^3 blocks
    {
        float nanv = NAN;
        void* args[] = {&g_field.surf, (void*)&e, &nanv};
        const unsigned bc = blocks_for(e, 8);
        if (launch(K.fill, dim3(bc, bc, bc), dim3(8, 8, 8), args)) return 1;
    }
    // per-call device vectors (DeviceVector<I3>, DeviceVector<real_type>)
    void* dn2i = nullptr;
    void* dval = nullptr;
    CKR(cudaMalloc(&dn2i, 6 * (size_t)n + 6));
    CKR(cudaMalloc(&dval, 4 * (size_t)n + 4));
    CKR(cudaMemcpy(dn2i, n2i, 6 * (size_t)n, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(dval, sparse, 4 * (size_t)n, cudaMemcpyHostToDevice));
    {
        void* args[] = {&g_field.surf, &dval, &dn2i, (void*)&n, (void*)&depth};
        if (n && launch(K.scatter, dim3(blocks_for(n, 32)), dim3(32), args)) return 1;
    }
    for (unsigned stage = 0; stage < depth; ++stage) {
        const unsigned ns = (1u << stage) + 1u;
        unsigned bs, bc;
        if (ns <= 8) {
            bs = ns;
            bc = 1;
        } else {
            bs = 8;
            bc = blocks_for(ns, bs - 1);
        }
        void* args[] = {&g_field.surf, (void*)&depth, &stage};
        if (launch(K.level, dim3(bc, bc, bc), dim3(bs, bs, bs), args)) return 1;
    }
    {
        char functor = 0;
        void* args[] = {&g_field.surf, (void*)&e, &functor};
        const unsigned bc = blocks_for(e, 8);
        if (launch(K.nan, dim3(bc, bc, bc), dim3(8, 8, 8), args)) return 1;
    }
    CKR(cudaFree(dn2i));
    CKR(cudaFree(dval));
    return 0;
}

int interp_into_field(const uint16_t* n2i, const float* sparse, uint32_t n, uint32_t depth)
{
    return interp_into(g_field, n2i, sparse, n, depth);
}

// renderKernel<mode> for one block (DenseFieldRenderer_cu.cu:317-482); pres == nullptr: Argb.
int render_block(const View& v, uint32_t depth, const uint32_t idx[3], const int32_t rect[4], uint32_t* viewport_dev,
                 const Pres* pres = nullptr, const Array3* f1 = &g_field, const Array3* f2 = &g_field2,
                 CUstream stream = nullptr)
{
    if (rect[2] <= 0 || rect[3] <= 0) return 0;
    RenderKernelParam p;
    std::memset(&p, 0, sizeof(p));
    p.viewport = {viewport_dev, v.W, v.H};
    p.primaryField = {f1->tex, depth, v.field_min, v.field_max};
    const float top = 5.f;
    const float h = top / (float)(1u << v.level);
    p.cube.halfSize = h;
    p.cube.center = make_float3(-top + h * (float)(1u + (idx[0] << 1)), -top + h * (float)(1u + (idx[1] << 1)),
                                -top + h * (float)(1u + (idx[2] << 1)));
    p.cube.level = v.level;
    p.eye.pos = make_float3(v.eye[0], v.eye[1], v.eye[2]);
    p.eye.e1 = make_float3(v.e1[0], v.e1[1], v.e1[2]);
    p.eye.e2 = make_float3(v.e2[0], v.e2[1], v.e2[2]);
    p.eye.n = make_float3(v.n[0], v.n[1], v.n[2]);
    p.eye.h = v.h;
    p.eye.pixelSize = v.h / (float)v.H;
    p.eye.w = p.eye.pixelSize * (float)v.W;
    p.view = {(unsigned)rect[0], (unsigned)rect[1], (unsigned)rect[2], (unsigned)rect[3]};
    p.presentation.threshold = v.threshold;
    p.presentation.colorTex = g_tf.tex;
    p.presentation.quality = v.quality;
    p.lights.sourceCount = 1;
    CUfunction kern = K.argb;
    if (pres) {
        if (pres->mode > 7 || !K.mode[pres->mode]) return fail("no kernel for mode " + std::to_string(pres->mode));
        kern = K.mode[pres->mode];
        p.presentation.isosurfaceOpacity = pres->isosurface_opacity;
        p.presentation.levelCount = pres->level_count;
        for (unsigned i = 0; i < pres->level_count && i < 50; ++i) p.presentation.levels[i] = pres->levels[i];
        p.lights.sourceCount = pres->light_count;
        for (unsigned i = 0; i < pres->light_count && i < 10; ++i) {
            const auto& L = pres->lights[i];
            p.lights.sources[i].pos = make_float3(L.pos[0], L.pos[1], L.pos[2]);
            p.lights.sources[i].ambient = make_float3(L.ambient[0], L.ambient[1], L.ambient[2]);
            p.lights.sources[i].diffuse = make_float3(L.diffuse[0], L.diffuse[1], L.diffuse[2]);
            p.lights.sources[i].specular = make_float3(L.specular[0], L.specular[1], L.specular[2]);
        }
        p.secondaryField = {f2->tex, depth, pres->secondary_min, pres->secondary_max};
    }
    // chooseKernelDim1d(view.W, 32), chooseKernelDim1d(view.H, 1)
    const unsigned W = rect[2], H = rect[3];
    dim3 grid(W <= 32 ? 1 : blocks_for(W, 32), H <= 1 ? 1 : H);
    dim3 block(W <= 32 ? W : 32, H <= 1 ? H : 1);
    void* args[] = {&p};
    return launch(kern, grid, block, args, stream);
}

} // namespace

extern "C" {

const char* ref_cuda_error(void) { return g_err.c_str(); }

// Loads both cubins (after the CUDA runtime made the primary context current).
int ref_cuda_init(const char* interp_cubin, const char* render_cubin)
{
    CKR(cudaFree(nullptr));
    CKD(cuModuleLoad(&K.interp, interp_cubin));
    CKD(cuModuleLoad(&K.render, render_cubin));
    if (find(K.interp, "fillKernel", nullptr, &K.fill) || find(K.interp, "scatterSparseFieldKernel", nullptr, &K.scatter) ||
        find(K.interp, "interpolateDense3dFieldKernel", nullptr, &K.level) ||
        find(K.interp, "transformInPlaceKernel", "ReplaceNoFieldValueWithNan", &K.nan) ||
        find(K.render, "renderKernel", "FieldModeE3", &K.argb))
        return 1;
    for (int m = 0; m < 8; ++m) {
        const std::string tag = "FieldModeE" + std::to_string(m) + "E";
        if (find(K.render, "renderKernel", tag.c_str(), &K.mode[m])) return 1;
    }
    size_t off = 0, size = 0;
    CKD(cuFuncGetParamInfo(K.argb, 0, &off, &size));
    if (size != sizeof(RenderKernelParam))
        return fail("RenderKernelParam size " + std::to_string(size) + " != " + std::to_string(sizeof(RenderKernelParam)));
    return 0;
}

int ref_cuda_interp(const uint16_t* n2i, const float* sparse, uint32_t n, uint32_t depth, float* dense)
{
    if (interp_into_field(n2i, sparse, n, depth)) return 1;
    const size_t e = g_field.edge;
    cudaMemcpy3DParms m;
    std::memset(&m, 0, sizeof(m));
    m.srcArray = g_field.a;
    m.dstPtr = make_cudaPitchedPtr(dense, e * 4, e, e);
    m.extent = make_cudaExtent(e, e, e);
    m.kind = cudaMemcpyDeviceToHost;
    CKR(cudaMemcpy3D(&m));
    return 0;
}

int ref_cuda_set_tf(const float* rgba, uint32_t n) { return g_tf.make(rgba, n); }

// One block into a host ARGB32 viewport (read-modify-write, as the reference).
int ref_cuda_render_block(const void* view, const uint16_t* n2i, const float* sparse, uint32_t n, uint32_t depth,
                          const uint32_t idx[3], const int32_t rect[4], uint32_t* viewport)
{
    const View& v = *static_cast<const View*>(view);
    if (interp_into_field(n2i, sparse, n, depth)) return 1;
    uint32_t* d = nullptr;
    const size_t bytes = (size_t)v.W * v.H * 4;
    CKR(cudaMalloc(&d, bytes));
    CKR(cudaMemcpy(d, viewport, bytes, cudaMemcpyHostToDevice));
    if (render_block(v, depth, idx, rect, d)) return 1;
    CKR(cudaMemcpy(viewport, d, bytes, cudaMemcpyDeviceToHost));
    CKR(cudaFree(d));
    return 0;
}

// One block in any field mode (pres: the product's s3r_presentation); sparse2:
// the secondary field's node values (same nodes) or NULL.
int ref_cuda_render_block_mode(const void* view, const void* pres, const uint16_t* n2i, const float* sparse,
                               const float* sparse2, uint32_t n, uint32_t depth, const uint32_t idx[3],
                               const int32_t rect[4], uint32_t* viewport)
{
    const View& v = *static_cast<const View*>(view);
    if (interp_into(g_field, n2i, sparse, n, depth)) return 1;
    if (sparse2 && interp_into(g_field2, n2i, sparse2, n, depth)) return 1;
    uint32_t* d = nullptr;
    const size_t bytes = (size_t)v.W * v.H * 4;
    CKR(cudaMalloc(&d, bytes));
    CKR(cudaMemcpy(d, viewport, bytes, cudaMemcpyHostToDevice));
    if (render_block(v, depth, idx, rect, d, static_cast<const Pres*>(pres))) return 1;
    CKR(cudaMemcpy(viewport, d, bytes, cudaMemcpyDeviceToHost));
    CKR(cudaFree(d));
    return 0;
}

// The worker loop over blocks already in back-to-front order: blocks[4*i] =
// {ix, iy, iz, depth}, their nodes at node_off[i]..node_off[i+1], rects[4*i]
// their view rectangles.  viewport receives the W*H ARGB32 image; crop[4] the
// non-transparent rectangle {x, y, w, h}; ms the wall time of the whole call.
int ref_cuda_worker(const void* view, uint32_t nblocks, const uint32_t* blocks, const uint64_t* node_off,
                    const uint16_t* n2i, const float* sparse, const int32_t* rects, uint32_t* viewport,
                    int32_t* crop, double* ms)
{
    const View& v = *static_cast<const View*>(view);
    const size_t npx = (size_t)v.W * v.H;
    static uint32_t* d = nullptr;
    static size_t dcap = 0;
    if (dcap < npx) {
        if (d) cudaFree(d);
        CKR(cudaMalloc(&d, npx * 4));
        dcap = npx;
    }
    CKR(cudaDeviceSynchronize());
    const auto t0 = std::chrono::steady_clock::now();
    CKR(cudaMemset(d, 0, npx * 4));
    std::vector<float> values;
    for (uint32_t i = 0; i < nblocks; ++i) {
        const uint64_t a = node_off[i], b = node_off[i + 1];
        // the reference reads these from the block's field file (fieldValues); here a host copy
        values.assign(sparse + a, sparse + b);
        if (interp_into_field(n2i + 3 * a, values.data(), (uint32_t)(b - a), blocks[4 * i + 3])) return 1;
        if (render_block(v, blocks[4 * i + 3], blocks + 4 * i, rects + 4 * i, d)) return 1;
    }
    CKR(cudaMemcpy(viewport, d, npx * 4, cudaMemcpyDeviceToHost));
    int minX = (int)v.W, maxX = 0, minY = (int)v.H, maxY = 0;
    for (uint32_t y = 0; y < v.H; ++y)
        for (uint32_t x = 0; x < v.W; ++x)
            if (viewport[(size_t)y * v.W + x] >> 24) {
                minX = std::min(minX, (int)x);
                maxX = std::max(maxX, (int)x);
                minY = std::min(minY, (int)y);
                maxY = std::max(maxY, (int)y);
            }
    if (minX > maxX) crop[0] = crop[1] = crop[2] = crop[3] = 0;
    else {
        crop[0] = minX;
        crop[1] = minY;
        crop[2] = maxX - minX + 1;
        crop[3] = maxY - minY + 1;
        std::vector<uint32_t> part((size_t)crop[2] * crop[3]);
        for (int y = 0; y < crop[3]; ++y)
            std::memcpy(&part[(size_t)y * crop[2]], viewport + (size_t)(minY + y) * v.W + minX, 4 * crop[2]);
    }
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

// The same worker loop with every kernel launch timed by CUDA events (each launch waited for, so the
// figures are kernel-only: no host copies, no launch overlap): interp_ms sums the interpolation kernels
// (fill, scatter, the d level passes, NaN transform), render_ms the renderKernel<Argb> launches.
int ref_cuda_worker_kernel_ms(const void* view, uint32_t nblocks, const uint32_t* blocks, const uint64_t* node_off,
                              const uint16_t* n2i, const float* sparse, const int32_t* rects, double* interp_ms,
                              double* render_ms)
{
    const View& v = *static_cast<const View*>(view);
    const size_t npx = (size_t)v.W * v.H;
    uint32_t* d = nullptr;
    CKR(cudaMalloc(&d, npx * 4));
    CKR(cudaMemset(d, 0, npx * 4));
    g_kernel_ms[0] = g_kernel_ms[1] = 0.0;
    g_timed = true;
    int rc = 0;
    for (uint32_t i = 0; i < nblocks && !rc; ++i) {
        const uint64_t a = node_off[i], b = node_off[i + 1];
        g_phase = 0;
        rc = interp_into_field(n2i + 3 * a, sparse + a, (uint32_t)(b - a), blocks[4 * i + 3]);
        g_phase = 1;
        if (!rc) rc = render_block(v, blocks[4 * i + 3], blocks + 4 * i, rects + 4 * i, d);
    }
    g_timed = false;
    cudaFree(d);
    *interp_ms = g_kernel_ms[0];
    *render_ms = g_kernel_ms[1];
    return rc;
}

} // extern "C"

extern "C" {

// Kernel time of the reference's renderKernel<mode> over a block set already in back-to-front order:
// per block its dense field interpolated (not timed; the secondary field too when sparse2 is given), then
// the render launch bracketed by CUDA events.  viewport (host, W*H) is the initial and final image;
// *ms the sum of the render launches' event times.
int ref_cuda_time_render(const void* view, const void* pres, uint32_t nblocks, const uint32_t* blocks,
                         const uint64_t* node_off, const uint16_t* n2i, const float* sparse, const float* sparse2,
                         const int32_t* rects, uint32_t* viewport, double* ms)
{
    const View& v = *static_cast<const View*>(view);
    const size_t npx = (size_t)v.W * v.H;
    uint32_t* d = nullptr;
    CKR(cudaMalloc(&d, npx * 4));
    CKR(cudaMemcpy(d, viewport, npx * 4, cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    CKR(cudaEventCreate(&e0));
    CKR(cudaEventCreate(&e1));
    double total = 0;
    for (uint32_t i = 0; i < nblocks; ++i) {
        const uint64_t a = node_off[i], b = node_off[i + 1];
        const uint32_t depth = blocks[4 * i + 3];
        if (interp_into_field(n2i + 3 * a, sparse + a, (uint32_t)(b - a), depth)) return 1;
        if (sparse2 && interp_into(g_field2, n2i + 3 * a, sparse2 + a, (uint32_t)(b - a), depth)) return 1;
        CKR(cudaDeviceSynchronize());
        CKR(cudaEventRecord(e0, 0));
        if (render_block(v, depth, blocks + 4 * i, rects + 4 * i, d, static_cast<const Pres*>(pres))) return 1;
        CKR(cudaEventRecord(e1, 0));
        CKR(cudaEventSynchronize(e1));
        float t = 0;
        CKR(cudaEventElapsedTime(&t, e0, e1));
        total += t;
    }
    CKR(cudaMemcpy(viewport, d, npx * 4, cudaMemcpyDeviceToHost));
    CKR(cudaEventDestroy(e0));
    CKR(cudaEventDestroy(e1));
    CKR(cudaFree(d));
    *ms = total;
    return 0;
}

// The same render launches timed back to back: every block's field interpolated into a texture of its
// own first (not timed), then the launches captured once into a CUDA graph and the graph replayed `reps`
// times; ms = GPU time per replay (CUDA events around the replays), free of per-launch host overhead.
int ref_cuda_time_render_graph(const void* view, const void* pres, uint32_t nblocks, const uint32_t* blocks,
                               const uint64_t* node_off, const uint16_t* n2i, const float* sparse,
                               const float* sparse2, const int32_t* rects, uint32_t reps, double* ms)
{
    const View& v = *static_cast<const View*>(view);
    const size_t npx = (size_t)v.W * v.H;
    std::vector<Array3> f1(nblocks), f2(sparse2 ? nblocks : 0);
    auto release = [&]() {
        for (auto& a : f1) a.release();
        for (auto& a : f2) a.release();
    };
    for (uint32_t i = 0; i < nblocks; ++i) {
        const uint64_t a = node_off[i], b = node_off[i + 1];
        const uint32_t depth = blocks[4 * i + 3];
        if (interp_into(f1[i], n2i + 3 * a, sparse + a, (uint32_t)(b - a), depth)) return release(), 1;
        if (sparse2 && interp_into(f2[i], n2i + 3 * a, sparse2 + a, (uint32_t)(b - a), depth)) return release(), 1;
    }
    uint32_t* d = nullptr;
    CKR(cudaMalloc(&d, npx * 4));
    CKR(cudaMemset(d, 0, npx * 4));
    CKR(cudaDeviceSynchronize());
    cudaStream_t s = nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CKR(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CKR(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (uint32_t i = 0; i < nblocks && !rc; ++i)
        rc = render_block(v, blocks[4 * i + 3], blocks + 4 * i, rects + 4 * i, d, static_cast<const Pres*>(pres),
                          &f1[i], sparse2 ? &f2[i] : &g_field2, (CUstream)s);
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (rc || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaStreamDestroy(s);
        cudaFree(d);
        release();
        return rc ? rc : fail(std::string("capture: ") + cudaGetErrorString(ce));
    }
    CKR(cudaGraphInstantiate(&ge, g, 0));
    cudaEvent_t e0, e1;
    CKR(cudaEventCreate(&e0));
    CKR(cudaEventCreate(&e1));
    CKR(cudaGraphLaunch(ge, s)); // warm-up
    CKR(cudaEventRecord(e0, s));
    for (uint32_t r = 0; r < reps; ++r) CKR(cudaGraphLaunch(ge, s));
    CKR(cudaEventRecord(e1, s));
    CKR(cudaEventSynchronize(e1));
    float t = 0;
    CKR(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / (reps ? reps : 1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    cudaStreamDestroy(s);
    cudaFree(d);
    release();
    return 0;
}

} // extern "C"
