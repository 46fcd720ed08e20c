// Image-part kernels for sm_103a: crop rectangle of the non-transparent
// pixels (getBoundRect, src/s3vs_worker/cuda/VsWorker_cu.cpp:51-88), the crop
// itself, and compositing of ARGB32 image parts with blendImagePart's integer
// src-over-dst arithmetic (src/s3vs_lib/BlendImagePart.hpp:61-145), one thread
// per destination pixel walking the parts in order.
#include "s3r_internal.h"

namespace s3r {
namespace {

__global__ void bound_rect_kernel(const uint32_t* __restrict__ img, uint32_t W, uint32_t H, int32_t* rect)
{
    // rect: {minX, minY, maxX, maxY}, pre-set to {W, H, -1, -1}
    int32_t mnx = INT32_MAX, mny = INT32_MAX, mxx = -1, mxy = -1;
    const uint64_t n = (uint64_t)W * H;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (img[i] >> 24) {
            const int32_t x = (int32_t)(i % W), y = (int32_t)(i / W);
            mnx = min(mnx, x);
            mny = min(mny, y);
            mxx = max(mxx, x);
            mxy = max(mxy, y);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxx = max(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = max(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    if ((threadIdx.x & 31) == 0 && mxx >= 0) {
        atomicMin(&rect[0], mnx);
        atomicMin(&rect[1], mny);
        atomicMax(&rect[2], mxx);
        atomicMax(&rect[3], mxy);
    }
}

__global__ void crop_kernel(const uint32_t* __restrict__ img, uint32_t W, int32_t x0, int32_t y0, int32_t w, int32_t h,
                            uint32_t* __restrict__ dst)
{
    const uint64_t n = (uint64_t)w * h;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t x = (int32_t)(i % w), y = (int32_t)(i / w);
        dst[i] = img[(uint64_t)(y0 + y) * W + (x0 + x)];
    }
}

__device__ __forceinline__ uint32_t blend_px(uint32_t d, uint32_t s)
{
    const uint32_t as = s >> 24;
    if (as == 0) return d;
    if (as == 255u) return s;
    const uint32_t ad = d >> 24;
    if (ad == 0) return s;
    const uint32_t a = as + ad * (255u - as) / 255u;
    uint32_t out = (a & 0xffu) << 24;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        const uint32_t cs = (s >> (8 * b)) & 0xffu, cd = (d >> (8 * b)) & 0xffu;
        out |= (((cs * as + cd * (a - as)) / a) & 0xffu) << (8 * b);
    }
    return out;
}

__global__ void compose_kernel(const s3r_image_part* __restrict__ parts, uint32_t nparts, int32_t just_copy_first,
                               uint32_t* __restrict__ dst, int32_t dw, int32_t dh, int32_t offx, int32_t offy)
{
    const int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    const int32_t gx = x + offx, gy = y + offy; // image-part coordinates
    uint32_t d = dst[(uint64_t)y * dw + x];
    bool touched = false;
    for (uint32_t p = 0; p < nparts; ++p) {
        const s3r_image_part pt = parts[p];
        const int32_t sx = gx - pt.origin[0], sy = gy - pt.origin[1];
        if (sx < 0 || sy < 0 || sx >= pt.size[0] || sy >= pt.size[1]) continue;
        const uint32_t s = pt.pixels[(uint64_t)sy * pt.size[0] + sx];
        d = (p == 0 && just_copy_first) ? s : blend_px(d, s);
        touched = true;
    }
    if (touched) dst[(uint64_t)y * dw + x] = d;
}

} // namespace

cudaError_t launch_bound_rect(const uint32_t* img, uint32_t W, uint32_t H, int32_t* rect_dev, cudaStream_t s)
{
    const uint64_t n = (uint64_t)W * H;
    uint32_t ctas = (uint32_t)((n + 255) / 256);
    if (ctas > 152 * 16) ctas = 152 * 16;
    if (ctas == 0) ctas = 1;
    bound_rect_kernel<<<ctas, 256, 0, s>>>(img, W, H, rect_dev);
    return cudaGetLastError();
}

cudaError_t launch_crop(const uint32_t* img, uint32_t W, const int32_t rect[4], uint32_t* dst, cudaStream_t s)
{
    const uint64_t n = (uint64_t)rect[2] * rect[3];
    if (n == 0) return cudaSuccess;
    uint32_t ctas = (uint32_t)((n + 255) / 256);
    if (ctas > 152 * 16) ctas = 152 * 16;
    crop_kernel<<<ctas, 256, 0, s>>>(img, W, rect[0], rect[1], rect[2], rect[3], dst);
    return cudaGetLastError();
}

cudaError_t launch_compose(const s3r_image_part* parts_dev, uint32_t nparts, int32_t just_copy_first, uint32_t* dst,
                           int32_t dw, int32_t dh, int32_t offx, int32_t offy, cudaStream_t s)
{
    if (dw <= 0 || dh <= 0 || nparts == 0) return cudaSuccess;
    dim3 block(32, 8);
    dim3 grid((dw + 31) / 32, (dh + 7) / 8);
    compose_kernel<<<grid, block, 0, s>>>(parts_dev, nparts, just_copy_first, dst, dw, dh, offx, offy);
    return cudaGetLastError();
}

} // namespace s3r
