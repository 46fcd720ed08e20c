// Test infrastructure only: runs the host side of the reference's own DenseFieldRenderer_cu
// (src/s3dmm_cuda/DenseFieldRenderer_cu.cu:279-486 -- cube, eye, view rectangle, presentation and light
// set-up of renderDenseField) on the CPU, linked against oracle/cuda_stub.cpp instead of the CUDA
// runtime, over a dataset in the reference's format.  For every block it returns the RenderKernelParam
// renderDenseField launches renderKernel<mode> with (or that no launch happened: an empty view
// rectangle).  Built from the staged reference sources by oracle/Makefile (target refsetup) into
// oracle/_ref/libs3r_refsetup.so; nothing in the product links or loads it.
#include "s3dmm_cuda/DenseFieldRenderer_cu.hpp"

#include "RenderKernelParam.hpp"

#include <atomic>
#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

namespace {

std::string g_err;
bool g_captured = false;
s3dmm::RenderKernelParam g_param;

} // namespace

// The stub runtime hands every launch here: keep renderKernel<mode>'s parameter block.
extern "C" void ref_stub_on_launch(const char* device_name, dim3, dim3, void** args)
{
    if (std::strstr(device_name, "renderKernel")) {
        std::memcpy(&g_param, args[0], sizeof(g_param));
        g_captured = true;
    }
}

extern "C" {

const char* ref_setup_error(void) { return g_err.c_str(); }

// Words per block record written by ref_setup_params.
uint32_t ref_setup_record_words(void) { return 88; }

// base: dataset base name (the reference's BlockTreeFieldService argument); view: the camera transform
// (world -> eye, column-major 4x4, VsRenderSharedState::cameraTransform); fovy: degrees; mode:
// s3vs::FieldMode; threshold / iso_level: relative values (fieldAllParam().threshold(), isosurfaceLevel());
// levels: relative isosurface levels; blocks: n x {x, y, z} at `level`.  out: n records of 88 32-bit words:
// [0..3] cube center, halfSize; [4] level; [5..16] eye pos, e1, e2, n; [17..19] w, h, pixelSize;
// [20..23] view x, y, W, H; [24..26] threshold, isosurfaceOpacity, quality; [27] texDepth;
// [28..29] field min, max; [30] light count; [31..33] light 0 position; [34] levelCount; [35..84] levels;
// [85] launched (0: empty view rectangle, no launch).
int ref_setup_params(const char* base, const float view[16], float fovy, uint32_t W, uint32_t H, uint32_t mode,
                     float threshold, float iso_level, float iso_opacity, const float* levels, uint32_t nlevels,
                     float quality, uint32_t level, uint32_t n, const uint32_t* blocks, uint32_t* out)
{
    try {
        s3vs::VsRenderSharedState st;
        st.fieldSvc = std::make_shared<s3dmm::BlockTreeFieldService<3>>(base);
        st.primaryFieldIndex = 0;
        st.secondaryFieldIndex = 0;
        auto& in = st.input;
        in.setFieldMode(static_cast<s3vs::FieldMode>(mode));
        in.setViewportSize(s3vs::Vec2i{static_cast<int>(W), static_cast<int>(H)});
        in.setFovY(fovy);
        in.setRenderQuality(quality);
        auto& fp = in.fieldAllParam();
        fp.setThreshold(threshold);
        fp.setIsosurfaceLevel(iso_level);
        fp.setIsosurfaceOpacity(iso_opacity);
        fp.setIsosurfaceLevels(std::vector<s3dmm::real_type>(levels, levels + nlevels));
        s3vs::ColorTransferFunction ctf;
        ctf[0] = s3vs::Vec4r{0, 0, 0, 0};
        ctf[1] = s3vs::Vec4r{1, 1, 1, 1};
        fp.setColorTransferFunction(ctf);
        for (int c = 0; c < 4; ++c)
            for (int r = 0; r < 4; ++r) st.cameraTransform.e[c][r] = view[4 * c + r];
        s3dmm::DenseFieldRenderer_cu renderer;
        renderer.setRenderSharedState(&st);
        s3dmm::DeviceVector<std::uint32_t> viewport(static_cast<std::size_t>(W) * H);
        std::atomic<bool> cancelled(false);
        for (uint32_t i = 0; i < n; ++i) {
            g_captured = false;
            renderer.renderDenseField(viewport, level,
                                      s3dmm::MultiIndex<3, unsigned int>{blocks[3 * i], blocks[3 * i + 1],
                                                                         blocks[3 * i + 2]},
                                      cancelled);
            uint32_t* o = out + (size_t)88 * i;
            std::memset(o, 0, 88 * 4);
            float* f = reinterpret_cast<float*>(o);
            const auto& p = g_param;
            o[85] = g_captured ? 1u : 0u;
            if (!g_captured) continue;
            f[0] = p.cube.center.x;
            f[1] = p.cube.center.y;
            f[2] = p.cube.center.z;
            f[3] = p.cube.halfSize;
            o[4] = p.cube.level;
            const float3 ev[4] = {p.eye.pos, p.eye.e1, p.eye.e2, p.eye.n};
            for (int k = 0; k < 4; ++k) {
                f[5 + 3 * k] = ev[k].x;
                f[6 + 3 * k] = ev[k].y;
                f[7 + 3 * k] = ev[k].z;
            }
            f[17] = p.eye.w;
            f[18] = p.eye.h;
            f[19] = p.eye.pixelSize;
            o[20] = p.view.x;
            o[21] = p.view.y;
            o[22] = p.view.W;
            o[23] = p.view.H;
            f[24] = p.presentation.threshold;
            f[25] = p.presentation.isosurfaceOpacity;
            f[26] = p.presentation.quality;
            o[27] = p.primaryField.texDepth;
            f[28] = p.primaryField.minValue;
            f[29] = p.primaryField.maxValue;
            o[30] = p.lights.sourceCount;
            f[31] = p.lights.sources[0].pos.x;
            f[32] = p.lights.sources[0].pos.y;
            f[33] = p.lights.sources[0].pos.z;
            o[34] = p.presentation.levelCount;
            for (int k = 0; k < 50; ++k) f[35 + k] = p.presentation.levels[k];
        }
        renderer.setRenderSharedState(nullptr);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

} // extern "C"
