// Drop-in block renderer for the reference's DenseFieldRenderer_cu
// (include/s3dmm_cuda/DenseFieldRenderer_cu.hpp:32-54, src/s3dmm_cuda/DenseFieldRenderer_cu.cu:222-486),
// backed by the s3r C ABI: the same public interface (setRenderSharedState, clearViewport,
// renderDenseField, timestamps), the same inputs (VsRenderSharedState: field service, field mode and
// parameters, camera transform, viewport size, field of view, quality, colour transfer function) and the
// same output (the block composited into the caller's device viewport, ARGB32).
//
// renderDenseField:
//   * the block's dense field goes into an s3r field texture (interpolated on the GPU from the subtree's
//     sparse values; DeviceField::makeField), the secondary field too in the value-on-isosurface modes;
//   * the transfer function is built with s3r_make_color_transfer (makeColorTransferVector, 512 entries)
//     into an s3r transfer-function texture whenever the control points change;
//   * the camera, cube, view rectangle, thresholds, levels and light follow DenseFieldRenderer_cu.cu:317-445
//     (s3r_camera_from_view, s3r_block_view_rect, s3r_default_light; relative values made absolute over the
//     field's global range in float, isosurface levels sorted and made unique);
//   * the block is ray-cast through the texture unit (s3r_render_block_texture).
// Errors throw std::runtime_error, as the reference's CU_CHECK does.  Compile with -ffp-contract=off so
// that the float set-up rounds as the reference's does.
#pragma once

#include "DenseFieldInterpolatorGb300.hpp"

#include "s3dmm_cuda/DeviceVector.hpp"
#include "s3vs/VsRenderSharedState.hpp"
#include "s3vs/VsWorkerTimestamps.hpp"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

namespace s3dmm {

class DenseFieldRendererGb300
{
public:
    DenseFieldRendererGb300() = default;
    ~DenseFieldRendererGb300()
    {
        s3r_tf_texture_destroy(m_tf);
        cudaFree(m_tfDev);
    }
    DenseFieldRendererGb300(const DenseFieldRendererGb300&) = delete;
    DenseFieldRendererGb300& operator=(const DenseFieldRendererGb300&) = delete;

    void setRenderSharedState(const s3vs::VsRenderSharedState* sharedState)
    {
        m_state = sharedState;
        m_tfPoints.reset();
    }

    const s3vs::VsRenderSharedState* renderSharedState() const { return m_state; }

    // Resizes the viewport to the view and fills it with 0, or with NaN bits for the maximum-intensity mode
    // (DenseFieldRenderer_cu.cu:268-277).
    void clearViewport(DeviceVector<std::uint32_t>& viewport) const
    {
        const auto vs = m_state->input.viewportSize();
        viewport.resize(static_cast<std::size_t>(vs[0]) * vs[1]);
        const std::uint32_t value =
            m_state->input.fieldMode() == s3vs::FieldMode::MaxIntensityProjection ? 0x7fc00000u : 0u;
        s3r_ctx* ctx = gb300::thread_context();
        gb300::check(s3r_clear_viewport(ctx, viewport.data(), vs[0], vs[1], value, nullptr), ctx,
                     "s3r_clear_viewport");
    }

    void renderDenseField(DeviceVector<std::uint32_t>& viewport, unsigned int level,
                          const MultiIndex<3, unsigned int>& index, const std::atomic<bool>& isCancelled)
    {
        m_timestamps = s3vs::BlockTimestamps();
        m_timestamps.blockIndex = index;
        s3r_ctx* ctx = gb300::thread_context();
        const auto& in = m_state->input;
        const auto mode = in.fieldMode();
        const bool secondary =
            mode == s3vs::FieldMode::ValueOnIsosurface || mode == s3vs::FieldMode::ValueOnIsosurfaces;
        auto* fs = m_state->fieldSvc.get();
        const auto subtreeRoot = fs->metadata().blockTree().blockAt(index, level);

        // the block's dense field(s), as textures
        Vec2<dfield_real> range;
        fs->template interpolateWith<DenseFieldInterpolatorGb300<Gb300TextureField&>>(
            range, m_field, m_state->primaryFieldIndex, in.timeFrame(), subtreeRoot, &m_timestamps.afterPrimaryField);
        if (secondary)
            fs->template interpolateWith<DenseFieldInterpolatorGb300<Gb300TextureField&>>(
                range, m_field2, m_state->secondaryFieldIndex, in.timeFrame(), subtreeRoot,
                &m_timestamps.afterSecondaryField);
        makeColorTransferTexture(ctx);
        if (isCancelled) return;

        const auto vs = in.viewportSize();
        const auto fr = fs->fieldRange(m_state->primaryFieldIndex);
        const float lo = static_cast<float>(fr[0]), hi = static_cast<float>(fr[1]);
        auto relToAbs = [&](float r) { return lo + (hi - lo) * r; };

        s3r_view view;
        std::memset(&view, 0, sizeof(view));
        float m[16];
        std::memcpy(m, m_state->cameraTransform.ptr(), sizeof(m));
        gb300::check(s3r_camera_from_view(m, static_cast<float>(in.fovY()), vs[0], vs[1], &view.cam), nullptr,
                     "s3r_camera_from_view");
        view.W = vs[0];
        view.H = vs[1];
        view.level = level;
        view.field_min = lo;
        view.field_max = hi;
        view.quality = static_cast<float>(in.renderQuality());
        view.tf_n = kColorTransferTexSize;
        view.alpha_stop = 2.f;
        view.filter = S3R_FILTER_TEXTURE;

        s3r_presentation pres;
        std::memset(&pres, 0, sizeof(pres));
        pres.mode = static_cast<uint32_t>(mode);
        const auto& fp = in.fieldAllParam();
        switch (mode) {
        case s3vs::FieldMode::Isosurface:
        case s3vs::FieldMode::ValueOnIsosurface:
            view.threshold = relToAbs(static_cast<float>(fp.isosurfaceLevel()));
            break;
        case s3vs::FieldMode::Isosurfaces:
        case s3vs::FieldMode::ValueOnIsosurfaces: {
            view.threshold = 0;
            std::vector<float> lv;
            for (auto r : fp.isosurfaceLevels()) lv.push_back(relToAbs(static_cast<float>(r)));
            std::sort(lv.begin(), lv.end());
            lv.erase(std::unique(lv.begin(), lv.end()), lv.end());
            pres.level_count = static_cast<uint32_t>(std::min<size_t>(lv.size(), S3R_MAX_LEVELS));
            std::copy(lv.begin(), lv.begin() + pres.level_count, pres.levels);
            break;
        }
        default:
            view.threshold = relToAbs(static_cast<float>(fp.threshold()));
            break;
        }
        pres.isosurface_opacity = static_cast<float>(fp.isosurfaceOpacity());
        pres.light_count = 1;
        gb300::check(s3r_default_light(&view, &pres.lights[0]), nullptr, "s3r_default_light");
        if (secondary) {
            const auto sr = fs->fieldRange(m_state->secondaryFieldIndex);
            pres.secondary_min = static_cast<float>(sr[0]);
            pres.secondary_max = static_cast<float>(sr[1]);
        }

        const uint32_t idx[3] = {index[0], index[1], index[2]};
        int32_t rect[4];
        gb300::check(s3r_block_view_rect(&view, idx, rect), nullptr, "s3r_block_view_rect");
        if (rect[2] == 0 || rect[3] == 0) {
            m_timestamps.afterRender = m_timestamps.beforeRender = hires_time();
            return;
        }
        m_timestamps.beforeRender = hires_time();
        gb300::check(s3r_render_block_texture(ctx, &view, &pres, m_field.current(),
                                              secondary ? m_field2.current() : nullptr, idx, rect, m_tf,
                                              viewport.data(), nullptr),
                     ctx, "s3r_render_block_texture");
        m_timestamps.afterRender = hires_time();
    }

    const s3vs::BlockTimestamps& timestamps() const { return m_timestamps; }

private:
    static constexpr uint32_t kColorTransferTexSize = 512; // DenseFieldRenderer_cu.cu:576

    void makeColorTransferTexture(s3r_ctx* ctx)
    {
        const auto& points = m_state->input.fieldAllParam().colorTransferFunction();
        if (m_tfPoints && *m_tfPoints == points && m_tf) return;
        std::vector<double> xs, rgba;
        for (const auto& [x, c] : points) {
            xs.push_back(static_cast<double>(x));
            for (int k = 0; k < 4; ++k) rgba.push_back(static_cast<double>(c[k]));
        }
        std::vector<float> table(4 * kColorTransferTexSize);
        gb300::check(s3r_make_color_transfer(xs.data(), rgba.data(), static_cast<uint32_t>(xs.size()),
                                             kColorTransferTexSize, table.data()),
                     nullptr, "s3r_make_color_transfer");
        if (!m_tfDev)
            gb300::check_cuda(cudaMalloc(reinterpret_cast<void**>(&m_tfDev), table.size() * sizeof(float)),
                              "cudaMalloc");
        gb300::check_cuda(cudaMemcpy(m_tfDev, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice),
                          "cudaMemcpy transfer function");
        if (!m_tf) gb300::check(s3r_tf_texture_create(ctx, kColorTransferTexSize, &m_tf), ctx, "s3r_tf_texture_create");
        gb300::check(s3r_tf_texture_set(ctx, m_tf, m_tfDev, nullptr), ctx, "s3r_tf_texture_set");
        m_tfPoints = std::make_unique<s3vs::ColorTransferFunction>(points);
    }

    const s3vs::VsRenderSharedState* m_state = nullptr;
    Gb300TextureField m_field, m_field2;
    s3r_tf_texture* m_tf = nullptr;
    float* m_tfDev = nullptr;
    std::unique_ptr<s3vs::ColorTransferFunction> m_tfPoints;
    s3vs::BlockTimestamps m_timestamps;
};

} // namespace s3dmm
