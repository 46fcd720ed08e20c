// Drop-in render worker for the reference's s3vs::VsWorkerInterface (include/s3vs/VsWorkerInterface.hpp:38-111),
// the GB300 counterpart of VsWorker_cu (src/s3vs_worker/cuda/VsWorker_cu.cpp): renderScenePart clears the
// viewport, orders the blocks of the subtree set's index box back to front for the camera's eye
// (s3r_b2f_order over the box's world extent, BackToFrontOrder<MacroBlock<3>>), renders them one by one with
// DenseFieldRendererGb300, and returns the part of the viewport holding non-transparent pixels
// (s3r_bound_rect, s3r_crop: getBoundRect and the QImage copy of VsWorker_cu.cpp:51-88, 296-309) as an
// RgbaImagePart of ARGB32 bytes.  A maintainer registers it with the worker factory as VsWorker_cu is
// registered (VsWorker_cu.cpp:41-45), e.g. SILVER_BULLETS_FACTORY_REGISTER_TYPE(s3dmm::VsWorkerGb300, "GB300").
#pragma once

#include "DenseFieldRendererGb300.hpp"

#include "s3vs/VsWorkerInterface.hpp"

#include <vector>

namespace s3dmm {

class VsWorkerGb300 : public s3vs::VsWorkerInterface
{
public:
    // The CUDA worker selects its GPU from the thread id (selectGpu); so does this one.
    void initialize(const std::string& /*shaderPath*/, bool /*logInfo*/, const std::string& /*logFileName*/,
                    size_t threadId) override
    {
        int n = 0;
        gb300::check_cuda(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (n > 0) gb300::check_cuda(cudaSetDevice(static_cast<int>(threadId % static_cast<size_t>(n))), "cudaSetDevice");
    }

    void setRenderSharedState(const s3vs::VsRenderSharedState* sharedState) override
    {
        m_state = sharedState;
        m_renderer.setRenderSharedState(sharedState);
    }

    const s3vs::VsRenderSharedState* renderSharedState() const override { return m_state; }

    void updateState(unsigned int /*flags*/) override {} // every renderScenePart reads the shared state afresh

    s3vs::RgbaImagePart renderScenePart(const s3vs::SubtreeSetDescription& subtrees,
                                        const silver_bullets::sync::CancelController::Checker& isCancelled) override
    {
        s3vs::RgbaImagePart part;
        if (subtrees.indexBox.empty()) return part;
        s3r_ctx* ctx = gb300::thread_context();
        m_renderer.clearViewport(m_viewport);
        const auto vs = m_state->input.viewportSize();

        // back-to-front order of the box's blocks for the camera's eye
        const auto& box = subtrees.indexBox;
        const uint32_t bmin[3] = {box.min()[0], box.min()[1], box.min()[2]};
        const uint32_t bmax[3] = {box.max()[0], box.max()[1], box.max()[2]};
        double cmin[3], cmax[3];
        gb300::check(s3r_index_box_world(subtrees.level, bmin, bmax, cmin, cmax), nullptr, "s3r_index_box_world");
        float m[16];
        std::memcpy(m, m_state->cameraTransform.ptr(), sizeof(m));
        s3r_camera cam;
        gb300::check(s3r_camera_from_view(m, static_cast<float>(m_state->input.fovY()), vs[0], vs[1], &cam), nullptr,
                     "s3r_camera_from_view");
        const double eye[3] = {cam.eye[0], cam.eye[1], cam.eye[2]};
        uint32_t count = 0;
        gb300::check(s3r_b2f_order(bmin, bmax, cmin, cmax, eye, nullptr, 0, &count), nullptr, "s3r_b2f_order");
        m_order.resize(3 * static_cast<size_t>(count));
        gb300::check(s3r_b2f_order(bmin, bmax, cmin, cmax, eye, m_order.data(), count, &count), nullptr,
                     "s3r_b2f_order");

        std::atomic<bool> cancelled(false);
        for (uint32_t i = 0; i < count; ++i) {
            if (isCancelled) {
                cancelled = true;
                break;
            }
            m_renderer.renderDenseField(m_viewport, subtrees.level,
                                        MultiIndex<3, unsigned int>{m_order[3 * i], m_order[3 * i + 1],
                                                                    m_order[3 * i + 2]},
                                        cancelled);
        }
        if (cancelled) return part;

        // the part of the viewport holding non-transparent pixels
        int32_t rect[4];
        gb300::check(s3r_bound_rect(ctx, m_viewport.data(), vs[0], vs[1], rect, nullptr), ctx, "s3r_bound_rect");
        if (rect[2] == 0 || rect[3] == 0) return part;
        m_crop.resize(static_cast<size_t>(rect[2]) * rect[3]);
        gb300::check(s3r_crop(ctx, m_viewport.data(), vs[0], rect, m_crop.data(), nullptr), ctx, "s3r_crop");
        part.image.bits.resize(4 * m_crop.size());
        m_crop.download(reinterpret_cast<std::uint32_t*>(part.image.bits.data()));
        part.image.size = s3vs::Vec2i{rect[2], rect[3]};
        part.origin = s3vs::Vec2i{rect[0], rect[1]};
        return part;
    }

#ifdef S3DMM_ENABLE_WORKER_TIME_ESTIMATION
    const std::vector<s3vs::VsWorkerTimestamps>& timestamps() const override { return m_timestamps; }
    void clearTimestamps() override { m_timestamps.clear(); }
    void enableNvProf() override {}

private:
    std::vector<s3vs::VsWorkerTimestamps> m_timestamps;
#endif // S3DMM_ENABLE_WORKER_TIME_ESTIMATION

private:
    const s3vs::VsRenderSharedState* m_state = nullptr;
    DenseFieldRendererGb300 m_renderer;
    DeviceVector<std::uint32_t> m_viewport;
    DeviceVector<std::uint32_t> m_crop;
    std::vector<uint32_t> m_order;
};

} // namespace s3dmm
