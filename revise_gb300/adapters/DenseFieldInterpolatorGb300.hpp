// Drop-in dense-field generator for the reference's plug-in point
// BlockTreeFieldService<3>::interpolateWith<DenseInterpolator>
// (include/s3dmm/BlockTreeFieldService.hpp:118-145), backed by the s3r C ABI.
//
// It models the same concept as DenseFieldInterpolator<3>
// (include/s3dmm/DenseFieldInterpolator.hpp:138-196) and
// DenseFieldInterpolatorTpl_cu_3 (include/s3dmm_cuda/DenseFieldInterpolatorTpl_cu_3.hpp:40-118):
// constructed from a BlockTreeFieldProvider<3>, it reads a subtree's sparse
// values (fieldValues), and interpolates them into the dense container.
// Three containers are accepted:
//   std::vector<dfield_real>&  host grid, the contract of DenseFieldInterpolator<3>
//                              (values copied back after the GPU computes them);
//   Gb300DenseField&           device grid that stays in HBM;
//   Gb300TextureField&         the grid as a 3-D texture (one per depth, kept), sampled by the texture
//                              unit as the reference's renderer samples its Device3DArray
//                              (the renderer adapter, DenseFieldRendererGb300.hpp).
// Errors throw std::runtime_error, as the reference's CU_CHECK does.
#pragma once

#include "s3dmm/BlockTreeFieldProvider.hpp"
#include "s3dmm/DenseFieldInterpolatorTimers.hpp"
#include "s3dmm/FieldTimestamps.hpp"
#include "s3dmm/Metadata.hpp"

#include "s3r.h"

#include <cuda_runtime_api.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace s3dmm {

namespace gb300 {

inline void check(int rc, const s3r_ctx* ctx, const char* what)
{
    if (rc != S3R_OK)
        throw std::runtime_error(std::string(what) + ": " + s3r_last_error(ctx));
}

inline void check_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess)
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// One s3r context per host thread and device (the reference keeps one renderer per worker thread).
inline s3r_ctx* thread_context()
{
    struct Holder {
        s3r_ctx* ctx = nullptr;
        int device = -1;
        ~Holder() { s3r_ctx_destroy(ctx); }
    };
    thread_local Holder h;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (!h.ctx || h.device != dev) {
        s3r_ctx_destroy(h.ctx);
        h.ctx = nullptr;
        check(s3r_ctx_create(dev, &h.ctx), nullptr, "s3r_ctx_create");
        h.device = dev;
    }
    return h.ctx;
}

// Growable device buffer.
template <class T> struct DeviceBuffer {
    T* data = nullptr;
    size_t capacity = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() { cudaFree(data); }
    void reserve(size_t n)
    {
        if (n <= capacity) return;
        cudaFree(data);
        data = nullptr;
        capacity = 0;
        check_cuda(cudaMalloc(reinterpret_cast<void**>(&data), n * sizeof(T)), "cudaMalloc");
        capacity = n;
    }
};

} // namespace gb300

// A dense grid resident in device memory: (2^depth+1)^3 floats, x fastest.
struct Gb300DenseField {
    gb300::DeviceBuffer<float> buf;
    unsigned int depth = 0;
    size_t size() const { return size_t((1u << depth) + 1) * ((1u << depth) + 1) * ((1u << depth) + 1); }
    const float* data() const { return buf.data; }
};

// A dense grid held as an s3r field texture: one texture per subtree depth, created on first use and kept.
struct Gb300TextureField {
    s3r_texture* tex[S3R_MAX_DEPTH + 1] = {};
    unsigned int depth = 0;
    Gb300TextureField() = default;
    Gb300TextureField(const Gb300TextureField&) = delete;
    Gb300TextureField& operator=(const Gb300TextureField&) = delete;
    ~Gb300TextureField()
    {
        for (s3r_texture* t : tex) s3r_texture_destroy(t);
    }
    s3r_texture* at(s3r_ctx* ctx, unsigned int d)
    {
        if (!tex[d]) gb300::check(s3r_texture_create(ctx, d, &tex[d]), ctx, "s3r_texture_create");
        return tex[d];
    }
    const s3r_texture* current() const { return tex[depth]; }
};

template <class ContainerRef>
class DenseFieldInterpolatorGb300
{
public:
    static constexpr const unsigned int N = 3;
    using BlockId = typename BlockTree<N>::BlockId;
    using BT = typename Metadata<N>::BT;
    using dense_field_container_ref = ContainerRef;
    using Timers = DenseFieldInterpolatorTimers;

    explicit DenseFieldInterpolatorGb300(BlockTreeFieldProvider<N>& fp) : m_fp(fp) {}

    std::shared_ptr<Timers> timers() const { return m_timers; }
    void setTimers(const std::shared_ptr<Timers>& timers) { m_timers = timers; }
    const FieldTimestamps& timestamps() const { return m_timestamps; }

    void interpolate(Vec2<real_type>& fieldRange, dense_field_container_ref dense, const BlockId& subtreeRoot)
    {
        auto nodes = m_fp.metadata().blockTreeNodes(subtreeRoot);
        interpolate(fieldRange, dense, nodes);
    }

    void interpolate(Vec2<real_type>& fieldRange, dense_field_container_ref dense,
                     const BlockTreeNodes<N, BT>& subtreeNodes)
    {
        m_fp.fieldValues(fieldRange, m_sparse, subtreeNodes);
        m_timestamps.afterReadSparseField = hires_time();
        if (m_timers) ++m_timers.get()->invocationCount;
        interpolate(dense, m_sparse, subtreeNodes);
        m_timestamps.afterComputeDenseField = hires_time();
    }

    // The static form of the reference's generators: dense <- sparse over subtreeNodes.
    void interpolate(dense_field_container_ref dense, const std::vector<real_type>& sparse,
                     const BlockTreeNodes<N, BT>& subtreeNodes)
    {
        s3r_ctx* ctx = gb300::thread_context();
        const auto& n2i = subtreeNodes.data().n2i;
        const unsigned int depth = subtreeNodes.maxDepth();
        const size_t n = n2i.size();
        static_assert(sizeof(n2i[0]) == 3 * sizeof(uint16_t), "BlockTreeNodes n2i must be 3 x uint16");
        m_n2i.reserve(3 * n + 1);
        m_values.reserve(n + 1);
        m_host.resize(n);
        for (size_t i = 0; i < n; ++i) m_host[i] = static_cast<float>(sparse[i]);
        gb300::check_cuda(cudaMemcpy(m_n2i.data, n2i.data(), 6 * n, cudaMemcpyHostToDevice), "cudaMemcpy n2i");
        gb300::check_cuda(cudaMemcpy(m_values.data, m_host.data(), 4 * n, cudaMemcpyHostToDevice),
                          "cudaMemcpy values");
        const size_t e = (size_t(1) << depth) + 1;
        if constexpr (std::is_same_v<std::decay_t<ContainerRef>, Gb300TextureField>) {
            if (depth > S3R_MAX_DEPTH) throw std::runtime_error("subtree depth exceeds S3R_MAX_DEPTH");
            dense.depth = depth;
            gb300::check(s3r_interp_dense_texture(ctx, m_n2i.data, m_values.data, uint32_t(n), dense.at(ctx, depth),
                                                  nullptr),
                         ctx, "s3r_interp_dense_texture");
        } else if constexpr (std::is_same_v<std::decay_t<ContainerRef>, Gb300DenseField>) {
            dense.buf.reserve(e * e * e);
            dense.depth = depth;
            gb300::check(s3r_interp_dense(ctx, m_n2i.data, m_values.data, uint32_t(n), depth, dense.buf.data, nullptr),
                         ctx, "s3r_interp_dense");
        } else {
            m_dense.reserve(e * e * e);
            gb300::check(s3r_interp_dense(ctx, m_n2i.data, m_values.data, uint32_t(n), depth, m_dense.data, nullptr),
                         ctx, "s3r_interp_dense");
            dense.resize(e * e * e);
            gb300::check_cuda(cudaMemcpy(dense.data(), m_dense.data, 4 * e * e * e, cudaMemcpyDeviceToHost),
                              "cudaMemcpy dense");
        }
    }

private:
    BlockTreeFieldProvider<N>& m_fp;
    std::vector<real_type> m_sparse;
    std::vector<float> m_host;
    gb300::DeviceBuffer<uint16_t> m_n2i;
    gb300::DeviceBuffer<float> m_values;
    gb300::DeviceBuffer<float> m_dense;
    std::shared_ptr<Timers> m_timers;
    FieldTimestamps m_timestamps;
};

} // namespace s3dmm
