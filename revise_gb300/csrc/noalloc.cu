// Allocation-free dense interpolation: s3r_interp_dense_noalloc.
//
// s3r_interp_dense needs a (2^d+1)^3 float scratch grid, which its context
// allocates with cudaMalloc when it first sees a depth.  Some callers cannot
// let a library call cudaMalloc: host applications that own all device memory
// through their own pool allocator or reserve it up front (a driver
// allocation then fails or competes with the pool), and render loops that
// must not stall, since cudaMalloc/cudaFree synchronize the whole device.
// This entry point serves them: it takes no context, allocates nothing, and
// uses as scratch a file-scope __device__ array of fixed size, held by every
// GPU that loads the library until the process exits.
//
// Limits and sharing:
//   * depth <= S3R_NOALLOC_MAX_DEPTH (7): the scratch holds 129^3 floats (8.6 MB);
//     deeper subtrees are rejected with S3R_ERR_INVALID.
//   * All calls on a device share the one scratch array.  Each call re-fills the
//     part it uses with NaN before scattering the nodes, so no state leaks from
//     the previous call, but calls that overlap on the GPU (different streams,
//     or host threads without ordering between them) race on the scratch and
//     produce wrong grids: order them on one stream or serialize them.
//   * The first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current and caches it; make that
//     first call before any stream capture.  The cache is keyed on the unique id
//     of the CUDA context current at the call (cuCtxGetId), so that a context
//     made after cudaDeviceReset, or a caller's own driver-API context on the
//     same device, gets its own lookup instead of a stale address.
#include "s3r_internal.h"

#include <mutex>

namespace s3r {
namespace {

constexpr uint32_t kNoAllocEdge = (1u << S3R_NOALLOC_MAX_DEPTH) + 1u;
constexpr size_t kNoAllocFloats = (size_t)kNoAllocEdge * kNoAllocEdge * kNoAllocEdge;

// The scratch grid.  In host code this name is only a host-side stand-in: its
// device address comes from cudaGetSymbolAddress, per device.
static __device__ __align__(256) float g_noalloc_grid[kNoAllocFloats];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct GridAddress {
    unsigned long long context_id = 0; // 0: none looked up yet
    float* grid = nullptr;
};
GridAddress g_grid_on_device[kMaxDevices];

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (no link against the driver
// library).  CUresult is an int-sized enum; 0 is success.
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_entry_points_looked_up = false;

// The unique id of the context current on this thread, 0 when there is none or it cannot be told.
unsigned long long current_context_id()
{
    if (!g_entry_points_looked_up) {
        g_entry_points_looked_up = true;
        cudaDriverEntryPointQueryResult q1, q2;
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
    }
    if (!g_ctx_get_current || !g_ctx_get_id) return 0;
    void* c = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&c) != 0 || !c || g_ctx_get_id(c, &id) != 0) return 0;
    return id;
}

} // namespace
} // namespace s3r

extern "C" int s3r_interp_dense_noalloc(const uint16_t* n2i_xyz, const float* sparse, uint32_t n, uint32_t depth,
                                        float* dense, void* stream)
{
    using namespace s3r;
    if (depth > S3R_NOALLOC_MAX_DEPTH)
        return record_error(S3R_ERR_INVALID, "s3r_interp_dense_noalloc: depth exceeds S3R_NOALLOC_MAX_DEPTH (7), "
                                             "the size of its fixed 8.6 MB scratch grid");
    if (!dense || (n > 0 && (!n2i_xyz || !sparse)))
        return record_error(S3R_ERR_INVALID, "s3r_interp_dense_noalloc: null pointer");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return record_cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return record_error(S3R_ERR_UNSUPPORTED, "s3r_interp_dense_noalloc: device ordinal beyond 63");
    float* grid = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        GridAddress& ga = g_grid_on_device[dev];
        // the context the call runs in; before the runtime's first use of the device there is none yet,
        // and the lookup below makes the device's primary context
        unsigned long long id = current_context_id();
        if (!ga.grid || id == 0 || id != ga.context_id) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_grid);
            if (e != cudaSuccess) return record_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_grid)");
            if (id == 0) id = current_context_id();
            ga.grid = static_cast<float*>(p);
            ga.context_id = id; // 0 (ids unavailable): looked up again on every call
        }
        grid = ga.grid;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t edge = (1ull << depth) + 1ull;
    if ((e = launch_fill_f32(grid, edge * edge * edge, __builtin_nanf(""), s)) != cudaSuccess)
        return record_cuda_error(e, "fill");
    if ((e = launch_scatter_nodes(grid, depth, n2i_xyz, sparse, n, s)) != cudaSuccess)
        return record_cuda_error(e, "scatter");
    if ((e = launch_interp_grid(grid, depth, dense, s, nullptr)) != cudaSuccess)
        return record_cuda_error(e, "interpolate");
    return S3R_OK;
}
