// Test infrastructure only: a stand-in for the CUDA runtime, linked instead of it into
// oracle/_ref/libs3r_refsetup.so so that the host side of the reference's renderer runs on a machine
// without a GPU.  Device allocations live in host memory (so the reference's copies move real bytes),
// arrays, textures and surfaces are opaque handles, no kernel runs, and every kernel launch is handed
// to ref_stub_on_launch() with its registered device name, launch shape and argument pointers.  Only
// the calls the reference's render and interpolation host code make are provided.
#include <cuda_runtime_api.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

// Called for each launch (defined by the harness).
extern "C" void ref_stub_on_launch(const char* device_name, dim3 grid, dim3 block, void** args);

namespace {

std::map<const void*, std::string>& kernels()
{
    static std::map<const void*, std::string> m;
    return m;
}

struct CallConfig {
    dim3 grid, block;
    size_t smem = 0;
    void* stream = nullptr;
} g_config;

cudaError_t g_last = cudaSuccess;
unsigned long long g_handles = 0;

struct FakeArray {
    cudaChannelFormatDesc desc;
    cudaExtent extent;
};

} // namespace

extern "C" {

// ---- module registration (the host code nvcc emits for every translation unit with kernels)
void** __cudaRegisterFatBinary(void*)
{
    static void* handle = nullptr;
    return &handle;
}
void __cudaRegisterFatBinaryEnd(void**) {}
void __cudaUnregisterFatBinary(void**) {}
void __cudaRegisterFunction(void**, const char* hostFun, char*, const char* deviceName, int, uint3*, uint3*, dim3*,
                            dim3*, int*)
{
    kernels()[hostFun] = deviceName;
}
void __cudaRegisterVar(void**, char*, char*, const char*, int, size_t, int, int) {}
void __cudaRegisterManagedVar(void**, void**, char*, const char*, int, size_t, int, int) {}
char __cudaInitModule(void**) { return 0; }

unsigned __cudaPushCallConfiguration(dim3 grid, dim3 block, size_t smem, struct CUstream_st* stream)
{
    g_config = CallConfig{grid, block, smem, stream};
    return 0;
}
cudaError_t __cudaPopCallConfiguration(dim3* grid, dim3* block, size_t* smem, void* stream)
{
    *grid = g_config.grid;
    *block = g_config.block;
    *smem = g_config.smem;
    *static_cast<void**>(stream) = g_config.stream;
    return cudaSuccess;
}

cudaError_t CUDARTAPI cudaLaunchKernel(const void* func, dim3 grid, dim3 block, void** args, size_t, cudaStream_t)
{
    auto it = kernels().find(func);
    ref_stub_on_launch(it == kernels().end() ? "" : it->second.c_str(), grid, block, args);
    return cudaSuccess;
}

// the launch path nvcc emits for <<<>>> (kernel handle = the host stub's address) and thrust's
cudaError_t CUDARTAPI __cudaGetKernel(cudaKernel_t* k, const void* fun)
{
    *k = reinterpret_cast<cudaKernel_t>(const_cast<void*>(fun));
    return cudaSuccess;
}
cudaError_t CUDARTAPI __cudaLaunchKernel(cudaKernel_t k, dim3 grid, dim3 block, void** args, size_t smem,
                                         cudaStream_t stream)
{
    return cudaLaunchKernel(reinterpret_cast<const void*>(k), grid, block, args, smem, stream);
}
cudaError_t CUDARTAPI cudaLaunchKernelExC(const cudaLaunchConfig_t* config, const void* func, void** args)
{
    return cudaLaunchKernel(func, config->gridDim, config->blockDim, args, config->dynamicSmemBytes, config->stream);
}

// ---- errors, devices, streams
cudaError_t CUDARTAPI cudaGetLastError(void)
{
    cudaError_t e = g_last;
    g_last = cudaSuccess;
    return e;
}
cudaError_t CUDARTAPI cudaPeekAtLastError(void) { return g_last; }
const char* CUDARTAPI cudaGetErrorString(cudaError_t) { return "cuda stub"; }
const char* CUDARTAPI cudaGetErrorName(cudaError_t) { return "cudaStub"; }
cudaError_t CUDARTAPI cudaGetDevice(int* d)
{
    *d = 0;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaSetDevice(int) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaGetDeviceCount(int* n)
{
    *n = 1;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaDeviceGetAttribute(int* v, cudaDeviceAttr attr, int)
{
    switch (attr) {
    case cudaDevAttrMaxSharedMemoryPerBlock: *v = 48 * 1024; break;
    case cudaDevAttrMultiProcessorCount: *v = 152; break;
    case cudaDevAttrMaxThreadsPerBlock: *v = 1024; break;
    case cudaDevAttrComputeCapabilityMajor: *v = 10; break;
    case cudaDevAttrComputeCapabilityMinor: *v = 3; break;
    case cudaDevAttrWarpSize: *v = 32; break;
    default: *v = 0; break;
    }
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaFuncGetAttributes(cudaFuncAttributes* a, const void*)
{
    std::memset(a, 0, sizeof(*a));
    a->maxThreadsPerBlock = 1024;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaOccupancyMaxActiveBlocksPerMultiprocessorWithFlags(int* n, const void*, int, size_t,
                                                                             unsigned int)
{
    *n = 1;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaOccupancyMaxActiveBlocksPerMultiprocessor(int* n, const void*, int, size_t)
{
    *n = 1;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaStreamIsCapturing(cudaStream_t, cudaStreamCaptureStatus* s)
{
    *s = cudaStreamCaptureStatusNone;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaProfilerStart(void) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaProfilerStop(void) { return cudaSuccess; }

// ---- memory: device pointers are host allocations
cudaError_t CUDARTAPI cudaMalloc(void** p, size_t n)
{
    *p = std::calloc(n ? n : 1, 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t CUDARTAPI cudaFree(void* p)
{
    std::free(p);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind)
{
    if (n) std::memmove(d, s, n);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t)
{
    if (n) std::memmove(d, s, n);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemset(void* p, int v, size_t n)
{
    std::memset(p, v, n);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemsetAsync(void* p, int v, size_t n, cudaStream_t)
{
    std::memset(p, v, n);
    return cudaSuccess;
}

// ---- arrays, textures, surfaces: handles only (their contents are never read on this path)
cudaError_t CUDARTAPI cudaMalloc3DArray(cudaArray_t* a, const cudaChannelFormatDesc* d, cudaExtent e, unsigned int)
{
    *a = reinterpret_cast<cudaArray_t>(new FakeArray{*d, e});
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMallocArray(cudaArray_t* a, const cudaChannelFormatDesc* d, size_t w, size_t h,
                                      unsigned int)
{
    cudaExtent e;
    e.width = w;
    e.height = h;
    e.depth = 0;
    *a = reinterpret_cast<cudaArray_t>(new FakeArray{*d, e});
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaFreeArray(cudaArray_t a)
{
    delete reinterpret_cast<FakeArray*>(a);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemcpy3D(const cudaMemcpy3DParms*) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaMemcpy2DToArray(cudaArray_t, size_t, size_t, const void*, size_t, size_t, size_t,
                                          cudaMemcpyKind)
{
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemcpy2DFromArray(void*, size_t, cudaArray_const_t, size_t, size_t, size_t, size_t,
                                            cudaMemcpyKind)
{
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaCreateTextureObject(cudaTextureObject_t* t, const cudaResourceDesc*,
                                              const cudaTextureDesc*, const cudaResourceViewDesc*)
{
    *t = ++g_handles;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaDestroyTextureObject(cudaTextureObject_t) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaCreateSurfaceObject(cudaSurfaceObject_t* s, const cudaResourceDesc*)
{
    *s = ++g_handles;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaDestroySurfaceObject(cudaSurfaceObject_t) { return cudaSuccess; }
cudaChannelFormatDesc CUDARTAPI cudaCreateChannelDesc(int x, int y, int z, int w, cudaChannelFormatKind f)
{
    cudaChannelFormatDesc d;
    d.x = x;
    d.y = y;
    d.z = z;
    d.w = w;
    d.f = f;
    return d;
}

} // extern "C"
