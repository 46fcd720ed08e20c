// Fixture generator (run by tests/golden/make_gpu_golden.py on a GPU host):
// the texture unit's linear-filter weights, read back from one-hot textures.
//
// For each of the 8 texels t of a 2x2x2 float texture (linear filtering, clamp
// addressing, unnormalized coordinates) a texture holding 1 at t and 0
// elsewhere is sampled at x = 0.5 + A[i]/256, y = 0.5 + A[j]/256,
// z = 0.5 + A[k]/256 over the lattice of fractions A; the result is texel t's
// weight there.  Then a ramp 0 -> 1 between two texel centres at 4096
// coordinates (the fraction quantization), then the NaN footprint: texel 0 set
// to NaN, the rest 1, over the same lattice.
//
// Then the ramp again at off-lattice coordinates: 65536 pseudo-random x in
// [0.5, 1.5) with full mantissas, and x just either side of every rounding
// boundary 0.5 + (j + 1/2)/256 at offsets of +-2^-e (e = 12 .. 23): how the unit
// forms the 8-bit fraction from a float coordinate.
//
// Output (binary, little endian): int32 na, int32 A[na], float W[8][na^3]
// (k slowest, i fastest), float ramp[4096], float nan_case[na^3],
// int32 m, float xs[m], float ramp_off[m].
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#define CHECK(x)                                                                                \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) {                                                                \
            std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
            return 1;                                                                           \
        }                                                                                       \
    } while (0)

__global__ void fetch(cudaTextureObject_t t, const float3* pos, float* out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = tex3D<float>(t, pos[i].x, pos[i].y, pos[i].z);
}

static int sample(const float vals[8], const std::vector<float3>& pos, std::vector<float>& out)
{
    cudaChannelFormatDesc d = cudaCreateChannelDesc<float>();
    cudaArray_t arr = nullptr;
    CHECK(cudaMalloc3DArray(&arr, &d, make_cudaExtent(2, 2, 2)));
    cudaMemcpy3DParms p = {};
    p.srcPtr = make_cudaPitchedPtr(const_cast<float*>(vals), 2 * sizeof(float), 2, 2);
    p.dstArray = arr;
    p.extent = make_cudaExtent(2, 2, 2);
    p.kind = cudaMemcpyHostToDevice;
    CHECK(cudaMemcpy3D(&p));
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td = {};
    td.normalizedCoords = 0;
    td.filterMode = cudaFilterModeLinear;
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.readMode = cudaReadModeElementType;
    cudaTextureObject_t tex = 0;
    CHECK(cudaCreateTextureObject(&tex, &rd, &td, nullptr));
    const int n = (int)pos.size();
    float3* dpos = nullptr;
    float* dout = nullptr;
    CHECK(cudaMalloc(&dpos, n * sizeof(float3)));
    CHECK(cudaMalloc(&dout, n * sizeof(float)));
    CHECK(cudaMemcpy(dpos, pos.data(), n * sizeof(float3), cudaMemcpyHostToDevice));
    fetch<<<(n + 255) / 256, 256>>>(tex, dpos, dout, n);
    CHECK(cudaGetLastError());
    out.resize(n);
    CHECK(cudaMemcpy(out.data(), dout, n * sizeof(float), cudaMemcpyDeviceToHost));
    cudaFree(dpos);
    cudaFree(dout);
    cudaDestroyTextureObject(tex);
    cudaFreeArray(arr);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: texture_probe <out.bin>\n");
        return 2;
    }
    const int A[] = {0,   1,   2,   3,   5,   8,   13,  17,  34,  51,  64,  85,  100, 119, 127,
                     128, 129, 137, 154, 171, 188, 200, 205, 222, 239, 250, 253, 254, 255};
    const int na = (int)(sizeof(A) / sizeof(A[0]));
    std::vector<float3> lattice;
    for (int k = 0; k < na; ++k)
        for (int j = 0; j < na; ++j)
            for (int i = 0; i < na; ++i)
                lattice.push_back(make_float3(0.5f + A[i] / 256.f, 0.5f + A[j] / 256.f, 0.5f + A[k] / 256.f));
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    std::fwrite(&na, sizeof(int), 1, f);
    std::fwrite(A, sizeof(int), na, f);
    std::vector<float> out;
    for (int t = 0; t < 8; ++t) {
        float v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        v[t] = 1.f;
        if (sample(v, lattice, out)) return 1;
        std::fwrite(out.data(), sizeof(float), out.size(), f);
    }
    std::vector<float3> ramp;
    for (int i = 0; i < 4096; ++i) ramp.push_back(make_float3(0.5f + i / 4096.f, 0.5f, 0.5f));
    {
        const float v[8] = {0, 1, 0, 1, 0, 1, 0, 1};
        if (sample(v, ramp, out)) return 1;
        std::fwrite(out.data(), sizeof(float), out.size(), f);
    }
    {
        const float v[8] = {NAN, 1, 1, 1, 1, 1, 1, 1};
        if (sample(v, lattice, out)) return 1;
        std::fwrite(out.data(), sizeof(float), out.size(), f);
    }
    {
        std::vector<float3> xs;
        unsigned long long st = 0x9E3779B97F4A7C15ull;
        for (int i = 0; i < 65536; ++i) {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            const float u = (float)((st >> 40) & 0xffffffull) / 16777216.f; // 24 random bits in [0, 1)
            xs.push_back(make_float3(0.5f + u, 0.5f, 0.5f));
        }
        for (int j = 0; j < 256; ++j)
            for (int e = 12; e <= 23; ++e)
                for (int sgn = -1; sgn <= 1; sgn += 2) {
                    const float x = 0.5f + (j + 0.5f) / 256.f + (float)sgn * std::ldexp(1.f, -e);
                    xs.push_back(make_float3(x, 0.5f, 0.5f));
                }
        const float v[8] = {0, 1, 0, 1, 0, 1, 0, 1};
        if (sample(v, xs, out)) return 1;
        const int m = (int)xs.size();
        std::fwrite(&m, sizeof(int), 1, f);
        for (const float3& p : xs) std::fwrite(&p.x, sizeof(float), 1, f);
        std::fwrite(out.data(), sizeof(float), out.size(), f);
    }
    std::fclose(f);
    std::printf("texture_probe: %d lattice points\n", (int)lattice.size());
    return 0;
}
