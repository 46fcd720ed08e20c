// Test driver (compiled and run by tests/test_gpu_adapters.py): the C++ drop-ins of revise_gb300/adapters
// used through the reference's own interfaces, on a dataset in the reference's format.
//
//   adapter_check interp <dataset base>
//       every subtree of every level through BlockTreeFieldService<3>::interpolateWith with
//       DenseFieldInterpolatorGb300 (host grid) and with the reference's DenseFieldInterpolator<3>;
//       prints "interp <subtrees> <vertices> <mismatches>" (bitwise comparison, NaN = NaN)
//   adapter_check worker <dataset base> <input file> <output file>
//       VsWorkerGb300 (seam 3, rendering with DenseFieldRendererGb300, seam 2) over one level's whole block
//       cube; the input file holds: level, field mode, W, H, fovY, quality, relative threshold, relative
//       isosurface level, isosurface opacity, the 16 floats of the camera transform (column-major), the
//       number of colour control points and per point x r g b a.  Writes origin x, y, width, height
//       (int32) and the part's ARGB32 pixels.
#include "s3dmm/BlockTreeFieldService.hpp"
#include "s3dmm/DenseFieldInterpolator.hpp"

#include "DenseFieldInterpolatorGb300.hpp"
#include "VsWorkerGb300.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <vector>

using namespace s3dmm;

static int run_interp(const std::string& base)
{
    BlockTreeFieldService<3> svc(base);
    const auto& md = svc.metadata();
    size_t subtrees = 0, vertices = 0, bad = 0;
    for (const auto& levelBlocks : md.levels()) {
        for (const auto& mb : levelBlocks) {
            const auto root = mb.subtreeRoot();
            Vec2<dfield_real> r1, r2;
            std::vector<dfield_real> gpu, cpu;
            svc.interpolateWith<DenseFieldInterpolatorGb300<std::vector<dfield_real>&>>(r1, gpu, 0, 0, root);
            svc.interpolateWith<DenseFieldInterpolator<3>>(r2, cpu, 0, 0, root);
            ++subtrees;
            vertices += cpu.size();
            if (gpu.size() != cpu.size() || r1[0] != r2[0] || r1[1] != r2[1]) {
                bad += cpu.size() ? cpu.size() : 1;
                continue;
            }
            for (size_t i = 0; i < cpu.size(); ++i) {
                const bool na = std::isnan(gpu[i]), nb = std::isnan(cpu[i]);
                if (na != nb || (!na && std::memcmp(&gpu[i], &cpu[i], sizeof(float)) != 0)) ++bad;
            }
        }
    }
    std::printf("interp %zu %zu %zu\n", subtrees, vertices, bad);
    return bad ? 1 : 0;
}

static int run_worker(const std::string& base, const std::string& in_path, const std::string& out_path)
{
    std::ifstream in(in_path);
    unsigned level, mode, W, H, npoints;
    float fovy, quality, thr, iso, opacity, m[16];
    in >> level >> mode >> W >> H >> fovy >> quality >> thr >> iso >> opacity;
    for (float& x : m) in >> x;
    in >> npoints;
    s3vs::ColorTransferFunction ctf;
    for (unsigned i = 0; i < npoints; ++i) {
        float x, r, g, b, a;
        in >> x >> r >> g >> b >> a;
        ctf[x] = s3vs::Vec4r{r, g, b, a};
    }
    if (!in) {
        std::fprintf(stderr, "bad input file\n");
        return 2;
    }
    s3vs::VsRenderSharedState st;
    st.fieldSvc = std::make_shared<BlockTreeFieldService<3>>(base);
    st.primaryFieldIndex = st.secondaryFieldIndex = 0;
    st.input.setFieldMode(static_cast<s3vs::FieldMode>(mode));
    st.input.setViewportSize(s3vs::Vec2i{static_cast<int>(W), static_cast<int>(H)});
    st.input.setFovY(fovy);
    st.input.setRenderQuality(quality);
    st.input.fieldAllParam().setThreshold(thr);
    st.input.fieldAllParam().setIsosurfaceLevel(iso);
    st.input.fieldAllParam().setIsosurfaceOpacity(opacity);
    st.input.fieldAllParam().setColorTransferFunction(ctf);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) st.cameraTransform.e[c][r] = m[4 * c + r];

    VsWorkerGb300 worker;
    worker.initialize("", false, "", 0);
    worker.setRenderSharedState(&st);
    // the level's whole block cube; an index box's max is one past its last block, as the reference's
    // splitter makes the boxes it hands to workers (BlockOrderUtil.hpp:45-47 takes 1 off it)
    const unsigned cubes = 1u << level;
    s3vs::SubtreeSetDescription subtrees(level, MultiIndex<3, unsigned int>{0, 0, 0},
                                         MultiIndex<3, unsigned int>{cubes, cubes, cubes});
    silver_bullets::sync::CancelController cc;
    const auto part = worker.renderScenePart(subtrees, cc.checker());
    std::ofstream out(out_path, std::ios::binary);
    const int32_t head[4] = {part.origin[0], part.origin[1], part.image.size[0], part.image.size[1]};
    out.write(reinterpret_cast<const char*>(head), sizeof(head));
    out.write(reinterpret_cast<const char*>(part.image.bits.data()), static_cast<std::streamsize>(part.image.bits.size()));
    return out ? 0 : 3;
}

int main(int argc, char** argv)
{
    try {
        if (argc >= 3 && std::string(argv[1]) == "interp") return run_interp(argv[2]);
        if (argc >= 5 && std::string(argv[1]) == "worker") return run_worker(argv[2], argv[3], argv[4]);
        std::fprintf(stderr, "usage: adapter_check interp <base> | worker <base> <in> <out>\n");
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 4;
    }
}
