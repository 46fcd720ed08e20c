// Test infrastructure only: a C-callable harness around the reference's own
// header-only hot-path code, compiled in place from the reference tree by
// oracle/Makefile (target `ref`) into oracle/_ref/libs3r_ref.so.  It is the
// checker the golden fixtures under tests/golden/ are generated from; nothing
// in the product links or loads it.
//
// Wrapped reference code:
//   ref_interp_dense      s3dmm::DenseFieldInterpolator<3>::interpolate(dense, sparse, nodes)
//                         include/s3dmm/DenseFieldInterpolator.hpp:198-419
//   ref_b2f_order         s3dmm::BackToFrontOrder<s3dmm::MacroBlock<3>>::range(eye)
//                         include/BackToFrontOrder.hpp:61-359, include/MacroBlock.hpp:29-67
//   ref_blend_image_part  s3vs::blendImagePart(dst, src, justCopySrc, dstOffset)
//                         src/s3vs_lib/BlendImagePart.hpp:61-145
//   ref_make_ctf          s3vs::makeColorTransferVector(ctmap, colorCount)
//                         include/s3vs/ColorTransferFunction.hpp:27-69
//   ref_split_cube        s3dmm::IndexCubeSplitter<3>(level, count, [-5,5]^3).all_blocks(trailing)
//                         include/IndexCubeSplitter.hpp:36-196
//   ref_split_b2f         BackToFrontOrder over that splitter for an eye
//                         (IndexCubeSplitStorage::getBoxesSorted, src/s3vs_lib/IndexCubeSplitStorage.hpp:54-74)
#include "s3dmm/DenseFieldInterpolator.hpp"
#include "IndexCubeSplitter.hpp"
#include "s3dmm/Metadata.hpp"
#include "BackToFrontOrder.hpp"
#include "MacroBlock.hpp"
#include "s3vs/ColorTransferFunction.hpp"
#include "BlendImagePart.hpp"

#include <cstdint>
#include <cstring>
#include <vector>

using namespace s3dmm;

extern "C" {

// Dense (2^depth+1)^3 grid from n sparse nodes; dense must hold that many floats.
int ref_interp_dense(const uint16_t* n2i_xyz, const float* sparse, uint32_t n, uint32_t depth,
                     float* dense)
{
    using BT = Metadata<3>::BT;
    using Nodes = BlockTreeNodes<3, BT>;
    typename Nodes::Data data;
    data.maxDepth = depth;
    data.n2i.resize(n);
    for (uint32_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d)
            data.n2i[i][d] = n2i_xyz[3 * i + d];
    auto nodes = Nodes::fromData(std::move(data));
    std::vector<real_type> sparseField(sparse, sparse + n);
    std::vector<dfield_real> denseField;
    DenseFieldInterpolator<3>::interpolate(denseField, sparseField, nodes);
    std::memcpy(dense, denseField.data(), denseField.size() * sizeof(float));
    return static_cast<int>(denseField.size());
}

// Visits the blocks of the index box [bmin, bmax) whose world box is
// [cmin, cmax], as BackToFrontOrder orders them for the eye; writes the
// block indices (3 per block) into out and returns how many it wrote.
int ref_b2f_order(const uint32_t* bmin, const uint32_t* bmax, const double* cmin,
                  const double* cmax, const double* eye, uint32_t* out, uint32_t capacity)
{
    BoundingBox<3, unsigned int> ib;
    ib << Vec3u{bmin[0], bmin[1], bmin[2]} << Vec3u{bmax[0], bmax[1], bmax[2]};
    BoundingBox<3, real_type> cb;
    cb << Vec<3, real_type>{real_type(cmin[0]), real_type(cmin[1]), real_type(cmin[2])}
       << Vec<3, real_type>{real_type(cmax[0]), real_type(cmax[1]), real_type(cmax[2])};
    MacroBlock<3> mb{ib, cb};
    BackToFrontOrder<MacroBlock<3>> b2fo{mb};
    uint32_t count = 0;
    Vec<3, real_type> e{real_type(eye[0]), real_type(eye[1]), real_type(eye[2])};
    for (const auto& block : b2fo.range(e)) {
        if (count < capacity) {
            out[3 * count] = block[0];
            out[3 * count + 1] = block[1];
            out[3 * count + 2] = block[2];
        }
        ++count;
    }
    return static_cast<int>(count);
}

// dst: dw x dh ARGB32 pixels; src: sw x sh pixels placed at (ox, oy).
void ref_blend_image_part(uint32_t* dst, int dw, int dh, const uint32_t* src, int sw, int sh,
                          int ox, int oy, int justCopySrc, int offx, int offy)
{
    s3vs::RgbaImage d;
    d.size = {dw, dh};
    d.bits.resize(size_t(dw) * dh * 4);
    std::memcpy(d.bits.data(), dst, d.bits.size());
    s3vs::RgbaImagePart s;
    s.origin = {ox, oy};
    s.image.size = {sw, sh};
    s.image.bits.resize(size_t(sw) * sh * 4);
    std::memcpy(s.image.bits.data(), src, s.image.bits.size());
    s3vs::blendImagePart(d, s, justCopySrc != 0, s3vs::Vec2i{offx, offy});
    std::memcpy(dst, d.bits.data(), d.bits.size());
}

// Control points (x[i], rgba[4i..4i+3]) -> colorCount RGBA entries.
void ref_make_ctf(const double* xs, const double* rgba, uint32_t npoints, uint32_t colorCount,
                  float* out)
{
    s3vs::ColorTransferFunction ctmap;
    for (uint32_t i = 0; i < npoints; ++i)
        ctmap[real_type(xs[i])] = s3vs::Vec4r{real_type(rgba[4 * i]), real_type(rgba[4 * i + 1]),
                                              real_type(rgba[4 * i + 2]), real_type(rgba[4 * i + 3])};
    auto v = s3vs::makeColorTransferVector(ctmap, colorCount);
    std::memcpy(out, v.data(), v.size() * sizeof(float));
}

} // extern "C"

extern "C" {

static BoundingBox<3, real_type> ref_cube_bbox()
{
    return BoundingBox<3, real_type>{} << Vec<3, real_type>{-5, -5, -5} << Vec<3, real_type>{5, 5, 5};
}

// Boxes of the splitter (6 per box: min xyz, max xyz; empty boxes as zeros); returns the count.
int ref_split_cube(uint32_t level, uint32_t count, int trailing, uint32_t* out, uint32_t capacity)
{
    IndexCubeSplitter<3> sp{level, count, ref_cube_bbox()};
    auto boxes = sp.all_blocks(trailing != 0);
    uint32_t n = 0;
    for (auto& b : boxes) {
        if (n < capacity)
            for (int a = 0; a < 3; ++a) {
                out[6 * n + a] = b.empty() ? 0u : b.min()[a];
                out[6 * n + 3 + a] = b.empty() ? 0u : b.max()[a];
            }
        ++n;
    }
    return (int)n;
}

int ref_split_b2f(uint32_t level, uint32_t count, const double* eye, uint32_t* out, uint32_t capacity)
{
    IndexCubeSplitter<3> sp{level, count, ref_cube_bbox()};
    BackToFrontOrder b2f{sp};
    Vec<3, real_type> e{real_type(eye[0]), real_type(eye[1]), real_type(eye[2])};
    uint32_t n = 0;
    for (const auto& b : b2f.range(e)) {
        if (n < capacity)
            for (int a = 0; a < 3; ++a) {
                out[6 * n + a] = b.min()[a];
                out[6 * n + 3 + a] = b.max()[a];
            }
        ++n;
    }
    return (int)n;
}

} // extern "C"
