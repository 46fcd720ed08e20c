// Test infrastructure only: writes small datasets with the reference's own
// writers and dumps what the reference's own readers return for them.  Built
// by oracle/Makefile (target `ref`) from the reference headers where they lie,
// into oracle/_ref/ref_dataset_gen; tests/golden/make_dataset.py runs it to
// make the committed dataset fixtures.  Nothing in the product links it.
//
// Reference code exercised:
//   writing   MetadataProvider<3>::metadata (include/s3dmm/MetadataProvider.hpp:61-92): block tree made
//             compressible, Metadata<3> generate (include/s3dmm/Metadata.hpp:401-443);
//             BlockTreeFieldProvider<3> with BlockTreeFieldGenerationPolicy::Propagate
//             (include/s3dmm/BlockTreeFieldProvider.hpp:270-389) and BlockTreeFieldFromFunc<3>
//             (include/s3dmm/BlockTreeFieldFromFunc.hpp:51-87)
//   reading   Metadata<3>(istream) (Metadata.hpp:182-214), levels(), blockTreeNodes(root) (:244-258),
//             BlockTreeFieldProvider<3>::fieldValues (BlockTreeFieldProvider.hpp:111-168)
//
// Usage:
//   ref_dataset_gen write <base> <variant>        variant: shell (1 frame, fields f, g) | frames (2 frames)
//   ref_dataset_gen dump <meta> <outdir> <field file>...
//       outdir/subtrees.txt   one line per subtree: level x y z depth tree_pos values_pos node_count
//                             (levels ascending, then z, y, x)
//       outdir/n2i.bin        the subtrees' n2i lists (uint16 x, y, z) in that order
//       outdir/values_<k>.bin per field file k: per subtree its range (2 floats) then its values
#include <math.h> // the reference's BlockTreeFieldFromFunc calls isnan unqualified

#include "filename_util.hpp"
#include "s3dmm/Metadata.hpp"
#include "s3dmm/MetadataProvider.hpp"
#include "s3dmm/BlockTreeFieldProvider.hpp"
#include "s3dmm/BlockTreeFieldFromFunc.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <string>
#include <tuple>
#include <vector>

using namespace s3dmm;

namespace {

// A block tree full down to level 2 of the cube [-5, 5]^3, refined to level
// `deep` at points on a sphere shell of radius 3 (golden-angle spiral).
struct ShellTreeGenerator {
    unsigned int deep;
    unsigned int points;
    BlockTree<3> makeBlockTree() const
    {
        BlockTree<3> bt(BoundingCube<3, real_type>({-5.f, -5.f, -5.f}, 10.f));
        MultiIndex<3, unsigned int> i;
        do {
            bt.ensureBlockAt(i, 2);
        } while (incMultiIndex(i, 4u));
        const double ga = M_PI * (3.0 - std::sqrt(5.0));
        for (unsigned int k = 0; k < points; ++k) {
            const double y = 1.0 - 2.0 * (k + 0.5) / points, r = std::sqrt(1.0 - y * y), a = ga * k;
            Vec<3, real_type> p{real_type(3.0 * r * std::cos(a)), real_type(3.0 * y), real_type(3.0 * r * std::sin(a))};
            bt.ensureBlockAt(p, deep);
        }
        return bt;
    }
    unsigned int maxTreeDepth() const { return deep; }
};

// Field functions: no field (NaN) inside radius 2.
struct FieldF {
    real_type operator()(const Vec<3, real_type>& p) const
    {
        const real_type r2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
        return r2 < 4 ? NAN : p[0] + 2 * p[1] - real_type(0.5) * p[2];
    }
};
struct FieldG {
    real_type t;
    real_type operator()(const Vec<3, real_type>& p) const
    {
        const real_type r2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
        return r2 < 4 ? NAN : p[0] * p[1] - p[2] + t;
    }
};

template <class Func>
void write_field(const Metadata<3>& md, const std::string& path, const Func& f)
{
    BlockTreeFieldFromFunc<3, Func> gen(md, f);
    BlockTreeFieldProvider<3> btf(md, path, gen, BlockTreeFieldGenerationPolicy::Propagate);
}

int write_dataset(const std::string& base, const std::string& variant)
{
    namespace fs = std::filesystem;
    const bool frames = variant == "frames";
    const unsigned int deep = frames ? 4 : 6, points = frames ? 120 : 1500;
    const unsigned int maxSubtreeDepth = frames ? 2 : 3, maxFullLevel = 1;
    std::vector<std::string> frameNames;
    if (frames) {
        const auto [dir, stem, ext] = splitFileName(base);
        fs::create_directories(fs::path(dir) / stem);
        for (unsigned int t = 0; t < 2; ++t) frameNames.push_back(frameOutputFileName(base, t, true));
    } else {
        frameNames.push_back(base);
        std::ofstream(base) << "mesh placeholder\n"; // the base name is a file, as for a preprocessed mesh
    }
    // every frame shares the block tree; each gets its own metadata file as the prep tools write it
    for (size_t t = 0; t < frameNames.size(); ++t) {
        MetadataProvider<3, ShellTreeGenerator> mp(frameNames[t] + ".s3dmm-meta", maxSubtreeDepth, deep,
                                                   maxFullLevel, ShellTreeGenerator{deep, points});
        auto& md = mp.metadata();
        if (frames) {
            write_field(md, frameNames[t] + ".s3dmm-field#g", FieldG{real_type(t)});
        } else {
            write_field(md, frameNames[t] + ".s3dmm-field#f", FieldF{});
            write_field(md, frameNames[t] + ".s3dmm-field#g", FieldG{0});
        }
    }
    std::string info;
    if (frames) {
        const auto [dir, stem, ext] = splitFileName(base);
        info = (fs::path(dir) / stem / (stem + ext + ".s3dmm-fields")).string();
    } else {
        info = base + ".s3dmm-fields";
    }
    std::ofstream os(info);
    os << "time_steps\n" << frameNames.size() << "\n\n" << "field\tmin\tmax\tanimated\n";
    if (frames) {
        os << "g\t-5\t6\t1\n";
    } else {
        os << "f\t-17.5\t17.5\t0\n" << "g\t-30\t30\t0\n";
    }
    return 0;
}

int dump(const std::string& meta, const std::string& outdir, const std::vector<std::string>& fieldFiles)
{
    std::ifstream is(meta, std::ios::binary);
    if (!is) {
        std::cerr << "cannot open " << meta << "\n";
        return 1;
    }
    Metadata<3> md(is);
    using Rec = std::tuple<unsigned, unsigned, unsigned, unsigned, Metadata<3>::MetadataBlock>;
    std::vector<Rec> recs;
    for (auto level : md.levels())
        for (auto& block : level)
            recs.emplace_back(block.level, block.blockIndex[2], block.blockIndex[1], block.blockIndex[0], block);
    std::sort(recs.begin(), recs.end(), [](const Rec& a, const Rec& b) {
        return std::make_tuple(std::get<0>(a), std::get<1>(a), std::get<2>(a), std::get<3>(a)) <
               std::make_tuple(std::get<0>(b), std::get<1>(b), std::get<2>(b), std::get<3>(b));
    });
    std::ofstream txt(outdir + "/subtrees.txt");
    std::ofstream n2i(outdir + "/n2i.bin", std::ios::binary);
    std::vector<std::unique_ptr<BlockTreeFieldProvider<3>>> btfs;
    std::vector<std::unique_ptr<std::ofstream>> vals;
    for (size_t k = 0; k < fieldFiles.size(); ++k) {
        btfs.emplace_back(new BlockTreeFieldProvider<3>(md, fieldFiles[k]));
        vals.emplace_back(new std::ofstream(outdir + "/values_" + std::to_string(k) + ".bin", std::ios::binary));
    }
    for (auto& r : recs) {
        const auto& b = std::get<4>(r);
        const auto root = b.subtreeRoot();
        const auto nodes = md.blockTreeNodes(root);
        txt << b.level << ' ' << b.blockIndex[0] << ' ' << b.blockIndex[1] << ' ' << b.blockIndex[2] << ' '
            << md.subtreeDepth(root) << ' ' << b.subtreeData.subtreeBlockTreePos << ' '
            << b.subtreeData.subtreeValuesPos << ' ' << nodes.nodeCount() << '\n';
        for (auto& ni : nodes.data().n2i)
            for (int d = 0; d < 3; ++d) {
                const uint16_t c = static_cast<uint16_t>(ni[d]);
                n2i.write(reinterpret_cast<const char*>(&c), 2);
            }
        for (size_t k = 0; k < btfs.size(); ++k) {
            Vec2<real_type> range;
            std::vector<real_type> v;
            btfs[k]->fieldValues(range, v, nodes);
            vals[k]->write(reinterpret_cast<const char*>(range.data()), 2 * sizeof(real_type));
            vals[k]->write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(real_type)));
        }
    }
    return 0;
}

} // namespace

int main(int argc, char** argv)
{
    try {
        if (argc == 4 && std::string(argv[1]) == "write") return write_dataset(argv[2], argv[3]);
        if (argc >= 4 && std::string(argv[1]) == "dump")
            return dump(argv[2], argv[3], std::vector<std::string>(argv + 4, argv + argc));
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
    std::cerr << "usage: ref_dataset_gen write <base> shell|frames | dump <meta> <outdir> <field file>...\n";
    return 2;
}
