// Reader of the reference's on-disk sparse fields (s3r_dataset_*): the field
// info text file, the binary metadata with its compressed block tree, and the
// per-field value files; plus the batched pinned-host upload of one level.
//
// Formats (paths relative to the reference project root):
//   metadata     include/s3dmm/Metadata.hpp:182-214 (reader), 401-443 (writer), 445-493 (header);
//                containers as include/binary_io.hpp:130-252 writes them (size_t counts, fields in
//                declaration order, no padding); the tree as include/s3dmm/BlockTree_io.hpp:63-81
//   block tree   include/s3dmm/CompressedBlockTree.hpp: one byte per block, bit 7-c set when child c
//                (c = x + 2y + 4z) exists; blocks in breadth-first order, so the children of block i
//                start at 1 + the number of set bits of blocks 0..i-1 (generateMilestones, :397-412;
//                getChildIndex, :427-437)
//   node order   include/s3dmm/BlockTreeNodes.hpp:60-74 and walkBlockNodesPriv :160-173
//   values       include/s3dmm/BlockTreeFieldProvider.hpp:157-168
//   field info   include/s3dmm/BlockTreeFieldService.hpp:178-251
//   file names   include/filename_util.hpp:28-46, 92-100

#include "s3r_internal.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <fcntl.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <sys/uio.h>
#include <unistd.h>

namespace fs = std::filesystem;

namespace {

struct FieldInfo {
    std::string name;
    float min = NAN, max = NAN;
    int32_t animated = 0;
};

struct Subtree {
    uint32_t level = 0, x = 0, y = 0, z = 0;
    uint32_t tree_index = 0;
    uint32_t depth = 0;
    uint64_t values_offset = 0;
    int64_t node_count = -1; // computed on first use
};

inline uint64_t loc_key(uint32_t x, uint32_t y, uint32_t z)
{
    return (uint64_t)x | ((uint64_t)y << 21) | ((uint64_t)z << 42);
}

int fail(int code, const std::string& msg)
{
    s3r::set_thread_error(msg.c_str());
    return code;
}

// Bounded binary reader over a file held in memory.
struct Bytes {
    std::vector<char> buf;
    size_t pos = 0;
    bool ok = true;
    template <typename T> T get()
    {
        T v{};
        if (pos + sizeof(T) > buf.size()) {
            ok = false;
            pos = buf.size();
            return v;
        }
        std::memcpy(&v, buf.data() + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
};

bool read_file(const std::string& path, std::vector<char>& out)
{
    std::ifstream is(path, std::ios::binary);
    if (!is) return false;
    is.seekg(0, std::ios::end);
    const std::streamoff n = is.tellg();
    if (n < 0) return false;
    is.seekg(0);
    out.resize((size_t)n);
    return n == 0 || (bool)is.read(out.data(), n);
}

// Device state of the propagation of one level (built on first use): per parent node the indices of
// the child nodes that land on it.
struct PropLevel {
    bool ready = false;
    int32_t* src = nullptr;           // 8 per parent node, -1 = none
    uint64_t parent_nodes = 0, child_nodes = 0;
    std::vector<uint8_t> child_count; // per parent subtree
};

// Reusable per-thread scratch of the node walk.
struct WalkScratch {
    std::vector<uint64_t> seen; // one bit per dense vertex of the subtree
    struct Item {
        uint32_t t, r, x, y, z;
    };
    std::vector<Item> stack;
};

} // namespace

struct s3r_dataset {
    std::string base;
    bool has_time_steps = false;
    uint32_t time_steps = 0;
    std::vector<FieldInfo> fields;
    uint32_t version = 0, max_subtree_depth = 0, max_full_level = 0;
    float bc_min[3] = {0.f, 0.f, 0.f};
    float bc_size = 0.f;
    std::vector<uint8_t> masks;        // children bits of every tree block, breadth-first
    std::vector<uint64_t> first_child; // tree index of the first child of each block
    std::vector<Subtree> subtrees;     // by level, then z, y, x
    std::vector<uint32_t> level_begin; // subtrees of level l: [level_begin[l], level_begin[l+1])
    std::vector<std::unordered_map<uint64_t, uint32_t>> level_map;
    uint64_t field_file_size = 0;
    // field file descriptors, by (frame, field)
    std::unordered_map<uint64_t, int> fds;
    // pinned staging of s3r_dataset_frame_upload
    float* pinned[2] = {nullptr, nullptr};
    size_t pinned_cap[2] = {0, 0};
    cudaEvent_t copied[2] = {nullptr, nullptr};
    bool pending[2] = {false, false};
    int next = 0;
    std::vector<PropLevel> prop; // per parent level
};

namespace {

std::string frame_name(const s3r_dataset& ds, uint32_t frame)
{
    if (!ds.has_time_steps) return ds.base;
    const fs::path p(ds.base);
    char num[16];
    std::snprintf(num, sizeof num, "_t%06u", frame);
    return (p.parent_path() / p.stem() / (p.stem().string() + num + p.extension().string())).string();
}

int parse_field_info(s3r_dataset& ds, const std::string& path)
{
    std::ifstream is(path);
    if (!is) return fail(S3R_ERR_INVALID, "cannot open the field info file '" + path + "'");
    std::string line;
    auto expect = [&](int n, const char* content) {
        if (!std::getline(is, line) || line != content)
            return fail(S3R_ERR_INVALID, "line " + std::to_string(n) + " of '" + path + "': expected '" + content +
                                             "', found '" + line + "'");
        return S3R_OK;
    };
    if (int st = expect(1, "time_steps")) return st;
    if (!std::getline(is, line)) return fail(S3R_ERR_INVALID, "'" + path + "' ends in line 2");
    {
        std::istringstream iss(line);
        if (!(iss >> ds.time_steps)) return fail(S3R_ERR_INVALID, "line 2 of '" + path + "': no time step count");
    }
    if (int st = expect(3, "")) return st;
    if (int st = expect(4, "field\tmin\tmax\tanimated")) return st;
    for (int n = 5; std::getline(is, line); ++n) {
        if (line.empty()) continue;
        std::istringstream iss(line);
        FieldInfo f;
        std::string smin, smax;
        if (!(iss >> f.name >> smin >> smax >> f.animated))
            return fail(S3R_ERR_INVALID, "line " + std::to_string(n) + " of '" + path + "': malformed field line");
        // "-" marks a field without a range (processMesh.cpp writes it for empty fields)
        f.min = smin == "-" ? NAN : std::strtof(smin.c_str(), nullptr);
        f.max = smax == "-" ? NAN : std::strtof(smax.c_str(), nullptr);
        ds.fields.push_back(f);
    }
    return S3R_OK;
}

int parse_metadata(s3r_dataset& ds, const std::string& path)
{
    Bytes b;
    if (!read_file(path, b.buf)) return fail(S3R_ERR_INVALID, "cannot read the metadata file '" + path + "'");
    static const char kId[] = "s3dmm-metadata";
    const size_t id_len = sizeof kId - 1;
    if (b.buf.size() >= id_len && std::memcmp(b.buf.data(), kId, id_len) == 0) {
        b.pos = id_len;
        ds.version = b.get<uint32_t>();
        if (b.ok && ds.version > 1)
            return fail(S3R_ERR_UNSUPPORTED, "metadata format version " + std::to_string(ds.version) + " in '" +
                                                 path + "' (1 is the newest known)");
        const uint64_t header = b.get<uint64_t>();
        const size_t p0 = b.pos;
        const uint32_t dim = b.get<uint32_t>();
        ds.max_subtree_depth = b.get<uint32_t>();
        ds.max_full_level = b.get<uint32_t>();
        if (!b.ok || dim != 3 || b.pos - p0 != header)
            return fail(S3R_ERR_INVALID, "'" + path + "': invalid metadata header");
    } else {
        ds.version = 0;
        ds.max_full_level = 0;
    }
    const uint64_t tree_pos = b.get<uint64_t>();
    if (!b.ok || tree_pos > b.buf.size()) return fail(S3R_ERR_INVALID, "'" + path + "': bad block tree offset");
    b.pos = (size_t)tree_pos;
    for (float& v : ds.bc_min) v = b.get<float>();
    ds.bc_size = b.get<float>();
    const uint64_t bits = b.get<uint64_t>();
    const uint64_t nbytes = b.get<uint64_t>();
    if (!b.ok || nbytes > b.buf.size() - b.pos || (bits >> 3) > nbytes)
        return fail(S3R_ERR_INVALID, "'" + path + "': truncated block tree");
    const uint64_t nblocks = bits >> 3;
    ds.masks.assign(b.buf.begin() + b.pos, b.buf.begin() + b.pos + nblocks);
    b.pos += nbytes;
    ds.first_child.resize(nblocks);
    uint64_t next = 1;
    for (uint64_t i = 0; i < nblocks; ++i) {
        ds.first_child[i] = next;
        next += (uint64_t)__builtin_popcount(ds.masks[i]);
    }
    if (nblocks && next != nblocks)
        return fail(S3R_ERR_INVALID, "'" + path + "': block tree children do not add up to its block count");
    if (ds.version == 0) ds.max_subtree_depth = b.get<uint32_t>();
    const uint64_t nlevels = b.get<uint64_t>();
    if (!b.ok || nlevels > 64) return fail(S3R_ERR_INVALID, "'" + path + "': bad level count");
    std::vector<Subtree> all;
    ds.level_begin.assign(1, 0);
    for (uint64_t l = 0; l < nlevels; ++l) {
        const uint64_t n = b.get<uint64_t>();
        if (!b.ok || n > b.buf.size()) return fail(S3R_ERR_INVALID, "'" + path + "': bad subtree count");
        std::vector<Subtree> lv((size_t)n);
        for (Subtree& s : lv) {
            s.level = (uint32_t)l;
            s.x = b.get<uint32_t>();
            s.y = b.get<uint32_t>();
            s.z = b.get<uint32_t>();
            s.tree_index = b.get<uint32_t>();
            s.values_offset = b.get<uint64_t>();
            s.depth = ds.version == 0 ? ds.max_subtree_depth : (uint32_t)b.get<uint64_t>();
            if (s.tree_index >= nblocks || s.depth > 15 || (l < 21 && (s.x >> l || s.y >> l || s.z >> l)))
                b.ok = false;
        }
        if (!b.ok) return fail(S3R_ERR_INVALID, "'" + path + "': bad subtree record at level " + std::to_string(l));
        std::sort(lv.begin(), lv.end(), [](const Subtree& a, const Subtree& c) {
            return a.z != c.z ? a.z < c.z : a.y != c.y ? a.y < c.y : a.x < c.x;
        });
        all.insert(all.end(), lv.begin(), lv.end());
        ds.level_begin.push_back((uint32_t)all.size());
    }
    ds.field_file_size = b.get<uint64_t>();
    if (!b.ok) return fail(S3R_ERR_INVALID, "'" + path + "': truncated after the subtree map");
    ds.subtrees.swap(all);
    ds.level_map.resize(nlevels);
    for (uint64_t l = 0; l < nlevels; ++l)
        for (uint32_t i = ds.level_begin[l]; i < ds.level_begin[l + 1]; ++i) {
            const Subtree& s = ds.subtrees[i];
            ds.level_map[l][loc_key(s.x, s.y, s.z)] = i;
        }
    return S3R_OK;
}

// BlockTreeNodes<3>(tree, root, depth): visits the subtree's blocks depth-first
// (pre-order, children in local index order), per block its 8 corners, and
// emits each node where it first appears.  Returns the node count, or -1 when
// the tree references a block it does not hold.
int64_t walk_nodes(const s3r_dataset& ds, const Subtree& st, uint16_t* n2i, WalkScratch& ws)
{
    const uint32_t d = st.depth;
    const uint64_t e = (1ull << d) + 1;
    ws.seen.assign((e * e * e + 63) / 64, 0ull);
    ws.stack.clear();
    ws.stack.push_back({st.tree_index, 0u, st.x, st.y, st.z});
    const uint64_t mask = (1ull << d) - 1;
    const uint64_t nblocks = ds.masks.size();
    int64_t count = 0;
    while (!ws.stack.empty()) {
        const WalkScratch::Item it = ws.stack.back();
        ws.stack.pop_back();
        const uint32_t shift = d - it.r;
        const uint64_t bx = ((uint64_t)it.x << shift) & mask, by = ((uint64_t)it.y << shift) & mask,
                       bz = ((uint64_t)it.z << shift) & mask;
        for (uint32_t k = 0; k < 8; ++k) {
            const uint64_t nx = bx + ((uint64_t)(k & 1) << shift), ny = by + ((uint64_t)((k >> 1) & 1) << shift),
                           nz = bz + ((uint64_t)(k >> 2) << shift);
            const uint64_t v = nx + e * (ny + e * nz);
            uint64_t& w = ws.seen[v >> 6];
            const uint64_t bit = 1ull << (v & 63);
            if (w & bit) continue;
            w |= bit;
            if (n2i) {
                n2i[3 * count + 0] = (uint16_t)nx;
                n2i[3 * count + 1] = (uint16_t)ny;
                n2i[3 * count + 2] = (uint16_t)nz;
            }
            ++count;
        }
        if (it.r >= d || it.t >= nblocks) continue;
        const uint8_t m = ds.masks[it.t];
        if (!m) continue;
        // push children last-to-first so child 0 is visited next
        uint64_t ci = ds.first_child[it.t] + (uint64_t)__builtin_popcount(m);
        for (int c = 7; c >= 0; --c) {
            if (!(m & (0x80u >> c))) continue;
            --ci;
            if (ci >= nblocks) return -1;
            ws.stack.push_back({(uint32_t)ci, it.r + 1, 2 * it.x + (c & 1), 2 * it.y + ((c >> 1) & 1),
                                2 * it.z + ((c >> 2) & 1)});
        }
    }
    return count;
}

const Subtree* find_subtree(const s3r_dataset& ds, uint32_t level, const uint32_t idx[3])
{
    if (level >= ds.level_map.size()) return nullptr;
    auto it = ds.level_map[level].find(loc_key(idx[0], idx[1], idx[2]));
    return it == ds.level_map[level].end() ? nullptr : &ds.subtrees[it->second];
}

int ensure_node_count(const s3r_dataset& ds, Subtree& st, WalkScratch& ws)
{
    if (st.node_count >= 0) return S3R_OK;
    const int64_t n = walk_nodes(ds, st, nullptr, ws);
    if (n < 0) return fail(S3R_ERR_INVALID, "block tree references a missing block");
    st.node_count = n;
    return S3R_OK;
}

void fill_info(const Subtree& s, s3r_subtree_info* o)
{
    o->level = s.level;
    o->x = s.x;
    o->y = s.y;
    o->z = s.z;
    o->depth = s.depth;
    o->tree_index = s.tree_index;
    o->values_offset = s.values_offset;
    o->node_count = s.node_count < 0 ? 0 : (uint64_t)s.node_count;
}

int field_fd(s3r_dataset& ds, uint32_t field, uint32_t frame, int* fd)
{
    if (field >= ds.fields.size()) return fail(S3R_ERR_INVALID, "field index out of range");
    if (frame >= std::max<uint32_t>(ds.time_steps, 1)) return fail(S3R_ERR_INVALID, "time frame out of range");
    const uint64_t key = ((uint64_t)frame << 32) | field;
    auto it = ds.fds.find(key);
    if (it != ds.fds.end()) {
        *fd = it->second;
        return S3R_OK;
    }
    const std::string path = frame_name(ds, frame) + ".s3dmm-field#" + ds.fields[field].name;
    const int f = ::open(path.c_str(), O_RDONLY | O_CLOEXEC);
    if (f < 0) return fail(S3R_ERR_INVALID, "cannot open the field file '" + path + "': " + std::strerror(errno));
    ds.fds[key] = f;
    *fd = f;
    return S3R_OK;
}

// Reads exactly the iovec's bytes at `offset`.
bool preadv_all(int fd, struct iovec* iov, int cnt, uint64_t offset)
{
    while (cnt > 0) {
        const ssize_t r = ::preadv(fd, iov, cnt, (off_t)offset);
        if (r < 0) {
            if (errno == EINTR) continue;
            return false;
        }
        if (r == 0) return false;
        offset += (uint64_t)r;
        size_t left = (size_t)r;
        while (cnt > 0 && left >= iov->iov_len) {
            left -= iov->iov_len;
            ++iov;
            --cnt;
        }
        if (cnt > 0 && left) {
            iov->iov_base = (char*)iov->iov_base + left;
            iov->iov_len -= left;
        }
    }
    return true;
}

uint32_t thread_count(uint32_t requested, uint32_t work)
{
    uint32_t t = requested ? requested : std::max(1u, std::thread::hardware_concurrency());
    return std::max(1u, std::min({t, work, 64u}));
}

// Runs f(begin, end, thread) over [0, n) split into `threads` contiguous ranges;
// returns the first nonzero status.
template <typename F> int parallel_ranges(uint32_t n, uint32_t threads, F&& f)
{
    if (threads <= 1) return f(0u, n, 0u);
    std::vector<int> st(threads, S3R_OK);
    std::vector<std::string> msg(threads);
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < threads; ++t) {
        const uint32_t b = (uint32_t)((uint64_t)n * t / threads), e = (uint32_t)((uint64_t)n * (t + 1) / threads);
        pool.emplace_back([&, b, e, t] {
            st[t] = f(b, e, t);
            if (st[t]) msg[t] = s3r_last_error(nullptr); // the worker's thread-local message
        });
    }
    for (auto& th : pool) th.join();
    for (uint32_t t = 0; t < threads; ++t)
        if (st[t]) return fail(st[t], msg[t]);
    return S3R_OK;
}

// Resolves the blocks of a frame request to subtree records.
int resolve_blocks(s3r_dataset& ds, uint32_t level, const uint32_t* idx, uint32_t nb, std::vector<Subtree*>& out)
{
    if (nb && !idx) return fail(S3R_ERR_INVALID, "null block index list");
    out.resize(nb);
    for (uint32_t b = 0; b < nb; ++b) {
        const Subtree* s = find_subtree(ds, level, idx + 3 * b);
        if (!s)
            return fail(S3R_ERR_INVALID, "block (" + std::to_string(idx[3 * b]) + ", " + std::to_string(idx[3 * b + 1]) +
                                             ", " + std::to_string(idx[3 * b + 2]) + ") of level " +
                                             std::to_string(level) + " is no subtree root");
        out[b] = const_cast<Subtree*>(s);
    }
    return S3R_OK;
}

} // namespace

extern "C" {

int s3r_dataset_open(const char* base_name, s3r_dataset** out)
{
    if (!base_name || !out) return fail(S3R_ERR_INVALID, "null argument");
    *out = nullptr;
    auto ds = new (std::nothrow) s3r_dataset();
    if (!ds) return fail(S3R_ERR_NOMEM, "out of host memory");
    ds->base = base_name;
    // firstOutputFrameFileName: a file (or its metadata) -> one frame; <dir>/<stem> a directory -> frames
    std::error_code ec;
    const fs::path p(ds->base);
    const bool as_file = fs::is_regular_file(p, ec) || fs::is_regular_file(ds->base + ".s3dmm-meta", ec);
    const bool as_dir = fs::is_directory(p.parent_path() / p.stem(), ec);
    std::string info;
    if (as_file) {
        info = ds->base + ".s3dmm-fields";
    } else if (as_dir) {
        ds->has_time_steps = true;
        info = (p.parent_path() / p.stem() / (p.stem().string() + p.extension().string() + ".s3dmm-fields")).string();
    } else {
        delete ds;
        return fail(S3R_ERR_INVALID, std::string("no dataset files match the name '") + base_name + "'");
    }
    int st = parse_field_info(*ds, info);
    if (!st) st = parse_metadata(*ds, frame_name(*ds, 0) + ".s3dmm-meta");
    if (st) {
        delete ds;
        return st;
    }
    *out = ds;
    return S3R_OK;
}

int s3r_dataset_close(s3r_dataset* ds)
{
    if (!ds) return S3R_OK;
    for (PropLevel& pl : ds->prop)
        if (pl.src) cudaFree(pl.src);
    for (auto& kv : ds->fds) ::close(kv.second);
    for (int i = 0; i < 2; ++i) {
        if (ds->copied[i]) {
            cudaEventSynchronize(ds->copied[i]);
            cudaEventDestroy(ds->copied[i]);
        }
        if (ds->pinned[i]) cudaFreeHost(ds->pinned[i]);
    }
    delete ds;
    return S3R_OK;
}

int s3r_dataset_info_get(const s3r_dataset* ds, s3r_dataset_info* o)
{
    if (!ds || !o) return fail(S3R_ERR_INVALID, "null argument");
    *o = s3r_dataset_info{};
    o->format_version = ds->version;
    o->time_steps = ds->time_steps;
    o->field_count = (uint32_t)ds->fields.size();
    o->max_subtree_depth = ds->max_subtree_depth;
    o->max_full_level = ds->max_full_level;
    o->level_count = (uint32_t)ds->level_map.size();
    o->subtree_count = (uint32_t)ds->subtrees.size();
    o->has_time_steps = ds->has_time_steps ? 1u : 0u;
    o->tree_blocks = ds->masks.size();
    o->field_file_size = ds->field_file_size;
    for (int i = 0; i < 3; ++i) o->bc_min[i] = ds->bc_min[i];
    o->bc_size = ds->bc_size;
    return S3R_OK;
}

int s3r_dataset_field(const s3r_dataset* ds, uint32_t index, char* name, size_t name_cap, float range[2],
                      int32_t* animated)
{
    if (!ds) return fail(S3R_ERR_INVALID, "null dataset");
    if (index >= ds->fields.size()) return fail(S3R_ERR_INVALID, "field index out of range");
    const FieldInfo& f = ds->fields[index];
    if (name && name_cap) {
        const size_t n = std::min(name_cap - 1, f.name.size());
        std::memcpy(name, f.name.data(), n);
        name[n] = 0;
    }
    if (range) {
        range[0] = f.min;
        range[1] = f.max;
    }
    if (animated) *animated = f.animated;
    return S3R_OK;
}

int s3r_dataset_field_index(const s3r_dataset* ds, const char* name, uint32_t* index)
{
    if (!ds || !name || !index) return fail(S3R_ERR_INVALID, "null argument");
    for (size_t i = 0; i < ds->fields.size(); ++i)
        if (ds->fields[i].name == name) {
            *index = (uint32_t)i;
            return S3R_OK;
        }
    return fail(S3R_ERR_INVALID, std::string("field '") + name + "' is not defined");
}

int s3r_dataset_tree_blocks(const s3r_dataset* ds, uint32_t level, uint32_t* xyz, uint64_t cap, uint64_t* count)
{
    if (!ds || !count || (cap && !xyz)) return fail(S3R_ERR_INVALID, "null argument");
    // breadth-first: a level's blocks in tree order, each block's children in local index order
    std::vector<uint64_t> t{0}, nt;
    std::vector<uint32_t> loc{0, 0, 0}, nloc;
    if (ds->masks.empty()) t.clear(), loc.clear();
    for (uint32_t l = 0; l < level && !t.empty(); ++l) {
        nt.clear();
        nloc.clear();
        for (size_t i = 0; i < t.size(); ++i) {
            const uint8_t m = ds->masks[t[i]];
            uint64_t ci = ds->first_child[t[i]];
            for (uint32_t c = 0; c < 8; ++c) {
                if (!(m & (0x80u >> c))) continue;
                if (ci >= ds->masks.size()) return fail(S3R_ERR_INVALID, "block tree references a missing block");
                nt.push_back(ci++);
                nloc.push_back(2 * loc[3 * i] + (c & 1));
                nloc.push_back(2 * loc[3 * i + 1] + ((c >> 1) & 1));
                nloc.push_back(2 * loc[3 * i + 2] + (c >> 2));
            }
        }
        t.swap(nt);
        loc.swap(nloc);
    }
    *count = t.size();
    const uint64_t n = std::min<uint64_t>(cap, t.size());
    if (n) std::memcpy(xyz, loc.data(), n * 3 * sizeof(uint32_t));
    return S3R_OK;
}

int s3r_dataset_subtrees(s3r_dataset* ds, uint32_t level, s3r_subtree_info* out, uint32_t cap, uint32_t* count)
{
    if (!ds || !count || (cap && !out)) return fail(S3R_ERR_INVALID, "null argument");
    if (level >= ds->level_map.size()) {
        *count = 0;
        return S3R_OK;
    }
    const uint32_t b = ds->level_begin[level], e = ds->level_begin[level + 1];
    *count = e - b;
    const uint32_t n = std::min(cap, e - b);
    const int st = parallel_ranges(n, thread_count(0, n / 64 + 1), [&](uint32_t i0, uint32_t i1, uint32_t) {
        WalkScratch ws;
        for (uint32_t i = i0; i < i1; ++i)
            if (int s = ensure_node_count(*ds, ds->subtrees[b + i], ws)) return s;
        return (int)S3R_OK;
    });
    if (st) return st;
    for (uint32_t i = 0; i < n; ++i) fill_info(ds->subtrees[b + i], out + i);
    return S3R_OK;
}

int s3r_dataset_subtree(s3r_dataset* ds, uint32_t level, const uint32_t idx[3], s3r_subtree_info* out)
{
    if (!ds || !idx || !out) return fail(S3R_ERR_INVALID, "null argument");
    std::vector<Subtree*> one;
    if (int st = resolve_blocks(*ds, level, idx, 1, one)) return st;
    WalkScratch ws;
    if (int st = ensure_node_count(*ds, *one[0], ws)) return st;
    fill_info(*one[0], out);
    return S3R_OK;
}

int s3r_dataset_subtree_nodes(s3r_dataset* ds, uint32_t level, const uint32_t idx[3], uint16_t* n2i,
                              uint64_t cap_nodes, uint64_t* count)
{
    if (!ds || !idx || !count) return fail(S3R_ERR_INVALID, "null argument");
    std::vector<Subtree*> one;
    if (int st = resolve_blocks(*ds, level, idx, 1, one)) return st;
    WalkScratch ws;
    if (int st = ensure_node_count(*ds, *one[0], ws)) return st;
    *count = (uint64_t)one[0]->node_count;
    if (!n2i) return S3R_OK;
    if (cap_nodes < *count) return fail(S3R_ERR_INVALID, "n2i buffer too small");
    walk_nodes(*ds, *one[0], n2i, ws);
    return S3R_OK;
}

int s3r_dataset_subtree_values(s3r_dataset* ds, uint32_t field, uint32_t frame, uint32_t level,
                               const uint32_t idx[3], float range[2], float* values, uint64_t cap_nodes,
                               uint64_t* count)
{
    if (!ds || !idx || !count) return fail(S3R_ERR_INVALID, "null argument");
    std::vector<Subtree*> one;
    if (int st = resolve_blocks(*ds, level, idx, 1, one)) return st;
    WalkScratch ws;
    if (int st = ensure_node_count(*ds, *one[0], ws)) return st;
    const uint64_t n = (uint64_t)one[0]->node_count;
    *count = n;
    if (!values && !range) return S3R_OK;
    if (values && cap_nodes < n) return fail(S3R_ERR_INVALID, "value buffer too small");
    int fd = -1;
    if (int st = field_fd(*ds, field, frame, &fd)) return st;
    float rng[2];
    struct iovec iov[2] = {{rng, sizeof rng}, {values, values ? n * sizeof(float) : 0}};
    if (!preadv_all(fd, iov, values ? 2 : 1, one[0]->values_offset))
        return fail(S3R_ERR_INVALID, "short read from the field file");
    if (range) {
        range[0] = rng[0];
        range[1] = rng[1];
    }
    return S3R_OK;
}

int s3r_dataset_frame_topology(s3r_dataset* ds, uint32_t level, const uint32_t* idx, uint32_t nb, uint32_t* blocks,
                               uint64_t* node_off, uint16_t* n2i, uint64_t n2i_cap_nodes, uint32_t threads)
{
    if (!ds || !blocks || !node_off) return fail(S3R_ERR_INVALID, "null argument");
    std::vector<Subtree*> sts;
    if (int st = resolve_blocks(*ds, level, idx, nb, sts)) return st;
    const uint32_t nt = thread_count(threads, nb);
    int st = parallel_ranges(nb, nt, [&](uint32_t b0, uint32_t b1, uint32_t) {
        WalkScratch ws;
        for (uint32_t b = b0; b < b1; ++b)
            if (int s = ensure_node_count(*ds, *sts[b], ws)) return s;
        return (int)S3R_OK;
    });
    if (st) return st;
    node_off[0] = 0;
    for (uint32_t b = 0; b < nb; ++b) {
        const Subtree& s = *sts[b];
        if (s.depth > S3R_MAX_DEPTH)
            return fail(S3R_ERR_UNSUPPORTED, "subtree depth " + std::to_string(s.depth) + " above S3R_MAX_DEPTH");
        blocks[4 * b + 0] = s.x;
        blocks[4 * b + 1] = s.y;
        blocks[4 * b + 2] = s.z;
        blocks[4 * b + 3] = s.depth;
        node_off[b + 1] = node_off[b] + (uint64_t)s.node_count;
    }
    if (!n2i) return S3R_OK;
    if (n2i_cap_nodes < node_off[nb]) return fail(S3R_ERR_INVALID, "n2i buffer too small");
    return parallel_ranges(nb, nt, [&](uint32_t b0, uint32_t b1, uint32_t) {
        WalkScratch ws;
        for (uint32_t b = b0; b < b1; ++b) walk_nodes(*ds, *sts[b], n2i + 3 * node_off[b], ws);
        return (int)S3R_OK;
    });
}

int s3r_dataset_frame_values(s3r_dataset* ds, uint32_t field, uint32_t frame, uint32_t level, const uint32_t* idx,
                             uint32_t nb, const uint64_t* node_off, float* values, float* ranges, uint32_t threads)
{
    if (!ds || !node_off || (nb && !values)) return fail(S3R_ERR_INVALID, "null argument");
    std::vector<Subtree*> sts;
    if (int st = resolve_blocks(*ds, level, idx, nb, sts)) return st;
    {
        WalkScratch ws; // node counts are cached after the first request for a block
        for (uint32_t b = 0; b < nb; ++b) {
            if (int st = ensure_node_count(*ds, *sts[b], ws)) return st;
            if (node_off[b + 1] - node_off[b] != (uint64_t)sts[b]->node_count)
                return fail(S3R_ERR_INVALID, "node_off does not match the subtrees' node counts");
        }
    }
    int fd = -1;
    if (int st = field_fd(*ds, field, frame, &fd)) return st;
    return parallel_ranges(nb, thread_count(threads, nb), [&](uint32_t b0, uint32_t b1, uint32_t) {
        for (uint32_t b = b0; b < b1; ++b) {
            float rng[2];
            struct iovec iov[2] = {{rng, sizeof rng},
                                   {values + node_off[b], (node_off[b + 1] - node_off[b]) * sizeof(float)}};
            if (!preadv_all(fd, iov, 2, sts[b]->values_offset))
                return fail(S3R_ERR_INVALID, "short read from the field file");
            if (ranges) {
                ranges[2 * b] = rng[0];
                ranges[2 * b + 1] = rng[1];
            }
        }
        return (int)S3R_OK;
    });
}

int s3r_dataset_frame_upload(s3r_ctx* ctx, s3r_dataset* ds, uint32_t field, uint32_t frame, uint32_t level,
                             const uint32_t* idx, uint32_t nb, const uint64_t* node_off, float* sparse, float* ranges,
                             uint32_t threads, void* stream)
{
    if (!ctx || !ds || !node_off || (nb && !sparse)) return fail(S3R_ERR_INVALID, "null argument");
    const cudaStream_t s = (cudaStream_t)stream;
    const int slot = ds->next;
    const size_t bytes = node_off[nb] * sizeof(float);
    cudaError_t e = cudaSuccess;
    if (ds->pending[slot]) {
        e = cudaEventSynchronize(ds->copied[slot]);
        ds->pending[slot] = false;
        if (e != cudaSuccess) return fail(S3R_ERR_CUDA, std::string("staging wait: ") + cudaGetErrorString(e));
    }
    if (bytes > ds->pinned_cap[slot]) {
        if (ds->pinned[slot]) cudaFreeHost(ds->pinned[slot]);
        ds->pinned[slot] = nullptr;
        ds->pinned_cap[slot] = 0;
        const size_t cap = bytes + bytes / 4;
        e = cudaHostAlloc((void**)&ds->pinned[slot], cap, cudaHostAllocDefault);
        if (e != cudaSuccess) return fail(S3R_ERR_NOMEM, std::string("pinned staging: ") + cudaGetErrorString(e));
        ds->pinned_cap[slot] = cap;
    }
    if (!ds->copied[slot]) {
        e = cudaEventCreateWithFlags(&ds->copied[slot], cudaEventDisableTiming);
        if (e != cudaSuccess) return fail(S3R_ERR_CUDA, std::string("staging event: ") + cudaGetErrorString(e));
    }
    if (int st = s3r_dataset_frame_values(ds, field, frame, level, idx, nb, node_off, ds->pinned[slot], ranges, threads))
        return st;
    if (bytes) {
        e = cudaMemcpyAsync(sparse, ds->pinned[slot], bytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return fail(S3R_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
    }
    e = cudaEventRecord(ds->copied[slot], s);
    if (e != cudaSuccess) return fail(S3R_ERR_CUDA, std::string("staging record: ") + cudaGetErrorString(e));
    ds->pending[slot] = true;
    ds->next = slot ^ 1;
    return S3R_OK;
}

} // extern "C"

namespace {

int prop_fail(s3r_ctx* ctx, cudaError_t e, const char* what)
{
    return fail(S3R_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Uploads what the propagation into `level` needs: both levels' node lists, the parent maps' layout,
// each child's parent, position and shift.
int prop_prepare(s3r_dataset& ds, uint32_t level, PropLevel& pl)
{
    const uint32_t nl = (uint32_t)ds.level_map.size();
    const uint32_t p0 = ds.level_begin[level], p1 = ds.level_begin[level + 1];
    const uint32_t c0 = level + 1 < nl ? ds.level_begin[level + 1] : 0, c1 = level + 1 < nl ? ds.level_begin[level + 2] : 0;
    const uint32_t np = p1 - p0, nc = c1 - c0;
    // node counts and node lists of both levels
    std::vector<uint64_t> poff(np + 1, 0), coff(nc + 1, 0);
    int st = parallel_ranges(np + nc, thread_count(0, (np + nc) / 16 + 1), [&](uint32_t b, uint32_t e, uint32_t) {
        WalkScratch ws;
        for (uint32_t i = b; i < e; ++i)
            if (int r = ensure_node_count(ds, ds.subtrees[i < np ? p0 + i : c0 + (i - np)], ws)) return r;
        return (int)S3R_OK;
    });
    if (st) return st;
    std::vector<s3r::PropParent> parents(np);
    uint64_t map_entries = 0;
    for (uint32_t i = 0; i < np; ++i) {
        const Subtree& t = ds.subtrees[p0 + i];
        if (t.depth < 1 || t.depth > S3R_MAX_DEPTH)
            return fail(S3R_ERR_UNSUPPORTED, "subtree depth " + std::to_string(t.depth) + " outside 1..S3R_MAX_DEPTH");
        poff[i + 1] = poff[i] + (uint64_t)t.node_count;
        const uint64_t e = (1ull << t.depth) + 1;
        parents[i] = {t.depth, 0u, map_entries};
        map_entries += e * e * e;
    }
    std::vector<s3r::PropChild> children(nc);
    pl.child_count.assign(np, 0);
    for (uint32_t k = 0; k < nc; ++k) {
        const Subtree& t = ds.subtrees[c0 + k];
        coff[k + 1] = coff[k] + (uint64_t)t.node_count;
        auto it = ds.level_map[level].find(loc_key(t.x >> 1, t.y >> 1, t.z >> 1));
        if (it == ds.level_map[level].end())
            return fail(S3R_ERR_INVALID, "a subtree of level " + std::to_string(level + 1) + " has no parent subtree");
        const uint32_t p = it->second - p0;
        children[k] = {p, (t.x & 1) + 2 * (t.y & 1) + 4 * (t.z & 1), (int32_t)t.depth + 1 - (int32_t)parents[p].depth, 0u};
        ++pl.child_count[p];
    }
    std::vector<uint16_t> pn2i(3 * poff[np]), cn2i(3 * coff[nc]);
    st = parallel_ranges(np + nc, thread_count(0, (np + nc) / 16 + 1), [&](uint32_t b, uint32_t e, uint32_t) {
        WalkScratch ws;
        for (uint32_t i = b; i < e; ++i) {
            if (i < np) walk_nodes(ds, ds.subtrees[p0 + i], pn2i.data() + 3 * poff[i], ws);
            else walk_nodes(ds, ds.subtrees[c0 + (i - np)], cn2i.data() + 3 * coff[i - np], ws);
        }
        return (int)S3R_OK;
    });
    if (st) return st;
    if (coff[nc] >= (1ull << 31)) return fail(S3R_ERR_UNSUPPORTED, "more than 2^31 child nodes in one level");
    // temporary device copies: node lists, layout, dense maps; kept: the gather indices
    const size_t sizes[8] = {np * sizeof(s3r::PropParent) + 1, (np + 1) * sizeof(uint64_t), pn2i.size() * 2 + 2,
                             nc * sizeof(s3r::PropChild) + 1, (nc + 1) * sizeof(uint64_t), cn2i.size() * 2 + 2,
                             map_entries * sizeof(int32_t) + 4, sizeof(uint32_t)};
    void* tmp[8] = {};
    auto release = [&]() {
        for (void*& p : tmp)
            if (p) cudaFree(p), p = nullptr;
    };
    cudaError_t e = cudaMalloc((void**)&pl.src, poff[np] * 8 * sizeof(int32_t) + 32);
    for (int i = 0; i < 8 && e == cudaSuccess; ++i) e = cudaMalloc(&tmp[i], sizes[i]);
    if (e != cudaSuccess) {
        release();
        if (pl.src) cudaFree(pl.src), pl.src = nullptr;
        return fail(S3R_ERR_NOMEM, std::string("propagation buffers: ") + cudaGetErrorString(e));
    }
    const void* from[6] = {parents.data(), poff.data(), pn2i.data(), children.data(), coff.data(), cn2i.data()};
    const size_t bytes[6] = {np * sizeof(s3r::PropParent), (np + 1) * sizeof(uint64_t), pn2i.size() * 2,
                             nc * sizeof(s3r::PropChild), (nc + 1) * sizeof(uint64_t), cn2i.size() * 2};
    for (int i = 0; i < 6 && e == cudaSuccess; ++i)
        if (bytes[i]) e = cudaMemcpy(tmp[i], from[i], bytes[i], cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(tmp[7], 0, sizeof(uint32_t));
    s3r::PropArgs a{};
    a.parents = (const s3r::PropParent*)tmp[0];
    a.parent_node_off = (const uint64_t*)tmp[1];
    a.parent_n2i = (const uint16_t*)tmp[2];
    a.children = (const s3r::PropChild*)tmp[3];
    a.child_node_off = (const uint64_t*)tmp[4];
    a.child_n2i = (const uint16_t*)tmp[5];
    a.map = (int32_t*)tmp[6];
    a.src = pl.src;
    a.error = (uint32_t*)tmp[7];
    a.parent_nodes = poff[np];
    a.child_nodes = coff[nc];
    a.nparents = np;
    a.nchildren = nc;
    uint32_t launches = 0, err = 0;
    if (e == cudaSuccess) e = s3r::launch_prop_index(a, nullptr, &launches);
    if (e == cudaSuccess) e = cudaMemcpy(&err, tmp[7], sizeof err, cudaMemcpyDeviceToHost); // synchronizes
    release();
    if (e != cudaSuccess || err) {
        cudaFree(pl.src);
        pl.src = nullptr;
        if (e != cudaSuccess) return prop_fail(nullptr, e, "propagation index");
        return fail(S3R_ERR_INVALID, err & 2u ? "a child node lands where its parent subtree has no node"
                                               : "a child node lands outside its parent subtree");
    }
    pl.parent_nodes = poff[np];
    pl.child_nodes = coff[nc];
    pl.ready = true;
    return S3R_OK;
}

} // namespace

extern "C" {

int s3r_dataset_propagate(s3r_ctx* ctx, s3r_dataset* ds, uint32_t level, const float* child_values, float* sums,
                          float* weights, uint8_t* child_count, void* stream)
{
    if (!ctx || !ds || !sums || !weights) return fail(S3R_ERR_INVALID, "null argument");
    if (level >= ds->level_map.size()) return fail(S3R_ERR_INVALID, "level out of range");
    if (ds->prop.size() < ds->level_map.size()) ds->prop.resize(ds->level_map.size());
    PropLevel& pl = ds->prop[level];
    if (!pl.ready)
        if (int st = prop_prepare(*ds, level, pl)) return st;
    if (pl.child_nodes && !child_values) return fail(S3R_ERR_INVALID, "null child values");
    const cudaError_t e =
        s3r::launch_prop_gather(pl.src, pl.child_nodes ? child_values : sums, pl.parent_nodes, sums, weights,
                                (cudaStream_t)stream);
    if (pl.parent_nodes) s3r::count_launches(ctx, 1);
    if (e != cudaSuccess) return prop_fail(ctx, e, "propagation kernel");
    if (child_count && !pl.child_count.empty()) std::memcpy(child_count, pl.child_count.data(), pl.child_count.size());
    return S3R_OK;
}

int s3r_field_divide(s3r_ctx* ctx, const float* sums, const float* weights, uint64_t n, float* values, void* stream)
{
    if (!ctx || (n && (!sums || !weights || !values))) return fail(S3R_ERR_INVALID, "null argument");
    const cudaError_t e = s3r::launch_divide(sums, weights, n, values, (cudaStream_t)stream);
    if (n) s3r::count_launches(ctx, 1);
    if (e != cudaSuccess) return prop_fail(ctx, e, "divide kernel");
    return S3R_OK;
}

} // extern "C"
