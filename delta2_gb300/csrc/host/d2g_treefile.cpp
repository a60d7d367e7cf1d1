// Versioned binary file of flattened surrogate trees (no counterpart in the
// reference, which builds its trees when it loads a mesh).  The arrays are the
// in-memory layout of d2g_trees: per node the child link, child count,
// inner flag and depth, and the node's bucket of up to 8 triangles with their
// eps and inner eps (model/surrogate_components.h:11-88), plus the mesh
// offsets and each mesh's triangle count.
//
// Layout, little-endian:
//   char     magic[8]      "D2GTREES"
//   uint32   version       2 (version 1 files came from a builder whose
//                          last-resort regrouping moved more triangles than
//                          the reference's divideAndFit does; they are refused
//                          so that a scene rebuilds its trees)
//   uint32   endian        0x01020304
//   uint32   n_meshes
//   uint32   reserved      0
//   uint64   n_nodes
//   uint64   checksum      FNV-1a 64 of the payload bytes
//   payload: int32 mesh_node_off[n_meshes + 1], int32 mesh_ntris[n_meshes],
//            int32 nodes[4 n_nodes], int32 ntris[n_nodes],
//            float64 tris[72 n_nodes], float64 eps[8 n_nodes],
//            float64 inner_eps[8 n_nodes]
#include <cstdio>
#include <cstring>

#include "d2g_scene.hpp"

namespace d2g {

namespace {

constexpr char kMagic[8] = {'D', '2', 'G', 'T', 'R', 'E', 'E', 'S'};
constexpr uint32_t kVersion = 2, kEndian = 0x01020304u;

struct Header {
    char magic[8];
    uint32_t version, endian, n_meshes, reserved;
    uint64_t n_nodes, checksum;
};
static_assert(sizeof(Header) == 40, "header layout");

uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 0x100000001b3ULL;
    }
    return h;
}

template <class T>
void add(std::vector<std::pair<const void*, size_t>>& parts, const std::vector<T>& v) {
    parts.push_back({v.data(), v.size() * sizeof(T)});
}

}  // namespace

bool save_trees(const TreeSet& t, const char* path, std::string* err) {
    const size_t nm = t.mesh_ntris.size(), nn = t.ntris.size();
    if (t.mesh_node_off.size() != nm + 1 || t.nodes.size() != 4 * nn || t.tris.size() != 72 * nn ||
        t.eps.size() != 8 * nn || t.inner_eps.size() != 8 * nn || (size_t)t.mesh_node_off.back() != nn) {
        if (err) *err = "inconsistent tree arrays";
        return false;
    }
    std::vector<std::pair<const void*, size_t>> parts;
    add(parts, t.mesh_node_off);
    add(parts, t.mesh_ntris);
    add(parts, t.nodes);
    add(parts, t.ntris);
    add(parts, t.tris);
    add(parts, t.eps);
    add(parts, t.inner_eps);
    Header h;
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.endian = kEndian;
    h.n_meshes = (uint32_t)nm;
    h.reserved = 0;
    h.n_nodes = nn;
    h.checksum = 0xcbf29ce484222325ULL;
    for (auto& p : parts) h.checksum = fnv1a(h.checksum, p.first, p.second);
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) {
        if (err) *err = std::string("cannot write ") + tmp;
        return false;
    }
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
    for (auto& p : parts) ok = ok && (p.second == 0 || std::fwrite(p.first, 1, p.second, f) == p.second);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        if (err) *err = std::string("writing ") + path + " failed";
        return false;
    }
    return true;
}

bool load_trees(const char* path, TreeSet& t, std::string* err) {
    auto fail = [&](const std::string& m) {
        if (err) *err = std::string(path) + ": " + m;
        return false;
    };
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail("cannot open");
    Header h;
    if (std::fread(&h, sizeof h, 1, f) != 1) {
        std::fclose(f);
        return fail("short header");
    }
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.endian != kEndian) {
        std::fclose(f);
        return fail("not a tree file of this byte order");
    }
    if (h.version != kVersion) {
        std::fclose(f);
        return fail("unsupported version " + std::to_string(h.version));
    }
    const size_t nm = h.n_meshes, nn = (size_t)h.n_nodes;
    if (nm > (1u << 28) || nn > (1ull << 32)) {
        std::fclose(f);
        return fail("implausible sizes");
    }
    t.mesh_node_off.resize(nm + 1);
    t.mesh_ntris.resize(nm);
    t.nodes.resize(4 * nn);
    t.ntris.resize(nn);
    t.tris.resize(72 * nn);
    t.eps.resize(8 * nn);
    t.inner_eps.resize(8 * nn);
    std::vector<std::pair<void*, size_t>> parts = {
        {t.mesh_node_off.data(), t.mesh_node_off.size() * 4}, {t.mesh_ntris.data(), t.mesh_ntris.size() * 4},
        {t.nodes.data(), t.nodes.size() * 4},                 {t.ntris.data(), t.ntris.size() * 4},
        {t.tris.data(), t.tris.size() * 8},                   {t.eps.data(), t.eps.size() * 8},
        {t.inner_eps.data(), t.inner_eps.size() * 8}};
    uint64_t sum = 0xcbf29ce484222325ULL;
    for (auto& p : parts) {
        if (p.second && std::fread(p.first, 1, p.second, f) != p.second) {
            std::fclose(f);
            return fail("truncated");
        }
        sum = fnv1a(sum, p.first, p.second);
    }
    const bool trailing = std::fgetc(f) != EOF;
    std::fclose(f);
    if (trailing) return fail("trailing bytes");
    if (sum != h.checksum) return fail("checksum mismatch");
    // structure: monotone offsets, links inside the mesh, at most 8 triangles per bucket
    if (t.mesh_node_off[0] != 0 || (size_t)t.mesh_node_off[nm] != nn) return fail("bad mesh offsets");
    for (size_t m = 0; m < nm; m++) {
        const int a = t.mesh_node_off[m], b = t.mesh_node_off[m + 1];
        if (b <= a) return fail("empty or decreasing mesh offsets");
        for (int i = a; i < b; i++) {
            const int child = t.nodes[4 * (size_t)i], count = t.nodes[4 * (size_t)i + 1];
            if (t.ntris[i] < 0 || t.ntris[i] > 8) return fail("bucket size out of range");
            if (child != -1 && (child < a || child >= b || count < 0 || child + count > b))
                return fail("child link outside its mesh");
        }
    }
    return true;
}

}  // namespace d2g
