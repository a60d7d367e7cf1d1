// Wavefront OBJ reading for the scene builder: the reference loads its meshes
// with igl::readOBJ (model/mesh.cpp:9-21) and keeps the vertices and the
// triangles.  Read here: `v x y z` records and `f` records of three or more
// vertex references (the first field of each `v/vt/vn` form; negative
// references count back from the last vertex read so far), polygons split
// into fans (0, j, j + 1).  Every other record is ignored.  The Python
// mirror (delta2_gb300.load_obj) applies the same rules.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "d2g_scene.hpp"

namespace d2g {

namespace {

// The whitespace-separated fields of one line.
void split_fields(const std::string& line, std::vector<std::string>& out) {
    out.clear();
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r' || line[i] == '\v' ||
                                   line[i] == '\f'))
            i++;
        const size_t j = i;
        while (i < line.size() && !(line[i] == ' ' || line[i] == '\t' || line[i] == '\r' || line[i] == '\v' ||
                                    line[i] == '\f'))
            i++;
        if (i > j) out.push_back(line.substr(j, i - j));
    }
}

// A whole field as a double (out-of-range magnitudes become +-inf or 0, as
// Python's float() gives for the mirror reader).
bool parse_double(const std::string& s, double* v) {
    if (s.empty()) return false;
    char* end = nullptr;
    *v = std::strtod(s.c_str(), &end);
    return end && *end == '\0';
}

// A whole field as an integer that fits 64 bits.
bool parse_int(const std::string& s, long long* v) {
    if (s.empty()) return false;
    char* end = nullptr;
    errno = 0;
    *v = std::strtoll(s.c_str(), &end, 10);
    return end && *end == '\0' && errno == 0;
}

}  // namespace

bool read_obj(const char* path, std::vector<double>& V, std::vector<int32_t>& F, std::string* err) {
    V.clear();
    F.clear();
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        if (err) *err = std::string(path) + ": cannot open";
        return false;
    }
    std::string line;
    std::vector<std::string> fields;
    std::vector<long long> idx;
    long long line_no = 0;
    bool ok = true;
    auto fail = [&](const std::string& m) {
        if (err) *err = std::string(path) + ":" + std::to_string(line_no) + ": " + m;
        ok = false;
    };
    char buf[4096];
    while (ok) {
        line.clear();
        bool got = false;
        while (std::fgets(buf, sizeof buf, f)) {
            got = true;
            line += buf;
            if (!line.empty() && line.back() == '\n') break;
        }
        if (!got) break;
        line_no++;
        if (!line.empty() && line.back() == '\n') line.pop_back();
        split_fields(line, fields);
        if (fields.empty()) continue;
        if (fields[0] == "v" && fields.size() >= 4) {
            double x[3];
            for (int k = 0; k < 3; k++)
                if (!parse_double(fields[1 + k], &x[k])) {
                    fail("bad vertex coordinate '" + fields[1 + k] + "'");
                    break;
                }
            if (!ok) break;
            V.insert(V.end(), x, x + 3);
        } else if (fields[0] == "f" && fields.size() >= 4) {
            idx.clear();
            const long long nv = (long long)(V.size() / 3);
            for (size_t t = 1; t < fields.size(); t++) {
                const std::string& tok = fields[t];
                long long k;
                if (!parse_int(tok.substr(0, tok.find('/')), &k)) {
                    fail("bad face reference '" + tok + "'");
                    break;
                }
                idx.push_back(k > 0 ? k - 1 : nv + k);
            }
            if (!ok) break;
            for (size_t j = 1; j + 1 < idx.size(); j++) {
                const long long tri[3] = {idx[0], idx[j], idx[j + 1]};
                for (long long v : tri) {
                    if (v < 0 || v > 2147483647LL) {
                        fail("face index out of range");
                        break;
                    }
                    F.push_back((int32_t)v);
                }
                if (!ok) break;
            }
        }
    }
    std::fclose(f);
    if (!ok) return false;
    const long long nv = (long long)(V.size() / 3);
    for (int32_t v : F)
        if (v >= nv) {
            if (err) *err = std::string(path) + ": face index out of range";
            return false;
        }
    return true;
}

}  // namespace d2g
