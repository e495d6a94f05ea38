// Scene input in the reference's format: hsr_read_obj, the C form of
// hussar::WavefrontFile::read (libhussar/include/hussar/io/wavefront.h:12-67).
//
// Line by line, as the reference parses: a line whose first character is '#' is a
// comment; otherwise the first token is the command: 'v' appends a vertex from the next
// three numbers (further components are ignored), 'f' a triangle from the next three
// 1-based vertex indices counted from the vertices the mesh had before this read
// (further indices are ignored), 's' and empty lines are skipped, and any other command
// is skipped and counted. The reference reads index tokens with `>> int`, which stops at
// the '/' of an 'a/b/c' token and leaves its stream failed for the rest of the file; here
// the vertex index before the first '/' is taken. Numbers are parsed with strtof/strtol
// (correctly rounded, as the reference's `>> float`). Host code only: no device is needed.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "hsr_internal.h"

namespace {

struct ObjData {
    std::vector<float> v;
    std::vector<int64_t> f;  // 1-based as in the file
    int64_t unsupported = 0;
};

// the next whitespace-separated token of `line` from `pos` (empty at the end)
std::string next_token(const std::string &line, size_t &pos) {
    while (pos < line.size() && (line[pos] == ' ' || line[pos] == '\t' || line[pos] == '\r')) ++pos;
    const size_t b = pos;
    while (pos < line.size() && line[pos] != ' ' && line[pos] != '\t' && line[pos] != '\r') ++pos;
    return line.substr(b, pos - b);
}

bool parse_obj(const char *path, ObjData &out, std::string &err) {
    FILE *fh = std::fopen(path, "rb");
    if (!fh) {
        err = std::string("invalid file passed to hsr_read_obj: ") + path;
        return false;
    }
    std::string line;
    int c;
    int64_t lineno = 0;
    bool ok = true;
    while (ok) {
        line.clear();
        bool any = false;
        while ((c = std::fgetc(fh)) != EOF) {
            any = true;
            if (c == '\n') break;
            line.push_back(char(c));
        }
        if (!any) break;
        ++lineno;
        if (!line.empty() && line[0] == '#') continue;
        size_t pos = 0;
        const std::string cmd = next_token(line, pos);
        if (cmd == "v") {
            for (int i = 0; i < 3; ++i) {
                const std::string t = next_token(line, pos);
                char *end = nullptr;
                errno = 0;
                const float x = std::strtof(t.c_str(), &end);
                if (t.empty() || end == t.c_str()) {
                    err = "line " + std::to_string(lineno) + ": a vertex needs three coordinates";
                    ok = false;
                    break;
                }
                out.v.push_back(x);
            }
        } else if (cmd == "f") {
            for (int i = 0; i < 3; ++i) {
                const std::string t = next_token(line, pos);
                char *end = nullptr;
                const long long k = std::strtoll(t.c_str(), &end, 10);
                if (t.empty() || end == t.c_str() || (*end != '\0' && *end != '/')) {
                    err = "line " + std::to_string(lineno) + ": a face needs three vertex indices";
                    ok = false;
                    break;
                }
                out.f.push_back(int64_t(k));
            }
        } else if (cmd == "s" || cmd.empty()) {
            // smoothing groups and empty lines carry nothing for the tracer
        } else {
            ++out.unsupported;
        }
    }
    std::fclose(fh);
    return ok;
}

}  // namespace

extern "C" hsr_status hsr_read_obj(const char *path, int64_t vertex_offset, float *vertices, int64_t vertex_capacity,
                                   int32_t *indices, int64_t triangle_capacity, int64_t *out_vertex_count,
                                   int64_t *out_triangle_count, int64_t *out_unsupported) {
    if (!path || !out_vertex_count || !out_triangle_count || vertex_offset < 0) {
        hsr::set_last_error("null argument or negative vertex offset");
        return HSR_ERR_INVALID_ARGUMENT;
    }
    ObjData d;
    std::string err;
    if (!parse_obj(path, d, err)) {
        hsr::set_last_error(err);
        return HSR_ERR_INVALID_ARGUMENT;
    }
    const int64_t nv = int64_t(d.v.size() / 3), nt = int64_t(d.f.size() / 3);
    *out_vertex_count = nv;
    *out_triangle_count = nt;
    if (out_unsupported) *out_unsupported = d.unsupported;
    if (!vertices && !indices) return HSR_OK;  // size query
    if (!vertices || !indices || vertex_capacity < nv || triangle_capacity < nt) {
        hsr::set_last_error("hsr_read_obj: buffers too small for " + std::to_string(nv) + " vertices and " +
                            std::to_string(nt) + " triangles");
        return HSR_ERR_INVALID_ARGUMENT;
    }
    std::memcpy(vertices, d.v.data(), sizeof(float) * d.v.size());
    for (size_t i = 0; i < d.f.size(); ++i) {
        // wavefront.h:42-48: 1-based, shifted by the vertices already in the mesh
        const int64_t k = d.f[i] + vertex_offset - 1;
        if (k < 0 || k > INT32_MAX) {
            hsr::set_last_error("hsr_read_obj: face " + std::to_string(i / 3 + 1) + " has a vertex index out of range");
            return HSR_ERR_INVALID_ARGUMENT;
        }
        indices[i] = int32_t(k);
    }
    return HSR_OK;
}
