// stl.cpp — STL ingest (host): format detection by content
// (stlformat::detect, aeros/src/stl_format.h:86-140) and the binary / ASCII
// parse of loadSTL (aeros/src/stl_loader.cpp:30-223), over an in-memory file
// or a path. The output feeds aeros_voxelize / aeros_voxel_plan: 9 floats per
// triangle, and 9 per triangle of per-vertex normals.
//
// Parsing text is host work; the parse follows the reference rule for rule
// (the same standard-library stream extraction for ASCII numbers, the same
// normal fix-ups in FP32), so that the triangles and normals are bit for bit
// the reference's. Compiled with -ffp-contract=off.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/aeros_lbm.h"

int set_error(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));

namespace {

uint32_t le32(const unsigned char* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

bool starts_with_solid(const unsigned char* d, uint64_t n) {
    static const char kw[] = "solid";
    if (n < 5) return false;
    for (int i = 0; i < 5; ++i) {
        char c = (char)d[i];
        if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
        if (c != kw[i]) return false;
    }
    return true;
}

// no NUL or control bytes but \t..\r in the first 2 KiB
bool looks_like_text(const unsigned char* d, uint64_t n) {
    const uint64_t lim = n < 2048 ? n : 2048;
    for (uint64_t i = 0; i < lim; ++i) {
        const unsigned char c = d[i];
        if (c == 0 || c < 9 || (c > 13 && c < 32) || c == 127) return false;
    }
    return true;
}

// "facet" or "vertex" (any case) in the first 4 KiB
bool has_keywords(const unsigned char* d, uint64_t n) {
    const uint64_t lim = n < 4096 ? n : 4096;
    for (uint64_t i = 0; i + 5 < lim; ++i) {
        const auto lc = [&](uint64_t k) { return (unsigned char)(d[i + k] | 0x20); };
        if (lc(0) == 'f' && lc(1) == 'a' && lc(2) == 'c' && lc(3) == 'e' && lc(4) == 't') return true;
        if (lc(0) == 'v' && lc(1) == 'e' && lc(2) == 'r' && lc(3) == 't' && lc(4) == 'e' && lc(5) == 'x') return true;
    }
    return false;
}

void detect(const unsigned char* d, uint64_t size, aeros_stl_info* out) {
    std::memset(out, 0, sizeof(*out));
    out->format = AEROS_STL_UNKNOWN;
    if (!d || size == 0) {
        out->reason = AEROS_STL_REASON_EMPTY;
        return;
    }
    const bool solid = starts_with_solid(d, size);
    const bool text = looks_like_text(d, size);
    const bool keywords = text && has_keywords(d, size);
    const uint32_t nt = size >= 84 ? le32(d + 80) : 0u;
    const uint64_t need = 84ull + (uint64_t)nt * 50ull;
    const bool fits = nt > 0 && need <= size;
    out->declared_triangles = nt;
    if (solid && keywords) {   // real text wins over a plausible count
        out->format = AEROS_STL_ASCII;
        out->reason = AEROS_STL_REASON_ASCII;
        return;
    }
    if (fits) {   // enough data for the declared triangles; a tail is allowed
        out->format = AEROS_STL_BINARY;
        out->payload_bytes = (uint64_t)nt * 50ull;
        out->trailing_bytes = size - need;
        out->reason = out->trailing_bytes ? AEROS_STL_REASON_BINARY_TAIL : AEROS_STL_REASON_BINARY;
        return;
    }
    if (text && !solid) {
        out->format = keywords ? AEROS_STL_ASCII : AEROS_STL_UNKNOWN;
        out->reason = keywords ? AEROS_STL_REASON_TEXT_NO_SOLID : AEROS_STL_REASON_TEXT_NO_KEYWORDS;
        return;
    }
    out->reason = (nt > 0 && need > size) ? AEROS_STL_REASON_TRUNCATED : AEROS_STL_REASON_UNRECOGNIZED;
}

struct Out {
    float* v;
    float* n;
    int64_t cap;
    int64_t count = 0;
    void put(const float* tri, const float* nrm3) {   // one triangle, one normal for its three vertices
        if (count < cap) {
            if (v) std::memcpy(v + 9 * count, tri, 36);
            if (n)
                for (int k = 0; k < 3; ++k) std::memcpy(n + 9 * count + 3 * k, nrm3, 12);
        }
        ++count;
    }
};

// binary records: normal (12 B), three vertices (36 B), attribute (2 B)
void parse_binary(const unsigned char* d, uint32_t nt, Out& o, aeros_stl_info* info) {
    uint64_t off = 84;
    for (uint32_t i = 0; i < nt; ++i, off += 50) {
        float n[3];
        std::memcpy(n, d + off, 12);
        if (!std::isfinite(n[0]) || !std::isfinite(n[1]) || !std::isfinite(n[2])) {
            n[0] = 0.0f; n[1] = 0.0f; n[2] = 1.0f;
        }
        const float len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (len > 1e-6f) {
            n[0] /= len; n[1] /= len; n[2] /= len;
        } else {
            n[0] = 0.0f; n[1] = 0.0f; n[2] = 1.0f;
        }
        float v[9];
        std::memcpy(v, d + off + 12, 36);
        bool bad = false;
        for (int k = 0; k < 9 && !bad; ++k) bad = !std::isfinite(v[k]);
        if (bad) {   // a triangle with a non-finite coordinate is dropped whole
            ++info->dropped;
            continue;
        }
        o.put(v, n);
    }
}

std::string lower(std::string s) {
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    return s;
}

// ASCII: "vertex x y z" lines in threes; facet normals are read but the
// output normal is the triangle's own (cross product of its edges).
void parse_ascii(const unsigned char* d, uint64_t size, Out& o, aeros_stl_info* info) {
    std::istringstream iss(std::string(reinterpret_cast<const char*>(d), (size_t)size));
    std::string line;
    std::vector<float> tv;
    uint64_t dropped = 0;
    while (std::getline(iss, line)) {
        line.erase(line.begin(),
                   std::find_if(line.begin(), line.end(), [](unsigned char ch) { return !std::isspace(ch); }));
        if (line.empty()) continue;
        std::istringstream ls(line);
        std::string t;
        ls >> t;
        t = lower(t);
        if (t == "vertex") {
            float x = 0.0f, y = 0.0f, z = 0.0f;
            ls >> x >> y >> z;
            if (!std::isfinite(x) || !std::isfinite(y) || !std::isfinite(z)) {
                ++dropped;
                continue;
            }
            tv.push_back(x);
            tv.push_back(y);
            tv.push_back(z);
        }
    }
    if (dropped % 3 != 0) dropped -= dropped % 3;
    info->dropped = (int64_t)dropped;
    const size_t nv = tv.size() / 3;
    for (size_t i = 0; i + 2 < nv; i += 3) {
        const float* a = &tv[3 * i];
        const float* b = a + 3;
        const float* c = a + 6;
        const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        // glm::cross(e1, e2) and glm::length
        float n[3] = {e1[1] * e2[2] - e2[1] * e1[2], e1[2] * e2[0] - e2[2] * e1[0], e1[0] * e2[1] - e2[0] * e1[1]};
        const float len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (len > 1e-9f) {
            n[0] /= len; n[1] /= len; n[2] /= len;
        } else {
            n[0] = 0.0f; n[1] = 1.0f; n[2] = 0.0f;
        }
        float tri[9];
        std::memcpy(tri, a, 36);
        o.put(tri, n);
    }
}

int parse(const unsigned char* d, uint64_t size, uint64_t budget, float* vertices, float* normals, int64_t capacity,
          aeros_stl_info* info) {
    detect(d, size, info);
    if (size < 10 || size > (2ull << 30)) return set_error(AEROS_ERR_INVALID, "STL size %llu bytes", (unsigned long long)size);
    if (info->format == AEROS_STL_UNKNOWN) return set_error(AEROS_ERR_INVALID, "STL format not recognized");
    Out o{vertices, normals, capacity};
    if (info->format == AEROS_STL_BINARY) {
        const uint64_t need = (uint64_t)info->declared_triangles * 9 * sizeof(float) * 2;
        if (budget && need > budget)
            return set_error(AEROS_ERR_ALLOC, "STL needs %llu bytes, budget %llu", (unsigned long long)need,
                             (unsigned long long)budget);
        parse_binary(d, info->declared_triangles, o, info);
    } else {
        parse_ascii(d, size, o, info);
    }
    info->triangles = o.count;
    if (o.count == 0) return set_error(AEROS_ERR_INVALID, "STL holds no usable triangle");
    return AEROS_OK;
}

}  // namespace

extern "C" int aeros_stl_detect(const uint8_t* data, uint64_t size, aeros_stl_info* info) {
    if (!info) return set_error(AEROS_ERR_INVALID, "info is NULL");
    detect(data, size, info);
    return AEROS_OK;
}

extern "C" int aeros_stl_parse(const uint8_t* data, uint64_t size, uint64_t budget, float* vertices, float* normals,
                               int64_t capacity, aeros_stl_info* info) {
    if (!info || (!data && size) || capacity < 0) return set_error(AEROS_ERR_INVALID, "NULL argument");
    return parse(data, size, budget, vertices, normals, capacity, info);
}

extern "C" int aeros_stl_read_file(const char* path, uint64_t budget, float* vertices, float* normals,
                                   int64_t capacity, aeros_stl_info* info) {
    if (!path || !info || capacity < 0) return set_error(AEROS_ERR_INVALID, "NULL argument");
    std::memset(info, 0, sizeof(*info));
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_error(AEROS_ERR_INVALID, "cannot open %s", path);
    std::vector<unsigned char> buf;
    int rc = AEROS_OK;
    if (std::fseek(f, 0, SEEK_END) != 0) rc = set_error(AEROS_ERR_INVALID, "cannot seek %s", path);
    long sz = rc == AEROS_OK ? std::ftell(f) : -1;
    if (rc == AEROS_OK && (sz < 10 || (unsigned long long)sz > (2ull << 30)))
        rc = set_error(AEROS_ERR_INVALID, "STL size %ld bytes", sz);
    if (rc == AEROS_OK) {
        buf.resize((size_t)sz);
        std::rewind(f);
        if (std::fread(buf.data(), 1, buf.size(), f) != buf.size()) rc = set_error(AEROS_ERR_INVALID, "read %s", path);
    }
    std::fclose(f);
    if (rc != AEROS_OK) return rc;
    return parse(buf.data(), buf.size(), budget, vertices, normals, capacity, info);
}
