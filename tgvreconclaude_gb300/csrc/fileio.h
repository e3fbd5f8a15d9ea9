// Whole-file readers and writers for the reference's binary formats (TGV1 cube
// files, octree_builder.hpp:8-19; TGVS / TGVH / TGVT 12- or 16-byte headers,
// tgv.cpp:16-46, histogram.cpp:167-218, treetop.cpp:93-108).  Host code.
#pragma once
#include <cstdio>
#include <cstring>
#include <vector>

#include "tgvg.h"

namespace tgvg {
namespace fileio {

inline int read_file(const char* path, std::vector<char>& out) {
    FILE* f = path ? std::fopen(path, "rb") : nullptr;
    if (!f) return TGVG_ERR_IO;
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out.resize(sz > 0 ? size_t(sz) : 0);
    size_t got = out.empty() ? 0 : std::fread(out.data(), 1, out.size(), f);
    std::fclose(f);
    return got == out.size() ? TGVG_OK : TGVG_ERR_IO;
}

inline int write_file(const char* path, const void* hdr, size_t nh, const void* body, size_t nb) {
    FILE* f = path ? std::fopen(path, "wb") : nullptr;
    if (!f) return TGVG_ERR_IO;
    bool ok = std::fwrite(hdr, 1, nh, f) == nh;
    if (ok && nb) ok = std::fwrite(body, 1, nb, f) == nb;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? TGVG_OK : TGVG_ERR_IO;
}

inline uint32_t u32_at(const std::vector<char>& b, size_t off) {
    uint32_t v;
    std::memcpy(&v, b.data() + off, 4);
    return v;
}

// TGV1 cube file (octree_builder.hpp:8-19): 16-byte header then cubes.
inline int load_cube_file(const char* path, std::vector<tgvg_cube>& cubes, float* r_root) {
    std::vector<char> b;
    int rc = read_file(path, b);
    if (rc) return rc;
    if (b.size() < 16 || std::memcmp(b.data(), "TGV1", 4) != 0) return TGVG_ERR_FORMAT;
    uint32_t n = u32_at(b, 12);
    if (b.size() < 16 + size_t(n) * sizeof(tgvg_cube)) return TGVG_ERR_FORMAT;
    if (r_root) std::memcpy(r_root, b.data() + 8, 4);
    cubes.resize(n);
    if (n) std::memcpy(cubes.data(), b.data() + 16, size_t(n) * sizeof(tgvg_cube));
    return TGVG_OK;
}


}  // namespace fileio
}  // namespace tgvg
