// Link-time replacement of the reference's src/octree_builder.cpp,
// src/merge.cpp and src/balance.cpp: every function their headers declare,
// with the reference's signatures and error behaviour.  Stage 1
// (build_cubes_from_depthmap), Stage 2 (kway_merge) and Stage 3
// (balance_octree) run on the GPU through the C ABI; the small host helpers
// (cube files, the depth rule, Morton neighbours) are plain C++ here.
#include <cmath>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "balance.hpp"
#include "dropin_ctx.h"
#include "merge.hpp"
#include "octree_builder.hpp"

static_assert(sizeof(OctreeCube) == sizeof(tgvg_cube), "OctreeCube layout");

// ---- octree_builder.hpp ------------------------------------------------------

// octree_builder.hpp:38-43: the depth whose cell r_root / 2^d is nearest
// 1.125 r_x on a log scale, nudged (at most three steps) into [0.75 r_x, 1.5 r_x),
// clamped to [0, max_depth]; max_depth for r_x <= 0.
int cube_depth_for_radius(float r_x, float r_root, int max_depth) {
    if (r_x <= 0.0f) return max_depth;
    const float l = std::round(std::log2(r_root / (r_x * 1.125f)));
    // (int) of a non-finite or huge value: the x86-64 result, INT_MIN
    int d = (l > -2147483904.0f && l < 2147483648.0f) ? static_cast<int>(l) : static_cast<int>(0x80000000u);
    d = d < 0 ? 0 : (d > max_depth ? max_depth : d);
    for (int step = 0; step < 3; ++step) {
        const float cell = r_root / static_cast<float>(1u << d);
        const bool small = cell < 0.75f * r_x, large = !(cell < 1.5f * r_x);
        if (!small && !large) break;
        if (small) {
            if (d == 0) break;
            --d;
        } else {
            if (d == max_depth) break;
            ++d;
        }
    }
    return d;
}

void build_cubes_from_depthmap(const DepthMap& dm, const Vec3f& scene_origin, float r_root,
                               const std::string& out_path) {
    tgvg_depthmap m{};
    m.fx = dm.K(0, 0);
    m.fy = dm.K(1, 1);
    m.cx = dm.K(0, 2);
    m.cy = dm.K(1, 2);
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m.rt[4 * r + c] = dm.Rt(r, c);
    m.width = dm.width;
    m.height = dm.height;
    m.depths = dm.depths.data();
    const float o[3] = {scene_origin[0], scene_origin[1], scene_origin[2]};
    tgvg_dropin_check(tgvg_build_cubes_file(tgvg_dropin_ctx(), &m, o, r_root, out_path.c_str()),
                      "build_cubes_from_depthmap");
}

static std::ifstream open_cube_file(const std::string& path, CubeFileHeader& hdr) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("Cannot open cube file: " + path);
    in.read(reinterpret_cast<char*>(&hdr), sizeof(hdr));
    if (std::memcmp(hdr.magic, "TGV1", 4) != 0) throw std::runtime_error("Bad magic in cube file: " + path);
    return in;
}

std::vector<OctreeCube> load_cubes(const std::string& path, float& r_root_out) {
    CubeFileHeader hdr;
    std::ifstream in = open_cube_file(path, hdr);
    r_root_out = hdr.r_root;
    std::vector<OctreeCube> cubes(hdr.cube_count);
    if (!cubes.empty()) in.read(reinterpret_cast<char*>(cubes.data()), cubes.size() * sizeof(OctreeCube));
    return cubes;
}

std::vector<OctreeCube> load_cubes_range(const std::string& path, uint32_t first_idx, uint32_t last_idx,
                                         float& r_root_out) {
    CubeFileHeader hdr;
    std::ifstream in = open_cube_file(path, hdr);
    r_root_out = hdr.r_root;
    if (first_idx >= hdr.cube_count || first_idx > last_idx) return {};
    const uint32_t end = last_idx + 1 < hdr.cube_count ? last_idx + 1 : hdr.cube_count;
    std::vector<OctreeCube> cubes(end - first_idx);
    in.seekg(static_cast<std::streamoff>(sizeof(CubeFileHeader)) +
             static_cast<std::streamoff>(first_idx) * static_cast<std::streamoff>(sizeof(OctreeCube)));
    in.read(reinterpret_cast<char*>(cubes.data()), cubes.size() * sizeof(OctreeCube));
    return cubes;
}

// ---- merge.hpp ----------------------------------------------------------------

void kway_merge(const std::vector<std::string>& in_paths, const std::string& out_path) {
    std::vector<const char*> p;
    for (const auto& s : in_paths) p.push_back(s.c_str());
    tgvg_dropin_check(tgvg_kway_merge(tgvg_dropin_ctx(), p.data(), static_cast<int32_t>(p.size()), out_path.c_str()),
                      "kway_merge");
}

// ---- balance.hpp --------------------------------------------------------------

static uint64_t as_u64(const MortonCode& m) { return (static_cast<uint64_t>(m.hi) << 32) | m.lo; }

MortonCode parent_code(const MortonCode& code, int current_depth) {
    // ancestor at current_depth - 1: clear the low 3 * (22 - current_depth) bits
    const unsigned sh = 3u * (21u - static_cast<unsigned>(current_depth - 1));
    const uint64_t v = sh >= 64u ? 0 : as_u64(code) & ~((uint64_t(1) << sh) - 1);
    return MortonCode{static_cast<uint32_t>(v >> 32), static_cast<uint32_t>(v)};
}

MortonCode face_neighbor(const MortonCode& code, int face, int depth) {
    const MortonCode none{UINT32_MAX, UINT32_MAX};
    if (face < 0 || face > 5) return none;
    uint32_t c[3];
    morton_decode(code, c[0], c[1], c[2]);
    const uint32_t step = 1u << (21 - depth);
    uint32_t& a = c[face / 2];
    if (face % 2 == 0) {
        if (a + step >= (1u << 21)) return none;
        a += step;
    } else {
        if (a < step) return none;
        a -= step;
    }
    return morton_encode(c[0], c[1], c[2]);
}

void balance_octree(const std::string& in_path, const std::string& out_path) {
    tgvg_dropin_check(tgvg_balance_octree(tgvg_dropin_ctx(), in_path.c_str(), out_path.c_str()), "balance_octree");
}
