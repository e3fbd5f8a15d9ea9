// Link-time drop-in for the reference's Stage-5/6 sources.
//
// Compile this file against the reference's own headers (src/histogram.hpp,
// src/tgv.hpp and what they include) and link it, together with
// libtgvg.so, in place of src/histogram.cpp and src/tgv.cpp.  Every function
// below keeps the reference's signature and behaviour (including
// std::runtime_error on I/O errors and empty results for empty inputs); the
// compute runs on the GPU through the C ABI in include/tgvg.h.
//
// Replaces, one for one:
//   CubeHistogram::mean_indicator / median_indicator  histogram.cpp:12-31
//   DepthMipmap::build / project / depth_at           histogram.cpp:35-113
//   compute_histograms                                histogram.cpp:127-163
//   save_histograms / load_histograms(_range)         histogram.cpp:175-218
//   compute_histograms_oc                             histogram.cpp:222-256
//   save_tgv / load_tgv                               tgv.cpp:24-46
//   tgv_minimize / tgv_minimize_oc                    tgv.cpp:356-511
//   tgv_minimize_streaming                            tgv.cpp:802-1070
#include "histogram.hpp"
#include "tgv.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <limits>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "tgvg.h"
#include "dropin_ctx.h"

static_assert(sizeof(OctreeCube) == sizeof(tgvg_cube), "OctreeCube layout");
static_assert(sizeof(TGVCube) == sizeof(tgvg_state), "TGVCube layout");
static_assert(sizeof(TreetopLeaf) == sizeof(tgvg_leaf), "TreetopLeaf layout");
static_assert(sizeof(CubeHistogram) == 32, "CubeHistogram layout");

namespace {

tgvg_ctx* ctx() { return tgvg_dropin_ctx(); }
void check(int rc, const char* what) { tgvg_dropin_check(rc, what); }

tgvg_camera camera_of(const DepthMipmap& m) {
    tgvg_camera c{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) c.rt_inv[i * 4 + j] = m.Rt_inv(i, j);
    const DepthMap& b = m.levels.front();
    c.fx = b.K(0, 0); c.fy = b.K(1, 1); c.cx = b.K(0, 2); c.cy = b.K(1, 2);
    c.width = b.width; c.height = b.height;
    c.lidar = m.lidar ? 1 : 0;
    return c;
}

tgvg_params params_of(const TGVParams& p) {
    tgvg_params q{};
    q.alpha0 = p.alpha0; q.alpha1 = p.alpha1; q.iters = p.iters;
    q.init = TGVG_INIT_MEDIAN; q.tol = 0.0f; q.check_every = 0;
    return q;
}

int trunc_i32(float x) {
    if (!(x > -2147483904.0f && x < 2147483648.0f)) return std::numeric_limits<int>::min();
    return static_cast<int>(x);
}

}  // namespace

// ---- CubeHistogram --------------------------------------------------------------
float CubeHistogram::mean_indicator() const {
    uint32_t tot = total();
    if (tot == 0) return 0.0f;
    float sum = 0.0f;
    for (int k = 0; k < 8; ++k) sum += bins[k] * (-1.0f + (k + 0.5f) / 4.0f);
    return sum / tot;
}

float CubeHistogram::median_indicator() const {
    uint32_t tot = total();
    if (tot == 0) return 0.0f;
    uint32_t cum = 0;
    for (int k = 0; k < 8; ++k) {
        cum += bins[k];
        if (cum * 2 >= tot) return -1.0f + (k + 0.5f) / 4.0f;
    }
    return 1.0f;
}

// ---- DepthMipmap: pyramid built on the GPU ------------------------------------------
void DepthMipmap::build(const DepthMap& base, bool is_lidar) {
    lidar = is_lidar;
    Rt_inv = base.Rt.inverse();
    levels.clear();
    int32_t dims[26];
    const int nl = tgvg_pyramid_dims(base.width, base.height, dims);
    if (nl <= 0) { levels.push_back(base); return; }
    std::vector<float> all;
    size_t total = 0;
    for (int l = 0; l < nl; ++l) total += size_t(dims[2 * l]) * dims[2 * l + 1];
    all.resize(total);
    tgvg_camera c{};
    c.width = base.width; c.height = base.height;
    const float* bp = base.depths.data();
    float* op = all.data();
    check(tgvg_build_pyramids(ctx(), &c, 1, &bp, &op), "DepthMipmap::build");
    size_t off = 0;
    for (int l = 0; l < nl; ++l) {
        DepthMap d;
        d.width = dims[2 * l];
        d.height = dims[2 * l + 1];
        d.K = base.K;
        for (int k = 0; k < l; ++k) {  // K halves per level (histogram.cpp:49-52)
            d.K(0, 0) *= 0.5f; d.K(1, 1) *= 0.5f;
            d.K(0, 2) = d.K(0, 2) * 0.5f; d.K(1, 2) = d.K(1, 2) * 0.5f;
        }
        d.Rt = base.Rt;
        d.depths.assign(all.begin() + off, all.begin() + off + size_t(d.width) * d.height);
        off += size_t(d.width) * d.height;
        levels.push_back(std::move(d));
    }
}

bool DepthMipmap::project(const Vec3f& P, float r_c, int& level_out, int& u_out, int& v_out,
                          float& cam_z_out) const {
    if (levels.empty()) return false;
    const DepthMap& base = levels[0];
    Eigen::Vector4f Pw{P.x(), P.y(), P.z(), 1.0f};
    Eigen::Vector4f cam = Rt_inv * Pw;
    float z = cam.z();
    if (z <= 0.0f) return false;
    float fx = base.K(0, 0), fy = base.K(1, 1), cx = base.K(0, 2), cy = base.K(1, 2);
    float u_f = cam.x() / z * fx + cx;
    float v_f = cam.y() / z * fy + cy;
    int u0 = trunc_i32(u_f), v0 = trunc_i32(v_f);
    if (u0 < 0 || u0 >= base.width || v0 < 0 || v0 >= base.height) return false;
    cam_z_out = z;
    float footprint = std::abs(fx) * r_c / z;
    int level = std::max(0, trunc_i32(std::log2(std::max(1.0f, footprint))));
    level = std::min(level, static_cast<int>(levels.size()) - 1);
    level_out = level;
    u_out = std::clamp(u0 >> level, 0, levels[level].width - 1);
    v_out = std::clamp(v0 >> level, 0, levels[level].height - 1);
    return true;
}

float DepthMipmap::depth_at(int level, int u, int v) const {
    if (level < 0 || level >= (int)levels.size()) return std::numeric_limits<float>::quiet_NaN();
    const DepthMap& lm = levels[level];
    if (u < 0 || u >= lm.width || v < 0 || v >= lm.height) return std::numeric_limits<float>::quiet_NaN();
    return lm.depths[v * lm.width + u];
}

// ---- histograms --------------------------------------------------------------------
std::vector<CubeHistogram> compute_histograms(const std::vector<OctreeCube>& cubes,
                                              const std::vector<DepthMipmap>& depth_maps,
                                              const Vec3f& scene_origin, float r_root) {
    std::vector<CubeHistogram> out(cubes.size());
    if (cubes.empty()) return out;
    std::vector<tgvg_camera> cams;
    std::vector<std::vector<float>> flat;
    std::vector<const float*> ptr;
    for (const auto& m : depth_maps) {
        if (m.levels.empty()) continue;
        cams.push_back(camera_of(m));
        std::vector<float> f;
        for (const auto& l : m.levels) f.insert(f.end(), l.depths.begin(), l.depths.end());
        flat.push_back(std::move(f));
    }
    for (auto& f : flat) ptr.push_back(f.data());
    const float o[3] = {scene_origin.x(), scene_origin.y(), scene_origin.z()};
    check(tgvg_compute_histograms_pyr(ctx(), reinterpret_cast<const tgvg_cube*>(cubes.data()),
                                      (int64_t)cubes.size(), cams.data(), (int32_t)cams.size(), ptr.data(), o,
                                      r_root, 8, reinterpret_cast<uint32_t*>(out.data())),
          "compute_histograms");
    return out;
}

void compute_histograms_oc(const std::string& balanced_cube_path, const std::vector<TreetopLeaf>& leaves,
                           const std::vector<DepthMipmap>& depth_maps, const Vec3f& scene_origin,
                           float r_root, const std::string& out_hist_path) {
    std::vector<tgvg_camera> cams;
    std::vector<const float*> base;
    for (const auto& m : depth_maps) {
        if (m.levels.empty()) continue;
        cams.push_back(camera_of(m));
        base.push_back(m.levels[0].depths.data());
    }
    const float o[3] = {scene_origin.x(), scene_origin.y(), scene_origin.z()};
    check(tgvg_compute_histograms_oc(ctx(), balanced_cube_path.c_str(),
                                     reinterpret_cast<const tgvg_leaf*>(leaves.data()), (int32_t)leaves.size(),
                                     cams.data(), (int32_t)cams.size(), base.data(), o, r_root,
                                     out_hist_path.c_str()),
          "compute_histograms_oc");
}

void save_histograms(const std::string& path, const std::vector<CubeHistogram>& hists) {
    if (tgvg_save_histograms(path.c_str(), reinterpret_cast<const uint32_t*>(hists.data()),
                             (int64_t)hists.size()) != TGVG_OK)
        throw std::runtime_error("Cannot open: " + path);
}

std::vector<CubeHistogram> load_histograms(const std::string& path) {
    int64_t n = tgvg_load_histograms(path.c_str(), nullptr, 0);
    if (n == TGVG_ERR_FORMAT) throw std::runtime_error("Bad histogram magic");
    if (n < 0) throw std::runtime_error("Cannot open: " + path);
    std::vector<CubeHistogram> h(n);
    if (n > 0) tgvg_load_histograms(path.c_str(), reinterpret_cast<uint32_t*>(h.data()), n);
    return h;
}

std::vector<CubeHistogram> load_histograms_range(const std::string& path, uint32_t first_idx,
                                                 uint32_t last_idx) {
    auto all = load_histograms(path);
    if (first_idx >= all.size() || first_idx > last_idx) return {};
    uint32_t end = std::min<uint32_t>(last_idx + 1, (uint32_t)all.size());
    return std::vector<CubeHistogram>(all.begin() + first_idx, all.begin() + end);
}

// ---- TGV -----------------------------------------------------------------------------
void save_tgv(const std::string& path, const std::vector<TGVCube>& state) {
    if (tgvg_save_tgv(path.c_str(), reinterpret_cast<const tgvg_state*>(state.data()),
                      (int64_t)state.size()) != TGVG_OK)
        throw std::runtime_error("Cannot open: " + path);
}

std::vector<TGVCube> load_tgv(const std::string& path) {
    int64_t n = tgvg_load_tgv(path.c_str(), nullptr, 0);
    if (n == TGVG_ERR_FORMAT) throw std::runtime_error("Bad TGV state magic");
    if (n < 0) throw std::runtime_error("Cannot open: " + path);
    std::vector<TGVCube> s(n);
    if (n > 0) tgvg_load_tgv(path.c_str(), reinterpret_cast<tgvg_state*>(s.data()), n);
    return s;
}

static std::vector<TGVCube> solve(const std::vector<OctreeCube>& cubes, const std::vector<CubeHistogram>& hists,
                                  const std::vector<TreetopLeaf>* leaves, int mode, const TGVParams& params) {
    std::vector<TGVCube> state(cubes.size());
    if (cubes.empty()) return state;
    tgvg_params p = params_of(params);
    check(tgvg_tgv_minimize(ctx(), reinterpret_cast<const tgvg_cube*>(cubes.data()),
                            reinterpret_cast<const uint32_t*>(hists.data()), (int64_t)cubes.size(), 8,
                            leaves ? reinterpret_cast<const tgvg_leaf*>(leaves->data()) : nullptr,
                            leaves ? (int32_t)leaves->size() : 0, mode, &p, nullptr,
                            reinterpret_cast<tgvg_state*>(state.data()), nullptr),
          "tgv_minimize");
    return state;
}

std::vector<TGVCube> tgv_minimize(const std::vector<OctreeCube>& cubes, const std::vector<CubeHistogram>& hists,
                                  const Vec3f& /*origin*/, float /*r_root*/, const TGVParams& params) {
    return solve(cubes, hists, nullptr, TGVG_MODE_INMEM, params);
}

std::vector<TGVCube> tgv_minimize_oc(const std::vector<OctreeCube>& cubes, const std::vector<CubeHistogram>& hists,
                                     const std::vector<TreetopLeaf>& leaves, const Vec3f& /*origin*/,
                                     float /*r_root*/, const TGVParams& params) {
    return solve(cubes, hists, &leaves, TGVG_MODE_OC, params);
}

void tgv_minimize_streaming(const std::string& balanced_cube_path, const std::string& hist_path,
                            const std::string& treetop_path, const Vec3f& /*origin*/, float /*r_root*/,
                            const std::string& out_state_path, const TGVParams& params) {
    tgvg_params p = params_of(params);
    check(tgvg_tgv_minimize_streaming(ctx(), balanced_cube_path.c_str(), hist_path.c_str(), treetop_path.c_str(),
                                      out_state_path.c_str(), &p, nullptr),
          "tgv_minimize_streaming");
}
