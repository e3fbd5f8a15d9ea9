// extern "C" wrapper over the reference's own Stage-5/Stage-6 functions
// (histogram.cpp, tgv.cpp), so that Python tests can call the unmodified
// reference through ctypes.
//
// TEST INFRASTRUCTURE ONLY.  It is compiled, together with the reference's
// src/*.cpp and the project-written Eigen/TBB shims under oracle/shim, into
// oracle/_ref/libref.so by oracle/Makefile.  It is used to pin the oracle
// restatement (oracle/tgv_oracle.cpp) and to generate the committed golden
// fixtures; nothing in the product links or loads it.
#include "histogram.hpp"
#include "tgv.hpp"
#include "treetop.hpp"
#include "balance.hpp"
#include "octree_builder.hpp"
#include "merge.hpp"
#include "marching_cubes.hpp"

#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

static_assert(sizeof(OctreeCube) == 16, "OctreeCube layout");
static_assert(sizeof(CubeHistogram) == 32, "CubeHistogram layout");
static_assert(sizeof(TGVCube) == 52, "TGVCube layout");
static_assert(sizeof(TreetopLeaf) == 20, "TreetopLeaf layout");

extern "C" {

// One base depth map: K (fx, fy, cx, cy), Rt row-major 4x4 (world<-camera),
// W x H depths row-major.
struct RefDepthMap {
    float fx, fy, cx, cy;
    float rt[16];
    int32_t width, height;
    int32_t lidar;
    const float* depths;
};

static void fill_dm(const RefDepthMap& s, DepthMap& dm) {
    dm.width = s.width;
    dm.height = s.height;
    dm.depths.assign(s.depths, s.depths + static_cast<size_t>(s.width) * s.height);
    dm.K = Eigen::Matrix3f::Identity();
    dm.K(0, 0) = s.fx; dm.K(1, 1) = s.fy; dm.K(0, 2) = s.cx; dm.K(1, 2) = s.cy;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) dm.Rt(i, j) = s.rt[i * 4 + j];
}

// DepthMipmap::build for one map.  Writes Rt_inv (row-major) and the level
// count; if `levels_out` is non-null it receives every level's texels
// concatenated (level 0 first).  Returns the total texel count.
int64_t ref_mipmap_build(const RefDepthMap* s, float* rt_inv_out, int32_t* n_levels_out,
                         int32_t* dims_out /* 2 per level, may be null */, float* levels_out) {
    DepthMap dm;
    fill_dm(*s, dm);
    DepthMipmap mm;
    mm.build(dm, s->lidar != 0);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) rt_inv_out[i * 4 + j] = mm.Rt_inv(i, j);
    *n_levels_out = static_cast<int32_t>(mm.levels.size());
    int64_t total = 0;
    for (size_t l = 0; l < mm.levels.size(); ++l) {
        const DepthMap& lv = mm.levels[l];
        if (dims_out) { dims_out[2 * l] = lv.width; dims_out[2 * l + 1] = lv.height; }
        if (levels_out)
            std::memcpy(levels_out + total, lv.depths.data(), lv.depths.size() * sizeof(float));
        total += static_cast<int64_t>(lv.depths.size());
    }
    return total;
}

// DepthMipmap::project for one point against one map.
int ref_project(const RefDepthMap* s, float px, float py, float pz, float r_c,
                int32_t* level, int32_t* u, int32_t* v, float* cam_z) {
    DepthMap dm;
    fill_dm(*s, dm);
    DepthMipmap mm;
    mm.build(dm, s->lidar != 0);
    int lv = -1, uu = -1, vv = -1;
    float cz = 0.0f;
    bool ok = mm.project(Vec3f{px, py, pz}, r_c, lv, uu, vv, cz);
    *level = lv; *u = uu; *v = vv; *cam_z = cz;
    return ok ? 1 : 0;
}

// compute_histograms over `n` cubes and `ncam` maps.  out: n * 8 uint32.
int ref_compute_histograms(const OctreeCube* cubes, int64_t n, const RefDepthMap* maps,
                           int32_t ncam, float ox, float oy, float oz, float r_root,
                           uint32_t* out) {
    try {
        std::vector<OctreeCube> cv(cubes, cubes + n);
        std::vector<DepthMipmap> mms(ncam);
        for (int c = 0; c < ncam; ++c) {
            DepthMap dm;
            fill_dm(maps[c], dm);
            mms[c].build(dm, maps[c].lidar != 0);
        }
        auto h = compute_histograms(cv, mms, Vec3f{ox, oy, oz}, r_root);
        std::memcpy(out, h.data(), h.size() * sizeof(CubeHistogram));
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// compute_histograms_oc: cubes and output through files, exactly like main.cpp.
int ref_compute_histograms_oc(const char* cube_path, const TreetopLeaf* leaves, int32_t nleaf,
                              const RefDepthMap* maps, int32_t ncam, float ox, float oy,
                              float oz, float r_root, const char* out_path) {
    try {
        std::vector<TreetopLeaf> lv(leaves, leaves + nleaf);
        std::vector<DepthMipmap> mms(ncam);
        for (int c = 0; c < ncam; ++c) {
            DepthMap dm;
            fill_dm(maps[c], dm);
            mms[c].build(dm, maps[c].lidar != 0);
        }
        compute_histograms_oc(cube_path, lv, mms, Vec3f{ox, oy, oz}, r_root, out_path);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

float ref_median_indicator(const uint32_t* bins8) {
    CubeHistogram h;
    std::memcpy(h.bins, bins8, sizeof(h.bins));
    return h.median_indicator();
}

float ref_mean_indicator(const uint32_t* bins8) {
    CubeHistogram h;
    std::memcpy(h.bins, bins8, sizeof(h.bins));
    return h.mean_indicator();
}

int ref_tgv_minimize(const OctreeCube* cubes, const CubeHistogram* hists, int64_t n,
                     float alpha0, float alpha1, int32_t iters, float r_root, TGVCube* out) {
    try {
        std::vector<OctreeCube> cv(cubes, cubes + n);
        std::vector<CubeHistogram> hv(hists, hists + n);
        TGVParams p;
        p.alpha0 = alpha0; p.alpha1 = alpha1; p.iters = iters;
        auto s = tgv_minimize(cv, hv, Vec3f::Zero(), r_root, p);
        std::memcpy(out, s.data(), s.size() * sizeof(TGVCube));
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

int ref_tgv_minimize_oc(const OctreeCube* cubes, const CubeHistogram* hists, int64_t n,
                        const TreetopLeaf* leaves, int32_t nleaf, float alpha0, float alpha1,
                        int32_t iters, float r_root, TGVCube* out) {
    try {
        std::vector<OctreeCube> cv(cubes, cubes + n);
        std::vector<CubeHistogram> hv(hists, hists + n);
        std::vector<TreetopLeaf> lv(leaves, leaves + nleaf);
        TGVParams p;
        p.alpha0 = alpha0; p.alpha1 = alpha1; p.iters = iters;
        auto s = tgv_minimize_oc(cv, hv, lv, Vec3f::Zero(), r_root, p);
        std::memcpy(out, s.data(), s.size() * sizeof(TGVCube));
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

int ref_tgv_minimize_streaming(const char* cube_path, const char* hist_path,
                               const char* treetop_path, float r_root, const char* out_path,
                               float alpha0, float alpha1, int32_t iters) {
    try {
        TGVParams p;
        p.alpha0 = alpha0; p.alpha1 = alpha1; p.iters = iters;
        tgv_minimize_streaming(cube_path, hist_path, treetop_path, Vec3f::Zero(), r_root,
                               out_path, p);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

void ref_parent_code(uint32_t hi, uint32_t lo, int32_t depth, uint32_t* out_hi, uint32_t* out_lo) {
    MortonCode m{hi, lo};
    MortonCode r = parent_code(m, depth);
    *out_hi = r.hi; *out_lo = r.lo;
}

void ref_face_neighbor(uint32_t hi, uint32_t lo, int32_t face, int32_t depth, uint32_t* out_hi,
                       uint32_t* out_lo) {
    MortonCode m{hi, lo};
    MortonCode r = face_neighbor(m, face, depth);
    *out_hi = r.hi; *out_lo = r.lo;
}

// Stage-1/2/3/4 (out of the hot path) are exposed only so that fixture scripts
// can produce realistic balanced cube sets from depth maps.
int ref_build_cubes_from_depthmap(const RefDepthMap* s, float ox, float oy, float oz,
                                  float r_root, const char* out_path) {
    try {
        DepthMap dm;
        fill_dm(*s, dm);
        build_cubes_from_depthmap(dm, Vec3f{ox, oy, oz}, r_root, out_path);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

int ref_kway_merge(const char* const* in_paths, int32_t n, const char* out_path) {
    try {
        std::vector<std::string> v;
        for (int i = 0; i < n; ++i) v.emplace_back(in_paths[i]);
        kway_merge(v, out_path);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

int ref_balance_octree(const char* in_path, const char* out_path) {
    try {
        balance_octree(in_path, out_path);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

int ref_build_treetop(const char* in_path, const char* out_path) {
    try {
        build_treetop(in_path, out_path);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// extract_surface (+ compute_normals) over caller arrays.  The mesh is kept in
// a heap object; ref_mesh_read copies it out and ref_mesh_free releases it.
struct RefMesh {
    Mesh m;
};

void* ref_extract_surface(const OctreeCube* cubes, const TGVCube* state, int64_t n, const uint8_t* has_data,
                          float ox, float oy, float oz, float r_root, int32_t normals, int64_t* nv,
                          int64_t* nf) {
    try {
        std::vector<OctreeCube> cv(cubes, cubes + n);
        std::vector<TGVCube> sv(state, state + n);
        std::vector<bool> hd;
        if (has_data) {
            hd.resize(static_cast<size_t>(n));
            for (int64_t i = 0; i < n; ++i) hd[i] = has_data[i] != 0;
        }
        auto* r = new RefMesh;
        r->m = extract_surface(cv, sv, Vec3f(ox, oy, oz), r_root, hd);
        if (normals) compute_normals(r->m);
        *nv = static_cast<int64_t>(r->m.verts.size());
        *nf = static_cast<int64_t>(r->m.tri_count());
        return r;
    } catch (const std::exception&) {
        return nullptr;
    }
}

void ref_mesh_read(void* h, float* verts, uint32_t* faces, float* normals) {
    const Mesh& m = static_cast<RefMesh*>(h)->m;
    for (size_t i = 0; i < m.verts.size(); ++i)
        for (int k = 0; k < 3; ++k) verts[3 * i + k] = m.verts[i][k];
    std::memcpy(faces, m.faces.data(), m.faces.size() * sizeof(uint32_t));
    if (normals)
        for (size_t i = 0; i < m.normals.size(); ++i)
            for (int k = 0; k < 3; ++k) normals[3 * i + k] = m.normals[i][k];
}

int ref_mesh_write_obj(void* h, const char* path) {
    try {
        write_obj(path, static_cast<RefMesh*>(h)->m);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

void ref_mesh_free(void* h) { delete static_cast<RefMesh*>(h); }

int ref_extract_surface_streaming(const char* cube_path, const char* state_path, const char* treetop_path,
                                  const char* hist_path, float ox, float oy, float oz, float r_root,
                                  const char* out_obj) {
    try {
        extract_surface_streaming(cube_path, state_path, treetop_path, hist_path, Vec3f(ox, oy, oz), r_root,
                                  out_obj);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

}  // extern "C"
