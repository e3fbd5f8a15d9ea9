// Link-time drop-in for the reference's Stage-7 surface extraction
// (src/marching_cubes.cpp).  Compile against the reference's headers and link
// with libtgvg.so in place of src/marching_cubes.cpp; the extraction runs on
// the GPU through include/tgvg.h with the reference's signatures, results
// (bit-identical meshes) and errors (std::runtime_error "Cannot open: ...").
//
// Replaces, one for one:
//   extract_surface             marching_cubes.cpp:63-181
//   compute_normals             marching_cubes.cpp:185-205
//   extract_surface_streaming   marching_cubes.cpp:374-580
//   write_obj                   marching_cubes.cpp:584-619
#include "marching_cubes.hpp"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "tgvg.h"
#include "dropin_ctx.h"

static_assert(sizeof(OctreeCube) == sizeof(tgvg_cube), "OctreeCube layout");
static_assert(sizeof(TGVCube) == sizeof(tgvg_state), "TGVCube layout");

namespace {

void flatten(const Mesh& m, std::vector<float>& v) {
    v.resize(m.verts.size() * 3);
    for (size_t i = 0; i < m.verts.size(); ++i)
        for (int k = 0; k < 3; ++k) v[3 * i + k] = m.verts[i][k];
}

}  // namespace

Mesh extract_surface(const std::vector<OctreeCube>& cubes, const std::vector<TGVCube>& state, const Vec3f& origin,
                     float r_root, const std::vector<bool>& has_data) {
    Mesh mesh;
    if (cubes.empty()) return mesh;
    std::vector<uint8_t> hd;
    if (!has_data.empty()) {
        hd.resize(cubes.size());
        for (size_t i = 0; i < cubes.size(); ++i) hd[i] = has_data[i] ? 1 : 0;
    }
    const float o[3] = {origin.x(), origin.y(), origin.z()};
    tgvg_mesh* m = nullptr;
    tgvg_dropin_check(tgvg_extract_surface(tgvg_dropin_ctx(), reinterpret_cast<const tgvg_cube*>(cubes.data()),
                                           reinterpret_cast<const tgvg_state*>(state.data()),
                                           int64_t(cubes.size()), hd.empty() ? nullptr : hd.data(), o, r_root, 0,
                                           &m),
                      "extract_surface");
    int64_t nv = 0, nf = 0;
    tgvg_mesh_size(m, &nv, &nf, nullptr);
    std::vector<float> v(size_t(nv) * 3);
    mesh.faces.resize(size_t(nf) * 3);
    tgvg_mesh_read(m, v.data(), mesh.faces.data(), nullptr);
    tgvg_mesh_free(m);
    mesh.verts.resize(size_t(nv));
    for (int64_t i = 0; i < nv; ++i) mesh.verts[i] = Vec3f(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    return mesh;
}

void compute_normals(Mesh& mesh) {
    std::vector<float> v, n(mesh.verts.size() * 3);
    flatten(mesh, v);
    tgvg_dropin_check(tgvg_compute_normals(tgvg_dropin_ctx(), v.data(), int64_t(mesh.verts.size()),
                                           mesh.faces.data(), int64_t(mesh.tri_count()), n.data()),
                      "compute_normals");
    mesh.normals.resize(mesh.verts.size());
    for (size_t i = 0; i < mesh.verts.size(); ++i) mesh.normals[i] = Vec3f(n[3 * i], n[3 * i + 1], n[3 * i + 2]);
}

void write_obj(const std::string& path, const Mesh& mesh) {
    std::vector<float> v, n;
    flatten(mesh, v);
    if (!mesh.normals.empty()) {
        n.resize(mesh.normals.size() * 3);
        for (size_t i = 0; i < mesh.normals.size(); ++i)
            for (int k = 0; k < 3; ++k) n[3 * i + k] = mesh.normals[i][k];
    }
    const int rc = tgvg_write_obj(path.c_str(), v.data(), int64_t(mesh.verts.size()), mesh.faces.data(),
                                  int64_t(mesh.tri_count()), n.empty() ? nullptr : n.data());
    if (rc != TGVG_OK) throw std::runtime_error("Cannot open: " + path);
}

void extract_surface_streaming(const std::string& balanced_cube_path, const std::string& tgv_state_path,
                               const std::string& treetop_path, const std::string& hist_path, const Vec3f& origin,
                               float r_root, const std::string& out_obj_path) {
    const float o[3] = {origin.x(), origin.y(), origin.z()};
    const int rc = tgvg_extract_surface_streaming(tgvg_dropin_ctx(), balanced_cube_path.c_str(),
                                                  tgv_state_path.c_str(), treetop_path.c_str(), hist_path.c_str(),
                                                  o, r_root, out_obj_path.c_str());
    if (rc == TGVG_ERR_IO || rc == TGVG_ERR_FORMAT) throw std::runtime_error(tgvg_last_error(tgvg_dropin_ctx()));
    tgvg_dropin_check(rc, "extract_surface_streaming");
}
