// Stage 1 on the GPU: the cubes of one depth map (the reference's
// build_cubes_from_depthmap, src/octree_builder.cpp:30-97, with
// cube_depth_for_radius :11-28 and DepthMap::unproject / sample_radius,
// src/depth_map.cpp:4-30).
//
// One thread per pixel: validity, the sample radius from the valid 4-neighbours,
// the world point, its place in the scene box, the cube depth for the radius
// and the Morton code; then a compaction and a stable radix sort by code.  The
// float arithmetic is the reference's, in its order, with explicitly rounded
// intrinsics (Eigen's 4x4 matvec and norms as the project's Eigen subset
// evaluates them).  round(log2(y)) of the depth rule is not evaluated on the
// device: the host finds, with its own log2f, the 21 thresholds where it
// reaches 1..21, and the kernel counts the thresholds below y.
//
// Cubes with equal codes come out in pixel order; the reference's std::sort
// leaves their order unspecified (and its parallel row loop makes the
// pre-sort order scheduling-dependent), so only the multiset of cubes is the
// reference's.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "common.cuh"
#include "fileio.h"

namespace tgvg {

struct DmDev {
    float fx, fy, cx, cy;
    float rt[16];  // world <- camera, row-major
    int w, h;
};

__device__ __forceinline__ bool dm_valid(const float* __restrict__ dep, const DmDev& m, int u, int v) {
    if (u < 0 || v < 0 || u >= m.w || v >= m.h) return false;
    const float d = dep[(size_t)v * m.w + u];
    return isfinite(d) && d > 0.0f;
}

// DepthMap::unproject (depth_map.cpp:4-11): cam = ((u - cx) d / fx, (v - cy) d / fy, d, 1), world = Rt cam.
__device__ __forceinline__ void dm_unproject(const float* __restrict__ dep, const DmDev& m, int u, int v, float* p) {
    const float d = dep[(size_t)v * m.w + u];
    const float c[4] = {fdiv(fmul(fsub((float)u, m.cx), d), m.fx), fdiv(fmul(fsub((float)v, m.cy), d), m.fy), d, 1.0f};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float acc = fmul(m.rt[4 * i], c[0]);
#pragma unroll
        for (int k = 1; k < 4; ++k) acc = fadd(acc, fmul(m.rt[4 * i + k], c[k]));
        p[i] = acc;
    }
}

__device__ __forceinline__ float norm3(float x, float y, float z) {
    return fsqrt(fadd(fadd(fmul(x, x), fmul(y, y)), fmul(z, z)));
}

// DepthMap::sample_radius (depth_map.cpp:13-30): half the mean distance to the
// valid 4-neighbours, in the order +u, -u, +v, -v.
__device__ __forceinline__ float dm_radius(const float* __restrict__ dep, const DmDev& m, int u, int v, const float* c) {
    const int du[4] = {1, -1, 0, 0}, dv[4] = {0, 0, 1, -1};
    float sum = 0.0f;
    int count = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int nu = u + du[i], nv = v + dv[i];
        if (!dm_valid(dep, m, nu, nv)) continue;
        float q[3];
        dm_unproject(dep, m, nu, nv, q);
        sum = fadd(sum, norm3(fsub(q[0], c[0]), fsub(q[1], c[1]), fsub(q[2], c[2])));
        ++count;
    }
    if (count == 0) return 0.0f;
    return fdiv(fmul(0.5f, sum), (float)count);
}

// cube_depth_for_radius (octree_builder.cpp:11-28) with max_depth 21.
__device__ __forceinline__ int depth_for_radius(float r_x, float r_root, const float* __restrict__ thr) {
    const float y = fdiv(r_root, fmul(r_x, 1.125f));
    int d = 0;
    if (!(isinf(y) && y > 0.0f)) {  // +inf: the cast of round(log2(inf)) gives INT_MIN on x86, clamped to 0
#pragma unroll
        for (int k = 0; k < 21; ++k) d += y >= thr[k] ? 1 : 0;
    }
    for (int tries = 0; tries < 3; ++tries) {
        const float cell = fdiv(r_root, (float)(1u << d));
        const float lo = fmul(0.75f, r_x), hi = fmul(1.5f, r_x);
        if (cell >= lo && cell < hi) break;
        if (cell < lo) { if (d > 0) --d; else break; }
        else { if (d < 21) ++d; else break; }
    }
    return d;
}

__global__ void k_stage1(DmDev m, const float* __restrict__ dep, float ox, float oy, float oz, float inv_2r,
                         float r_root, const float* __restrict__ thr, unsigned long long* __restrict__ key,
                         float* __restrict__ rc, int* __restrict__ dpt, int* __restrict__ keep) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)m.w * m.h) return;
    const int u = (int)(t % m.w), v = (int)(t / m.w);
    keep[t] = 0;
    if (!dm_valid(dep, m, u, v)) return;
    float p[3];
    dm_unproject(dep, m, u, v, p);
    const float r_x = dm_radius(dep, m, u, v, p);
    if (!(r_x > 0.0f)) return;
    const float n[3] = {fmul(fsub(p[0], ox), inv_2r), fmul(fsub(p[1], oy), inv_2r), fmul(fsub(p[2], oz), inv_2r)};
    for (int k = 0; k < 3; ++k)
        if (n[k] < 0.0f || n[k] >= 1.0f) return;  // the reference's test (a NaN passes it)
    const int d = depth_for_radius(r_x, r_root, thr);
    const uint32_t g = 1u << d;
    uint32_t ix[3];
    for (int k = 0; k < 3; ++k) {
        uint32_t q = __float2uint_rz(fmul(n[k], (float)g));
        ix[k] = q >= g ? g - 1 : q;
    }
    const int sh = 21 - d;
    key[t] = spread3(ix[0] << sh) | (spread3(ix[1] << sh) << 1) | (spread3(ix[2] << sh) << 2);
    rc[t] = r_x;
    dpt[t] = d;
    keep[t] = 1;
}

__global__ void k_stage1_compact(int64_t npix, const int* __restrict__ keep, const int* __restrict__ pos,
                                 const unsigned long long* __restrict__ key, unsigned long long* __restrict__ ckey,
                                 int* __restrict__ cidx) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npix || !keep[t]) return;
    ckey[pos[t]] = key[t];
    cidx[pos[t]] = (int)t;
}

__global__ void k_stage1_emit(int nc, const unsigned long long* __restrict__ skey, const int* __restrict__ sidx,
                              const float* __restrict__ rc, const int* __restrict__ dpt, tgvg_cube* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const unsigned long long k = skey[i];
    const int t = sidx[i];
    tgvg_cube c;
    c.hi = (uint32_t)(k >> 32);
    c.lo = (uint32_t)k;
    c.r_c = rc[t];
    c.depth = dpt[t];
    out[i] = c;
}

// Thresholds t[k-1] = smallest float y > 0 with (int)round(log2f(y)) >= k, k = 1..21,
// found by bisection over the positive float bit patterns with the host's log2f.
static void radius_thresholds(float* t) {
    for (int k = 1; k <= 21; ++k) {
        uint32_t lo = 1u, hi = 0x7f7fffffu;  // smallest subnormal .. largest finite
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            float y;
            std::memcpy(&y, &mid, 4);
            if ((int)std::round(std::log2(y)) >= k) hi = mid; else lo = mid + 1;
        }
        std::memcpy(&t[k - 1], &lo, 4);
    }
}

// The cubes of one map.  *count receives their number; they are copied to
// out when it has room for them (cap), else TGVG_ERR_LIMIT; out == nullptr
// asks for the count only.
static int build_cubes(tgvg_ctx* ctx, const tgvg_depthmap* dm, const float* origin, float r_root,
                       tgvg_cube* out, int64_t cap, int64_t* count) {
    const int64_t npix = int64_t(dm->width) * dm->height;
    *count = 0;
    if (npix <= 0) return TGVG_OK;
    if (npix > (int64_t(1) << 30)) return ctx->fail(TGVG_ERR_LIMIT, "depth map larger than 2^30 pixels");
    float thr[21];
    radius_thresholds(thr);
    DmDev m;
    m.fx = dm->fx; m.fy = dm->fy; m.cx = dm->cx; m.cy = dm->cy;
    std::memcpy(m.rt, dm->rt, sizeof(m.rt));
    m.w = dm->width; m.h = dm->height;
    const float inv_2r = 1.0f / (2.0f * r_root);
    auto B = [&](int id, size_t b) { return ctx->buf(id, b); };
    auto* dep = (float*)B(B_P_DEP, 4ull * npix);
    auto* key = (unsigned long long*)B(B_P_KEY, 8ull * npix);
    auto* rc = (float*)B(B_P_RC, 4ull * npix);
    auto* dpt = (int*)B(B_P_DPT, 4ull * npix);
    auto* keep = (int*)B(B_P_KEEP, 4ull * npix);
    auto* pos = (int*)B(B_P_POS, 4ull * npix);
    auto* d_thr = (float*)B(B_P_THR, sizeof(thr));
    if (!dep || !key || !rc || !dpt || !keep || !pos || !d_thr) return TGVG_ERR_NOMEM;
    cudaStream_t st = ctx->stream;
    TGVG_CK(ctx, cudaMemcpyAsync(dep, dm->depths, 4ull * npix, cudaMemcpyHostToDevice, st));
    TGVG_CK(ctx, cudaMemcpyAsync(d_thr, thr, sizeof(thr), cudaMemcpyHostToDevice, st));
    k_stage1<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(m, dep, origin[0], origin[1], origin[2], inv_2r, r_root,
                                                             d_thr, key, rc, dpt, keep);
    TGVG_LAUNCHED(ctx);
    int64_t nc = 0;
    int rc2 = scan_exclusive(ctx, keep, npix, pos, &nc);
    if (rc2) return rc2;
    *count = nc;
    if (nc == 0 || !out) return TGVG_OK;
    if (cap < nc) return TGVG_ERR_LIMIT;
    auto* ckey = (unsigned long long*)B(B_P_CKEY, 8ull * nc);
    auto* cidx = (int*)B(B_P_CIDX, 4ull * nc);
    auto* skey = (unsigned long long*)B(B_P_SKEY, 8ull * nc);
    auto* sidx = (int*)B(B_P_SIDX, 4ull * nc);
    auto* cub_out = (tgvg_cube*)B(B_P_OUT, sizeof(tgvg_cube) * nc);
    if (!ckey || !cidx || !skey || !sidx || !cub_out) return TGVG_ERR_NOMEM;
    k_stage1_compact<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(npix, keep, pos, key, ckey, cidx);
    TGVG_LAUNCHED(ctx);
    // stable LSD radix sort by the 63-bit code (library sort: the cube list is
    // input preparation, not the iterated path)
    size_t tmp_bytes = 0;
    TGVG_CK(ctx, cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, ckey, skey, cidx, sidx, (int)nc, 0, 63, st));
    void* tmp = B(B_P_TMP, std::max<size_t>(tmp_bytes, 16));
    if (!tmp) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, ckey, skey, cidx, sidx, (int)nc, 0, 63, st));
    k_stage1_emit<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>((int)nc, skey, sidx, rc, dpt, cub_out);
    TGVG_LAUNCHED(ctx);
    TGVG_CK(ctx, cudaMemcpyAsync(out, cub_out, sizeof(tgvg_cube) * nc, cudaMemcpyDeviceToHost, st));
    TGVG_CK(ctx, cudaStreamSynchronize(st));
    return TGVG_OK;
}

}  // namespace tgvg

using namespace tgvg;

extern "C" int tgvg_build_cubes(tgvg_ctx* ctx, const tgvg_depthmap* dm, const float* origin3, float r_root,
                                tgvg_cube* out, int64_t cap, int64_t* count) {
    if (!ctx || !dm || !origin3 || !count || dm->width < 0 || dm->height < 0 ||
        (int64_t(dm->width) * dm->height > 0 && !dm->depths) || !std::isfinite(r_root) || !(r_root > 0.0f))
        return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return build_cubes(ctx, dm, origin3, r_root, out, cap, count);
}

extern "C" int tgvg_build_cubes_file(tgvg_ctx* ctx, const tgvg_depthmap* dm, const float* origin3, float r_root,
                                     const char* out_path) {
    int64_t n = 0;
    std::vector<tgvg_cube> cubes(size_t(std::max(0, dm ? dm->width : 0)) * size_t(std::max(0, dm ? dm->height : 0)));
    int rc = tgvg_build_cubes(ctx, dm, origin3, r_root, cubes.data(), int64_t(cubes.size()), &n);
    if (rc) return rc;
    cubes.resize(size_t(n));
    char hdr[16] = {'T', 'G', 'V', '1'};
    const uint32_t ver = 1, cnt = uint32_t(n);
    std::memcpy(hdr + 4, &ver, 4);
    std::memcpy(hdr + 8, &r_root, 4);
    std::memcpy(hdr + 12, &cnt, 4);
    rc = tgvg::fileio::write_file(out_path, hdr, 16, cubes.data(), sizeof(tgvg_cube) * size_t(n));
    return rc ? ctx->fail(rc, std::string("Cannot open output: ") + (out_path ? out_path : "")) : TGVG_OK;
}
