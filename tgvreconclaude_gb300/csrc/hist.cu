// Stage 5 on sm_103a: depth-map pyramids and cube histograms.
//
// K1 k_pyramid_level  -- DepthMipmap::build (reference src/histogram.cpp:35-74):
//    one launch per pyramid level covers every map; each thread averages the
//    finite, positive texels among its (up to) four children in the
//    reference's dv-outer / du-inner order.  HBM-bound: 4 B read per child
//    texel, 4 B written per coarse texel.
// K2 k_histograms     -- compute_histograms + project + cube_center
//    (reference src/histogram.cpp:76-163): one thread per cube walks every map,
//    keeps the bins in registers and writes its row once, so no atomics are
//    needed.  Cameras are staged through shared memory in batches and read as
//    warp-uniform broadcasts.  Bound: the texel gather (4 B per accepted pair,
//    sector-granular) plus 16 B cube + 4*nbins B row per cube.
//
// Every float operation is an explicitly rounded __f*_rn intrinsic in the
// reference's evaluation order, so the bins are bit-identical to the CPU
// reference (no contraction, IEEE division).
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace tgvg {

// Laid out so that the fields the binning loop reads for every pair come as
// five 16-byte shared-memory loads: the three rows of Rt_inv, (fx, fy, cx, cy)
// and (|fx|, W, H, nlev).
struct __align__(16) DevCam {
    float m[12];      // rows 0..2 of Rt_inv (row-major)
    float fx, fy, cx, cy;
    float absfx;
    int W, H, nlev;
    long long base;   // element offset of level 0 in the texel buffer
    int vote;
    int off[13];      // element offset of level l relative to base
};
static_assert(sizeof(DevCam) == 144, "DevCam layout");

// Level dimensions: the reference halves with integer division and stops once a
// side reaches 1 (histogram.cpp:42-53), so level l is max(1, W >> l) wide.
int pyramid_dims(int32_t w, int32_t h, int32_t* dims) {
    int n = 1;
    dims[0] = w; dims[1] = h;
    for (int l = 0; l < 12; ++l) {
        int pw = dims[2 * (n - 1)], ph = dims[2 * (n - 1) + 1];
        if (pw <= 1 || ph <= 1) break;
        dims[2 * n] = pw / 2 > 1 ? pw / 2 : 1;
        dims[2 * n + 1] = ph / 2 > 1 ? ph / 2 : 1;
        ++n;
    }
    return n;
}

static int64_t pyramid_size(int32_t w, int32_t h) {
    int32_t d[26];
    int n = pyramid_dims(w, h, d);
    int64_t t = 0;
    for (int l = 0; l < n; ++l) t += int64_t(d[2 * l]) * d[2 * l + 1];
    return t;
}

static void make_devcams(const tgvg_camera* cams, int32_t ncam, const int64_t* level_offset,
                         std::vector<DevCam>& out) {
    out.resize(ncam);
    for (int c = 0; c < ncam; ++c) {
        DevCam& d = out[c];
        std::memset(&d, 0, sizeof(d));
        d.base = level_offset[c];
        for (int i = 0; i < 12; ++i) d.m[i] = cams[c].rt_inv[i];
        d.fx = cams[c].fx; d.fy = cams[c].fy; d.cx = cams[c].cx; d.cy = cams[c].cy;
        d.absfx = std::fabs(cams[c].fx);
        d.W = cams[c].width; d.H = cams[c].height;
        d.vote = cams[c].lidar ? 5 : 1;
        int32_t dims[26];
        d.nlev = pyramid_dims(d.W, d.H, dims);
        int o = 0;
        for (int l = 0; l < d.nlev; ++l) { d.off[l] = o; o += dims[2 * l] * dims[2 * l + 1]; }
    }
}

// ---------------------------------------------------------------- K1 ---
__global__ void k_pyramid_level(const DevCam* __restrict__ cams, float* __restrict__ tex, int level) {
    const DevCam& c = cams[blockIdx.y];
    if (level >= c.nlev) return;
    const int pw = max(1, c.W >> (level - 1)), ph = max(1, c.H >> (level - 1));
    const int w = max(1, c.W >> level), h = max(1, c.H >> level);
    const float* prev = tex + c.base + c.off[level - 1];
    float* cur = tex + c.base + c.off[level];
    const int total = w * h;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int v = t / w, u = t - v * w;
        float sum = 0.0f;
        int cnt = 0;
#pragma unroll
        for (int dv = 0; dv < 2; ++dv)
#pragma unroll
            for (int du = 0; du < 2; ++du) {
                const int pu = 2 * u + du, pv = 2 * v + dv;
                if (pu < pw && pv < ph) {
                    const float d = __ldg(prev + pv * pw + pu);
                    if (d > 0.0f && d < INFINITY) { sum = fadd(sum, d); ++cnt; }
                }
            }
        cur[t] = cnt > 0 ? fdiv(sum, (float)cnt) : __int_as_float(0x7fc00000);
    }
}

// ---------------------------------------------------------------- K2 ---
static constexpr int HIST_BLOCK = 256;
static constexpr int CAM_BATCH = 64;

// t[k] (k = 1..12): the smallest float x with (int)log2f(x) >= k.  expo: every
// t[k] lies in (2^(k-1), 2^k], so for x >= 1 the level is the float exponent e
// of x, plus one when x >= t[e+1].
struct Thresholds {
    float t[13];
    int expo;
};

// Host side of the thresholds: the expo property checked on the values.
static inline void finish_thresholds(Thresholds& thr) {
    thr.expo = 1;
    for (int k = 1; k < 13; ++k)
        if (!(thr.t[k] > std::ldexp(1.0f, k - 1) && thr.t[k] <= std::ldexp(1.0f, k))) thr.expo = 0;
}

// Camera cull for one block of cubes (no counterpart in the reference; it
// only skips pairs that project() rejects, histogram.cpp:76-106).  The
// block's cube centres lie in the box ctr +- ext.  A pair is accepted only if
// its camera-space z > 0 and the truncated pixel coordinates fall inside the
// image, i.e. -1 < x fx / z + cx < W and -1 < y fy / z + cy < H; for z > 0 these
// are half-spaces g(P) > 0 with g linear in the world point P.  The float
// evaluation of project() differs from exact arithmetic by a few units of
// 2^-24 of the magnitudes involved, so if the largest g over the box is below
// minus 1e-3 of those magnitudes, no centre in the box can pass: the camera is
// skipped for the whole block.  Cameras with a non-finite parameter are never
// skipped.
__device__ __noinline__ bool camera_may_see(const DevCam& c, const float* ctr, const float* ext) {
    const float* m = c.m;
    bool finite = isfinite(c.fx) && isfinite(c.fy) && isfinite(c.cx) && isfinite(c.cy);
#pragma unroll
    for (int k = 0; k < 12; ++k) finite = finite && isfinite(m[k]);
    if (!finite) return true;
    // S_r: the magnitude of row r's terms over the box (rows x, y, z of Rt_inv)
    float S[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float t = fabsf(m[4 * r + 3]);
#pragma unroll
        for (int k = 0; k < 3; ++k) t += fabsf(m[4 * r + k]) * (fabsf(ctr[k]) + ext[k]);
        S[r] = t;
    }
    // largest value over the box of g = wr * (row r) + wz * (row z); the error of
    // this float evaluation is a few 1e-7 of the magnitudes, far inside the margin
    auto max_g = [&](int r, float wr, float wz) {
        float g = wr * m[4 * r + 3] + wz * m[11];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float a = wr * m[4 * r + k] + wz * m[8 + k];
            g += a * ctr[k] + fabsf(a) * ext[k];
        }
        return g;
    };
    if (max_g(0, 0.0f, 1.0f) < -1e-3f * S[2]) return false;  // z > 0
    const float W = (float)c.W, H = (float)c.H;
    const float tu = 1e-3f * (fabsf(c.fx) * S[0] + (fabsf(c.cx) + W + 2.0f) * S[2]);
    const float tv = 1e-3f * (fabsf(c.fy) * S[1] + (fabsf(c.cy) + H + 2.0f) * S[2]);
    if (max_g(0, c.fx, c.cx + 1.0f) < -tu) return false;  // x fx / z + cx > -1
    if (max_g(0, -c.fx, W - c.cx) < -tu) return false;    // x fx / z + cx < W
    if (max_g(1, c.fy, c.cy + 1.0f) < -tv) return false;  // y fy / z + cy > -1
    if (max_g(1, -c.fy, H - c.cy) < -tv) return false;    // y fy / z + cy < H
    return true;
}

// PACK: the bin counts are kept as 16-bit fields of 64-bit words (four bins a
// word), which holds when no cube can collect more than 65535 votes; one shift
// and a few predicated adds per pair instead of a compare and add per bin.
template <int NB, bool PACK>
__global__ void __launch_bounds__(HIST_BLOCK)
k_histograms(const uint4* __restrict__ cubes, int64_t n, const DevCam* __restrict__ cams, int ncam,
             const float* __restrict__ tex, float ox, float oy, float oz, float r_root,
             Thresholds thr, uint32_t* __restrict__ out) {
    __shared__ DevCam s_cam[CAM_BATCH];
    __shared__ float s_thr[13];
    __shared__ bool s_vis[CAM_BATCH];
    __shared__ float s_box[HIST_BLOCK / 32][6];
    __shared__ float s_geo[6];  // centre and half extent of the block's box; ext < 0: no active cube
    if (threadIdx.x < 13) s_thr[threadIdx.x] = thr.t[threadIdx.x];
    const int64_t i = int64_t(blockIdx.x) * HIST_BLOCK + threadIdx.x;
    const bool valid = i < n;
    constexpr int NW = (NB + 3) / 4;
    uint32_t bins[NB];
    uint64_t pk[NW];
#pragma unroll
    for (int k = 0; k < NB; ++k) bins[k] = 0;
#pragma unroll
    for (int k = 0; k < NW; ++k) pk[k] = 0;

    // cube_center (histogram.cpp:118-125)
    float px = 0.f, py = 0.f, pz = 0.f, r_c = 0.f;
    bool active = false;
    if (valid) {
        const uint4 cb = cubes[i];
        const uint64_t key = (uint64_t(cb.x) << 32) | cb.y;
        r_c = __uint_as_float(cb.z);
        const int depth = (int)cb.w;
        const uint32_t fxg = gather3(key), fyg = gather3(key >> 1), fzg = gather3(key >> 2);
        const int shift = 21 - depth;
        const uint32_t ix = fxg >> shift, iy = fyg >> shift, iz = fzg >> shift;
        const float cs = fdiv(fmul(2.0f, r_root), (float)(1u << depth));
        px = fadd(ox, fmul(fadd((float)ix, 0.5f), cs));
        py = fadd(oy, fmul(fadd((float)iy, 0.5f), cs));
        pz = fadd(oz, fmul(fadd((float)iz, 0.5f), cs));
        active = !(r_c <= 0.0f);  // histogram.cpp:141 (NaN r_c proceeds)
    }
    const float delta = fmul(6.0f, r_c);
    const float eta = fmul(18.0f, r_c);
    const float HALF = NB / 2.0f;

    // bounding box of the block's active cube centres (empty: every camera skipped,
    // which changes nothing since no thread of the block is active)
    {
        float b[6] = {active ? px : INFINITY, active ? py : INFINITY, active ? pz : INFINITY,
                      active ? px : -INFINITY, active ? py : -INFINITY, active ? pz : -INFINITY};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                b[k] = fminf(b[k], __shfl_xor_sync(0xffffffffu, b[k], o));
                b[k + 3] = fmaxf(b[k + 3], __shfl_xor_sync(0xffffffffu, b[k + 3], o));
            }
        }
        if ((threadIdx.x & 31) == 0) {
#pragma unroll
            for (int k = 0; k < 6; ++k) s_box[threadIdx.x >> 5][k] = b[k];
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        float lo = INFINITY, hi = -INFINITY;
        for (int w = 0; w < HIST_BLOCK / 32; ++w) { lo = fminf(lo, s_box[w][k]); hi = fmaxf(hi, s_box[w][k + 3]); }
        const bool any = lo <= hi;
        // the centre's rounding is covered by rounding the half extent up
        const float ctr = 0.5f * (lo + hi);
        s_geo[k] = any ? ctr : 0.0f;
        s_geo[k + 3] = any ? fmaxf(hi - ctr, ctr - lo) * 1.0001f : -1.0f;
    }

    for (int c0 = 0; c0 < ncam; c0 += CAM_BATCH) {
        const int nb = min(CAM_BATCH, ncam - c0);
        __syncthreads();
        {
            const int words = nb * (int)(sizeof(DevCam) / 4);
            const int* src = reinterpret_cast<const int*>(cams + c0);
            int* dst = reinterpret_cast<int*>(s_cam);
            for (int w = threadIdx.x; w < words; w += HIST_BLOCK) dst[w] = src[w];
        }
        __syncthreads();
        if (threadIdx.x < nb)
            s_vis[threadIdx.x] = s_geo[3] >= 0.0f && camera_may_see(s_cam[threadIdx.x], s_geo, s_geo + 3);
        __syncthreads();
        if (!active) continue;
        for (int cc = 0; cc < nb; ++cc) {
            if (!s_vis[cc]) continue;  // block-uniform: no centre of the block can pass project()
            const DevCam& c = s_cam[cc];
            const float4* c4 = reinterpret_cast<const float4*>(&c);
            const float4 r0 = c4[0], r1 = c4[1], r2 = c4[2], k4 = c4[3], e4 = c4[4];
            const int cW = __float_as_int(e4.y), cH = __float_as_int(e4.z), cL = __float_as_int(e4.w);
            // project (histogram.cpp:76-106): cam = Rt_inv * [P, 1]
            float X = fmul(r0.x, px); X = fadd(X, fmul(r0.y, py)); X = fadd(X, fmul(r0.z, pz));
            X = fadd(X, fmul(r0.w, 1.0f));
            float Y = fmul(r1.x, px); Y = fadd(Y, fmul(r1.y, py)); Y = fadd(Y, fmul(r1.z, pz));
            Y = fadd(Y, fmul(r1.w, 1.0f));
            float Z = fmul(r2.x, px); Z = fadd(Z, fmul(r2.y, py)); Z = fadd(Z, fmul(r2.z, pz));
            Z = fadd(Z, fmul(r2.w, 1.0f));
            if (Z <= 0.0f) continue;
            const float u_f = fadd(fmul(fdiv(X, Z), k4.x), k4.z);
            const float v_f = fadd(fmul(fdiv(Y, Z), k4.y), k4.w);
            const int u0 = trunc_i32(u_f), v0 = trunc_i32(v_f);
            if (u0 < 0 || u0 >= cW || v0 < 0 || v0 >= cH) continue;
            // level = clamp((int)log2(max(1, |fx| r_c / z)), 0, L-1) through the
            // host-computed thresholds of (int)log2f; +inf gives level 0 as the
            // reference's int conversion of log2f(inf) does on x86-64.
            const float fp = fdiv(fmul(e4.x, r_c), Z);
            const float xm = (1.0f < fp) ? fp : 1.0f;
            int lv = 0;
            if (xm < INFINITY) {
                if (thr.expo) {
                    const int e = min((int)(__float_as_uint(xm) >> 23) - 127, 12);  // xm >= 1
                    lv = e + ((e < 12 && xm >= s_thr[e + 1]) ? 1 : 0);
                } else {
#pragma unroll
                    for (int k = 1; k < 13; ++k) lv += (xm >= s_thr[k]) ? 1 : 0;
                }
            }
            lv = min(lv, cL - 1);
            const int lw = max(1, cW >> lv), lh = max(1, cH >> lv);
            int uu = u0 >> lv, vv = v0 >> lv;
            uu = uu < 0 ? 0 : (lw - 1 < uu ? lw - 1 : uu);
            vv = vv < 0 ? 0 : (lh - 1 < vv ? lh - 1 : vv);
            const float sd = __ldg(tex + c.base + c.off[lv] + (int64_t)vv * lw + uu);
            if (!(sd > 0.0f && sd < INFINITY)) continue;  // !isfinite || <= 0
            float a = fsub(sd, Z);
            if (a < -eta) continue;
            a = fdiv(a, delta);
            a = (a < -1.0f) ? -1.0f : ((1.0f < a) ? 1.0f : a);  // std::clamp
            int bin = trunc_i32(fmul(fadd(a, 1.0f), HALF));
            bin = bin < 0 ? 0 : (NB - 1 < bin ? NB - 1 : bin);
            if (PACK) {
                const uint64_t inc = (uint64_t)c.vote << (16 * (bin & 3));
#pragma unroll
                for (int w = 0; w < NW; ++w) pk[w] += ((bin >> 2) == w) ? inc : 0ull;
            } else {
#pragma unroll
                for (int k = 0; k < NB; ++k) bins[k] += (bin == k) ? (uint32_t)c.vote : 0u;
            }
        }
    }
    if (!valid) return;
    if (PACK) {
#pragma unroll
        for (int k = 0; k < NB; ++k) bins[k] = (uint32_t)(pk[k >> 2] >> (16 * (k & 3))) & 0xffffu;
    }
    uint32_t* row = out + i * NB;
    if (NB == 8) {
        reinterpret_cast<uint4*>(row)[0] = make_uint4(bins[0], bins[1], bins[2], bins[3]);
        reinterpret_cast<uint4*>(row)[1] = make_uint4(bins[4], bins[5], bins[6], bins[7]);
    } else {
#pragma unroll
        for (int k = 0; k < NB; k += 2) reinterpret_cast<uint2*>(row)[k / 2] = make_uint2(bins[k], bins[k + 1]);
    }
}

int build_pyramids_dev(tgvg_ctx* ctx, const tgvg_camera* cams, int32_t ncam, float* d_levels,
                       const int64_t* level_offset) {
    std::vector<DevCam> dc;
    make_devcams(cams, ncam, level_offset, dc);
    DevCam* d_cams = (DevCam*)ctx->buf(B_H_CAMS, sizeof(DevCam) * dc.size());
    if (!d_cams) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemcpyAsync(d_cams, dc.data(), sizeof(DevCam) * dc.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    int maxlev = 0, maxpix = 0;
    for (auto& c : dc) { maxlev = std::max(maxlev, c.nlev); maxpix = std::max(maxpix, c.W * c.H); }
    for (int l = 1; l < maxlev; ++l) {
        const int texels = std::max(1, maxpix >> (2 * l));
        dim3 grid((unsigned)std::min(1024, (texels + 255) / 256), (unsigned)ncam);
        k_pyramid_level<<<grid, 256, 0, ctx->stream>>>(d_cams, d_levels, l);
        TGVG_LAUNCHED(ctx);
    }
    return TGVG_OK;
}

// The binning launch: the packed counters when no cube can collect more than
// 65535 votes (every camera's vote counted once), else the per-bin counters.
static void launch_histograms(const tgvg_camera* cams, int32_t ncam, unsigned grid, cudaStream_t s,
                              const uint4* cubes, int64_t n, const DevCam* d_cams, const float* tex, const float* o,
                              float r_root, Thresholds thr, int32_t nbins, uint32_t* out) {
    finish_thresholds(thr);
    int64_t votes = 0;
    for (int c = 0; c < ncam; ++c) votes += cams[c].lidar ? 5 : 1;
    const bool pack = votes <= 65535;
#define TGVG_HIST(NBV, PK) \
    k_histograms<NBV, PK><<<grid, HIST_BLOCK, 0, s>>>(cubes, n, d_cams, ncam, tex, o[0], o[1], o[2], r_root, thr, out)
    if (nbins == 8) {
        if (pack) TGVG_HIST(8, true); else TGVG_HIST(8, false);
    } else {
        if (pack) TGVG_HIST(10, true); else TGVG_HIST(10, false);
    }
#undef TGVG_HIST
}

int histograms_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, int64_t n, const tgvg_camera* cams,
                   int32_t ncam, const float* d_levels, const int64_t* level_offset,
                   const float origin[3], float r_root, int32_t nbins, uint32_t* d_out) {
    if (n == 0) return TGVG_OK;
    std::vector<DevCam> dc;
    make_devcams(cams, ncam, level_offset, dc);
    DevCam* d_cams = (DevCam*)ctx->buf(B_H_CAMS, sizeof(DevCam) * std::max<size_t>(1, dc.size()));
    if (!d_cams) return TGVG_ERR_NOMEM;
    if (ncam > 0)
        TGVG_CK(ctx, cudaMemcpyAsync(d_cams, dc.data(), sizeof(DevCam) * dc.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
    Thresholds thr;
    std::memcpy(thr.t, ctx->lvl_thresh, sizeof(thr.t));
    const unsigned grid = (unsigned)((n + HIST_BLOCK - 1) / HIST_BLOCK);
    launch_histograms(cams, ncam, grid, ctx->stream, reinterpret_cast<const uint4*>(d_cubes), n, d_cams, d_levels,
                      origin, r_root, thr, nbins, d_out);
    TGVG_LAUNCHED(ctx);
    return TGVG_OK;
}

}  // namespace tgvg

// ---------------------------------------------------------- C ABI (Stage 5) ---
using namespace tgvg;

static int check_cams(const tgvg_camera* cams, int32_t ncam) {
    if (ncam < 0 || (ncam > 0 && !cams)) return TGVG_ERR_INVALID;
    for (int c = 0; c < ncam; ++c)
        if (cams[c].width <= 0 || cams[c].height <= 0 ||
            int64_t(cams[c].width) * cams[c].height > (int64_t(1) << 30))
            return TGVG_ERR_INVALID;
    return TGVG_OK;
}

static int check_cubes_depth(const tgvg_cube* cubes, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
        if (cubes[i].depth < 0 || cubes[i].depth > 21) return TGVG_ERR_INVALID;
    return TGVG_OK;
}

// Shared body of the host-buffer histogram calls.  `pyr` selects whether
// maps[c] holds level 0 only (pyramids built here) or every level.
static int histograms_host(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n,
                           const tgvg_camera* cams, int32_t ncam, const float* const* maps, bool pyr,
                           const float origin[3], float r_root, int32_t nbins, uint32_t* out) {
    if (!ctx || n < 0 || (n > 0 && (!cubes || !out)) || !origin || (nbins != 8 && nbins != 10))
        return TGVG_ERR_INVALID;
    int rc = check_cams(cams, ncam);
    if (rc) return rc;
    if (ncam > 0 && !maps) return TGVG_ERR_INVALID;
    if ((rc = check_cubes_depth(cubes, n))) return rc;
    if (n == 0) return TGVG_OK;
    std::vector<int64_t> off(ncam + 1, 0);
    for (int c = 0; c < ncam; ++c) off[c + 1] = off[c] + pyramid_size(cams[c].width, cams[c].height);
    // Under a device budget (tgvg_set_device_budget) the cubes go through in
    // batches whose cube and histogram buffers take at most half of it; the
    // pyramids stay on the device.  Cubes are binned independently, so the
    // batches give the one-pass result.
    int64_t batch = n;
    if (ctx->device_budget > 0) {
        const int64_t per = int64_t(sizeof(tgvg_cube)) + 4ll * nbins;
        batch = std::min<int64_t>(n, std::max<int64_t>(4096, int64_t(ctx->device_budget / 2) / per));
    }
    float* d_tex = (float*)ctx->buf(B_H_TEX, sizeof(float) * std::max<int64_t>(1, off[ncam]));
    tgvg_cube* d_cubes = (tgvg_cube*)ctx->buf(B_H_CUBES, sizeof(tgvg_cube) * batch);
    uint32_t* d_out = (uint32_t*)ctx->buf(B_H_OUT, sizeof(uint32_t) * nbins * batch);
    if (!d_tex || !d_cubes || !d_out) return TGVG_ERR_NOMEM;
    for (int c = 0; c < ncam; ++c) {
        if (!maps[c]) return TGVG_ERR_INVALID;
        const int64_t cnt = pyr ? off[c + 1] - off[c] : int64_t(cams[c].width) * cams[c].height;
        TGVG_CK(ctx, cudaMemcpyAsync(d_tex + off[c], maps[c], sizeof(float) * cnt,
                                     cudaMemcpyHostToDevice, ctx->stream));
    }
    if (!pyr && ncam > 0 && (rc = build_pyramids_dev(ctx, cams, ncam, d_tex, off.data()))) return rc;
    for (int64_t s0 = 0; s0 < n; s0 += batch) {
        const int64_t m = std::min(batch, n - s0);
        TGVG_CK(ctx, cudaMemcpyAsync(d_cubes, cubes + s0, sizeof(tgvg_cube) * m, cudaMemcpyHostToDevice,
                                     ctx->stream));
        if ((rc = histograms_dev(ctx, d_cubes, m, cams, ncam, d_tex, off.data(), origin, r_root, nbins,
                                 d_out)))
            return rc;
        TGVG_CK(ctx, cudaMemcpyAsync(out + s0 * nbins, d_out, sizeof(uint32_t) * nbins * m,
                                     cudaMemcpyDeviceToHost, ctx->stream));
    }
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

extern "C" int tgvg_pyramid_dims(int32_t width, int32_t height, int32_t* dims) {
    if (width <= 0 || height <= 0 || !dims) return TGVG_ERR_INVALID;
    return pyramid_dims(width, height, dims);
}

extern "C" int tgvg_build_pyramids(tgvg_ctx* ctx, const tgvg_camera* cams, int32_t ncam,
                                   const float* const* base, float* const* levels_out) {
    if (!ctx) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int rc = check_cams(cams, ncam);
    if (rc) return rc;
    if (ncam == 0) return TGVG_OK;
    if (!base) return TGVG_ERR_INVALID;
    std::vector<int64_t> off(ncam + 1, 0);
    for (int c = 0; c < ncam; ++c) off[c + 1] = off[c] + pyramid_size(cams[c].width, cams[c].height);
    float* d_tex = (float*)ctx->buf(B_H_TEX, sizeof(float) * off[ncam]);
    if (!d_tex) return TGVG_ERR_NOMEM;
    for (int c = 0; c < ncam; ++c) {
        if (!base[c]) return TGVG_ERR_INVALID;
        TGVG_CK(ctx, cudaMemcpyAsync(d_tex + off[c], base[c],
                                     sizeof(float) * cams[c].width * cams[c].height,
                                     cudaMemcpyHostToDevice, ctx->stream));
    }
    if ((rc = build_pyramids_dev(ctx, cams, ncam, d_tex, off.data()))) return rc;
    if (levels_out)
        for (int c = 0; c < ncam; ++c)
            if (levels_out[c])
                TGVG_CK(ctx, cudaMemcpyAsync(levels_out[c], d_tex + off[c],
                                             sizeof(float) * (off[c + 1] - off[c]),
                                             cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

extern "C" int tgvg_compute_histograms(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n,
                                       const tgvg_camera* cams, int32_t ncam,
                                       const float* const* base, const float origin[3],
                                       float r_root, int32_t nbins, uint32_t* out) {
    if (!ctx) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return histograms_host(ctx, cubes, n, cams, ncam, base, false, origin, r_root, nbins, out);
}

extern "C" int tgvg_compute_histograms_pyr(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n,
                                           const tgvg_camera* cams, int32_t ncam,
                                           const float* const* levels, const float origin[3],
                                           float r_root, int32_t nbins, uint32_t* out) {
    if (!ctx) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return histograms_host(ctx, cubes, n, cams, ncam, levels, true, origin, r_root, nbins, out);
}

extern "C" int tgvg_compute_histograms_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, int64_t n,
                                           const tgvg_camera* cams, int32_t ncam,
                                           const float* d_levels, const int64_t* level_offset,
                                           const float origin[3], float r_root, int32_t nbins,
                                           uint32_t* d_out) {
    if (!ctx || n < 0 || (n > 0 && (!d_cubes || !d_out)) || !origin || (nbins != 8 && nbins != 10))
        return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    int rc = check_cams(cams, ncam);
    if (rc) return rc;
    if (ncam > 0 && (!d_levels || !level_offset)) return TGVG_ERR_INVALID;
    if ((rc = histograms_dev(ctx, d_cubes, n, cams, ncam, d_levels, level_offset, origin, r_root,
                             nbins, d_out)))
        return rc;
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

// ------------------------------------------- no-allocation histogram entry ---
// Some host programs cannot call cudaMalloc once they are running: a service
// that reserves all device memory up front for its own pool, a real-time loop
// in which an allocation's implicit device synchronisation would stall other
// work, or a runtime that routes every device allocation through its own
// allocator.  tgvg_compute_histograms_noalloc serves them: the caller passes
// device inputs and outputs, and the only scratch this path needs (the depth
// pyramids and the camera table) lives in the fixed array below, which every
// GPU that loads this library holds until the process exits.
static constexpr int64_t NOALLOC_CAM_FLOATS = 9216;                   // 256 DevCam records
static constexpr int64_t NOALLOC_TEX_FLOATS = int64_t(16) << 20;      // 16 Mi texels = 64 MiB
static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_CAM_FLOATS + NOALLOC_TEX_FLOATS];

// Device address of the scratch array in the current context.  It is looked
// up on every call (the first call on a device may load the module): a cached
// address would go stale if the context were reset and the module reloaded.
static int noalloc_scratch(float** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return TGVG_ERR_NODEVICE;
    float* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return TGVG_ERR_CUDA;
    }
    *out = p;
    return TGVG_OK;
}

extern "C" int tgvg_compute_histograms_noalloc(const tgvg_cube* d_cubes, int64_t n, const tgvg_camera* cams,
                                               int32_t ncam, const float* const* d_base, const float origin[3],
                                               float r_root, int32_t nbins, uint32_t* d_out, void* stream) {
    if (n < 0 || (n > 0 && (!d_cubes || !d_out)) || !origin || (nbins != 8 && nbins != 10))
        return TGVG_ERR_INVALID;
    int rc = check_cams(cams, ncam);
    if (rc) return rc;
    if (ncam > 0 && !d_base) return TGVG_ERR_INVALID;
    if (int64_t(ncam) * (int64_t)sizeof(DevCam) > NOALLOC_CAM_FLOATS * 4) return TGVG_ERR_LIMIT;
    std::vector<int64_t> off(ncam + 1, 0);
    for (int c = 0; c < ncam; ++c) off[c + 1] = off[c] + pyramid_size(cams[c].width, cams[c].height);
    if (off[ncam] > NOALLOC_TEX_FLOATS) return TGVG_ERR_LIMIT;
    if (n == 0) return TGVG_OK;
    float* scratch = nullptr;
    if ((rc = noalloc_scratch(&scratch))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    DevCam* d_cams = reinterpret_cast<DevCam*>(scratch);
    float* d_tex = scratch + NOALLOC_CAM_FLOATS;
    std::vector<DevCam> dc;
    make_devcams(cams, ncam, off.data(), dc);
    // Every texel and camera record the kernels read is written earlier in this
    // call, so nothing left in the array by a previous call is ever used.
    if (ncam > 0 &&
        cudaMemcpyAsync(d_cams, dc.data(), sizeof(DevCam) * dc.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return TGVG_ERR_CUDA;
    int maxlev = 0, maxpix = 0;
    for (int c = 0; c < ncam; ++c) {
        if (!d_base[c]) return TGVG_ERR_INVALID;
        if (cudaMemcpyAsync(d_tex + off[c], d_base[c], sizeof(float) * cams[c].width * cams[c].height,
                            cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return TGVG_ERR_CUDA;
        maxlev = std::max(maxlev, dc[c].nlev);
        maxpix = std::max(maxpix, dc[c].W * dc[c].H);
    }
    for (int l = 1; l < maxlev; ++l) {
        const int texels = std::max(1, maxpix >> (2 * l));
        dim3 grid((unsigned)std::min(1024, (texels + 255) / 256), (unsigned)ncam);
        k_pyramid_level<<<grid, 256, 0, s>>>(d_cams, d_tex, l);
    }
    Thresholds thr;
    tgvg_level_thresholds(thr.t);
    const unsigned grid = (unsigned)((n + HIST_BLOCK - 1) / HIST_BLOCK);
    launch_histograms(cams, ncam, grid, s, reinterpret_cast<const uint4*>(d_cubes), n, d_cams, d_tex, origin, r_root,
                      thr, nbins, d_out);
    return cudaGetLastError() == cudaSuccess ? TGVG_OK : TGVG_ERR_CUDA;
}
