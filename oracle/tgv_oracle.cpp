// CPU restatement of the reference's Stage-5 (histogram) and Stage-6 (TGV)
// algorithms, used as the parity ORACLE for the CUDA path.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py load this library (oracle/_build/liboracle.so), and
// only to check results or as the timed CPU baseline; the product never calls it.
//
// Pinning: the float instantiation at NBINS=8 is checked bit-for-bit against
// the reference's own src/histogram.cpp and src/tgv.cpp compiled unmodified
// (oracle/Makefile -> oracle/_ref/libref.so) on seeded multi-level octrees and
// on the fixtures in tests/golden/.  The double instantiation is the FP64 oracle;
// NBINS=10 is the 10-bin extension (same formulas with 10 bins).
//
// Each routine cites the reference lines whose behaviour it restates.  Build with
// -ffp-contract=off: the float results must not depend on FMA contraction.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---- data layouts (reference src/types.hpp:18-35, src/histogram.hpp:10-19,
//      src/tgv.hpp:12-17, src/treetop.hpp:8-13) --------------------------------
struct Cube { uint32_t hi, lo; float r_c; int32_t depth; };
struct Leaf { uint32_t hi, lo; int32_t depth; uint32_t first_idx, last_idx; };
struct State { float u, v[3], p[3], q[6]; };
struct StateD { double u, v[3], p[3], q[6]; };
static_assert(sizeof(Cube) == 16, "cube");
static_assert(sizeof(Leaf) == 20, "leaf");
static_assert(sizeof(State) == 52, "state");

// ---- Morton helpers (reference src/types.hpp:39-73, src/balance.cpp:13-49) --
static inline uint64_t spread3(uint32_t v) {
    // Insert two zero bits between the 21 low bits of v.
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x001f00000000ffffull;
    x = (x | (x << 16)) & 0x001f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}
static inline uint32_t gather3(uint64_t v) {
    v &= 0x1249249249249249ull;
    v = (v | (v >> 2)) & 0x10c30c30c30c30c3ull;
    v = (v | (v >> 4)) & 0x100f00f00f00f00full;
    v = (v | (v >> 8)) & 0x001f0000ff0000ffull;
    v = (v | (v >> 16)) & 0x001f00000000ffffull;
    v = (v | (v >> 32)) & 0x00000000001fffffull;
    return static_cast<uint32_t>(v);
}
static inline uint64_t key_of(uint32_t hi, uint32_t lo) { return (uint64_t(hi) << 32) | lo; }
static inline uint64_t encode(uint32_t x, uint32_t y, uint32_t z) {
    return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}
static inline void decode(uint64_t k, uint32_t& x, uint32_t& y, uint32_t& z) {
    x = gather3(k); y = gather3(k >> 1); z = gather3(k >> 2);
}
// ancestor at target depth: clear the low 3*(21-d) bits (balance.cpp:22-26)
static inline uint64_t ancestor(uint64_t k, int d) {
    unsigned sh = 3u * (21u - static_cast<unsigned>(d));
    if (sh >= 64u) return 0;
    return k & ~((1ull << sh) - 1ull);
}
static inline uint64_t parent_key(uint64_t k, int depth) { return ancestor(k, depth - 1); }
static const uint64_t NO_KEY = ~0ull;  // {UINT32_MAX, UINT32_MAX}
// same-depth face neighbour, faces 0..5 = +x,-x,+y,-y,+z,-z (balance.cpp:32-49)
static inline uint64_t face_key(uint64_t k, int face, int depth) {
    uint32_t x, y, z;
    decode(k, x, y, z);
    const uint32_t step = 1u << (21 - depth), bound = 1u << 21;
    switch (face) {
        case 0: if (x + step >= bound) return NO_KEY; x += step; break;
        case 1: if (x < step) return NO_KEY; x -= step; break;
        case 2: if (y + step >= bound) return NO_KEY; y += step; break;
        case 3: if (y < step) return NO_KEY; y -= step; break;
        case 4: if (z + step >= bound) return NO_KEY; z += step; break;
        case 5: if (z < step) return NO_KEY; z -= step; break;
        default: return NO_KEY;
    }
    return encode(x, y, z);
}
static inline bool is_none(uint64_t k) { return (k >> 32) == 0xffffffffu; }

// ---- float -> int truncation with x86 semantics ------------------------------
// The reference uses static_cast<int>(float) (histogram.cpp:91-92,99,155), which
// is undefined for NaN and out-of-range values; on x86-64, where the golden
// fixtures are made, cvttss2si returns INT_MIN for them.  The oracle and the
// CUDA kernels both implement that result explicitly so that neither depends on
// the host ISA.
static inline int trunc_i32(float x) {
    if (!(x > -2147483904.0f && x < 2147483648.0f)) return std::numeric_limits<int>::min();
    return static_cast<int>(x);
}

// ---- histogram statistics (histogram.cpp:12-31) -----------------------------
template <int NB>
static float median_indicator(const uint32_t* b) {
    uint32_t tot = 0;
    for (int k = 0; k < NB; ++k) tot += b[k];
    if (tot == 0) return 0.0f;
    uint32_t cum = 0;
    for (int k = 0; k < NB; ++k) {
        cum += b[k];
        if (cum * 2 >= tot) return -1.0f + (k + 0.5f) / (NB / 2.0f);
    }
    return 1.0f;
}
template <int NB>
static float mean_indicator(const uint32_t* b) {
    uint32_t tot = 0;
    for (int k = 0; k < NB; ++k) tot += b[k];
    if (tot == 0) return 0.0f;
    float sum = 0.0f;
    for (int k = 0; k < NB; ++k) sum += b[k] * (-1.0f + (k + 0.5f) / (NB / 2.0f));
    return sum / tot;
}

// ---- depth-map pyramid (histogram.cpp:35-74) --------------------------------
// Level dimensions: halve (integer division, at least 1) while both sides of the
// previous level exceed 1, at most 12 times.
static int pyramid_dims(int W, int H, int32_t* dims /* 2*13 */) {
    int n = 0;
    dims[0] = W; dims[1] = H; n = 1;
    for (int l = 0; l < 12; ++l) {
        int pw = dims[2 * (n - 1)], ph = dims[2 * (n - 1) + 1];
        if (pw <= 1 || ph <= 1) break;
        dims[2 * n] = std::max(1, pw / 2);
        dims[2 * n + 1] = std::max(1, ph / 2);
        ++n;
    }
    return n;
}
// Each coarse texel is the mean of the finite, positive texels among its (up to)
// four children, visited dv-outer / du-inner; NaN when none qualifies.
static void pyramid_build(const float* base, int W, int H, float* out, int32_t* n_levels,
                          int32_t* dims) {
    int n = pyramid_dims(W, H, dims);
    *n_levels = n;
    std::memcpy(out, base, sizeof(float) * size_t(W) * H);
    size_t prev_off = 0, off = size_t(W) * H;
    for (int l = 1; l < n; ++l) {
        int pw = dims[2 * (l - 1)], ph = dims[2 * (l - 1) + 1];
        int w = dims[2 * l], h = dims[2 * l + 1];
        const float* prev = out + prev_off;
        float* cur = out + off;
        for (int v = 0; v < h; ++v)
            for (int u = 0; u < w; ++u) {
                float sum = 0.0f;
                int cnt = 0;
                for (int dv = 0; dv < 2; ++dv)
                    for (int du = 0; du < 2; ++du) {
                        int pu = 2 * u + du, pv = 2 * v + dv;
                        if (pu < pw && pv < ph) {
                            float d = prev[size_t(pv) * pw + pu];
                            if (std::isfinite(d) && d > 0.0f) { sum += d; ++cnt; }
                        }
                    }
                cur[size_t(v) * w + u] = cnt > 0 ? sum / cnt : std::numeric_limits<float>::quiet_NaN();
            }
        prev_off = off;
        off += size_t(w) * h;
    }
}

// Camera as the histogram kernel sees it: the pyramid plus Rt_inv (row-major)
// and the base-level intrinsics.
struct Camera {
    float rt_inv[16];
    float fx, fy, cx, cy;
    int32_t width, height;
    int32_t lidar;
    int32_t n_levels;
    int32_t dims[26];
    int64_t offs[13];
    const float* texels;
};

// DepthMipmap::project (histogram.cpp:76-106).  Matrix-vector product in the
// pinned order (((m0*x + m1*y) + m2*z) + m3*1).
static bool project(const Camera& c, float px, float py, float pz, float r_c, int& level,
                    int& uo, int& vo, float& cam_z) {
    if (c.n_levels <= 0) return false;
    const float* m = c.rt_inv;
    float cx_ = m[0] * px; cx_ = cx_ + m[1] * py; cx_ = cx_ + m[2] * pz; cx_ = cx_ + m[3] * 1.0f;
    float cy_ = m[4] * px; cy_ = cy_ + m[5] * py; cy_ = cy_ + m[6] * pz; cy_ = cy_ + m[7] * 1.0f;
    float cz_ = m[8] * px; cz_ = cz_ + m[9] * py; cz_ = cz_ + m[10] * pz; cz_ = cz_ + m[11] * 1.0f;
    float z = cz_;
    if (z <= 0.0f) return false;
    float u_f = cx_ / z * c.fx + c.cx;
    float v_f = cy_ / z * c.fy + c.cy;
    int u0 = trunc_i32(u_f), v0 = trunc_i32(v_f);
    if (u0 < 0 || u0 >= c.width || v0 < 0 || v0 >= c.height) return false;
    cam_z = z;
    float fp = std::abs(c.fx) * r_c / z;
    int lv = std::max(0, trunc_i32(std::log2(std::max(1.0f, fp))));
    lv = std::min(lv, c.n_levels - 1);
    level = lv;
    uo = std::clamp(u0 >> lv, 0, c.dims[2 * lv] - 1);
    vo = std::clamp(v0 >> lv, 0, c.dims[2 * lv + 1] - 1);
    return true;
}

// cube_center (histogram.cpp:118-125)
static void cube_center(const Cube& cb, const float* origin, float r_root, float* P) {
    uint32_t fx, fy, fz;
    decode(key_of(cb.hi, cb.lo), fx, fy, fz);
    int shift = 21 - cb.depth;
    uint32_t ix = fx >> shift, iy = fy >> shift, iz = fz >> shift;
    float cs = 2.0f * r_root / static_cast<float>(1u << cb.depth);
    P[0] = origin[0] + (ix + 0.5f) * cs;
    P[1] = origin[1] + (iy + 0.5f) * cs;
    P[2] = origin[2] + (iz + 0.5f) * cs;
}

// compute_histograms (histogram.cpp:127-163), NB bins: bin = (int)((a+1)*NB/2).
template <int NB>
static void compute_histograms(const Cube* cubes, int64_t n, const Camera* cams, int ncam,
                               const float* origin, float r_root, uint32_t* out, int nthreads) {
    std::memset(out, 0, sizeof(uint32_t) * NB * size_t(n));
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads) if (nthreads > 1)
    for (int64_t ci = 0; ci < n; ++ci) {
        const Cube& cb = cubes[ci];
        float P[3];
        cube_center(cb, origin, r_root, P);
        float r_c = cb.r_c;
        float delta = 6.0f * r_c;
        float eta = 18.0f * r_c;
        if (r_c <= 0.0f) continue;
        uint32_t* h = out + size_t(ci) * NB;
        for (int c = 0; c < ncam; ++c) {
            int lv, uu, vv;
            float cz;
            if (!project(cams[c], P[0], P[1], P[2], r_c, lv, uu, vv, cz)) continue;
            float sd = cams[c].texels[cams[c].offs[lv] + int64_t(vv) * cams[c].dims[2 * lv] + uu];
            if (!std::isfinite(sd) || sd <= 0.0f) continue;
            float a = sd - cz;
            if (a < -eta) continue;
            a = std::clamp(a / delta, -1.0f, 1.0f);
            int bin = trunc_i32((a + 1.0f) * (NB / 2.0f));
            bin = std::clamp(bin, 0, NB - 1);
            h[bin] += cams[c].lidar ? 5u : 1u;
        }
    }
}

// ---- TGV (tgv.cpp) -----------------------------------------------------------
enum Mode { INMEM = 0, OC = 1, STREAM = 2 };

// Data term of one cube: median of the histogram and the shrink step tau*tot
// (prox_data, tgv.cpp:75-94).  `has` is false for an empty histogram (prox is
// the identity there).
template <typename S>
struct DataTerm { S med; S shrink; bool has; };

template <typename S, int NB>
static DataTerm<S> data_term(const uint32_t* b, S tau) {
    uint32_t tot = 0;
    for (int k = 0; k < NB; ++k) tot += b[k];
    DataTerm<S> d{S(0), S(0), tot != 0};
    if (!d.has) return d;
    uint32_t cum = 0;
    for (int k = 0; k < NB; ++k) {
        cum += b[k];
        if (cum * 2 >= tot) { d.med = S(-1) + (S(k) + S(0.5)) / S(NB / 2.0); break; }
    }
    d.shrink = tau * static_cast<S>(tot);
    return d;
}
template <typename S>
static inline S prox(S z, const DataTerm<S>& d) {
    if (!d.has) return z;
    S diff = z - d.med;
    if (diff > d.shrink) return z - d.shrink;
    if (diff < -d.shrink) return z + d.shrink;
    return d.med;
}
template <typename S>
static inline void clip3(S* p, S r) {
    S n2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
    if (n2 > r * r) {
        S s = r / std::sqrt(n2);
        p[0] *= s; p[1] *= s; p[2] *= s;
    }
}
template <typename S>
static inline void clip6(S* q, S r) {
    S n2 = 0;
    for (int i = 0; i < 6; ++i) n2 += q[i] * q[i];
    if (n2 > r * r) {
        S s = r / std::sqrt(n2);
        for (int i = 0; i < 6; ++i) q[i] *= s;
    }
}

template <typename S>
struct St { S u, v[3], p[3], q[6]; };

// Counters reported by the oracle solve (per level: iterations actually run,
// final residual).
struct LevelStats { int32_t depth; int32_t iters_run; int64_t active; double residual; double energy; };

// One level of primal-dual iterations over `act` (indices into the arrays
// below), restating run_level / run_level_frozen / run_level_streaming
// (tgv.cpp:137-232, 241-352, 704-798).  Neighbour reads go through `nb`
// (6 per active entry).  `live(j)` decides whether an out-of-set neighbour's
// bars come from the live arrays (true) or the frozen ones; dual values are
// always read from `st`.
template <typename S, typename LiveFn>
static void run_level(const std::vector<uint32_t>& act, const std::vector<int32_t>& nb,
                      const std::vector<DataTerm<S>>& dt, std::vector<St<S>>& st,
                      std::vector<S>& ub, std::vector<S>& vbx, std::vector<S>& vby,
                      std::vector<S>& vbz, const std::vector<S>* fu, const std::vector<S>* fvx,
                      const std::vector<S>* fvy, const std::vector<S>* fvz, LiveFn live,
                      S alpha0, S alpha1, int iters, S tol, int check_every, LevelStats* ls,
                      int nthreads) {
    const S sigma = S(0.25), tau = S(0.25);
    const int64_t na = static_cast<int64_t>(act.size());
    std::vector<S> un(na), vxn(na), vyn(na), vzn(na);
    auto UB = [&](int32_t j) -> S { return live(j) ? ub[j] : (*fu)[j]; };
    auto VB = [&](int32_t j, int c) -> S {
        if (live(j)) return c == 0 ? vbx[j] : c == 1 ? vby[j] : vbz[j];
        return c == 0 ? (*fvx)[j] : c == 1 ? (*fvy)[j] : (*fvz)[j];
    };
    int it = 0;
    double resid = 0.0;
    for (; it < iters; ++it) {
        const bool check = tol > S(0) && check_every > 0 && ((it + 1) % check_every == 0 || it + 1 == iters);
        double dprim = 0, ddual = 0, nprim = 0, ndual = 0;
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) reduction(+ : ddual)
        for (int64_t a = 0; a < na; ++a) {
            const uint32_t i = act[a];
            const int32_t* n6 = &nb[size_t(a) * 6];
            auto ubf = [&](int f) -> S { return n6[f] >= 0 ? UB(n6[f]) : ub[i]; };
            S p_old[3] = {st[i].p[0], st[i].p[1], st[i].p[2]};
            st[i].p[0] += sigma * (ubf(0) - ub[i] - vbx[i]);
            st[i].p[1] += sigma * (ubf(2) - ub[i] - vby[i]);
            st[i].p[2] += sigma * (ubf(4) - ub[i] - vbz[i]);
            clip3(st[i].p, alpha1);
            auto vb = [&](int f, int c) -> S {
                if (n6[f] < 0) return c == 0 ? vbx[i] : c == 1 ? vby[i] : vbz[i];
                return VB(n6[f], c);
            };
            S e[6] = {vb(0, 0) - vbx[i],
                      vb(2, 1) - vby[i],
                      vb(4, 2) - vbz[i],
                      S(0.5) * (vb(2, 0) - vbx[i] + vb(0, 1) - vby[i]),
                      S(0.5) * (vb(4, 0) - vbx[i] + vb(0, 2) - vbz[i]),
                      S(0.5) * (vb(4, 1) - vby[i] + vb(2, 2) - vbz[i])};
            S q_old[6];
            for (int k = 0; k < 6; ++k) { q_old[k] = st[i].q[k]; st[i].q[k] += sigma * e[k]; }
            clip6(st[i].q, alpha0);
            if (check) {
                // per-cube terms in S, in component order; sums over cubes in FP64
                S d = S(0);
                for (int k = 0; k < 3; ++k) { S t = st[i].p[k] - p_old[k]; d = d + t * t; }
                for (int k = 0; k < 6; ++k) { S t = st[i].q[k] - q_old[k]; d = d + t * t; }
                ddual += double(d);
            }
        }
        // The p and q sweeps of the reference are separate loops; fusing them per
        // cube is exact because q reads only the bars, which p does not write.
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1)
        for (int64_t a = 0; a < na; ++a) {
            const uint32_t i = act[a];
            const int32_t* n6 = &nb[size_t(a) * 6];
            auto gp = [&](int f, int c) -> S { return n6[f] >= 0 ? st[n6[f]].p[c] : S(0); };
            auto gq = [&](int f, int c) -> S { return n6[f] >= 0 ? st[n6[f]].q[c] : S(0); };
            S div_p = (st[i].p[0] - gp(1, 0)) + (st[i].p[1] - gp(3, 1)) + (st[i].p[2] - gp(5, 2));
            un[a] = prox(st[i].u + tau * div_p, dt[i]);
            S dqx = (st[i].q[0] - gq(1, 0)) + (st[i].q[3] - gq(3, 3)) + (st[i].q[4] - gq(5, 4));
            S dqy = (st[i].q[3] - gq(1, 3)) + (st[i].q[1] - gq(3, 1)) + (st[i].q[5] - gq(5, 5));
            S dqz = (st[i].q[4] - gq(1, 4)) + (st[i].q[5] - gq(3, 5)) + (st[i].q[2] - gq(5, 2));
            vxn[a] = st[i].v[0] + tau * (st[i].p[0] + dqx);
            vyn[a] = st[i].v[1] + tau * (st[i].p[1] + dqy);
            vzn[a] = st[i].v[2] + tau * (st[i].p[2] + dqz);
        }
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) reduction(+ : dprim, nprim, ndual)
        for (int64_t a = 0; a < na; ++a) {
            const uint32_t i = act[a];
            if (check) {
                const S t0 = un[a] - st[i].u, t1 = vxn[a] - st[i].v[0];
                const S t2 = vyn[a] - st[i].v[1], t3 = vzn[a] - st[i].v[2];
                S dp = t0 * t0;
                dp = dp + t1 * t1; dp = dp + t2 * t2; dp = dp + t3 * t3;
                dprim += double(dp);
                S np = un[a] * un[a];
                np = np + vxn[a] * vxn[a]; np = np + vyn[a] * vyn[a]; np = np + vzn[a] * vzn[a];
                nprim += double(np);
                S nd = S(0);
                for (int k = 0; k < 3; ++k) nd = nd + st[i].p[k] * st[i].p[k];
                for (int k = 0; k < 6; ++k) nd = nd + st[i].q[k] * st[i].q[k];
                ndual += double(nd);
            }
            ub[i] = S(2) * un[a] - st[i].u;
            vbx[i] = S(2) * vxn[a] - st[i].v[0];
            vby[i] = S(2) * vyn[a] - st[i].v[1];
            vbz[i] = S(2) * vzn[a] - st[i].v[2];
            st[i].u = un[a];
            st[i].v[0] = vxn[a];
            st[i].v[1] = vyn[a];
            st[i].v[2] = vzn[a];
        }
        if (check) {
            // Relative fixed-point residual of the primal-dual iteration
            // (sigma = tau): (|x+ - x| + |y+ - y|) / (|x+| + |y+|), FP64.
            double num = std::sqrt(dprim) + std::sqrt(ddual);
            double den = std::sqrt(nprim) + std::sqrt(ndual);
            resid = den > 0 ? num / den : 0.0;
            if (resid <= double(tol)) { ++it; break; }
        }
    }
    if (ls) { ls->iters_run = it; ls->residual = resid; }
}

template <typename S, int NB>
struct Problem {
    const Cube* cubes;
    int64_t n;
    const uint32_t* hists;
    const Leaf* leaves;
    int nleaf;
    int mode;
    S alpha0, alpha1;
    int iters;
    int init;            // 0 = median, 1 = zero, 2 = caller u
    const float* u_init; // init == 2
    S tol;
    int check_every;
    int nthreads;
    // Sharded streaming (one rank's share of one level): iterate only the
    // leaves with a nonzero mask entry, run only level `only_level`, start from
    // `state_in` instead of the initial state.
    const uint8_t* leaf_mask = nullptr;
    int only_level = -1;
    const State* state_in = nullptr;
    int keep_init_u = 0;  // extension: parent init copies only v (warm / zero start per level)
    // Extension (warm start of the whole primal-dual state): when set, every
    // cube takes level_init's (u, v, p, q) at its own level's start, in place of
    // the parent copy and the zeroing of p and q; until then it holds the
    // initial state `init` gives, like every cube of the plain solve.
    const State* level_init = nullptr;
};

// Reference binary search over the Morton-sorted cube array: returns the first
// probed index whose code equals `k` (CubeFileReader::lookup, tgv.cpp:673-683).
static uint32_t file_lookup(const std::vector<uint64_t>& keys, uint64_t k) {
    uint32_t lo = 0, hi = static_cast<uint32_t>(keys.size());
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (keys[mid] == k) return mid;
        if (keys[mid] < k) lo = mid + 1; else hi = mid;
    }
    return 0xffffffffu;
}

template <typename S>
static void set_state(St<S>& d, const State& s) {
    d.u = S(s.u);
    for (int c = 0; c < 3; ++c) { d.v[c] = S(s.v[c]); d.p[c] = S(s.p[c]); }
    for (int c = 0; c < 6; ++c) d.q[c] = S(s.q[c]);
}

template <typename S, int NB>
static int solve(const Problem<S, NB>& P, St<S>* out, LevelStats* lstats, int* n_lstats) {
    const int64_t N = P.n;
    const S tau = S(0.25);
    std::vector<St<S>> st(N);
    std::vector<DataTerm<S>> dt(N);
    std::vector<uint64_t> keys(N);
    for (int64_t i = 0; i < N; ++i) {
        keys[i] = key_of(P.cubes[i].hi, P.cubes[i].lo);
        dt[i] = data_term<S, NB>(P.hists + size_t(i) * NB, tau);
        st[i] = St<S>{};
        if (P.init == 0) st[i].u = dt[i].has ? dt[i].med : S(0);  // median_indicator
        else if (P.init == 2) st[i].u = S(P.u_init[i]);
        if (P.state_in) {
            const State& s = P.state_in[i];
            st[i].u = S(s.u);
            for (int c = 0; c < 3; ++c) { st[i].v[c] = S(s.v[c]); st[i].p[c] = S(s.p[c]); }
            for (int c = 0; c < 6; ++c) st[i].q[c] = S(s.q[c]);
        }
    }
    int nls = 0;
    if (N == 0) { if (n_lstats) *n_lstats = 0; return 0; }
    int min_d = 21, max_d = 0;
    for (int64_t i = 0; i < N; ++i) {
        min_d = std::min(min_d, int(P.cubes[i].depth));
        max_d = std::max(max_d, int(P.cubes[i].depth));
    }
    std::vector<S> ub(N), vbx(N, S(0)), vby(N, S(0)), vbz(N, S(0));
    for (int64_t i = 0; i < N; ++i) ub[i] = st[i].u;

    if (P.mode == INMEM || P.mode == OC) {
        // cmap: code -> max index (tgv.cpp:367-370)
        std::unordered_map<uint64_t, uint32_t> cmap;
        cmap.reserve(size_t(N) * 2);
        for (int64_t i = 0; i < N; ++i) cmap[keys[i]] = uint32_t(i);
        auto find = [&](uint64_t k) -> int32_t {
            auto it = cmap.find(k);
            return it == cmap.end() ? -1 : int32_t(it->second);
        };
        // neighbor_idx_ctf (tgv.cpp:97-109)
        auto nb_of = [&](uint32_t i, int f) -> int32_t {
            int d = P.cubes[i].depth;
            uint64_t nk = face_key(keys[i], f, d);
            if (is_none(nk)) return -1;
            int32_t r = find(nk);
            if (r >= 0) return r;
            if (d > 0) return find(parent_key(nk, d));
            return -1;
        };
        // FP64 primal energy of a level's state (the GPU library reports it per
        // level; no counterpart in the reference): tot |u - med| + alpha1 |grad u - v|
        // + alpha0 |e(v)|, forward differences to the in-memory neighbour (a
        // missing one counts as the cube itself), e(v) in Voigt form with the
        // off-diagonals halved and counted once.
        auto energy_of = [&](const std::vector<uint32_t>& lv) -> double {
            double e = 0.0;
            for (uint32_t i : lv) {
                const St<S>& c0 = st[i];
                uint32_t tot = 0;
                for (int k = 0; k < NB; ++k) tot += P.hists[size_t(i) * NB + k];
                if (tot) e += double(tot) * std::fabs(double(c0.u) - double(dt[i].med));
                double nu[3], nv[3][3];
                for (int c = 0; c < 3; ++c) {
                    const int32_t j = nb_of(i, 2 * c);
                    const St<S>& t = j < 0 ? c0 : st[j];
                    nu[c] = double(t.u);
                    for (int k = 0; k < 3; ++k) nv[c][k] = double(t.v[k]);
                }
                const double u = c0.u, v0 = c0.v[0], v1 = c0.v[1], v2 = c0.v[2];
                const double g0 = (nu[0] - u) - v0, g1 = (nu[1] - u) - v1, g2 = (nu[2] - u) - v2;
                e += double(P.alpha1) * std::sqrt(g0 * g0 + g1 * g1 + g2 * g2);
                const double e0 = nv[0][0] - v0, e1 = nv[1][1] - v1, e2 = nv[2][2] - v2;
                const double e3 = 0.5 * ((nv[1][0] - v0) + (nv[0][1] - v1));
                const double e4 = 0.5 * ((nv[2][0] - v0) + (nv[0][2] - v2));
                const double e5 = 0.5 * ((nv[2][1] - v1) + (nv[1][2] - v2));
                e += double(P.alpha0) * std::sqrt(e0 * e0 + e1 * e1 + e2 * e2 + e3 * e3 + e4 * e4 + e5 * e5);
            }
            return e;
        };
        std::vector<std::vector<uint32_t>> by_d(max_d + 1);
        for (int64_t i = 0; i < N; ++i) by_d[P.cubes[i].depth].push_back(uint32_t(i));
        for (int L = min_d; L <= max_d; ++L) {
            const auto& all = by_d[L];
            if (all.empty()) continue;
            if (P.level_init) {  // whole given state at the level's start
                for (uint32_t i : all) {
                    set_state(st[i], P.level_init[i]);
                    ub[i] = st[i].u; vbx[i] = st[i].v[0]; vby[i] = st[i].v[1]; vbz[i] = st[i].v[2];
                }
            } else if (L > min_d) {  // parent copy (tgv.cpp:391-409)
                for (uint32_t i : all) {
                    int32_t pi = find(parent_key(keys[i], L));
                    if (pi >= 0) {
                        if (!P.keep_init_u) st[i].u = st[pi].u;
                        for (int c = 0; c < 3; ++c) st[i].v[c] = st[pi].v[c];
                    }
                    for (int c = 0; c < 3; ++c) st[i].p[c] = S(0);
                    for (int c = 0; c < 6; ++c) st[i].q[c] = S(0);
                    ub[i] = st[i].u; vbx[i] = st[i].v[0]; vby[i] = st[i].v[1]; vbz[i] = st[i].v[2];
                }
            }
            LevelStats ls{L, 0, int64_t(all.size()), 0.0, 0.0};
            if (P.mode == INMEM) {
                std::vector<int32_t> nb(all.size() * 6);
                for (size_t a = 0; a < all.size(); ++a)
                    for (int f = 0; f < 6; ++f) nb[a * 6 + f] = nb_of(all[a], f);
                run_level(all, nb, dt, st, ub, vbx, vby, vbz, (const std::vector<S>*)nullptr,
                          (const std::vector<S>*)nullptr, (const std::vector<S>*)nullptr,
                          (const std::vector<S>*)nullptr, [](int32_t) { return true; }, P.alpha0,
                          P.alpha1, P.iters, P.tol, P.check_every, &ls, P.nthreads);
            } else {
                // frozen snapshot of the bars (tgv.cpp:484-487), then leaves in order
                const std::vector<S> fu = ub, fvx = vbx, fvy = vby, fvz = vbz;
                int it_max = 0;
                for (int l = 0; l < P.nleaf; ++l) {
                    const uint32_t f0 = P.leaves[l].first_idx, f1 = P.leaves[l].last_idx;
                    auto lo = std::lower_bound(all.begin(), all.end(), f0);
                    auto hi = std::upper_bound(all.begin(), all.end(), f1);
                    if (lo == hi) continue;
                    std::vector<uint32_t> la(lo, hi);
                    std::vector<int32_t> nb(la.size() * 6);
                    for (size_t a = 0; a < la.size(); ++a)
                        for (int f = 0; f < 6; ++f) nb[a * 6 + f] = nb_of(la[a], f);
                    auto live = [&](int32_t j) { return uint32_t(j) >= f0 && uint32_t(j) <= f1; };
                    LevelStats lls = ls;
                    run_level(la, nb, dt, st, ub, vbx, vby, vbz, &fu, &fvx, &fvy, &fvz, live,
                              P.alpha0, P.alpha1, P.iters, P.tol, P.check_every, &lls, P.nthreads);
                    it_max = std::max(it_max, lls.iters_run);
                    ls.residual = std::max(ls.residual, lls.residual);
                }
                ls.iters_run = it_max;
            }
            ls.energy = energy_of(all);
            if (lstats) lstats[nls] = ls;
            ++nls;
        }
    } else {
        // ---- streaming semantics (tgv.cpp:802-1070), held in memory ----------
        auto leaf_range = [&](int l, uint32_t& f0, uint32_t& n_leaf) -> bool {
            uint32_t a = P.leaves[l].first_idx, b = P.leaves[l].last_idx;
            if (int64_t(a) >= N || a > b) return false;
            uint32_t end = uint32_t(std::min<int64_t>(int64_t(b) + 1, N));
            f0 = a; n_leaf = end - a;
            return true;
        };
        for (int L = min_d; L <= max_d; ++L) {
            if (P.only_level >= 0 && L != P.only_level) continue;
            if (P.level_init) {  // whole given state at the level's start, leaf by leaf
                for (int l = 0; l < P.nleaf; ++l) {
                    uint32_t f0, nl;
                    if (!leaf_range(l, f0, nl)) continue;
                    for (uint32_t li = 0; li < nl; ++li)
                        if (P.cubes[f0 + li].depth == L) set_state(st[f0 + li], P.level_init[f0 + li]);
                }
            } else if (L > min_d) {  // parent init, leaf by leaf (tgv.cpp:878-934)
                for (int l = 0; l < P.nleaf; ++l) {
                    uint32_t f0, nl;
                    if (!leaf_range(l, f0, nl)) continue;
                    for (uint32_t li = 0; li < nl; ++li) {
                        uint32_t i = f0 + li;
                        if (P.cubes[i].depth != L) continue;
                        uint32_t g = file_lookup(keys, parent_key(keys[i], L));
                        if (g != 0xffffffffu) {
                            if (!P.keep_init_u) st[i].u = st[g].u;
                            for (int c = 0; c < 3; ++c) st[i].v[c] = st[g].v[c];
                        }
                        for (int c = 0; c < 3; ++c) st[i].p[c] = S(0);
                        for (int c = 0; c < 6; ++c) st[i].q[c] = S(0);
                    }
                }
            }
            // frozen bars = state u/v of every cube (build_bars_frozen, tgv.cpp:606-635)
            std::vector<S> fu(N), fvx(N), fvy(N), fvz(N);
            for (int64_t i = 0; i < N; ++i) {
                fu[i] = st[i].u; fvx[i] = st[i].v[0]; fvy[i] = st[i].v[1]; fvz[i] = st[i].v[2];
            }
            LevelStats ls{L, 0, 0, 0.0, 0.0};
            bool any = false;
            for (int l = 0; l < P.nleaf; ++l) {
                uint32_t f0, nl;
                if (!leaf_range(l, f0, nl)) continue;
                if (P.leaf_mask && !P.leaf_mask[l]) continue;  // another rank's leaf
                std::vector<uint32_t> act;
                for (uint32_t li = 0; li < nl; ++li)
                    if (P.cubes[f0 + li].depth == L) act.push_back(li);
                if (act.empty()) continue;
                any = true;
                // leaf-local code map: code -> max local index (tgv.cpp:955-958)
                std::unordered_map<uint64_t, uint32_t> lmap;
                lmap.reserve(nl * 2);
                for (uint32_t li = 0; li < nl; ++li) lmap[keys[f0 + li]] = li;
                // border codes (tgv.cpp:960-979)
                std::vector<uint64_t> bcodes;
                for (uint32_t li : act) {
                    for (int f = 0; f < 6; ++f) {
                        uint64_t nk = face_key(keys[f0 + li], f, L);
                        if (is_none(nk)) continue;
                        if (lmap.count(nk)) continue;
                        bcodes.push_back(nk);
                        if (L > 0) {
                            uint64_t pk = parent_key(nk, L);
                            if (!lmap.count(pk)) bcodes.push_back(pk);
                        }
                    }
                }
                std::sort(bcodes.begin(), bcodes.end());
                bcodes.erase(std::unique(bcodes.begin(), bcodes.end()), bcodes.end());
                std::vector<uint32_t> bglob;
                std::unordered_map<uint64_t, uint32_t> local = lmap;
                for (uint64_t k : bcodes) {
                    uint32_t g = file_lookup(keys, k);
                    if (g == 0xffffffffu) continue;
                    if (g >= f0 && g <= f0 + nl - 1) continue;
                    local[keys[g]] = nl + uint32_t(bglob.size());
                    bglob.push_back(g);
                }
                const uint32_t nb_n = uint32_t(bglob.size());
                auto lfind = [&](uint64_t k) -> int32_t {
                    auto it = local.find(k);
                    return it == local.end() ? -1 : int32_t(it->second);
                };
                std::vector<int32_t> nbt(act.size() * 6, -1);
                for (size_t a = 0; a < act.size(); ++a)
                    for (int f = 0; f < 6; ++f) {
                        uint64_t nk = face_key(keys[f0 + act[a]], f, L);
                        if (is_none(nk)) continue;
                        int32_t r = lfind(nk);
                        if (r < 0 && L > 0) r = lfind(parent_key(nk, L));
                        nbt[a * 6 + f] = r;
                    }
                // local state: leaf cubes then border cubes with p/q zeroed
                std::vector<St<S>> sl(nl + nb_n);
                std::vector<DataTerm<S>> dl(nl + nb_n);
                for (uint32_t li = 0; li < nl; ++li) { sl[li] = st[f0 + li]; dl[li] = dt[f0 + li]; }
                for (uint32_t b = 0; b < nb_n; ++b) {
                    sl[nl + b] = st[bglob[b]];
                    for (int c = 0; c < 3; ++c) sl[nl + b].p[c] = S(0);
                    for (int c = 0; c < 6; ++c) sl[nl + b].q[c] = S(0);
                }
                std::vector<S> lub(nl + nb_n), lvx(nl + nb_n), lvy(nl + nb_n), lvz(nl + nb_n);
                for (uint32_t li = 0; li < nl; ++li) {
                    lub[li] = sl[li].u; lvx[li] = sl[li].v[0]; lvy[li] = sl[li].v[1]; lvz[li] = sl[li].v[2];
                }
                for (uint32_t b = 0; b < nb_n; ++b) {
                    lub[nl + b] = fu[bglob[b]]; lvx[nl + b] = fvx[bglob[b]];
                    lvy[nl + b] = fvy[bglob[b]]; lvz[nl + b] = fvz[bglob[b]];
                }
                LevelStats lls = ls;
                run_level(act, nbt, dl, sl, lub, lvx, lvy, lvz, (const std::vector<S>*)nullptr,
                          (const std::vector<S>*)nullptr, (const std::vector<S>*)nullptr,
                          (const std::vector<S>*)nullptr, [](int32_t) { return true; }, P.alpha0,
                          P.alpha1, P.iters, P.tol, P.check_every, &lls, P.nthreads);
                ls.iters_run = std::max(ls.iters_run, lls.iters_run);
                ls.residual = std::max(ls.residual, lls.residual);
                ls.active += int64_t(act.size());
                for (uint32_t li = 0; li < nl; ++li) st[f0 + li] = sl[li];
            }
            if (any) {
                if (lstats) lstats[nls] = ls;
                ++nls;
            }
        }
    }
    for (int64_t i = 0; i < N; ++i) out[i] = st[i];
    if (n_lstats) *n_lstats = nls;
    return 0;
}

// ---- Stage 1: cubes from a depth map (reference src/octree_builder.cpp:11-97,
//      src/depth_map.cpp:4-30) --------------------------------------------------
struct DepthMapO { float fx, fy, cx, cy; float rt[16]; int32_t width, height; const float* depths; };

static inline bool dm_valid(const DepthMapO& m, int u, int v) {
    if (u < 0 || v < 0 || u >= m.width || v >= m.height) return false;
    const float d = m.depths[size_t(v) * m.width + u];
    return std::isfinite(d) && d > 0.0f;
}
// unproject: cam = ((u - cx) d / fx, (v - cy) d / fy, d, 1); world = Rt cam (row sums left to right)
static inline void dm_unproject(const DepthMapO& m, int u, int v, float* p) {
    const float d = m.depths[size_t(v) * m.width + u];
    const float c[4] = {(float(u) - m.cx) * d / m.fx, (float(v) - m.cy) * d / m.fy, d, 1.0f};
    for (int i = 0; i < 3; ++i) {
        float acc = m.rt[4 * i] * c[0];
        for (int k = 1; k < 4; ++k) acc = acc + m.rt[4 * i + k] * c[k];
        p[i] = acc;
    }
}
static inline float dm_radius(const DepthMapO& m, int u, int v) {
    if (!dm_valid(m, u, v)) return 0.0f;
    float c[3];
    dm_unproject(m, u, v, c);
    const int du[4] = {1, -1, 0, 0}, dv[4] = {0, 0, 1, -1};
    float sum = 0.0f;
    int count = 0;
    for (int i = 0; i < 4; ++i) {
        const int nu = u + du[i], nv = v + dv[i];
        if (!dm_valid(m, nu, nv)) continue;
        float q[3];
        dm_unproject(m, nu, nv, q);
        const float x = q[0] - c[0], y = q[1] - c[1], z = q[2] - c[2];
        sum += std::sqrt(x * x + y * y + z * z);
        ++count;
    }
    if (count == 0) return 0.0f;
    return 0.5f * sum / count;
}
// cube_depth_for_radius; (int) of round(log2(y)) with the x86 result for inf/NaN (INT_MIN)
static int depth_for_radius(float r_x, float r_root, int max_depth) {
    if (r_x <= 0.0f) return max_depth;
    const float l = std::round(std::log2(r_root / (r_x * 1.125f)));
    int d = trunc_i32(l);
    if (d < 0) d = 0;
    if (d > max_depth) d = max_depth;
    for (int tries = 0; tries < 3; ++tries) {
        const float cell = r_root / static_cast<float>(1u << d);
        if (cell >= 0.75f * r_x && cell < 1.5f * r_x) break;
        if (cell < 0.75f * r_x) { if (d > 0) --d; else break; }
        else { if (d < max_depth) ++d; else break; }
    }
    return d;
}
// build_cubes_from_depthmap: pixel order, then a stable sort by code.
static void build_cubes(const DepthMapO& m, const float* o, float r_root, std::vector<Cube>& out) {
    const float inv_2r = 1.0f / (2.0f * r_root);
    std::vector<std::pair<uint64_t, Cube>> cs;
    for (int v = 0; v < m.height; ++v)
        for (int u = 0; u < m.width; ++u) {
            if (!dm_valid(m, u, v)) continue;
            const float r_x = dm_radius(m, u, v);
            if (r_x <= 0.0f) continue;
            float p[3];
            dm_unproject(m, u, v, p);
            const float n[3] = {(p[0] - o[0]) * inv_2r, (p[1] - o[1]) * inv_2r, (p[2] - o[2]) * inv_2r};
            if (n[0] < 0 || n[0] >= 1 || n[1] < 0 || n[1] >= 1 || n[2] < 0 || n[2] >= 1) continue;
            const int d = depth_for_radius(r_x, r_root, 21);
            const uint32_t g = 1u << d;
            uint32_t ix[3];
            for (int k = 0; k < 3; ++k) {
                const float f = n[k] * static_cast<float>(g);
                uint32_t q = f >= 0.0f ? static_cast<uint32_t>(f) : 0u;  // NaN -> 0 (x86 result)
                ix[k] = q >= g ? g - 1 : q;
            }
            const int sh = 21 - d;
            const uint64_t key = encode(ix[0] << sh, ix[1] << sh, ix[2] << sh);
            cs.push_back({key, Cube{uint32_t(key >> 32), uint32_t(key), r_x, d}});
        }
    std::stable_sort(cs.begin(), cs.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    out.resize(cs.size());
    for (size_t i = 0; i < cs.size(); ++i) out[i] = cs[i].second;
}

// ---- surface extraction (reference src/marching_cubes.cpp) ------------------
// A quad at the zero crossing of u is placed on every face pair of cubes whose
// u changes sign; vertices are merged by a 60-bit quantised key.
struct SurfMesh {
    std::vector<float> v;         // 3 per vertex
    std::vector<uint32_t> f;      // 3 per triangle
    std::vector<float> nrm;       // 3 per vertex (optional)
};

// World lower corner of a cube (cube_corner, marching_cubes.cpp:21-30).
static inline void cube_corner(const Cube& c, const float* o, float r_root, float* out, float& cs) {
    uint32_t fx, fy, fz;
    decode(key_of(c.hi, c.lo), fx, fy, fz);
    const int sh = 21 - c.depth;
    cs = 2.0f * r_root / static_cast<float>(1u << c.depth);
    out[0] = o[0] + static_cast<float>(fx >> sh) * cs;
    out[1] = o[1] + static_cast<float>(fy >> sh) * cs;
    out[2] = o[2] + static_cast<float>(fz >> sh) * cs;
}

// 20-bit quantisation and the packed 60-bit vertex key (marching_cubes.cpp:34-47).
static inline uint64_t vertex_key(const float* p, const float* o, float inv) {
    uint64_t k = 0;
    for (int a = 0; a < 3; ++a) {
        int q = trunc_i32((p[a] - o[a]) * inv + 0.5f);
        if (q < 0) q = 0;
        if (q > (1 << 20) - 1) q = (1 << 20) - 1;
        k |= static_cast<uint64_t>(q) << (20 * a);
    }
    return k;
}

// The quad of face pair (i, j) seen from cube i across face f: corners v0..v3
// (marching_cubes.cpp:124-158) and the winding flag (:167-168).
static inline bool face_quad(const Cube& ci, const Cube& cj, float ui, float uj, int f, const float* o,
                             float r_root, float q[4][3]) {
    float pi[3], pj[3], cs_i, cs_j;
    cube_corner(ci, o, r_root, pi, cs_i);
    cube_corner(cj, o, r_root, pj, cs_j);
    const float cs_min = cs_i < cs_j ? cs_i : cs_j;
    const float h = cs_min * 0.5f;
    const float t = ui / (ui - uj);
    const int ax = f / 2;
    float surf[3];
    const float ci_c = pi[ax] + cs_i * 0.5f, cj_c = pj[ax] + cs_j * 0.5f;
    surf[ax] = ci_c + t * (cj_c - ci_c);
    const float* small = cs_i <= cs_j ? pi : pj;
    for (int b = 0; b < 3; ++b)
        if (b != ax) surf[b] = small[b] + h;
    // tangential half-extents: x normal -> (y, z); y -> (z, x); z -> (x, y)
    const int t1 = ax == 0 ? 1 : ax == 1 ? 2 : 0;
    const int t2 = ax == 0 ? 2 : ax == 1 ? 0 : 1;
    float a1[3] = {0.0f, 0.0f, 0.0f}, a2[3] = {0.0f, 0.0f, 0.0f};
    a1[t1] = h;
    a2[t2] = h;
    for (int b = 0; b < 3; ++b) {
        q[0][b] = (surf[b] - a1[b]) - a2[b];
        q[1][b] = (surf[b] + a1[b]) - a2[b];
        q[2][b] = (surf[b] + a1[b]) + a2[b];
        q[3][b] = (surf[b] - a1[b]) + a2[b];
    }
    return (f % 2 == 0) ? (ui > 0.0f) : (ui < 0.0f);
}

static inline void push_quad(std::vector<uint32_t>& f, const uint32_t id[4], bool flip) {
    if (!flip) {
        f.insert(f.end(), {id[0], id[1], id[2], id[0], id[2], id[3]});
    } else {
        f.insert(f.end(), {id[0], id[2], id[1], id[0], id[3], id[2]});
    }
}

// extract_surface (marching_cubes.cpp:63-181): neighbour by code (largest
// index), else the parent code; self links skipped; each unordered index pair
// judged once, by its first visitor in (cube, face) order.
static void extract_surface(const Cube* cubes, const State* st, int64_t n, const uint8_t* has_data,
                            const float* o, float r_root, SurfMesh& m) {
    const float inv = static_cast<float>(1u << 20) / (2.0f * r_root);
    std::unordered_map<uint64_t, uint32_t> cmap;
    cmap.reserve(size_t(n) * 2);
    for (int64_t i = 0; i < n; ++i) cmap[key_of(cubes[i].hi, cubes[i].lo)] = uint32_t(i);
    auto find = [&](uint64_t k) -> int64_t {
        auto it = cmap.find(k);
        return it == cmap.end() ? -1 : int64_t(it->second);
    };
    std::unordered_map<uint64_t, char> seen;
    std::unordered_map<uint64_t, uint32_t> vmap;
    for (int64_t i = 0; i < n; ++i) {
        const uint64_t ki = key_of(cubes[i].hi, cubes[i].lo);
        for (int f = 0; f < 6; ++f) {
            const uint64_t nk = face_key(ki, f, cubes[i].depth);
            if (is_none(nk)) continue;
            int64_t j = find(nk);
            if (j < 0 && cubes[i].depth > 0) j = find(parent_key(nk, cubes[i].depth));
            if (j < 0 || j == i) continue;
            const uint64_t lo = uint64_t(std::min<int64_t>(i, j)), hi = uint64_t(std::max<int64_t>(i, j));
            if (!seen.emplace((lo << 32) | hi, 1).second) continue;
            if (has_data && !(has_data[i] && has_data[j])) continue;
            const float ui = st[i].u, uj = st[j].u;
            if ((ui >= 0.0f) == (uj >= 0.0f)) continue;
            float q[4][3];
            const bool flip = face_quad(cubes[i], cubes[j], ui, uj, f, o, r_root, q);
            uint32_t id[4];
            for (int c = 0; c < 4; ++c) {
                auto r = vmap.emplace(vertex_key(q[c], o, inv), uint32_t(m.v.size() / 3));
                if (r.second) m.v.insert(m.v.end(), {q[c][0], q[c][1], q[c][2]});
                id[c] = r.first->second;
            }
            push_quad(m.f, id, flip);
        }
    }
}

// compute_normals (marching_cubes.cpp:185-205): face normals (b-a) x (c-a)
// summed per vertex in triangle order, then divided by their length when it
// exceeds 1e-12.
static void compute_normals(SurfMesh& m) {
    const size_t nv = m.v.size() / 3, nt = m.f.size() / 3;
    m.nrm.assign(nv * 3, 0.0f);
    for (size_t t = 0; t < nt; ++t) {
        const float* a = &m.v[3 * m.f[3 * t]];
        const float* b = &m.v[3 * m.f[3 * t + 1]];
        const float* c = &m.v[3 * m.f[3 * t + 2]];
        const float d0 = b[0] - a[0], d1 = b[1] - a[1], d2 = b[2] - a[2];
        const float e0 = c[0] - a[0], e1 = c[1] - a[1], e2 = c[2] - a[2];
        const float nn[3] = {d1 * e2 - d2 * e1, d2 * e0 - d0 * e2, d0 * e1 - d1 * e0};
        for (int k = 0; k < 3; ++k)
            for (int ax = 0; ax < 3; ++ax) m.nrm[3 * m.f[3 * t + k] + ax] += nn[ax];
    }
    for (size_t vtx = 0; vtx < nv; ++vtx) {
        float* x = &m.nrm[3 * vtx];
        const float len = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        if (len > 1e-12f) { x[0] /= len; x[1] /= len; x[2] /= len; }
    }
}

// extract_surface_streaming (marching_cubes.cpp:374-580), held in memory:
// leaves in the given order; neighbour candidates in the order in-leaf exact,
// file bisection exact, in-leaf parent, file bisection parent, a candidate equal
// to the cube itself skipped; the finer side (equal depth: smaller index) owns
// a pair; both cubes need votes.  Vertices are numbered by first appearance and
// placed at their dequantised keys.
static void extract_surface_streaming(const Cube* cubes, const State* st, const uint32_t* tot, int64_t n,
                                      const Leaf* leaves, int nleaf, const float* o, float r_root,
                                      SurfMesh& m) {
    const float inv = static_cast<float>(1u << 20) / (2.0f * r_root);
    const float scale = 1.0f / inv;
    std::vector<uint64_t> keys(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) keys[i] = key_of(cubes[i].hi, cubes[i].lo);
    std::unordered_map<uint64_t, uint32_t> vmap;
    std::vector<uint64_t> vkeys;
    for (int l = 0; l < nleaf; ++l) {
        const uint32_t a = leaves[l].first_idx, b = leaves[l].last_idx;
        if (int64_t(a) >= n || a > b) continue;  // load_cubes_range clamps (octree_builder.cpp:131-135)
        const uint32_t e = uint32_t(std::min<int64_t>(int64_t(b), n - 1));
        std::unordered_map<uint64_t, uint32_t> lmap;
        for (uint32_t g = a; g <= e; ++g) lmap[keys[g]] = g;
        for (uint32_t gi = a; gi <= e; ++gi) {
            const Cube& ci = cubes[gi];
            for (int f = 0; f < 6; ++f) {
                const uint64_t nk = face_key(keys[gi], f, ci.depth);
                if (is_none(nk)) continue;
                uint32_t gj = 0xffffffffu;
                auto in_leaf = [&](uint64_t k) {
                    if (gj != 0xffffffffu) return;
                    auto it = lmap.find(k);
                    if (it != lmap.end() && it->second != gi) gj = it->second;
                };
                auto in_file = [&](uint64_t k) {
                    if (gj != 0xffffffffu) return;
                    const uint32_t g = file_lookup(keys, k);
                    if (g != 0xffffffffu && g != gi) gj = g;
                };
                in_leaf(nk);
                in_file(nk);
                if (ci.depth > 0) {
                    const uint64_t pk = parent_key(nk, ci.depth);
                    in_leaf(pk);
                    in_file(pk);
                }
                if (gj == 0xffffffffu) continue;
                const Cube& cj = cubes[gj];
                if (cj.depth > ci.depth) continue;
                if (cj.depth == ci.depth && gi > gj) continue;
                if (tot[gi] == 0 || tot[gj] == 0) continue;
                const float ui = st[gi].u, uj = st[gj].u;
                if ((ui >= 0.0f) == (uj >= 0.0f)) continue;
                float q[4][3];
                const bool flip = face_quad(ci, cj, ui, uj, f, o, r_root, q);
                uint32_t id[4];
                for (int c = 0; c < 4; ++c) {
                    const uint64_t k = vertex_key(q[c], o, inv);
                    auto r = vmap.emplace(k, uint32_t(vkeys.size()));
                    if (r.second) vkeys.push_back(k);
                    id[c] = r.first->second;
                }
                push_quad(m.f, id, flip);
            }
        }
    }
    m.v.resize(vkeys.size() * 3);
    for (size_t k = 0; k < vkeys.size(); ++k)
        for (int a = 0; a < 3; ++a)
            m.v[3 * k + a] = o[a] + static_cast<float>((vkeys[k] >> (20 * a)) & 0xFFFFFull) * scale;
}

}  // namespace orc

// ============================ C API (ctypes) =================================
extern "C" {

struct orc_params {
    float alpha0, alpha1;
    int32_t iters;
    int32_t init;         // 0 median (reference), 1 zero, 2 caller u
    float tol;            // 0: fixed iteration count (reference behaviour)
    int32_t check_every;  // residual period when tol > 0
    int32_t keep_init_u;  // 1: levels keep their initial u, copy only v from the parent
};

int orc_abi_version() { return 1; }

float orc_median_indicator(const uint32_t* bins, int nbins) {
    return nbins == 10 ? orc::median_indicator<10>(bins) : orc::median_indicator<8>(bins);
}
float orc_mean_indicator(const uint32_t* bins, int nbins) {
    return nbins == 10 ? orc::mean_indicator<10>(bins) : orc::mean_indicator<8>(bins);
}

// Pyramid level count and dims (2 per level, up to 13 levels) for a W x H map.
int orc_pyramid_dims(int W, int H, int32_t* dims) { return orc::pyramid_dims(W, H, dims); }

void orc_pyramid_build(const float* base, int W, int H, float* out, int32_t* n_levels, int32_t* dims) {
    orc::pyramid_build(base, W, H, out, n_levels, dims);
}

// Camera descriptor for the oracle: as in orc::Camera.
int orc_compute_histograms(const orc::Cube* cubes, int64_t n, const orc::Camera* cams, int ncam,
                           const float* origin, float r_root, int nbins, uint32_t* out,
                           int nthreads) {
    if (nbins == 8) orc::compute_histograms<8>(cubes, n, cams, ncam, origin, r_root, out, nthreads);
    else if (nbins == 10) orc::compute_histograms<10>(cubes, n, cams, ncam, origin, r_root, out, nthreads);
    else return -1;
    return 0;
}

int orc_project(const orc::Camera* cam, float px, float py, float pz, float r_c, int32_t* level,
                int32_t* u, int32_t* v, float* cam_z) {
    int lv = -1, uu = -1, vv = -1;
    float cz = 0.0f;
    bool ok = orc::project(*cam, px, py, pz, r_c, lv, uu, vv, cz);
    *level = lv; *u = uu; *v = vv; *cam_z = cz;
    return ok ? 1 : 0;
}

static int solve_f32(const orc::Cube* cubes, const uint32_t* hists, int64_t n, int nbins,
                     const orc::Leaf* leaves, int nleaf, int mode, const orc_params* p,
                     const float* u_init, orc::State* out, orc::LevelStats* ls, int* nls,
                     int nthreads, const orc::State* level_init = nullptr) {
    std::vector<orc::St<float>> s(static_cast<size_t>(n));
    int rc;
    if (nbins == 8) {
        orc::Problem<float, 8> P{cubes, n, hists, leaves, nleaf, mode, p->alpha0, p->alpha1, p->iters,
                                 p->init, u_init, p->tol, p->check_every, nthreads};
        P.keep_init_u = p->keep_init_u;
        P.level_init = level_init;
        rc = orc::solve<float, 8>(P, s.data(), ls, nls);
    } else if (nbins == 10) {
        orc::Problem<float, 10> P{cubes, n, hists, leaves, nleaf, mode, p->alpha0, p->alpha1, p->iters,
                                  p->init, u_init, p->tol, p->check_every, nthreads};
        P.keep_init_u = p->keep_init_u;
        P.level_init = level_init;
        rc = orc::solve<float, 10>(P, s.data(), ls, nls);
    } else {
        return -1;
    }
    static_assert(sizeof(orc::St<float>) == sizeof(orc::State), "state");
    std::memcpy(out, s.data(), sizeof(orc::State) * size_t(n));
    return rc;
}

// Float solve: mode 0 in-memory (tgv_minimize), 1 chunked (tgv_minimize_oc),
// 2 streaming (tgv_minimize_streaming).  out: n TGVCube records (52 B).
int orc_tgv_solve(const orc::Cube* cubes, const uint32_t* hists, int64_t n, int nbins,
                  const orc::Leaf* leaves, int nleaf, int mode, const orc_params* p,
                  const float* u_init, orc::State* out, orc::LevelStats* ls, int* nls,
                  int nthreads) {
    return solve_f32(cubes, hists, n, nbins, leaves, nleaf, mode, p, u_init, out, ls, nls, nthreads);
}

// Float solve in which every cube starts its level from the whole given state
// (u, v, p, q; TGVCube records) instead of the parent copy; the initial state
// of not-yet-run cubes comes from p->init as in the plain solve.  Warm start of
// the whole primal-dual state; no counterpart in the reference.
int orc_tgv_solve_level_init(const orc::Cube* cubes, const uint32_t* hists, int64_t n, int nbins,
                             const orc::Leaf* leaves, int nleaf, int mode, const orc_params* p,
                             const float* u_init, const orc::State* level_init, orc::State* out,
                             orc::LevelStats* ls, int* nls, int nthreads) {
    return solve_f32(cubes, hists, n, nbins, leaves, nleaf, mode, p, u_init, out, ls, nls, nthreads,
                     level_init);
}

// FP64 oracle of the same solver.  out: n * 13 doubles (u, v[3], p[3], q[6]).
int orc_tgv_solve_f64(const orc::Cube* cubes, const uint32_t* hists, int64_t n, int nbins,
                      const orc::Leaf* leaves, int nleaf, int mode, const orc_params* p,
                      const float* u_init, double* out, orc::LevelStats* ls, int* nls,
                      int nthreads) {
    std::vector<orc::St<double>> s(static_cast<size_t>(n));
    int rc;
    if (nbins == 8) {
        orc::Problem<double, 8> P{cubes, n, hists, leaves, nleaf, mode, double(p->alpha0),
                                  double(p->alpha1), p->iters, p->init, u_init, double(p->tol),
                                  p->check_every, nthreads};
        P.keep_init_u = p->keep_init_u;
        rc = orc::solve<double, 8>(P, s.data(), ls, nls);
    } else if (nbins == 10) {
        orc::Problem<double, 10> P{cubes, n, hists, leaves, nleaf, mode, double(p->alpha0),
                                   double(p->alpha1), p->iters, p->init, u_init, double(p->tol),
                                   p->check_every, nthreads};
        P.keep_init_u = p->keep_init_u;
        rc = orc::solve<double, 10>(P, s.data(), ls, nls);
    } else {
        return -1;
    }
    std::memcpy(out, s.data(), sizeof(double) * 13 * size_t(n));
    return rc;
}

}  // extern "C"

extern "C" {
// Exhaustive check of pyramid-level thresholds against this host's log2f:
// returns how many floats x in [1, 2^14) have (int)log2f(x) != #{k : x >= t[k]}
// (k = 1..12, capped at 12), plus checks at the top of the float range.
int64_t orc_check_thresholds(const float* t) {
    int64_t bad = 0;
    uint32_t a, b;
    float one = 1.0f, top = 16384.0f;
    std::memcpy(&a, &one, 4);
    std::memcpy(&b, &top, 4);
    auto lvl = [&](float x) {
        int l = 0;
        for (int k = 1; k < 13; ++k) l += x >= t[k] ? 1 : 0;
        return l;
    };
    for (uint32_t u = a; u < b; ++u) {
        float x;
        std::memcpy(&x, &u, 4);
        int r = std::min(12, orc::trunc_i32(std::log2(x)));
        if (r != lvl(x)) ++bad;
    }
    const float big[] = {16384.0f, 1e6f, 3.0e38f, std::numeric_limits<float>::max()};
    for (float x : big)
        if (std::min(12, orc::trunc_i32(std::log2(x))) != lvl(x)) ++bad;
    return bad;
}
}

extern "C" {
// One rank's share of one level of the streaming semantics: parent init of
// every leaf's level-L cubes, the level-start snapshot of every cube, then
// iterations of the leaves whose mask entry is nonzero.  `state` (n TGVCube
// records) is read as the state before the level and overwritten with the
// state after it.  Float, fixed iteration count.
int orc_stream_level(const orc::Cube* cubes, const uint32_t* hists, int64_t n, int nbins,
                     const orc::Leaf* leaves, int nleaf, const uint8_t* leaf_mask, int level,
                     const orc_params* p, orc::State* state, int nthreads) {
    std::vector<orc::St<float>> s(static_cast<size_t>(n));
    int rc;
    if (nbins == 8) {
        orc::Problem<float, 8> P{cubes, n, hists, leaves, nleaf, orc::STREAM, p->alpha0, p->alpha1, p->iters,
                                 0, nullptr, 0.0f, 1, nthreads};
        P.leaf_mask = leaf_mask; P.only_level = level; P.state_in = state;
        rc = orc::solve<float, 8>(P, s.data(), nullptr, nullptr);
    } else if (nbins == 10) {
        orc::Problem<float, 10> P{cubes, n, hists, leaves, nleaf, orc::STREAM, p->alpha0, p->alpha1, p->iters,
                                  0, nullptr, 0.0f, 1, nthreads};
        P.leaf_mask = leaf_mask; P.only_level = level; P.state_in = state;
        rc = orc::solve<float, 10>(P, s.data(), nullptr, nullptr);
    } else {
        return -1;
    }
    std::memcpy(state, s.data(), sizeof(orc::State) * size_t(n));
    return rc;
}
}

// ---- surface extraction entry points ----------------------------------------
extern "C" {
void* orc_extract_surface(const orc::Cube* cubes, const orc::State* state, int64_t n, const uint8_t* has_data,
                          const float* origin, float r_root, int32_t normals, int64_t* nv, int64_t* nf) {
    auto* m = new orc::SurfMesh;
    orc::extract_surface(cubes, state, n, has_data, origin, r_root, *m);
    if (normals) orc::compute_normals(*m);
    *nv = int64_t(m->v.size() / 3);
    *nf = int64_t(m->f.size() / 3);
    return m;
}

void* orc_extract_surface_streaming(const orc::Cube* cubes, const orc::State* state, const uint32_t* hist_total,
                                    int64_t n, const orc::Leaf* leaves, int32_t nleaf, const float* origin,
                                    float r_root, int64_t* nv, int64_t* nf) {
    auto* m = new orc::SurfMesh;
    orc::extract_surface_streaming(cubes, state, hist_total, n, leaves, nleaf, origin, r_root, *m);
    *nv = int64_t(m->v.size() / 3);
    *nf = int64_t(m->f.size() / 3);
    return m;
}

void orc_mesh_read(void* h, float* verts, uint32_t* faces, float* normals) {
    const auto* m = static_cast<const orc::SurfMesh*>(h);
    std::memcpy(verts, m->v.data(), m->v.size() * sizeof(float));
    std::memcpy(faces, m->f.data(), m->f.size() * sizeof(uint32_t));
    if (normals && !m->nrm.empty()) std::memcpy(normals, m->nrm.data(), m->nrm.size() * sizeof(float));
}

void orc_mesh_free(void* h) { delete static_cast<orc::SurfMesh*>(h); }
}

extern "C" int64_t orc_build_cubes(const orc::DepthMapO* m, const float* origin, float r_root, orc::Cube* out,
                                   int64_t cap) {
    std::vector<orc::Cube> cs;
    orc::build_cubes(*m, origin, r_root, cs);
    if (out && cap >= int64_t(cs.size())) std::memcpy(out, cs.data(), cs.size() * sizeof(orc::Cube));
    return int64_t(cs.size());
}

// ---- Stage 2: merge of sorted cube arrays (reference src/merge.cpp:7-97) -----
// The reference pops a min-heap keyed on the code alone, so when two inputs
// hold equal codes the pop order is whatever std::priority_queue does with
// ties.  This restatement takes them in input order (a stable merge); the two
// agree whenever no code occurs in more than one input.  A run of consecutive
// entries with equal (code, depth) becomes one cube whose r_c is the float sum
// of the run in pop order divided by its length (merge.cpp:64-88); equal codes
// of different depths that alternate are not merged, as in the reference.
namespace orc {
static void merge_cubes(const Cube* const* in, const int64_t* n, int k, std::vector<Cube>& out) {
    struct Ent { uint64_t code; int src; int64_t pos; };
    std::vector<Ent> all;
    for (int s = 0; s < k; ++s)
        for (int64_t i = 0; i < n[s]; ++i) all.push_back({key_of(in[s][i].hi, in[s][i].lo), s, i});
    std::stable_sort(all.begin(), all.end(), [](const Ent& a, const Ent& b) { return a.code < b.code; });
    out.clear();
    float sum = 0.0f;
    uint32_t cnt = 0;
    for (const Ent& e : all) {
        const Cube& c = in[e.src][e.pos];
        if (cnt && key_of(out.back().hi, out.back().lo) == e.code && out.back().depth == c.depth) {
            sum += c.r_c;
            ++cnt;
            continue;
        }
        if (cnt) out.back().r_c = sum / static_cast<float>(cnt);
        out.push_back(c);
        sum = c.r_c;
        cnt = 1;
    }
    if (cnt) out.back().r_c = sum / static_cast<float>(cnt);
}

// ---- Stage 3: 2:1 balance (reference src/balance.cpp:60-150) -----------------
// Cells are (depth, code).  Presence is tested on the exact code per depth; the
// output table is keyed like the reference's dc_key, depth << 60 | (code & (2^60 - 1))
// in 64-bit arithmetic (balance.cpp:57-59), so the code's top three bits are
// dropped and depths 16..21 share keys with depths 0..5.  Output cubes are
// decoded from that key.  Duplicate keys average their r_c in input order
// (balance.cpp:66-75).  A FIFO of cells, seeded with every input cube in input
// order, is processed one cell at a time: for each face whose same-depth
// neighbour is absent, whose neighbour's parent is absent, and which has any
// coarser ancestor present at depth <= d-2, the parent is added as a bridge with
// r_c = r_root / 2^(d-1), unless its key is already in the output table, and is
// queued (balance.cpp:82-121).  Cells of depth < 2 are skipped.
struct CellHash {
    size_t operator()(const std::pair<uint64_t, int>& c) const {
        uint64_t h = c.first * 0x9e3779b97f4a7c15ull ^ (uint64_t(c.second) * 0xc2b2ae3d27d4eb4full);
        return size_t(h ^ (h >> 29));
    }
};
static inline uint64_t table_key(int depth, uint64_t code) {
    return (uint64_t(uint32_t(depth)) << 60) | (code & 0x0fffffffffffffffull);
}
static void balance_cubes(const Cube* in, int64_t n, float r_root, std::vector<Cube>& out) {
    std::unordered_map<uint64_t, std::pair<float, uint32_t>> table;  // key -> (r_c sum, count)
    std::vector<uint64_t> order;                                       // keys in first-seen order
    table.reserve(size_t(n) * 2 + 16);
    for (int64_t i = 0; i < n; ++i) {
        auto r = table.emplace(table_key(in[i].depth, key_of(in[i].hi, in[i].lo)), std::make_pair(0.0f, 0u));
        if (r.second) order.push_back(r.first->first);
        r.first->second.first += in[i].r_c;
        r.first->second.second += 1;
    }
    for (size_t j = 0; j < order.size(); ++j) {
        auto& e = table[order[j]];
        e.first /= static_cast<float>(e.second);
    }
    std::unordered_set<std::pair<uint64_t, int>, CellHash> present;
    present.reserve(size_t(n) * 2 + 16);
    std::vector<std::pair<int, uint64_t>> fifo;
    fifo.reserve(size_t(n) + 16);
    for (int64_t i = 0; i < n; ++i) {
        const uint64_t c = key_of(in[i].hi, in[i].lo);
        present.insert({c, in[i].depth});
        fifo.push_back({in[i].depth, c});
    }
    for (size_t h = 0; h < fifo.size(); ++h) {
        const int d = fifo[h].first;
        const uint64_t c = fifo[h].second;
        if (d < 2) continue;
        for (int f = 0; f < 6; ++f) {
            const uint64_t nb = face_key(c, f, d);
            if (is_none(nb)) continue;
            if (present.count({nb, d})) continue;
            const uint64_t par = ancestor(nb, d - 1);
            if (present.count({par, d - 1})) continue;
            bool coarser = false;
            for (int d2 = d - 2; d2 >= 0 && !coarser; --d2) coarser = present.count({ancestor(nb, d2), d2}) != 0;
            if (!coarser) continue;
            auto r = table.emplace(table_key(d - 1, par),
                                   std::make_pair(r_root / static_cast<float>(1u << (d - 1)), 1u));
            if (!r.second) continue;
            order.push_back(r.first->first);
            present.insert({par, d - 1});
            fifo.push_back({d - 1, par});
        }
    }
    out.resize(order.size());
    for (size_t j = 0; j < order.size(); ++j) {
        const uint64_t k = order[j];
        const uint64_t code = k & 0x0fffffffffffffffull;
        out[j] = Cube{uint32_t(code >> 32), uint32_t(code), table[k].first, int32_t(k >> 60)};
    }
    // The reference sorts by code only, leaving equal codes in hash-table
    // order; here they are ordered by depth.
    std::stable_sort(out.begin(), out.end(), [](const Cube& a, const Cube& b) {
        const uint64_t ka = key_of(a.hi, a.lo), kb = key_of(b.hi, b.lo);
        return ka != kb ? ka < kb : a.depth < b.depth;
    });
}
}  // namespace orc

extern "C" int64_t orc_merge_cubes(const orc::Cube* const* in, const int64_t* n, int k, orc::Cube* out, int64_t cap) {
    std::vector<orc::Cube> cs;
    orc::merge_cubes(in, n, k, cs);
    if (out && cap >= int64_t(cs.size())) std::memcpy(out, cs.data(), cs.size() * sizeof(orc::Cube));
    return int64_t(cs.size());
}

extern "C" int64_t orc_balance_cubes(const orc::Cube* in, int64_t n, float r_root, orc::Cube* out, int64_t cap) {
    std::vector<orc::Cube> cs;
    orc::balance_cubes(in, n, r_root, cs);
    if (out && cap >= int64_t(cs.size())) std::memcpy(out, cs.data(), cs.size() * sizeof(orc::Cube));
    return int64_t(cs.size());
}

extern "C" {
// In-memory neighbour table of every cube (neighbor_idx_ctf over the code map
// code -> largest index, tgv.cpp:97-109, 367-370): nb[6 i + f] = the index of
// cube i's face-f neighbour, else -1 (faces +x, -x, +y, -y, +z, -z).
void orc_neighbour_table(const orc::Cube* cubes, int64_t n, int32_t* nb) {
    std::unordered_map<uint64_t, uint32_t> cmap;
    cmap.reserve(size_t(n) * 2);
    std::vector<uint64_t> keys(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        keys[i] = orc::key_of(cubes[i].hi, cubes[i].lo);
        cmap[keys[i]] = uint32_t(i);
    }
    auto find = [&](uint64_t k) -> int32_t {
        auto it = cmap.find(k);
        return it == cmap.end() ? -1 : int32_t(it->second);
    };
    for (int64_t i = 0; i < n; ++i) {
        const int d = cubes[i].depth;
        for (int f = 0; f < 6; ++f) {
            int32_t r = -1;
            const uint64_t nk = orc::face_key(keys[i], f, d);
            if (!orc::is_none(nk)) {
                r = find(nk);
                if (r < 0 && d > 0) r = find(orc::parent_key(nk, d));
            }
            nb[size_t(i) * 6 + f] = r;
        }
    }
}
}
