// Stage 6 on sm_103a: coarse-to-fine primal-dual TGV with a histogram data term
// over a Morton-ordered octree (reference src/tgv.cpp).
//
// Device layout ("level-major"): cubes are stably bucketed by depth, so level
// L's active cubes occupy one contiguous position range and keep their
// (Morton) index order inside it.  Per position, structure-of-arrays:
//   uv   float4 {u, vx, vy, vz}        bar  float4 {u_bar, vx_bar, vy_bar, vz_bar}
//   P4   float4 {p0, p1, p2, q0}       Q4   float4 {q1, q2, q3, q4}     Q1 float {q5}
//   dat  float2 {median, tau*tot or -1 for an empty histogram}
//   nb   int32 [6][npos] neighbour positions (-1 none, BORDER flag), par int32
// = 100 B of state per cube, every per-cube record a single vector access.
//
// Kernels (one thread per active cube, block-contiguous chunks):
//   K3 setup: k_prep / k_bucket_* (stable counting sort) / k_hash_insert /
//      k_neighbours<MODE> -- replaces CodeMap + NeighbourTable + the streaming
//      path's on-disk lookups (tgv.cpp:97-133, 367-370, 651-688, 955-1021)
//   K4 k_init -- median / data term once per solve instead of per iteration
//      (prox_data, tgv.cpp:75-94)
//   K5 k_parent_init / k_stream_snapshot -- level start (tgv.cpp:391-409,
//      484-487, 878-937, 1029-1057)
//   K6 k_dual<MODE>   -- p and q sweeps (tgv.cpp:158-189): 100 B/cube
//   K7 k_primal<MODE> -- u, v and extrapolation sweeps (tgv.cpp:191-230): 104 B/cube
//      Both optionally accumulate the FP64 residual sums of the stopping test.
// The reference's five Jacobi sweeps are exact as two kernels: q reads only
// the bars, which the p sweep does not write; u and v read only p/q, which
// they do not write, and the extrapolation is per cube.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace tgvg {

static constexpr int NBUCKET = 23;  // depths 0..21, 22 = never active
static constexpr int SORT_BLOCK = 1024;
static constexpr int ITER_BLOCK = 256;

enum { M_INMEM = 0, M_OC = 1, M_STREAM = 2 };

// ---------------------------------------------------------------- setup ---

// keys, depth, flags: [0] unsorted, [1] bad depth, [2] min depth, [3] max depth
__global__ void k_prep(int n, const uint4* __restrict__ cubes, unsigned long long* __restrict__ keys,
                       int* __restrict__ depth, int* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool v = i < n;
    int lo = 21, hi = 0;
    if (v) {
        const uint4 c = cubes[i];
        const unsigned long long k = ((unsigned long long)c.x << 32) | c.y;
        keys[i] = k;
        const int d = (int)c.w;
        depth[i] = d;
        if (d < 0 || d > 21) atomicOr(flags + 1, 1);
        if (i > 0) {
            const uint4 pc = cubes[i - 1];
            const unsigned long long pk = ((unsigned long long)pc.x << 32) | pc.y;
            if (pk > k) atomicOr(flags + 0, 1);
        }
        lo = hi = d;
    }
    // warp-reduced depth range (block size is a multiple of 32, all lanes present)
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0 && (blockIdx.x * blockDim.x + threadIdx.x) < n) {
        atomicMin(flags + 2, lo);
        atomicMax(flags + 3, hi);
    }
}

// leaf_of[i] = caller index of the leaf holding cube i, or -1.  Leaves arrive
// sorted by first index (non-overlapping) with their caller indices.
__global__ void k_leaf_of(int n, int nleaf, const int* __restrict__ s_first,
                          const int* __restrict__ s_last, const int* __restrict__ s_id,
                          int* __restrict__ leaf_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lo = 0, hi = nleaf;  // first s with s_first[s] > i
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s_first[mid] <= i) lo = mid + 1; else hi = mid;
    }
    const int s = lo - 1;
    leaf_of[i] = (s >= 0 && i <= s_last[s]) ? s_id[s] : -1;
}

__device__ __forceinline__ int bucket_of(int mode, int d, int leaf) {
    return (d < 0 || d > 21 || (mode == M_STREAM && leaf < 0)) ? 22 : d;
}

__global__ void k_bucket_count(int n, int mode, const int* __restrict__ depth,
                               const int* __restrict__ leaf_of, int* __restrict__ counts, int nblk) {
    __shared__ int sc[NBUCKET];
    if (threadIdx.x < NBUCKET) sc[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * SORT_BLOCK + threadIdx.x;
    if (i < n) atomicAdd(&sc[bucket_of(mode, depth[i], leaf_of[i])], 1);
    __syncthreads();
    if (threadIdx.x < NBUCKET) counts[threadIdx.x * nblk + blockIdx.x] = sc[threadIdx.x];
}

// In-place exclusive scan of counts[NBUCKET * nblk] (bucket-major), one block.
// bstart[b] = first position of bucket b, bstart[NBUCKET] = n.
__global__ void k_bucket_scan(int total, int* __restrict__ counts, int nblk, int* __restrict__ bstart) {
    __shared__ int part[SORT_BLOCK];
    const int t = threadIdx.x;
    const int per = (total + SORT_BLOCK - 1) / SORT_BLOCK;
    const int a = min(total, t * per), b = min(total, a + per);
    int s = 0;
    for (int k = a; k < b; ++k) s += counts[k];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < SORT_BLOCK; off <<= 1) {
        int v = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;  // exclusive
    for (int k = a; k < b; ++k) { const int c = counts[k]; counts[k] = run; run += c; }
    __syncthreads();
    if (t < NBUCKET) bstart[t] = counts[t * nblk];
    if (t == 0) bstart[NBUCKET] = part[SORT_BLOCK - 1];
}

// Stable scatter: rank inside the block = earlier warps' count + lanes below.
__global__ void k_bucket_scatter(int n, int mode, const int* __restrict__ depth,
                                 const int* __restrict__ leaf_of, const int* __restrict__ offs, int nblk,
                                 int* __restrict__ perm, int* __restrict__ inv) {
    __shared__ int wcnt[SORT_BLOCK / 32][NBUCKET];
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    const int i = blockIdx.x * SORT_BLOCK + t;
    const int b = i < n ? bucket_of(mode, depth[i], leaf_of[i]) : NBUCKET;
    for (int k = lane; k < NBUCKET; k += 32) wcnt[w][k] = 0;
    __syncwarp();
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (b < NBUCKET && rank == 0) wcnt[w][b] = __popc(peers);
    __syncthreads();
    if (t < NBUCKET) {
        int run = 0;
        for (int ww = 0; ww < SORT_BLOCK / 32; ++ww) { const int c = wcnt[ww][t]; wcnt[ww][t] = run; run += c; }
    }
    __syncthreads();
    if (i < n) {
        const int pos = offs[b * nblk + blockIdx.x] + wcnt[w][b] + rank;
        perm[pos] = i;
        inv[i] = pos;
    }
}

__global__ void k_hash_insert(int n, const unsigned long long* __restrict__ keys, HashView h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) hash_insert(h, keys[i], i);
}

// Resolve one neighbour code into a position (or -1), with the semantics of
// the selected entry point.  INMEM/OC: largest index with the code, falling
// back to the code of its parent (neighbor_idx_ctf, tgv.cpp:97-109); OC flags
// neighbours of other leaves.  STREAM: the leaf's own largest index with the
// code, else the cube file's bisection hit as a frozen border cube, else the
// same two steps for the parent code (tgv.cpp:960-1021).
template <int MODE>
__device__ __forceinline__ int resolve(uint64_t nk, int d, int lid, int f0, int l0, const HashView& h,
                                       int n, const int* __restrict__ inv, const int* __restrict__ leaf_of) {
    if (nk == NO_KEY) return -1;
    for (int step = 0; step < 2; ++step) {
        if (step == 1) {
            if (d <= 0) return -1;
            nk = parent_key(nk, d);
        }
        const int s = hash_find(h, nk);
        if (s < 0) continue;
        const int r0 = h.rmin[s], r1 = h.rmax[s];
        if (MODE == M_STREAM) {
            const int hi = min(r1, l0);
            if (max(r0, f0) <= hi) return inv[hi];
            const int g = bisect_hit(n, r0, r1);
            return g < 0 ? -1 : (inv[g] | BORDER);
        } else {
            int pos = inv[r1];
            if (MODE == M_OC && leaf_of[r1] != lid) pos |= BORDER;
            return pos;
        }
    }
    return -1;
}

template <int MODE>
__global__ void k_neighbours(int n_act, int n, const int* __restrict__ perm, const int* __restrict__ inv,
                             const unsigned long long* __restrict__ keys, const int* __restrict__ depth,
                             const int* __restrict__ leaf_of, const int* __restrict__ leaf_first,
                             const int* __restrict__ leaf_last, HashView h, int npos,
                             int* __restrict__ nb, int* __restrict__ par) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_act) return;
    const int i = perm[p];
    const uint64_t key = keys[i];
    const int d = depth[i];
    const int lid = leaf_of[i];
    int f0 = 0, l0 = n - 1;
    if (MODE == M_STREAM && lid >= 0) { f0 = leaf_first[lid]; l0 = leaf_last[lid]; }
#pragma unroll
    for (int f = 0; f < 6; ++f)
        nb[f * npos + p] = resolve<MODE>(face_key(key, f, d), d, lid, f0, l0, h, n, inv, leaf_of);
    int pp = -1;
    if (d > 0) {
        const int s = hash_find(h, parent_key(key, d));
        if (s >= 0) {
            const int j = (MODE == M_STREAM) ? bisect_hit(n, h.rmin[s], h.rmax[s]) : h.rmax[s];
            pp = j >= 0 ? inv[j] : -1;
        }
    }
    par[p] = pp;
}

// Data term and initial state (tgv.cpp:372-373, 384-385; prox_data 75-94).
template <int NB>
__global__ void k_init(int npos, const int* __restrict__ perm, const uint32_t* __restrict__ hists, int init,
                       const float* __restrict__ u_init, const int* __restrict__ leaf_of,
                       float4* __restrict__ uv, float4* __restrict__ bar, float4* __restrict__ P4,
                       float4* __restrict__ Q4, float* __restrict__ Q1, float2* __restrict__ dat,
                       int* __restrict__ lid) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npos) return;
    const int i = perm[p];
    const uint32_t* row = hists + (size_t)i * NB;
    uint32_t b[NB];
    uint32_t tot = 0;
#pragma unroll
    for (int k = 0; k < NB; ++k) { b[k] = row[k]; tot += b[k]; }
    float med = 0.0f, shrink = -1.0f;
    if (tot != 0) {
        uint32_t cum = 0;
        int km = NB;
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            cum += b[k];
            if (km == NB && cum * 2u >= tot) km = k;
        }
        med = km < NB ? fadd(-1.0f, fdiv(fadd((float)km, 0.5f), NB / 2.0f)) : 1.0f;
        shrink = fmul(0.25f, (float)tot);
    }
    // TGVG_INIT_STATE: until its level starts a cube holds the reference's
    // initial state; the caller's state replaces it at the level start.
    float u0 = (init == TGVG_INIT_MEDIAN || init == TGVG_INIT_STATE) ? med
             : (init == TGVG_INIT_ZERO ? 0.0f : u_init[i]);
    const float4 s = make_float4(u0, 0.f, 0.f, 0.f);
    uv[p] = s;
    bar[p] = s;
    P4[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    Q4[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    Q1[p] = 0.f;
    dat[p] = make_float2(med, shrink);
    lid[p] = leaf_of[i];
}

// Per-(leaf, level) position ranges inside each level's segment, whose
// positions are sorted by cube index: ranges[(leaf*NBUCKET + b)*2 + {0,1}].
__global__ void k_leaf_ranges(int nleaf, const int* __restrict__ leaf_first, const int* __restrict__ leaf_last,
                              const int* __restrict__ bstart, const int* __restrict__ perm,
                              int* __restrict__ ranges) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nleaf * 22) return;
    const int leaf = t / 22, b = t % 22;
    const int s = bstart[b], e = bstart[b + 1];
    const int f0 = leaf_first[leaf], l0 = leaf_last[leaf];
    int lo = s, hi = e;
    while (lo < hi) { const int m = (lo + hi) >> 1; if (perm[m] < f0) lo = m + 1; else hi = m; }
    const int a = lo;
    hi = e;
    while (lo < hi) { const int m = (lo + hi) >> 1; if (perm[m] <= l0) lo = m + 1; else hi = m; }
    ranges[(leaf * NBUCKET + b) * 2 + 0] = (l0 >= f0) ? a : s;
    ranges[(leaf * NBUCKET + b) * 2 + 1] = (l0 >= f0) ? lo : s;
}

// ------------------------------------------------------------- per level ---

__global__ void k_parent_init(int o, int n, const int* __restrict__ par, int keep_u, float4* __restrict__ uv,
                              float4* __restrict__ bar, float4* __restrict__ P4, float4* __restrict__ Q4,
                              float* __restrict__ Q1) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int p = o + t;
    const int j = par[p];
    float4 s = uv[p];
    // A parent at this same level is a cube whose own parent lookup returns
    // itself, so it never changes here and can be read concurrently.
    if (j >= 0 && j != p) {
        const float4 q = uv[j];
        s = keep_u ? make_float4(s.x, q.y, q.z, q.w) : q;  // keep_u: warm start keeps its own u
        uv[p] = s;
    }
    bar[p] = s;
    P4[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    Q4[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    Q1[p] = 0.f;
}

// Level start of a whole-state warm start (TGVG_INIT_STATE, no counterpart in
// the reference): every cube of the level takes the caller's u, v, p and q
// (TGVCube record of its caller index) in place of the parent copy and the
// zeroing of p and q; its bars restart from u and v.
__global__ void k_level_state(int o, int n, const int* __restrict__ perm, const float* __restrict__ st,
                              float4* __restrict__ uv, float4* __restrict__ bar, float4* __restrict__ P4,
                              float4* __restrict__ Q4, float* __restrict__ Q1) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int p = o + t;
    const float* r = st + (size_t)perm[p] * 13;  // 52-byte records: scalar loads
    const float4 s = make_float4(r[0], r[1], r[2], r[3]);
    uv[p] = s;
    bar[p] = s;
    P4[p] = make_float4(r[4], r[5], r[6], r[7]);
    Q4[p] = make_float4(r[8], r[9], r[10], r[11]);
    Q1[p] = r[12];
}

// Streaming level start: every cube's bars restart from its state u/v, and the
// frozen copy for border reads is taken (build_bars_frozen, tgv.cpp:606-635).
__global__ void k_stream_snapshot(int npos, const float4* __restrict__ uv, float4* __restrict__ bar,
                                  float4* __restrict__ snap) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npos) return;
    const float4 s = uv[p];
    bar[p] = s;
    snap[p] = s;
}

__global__ void k_copy4(int npos, const float4* __restrict__ src, float4* __restrict__ dst) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < npos) dst[p] = src[p];
}

struct IterArgs {
    int o, n, chunk, npos;
    const int* nb;
    float4* uv;
    float4* bar;
    float4* P4;
    float4* Q4;
    float* Q1;
    const float2* dat;
    const float4* snap;
    const int* lid;     // STREAM: stop/residual slot per position
    double* acc;        // [slot][4]: d_primal, d_dual, n_primal, n_dual
    int* done;          // [slot]
    int slot0;          // INMEM/OC: the slot of this launch
    float alpha0, alpha1;
    // persistent (one launch per level) schedule only
    int iters, check_every, nslot, it0, iters_total;
    float tol;
    unsigned* bar_count;  // grid barrier state
    unsigned* bar_gen;
    int* err;             // set when a bounded wait gives up
    int* iters_run;
    double* resid;
    int pf;               // per-launch schedules: L2 prefetch of the warp's next group (0 = off)
    int swap;             // per-launch schedules: dual sweep in reverse order, primal forward
    int band;             // per-launch schedules: warps stride over the whole unit (grid-stride band)
    int lend;             // end of the level's positions; cubes at lend and beyond are deeper
    int gcap;             // single-block shared-memory schedule: room for staged out-of-unit values
    // per-launch sweep schedules (in-memory and streaming semantics): the unit's
    // -x/-y/-z neighbour table [3][n] with coarser neighbours replaced by
    // -2 - entry of gh, the compact copies of their gathered p/q values (or null)
    const int* pnb;
    const float4* gh;
    // the same for the dual sweep's +x/+y/+z faces on levels with many deeper
    // neighbours: neighbours on other levels redirected to dgh, copies of their
    // bars (or null)
    const int* dnb;
    const float4* dgh;
};

// Error-free addition (Knuth's TwoSum, TAOCP vol. 2, 4.2.2): hi + x = s + e
// exactly in round-to-nearest.  hi gets s and lo collects e, so (hi, lo) carries
// a sum of FP32 terms to about 48 bits with FP32 arithmetic only.
__device__ __forceinline__ void two_sum(float& hi, float& lo, float x) {
    const float s = fadd(hi, x);
    const float bp = fsub(s, hi);
    const float e = fadd(fsub(hi, fsub(s, bp)), fsub(x, bp));
    hi = s;
    lo = fadd(lo, e);
}

// Accumulate two sums of per-cube FP32 terms over a warp's cubes of one slot,
// and add them to acc[slot*4+k0..] in FP64 with one atomic per warp per slot
// run (positions are sorted by leaf).  Within the warp the sums are two-term
// floats, so the per-cube path has no FP64 arithmetic (GB300's FP64 rate is a
// small fraction of its FP32 rate); only lane 0 converts to FP64, for the
// atomic.
struct WarpAcc {
    float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f;
    int cur = -1;
    __device__ __forceinline__ void flush(double* acc, int k0, int lane) {
        float ah = xh, al = xl, bh = yh, bl = yl;
        for (int o = 16; o > 0; o >>= 1) {
            const float oah = __shfl_xor_sync(0xffffffffu, ah, o), oal = __shfl_xor_sync(0xffffffffu, al, o);
            const float obh = __shfl_xor_sync(0xffffffffu, bh, o), obl = __shfl_xor_sync(0xffffffffu, bl, o);
            two_sum(ah, al, oah);
            al = fadd(al, oal);
            two_sum(bh, bl, obh);
            bl = fadd(bl, obl);
        }
        if (lane == 0 && cur >= 0) {
            atomicAdd(acc + cur * 4 + k0, (double)ah + (double)al);
            atomicAdd(acc + cur * 4 + k0 + 2, (double)bh + (double)bl);
        }
        xh = xl = yh = yl = 0.f;
    }
    // slot: this lane's slot (-1 if the lane has no cube); whole warp calls.
    __device__ __forceinline__ void add(int slot, float dx, float dy, double* acc, int k0, int lane) {
        const int s0 = __shfl_sync(0xffffffffu, slot, __ffs(__ballot_sync(0xffffffffu, slot >= 0)) - 1);
        const bool uniform = __all_sync(0xffffffffu, slot < 0 || slot == s0);
        if (uniform) {
            if (s0 != cur) { flush(acc, k0, lane); cur = s0; }
            two_sum(xh, xl, dx);
            two_sum(yh, yl, dy);
        } else if (slot >= 0) {
            atomicAdd(acc + slot * 4 + k0, (double)dx);
            atomicAdd(acc + slot * 4 + k0 + 2, (double)dy);
        }
    }
};

__device__ __forceinline__ void clip3(float& a, float& b, float& c, float r) {
    const float n2 = fadd(fadd(fmul(a, a), fmul(b, b)), fmul(c, c));
    if (n2 > fmul(r, r)) {
        const float s = fdiv(r, fsqrt(n2));
        a = fmul(a, s); b = fmul(b, s); c = fmul(c, s);
    }
}
__device__ __forceinline__ void clip6(float* q, float r) {
    float n2 = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; ++k) n2 = fadd(n2, fmul(q[k], q[k]));
    if (n2 > fmul(r, r)) {
        const float s = fdiv(r, fsqrt(n2));
#pragma unroll
        for (int k = 0; k < 6; ++k) q[k] = fmul(q[k], s);
    }
}

// Loads of state that other blocks rewrite while a persistent kernel runs go
// to L2 (.cg) so no stale L1 line is ever read; the per-launch kernels use
// ordinary loads.
// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start while the previous kernel of the stream finishes;
// pdl_wait() blocks until that kernel has completed and its writes are
// visible (a no-op for an ordinary launch), and pdl_release() lets the next
// such kernel start launching its blocks as this one's blocks retire.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <bool CG> __device__ __forceinline__ float4 ld4(const float4* p) { return CG ? __ldcg(p) : *p; }
// p/q lines marked evict-last in L2: the dual sweep's stores and the primal
// sweep's loads of P4/Q4/Q1.  A primal gather of a -x/-y/-z neighbour then
// more often finds the line the dual sweep wrote still in L2, while the
// once-read streams (u/v, data term, neighbour indices) go first.  Measured on
// the largest three64 levels: k_dual 52.2-53.3 -> 48.9 us per launch, the
// solve 243-245 -> 235 ms, results unchanged.
__device__ __forceinline__ uint64_t pol_last() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float4 ld4L(const float4* p, uint64_t pol) {
    float4 r;
    asm volatile("ld.global.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p), "l"(pol));
    return r;
}
__device__ __forceinline__ float ld1L(const float* p, uint64_t pol) {
    float r;
    asm volatile("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(r) : "l"(p), "l"(pol));
    return r;
}
__device__ __forceinline__ void st4L(float4* p, float4 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1,%2,%3,%4}, %5;"
                 :: "l"(p), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "l"(pol) : "memory");
}
__device__ __forceinline__ void st1L(float* p, float v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" :: "l"(p), "f"(v), "l"(pol) : "memory");
}
template <bool CG> __device__ __forceinline__ float ld1(const float* p) { return CG ? __ldcg(p) : *p; }

template <int MODE, bool CG>
__device__ __forceinline__ float4 fetch_bar(int j, const float4& own, const float4* __restrict__ bar,
                                            const float4* __restrict__ snap, const float4* __restrict__ gh) {
    if (j < 0) return (!CG && j <= -2) ? __ldg(gh + (-2 - j)) : own;
    if (MODE != M_INMEM && (j & BORDER)) return snap[j & POS_MASK];
    return ld4<CG>(bar + j);
}

// One cube's terms of the stopping test: the squared change and the squared
// new value of its K state components, each summed in FP32 with explicit
// rounding in component order (the oracle sums them the same way); the sums
// over cubes are two-term floats within a warp and FP64 across warps (WarpAcc).
// GB300's FP64 rate is a small fraction of its FP32 rate: with the per-cube
// terms in FP64 a checking iteration cost about five times a plain one on the
// largest levels.
template <int K>
__device__ __forceinline__ void res_terms(const float* w, const float* o, float& dd, float& nd) {
    float t = fsub(w[0], o[0]);
    float ds = fmul(t, t), ns = fmul(w[0], w[0]);
#pragma unroll
    for (int k = 1; k < K; ++k) {
        t = fsub(w[k], o[k]);
        ds = fadd(ds, fmul(t, t));
        ns = fadd(ns, fmul(w[k], w[k]));
    }
    dd = ds;
    nd = ns;
}

// One cube's dual ascent: p on |grad u - v| (radius alpha1) and q on |e(v)|
// (radius alpha0), in the reference's operation order (tgv.cpp:158-189).
// Split into the loads (dual_load) and the arithmetic and stores (dual_finish)
// so that a warp can issue the loads of two cubes before either's stores.
// Returns the residual contributions through dd / nd when RES.
struct DualLd { float4 b, B0, B2, B4, P, Q; float q5; };

template <int MODE, bool CG>
__device__ __forceinline__ void dual_load(const IterArgs& a, int p, DualLd& L) {
    L.b = ld4<CG>(a.bar + p);
    const bool g = !CG && a.dnb;
    const int* jb = g ? a.dnb + (p - a.o) : a.nb + p;
    const int js = g ? a.n : 2 * a.npos;
    const int j0 = __ldg(jb), j2 = __ldg(jb + js), j4 = __ldg(jb + 2 * js);
    L.P = ld4<CG>(a.P4 + p);
    L.Q = ld4<CG>(a.Q4 + p);
    L.q5 = ld1<CG>(a.Q1 + p);
    L.B0 = fetch_bar<MODE, CG>(j0, L.b, a.bar, a.snap, a.dgh);
    L.B2 = fetch_bar<MODE, CG>(j2, L.b, a.bar, a.snap, a.dgh);
    L.B4 = fetch_bar<MODE, CG>(j4, L.b, a.bar, a.snap, a.dgh);
}

template <bool RES>
__device__ __forceinline__ void dual_finish(const IterArgs& a, int p, const DualLd& L, float& dd, float& nd) {
    const float4 b = L.b, B0 = L.B0, B2 = L.B2, B4 = L.B4, P = L.P, Q = L.Q;
    const float q5o = L.q5;
    float p0 = fadd(P.x, fmul(0.25f, fsub(fsub(B0.x, b.x), b.y)));
    float p1 = fadd(P.y, fmul(0.25f, fsub(fsub(B2.x, b.x), b.z)));
    float p2 = fadd(P.z, fmul(0.25f, fsub(fsub(B4.x, b.x), b.w)));
    clip3(p0, p1, p2, a.alpha1);
    const float e0 = fsub(B0.y, b.y);
    const float e1 = fsub(B2.z, b.z);
    const float e2 = fsub(B4.w, b.w);
    const float e3 = fmul(0.5f, fsub(fadd(fsub(B2.y, b.y), B0.z), b.z));
    const float e4 = fmul(0.5f, fsub(fadd(fsub(B4.y, b.y), B0.w), b.w));
    const float e5 = fmul(0.5f, fsub(fadd(fsub(B4.z, b.z), B2.w), b.w));
    float q[6] = {fadd(P.w, fmul(0.25f, e0)), fadd(Q.x, fmul(0.25f, e1)), fadd(Q.y, fmul(0.25f, e2)),
                  fadd(Q.z, fmul(0.25f, e3)), fadd(Q.w, fmul(0.25f, e4)), fadd(q5o, fmul(0.25f, e5))};
    clip6(q, a.alpha0);
    const uint64_t pol = pol_last();
    st4L(a.P4 + p, make_float4(p0, p1, p2, q[0]), pol);
    st4L(a.Q4 + p, make_float4(q[1], q[2], q[3], q[4]), pol);
    st1L(a.Q1 + p, q[5], pol);
    if (RES) {
        const float o[9] = {P.x, P.y, P.z, P.w, Q.x, Q.y, Q.z, Q.w, q5o};
        const float w[9] = {p0, p1, p2, q[0], q[1], q[2], q[3], q[4], q[5]};
        res_terms<9>(w, o, dd, nd);
    }
}

template <int MODE, bool RES, bool CG>
__device__ __forceinline__ void dual_cube(const IterArgs& a, int p, float& dd, float& nd) {
    DualLd L;
    dual_load<MODE, CG>(a, p, L);
    dual_finish<RES>(a, p, L, dd, nd);
}

// One cube's primal descent: u by the prox of tot*|u - median|, v, then the
// extrapolated bars (tgv.cpp:191-230); loads (primal_load) and arithmetic and
// stores (primal_finish) as for the dual.  Neighbours across faces 1/3/5 give
// their p/q components, or zero when missing (streaming: also for border cubes).
struct PrimalLd {
    float4 U, P, Q;
    float q5;
    float2 D;
    int j1, j3, j5;
    float gp10, gq10, gq13, gq14, gp31, gq31, gq33, gq35, gp52, gq52, gq54, gq55;
};

// The cube's own records and neighbour indices ...
template <int MODE, bool CG>
__device__ __forceinline__ void primal_load_own(const IterArgs& a, int p, PrimalLd& L) {
    L.U = ld4<CG>(a.uv + p);
    const uint64_t pol = pol_last();
    L.P = CG ? ld4<CG>(a.P4 + p) : ld4L(a.P4 + p, pol);
    L.Q = CG ? ld4<CG>(a.Q4 + p) : ld4L(a.Q4 + p, pol);
    L.q5 = CG ? ld1<CG>(a.Q1 + p) : ld1L(a.Q1 + p, pol);
    L.D = __ldg(a.dat + p);
    const bool g = !CG && a.pnb;
    const int* jb = g ? a.pnb + (p - a.o) : a.nb + a.npos + p;
    const int js = g ? a.n : 2 * a.npos;
    L.j1 = __ldg(jb);
    L.j3 = __ldg(jb + js);
    L.j5 = __ldg(jb + 2 * js);
}

// ... and the p/q of its -x/-y/-z neighbours.  A neighbour found by code can be
// a deeper cube (an octant-0 descendant shares the code, tgv.cpp:97-109,369-370).
// Levels run coarse to fine, so a deeper cube's p/q still hold their initial
// zeros while this level runs: such a neighbour reads as 0 without a load.
template <int MODE, bool CG>
__device__ __forceinline__ void primal_load_gather(const IterArgs& a, int p, PrimalLd& L) {
    const int j1 = L.j1, j3 = L.j3, j5 = L.j5;
    L.gp10 = L.gq10 = L.gq13 = L.gq14 = 0.f;
    L.gp31 = L.gq31 = L.gq33 = L.gq35 = 0.f;
    L.gp52 = L.gq52 = L.gq54 = L.gq55 = 0.f;
    if (j1 >= 0 && !(MODE == M_STREAM && (j1 & BORDER)) && (j1 & POS_MASK) < a.lend) {
        const int j = j1 & POS_MASK;
        const uint64_t pol = pol_last();
        const float4 a4 = CG ? ld4<CG>(a.P4 + j) : ld4L(a.P4 + j, pol);
        const float4 b4 = CG ? ld4<CG>(a.Q4 + j) : ld4L(a.Q4 + j, pol);
        L.gp10 = a4.x; L.gq10 = a4.w; L.gq13 = b4.z; L.gq14 = b4.w;
    } else if (!CG && j1 <= -2) {
        const float4 g = __ldg(a.gh + (-2 - j1));
        L.gp10 = g.x; L.gq10 = g.y; L.gq13 = g.z; L.gq14 = g.w;
    }
    if (j3 >= 0 && !(MODE == M_STREAM && (j3 & BORDER)) && (j3 & POS_MASK) < a.lend) {
        const int j = j3 & POS_MASK;
        const uint64_t pol = pol_last();
        const float4 a4 = CG ? ld4<CG>(a.P4 + j) : ld4L(a.P4 + j, pol);
        const float4 b4 = CG ? ld4<CG>(a.Q4 + j) : ld4L(a.Q4 + j, pol);
        L.gp31 = a4.y; L.gq31 = b4.x; L.gq33 = b4.z; L.gq35 = (CG ? ld1<CG>(a.Q1 + j) : ld1L(a.Q1 + j, pol));
    } else if (!CG && j3 <= -2) {
        const float4 g = __ldg(a.gh + (-2 - j3));
        L.gp31 = g.x; L.gq31 = g.y; L.gq33 = g.z; L.gq35 = g.w;
    }
    if (j5 >= 0 && !(MODE == M_STREAM && (j5 & BORDER)) && (j5 & POS_MASK) < a.lend) {
        const int j = j5 & POS_MASK;
        const uint64_t pol = pol_last();
        const float4 a4 = CG ? ld4<CG>(a.P4 + j) : ld4L(a.P4 + j, pol);
        const float4 b4 = CG ? ld4<CG>(a.Q4 + j) : ld4L(a.Q4 + j, pol);
        L.gp52 = a4.z; L.gq52 = b4.y; L.gq54 = b4.w; L.gq55 = (CG ? ld1<CG>(a.Q1 + j) : ld1L(a.Q1 + j, pol));
    } else if (!CG && j5 <= -2) {
        const float4 g = __ldg(a.gh + (-2 - j5));
        L.gp52 = g.x; L.gq52 = g.y; L.gq54 = g.z; L.gq55 = g.w;
    }
}

template <int MODE, bool CG>
__device__ __forceinline__ void primal_load(const IterArgs& a, int p, PrimalLd& L) {
    primal_load_own<MODE, CG>(a, p, L);
    primal_load_gather<MODE, CG>(a, p, L);
}

template <bool RES>
__device__ __forceinline__ void primal_math(const PrimalLd& L, float4& uvn, float4& barn, float& dd, float& nd) {
    const float4 U = L.U, P = L.P, Q = L.Q;
    const float q5 = L.q5;
    const float2 D = L.D;
    const float p0 = P.x, p1 = P.y, p2 = P.z;
    const float q0 = P.w, q1 = Q.x, q2 = Q.y, q3 = Q.z, q4 = Q.w;
    const float div_p = fadd(fadd(fsub(p0, L.gp10), fsub(p1, L.gp31)), fsub(p2, L.gp52));
    const float z = fadd(U.x, fmul(0.25f, div_p));
    float un;
    if (D.y < 0.0f) {
        un = z;
    } else {
        const float diff = fsub(z, D.x);
        if (diff > D.y) un = fsub(z, D.y);
        else if (diff < -D.y) un = fadd(z, D.y);
        else un = D.x;
    }
    const float dqx = fadd(fadd(fsub(q0, L.gq10), fsub(q3, L.gq33)), fsub(q4, L.gq54));
    const float dqy = fadd(fadd(fsub(q3, L.gq13), fsub(q1, L.gq31)), fsub(q5, L.gq55));
    const float dqz = fadd(fadd(fsub(q4, L.gq14), fsub(q5, L.gq35)), fsub(q2, L.gq52));
    const float vxn = fadd(U.y, fmul(0.25f, fadd(p0, dqx)));
    const float vyn = fadd(U.z, fmul(0.25f, fadd(p1, dqy)));
    const float vzn = fadd(U.w, fmul(0.25f, fadd(p2, dqz)));
    barn = make_float4(fsub(fmul(2.0f, un), U.x), fsub(fmul(2.0f, vxn), U.y), fsub(fmul(2.0f, vyn), U.z),
                       fsub(fmul(2.0f, vzn), U.w));
    uvn = make_float4(un, vxn, vyn, vzn);
    if (RES) {
        const float o[4] = {U.x, U.y, U.z, U.w};
        const float w[4] = {un, vxn, vyn, vzn};
        res_terms<4>(w, o, dd, nd);
    }
}

template <bool RES>
__device__ __forceinline__ void primal_finish(const IterArgs& a, int p, const PrimalLd& L, float& dd, float& nd) {
    float4 uvn, barn;
    primal_math<RES>(L, uvn, barn, dd, nd);
    a.bar[p] = barn;
    a.uv[p] = uvn;
}

template <int MODE, bool RES, bool CG>
__device__ __forceinline__ void primal_cube(const IterArgs& a, int p, float& dd, float& nd) {
    PrimalLd L;
    primal_load<MODE, CG>(a, p, L);
    primal_finish<RES>(a, p, L, dd, nd);
}

// A block's share of one sweep over positions [beg, end): warps take 32-cube
// groups in order (or in reverse order with REV, so that a sweep starts where
// the previous one ended and finds its last writes still in L2).
// L2 prefetch of the contiguous per-position streams of the 32-cube group at
// position q0 (one 128-byte line per lane): the own-cube records a sweep reads,
// so that their DRAM latency overlaps the current group's work without holding
// registers.  The neighbour gathers are left to the caches.
template <bool DUAL>
__device__ __forceinline__ void prefetch_group(const IterArgs& a, int q0, int end, int lane) {
    // every line starts at a position below `end`, so each address is inside its array
    const void* line = nullptr;
    const int k4 = lane & 3;        // float4 streams: line k covers positions q0 + 8k ..
    const bool in4 = q0 + 8 * k4 < end;
    if (DUAL) {
        if (lane < 4) line = in4 ? a.bar + q0 + 8 * k4 : nullptr;
        else if (lane < 8) line = in4 ? a.P4 + q0 + 8 * k4 : nullptr;
        else if (lane < 12) line = in4 ? a.Q4 + q0 + 8 * k4 : nullptr;
        else if (lane == 12) line = a.Q1 + q0;
        else if (lane < 16)
            line = a.dnb ? a.dnb + (size_t)(lane - 13) * a.n + (q0 - a.o)
                         : a.nb + (size_t)(2 * (lane - 13)) * a.npos + q0;
    } else {
        if (lane < 4) line = in4 ? a.uv + q0 + 8 * k4 : nullptr;
        else if (lane < 8) line = in4 ? a.P4 + q0 + 8 * k4 : nullptr;
        else if (lane < 12) line = in4 ? a.Q4 + q0 + 8 * k4 : nullptr;
        else if (lane == 12) line = a.Q1 + q0;
        else if (lane < 15) line = q0 + 16 * (lane - 13) < end ? a.dat + q0 + 16 * (lane - 13) : nullptr;
        else if (lane < 18)
            line = a.pnb ? a.pnb + (size_t)(lane - 15) * a.n + (q0 - a.o)
                         : a.nb + (size_t)(2 * (lane - 15) + 1) * a.npos + q0;
    }
    if (line && q0 < end) asm volatile("prefetch.global.L2 [%0];" ::"l"(line));
}

// Warp w of the block takes groups w, w + nw, ... of [beg, end); in band mode
// (per-launch schedules with a.band) the range is the whole unit and the
// global warp g takes groups g, g + (all warps), ..., so that all warps work
// on one narrow band of positions that moves through the unit and a cube's
// neighbours are read while their lines are still in L2.
// With ILP = 2 a warp takes two of its groups per step and issues the loads
// of both cubes before either's arithmetic and stores (more loads in flight
// per warp at the same occupancy).
// chk = false (streaming semantics, per-launch schedules): no slot of the unit
// has met its tolerance, so no cube reads its slot's stopping flag.
template <int MODE, bool RES, bool STOP, bool CG, bool DUAL, bool REV, int ILP = 1>
__device__ __forceinline__ void sweep(const IterArgs& a, int beg, int end, WarpAcc& wa, bool chk = true) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int g0 = warp, gs = blockDim.x >> 5;
    if (!CG && a.band) {
        beg = a.o;
        end = a.o + a.n;
        g0 = blockIdx.x * gs + warp;
        gs *= gridDim.x;
    }
    const int ngroups = (end - beg + 31) >> 5;
    const bool rev = CG ? REV : (REV != (a.swap != 0));
    for (int gi = g0; gi < ngroups; gi += ILP * gs) {
        if (ILP == 1 && !CG && a.pf > 0 && gi + a.pf * gs < ngroups) {
            const int gn = rev ? (ngroups - 1 - (gi + a.pf * gs)) : gi + a.pf * gs;
            prefetch_group<DUAL>(a, beg + gn * 32, end, lane);
        }
        int pos[ILP], slot[ILP];
        bool work[ILP];
#pragma unroll
        for (int u = 0; u < ILP; ++u) {
            const int gu = gi + u * gs;
            const int g = rev ? (ngroups - 1 - gu) : gu;
            pos[u] = beg + g * 32 + lane;
            work[u] = gu < ngroups && pos[u] < end;
            slot[u] = -1;
            if (work[u] && (MODE != M_STREAM || RES || (STOP && chk)))
                slot[u] = (MODE == M_STREAM) ? __ldg(a.lid + pos[u]) : a.slot0;
            // The stopping flags change only between launches of the per-launch
            // schedules (k_check is its own launch), so they are read through L1
            // there; the one-launch schedules re-read them from L2.
            if (STOP && chk && work[u] && MODE == M_STREAM)
                work[u] = (CG ? __ldcg(a.done + slot[u]) : __ldg(a.done + slot[u])) == 0;
        }
        if (DUAL) {
            DualLd L[ILP];
#pragma unroll
            for (int u = 0; u < ILP; ++u)
                if (work[u]) dual_load<MODE, CG>(a, pos[u], L[u]);
#pragma unroll
            for (int u = 0; u < ILP; ++u) {
                float dd = 0.f, nd = 0.f;
                if (work[u]) dual_finish<RES>(a, pos[u], L[u], dd, nd);
                if (RES) wa.add(work[u] ? slot[u] : -1, dd, nd, a.acc, 1, lane);
            }
        } else {
            PrimalLd L[ILP];
#pragma unroll
            for (int u = 0; u < ILP; ++u)
                if (work[u]) primal_load<MODE, CG>(a, pos[u], L[u]);
#pragma unroll
            for (int u = 0; u < ILP; ++u) {
                float dd = 0.f, nd = 0.f;
                if (work[u]) primal_finish<RES>(a, pos[u], L[u], dd, nd);
                if (RES) wa.add(work[u] ? slot[u] : -1, dd, nd, a.acc, 0, lane);
            }
        }
    }
}

// K6 / K7 as one launch per sweep.  The primal sweep runs in reverse block
// order so it starts on the cubes whose p/q the dual sweep wrote last.
// MINB = 8 caps registers at 32 so that 64 warps fit per SM (more loads in
// flight); MINB = 6 (the default) allows about 42.
// Streaming semantics: the block first reads the unit's stopping flags (they
// change only between launches).  All set: nothing to do.  None set by a met
// tolerance (a slot with no cube on the level holds 2, not 1): no cube needs its
// own flag, which saves each cube a dependent read of its slot and flag before
// its loads.  Units with more slots than this bound keep the per-cube reads.
constexpr int STOP_SCAN_MAX = 4 * ITER_BLOCK;
template <int MODE, bool STOP>
__device__ __forceinline__ bool unit_flags(const IterArgs& a, bool& chk) {
    chk = true;
    if (!STOP) return true;
    if (MODE != M_STREAM) return a.done[a.slot0] == 0;
    if (a.nslot > STOP_SCAN_MAX) return true;
    int any = 0, all = 1;
    for (int s = threadIdx.x; s < a.nslot; s += blockDim.x) {
        const int d = __ldg(a.done + a.slot0 + s);
        any |= d == 1;
        all &= d != 0;
    }
    any = __syncthreads_or(any);
    all = __syncthreads_and(all);
    chk = any != 0;
    return all == 0;
}

template <int MODE, bool RES, bool STOP, int MINB, int ILP = 1>
__global__ void __launch_bounds__(ITER_BLOCK, MINB) k_dual(IterArgs a) {
    pdl_wait();
    pdl_release();
    bool chk;
    if (!unit_flags<MODE, STOP>(a, chk)) return;
    const int beg = a.o + blockIdx.x * a.chunk;
    const int end = min(a.o + a.n, beg + a.chunk);
    WarpAcc wa;
    sweep<MODE, RES, STOP, false, true, false, ILP>(a, beg, end, wa, chk);
    if (RES) wa.flush(a.acc, 1, threadIdx.x & 31);
}

template <int MODE, bool RES, bool STOP, int MINB, int ILP = 1>
__global__ void __launch_bounds__(ITER_BLOCK, MINB) k_primal(IterArgs a) {
    pdl_wait();
    pdl_release();
    bool chk;
    if (!unit_flags<MODE, STOP>(a, chk)) return;
    const int blk = gridDim.x - 1 - blockIdx.x;
    const int beg = a.o + blk * a.chunk;
    const int end = min(a.o + a.n, beg + a.chunk);
    WarpAcc wa;
    sweep<MODE, RES, STOP, false, false, true, ILP>(a, beg, end, wa, chk);
    if (RES) wa.flush(a.acc, 0, threadIdx.x & 31);
}

// Grid-wide barrier of a co-resident (cooperatively launched) grid, with a
// bounded wait: thread 0 of each block arrives on a counter; the last one
// bumps the generation; the others poll it at most ~2^25 times (>= 1 s), then
// set *err and give up, so a broken grid ends instead of hanging.
__device__ __forceinline__ bool grid_sync(unsigned* count, unsigned* gen, int* err) {
    __syncthreads();
    if (gridDim.x > 1 && threadIdx.x == 0) {
        volatile unsigned* vg = gen;
        const unsigned g = *vg;
        __threadfence();
        if (atomicAdd(count, 1u) == gridDim.x - 1) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            unsigned spins = 0;
            while (*vg == g) {
                if (++spins > (1u << 25)) { atomicOr(err, 1); break; }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)err == 0;
}

// Stopping slots a unit owns: every leaf's slot when all leaves of a level run
// together (streaming semantics), else its own one (the level in in-memory
// semantics, one leaf in OC semantics, where leaves run one after another and
// a leaf that has not run yet must not be judged on empty sums).
template <int MODE>
__host__ __device__ __forceinline__ int unit_slots(int nslot) { return MODE == M_STREAM ? nslot : 1; }

// Stopping test of the unit's slots, run by block 0 between barriers (k_check's logic).
template <int MODE>
__device__ __forceinline__ void check_slots(const IterArgs& a, int it) {
    for (int s = a.slot0 + threadIdx.x; s < a.slot0 + unit_slots<MODE>(a.nslot); s += blockDim.x) {
        if (a.done[s]) continue;
        double* q = a.acc + s * 4;
        const double num = sqrt(__ldcg(q + 0)) + sqrt(__ldcg(q + 1));
        const double den = sqrt(__ldcg(q + 2)) + sqrt(__ldcg(q + 3));
        const double rel = den > 0.0 ? num / den : 0.0;
        a.resid[s] = rel;
        if (rel <= (double)a.tol) { a.done[s] = 1; a.iters_run[s] = it + 1; }
        q[0] = q[1] = q[2] = q[3] = 0.0;
    }
}

// Every iteration of one level in ONE cooperative launch (levels small enough
// that launch latency, not bandwidth, dominates).  Blocks own contiguous
// chunks; two grid barriers per iteration order the dual and primal sweeps.
template <int MODE, bool STOP>
__global__ void __launch_bounds__(ITER_BLOCK) k_level_persistent(IterArgs a) {
    const int beg = a.o + blockIdx.x * a.chunk;
    const int end = min(a.o + a.n, beg + a.chunk);
    for (int i = 0; i < a.iters; ++i) {
        const int it = a.it0 + i;
        if (STOP && MODE != M_STREAM && *(volatile int*)(a.done + a.slot0)) break;
        const bool res = STOP && ((it + 1) % a.check_every == 0 || it + 1 == a.iters_total);
        WarpAcc wd, wp;
        if (res) sweep<MODE, true, STOP, true, true, false>(a, beg, end, wd);
        else sweep<MODE, false, STOP, true, true, false>(a, beg, end, wd);
        if (res) wd.flush(a.acc, 1, threadIdx.x & 31);
        if (!grid_sync(a.bar_count, a.bar_gen, a.err)) return;
        if (res) sweep<MODE, true, STOP, true, false, false>(a, beg, end, wp);
        else sweep<MODE, false, STOP, true, false, false>(a, beg, end, wp);
        if (res) {
            wp.flush(a.acc, 0, threadIdx.x & 31);
            if (!grid_sync(a.bar_count, a.bar_gen, a.err)) return;
            if (blockIdx.x == 0) check_slots<MODE>(a, it);
        }
        if (!grid_sync(a.bar_count, a.bar_gen, a.err)) return;
    }
}

// Cluster-wide barrier of all threads of a thread-block cluster, with release /
// acquire ordering at cluster scope (the hardware barrier: nothing to poll).
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Every iteration of one small level in ONE launch of a single thread-block
// cluster (8 or 16 CTAs of 1024 threads on one GPC): as k_level_persistent,
// with the hardware cluster barrier in place of the software grid barrier, so
// an iteration costs two sweeps of L2-resident state plus two barriers.
constexpr int CLUSTER_BLOCK = 1024;
template <int MODE, bool STOP>
__global__ void __launch_bounds__(CLUSTER_BLOCK) k_level_cluster(IterArgs a) {
    const int beg = a.o + blockIdx.x * a.chunk;
    const int end = min(a.o + a.n, beg + a.chunk);
    for (int i = 0; i < a.iters; ++i) {
        const int it = a.it0 + i;
        if (STOP && MODE != M_STREAM && *(volatile int*)(a.done + a.slot0)) break;
        const bool res = STOP && ((it + 1) % a.check_every == 0 || it + 1 == a.iters_total);
        WarpAcc wd, wp;
        if (res) sweep<MODE, true, STOP, true, true, false>(a, beg, end, wd);
        else sweep<MODE, false, STOP, true, true, false>(a, beg, end, wd);
        if (res) wd.flush(a.acc, 1, threadIdx.x & 31);
        cluster_barrier();
        if (res) sweep<MODE, true, STOP, true, false, false>(a, beg, end, wp);
        else sweep<MODE, false, STOP, true, false, false>(a, beg, end, wp);
        if (res) {
            wp.flush(a.acc, 0, threadIdx.x & 31);
            cluster_barrier();
            if (blockIdx.x == 0) check_slots<MODE>(a, it);
        }
        cluster_barrier();
    }
}

// Every iteration of one tiny level in ONE launch of ONE block of 1024 threads:
// as k_level_cluster with __syncthreads in place of the cluster barrier.  All
// readers and writers share one SM, so the sweeps read through L1 (plain loads:
// a block's global writes are visible to the block after __syncthreads), and
// a level of up to a couple of thousand cubes stays in L1 for all its
// iterations.
template <int MODE, bool STOP>
__global__ void __launch_bounds__(CLUSTER_BLOCK) k_level_cta(IterArgs a) {
    const int beg = a.o, end = a.o + a.n;
    for (int i = 0; i < a.iters; ++i) {
        const int it = a.it0 + i;
        if (STOP && MODE != M_STREAM && *(volatile int*)(a.done + a.slot0)) break;
        const bool res = STOP && ((it + 1) % a.check_every == 0 || it + 1 == a.iters_total);
        WarpAcc wd, wp;
        if (res) sweep<MODE, true, STOP, false, true, false>(a, beg, end, wd);
        else sweep<MODE, false, STOP, false, true, false>(a, beg, end, wd);
        if (res) wd.flush(a.acc, 1, threadIdx.x & 31);
        __syncthreads();
        if (res) sweep<MODE, true, STOP, false, false, false>(a, beg, end, wp);
        else sweep<MODE, false, STOP, false, false, false>(a, beg, end, wp);
        if (res) {
            wp.flush(a.acc, 0, threadIdx.x & 31);
            __syncthreads();
            check_slots<MODE>(a, it);
        }
        __syncthreads();
    }
}

// Primal energy of one level's state in FP64 (no counterpart in the reference;
// reported per level):  sum over the level's cubes of  tot |u - median|  +
// alpha1 |grad u - v|  +  alpha0 |e(v)|, with the iteration's own operators:
// forward differences along +x/+y/+z to the neighbour the sweeps use (a
// missing neighbour counts as the cube itself) and e(v) in Voigt form with the
// off-diagonal terms halved and counted once, as in the q ball.  Neighbour
// values are the current state (u, v), whatever the semantics' border rule.
template <int MODE>
__global__ void k_energy(int o, int cnt, int npos, const int* __restrict__ nb, const float4* __restrict__ uv,
                         const float2* __restrict__ dat, float alpha0, float alpha1, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (i < cnt) {
        const int p = o + i;
        const float4 s = uv[p];
        const float2 D = dat[p];
        if (D.y >= 0.0f) e += 4.0 * (double)D.y * fabs((double)s.x - (double)D.x);  // tot = 4 * (tau tot)
        double nu[3], nv[3][3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int j = __ldg(nb + (size_t)(2 * c) * npos + p);
            const float4 t = j < 0 ? s : uv[j & POS_MASK];
            nu[c] = (double)t.x;
            nv[c][0] = (double)t.y; nv[c][1] = (double)t.z; nv[c][2] = (double)t.w;
        }
        const double u = s.x, v0 = s.y, v1 = s.z, v2 = s.w;
        const double g0 = (nu[0] - u) - v0, g1 = (nu[1] - u) - v1, g2 = (nu[2] - u) - v2;
        e += (double)alpha1 * sqrt(g0 * g0 + g1 * g1 + g2 * g2);
        const double e0 = nv[0][0] - v0, e1 = nv[1][1] - v1, e2 = nv[2][2] - v2;
        const double e3 = 0.5 * ((nv[1][0] - v0) + (nv[0][1] - v1));
        const double e4 = 0.5 * ((nv[2][0] - v0) + (nv[0][2] - v2));
        const double e5 = 0.5 * ((nv[2][1] - v1) + (nv[1][2] - v2));
        e += (double)alpha0 * sqrt(e0 * e0 + e1 * e1 + e2 * e2 + e3 * e3 + e4 * e4 + e5 * e5);
    }
    for (int w = 16; w > 0; w >>= 1) e += __shfl_xor_sync(0xffffffffu, e, w);
    if ((threadIdx.x & 31) == 0 && e != 0.0) atomicAdd(out, e);
}

// ---- coarser-neighbour ghosts (per-launch sweep schedules) -------------------
// A -x/-y/-z neighbour on a coarser level (a position before the level) does
// not change while the level runs.  On the finest level of a ray-cast octree
// about 40 % of those faces have one, and each gather of it read two or three
// 32-byte sectors of P4/Q4/Q1 for the coarse cube's four values, in every
// iteration.  At the level's start the four values of each referenced (coarse
// cube, face) pair are copied to one float4 of a compact array, in the order
// of first reference, and the level's own -face table points to it
// (-2 - entry).  Cubes that share a coarse neighbour across a face are the
// children of at most two parents (the coarse cube's neighbour, and the coarse
// cube itself where the octree keeps a cube together with cubes inside it);
// siblings sit in at most 8 consecutive positions, so a pair is stored once per
// sibling run, at most twice.  The copied values are the ones the gather would
// read, so results are bit-identical.
static constexpr int GHOST_MIN = 16384;  // smaller levels keep the plain gathers
// entry numbers are int: at most three per cube of the level
static constexpr int GHOST_MAX = (int)((((int64_t)1 << 31) - 1) / 3);

template <int MODE>
__device__ __forceinline__ bool coarse_face(int raw, int o) {
    return raw >= 0 && !(MODE == M_STREAM && (raw & BORDER)) && (raw & POS_MASK) < o;
}

// The first position of p's sibling run whose neighbour across the face is the
// same (raw) value; p when none before it.  Positions without a parent form no run.
__device__ __forceinline__ int ghost_first(const int* __restrict__ nbf, const int* __restrict__ par, int o, int p,
                                           int raw) {
    const int pp = par[p];
    int q0 = p;
    if (pp < 0) return q0;
    for (int q = p - 1; q >= max(o, p - 7); --q) {
        if (par[q] != pp) break;
        if (nbf[q] == raw) q0 = q;
    }
    return q0;
}

// mark[f*cnt + i] = 1 where position o + i starts a new ghost entry for face
// 2f+1 (f = 0, 1, 2: -x, -y, -z).
template <int MODE>
__global__ void k_ghost_mark(int o, int cnt, int npos, const int* __restrict__ nb, const int* __restrict__ par,
                             int* __restrict__ mark) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * (int64_t)cnt) return;
    const int f = int(t / cnt), i = int(t - (int64_t)f * cnt), p = o + i;
    const int* nbf = nb + (size_t)(2 * f + 1) * npos;
    const int raw = nbf[p];
    mark[t] = coarse_face<MODE>(raw, o) && ghost_first(nbf, par, o, p, raw) == p;
}

// The level's -face table (pnb[f*cnt + i]) and the ghost entries; ids is the
// exclusive scan of mark.  A face whose run start did not open an entry (a run
// longer than a sibling group, which a 2:1-balanced octree does not have) keeps
// its plain neighbour index.
template <int MODE>
__global__ void k_ghost_fill(int o, int cnt, int npos, const int* __restrict__ nb, const int* __restrict__ par,
                             const int* __restrict__ mark, const int* __restrict__ ids, const float4* __restrict__ P4,
                             const float4* __restrict__ Q4, const float* __restrict__ Q1, int* __restrict__ pnb,
                             float4* __restrict__ gh) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * (int64_t)cnt) return;
    const int f = int(t / cnt), i = int(t - (int64_t)f * cnt), p = o + i;
    const int* nbf = nb + (size_t)(2 * f + 1) * npos;
    const int raw = nbf[p];
    if (!coarse_face<MODE>(raw, o)) {
        pnb[t] = raw;
        return;
    }
    const int q = ghost_first(nbf, par, o, p, raw);
    if (!mark[(int64_t)f * cnt + (q - o)]) {
        pnb[t] = raw;
        return;
    }
    const int e = ids[(int64_t)f * cnt + (q - o)];
    pnb[t] = -2 - e;
    if (q != p) return;
    const int j = raw & POS_MASK;
    const float4 A = P4[j], B = Q4[j];
    // the values each face's gather takes (primal_load_gather)
    gh[e] = f == 0 ? make_float4(A.x, A.w, B.z, B.w)
          : f == 1 ? make_float4(A.y, B.x, B.z, Q1[j])
                   : make_float4(A.z, B.y, B.w, Q1[j]);
}

// The dual sweep's ghosts: +x/+y/+z faces whose neighbour is on another level
// (coarser: finished; deeper: not started) and not a frozen border cube; the
// copy is the neighbour's bar.  Built only on levels of at least
// DUAL_GHOST_MIN cubes whose next deeper level is at least twice as large,
// where many faces have a deeper neighbour: on the finest levels the dual's bar
// gathers already come from L2, and on smaller levels, which are bound by
// latency, the redirect only adds work.
static constexpr int DUAL_GHOST_MIN = 262144;
template <int MODE>
__device__ __forceinline__ bool dual_ghost_face(int raw, int o, int lend) {
    if (raw < 0 || (MODE == M_STREAM && (raw & BORDER))) return false;
    const int j = raw & POS_MASK;
    return j < o || j >= lend;
}

template <int MODE>
__global__ void k_ghost_mark_dual(int o, int cnt, int npos, const int* __restrict__ nb, const int* __restrict__ par,
                                  int* __restrict__ mark) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * (int64_t)cnt) return;
    const int f = int(t / cnt), i = int(t - (int64_t)f * cnt), p = o + i;
    const int* nbf = nb + (size_t)(2 * f) * npos;
    const int raw = nbf[p];
    mark[t] = dual_ghost_face<MODE>(raw, o, o + cnt) && ghost_first(nbf, par, o, p, raw) == p;
}

template <int MODE>
__global__ void k_ghost_fill_dual(int o, int cnt, int npos, const int* __restrict__ nb, const int* __restrict__ par,
                                  const int* __restrict__ mark, const int* __restrict__ ids,
                                  const float4* __restrict__ bar, int* __restrict__ dnb, float4* __restrict__ gh) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * (int64_t)cnt) return;
    const int f = int(t / cnt), i = int(t - (int64_t)f * cnt), p = o + i;
    const int* nbf = nb + (size_t)(2 * f) * npos;
    const int raw = nbf[p];
    if (!dual_ghost_face<MODE>(raw, o, o + cnt)) {
        dnb[t] = raw;
        return;
    }
    const int q = ghost_first(nbf, par, o, p, raw);
    if (!mark[(int64_t)f * cnt + (q - o)]) {
        dnb[t] = raw;
        return;
    }
    const int e = ids[(int64_t)f * cnt + (q - o)];
    dnb[t] = -2 - e;
    if (q == p) gh[e] = bar[raw & POS_MASK];
}

// Streaming semantics, tolerance-stopped solve: at each level's start a leaf's
// stopping flag is 0 when the leaf has cubes on the level, else 2 (finished,
// but not by a met tolerance, which sets 1).
__global__ void k_done_init(int nleaf, int level, const int* __restrict__ ranges, int* __restrict__ done) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nleaf) return;
    const int* r = ranges + (l * NBUCKET + level) * 2;
    done[l] = r[1] > r[0] ? 0 : 2;
}

// Stopping test after a residual iteration: relative fixed-point residual
// (|x+ - x| + |y+ - y|) / (|x+| + |y+|) in FP64 per slot (sigma = tau).
__global__ void k_check(int s0, int ns, double* __restrict__ acc, int* __restrict__ done, float tol, int iter,
                        int* __restrict__ iters_run, double* __restrict__ resid) {
    pdl_wait();
    pdl_release();
    const int s = s0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= s0 + ns || done[s]) return;
    double* q = acc + s * 4;
    const double num = sqrt(q[0]) + sqrt(q[1]);
    const double den = sqrt(q[2]) + sqrt(q[3]);
    const double rel = den > 0.0 ? num / den : 0.0;
    resid[s] = rel;
    if (rel <= (double)tol) { done[s] = 1; iters_run[s] = iter + 1; }
    q[0] = q[1] = q[2] = q[3] = 0.0;
}

// ---- fused iteration (schedule 18) ------------------------------------------
// One launch per iteration.  Blocks take 256-cube tiles of the level (grid-
// stride over tiles, so concurrent tiles are neighbours in Morton order).  A
// tile's dual updates go to shared memory as well as to global memory; the
// dual updates of the tile's halo -- active cubes outside the tile that are a
// tile cube's -x/-y/-z neighbour -- are recomputed into shared memory from the
// same inputs their owners use, so they are bit-identical; the primal updates
// then read every p/q they need from shared memory.  p, q and the bars are
// ping-pong buffers (iteration k reads set k & 1 and writes the other), so no
// block ever reads a value another block of the same launch writes.  Cubes of
// other levels are read from set 0, which holds every finished level.
// Per cube and iteration that is 168 B of compulsory traffic instead of the
// two-kernel split's 204 B (p/q are not written by one kernel and re-read by
// the next).
constexpr int FT = 256;       // cubes per tile = threads per block
constexpr int FH = 3 * FT;    // halo capacity per tile (three faces per cube)
constexpr int FHASH = 2048;   // shared hash slots for building a tile's halo

struct FuseArgs {
    const float4* bar_r; float4* bar_w;
    const float4* P4_r; float4* P4_w;
    const float4* Q4_r; float4* Q4_w;
    const float* Q1_r; float* Q1_w;
    const int* slot;    // [3][npos]: primal neighbour of faces 1/3/5: tile index, FT + halo index,
                        // -1 (none: p/q read as zero), or -(j + 2) for a cube j of another level
    const int* halo;    // [tile][FH] halo positions
    const int* hcount;  // [tile] halo size
    int ntiles;
};

// Halo and neighbour slots of the level's tiles (one block per tile).
template <int MODE>
__global__ void __launch_bounds__(FT) k_fuse_tiles(int o, int n, int npos, const int* __restrict__ nb,
                                                   int* __restrict__ slot, int* __restrict__ halo,
                                                   int* __restrict__ hcount) {
    __shared__ int hk[FHASH];
    __shared__ short hv[FHASH];
    __shared__ int cnt;
    for (int k = threadIdx.x; k < FHASH; k += FT) hk[k] = -1;
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    const int t = blockIdx.x, t0 = o + t * FT;
    const int p = t0 + threadIdx.x;
    if (p < o + n) {
        for (int k = 0; k < 3; ++k) {
            const int j = nb[(2 * k + 1) * npos + p];
            int sl;
            if (j < 0 || (MODE == M_STREAM && (j & BORDER))) {
                sl = -1;
            } else {
                const int jj = j & POS_MASK;
                if (jj < o || jj >= o + n) sl = -(jj + 2);
                else if (jj >= t0 && jj < t0 + FT) sl = jj - t0;
                else {
                    unsigned h = ((unsigned)jj * 2654435761u) & (FHASH - 1);
                    // at most 3 * FT distinct keys in FHASH > 3 * FT slots: a free or equal slot
                    // is met within FHASH probes
                    for (int probe = 0; probe < FHASH; ++probe) {
                        const int prev = atomicCAS(&hk[h], -1, jj);
                        if (prev == -1) {
                            const int id = atomicAdd(&cnt, 1);
                            hv[h] = (short)id;
                            halo[(size_t)t * FH + id] = jj;
                            break;
                        }
                        if (prev == jj) break;
                        h = (h + 1) & (FHASH - 1);
                    }
                    sl = -3 - (int)h;  // resolved to FT + id below, once every id is written
                }
            }
            slot[(size_t)k * npos + p] = sl;
        }
    }
    __syncthreads();
    if (p < o + n)
        for (int k = 0; k < 3; ++k) {
            int* s = slot + (size_t)k * npos + p;
            const int sl = *s;
            const int j = nb[(2 * k + 1) * npos + p];
            const int jj = j & POS_MASK;
            const bool is_halo = j >= 0 && !(MODE == M_STREAM && (j & BORDER)) && jj >= o && jj < o + n &&
                                 !(jj >= t0 && jj < t0 + FT);
            if (is_halo) *s = FT + hv[-3 - sl];
        }
    if (threadIdx.x == 0) hcount[t] = cnt;
}

// Bars of a neighbour: own value when missing, the level-start snapshot for a
// border cube (streaming), the current set for this level's cubes, set 0 for others.
template <int MODE>
__device__ __forceinline__ float4 fused_bar(int j, const float4& own, const IterArgs& a, const FuseArgs& f) {
    if (j < 0) return own;
    if (MODE != M_INMEM && (j & BORDER)) return a.snap[j & POS_MASK];
    return (j >= a.o && j < a.o + a.n) ? __ldcg(f.bar_r + j) : __ldcg(a.bar + j);
}

template <int MODE>
__device__ __forceinline__ void fused_dual_load(const IterArgs& a, const FuseArgs& f, int p, DualLd& L) {
    L.b = __ldcg(f.bar_r + p);
    const int j0 = __ldg(a.nb + p), j2 = __ldg(a.nb + 2 * a.npos + p), j4 = __ldg(a.nb + 4 * a.npos + p);
    L.P = __ldcg(f.P4_r + p);
    L.Q = __ldcg(f.Q4_r + p);
    L.q5 = __ldcg(f.Q1_r + p);
    L.B0 = fused_bar<MODE>(j0, L.b, a, f);
    L.B2 = fused_bar<MODE>(j2, L.b, a, f);
    L.B4 = fused_bar<MODE>(j4, L.b, a, f);
}

// The dual arithmetic of dual_finish, results to registers.
__device__ __forceinline__ void dual_math(const IterArgs& a, const DualLd& L, float4& Po, float4& Qo, float& q5n) {
    const float4 b = L.b, B0 = L.B0, B2 = L.B2, B4 = L.B4, P = L.P, Q = L.Q;
    float p0 = fadd(P.x, fmul(0.25f, fsub(fsub(B0.x, b.x), b.y)));
    float p1 = fadd(P.y, fmul(0.25f, fsub(fsub(B2.x, b.x), b.z)));
    float p2 = fadd(P.z, fmul(0.25f, fsub(fsub(B4.x, b.x), b.w)));
    clip3(p0, p1, p2, a.alpha1);
    const float e0 = fsub(B0.y, b.y);
    const float e1 = fsub(B2.z, b.z);
    const float e2 = fsub(B4.w, b.w);
    const float e3 = fmul(0.5f, fsub(fadd(fsub(B2.y, b.y), B0.z), b.z));
    const float e4 = fmul(0.5f, fsub(fadd(fsub(B4.y, b.y), B0.w), b.w));
    const float e5 = fmul(0.5f, fsub(fadd(fsub(B4.z, b.z), B2.w), b.w));
    float q[6] = {fadd(P.w, fmul(0.25f, e0)), fadd(Q.x, fmul(0.25f, e1)), fadd(Q.y, fmul(0.25f, e2)),
                  fadd(Q.z, fmul(0.25f, e3)), fadd(Q.w, fmul(0.25f, e4)), fadd(L.q5, fmul(0.25f, e5))};
    clip6(q, a.alpha0);
    Po = make_float4(p0, p1, p2, q[0]);
    Qo = make_float4(q[1], q[2], q[3], q[4]);
    q5n = q[5];
}

// Residual terms of one dual update (as dual_finish computes them).
__device__ __forceinline__ void dual_res(const DualLd& L, const float4& Po, const float4& Qo, float q5n, float& dd,
                                         float& nd) {
    const float o[9] = {L.P.x, L.P.y, L.P.z, L.P.w, L.Q.x, L.Q.y, L.Q.z, L.Q.w, L.q5};
    const float w[9] = {Po.x, Po.y, Po.z, Po.w, Qo.x, Qo.y, Qo.z, Qo.w, q5n};
    res_terms<9>(w, o, dd, nd);
}

// ---- tiny levels in shared memory (schedule 23) -------------------------------
// Every iteration of a unit of at most SMEM_MAX_N cubes in ONE launch of ONE
// 1024-thread block that holds the unit's state, data term and neighbour
// indices in shared memory (100 B per cube) for the whole launch: loaded once,
// iterated with __syncthreads between the sweeps, written back once.  Cubes
// outside the unit (coarser levels, the snapshot, other leaves) are read from
// global memory; nothing writes them during the launch.  The arithmetic is the
// split kernels' (dual_math, primal_math).
constexpr int SMEM_MAX_N = 2048;
static inline size_t smem_level_bytes(int n) { return size_t(n) * 100; }
// Staged out-of-unit values follow the unit's arrays at a 16-byte boundary.
static inline size_t smem_ghost_offset(int n) { return (smem_level_bytes(n) + 15) & ~size_t(15); }

template <int MODE>
__device__ __forceinline__ float4 smem_bar(const IterArgs& a, const float4* s_bar, int j, const float4& own) {
    if (j < 0) return own;
    if (MODE != M_INMEM && (j & BORDER)) return a.snap[j & POS_MASK];
    const unsigned li = (unsigned)(j - a.o);
    return li < (unsigned)a.n ? s_bar[li] : a.bar[j];
}

template <int MODE>
__device__ __forceinline__ bool smem_pq(const IterArgs& a, const float4* s_P, const float4* s_Q, const float* s_q5,
                                        int jf, float4& A, float4& B, float& c5) {
    if (jf < 0 || (MODE == M_STREAM && (jf & BORDER))) return false;
    const int j = jf & POS_MASK;
    const unsigned li = (unsigned)(j - a.o);
    if (li < (unsigned)a.n) { A = s_P[li]; B = s_Q[li]; c5 = s_q5[li]; }
    else { A = a.P4[j]; B = a.Q4[j]; c5 = a.Q1[j]; }
    return true;
}

template <int MODE, bool STOP>
__global__ void __launch_bounds__(CLUSTER_BLOCK) k_level_smem(IterArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = a.n, o = a.o;
    float4* s_uv = reinterpret_cast<float4*>(smem_raw);
    float4* s_bar = s_uv + n;
    float4* s_P = s_bar + n;
    float4* s_Q = s_P + n;
    float2* s_dat = reinterpret_cast<float2*>(s_Q + n);
    float* s_q5 = reinterpret_cast<float*>(s_dat + n);
    int* s_nb = reinterpret_cast<int*>(s_q5 + n);  // [6][n]
    float4* s_gh = reinterpret_cast<float4*>(smem_raw + ((size_t(n) * 100 + 15) & ~size_t(15)));
    __shared__ int s_ng;
    if (threadIdx.x == 0) s_ng = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int p = o + i;
        s_uv[i] = a.uv[p]; s_bar[i] = a.bar[p]; s_P[i] = a.P4[p]; s_Q[i] = a.Q4[p];
        s_dat[i] = a.dat[p]; s_q5[i] = a.Q1[p];
#pragma unroll
        for (int f = 0; f < 6; ++f) s_nb[f * n + i] = a.nb[(size_t)f * a.npos + p];
    }
    __syncthreads();
    // Cubes outside the unit (coarser and deeper levels, other leaves, the
    // snapshot) do not change during the launch: the values a face reads from
    // one are staged once, so the iterations touch only shared memory.  A
    // staged face holds slot -2 - g of s_gh: the neighbour's bars for the dual
    // faces +x/+y/+z, the four gathered p/q values for the primal faces
    // -x/-y/-z.  Faces beyond the room left in shared memory keep reading
    // global memory.
    for (int idx = threadIdx.x; idx < 6 * n; idx += blockDim.x) {
        const int f = idx / n;
        const int j = s_nb[idx];
        if (j < 0) continue;
        const bool border = MODE != M_INMEM && (j & BORDER);
        const int jj = j & POS_MASK;
        if (!border && (unsigned)(jj - o) < (unsigned)n) continue;  // inside the unit
        if ((f & 1) && MODE == M_STREAM && border) continue;         // reads as zero already
        float4 g;
        if (!(f & 1)) {
            g = border ? a.snap[jj] : a.bar[jj];
        } else {
            const float4 A = a.P4[jj], B = a.Q4[jj];
            const float c5 = a.Q1[jj];
            g = f == 1 ? make_float4(A.x, A.w, B.z, B.w)
              : f == 3 ? make_float4(A.y, B.x, B.z, c5) : make_float4(A.z, B.y, B.w, c5);
        }
        const int slot = atomicAdd(&s_ng, 1);
        if (slot < a.gcap) { s_gh[slot] = g; s_nb[idx] = -2 - slot; }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int k = 0; k < a.iters; ++k) {
        const int it = a.it0 + k;
        if (STOP && MODE != M_STREAM && *(volatile int*)(a.done + a.slot0)) break;
        const bool res = STOP && ((it + 1) % a.check_every == 0 || it + 1 == a.iters_total);
        WarpAcc wd, wp;
        for (int i0 = 0; i0 < n; i0 += blockDim.x) {  // dual sweep (tgv.cpp:158-189)
            const int i = i0 + (int)threadIdx.x;
            bool work = i < n;
            int slot = -1;
            if (work) slot = (MODE == M_STREAM) ? __ldg(a.lid + o + i) : a.slot0;
            if (STOP && work && MODE == M_STREAM) work = __ldcg(a.done + slot) == 0;
            float dd = 0.f, nd = 0.f;
            if (work) {
                DualLd L;
                L.b = s_bar[i]; L.P = s_P[i]; L.Q = s_Q[i]; L.q5 = s_q5[i];
                const int j0 = s_nb[i], j2 = s_nb[2 * n + i], j4 = s_nb[4 * n + i];
                L.B0 = j0 <= -2 ? s_gh[-2 - j0] : smem_bar<MODE>(a, s_bar, j0, L.b);
                L.B2 = j2 <= -2 ? s_gh[-2 - j2] : smem_bar<MODE>(a, s_bar, j2, L.b);
                L.B4 = j4 <= -2 ? s_gh[-2 - j4] : smem_bar<MODE>(a, s_bar, j4, L.b);
                float4 Po, Qo;
                float q5n;
                dual_math(a, L, Po, Qo, q5n);
                if (res) dual_res(L, Po, Qo, q5n, dd, nd);
                s_P[i] = Po; s_Q[i] = Qo; s_q5[i] = q5n;
            }
            if (res) wd.add(work ? slot : -1, dd, nd, a.acc, 1, lane);
        }
        if (res) wd.flush(a.acc, 1, lane);
        __syncthreads();
        for (int i0 = 0; i0 < n; i0 += blockDim.x) {  // primal sweep (tgv.cpp:191-230)
            const int i = i0 + (int)threadIdx.x;
            bool work = i < n;
            int slot = -1;
            if (work) slot = (MODE == M_STREAM) ? __ldg(a.lid + o + i) : a.slot0;
            if (STOP && work && MODE == M_STREAM) work = __ldcg(a.done + slot) == 0;
            float dd = 0.f, nd = 0.f;
            if (work) {
                PrimalLd L;
                L.U = s_uv[i]; L.P = s_P[i]; L.Q = s_Q[i]; L.q5 = s_q5[i]; L.D = s_dat[i];
                L.gp10 = L.gq10 = L.gq13 = L.gq14 = 0.f;
                L.gp31 = L.gq31 = L.gq33 = L.gq35 = 0.f;
                L.gp52 = L.gq52 = L.gq54 = L.gq55 = 0.f;
                float4 A, B;
                float c5;
                const int j1 = s_nb[n + i], j3 = s_nb[3 * n + i], j5 = s_nb[5 * n + i];
                if (j1 <= -2) {
                    const float4 g = s_gh[-2 - j1];
                    L.gp10 = g.x; L.gq10 = g.y; L.gq13 = g.z; L.gq14 = g.w;
                } else if (smem_pq<MODE>(a, s_P, s_Q, s_q5, j1, A, B, c5)) {
                    L.gp10 = A.x; L.gq10 = A.w; L.gq13 = B.z; L.gq14 = B.w;
                }
                if (j3 <= -2) {
                    const float4 g = s_gh[-2 - j3];
                    L.gp31 = g.x; L.gq31 = g.y; L.gq33 = g.z; L.gq35 = g.w;
                } else if (smem_pq<MODE>(a, s_P, s_Q, s_q5, j3, A, B, c5)) {
                    L.gp31 = A.y; L.gq31 = B.x; L.gq33 = B.z; L.gq35 = c5;
                }
                if (j5 <= -2) {
                    const float4 g = s_gh[-2 - j5];
                    L.gp52 = g.x; L.gq52 = g.y; L.gq54 = g.z; L.gq55 = g.w;
                } else if (smem_pq<MODE>(a, s_P, s_Q, s_q5, j5, A, B, c5)) {
                    L.gp52 = A.z; L.gq52 = B.y; L.gq54 = B.w; L.gq55 = c5;
                }
                float4 uvn, barn;
                if (res) primal_math<true>(L, uvn, barn, dd, nd);
                else primal_math<false>(L, uvn, barn, dd, nd);
                s_uv[i] = uvn; s_bar[i] = barn;
            }
            if (res) wp.add(work ? slot : -1, dd, nd, a.acc, 0, lane);
        }
        if (res) {
            wp.flush(a.acc, 0, lane);
            __syncthreads();
            check_slots<MODE>(a, it);
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int p = o + i;
        a.uv[p] = s_uv[i]; a.bar[p] = s_bar[i]; a.P4[p] = s_P[i]; a.Q4[p] = s_Q[i]; a.Q1[p] = s_q5[i];
    }
}

// ---- small levels in distributed shared memory (schedule 24) -------------------
// As k_level_smem for a unit of up to DSM_MAX_CHUNK cubes per CTA of one
// thread-block cluster (8 or 16 CTAs of 1024 threads): each CTA holds the
// state and data term of its contiguous chunk in its own shared memory (76 B
// per cube; the neighbour indices stay in global memory), and a neighbour in
// another CTA's chunk is read from that CTA's shared memory through the
// cluster's distributed shared memory.  The hardware cluster barrier orders
// the sweeps and makes each CTA's shared-memory writes visible to the others;
// the last barrier of every iteration also keeps every CTA's shared memory
// alive until no other CTA reads it.
constexpr int DSM_MAX_CHUNK = 2816;
static inline size_t dsm_level_bytes(int chunk) { return size_t(chunk) * 76; }

struct DsmView {  // this CTA's arrays; a remote rank's through map_shared_rank
    float4* uv; float4* bar; float4* P; float4* Q; float2* dat; float* q5;
};

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// Generic address of the same shared-memory location in CTA `rank` of the cluster.
template <class T>
__device__ __forceinline__ T* dsm_map(T* p, unsigned rank) {
    unsigned long long in = (unsigned long long)p, out;
    asm volatile("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"(in), "r"(rank));
    return reinterpret_cast<T*>(out);
}

template <int MODE>
__device__ __forceinline__ float4 dsm_bar(const IterArgs& a, const DsmView& v, int chunk, unsigned me, int j,
                                          const float4& own) {
    if (j < 0) return own;
    if (MODE != M_INMEM && (j & BORDER)) return a.snap[j & POS_MASK];
    const unsigned li = (unsigned)(j - a.o);
    if (li >= (unsigned)a.n) return a.bar[j];
    const unsigned r = li / (unsigned)chunk, l = li - r * (unsigned)chunk;
    return r == me ? v.bar[l] : dsm_map(v.bar, r)[l];
}

template <int MODE>
__device__ __forceinline__ bool dsm_pq(const IterArgs& a, const DsmView& v, int chunk, unsigned me, int jf, float4& A,
                                       float4& B, float& c5) {
    if (jf < 0 || (MODE == M_STREAM && (jf & BORDER))) return false;
    const int j = jf & POS_MASK;
    const unsigned li = (unsigned)(j - a.o);
    if (li >= (unsigned)a.n) { A = a.P4[j]; B = a.Q4[j]; c5 = a.Q1[j]; return true; }
    const unsigned r = li / (unsigned)chunk, l = li - r * (unsigned)chunk;
    if (r == me) { A = v.P[l]; B = v.Q[l]; c5 = v.q5[l]; }
    else { A = dsm_map(v.P, r)[l]; B = dsm_map(v.Q, r)[l]; c5 = dsm_map(v.q5, r)[l]; }
    return true;
}

template <int MODE, bool STOP>
__global__ void __launch_bounds__(CLUSTER_BLOCK) k_level_dsm(IterArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int chunk = a.chunk;
    const unsigned me = cluster_rank();
    DsmView v;
    v.uv = reinterpret_cast<float4*>(smem_raw);
    v.bar = v.uv + chunk;
    v.P = v.bar + chunk;
    v.Q = v.P + chunk;
    v.dat = reinterpret_cast<float2*>(v.Q + chunk);
    v.q5 = reinterpret_cast<float*>(v.dat + chunk);
    const int beg = a.o + (int)me * chunk, cnt = max(0, min(chunk, a.o + a.n - beg));
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int p = beg + i;
        v.uv[i] = a.uv[p]; v.bar[i] = a.bar[p]; v.P[i] = a.P4[p]; v.Q[i] = a.Q4[p];
        v.dat[i] = a.dat[p]; v.q5[i] = a.Q1[p];
    }
    cluster_barrier();
    const int lane = threadIdx.x & 31;
    for (int k = 0; k < a.iters; ++k) {
        const int it = a.it0 + k;
        if (STOP && MODE != M_STREAM && *(volatile int*)(a.done + a.slot0)) break;
        const bool res = STOP && ((it + 1) % a.check_every == 0 || it + 1 == a.iters_total);
        WarpAcc wd, wp;
        for (int i0 = 0; i0 < cnt; i0 += blockDim.x) {  // dual sweep (tgv.cpp:158-189)
            const int i = i0 + (int)threadIdx.x, p = beg + i;
            bool work = i < cnt;
            int slot = -1;
            if (work) slot = (MODE == M_STREAM) ? __ldg(a.lid + p) : a.slot0;
            if (STOP && work && MODE == M_STREAM) work = __ldcg(a.done + slot) == 0;
            float dd = 0.f, nd = 0.f;
            if (work) {
                DualLd L;
                L.b = v.bar[i]; L.P = v.P[i]; L.Q = v.Q[i]; L.q5 = v.q5[i];
                L.B0 = dsm_bar<MODE>(a, v, chunk, me, __ldg(a.nb + p), L.b);
                L.B2 = dsm_bar<MODE>(a, v, chunk, me, __ldg(a.nb + 2 * a.npos + p), L.b);
                L.B4 = dsm_bar<MODE>(a, v, chunk, me, __ldg(a.nb + 4 * a.npos + p), L.b);
                float4 Po, Qo;
                float q5n;
                dual_math(a, L, Po, Qo, q5n);
                if (res) dual_res(L, Po, Qo, q5n, dd, nd);
                v.P[i] = Po; v.Q[i] = Qo; v.q5[i] = q5n;
            }
            if (res) wd.add(work ? slot : -1, dd, nd, a.acc, 1, lane);
        }
        if (res) wd.flush(a.acc, 1, lane);
        cluster_barrier();
        for (int i0 = 0; i0 < cnt; i0 += blockDim.x) {  // primal sweep (tgv.cpp:191-230)
            const int i = i0 + (int)threadIdx.x, p = beg + i;
            bool work = i < cnt;
            int slot = -1;
            if (work) slot = (MODE == M_STREAM) ? __ldg(a.lid + p) : a.slot0;
            if (STOP && work && MODE == M_STREAM) work = __ldcg(a.done + slot) == 0;
            float dd = 0.f, nd = 0.f;
            if (work) {
                PrimalLd L;
                L.U = v.uv[i]; L.P = v.P[i]; L.Q = v.Q[i]; L.q5 = v.q5[i]; L.D = v.dat[i];
                L.gp10 = L.gq10 = L.gq13 = L.gq14 = 0.f;
                L.gp31 = L.gq31 = L.gq33 = L.gq35 = 0.f;
                L.gp52 = L.gq52 = L.gq54 = L.gq55 = 0.f;
                float4 A, B;
                float c5;
                if (dsm_pq<MODE>(a, v, chunk, me, __ldg(a.nb + a.npos + p), A, B, c5)) {
                    L.gp10 = A.x; L.gq10 = A.w; L.gq13 = B.z; L.gq14 = B.w;
                }
                if (dsm_pq<MODE>(a, v, chunk, me, __ldg(a.nb + 3 * a.npos + p), A, B, c5)) {
                    L.gp31 = A.y; L.gq31 = B.x; L.gq33 = B.z; L.gq35 = c5;
                }
                if (dsm_pq<MODE>(a, v, chunk, me, __ldg(a.nb + 5 * a.npos + p), A, B, c5)) {
                    L.gp52 = A.z; L.gq52 = B.y; L.gq54 = B.w; L.gq55 = c5;
                }
                float4 uvn, barn;
                if (res) primal_math<true>(L, uvn, barn, dd, nd);
                else primal_math<false>(L, uvn, barn, dd, nd);
                v.uv[i] = uvn; v.bar[i] = barn;
            }
            if (res) wp.add(work ? slot : -1, dd, nd, a.acc, 0, lane);
        }
        if (res) {
            wp.flush(a.acc, 0, lane);
            cluster_barrier();
            if (me == 0) check_slots<MODE>(a, it);
        }
        cluster_barrier();
    }
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int p = beg + i;
        a.uv[p] = v.uv[i]; a.bar[p] = v.bar[i]; a.P4[p] = v.P[i]; a.Q4[p] = v.Q[i]; a.Q1[p] = v.q5[i];
    }
}

// The primal's neighbour p/q of faces 1/3/5 from their slots: shared memory
// (tile or halo), zero (none / border), or set 0 of global memory (another level).
__device__ __forceinline__ void fused_gather(const IterArgs& a, const float4* sP, const float4* sQ, const float* s5,
                                             const int* sl, PrimalLd& L) {
    float g[3][4];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A;
        float c5 = 0.f;
        if (sl[k] >= 0) {
            A = sP[sl[k]]; B = sQ[sl[k]]; c5 = s5[sl[k]];
        } else if (sl[k] <= -2) {
            const int j = -(sl[k] + 2);
            A = __ldcg(a.P4 + j); B = __ldcg(a.Q4 + j); c5 = __ldcg(a.Q1 + j);
        }
        // face 1 needs p0, q0, q3, q4; face 3: p1, q1, q3, q5; face 5: p2, q2, q4, q5
        if (k == 0) { g[0][0] = A.x; g[0][1] = A.w; g[0][2] = B.z; g[0][3] = B.w; }
        else if (k == 1) { g[1][0] = A.y; g[1][1] = B.x; g[1][2] = B.z; g[1][3] = c5; }
        else { g[2][0] = A.z; g[2][1] = B.y; g[2][2] = B.w; g[2][3] = c5; }
    }
    L.gp10 = g[0][0]; L.gq10 = g[0][1]; L.gq13 = g[0][2]; L.gq14 = g[0][3];
    L.gp31 = g[1][0]; L.gq31 = g[1][1]; L.gq33 = g[1][2]; L.gq35 = g[1][3];
    L.gp52 = g[2][0]; L.gq52 = g[2][1]; L.gq54 = g[2][2]; L.gq55 = g[2][3];
}

template <int MODE, bool RES, bool STOP>
__global__ void __launch_bounds__(FT) k_fused(IterArgs a, FuseArgs f) {
    __shared__ float4 sP[FT + FH], sQ[FT + FH];
    __shared__ float s5[FT + FH];
    pdl_wait();
    pdl_release();
    if (MODE != M_STREAM && STOP && a.done[a.slot0]) return;
    const int lane = threadIdx.x & 31;
    WarpAcc wd, wp;
    for (int t = blockIdx.x; t < f.ntiles; t += gridDim.x) {
        const int p = a.o + t * FT + threadIdx.x;
        bool own = p < a.o + a.n;
        int slot = -1;
        if (own) slot = (MODE == M_STREAM) ? __ldg(a.lid + p) : a.slot0;
        if (STOP && own && MODE == M_STREAM) own = __ldg(a.done + slot) == 0;
        // dual: the tile's own cubes
        float dd = 0.f, nd = 0.f;
        if (own) {
            DualLd L;
            fused_dual_load<MODE>(a, f, p, L);
            float4 Po, Qo;
            float q5n;
            dual_math(a, L, Po, Qo, q5n);
            f.P4_w[p] = Po; f.Q4_w[p] = Qo; f.Q1_w[p] = q5n;
            sP[threadIdx.x] = Po; sQ[threadIdx.x] = Qo; s5[threadIdx.x] = q5n;
            if (RES) dual_res(L, Po, Qo, q5n, dd, nd);
        }
        if (RES) wd.add(own ? slot : -1, dd, nd, a.acc, 1, lane);
        // dual: the halo, recomputed (not stored globally)
        const int nh = __ldg(f.hcount + t);
        for (int h = threadIdx.x; h < nh; h += FT) {
            const int q = __ldg(f.halo + (size_t)t * FH + h);
            DualLd L;
            fused_dual_load<MODE>(a, f, q, L);
            float4 Po, Qo;
            float q5n;
            dual_math(a, L, Po, Qo, q5n);
            sP[FT + h] = Po; sQ[FT + h] = Qo; s5[FT + h] = q5n;
        }
        __syncthreads();
        // primal
        dd = 0.0; nd = 0.0;
        if (own) {
            PrimalLd L;
            L.U = __ldcg(a.uv + p);
            L.P = sP[threadIdx.x]; L.Q = sQ[threadIdx.x]; L.q5 = s5[threadIdx.x];
            L.D = __ldg(a.dat + p);
            int sl[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) sl[k] = __ldg(f.slot + (size_t)k * a.npos + p);
            fused_gather(a, sP, sQ, s5, sl, L);
            IterArgs w = a;
            w.bar = f.bar_w;
            primal_finish<RES>(w, p, L, dd, nd);
        }
        if (RES) wp.add(own ? slot : -1, dd, nd, a.acc, 0, lane);
        __syncthreads();
    }
    if (RES) { wd.flush(a.acc, 1, lane); wp.flush(a.acc, 0, lane); }
}

// ---- fused iteration with TMA staging (schedule 19) ---------------------------
// As k_fused, with each tile's contiguous per-cube streams (bars, p/q, u/v,
// data term, neighbour ids and slots: 25.7 KB) brought into shared memory by
// 1-D bulk async copies (cp.async.bulk, completion counted on an mbarrier),
// double-buffered: one thread issues tile t + 1's copies before the block works
// on tile t.  Only neighbour bars, halo cubes and other levels' cubes are
// read with ordinary loads.  Every mbarrier wait is bounded; a wait that runs
// out sets the error flag, waits (bounded) for the copies in flight and ends
// the kernel, and the solve returns TGVG_ERR_TIMEOUT.
struct TileStage {                 // one buffer; every member starts on a 16-byte boundary
    float4 bar[FT], P4[FT], Q4[FT], uv[FT];
    float Q1[FT + 4];
    int nb[3][FT + 4];             // faces 0, 2, 4
    int sl[3][FT + 4];             // slots of faces 1, 3, 5
    float2 dat[FT + 2];
};
static_assert(sizeof(TileStage) % 16 == 0, "TileStage alignment");
struct FusedSmem {
    TileStage st[2];
    float4 sP[FT + FH], sQ[FT + FH];
    float s5[FT + FH];
    unsigned long long mbar[2];
};
static constexpr size_t FUSED_TMA_SMEM = sizeof(FusedSmem);

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(b))
                 : "memory");
}

// Copy elements [t0, t0 + cnt) of a 4- or 8-byte array into dst: the copy
// starts at the 16-byte boundary at or below the first element (dst is indexed
// from `off` = the elements before it) and is rounded up to 16 bytes.  The
// arrays carry at least 16 bytes of padding past their end.
__device__ __forceinline__ uint32_t slice_bytes(const void* first, int es, int cnt, int& off) {
    const uintptr_t a = (uintptr_t)first, al = a & ~(uintptr_t)15;
    off = (int)((a - al) / es);
    return ((uint32_t)((off + cnt) * es) + 15u) & ~15u;
}
__device__ __forceinline__ const void* slice_src(const void* first) {
    return (const void*)((uintptr_t)first & ~(uintptr_t)15);
}

// Issue tile t's copies into stage buffer S (one thread).  The fence orders
// the block's earlier ordinary reads of S (the barrier before this call made
// them complete) before the asynchronous writes.
__device__ __forceinline__ void stage_tile(const IterArgs& a, const FuseArgs& f, int t, TileStage& S,
                                           unsigned long long* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const int t0 = a.o + t * FT;
    const int cnt = min(FT, a.o + a.n - t0);
    int off;
    uint32_t total = 16u * cnt * 4;
    const float* q1 = f.Q1_r + t0;
    const uint32_t bq1 = slice_bytes(q1, 4, cnt, off);
    total += bq1;
    uint32_t bnb[3], bsl[3];
    for (int k = 0; k < 3; ++k) {
        bnb[k] = slice_bytes(a.nb + (size_t)(2 * k) * a.npos + t0, 4, cnt, off);
        bsl[k] = slice_bytes(f.slot + (size_t)k * a.npos + t0, 4, cnt, off);
        total += bnb[k] + bsl[k];
    }
    const uint32_t bdat = slice_bytes(a.dat + t0, 8, cnt, off);
    total += bdat;
    mbar_expect_tx(bar, total);
    bulk_load(S.bar, f.bar_r + t0, 16u * cnt, bar);
    bulk_load(S.P4, f.P4_r + t0, 16u * cnt, bar);
    bulk_load(S.Q4, f.Q4_r + t0, 16u * cnt, bar);
    bulk_load(S.uv, a.uv + t0, 16u * cnt, bar);
    bulk_load(S.Q1, slice_src(q1), bq1, bar);
    for (int k = 0; k < 3; ++k) {
        bulk_load(S.nb[k], slice_src(a.nb + (size_t)(2 * k) * a.npos + t0), bnb[k], bar);
        bulk_load(S.sl[k], slice_src(f.slot + (size_t)k * a.npos + t0), bsl[k], bar);
    }
    bulk_load(S.dat, slice_src(a.dat + t0), bdat, bar);
}

// Bounded wait of every thread of the block for a stage buffer; true when all
// saw it complete.
__device__ __forceinline__ bool stage_wait(unsigned long long* bar, uint32_t parity) {
    bool ok = false;
    for (int spin = 0; spin < (1 << 22) && !ok; ++spin) {
        ok = mbar_try_wait(bar, parity);
        if (!ok) __nanosleep(64);
    }
    return __syncthreads_and(ok) != 0;
}

template <int MODE, bool RES, bool STOP>
__global__ void __launch_bounds__(FT) k_fused_tma(IterArgs a, FuseArgs f) {
    extern __shared__ __align__(128) unsigned char dsm[];
    FusedSmem& sm = *reinterpret_cast<FusedSmem*>(dsm);
    pdl_wait();
    pdl_release();
    if (MODE != M_STREAM && STOP && a.done[a.slot0]) return;
    if (threadIdx.x == 0) {
        mbar_init(&sm.mbar[0]);
        mbar_init(&sm.mbar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    WarpAcc wd, wp;
    if (threadIdx.x == 0 && (int)blockIdx.x < f.ntiles) stage_tile(a, f, blockIdx.x, sm.st[0], &sm.mbar[0]);
    int i = 0;
    for (int t = blockIdx.x; t < f.ntiles; t += gridDim.x, ++i) {
        const int b = i & 1;
        const int tn = t + gridDim.x;
        if (threadIdx.x == 0 && tn < f.ntiles) stage_tile(a, f, tn, sm.st[b ^ 1], &sm.mbar[b ^ 1]);
        if (!stage_wait(&sm.mbar[b], (uint32_t)(i >> 1) & 1u)) {
            if (threadIdx.x == 0) {
                atomicOr(a.err, 4);
                // let the copies in flight land before the block's shared memory goes away (bounded)
                for (int spin = 0; spin < (1 << 22) && !mbar_try_wait(&sm.mbar[b], (uint32_t)(i >> 1) & 1u); ++spin)
                    __nanosleep(64);
                if (tn < f.ntiles)
                    for (int spin = 0;
                         spin < (1 << 22) && !mbar_try_wait(&sm.mbar[b ^ 1], (uint32_t)((i + 1) >> 1) & 1u); ++spin)
                        __nanosleep(64);
            }
            return;
        }
        const TileStage& S = sm.st[b];
        const int t0 = a.o + t * FT;
        const int cnt = min(FT, a.o + a.n - t0);
        const int p = t0 + threadIdx.x;
        bool own = threadIdx.x < cnt;
        int slot = -1;
        if (own) slot = (MODE == M_STREAM) ? __ldg(a.lid + p) : a.slot0;
        if (STOP && own && MODE == M_STREAM) own = __ldg(a.done + slot) == 0;
        // offsets of the 4- and 8-byte slices inside their stage arrays
        int oq1, onb[3], osl[3], odat;
        slice_bytes(f.Q1_r + t0, 4, cnt, oq1);
        for (int k = 0; k < 3; ++k) {
            slice_bytes(a.nb + (size_t)(2 * k) * a.npos + t0, 4, cnt, onb[k]);
            slice_bytes(f.slot + (size_t)k * a.npos + t0, 4, cnt, osl[k]);
        }
        slice_bytes(a.dat + t0, 8, cnt, odat);
        float dd = 0.f, nd = 0.f;
        if (own) {
            const int x = threadIdx.x;
            DualLd L;
            L.b = S.bar[x]; L.P = S.P4[x]; L.Q = S.Q4[x]; L.q5 = S.Q1[oq1 + x];
            L.B0 = fused_bar<MODE>(S.nb[0][onb[0] + x], L.b, a, f);
            L.B2 = fused_bar<MODE>(S.nb[1][onb[1] + x], L.b, a, f);
            L.B4 = fused_bar<MODE>(S.nb[2][onb[2] + x], L.b, a, f);
            float4 Po, Qo;
            float q5n;
            dual_math(a, L, Po, Qo, q5n);
            f.P4_w[p] = Po; f.Q4_w[p] = Qo; f.Q1_w[p] = q5n;
            sm.sP[x] = Po; sm.sQ[x] = Qo; sm.s5[x] = q5n;
            if (RES) dual_res(L, Po, Qo, q5n, dd, nd);
        }
        if (RES) wd.add(own ? slot : -1, dd, nd, a.acc, 1, lane);
        const int nh = __ldg(f.hcount + t);
        for (int h = threadIdx.x; h < nh; h += FT) {
            const int q = __ldg(f.halo + (size_t)t * FH + h);
            DualLd L;
            fused_dual_load<MODE>(a, f, q, L);
            float4 Po, Qo;
            float q5n;
            dual_math(a, L, Po, Qo, q5n);
            sm.sP[FT + h] = Po; sm.sQ[FT + h] = Qo; sm.s5[FT + h] = q5n;
        }
        __syncthreads();
        dd = 0.0; nd = 0.0;
        if (own) {
            const int x = threadIdx.x;
            PrimalLd L;
            L.U = S.uv[x];
            L.P = sm.sP[x]; L.Q = sm.sQ[x]; L.q5 = sm.s5[x];
            L.D = S.dat[odat + x];
            const int sl[3] = {S.sl[0][osl[0] + x], S.sl[1][osl[1] + x], S.sl[2][osl[2] + x]};
            fused_gather(a, sm.sP, sm.sQ, sm.s5, sl, L);
            IterArgs w = a;
            w.bar = f.bar_w;
            primal_finish<RES>(w, p, L, dd, nd);
        }
        if (RES) wp.add(own ? slot : -1, dd, nd, a.acc, 0, lane);
        __syncthreads();
    }
    if (RES) { wd.flush(a.acc, 1, lane); wp.flush(a.acc, 0, lane); }
}

// After a fused segment [it0, it0 + count): every cube whose slot ran an odd
// number of the segment's iterations has its state in set 1; copy it to set 0.
__global__ void k_fuse_settle(int o, int n, int it0, int count, int slot0, const int* __restrict__ lid,
                              const int* __restrict__ iters_run, int mode, const float4* __restrict__ barB,
                              const float4* __restrict__ P4B, const float4* __restrict__ Q4B,
                              const float* __restrict__ Q1B, float4* __restrict__ bar, float4* __restrict__ P4,
                              float4* __restrict__ Q4, float* __restrict__ Q1) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int p = o + t;
    const int s = mode == M_STREAM ? lid[p] : slot0;
    const int e = min(iters_run[s], it0 + count) - it0;
    if (e <= 0 || !(e & 1)) return;
    bar[p] = barB[p];
    P4[p] = P4B[p];
    Q4[p] = Q4B[p];
    Q1[p] = Q1B[p];
}

// ---- ordered wavefront: one launch per iteration, dual then primal per tile --
// The level is cut into tiles of 512 positions (two cubes, one after the other,
// per thread of a 256-thread block), aligned to multiples of 32 positions so that no 128-byte
// line of any per-cube array is shared by two tiles.  Tile c depends on tile d
// when a cube of c has an active -x/-y/-z neighbour in d (c's primal step reads
// its p/q), or a cube of d has an active +x/+y/+z neighbour in c (d's dual step
// reads the bar that c's primal step overwrites).  In Morton order d < c for
// nearly every pair; the exceptions come from the parent-code lookup, which
// can land on the octant-0 cube of the parent a few positions back.
// Consecutive tiles are therefore joined into groups so that every dependency
// points to an earlier group or into its own.  Blocks claim groups in
// increasing order from a counter; for its group a block runs the dual steps
// of all its tiles, publishes their flags (the iteration's epoch), waits for
// the flags of the tiles the group's primal steps depend on, and runs the
// primal steps.  A block only ever waits for tiles of groups claimed before
// its own (or its own, already published), whose dual steps never wait: the
// wavefront cannot deadlock.  The waits are bounded anyway.
// Every cube gets exactly the split schedule's arithmetic, so the results are
// the same bit for bit; the pass reads and writes each record once per
// iteration instead of twice.
static constexpr int WAVE_BLOCK = 256;            // threads per block
static constexpr int WT = 2 * WAVE_BLOCK;          // cubes per tile: two per thread

struct WaveArgs {
    const int* doff;   // [ntiles + 1] offsets into dep
    const int* dep;    // tiles each tile's primal step waits for
    const int* gstart; // [ngroups + 1] first tile of each group
    int* flag;         // [ntiles] epoch of the last published dual step
    int* claim;        // [2] group counters of alternate iterations
    int ngroups, base, epoch;
};

__device__ __forceinline__ int wave_tile_of(int p, int base) { return (p - base) / WT; }

// Dependency pairs (consumer tile << 32 | producer tile) of one level, or only
// their count (out == nullptr); reach[c] = the last tile after c that c depends
// on (when out == nullptr).
template <int MODE>
__global__ void k_wave_pairs(int o, int cnt, int base, int npos, const int* __restrict__ nb,
                             unsigned long long* __restrict__ out, int* __restrict__ count, int* __restrict__ reach) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long key[6];
    int k = 0;
    if (i < cnt) {
        const int p = o + i, tp = wave_tile_of(p, base);
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            int j = __ldg(nb + (size_t)f * npos + p);
            if (j < 0 || (MODE == M_STREAM && (j & BORDER))) continue;
            j &= POS_MASK;
            if (j < o || j >= o + cnt) continue;  // not active on this level
            const int tj = wave_tile_of(j, base);
            const int cons = (f & 1) ? tp : tj, prod = (f & 1) ? tj : tp;
            if (cons == prod) continue;
            if (prod > cons && !out) atomicMax(reach + cons, prod);
            key[k++] = ((unsigned long long)cons << 32) | (unsigned)prod;
        }
    }
    // warp-aggregated reservation of the output slots
    const int lane = threadIdx.x & 31;
    int incl = k;
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    int base_slot = 0;
    if (lane == 31) base_slot = atomicAdd(count, incl);
    base_slot = __shfl_sync(0xffffffffu, base_slot, 31);
    if (out)
        for (int m = 0; m < k; ++m) out[base_slot + incl - k + m] = key[m];
}

__global__ void k_wave_unique(int m, const unsigned long long* __restrict__ keys, int* __restrict__ keep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) keep[i] = i == 0 || keys[i] != keys[i - 1];
}

__global__ void k_wave_compact(int m, const unsigned long long* __restrict__ keys, const int* __restrict__ keep,
                               const int* __restrict__ pos, unsigned long long* __restrict__ ukeys,
                               int* __restrict__ dep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m && keep[i]) {
        ukeys[pos[i]] = keys[i];
        dep[pos[i]] = (int)(keys[i] & 0xffffffffu);
    }
}

// doff[t] = first unique pair whose consumer is >= t (binary search).
__global__ void k_wave_offsets(int ntiles, int nu, const unsigned long long* __restrict__ ukeys, int* __restrict__ doff) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > ntiles) return;
    const unsigned long long want = (unsigned long long)t << 32;
    int lo = 0, hi = nu;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ukeys[mid] < want) lo = mid + 1; else hi = mid;
    }
    doff[t] = lo;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Position of cube u (0 or 1) of this thread in tile t, whether it is active
// (in the unit and, when streaming with stopping tests, its slot still
// running), and its stopping slot.
template <int MODE, bool STOP>
__device__ __forceinline__ int wave_cube(const IterArgs& a, const WaveArgs& w, int t, int u, bool& work, int& slot) {
    const int p = w.base + t * WT + u * WAVE_BLOCK + (int)threadIdx.x;
    work = p >= a.o && p < a.o + a.n;
    slot = -1;
    if (work) slot = (MODE == M_STREAM) ? __ldg(a.lid + p) : a.slot0;
    if (STOP && work && MODE == M_STREAM) work = __ldg(a.done + slot) == 0;
    return p;
}

template <int MODE, bool RES, bool STOP, bool CG>
__global__ void __launch_bounds__(WAVE_BLOCK, 5) k_wave(IterArgs a, WaveArgs w) {
    __shared__ int s_group;
    if (blockIdx.x == 0 && threadIdx.x == 0) w.claim[(w.epoch + 1) & 1] = 0;  // the next iteration's counter
    if (MODE != M_STREAM && STOP && a.done[a.slot0]) return;
    const int lane = threadIdx.x & 31;
    WarpAcc wd, wp;
    for (;;) {
        if (threadIdx.x == 0) s_group = atomicAdd(w.claim + (w.epoch & 1), 1);
        __syncthreads();
        const int g = s_group;
        if (g >= w.ngroups) break;
        const int t0 = __ldg(w.gstart + g), t1 = __ldg(w.gstart + g + 1);
        for (int t = t0; t < t1; ++t)
#pragma unroll 1
            for (int u = 0; u < 2; ++u) {
                bool wk;
                int sl;
                const int p = wave_cube<MODE, STOP>(a, w, t, u, wk, sl);
                float dd = 0.f, nd = 0.f;
                if (wk) dual_cube<MODE, RES, CG>(a, p, dd, nd);
                if (RES) wd.add(wk ? sl : -1, dd, nd, a.acc, 1, lane);
            }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            for (int t = t0; t < t1; ++t) st_release(w.flag + t, w.epoch);
        }
        // wait for the tiles the group's primal steps read from or overwrite for
        bool ok = true;
        for (int t = t0; t < t1 && ok; ++t)
            for (int k = __ldg(w.doff + t) + (int)threadIdx.x; k < __ldg(w.doff + t + 1) && ok; k += WAVE_BLOCK) {
                const int* f = w.flag + __ldg(w.dep + k);
                for (int spin = 0; ld_acquire(f) != w.epoch; ++spin) {
                    if (spin > (1 << 20)) { ok = false; break; }  // about 0.1 s and more: give up, report
                    __nanosleep(32);
                }
            }
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) atomicOr(a.err, 8);
            break;
        }
        for (int t = t0; t < t1; ++t)
#pragma unroll 1
            for (int u = 0; u < 2; ++u) {
                bool wk;
                int sl;
                const int p = wave_cube<MODE, STOP>(a, w, t, u, wk, sl);
                float dd = 0.f, nd = 0.f;
                if (wk) primal_cube<MODE, RES, CG>(a, p, dd, nd);
                if (RES) wp.add(wk ? sl : -1, dd, nd, a.acc, 0, lane);
            }
        __syncthreads();  // s_group is rewritten for the next group
    }
    if (RES) {
        wd.flush(a.acc, 1, lane);
        wp.flush(a.acc, 0, lane);
    }
}

__global__ void k_unpermute(int n, const int* __restrict__ inv, const float4* __restrict__ uv,
                            const float4* __restrict__ P4, const float4* __restrict__ Q4,
                            const float* __restrict__ Q1, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int p = inv[i];
    const float4 u = uv[p], a = P4[p], b = Q4[p];
    float* r = out + (size_t)i * 13;
    r[0] = u.x; r[1] = u.y; r[2] = u.z; r[3] = u.w;
    r[4] = a.x; r[5] = a.y; r[6] = a.z; r[7] = a.w;
    r[8] = b.x; r[9] = b.y; r[10] = b.z; r[11] = b.w;
    r[12] = Q1[p];
}

// ------------------------------------------------------------------ host ---

static inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Launch with programmatic stream serialisation (the kernel calls pdl_wait()
// before it touches memory): the launch and the first blocks overlap the end
// of the previous kernel.  Errors surface through cudaGetLastError.
template <class... KArgs, class... Args>
static void launch_pdl_smem(void (*k)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                            Args... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(block);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    cudaLaunchKernelEx(&lc, k, args...);
}
template <class... KArgs, class... Args>
static void launch_pdl(void (*k)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args) {
    launch_pdl_smem(k, grid, block, 0, s, args...);
}

// The residual-summing variants (one iteration in check_every) keep the old
// and new state of a cube and the slot's sums live: at the 40-register bound of
// six blocks per SM they spilled 60-124 bytes per thread, and a checking
// iteration cost about twice a plain one.  They run at four blocks per SM.
constexpr int RES_MINB = 4;
template <int MODE>
static void launch_iter(tgvg_ctx* ctx, IterArgs a, bool res, bool stop, bool dual, bool lean, bool ilp2) {
    // One full wave: as many blocks as fit on the GPU at once (occupancy of the
    // variant), each owning an equal contiguous chunk of the unit.
    const int occ = ilp2  ? ctx->iter_occ_ilp2[MODE][dual ? 0 : 1]
                    : res ? ctx->iter_occ_res[MODE][dual ? 0 : 1]
                          : ctx->iter_occ[MODE][lean ? 1 : 0][dual ? 0 : 1];
    const int want = std::max(1, std::min((a.n + ITER_BLOCK - 1) / ITER_BLOCK, occ * ctx->sm_count));
    a.chunk = ((a.n + want - 1) / want + 31) / 32 * 32;
    const unsigned grid = (unsigned)((a.n + a.chunk - 1) / a.chunk);
    void (*k)(IterArgs);
#define TGVG_ITER(K)                                      \
    if (ilp2 && res && stop) k = K<MODE, true, true, 4, 2>; \
    else if (ilp2 && res) k = K<MODE, true, false, 4, 2>;   \
    else if (ilp2 && stop) k = K<MODE, false, true, 4, 2>;  \
    else if (ilp2) k = K<MODE, false, false, 4, 2>;         \
    else if (res && stop) k = K<MODE, true, true, RES_MINB>; \
    else if (res) k = K<MODE, true, false, RES_MINB>;        \
    else if (stop) k = K<MODE, false, true, 6>;             \
    else if (lean) k = K<MODE, false, false, 8>;            \
    else k = K<MODE, false, false, 6>;
    if (dual) { TGVG_ITER(k_dual) } else { TGVG_ITER(k_primal) }
#undef TGVG_ITER
    launch_pdl(k, grid, ITER_BLOCK, ctx->stream, a);
}

// Blocks per SM of the plain (and register-capped) sweep kernels, per mode.
template <int MODE>
static int iter_occupancy(tgvg_ctx* ctx) {
    int* o = &ctx->iter_occ[MODE][0][0];
    if (o[0] > 0) return TGVG_OK;
    int v[4] = {0, 0, 0, 0};
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v[0], k_dual<MODE, false, false, 6>, ITER_BLOCK, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v[1], k_primal<MODE, false, false, 6>, ITER_BLOCK, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v[2], k_dual<MODE, false, false, 8>, ITER_BLOCK, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v[3], k_primal<MODE, false, false, 8>, ITER_BLOCK, 0);
    int r[2] = {0, 0};
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r[0], k_dual<MODE, true, true, RES_MINB>, ITER_BLOCK, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r[1], k_primal<MODE, true, true, RES_MINB>, ITER_BLOCK, 0);
    int w[2] = {0, 0};
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&w[0], k_dual<MODE, false, false, 4, 2>, ITER_BLOCK, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&w[1], k_primal<MODE, false, false, 4, 2>, ITER_BLOCK, 0);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "occupancy query");
    o[0] = std::max(1, v[0]); o[1] = std::max(1, v[1]); o[2] = std::max(1, v[2]); o[3] = std::max(1, v[3]);
    ctx->iter_occ_res[MODE][0] = std::max(1, r[0]);
    ctx->iter_occ_res[MODE][1] = std::max(1, r[1]);
    ctx->iter_occ_ilp2[MODE][0] = std::max(1, w[0]);
    ctx->iter_occ_ilp2[MODE][1] = std::max(1, w[1]);
    return TGVG_OK;
}

// ---- launch schedules of one unit (a level, or one leaf's slice of it in OC) ----
// cfg 0: two launches per iteration (K6, K7) over a grid of up to 8 blocks per SM.
// cfg k in 1..6: one cooperative launch of k_level_persistent running all the
//   unit's iterations, with about 256 << k cubes per block.
// Every schedule applies the identical per-cube arithmetic, so the choice never
// changes a result, only the time.
// cfg 7 (CFG_LEAN): as cfg 0 with the sweep kernels capped at 32 registers.
// cfg 8 / 9: as cfg 0 / 7 with an L2 prefetch of each warp's next group.
// cfg 10 / 11: every iteration in one launch of one thread-block cluster of
//   8 / 16 CTAs (k_level_cluster), for small units.
// cfg 12 / 13: as cfg 0 / 8 with the sweep directions swapped (dual sweep from
//   the chunk's end, primal from its start), so that each sweep meets the
//   neighbours it gathers right after visiting them.
// cfg 14 / 15: as cfg 0 / 12 in band order (all warps stride over the whole
//   unit together instead of each block owning a contiguous chunk).
// cfg 16 / 17: as cfg 14 / 15 with two cubes per thread and step (ILP 2).
// cfg 18: one fused launch per iteration over 256-cube tiles (k_fused);
//   in-memory and streaming semantics (OC semantics run cfg 14 instead).
// cfg 19: as 18 with the tiles' contiguous streams staged by TMA bulk copies
//   (k_fused_tma).
// cfg 22: every iteration in one launch of a single 1024-thread block
//   (k_level_cta), reading through L1, for units of up to 4096 cubes.
// cfg 23: as 22 with the unit's state, data term and neighbour indices held in
//   shared memory for the whole launch (k_level_smem), units of up to 2048 cubes.
// cfg 24: one thread-block cluster of 16 (else 8) CTAs whose shared memories
//   hold the unit's state, neighbours in other CTAs read through distributed
//   shared memory (k_level_dsm), units of up to 16 (8) x 2816 cubes.
// cfg 20 / 21: one ordered-wavefront launch per iteration (k_wave): each
//   block runs the dual then the primal step of a group of 512-cube tiles,
//   after the tiles the primal step depends on have published their dual
//   step; 20 reads through L2 only (ld.global.cg), 21 through L1 as well.
//   In-memory and streaming semantics, on levels whose forward dependencies
//   fit in small tile groups (OC semantics and other levels run 14).  Set by
//   tgvg_set_schedule only: the autotuner does not try them, as on GB300 the
//   tile hand-offs cost more than the traffic they save (largest three64
//   level: 152 us per iteration against 119 us for schedule 14).
static constexpr int TUNE_SEG = 16;
static constexpr int N_PERSIST_CFG = 6;
static constexpr int CFG_LEAN = 7;
static constexpr int CFG_PF = 8, CFG_LEAN_PF = 9;
static constexpr int CFG_SWAP = 12, CFG_SWAP_PF = 13, CFG_BAND = 14, CFG_BAND_SWAP = 15;
static constexpr int CFG_BAND_ILP = 16, CFG_BAND_SWAP_ILP = 17, CFG_FUSED = 18, CFG_FUSED_TMA = 19;
static constexpr int CFG_WAVE = 20, CFG_WAVE_L1 = 21, CFG_CTA = 22, CFG_SMEM = 23, CFG_DSM = 24;
static constexpr int CTA_MAX_N = 4096;  // the single-block schedule is a candidate up to this unit size
static inline bool fused_cfg(int cfg) { return cfg == CFG_FUSED || cfg == CFG_FUSED_TMA; }
static inline bool wave_cfg(int cfg) { return cfg == CFG_WAVE || cfg == CFG_WAVE_L1; }

// Host-side tables of the wavefront schedule for one level (ok: the groups
// that make every dependency point backwards are small, so the schedule is
// usable).
struct WaveSet {
    const int* doff; const int* dep; const int* gstart; int* flag; int* claim;
    int ntiles, ngroups, base;
    bool ok;
};
static constexpr int WAVE_MAX_GROUP = 8;  // tiles; larger groups leave too few blocks busy

// Host-side tables of the fused schedule for one level: the second (ping-pong)
// set of bars and p/q, the neighbour slots, the tiles' halos.
struct FuseSet {
    float4* barB; float4* P4B; float4* Q4B; float* Q1B;
    const int* slot; const int* halo; const int* hcount;
    int ntiles;
};
static inline bool per_launch_cfg(int cfg) {
    return cfg == 0 || cfg == CFG_LEAN || cfg == CFG_PF || cfg == CFG_LEAN_PF || (cfg >= CFG_SWAP && cfg <= CFG_BAND_SWAP_ILP);
}
static constexpr int CFG_CLUSTER8 = 10, CFG_CLUSTER16 = 11;
static constexpr int CLUSTER_MAX_N = 1 << 17;  // cluster schedules are candidates up to this unit size

// Largest usable cluster size of k_level_cluster for this mode / stop variant
// (16 when the device accepts non-portable clusters of 16 such CTAs, else 8, or
// 0 when not even 8 fit), cached in the context.
template <int MODE>
static int cluster_capacity(tgvg_ctx* ctx, bool stop, int* out) {
    int& c = ctx->cluster_max[MODE][stop ? 1 : 0];
    if (c < 0) {
        const void* k = stop ? (const void*)k_level_cluster<MODE, true> : (const void*)k_level_cluster<MODE, false>;
        c = 0;
        for (int cs : {16, 8}) {
            if (cs == 16 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(cs);
            cfg.blockDim = dim3(CLUSTER_BLOCK);
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = cs; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nc = 0;
            if (cudaOccupancyMaxActiveClusters(&nc, k, &cfg) == cudaSuccess && nc > 0) { c = cs; break; }
            cudaGetLastError();
        }
    }
    *out = c;
    return TGVG_OK;
}

static int persist_grid(int n, int cfg, int cmax) {
    const int cpb = 256 << cfg;
    return std::max(1, std::min((n + cpb - 1) / cpb, cmax));
}

template <int MODE>
static int coop_capacity(tgvg_ctx* ctx, bool stop, int* out) {
    int& cmax = ctx->coop_max[MODE][stop ? 1 : 0];
    if (cmax <= 0) {
        int per = 0;
        cudaError_t e = stop ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_level_persistent<MODE, true>,
                                                                            ITER_BLOCK, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_level_persistent<MODE, false>,
                                                                            ITER_BLOCK, 0);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "occupancy query");
        cmax = std::max(1, per) * ctx->sm_count;
    }
    *out = cmax;
    return TGVG_OK;
}

// An event record: inside a stream capture it becomes an event record node of
// the graph (so graph replays are timed too); outside, a plain record.
static cudaError_t record_event(cudaEvent_t e, cudaStream_t s, bool capturing) {
    return capturing ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s);
}

// Per-launch timing samples every TIMING_STRIDE-th iteration of the timed level.
static constexpr int TIMING_STRIDE = 10;

// Blocks per SM of the fused kernels (tma: the staged variant, which also gets
// its dynamic shared memory limit raised here, before any stream capture).
template <int MODE>
static int fused_occupancy(tgvg_ctx* ctx, bool tma, int* out) {
    int& o = ctx->fused_occ[MODE][tma ? 1 : 0];
    if (o <= 0) {
        int v = 0;
        cudaError_t e;
        if (tma) {
            e = cudaSuccess;
            const void* ks[] = {(const void*)k_fused_tma<MODE, false, false>, (const void*)k_fused_tma<MODE, true, false>,
                                (const void*)k_fused_tma<MODE, false, true>, (const void*)k_fused_tma<MODE, true, true>};
            for (const void* k : ks)
                if (e == cudaSuccess)
                    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FUSED_TMA_SMEM);
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_fused_tma<MODE, false, false>, FT,
                                                                  FUSED_TMA_SMEM);
        } else {
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_fused<MODE, false, false>, FT, 0);
        }
        if (e != cudaSuccess) return ctx->cuda_fail(e, "occupancy query");
        o = std::max(1, v);
    }
    *out = o;
    return TGVG_OK;
}

// The schedule a unit really runs: the fused and wavefront schedules need their
// tables (in-memory and streaming semantics; for the wavefront, a level whose
// dependencies all point backwards), else band order.
template <int MODE>
static int effective_cfg(const tgvg_ctx* ctx, int cfg, int n) {
    const WaveSet* wz = static_cast<const WaveSet*>(ctx->wave_cur);
    if (fused_cfg(cfg) && (MODE == M_OC || !ctx->fuse_cur)) return CFG_BAND;
    if (wave_cfg(cfg) && (MODE == M_OC || !wz || !wz->ok)) return CFG_BAND;
    if (cfg == CFG_SMEM && n > SMEM_MAX_N) return CFG_CTA;
    if (cfg == CFG_DSM) {  // the cluster size is known once dsm_capacity ran (plan and tuning call it)
        const int cs = ctx->dsm_max[MODE];
        if (cs >= 0 && (cs == 0 || n > cs * DSM_MAX_CHUNK)) return CFG_BAND;
    }
    return cfg;
}

// Shared-memory limit of the tiny-level kernel, raised once (before any capture).
template <int MODE>
static int smem_level_setup(tgvg_ctx* ctx) {
    if (ctx->smem_level_ready[MODE]) return TGVG_OK;
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) != cudaSuccess)
        return ctx->cuda_fail(cudaGetLastError(), "shared memory opt-in limit");
    // the unit's arrays at the largest unit size, plus what is left for staged values
    const int bytes = std::max((int)smem_ghost_offset(SMEM_MAX_N), optin - 1024);
    ctx->smem_level_max = bytes;
    cudaError_t e = cudaFuncSetAttribute((const void*)k_level_smem<MODE, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void*)k_level_smem<MODE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 bytes);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "shared memory limit");
    ctx->smem_level_ready[MODE] = true;
    return TGVG_OK;
}

// Cluster size of the distributed-shared-memory kernel (16 when the device
// runs such clusters with the full shared-memory carve-out, else 8, else 0),
// with the kernel's attributes set; cached in the context.
template <int MODE>
static int dsm_capacity(tgvg_ctx* ctx, int* out) {
    int& c = ctx->dsm_max[MODE];
    if (c < 0) {
        c = 0;
        const int bytes = (int)dsm_level_bytes(DSM_MAX_CHUNK);
        const void* ks[2] = {(const void*)k_level_dsm<MODE, false>, (const void*)k_level_dsm<MODE, true>};
        bool ok = true;
        for (const void* k : ks)
            ok = ok && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
        } else {
            for (int cs : {16, 8}) {
                bool allowed = true;
                if (cs == 16)
                    for (const void* k : ks)
                        allowed = allowed &&
                                  cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
                if (!allowed) { cudaGetLastError(); continue; }
                bool fits = true;
                for (const void* k : ks) {
                    cudaLaunchConfig_t lc = {};
                    lc.gridDim = dim3(cs);
                    lc.blockDim = dim3(CLUSTER_BLOCK);
                    lc.dynamicSmemBytes = (size_t)bytes;
                    cudaLaunchAttribute at[1];
                    at[0].id = cudaLaunchAttributeClusterDimension;
                    at[0].val.clusterDim.x = cs; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
                    lc.attrs = at;
                    lc.numAttrs = 1;
                    int nc = 0;
                    fits = fits && cudaOccupancyMaxActiveClusters(&nc, k, &lc) == cudaSuccess && nc > 0;
                }
                if (fits) { c = cs; break; }
                cudaGetLastError();
            }
        }
    }
    *out = c;
    return TGVG_OK;
}

// Blocks per SM of the wavefront kernel.
template <int MODE>
static int wave_occupancy(tgvg_ctx* ctx, bool l1, int* out) {
    int& o = ctx->wave_occ[MODE][l1 ? 1 : 0];
    if (o <= 0) {
        int v = 0;
        // the smallest over the variants (blocks claim work, so any grid is safe;
        // this one fills the GPU once)
        int u = 0;
        cudaError_t e = l1 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_wave<MODE, true, true, false>, WAVE_BLOCK, 0)
                           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_wave<MODE, true, true, true>, WAVE_BLOCK, 0);
        if (e == cudaSuccess)
            e = l1 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&u, k_wave<MODE, false, false, false>, WAVE_BLOCK, 0)
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&u, k_wave<MODE, false, false, true>, WAVE_BLOCK, 0);
        v = std::min(v, u);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "occupancy query");
        o = std::max(1, v);
    }
    *out = o;
    return TGVG_OK;
}

template <int MODE>
static int run_segment(tgvg_ctx* ctx, IterArgs a, int cfg, int it0, int count, bool stop, bool timed) {
    if (count <= 0) return TGVG_OK;
    const FuseSet* fz = static_cast<const FuseSet*>(ctx->fuse_cur);
    const WaveSet* wz = static_cast<const WaveSet*>(ctx->wave_cur);
    cfg = effective_cfg<MODE>(ctx, cfg, a.n);
    if (wave_cfg(cfg)) {
        const bool l1 = cfg == CFG_WAVE_L1;
        int occ = 0, rc = wave_occupancy<MODE>(ctx, l1, &occ);
        if (rc) return rc;
        const unsigned grid = (unsigned)std::max(1, std::min(wz->ngroups, occ * ctx->sm_count));
        // fresh flags and counters for this run of consecutive epochs
        TGVG_CK(ctx, cudaMemsetAsync(wz->flag, 0, 4ull * std::max(1, wz->ntiles), ctx->stream));
        TGVG_CK(ctx, cudaMemsetAsync(wz->claim, 0, 8, ctx->stream));
        for (int it = it0; it < it0 + count; ++it) {
            const bool res = stop && ((it + 1) % a.check_every == 0 || it + 1 == a.iters_total);
            WaveArgs w{wz->doff, wz->dep, wz->gstart, wz->flag, wz->claim, wz->ngroups, wz->base, it - it0 + 1};
            const bool mark = timed && it % TIMING_STRIDE == 0;
            cudaEvent_t* te = mark ? &ctx->tev[3 * (it / TIMING_STRIDE)] : nullptr;
            if (mark) TGVG_CK(ctx, record_event(te[0], ctx->stream, ctx->capturing));
#define TGVG_WAVE(CGV)                                                                                  \
    if (res && stop) k_wave<MODE, true, true, CGV><<<grid, WAVE_BLOCK, 0, ctx->stream>>>(a, w);         \
    else if (res) k_wave<MODE, true, false, CGV><<<grid, WAVE_BLOCK, 0, ctx->stream>>>(a, w);           \
    else if (stop) k_wave<MODE, false, true, CGV><<<grid, WAVE_BLOCK, 0, ctx->stream>>>(a, w);          \
    else k_wave<MODE, false, false, CGV><<<grid, WAVE_BLOCK, 0, ctx->stream>>>(a, w);
            if (l1) { TGVG_WAVE(false) } else { TGVG_WAVE(true) }
#undef TGVG_WAVE
            TGVG_LAUNCHED(ctx);
            if (mark) {
                TGVG_CK(ctx, record_event(te[1], ctx->stream, ctx->capturing));
                TGVG_CK(ctx, record_event(te[2], ctx->stream, ctx->capturing));
            }
            if (res) {
                const int ns = unit_slots<MODE>(a.nslot);
                launch_pdl(k_check, blocks_for(ns, 128), 128, ctx->stream, a.slot0, ns, a.acc, a.done, a.tol, it,
                           a.iters_run, a.resid);
                TGVG_LAUNCHED(ctx);
            }
        }
        return TGVG_OK;
    }
    if (fused_cfg(cfg)) {
        const bool tma = cfg == CFG_FUSED_TMA;
        int occ = 0, rc = fused_occupancy<MODE>(ctx, tma, &occ);
        if (rc) return rc;
        const unsigned grid = (unsigned)std::max(1, std::min(fz->ntiles, occ * ctx->sm_count));
        for (int it = it0; it < it0 + count; ++it) {
            const bool res = stop && ((it + 1) % a.check_every == 0 || it + 1 == a.iters_total);
            const bool odd = ((it - it0) & 1) != 0;
            FuseArgs f;
            f.bar_r = odd ? fz->barB : a.bar; f.bar_w = odd ? a.bar : fz->barB;
            f.P4_r = odd ? fz->P4B : a.P4;   f.P4_w = odd ? a.P4 : fz->P4B;
            f.Q4_r = odd ? fz->Q4B : a.Q4;   f.Q4_w = odd ? a.Q4 : fz->Q4B;
            f.Q1_r = odd ? fz->Q1B : a.Q1;   f.Q1_w = odd ? a.Q1 : fz->Q1B;
            f.slot = fz->slot; f.halo = fz->halo; f.hcount = fz->hcount; f.ntiles = fz->ntiles;
            const bool mark = timed && it % TIMING_STRIDE == 0;
            cudaEvent_t* te = mark ? &ctx->tev[3 * (it / TIMING_STRIDE)] : nullptr;
            if (mark) TGVG_CK(ctx, record_event(te[0], ctx->stream, ctx->capturing));
            const size_t sh = tma ? FUSED_TMA_SMEM : 0;
            void (*k)(IterArgs, FuseArgs);
            if (tma) k = res && stop ? k_fused_tma<MODE, true, true> : res ? k_fused_tma<MODE, true, false>
                         : stop ? k_fused_tma<MODE, false, true> : k_fused_tma<MODE, false, false>;
            else k = res && stop ? k_fused<MODE, true, true> : res ? k_fused<MODE, true, false>
                     : stop ? k_fused<MODE, false, true> : k_fused<MODE, false, false>;
            launch_pdl_smem(k, grid, FT, sh, ctx->stream, a, f);
            TGVG_LAUNCHED(ctx);
            if (mark) {
                TGVG_CK(ctx, record_event(te[1], ctx->stream, ctx->capturing));
                TGVG_CK(ctx, record_event(te[2], ctx->stream, ctx->capturing));
            }
            if (res) {
                const int ns = unit_slots<MODE>(a.nslot);
                launch_pdl(k_check, blocks_for(ns, 128), 128, ctx->stream, a.slot0, ns, a.acc, a.done, a.tol, it,
                           a.iters_run, a.resid);
                TGVG_LAUNCHED(ctx);
            }
        }
        k_fuse_settle<<<blocks_for(a.n, 256), 256, 0, ctx->stream>>>(a.o, a.n, it0, count, a.slot0, a.lid, a.iters_run,
                                                                      MODE, fz->barB, fz->P4B, fz->Q4B, fz->Q1B,
                                                                      a.bar, a.P4, a.Q4, a.Q1);
        TGVG_LAUNCHED(ctx);
        return TGVG_OK;
    }
    if (per_launch_cfg(cfg)) {
        const bool lean = cfg == CFG_LEAN || cfg == CFG_LEAN_PF;
        a.pf = (cfg == CFG_PF || cfg == CFG_LEAN_PF || cfg == CFG_SWAP_PF) ? 1 : 0;
        a.swap = (cfg == CFG_SWAP || cfg == CFG_SWAP_PF || cfg == CFG_BAND_SWAP || cfg == CFG_BAND_SWAP_ILP) ? 1 : 0;
        a.band = (cfg >= CFG_BAND && cfg <= CFG_BAND_SWAP_ILP) ? 1 : 0;
        const bool ilp2 = cfg == CFG_BAND_ILP || cfg == CFG_BAND_SWAP_ILP;
        int rc = iter_occupancy<MODE>(ctx);
        if (rc) return rc;
        for (int it = it0; it < it0 + count; ++it) {
            const bool res = stop && ((it + 1) % a.check_every == 0 || it + 1 == a.iters_total);
            const bool mark = timed && it % TIMING_STRIDE == 0;
            cudaEvent_t* te = mark ? &ctx->tev[3 * (it / TIMING_STRIDE)] : nullptr;
            if (mark) TGVG_CK(ctx, record_event(te[0], ctx->stream, ctx->capturing));
            launch_iter<MODE>(ctx, a, res, stop, true, lean, ilp2);
            if (mark) TGVG_CK(ctx, record_event(te[1], ctx->stream, ctx->capturing));
            launch_iter<MODE>(ctx, a, res, stop, false, lean, ilp2);
            if (mark) TGVG_CK(ctx, record_event(te[2], ctx->stream, ctx->capturing));
            cudaError_t le = cudaGetLastError();
            if (le != cudaSuccess) return ctx->cuda_fail(le, "iteration launch");
            ctx->kernels += 2;
            if (res) {
                const int ns = unit_slots<MODE>(a.nslot);
                launch_pdl(k_check, blocks_for(ns, 128), 128, ctx->stream, a.slot0, ns, a.acc, a.done, a.tol, it,
                           a.iters_run, a.resid);
                TGVG_LAUNCHED(ctx);
            }
        }
        return TGVG_OK;
    }
    if (cfg == CFG_DSM) {
        int cs = 0;
        const int rc = dsm_capacity<MODE>(ctx, &cs);
        if (rc) return rc;
        if (cs == 0 || a.n > cs * DSM_MAX_CHUNK) {
            cfg = CFG_BAND;  // does not fit: band order
        } else {
            a.chunk = (a.n + cs - 1) / cs;
            a.it0 = it0;
            a.iters = count;
            cudaLaunchConfig_t lc = {};
            lc.gridDim = dim3(cs);
            lc.blockDim = dim3(CLUSTER_BLOCK);
            lc.dynamicSmemBytes = dsm_level_bytes(a.chunk);
            lc.stream = ctx->stream;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = cs; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
            lc.attrs = at;
            lc.numAttrs = 1;
            cudaError_t e = stop ? cudaLaunchKernelEx(&lc, k_level_dsm<MODE, true>, a)
                                 : cudaLaunchKernelEx(&lc, k_level_dsm<MODE, false>, a);
            if (e != cudaSuccess) return ctx->cuda_fail(e, "cluster launch");
            ++ctx->kernels;
            return TGVG_OK;
        }
    }
    if (cfg == CFG_SMEM && a.n > SMEM_MAX_N) cfg = CFG_CTA;
    if (cfg == CFG_SMEM) {
        const int rc = smem_level_setup<MODE>(ctx);
        if (rc) return rc;
        a.it0 = it0;
        a.iters = count;
        const size_t base = smem_ghost_offset(a.n);
        const size_t sh = std::min((size_t)ctx->smem_level_max, base + size_t(16) * 6 * a.n);
        a.gcap = (int)((sh - base) / 16);
        if (stop) k_level_smem<MODE, true><<<1, CLUSTER_BLOCK, sh, ctx->stream>>>(a);
        else k_level_smem<MODE, false><<<1, CLUSTER_BLOCK, sh, ctx->stream>>>(a);
        TGVG_LAUNCHED(ctx);
        return TGVG_OK;
    }
    if (cfg == CFG_CTA) {
        a.chunk = a.n;
        a.it0 = it0;
        a.iters = count;
        a.pf = a.swap = a.band = 0;
        if (stop) k_level_cta<MODE, true><<<1, CLUSTER_BLOCK, 0, ctx->stream>>>(a);
        else k_level_cta<MODE, false><<<1, CLUSTER_BLOCK, 0, ctx->stream>>>(a);
        TGVG_LAUNCHED(ctx);
        return TGVG_OK;
    }
    if (cfg == CFG_CLUSTER8 || cfg == CFG_CLUSTER16) {
        const int cs = cfg == CFG_CLUSTER16 ? 16 : 8;
        int cmax = 0;
        const int rc = cluster_capacity<MODE>(ctx, stop, &cmax);  // also opts the kernel in to 16-CTA clusters
        if (rc) return rc;
        if (cs > cmax) return ctx->fail(TGVG_ERR_INVALID, "thread-block cluster size not supported by the device");
        a.chunk = ((a.n + cs - 1) / cs + 31) / 32 * 32;
        a.it0 = it0;
        a.iters = count;
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(cs);
        lc.blockDim = dim3(CLUSTER_BLOCK);
        lc.stream = ctx->stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs; at[0].val.clusterDim.y = 1; at[0].val.clusterDim.z = 1;
        lc.attrs = at;
        lc.numAttrs = 1;
        cudaError_t e = stop ? cudaLaunchKernelEx(&lc, k_level_cluster<MODE, true>, a)
                             : cudaLaunchKernelEx(&lc, k_level_cluster<MODE, false>, a);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "cluster launch");
        ++ctx->kernels;
        return TGVG_OK;
    }
    int cmax = 0, rc = coop_capacity<MODE>(ctx, stop, &cmax);
    if (rc) return rc;
    const int G = persist_grid(a.n, cfg, cmax);
    a.chunk = ((a.n + G - 1) / G + 31) / 32 * 32;
    const unsigned grid = (unsigned)((a.n + a.chunk - 1) / a.chunk);
    a.it0 = it0;
    a.iters = count;
    TGVG_CK(ctx, cudaMemsetAsync(a.bar_count, 0, sizeof(unsigned), ctx->stream));
    void* args[] = {&a};
    cudaError_t e = stop ? cudaLaunchCooperativeKernel((const void*)k_level_persistent<MODE, true>, dim3(grid),
                                                       dim3(ITER_BLOCK), args, 0, ctx->stream)
                         : cudaLaunchCooperativeKernel((const void*)k_level_persistent<MODE, false>, dim3(grid),
                                                       dim3(ITER_BLOCK), args, 0, ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "cooperative launch");
    ++ctx->kernels;
    return TGVG_OK;
}

// Candidate schedules the autotuner times for a unit of n cubes: the two
// per-iteration-launch variants and every persistent cfg whose grid differs.
template <int MODE>
static int tune_candidates(tgvg_ctx* ctx, int n, bool stop, std::vector<int>& cands) {
    int cmax = 0, rc = coop_capacity<MODE>(ctx, stop, &cmax);
    if (rc) return rc;
    cands = {0, CFG_LEAN, CFG_PF, CFG_LEAN_PF, CFG_SWAP, CFG_SWAP_PF, CFG_BAND, CFG_BAND_SWAP, CFG_BAND_ILP,
             CFG_BAND_SWAP_ILP};
    int last_grid = -1;
    if (n <= (1 << 22))
        for (int k = 1; k <= N_PERSIST_CFG; ++k) {
            const int g = persist_grid(n, k, cmax);
            if (g != last_grid) cands.push_back(k);
            last_grid = g;
        }
    if (n <= CTA_MAX_N) cands.push_back(CFG_CTA);
    if (n <= SMEM_MAX_N) {
        if ((rc = smem_level_setup<MODE>(ctx))) return rc;
        cands.push_back(CFG_SMEM);
    }
    if (n <= 16 * DSM_MAX_CHUNK) {
        int cs = 0;
        if ((rc = dsm_capacity<MODE>(ctx, &cs))) return rc;
        if (cs > 0 && n <= cs * DSM_MAX_CHUNK) cands.push_back(CFG_DSM);
    }
    if (n <= CLUSTER_MAX_N) {
        int cs = 0;
        if ((rc = cluster_capacity<MODE>(ctx, stop, &cs))) return rc;
        if (cs >= 8) cands.push_back(CFG_CLUSTER8);
        if (cs >= 16) cands.push_back(CFG_CLUSTER16);
    }
    if (MODE != M_OC && ctx->fuse_cur) {
        cands.push_back(CFG_FUSED);
        if (!ctx->paged_now) cands.push_back(CFG_FUSED_TMA);  // bulk copies stay on device-resident state
    }
    return TGVG_OK;
}

// The schedule a unit of n cubes runs with, or -1 when the online autotuner
// will first time the candidates on it.  The schedule for the unit's size
// class (floor(log2 n)) is taken from the context's table; the first time a
// class is met in a fixed-count solve with enough iterations, its first
// segments try each candidate for TUNE_SEG iterations and keep the fastest
// (the tried iterations count toward the solve).  Also makes sure the
// occupancy figures the launches need are cached.
template <int MODE>
static int plan_schedule(tgvg_ctx* ctx, int n, int iters, bool stop, bool timed, int* cfg) {
    int rc = iter_occupancy<MODE>(ctx), cmax = 0;
    if (!rc) rc = coop_capacity<MODE>(ctx, stop, &cmax);
    if (rc) return rc;
    int tuned = ctx->tune[MODE][31 - __builtin_clz((unsigned)std::max(1, n))];
    if (tuned == CFG_FUSED_TMA && ctx->paged_now) tuned = CFG_FUSED;  // bulk copies stay on device-resident state
    if (timed) {  // per-launch event timing needs one of the per-sweep-launch or fused schedules
        *cfg = (per_launch_cfg(tuned) || ((fused_cfg(tuned) || wave_cfg(tuned)) && MODE != M_OC)) ? tuned : CFG_BAND;
        if (fused_cfg(*cfg)) {
            int occ = 0;
            return fused_occupancy<MODE>(ctx, *cfg == CFG_FUSED_TMA, &occ);
        }
        *cfg = effective_cfg<MODE>(ctx, *cfg, n);
        if (wave_cfg(*cfg)) {
            int occ = 0;
            return wave_occupancy<MODE>(ctx, *cfg == CFG_WAVE_L1, &occ);
        }
        return TGVG_OK;
    }
    if (tuned >= 0) {
        *cfg = tuned;
        if (tuned == CFG_CLUSTER8 || tuned == CFG_CLUSTER16) {  // set up before any stream capture
            int cs = 0;
            return cluster_capacity<MODE>(ctx, stop, &cs);
        }
        if (tuned == CFG_SMEM) {
            *cfg = effective_cfg<MODE>(ctx, tuned, n);
            return smem_level_setup<MODE>(ctx);
        }
        if (tuned == CFG_DSM) {
            int cs = 0;
            rc = dsm_capacity<MODE>(ctx, &cs);
            *cfg = effective_cfg<MODE>(ctx, tuned, n);
            return rc;
        }
        if (fused_cfg(tuned)) {
            if (MODE == M_OC) *cfg = CFG_BAND;
            int occ = 0;
            return fused_occupancy<MODE>(ctx, tuned == CFG_FUSED_TMA, &occ);
        }
        if (wave_cfg(tuned)) {
            *cfg = effective_cfg<MODE>(ctx, tuned, n);
            int occ = 0;
            return wave_cfg(*cfg) ? wave_occupancy<MODE>(ctx, tuned == CFG_WAVE_L1, &occ) : TGVG_OK;
        }
        return TGVG_OK;
    }
    std::vector<int> cands;
    if ((rc = tune_candidates<MODE>(ctx, n, stop, cands))) return rc;
    // Tune when the trials are at most half the iterations: fixed-count solves,
    // and tolerance-stopped solves with a large cap (a unit that meets its
    // tolerance during the trials ends there without recording a pick).
    if ((int)cands.size() * TUNE_SEG * 2 <= iters) { *cfg = -1; return TGVG_OK; }
    // Untuned default (a tolerance-stopped solve, or too few iterations to
    // tune), after the autotuner's picks on the benchmark octrees: the unit's
    // state held on chip by one block (small units) or one cluster of 16 CTAs
    // (mid-size units), else band order.  Each is a single launch for all of
    // the unit's iterations or one launch per sweep, with no grid-wide barrier.
    *cfg = CFG_BAND;
    if (n <= SMEM_MAX_N) {
        if ((rc = smem_level_setup<MODE>(ctx))) return rc;
        *cfg = effective_cfg<MODE>(ctx, CFG_SMEM, n);
    } else if (n <= CTA_MAX_N) {
        *cfg = CFG_CTA;
    } else if (n <= 8192) {  // one cluster covers 16 SMs: beyond this per-sweep launches are faster
        int cs = 0;
        if ((rc = cluster_capacity<MODE>(ctx, stop, &cs))) return rc;
        if (cs >= 16) *cfg = CFG_CLUSTER16;
        else if (cs >= 8) *cfg = CFG_CLUSTER8;
    }
    return TGVG_OK;
}

// Run `iters` iterations of one unit with schedule `cfg` (-1: autotune first).
template <int MODE>
static int run_unit_t(tgvg_ctx* ctx, IterArgs& a, int iters, bool stop, bool timed, int cfg, int* used) {
    int it = 0, rc;
    if (cfg < 0) {
        std::vector<int> cands;
        if ((rc = tune_candidates<MODE>(ctx, a.n, stop, cands))) return rc;
        float best_ms = 1e30f;
        int best = 0;
        const int ns = unit_slots<MODE>(a.nslot);
        std::vector<int> done_h(stop ? ns : 0);
        for (int c : cands) {
            TGVG_CK(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
            if ((rc = run_segment<MODE>(ctx, a, c, it, TUNE_SEG, stop, false))) return rc;
            TGVG_CK(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
            TGVG_CK(ctx, cudaEventSynchronize(ctx->ev[3]));
            it += TUNE_SEG;
            if (stop) {
                // A unit that met its tolerance during the trials is finished.  Its
                // last segment stopped early and is not compared; the class keeps the
                // fastest complete trial (or this candidate when there is none), so
                // that later units of the class do not pay for the trials again.
                TGVG_CK(ctx, cudaMemcpy(done_h.data(), a.done + a.slot0, sizeof(int) * ns, cudaMemcpyDeviceToHost));
                bool all = true;
                for (int d : done_h) all = all && d != 0;
                if (all) {
                    ctx->tune[MODE][31 - __builtin_clz((unsigned)std::max(1, a.n))] = best_ms < 1e30f ? best : c;
                    *used = effective_cfg<MODE>(ctx, c, a.n);
                    return TGVG_OK;
                }
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
            if (ms < best_ms) { best_ms = ms; best = c; }
        }
        ctx->tune[MODE][31 - __builtin_clz((unsigned)std::max(1, a.n))] = best;
        cfg = best;
    }
    if (cfg == CFG_DSM) {
        int cs = 0;
        if ((rc = dsm_capacity<MODE>(ctx, &cs))) return rc;
    }
    *used = effective_cfg<MODE>(ctx, cfg, a.n);
    const int eff = *used;
    if (!stop || ctx->capturing || !(per_launch_cfg(eff) || fused_cfg(eff) || wave_cfg(eff)))
        return run_segment<MODE>(ctx, a, cfg, it, iters - it, stop, timed);
    // A tolerance-stopped unit on a schedule with launches per iteration: its
    // launches after convergence would return at once but still cost a launch
    // each (at a 6000-iteration cap, about 20 ms).  So the iterations are
    // enqueued in chunks of growing length, and each chunk's stopping flags are
    // copied back while the next chunk runs; once they show the unit finished,
    // nothing more is enqueued.  At most one chunk runs after convergence.
    const int ns = unit_slots<MODE>(a.nslot);
    if (ctx->chk_cap < ns) {
        if (ctx->chk_host) cudaFreeHost(ctx->chk_host);
        ctx->chk_host = nullptr;
        ctx->chk_cap = 0;
        TGVG_CK(ctx, cudaHostAlloc((void**)&ctx->chk_host, sizeof(int) * 2 * ns, cudaHostAllocDefault));
        ctx->chk_cap = ns;
    }
    int seg = 64;
    for (int k = 0; it < iters; ++k) {
        const int cnt = std::min(seg, iters - it);
        if ((rc = run_segment<MODE>(ctx, a, cfg, it, cnt, stop, timed))) return rc;
        it += cnt;
        int* h = ctx->chk_host + (k & 1) * ns;
        TGVG_CK(ctx, cudaMemcpyAsync(h, a.done + a.slot0, sizeof(int) * ns, cudaMemcpyDeviceToHost, ctx->stream));
        TGVG_CK(ctx, cudaEventRecord(ctx->chk_ev[k & 1], ctx->stream));
        if (k > 0) {
            TGVG_CK(ctx, cudaEventSynchronize(ctx->chk_ev[(k - 1) & 1]));
            const int* hp = ctx->chk_host + ((k - 1) & 1) * ns;
            bool all = true;
            for (int s = 0; s < ns && all; ++s) all = hp[s] != 0;
            if (all) break;
        }
        seg = std::min(seg * 2, 1024);
    }
    return TGVG_OK;
}

static int plan_unit(tgvg_ctx* ctx, int mode, int n, int iters, bool stop, bool timed, int* cfg) {
    if (mode == M_INMEM) return plan_schedule<M_INMEM>(ctx, n, iters, stop, timed, cfg);
    if (mode == M_OC) return plan_schedule<M_OC>(ctx, n, iters, stop, timed, cfg);
    return plan_schedule<M_STREAM>(ctx, n, iters, stop, timed, cfg);
}

static int run_unit(tgvg_ctx* ctx, int mode, IterArgs& a, int iters, bool stop, bool timed, int cfg, int* used) {
    if (mode == M_INMEM) return run_unit_t<M_INMEM>(ctx, a, iters, stop, timed, cfg, used);
    if (mode == M_OC) return run_unit_t<M_OC>(ctx, a, iters, stop, timed, cfg, used);
    return run_unit_t<M_STREAM>(ctx, a, iters, stop, timed, cfg, used);
}

__global__ void k_fill_i32(int n, int* __restrict__ p, int v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// Wavefront tables of every level of a solve: per level, the dependency pairs
// of its tiles, sorted and made unique, as per-tile lists (doff / dep); the
// groups of consecutive tiles that contain every forward dependency (gstart);
// and whether those groups are small enough for the schedule (ok).  Levels are
// processed one at a time on scratch sized for the largest; the lists of all
// levels share one array.
static int build_wave_tables(tgvg_ctx* ctx, int mode, int min_d, int max_d, const int* h_bstart,
                             int npos, const int* nb, std::vector<WaveSet>& ws) {
    auto B = [&](int id, size_t b) { return ctx->buf(id, b); };
    cudaStream_t st = ctx->stream;
    const int nl = max_d - min_d + 1;
    int64_t tiles_total = 0;
    int max_tiles = 1;
    std::vector<int> base(nl), ntiles(nl);
    std::vector<int64_t> toff(nl);
    for (int Ld = min_d; Ld <= max_d; ++Ld) {
        const int k = Ld - min_d, o = h_bstart[Ld], c = h_bstart[Ld + 1] - h_bstart[Ld];
        base[k] = o & ~31;
        ntiles[k] = c > 0 ? (o + c - base[k] + WT - 1) / WT : 0;
        max_tiles = std::max(max_tiles, ntiles[k]);
        toff[k] = tiles_total;
        tiles_total += ntiles[k];
    }
    auto* cnt = (int*)B(B_W_CNT, 4ull * (nl + 2));
    auto* reach = (int*)B(B_W_POS, 4ull * std::max<int64_t>(1, tiles_total));
    if (!cnt || !reach) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemsetAsync(cnt, 0, 4ull * (nl + 2), st));
    TGVG_CK(ctx, cudaMemsetAsync(reach, 0xff, 4ull * std::max<int64_t>(1, tiles_total), st));
    for (int Ld = min_d; Ld <= max_d; ++Ld) {
        const int k = Ld - min_d, o = h_bstart[Ld], c = h_bstart[Ld + 1] - h_bstart[Ld];
        if (c <= 0) continue;
        if (mode == M_INMEM)
            k_wave_pairs<M_INMEM><<<blocks_for(c, 256), 256, 0, st>>>(o, c, base[k], npos, nb, nullptr, cnt + k,
                                                                    reach + toff[k]);
        else
            k_wave_pairs<M_STREAM><<<blocks_for(c, 256), 256, 0, st>>>(o, c, base[k], npos, nb, nullptr, cnt + k,
                                                                     reach + toff[k]);
        TGVG_LAUNCHED(ctx);
    }
    std::vector<int> h_cnt(nl), h_reach(size_t(std::max<int64_t>(1, tiles_total)));
    TGVG_CK(ctx, cudaMemcpyAsync(h_cnt.data(), cnt, 4ull * nl, cudaMemcpyDeviceToHost, st));
    TGVG_CK(ctx, cudaMemcpyAsync(h_reach.data(), reach, 4ull * h_reach.size(), cudaMemcpyDeviceToHost, st));
    TGVG_CK(ctx, cudaStreamSynchronize(st));
    // groups: extend each group until no tile in it depends on a tile after it
    std::vector<int> h_gstart;
    std::vector<int64_t> goff(nl);
    std::vector<int> ngroups(nl), maxg(nl, 0);
    for (int k = 0; k < nl; ++k) {
        goff[k] = (int64_t)h_gstart.size();
        int t = 0;
        while (t < ntiles[k]) {
            const int g0 = t;
            int end = t + 1;
            for (; t < end; ++t) end = std::max(end, h_reach[toff[k] + t] + 1);
            h_gstart.push_back(g0);
            maxg[k] = std::max(maxg[k], t - g0);
        }
        h_gstart.push_back(ntiles[k]);
        ngroups[k] = (int)(h_gstart.size() - goff[k]) - 1;
    }
    int64_t max_pairs = 1, dep_total = 1, off_total = 0;
    for (int k = 0; k < nl; ++k) {
        max_pairs = std::max<int64_t>(max_pairs, h_cnt[k]);
        dep_total += h_cnt[k];
        off_total += ntiles[k] + 1;
    }
    auto* keys = (unsigned long long*)B(B_W_KEYS, 8ull * max_pairs);
    auto* skeys = (unsigned long long*)B(B_W_SKEYS, 8ull * max_pairs);
    auto* keep = (int*)B(B_W_KEEP, 4ull * max_pairs);
    auto* kpos = (int*)B(B_W_TMP2, 4ull * max_pairs);
    auto* ukeys = (unsigned long long*)B(B_W_UKEYS, 8ull * max_pairs);
    auto* dep = (int*)B(B_W_DEP, 4ull * dep_total);
    auto* doff = (int*)B(B_W_DOFF, 4ull * std::max<int64_t>(1, off_total));
    auto* gst = (int*)B(B_W_GSTART, 4ull * h_gstart.size());
    auto* flag = (int*)B(B_W_FLAG, 4ull * max_tiles + 64);
    if (!keys || !skeys || !keep || !kpos || !ukeys || !dep || !doff || !gst || !flag) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemcpyAsync(gst, h_gstart.data(), 4ull * h_gstart.size(), cudaMemcpyHostToDevice, st));
    int64_t dep_at = 0, off_at = 0;
    for (int Ld = min_d; Ld <= max_d; ++Ld) {
        const int k = Ld - min_d, o = h_bstart[Ld], c = h_bstart[Ld + 1] - h_bstart[Ld];
        if (c <= 0) continue;
        WaveSet& w = ws[Ld];
        w = WaveSet{doff + off_at, dep + dep_at, gst + goff[k], flag, flag + max_tiles, ntiles[k], ngroups[k],
                    base[k], maxg[k] <= WAVE_MAX_GROUP};
        const int m = h_cnt[k];
        int nu = 0;
        if (w.ok && m > 0) {
            TGVG_CK(ctx, cudaMemsetAsync(cnt + nl, 0, 4, st));
            if (mode == M_INMEM)
                k_wave_pairs<M_INMEM><<<blocks_for(c, 256), 256, 0, st>>>(o, c, base[k], npos, nb, keys, cnt + nl,
                                                                        nullptr);
            else
                k_wave_pairs<M_STREAM><<<blocks_for(c, 256), 256, 0, st>>>(o, c, base[k], npos, nb, keys, cnt + nl,
                                                                         nullptr);
            TGVG_LAUNCHED(ctx);
            int bits = 1;
            while ((1 << bits) < ntiles[k] + 1) ++bits;
            size_t tb = 0;
            TGVG_CK(ctx, cub::DeviceRadixSort::SortKeys(nullptr, tb, keys, skeys, m, 0, 32 + bits, st));
            void* tmp = B(B_W_TMP, std::max<size_t>(tb, 16));
            if (!tmp) return TGVG_ERR_NOMEM;
            TGVG_CK(ctx, cub::DeviceRadixSort::SortKeys(tmp, tb, keys, skeys, m, 0, 32 + bits, st));
            k_wave_unique<<<blocks_for(m, 256), 256, 0, st>>>(m, skeys, keep);
            TGVG_LAUNCHED(ctx);
            int64_t nu64 = 0;
            int rc = scan_exclusive(ctx, keep, m, kpos, &nu64);
            if (rc) return rc;
            nu = (int)nu64;
            k_wave_compact<<<blocks_for(m, 256), 256, 0, st>>>(m, skeys, keep, kpos, ukeys, dep + dep_at);
            TGVG_LAUNCHED(ctx);
        }
        k_wave_offsets<<<blocks_for(ntiles[k] + 1, 256), 256, 0, st>>>(ntiles[k], nu, ukeys, doff + off_at);
        TGVG_LAUNCHED(ctx);
        dep_at += nu;
        off_at += ntiles[k] + 1;
    }
    return TGVG_OK;
}

int tgv_solve_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, const uint32_t* d_hists, int64_t n64,
                  int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, int32_t mode,
                  const tgvg_params* prm, const float* d_u_init, tgvg_state* d_out, tgvg_stats* stats,
                  const tgvg_state* d_state_init) {
    tgvg_stats st;
    std::memset(&st, 0, sizeof(st));
    const int64_t k0 = ctx->kernels;
    if (mode < 0 || mode > 2 || (nbins != 8 && nbins != 10) || !prm || n64 < 0 || n64 > POS_MASK)
        return TGVG_ERR_INVALID;
    if (prm->init < 0 || prm->init > TGVG_INIT_STATE || (prm->init == TGVG_INIT_GIVEN && n64 > 0 && !d_u_init) ||
        (prm->init == TGVG_INIT_STATE && n64 > 0 && !d_state_init))
        return TGVG_ERR_INVALID;
    const bool level_state = prm->init == TGVG_INIT_STATE;
    if (mode != M_INMEM && nleaf > 0 && !leaves) return TGVG_ERR_INVALID;
    const int n = (int)n64;
    if (n == 0) { if (stats) *stats = st; return TGVG_OK; }
    if (!d_cubes || !d_hists || !d_out) return TGVG_ERR_INVALID;

    // ---- leaves: clamp like load_cubes_range (octree_builder.cpp:131-135), sort, reject overlap
    std::vector<int> lf, ll;  // by caller index (empty leaf: first > last)
    if (mode == M_INMEM) {
        lf.assign(1, 0); ll.assign(1, n - 1);
    } else {
        lf.resize(std::max(0, nleaf)); ll.resize(std::max(0, nleaf));
        for (int l = 0; l < nleaf; ++l) {
            const uint32_t a = leaves[l].first_idx, b = leaves[l].last_idx;
            if (int64_t(a) >= n || a > b) { lf[l] = 1; ll[l] = 0; continue; }
            lf[l] = (int)a;
            ll[l] = (int)std::min<int64_t>(int64_t(b), n - 1);
        }
    }
    const int L = (int)lf.size();
    std::vector<int> order;
    for (int l = 0; l < L; ++l) if (lf[l] <= ll[l]) order.push_back(l);
    std::sort(order.begin(), order.end(), [&](int x, int y) { return lf[x] < lf[y]; });
    for (size_t k = 1; k < order.size(); ++k)
        if (lf[order[k]] <= ll[order[k - 1]]) return TGVG_ERR_OVERLAP;
    std::vector<int> s_first, s_last, s_id;
    for (int l : order) { s_first.push_back(lf[l]); s_last.push_back(ll[l]); s_id.push_back(l); }
    const int nsl = (int)s_first.size();
    const int nslot = std::max(1, L);

    cudaEvent_t e0 = ctx->ev[0], e1 = ctx->ev[1], e2 = ctx->ev[2];
    TGVG_CK(ctx, cudaEventRecord(e0, ctx->stream));

    // ---- buffers
    const int nblk = (n + SORT_BLOCK - 1) / SORT_BLOCK;
    uint64_t cap = 1024;
    while (cap < 2ull * (uint64_t)n) cap <<= 1;
    auto B = [&](int id, size_t bytes) { return ctx->buf(id, bytes); };
    auto* keys = (unsigned long long*)B(B_KEYS, 8ull * n);
    auto* depth = (int*)B(B_DEPTH, 4ull * n);
    auto* leaf_of = (int*)B(B_LEAFOF, 4ull * n);
    auto* counts = (int*)B(B_BCOUNT, 4ull * NBUCKET * nblk);
    auto* bstart = (int*)B(B_BTOT, 4ull * (NBUCKET + 1));
    auto* perm = (int*)B(B_PERM, 4ull * n);
    auto* inv = (int*)B(B_INV, 4ull * n);
    auto* hk = (unsigned long long*)B(B_HKEYS, 8ull * cap);
    auto* hmin = (int*)B(B_HMIN, 4ull * cap);
    auto* hmax = (int*)B(B_HMAX, 4ull * cap);
    auto* nb = (int*)B(B_NB, 4ull * 6 * n + 64);  // padded: staged slices round up to 16 B
    auto* par = (int*)B(B_PAR, 4ull * n);
    // Beyond the device budget the per-cube state (and its snapshot and second
    // set) lives in host memory and each level's slice is prefetched to the
    // device while the level runs; keys, hash and neighbour tables stay resident.
    const bool paged = state_paged(ctx, n64);
    ctx->paged_now = paged;
    auto SB = [&](int id, size_t bytes) { return paged ? ctx->host_backed(id, bytes) : ctx->buf(id, bytes); };
    auto* uv = (float4*)SB(B_UV, 16ull * n);
    auto* bar = (float4*)SB(B_BAR, 16ull * n);
    auto* P4 = (float4*)SB(B_P4, 16ull * n);
    auto* Q4 = (float4*)SB(B_Q4, 16ull * n);
    auto* Q1 = (float*)SB(B_Q1, 4ull * n + 64);
    auto* dat = (float2*)B(B_DAT, 8ull * n + 64);
    auto* snap = (float4*)SB(B_SNAP, mode == M_INMEM ? 16 : 16ull * n);
    auto* lid = (int*)B(B_LID, 4ull * n);
    auto* lv = (int*)B(B_LEAVES, 4ull * (3 * std::max(1, nsl) + 2 * std::max(1, L)));
    auto* acc = (double*)B(B_ACC, 32ull * nslot);
    auto* flags = (int*)B(B_FLAGS, 4ull * (8 + 2 * nslot));
    auto* ranges = (int*)B(B_RANGES, 8ull * NBUCKET * std::max(1, L));
    auto* resid = (double*)B(B_RESID, 8ull * nslot);
    if (!keys || !depth || !leaf_of || !counts || !bstart || !perm || !inv || !hk || !hmin || !hmax ||
        !nb || !par || !uv || !bar || !P4 || !Q4 || !Q1 || !dat || !snap || !lid || !lv || !acc ||
        !flags || !ranges || !resid)
        return TGVG_ERR_NOMEM;
    int* d_sfirst = lv;
    int* d_slast = lv + std::max(1, nsl);
    int* d_sid = lv + 2 * std::max(1, nsl);
    int* d_lfirst = lv + 3 * std::max(1, nsl);
    int* d_llast = d_lfirst + std::max(1, L);
    int* done = flags + 8;
    int* iters_run = flags + 8 + nslot;

    std::vector<int> hostleaf(3 * std::max(1, nsl) + 2 * std::max(1, L), 0);
    for (int k = 0; k < nsl; ++k) {
        hostleaf[k] = s_first[k];
        hostleaf[std::max(1, nsl) + k] = s_last[k];
        hostleaf[2 * std::max(1, nsl) + k] = s_id[k];
    }
    for (int l = 0; l < L; ++l) {
        hostleaf[3 * std::max(1, nsl) + l] = lf[l];
        hostleaf[3 * std::max(1, nsl) + std::max(1, L) + l] = ll[l];
    }
    TGVG_CK(ctx, cudaMemcpyAsync(lv, hostleaf.data(), 4 * hostleaf.size(), cudaMemcpyHostToDevice, ctx->stream));
    // [0] unsorted [1] bad depth [2] min depth [3] max depth [4] barrier count [5] barrier
    // generation [6] bounded-wait timeout [7] unused
    const int init_flags[8] = {0, 0, 21, 0, 0, 0, 0, 0};
    TGVG_CK(ctx, cudaMemcpyAsync(flags, init_flags, sizeof(init_flags), cudaMemcpyHostToDevice, ctx->stream));

    // ---- K3: keys, leaves, level-major order, hash, neighbours
    k_prep<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, reinterpret_cast<const uint4*>(d_cubes), keys,
                                                         depth, flags);
    TGVG_LAUNCHED(ctx);
    k_leaf_of<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, nsl, d_sfirst, d_slast, d_sid, leaf_of);
    TGVG_LAUNCHED(ctx);
    k_bucket_count<<<nblk, SORT_BLOCK, 0, ctx->stream>>>(n, mode, depth, leaf_of, counts, nblk);
    TGVG_LAUNCHED(ctx);
    k_bucket_scan<<<1, SORT_BLOCK, 0, ctx->stream>>>(NBUCKET * nblk, counts, nblk, bstart);
    TGVG_LAUNCHED(ctx);
    k_bucket_scatter<<<nblk, SORT_BLOCK, 0, ctx->stream>>>(n, mode, depth, leaf_of, counts, nblk, perm, inv);
    TGVG_LAUNCHED(ctx);
    int h_flags[4], h_bstart[NBUCKET + 1];
    TGVG_CK(ctx, cudaMemcpyAsync(h_flags, flags, sizeof(h_flags), cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaMemcpyAsync(h_bstart, bstart, sizeof(h_bstart), cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaMemsetAsync(hk, 0xff, 8ull * cap, ctx->stream));
    TGVG_CK(ctx, cudaMemsetAsync(hmin, 0x7f, 4ull * cap, ctx->stream));
    TGVG_CK(ctx, cudaMemsetAsync(hmax, 0xff, 4ull * cap, ctx->stream));
    HashView hv{hk, hmin, hmax, cap - 1};
    k_hash_insert<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, keys, hv);
    TGVG_LAUNCHED(ctx);
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (h_flags[1]) return ctx->fail(TGVG_ERR_INVALID, "cube depth outside 0..21");
    if (mode == M_STREAM && h_flags[0])
        return ctx->fail(TGVG_ERR_UNSORTED, "streaming semantics need Morton-sorted cubes");
    const int min_d = h_flags[2], max_d = h_flags[3];
    const int n_act = h_bstart[22];

    if (n_act > 0) {
        if (mode == M_INMEM)
            k_neighbours<M_INMEM><<<blocks_for(n_act, 256), 256, 0, ctx->stream>>>(
                n_act, n, perm, inv, keys, depth, leaf_of, d_lfirst, d_llast, hv, n, nb, par);
        else if (mode == M_OC)
            k_neighbours<M_OC><<<blocks_for(n_act, 256), 256, 0, ctx->stream>>>(
                n_act, n, perm, inv, keys, depth, leaf_of, d_lfirst, d_llast, hv, n, nb, par);
        else
            k_neighbours<M_STREAM><<<blocks_for(n_act, 256), 256, 0, ctx->stream>>>(
                n_act, n, perm, inv, keys, depth, leaf_of, d_lfirst, d_llast, hv, n, nb, par);
        TGVG_LAUNCHED(ctx);
    }
    if (nbins == 8)
        k_init<8><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, perm, d_hists, prm->init, d_u_init, leaf_of,
                                                               uv, bar, P4, Q4, Q1, dat, lid);
    else
        k_init<10><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, perm, d_hists, prm->init, d_u_init, leaf_of,
                                                                uv, bar, P4, Q4, Q1, dat, lid);
    TGVG_LAUNCHED(ctx);
    std::vector<int> h_ranges;
    if (mode != M_INMEM && L > 0) {
        k_leaf_ranges<<<blocks_for(int64_t(L) * 22, 128), 128, 0, ctx->stream>>>(L, d_lfirst, d_llast, bstart,
                                                                                perm, ranges);
        TGVG_LAUNCHED(ctx);
        h_ranges.resize(2ull * NBUCKET * L);
        TGVG_CK(ctx, cudaMemcpyAsync(h_ranges.data(), ranges, 4 * h_ranges.size(), cudaMemcpyDeviceToHost,
                                     ctx->stream));
        TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    }
    // ---- fused-schedule tables, per level (in-memory and streaming semantics)
    std::vector<FuseSet> fsets(NBUCKET);
    bool fused_ok = false;
    const int fiters = std::max(0, prm->iters);
    if (mode != M_OC && fiters > 0 && n_act > 0) {
        int64_t total_tiles = 0;
        for (int Ld = min_d; Ld <= max_d; ++Ld) total_tiles += (h_bstart[Ld + 1] - h_bstart[Ld] + FT - 1) / FT;
        auto* barB = (float4*)SB(B_BARB, 16ull * n);
        auto* P4B = (float4*)SB(B_P4B, 16ull * n);
        auto* Q4B = (float4*)SB(B_Q4B, 16ull * n);
        auto* Q1B = (float*)SB(B_Q1B, 4ull * n + 64);
        auto* fslot = (int*)B(B_FSLOT, 12ull * n + 64);
        auto* fhalo = (int*)B(B_FHALO, 4ull * FH * std::max<int64_t>(1, total_tiles));
        auto* fhcnt = (int*)B(B_FHCNT, 4ull * std::max<int64_t>(1, total_tiles));
        if (!barB || !P4B || !Q4B || !Q1B || !fslot || !fhalo || !fhcnt) return TGVG_ERR_NOMEM;
        int64_t base = 0;
        for (int Ld = min_d; Ld <= max_d; ++Ld) {
            const int o = h_bstart[Ld], cnt = h_bstart[Ld + 1] - h_bstart[Ld];
            if (cnt <= 0) continue;
            const int tiles = (cnt + FT - 1) / FT;
            if (mode == M_INMEM)
                k_fuse_tiles<M_INMEM><<<tiles, FT, 0, ctx->stream>>>(o, cnt, n, nb, fslot, fhalo + base * FH, fhcnt + base);
            else
                k_fuse_tiles<M_STREAM><<<tiles, FT, 0, ctx->stream>>>(o, cnt, n, nb, fslot, fhalo + base * FH, fhcnt + base);
            TGVG_LAUNCHED(ctx);
            fsets[Ld] = FuseSet{barB, P4B, Q4B, Q1B, fslot, fhalo + base * FH, fhcnt + base, tiles};
            base += tiles;
        }
        fused_ok = true;
    }
    // ---- wavefront-schedule tables, per level (in-memory and streaming semantics)
    std::vector<WaveSet> wsets(NBUCKET, WaveSet{nullptr, nullptr, nullptr, nullptr, nullptr, 0, 0, 0, false});
    bool wave_wanted = false;  // only a schedule set by tgvg_set_schedule runs it
    for (int c : ctx->tune[mode]) wave_wanted |= wave_cfg(c);
    if (wave_wanted && mode != M_OC && fiters > 0 && n_act > 0) {
        const int rc = build_wave_tables(ctx, mode, min_d, max_d, h_bstart, n, nb, wsets);
        if (rc) return rc;
    }
    // the level being planned or run; cleared on every return
    struct FuseCur {
        tgvg_ctx* c;
        ~FuseCur() { c->fuse_cur = nullptr; c->wave_cur = nullptr; }
    } fuse_guard{ctx};
    auto set_fuse = [&](int Ld) {
        ctx->fuse_cur = fused_ok ? &fsets[Ld] : nullptr;
        ctx->wave_cur = wsets[Ld].doff ? &wsets[Ld] : nullptr;
    };
    TGVG_CK(ctx, cudaEventRecord(e1, ctx->stream));

    // ---- levels
    const bool stop = prm->tol > 0.0f && prm->check_every > 0;
    const int iters = std::max(0, prm->iters);
    st.min_depth = min_d;
    st.max_depth = max_d;
    // optional per-launch timing of the largest level (not for sequential OC leaves)
    int big_level = -1, t_level = -1;
    {
        int best = 0;
        for (int Ld = min_d; Ld <= max_d; ++Ld)
            if (h_bstart[Ld + 1] - h_bstart[Ld] > best) { best = h_bstart[Ld + 1] - h_bstart[Ld]; big_level = Ld; }
    }
    if (ctx->timing && mode != M_OC && iters > 0) {
        t_level = big_level;
        while ((int)ctx->tev.size() < 3 * ((iters + TIMING_STRIDE - 1) / TIMING_STRIDE)) {
            cudaEvent_t e;
            TGVG_CK(ctx, cudaEventCreate(&e));
            ctx->tev.push_back(e);
        }
    }
    // Plan: the levels, their launch units (INMEM / STREAM the whole level, OC
    // one per leaf in caller order) and each unit's schedule.
    struct Unit { int slot, o, n, cfg; };
    struct Level { int d, o, cnt; std::vector<Unit> us; };
    std::vector<Level> levels;
    bool tuning = false;
    for (int Ld = min_d; Ld <= max_d; ++Ld) {
        const int o = h_bstart[Ld], cnt = h_bstart[Ld + 1] - h_bstart[Ld];
        if (cnt <= 0) continue;
        Level lvl{Ld, o, cnt, {}};
        if (mode == M_OC) {
            for (int l = 0; l < L; ++l) {
                const int a0 = h_ranges[(l * NBUCKET + Ld) * 2], a1 = h_ranges[(l * NBUCKET + Ld) * 2 + 1];
                if (a1 > a0) lvl.us.push_back({l, a0, a1 - a0, 0});
            }
        } else {
            lvl.us.push_back({0, o, cnt, 0});
        }
        for (Unit& u : lvl.us) {
            set_fuse(Ld);
            const int rc = plan_unit(ctx, mode, u.n, iters, stop, Ld == t_level, &u.cfg);
            if (rc) return rc;
            tuning |= u.cfg < 0;
        }
        levels.push_back(std::move(lvl));
    }
    // coarser-neighbour ghost tables for levels run by the per-launch sweep
    // schedules (in-memory and streaming semantics, state on the device)
    int gmax = 0, dmax = 0;
    std::vector<char> dual_ghosts(levels.size(), 0);
    if (mode != M_OC && !paged)
        for (size_t k = 0; k < levels.size(); ++k) {
            const Level& lvl = levels[k];
            if (lvl.cnt < GHOST_MIN || lvl.cnt > GHOST_MAX) continue;
            gmax = std::max(gmax, lvl.cnt);
            if (lvl.cnt >= DUAL_GHOST_MIN && k + 1 < levels.size() && levels[k + 1].d == lvl.d + 1 &&
                levels[k + 1].cnt >= 2ll * lvl.cnt) {
                dual_ghosts[k] = 1;
                dmax = std::max(dmax, lvl.cnt);
            }
        }
    int *g_pnb = nullptr, *g_mark = nullptr, *g_ids = nullptr, *g_sums = nullptr, *g_dnb = nullptr;
    float4 *g_val = nullptr, *g_dval = nullptr;
    if (gmax > 0) {
        g_pnb = (int*)B(B_G_PNB, 12ull * gmax);
        g_val = (float4*)B(B_G_VAL, 48ull * gmax);
        g_mark = (int*)B(B_G_MARK, 12ull * gmax);
        g_ids = (int*)B(B_G_IDS, 12ull * gmax);
        g_sums = (int*)B(B_G_SUMS, 4ull * scan_sums_len(3ll * gmax));
        if (!g_pnb || !g_val || !g_mark || !g_ids || !g_sums) return TGVG_ERR_NOMEM;
        if (dmax > 0) {
            g_dnb = (int*)B(B_G_DNB, 12ull * dmax);
            g_dval = (float4*)B(B_G_DVAL, 48ull * dmax);
            if (!g_dnb || !g_dval) return TGVG_ERR_NOMEM;
        }
    }
    const int nlv = std::min<int>((int)levels.size(), TGVG_MAX_LEVELS);
    double* lv_res = nullptr;
    int* lv_it = nullptr;
    if (stop) {
        auto* lvstat = (double*)B(B_LVSTAT, 12ull * TGVG_MAX_LEVELS * nslot);
        if (!lvstat) return TGVG_ERR_NOMEM;
        lv_res = lvstat;
        lv_it = reinterpret_cast<int*>(lvstat + TGVG_MAX_LEVELS * nslot);
    }
    std::vector<int> used(nlv, -1);
    auto* lv_en = (double*)B(B_LVENERGY, 8ull * TGVG_MAX_LEVELS);
    if (!lv_en) return TGVG_ERR_NOMEM;

    // Enqueue every level.  Device-only work: stopping flags and per-level
    // iteration counts / residuals stay on the device (copied per level into
    // lv_it / lv_res) and are read once after the loop, so the sequence can be
    // captured into a CUDA graph.
    // Host-backed state: move a level's slice of every state array to the
    // device before the level runs, and back to host memory after it.
    auto page = [&](int o, int cnt, bool in) -> int {
        cudaMemLocation loc{};
        loc.type = in ? cudaMemLocationTypeDevice : cudaMemLocationTypeHost;
        loc.id = in ? ctx->device : 0;
        float4* a16[] = {uv, bar, P4, Q4};
        for (float4* a : a16) TGVG_CK(ctx, cudaMemPrefetchAsync(a + o, 16ull * cnt, loc, 0, ctx->stream));
        TGVG_CK(ctx, cudaMemPrefetchAsync(Q1 + o, 4ull * cnt, loc, 0, ctx->stream));
        return TGVG_OK;
    };
    auto enqueue = [&](bool capturing) -> int {
        TGVG_CK(ctx, cudaMemsetAsync(lv_en, 0, 8ull * TGVG_MAX_LEVELS, ctx->stream));
        for (int k = 0; k < (int)levels.size(); ++k) {
            const Level& lvl = levels[k];
            const int Ld = lvl.d, o = lvl.o, cnt = lvl.cnt;
            if (paged) {
                const int rc = page(o, cnt, true);
                if (rc) return rc;
            }
            if (k < TGVG_MAX_LEVELS)
                TGVG_CK(ctx, record_event(ctx->lev_ev[2 * k], ctx->stream, capturing));
            if (level_state) {
                k_level_state<<<blocks_for(cnt, 256), 256, 0, ctx->stream>>>(
                    o, cnt, perm, reinterpret_cast<const float*>(d_state_init), uv, bar, P4, Q4, Q1);
                TGVG_LAUNCHED(ctx);
            }
            if (Ld > min_d && !level_state) {
                k_parent_init<<<blocks_for(cnt, 256), 256, 0, ctx->stream>>>(
                    o, cnt, par, prm->keep_init_u ? 1 : 0, uv, bar, P4, Q4, Q1);
                TGVG_LAUNCHED(ctx);
            }
            if (mode == M_STREAM) {
                k_stream_snapshot<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, uv, bar, snap);
                TGVG_LAUNCHED(ctx);
            } else if (mode == M_OC) {
                k_copy4<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, bar, snap);
                TGVG_LAUNCHED(ctx);
            }
            const bool ghosts = gmax > 0 && cnt >= GHOST_MIN && cnt <= GHOST_MAX;
            if (ghosts) {
                const unsigned gb = (unsigned)((3ll * cnt + 255) / 256);
                if (mode == M_STREAM)
                    k_ghost_mark<M_STREAM><<<gb, 256, 0, ctx->stream>>>(o, cnt, n, nb, par, g_mark);
                else
                    k_ghost_mark<M_INMEM><<<gb, 256, 0, ctx->stream>>>(o, cnt, n, nb, par, g_mark);
                TGVG_LAUNCHED(ctx);
                const int rc = scan_exclusive_async(ctx, g_mark, 3ll * cnt, g_ids, g_sums);
                if (rc) return rc;
                if (mode == M_STREAM)
                    k_ghost_fill<M_STREAM><<<gb, 256, 0, ctx->stream>>>(o, cnt, n, nb, par, g_mark, g_ids, P4, Q4,
                                                                        Q1, g_pnb, g_val);
                else
                    k_ghost_fill<M_INMEM><<<gb, 256, 0, ctx->stream>>>(o, cnt, n, nb, par, g_mark, g_ids, P4, Q4,
                                                                       Q1, g_pnb, g_val);
                TGVG_LAUNCHED(ctx);
                if (dual_ghosts[k]) {  // mark and ids are reused: the primal fill above has read them
                    if (mode == M_STREAM)
                        k_ghost_mark_dual<M_STREAM><<<gb, 256, 0, ctx->stream>>>(o, cnt, n, nb, par, g_mark);
                    else
                        k_ghost_mark_dual<M_INMEM><<<gb, 256, 0, ctx->stream>>>(o, cnt, n, nb, par, g_mark);
                    TGVG_LAUNCHED(ctx);
                    const int rc2 = scan_exclusive_async(ctx, g_mark, 3ll * cnt, g_ids, g_sums);
                    if (rc2) return rc2;
                    if (mode == M_STREAM)
                        k_ghost_fill_dual<M_STREAM><<<gb, 256, 0, ctx->stream>>>(o, cnt, n, nb, par, g_mark, g_ids,
                                                                                 bar, g_dnb, g_dval);
                    else
                        k_ghost_fill_dual<M_INMEM><<<gb, 256, 0, ctx->stream>>>(o, cnt, n, nb, par, g_mark, g_ids,
                                                                                bar, g_dnb, g_dval);
                    TGVG_LAUNCHED(ctx);
                }
            }
            // Every slot's iteration count starts at the full count: the fused
            // schedules' settle step reads it in fixed-count solves too, so a
            // count left by an earlier tolerance-stopped solve must not survive.
            k_fill_i32<<<blocks_for(nslot, 128), 128, 0, ctx->stream>>>(nslot, iters_run, iters);
            TGVG_LAUNCHED(ctx);
            if (stop) {
                TGVG_CK(ctx, cudaMemsetAsync(acc, 0, 32ull * nslot, ctx->stream));
                if (mode == M_STREAM && L > 0) {
                    k_done_init<<<blocks_for(L, 128), 128, 0, ctx->stream>>>(L, Ld, ranges, done);
                    TGVG_LAUNCHED(ctx);
                } else {
                    TGVG_CK(ctx, cudaMemsetAsync(done, 0, 4ull * nslot, ctx->stream));
                }
                TGVG_CK(ctx, cudaMemsetAsync(resid, 0, 8ull * nslot, ctx->stream));
            }
            // NVTX range per level so profilers can select the largest level's launches
            nvtxRangePushA(Ld == big_level ? "tgv_largest_level" : "tgv_level");
            int used_cfg = -1;
            for (const Unit& u : lvl.us) {
                IterArgs a;
                std::memset(&a, 0, sizeof(a));
                a.o = u.o; a.n = u.n; a.npos = n; a.lend = o + cnt;
                a.nb = nb; a.uv = uv; a.bar = bar; a.P4 = P4; a.Q4 = Q4; a.Q1 = Q1; a.dat = dat; a.snap = snap;
                a.lid = lid; a.acc = acc; a.done = done; a.slot0 = u.slot;
                a.alpha0 = prm->alpha0; a.alpha1 = prm->alpha1;
                a.check_every = std::max(1, prm->check_every); a.nslot = nslot; a.tol = prm->tol;
                a.iters_total = iters;
                a.bar_count = reinterpret_cast<unsigned*>(flags + 4);
                a.bar_gen = reinterpret_cast<unsigned*>(flags + 5);
                a.err = flags + 6;
                a.iters_run = iters_run; a.resid = resid;
                a.pnb = ghosts ? g_pnb : nullptr;
                a.gh = ghosts ? g_val : nullptr;
                a.dnb = ghosts && dual_ghosts[k] ? g_dnb : nullptr;
                a.dgh = ghosts && dual_ghosts[k] ? g_dval : nullptr;
                set_fuse(Ld);
                const int rc = run_unit(ctx, mode, a, iters, stop, Ld == t_level, u.cfg, &used_cfg);
                if (rc) { nvtxRangePop(); return rc; }
            }
            nvtxRangePop();
            if (k < TGVG_MAX_LEVELS) {
                used[k] = used_cfg;
                TGVG_CK(ctx, record_event(ctx->lev_ev[2 * k + 1], ctx->stream, capturing));
                if (stop) {
                    TGVG_CK(ctx, cudaMemcpyAsync(lv_it + k * nslot, iters_run, 4ull * nslot,
                                                 cudaMemcpyDeviceToDevice, ctx->stream));
                    TGVG_CK(ctx, cudaMemcpyAsync(lv_res + k * nslot, resid, 8ull * nslot,
                                                 cudaMemcpyDeviceToDevice, ctx->stream));
                }
                if (mode == M_INMEM)
                    k_energy<M_INMEM><<<blocks_for(cnt, 256), 256, 0, ctx->stream>>>(o, cnt, n, nb, uv, dat, prm->alpha0,
                                                                                   prm->alpha1, lv_en + k);
                else
                    k_energy<M_STREAM><<<blocks_for(cnt, 256), 256, 0, ctx->stream>>>(o, cnt, n, nb, uv, dat,
                                                                                    prm->alpha0, prm->alpha1, lv_en + k);
                TGVG_LAUNCHED(ctx);
            }
            if (paged) {
                const int rc = page(o, cnt, false);
                if (rc) return rc;
            }
        }
        return TGVG_OK;
    };

    // (host-backed state runs with direct launches: its prefetches are not captured)
    if (ctx->graphs && !tuning && !levels.empty() && !paged) {
        // Problem signature: everything the captured launches bake in.
        std::vector<uint64_t> key = {
            (uint64_t)mode, (uint64_t)n, (uint64_t)nslot, (uint64_t)iters, (uint64_t)stop,
            (uint64_t)std::max(1, prm->check_every), (uint64_t)(prm->keep_init_u ? 1 : 0), (uint64_t)min_d,
            (uint64_t)(t_level + 1), (uint64_t)level_state, (uint64_t)(uintptr_t)d_state_init};
        uint32_t fb[3];
        std::memcpy(&fb[0], &prm->alpha0, 4);
        std::memcpy(&fb[1], &prm->alpha1, 4);
        std::memcpy(&fb[2], &prm->tol, 4);
        for (uint32_t f : fb) key.push_back(f);
        const FuseSet& fz0 = fsets[levels.front().d];
        const void* ptrs[] = {nb, par, uv, bar, P4, Q4, Q1, dat, snap, lid, acc, flags, resid, lv_res,
                              fused_ok ? fz0.barB : nullptr, fused_ok ? fz0.P4B : nullptr,
                              fused_ok ? fz0.Q4B : nullptr, fused_ok ? fz0.Q1B : nullptr,
                              fused_ok ? fz0.slot : nullptr, fused_ok ? fz0.halo : nullptr,
                              g_pnb, g_val, g_mark, g_ids, g_sums, g_dnb, g_dval};
        for (const void* q : ptrs) key.push_back((uint64_t)(uintptr_t)q);
        for (const Level& lvl : levels) {
            key.push_back(((uint64_t)lvl.d << 32) | (uint32_t)lvl.o);
            key.push_back((uint64_t)lvl.cnt);
            for (const Unit& u : lvl.us) {
                key.push_back(((uint64_t)u.slot << 32) | (uint32_t)u.o);
                key.push_back(((uint64_t)u.n << 8) | (uint32_t)u.cfg);
            }
        }
        if (ctx->graph_exec && key == ctx->graph_key) {
            TGVG_CK(ctx, cudaGraphLaunch(ctx->graph_exec, ctx->stream));
            ctx->kernels += ctx->graph_kernels;
            for (int k = 0; k < nlv; ++k) used[k] = levels[k].us.empty() ? -1 : levels[k].us.back().cfg;
            st.graph = 2;
        } else if (key != ctx->graph_seen) {
            // first sighting of this problem: direct launches (a one-shot solve
            // never pays for capture and instantiation); the next one captures
            ctx->graph_seen = std::move(key);
            const int rc = enqueue(false);
            if (rc) return rc;
        } else {
            ctx->graph_seen.clear();
            if (ctx->graph_exec) {
                cudaGraphExecDestroy(ctx->graph_exec);
                ctx->graph_exec = nullptr;
                ctx->graph_key.clear();
            }
            const int64_t kbefore = ctx->kernels;
            TGVG_CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            ctx->capturing = true;
            const int rc = enqueue(true);
            ctx->capturing = false;
            cudaGraph_t g = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
            if (rc || ce != cudaSuccess || !g) {
                if (g) cudaGraphDestroy(g);
                return rc ? rc : ctx->cuda_fail(ce, "level loop capture");
            }
            cudaGraphExec_t ex = nullptr;
            const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) return ctx->cuda_fail(ie, "level loop graph instantiate");
            ctx->graph_exec = ex;
            ctx->graph_key = std::move(key);
            ctx->graph_kernels = ctx->kernels - kbefore;
            TGVG_CK(ctx, cudaGraphLaunch(ex, ctx->stream));
            st.graph = 1;
        }
    } else {
        const int rc = enqueue(false);
        if (rc) return rc;
    }

    TGVG_CK(ctx, cudaEventRecord(e2, ctx->stream));
    k_unpermute<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(n, inv, uv, P4, Q4, Q1, reinterpret_cast<float*>(d_out));
    TGVG_LAUNCHED(ctx);
    // level stats
    std::vector<int> h_it;
    std::vector<double> h_rs;
    if (stop && nlv > 0) {
        h_it.resize((size_t)nlv * nslot);
        h_rs.resize((size_t)nlv * nslot);
        TGVG_CK(ctx, cudaMemcpyAsync(h_it.data(), lv_it, 4ull * nlv * nslot, cudaMemcpyDeviceToHost, ctx->stream));
        TGVG_CK(ctx, cudaMemcpyAsync(h_rs.data(), lv_res, 8ull * nlv * nslot, cudaMemcpyDeviceToHost, ctx->stream));
    }
    double h_en[TGVG_MAX_LEVELS] = {};
    if (nlv > 0)
        TGVG_CK(ctx, cudaMemcpyAsync(h_en, lv_en, 8ull * nlv, cudaMemcpyDeviceToHost, ctx->stream));
    int h_err = 0;
    TGVG_CK(ctx, cudaMemcpyAsync(&h_err, flags + 6, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (h_err)
        return ctx->fail(TGVG_ERR_TIMEOUT, (h_err & 1) ? "a grid barrier of the persistent iteration kernel timed out"
                                           : (h_err & 4) ? "a TMA stage wait of the fused iteration kernel timed out"
                                                         : "a tile wait of the wavefront iteration kernel timed out");
    for (int k = 0; k < nlv; ++k) {
        const Level& lvl = levels[k];
        st.n_levels = k + 1;
        st.schedule[k] = used[k];
        st.energy[k] = h_en[k];
        st.depth[k] = lvl.d;
        st.active[k] = lvl.cnt;
        if (stop) {
            const int* it_k = h_it.data() + (size_t)k * nslot;
            const double* rs_k = h_rs.data() + (size_t)k * nslot;
            int itmax = 0;
            double rmax = 0.0;
            int64_t li = 0;
            if (mode == M_INMEM) {
                itmax = it_k[0]; rmax = rs_k[0]; li = int64_t(lvl.cnt) * itmax;
            } else {  // one stopping slot per leaf
                for (int l = 0; l < L; ++l) {
                    const int a0 = h_ranges[(l * NBUCKET + lvl.d) * 2], a1 = h_ranges[(l * NBUCKET + lvl.d) * 2 + 1];
                    if (a1 <= a0) continue;
                    itmax = std::max(itmax, it_k[l]);
                    rmax = std::max(rmax, rs_k[l]);
                    li += int64_t(a1 - a0) * it_k[l];
                }
            }
            st.iters_run[k] = itmax;
            st.residual[k] = rmax;
            st.leaf_iters += li;
        } else {
            st.iters_run[k] = iters;
            st.leaf_iters += int64_t(lvl.cnt) * iters;
        }
    }
    float ms_setup = 0.f, ms_iter = 0.f;
    cudaEventElapsedTime(&ms_setup, e0, e1);
    cudaEventElapsedTime(&ms_iter, e1, e2);
    st.setup_ms = ms_setup;
    st.iterate_ms = ms_iter;
    st.total_ms = ms_setup + ms_iter;
    st.kernel_launches = (int32_t)(ctx->kernels - k0);
    for (int k = 0; k < st.n_levels; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->lev_ev[2 * k], ctx->lev_ev[2 * k + 1]);
        st.level_ms[k] = ms;
    }
    if (t_level >= 0) {
        double dsum = 0.0, psum = 0.0;
        const int nt = (iters + TIMING_STRIDE - 1) / TIMING_STRIDE;
        for (int k = 0; k < nt; ++k) {
            float a = 0.f, b = 0.f;
            cudaEventElapsedTime(&a, ctx->tev[3 * k], ctx->tev[3 * k + 1]);
            cudaEventElapsedTime(&b, ctx->tev[3 * k + 1], ctx->tev[3 * k + 2]);
            dsum += a;
            psum += b;
        }
        st.kt_depth = t_level;
        st.kt_launches = nt;
        for (int k = 0; k < nlv; ++k)
            if (levels[k].d == t_level) st.kt_fused = fused_cfg(used[k]) ? 1 : (wave_cfg(used[k]) ? 2 : 0);
        st.kt_active = h_bstart[t_level + 1] - h_bstart[t_level];
        st.kt_dual_ms = dsum;
        st.kt_primal_ms = psum;
    }
    st.placement = paged ? 1 : 0;
    if (stats) *stats = st;
    return TGVG_OK;
}

}  // namespace tgvg
