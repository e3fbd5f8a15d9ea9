// Shared host/device definitions of the sm_103a Stage-5/6 library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "tgvg.h"

namespace tgvg {

// ---- arithmetic that must match the CPU reference bit for bit ---------------
// The reference is plain float C++ evaluated without fused multiply-adds; every
// multiply and add below is an explicitly rounded single operation, never
// contracted.  Division and square root are the IEEE round-to-nearest ones.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// float -> int truncation with the x86-64 result for NaN / out-of-range input
// (INT_MIN), which is what the reference's static_cast<int> yields on the
// platform its fixtures come from.
__host__ __device__ __forceinline__ int trunc_i32(float x) {
    if (!(x > -2147483904.0f && x < 2147483648.0f)) return (int)0x80000000;
#ifdef __CUDA_ARCH__
    return __float2int_rz(x);
#else
    return (int)x;
#endif
}

// ---- Morton helpers (reference src/types.hpp:39-73, src/balance.cpp:13-49) --
__host__ __device__ __forceinline__ uint64_t spread3(uint32_t v) {
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x001f00000000ffffull;
    x = (x | (x << 16)) & 0x001f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}
__host__ __device__ __forceinline__ uint32_t gather3(uint64_t v) {
    v &= 0x1249249249249249ull;
    v = (v | (v >> 2)) & 0x10c30c30c30c30c3ull;
    v = (v | (v >> 4)) & 0x100f00f00f00f00full;
    v = (v | (v >> 8)) & 0x001f0000ff0000ffull;
    v = (v | (v >> 16)) & 0x001f00000000ffffull;
    v = (v | (v >> 32)) & 0x00000000001fffffull;
    return (uint32_t)v;
}
static constexpr uint64_t NO_KEY = ~0ull;
__host__ __device__ __forceinline__ uint64_t ancestor_key(uint64_t k, int d) {
    unsigned sh = 3u * (21u - (unsigned)d);
    if (sh >= 64u) return 0;
    return k & ~((1ull << sh) - 1ull);
}
__host__ __device__ __forceinline__ uint64_t parent_key(uint64_t k, int depth) {
    return ancestor_key(k, depth - 1);
}
// Same-depth face neighbour; faces 0..5 = +x,-x,+y,-y,+z,-z.  NO_KEY outside.
__host__ __device__ __forceinline__ uint64_t face_key(uint64_t k, int face, int depth) {
    uint32_t x = gather3(k), y = gather3(k >> 1), z = gather3(k >> 2);
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
    return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

// ---- device hash table: code -> (smallest index, largest index) -------------
// Open addressing, linear probing, capacity a power of two >= 2n.  Built once
// per solve with atomicCAS on the key and atomicMin/atomicMax on the index
// range, read-only afterwards.  The largest index is the reference's
// std::unordered_map lookup result ("last assignment wins", tgv.cpp:367-370);
// the range also reproduces its binary-search lookup in the streaming path.
struct HashView {
    unsigned long long* keys;  // NO_KEY = empty
    int* rmin;
    int* rmax;
    uint64_t mask;
};
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}
// Insert `key` for index i: the slot keeps the smallest and largest index.
__device__ __forceinline__ void hash_insert(const HashView& h, uint64_t key, int i) {
    uint64_t s = mix64(key) & h.mask;
    for (uint64_t probe = 0; probe <= h.mask; ++probe) {
        const unsigned long long prev = atomicCAS(h.keys + s, (unsigned long long)NO_KEY, (unsigned long long)key);
        if (prev == (unsigned long long)NO_KEY || prev == key) {
            if (h.rmin) atomicMin(h.rmin + s, i);
            if (h.rmax) atomicMax(h.rmax + s, i);
            return;
        }
        s = (s + 1) & h.mask;
    }
}
__device__ __forceinline__ int hash_find(const HashView& h, uint64_t key) {
    uint64_t s = mix64(key) & h.mask;
    for (uint64_t probe = 0; probe <= h.mask; ++probe) {
        unsigned long long k = h.keys[s];
        if (k == key) return (int)s;
        if (k == NO_KEY) return -1;
        s = (s + 1) & h.mask;
    }
    return -1;
}

// The index the reference's CubeFileReader::lookup (tgv.cpp:673-683) returns for
// a code whose equal-code run in the sorted array is [r0, r1]: its bisection
// only compares against the probed code, so the answer depends on n and the
// run bounds alone.
__host__ __device__ __forceinline__ int bisect_hit(int n, int r0, int r1) {
    uint32_t lo = 0, hi = (uint32_t)n;
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if ((int)mid >= r0 && (int)mid <= r1) return (int)mid;
        if ((int)mid < r0) lo = mid + 1; else hi = mid;
    }
    return -1;
}

// Neighbour slots hold a level-major position; BORDER marks a neighbour whose
// bars come from the level-start snapshot (and, in streaming semantics, whose
// p/q read as zero).
static constexpr int BORDER = 0x40000000;
static constexpr int POS_MASK = 0x3fffffff;

}  // namespace tgvg

// ---- context ----------------------------------------------------------------
enum BufId {
    // Stage 5
    B_H_CUBES, B_H_TEX, B_H_OUT, B_H_CAMS,
    // Stage 6
    B_T_CUBES, B_T_HISTS, B_T_UINIT, B_T_SINIT, B_T_OUT, B_KEYS, B_DEPTH, B_LEAFOF, B_BUCKET, B_BCOUNT,
    B_BOFF, B_BTOT, B_PERM, B_INV, B_HKEYS, B_HMIN, B_HMAX, B_NB, B_PAR, B_UV, B_BAR, B_P4, B_Q4,
    B_Q1, B_DAT, B_SNAP, B_LID, B_LEAVES, B_ACC, B_FLAGS, B_RANGES, B_RESID, B_LVSTAT,
    B_BARB, B_P4B, B_Q4B, B_Q1B, B_FSLOT, B_FHALO, B_FHCNT,
    // learned warm start
    B_M_X, B_M_T, B_M_IDX, B_M_Y, B_M_LEAVES, B_M_LEAFID,
    // surface extraction
    B_S_CUBES, B_S_STATE, B_S_KEYS, B_S_DEPTH, B_S_U, B_S_HD, B_S_HKEYS, B_S_HMIN, B_S_HMAX, B_S_NBR,
    B_S_FLAGS, B_S_QIDX, B_S_SCAN, B_S_RANK, B_S_LEAF, B_S_QKEY, B_S_QPOS, B_S_QFLIP, B_S_VTK, B_S_VTF,
    B_S_SLOT, B_S_VFLAG, B_S_VID, B_S_VERTS, B_S_FACES, B_S_TN, B_S_VCNT, B_S_VSTART, B_S_VCUR, B_S_VLIST,
    B_S_NRM,
    // Stage 1
    B_P_DEP, B_P_KEY, B_P_RC, B_P_DPT, B_P_KEEP, B_P_POS, B_P_THR, B_P_CKEY, B_P_CIDX, B_P_SKEY, B_P_SIDX,
    B_P_OUT, B_P_TMP,
    // ordered-wavefront schedule tables
    B_W_KEYS, B_W_SKEYS, B_W_KEEP, B_W_POS, B_W_UKEYS, B_W_DEP, B_W_DOFF, B_W_FLAG, B_W_CNT, B_W_TMP, B_W_TMP2,
    B_W_GSTART, B_LVENERGY,
    // coarser-neighbour ghost tables of the per-launch sweep schedules
    B_G_PNB, B_G_VAL, B_G_MARK, B_G_IDS, B_G_SUMS, B_G_DNB, B_G_DVAL,
    B_COUNT
};

struct tgvg_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::string last_error;
    int64_t kernels = 0;
    struct Buf { void* p = nullptr; size_t cap = 0; bool managed = false; };
    Buf bufs[B_COUNT];
    float lvl_thresh[13] = {};  // footprint thresholds of pyramid levels 1..12
    cudaEvent_t ev[4] = {};
    bool timing = false;               // per-launch events on the largest level
    std::vector<cudaEvent_t> tev;      // pool for those events
    int tune[3][32];                   // chosen iteration schedule per mode and log2(size) class, -1 = untuned
    int coop_max[3][2] = {};           // co-resident blocks of the persistent kernel per mode / stop
    int cluster_max[3][2] = {{-1, -1}, {-1, -1}, {-1, -1}};  // usable cluster size per mode / stop (-1 unknown)
    int iter_occ[3][2][2] = {};        // blocks/SM of the sweep kernels [mode][register-capped][dual, primal]
    int iter_occ_ilp2[3][2] = {};      // blocks/SM of the two-cubes-per-thread sweep kernels [mode][dual, primal]
    int iter_occ_res[3][2] = {};       // blocks/SM of the residual-summing sweep kernels [mode][dual, primal]
    int fused_occ[3][2] = {};          // blocks/SM of the fused iteration kernels per mode [plain, TMA-staged]
    const void* fuse_cur = nullptr;    // the fused-schedule tables of the level being run (tgv.cu), or null
    const void* wave_cur = nullptr;    // the wavefront-schedule tables of the level being run (tgv.cu), or null
    int wave_occ[3][2] = {};           // blocks/SM of the wavefront kernel per mode [L2 loads, L1 loads]
    bool smem_level_ready[3] = {};     // shared-memory limit of the tiny-level kernel raised, per mode
    int smem_level_max = 0;            // dynamic shared memory that kernel may use (bytes)
    cudaEvent_t chk_ev[2] = {};        // stopping flags copied back while the next chunk of iterations runs
    int* chk_host = nullptr;           // pinned host copies of those flags (2 x chk_cap)
    int chk_cap = 0;
    int dsm_max[3] = {-1, -1, -1};     // cluster size of the distributed-shared-memory kernel per mode (-1 unknown)
    cudaEvent_t lev_ev[2 * TGVG_MAX_LEVELS] = {};  // per-level start/end
    bool graphs = true;                // capture the level loop into a CUDA graph when possible
    std::vector<uint64_t> graph_key;   // problem signature of the cached graph
    std::vector<uint64_t> graph_seen;  // signature of the last solve run without a graph
    cudaGraphExec_t graph_exec = nullptr;
    int64_t graph_kernels = 0;         // kernel nodes in the cached graph
    bool capturing = false;            // the level loop is being captured
    size_t device_budget = 0;          // solve footprint above which the state lives in host memory (0: never)
    bool paged_now = false;            // the running solve's state lives in host memory (no TMA-staged schedule)
    tgvg_ctx() {
        for (auto& m : tune)
            for (int& c : m) c = -1;
    }

    // Device buffer `id` with room for `bytes` (grow-only; contents are not kept
    // across growth).  Returns nullptr after recording the error.
    void* buf(int id, size_t bytes);
    // The same as managed memory whose pages live in host memory until they
    // are prefetched to the device (the state of solves larger than the
    // device budget).  A buffer changes kind by being reallocated.
    void* host_backed(int id, size_t bytes);
    int fail(int rc, const std::string& what);
    int cuda_fail(cudaError_t e, const char* what);
};

// Device bytes of a solve of n cubes, in round figures: state and its second
// set 136 B, keys, hash, neighbour and order tables about 150 B, inputs and
// output of a host-buffer call about 110 B per cube.
static inline bool state_paged(const tgvg_ctx* ctx, int64_t n) {
    return ctx->device_budget > 0 && uint64_t(n) * 400ull > ctx->device_budget;
}

#define TGVG_CK(ctx, call)                                                   \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) return (ctx)->cuda_fail(e_, #call);           \
    } while (0)

#define TGVG_LAUNCHED(ctx)                                                   \
    do {                                                                     \
        cudaError_t e_ = cudaGetLastError();                                 \
        if (e_ != cudaSuccess) return (ctx)->cuda_fail(e_, "kernel launch"); \
        ++(ctx)->kernels;                                                    \
    } while (0)

// Entry points implemented in the .cu files (called with ctx->mu held).
namespace tgvg {
int histograms_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, int64_t n, const tgvg_camera* cams,
                   int32_t ncam, const float* d_levels, const int64_t* level_offset,
                   const float origin[3], float r_root, int32_t nbins, uint32_t* d_out);
int build_pyramids_dev(tgvg_ctx* ctx, const tgvg_camera* cams, int32_t ncam, float* d_levels,
                       const int64_t* level_offset);
int tgv_solve_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, const uint32_t* d_hists, int64_t n,
                  int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, int32_t mode,
                  const tgvg_params* params, const float* d_u_init, tgvg_state* d_out,
                  tgvg_stats* stats, const tgvg_state* d_state_init = nullptr);
int pyramid_dims(int32_t w, int32_t h, int32_t* dims);
// Exclusive scan of n ints on the context stream; *total receives the sum (synchronises).
int scan_exclusive(tgvg_ctx* ctx, const int* d_in, int64_t n, int* d_out, int64_t* total);
int64_t scan_sums_len(int64_t n);
int scan_exclusive_async(tgvg_ctx* ctx, const int* d_in, int64_t n, int* d_out, int* sums);
}  // namespace tgvg
