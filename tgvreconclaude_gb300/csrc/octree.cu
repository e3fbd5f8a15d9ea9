// Stages 2 and 3 on the GPU: the k-way merge of sorted cube lists (the
// reference's kway_merge, src/merge.cpp:7-97) and the 2:1 balance
// (balance_octree, src/balance.cpp:60-150).
//
// Merge.  The inputs are concatenated in order and stably radix-sorted by code,
// so equal codes keep input order (the reference's heap leaves the order of
// equal codes from different inputs to std::priority_queue; the two agree
// whenever no code occurs in more than one input).  Runs of consecutive equal
// (code, depth) collapse into one cube whose r_c is the run's float sum in
// order divided by its length (merge.cpp:64-88).
//
// Balance.  The reference processes a FIFO of cells one at a time, and each
// cell's decisions read the cell sets as the cells before it left them.  The
// kernels reproduce that order exactly.  A window of pending FIFO entries is
// evaluated in parallel: every (entry, face) slot computes its bridge
// proposal against the sets at the window start plus the bridges that slots
// before it propose, and the evaluation repeats until the proposals stop
// changing.  A slot's result depends only on slots before it, so the fixed
// point is the sequential result, and a prefix of slots that did not change
// is already exact (used to bound the repetitions).  The accepted bridges are
// appended to the FIFO in slot order, which is the reference's push order.
//
// Presence is tested per exact (depth, code) cell; the output table is keyed
// like the reference's dc_key, depth << 60 | (code & (2^60 - 1)) in 64-bit
// arithmetic (balance.cpp:57-59), so the output drops the code's top three
// bits and folds depths 16..21 onto 0..5, as the reference's does.  Input
// cubes must be valid cells (depth 0..21, code aligned to its depth's grid).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "common.cuh"
#include "fileio.h"

namespace tgvg {
namespace {

constexpr uint64_t DC_MASK = 0x0fffffffffffffffull;
constexpr unsigned long long CELL_EMPTY = 0ull;   // cell keys are never 0
constexpr unsigned long long DC_EMPTY = ~0ull;    // no aligned cell has this output key
constexpr unsigned long long IDX_NONE = ~0ull;
constexpr int64_t WINDOW = int64_t(1) << 22;      // FIFO entries evaluated together
constexpr int MAX_ROUNDS = 24;                    // evaluations of one window before a prefix is committed

inline unsigned grid_of(int64_t n, int t) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

// Locational key of an aligned cell: its depth-d index under a marker bit 3d.
__host__ __device__ __forceinline__ uint64_t cell_key(uint64_t code, int d) {
    return (code >> (3 * (21 - d))) | (1ull << (3 * d));
}
// The reference's output-table key (balance.cpp:57-59).
__host__ __device__ __forceinline__ uint64_t dc_key(int d, uint64_t code) {
    return ((uint64_t)(uint32_t)d << 60) | (code & DC_MASK);
}

// Insert-only open-addressing key set, linear probing, power-of-two capacity.
struct KeySet {
    unsigned long long* keys;
    uint64_t mask;
    unsigned long long empty;
};
__device__ __forceinline__ long long set_slot(const KeySet& s, uint64_t k) {
    uint64_t i = mix64(k) & s.mask;
    for (uint64_t p = 0; p <= s.mask; ++p) {
        const unsigned long long v = s.keys[i];
        if (v == k) return (long long)i;
        if (v == s.empty) return -1;
        i = (i + 1) & s.mask;
    }
    return -1;
}
__device__ __forceinline__ long long set_insert(const KeySet& s, uint64_t k) {
    uint64_t i = mix64(k) & s.mask;
    for (uint64_t p = 0; p <= s.mask; ++p) {
        const unsigned long long prev = atomicCAS(s.keys + i, s.empty, (unsigned long long)k);
        if (prev == s.empty || prev == k) return (long long)i;
        i = (i + 1) & s.mask;
    }
    return -1;  // full: the host sizes every set to at most half load
}

struct Cell {
    unsigned long long code;
    int depth;
    int pad;
};

// ---------------------------------------------------------------- merge ---

__global__ void k_merge_keys(int64_t n, const tgvg_cube* __restrict__ c, unsigned long long* __restrict__ key,
                             long long* __restrict__ idx) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = ((unsigned long long)c[i].hi << 32) | c[i].lo;
    idx[i] = i;
}

__global__ void k_merge_starts(int64_t n, const tgvg_cube* __restrict__ c, const long long* __restrict__ sidx,
                               int* __restrict__ start) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = 1;
    if (i > 0) {
        const tgvg_cube a = c[sidx[i - 1]], b = c[sidx[i]];
        s = !(a.hi == b.hi && a.lo == b.lo && a.depth == b.depth);
    }
    start[i] = s;
}

// One thread per run: the reference's pending-cube accumulation (merge.cpp:64-88).
__global__ void k_merge_runs(int64_t n, const tgvg_cube* __restrict__ c, const long long* __restrict__ sidx,
                             const int* __restrict__ start, const int* __restrict__ pos, tgvg_cube* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !start[i]) return;
    tgvg_cube p = c[sidx[i]];
    float sum = p.r_c;
    uint32_t cnt = 1;
    for (int64_t j = i + 1; j < n && !start[j]; ++j) {
        sum = fadd(sum, c[sidx[j]].r_c);
        ++cnt;
    }
    p.r_c = fdiv(sum, (float)cnt);
    out[pos[i]] = p;
}

// -------------------------------------------------------------- balance ---

// Validity of the input cells: depth 0..21 and a code on its depth's grid.
__global__ void k_bal_check(int64_t n, const tgvg_cube* __restrict__ c, int* __restrict__ bad) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int d = c[i].depth;
    const uint64_t code = ((uint64_t)c[i].hi << 32) | c[i].lo;
    if (d < 0 || d > 21 || (code >> 63) != 0 || ancestor_key(code, d) != code) atomicOr(bad, 1);
}

__global__ void k_bal_seed(int64_t n, const tgvg_cube* __restrict__ c, Cell* __restrict__ q,
                           unsigned long long* __restrict__ dck, long long* __restrict__ dci) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t code = ((uint64_t)c[i].hi << 32) | c[i].lo;
    q[i] = Cell{code, c[i].depth, 0};
    dck[i] = dc_key(c[i].depth, code);
    dci[i] = i;
}

// Insert FIFO entries [0, t) into the cell set and the output-key set.
__global__ void k_bal_insert(int64_t t0, int64_t t, const Cell* __restrict__ q, KeySet cells, KeySet dcs) {
    const int64_t i = t0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= t) return;
    const Cell c = q[i];
    set_insert(cells, cell_key(c.code, c.depth));
    set_insert(dcs, dc_key(c.depth, c.code));
}

// The bridges proposed in the window, as found so far: a set of cell keys with
// the slot that proposes each (only accepted proposals are in it).
struct Window {
    KeySet cells;
    const unsigned long long* slot;
    bool on;
};

// Is (code, d) present for slot `me`: at the window start, or added by an
// earlier slot of the window.
__device__ __forceinline__ bool present(const KeySet& cells, const Window& w, uint64_t code, int d,
                                        unsigned long long me) {
    const uint64_t k = cell_key(code, d);
    if (set_slot(cells, k) >= 0) return true;
    if (!w.on) return false;
    const long long s = set_slot(w.cells, k);
    return s >= 0 && w.slot[s] < me;
}

// One (entry, face) slot of the reference's queue loop (balance.cpp:82-121):
// the bridge it would add, or NO_KEY.
__global__ void k_bal_propose(int64_t h, int64_t wn, const Cell* __restrict__ q, KeySet cells, Window w,
                              unsigned long long* __restrict__ prop, const unsigned long long* __restrict__ prev,
                              unsigned long long* __restrict__ first_change) {
    const int64_t me = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (me >= wn * 6) return;
    const Cell c = q[h + me / 6];
    const int f = (int)(me % 6), d = c.depth;
    uint64_t out = NO_KEY;
    if (d >= 2) {
        const uint64_t nb = face_key(c.code, f, d);
        if (nb != NO_KEY && !present(cells, w, nb, d, me)) {
            const uint64_t par = ancestor_key(nb, d - 1);
            if (!present(cells, w, par, d - 1, me)) {
                bool coarser = false;
                for (int d2 = d - 2; d2 >= 0 && !coarser; --d2)
                    coarser = present(cells, w, ancestor_key(nb, d2), d2, me);
                if (coarser) out = par;
            }
        }
    }
    prop[me] = out;
    if (prev && prev[me] != out) atomicMin(first_change, (unsigned long long)me);
}

__global__ void k_bal_flags(int64_t m, const unsigned long long* __restrict__ prop, int* __restrict__ flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) flag[i] = prop[i] != NO_KEY;
}

__global__ void k_bal_compact(int64_t m, const unsigned long long* __restrict__ prop, const int* __restrict__ flag,
                              const int* __restrict__ pos, unsigned long long* __restrict__ lslot) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m && flag[i]) lslot[pos[i]] = (unsigned long long)i;
}

// Proposals whose output key is new compete for it; the earliest slot wins
// (the reference's emplace succeeds for the first one only).
__global__ void k_bal_claim(int64_t nl, int64_t h, const Cell* __restrict__ q, const unsigned long long* __restrict__ prop,
                            const unsigned long long* __restrict__ lslot, KeySet dcs, KeySet wdc,
                            unsigned long long* __restrict__ wdc_slot) {
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nl) return;
    const unsigned long long me = lslot[l];
    const int d = q[h + me / 6].depth - 1;
    const uint64_t k = dc_key(d, prop[me]);
    if (set_slot(dcs, k) >= 0) return;
    const long long s = set_insert(wdc, k);
    if (s >= 0) atomicMin(wdc_slot + s, me);
}

__global__ void k_bal_accept(int64_t nl, int64_t h, const Cell* __restrict__ q, const unsigned long long* __restrict__ prop,
                             const unsigned long long* __restrict__ lslot, KeySet dcs, KeySet wdc,
                             const unsigned long long* __restrict__ wdc_slot, KeySet wcell,
                             unsigned long long* __restrict__ wcell_slot, int* __restrict__ acc) {
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nl) return;
    const unsigned long long me = lslot[l];
    const int d = q[h + me / 6].depth - 1;
    const uint64_t par = prop[me];
    const uint64_t k = dc_key(d, par);
    int a = 0;
    if (set_slot(dcs, k) < 0) {
        const long long s = set_slot(wdc, k);
        a = s >= 0 && wdc_slot[s] == me;
    }
    acc[l] = a;
    if (a) {
        const long long s = set_insert(wcell, cell_key(par, d));
        if (s >= 0) wcell_slot[s] = me;
    }
}

// Append the accepted bridges of slots below `limit` to the FIFO, in slot order.
__global__ void k_bal_append(int64_t nl, int64_t h, int64_t t, unsigned long long limit, const Cell* __restrict__ qin,
                             Cell* __restrict__ qout, const unsigned long long* __restrict__ prop,
                             const unsigned long long* __restrict__ lslot, const int* __restrict__ acc,
                             const int* __restrict__ apos) {
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nl || !acc[l] || lslot[l] >= limit) return;
    const unsigned long long me = lslot[l];
    qout[t + apos[l]] = Cell{prop[me], qin[h + me / 6].depth - 1, 0};
}

__global__ void k_bal_limit(int64_t nl, const unsigned long long* __restrict__ lslot, unsigned long long limit,
                            const int* __restrict__ acc, int* __restrict__ acc_lim) {
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l < nl) acc_lim[l] = acc[l] && lslot[l] < limit;
}

// Output cubes: the input cells averaged per output key in input order
// (balance.cpp:66-75), then the bridges with r_c = r_root / 2^depth (:113).
__global__ void k_bal_starts(int64_t n, const unsigned long long* __restrict__ skey, int* __restrict__ start) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) start[i] = i == 0 || skey[i] != skey[i - 1];
}

__global__ void k_bal_avg(int64_t n, const unsigned long long* __restrict__ skey, const long long* __restrict__ sidx,
                          const tgvg_cube* __restrict__ c, const int* __restrict__ start, const int* __restrict__ pos,
                          unsigned long long* __restrict__ okey, float* __restrict__ orc) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !start[i]) return;
    float sum = 0.0f;
    uint32_t cnt = 0;
    for (int64_t j = i; j < n && (j == i || !start[j]); ++j) {
        sum = fadd(sum, c[sidx[j]].r_c);
        ++cnt;
    }
    const uint64_t k = skey[i];
    okey[pos[i]] = ((k & DC_MASK) << 4) | (k >> 60);
    orc[pos[i]] = fdiv(sum, (float)cnt);
}

__global__ void k_bal_bridges(int64_t nb, const Cell* __restrict__ q, float r_root, int64_t off,
                              unsigned long long* __restrict__ okey, float* __restrict__ orc) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const Cell c = q[i];
    const uint64_t k = dc_key(c.depth, c.code);
    okey[off + i] = ((k & DC_MASK) << 4) | (k >> 60);
    orc[off + i] = fdiv(r_root, (float)(1u << c.depth));
}

__global__ void k_bal_emit(int64_t n, const unsigned long long* __restrict__ skey, const int* __restrict__ sidx,
                           const float* __restrict__ rc, tgvg_cube* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t k = skey[i];
    const uint64_t code = k >> 4;
    out[i] = tgvg_cube{(uint32_t)(code >> 32), (uint32_t)code, rc[sidx[i]], (int32_t)(k & 15)};
}

__global__ void k_iota(int64_t n, int* __restrict__ v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (int)i;
}

uint64_t pow2_at_least(uint64_t x) {
    uint64_t c = 1024;
    while (c < x) c <<= 1;
    return c;
}

// Device memory of one balance run (owned here: the FIFO grows with its contents).
struct Dev {
    std::vector<void*> ptrs;
    ~Dev() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (T*)p;
    }
    void release(void* p) {
        auto it = std::find(ptrs.begin(), ptrs.end(), p);
        if (it != ptrs.end()) {
            cudaFree(p);
            ptrs.erase(it);
        }
    }
};

// Results go to `vec` (resized) when given, else to `out` when it has room
// (cap), else TGVG_ERR_LIMIT; *count receives their number.
int merge_dev(tgvg_ctx* ctx, const tgvg_cube* const* in, const int64_t* counts, int k, std::vector<tgvg_cube>* vec,
              tgvg_cube* out, int64_t cap, int64_t* count) {
    int64_t n = 0;
    for (int s = 0; s < k; ++s) n += counts[s];
    *count = 0;
    if (vec) vec->clear();
    if (n == 0) return TGVG_OK;
    if (n > (int64_t(1) << 31) - 1) return ctx->fail(TGVG_ERR_LIMIT, "more than 2^31 - 1 cubes");
    cudaStream_t st = ctx->stream;
    Dev D;
    auto* cat = D.get<tgvg_cube>(n);
    auto* key = D.get<unsigned long long>(n);
    auto* skey = D.get<unsigned long long>(n);
    auto* idx = D.get<long long>(n);
    auto* sidx = D.get<long long>(n);
    auto* start = D.get<int>(n);
    auto* pos = D.get<int>(n);
    if (!cat || !key || !skey || !idx || !sidx || !start || !pos) return ctx->fail(TGVG_ERR_NOMEM, "merge buffers");
    int64_t off = 0;
    for (int s = 0; s < k; ++s) {
        if (counts[s])
            TGVG_CK(ctx, cudaMemcpyAsync(cat + off, in[s], sizeof(tgvg_cube) * counts[s], cudaMemcpyHostToDevice, st));
        off += counts[s];
    }
    k_merge_keys<<<grid_of(n, 256), 256, 0, st>>>(n, cat, key, idx);
    TGVG_LAUNCHED(ctx);
    size_t tb = 0;
    TGVG_CK(ctx, cub::DeviceRadixSort::SortPairs(nullptr, tb, key, skey, idx, sidx, (int)n, 0, 63, st));
    void* tmp = D.get<char>(tb);
    if (!tmp) return ctx->fail(TGVG_ERR_NOMEM, "merge sort buffer");
    TGVG_CK(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, key, skey, idx, sidx, (int)n, 0, 63, st));
    k_merge_starts<<<grid_of(n, 256), 256, 0, st>>>(n, cat, sidx, start);
    TGVG_LAUNCHED(ctx);
    int64_t runs = 0;
    int rc = scan_exclusive(ctx, start, n, pos, &runs);
    if (rc) return rc;
    auto* res = D.get<tgvg_cube>(runs);
    if (!res) return ctx->fail(TGVG_ERR_NOMEM, "merge output");
    k_merge_runs<<<grid_of(n, 256), 256, 0, st>>>(n, cat, sidx, start, pos, res);
    TGVG_LAUNCHED(ctx);
    *count = runs;
    if (vec) {
        vec->resize(size_t(runs));
        out = vec->data();
    } else if (!out) {
        return TGVG_OK;
    } else if (cap < runs) {
        return TGVG_ERR_LIMIT;
    }
    TGVG_CK(ctx, cudaMemcpyAsync(out, res, sizeof(tgvg_cube) * runs, cudaMemcpyDeviceToHost, st));
    TGVG_CK(ctx, cudaStreamSynchronize(st));
    return TGVG_OK;
}

struct BalanceSets {
    unsigned long long* cell_keys = nullptr;
    unsigned long long* dc_keys = nullptr;
    uint64_t cap = 0;
    KeySet cells() const { return KeySet{cell_keys, cap - 1, CELL_EMPTY}; }
    KeySet dcs() const { return KeySet{dc_keys, cap - 1, DC_EMPTY}; }
};

// Results as merge_dev's.
int balance_dev(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n, float r_root, std::vector<tgvg_cube>* vec,
                tgvg_cube* out, int64_t cap, int64_t* count) {
    *count = 0;
    if (vec) vec->clear();
    if (n == 0) return TGVG_OK;
    if (n > (int64_t(1) << 30)) return ctx->fail(TGVG_ERR_LIMIT, "more than 2^30 cubes");
    cudaStream_t st = ctx->stream;
    Dev D;
    auto* c = D.get<tgvg_cube>(n);
    auto* bad = D.get<int>(1);
    unsigned long long* fc = D.get<unsigned long long>(1);
    if (!c || !bad || !fc) return ctx->fail(TGVG_ERR_NOMEM, "balance buffers");
    TGVG_CK(ctx, cudaMemcpyAsync(c, cubes, sizeof(tgvg_cube) * n, cudaMemcpyHostToDevice, st));
    TGVG_CK(ctx, cudaMemsetAsync(bad, 0, sizeof(int), st));
    k_bal_check<<<grid_of(n, 256), 256, 0, st>>>(n, c, bad);
    TGVG_LAUNCHED(ctx);
    int hbad = 0;
    TGVG_CK(ctx, cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    TGVG_CK(ctx, cudaStreamSynchronize(st));
    if (hbad) return ctx->fail(TGVG_ERR_INVALID, "balance input holds a cube whose depth is outside 0..21 or "
                                                 "whose code is not on its depth's grid");

    // FIFO (grows), the two sets (rebuilt larger when half full), output keys of the inputs.
    int64_t qcap = std::max<int64_t>(2 * n, 4096);
    Cell* q = D.get<Cell>(qcap);
    auto* dck = D.get<unsigned long long>(n);
    auto* sdck = D.get<unsigned long long>(n);
    auto* dci = D.get<long long>(n);
    auto* sdci = D.get<long long>(n);
    if (!q || !dck || !sdck || !dci || !sdci) return ctx->fail(TGVG_ERR_NOMEM, "balance buffers");
    k_bal_seed<<<grid_of(n, 256), 256, 0, st>>>(n, c, q, dck, dci);
    TGVG_LAUNCHED(ctx);
    BalanceSets S;
    auto build_sets = [&](uint64_t cap, int64_t t) -> int {
        if (S.cell_keys) D.release(S.cell_keys);
        if (S.dc_keys) D.release(S.dc_keys);
        S.cap = cap;
        S.cell_keys = D.get<unsigned long long>(cap);
        S.dc_keys = D.get<unsigned long long>(cap);
        if (!S.cell_keys || !S.dc_keys) return ctx->fail(TGVG_ERR_NOMEM, "balance sets");
        TGVG_CK(ctx, cudaMemsetAsync(S.cell_keys, 0x00, sizeof(unsigned long long) * cap, st));
        TGVG_CK(ctx, cudaMemsetAsync(S.dc_keys, 0xff, sizeof(unsigned long long) * cap, st));
        k_bal_insert<<<grid_of(t, 256), 256, 0, st>>>(0, t, q, S.cells(), S.dcs());
        TGVG_LAUNCHED(ctx);
        return TGVG_OK;
    };
    int rc = build_sets(pow2_at_least(4 * uint64_t(n)), n);
    if (rc) return rc;

    // Window buffers, sized for the largest window.
    const int64_t wmax = std::min<int64_t>(WINDOW, qcap);
    int64_t slots_cap = 6 * wmax;
    auto* prop = D.get<unsigned long long>(slots_cap);
    auto* prop2 = D.get<unsigned long long>(slots_cap);
    auto* flag = D.get<int>(slots_cap);
    auto* fpos = D.get<int>(slots_cap);
    auto* lslot = D.get<unsigned long long>(slots_cap);
    auto* acc = D.get<int>(slots_cap);
    auto* acc_lim = D.get<int>(slots_cap);
    auto* apos = D.get<int>(slots_cap);
    if (!prop || !prop2 || !flag || !fpos || !lslot || !acc || !acc_lim || !apos)
        return ctx->fail(TGVG_ERR_NOMEM, "balance window buffers");
    uint64_t wcap = 0;
    unsigned long long *wdc = nullptr, *wdc_slot = nullptr, *wcell = nullptr, *wcell_slot = nullptr;

    int64_t h = 0, t = n;
    while (h < t) {
        const int64_t wn = std::min<int64_t>(t - h, wmax);
        const int64_t m = 6 * wn;
        k_bal_propose<<<grid_of(m, 256), 256, 0, st>>>(h, wn, q, S.cells(), Window{S.cells(), nullptr, false}, prop,
                                                        nullptr, nullptr);
        TGVG_LAUNCHED(ctx);
        int64_t nl = 0;
        unsigned long long limit = (unsigned long long)m;
        for (int it = 0;; ++it) {
            // the proposals of `prop`, compacted in slot order
            k_bal_flags<<<grid_of(m, 256), 256, 0, st>>>(m, prop, flag);
            TGVG_LAUNCHED(ctx);
            rc = scan_exclusive(ctx, flag, m, fpos, &nl);
            if (rc) return rc;
            if (nl == 0 && it == 0) break;  // nothing proposed against the start sets: already the fixed point
            k_bal_compact<<<grid_of(m, 256), 256, 0, st>>>(m, prop, flag, fpos, lslot);
            TGVG_LAUNCHED(ctx);
            const uint64_t need = pow2_at_least(2 * uint64_t(nl));
            if (need > wcap) {
                for (void* p : {(void*)wdc, (void*)wdc_slot, (void*)wcell, (void*)wcell_slot})
                    if (p) D.release(p);
                wcap = need;
                wdc = D.get<unsigned long long>(wcap);
                wdc_slot = D.get<unsigned long long>(wcap);
                wcell = D.get<unsigned long long>(wcap);
                wcell_slot = D.get<unsigned long long>(wcap);
                if (!wdc || !wdc_slot || !wcell || !wcell_slot) return ctx->fail(TGVG_ERR_NOMEM, "balance window sets");
            }
            const uint64_t wc = pow2_at_least(2 * uint64_t(nl));
            TGVG_CK(ctx, cudaMemsetAsync(wdc, 0xff, sizeof(unsigned long long) * wc, st));
            TGVG_CK(ctx, cudaMemsetAsync(wdc_slot, 0xff, sizeof(unsigned long long) * wc, st));
            TGVG_CK(ctx, cudaMemsetAsync(wcell, 0x00, sizeof(unsigned long long) * wc, st));
            const KeySet kwdc{wdc, wc - 1, DC_EMPTY}, kwcell{wcell, wc - 1, CELL_EMPTY};
            k_bal_claim<<<grid_of(nl, 256), 256, 0, st>>>(nl, h, q, prop, lslot, S.dcs(), kwdc, wdc_slot);
            TGVG_LAUNCHED(ctx);
            k_bal_accept<<<grid_of(nl, 256), 256, 0, st>>>(nl, h, q, prop, lslot, S.dcs(), kwdc, wdc_slot, kwcell,
                                                           wcell_slot, acc);
            TGVG_LAUNCHED(ctx);
            // re-evaluate every slot against the accepted bridges of earlier slots
            TGVG_CK(ctx, cudaMemsetAsync(fc, 0xff, sizeof(unsigned long long), st));
            k_bal_propose<<<grid_of(m, 256), 256, 0, st>>>(h, wn, q, S.cells(), Window{kwcell, wcell_slot, true},
                                                            prop2, prop, fc);
            TGVG_LAUNCHED(ctx);
            unsigned long long first = 0;
            TGVG_CK(ctx, cudaMemcpyAsync(&first, fc, sizeof(first), cudaMemcpyDeviceToHost, st));
            TGVG_CK(ctx, cudaStreamSynchronize(st));
            if (first == IDX_NONE) break;          // fixed point: `prop` is the sequential result
            if (it + 1 >= MAX_ROUNDS) {            // slots below `first` are already exact
                limit = (first / 6) * 6;
                break;
            }
            std::swap(prop, prop2);
        }
        const int64_t done = int64_t(limit / 6);  // FIFO entries finished in this window
        int64_t na = 0;
        if (nl > 0) {
            k_bal_limit<<<grid_of(nl, 256), 256, 0, st>>>(nl, lslot, limit, acc, acc_lim);
            TGVG_LAUNCHED(ctx);
            rc = scan_exclusive(ctx, acc_lim, nl, apos, &na);
            if (rc) return rc;
        }
        if (na > 0) {
            Cell* qout = q;
            const int64_t ncap = std::max<int64_t>(2 * qcap, t + na);
            if (t + na > qcap) {  // grow the FIFO, keeping its contents
                qout = D.get<Cell>(ncap);
                if (!qout) return ctx->fail(TGVG_ERR_NOMEM, "balance queue");
                TGVG_CK(ctx, cudaMemcpyAsync(qout, q, sizeof(Cell) * t, cudaMemcpyDeviceToDevice, st));
            }
            k_bal_append<<<grid_of(nl, 256), 256, 0, st>>>(nl, h, t, limit, q, qout, prop, lslot, acc_lim, apos);
            TGVG_LAUNCHED(ctx);
            if (qout != q) {
                TGVG_CK(ctx, cudaStreamSynchronize(st));
                D.release(q);
                q = qout;
                qcap = ncap;
            }
            if (uint64_t(t + na) * 2 > S.cap) {
                rc = build_sets(pow2_at_least(4 * uint64_t(t + na)), t + na);
                if (rc) return rc;
            } else {
                k_bal_insert<<<grid_of(na, 256), 256, 0, st>>>(t, t + na, q, S.cells(), S.dcs());
                TGVG_LAUNCHED(ctx);
            }
        }
        h += done;
        t += na;
    }

    // Output: averaged input keys, then the bridges, sorted by (code, depth).
    size_t tb = 0;
    TGVG_CK(ctx, cub::DeviceRadixSort::SortPairs(nullptr, tb, dck, sdck, dci, sdci, (int)n, 0, 64, st));
    void* tmp = D.get<char>(tb);
    if (!tmp) return ctx->fail(TGVG_ERR_NOMEM, "balance sort buffer");
    TGVG_CK(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, dck, sdck, dci, sdci, (int)n, 0, 64, st));
    auto* start = D.get<int>(n);
    auto* spos = D.get<int>(n);
    if (!start || !spos) return ctx->fail(TGVG_ERR_NOMEM, "balance buffers");
    k_bal_starts<<<grid_of(n, 256), 256, 0, st>>>(n, sdck, start);
    TGVG_LAUNCHED(ctx);
    int64_t nu = 0;
    rc = scan_exclusive(ctx, start, n, spos, &nu);
    if (rc) return rc;
    const int64_t nb = t - n, no = nu + nb;
    auto* okey = D.get<unsigned long long>(no);
    auto* sokey = D.get<unsigned long long>(no);
    auto* orc = D.get<float>(no);
    auto* oidx = D.get<int>(no);
    auto* soidx = D.get<int>(no);
    auto* res = D.get<tgvg_cube>(no);
    if (!okey || !sokey || !orc || !oidx || !soidx || !res) return ctx->fail(TGVG_ERR_NOMEM, "balance output");
    k_bal_avg<<<grid_of(n, 256), 256, 0, st>>>(n, sdck, sdci, c, start, spos, okey, orc);
    TGVG_LAUNCHED(ctx);
    if (nb > 0) {
        k_bal_bridges<<<grid_of(nb, 256), 256, 0, st>>>(nb, q + n, r_root, nu, okey, orc);
        TGVG_LAUNCHED(ctx);
    }
    k_iota<<<grid_of(no, 256), 256, 0, st>>>(no, oidx);
    TGVG_LAUNCHED(ctx);
    tb = 0;
    TGVG_CK(ctx, cub::DeviceRadixSort::SortPairs(nullptr, tb, okey, sokey, oidx, soidx, (int)no, 0, 64, st));
    void* tmp2 = D.get<char>(tb);
    if (!tmp2) return ctx->fail(TGVG_ERR_NOMEM, "balance sort buffer");
    TGVG_CK(ctx, cub::DeviceRadixSort::SortPairs(tmp2, tb, okey, sokey, oidx, soidx, (int)no, 0, 64, st));
    k_bal_emit<<<grid_of(no, 256), 256, 0, st>>>(no, sokey, soidx, orc, res);
    TGVG_LAUNCHED(ctx);
    *count = no;
    if (vec) {
        vec->resize(size_t(no));
        out = vec->data();
    } else if (!out) {
        return TGVG_OK;
    } else if (cap < no) {
        return TGVG_ERR_LIMIT;
    }
    TGVG_CK(ctx, cudaMemcpyAsync(out, res, sizeof(tgvg_cube) * no, cudaMemcpyDeviceToHost, st));
    TGVG_CK(ctx, cudaStreamSynchronize(st));
    return TGVG_OK;
}

int write_cube_file(const char* path, float r_root, const std::vector<tgvg_cube>& cubes) {
    char hdr[16] = {'T', 'G', 'V', '1'};
    const uint32_t ver = 1, cnt = uint32_t(cubes.size());
    std::memcpy(hdr + 4, &ver, 4);
    std::memcpy(hdr + 8, &r_root, 4);
    std::memcpy(hdr + 12, &cnt, 4);
    return fileio::write_file(path, hdr, 16, cubes.data(), sizeof(tgvg_cube) * cubes.size());
}

}  // namespace
}  // namespace tgvg

using namespace tgvg;

extern "C" int tgvg_merge_cubes(tgvg_ctx* ctx, const tgvg_cube* const* arrays, const int64_t* counts, int32_t k,
                                tgvg_cube* out, int64_t cap, int64_t* count) {
    if (!ctx || !count || k < 0 || (k > 0 && (!arrays || !counts))) return TGVG_ERR_INVALID;
    for (int s = 0; s < k; ++s)
        if (counts[s] < 0 || (counts[s] > 0 && !arrays[s])) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return merge_dev(ctx, arrays, counts, k, nullptr, out, cap, count);
}

extern "C" int tgvg_kway_merge(tgvg_ctx* ctx, const char* const* in_paths, int32_t k, const char* out_path) {
    if (!ctx || k < 0 || (k > 0 && !in_paths) || !out_path) return TGVG_ERR_INVALID;
    std::vector<std::vector<tgvg_cube>> ins(size_t(std::max(k, 0)));
    float r_root = 0.0f;
    for (int s = 0; s < k; ++s) {
        // merge.cpp:30-40 reads each stream's cubes until the file ends
        std::vector<char> b;
        int rc = fileio::read_file(in_paths[s], b);
        if (rc) return ctx->fail(rc, std::string("Cannot open: ") + (in_paths[s] ? in_paths[s] : ""));
        if (b.size() < 16 || std::memcmp(b.data(), "TGV1", 4) != 0)
            return ctx->fail(TGVG_ERR_FORMAT, std::string("Bad magic: ") + in_paths[s]);
        if (s == 0) std::memcpy(&r_root, b.data() + 8, 4);
        const size_t nc = (b.size() - 16) / sizeof(tgvg_cube);
        ins[s].resize(nc);
        if (nc) std::memcpy(ins[s].data(), b.data() + 16, nc * sizeof(tgvg_cube));
    }
    std::vector<const tgvg_cube*> ptr;
    std::vector<int64_t> cnt;
    for (auto& v : ins) {
        ptr.push_back(v.data());
        cnt.push_back(int64_t(v.size()));
    }
    std::vector<tgvg_cube> res;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        int64_t nres = 0;
        const int rc = merge_dev(ctx, ptr.data(), cnt.data(), k, &res, nullptr, 0, &nres);
        if (rc) return rc;
    }
    const int rc = write_cube_file(out_path, r_root, res);
    return rc ? ctx->fail(rc, std::string("Cannot open output: ") + out_path) : TGVG_OK;
}

extern "C" int tgvg_balance_cubes(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n, float r_root, tgvg_cube* out,
                                  int64_t cap, int64_t* count) {
    if (!ctx || !count || n < 0 || (n > 0 && !cubes)) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return balance_dev(ctx, cubes, n, r_root, nullptr, out, cap, count);
}

extern "C" int tgvg_balance_octree(tgvg_ctx* ctx, const char* in_path, const char* out_path) {
    if (!ctx || !in_path || !out_path) return TGVG_ERR_INVALID;
    std::vector<tgvg_cube> cubes;
    float r_root = 0.0f;
    int rc = fileio::load_cube_file(in_path, cubes, &r_root);
    if (rc) return ctx->fail(rc, std::string(rc == TGVG_ERR_IO ? "Cannot open cube file: " : "Bad magic in cube file: ") +
                                     in_path);
    std::vector<tgvg_cube> res;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        int64_t nres = 0;
        rc = balance_dev(ctx, cubes.data(), int64_t(cubes.size()), r_root, &res, nullptr, 0, &nres);
        if (rc) return rc;
    }
    rc = write_cube_file(out_path, r_root, res);
    return rc ? ctx->fail(rc, std::string("Cannot open output: ") + out_path) : TGVG_OK;
}
