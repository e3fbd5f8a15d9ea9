// Context, device buffer pool and the file-level / host-buffer entry points of
// the C ABI declared in include/tgvg.h.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "common.cuh"
#include "fileio.h"

// ------------------------------------------------------------------ ctx ---

void* tgvg_ctx::buf(int id, size_t bytes) {
    if (bytes == 0) bytes = 16;
    Buf& b = bufs[id];
    if (b.cap >= bytes && !b.managed) return b.p;
    if (b.p && b.managed) {
        cudaStreamSynchronize(stream);
        cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
        b.managed = false;
    }
    if (b.cap >= bytes) return b.p;
    if (b.p) {
        cudaStreamSynchronize(stream);
        cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
    }
    size_t want = bytes + bytes / 8;  // headroom so slowly growing inputs do not realloc every call
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaMalloc(&b.p, bytes);
        want = bytes;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        last_error = "cudaMalloc of " + std::to_string(bytes) + " bytes failed";
        return nullptr;
    }
    b.cap = want;
    return b.p;
}

void* tgvg_ctx::host_backed(int id, size_t bytes) {
    if (bytes == 0) bytes = 16;
    Buf& b = bufs[id];
    if (b.cap >= bytes && b.managed) return b.p;
    if (b.p) {
        cudaStreamSynchronize(stream);
        cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
    }
    b.managed = false;
    cudaError_t e = cudaMallocManaged(&b.p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        last_error = "cudaMallocManaged of " + std::to_string(bytes) + " bytes failed";
        return nullptr;
    }
    cudaMemLocation host{};
    host.type = cudaMemLocationTypeHost;
    cudaMemLocation dev{};
    dev.type = cudaMemLocationTypeDevice;
    dev.id = device;
    // pages stay in host memory unless prefetched; the device maps what it
    // touches otherwise instead of faulting it over page by page
    if (cudaMemAdvise(b.p, bytes, cudaMemAdviseSetPreferredLocation, host) != cudaSuccess ||
        cudaMemAdvise(b.p, bytes, cudaMemAdviseSetAccessedBy, dev) != cudaSuccess)
        cudaGetLastError();  // advice only: placement stays correct without it
    b.cap = bytes;
    b.managed = true;
    return b.p;
}

int tgvg_ctx::fail(int rc, const std::string& what) {
    last_error = what;
    return rc;
}

int tgvg_ctx::cuda_fail(cudaError_t e, const char* what) {
    last_error = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();  // a failed call also sets the runtime's last error; clear it for the next call
    return e == cudaErrorMemoryAllocation ? TGVG_ERR_NOMEM : TGVG_ERR_CUDA;
}

// Thresholds t_k = smallest float x >= 1 whose (int)log2f(x) reaches k, for
// k = 1..12, found by bisection over the float bit patterns with the host's
// own log2f -- the function the reference calls (histogram.cpp:99).  A
// footprint's pyramid level is then the number of thresholds it reaches.
static void level_thresholds(float* t) {
    t[0] = 1.0f;
    for (int k = 1; k < 13; ++k) {
        uint32_t lo, hi;
        float one = 1.0f, big = std::numeric_limits<float>::max();
        std::memcpy(&lo, &one, 4);
        std::memcpy(&hi, &big, 4);
        while (lo < hi) {
            uint32_t mid = lo + (hi - lo) / 2;
            float x;
            std::memcpy(&x, &mid, 4);
            if (tgvg::trunc_i32(std::log2(x)) >= k) hi = mid; else lo = mid + 1;
        }
        std::memcpy(&t[k], &lo, 4);
    }
}

extern "C" int tgvg_abi_version(void) { return TGVG_ABI_VERSION; }

extern "C" void tgvg_level_thresholds(float* t13) {
    if (t13) level_thresholds(t13);
}

extern "C" int tgvg_set_schedule(tgvg_ctx* ctx, int32_t mode, int32_t cls, int32_t cfg) {
    if (!ctx || mode < 0 || mode > 2 || cls < -1 || cls > 31 || cfg < -1 || cfg > 24) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    for (int c = 0; c < 32; ++c)
        if (cls < 0 || c == cls) ctx->tune[mode][c] = cfg;
    return TGVG_OK;
}

extern "C" int tgvg_set_graphs(tgvg_ctx* ctx, int on) {
    if (!ctx) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->graphs = on != 0;
    return TGVG_OK;
}

extern "C" int tgvg_set_device_budget(tgvg_ctx* ctx, int64_t bytes) {
    if (!ctx || bytes < 0) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->device_budget = (size_t)bytes;
    return TGVG_OK;
}

extern "C" int tgvg_set_timing(tgvg_ctx* ctx, int on) {
    if (!ctx) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->timing = on != 0;
    return TGVG_OK;
}

extern "C" const char* tgvg_strerror(int rc) {
    switch (rc) {
        case TGVG_OK: return "ok";
        case TGVG_ERR_INVALID: return "invalid argument";
        case TGVG_ERR_CUDA: return "CUDA error";
        case TGVG_ERR_NOMEM: return "out of device memory";
        case TGVG_ERR_UNSORTED: return "cubes are not sorted by Morton code";
        case TGVG_ERR_IO: return "cannot open or read/write file";
        case TGVG_ERR_FORMAT: return "bad file magic or truncated file";
        case TGVG_ERR_TIMEOUT: return "device wait timed out";
        case TGVG_ERR_NODEVICE: return "no usable sm_103 device";
        case TGVG_ERR_OVERLAP: return "treetop leaves overlap";
        case TGVG_ERR_LIMIT: return "request exceeds the fixed scratch of the no-allocation entry point";
        default: return "unknown error";
    }
}

extern "C" const char* tgvg_last_error(tgvg_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

extern "C" void* tgvg_stream(tgvg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

extern "C" int64_t tgvg_kernel_count(tgvg_ctx* ctx) { return ctx ? ctx->kernels : 0; }

extern "C" int tgvg_create(int device, tgvg_ctx** out) {
    if (!out) return TGVG_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return TGVG_ERR_NODEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major != 10 || prop.minor != 3)
        return TGVG_ERR_NODEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return TGVG_ERR_NODEVICE;
    auto* c = new tgvg_ctx();
    c->device = device;
    c->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return TGVG_ERR_CUDA;
    }
    for (auto& e : c->ev) cudaEventCreate(&e);
    for (auto& e : c->lev_ev) cudaEventCreate(&e);
    for (auto& e : c->chk_ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    level_thresholds(c->lvl_thresh);
    *out = c;
    return TGVG_OK;
}

extern "C" int tgvg_destroy(tgvg_ctx* ctx) {
    if (!ctx) return TGVG_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        for (auto& b : ctx->bufs)
            if (b.p) cudaFree(b.p);
        for (auto& e : ctx->ev) cudaEventDestroy(e);
        for (auto& e : ctx->tev) cudaEventDestroy(e);
        for (auto& e : ctx->lev_ev) cudaEventDestroy(e);
        for (auto& e : ctx->chk_ev) cudaEventDestroy(e);
        if (ctx->chk_host) cudaFreeHost(ctx->chk_host);
        if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
        cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
    return TGVG_OK;
}

// ---------------------------------------------------------------- files ---
using namespace tgvg::fileio;


extern "C" int tgvg_save_tgv(const char* path, const tgvg_state* state, int64_t n) {
    if (n < 0 || (n > 0 && !state) || n > 0xffffffffll) return TGVG_ERR_INVALID;
    char hdr[12] = {'T', 'G', 'V', 'S'};
    uint32_t v = 1, c = (uint32_t)n;
    std::memcpy(hdr + 4, &v, 4);
    std::memcpy(hdr + 8, &c, 4);
    return write_file(path, hdr, 12, state, sizeof(tgvg_state) * size_t(n));
}

extern "C" int64_t tgvg_load_tgv(const char* path, tgvg_state* out, int64_t cap) {
    std::vector<char> b;
    int rc = read_file(path, b);
    if (rc) return rc;
    if (b.size() < 12 || std::memcmp(b.data(), "TGVS", 4) != 0) return TGVG_ERR_FORMAT;
    uint32_t n = u32_at(b, 8);
    if (b.size() < 12 + size_t(n) * sizeof(tgvg_state)) return TGVG_ERR_FORMAT;
    if (out) {
        if (cap < int64_t(n)) return TGVG_ERR_INVALID;
        std::memcpy(out, b.data() + 12, size_t(n) * sizeof(tgvg_state));
    }
    return int64_t(n);
}

extern "C" int tgvg_save_histograms(const char* path, const uint32_t* hists, int64_t n) {
    if (n < 0 || (n > 0 && !hists) || n > 0xffffffffll) return TGVG_ERR_INVALID;
    char hdr[12] = {'T', 'G', 'V', 'H'};
    uint32_t v = 1, c = (uint32_t)n;
    std::memcpy(hdr + 4, &v, 4);
    std::memcpy(hdr + 8, &c, 4);
    return write_file(path, hdr, 12, hists, 32 * size_t(n));
}

extern "C" int64_t tgvg_load_histograms(const char* path, uint32_t* out, int64_t cap) {
    std::vector<char> b;
    int rc = read_file(path, b);
    if (rc) return rc;
    if (b.size() < 12 || std::memcmp(b.data(), "TGVH", 4) != 0) return TGVG_ERR_FORMAT;
    uint32_t n = u32_at(b, 8);
    if (b.size() < 12 + size_t(n) * 32) return TGVG_ERR_FORMAT;
    if (out) {
        if (cap < int64_t(n)) return TGVG_ERR_INVALID;
        std::memcpy(out, b.data() + 12, size_t(n) * 32);
    }
    return int64_t(n);
}

// --------------------------------------------------------- Stage 6 host ---

extern "C" int tgvg_tgv_minimize_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, const uint32_t* d_hists,
                                     int64_t n, int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf,
                                     int32_t mode, const tgvg_params* params, const float* d_u_init,
                                     tgvg_state* d_out, tgvg_stats* stats) {
    if (!ctx) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return tgvg::tgv_solve_dev(ctx, d_cubes, d_hists, n, nbins, leaves, nleaf, mode, params, d_u_init,
                               d_out, stats);
}

extern "C" int tgvg_tgv_minimize_state_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, const uint32_t* d_hists,
                                           int64_t n, int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf,
                                           int32_t mode, const tgvg_params* params,
                                           const tgvg_state* d_init_state, tgvg_state* d_out, tgvg_stats* stats) {
    if (!ctx || !params || params->init != TGVG_INIT_STATE) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return tgvg::tgv_solve_dev(ctx, d_cubes, d_hists, n, nbins, leaves, nleaf, mode, params, nullptr, d_out, stats,
                               d_init_state);
}

static int minimize_host(tgvg_ctx* ctx, const tgvg_cube* cubes, const uint32_t* hists, int64_t n,
                         int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, int32_t mode,
                         const tgvg_params* params, const float* u_init, tgvg_state* out,
                         tgvg_stats* stats, const tgvg_state* init_state = nullptr) {
    if (n < 0 || (n > 0 && (!cubes || !hists || !out)) || (nbins != 8 && nbins != 10) || !params)
        return TGVG_ERR_INVALID;
    if (n == 0) {
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return TGVG_OK;
    }
    if (params->init == TGVG_INIT_GIVEN && !u_init) return TGVG_ERR_INVALID;
    if ((params->init == TGVG_INIT_STATE) != (init_state != nullptr)) return TGVG_ERR_INVALID;
    // beyond the device budget the staged inputs and the output live in host memory too
    auto TB = [&](int id, size_t bytes) {
        return state_paged(ctx, n) ? ctx->host_backed(id, bytes) : ctx->buf(id, bytes);
    };
    auto* d_cubes = (tgvg_cube*)TB(B_T_CUBES, sizeof(tgvg_cube) * n);
    auto* d_hists = (uint32_t*)TB(B_T_HISTS, sizeof(uint32_t) * nbins * n);
    auto* d_out = (tgvg_state*)TB(B_T_OUT, sizeof(tgvg_state) * n);
    float* d_u = nullptr;
    if (params->init == TGVG_INIT_GIVEN) d_u = (float*)ctx->buf(B_T_UINIT, sizeof(float) * n);
    tgvg_state* d_s = nullptr;
    if (init_state) d_s = (tgvg_state*)ctx->buf(B_T_SINIT, sizeof(tgvg_state) * n);
    if (!d_cubes || !d_hists || !d_out || (params->init == TGVG_INIT_GIVEN && !d_u) || (init_state && !d_s))
        return TGVG_ERR_NOMEM;
    if (d_s)
        TGVG_CK(ctx, cudaMemcpyAsync(d_s, init_state, sizeof(tgvg_state) * n, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaMemcpyAsync(d_cubes, cubes, sizeof(tgvg_cube) * n, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaMemcpyAsync(d_hists, hists, sizeof(uint32_t) * nbins * n, cudaMemcpyHostToDevice,
                                 ctx->stream));
    if (d_u)
        TGVG_CK(ctx, cudaMemcpyAsync(d_u, u_init, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    int rc = tgvg::tgv_solve_dev(ctx, d_cubes, d_hists, n, nbins, leaves, nleaf, mode, params, d_u, d_out,
                                 stats, d_s);
    if (rc) return rc;
    TGVG_CK(ctx, cudaMemcpyAsync(out, d_out, sizeof(tgvg_state) * n, cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

extern "C" int tgvg_tgv_minimize(tgvg_ctx* ctx, const tgvg_cube* cubes, const uint32_t* hists, int64_t n,
                                 int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, int32_t mode,
                                 const tgvg_params* params, const float* u_init, tgvg_state* out,
                                 tgvg_stats* stats) {
    if (!ctx) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return minimize_host(ctx, cubes, hists, n, nbins, leaves, nleaf, mode, params, u_init, out, stats);
}

extern "C" int tgvg_tgv_minimize_state(tgvg_ctx* ctx, const tgvg_cube* cubes, const uint32_t* hists, int64_t n,
                                       int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, int32_t mode,
                                       const tgvg_params* params, const tgvg_state* init_state, tgvg_state* out,
                                       tgvg_stats* stats) {
    if (!ctx || !params || params->init != TGVG_INIT_STATE || (n > 0 && !init_state)) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    return minimize_host(ctx, cubes, hists, n, nbins, leaves, nleaf, mode, params, nullptr, out, stats, init_state);
}

extern "C" int tgvg_tgv_minimize_streaming(tgvg_ctx* ctx, const char* cube_path, const char* hist_path,
                                           const char* treetop_path, const char* out_state_path,
                                           const tgvg_params* params, tgvg_stats* stats) {
    if (!ctx || !params) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    // treetop (treetop.cpp:93-108)
    std::vector<char> tb;
    int rc = read_file(treetop_path, tb);
    if (rc) return ctx->fail(rc, std::string("Cannot open treetop: ") + (treetop_path ? treetop_path : ""));
    if (tb.size() < 16 || std::memcmp(tb.data(), "TGVT", 4) != 0)
        return ctx->fail(TGVG_ERR_FORMAT, "Bad treetop magic");
    const uint32_t nleaf = u32_at(tb, 12);
    if (tb.size() < 16 + size_t(nleaf) * sizeof(tgvg_leaf)) return ctx->fail(TGVG_ERR_FORMAT, "short treetop");
    std::vector<tgvg_leaf> leaves(nleaf);
    if (nleaf) std::memcpy(leaves.data(), tb.data() + 16, nleaf * sizeof(tgvg_leaf));
    std::vector<tgvg_cube> cubes;
    if ((rc = load_cube_file(cube_path, cubes, nullptr)))
        return ctx->fail(rc, std::string("cube file: ") + (cube_path ? cube_path : ""));
    const int64_t n = int64_t(cubes.size());
    std::vector<tgvg_state> state(n);
    if (n > 0) {
        std::vector<char> hb;
        if ((rc = read_file(hist_path, hb))) return ctx->fail(rc, "Cannot open histograms");
        if (hb.size() < 12 || std::memcmp(hb.data(), "TGVH", 4) != 0)
            return ctx->fail(TGVG_ERR_FORMAT, "Bad histogram magic");
        if (hb.size() < 12 + size_t(n) * 32 || u32_at(hb, 8) < uint32_t(n))
            return ctx->fail(TGVG_ERR_FORMAT, "histogram file shorter than the cube file");
        rc = minimize_host(ctx, cubes.data(), reinterpret_cast<const uint32_t*>(hb.data() + 12), n, 8,
                           leaves.data(), int32_t(nleaf), TGVG_MODE_STREAM, params, nullptr, state.data(),
                           stats);
        if (rc) return rc;
    } else if (stats) {
        std::memset(stats, 0, sizeof(*stats));
    }
    rc = tgvg_save_tgv(out_state_path, state.data(), n);
    return rc ? ctx->fail(rc, "Cannot open state output") : TGVG_OK;
}

// ------------------------------------------------------- Stage 5 files ---

extern "C" int tgvg_compute_histograms(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n,
                                       const tgvg_camera* cams, int32_t ncam, const float* const* base,
                                       const float origin[3], float r_root, int32_t nbins, uint32_t* out);

extern "C" int tgvg_compute_histograms_oc(tgvg_ctx* ctx, const char* cube_path, const tgvg_leaf* leaves,
                                          int32_t nleaf, const tgvg_camera* cams, int32_t ncam,
                                          const float* const* base, const float origin[3], float r_root,
                                          const char* out_hist_path) {
    if (!ctx || nleaf < 0 || (nleaf > 0 && !leaves)) return TGVG_ERR_INVALID;
    char hdr[12] = {'T', 'G', 'V', 'H'};
    uint32_t ver = 1;
    std::memcpy(hdr + 4, &ver, 4);
    if (nleaf == 0) {
        uint32_t z = 0;
        std::memcpy(hdr + 8, &z, 4);
        return write_file(out_hist_path, hdr, 12, nullptr, 0);
    }
    std::vector<tgvg_cube> cubes;
    int rc = load_cube_file(cube_path, cubes, nullptr);
    if (rc) return rc;
    const int64_t n = int64_t(cubes.size());
    std::vector<uint32_t> h(size_t(n) * 8);
    if (n > 0 && (rc = tgvg_compute_histograms(ctx, cubes.data(), n, cams, ncam, base, origin, r_root, 8,
                                               h.data())))
        return rc;
    // The reference streams each leaf's slice in leaf order under a header
    // counting leaves.back().last_idx + 1 rows (histogram.cpp:237-255).
    const uint32_t total = leaves[nleaf - 1].last_idx + 1;
    std::memcpy(hdr + 8, &total, 4);
    std::vector<uint32_t> body;
    for (int l = 0; l < nleaf; ++l) {
        const uint32_t a = leaves[l].first_idx, b = leaves[l].last_idx;
        if (int64_t(a) >= n || a > b) continue;
        const int64_t e = std::min<int64_t>(int64_t(b) + 1, n);
        body.insert(body.end(), h.begin() + int64_t(a) * 8, h.begin() + e * 8);
    }
    return write_file(out_hist_path, hdr, 12, body.data(), body.size() * 4);
}
