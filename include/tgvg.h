/*
 * tgvg.h -- C ABI of the GB300 (sm_103a) implementation of the TGVReconClaude
 * Stage-5 (depth maps -> per-cube histograms) and Stage-6 (histogram-data-term
 * primal-dual TGV over a Morton-ordered octree) hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns 0
 * (TGVG_OK) or a negative TGVG_ERR_* code, and never throws.  A C++ caller that
 * wants the reference's exception behaviour maps a nonzero code to
 * std::runtime_error(tgvg_strerror(rc)).  Records are byte-identical to the
 * reference's structs, so std::vector<OctreeCube>::data() etc. can be passed as
 * they are.
 *
 * The reference interface each entry point replaces is cited as
 * reference-path:line (paths inside the reference project).
 */
#ifndef TGVG_H
#define TGVG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TGVG_ABI_VERSION 4

/* ---- status codes -------------------------------------------------------- */
#define TGVG_OK             0
#define TGVG_ERR_INVALID   -1  /* bad argument (null pointer, size, depth outside 0..21, mode) */
#define TGVG_ERR_CUDA      -2  /* a CUDA runtime call failed; tgvg_last_error() has the text  */
#define TGVG_ERR_NOMEM     -3  /* device memory exhausted                                      */
#define TGVG_ERR_UNSORTED  -4  /* streaming semantics need cubes sorted by Morton code         */
#define TGVG_ERR_IO        -5  /* cannot open / short read / short write   (runtime_error)     */
#define TGVG_ERR_FORMAT    -6  /* bad magic in a TGV1/TGVH/TGVT/TGVS file    (runtime_error)   */
#define TGVG_ERR_TIMEOUT   -7  /* a bounded device wait ran out of iterations                  */
#define TGVG_ERR_NODEVICE  -8  /* no CUDA device, or not an sm_103 part                        */
#define TGVG_ERR_OVERLAP   -9  /* treetop leaves overlap                                       */
#define TGVG_ERR_LIMIT    -10  /* request exceeds the fixed scratch of a no-allocation entry   */

/* ---- records (byte-identical to the reference) --------------------------- */

/* OctreeCube, reference src/types.hpp:30-34 (16 B). code = {hi, lo} 63-bit Z-code
 * of the cube's lower corner on the 2^21 fine grid. */
typedef struct tgvg_cube {
    uint32_t hi, lo;
    float r_c;
    int32_t depth;
} tgvg_cube;

/* TreetopLeaf, reference src/treetop.hpp:8-13 (20 B): inclusive index range. */
typedef struct tgvg_leaf {
    uint32_t hi, lo;
    int32_t depth;
    uint32_t first_idx, last_idx;
} tgvg_leaf;

/* TGVCube, reference src/tgv.hpp:12-17 (52 B). q in Voigt order xx yy zz xy xz yz. */
typedef struct tgvg_state {
    float u;
    float v[3];
    float p[3];
    float q[6];
} tgvg_state;

/* Histogram rows are uint32[nbins]: nbins = 8 is CubeHistogram
 * (reference src/histogram.hpp:10-19); nbins = 10 is the 10-bin extension. */

/* One depth map as DepthMipmap holds it (reference src/histogram.hpp:22-38),
 * without the texels. */
typedef struct tgvg_camera {
    float rt_inv[16];        /* camera<-world, ROW-major (DepthMipmap::Rt_inv)           */
    float fx, fy, cx, cy;    /* level-0 intrinsics K(0,0), K(1,1), K(0,2), K(1,2)        */
    int32_t width, height;   /* level-0 size                                             */
    int32_t lidar;           /* nonzero: vote 5 instead of 1 (histogram.cpp:158)         */
    int32_t reserved;        /* must be 0                                                */
} tgvg_camera;

/* TGVParams (reference src/tgv.hpp:24-28) plus the stopping extension. */
typedef struct tgvg_params {
    float alpha0;            /* weight on |e(v)|  (reference default 0.02)              */
    float alpha1;            /* weight on |grad u - v| (reference default 0.04)         */
    int32_t iters;           /* primal-dual iterations per level (maximum when tol > 0) */
    int32_t init;            /* TGVG_INIT_*                                             */
    float tol;               /* relative residual stop; 0 = fixed count (reference)     */
    int32_t check_every;     /* residual evaluated every this many iterations           */
    int32_t keep_init_u;     /* 0 (reference): a level's cubes copy u and v from their  */
                             /* parent; 1: they keep their initial u and copy only v     */
                             /* (a warm start or a literal zero start at every level)   */
} tgvg_params;

#define TGVG_INIT_MEDIAN 0   /* u = median_indicator (reference, tgv.cpp:372-373) */
#define TGVG_INIT_ZERO   1   /* u = 0 ("plain solver from a zero start")          */
#define TGVG_INIT_GIVEN  2   /* u = caller array (learned warm start)             */
#define TGVG_INIT_STATE  3   /* whole-state warm start: tgvg_tgv_minimize_state   */

#define TGVG_MODE_INMEM  0   /* tgv_minimize           (tgv.cpp:356-419) */
#define TGVG_MODE_OC     1   /* tgv_minimize_oc        (tgv.cpp:423-511) */
#define TGVG_MODE_STREAM 2   /* tgv_minimize_streaming (tgv.cpp:802-1070), all leaves batched */

#define TGVG_MAX_LEVELS 22

/* Per-solve counters. */
typedef struct tgvg_stats {
    int32_t n_levels;                    /* levels that had active cubes            */
    int32_t min_depth, max_depth;
    int32_t depth[TGVG_MAX_LEVELS];      /* depth of level slot k                   */
    int64_t active[TGVG_MAX_LEVELS];     /* active cubes of level slot k            */
    int32_t iters_run[TGVG_MAX_LEVELS];  /* iterations run (max over leaves)        */
    double residual[TGVG_MAX_LEVELS];    /* last relative residual (max over leaves)*/
    int64_t leaf_iters;                  /* sum over levels of active x iterations  */
    int32_t kernel_launches;             /* kernels this call enqueued              */
    int32_t graph;                       /* level loop: 0 direct launches, 1 captured
                                            into a new CUDA graph and launched, 2 a
                                            cached graph of the same problem relaunched */
    double setup_ms, iterate_ms, total_ms; /* device time of the phases             */
    /* Per-launch timing of the iteration kernels on the level with the most
     * active cubes (filled when tgvg_set_timing(ctx, 1) is on): CUDA event
     * durations on the context stream, summed over the launches of every 10th
     * iteration, and the number of launches timed per kernel.  That level then
     * runs with per-sweep launches (schedule 0, or 7 when tuned to it). */
    int32_t kt_depth;
    int32_t kt_launches;
    int64_t kt_active;
    double kt_dual_ms, kt_primal_ms;
    double level_ms[TGVG_MAX_LEVELS];    /* device time of level slot k (init + iterations) */
    int32_t schedule[TGVG_MAX_LEVELS];   /* iteration schedule used for level slot k       */
    int32_t kt_fused;                    /* 1: the timed level ran the fused kernel, 2: the
                                            wavefront kernel (kt_dual_ms holds its time,
                                            kt_primal_ms 0)                                   */
    int32_t placement;                   /* 0: state in device memory; 1: the solve exceeded
                                            the device budget (tgvg_set_device_budget) and its
                                            state lived in host memory, each level's slice
                                            prefetched to the device while it ran            */
    /* No counterpart in the reference: the FP64 primal energy of level slot k's
     * state when the level ends, sum over its cubes of tot |u - median| +
     * alpha1 |grad u - v| + alpha0 |e(v)| with the iteration's own difference
     * operators (a missing neighbour counts as the cube itself; e(v) in Voigt
     * form, off-diagonals halved and counted once).  Neighbours are read from the
     * current state in every semantics. */
    double energy[TGVG_MAX_LEVELS];
} tgvg_stats;

typedef struct tgvg_ctx tgvg_ctx;

/* ---- context ---------------------------------------------------------------
 * One context per process and device: it owns the CUDA stream all calls run on
 * and a grow-only pool of device buffers reused across calls.  Calls on one
 * context are serialised by a mutex (the reference is single-threaded). */
int tgvg_create(int device, tgvg_ctx** out);
int tgvg_destroy(tgvg_ctx* ctx);
const char* tgvg_strerror(int rc);
const char* tgvg_last_error(tgvg_ctx* ctx);
int tgvg_abi_version(void);
/* The stream the context runs on (cudaStream_t as void*). */
void* tgvg_stream(tgvg_ctx* ctx);
/* Count of this library's kernels launched on the context since creation. */
int64_t tgvg_kernel_count(tgvg_ctx* ctx);
/* The 13 footprint thresholds the histogram kernel uses for the pyramid level
 * (t[k] = smallest float >= 1 whose (int)log2f reaches k; t[0] = 1).  Host-only,
 * needs no device: it reproduces `(int)std::log2(std::max(1.0f, footprint))`
 * of histogram.cpp:99 without calling log2 on the GPU. */
void tgvg_level_thresholds(float* t13);
/* Turn per-launch event timing of the largest level's iteration kernels on (1)
 * or off (0); results land in tgvg_stats.kt_*. */
int tgvg_set_timing(tgvg_ctx* ctx, int on);
/* Iteration schedule of a level whose active count n has floor(log2 n) == cls
 * (cls = -1: every class), for one mode: 0 = two launches per iteration, 1..6 =
 * one cooperative launch per level with about 256 << k cubes per block, 7 = as 0
 * with the sweep kernels capped at 32 registers, 8 / 9 = as 0 / 7 with an L2
 * prefetch of each warp's next group, 10 / 11 = one launch of one thread-block
 * cluster of 8 / 16 CTAs running every iteration (units of at most 131072
 * cubes), 12 / 13 = as 0 / 8 with the dual sweep run from the chunk's end and
 * the primal from its start, 14 / 15 = as 0 / 12 with all warps striding over
 * the whole level together (band order), 16 / 17 = as 14 / 15 with two cubes
 * per thread and step, 18 = one fused launch per iteration over 256-cube tiles
 * with the tile's p/q in shared memory (in-memory and streaming semantics; OC
 * runs 14), 19 = as 18 with the tiles' streams staged by TMA bulk copies,
 * 20 / 21 = one ordered-wavefront launch per iteration, each block running the
 * dual then the primal step of a 512-cube tile once the tiles it depends on
 * have run their dual step, with loads through L2 only (20) or through L1 too
 * (21) (in-memory and streaming semantics on levels whose dependencies all
 * point to earlier tiles once short runs of tiles are grouped, which holds for
 * Morton-sorted cubes; otherwise 14; never chosen by the autotuner), 22 = one
 * launch of a single 1024-thread block running every iteration, reading through
 * L1 (units of at most 4096 cubes), 23 = as 22 with the unit's state held in
 * shared memory for the whole launch (units of at most 2048 cubes; larger
 * units run 22), 24 = one thread-block cluster of 16 (else 8) CTAs whose
 * shared memories hold the unit's state, neighbours in other CTAs read through
 * distributed shared memory (units of at most 16 x 2816 cubes; larger units
 * run 14), -1 = let the online autotuner choose (default).  Results do not
 * depend on it. */
int tgvg_set_schedule(tgvg_ctx* ctx, int32_t mode, int32_t cls, int32_t cfg);
/* CUDA graphs for the level loop (1 = on, the default; 0 = off).  When every
 * level's schedule is already fixed (chosen by the autotuner in an earlier
 * call, set with tgvg_set_schedule, or the default of a tolerance-stopped
 * solve) and per-launch timing is off, the whole level loop -- parent init,
 * snapshots, the iteration launches and the stopping tests of every level --
 * is captured into one CUDA graph, kept in the context and relaunched by
 * later solves of a problem with the same level sizes, leaves, parameters and
 * buffers.  Capture happens on the second consecutive solve of such a problem
 * (graph = 1), so one-shot solves run with direct launches (graph = 0).
 * Results do not depend on it. */
int tgvg_set_graphs(tgvg_ctx* ctx, int on);
/* Device budget for one solve, in bytes (0 = none, the default).  A solve whose
 * device footprint (about 400 B per cube) would exceed it keeps its per-cube
 * state -- u, v, p, q, bars, the streaming snapshot and the fused schedules'
 * second set -- in host memory (CUDA managed memory preferring the host), and
 * moves each level's slice to the device while that level runs and back after
 * it; keys, hash and neighbour tables stay in device memory.  On a GB300 the
 * host memory is the Grace CPU's, reached over NVLink-C2C.  Such solves run
 * with direct launches (no level-loop graph).  This is the out-of-core
 * streaming of tgv_minimize_streaming (reference tgv.cpp:802-1070) for
 * problems beyond device memory; results do not depend on it. */
int tgvg_set_device_budget(tgvg_ctx* ctx, int64_t bytes);

/* ---- Stage 5: depth maps -> histograms ------------------------------------ */

/* Pyramid geometry of a W x H map: writes (w, h) of every level into dims
 * (2 entries per level, room for 13) and returns the level count
 * (DepthMipmap::build level rule, reference src/histogram.cpp:42-53). */
int tgvg_pyramid_dims(int32_t width, int32_t height, int32_t* dims);

/* DepthMipmap::build (reference src/histogram.cpp:35-74) for ncam maps on the
 * device.  base[c] is map c's level-0 texels (host); levels_out[c] (host,
 * optional) receives all of map c's levels concatenated, level 0 first.
 * Rt_inv stays with the caller (the reference computes it with Eigen). */
int tgvg_build_pyramids(tgvg_ctx* ctx, const tgvg_camera* cams, int32_t ncam,
                        const float* const* base, float* const* levels_out);

/* compute_histograms (reference src/histogram.hpp:44-48, histogram.cpp:127-163).
 * Host buffers in and out.  base[c]: map c's level-0 texels; the pyramids are
 * built on the device.  out: n * nbins uint32.  Bit-exact with the reference
 * at nbins = 8. */
int tgvg_compute_histograms(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n,
                            const tgvg_camera* cams, int32_t ncam, const float* const* base,
                            const float origin[3], float r_root, int32_t nbins, uint32_t* out);

/* Same, for callers that already hold the pyramids (std::vector<DepthMipmap>):
 * levels[c] = map c's levels concatenated (host). */
int tgvg_compute_histograms_pyr(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n,
                                const tgvg_camera* cams, int32_t ncam,
                                const float* const* levels, const float origin[3],
                                float r_root, int32_t nbins, uint32_t* out);

/* Device-resident form: d_cubes, d_levels (all maps' pyramids back to back,
 * map c at element offset level_offset[c], host array) and d_out are device
 * pointers; runs on the context stream. */
int tgvg_compute_histograms_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, int64_t n,
                                const tgvg_camera* cams, int32_t ncam, const float* d_levels,
                                const int64_t* level_offset, const float origin[3],
                                float r_root, int32_t nbins, uint32_t* d_out);

/* No counterpart in the reference.  The device-resident histogram pass for
 * callers that cannot allocate device memory while they run: a service that
 * reserves all device memory up front for its own pool, a real-time loop where
 * an allocation's implicit synchronisation would stall other work, or a runtime
 * that routes every allocation through its own allocator.  It calls no
 * cudaMalloc/cudaFree and needs no context: d_cubes, d_base[c] (map c's level-0
 * texels) and d_out are the caller's device memory; cams stays on the host.
 * The pyramids and camera table are built in one fixed scratch array that the
 * library holds on every GPU that loads it: at most 256 cameras and
 * 16 Mi pyramid texels (64 MiB, levels 0.. of all maps together); larger
 * requests return TGVG_ERR_LIMIT.  The first call on a device looks the array
 * up on that device, which may load this library's device code and the array
 * with it: make that first call before any stream capture, and before the
 * caller reserves the device's memory for its own pool.  Work is enqueued on
 * `stream` (a cudaStream_t; null = the legacy default stream) and the call
 * returns without waiting.  The call copies the camera table from host memory
 * on `stream`, so it cannot be captured into a CUDA graph.  All calls share the
 * one array, so calls that may
 * overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  Output is bit-identical to
 * tgvg_compute_histograms_dev. */
int tgvg_compute_histograms_noalloc(const tgvg_cube* d_cubes, int64_t n, const tgvg_camera* cams,
                                    int32_t ncam, const float* const* d_base, const float origin[3],
                                    float r_root, int32_t nbins, uint32_t* d_out, void* stream);

/* compute_histograms_oc (reference src/histogram.hpp:55-61, histogram.cpp:222-256):
 * cubes from a TGV1 file, leaves from the caller, output written as a TGVH file
 * (8 bins).  The whole cube file is processed in one device pass, or in
 * batches of cubes under a device budget (tgvg_set_device_budget). */
int tgvg_compute_histograms_oc(tgvg_ctx* ctx, const char* cube_path, const tgvg_leaf* leaves,
                               int32_t nleaf, const tgvg_camera* cams, int32_t ncam,
                               const float* const* base, const float origin[3], float r_root,
                               const char* out_hist_path);

/* ---- Stage 6: TGV ------------------------------------------------------------
 * tgv_minimize / tgv_minimize_oc (reference src/tgv.hpp:31-48).  mode selects the
 * semantics (TGVG_MODE_*); leaves may be null for INMEM (one leaf covering all
 * cubes is implied).  hists: n * nbins uint32 (host).  u_init: n floats when
 * params->init == TGVG_INIT_GIVEN, else null.  out: n TGVCube records (host).
 * stats may be null. */
int tgvg_tgv_minimize(tgvg_ctx* ctx, const tgvg_cube* cubes, const uint32_t* hists, int64_t n,
                      int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, int32_t mode,
                      const tgvg_params* params, const float* u_init, tgvg_state* out,
                      tgvg_stats* stats);

/* Device-resident form: every array pointer is a device pointer (leaves stays
 * on the host).  Runs on the context stream; returns after the solve finished. */
int tgvg_tgv_minimize_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, const uint32_t* d_hists,
                          int64_t n, int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf,
                          int32_t mode, const tgvg_params* params, const float* d_u_init,
                          tgvg_state* d_out, tgvg_stats* stats);

/* Whole-state warm start (no counterpart in the reference; params->init must be
 * TGVG_INIT_STATE).  Every cube starts its own level from init_state[i] (u, v,
 * p and q of a TGVCube record) in place of the reference's parent copy of u, v
 * and zeroing of p, q (tgv.cpp:391-409, 878-934); until its level starts it
 * holds the reference's initial state (u = median indicator, v = p = q = 0),
 * so coarser levels that read it as a deeper neighbour see exactly what the
 * plain solve shows them, and every level solves the reference's problem.
 * Records equal to what the parent copy would give reproduce the plain solve;
 * all-zero records are a zero start of every level.  keep_init_u is ignored.
 * Host arrays (the _dev form: device arrays, leaves on the host), otherwise as
 * tgvg_tgv_minimize. */
int tgvg_tgv_minimize_state(tgvg_ctx* ctx, const tgvg_cube* cubes, const uint32_t* hists, int64_t n,
                            int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, int32_t mode,
                            const tgvg_params* params, const tgvg_state* init_state, tgvg_state* out,
                            tgvg_stats* stats);
int tgvg_tgv_minimize_state_dev(tgvg_ctx* ctx, const tgvg_cube* d_cubes, const uint32_t* d_hists, int64_t n,
                                int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, int32_t mode,
                                const tgvg_params* params, const tgvg_state* d_init_state, tgvg_state* d_out,
                                tgvg_stats* stats);

/* tgv_minimize_streaming (reference src/tgv.hpp:57-64, tgv.cpp:802-1070): TGV1
 * cube file, TGVH histogram file (8 bins) and TGVT treetop file in, TGVS state
 * file out.  All leaves of a level run batched in one pass on the device; the
 * result equals the reference's leaf-by-leaf order because its leaves only see
 * one another through the level-start snapshot. */
int tgvg_tgv_minimize_streaming(tgvg_ctx* ctx, const char* cube_path, const char* hist_path,
                                const char* treetop_path, const char* out_state_path,
                                const tgvg_params* params, tgvg_stats* stats);

/* ---- learned warm start (no counterpart in the reference) -------------------
 * A per-cube MLP F -> 64 -> 64 -> 1 (F = nbins + 5: histogram / total,
 * depth / 21, the cube centre's position in its chunk's node, the median
 * indicator), ReLU, BF16 weights and activations with FP32 accumulation on the
 * tensor cores.  It is trained on (features, converged u - median indicator)
 * pairs from the plain solver; the warm-start u is median indicator + network
 * (tgvg_mlp_warm_start).  Solve with params.init = TGVG_INIT_GIVEN and
 * keep_init_u = 1.  Features are 16 bf16 values per cube (uint16 bit
 * patterns, zero padded). */
typedef struct tgvg_mlp tgvg_mlp;
int tgvg_mlp_create(tgvg_ctx* ctx, int32_t nbins, uint64_t seed, tgvg_mlp** out);
int tgvg_mlp_destroy(tgvg_mlp* m);
int32_t tgvg_mlp_num_params(void);
/* Copy the fp32 parameters out (get) and/or in (set); either may be null. */
int tgvg_mlp_params(tgvg_ctx* ctx, tgvg_mlp* m, float* get, const float* set);
/* Features of n cubes (host arrays in and out). */
int tgvg_mlp_features(tgvg_ctx* ctx, const tgvg_cube* cubes, const uint32_t* hists, int64_t n,
                      int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, uint16_t* X);
/* Prediction for n feature rows (host arrays). */
int tgvg_mlp_predict(tgvg_ctx* ctx, tgvg_mlp* m, const uint16_t* X, int64_t n, float* y);
/* Warm-start u of n cubes: features, forward pass and the median indicator
 * (FP32, reference order) added, all on the device.  Host arrays in and out;
 * the _dev form takes device cubes / histograms / u and host leaves, and
 * leaves u on the context stream for tgvg_tgv_minimize_dev. */
int tgvg_mlp_warm_start(tgvg_ctx* ctx, tgvg_mlp* m, const tgvg_cube* cubes, const uint32_t* hists, int64_t n,
                        int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, float* u);
int tgvg_mlp_warm_start_dev(tgvg_ctx* ctx, tgvg_mlp* m, const tgvg_cube* d_cubes, const uint32_t* d_hists,
                            int64_t n, int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, float* d_u);
/* Gradient of the mean squared error over all n rows (for checks; host arrays). */
int tgvg_mlp_grad(tgvg_ctx* ctx, tgvg_mlp* m, const uint16_t* X, const float* t, int64_t n, float* grad,
                  float* loss);
/* Adam training over shuffled mini-batches; last_loss = mean loss of the last epoch. */
int tgvg_mlp_train(tgvg_ctx* ctx, tgvg_mlp* m, const uint16_t* X, const float* t, int64_t n, int32_t epochs,
                   int32_t batch, float lr, uint64_t seed, float* last_loss);

/* ---- Stage 1: cubes from a depth map (reference src/octree_builder.hpp) ---- */
/* One base depth map: K (fx, fy, cx, cy), Rt row-major 4x4 (world <- camera),
 * width x height depths row-major (NaN / <= 0 invalid), host memory. */
typedef struct tgvg_depthmap {
    float fx, fy, cx, cy;
    float rt[16];
    int32_t width, height;
    const float* depths;
} tgvg_depthmap;
/* build_cubes_from_depthmap (octree_builder.hpp:21-29, octree_builder.cpp:30-97):
 * one cube per valid pixel with a sample radius, at the depth
 * cube_depth_for_radius gives, sorted by Morton code (equal codes in pixel
 * order; the reference leaves their order unspecified).  `out` may be null
 * (count only); else it needs room for *count cubes (width*height always
 * suffices), else TGVG_ERR_LIMIT.  The _file form writes the TGV1 file. */
int tgvg_build_cubes(tgvg_ctx* ctx, const tgvg_depthmap* dm, const float* origin3, float r_root, tgvg_cube* out,
                     int64_t cap, int64_t* count);
int tgvg_build_cubes_file(tgvg_ctx* ctx, const tgvg_depthmap* dm, const float* origin3, float r_root,
                          const char* out_path);

/* ---- Stages 2 and 3: merge and 2:1 balance (reference src/merge.hpp,
 * src/balance.hpp) ----------------------------------------------------------
 * kway_merge (merge.hpp:6-8, merge.cpp:7-97): k code-sorted cube lists merged by
 * code; consecutive cubes with equal (code, depth) become one cube with the
 * mean r_c (float sum in merge order / count).  Equal codes from different
 * lists are taken in list order; the reference's heap takes them in an
 * unspecified order, so the results agree whenever no code occurs in two
 * lists.  `out` may be null (count only); else it needs room for *count cubes
 * (the total input count always suffices), else TGVG_ERR_LIMIT.  The file form
 * reads TGV1 files (all cubes up to the end of each file, the first file's
 * r_root) and writes one; no inputs writes an empty file with r_root 0. */
int tgvg_merge_cubes(tgvg_ctx* ctx, const tgvg_cube* const* arrays, const int64_t* counts, int32_t k,
                     tgvg_cube* out, int64_t cap, int64_t* count);
int tgvg_kway_merge(tgvg_ctx* ctx, const char* const* in_paths, int32_t k, const char* out_path);
/* balance_octree (balance.hpp:15-16, balance.cpp:60-150): the reference's
 * bridge cubes for 2:1 balance, added in its queue order, and its output
 * table: one cube per key depth << 60 | (code & (2^60 - 1)), with the mean r_c
 * of the input cubes holding the key and r_root / 2^depth for a bridge.  The
 * output cubes are decoded from the key (so codes lose bits 60..62 and depths
 * 16..21 read as 0..5, as in the reference) and sorted by code, then depth
 * (the reference leaves equal codes in hash-table order).  Every input cube
 * must have depth 0..21 and a code on its depth's grid, else
 * TGVG_ERR_INVALID.  The file form reads and writes TGV1 files. */
int tgvg_balance_cubes(tgvg_ctx* ctx, const tgvg_cube* cubes, int64_t n, float r_root, tgvg_cube* out, int64_t cap,
                       int64_t* count);
int tgvg_balance_octree(tgvg_ctx* ctx, const char* in_path, const char* out_path);

/* ---- surface extraction (reference src/marching_cubes.hpp) -----------------
 * The u = 0 iso-surface of a TGV state as an indexed quad mesh, two triangles
 * per quad, vertices merged by the reference's 60-bit quantised position.
 * Vertices, indices and normals are bit-identical to the reference's. */
typedef struct tgvg_mesh tgvg_mesh;
/* extract_surface (marching_cubes.hpp:28-33, marching_cubes.cpp:63-181), with
 * compute_normals (:185-205) when normals != 0.  has_data may be null (no
 * filter); else one byte per cube, nonzero = has votes.  Host arrays in; the
 * mesh is returned as a handle. */
int tgvg_extract_surface(tgvg_ctx* ctx, const tgvg_cube* cubes, const tgvg_state* state, int64_t n,
                         const uint8_t* has_data, const float* origin3, float r_root, int32_t normals,
                         tgvg_mesh** out);
/* The semantics of extract_surface_streaming (marching_cubes.cpp:374-580) over
 * arrays: leaves in the caller's (treetop) order, Morton-sorted cubes, votes
 * from the histograms (nbins 8 or 10); vertices are the dequantised keys. */
int tgvg_extract_surface_leaves(tgvg_ctx* ctx, const tgvg_cube* cubes, const tgvg_state* state,
                                const uint32_t* hists, int32_t nbins, int64_t n, const tgvg_leaf* leaves,
                                int32_t nleaf, const float* origin3, float r_root, tgvg_mesh** out);
/* extract_surface_streaming (marching_cubes.hpp:44-51): TGV1 cube, TGVS state,
 * TGVT treetop and TGVH histogram files in, Wavefront file out. */
int tgvg_extract_surface_streaming(tgvg_ctx* ctx, const char* balanced_cube_path, const char* tgv_state_path,
                                   const char* treetop_path, const char* hist_path, const float* origin3,
                                   float r_root, const char* out_obj_path);
int tgvg_mesh_size(const tgvg_mesh* m, int64_t* n_verts, int64_t* n_tris, int32_t* has_normals);
/* Copy out 3 floats per vertex, 3 indices per triangle, 3 floats per normal
 * (any pointer may be null). */
int tgvg_mesh_read(const tgvg_mesh* m, float* verts, uint32_t* faces, float* normals);
void tgvg_mesh_free(tgvg_mesh* m);
/* compute_normals (marching_cubes.hpp:55) over host arrays. */
int tgvg_compute_normals(tgvg_ctx* ctx, const float* verts, int64_t n_verts, const uint32_t* faces,
                         int64_t n_tris, float* normals);
/* write_obj (marching_cubes.hpp:58): `v`, `vn` when normals is non-null, `f`. */
int tgvg_write_obj(const char* path, const float* verts, int64_t n_verts, const uint32_t* faces, int64_t n_tris,
                   const float* normals);

/* ---- state / histogram files (reference tgv.cpp:24-46, histogram.cpp:175-218) */
int tgvg_save_tgv(const char* path, const tgvg_state* state, int64_t n);
/* Returns the record count (>= 0) and fills `out` when non-null (capacity cap). */
int64_t tgvg_load_tgv(const char* path, tgvg_state* out, int64_t cap);
int tgvg_save_histograms(const char* path, const uint32_t* hists, int64_t n);
int64_t tgvg_load_histograms(const char* path, uint32_t* out, int64_t cap);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* TGVG_H */
