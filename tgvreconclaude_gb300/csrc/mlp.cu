// Learned warm start: a per-cube MLP  F -> 64 -> 64 -> 1  (F = nbins + 5 inputs:
// the histogram normalised by its total, depth / 21, the cube's position inside
// its chunk's node, and the histogram's median indicator), ReLU hidden layers,
// linear output predicting the converged u minus the median indicator (the
// reference's own start), so that the warm start is median + network.  BF16 weights and activations, FP32 accumulation, on the tensor
// cores through mma.sync m16n8k16 (row.col, bf16 x bf16 -> f32).
//
// The network is under 1 % of a solve's device time (about 10 KFLOP per cube
// against ~1000 HBM-bound iterations per cube), so it uses the warp-level
// mma path; the training backward pass runs in FP32 on the CUDA cores from
// the BF16-rounded activations the forward pass produced.
//
// Fragment layouts of mma.m16n8k16 (lane t, g = t / 4, c = t % 4):
//   A (16x16, row-major): a0 = A[g][2c..2c+1], a1 = A[g+8][2c..], a2 = A[g][2c+8..], a3 = A[g+8][2c+8..]
//   B (16x8, col-major):  b0 = B[2c..2c+1][g],   b1 = B[2c+8..2c+9][g]
//   C/D (16x8, f32):      c0 = C[g][2c], c1 = C[g][2c+1], c2 = C[g+8][2c], c3 = C[g+8][2c+1]
// so the C tiles of output columns 16j..16j+15 are, packed to bf16, exactly the
// A fragment of input chunk j of the next layer.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"

namespace tgvg {

constexpr int MLP_K1 = 16;  // padded input width
constexpr int MLP_H = 64;
// fp32 master parameters
constexpr int P_W1 = 0;                  // W1[k][j], k < 16, j < 64
constexpr int P_B1 = P_W1 + MLP_K1 * MLP_H;
constexpr int P_W2 = P_B1 + MLP_H;       // W2[k][j]
constexpr int P_B2 = P_W2 + MLP_H * MLP_H;
constexpr int P_W3 = P_B2 + MLP_H;       // W3[k]
constexpr int P_B3 = P_W3 + MLP_H;
constexpr int P_N = P_B3 + 1;            // 5249
// bf16 B fragments: 64 words per (k-chunk, n-tile)
constexpr int F_W1 = 0;                  // 1 x 8 tiles
constexpr int F_W2 = F_W1 + 8 * 64;      // 4 x 8 tiles
constexpr int F_W3 = F_W2 + 32 * 64;     // 4 x 1 tile (column 0 = W3)
constexpr int F_N = F_W3 + 4 * 64;       // 2816 words

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ void mma_bf16(float& d0, float& d1, float& d2, float& d3, uint32_t a0, uint32_t a1,
                                         uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Weight fragments (and a bf16-rounded float copy used by the backward pass)
// from the fp32 master parameters.
__global__ void k_mlp_pack(const float* __restrict__ prm, uint32_t* __restrict__ frag, float* __restrict__ wr) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < P_N) wr[t] = bf16r(prm[t]);
    if (t >= F_N) return;
    const int tile = t / 64, w = t % 64, lane = w / 2, half = w % 2;
    const int g = lane / 4, c = lane % 4;
    int kc, nt, base;
    if (t < F_W2) { kc = 0; nt = tile; base = P_W1; }
    else if (t < F_W3) { kc = (tile - 8) / 8; nt = (tile - 8) % 8; base = P_W2; }
    else { kc = tile - 40; nt = 0; base = P_W3; }
    const int k = kc * 16 + 2 * c + 8 * half;
    const int n = nt * 8 + g;
    float lo, hi;
    if (base == P_W3) {
        lo = n == 0 ? prm[P_W3 + k] : 0.f;
        hi = n == 0 ? prm[P_W3 + k + 1] : 0.f;
    } else {
        lo = prm[base + k * MLP_H + n];
        hi = prm[base + (k + 1) * MLP_H + n];
    }
    frag[t] = pack_bf16(lo, hi);
}

// Features: bins / total, depth / 21, the position of the cube's centre
// inside its chunk's node (TreetopLeaf code/depth; the root without leaves) and
// the median indicator.  `med` (optional) receives the median indicator in
// FP32 as the reference computes it (src/histogram.cpp:12-31; 0 when empty).
template <int NB>
__global__ void k_mlp_features(int n, const uint4* __restrict__ cubes, const uint32_t* __restrict__ hists,
                               const int* __restrict__ leaf_id, const tgvg_leaf* __restrict__ leaves,
                               uint32_t* __restrict__ X, float* __restrict__ med) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* row = hists + (size_t)i * NB;
    float f[MLP_K1];
#pragma unroll
    for (int k = 0; k < MLP_K1; ++k) f[k] = 0.f;
    uint32_t tot = 0;
#pragma unroll
    for (int k = 0; k < NB; ++k) tot += row[k];
    const float inv = tot ? 1.0f / (float)tot : 0.f;
    uint32_t cum = 0;
    int km = -1;
#pragma unroll
    for (int k = 0; k < NB; ++k) {
        f[k] = (float)row[k] * inv;
        cum += row[k];
        if (km < 0 && cum * 2 >= tot) km = k;
    }
    const float m = tot ? fadd(-1.0f, fdiv(fadd((float)km, 0.5f), NB / 2.0f)) : 0.0f;
    f[NB + 4] = m;
    if (med) med[i] = m;
    const uint4 cb = cubes[i];
    const uint64_t key = (uint64_t(cb.x) << 32) | cb.y;
    const int d = min(21, max(0, (int)cb.w));
    f[NB] = d / 21.0f;
    uint64_t nkey = 0;
    int nd = 0;
    const int l = leaf_id ? leaf_id[i] : -1;
    if (l >= 0) { nkey = (uint64_t(leaves[l].hi) << 32) | leaves[l].lo; nd = min(21, max(0, leaves[l].depth)); }
    const float nsize = (float)(1u << (21 - nd)), half = 0.5f * (float)(1u << (21 - d));
    const uint32_t cx = gather3(key), cy = gather3(key >> 1), cz = gather3(key >> 2);
    const uint32_t nx = gather3(nkey), ny = gather3(nkey >> 1), nz = gather3(nkey >> 2);
    f[NB + 1] = fminf(fmaxf(((float)cx - (float)nx + half) / nsize, 0.f), 1.f);
    f[NB + 2] = fminf(fmaxf(((float)cy - (float)ny + half) / nsize, 0.f), 1.f);
    f[NB + 3] = fminf(fmaxf(((float)cz - (float)nz + half) / nsize, 0.f), 1.f);
    uint32_t* out = X + (size_t)i * 8;
#pragma unroll
    for (int k = 0; k < 8; ++k) out[k] = pack_bf16(f[2 * k], f[2 * k + 1]);
}

__global__ void k_leaf_id(int n, int nleaf, const tgvg_leaf* __restrict__ leaves, int* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int id = -1;
    for (int l = 0; l < nleaf; ++l)
        if ((uint32_t)i >= leaves[l].first_idx && (uint32_t)i <= leaves[l].last_idx) { id = l; break; }
    out[i] = id;
}

// One warp's forward pass over a 16-row tile whose input is the A fragment
// a0..a3.  Returns y for rows g and g+8 in y0/y1 (valid on lanes with c == 0);
// with SAVE it also stores the bf16-rounded hidden activations (as float,
// [16][64] each) for the backward pass.
template <bool SAVE>
__device__ __forceinline__ void mlp_tile(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         const uint32_t* __restrict__ sfrag, const float* __restrict__ sbias,
                                         float& y0, float& y1, float* h1s, float* h2s) {
    const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
    uint32_t h[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bl = sbias[nt * 8 + 2 * c], bh = sbias[nt * 8 + 2 * c + 1];
        float d0 = bl, d1 = bh, d2 = bl, d3 = bh;
        const uint32_t* bf = sfrag + F_W1 + nt * 64 + lane * 2;
        mma_bf16(d0, d1, d2, d3, a0, a1, a2, a3, bf[0], bf[1]);
        d0 = fmaxf(d0, 0.f); d1 = fmaxf(d1, 0.f); d2 = fmaxf(d2, 0.f); d3 = fmaxf(d3, 0.f);
        if (SAVE) {
            const int col = nt * 8 + 2 * c;
            h1s[g * 64 + col] = bf16r(d0); h1s[g * 64 + col + 1] = bf16r(d1);
            h1s[(g + 8) * 64 + col] = bf16r(d2); h1s[(g + 8) * 64 + col + 1] = bf16r(d3);
        }
        const int kc = nt >> 1;
        if ((nt & 1) == 0) { h[kc][0] = pack_bf16(d0, d1); h[kc][1] = pack_bf16(d2, d3); }
        else { h[kc][2] = pack_bf16(d0, d1); h[kc][3] = pack_bf16(d2, d3); }
    }
    uint32_t h2[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bl = sbias[64 + nt * 8 + 2 * c], bh = sbias[64 + nt * 8 + 2 * c + 1];
        float d0 = bl, d1 = bh, d2 = bl, d3 = bh;
#pragma unroll
        for (int kc = 0; kc < 4; ++kc) {
            const uint32_t* bf = sfrag + F_W2 + (kc * 8 + nt) * 64 + lane * 2;
            mma_bf16(d0, d1, d2, d3, h[kc][0], h[kc][1], h[kc][2], h[kc][3], bf[0], bf[1]);
        }
        d0 = fmaxf(d0, 0.f); d1 = fmaxf(d1, 0.f); d2 = fmaxf(d2, 0.f); d3 = fmaxf(d3, 0.f);
        if (SAVE) {
            const int col = nt * 8 + 2 * c;
            h2s[g * 64 + col] = bf16r(d0); h2s[g * 64 + col + 1] = bf16r(d1);
            h2s[(g + 8) * 64 + col] = bf16r(d2); h2s[(g + 8) * 64 + col + 1] = bf16r(d3);
        }
        const int kc = nt >> 1;
        if ((nt & 1) == 0) { h2[kc][0] = pack_bf16(d0, d1); h2[kc][1] = pack_bf16(d2, d3); }
        else { h2[kc][2] = pack_bf16(d0, d1); h2[kc][3] = pack_bf16(d2, d3); }
    }
    const float b3 = (c == 0) ? sbias[128] : 0.f;
    float d0 = b3, d1 = 0.f, d2 = b3, d3 = 0.f;
#pragma unroll
    for (int kc = 0; kc < 4; ++kc) {
        const uint32_t* bf = sfrag + F_W3 + kc * 64 + lane * 2;
        mma_bf16(d0, d1, d2, d3, h2[kc][0], h2[kc][1], h2[kc][2], h2[kc][3], bf[0], bf[1]);
    }
    y0 = d0;
    y1 = d2;
}

__device__ __forceinline__ void load_net(const uint32_t* __restrict__ frag, const float* __restrict__ prm,
                                         uint32_t* sfrag, float* sbias) {
    for (int w = threadIdx.x; w < F_N; w += blockDim.x) sfrag[w] = frag[w];
    for (int k = threadIdx.x; k < 64; k += blockDim.x) {
        sbias[k] = prm[P_B1 + k];
        sbias[64 + k] = prm[P_B2 + k];
    }
    if (threadIdx.x == 0) sbias[128] = prm[P_B3];
    __syncthreads();
}

// Inference: y[i] for i < n, plus base[i] when base is given.
__global__ void __launch_bounds__(256) k_mlp_forward(const uint32_t* __restrict__ X, int n,
                                                     const uint32_t* __restrict__ frag,
                                                     const float* __restrict__ prm, const float* __restrict__ base,
                                                     float* __restrict__ y) {
    __shared__ uint32_t sfrag[F_N];
    __shared__ float sbias[132];
    load_net(frag, prm, sfrag, sbias);
    const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n; tile += warps) {
        const int r0 = tile * 16 + g, r1 = r0 + 8;
        uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        if (r0 < n) { a0 = X[(size_t)r0 * 8 + c]; a2 = X[(size_t)r0 * 8 + c + 4]; }
        if (r1 < n) { a1 = X[(size_t)r1 * 8 + c]; a3 = X[(size_t)r1 * 8 + c + 4]; }
        float y0, y1;
        mlp_tile<false>(a0, a1, a2, a3, sfrag, sbias, y0, y1, nullptr, nullptr);
        if (c == 0) {
            if (r0 < n) y[r0] = base ? fadd(base[r0], y0) : y0;
            if (r1 < n) y[r1] = base ? fadd(base[r1], y1) : y1;
        }
    }
}

// Gradient of the mean squared error over rows idx[0..m) (idx may be null:
// rows 0..m).  Gradients and the loss sum are added into grad[P_N] and loss[0].
constexpr int TRAIN_WARPS = 4;
__global__ void __launch_bounds__(TRAIN_WARPS * 32) k_mlp_grad(const uint32_t* __restrict__ X, const float* __restrict__ t,
                                                              const int* __restrict__ idx, int m, float inv_m,
                                                              const uint32_t* __restrict__ frag,
                                                              const float* __restrict__ prm,
                                                              const float* __restrict__ wr, float* __restrict__ grad,
                                                              float* __restrict__ loss) {
    extern __shared__ float smem[];
    uint32_t* sfrag = reinterpret_cast<uint32_t*>(smem);           // F_N
    float* sbias = smem + F_N;                                      // 132
    float* sg = sbias + 132;                                        // P_N block gradient
    float* swr = sg + P_N;                                          // P_N rounded weights
    float* wbase = swr + P_N;                                       // per warp: X 256, h1 1024, h2 1024, dz2 1024, y/t 32
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
    float* xs = wbase + warp * (256 + 3 * 1024 + 32);
    float* h1s = xs + 256;
    float* h2s = h1s + 1024;
    float* dz2 = h2s + 1024;
    float* dys = dz2 + 1024;
    load_net(frag, prm, sfrag, sbias);
    for (int k = threadIdx.x; k < P_N; k += blockDim.x) { sg[k] = 0.f; swr[k] = wr[k]; }
    __syncthreads();
    const int warps = gridDim.x * TRAIN_WARPS;
    float lsum = 0.f;
    for (int tile = blockIdx.x * TRAIN_WARPS + warp; tile * 16 < m; tile += warps) {
        // stage this tile's X rows (bf16 -> float) and its row indices
        int rows[2] = {-1, -1};
        for (int rr = 0; rr < 2; ++rr) {
            const int s = g + 8 * rr;
            const int b = tile * 16 + s;
            rows[rr] = b < m ? (idx ? idx[b] : b) : -1;
        }
        // X as float for the dW1 term (lanes c cover words 2c, 2c+1 of each row)
        for (int rr = 0; rr < 2; ++rr) {
            const int s = g + 8 * rr;
            for (int wi = 0; wi < 2; ++wi) {
                const int word = c * 2 + wi;
                float lo = 0.f, hi = 0.f;
                if (rows[rr] >= 0) {
                    uint32_t v = X[(size_t)rows[rr] * 8 + word];
                    __nv_bfloat162 b2 = *reinterpret_cast<__nv_bfloat162*>(&v);
                    lo = __bfloat162float(b2.x); hi = __bfloat162float(b2.y);
                }
                xs[s * 16 + 2 * word] = lo;
                xs[s * 16 + 2 * word + 1] = hi;
            }
        }
        __syncwarp();
        // forward on the staged rows (already bf16 values, so packing is exact)
        float y0, y1;
        mlp_tile<true>(pack_bf16(xs[g * 16 + 2 * c], xs[g * 16 + 2 * c + 1]),
                       pack_bf16(xs[(g + 8) * 16 + 2 * c], xs[(g + 8) * 16 + 2 * c + 1]),
                       pack_bf16(xs[g * 16 + 2 * c + 8], xs[g * 16 + 2 * c + 9]),
                       pack_bf16(xs[(g + 8) * 16 + 2 * c + 8], xs[(g + 8) * 16 + 2 * c + 9]), sfrag, sbias, y0, y1,
                       h1s, h2s);
        // dy = 2 (y - t) / m on lanes c == 0
        if (c == 0) {
            for (int rr = 0; rr < 2; ++rr) {
                const int s = g + 8 * rr;
                float dy = 0.f;
                if (rows[rr] >= 0) {
                    const float e = (rr ? y1 : y0) - t[rows[rr]];
                    lsum += e * e;
                    dy = 2.f * e * inv_m;
                }
                dys[s] = dy;
            }
        }
        __syncwarp();
        // W3, b3 and dZ2 (lane owns hidden columns lane and lane + 32)
        for (int jj = 0; jj < 2; ++jj) {
            const int j = lane + 32 * jj;
            float gw = 0.f;
            for (int s = 0; s < 16; ++s) {
                const float hv = h2s[s * 64 + j];
                gw += hv * dys[s];
                dz2[s * 64 + j] = hv > 0.f ? dys[s] * swr[P_W3 + j] : 0.f;
            }
            atomicAdd(&sg[P_W3 + j], gw);
        }
        if (lane == 0) {
            float gb = 0.f;
            for (int s = 0; s < 16; ++s) gb += dys[s];
            atomicAdd(&sg[P_B3], gb);
        }
        __syncwarp();
        // W2 (k rows x j = lane, lane + 32), b2, and dZ1 into h1s (overwritten in place)
        for (int jj = 0; jj < 2; ++jj) {
            const int j = lane + 32 * jj;
            float gb = 0.f;
            for (int s = 0; s < 16; ++s) gb += dz2[s * 64 + j];
            atomicAdd(&sg[P_B2 + j], gb);
            for (int k = 0; k < 64; ++k) {
                float acc = 0.f;
                for (int s = 0; s < 16; ++s) acc += h1s[s * 64 + k] * dz2[s * 64 + j];
                atomicAdd(&sg[P_W2 + k * 64 + j], acc);
            }
        }
        __syncwarp();
        float dz1v[2][16];
        for (int kk = 0; kk < 2; ++kk) {
            const int k = lane + 32 * kk;
            for (int s = 0; s < 16; ++s) {
                float acc = 0.f;
                for (int j = 0; j < 64; ++j) acc += dz2[s * 64 + j] * swr[P_W2 + k * 64 + j];
                dz1v[kk][s] = h1s[s * 64 + k] > 0.f ? acc : 0.f;
            }
        }
        // W1 (16 inputs x k = lane, lane + 32) and b1
        for (int kk = 0; kk < 2; ++kk) {
            const int k = lane + 32 * kk;
            float gb = 0.f;
            for (int s = 0; s < 16; ++s) gb += dz1v[kk][s];
            atomicAdd(&sg[P_B1 + k], gb);
            for (int i = 0; i < MLP_K1; ++i) {
                float acc = 0.f;
                for (int s = 0; s < 16; ++s) acc += xs[s * 16 + i] * dz1v[kk][s];
                atomicAdd(&sg[P_W1 + i * 64 + k], acc);
            }
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0) atomicAdd(loss, lsum);
    __syncthreads();
    for (int k = threadIdx.x; k < P_N; k += blockDim.x) atomicAdd(&grad[k], sg[k]);
}

__global__ void k_adam(float* __restrict__ prm, float* __restrict__ m1, float* __restrict__ m2,
                       const float* __restrict__ grad, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P_N) return;
    const float gk = grad[k];
    const float a = b1 * m1[k] + (1.f - b1) * gk;
    const float b = b2 * m2[k] + (1.f - b2) * gk * gk;
    m1[k] = a;
    m2[k] = b;
    prm[k] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

}  // namespace tgvg

// ------------------------------------------------------------------ C ABI ---
using namespace tgvg;

struct tgvg_mlp {
    int nbins;
    float* d_prm = nullptr;
    float* d_m1 = nullptr;
    float* d_m2 = nullptr;
    float* d_grad = nullptr;
    float* d_wr = nullptr;
    float* d_loss = nullptr;
    uint32_t* d_frag = nullptr;
    int step = 0;
};

static constexpr size_t GRAD_SMEM = sizeof(float) * (F_N + 132 + 2 * P_N + TRAIN_WARPS * (256 + 3 * 1024 + 32));

static int mlp_repack(tgvg_ctx* ctx, tgvg_mlp* m) {
    k_mlp_pack<<<(P_N + 255) / 256, 256, 0, ctx->stream>>>(m->d_prm, m->d_frag, m->d_wr);
    TGVG_LAUNCHED(ctx);
    return TGVG_OK;
}

extern "C" int tgvg_mlp_create(tgvg_ctx* ctx, int32_t nbins, uint64_t seed, tgvg_mlp** out) {
    if (!ctx || !out || (nbins != 8 && nbins != 10)) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto* m = new tgvg_mlp();
    m->nbins = nbins;
    float** bufs[] = {&m->d_prm, &m->d_m1, &m->d_m2, &m->d_grad, &m->d_wr};
    for (float** b : bufs)
        if (cudaMalloc(b, sizeof(float) * P_N) != cudaSuccess) { delete m; return TGVG_ERR_NOMEM; }
    if (cudaMalloc(&m->d_loss, sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->d_frag, sizeof(uint32_t) * F_N) != cudaSuccess) {
        delete m;
        return TGVG_ERR_NOMEM;
    }
    // He-uniform weights over the real fan-in (the padded inputs stay zero), zero biases.
    std::mt19937_64 rng(seed);
    std::vector<float> p(P_N, 0.f);
    const int fan1 = nbins + 4;
    std::uniform_real_distribution<float> u1(-std::sqrt(6.f / fan1), std::sqrt(6.f / fan1));
    std::uniform_real_distribution<float> u2(-std::sqrt(6.f / 64), std::sqrt(6.f / 64));
    std::uniform_real_distribution<float> u3(-std::sqrt(3.f / 64), std::sqrt(3.f / 64));
    for (int k = 0; k < fan1; ++k)
        for (int j = 0; j < 64; ++j) p[P_W1 + k * 64 + j] = u1(rng);
    for (int k = 0; k < 64 * 64; ++k) p[P_W2 + k] = u2(rng);
    for (int k = 0; k < 64; ++k) p[P_W3 + k] = u3(rng);
    TGVG_CK(ctx, cudaMemcpyAsync(m->d_prm, p.data(), sizeof(float) * P_N, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaMemsetAsync(m->d_m1, 0, sizeof(float) * P_N, ctx->stream));
    TGVG_CK(ctx, cudaMemsetAsync(m->d_m2, 0, sizeof(float) * P_N, ctx->stream));
    int rc = mlp_repack(ctx, m);
    if (rc) return rc;
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    *out = m;
    return TGVG_OK;
}

extern "C" int tgvg_mlp_destroy(tgvg_mlp* m) {
    if (!m) return TGVG_ERR_INVALID;
    cudaFree(m->d_prm); cudaFree(m->d_m1); cudaFree(m->d_m2); cudaFree(m->d_grad); cudaFree(m->d_wr);
    cudaFree(m->d_loss); cudaFree(m->d_frag);
    delete m;
    return TGVG_OK;
}

extern "C" int32_t tgvg_mlp_num_params(void) { return P_N; }

extern "C" int tgvg_mlp_params(tgvg_ctx* ctx, tgvg_mlp* m, float* get, const float* set) {
    if (!ctx || !m) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set) {
        TGVG_CK(ctx, cudaMemcpyAsync(m->d_prm, set, sizeof(float) * P_N, cudaMemcpyHostToDevice, ctx->stream));
        int rc = mlp_repack(ctx, m);
        if (rc) return rc;
    }
    if (get) TGVG_CK(ctx, cudaMemcpyAsync(get, m->d_prm, sizeof(float) * P_N, cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

extern "C" int tgvg_mlp_features(tgvg_ctx* ctx, const tgvg_cube* cubes, const uint32_t* hists, int64_t n,
                                 int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, uint16_t* X) {
    if (!ctx || n < 0 || (n > 0 && (!cubes || !hists || !X)) || (nbins != 8 && nbins != 10) || nleaf < 0 ||
        (nleaf > 0 && !leaves) || n > (int64_t(1) << 30))
        return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (n == 0) return TGVG_OK;
    auto* d_c = (tgvg_cube*)ctx->buf(B_T_CUBES, sizeof(tgvg_cube) * n);
    auto* d_h = (uint32_t*)ctx->buf(B_T_HISTS, sizeof(uint32_t) * nbins * n);
    auto* d_x = (uint32_t*)ctx->buf(B_M_X, sizeof(uint32_t) * 8 * n);
    auto* d_l = (tgvg_leaf*)ctx->buf(B_M_LEAVES, sizeof(tgvg_leaf) * std::max(1, nleaf));
    auto* d_id = (int*)ctx->buf(B_M_LEAFID, sizeof(int) * n);
    if (!d_c || !d_h || !d_x || !d_l || !d_id) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemcpyAsync(d_c, cubes, sizeof(tgvg_cube) * n, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaMemcpyAsync(d_h, hists, sizeof(uint32_t) * nbins * n, cudaMemcpyHostToDevice, ctx->stream));
    if (nleaf > 0)
        TGVG_CK(ctx, cudaMemcpyAsync(d_l, leaves, sizeof(tgvg_leaf) * nleaf, cudaMemcpyHostToDevice, ctx->stream));
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (nleaf > 0) {
        k_leaf_id<<<grid, 256, 0, ctx->stream>>>((int)n, nleaf, d_l, d_id);
        TGVG_LAUNCHED(ctx);
    }
    if (nbins == 8)
        k_mlp_features<8><<<grid, 256, 0, ctx->stream>>>((int)n, reinterpret_cast<const uint4*>(d_c), d_h,
                                                         nleaf > 0 ? d_id : nullptr, d_l, d_x, nullptr);
    else
        k_mlp_features<10><<<grid, 256, 0, ctx->stream>>>((int)n, reinterpret_cast<const uint4*>(d_c), d_h,
                                                          nleaf > 0 ? d_id : nullptr, d_l, d_x, nullptr);
    TGVG_LAUNCHED(ctx);
    TGVG_CK(ctx, cudaMemcpyAsync(X, d_x, sizeof(uint32_t) * 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

extern "C" int tgvg_mlp_predict(tgvg_ctx* ctx, tgvg_mlp* m, const uint16_t* X, int64_t n, float* y) {
    if (!ctx || !m || n < 0 || (n > 0 && (!X || !y)) || n > (int64_t(1) << 30)) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (n == 0) return TGVG_OK;
    auto* d_x = (uint32_t*)ctx->buf(B_M_X, sizeof(uint32_t) * 8 * n);
    auto* d_y = (float*)ctx->buf(B_M_Y, sizeof(float) * n);
    if (!d_x || !d_y) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemcpyAsync(d_x, X, sizeof(uint32_t) * 8 * n, cudaMemcpyHostToDevice, ctx->stream));
    const int tiles = (int)((n + 15) / 16);
    const unsigned grid = (unsigned)std::min((tiles + 7) / 8, ctx->sm_count * 8);
    k_mlp_forward<<<grid, 256, 0, ctx->stream>>>(d_x, (int)n, m->d_frag, m->d_prm, nullptr, d_y);
    TGVG_LAUNCHED(ctx);
    TGVG_CK(ctx, cudaMemcpyAsync(y, d_y, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

// Warm-start u on the device: features, forward pass, plus the median
// indicator (u = median + network).  Device cubes / histograms / output, host
// leaves.  Called with ctx->mu held.
static int warm_start_dev(tgvg_ctx* ctx, tgvg_mlp* m, const tgvg_cube* d_c, const uint32_t* d_h, int64_t n,
                          int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, float* d_u) {
    auto* d_x = (uint32_t*)ctx->buf(B_M_X, sizeof(uint32_t) * 8 * n);
    auto* d_med = (float*)ctx->buf(B_M_T, sizeof(float) * n);
    auto* d_l = (tgvg_leaf*)ctx->buf(B_M_LEAVES, sizeof(tgvg_leaf) * std::max(1, nleaf));
    auto* d_id = (int*)ctx->buf(B_M_LEAFID, sizeof(int) * n);
    if (!d_x || !d_med || !d_l || !d_id) return TGVG_ERR_NOMEM;
    if (nleaf > 0)
        TGVG_CK(ctx, cudaMemcpyAsync(d_l, leaves, sizeof(tgvg_leaf) * nleaf, cudaMemcpyHostToDevice, ctx->stream));
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (nleaf > 0) {
        k_leaf_id<<<grid, 256, 0, ctx->stream>>>((int)n, nleaf, d_l, d_id);
        TGVG_LAUNCHED(ctx);
    }
    if (nbins == 8)
        k_mlp_features<8><<<grid, 256, 0, ctx->stream>>>((int)n, reinterpret_cast<const uint4*>(d_c), d_h,
                                                         nleaf > 0 ? d_id : nullptr, d_l, d_x, d_med);
    else
        k_mlp_features<10><<<grid, 256, 0, ctx->stream>>>((int)n, reinterpret_cast<const uint4*>(d_c), d_h,
                                                          nleaf > 0 ? d_id : nullptr, d_l, d_x, d_med);
    TGVG_LAUNCHED(ctx);
    const int tiles = (int)((n + 15) / 16);
    const unsigned fgrid = (unsigned)std::min((tiles + 7) / 8, ctx->sm_count * 8);
    k_mlp_forward<<<fgrid, 256, 0, ctx->stream>>>(d_x, (int)n, m->d_frag, m->d_prm, d_med, d_u);
    TGVG_LAUNCHED(ctx);
    return TGVG_OK;
}

static bool warm_start_args_ok(tgvg_ctx* ctx, tgvg_mlp* m, const void* c, const void* h, int64_t n, int32_t nbins,
                               const tgvg_leaf* leaves, int32_t nleaf, const void* u) {
    return ctx && m && n >= 0 && (n == 0 || (c && h && u)) && (nbins == 8 || nbins == 10) && nbins == m->nbins &&
           nleaf >= 0 && (nleaf == 0 || leaves) && n <= (int64_t(1) << 30);
}

extern "C" int tgvg_mlp_warm_start(tgvg_ctx* ctx, tgvg_mlp* m, const tgvg_cube* cubes, const uint32_t* hists,
                                   int64_t n, int32_t nbins, const tgvg_leaf* leaves, int32_t nleaf, float* u) {
    if (!warm_start_args_ok(ctx, m, cubes, hists, n, nbins, leaves, nleaf, u)) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (n == 0) return TGVG_OK;
    auto* d_c = (tgvg_cube*)ctx->buf(B_T_CUBES, sizeof(tgvg_cube) * n);
    auto* d_h = (uint32_t*)ctx->buf(B_T_HISTS, sizeof(uint32_t) * nbins * n);
    auto* d_u = (float*)ctx->buf(B_M_Y, sizeof(float) * n);
    if (!d_c || !d_h || !d_u) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemcpyAsync(d_c, cubes, sizeof(tgvg_cube) * n, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaMemcpyAsync(d_h, hists, sizeof(uint32_t) * nbins * n, cudaMemcpyHostToDevice, ctx->stream));
    int rc = warm_start_dev(ctx, m, d_c, d_h, n, nbins, leaves, nleaf, d_u);
    if (rc) return rc;
    TGVG_CK(ctx, cudaMemcpyAsync(u, d_u, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

extern "C" int tgvg_mlp_warm_start_dev(tgvg_ctx* ctx, tgvg_mlp* m, const tgvg_cube* d_cubes,
                                       const uint32_t* d_hists, int64_t n, int32_t nbins, const tgvg_leaf* leaves,
                                       int32_t nleaf, float* d_u) {
    if (!warm_start_args_ok(ctx, m, d_cubes, d_hists, n, nbins, leaves, nleaf, d_u)) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (n == 0) return TGVG_OK;
    return warm_start_dev(ctx, m, d_cubes, d_hists, n, nbins, leaves, nleaf, d_u);
}

// Gradient of the mean squared error of the whole set (one batch), for checks.
extern "C" int tgvg_mlp_grad(tgvg_ctx* ctx, tgvg_mlp* m, const uint16_t* X, const float* t, int64_t n,
                             float* grad, float* loss) {
    if (!ctx || !m || n <= 0 || !X || !t || !grad || n > (int64_t(1) << 30)) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto* d_x = (uint32_t*)ctx->buf(B_M_X, sizeof(uint32_t) * 8 * n);
    auto* d_t = (float*)ctx->buf(B_M_T, sizeof(float) * n);
    if (!d_x || !d_t) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemcpyAsync(d_x, X, sizeof(uint32_t) * 8 * n, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaMemcpyAsync(d_t, t, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaMemsetAsync(m->d_grad, 0, sizeof(float) * P_N, ctx->stream));
    TGVG_CK(ctx, cudaMemsetAsync(m->d_loss, 0, sizeof(float), ctx->stream));
    TGVG_CK(ctx, cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GRAD_SMEM));
    const int tiles = (int)((n + 15) / 16);
    const unsigned grid = (unsigned)std::max(1, std::min((tiles + TRAIN_WARPS - 1) / TRAIN_WARPS, ctx->sm_count * 2));
    k_mlp_grad<<<grid, TRAIN_WARPS * 32, GRAD_SMEM, ctx->stream>>>(d_x, d_t, nullptr, (int)n, 1.0f / (float)n,
                                                                  m->d_frag, m->d_prm, m->d_wr, m->d_grad, m->d_loss);
    TGVG_LAUNCHED(ctx);
    TGVG_CK(ctx, cudaMemcpyAsync(grad, m->d_grad, sizeof(float) * P_N, cudaMemcpyDeviceToHost, ctx->stream));
    float l = 0.f;
    TGVG_CK(ctx, cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (loss) *loss = l / (float)n;
    return TGVG_OK;
}

// Adam on the mean squared error over shuffled mini-batches; returns the mean
// loss of the last epoch.
extern "C" int tgvg_mlp_train(tgvg_ctx* ctx, tgvg_mlp* m, const uint16_t* X, const float* t, int64_t n,
                              int32_t epochs, int32_t batch, float lr, uint64_t seed, float* last_loss) {
    if (!ctx || !m || n <= 0 || !X || !t || epochs < 0 || batch <= 0 || n > (int64_t(1) << 30))
        return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto* d_x = (uint32_t*)ctx->buf(B_M_X, sizeof(uint32_t) * 8 * n);
    auto* d_t = (float*)ctx->buf(B_M_T, sizeof(float) * n);
    auto* d_idx = (int*)ctx->buf(B_M_IDX, sizeof(int) * n);
    if (!d_x || !d_t || !d_idx) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemcpyAsync(d_x, X, sizeof(uint32_t) * 8 * n, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaMemcpyAsync(d_t, t, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    TGVG_CK(ctx, cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GRAD_SMEM));
    std::vector<int> perm(n);
    for (int64_t i = 0; i < n; ++i) perm[i] = (int)i;
    std::mt19937_64 rng(seed);
    float epoch_loss = 0.f;
    for (int e = 0; e < epochs; ++e) {
        std::shuffle(perm.begin(), perm.end(), rng);
        TGVG_CK(ctx, cudaMemcpyAsync(d_idx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
        TGVG_CK(ctx, cudaMemsetAsync(m->d_loss, 0, sizeof(float), ctx->stream));
        for (int64_t b0 = 0; b0 < n; b0 += batch) {
            const int mb = (int)std::min<int64_t>(batch, n - b0);
            TGVG_CK(ctx, cudaMemsetAsync(m->d_grad, 0, sizeof(float) * P_N, ctx->stream));
            const int tiles = (mb + 15) / 16;
            const unsigned grid = (unsigned)std::max(1, std::min((tiles + TRAIN_WARPS - 1) / TRAIN_WARPS,
                                                                 ctx->sm_count * 2));
            k_mlp_grad<<<grid, TRAIN_WARPS * 32, GRAD_SMEM, ctx->stream>>>(
                d_x, d_t, d_idx + b0, mb, 1.0f / (float)mb, m->d_frag, m->d_prm, m->d_wr, m->d_grad, m->d_loss);
            TGVG_LAUNCHED(ctx);
            ++m->step;
            const float c1 = 1.f - std::pow(0.9f, (float)m->step), c2 = 1.f - std::pow(0.999f, (float)m->step);
            k_adam<<<(P_N + 255) / 256, 256, 0, ctx->stream>>>(m->d_prm, m->d_m1, m->d_m2, m->d_grad, lr, 0.9f,
                                                               0.999f, 1e-8f, c1, c2);
            TGVG_LAUNCHED(ctx);
            int rc = mlp_repack(ctx, m);
            if (rc) return rc;
        }
        float l = 0.f;
        TGVG_CK(ctx, cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
        epoch_loss = l / (float)n;
    }
    if (last_loss) *last_loss = epoch_loss;
    return TGVG_OK;
}
