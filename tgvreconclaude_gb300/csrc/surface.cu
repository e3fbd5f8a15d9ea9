// Surface extraction on the GPU: the u = 0 iso-surface of a TGV state as an
// indexed quad mesh, with the semantics of the reference's
// src/marching_cubes.cpp (extract_surface :63-181, compute_normals :185-205,
// extract_surface_streaming :374-580, write_obj :584-619).
//
// For every cube and face, the neighbour is resolved by code (as the TGV
// setup does), and a face pair whose u changes sign contributes one quad at
// the interpolated zero crossing.  The reference walks cubes and faces in
// order and keeps hash maps of emitted pairs and of vertices; here every
// (cube, face) slot decides in parallel whether it is the pair's emitter,
// an exclusive scan over the slots gives each quad its place in the
// reference's emission order, and vertices are merged through a device hash
// table keyed by the reference's 60-bit quantised position, numbered by first
// occurrence with a second scan.  Float arithmetic uses explicitly rounded
// intrinsics in the reference's expression order, so positions, indices and
// normals are bit-identical to the reference's.
//
//   S1 k_surf_prep       keys, depth check, u gathered from the 13-float state
//   S2 k_surf_hash       code -> smallest / largest index
//   S3 k_surf_nbrs<STR>  resolved neighbour per (cube, face)
//   S4 k_surf_flags<STR> emitter test per (cube, face)
//   S5 k_surf_quads<STR> four corners, keys and winding per quad
//   S6 k_vert_*          vertex merge and numbering; k_faces: index triangles
//   S7 k_tri_normal / k_vert_normal: per-vertex normals in triangle order
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "fileio.h"

struct tgvg_mesh {
    std::vector<float> verts;     // 3 per vertex
    std::vector<uint32_t> faces;  // 3 per triangle
    std::vector<float> normals;   // 3 per vertex, or empty
};

namespace tgvg {

// ------------------------------------------------------- exclusive scan ---
static constexpr int SCAN_THREADS = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void k_scan_tiles(const int* __restrict__ in, int64_t n, int* __restrict__ sums) {
    __shared__ int ws[SCAN_THREADS / 32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const int64_t i = base + (int64_t)k * SCAN_THREADS + threadIdx.x;
        if (i < n) s += in[i];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < SCAN_THREADS / 32; ++w) t += ws[w];
        sums[blockIdx.x] = t;
    }
}

// One block: exclusive scan of nt tile sums in place; sums[nt] = total.
__global__ void k_scan_sums(int* __restrict__ sums, int nt) {
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int per = (nt + 1023) / 1024;
    const int a = min(nt, t * per), b = min(nt, a + per);
    int s = 0;
    for (int k = a; k < b; ++k) s += sums[k];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int v = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;
    for (int k = a; k < b; ++k) { const int c = sums[k]; sums[k] = run; run += c; }
    if (t == 1023) sums[nt] = part[1023];
}

__global__ void k_scan_apply(const int* __restrict__ in, int64_t n, const int* __restrict__ offs,
                             int* __restrict__ out) {
    __shared__ int ws[SCAN_THREADS / 32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = s;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int z = lane < SCAN_THREADS / 32 ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o) z += y;
        }
        if (lane < SCAN_THREADS / 32) ws[lane] = z;
    }
    __syncthreads();
    int run = x - s + (w > 0 ? ws[w - 1] : 0) + offs[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

// out[i] = sum of in[0..i) for i < n, enqueued only (no host synchronisation,
// so it can be captured into a CUDA graph); sums holds scan_sums_len(n) ints.
int64_t scan_sums_len(int64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }
int scan_exclusive_async(tgvg_ctx* ctx, const int* d_in, int64_t n, int* d_out, int* sums) {
    if (n <= 0) return TGVG_OK;
    const int64_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nt > (int64_t(1) << 30)) return ctx->fail(TGVG_ERR_LIMIT, "scan too long");
    k_scan_tiles<<<(unsigned)nt, SCAN_THREADS, 0, ctx->stream>>>(d_in, n, sums);
    TGVG_LAUNCHED(ctx);
    k_scan_sums<<<1, 1024, 0, ctx->stream>>>(sums, (int)nt);
    TGVG_LAUNCHED(ctx);
    k_scan_apply<<<(unsigned)nt, SCAN_THREADS, 0, ctx->stream>>>(d_in, n, sums, d_out);
    TGVG_LAUNCHED(ctx);
    return TGVG_OK;
}

// out[i] = sum of in[0..i) for i < n; returns the total through *total (host).
int scan_exclusive(tgvg_ctx* ctx, const int* d_in, int64_t n, int* d_out, int64_t* total) {
    *total = 0;
    if (n <= 0) return TGVG_OK;
    const int64_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nt > (int64_t(1) << 30)) return ctx->fail(TGVG_ERR_LIMIT, "scan too long");
    auto* sums = (int*)ctx->buf(B_S_SCAN, sizeof(int) * (nt + 1));
    if (!sums) return TGVG_ERR_NOMEM;
    k_scan_tiles<<<(unsigned)nt, SCAN_THREADS, 0, ctx->stream>>>(d_in, n, sums);
    TGVG_LAUNCHED(ctx);
    k_scan_sums<<<1, 1024, 0, ctx->stream>>>(sums, (int)nt);
    TGVG_LAUNCHED(ctx);
    k_scan_apply<<<(unsigned)nt, SCAN_THREADS, 0, ctx->stream>>>(d_in, n, sums, d_out);
    TGVG_LAUNCHED(ctx);
    int h = 0;
    TGVG_CK(ctx, cudaMemcpyAsync(&h, sums + nt, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    *total = h;
    return TGVG_OK;
}

// ------------------------------------------------------------ geometry ---
__device__ __forceinline__ float corner_axis(uint32_t fine, int d, float cs, float o) {
    return fadd(o, fmul((float)(fine >> (21 - d)), cs));
}

// World lower corner and edge of a cube (cube_corner, marching_cubes.cpp:21-30).
__device__ __forceinline__ void cube_corner(uint64_t key, int d, const float* o, float r_root, float* p, float& cs) {
    cs = fdiv(fmul(2.0f, r_root), (float)(1u << d));
    p[0] = corner_axis(gather3(key), d, cs, o[0]);
    p[1] = corner_axis(gather3(key >> 1), d, cs, o[1]);
    p[2] = corner_axis(gather3(key >> 2), d, cs, o[2]);
}

// 20-bit quantisation and the packed 60-bit vertex key (marching_cubes.cpp:34-47).
__device__ __forceinline__ unsigned long long vertex_key(const float* p, const float* o, float inv) {
    unsigned long long k = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int q = trunc_i32(fadd(fmul(fsub(p[a], o[a]), inv), 0.5f));
        q = q < 0 ? 0 : (q > (1 << 20) - 1 ? (1 << 20) - 1 : q);
        k |= (unsigned long long)q << (20 * a);
    }
    return k;
}

// Quad of the pair (i, j) seen from i across face f (marching_cubes.cpp:124-158)
// and its winding flag (:167-168).
__device__ __forceinline__ bool face_quad(uint64_t ki, int di, uint64_t kj, int dj, float ui, float uj, int f,
                                          const float* o, float r_root, float q[4][3]) {
    float pi[3], pj[3], cs_i, cs_j;
    cube_corner(ki, di, o, r_root, pi, cs_i);
    cube_corner(kj, dj, o, r_root, pj, cs_j);
    const float cs_min = cs_i < cs_j ? cs_i : cs_j;
    const float h = fmul(cs_min, 0.5f);
    const float t = fdiv(ui, fsub(ui, uj));
    const int ax = f / 2;
    float surf[3];
    const float ci = fadd(pi[ax], fmul(cs_i, 0.5f)), cj = fadd(pj[ax], fmul(cs_j, 0.5f));
    const float* small = cs_i <= cs_j ? pi : pj;
#pragma unroll
    for (int b = 0; b < 3; ++b) surf[b] = b == ax ? fadd(ci, fmul(t, fsub(cj, ci))) : fadd(small[b], h);
    const int t1 = ax == 0 ? 1 : (ax == 1 ? 2 : 0);
    const int t2 = ax == 0 ? 2 : (ax == 1 ? 0 : 1);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        const float a1 = b == t1 ? h : 0.0f, a2 = b == t2 ? h : 0.0f;
        q[0][b] = fsub(fsub(surf[b], a1), a2);
        q[1][b] = fsub(fadd(surf[b], a1), a2);
        q[2][b] = fadd(fadd(surf[b], a1), a2);
        q[3][b] = fadd(fsub(surf[b], a1), a2);
    }
    return (f % 2 == 0) ? (ui > 0.0f) : (ui < 0.0f);
}

// ------------------------------------------------------------- kernels ---
__global__ void k_surf_prep(int n, const uint4* __restrict__ cubes, const float* __restrict__ state,
                            unsigned long long* __restrict__ keys, int* __restrict__ depth,
                            float* __restrict__ u, int* __restrict__ bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 c = cubes[i];
    const int d = (int)c.w;
    if (d < 0 || d > 21) atomicOr(bad, 1);
    const unsigned long long k = ((unsigned long long)c.x << 32) | c.y;
    if (i > 0) {
        const uint4 pc = cubes[i - 1];
        if ((((unsigned long long)pc.x << 32) | pc.y) > k) atomicOr(bad, 2);
    }
    keys[i] = k;
    depth[i] = min(21, max(0, d));
    u[i] = state[(size_t)i * 13];
}

__global__ void k_surf_hash(int n, const unsigned long long* __restrict__ keys, HashView h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) hash_insert(h, keys[i], i);
}

// The reference's bisection over the cube file (CubeReader::lookup,
// marching_cubes.cpp:243-252): the first probed index whose code equals k.  It
// is run on the key array itself, so it answers as the reference does for any
// order of the cubes.
__device__ __forceinline__ int file_bisect(const unsigned long long* __restrict__ keys, int n, uint64_t k) {
    uint32_t lo = 0, hi = (uint32_t)n;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        const uint64_t c = keys[mid];
        if (c == k) return (int)mid;
        if (c < k) lo = mid + 1; else hi = mid;
    }
    return -1;
}

// Resolved neighbour of (cube i, face f), or -1.  In-memory semantics: the
// largest index with the face neighbour's code, else with its parent code; a
// self link is dropped (marching_cubes.cpp:92-107).  Streaming semantics:
// candidates in-leaf exact, file bisection exact, in-leaf parent, file
// bisection parent; a candidate equal to the cube itself is passed over
// (:451-488).  `leaf` holds each cube's leaf range (first, last), or (1, 0).
// The in-leaf candidate is the leaf's largest index with the code: from the
// code's index range when the cubes are Morton-sorted (equal codes are then
// contiguous), else by a scan of the leaf.
template <bool STR>
__global__ void k_surf_nbrs(int n, const unsigned long long* __restrict__ keys, const int* __restrict__ depth,
                            HashView h, const int2* __restrict__ leaf, int sorted, int* __restrict__ nbr) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * 6) return;
    const int i = (int)(t / 6), f = (int)(t % 6);
    const int d = depth[i];
    int j = -1;
    const uint64_t nk = face_key(keys[i], f, d);
    if (nk != NO_KEY) {
        if (!STR) {
            int s = hash_find(h, nk);
            if (s < 0 && d > 0) s = hash_find(h, parent_key(nk, d));
            if (s >= 0) j = h.rmax[s];
            if (j == i) j = -1;
        } else {
            const int2 lr = leaf[i];
            for (int step = 0; step < 2 && j < 0; ++step) {
                if (step == 1 && d <= 0) break;
                const uint64_t k = step ? parent_key(nk, d) : nk;
                const int s = hash_find(h, k);
                if (s < 0) continue;  // no cube has the code
                int cand = -1;
                if (sorted) {
                    const int hi = min(h.rmax[s], lr.y);
                    if (max(h.rmin[s], lr.x) <= hi) cand = hi;
                } else {
                    for (int g = lr.y; g >= lr.x; --g)
                        if (keys[g] == k) { cand = g; break; }
                }
                if (cand >= 0 && cand != i) { j = cand; break; }
                const int g = file_bisect(keys, n, k);
                if (g >= 0 && g != i) j = g;
            }
        }
    }
    nbr[t] = j;
}

// Emitter test of (cube i, face f), written at slot rank(i) * 6 + f of the
// emission order.  In-memory: the pair's first visitor in (cube, face) order
// (the reference's `seen` set, :110-114), both cubes with data when given, a
// sign change (:119).  Streaming: the finer cube (equal depth: the smaller
// index) owns the pair (:490-493), both cubes have votes, a sign change.
template <bool STR>
__global__ void k_surf_flags(int n, const int* __restrict__ nbr, const int* __restrict__ depth,
                             const float* __restrict__ u, const uint8_t* __restrict__ ok,
                             const int* __restrict__ rank, int* __restrict__ flag) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * 6) return;
    const int i = (int)(t / 6), f = (int)(t % 6);
    const int r = STR ? rank[i] : i;
    if (r < 0) return;
    const int j = nbr[t];
    bool e = j >= 0;
    if (e && !STR) {
        for (int g = 0; g < f; ++g) e &= nbr[(int64_t)i * 6 + g] != j;
        if (j < i)
            for (int g = 0; g < 6; ++g) e &= nbr[(int64_t)j * 6 + g] != i;
    }
    if (e && STR) e = depth[j] < depth[i] || (depth[j] == depth[i] && i < j);
    if (e && ok) e = ok[i] && ok[j];
    if (e) e = (u[i] >= 0.0f) != (u[j] >= 0.0f);
    flag[(int64_t)r * 6 + f] = e ? 1 : 0;
}

template <bool STR>
__global__ void k_surf_quads(int n, const int* __restrict__ nbr, const unsigned long long* __restrict__ keys,
                             const int* __restrict__ depth, const float* __restrict__ u,
                             const int* __restrict__ rank, const int* __restrict__ flag,
                             const int* __restrict__ qidx, float3 o3, float r_root, float inv,
                             unsigned long long* __restrict__ qkey, float* __restrict__ qpos,
                             uint8_t* __restrict__ qflip) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * 6) return;
    const int i = (int)(t / 6), f = (int)(t % 6);
    const int r = STR ? rank[i] : i;
    if (r < 0) return;
    const int64_t slot = (int64_t)r * 6 + f;
    if (!flag[slot]) return;
    const int j = nbr[t];
    const float o[3] = {o3.x, o3.y, o3.z};
    float q[4][3];
    const bool flip = face_quad(keys[i], depth[i], keys[j], depth[j], u[i], u[j], f, o, r_root, q);
    const int64_t qi = qidx[slot];
    qflip[qi] = flip ? 1 : 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        qkey[qi * 4 + c] = vertex_key(q[c], o, inv);
        if (!STR)
            for (int a = 0; a < 3; ++a) qpos[(qi * 4 + c) * 3 + a] = q[c][a];
    }
}

// Vertex merge: every corner occurrence o (quad-major, corner-minor: the
// reference's insertion order) meets its key's slot; the slot keeps the
// smallest occurrence.
__global__ void k_vert_hash(int64_t no, const unsigned long long* __restrict__ qkey, unsigned long long* hk,
                            int* __restrict__ first, uint64_t mask, int* __restrict__ slot) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= no) return;
    const unsigned long long key = qkey[o];
    uint64_t s = mix64(key) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS(hk + s, (unsigned long long)NO_KEY, key);
        if (prev == (unsigned long long)NO_KEY || prev == key) {
            atomicMin(first + s, (int)o);
            slot[o] = (int)s;
            return;
        }
        s = (s + 1) & mask;
    }
}

__global__ void k_vert_first(int64_t no, const int* __restrict__ slot, const int* __restrict__ first,
                             int* __restrict__ isfirst) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o < no) isfirst[o] = first[slot[o]] == (int)o ? 1 : 0;
}

// Vertex positions: the first occurrence's corner (in-memory) or the
// dequantised key (streaming: origin + q * scale, :372-377).
template <bool STR>
__global__ void k_vert_emit(int64_t no, const int* __restrict__ isfirst, const int* __restrict__ vid,
                            const float* __restrict__ qpos, const unsigned long long* __restrict__ qkey,
                            float3 o3, float scale, float* __restrict__ verts) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= no || !isfirst[o]) return;
    float* v = verts + (int64_t)vid[o] * 3;
    if (!STR) {
        v[0] = qpos[o * 3]; v[1] = qpos[o * 3 + 1]; v[2] = qpos[o * 3 + 2];
    } else {
        const unsigned long long k = qkey[o];
        v[0] = fadd(o3.x, fmul((float)(k & 0xFFFFFull), scale));
        v[1] = fadd(o3.y, fmul((float)((k >> 20) & 0xFFFFFull), scale));
        v[2] = fadd(o3.z, fmul((float)((k >> 40) & 0xFFFFFull), scale));
    }
}

// Two triangles per quad, winding by its flag (:170-176).
__global__ void k_faces(int64_t nq, const int* __restrict__ slot, const int* __restrict__ first,
                        const int* __restrict__ vid, const uint8_t* __restrict__ qflip, uint32_t* __restrict__ faces) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    uint32_t id[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) id[c] = (uint32_t)vid[first[slot[q * 4 + c]]];
    uint32_t* f = faces + q * 6;
    if (!qflip[q]) {
        f[0] = id[0]; f[1] = id[1]; f[2] = id[2]; f[3] = id[0]; f[4] = id[2]; f[5] = id[3];
    } else {
        f[0] = id[0]; f[1] = id[2]; f[2] = id[1]; f[3] = id[0]; f[4] = id[3]; f[5] = id[2];
    }
}

// Face normal (b - a) x (c - a) of triangle t (compute_normals, :191-195).
__global__ void k_tri_normal(int64_t nt, const float* __restrict__ v, const uint32_t* __restrict__ faces,
                             float* __restrict__ tn, int* __restrict__ cnt) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const uint32_t ia = faces[t * 3], ib = faces[t * 3 + 1], ic = faces[t * 3 + 2];
    const float* a = v + (int64_t)ia * 3;
    const float* b = v + (int64_t)ib * 3;
    const float* c = v + (int64_t)ic * 3;
    const float d0 = fsub(b[0], a[0]), d1 = fsub(b[1], a[1]), d2 = fsub(b[2], a[2]);
    const float e0 = fsub(c[0], a[0]), e1 = fsub(c[1], a[1]), e2 = fsub(c[2], a[2]);
    tn[t * 3] = fsub(fmul(d1, e2), fmul(d2, e1));
    tn[t * 3 + 1] = fsub(fmul(d2, e0), fmul(d0, e2));
    tn[t * 3 + 2] = fsub(fmul(d0, e1), fmul(d1, e0));
    atomicAdd(cnt + ia, 1);
    atomicAdd(cnt + ib, 1);
    atomicAdd(cnt + ic, 1);
}

__global__ void k_vert_list(int64_t ne, const uint32_t* __restrict__ faces, const int* __restrict__ start,
                            int* __restrict__ cur, int* __restrict__ list) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const uint32_t vtx = faces[e];
    list[start[vtx] + atomicAdd(cur + vtx, 1)] = (int)e;
}

// Per vertex: its (triangle, corner) entries in ascending order -- the order
// in which the reference adds face normals -- summed, then divided by the
// length when it exceeds 1e-12 (:197-204).
__global__ void k_vert_normal(int64_t nv, const int* __restrict__ start, const int* __restrict__ cnt,
                              const int* __restrict__ list, const float* __restrict__ tn, float* __restrict__ nrm) {
    const int64_t vtx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (vtx >= nv) return;
    const int s0 = start[vtx], m = cnt[vtx];
    float x = 0.0f, y = 0.0f, z = 0.0f;
    int last = -1;
    for (int k = 0; k < m; ++k) {
        int next = 0x7fffffff;
        for (int r = 0; r < m; ++r) {
            const int e = list[s0 + r];
            if (e > last && e < next) next = e;
        }
        last = next;
        const float* n = tn + (int64_t)(next / 3) * 3;
        x = fadd(x, n[0]); y = fadd(y, n[1]); z = fadd(z, n[2]);
    }
    const float len = fsqrt(fadd(fadd(fmul(x, x), fmul(y, y)), fmul(z, z)));
    if (len > 1e-12f) { x = fdiv(x, len); y = fdiv(y, len); z = fdiv(z, len); }
    nrm[vtx * 3] = x; nrm[vtx * 3 + 1] = y; nrm[vtx * 3 + 2] = z;
}

// ---------------------------------------------------------------- host ---
static inline unsigned grid_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Normals of a device mesh into d_nrm.
static int normals_dev(tgvg_ctx* ctx, const float* d_v, int64_t nv, const uint32_t* d_f, int64_t nf, float* d_nrm) {
    if (nv == 0) return TGVG_OK;
    auto* tn = (float*)ctx->buf(B_S_TN, sizeof(float) * 3 * std::max<int64_t>(1, nf));
    auto* cnt = (int*)ctx->buf(B_S_VCNT, sizeof(int) * nv);
    auto* start = (int*)ctx->buf(B_S_VSTART, sizeof(int) * nv);
    auto* cur = (int*)ctx->buf(B_S_VCUR, sizeof(int) * nv);
    auto* list = (int*)ctx->buf(B_S_VLIST, sizeof(int) * 3 * std::max<int64_t>(1, nf));
    if (!tn || !cnt || !start || !cur || !list) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemsetAsync(cnt, 0, sizeof(int) * nv, ctx->stream));
    TGVG_CK(ctx, cudaMemsetAsync(cur, 0, sizeof(int) * nv, ctx->stream));
    if (nf > 0) {
        k_tri_normal<<<grid_for(nf, 256), 256, 0, ctx->stream>>>(nf, d_v, d_f, tn, cnt);
        TGVG_LAUNCHED(ctx);
    }
    int64_t tot = 0;
    int rc = scan_exclusive(ctx, cnt, nv, start, &tot);
    if (rc) return rc;
    if (nf > 0) {
        k_vert_list<<<grid_for(3 * nf, 256), 256, 0, ctx->stream>>>(3 * nf, d_f, start, cur, list);
        TGVG_LAUNCHED(ctx);
    }
    k_vert_normal<<<grid_for(nv, 128), 128, 0, ctx->stream>>>(nv, start, cnt, list, tn, d_nrm);
    TGVG_LAUNCHED(ctx);
    return TGVG_OK;
}

// The whole extraction over host arrays.  STR selects the streaming semantics
// (leaves in caller order, per-cube vote totals); otherwise `ok` is the
// optional has_data mask.
template <bool STR>
static int extract(tgvg_ctx* ctx, const tgvg_cube* cubes, const tgvg_state* state, int64_t n64, const uint8_t* ok,
                   const uint32_t* tot, const tgvg_leaf* leaves, int32_t nleaf, const float* origin, float r_root,
                   bool normals, tgvg_mesh* out) {
    if (n64 > (int64_t(1) << 28)) return ctx->fail(TGVG_ERR_LIMIT, "surface extraction: more than 2^28 cubes");
    const int n = (int)n64;
    if (n == 0) return TGVG_OK;
    // emission rank of every cube: its place in the caller's leaf order (streaming)
    std::vector<int> rank;
    std::vector<int2> lrange;
    std::vector<uint8_t> hasv;
    if (STR) {
        rank.assign(n, -1);
        lrange.assign(n, make_int2(1, 0));
        hasv.resize(n);
        for (int i = 0; i < n; ++i) hasv[i] = tot[i] != 0;
        int r = 0;
        for (int l = 0; l < nleaf; ++l) {
            const uint32_t a = leaves[l].first_idx, b = leaves[l].last_idx;
            if (int64_t(a) >= n64 || a > b) continue;  // load_cubes_range clamps (octree_builder.cpp:131-135)
            const int e = (int)std::min<int64_t>(int64_t(b), n64 - 1);
            for (int g = (int)a; g <= e; ++g) {
                if (rank[g] >= 0) return ctx->fail(TGVG_ERR_OVERLAP, "treetop leaves overlap");
                rank[g] = r++;
                lrange[g] = make_int2((int)a, e);
            }
        }
    }
    uint64_t cap = 1024;
    while (cap < 2ull * (uint64_t)n) cap <<= 1;
    auto B = [&](int id, size_t bytes) { return ctx->buf(id, bytes); };
    auto* d_c = (tgvg_cube*)B(B_S_CUBES, sizeof(tgvg_cube) * n);
    auto* d_s = (float*)B(B_S_STATE, sizeof(tgvg_state) * n);
    auto* keys = (unsigned long long*)B(B_S_KEYS, 8ull * n);
    auto* depth = (int*)B(B_S_DEPTH, 4ull * n);
    auto* u = (float*)B(B_S_U, 4ull * n);
    auto* hd = (uint8_t*)B(B_S_HD, (size_t)n + 16);
    auto* hk = (unsigned long long*)B(B_S_HKEYS, 8ull * cap);
    auto* hmin = (int*)B(B_S_HMIN, 4ull * cap);
    auto* hmax = (int*)B(B_S_HMAX, 4ull * cap);
    auto* nbr = (int*)B(B_S_NBR, 24ull * n);
    auto* flag = (int*)B(B_S_FLAGS, 24ull * n);
    auto* qidx = (int*)B(B_S_QIDX, 24ull * n);
    auto* d_rank = (int*)B(B_S_RANK, 4ull * n);
    auto* d_leaf = (int2*)B(B_S_LEAF, 8ull * n);
    if (!d_c || !d_s || !keys || !depth || !u || !hd || !hk || !hmin || !hmax || !nbr || !flag || !qidx || !d_rank ||
        !d_leaf)
        return TGVG_ERR_NOMEM;
    cudaStream_t st = ctx->stream;
    TGVG_CK(ctx, cudaMemcpyAsync(d_c, cubes, sizeof(tgvg_cube) * n, cudaMemcpyHostToDevice, st));
    TGVG_CK(ctx, cudaMemcpyAsync(d_s, state, sizeof(tgvg_state) * n, cudaMemcpyHostToDevice, st));
    const uint8_t* d_ok = nullptr;
    if (STR || ok) {
        TGVG_CK(ctx, cudaMemcpyAsync(hd, STR ? hasv.data() : ok, (size_t)n, cudaMemcpyHostToDevice, st));
        d_ok = hd;
    }
    if (STR) {
        TGVG_CK(ctx, cudaMemcpyAsync(d_rank, rank.data(), 4ull * n, cudaMemcpyHostToDevice, st));
        TGVG_CK(ctx, cudaMemcpyAsync(d_leaf, lrange.data(), 8ull * n, cudaMemcpyHostToDevice, st));
    }
    TGVG_CK(ctx, cudaMemsetAsync(hk, 0xff, 8ull * cap, st));
    TGVG_CK(ctx, cudaMemsetAsync(hmin, 0x7f, 4ull * cap, st));
    TGVG_CK(ctx, cudaMemsetAsync(hmax, 0xff, 4ull * cap, st));
    TGVG_CK(ctx, cudaMemsetAsync(flag, 0, 24ull * n, st));
    int* bad = qidx;  // scratch word before the scan overwrites qidx
    TGVG_CK(ctx, cudaMemsetAsync(bad, 0, sizeof(int), st));
    k_surf_prep<<<grid_for(n, 256), 256, 0, st>>>(n, reinterpret_cast<const uint4*>(d_c), d_s, keys, depth, u, bad);
    TGVG_LAUNCHED(ctx);
    int h_bad = 0;
    TGVG_CK(ctx, cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    const HashView hv{hk, hmin, hmax, cap - 1};
    k_surf_hash<<<grid_for(n, 256), 256, 0, st>>>(n, keys, hv);
    TGVG_LAUNCHED(ctx);
    TGVG_CK(ctx, cudaStreamSynchronize(st));
    if (h_bad & 1) return ctx->fail(TGVG_ERR_INVALID, "cube depth outside 0..21");
    const int sorted = (h_bad & 2) ? 0 : 1;
    const int64_t ns = 6ll * n;
    k_surf_nbrs<STR><<<grid_for(ns, 256), 256, 0, st>>>(n, keys, depth, hv, d_leaf, sorted, nbr);
    TGVG_LAUNCHED(ctx);
    k_surf_flags<STR><<<grid_for(ns, 256), 256, 0, st>>>(n, nbr, depth, u, d_ok, d_rank, flag);
    TGVG_LAUNCHED(ctx);
    int64_t nq = 0;
    int rc = scan_exclusive(ctx, flag, ns, qidx, &nq);
    if (rc) return rc;
    if (nq > (int64_t(1) << 28)) return ctx->fail(TGVG_ERR_LIMIT, "surface extraction: more than 2^28 quads");
    const int64_t no = 4 * nq;
    auto* qkey = (unsigned long long*)B(B_S_QKEY, 8ull * std::max<int64_t>(1, no));
    auto* qpos = (float*)B(B_S_QPOS, 12ull * std::max<int64_t>(1, STR ? 1 : no));
    auto* qflip = (uint8_t*)B(B_S_QFLIP, (size_t)std::max<int64_t>(1, nq));
    uint64_t vcap = 1024;
    while (vcap < 2ull * (uint64_t)no) vcap <<= 1;
    auto* vk = (unsigned long long*)B(B_S_VTK, 8ull * vcap);
    auto* vfirst = (int*)B(B_S_VTF, 4ull * vcap);
    auto* slot = (int*)B(B_S_SLOT, 4ull * std::max<int64_t>(1, no));
    auto* isfirst = (int*)B(B_S_VFLAG, 4ull * std::max<int64_t>(1, no));
    auto* vid = (int*)B(B_S_VID, 4ull * std::max<int64_t>(1, no));
    if (!qkey || !qpos || !qflip || !vk || !vfirst || !slot || !isfirst || !vid) return TGVG_ERR_NOMEM;
    const float3 o3 = make_float3(origin[0], origin[1], origin[2]);
    const float inv = (float)(1u << 20) / (2.0f * r_root);
    const float scale = 1.0f / inv;
    if (nq > 0) {
        k_surf_quads<STR><<<grid_for(ns, 256), 256, 0, st>>>(n, nbr, keys, depth, u, d_rank, flag, qidx, o3, r_root,
                                                             inv, qkey, qpos, qflip);
        TGVG_LAUNCHED(ctx);
        TGVG_CK(ctx, cudaMemsetAsync(vk, 0xff, 8ull * vcap, st));
        TGVG_CK(ctx, cudaMemsetAsync(vfirst, 0x7f, 4ull * vcap, st));
        k_vert_hash<<<grid_for(no, 256), 256, 0, st>>>(no, qkey, vk, vfirst, vcap - 1, slot);
        TGVG_LAUNCHED(ctx);
        k_vert_first<<<grid_for(no, 256), 256, 0, st>>>(no, slot, vfirst, isfirst);
        TGVG_LAUNCHED(ctx);
    }
    int64_t nv = 0;
    if ((rc = scan_exclusive(ctx, isfirst, no, vid, &nv))) return rc;
    auto* verts = (float*)B(B_S_VERTS, 12ull * std::max<int64_t>(1, nv));
    auto* faces = (uint32_t*)B(B_S_FACES, 24ull * std::max<int64_t>(1, nq));
    auto* nrm = (float*)B(B_S_NRM, 12ull * std::max<int64_t>(1, nv));
    if (!verts || !faces || !nrm) return TGVG_ERR_NOMEM;
    if (nq > 0) {
        k_vert_emit<STR><<<grid_for(no, 256), 256, 0, st>>>(no, isfirst, vid, qpos, qkey, o3, scale, verts);
        TGVG_LAUNCHED(ctx);
        k_faces<<<grid_for(nq, 256), 256, 0, st>>>(nq, slot, vfirst, vid, qflip, faces);
        TGVG_LAUNCHED(ctx);
    }
    if (normals && (rc = normals_dev(ctx, verts, nv, faces, 2 * nq, nrm))) return rc;
    out->verts.resize(3 * nv);
    out->faces.resize(6 * nq);
    out->normals.resize(normals ? 3 * nv : 0);
    if (nv) TGVG_CK(ctx, cudaMemcpyAsync(out->verts.data(), verts, 12ull * nv, cudaMemcpyDeviceToHost, st));
    if (nq) TGVG_CK(ctx, cudaMemcpyAsync(out->faces.data(), faces, 24ull * nq, cudaMemcpyDeviceToHost, st));
    if (normals && nv)
        TGVG_CK(ctx, cudaMemcpyAsync(out->normals.data(), nrm, 12ull * nv, cudaMemcpyDeviceToHost, st));
    TGVG_CK(ctx, cudaStreamSynchronize(st));
    return TGVG_OK;
}

}  // namespace tgvg

using namespace tgvg;

namespace {

bool surface_args_ok(tgvg_ctx* ctx, const void* cubes, const void* state, int64_t n, const float* origin,
                     float r_root) {
    return ctx && n >= 0 && (n == 0 || (cubes && state)) && origin && std::isfinite(r_root) && r_root > 0.0f;
}

// One Wavefront line of three floats as the reference's streams write them
// (default formatting: %g with 6 significant digits).
void put_v(FILE* f, const char* tag, const float* p) {
    std::fprintf(f, "%s %g %g %g\n", tag, (double)p[0], (double)p[1], (double)p[2]);
}

int write_obj_file(const char* path, const float* v, int64_t nv, const uint32_t* faces, int64_t nf, const float* nrm) {
    FILE* f = path ? std::fopen(path, "w") : nullptr;
    if (!f) return TGVG_ERR_IO;
    for (int64_t i = 0; i < nv; ++i) put_v(f, "v", v + 3 * i);
    if (nrm)
        for (int64_t i = 0; i < nv; ++i) put_v(f, "vn", nrm + 3 * i);
    for (int64_t t = 0; t < nf; ++t) {
        const unsigned long long a = faces[3 * t] + 1ull, b = faces[3 * t + 1] + 1ull, c = faces[3 * t + 2] + 1ull;
        if (nrm) std::fprintf(f, "f %llu//%llu %llu//%llu %llu//%llu\n", a, a, b, b, c, c);
        else std::fprintf(f, "f %llu %llu %llu\n", a, b, c);
    }
    return std::fclose(f) == 0 ? TGVG_OK : TGVG_ERR_IO;
}

}  // namespace

extern "C" int tgvg_extract_surface(tgvg_ctx* ctx, const tgvg_cube* cubes, const tgvg_state* state, int64_t n,
                                    const uint8_t* has_data, const float* origin, float r_root, int32_t normals,
                                    tgvg_mesh** out) {
    if (!surface_args_ok(ctx, cubes, state, n, origin, r_root) || !out) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto* m = new tgvg_mesh;
    const int rc = extract<false>(ctx, cubes, state, n, has_data, nullptr, nullptr, 0, origin, r_root, normals != 0, m);
    if (rc) { delete m; return rc; }
    *out = m;
    return TGVG_OK;
}

extern "C" int tgvg_extract_surface_leaves(tgvg_ctx* ctx, const tgvg_cube* cubes, const tgvg_state* state,
                                           const uint32_t* hists, int32_t nbins, int64_t n, const tgvg_leaf* leaves,
                                           int32_t nleaf, const float* origin, float r_root, tgvg_mesh** out) {
    if (!surface_args_ok(ctx, cubes, state, n, origin, r_root) || !out || (n > 0 && !hists) ||
        (nbins != 8 && nbins != 10) || nleaf < 0 || (nleaf > 0 && !leaves))
        return TGVG_ERR_INVALID;
    std::vector<uint32_t> tot(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        uint32_t s = 0;
        for (int k = 0; k < nbins; ++k) s += hists[i * nbins + k];
        tot[i] = s;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto* m = new tgvg_mesh;
    const int rc = extract<true>(ctx, cubes, state, n, nullptr, tot.data(), leaves, nleaf, origin, r_root, false, m);
    if (rc) { delete m; return rc; }
    *out = m;
    return TGVG_OK;
}

extern "C" int tgvg_mesh_size(const tgvg_mesh* m, int64_t* nv, int64_t* nf, int32_t* has_normals) {
    if (!m) return TGVG_ERR_INVALID;
    if (nv) *nv = int64_t(m->verts.size() / 3);
    if (nf) *nf = int64_t(m->faces.size() / 3);
    if (has_normals) *has_normals = m->normals.empty() ? 0 : 1;
    return TGVG_OK;
}

extern "C" int tgvg_mesh_read(const tgvg_mesh* m, float* verts, uint32_t* faces, float* normals) {
    if (!m) return TGVG_ERR_INVALID;
    if (verts && !m->verts.empty()) std::memcpy(verts, m->verts.data(), m->verts.size() * sizeof(float));
    if (faces && !m->faces.empty()) std::memcpy(faces, m->faces.data(), m->faces.size() * sizeof(uint32_t));
    if (normals && !m->normals.empty()) std::memcpy(normals, m->normals.data(), m->normals.size() * sizeof(float));
    return TGVG_OK;
}

extern "C" void tgvg_mesh_free(tgvg_mesh* m) { delete m; }

extern "C" int tgvg_compute_normals(tgvg_ctx* ctx, const float* verts, int64_t nv, const uint32_t* faces, int64_t nf,
                                    float* normals) {
    if (!ctx || nv < 0 || nf < 0 || (nv > 0 && (!verts || !normals)) || (nf > 0 && !faces) ||
        nv > (int64_t(1) << 28) || nf > (int64_t(1) << 29))
        return TGVG_ERR_INVALID;
    for (int64_t e = 0; e < 3 * nf; ++e)
        if (faces[e] >= uint64_t(nv)) return TGVG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (nv == 0) return TGVG_OK;
    auto* d_v = (float*)ctx->buf(B_S_VERTS, 12ull * nv);
    auto* d_f = (uint32_t*)ctx->buf(B_S_FACES, 12ull * std::max<int64_t>(1, nf));
    auto* d_n = (float*)ctx->buf(B_S_NRM, 12ull * nv);
    if (!d_v || !d_f || !d_n) return TGVG_ERR_NOMEM;
    TGVG_CK(ctx, cudaMemcpyAsync(d_v, verts, 12ull * nv, cudaMemcpyHostToDevice, ctx->stream));
    if (nf) TGVG_CK(ctx, cudaMemcpyAsync(d_f, faces, 12ull * nf, cudaMemcpyHostToDevice, ctx->stream));
    int rc = normals_dev(ctx, d_v, nv, d_f, nf, d_n);
    if (rc) return rc;
    TGVG_CK(ctx, cudaMemcpyAsync(normals, d_n, 12ull * nv, cudaMemcpyDeviceToHost, ctx->stream));
    TGVG_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TGVG_OK;
}

extern "C" int tgvg_write_obj(const char* path, const float* verts, int64_t nv, const uint32_t* faces, int64_t nf,
                              const float* normals) {
    if (nv < 0 || nf < 0 || (nv > 0 && !verts) || (nf > 0 && !faces)) return TGVG_ERR_INVALID;
    return write_obj_file(path, verts, nv, faces, nf, normals);
}

// extract_surface_streaming (marching_cubes.cpp:374-580): cube, state,
// treetop and histogram files in, Wavefront file out.
extern "C" int tgvg_extract_surface_streaming(tgvg_ctx* ctx, const char* cube_path, const char* state_path,
                                              const char* treetop_path, const char* hist_path, const float* origin,
                                              float r_root, const char* out_obj_path) {
    using namespace tgvg::fileio;
    if (!ctx || !origin || !std::isfinite(r_root) || !(r_root > 0.0f)) return TGVG_ERR_INVALID;
    std::vector<char> tb, sb, hb;
    int rc = read_file(treetop_path, tb);
    if (rc) return ctx->fail(rc, std::string("Cannot open: ") + (treetop_path ? treetop_path : ""));
    if (tb.size() < 16 || std::memcmp(tb.data(), "TGVT", 4) != 0) return ctx->fail(TGVG_ERR_FORMAT, "Bad treetop magic");
    const uint32_t nleaf = u32_at(tb, 12);
    if (tb.size() < 16 + size_t(nleaf) * sizeof(tgvg_leaf)) return ctx->fail(TGVG_ERR_FORMAT, "short treetop file");
    std::vector<tgvg_leaf> leaves(nleaf);
    if (nleaf) std::memcpy(leaves.data(), tb.data() + 16, nleaf * sizeof(tgvg_leaf));
    std::vector<tgvg_cube> cubes;
    if ((rc = load_cube_file(cube_path, cubes, nullptr)))
        return ctx->fail(rc, std::string("Bad cube file: ") + (cube_path ? cube_path : ""));
    const size_t n = cubes.size();
    if ((rc = read_file(state_path, sb))) return ctx->fail(rc, std::string("Cannot open: ") + (state_path ? state_path : ""));
    if (sb.size() < 12 || std::memcmp(sb.data(), "TGVS", 4) != 0) return ctx->fail(TGVG_ERR_FORMAT, "Bad TGV state magic");
    if (u32_at(sb, 8) < n || sb.size() < 12 + n * sizeof(tgvg_state))
        return ctx->fail(TGVG_ERR_FORMAT, "state file shorter than the cube file");
    if ((rc = read_file(hist_path, hb))) return ctx->fail(rc, std::string("Cannot open: ") + (hist_path ? hist_path : ""));
    if (hb.size() < 12 || std::memcmp(hb.data(), "TGVH", 4) != 0) return ctx->fail(TGVG_ERR_FORMAT, "Bad histogram magic");
    if (u32_at(hb, 8) < n || hb.size() < 12 + n * 32)
        return ctx->fail(TGVG_ERR_FORMAT, "histogram file shorter than the cube file");
    std::vector<tgvg_state> state(n);
    std::vector<uint32_t> tot(n);
    if (n) std::memcpy(state.data(), sb.data() + 12, n * sizeof(tgvg_state));
    for (size_t i = 0; i < n; ++i) {
        uint32_t b[8], s = 0;
        std::memcpy(b, hb.data() + 12 + 32 * i, 32);
        for (int k = 0; k < 8; ++k) s += b[k];
        tot[i] = s;
    }
    tgvg_mesh m;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        rc = extract<true>(ctx, cubes.data(), state.data(), int64_t(n), nullptr, tot.data(), leaves.data(),
                           int32_t(nleaf), origin, r_root, false, &m);
        if (rc) return rc;
    }
    rc = write_obj_file(out_obj_path, m.verts.data(), int64_t(m.verts.size() / 3), m.faces.data(),
                        int64_t(m.faces.size() / 3), nullptr);
    return rc ? ctx->fail(rc, std::string("Cannot open: ") + (out_obj_path ? out_obj_path : "")) : TGVG_OK;
}
