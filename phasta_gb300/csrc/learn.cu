// learn.cu -- the learned right preconditioner of flexible GMRES: a message-passing network
// over the mesh edges that maps a Krylov vector v of the block-diagonal preconditioned
// operator L^-1 J U^-1 (au1mfg.f:57-83, i3lu.f) to z ~ (L^-1 J U^-1)^-1 v.  It has no
// counterpart in the reference, whose matrix-free GMRES (solmfg.f:221-340) is preconditioned
// by the 5x5 block-diagonal LU alone; that method stays the fallback (solver.cu).
//
// Network (the oracle restates it as test infrastructure, oracle/net_oracle.py):
//   x_i  = [ctx_i (32) | bf16(s alpha_d v_i,d) (5) | 0 (11)],  s = sqrt(5 nshg)
//   h0   = bf16(relu(W_e x + b_e))
//   per layer: P = bf16(W_p h), Q = W_q h + b_m, m_ij = relu(Q_i + P_j + C e_ij),
//              a_i = bf16(mean_j m_ij), h' = bf16(h + relu(W_u [h; a] + b_u))
//   out  = W_d h3 + b_d,  z_i = v_i + act_i beta out_i / s
// Every GEMM runs on the tensor cores (mma.sync m16n8k16, bf16 operands, FP32
// accumulation); edges are gathered per node from a CSR over periodic masters whose entries
// carry the periodic shift of the element edge they came from.
//
// Kernels: one warp owns 16 nodes (a "slab") from staging through both GEMMs, so the
// inference layers need no block barrier after their weights are staged; the persistent grid
// keeps the weights (bf16, in shared memory) for all of its slabs.  The training backward
// works on 128-node tiles: per-warp data GEMMs, then block-wide weight-gradient GEMMs over
// the tile (K = nodes), with per-CTA partial gradients summed in a fixed order (deterministic).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "phgpu_impl.cuh"

namespace phgpu {

namespace netk {

using bf16 = __nv_bfloat16;
using bf162 = __nv_bfloat162;

constexpr int H = 64, FIN = 48, FCTX = 32, NL = 3, NOUT = 5;
// flat parameter layout (include/phgpu.h)
constexpr int O_WE = 0, O_BE = O_WE + H * FIN, O_L0 = O_BE + H;
constexpr int L_WP = 0, L_WQ = H * H, L_BM = 2 * H * H, L_C = L_BM + H, L_WU = L_C + 3 * H, L_BU = L_WU + 2 * H * H,
              L_SIZE = L_BU + H;
constexpr int O_WD = O_L0 + NL * L_SIZE, O_BD = O_WD + NOUT * H, O_AL = O_BD + NOUT, O_BT = O_AL + NOUT,
              NPARAM = O_BT + NOUT;
static_assert(NPARAM == PHGPU_NET_NPARAM, "parameter layout");
static_assert(O_AL == PHGPU_NET_NTRAIN, "trained parameters");
constexpr int PSTRIDE = NPARAM + 1;  // partial row: the gradient, then the loss
constexpr int SHIFT = 26;
constexpr unsigned NBMASK = (1u << SHIFT) - 1;
__host__ __device__ constexpr int OL(int l) { return O_L0 + l * L_SIZE; }

// shared-memory row strides (bf16 elements): K = 48, 64, 128 operands + 8 of padding, so that the
// 32-bit fragment loads of one mma hit 32 different banks
constexpr int LD48 = 56, LD64 = 72, LD128 = 136, LDQ = 68;
constexpr int TILE = 128;  // nodes per backward tile (8 warps x 16)

// ---------------------------------------------------------------------------
// tensor-core fragment helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// c[nt] += A (16 x K, row-major, lda) . B^T, B stored [n][k] (ldb): one warp, NT n-tiles of 8.
// Fragment layout of m16n8k16 (g = lane/4, t = lane%4): a0 (g, 2t..2t+1), a1 (g+8, 2t..),
// a2 (g, 2t+8..), a3 (g+8, 2t+8..); b0 (k 2t..2t+1, n g), b1 (k 2t+8.., n g);
// c0,c1 (g, 2t..2t+1), c2,c3 (g+8, 2t..2t+1).
template <int NT>
__device__ __forceinline__ void warp_gemm(float (&c)[NT][4], const bf16* A, int lda, const bf16* B, int ldb, int K) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[4];
        a[0] = ld32(A + g * lda + k0 + 2 * t);
        a[1] = ld32(A + (g + 8) * lda + k0 + 2 * t);
        a[2] = ld32(A + g * lda + k0 + 8 + 2 * t);
        a[3] = ld32(A + (g + 8) * lda + k0 + 8 + 2 * t);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            uint32_t b[2];
            b[0] = ld32(B + (nt * 8 + g) * ldb + k0 + 2 * t);
            b[1] = ld32(B + (nt * 8 + g) * ldb + k0 + 8 + 2 * t);
            mma16816(c[nt], a, b);
        }
    }
}
template <int NT>
__device__ __forceinline__ void zero(float (&c)[NT][4]) {
#pragma unroll
    for (int i = 0; i < NT; ++i) c[i][0] = c[i][1] = c[i][2] = c[i][3] = 0.f;
}

// W[rows][cols] (FP32, global) -> dst[o][ld] bf16; rows rows..rows_pad-1 are zero
__device__ void stage_w(bf16* dst, int ld, const float* W, int rows, int cols, int rows_pad) {
    for (int idx = threadIdx.x; idx < rows_pad * cols; idx += blockDim.x) {
        const int o = idx / cols, i = idx - o * cols;
        dst[o * ld + i] = __float2bfloat16_rn(o < rows ? W[o * cols + i] : 0.f);
    }
}
// transposed: dst[i][ld] = W[o][i] for W[rows][cols]; extra_off shifts the output row index
__device__ void stage_wT(bf16* dst, int ld, const float* W, int rows, int cols, int col_off) {
    for (int idx = threadIdx.x; idx < rows * cols; idx += blockDim.x) {
        const int o = idx / cols, i = idx - o * cols;
        dst[i * ld + o + col_off] = __float2bfloat16_rn(W[o * cols + i]);
    }
}

// 16 rows x 64 bf16 between global (row stride 64) and shared memory (row stride lds), 16-byte vectors
__device__ __forceinline__ void load_slab(bf16* s, int lds, const bf16* g, int n0, int N) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int it = 0; it < 4; ++it) {
        const int idx = it * 32 + lane, r = idx >> 3, c = (idx & 7) * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (n0 + r < N) v = *reinterpret_cast<const uint4*>(g + (size_t)(n0 + r) * H + c);
        *reinterpret_cast<uint4*>(s + r * lds + c) = v;
    }
}
__device__ __forceinline__ void store_slab(bf16* g, const bf16* s, int lds, int n0, int N) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int it = 0; it < 4; ++it) {
        const int idx = it * 32 + lane, r = idx >> 3, c = (idx & 7) * 8;
        if (n0 + r < N) *reinterpret_cast<uint4*>(g + (size_t)(n0 + r) * H + c) = *reinterpret_cast<const uint4*>(s + r * lds + c);
    }
}

struct Geo {
    const int* nstart;
    const unsigned* nbr;
    const float* xf;
    float L0, L1, L2, rh;
    int N;
};

// edge vector (x_j - x_i + shift) / hbar of neighbour entry nb of node i; the same rounding in
// every kernel (the reverse edge's vector is the exact negation)
__device__ __forceinline__ int edge_vec(const Geo& G, float xi0, float xi1, float xi2, unsigned nb, float* e) {
    const int j = (int)(nb & NBMASK);
    const unsigned code = nb >> SHIFT;
    const float xj0 = __ldg(G.xf + 3 * (size_t)j), xj1 = __ldg(G.xf + 3 * (size_t)j + 1),
                xj2 = __ldg(G.xf + 3 * (size_t)j + 2);
    const unsigned c0 = code & 3, c1 = (code >> 2) & 3, c2 = (code >> 4) & 3;
    const float s0 = c0 == 1 ? G.L0 : (c0 == 2 ? -G.L0 : 0.f);
    const float s1 = c1 == 1 ? G.L1 : (c1 == 2 ? -G.L1 : 0.f);
    const float s2 = c2 == 1 ? G.L2 : (c2 == 2 ? -G.L2 : 0.f);
    e[0] = __fmul_rn(__fadd_rn(__fsub_rn(xj0, xi0), s0), G.rh);
    e[1] = __fmul_rn(__fadd_rn(__fsub_rn(xj1, xi1), s1), G.rh);
    e[2] = __fmul_rn(__fadd_rn(__fsub_rn(xj2, xi2), s2), G.rh);
    return j;
}
// the same from coordinates already loaded (x.w unused)
__device__ __forceinline__ void edge_vec4(const Geo& G, const float4& xi, const float4& xj, unsigned nb, float* e) {
    const unsigned code = nb >> SHIFT;
    const unsigned c0 = code & 3, c1 = (code >> 2) & 3, c2 = (code >> 4) & 3;
    const float s0 = c0 == 1 ? G.L0 : (c0 == 2 ? -G.L0 : 0.f);
    const float s1 = c1 == 1 ? G.L1 : (c1 == 2 ? -G.L1 : 0.f);
    const float s2 = c2 == 1 ? G.L2 : (c2 == 2 ? -G.L2 : 0.f);
    e[0] = __fmul_rn(__fadd_rn(__fsub_rn(xj.x, xi.x), s0), G.rh);
    e[1] = __fmul_rn(__fadd_rn(__fsub_rn(xj.y, xi.y), s1), G.rh);
    e[2] = __fmul_rn(__fadd_rn(__fsub_rn(xj.z, xi.z), s2), G.rh);
}
// message pre-activation Q_i + P_j + C e (one rounding sequence for the forward and backward)
__device__ __forceinline__ float edge_pre(float q, float p, float c0, float c1, float c2, const float* e) {
    return __fadd_rn(__fadd_rn(q, p), __fmaf_rn(c2, e[2], __fmaf_rn(c1, e[1], __fmul_rn(c0, e[0]))));
}

__device__ __forceinline__ float bflo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bfhi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

// input feature f of node n (the encoder's x, rebuilt identically by the backward)
__device__ __forceinline__ float feat(const float* v, const bf16* ctx, const float* alpha, float s, int n, int f) {
    if (f < FCTX) return __bfloat162float(ctx[(size_t)FCTX * n + f]);
    if (f < FCTX + NOUT) return __fmul_rn(__fmul_rn(s, v[5 * (size_t)n + (f - FCTX)]), alpha[f - FCTX]);
    return 0.f;
}

// ---------------------------------------------------------------------------
// context features
// ---------------------------------------------------------------------------
constexpr int kStatN = 28;   // 25 sums of squares of the factored BDiag, sum p, sum T, count
constexpr int kStatBlocks = 2 * 152, kStatThreads = 256;

__global__ void __launch_bounds__(kStatThreads) k_ctx_stats(const float* __restrict__ bdf, const double* __restrict__ y,
                                                           const unsigned char* __restrict__ act, int N,
                                                           double* __restrict__ part) {
    double acc[kStatN];
#pragma unroll
    for (int k = 0; k < kStatN; ++k) acc[k] = 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        if (!act[n]) continue;
#pragma unroll
        for (int k = 0; k < 25; ++k) {
            const double b = (double)bdf[25 * (size_t)n + k];
            acc[k] += b * b;
        }
        acc[25] += y[5 * (size_t)n];
        acc[26] += y[5 * (size_t)n + 4];
        acc[27] += 1.0;
    }
    __shared__ double sh[kStatThreads / 32][kStatN];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kStatN; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kStatN) {
        double s = 0.0;
        for (int w = 0; w < kStatThreads / 32; ++w) s += sh[w][threadIdx.x];
        part[(size_t)blockIdx.x * kStatN + threadIdx.x] = s;
    }
}

// stat[0..24] = 1/rms of each BDiag entry, [25] 1/pbar, [26] 1/Tbar, [27] 1/cbar
__global__ void k_ctx_final(const double* __restrict__ part, int nb, double Rgas, double gamma, float* __restrict__ stat) {
    __shared__ double tot[kStatN];
    if (threadIdx.x < kStatN) {
        double s = 0.0;
        for (int b = 0; b < nb; ++b) s += part[(size_t)b * kStatN + threadIdx.x];
        tot[threadIdx.x] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double na = tot[27] > 0 ? tot[27] : 1.0;
        for (int k = 0; k < 25; ++k) {
            const float rms = (float)sqrt(tot[k] / na);
            stat[k] = rms > 0.f ? 1.f / rms : 1.f;
        }
        const double pbar = tot[25] / na, Tbar = tot[26] / na;
        stat[25] = (float)(1.0 / pbar);
        stat[26] = (float)(1.0 / Tbar);
        stat[27] = (float)(1.0 / sqrt(gamma * Rgas * Tbar));
    }
}

__global__ void k_ctx_features(const float* __restrict__ bdf, const double* __restrict__ y,
                               const unsigned char* __restrict__ act, const float* __restrict__ stat, int N,
                               bf16* __restrict__ ctx) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float f[FCTX];
#pragma unroll
    for (int k = 0; k < 25; ++k) f[k] = __fmul_rn(bdf[25 * (size_t)n + k], stat[k]);
    const double* yn = y + 5 * (size_t)n;
    f[25] = 10.f * (float)(yn[0] * (double)stat[25] - 1.0);
    f[26] = (float)yn[1] * stat[27];
    f[27] = (float)yn[2] * stat[27];
    f[28] = (float)yn[3] * stat[27];
    f[29] = 10.f * (float)(yn[4] * (double)stat[26] - 1.0);
    f[30] = act[n] ? 1.f : 0.f;
    f[31] = 0.f;
    uint4* o = reinterpret_cast<uint4*>(ctx + (size_t)FCTX * n);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        bf162 p0 = __floats2bfloat162_rn(f[8 * q], f[8 * q + 1]), p1 = __floats2bfloat162_rn(f[8 * q + 2], f[8 * q + 3]);
        bf162 p2 = __floats2bfloat162_rn(f[8 * q + 4], f[8 * q + 5]), p3 = __floats2bfloat162_rn(f[8 * q + 6], f[8 * q + 7]);
        uint4 u;
        u.x = *reinterpret_cast<uint32_t*>(&p0);
        u.y = *reinterpret_cast<uint32_t*>(&p1);
        u.z = *reinterpret_cast<uint32_t*>(&p2);
        u.w = *reinterpret_cast<uint32_t*>(&p3);
        o[q] = u;
    }
}

// ---------------------------------------------------------------------------
// forward: encoder (+ layer-0 projection) and message-passing layers
// ---------------------------------------------------------------------------
struct Fwd {
    const float* w;
    const float* v;            // [N][5] direction
    float* z;                  // [N][5] output (last layer)
    const bf16* ctx;           // [N][32]
    const unsigned char* act;  // [N]
    Geo G;
    const float4* x4;          // [N] coordinates padded to 16 bytes (the same FP32 values as G.xf)
    const bf16* h_in;
    bf16* h_out;
    const bf16* P_in;
    bf16* P_out;
    float s;
    int layer;
    // training: what the backward needs
    float* Q_st;
    bf16* a_st;
    float* u_st;
    float* out_st;
};

constexpr int kEncSmem = (64 * LD48 + 64 * LD64) * 2 + (64 + 8) * 4 + 8 * (2 * 16 * LD64) * 2;

__global__ void __launch_bounds__(256, 2) k_net_enc(Fwd a) {
    extern __shared__ __align__(16) unsigned char smem[];
    bf16* sWe = reinterpret_cast<bf16*>(smem);
    bf16* sWp = sWe + 64 * LD48;
    float* sbe = reinterpret_cast<float*>(sWp + 64 * LD64);
    float* sal = sbe + 64;
    bf16* slabs = reinterpret_cast<bf16*>(sal + 8);
    stage_w(sWe, LD48, a.w + O_WE, H, FIN, H);
    stage_w(sWp, LD64, a.w + OL(0) + L_WP, H, H, H);
    for (int i = threadIdx.x; i < H; i += blockDim.x) sbe[i] = a.w[O_BE + i];
    if (threadIdx.x < 8) sal[threadIdx.x] = threadIdx.x < NOUT ? a.w[O_AL + threadIdx.x] : 0.f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    bf16* sx = slabs + warp * (2 * 16 * LD64);   // x (stride LD48), later the projection (stride LD64)
    bf16* sh = sx + 16 * LD64;
    const int N = a.G.N, nslab = (N + 15) / 16;
    for (int slab = blockIdx.x * 8 + warp; slab < nslab; slab += gridDim.x * 8) {
        const int n0 = slab * 16;
        // context features: 4 x 16 bytes per node
#pragma unroll
        for (int it = 0; it < 2; ++it) {
            const int idx = it * 32 + lane, r = idx >> 2, q = idx & 3, n = n0 + r;
            uint4 u = make_uint4(0, 0, 0, 0);
            if (n < N) u = __ldg(reinterpret_cast<const uint4*>(a.ctx + (size_t)FCTX * n) + q);
            *reinterpret_cast<uint4*>(sx + r * LD48 + 8 * q) = u;
        }
        // direction (5) and zeros (columns 37..55) as bf16 pairs from column 32
        for (int idx = lane; idx < 16 * 12; idx += 32) {
            const int r = idx / 12, f = FCTX + 2 * (idx - r * 12), n = n0 + r;
            float x0 = 0.f, x1 = 0.f;
            if (n < N) {
                x0 = feat(a.v, a.ctx, sal, a.s, n, f);
                x1 = feat(a.v, a.ctx, sal, a.s, n, f + 1);
            }
            *reinterpret_cast<bf162*>(sx + r * LD48 + f) = __floats2bfloat162_rn(x0, x1);
        }
        __syncwarp();
        float c[8][4];
        zero(c);
        warp_gemm<8>(c, sx, LD48, sWe, LD48, FIN);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = nt * 8 + 2 * t;
            *reinterpret_cast<bf162*>(sh + g * LD64 + col) =
                __floats2bfloat162_rn(fmaxf(c[nt][0] + sbe[col], 0.f), fmaxf(c[nt][1] + sbe[col + 1], 0.f));
            *reinterpret_cast<bf162*>(sh + (g + 8) * LD64 + col) =
                __floats2bfloat162_rn(fmaxf(c[nt][2] + sbe[col], 0.f), fmaxf(c[nt][3] + sbe[col + 1], 0.f));
        }
        __syncwarp();
        store_slab(a.h_out, sh, LD64, n0, N);
        zero(c);
        warp_gemm<8>(c, sh, LD64, sWp, LD64, H);
        __syncwarp();
        // the projection through the x area (free now) for 16-byte stores
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = nt * 8 + 2 * t;
            *reinterpret_cast<bf162*>(sx + g * LD64 + col) = __floats2bfloat162_rn(c[nt][0], c[nt][1]);
            *reinterpret_cast<bf162*>(sx + (g + 8) * LD64 + col) = __floats2bfloat162_rn(c[nt][2], c[nt][3]);
        }
        __syncwarp();
        store_slab(a.P_out, sx, LD64, n0, N);
        __syncwarp();
    }
}

constexpr int kEdgeCap = 16 * LD64 / 2;  // CSR entries of a slab that fit in the h area (576)
constexpr int kMpSmemW = (64 * LD64 + 64 * LD128 + 64 * LD64) * 2 + (64 + 64 + 192 + 8 + 8) * 4;
constexpr int kMpSmemWarp = (16 * LD64 + 16 * LD64) * 2 + 16 * LDQ * 4;
constexpr int kMpSmem = kMpSmemW + 8 * kMpSmemWarp;

// Sum over the neighbours of node n (edges [beg, end), their entries from the staged slab
// segment eb when given) of relu(Q_i + P_j + C e_ij), for the 8 channels [8 chunk, 8 chunk + 8)
// of this lane, in edge order; the gathers of eight edges are in flight at once.
constexpr int kAggU = 6;
__device__ __forceinline__ void aggregate(const Geo& G, const float4* __restrict__ x4, const bf16* __restrict__ P,
                                          int n, int beg, int end, const unsigned* eb, int eb0, const float* q,
                                          const float (*cw)[3], int chunk, float* acc) {
    const float4 xi = __ldg(x4 + n);
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = 0.f;
    for (int kb = beg; kb < end; kb += kAggU) {
        unsigned nb[kAggU];
        uint4 pv[kAggU];
        float4 xj[kAggU];
#pragma unroll
        for (int u = 0; u < kAggU; ++u) {
            const int k = kb + u;
            nb[u] = k < end ? (eb ? eb[k - eb0] : __ldg(G.nbr + k)) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kAggU; ++u) {
            if (kb + u < end) {
                const int j = (int)(nb[u] & NBMASK);
                pv[u] = __ldg(reinterpret_cast<const uint4*>(P + (size_t)j * H + 8 * chunk));
                xj[u] = __ldg(x4 + j);
            }
        }
#pragma unroll
        for (int u = 0; u < kAggU; ++u) {
            if (kb + u >= end) break;
            float e[3];
            edge_vec4(G, xi, xj[u], nb[u], e);
            const uint32_t pw[4] = {pv[u].x, pv[u].y, pv[u].z, pv[u].w};
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const float p = (c & 1) ? bfhi(pw[c >> 1]) : bflo(pw[c >> 1]);
                acc[c] += fmaxf(edge_pre(q[c], p, cw[c][0], cw[c][1], cw[c][2], e), 0.f);
            }
        }
    }
}

template <bool LAST, bool TRAIN>
__global__ void __launch_bounds__(256, 2) k_net_mp(Fwd a) {
    extern __shared__ __align__(16) unsigned char smem[];
    bf16* sWq = reinterpret_cast<bf16*>(smem);
    bf16* sWu = sWq + 64 * LD64;
    bf16* sWn = sWu + 64 * LD128;
    float* sbm = reinterpret_cast<float*>(sWn + 64 * LD64);
    float* sbu = sbm + 64;
    float* sC = sbu + 64;
    float* sbd = sC + 192;
    float* sbt = sbd + 8;
    unsigned char* wbase = reinterpret_cast<unsigned char*>(sbt + 8);
    const int l = a.layer;
    const float* wl = a.w + OL(l);
    stage_w(sWq, LD64, wl + L_WQ, H, H, H);
    stage_w(sWu, LD128, wl + L_WU, H, 2 * H, H);
    if (LAST) stage_w(sWn, LD64, a.w + O_WD, NOUT, H, 8);
    else stage_w(sWn, LD64, a.w + OL(l + 1) + L_WP, H, H, H);
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        sbm[i] = wl[L_BM + i];
        sbu[i] = wl[L_BU + i];
    }
    for (int i = threadIdx.x; i < 3 * H; i += blockDim.x) sC[i] = wl[L_C + i];
    if (threadIdx.x < 8) {
        sbd[threadIdx.x] = threadIdx.x < NOUT ? a.w[O_BD + threadIdx.x] : 0.f;
        sbt[threadIdx.x] = threadIdx.x < NOUT ? a.w[O_BT + threadIdx.x] : 0.f;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int slot = lane >> 3, chunk = lane & 7;
    bf16* sh = reinterpret_cast<bf16*>(wbase + warp * kMpSmemWarp);
    bf16* sa = sh + 16 * LD64;
    float* sQ = reinterpret_cast<float*>(sa + 16 * LD64);
    float cw[8][3];
#pragma unroll
    for (int c = 0; c < 8; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) cw[c][d] = sC[(8 * chunk + c) * 3 + d];
    const int N = a.G.N, nslab = (N + 15) / 16;
    for (int slab = blockIdx.x * 8 + warp; slab < nslab; slab += gridDim.x * 8) {
        const int n0 = slab * 16;
        load_slab(sh, LD64, a.h_in, n0, N);
        __syncwarp();
        // Q = W_q h + b_m (FP32, kept in shared memory for the edge loop)
        {
            float c[8][4];
            zero(c);
            warp_gemm<8>(c, sh, LD64, sWq, LD64, H);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int col = nt * 8 + 2 * t;
                const float2 q0 = make_float2(c[nt][0] + sbm[col], c[nt][1] + sbm[col + 1]);
                const float2 q1 = make_float2(c[nt][2] + sbm[col], c[nt][3] + sbm[col + 1]);
                *reinterpret_cast<float2*>(sQ + g * LDQ + col) = q0;
                *reinterpret_cast<float2*>(sQ + (g + 8) * LDQ + col) = q1;
                if (TRAIN) {
                    if (n0 + g < N) *reinterpret_cast<float2*>(a.Q_st + (size_t)(n0 + g) * H + col) = q0;
                    if (n0 + g + 8 < N) *reinterpret_cast<float2*>(a.Q_st + (size_t)(n0 + g + 8) * H + col) = q1;
                }
            }
        }
        __syncwarp();
        // the slab's CSR segment into the h area (free until h is loaded again below)
        const int st = lane <= 16 ? __ldg(a.G.nstart + min(n0 + lane, N)) : 0;
        const int sb = __shfl_sync(0xffffffffu, st, 0), se = __shfl_sync(0xffffffffu, st, 16);
        unsigned* eb = reinterpret_cast<unsigned*>(sh);
        const bool staged = se - sb <= kEdgeCap;
        if (staged)
            for (int k = lane; k < se - sb; k += 32) eb[k] = __ldg(a.G.nbr + sb + k);
        __syncwarp();
        // mean message of every node of the slab, four nodes at a time (lanes 8 slot + chunk)
        for (int it = 0; it < 4; ++it) {
            const int r = 4 * it + slot, n = n0 + r;
            const int beg = __shfl_sync(0xffffffffu, st, r), end = __shfl_sync(0xffffffffu, st, r + 1);
            const int deg = n < N ? end - beg : 0;
            float acc[8];
            if (n < N) {
                float q[8];
                const float4 qa = *reinterpret_cast<const float4*>(sQ + r * LDQ + 8 * chunk);
                const float4 qb = *reinterpret_cast<const float4*>(sQ + r * LDQ + 8 * chunk + 4);
                q[0] = qa.x; q[1] = qa.y; q[2] = qa.z; q[3] = qa.w;
                q[4] = qb.x; q[5] = qb.y; q[6] = qb.z; q[7] = qb.w;
                aggregate(a.G, a.x4, a.P_in, n, beg, end, staged ? eb : nullptr, sb, q, cw, chunk, acc);
            } else {
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[c] = 0.f;
            }
            {
                float m[8];
#pragma unroll
                for (int c = 0; c < 8; ++c) m[c] = deg > 0 ? __fdiv_rn(acc[c], (float)deg) : 0.f;
                bf162 p0 = __floats2bfloat162_rn(m[0], m[1]), p1 = __floats2bfloat162_rn(m[2], m[3]);
                bf162 p2 = __floats2bfloat162_rn(m[4], m[5]), p3 = __floats2bfloat162_rn(m[6], m[7]);
                uint4 u;
                u.x = *reinterpret_cast<uint32_t*>(&p0);
                u.y = *reinterpret_cast<uint32_t*>(&p1);
                u.z = *reinterpret_cast<uint32_t*>(&p2);
                u.w = *reinterpret_cast<uint32_t*>(&p3);
                *reinterpret_cast<uint4*>(sa + r * LD64 + 8 * chunk) = u;
            }
        }
        __syncwarp();
        load_slab(sh, LD64, a.h_in, n0, N);
        __syncwarp();
        if (TRAIN) store_slab(a.a_st, sa, LD64, n0, N);
        // h' = h + relu(W_u [h; a] + b_u), in place
        {
            float c[8][4];
            zero(c);
            warp_gemm<8>(c, sh, LD64, sWu, LD128, H);
            warp_gemm<8>(c, sa, LD64, sWu + H, LD128, H);
            __syncwarp();
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int col = nt * 8 + 2 * t;
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int r = g + 8 * hh;
                    const float u0 = c[nt][2 * hh] + sbu[col], u1 = c[nt][2 * hh + 1] + sbu[col + 1];
                    if (TRAIN && n0 + r < N)
                        *reinterpret_cast<float2*>(a.u_st + (size_t)(n0 + r) * H + col) = make_float2(u0, u1);
                    const uint32_t hv = ld32(sh + r * LD64 + col);
                    *reinterpret_cast<bf162*>(sh + r * LD64 + col) =
                        __floats2bfloat162_rn(bflo(hv) + fmaxf(u0, 0.f), bfhi(hv) + fmaxf(u1, 0.f));
                }
            }
        }
        __syncwarp();
        if (!LAST) {
            store_slab(a.h_out, sh, LD64, n0, N);
            float c[8][4];
            zero(c);
            warp_gemm<8>(c, sh, LD64, sWn, LD64, H);
            __syncwarp();
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int col = nt * 8 + 2 * t;
                *reinterpret_cast<bf162*>(sa + g * LD64 + col) = __floats2bfloat162_rn(c[nt][0], c[nt][1]);
                *reinterpret_cast<bf162*>(sa + (g + 8) * LD64 + col) = __floats2bfloat162_rn(c[nt][2], c[nt][3]);
            }
            __syncwarp();
            store_slab(a.P_out, sa, LD64, n0, N);
        } else {
            if (TRAIN) store_slab(a.h_out, sh, LD64, n0, N);
            float c[1][4];
            zero(c);
            warp_gemm<1>(c, sh, LD64, sWn, LD64, H);
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int n = n0 + g + 8 * hh;
                if (n >= N) continue;
                const bool on = a.act[n] != 0;
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int col = 2 * t + q;
                    const float o = c[0][2 * hh + q] + sbd[col];
                    if (TRAIN) a.out_st[8 * (size_t)n + col] = col < NOUT ? o : 0.f;
                    if (col < NOUT) {
                        const float vv = a.v[5 * (size_t)n + col];
                        a.z[5 * (size_t)n + col] = on ? vv + __fdiv_rn(__fmul_rn(sbt[col], o), a.s) : vv;
                    }
                }
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// backward (training)
// ---------------------------------------------------------------------------
struct Bwd {
    const float* w;
    Geo G;
    const unsigned char* act;
    const float* v;
    const float* t;
    const bf16* ctx;
    float s, nm;               // s = sqrt(5N); nm = 5 x active nodes
    const bf16* hs;            // 4 x 64N
    const bf16* ps;            // 3 x 64N
    const bf16* as;            // 3 x 64N
    const float* qs;           // 3 x 64N
    const float* us;           // 3 x 64N
    const float* out;          // 8N
    float* dh;                 // 64N
    float* dms;                // 64N
    bf16* dqp;                 // 128N
    float* part;               // grid x PSTRIDE
    int layer;
};

__device__ __forceinline__ size_t HN(const Geo& G) { return (size_t)G.N * H; }

// per-lane sums of a column pair (cols nt*8+2t, +1 over rows g, g+8) reduced over g (lanes
// t, t+4, ..., t+28) in a fixed tree; lanes 0..3 then hold the warp's sums
__device__ __forceinline__ float red_g(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    return v;
}

constexpr int kTopSmem = 128 * LD64 * 2 + 5 * 64 * 4 + 8 * (16 * LD64 * 2 + 16 * LDQ * 4 + 16 * 8 * 4) +
                         64 * LD128 * 2 + 128 * LD128 * 2 + 8 * (64 + 5 * 64 + 8) * 4;

// decoder backward and the update backward of the last layer
__global__ void __launch_bounds__(256, 1) k_bwd_top(Bwd a) {
    extern __shared__ __align__(16) unsigned char smem[];
    bf16* sWuT = reinterpret_cast<bf16*>(smem);                 // [128][LD64]: W_u^T of layer 2
    float* sWd = reinterpret_cast<float*>(sWuT + 128 * LD64);   // [5][64]
    unsigned char* wb = reinterpret_cast<unsigned char*>(sWd + 5 * 64);
    constexpr int WARPB = 16 * LD64 * 2 + 16 * LDQ * 4 + 16 * 8 * 4;
    bf16* sduT = reinterpret_cast<bf16*>(wb + 8 * WARPB);       // [64][LD128]
    bf16* shaT = sduT + 64 * LD128;                             // [128][LD128]
    float* sred = reinterpret_cast<float*>(shaT + 128 * LD128); // [8][64 + 320 + 8]
    const int l = NL - 1;
    const float* wl = a.w + OL(l);
    stage_wT(sWuT, LD64, wl + L_WU, H, 2 * H, 0);
    for (int i = threadIdx.x; i < 5 * 64; i += blockDim.x) sWd[i] = __bfloat162float(__float2bfloat16_rn(a.w[O_WD + i]));
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    bf16* sdu = reinterpret_cast<bf16*>(wb + warp * WARPB);
    float* sdh = reinterpret_cast<float*>(sdu + 16 * LD64);
    float* sdo = sdh + 16 * LDQ;
    const Geo& G = a.G;
    const int N = G.N, ntile = (N + TILE - 1) / TILE;
    const bf16* h3 = a.hs + 3 * HN(G);
    const bf16* h2 = a.hs + 2 * HN(G);
    const bf16* a2 = a.as + 2 * HN(G);
    const float* u2 = a.us + 2 * HN(G);
    float accw[8][4];
    zero(accw);
    float wd[5][2] = {}, bu[2] = {0.f, 0.f}, bd = 0.f, lacc = 0.f;
    const int c0 = 2 * lane;
    float beta[NOUT];
#pragma unroll
    for (int d = 0; d < NOUT; ++d) beta[d] = a.w[O_BT + d];
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int n0 = tile * TILE + warp * 16;
        for (int idx = lane; idx < 16 * 8; idx += 32) {
            const int r = idx >> 3, d = idx & 7, n = n0 + r;
            float dout = 0.f;
            if (d < NOUT && n < N && a.act[n]) {
                const float rt = __fdiv_rn(__fmul_rn(a.s, a.t[5 * (size_t)n + d] - a.v[5 * (size_t)n + d]), beta[d]);
                const float diff = a.out[8 * (size_t)n + d] - rt;
                lacc += diff * diff;
                dout = 2.f * diff / a.nm;
            }
            sdo[r * 8 + d] = dout;
        }
        __syncwarp();
        for (int r = 0; r < 16; ++r) {
            const int n = n0 + r;
            float h0 = 0.f, h1 = 0.f, uu0 = 0.f, uu1 = 0.f;
            if (n < N) {
                const uint32_t hv = ld32(h3 + (size_t)n * H + c0);
                h0 = bflo(hv);
                h1 = bfhi(hv);
                const float2 uv = *reinterpret_cast<const float2*>(u2 + (size_t)n * H + c0);
                uu0 = uv.x;
                uu1 = uv.y;
            }
            float dh0 = 0.f, dh1 = 0.f;
#pragma unroll
            for (int d = 0; d < NOUT; ++d) {
                const float o = sdo[r * 8 + d];
                wd[d][0] += o * h0;
                wd[d][1] += o * h1;
                dh0 += o * sWd[d * 64 + c0];
                dh1 += o * sWd[d * 64 + c0 + 1];
            }
            const float du0 = uu0 > 0.f ? dh0 : 0.f, du1 = uu1 > 0.f ? dh1 : 0.f;
            bu[0] += du0;
            bu[1] += du1;
            sdh[r * LDQ + c0] = dh0;
            sdh[r * LDQ + c0 + 1] = dh1;
            const bf162 db = __floats2bfloat162_rn(du0, du1);
            *reinterpret_cast<bf162*>(sdu + r * LD64 + c0) = db;
            sduT[c0 * LD128 + warp * 16 + r] = db.x;
            sduT[(c0 + 1) * LD128 + warp * 16 + r] = db.y;
        }
        if (lane < NOUT)
            for (int r = 0; r < 16; ++r) bd += sdo[r * 8 + lane];
        // [h2; a2]^T of the tile for the weight gradient
        for (int idx = lane; idx < 16 * 64; idx += 32) {
            const int r = idx >> 6, cp = idx & 63, n = n0 + r, col = 2 * cp;
            uint32_t v = 0;
            if (n < N) v = col < H ? ld32(h2 + (size_t)n * H + col) : ld32(a2 + (size_t)n * H + col - H);
            const bf162 b = *reinterpret_cast<bf162*>(&v);
            shaT[col * LD128 + warp * 16 + r] = b.x;
            shaT[(col + 1) * LD128 + warp * 16 + r] = b.y;
        }
        __syncwarp();
        // d[h; a] = du W_u: the h part adds into dh, the a part over deg is the message gradient
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            float c[8][4];
            zero(c);
            warp_gemm<8>(c, sdu, LD64, sWuT + half * 64 * LD64, LD64, H);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int col = nt * 8 + 2 * t;
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int r = g + 8 * hh, n = n0 + r;
                    if (n >= N) continue;
                    if (half == 0) {
                        const float2 o = make_float2(sdh[r * LDQ + col] + c[nt][2 * hh], sdh[r * LDQ + col + 1] + c[nt][2 * hh + 1]);
                        *reinterpret_cast<float2*>(a.dh + (size_t)n * H + col) = o;
                    } else {
                        const int deg = G.nstart[n + 1] - G.nstart[n];
                        const float2 o = deg > 0 ? make_float2(__fdiv_rn(c[nt][2 * hh], (float)deg), __fdiv_rn(c[nt][2 * hh + 1], (float)deg))
                                                 : make_float2(0.f, 0.f);
                        *reinterpret_cast<float2*>(a.dms + (size_t)n * H + col) = o;
                    }
                }
            }
        }
        __syncthreads();
        warp_gemm<8>(accw, sduT + (warp & 3) * 16 * LD128, LD128, shaT + (warp >> 2) * 64 * LD128, LD128, TILE);
        __syncthreads();
    }
    // partials of this CTA
    float* part = a.part + (size_t)blockIdx.x * PSTRIDE;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int o = (warp & 3) * 16 + g + 8 * (q >> 1), i = (warp >> 2) * 64 + nt * 8 + 2 * t + (q & 1);
            part[OL(l) + L_WU + o * 2 * H + i] = accw[nt][q];
        }
    float* sr = sred + warp * (64 + 320 + 8);
    sr[c0] = bu[0];
    sr[c0 + 1] = bu[1];
#pragma unroll
    for (int d = 0; d < NOUT; ++d) {
        sr[64 + d * 64 + c0] = wd[d][0];
        sr[64 + d * 64 + c0 + 1] = wd[d][1];
    }
    if (lane < NOUT) sr[384 + lane] = bd;
    float lw = lacc;
    for (int o = 16; o > 0; o >>= 1) lw += __shfl_xor_sync(0xffffffffu, lw, o);
    if (lane == 0) sr[389] = lw;
    __syncthreads();
    for (int i = threadIdx.x; i < 390; i += blockDim.x) {
        float s = 0.f;
        for (int w8 = 0; w8 < 8; ++w8) s += sred[w8 * (64 + 320 + 8) + i];
        if (i < 64) part[OL(l) + L_BU + i] = s;
        else if (i < 384) part[O_WD + (i - 64)] = s;
        else if (i < 389) part[O_BD + (i - 384)] = s;
        else part[NPARAM] = s;
    }
}

// message backward of layer l: dQ_i = sum_j [pre_ij > 0] dms_i, dP_i = sum_j [pre_ji > 0] dms_j,
// dC and db_m partials
__global__ void __launch_bounds__(256) k_bwd_edge(Bwd a) {
    __shared__ float sred[8][H * 4];
    const int l = a.layer;
    const float* wl = a.w + OL(l);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, c0 = 2 * lane;
    float cw[2][3];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) cw[c][d] = wl[L_C + (c0 + c) * 3 + d];
    const Geo& G = a.G;
    const int N = G.N;
    const float* Q = a.qs + l * HN(G);
    const bf16* P = a.ps + l * HN(G);
    float bm[2] = {0.f, 0.f}, dC[2][3] = {};
    for (int n = blockIdx.x * 8 + warp; n < N; n += gridDim.x * 8) {
        const int beg = G.nstart[n], end = G.nstart[n + 1];
        const float xi0 = G.xf[3 * (size_t)n], xi1 = G.xf[3 * (size_t)n + 1], xi2 = G.xf[3 * (size_t)n + 2];
        const float2 qi = *reinterpret_cast<const float2*>(Q + (size_t)n * H + c0);
        const uint32_t pu = ld32(P + (size_t)n * H + c0);
        const float pi[2] = {bflo(pu), bfhi(pu)};
        const float2 di = *reinterpret_cast<const float2*>(a.dms + (size_t)n * H + c0);
        const float qv[2] = {qi.x, qi.y}, dv[2] = {di.x, di.y};
        float dq[2] = {0.f, 0.f}, dp[2] = {0.f, 0.f};
        for (int k = beg; k < end; ++k) {
            const unsigned nb = G.nbr[k];
            float e[3], ne[3];
            const int j = edge_vec(G, xi0, xi1, xi2, nb, e);
            ne[0] = -e[0];
            ne[1] = -e[1];
            ne[2] = -e[2];
            const uint32_t pju = ld32(P + (size_t)j * H + c0);
            const float pj[2] = {bflo(pju), bfhi(pju)};
            const float2 qj = *reinterpret_cast<const float2*>(Q + (size_t)j * H + c0);
            const float2 dj = *reinterpret_cast<const float2*>(a.dms + (size_t)j * H + c0);
            const float qjv[2] = {qj.x, qj.y}, djv[2] = {dj.x, dj.y};
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                if (edge_pre(qv[c], pj[c], cw[c][0], cw[c][1], cw[c][2], e) > 0.f) {
                    dq[c] += dv[c];
                    dC[c][0] += dv[c] * e[0];
                    dC[c][1] += dv[c] * e[1];
                    dC[c][2] += dv[c] * e[2];
                }
                if (edge_pre(qjv[c], pi[c], cw[c][0], cw[c][1], cw[c][2], ne) > 0.f) dp[c] += djv[c];
            }
        }
        *reinterpret_cast<bf162*>(a.dqp + (size_t)n * 2 * H + c0) = __floats2bfloat162_rn(dq[0], dq[1]);
        *reinterpret_cast<bf162*>(a.dqp + (size_t)n * 2 * H + H + c0) = __floats2bfloat162_rn(dp[0], dp[1]);
        bm[0] += dq[0];
        bm[1] += dq[1];
    }
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        sred[warp][c0 + c] = bm[c];
#pragma unroll
        for (int d = 0; d < 3; ++d) sred[warp][H + (c0 + c) * 3 + d] = dC[c][d];
    }
    __syncthreads();
    float* part = a.part + (size_t)blockIdx.x * PSTRIDE;
    for (int i = threadIdx.x; i < 4 * H; i += blockDim.x) {
        float s = 0.f;
        for (int w8 = 0; w8 < 8; ++w8) s += sred[w8][i];
        if (i < H) part[OL(l) + L_BM + i] = s;
        else part[OL(l) + L_C + (i - H)] = s;
    }
}

constexpr int kNodeWarpB = 16 * LD128 * 2 + 16 * LD64 * 2;  // sdq (aliased by sdh: 16 x LDQ floats) + sdu
static_assert(16 * LD128 * 2 >= 16 * LDQ * 4, "sdh fits in the sdq area");
constexpr int kNodeSmem = 64 * LD128 * 2 + 128 * LD64 * 2 + 8 * kNodeWarpB + 128 * LD128 * 2 + 64 * LD128 * 2 +
                          64 * LD128 * 2 + 128 * LD128 * 2 + 8 * 64 * 4 + 64;

// projection backward of layer l (dh += [dQ dP] [W_q; W_p], dW_q, dW_p), then either the update
// backward of layer l - 1 (l >= 1) or the encoder backward (l == 0)
template <bool ENC>
__global__ void __launch_bounds__(256, 1) k_bwd_node(Bwd a) {
    extern __shared__ __align__(16) unsigned char smem[];
    bf16* sWqpT = reinterpret_cast<bf16*>(smem);               // [64][LD128]: [W_q; W_p]^T
    bf16* sWuT = sWqpT + 64 * LD128;                           // [128][LD64]: W_u^T of layer l-1
    unsigned char* wb = reinterpret_cast<unsigned char*>(sWuT + 128 * LD64);
    bf16* sdqpT = reinterpret_cast<bf16*>(wb + 8 * kNodeWarpB); // [128][LD128]
    bf16* shT = sdqpT + 128 * LD128;                           // [64][LD128]
    bf16* sduT = shT + 64 * LD128;                             // [64][LD128] (ENC: dpre_e^T)
    bf16* shaT = sduT + 64 * LD128;                            // [128][LD128] (ENC: x^T, 48 rows)
    float* sred = reinterpret_cast<float*>(shaT + 128 * LD128); // [8][64]
    float* sal = sred + 8 * 64;                                 // alpha
    const int l = a.layer;
    const float* wl = a.w + OL(l);
    stage_wT(sWqpT, LD128, wl + L_WQ, H, H, 0);
    stage_wT(sWqpT, LD128, wl + L_WP, H, H, H);
    if (!ENC) stage_wT(sWuT, LD64, a.w + OL(l - 1) + L_WU, H, 2 * H, 0);
    if (threadIdx.x < 8) sal[threadIdx.x] = threadIdx.x < NOUT ? a.w[O_AL + threadIdx.x] : 0.f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    bf16* sdq = reinterpret_cast<bf16*>(wb + warp * kNodeWarpB);
    float* sdh = reinterpret_cast<float*>(sdq);
    bf16* sdu = sdq + 16 * LD128;
    const Geo& G = a.G;
    const int N = G.N, ntile = (N + TILE - 1) / TILE;
    const bf16* hl = a.hs + l * HN(G);                       // input of layer l
    const bf16* hp = ENC ? a.hs : a.hs + (l - 1) * HN(G);    // input of layer l-1 (ENC: h0 for its mask)
    const bf16* ap = ENC ? nullptr : a.as + (l - 1) * HN(G);
    const float* up = ENC ? nullptr : a.us + (l - 1) * HN(G);
    float accq[8][4], accu[8][4], acce[3][4];
    zero(accq);
    zero(accu);
    zero(acce);
    float bsum[8][2] = {};
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int n0 = tile * TILE + warp * 16, rb = warp * 16;
        // [dQ dP] rows (A operand) and transposed (weight gradient), h_l transposed
        for (int idx = lane; idx < 16 * 16; idx += 32) {
            const int r = idx >> 4, c = (idx & 15) * 8, n = n0 + r;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (n < N) v = *reinterpret_cast<const uint4*>(a.dqp + (size_t)n * 2 * H + c);
            *reinterpret_cast<uint4*>(sdq + r * LD128 + c) = v;
            const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
            for (int k = 0; k < 8; ++k) sdqpT[(c + k) * LD128 + rb + r] = e[k];
        }
        for (int idx = lane; idx < 16 * 8; idx += 32) {
            const int r = idx >> 3, c = (idx & 7) * 8, n = n0 + r;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (n < N) v = *reinterpret_cast<const uint4*>(hl + (size_t)n * H + c);
            const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
            for (int k = 0; k < 8; ++k) shT[(c + k) * LD128 + rb + r] = e[k];
        }
        if (!ENC) {
            for (int idx = lane; idx < 16 * 16; idx += 32) {
                const int r = idx >> 4, c = (idx & 15) * 8, n = n0 + r;
                uint4 v = make_uint4(0, 0, 0, 0);
                if (n < N) v = c < H ? *reinterpret_cast<const uint4*>(hp + (size_t)n * H + c)
                                     : *reinterpret_cast<const uint4*>(ap + (size_t)n * H + c - H);
                const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
                for (int k = 0; k < 8; ++k) shaT[(c + k) * LD128 + rb + r] = e[k];
            }
        } else {
            for (int idx = lane; idx < 16 * FIN; idx += 32) {
                const int r = idx / FIN, f = idx - r * FIN, n = n0 + r;
                const float x = n < N ? feat(a.v, a.ctx, sal, a.s, n, f) : 0.f;
                shaT[f * LD128 + rb + r] = __float2bfloat16_rn(x);
            }
        }
        __syncwarp();
        float c[8][4];
        zero(c);
        warp_gemm<8>(c, sdq, LD128, sWqpT, LD128, 2 * H);
        __syncwarp();
        // dh = dh_in + [dQ dP][W_q; W_p]; then the relu mask of layer l-1's update (or of h0)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = nt * 8 + 2 * t;
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int r = g + 8 * hh, n = n0 + r;
                float d0 = 0.f, d1 = 0.f, m0 = 0.f, m1 = 0.f;
                if (n < N) {
                    const float2 din = *reinterpret_cast<const float2*>(a.dh + (size_t)n * H + col);
                    d0 = din.x + c[nt][2 * hh];
                    d1 = din.y + c[nt][2 * hh + 1];
                    if (ENC) {
                        const uint32_t hv = ld32(hp + (size_t)n * H + col);
                        m0 = bflo(hv) > 0.f ? d0 : 0.f;
                        m1 = bfhi(hv) > 0.f ? d1 : 0.f;
                    } else {
                        const float2 uv = *reinterpret_cast<const float2*>(up + (size_t)n * H + col);
                        m0 = uv.x > 0.f ? d0 : 0.f;
                        m1 = uv.y > 0.f ? d1 : 0.f;
                    }
                }
                bsum[nt][0] += m0;
                bsum[nt][1] += m1;
                const bf162 mb = __floats2bfloat162_rn(m0, m1);
                sduT[col * LD128 + rb + r] = mb.x;
                sduT[(col + 1) * LD128 + rb + r] = mb.y;
                if (!ENC) {
                    sdh[r * LDQ + col] = d0;
                    sdh[r * LDQ + col + 1] = d1;
                    *reinterpret_cast<bf162*>(sdu + r * LD64 + col) = mb;
                }
            }
        }
        __syncwarp();
        if (!ENC) {
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                float c2[8][4];
                zero(c2);
                warp_gemm<8>(c2, sdu, LD64, sWuT + half * 64 * LD64, LD64, H);
#pragma unroll
                for (int nt = 0; nt < 8; ++nt) {
                    const int col = nt * 8 + 2 * t;
#pragma unroll
                    for (int hh = 0; hh < 2; ++hh) {
                        const int r = g + 8 * hh, n = n0 + r;
                        if (n >= N) continue;
                        if (half == 0) {
                            *reinterpret_cast<float2*>(a.dh + (size_t)n * H + col) =
                                make_float2(sdh[r * LDQ + col] + c2[nt][2 * hh], sdh[r * LDQ + col + 1] + c2[nt][2 * hh + 1]);
                        } else {
                            const int deg = G.nstart[n + 1] - G.nstart[n];
                            *reinterpret_cast<float2*>(a.dms + (size_t)n * H + col) =
                                deg > 0 ? make_float2(__fdiv_rn(c2[nt][2 * hh], (float)deg), __fdiv_rn(c2[nt][2 * hh + 1], (float)deg))
                                        : make_float2(0.f, 0.f);
                        }
                    }
                }
            }
        }
        __syncthreads();
        // weight gradients over the tile's 128 nodes
        warp_gemm<8>(accq, sdqpT + warp * 16 * LD128, LD128, shT, LD128, TILE);
        if (!ENC) {
            warp_gemm<8>(accu, sduT + (warp & 3) * 16 * LD128, LD128, shaT + (warp >> 2) * 64 * LD128, LD128, TILE);
        } else {
            warp_gemm<3>(acce, sduT + (warp & 3) * 16 * LD128, LD128, shaT + (warp >> 2) * 24 * LD128, LD128, TILE);
        }
        __syncthreads();
    }
    float* part = a.part + (size_t)blockIdx.x * PSTRIDE;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int o = warp * 16 + g + 8 * (q >> 1), i = nt * 8 + 2 * t + (q & 1);
            if (o < H) part[OL(l) + L_WQ + o * H + i] = accq[nt][q];
            else part[OL(l) + L_WP + (o - H) * H + i] = accq[nt][q];
        }
    if (!ENC) {
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int o = (warp & 3) * 16 + g + 8 * (q >> 1), i = (warp >> 2) * 64 + nt * 8 + 2 * t + (q & 1);
                part[OL(l - 1) + L_WU + o * 2 * H + i] = accu[nt][q];
            }
    } else {
#pragma unroll
        for (int nt = 0; nt < 3; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int o = (warp & 3) * 16 + g + 8 * (q >> 1), f = (warp >> 2) * 24 + nt * 8 + 2 * t + (q & 1);
                part[O_WE + o * FIN + f] = acce[nt][q];
            }
    }
    // bias of layer l-1's update (or of the encoder): fixed-order reduction over g, then warps
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float s0 = red_g(bsum[nt][0]), s1 = red_g(bsum[nt][1]);
        if (g == 0) {
            sred[warp * 64 + nt * 8 + 2 * t] = s0;
            sred[warp * 64 + nt * 8 + 2 * t + 1] = s1;
        }
    }
    __syncthreads();
    if (threadIdx.x < H) {
        float s = 0.f;
        for (int w8 = 0; w8 < 8; ++w8) s += sred[w8 * 64 + threadIdx.x];
        if (ENC) part[O_BE + threadIdx.x] = s;
        else part[OL(l - 1) + L_BU + threadIdx.x] = s;
    }
}

// gradient (and loss) = sum of the CTAs' partials in CTA order
__global__ void k_grad_reduce(const float* __restrict__ part, int G, float* __restrict__ grad, double* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > NPARAM) return;
    double s = 0.0;
    for (int c = 0; c < G; ++c) s += (double)part[(size_t)c * PSTRIDE + p];
    if (p < NPARAM) grad[p] = p < O_AL ? (float)s : 0.f;
    else if (loss) *loss = s;
}

__global__ void __launch_bounds__(1024) k_grad_norm(const float* __restrict__ grad, double* __restrict__ out) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int p = threadIdx.x; p < O_AL; p += blockDim.x) s += (double)grad[p] * grad[p];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < 32; ++w) tot += sh[w];
        *out = tot;
    }
}

struct AdamP {
    float lr, b1, b2, eps, clip, c1, c2;  // c1 = 1 - b1^t, c2 = 1 - b2^t
};
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, AdamP p, const double* __restrict__ gn2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= O_AL) return;
    float sc = 1.f;
    if (p.clip > 0.f) {
        const float gn = (float)sqrt(*gn2);
        if (gn > p.clip) sc = p.clip / gn;
    }
    const float gi = grad[i] * sc;
    const float mi = p.b1 * m[i] + (1.f - p.b1) * gi;
    const float vi = p.b2 * v[i] + (1.f - p.b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= p.lr * (mi / p.c1) / (sqrtf(vi / p.c2) + p.eps);
}

// per-dof sums of (s v)^2 and (s (t - v))^2 over the active nodes of all pairs
__global__ void __launch_bounds__(256) k_pair_stats(const float* __restrict__ V, const float* __restrict__ T,
                                                    const unsigned char* __restrict__ act, int N, int npairs, float s,
                                                    double* __restrict__ part) {
    double acc[10] = {};
    const size_t tot = (size_t)npairs * N;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const int n = (int)(i % N);
        if (!act[n]) continue;
#pragma unroll
        for (int d = 0; d < 5; ++d) {
            const double vv = (double)s * V[5 * i + d], dd = (double)s * ((double)T[5 * i + d] - V[5 * i + d]);
            acc[d] += vv * vv;
            acc[5 + d] += dd * dd;
        }
    }
    __shared__ double sh[8][10];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 10) {
        double v = 0.0;
        for (int w8 = 0; w8 < 8; ++w8) v += sh[w8][threadIdx.x];
        part[(size_t)blockIdx.x * 10 + threadIdx.x] = v;
    }
}

// pair slot: v = Aw / ||Aw||, t = w / ||Aw||  (||Aw||^2 in *nrm2)
__global__ void k_pair_store(const float* __restrict__ Aw, const float* __restrict__ w, const double* __restrict__ nrm2,
                             size_t n5, float* __restrict__ V, float* __restrict__ T) {
    const double inv = 1.0 / sqrt(*nrm2);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n5; i += (size_t)gridDim.x * blockDim.x) {
        V[i] = (float)(Aw[i] * inv);
        T[i] = (float)(w[i] * inv);
    }
}

}  // namespace netk

// ============================================================================
// host side
// ============================================================================
namespace {

using namespace netk;

template <typename T>
int nalloc(Ctx& C, T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    const cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
    if (e != cudaSuccess) return fail(C, PHGPU_ERR_NOMEM, std::string("cudaMalloc (network): ") + cudaGetErrorString(e));
    return PHGPU_OK;
}
#define NT_TRY(x)                      \
    do {                               \
        int _s = (x);                  \
        if (_s != PHGPU_OK) return _s; \
    } while (0)

const int kTetE[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
const int kHexE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int kWedE[9][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 4}, {4, 5}, {5, 3}, {0, 3}, {1, 4}, {2, 5}};

// The CSR of directed edges between periodic masters with the shift code of each (see the file
// header); built once per context on the host from the element blocks.
int build_graph(Ctx& C) {
    const int N = C.N;
    if (N >= (1 << SHIFT)) return fail(C, PHGPU_ERR_UNSUPPORTED, "learned preconditioner: more than 2^26 nodes");
    std::vector<double> x(3 * (size_t)N);
    std::vector<int> iper(N), iBC(N);
    NT_TRY(d2h(C, x.data(), C.d_x, sizeof(double) * x.size(), "graph: x"));
    NT_TRY(d2h(C, iper.data(), C.d_iper, sizeof(int) * N, "graph: iper"));
    NT_TRY(d2h(C, iBC.data(), C.d_iBC, sizeof(int) * N, "graph: iBC"));
    struct Blk {
        const int* ien;
        size_t ne;
        int nen, nedge;
        const int (*edges)[2];
    };
    const Blk blks[3] = {{C.h_ien.data(), (size_t)C.E, 4, 6, kTetE},
                         {C.h_ienh.data(), (size_t)C.nhex, 8, 12, kHexE},
                         {C.h_ienw.data(), (size_t)C.nwedge, 6, 9, kWedE}};
    // pass 1: periods and counts
    double L[3] = {0.0, 0.0, 0.0};
    std::vector<long long> cnt((size_t)N + 1, 0);
    for (const Blk& b : blks)
        for (size_t e = 0; e < b.ne; ++e) {
            const int* c = b.ien + b.nen * e;
            for (int k = 0; k < b.nedge; ++k) {
                const int pa = c[b.edges[k][0]], pb = c[b.edges[k][1]];
                const int i = iper[pa], j = iper[pb];
                if (i == j) continue;
                for (int d = 0; d < 3; ++d) {
                    const double diff = (x[3 * (size_t)pb + d] - x[3 * (size_t)pa + d]) - (x[3 * (size_t)j + d] - x[3 * (size_t)i + d]);
                    L[d] = std::max(L[d], std::fabs(diff));
                }
                ++cnt[i];
                ++cnt[j];
            }
        }
    std::vector<long long> off((size_t)N + 1, 0);
    for (int n = 0; n < N; ++n) off[n + 1] = off[n] + cnt[n];
    std::vector<unsigned> ent((size_t)off[N]);
    std::vector<long long> pos(off.begin(), off.end() - 1);
    auto code_of = [&](double diff, int d, bool& ok) -> unsigned {
        if (L[d] <= 0.0) {
            ok = ok && std::fabs(diff) <= 1e-12;
            return 0u;
        }
        const double k = std::nearbyint(diff / L[d]);
        ok = ok && std::fabs(diff - k * L[d]) <= 1e-9 * std::max(L[d], 1.0) && std::fabs(k) <= 1.0;
        return k > 0.5 ? 1u : (k < -0.5 ? 2u : 0u);
    };
    bool ok = true;
    for (const Blk& b : blks)
        for (size_t e = 0; e < b.ne; ++e) {
            const int* c = b.ien + b.nen * e;
            for (int k = 0; k < b.nedge; ++k) {
                const int pa = c[b.edges[k][0]], pb = c[b.edges[k][1]];
                const int i = iper[pa], j = iper[pb];
                if (i == j) continue;
                unsigned code = 0, neg = 0;
                for (int d = 0; d < 3; ++d) {
                    const double diff = (x[3 * (size_t)pb + d] - x[3 * (size_t)pa + d]) - (x[3 * (size_t)j + d] - x[3 * (size_t)i + d]);
                    const unsigned cd = code_of(diff, d, ok);
                    code |= cd << (2 * d);
                    neg |= (cd == 1 ? 2u : cd == 2 ? 1u : 0u) << (2 * d);
                }
                ent[pos[i]++] = (unsigned)j | (code << SHIFT);
                ent[pos[j]++] = (unsigned)i | (neg << SHIFT);
            }
        }
    if (!ok) return fail(C, PHGPU_ERR_UNSUPPORTED, "learned preconditioner: periodicity is not a translation by the box size");
    // ascending (neighbour, code) per node, duplicates removed
    std::vector<int> nstart((size_t)N + 1, 0);
    long long w = 0;
    for (int n = 0; n < N; ++n) {
        unsigned* b = ent.data() + off[n];
        unsigned* e = ent.data() + off[n + 1];
        std::sort(b, e, [](unsigned p, unsigned q) {
            const unsigned jp = p & NBMASK, jq = q & NBMASK;
            return jp != jq ? jp < jq : (p >> SHIFT) < (q >> SHIFT);
        });
        unsigned* u = std::unique(b, e);
        nstart[n] = (int)w;
        for (unsigned* p = b; p < u; ++p) ent[w++] = *p;
        if (w > 0x7fffffffLL) return fail(C, PHGPU_ERR_TOO_LARGE, "learned preconditioner: more than 2^31 edges");
    }
    nstart[N] = (int)w;
    ent.resize(w);
    // mean edge length and the active nodes
    double hs = 0.0;
    for (int n = 0; n < N; ++n)
        for (int k = nstart[n]; k < nstart[n + 1]; ++k) {
            const unsigned nb = ent[k];
            const int j = (int)(nb & NBMASK);
            double s2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                const unsigned cd = (nb >> (SHIFT + 2 * d)) & 3;
                const double dd = x[3 * (size_t)j + d] - x[3 * (size_t)n + d] + (cd == 1 ? L[d] : cd == 2 ? -L[d] : 0.0);
                s2 += dd * dd;
            }
            hs += std::sqrt(s2);
        }
    NetCtx& T = C.net;
    T.hbar = w > 0 ? hs / (double)w : 1.0;
    T.rh = (float)(1.0 / T.hbar);
    for (int d = 0; d < 3; ++d) T.L[d] = (float)L[d];
    std::vector<unsigned char> act(N);
    T.nact = 0;
    for (int n = 0; n < N; ++n) {
        act[n] = (iper[n] == n && (iBC[n] & 63) == 0) ? 1 : 0;
        T.nact += act[n];
    }
    T.nnz = w;
    NT_TRY(nalloc(C, &T.d_nstart, (size_t)N + 1));
    NT_TRY(nalloc(C, &T.d_nbr, (size_t)std::max<long long>(w, 1)));
    NT_TRY(nalloc(C, &T.d_act, (size_t)N));
    {
        std::vector<float4> x4(N);
        for (int n = 0; n < N; ++n)
            x4[n] = make_float4((float)x[3 * (size_t)n], (float)x[3 * (size_t)n + 1], (float)x[3 * (size_t)n + 2], 0.f);
        NT_TRY(nalloc(C, &T.d_x4, (size_t)N));
        NT_TRY(h2d(C, T.d_x4, x4.data(), sizeof(float4) * N, "graph"));
    }
    NT_TRY(h2d(C, T.d_nstart, nstart.data(), sizeof(int) * nstart.size(), "graph"));
    if (w > 0) NT_TRY(h2d(C, T.d_nbr, ent.data(), sizeof(unsigned) * w, "graph"));
    NT_TRY(h2d(C, T.d_act, act.data(), N, "graph"));
    T.graph = true;
    return PHGPU_OK;
}

Geo geo(const Ctx& C) {
    Geo G;
    G.nstart = C.net.d_nstart;
    G.nbr = C.net.d_nbr;
    G.xf = C.d_xf;
    G.L0 = C.net.L[0];
    G.L1 = C.net.L[1];
    G.L2 = C.net.L[2];
    G.rh = C.net.rh;
    G.N = C.N;
    return G;
}

int num_sms() {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 152;
}

// once per context (function attributes belong to the device the context runs on)
int set_attrs(Ctx& C) {
    if (C.net.attrs_set) return PHGPU_OK;
    NT_TRY(check(C, smem_attr(k_net_enc, cudaFuncAttributeMaxDynamicSharedMemorySize, kEncSmem), "attr"));
    NT_TRY(check(C, smem_attr(k_net_mp<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMpSmem), "attr"));
    NT_TRY(check(C, smem_attr(k_net_mp<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMpSmem), "attr"));
    NT_TRY(check(C, smem_attr(k_net_mp<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMpSmem), "attr"));
    NT_TRY(check(C, smem_attr(k_net_mp<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMpSmem), "attr"));
    NT_TRY(check(C, smem_attr(k_bwd_top, cudaFuncAttributeMaxDynamicSharedMemorySize, kTopSmem), "attr"));
    NT_TRY(check(C, smem_attr(k_bwd_node<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kNodeSmem), "attr"));
    NT_TRY(check(C, smem_attr(k_bwd_node<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kNodeSmem), "attr"));
    C.net.attrs_set = true;
    return PHGPU_OK;
}

// forward over all layers; train: keep the activations in the training buffers
void forward(Ctx& C, const float* v, float* z, const bf16* ctx, bool train) {
    NetCtx& T = C.net;
    NetTrain& R = T.tr;
    const size_t HNs = (size_t)C.N * H;
    const int genc = T.grid_mp;
    Fwd a{};
    a.w = T.d_w;
    a.v = v;
    a.z = z;
    a.ctx = ctx;
    a.act = T.d_act;
    a.G = geo(C);
    a.x4 = T.d_x4;
    a.s = (float)std::sqrt(5.0 * C.N);
    a.h_out = train ? R.d_hs : T.d_h;
    a.P_out = train ? R.d_ps : T.d_P0;
    k_net_enc<<<genc, 256, kEncSmem, C.stream>>>(a);
    ++C.launches;
    for (int l = 0; l < NL; ++l) {
        Fwd b = a;
        b.layer = l;
        if (train) {
            b.h_in = R.d_hs + l * HNs;
            b.h_out = R.d_hs + (l + 1) * HNs;
            b.P_in = R.d_ps + l * HNs;
            b.P_out = l + 1 < NL ? R.d_ps + (l + 1) * HNs : nullptr;
            b.Q_st = R.d_qs + l * HNs;
            b.a_st = R.d_as + l * HNs;
            b.u_st = R.d_us + l * HNs;
            b.out_st = R.d_out;
        } else {
            b.h_in = T.d_h;
            b.h_out = T.d_h;
            b.P_in = (l & 1) ? T.d_P1 : T.d_P0;
            b.P_out = (l & 1) ? T.d_P0 : T.d_P1;
        }
        if (l + 1 < NL) {
            if (train) k_net_mp<false, true><<<genc, 256, kMpSmem, C.stream>>>(b);
            else k_net_mp<false, false><<<genc, 256, kMpSmem, C.stream>>>(b);
        } else {
            if (train) k_net_mp<true, true><<<genc, 256, kMpSmem, C.stream>>>(b);
            else k_net_mp<true, false><<<genc, 256, kMpSmem, C.stream>>>(b);
        }
        ++C.launches;
    }
}

int train_alloc(Ctx& C) {
    NetTrain& R = C.net.tr;
    if (R.d_hs) return PHGPU_OK;
    const size_t HNs = (size_t)C.N * H;
    NT_TRY(nalloc(C, &R.d_hs, 4 * HNs));
    NT_TRY(nalloc(C, &R.d_ps, 3 * HNs));
    NT_TRY(nalloc(C, &R.d_as, 3 * HNs));
    NT_TRY(nalloc(C, &R.d_qs, 3 * HNs));
    NT_TRY(nalloc(C, &R.d_us, 3 * HNs));
    NT_TRY(nalloc(C, &R.d_out, 8 * (size_t)C.N));
    NT_TRY(nalloc(C, &R.d_dh, HNs));
    NT_TRY(nalloc(C, &R.d_dms, HNs));
    NT_TRY(nalloc(C, &R.d_dqp, 2 * HNs));
    const int ntile = (C.N + TILE - 1) / TILE;
    R.grid = std::max(1, std::min(ntile, num_sms()));
    NT_TRY(nalloc(C, &R.d_part, (size_t)R.grid * PSTRIDE));
    NT_TRY(dzero(C, R.d_part, sizeof(float) * (size_t)R.grid * PSTRIDE, "memset"));
    NT_TRY(nalloc(C, &R.d_grad, NPARAM));
    NT_TRY(nalloc(C, &R.d_m, NPARAM));
    NT_TRY(nalloc(C, &R.d_v, NPARAM));
    NT_TRY(dzero(C, R.d_m, sizeof(float) * NPARAM, "memset"));
    NT_TRY(dzero(C, R.d_v, sizeof(float) * NPARAM, "memset"));
    return PHGPU_OK;
}

int scal_room(Ctx& C, int n) {
    NetTrain& R = C.net.tr;
    if (R.scal_cap >= n) return PHGPU_OK;
    if (R.d_scal) cudaFree(R.d_scal);
    R.d_scal = nullptr;
    R.scal_cap = 0;
    NT_TRY(nalloc(C, &R.d_scal, (size_t)n));
    R.scal_cap = n;
    return PHGPU_OK;
}

// loss and gradient of one pair (forward with stored activations, backward, fixed-order reduce)
void backward(Ctx& C, const float* v, const float* t, const bf16* ctx, double* loss_slot) {
    NetCtx& T = C.net;
    NetTrain& R = T.tr;
    Bwd b{};
    b.w = T.d_w;
    b.G = geo(C);
    b.act = T.d_act;
    b.v = v;
    b.t = t;
    b.ctx = ctx;
    b.s = (float)std::sqrt(5.0 * C.N);
    b.nm = (float)std::max(5.0 * T.nact, 1.0);
    b.hs = R.d_hs;
    b.ps = R.d_ps;
    b.as = R.d_as;
    b.qs = R.d_qs;
    b.us = R.d_us;
    b.out = R.d_out;
    b.dh = R.d_dh;
    b.dms = R.d_dms;
    b.dqp = R.d_dqp;
    b.part = R.d_part;
    const int G = R.grid;
    k_bwd_top<<<G, 256, kTopSmem, C.stream>>>(b);
    ++C.launches;
    for (int l = NL - 1; l >= 0; --l) {
        b.layer = l;
        k_bwd_edge<<<G, 256, 0, C.stream>>>(b);
        if (l > 0) k_bwd_node<false><<<G, 256, kNodeSmem, C.stream>>>(b);
        else k_bwd_node<true><<<G, 256, kNodeSmem, C.stream>>>(b);
        C.launches += 2;
    }
    k_grad_reduce<<<(NPARAM + 1 + 255) / 256, 256, 0, C.stream>>>(R.d_part, G, R.d_grad, loss_slot);
    ++C.launches;
}

}  // namespace

// ---------------------------------------------------------------------------
// interface to the solver
// ---------------------------------------------------------------------------
bool net_usable(const Ctx& C) { return C.net.have_w; }

int net_setup(Ctx& C) {
    NetCtx& T = C.net;
    NT_TRY(set_attrs(C));
    if (!T.graph) NT_TRY(build_graph(C));
    const size_t HNs = (size_t)C.N * H;
    if (!T.d_w) {
        NT_TRY(nalloc(C, &T.d_w, NPARAM));
        NT_TRY(dzero(C, T.d_w, sizeof(float) * NPARAM, "memset"));
    }
    if (!T.d_ctx) {
        NT_TRY(nalloc(C, &T.d_ctx, (size_t)FCTX * C.N));
        NT_TRY(nalloc(C, &T.d_stat, 32));
        NT_TRY(nalloc(C, &T.d_spart, (size_t)kStatBlocks * kStatN));
        NT_TRY(nalloc(C, &T.d_h, HNs));
        NT_TRY(nalloc(C, &T.d_P0, HNs));
        NT_TRY(nalloc(C, &T.d_P1, HNs));
    }
    if (!T.d_Z && C.cfg.precision == PHGPU_MIXED) NT_TRY(nalloc(C, &T.d_Z, C.ldU * (size_t)C.Ucap));
    if (!T.ev0) {
        NT_TRY(check(C, cudaEventCreate(&T.ev0), "event"));
        NT_TRY(check(C, cudaEventCreate(&T.ev1), "event"));
    }
    // persistent grid of the forward kernels: two CTAs per SM (shared memory and 128 registers
    // allow two), 8 slabs of 16 nodes per CTA pass
    const int nslab = (C.N + 15) / 16;
    T.grid_mp = std::max(1, std::min((nslab + 7) / 8, 2 * num_sms()));
    T.grid_enc = T.grid_mp;
    return PHGPU_OK;
}

int net_prepare(Ctx& C) {
    NT_TRY(net_setup(C));
    NetCtx& T = C.net;
    k_ctx_stats<<<kStatBlocks, kStatThreads, 0, C.stream>>>(C.d_bdf, C.d_y, T.d_act, C.N, T.d_spart);
    k_ctx_final<<<1, 32, 0, C.stream>>>(T.d_spart, kStatBlocks, C.cfg.Rgas, C.cfg.gamma, T.d_stat);
    k_ctx_features<<<(C.N + 255) / 256, 256, 0, C.stream>>>(C.d_bdf, C.d_y, T.d_act, T.d_stat, C.N, T.d_ctx);
    C.launches += 3;
    return check(C, cudaGetLastError(), "network context features");
}

void net_apply(Ctx& C, const float* v, float* z) { forward(C, v, z, C.net.d_ctx, false); }

int net_store_pair(Ctx& C, int slot, const float* Aw, const float* w, const double* nrm2) {
    NetTrain& R = C.net.tr;
    if (slot < 0 || slot >= R.cap) return fail(C, PHGPU_ERR_INVALID, "pair slot outside the allocated training set");
    const size_t n5 = 5 * (size_t)C.N;
    k_pair_store<<<kRedBlocks, 256, 0, C.stream>>>(Aw, w, nrm2, n5, R.d_pv + n5 * slot, R.d_pt + n5 * slot);
    ++C.launches;
    NT_TRY(check(C, cudaMemcpyAsync(R.d_pctx + (size_t)FCTX * C.N * slot, C.net.d_ctx, sizeof(bf16) * FCTX * (size_t)C.N,
                                    cudaMemcpyDeviceToDevice, C.stream), "pair features"));
    R.npairs = std::max(R.npairs, slot + 1);
    return check(C, cudaGetLastError(), "pair store");
}

void net_free(Ctx& C) {
    NetCtx& T = C.net;
    NetTrain& R = T.tr;
    void* ptrs[] = {T.d_nstart, T.d_nbr, T.d_act, T.d_x4, T.d_w, T.d_ctx, T.d_stat, T.d_spart, T.d_h, T.d_P0, T.d_P1, T.d_Z,
                    R.d_pv, R.d_pt, R.d_pctx, R.d_hs, R.d_ps, R.d_as, R.d_qs, R.d_us, R.d_out, R.d_dh, R.d_dms,
                    R.d_dqp, R.d_part, R.d_grad, R.d_m, R.d_v, R.d_scal};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (T.ev0) cudaEventDestroy(T.ev0);
    if (T.ev1) cudaEventDestroy(T.ev1);
    T = NetCtx{};
}

}  // namespace phgpu

// ============================================================================
// C ABI
// ============================================================================
using phgpu::Ctx;

namespace {

int sync_net(Ctx& C) {
    NT_TRY(phgpu::check(C, cudaGetLastError(), "network kernel launch"));
    return phgpu::check(C, cudaStreamSynchronize(C.stream), "network synchronize");
}

// host (nshg, 5) column-major <-> device [node][5] floats
int upload_vec(Ctx& C, const double* h, float* d) {
    const int N = C.N;
    std::vector<float> t(5 * (size_t)N);
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < 5; ++k) t[5 * (size_t)n + k] = (float)h[(size_t)k * N + n];
    return phgpu::h2d(C, d, t.data(), sizeof(float) * t.size(), "upload vector");
}
int download_vec(Ctx& C, const float* d, double* h) {
    const int N = C.N;
    std::vector<float> t(5 * (size_t)N);
    NT_TRY(phgpu::d2h(C, t.data(), d, sizeof(float) * t.size(), "download vector"));
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < 5; ++k) h[(size_t)k * N + n] = t[5 * (size_t)n + k];
    return PHGPU_OK;
}

int need_mixed(Ctx& C) {
    if (C.cfg.precision != PHGPU_MIXED)
        return phgpu::fail(C, PHGPU_ERR_UNSUPPORTED, "the learned preconditioner works on the mixed-precision (FP32) Krylov vectors");
    return PHGPU_OK;
}

}  // namespace

extern "C" {

int phgpu_net_set_weights(phgpu_ctx* h, const float* w, int n) {
    if (!h || !w || n != PHGPU_NET_NPARAM) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(w[i])) return phgpu::fail(C, PHGPU_ERR_NONFINITE, "non-finite network weight");
    NT_TRY(phgpu::net_setup(C));
    NT_TRY(phgpu::check(C, cudaMemcpyAsync(C.net.d_w, w, sizeof(float) * n, cudaMemcpyHostToDevice, C.stream), "weights"));
    C.net.have_w = true;
    C.net.its_ref = -1;
    C.net.fails = 0;
    C.net.disabled = false;
    return sync_net(C);
}

int phgpu_net_get_weights(phgpu_ctx* h, float* w, int n) {
    if (!h || !w || n != PHGPU_NET_NPARAM) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    if (!C.net.d_w) return phgpu::fail(C, PHGPU_ERR_INVALID, "no network weights");
    NT_TRY(phgpu::check(C, cudaMemcpyAsync(w, C.net.d_w, sizeof(float) * n, cudaMemcpyDeviceToHost, C.stream), "weights"));
    return sync_net(C);
}

int phgpu_net_graph(phgpu_ctx* h, int* nstart, unsigned* nbr, long long cap, long long* nnz, float* geo) {
    if (!h || !nnz) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    NT_TRY(phgpu::net_setup(C));
    *nnz = C.net.nnz;
    if (geo) {
        geo[0] = C.net.L[0];
        geo[1] = C.net.L[1];
        geo[2] = C.net.L[2];
        geo[3] = C.net.rh;
    }
    if (nstart)
        NT_TRY(phgpu::d2h(C, nstart, C.net.d_nstart, sizeof(int) * ((size_t)C.N + 1), "graph"));
    if (nbr) {
        if (cap < C.net.nnz) return phgpu::fail(C, PHGPU_ERR_TOO_LARGE, "phgpu_net_graph: nbr holds fewer than nnz entries");
        NT_TRY(phgpu::d2h(C, nbr, C.net.d_nbr, sizeof(unsigned) * C.net.nnz, "graph"));
    }
    return PHGPU_OK;
}

int phgpu_net_usage(phgpu_ctx* h, long long* counts) {
    if (!h || !counts) return PHGPU_ERR_INVALID;
    const phgpu::NetCtx& T = h->c.net;
    counts[0] = T.n_used;
    counts[1] = T.n_fell_back;
    counts[2] = T.n_plain;
    counts[3] = T.disabled ? 1 : 0;
    return PHGPU_OK;
}

int phgpu_net_features(phgpu_ctx* h, float* out) {
    if (!h) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    NT_TRY(need_mixed(C));
    NT_TRY(phgpu::net_prepare(C));
    NT_TRY(sync_net(C));
    if (out) {
        std::vector<__nv_bfloat16> t((size_t)phgpu::netk::FCTX * C.N);
        NT_TRY(phgpu::d2h(C, t.data(), C.net.d_ctx, sizeof(__nv_bfloat16) * t.size(), "features"));
        for (size_t i = 0; i < t.size(); ++i) out[i] = __bfloat162float(t[i]);
    }
    return PHGPU_OK;
}

int phgpu_net_apply(phgpu_ctx* h, const double* v, double* z, float* hidden, float* out) {
    using namespace phgpu::netk;
    if (!h || !v || !z) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    NT_TRY(need_mixed(C));
    if (!C.net.have_w) return phgpu::fail(C, PHGPU_ERR_INVALID, "no network weights");
    NT_TRY(phgpu::net_setup(C));
    const bool keep = hidden || out;
    if (keep) NT_TRY(phgpu::train_alloc(C));
    NT_TRY(upload_vec(C, v, C.d_t32));
    phgpu::forward(C, C.d_t32, C.d_t32b, C.net.d_ctx, keep);
    NT_TRY(sync_net(C));
    NT_TRY(download_vec(C, C.d_t32b, z));
    const size_t HNs = (size_t)C.N * H;
    if (hidden) {
        std::vector<__nv_bfloat16> t(4 * HNs);
        NT_TRY(phgpu::d2h(C, t.data(), C.net.tr.d_hs, sizeof(__nv_bfloat16) * t.size(), "hidden"));
        for (size_t i = 0; i < t.size(); ++i) hidden[i] = __bfloat162float(t[i]);
    }
    if (out) NT_TRY(phgpu::d2h(C, out, C.net.tr.d_out, sizeof(float) * 8 * (size_t)C.N, "out"));
    return PHGPU_OK;
}

int phgpu_net_loss_grad(phgpu_ctx* h, const double* v, const double* t, double* loss, float* grad) {
    using namespace phgpu::netk;
    if (!h || !v || !t) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    NT_TRY(need_mixed(C));
    if (!C.net.have_w) return phgpu::fail(C, PHGPU_ERR_INVALID, "no network weights");
    NT_TRY(phgpu::net_setup(C));
    NT_TRY(phgpu::train_alloc(C));
    NT_TRY(phgpu::scal_room(C, 2));
    NT_TRY(upload_vec(C, v, C.d_t32));
    NT_TRY(upload_vec(C, t, C.d_t32b));
    phgpu::forward(C, C.d_t32, C.d_resf, C.net.d_ctx, true);
    phgpu::backward(C, C.d_t32, C.d_t32b, C.net.d_ctx, C.net.tr.d_scal + 1);
    NT_TRY(sync_net(C));
    double l = 0.0;
    NT_TRY(phgpu::d2h(C, &l, C.net.tr.d_scal + 1, sizeof(double), "loss"));
    if (loss) *loss = l / std::max(5.0 * C.net.nact, 1.0);
    if (grad) NT_TRY(phgpu::d2h(C, grad, C.net.tr.d_grad, sizeof(float) * NPARAM, "grad"));
    return PHGPU_OK;
}

int phgpu_net_pairs(phgpu_ctx* h, int cap) {
    if (!h || cap < 1) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    NT_TRY(need_mixed(C));
    NT_TRY(phgpu::net_setup(C));
    phgpu::NetTrain& R = C.net.tr;
    for (void* p : {(void*)R.d_pv, (void*)R.d_pt, (void*)R.d_pctx})
        if (p) cudaFree(p);
    R.d_pv = R.d_pt = nullptr;
    R.d_pctx = nullptr;
    R.cap = R.npairs = 0;
    const size_t n5 = 5 * (size_t)C.N;
    NT_TRY(phgpu::nalloc(C, &R.d_pv, n5 * cap));
    NT_TRY(phgpu::nalloc(C, &R.d_pt, n5 * cap));
    NT_TRY(phgpu::nalloc(C, &R.d_pctx, (size_t)phgpu::netk::FCTX * C.N * cap));
    R.cap = cap;
    return PHGPU_OK;
}

int phgpu_net_train(phgpu_ctx* h, const phgpu_net_train_config* cfg, phgpu_net_train_stats* out) {
    using namespace phgpu::netk;
    if (!h || !cfg || cfg->epochs < 1 || !(cfg->lr > 0.f)) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    NT_TRY(need_mixed(C));
    phgpu::NetCtx& T = C.net;
    phgpu::NetTrain& R = T.tr;
    if (!T.have_w) return phgpu::fail(C, PHGPU_ERR_INVALID, "set initial weights before training");
    if (R.npairs < 1) return phgpu::fail(C, PHGPU_ERR_INVALID, "no training pairs collected");
    const int np = cfg->npairs > 0 ? std::min(cfg->npairs, R.npairs) : R.npairs;
    NT_TRY(phgpu::net_setup(C));
    NT_TRY(phgpu::train_alloc(C));
    const long long nsteps = (long long)cfg->epochs * np;
    if (nsteps + 1 > (1LL << 30)) return PHGPU_ERR_TOO_LARGE;
    NT_TRY(phgpu::scal_room(C, (int)nsteps + 1));
    const size_t n5 = 5 * (size_t)C.N, nc = (size_t)FCTX * C.N;
    const float s = (float)std::sqrt(5.0 * C.N);
    if (cfg->renormalize) {
        k_pair_stats<<<kStatBlocks, 256, 0, C.stream>>>(R.d_pv, R.d_pt, T.d_act, C.N, np, s, T.d_spart);
        ++C.launches;
        std::vector<double> part((size_t)kStatBlocks * 10);
        NT_TRY(phgpu::check(C, cudaMemcpyAsync(part.data(), T.d_spart, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, C.stream), "pair stats"));
        NT_TRY(sync_net(C));
        double tot[10] = {};
        for (int b = 0; b < kStatBlocks; ++b)
            for (int k = 0; k < 10; ++k) tot[k] += part[(size_t)b * 10 + k];
        const double cnt = std::max(1.0, (double)T.nact * np);
        float ab[10];
        for (int d = 0; d < 5; ++d) {
            const double rv = std::sqrt(tot[d] / cnt), rt = std::sqrt(tot[5 + d] / cnt);
            ab[d] = rv > 0 ? (float)(1.0 / rv) : 1.f;
            ab[5 + d] = rt > 0 ? (float)rt : 1.f;
        }
        NT_TRY(phgpu::check(C, cudaMemcpyAsync(T.d_w + O_AL, ab, sizeof(ab), cudaMemcpyHostToDevice, C.stream), "alpha/beta"));
        NT_TRY(sync_net(C));
    }
    std::mt19937 rng(cfg->seed);
    std::vector<int> order(np);
    std::iota(order.begin(), order.end(), 0);
    cudaEvent_t e0 = C.ev[2], e1 = C.ev[3];
    cudaEventRecord(e0, C.stream);
    const float b1 = cfg->beta1 > 0.f ? cfg->beta1 : 0.9f, b2 = cfg->beta2 > 0.f ? cfg->beta2 : 0.999f;
    const float eps = cfg->eps > 0.f ? cfg->eps : 1e-8f;
    long long k = 0;
    for (int ep = 0; ep < cfg->epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        for (int q = 0; q < np; ++q, ++k) {
            const int p = order[q];
            const float* v = R.d_pv + n5 * p;
            const float* t = R.d_pt + n5 * p;
            const __nv_bfloat16* cx = R.d_pctx + nc * p;
            phgpu::forward(C, v, C.d_resf, cx, true);
            phgpu::backward(C, v, t, cx, R.d_scal + 1 + k);
            k_grad_norm<<<1, 1024, 0, C.stream>>>(R.d_grad, R.d_scal);
            ++R.step;
            AdamP ap{cfg->lr, b1, b2, eps, cfg->clip, (float)(1.0 - std::pow((double)b1, (double)R.step)),
                     (float)(1.0 - std::pow((double)b2, (double)R.step))};
            k_adam<<<(O_AL + 255) / 256, 256, 0, C.stream>>>(T.d_w, R.d_grad, R.d_m, R.d_v, ap, R.d_scal);
            C.launches += 2;
        }
    }
    cudaEventRecord(e1, C.stream);
    NT_TRY(sync_net(C));
    std::vector<double> losses((size_t)nsteps);
    NT_TRY(phgpu::d2h(C, losses.data(), R.d_scal + 1, sizeof(double) * nsteps, "losses"));
    const double nm = std::max(5.0 * T.nact, 1.0);
    if (out) {
        double f = 0.0, l = 0.0;
        for (int q = 0; q < np; ++q) {
            f += losses[q] / nm;
            l += losses[(size_t)(nsteps - np) + q] / nm;
        }
        out->loss_first = f / np;
        out->loss_last = l / np;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        out->ms = ms;
        out->steps = nsteps;
    }
    // new weights: the fallback statistics start again
    T.its_ref = -1;
    T.fails = 0;
    T.disabled = false;
    return PHGPU_OK;
}

}  // extern "C"
