// tangent.cu -- the assembled element tangent of the sparse solver (ElmGMRs
// with lhs = 1, elmgmr.f:280-470) for linear tets, hexes and wedges.
//
// For each element the tangent EGmass of e3.f is the quadrature sum of
//   e3conv.f   N_a A_i N_b,i
//   e3ls.f     fct N_a,i A_i tau A0 N_b + N_a,i A_i tau A_j N_b,j
//   e3massl.f  fct N_a N_b A0                       (no sponge: bcool = 0)
//   e3wmlt.f   N_a,i K_ij N_b,j                     (K of e3visc.f:65-127)
// with fct = almi/(gami alfi) Dtgl.  Block (a,b) is evaluated here as the
// regrouped product
//   W [ (N_a I + B_a tau)(B_b + fct N_b A0) + K_ab ],   B_c = sum_i N_c,i A_i,
// from the closed forms of B_c and A0 (the same sum).  bc3LHS (bc3lhs.f) is
// then applied block by block: its row operations belong to the row node and
// its column operations to the column node, and a block sees only those of
// its own two nodes, in the routine's order.  fillsparseC (fillsparse.f) adds
// the block to lhsK at a position found on the host (the element's block map).
//
// Threads: one per (element, a, b); the NEN threads of an element first
// evaluate one quadrature point each (the linear rules have NEN points) and
// share it in shared memory.  Elements of one colour share no node, so the
// read-modify-write of lhsK blocks is deterministic and atomic-free.
#include "phgpu_impl.cuh"
#include "qpoint.cuh"

// resident CTAs per SM of the FP32 tangent (register budget 65536 / (128 x this))
#ifndef PHGPU_TAN32_MINB
#define PHGPU_TAN32_MINB 7
#endif

namespace phgpu {
namespace {

__constant__ TopoTabD c_tt[3];   // 0 hex, 1 wedge, 2 tet
__constant__ TopoTabF c_ttf[3];

template <typename R> __device__ __forceinline__ R t_shp(int t, int q, int a);
template <> __device__ __forceinline__ double t_shp<double>(int t, int q, int a) { return c_tt[t].shp[q][a]; }
template <> __device__ __forceinline__ float t_shp<float>(int t, int q, int a) { return c_ttf[t].shp[q][a]; }
template <typename R> __device__ __forceinline__ R t_shgl(int t, int q, int i, int a);
template <> __device__ __forceinline__ double t_shgl<double>(int t, int q, int i, int a) { return c_tt[t].shgl[q][i][a]; }
template <> __device__ __forceinline__ float t_shgl<float>(int t, int q, int i, int a) { return c_ttf[t].shgl[q][i][a]; }
template <typename R> __device__ __forceinline__ R t_qwt(int t, int q);
template <> __device__ __forceinline__ double t_qwt<double>(int t, int q) { return c_tt[t].qwt[q]; }
template <> __device__ __forceinline__ float t_qwt<float>(int t, int q) { return c_ttf[t].qwt[q]; }

constexpr int kTanThreads = 128;
constexpr int kTanNode = 8;  // staged per node: x(3) y(5)

// one quadrature point in shared memory
template <int NEN>
struct TanQp {
    static constexpr int kShg = 0;           // shg[b][i]
    static constexpr int kW = 3 * NEN;       // WdetJ
    static constexpr int kS = kW + 1;        // u(3) rho drdp drdT e1p e2p e3p e4p tau(3)
    static constexpr int kN = kS + 13;
};

template <int NEN>
constexpr int tan_epb() { return kTanThreads / (NEN * NEN); }  // elements per CTA: tet 8, hex 2, wedge 3

// per (element, point q, node a): W_q (N_a I + B_a tau) and B_a + fct N_a A0, 25 + 25 values
constexpr int kTanDC = 50;

template <typename R, int NEN>
constexpr size_t tan_smem() {
    return sizeof(R) * (size_t)tan_epb<NEN>() * NEN * (kTanNode + TanQp<NEN>::kN + NEN * kTanDC) +
           sizeof(int) * tan_epb<NEN>() * NEN * (1 + NEN);
}

// B = sum_i s_i A_i for the direction s (e3mtrx.f closed form); Us = s . u
template <typename R>
__device__ __forceinline__ void bmat(const R (&s)[3], R Us, const R (&u)[3], R rho, R drdp, R drdT, R e2p, R e3p,
                                     R e4p, R (&B)[5][5]) {
    B[0][0] = drdp * Us;
    B[0][4] = drdT * Us;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        B[0][1 + j] = rho * s[j];
        B[1 + j][0] = drdp * Us * u[j] + s[j];
        B[1 + j][4] = drdT * Us * u[j];
#pragma unroll
        for (int k = 0; k < 3; ++k) B[1 + j][1 + k] = rho * (u[j] * s[k] + (j == k ? Us : R(0)));
        B[4][1 + j] = e3p * s[j] + rho * Us * u[j];
    }
    B[4][0] = e2p * Us;
    B[4][4] = e4p * Us;
}

// bc3LHS (bc3lhs.f, intpres = 0) on block (a,b): the row operations of node a (code ia,
// BC values ba) and the column operations of node b; unit diagonals on a diagonal block
template <typename R>
__device__ __forceinline__ void bc3lhs_block(R (&M)[5][5], int ia, const double* __restrict__ ba, int ib,
                                             const double* __restrict__ bb, bool diag) {
    auto zrow = [&](int r) {
#pragma unroll
        for (int c = 0; c < 5; ++c) M[r][c] = R(0);
    };
    auto zcol = [&](int c) {
#pragma unroll
        for (int r = 0; r < 5; ++r) M[r][c] = R(0);
    };
    // pressure (bit 2)
    if (ia & 4) zrow(0);
    if (ib & 4) zcol(0);
    if (diag && (ia & 4)) M[0][0] = R(1);
    // velocity (bits 3-5)
    const int va = (ia >> 3) & 7, vb = (ib >> 3) & 7;
    if (va) {
        const R b4 = (R)ba[3], b5 = (R)ba[4], b6 = (R)ba[5];
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            switch (va) {
                case 1: M[2][c] = M[2][c] - b4 * M[1][c]; M[3][c] = M[3][c] - b5 * M[1][c]; break;
                case 2: M[1][c] = M[1][c] - b4 * M[2][c]; M[3][c] = M[3][c] - b5 * M[2][c]; break;
                case 3: M[3][c] = M[3][c] - b4 * M[1][c] - b6 * M[2][c]; break;
                case 4: M[1][c] = M[1][c] - b4 * M[3][c]; M[2][c] = M[2][c] - b5 * M[3][c]; break;
                case 5: M[2][c] = M[2][c] - b4 * M[1][c] - b6 * M[3][c]; break;
                case 6: M[1][c] = M[1][c] - b4 * M[2][c] - b6 * M[3][c]; break;
                default: break;
            }
        }
    }
    if (vb) {
        const R b4 = (R)bb[3], b5 = (R)bb[4], b6 = (R)bb[5];
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            switch (vb) {
                case 1: M[r][2] = M[r][2] - b4 * M[r][1]; M[r][3] = M[r][3] - b5 * M[r][1]; break;
                case 2: M[r][1] = M[r][1] - b4 * M[r][2]; M[r][3] = M[r][3] - b5 * M[r][2]; break;
                case 3: M[r][3] = M[r][3] - b4 * M[r][1] - b6 * M[r][2]; break;
                case 4: M[r][1] = M[r][1] - b4 * M[r][3]; M[r][2] = M[r][2] - b5 * M[r][3]; break;
                case 5: M[r][2] = M[r][2] - b4 * M[r][1] - b6 * M[r][3]; break;
                case 6: M[r][1] = M[r][1] - b4 * M[r][2] - b6 * M[r][3]; break;
                default: break;
            }
        }
    }
    // constrained velocity components of each case: 1 {u}, 2 {v}, 3 {u,v}, 4 {w}, 5 {u,w}, 6 {v,w}, 7 all
    auto vset = [](int v, int d) {
        const int m = (v == 1) ? 1 : (v == 2) ? 2 : (v == 3) ? 3 : (v == 4) ? 4 : (v == 5) ? 5 : (v == 6) ? 6 : 7;
        return v != 0 && ((m >> d) & 1);
    };
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (vset(va, d)) zrow(1 + d);
        if (vset(vb, d)) zcol(1 + d);
        if (diag && vset(va, d)) M[1 + d][1 + d] = R(1);
    }
    // temperature (bit 1)
    if (ia & 2) zrow(4);
    if (ib & 2) zcol(4);
    if (diag && (ia & 2)) M[4][4] = R(1);
}

template <typename R, int NEN, int TOPO>
__global__ void __launch_bounds__(kTanThreads, sizeof(R) == 4 ? PHGPU_TAN32_MINB : 2)
k_tangent(const int* __restrict__ ien, const int* __restrict__ bmap, int ne, const R* __restrict__ x,
          const R* __restrict__ y, const int* __restrict__ iBC, const double* __restrict__ BC,
          R* __restrict__ lhsK, R* __restrict__ bd, Phys<R> P) {
    using Q = TanQp<NEN>;
    constexpr int EPB = tan_epb<NEN>();
    constexpr int NB = NEN * NEN;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* snode = reinterpret_cast<R*>(smem_raw);                 // [EPB][NEN][kTanNode]
    R* sqp = snode + EPB * NEN * kTanNode;                     // [EPB][NEN][kN]
    R* sdc = sqp + EPB * NEN * Q::kN;                          // [EPB][NEN q][NEN a][kTanDC]
    int* sid = reinterpret_cast<int*>(sdc + EPB * NB * kTanDC);  // [EPB][NEN]
    int* sk = sid + EPB * NEN;                                 // [EPB * NB] output block of each thread
    const int e0 = blockIdx.x * EPB;
    // start the block's lines on their way to L2 for the read-modify-write at the end
    if (bmap && threadIdx.x < EPB * NB && e0 + (int)threadIdx.x / NB < ne) {
        const char* o = reinterpret_cast<const char*>(
            lhsK + 25 * (size_t)bmap[(size_t)(e0 + threadIdx.x / NB) * NB + threadIdx.x % NB]);
#pragma unroll
        for (int off = 0; off < 25 * (int)sizeof(R); off += 96)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(o + off));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(o + 25 * sizeof(R) - 1));
    }
    // stage the nodes
    for (int i = threadIdx.x; i < EPB * NEN; i += blockDim.x) {
        const int le = i / NEN, a = i % NEN, e = e0 + le;
        if (e >= ne) continue;
        const int n = ien[(size_t)e * NEN + a];
        sid[i] = n;
        R* s = snode + kTanNode * i;
#pragma unroll
        for (int d = 0; d < 3; ++d) s[d] = ldg(x + 3 * (size_t)n + d);
#pragma unroll
        for (int k = 0; k < 5; ++k) s[3 + k] = ldg(y + 5 * (size_t)n + k);
    }
    __syncthreads();
    // quadrature point q of element le: metric (e3metric.f:22-77), state, tau
    for (int i = threadIdx.x; i < EPB * NEN; i += blockDim.x) {
        const int le = i / NEN, q = i % NEN;
        if (e0 + le >= ne) continue;
        const R* sx = snode + kTanNode * NEN * le;
        R dxdxi[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                R acc = R(0);
#pragma unroll
                for (int b = 0; b < NEN; ++b) acc += sx[kTanNode * b + r] * t_shgl<R>(TOPO, q, j, b);
                dxdxi[r][j] = acc;
            }
        R di[3][3];
        di[0][0] = dxdxi[1][1] * dxdxi[2][2] - dxdxi[2][1] * dxdxi[1][2];
        di[0][1] = dxdxi[2][1] * dxdxi[0][2] - dxdxi[0][1] * dxdxi[2][2];
        di[0][2] = dxdxi[0][1] * dxdxi[1][2] - dxdxi[0][2] * dxdxi[1][1];
        const R tmp = R(1) / (di[0][0] * dxdxi[0][0] + di[0][1] * dxdxi[1][0] + di[0][2] * dxdxi[2][0]);
        di[0][0] *= tmp;
        di[0][1] *= tmp;
        di[0][2] *= tmp;
        di[1][0] = (dxdxi[1][2] * dxdxi[2][0] - dxdxi[1][0] * dxdxi[2][2]) * tmp;
        di[1][1] = (dxdxi[0][0] * dxdxi[2][2] - dxdxi[2][0] * dxdxi[0][2]) * tmp;
        di[1][2] = (dxdxi[1][0] * dxdxi[0][2] - dxdxi[0][0] * dxdxi[1][2]) * tmp;
        di[2][0] = (dxdxi[1][0] * dxdxi[2][1] - dxdxi[1][1] * dxdxi[2][0]) * tmp;
        di[2][1] = (dxdxi[2][0] * dxdxi[0][1] - dxdxi[0][0] * dxdxi[2][1]) * tmp;
        di[2][2] = (dxdxi[0][0] * dxdxi[1][1] - dxdxi[0][1] * dxdxi[1][0]) * tmp;
        R* o = sqp + Q::kN * i;
        o[Q::kW] = t_qwt<R>(TOPO, q) / tmp;
        R yq[5] = {R(0), R(0), R(0), R(0), R(0)};
#pragma unroll
        for (int b = 0; b < NEN; ++b) {
#pragma unroll
            for (int r = 0; r < 3; ++r)
                o[Q::kShg + 3 * b + r] = t_shgl<R>(TOPO, q, 0, b) * di[0][r] + t_shgl<R>(TOPO, q, 1, b) * di[1][r] +
                                         t_shgl<R>(TOPO, q, 2, b) * di[2][r];
            const R Nb = t_shp<R>(TOPO, q, b);
#pragma unroll
            for (int k = 0; k < 5; ++k) yq[k] += Nb * sx[kTanNode * b + 3 + k];
        }
        Qp<R> st;
        qp_state(P, yq[0], yq[1], yq[2], yq[3], yq[4], st);
        Geo<R> gm;
        auto cij = [&](int r, int j) { return di[0][r] * di[0][j] + di[1][r] * di[1][j] + di[2][r] * di[2][j]; };
        const int ord[6][2] = {{0, 0}, {0, 1}, {1, 1}, {0, 2}, {1, 2}, {2, 2}};
        if (TOPO == 2) {
            // tets: dxidx^T M dxidx, M = c2 ones + (c1 - c2) I (e3tau.f:1440-1470)
            const R c2 = R(6.299605249474365e-01), cm = R(1.259921049894873e+00 - 6.299605249474365e-01);
            R s[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) s[r] = di[0][r] + di[1][r] + di[2][r];
#pragma unroll
            for (int k = 0; k < 6; ++k) gm.G[k] = cm * cij(ord[k][0], ord[k][1]) + c2 * s[ord[k][0]] * s[ord[k][1]];
        } else {
            // hexes and wedges: dxidx^T dxidx (e3tau.f:1408-1425)
#pragma unroll
            for (int k = 0; k < 6; ++k) gm.G[k] = cij(ord[k][0], ord[k][1]);
        }
        gm.GG = gm.G[0] * gm.G[0] + gm.G[2] * gm.G[2] + gm.G[5] * gm.G[5] +
                R(2) * (gm.G[1] * gm.G[1] + gm.G[3] * gm.G[3] + gm.G[4] * gm.G[4]);
        gm.trG = gm.G[0] + gm.G[2] + gm.G[5];
        qp_tau(P, gm, st);
        R* os = o + Q::kS;
        os[0] = st.u[0];
        os[1] = st.u[1];
        os[2] = st.u[2];
        os[3] = st.rho;
        os[4] = st.drdp;
        os[5] = st.drdT;
        os[6] = st.e1p;
        os[7] = st.e2p;
        os[8] = st.e3p;
        os[9] = st.e4p;
        os[10] = st.tau[0];
        os[11] = st.tau[1];
        os[12] = st.tau[2];
    }
    __syncthreads();
    // the two factors of every (point, node): W (N_a I + B_a tau) and B_a + fct N_a A0
    if (threadIdx.x < EPB * NB && e0 + (int)threadIdx.x / NB < ne) {
        const int le = threadIdx.x / NB, r = threadIdx.x % NB, q = r / NEN, a = r % NEN;
        const R* v = sqp + Q::kN * (NEN * le + q);
        const R w = v[Q::kW];
        const R sa[3] = {v[Q::kShg + 3 * a], v[Q::kShg + 3 * a + 1], v[Q::kShg + 3 * a + 2]};
        const R* st = v + Q::kS;
        const R u[3] = {st[0], st[1], st[2]};
        const R rho = st[3], drdp = st[4], drdT = st[5], e1p = st[6], e2p = st[7], e3p = st[8], e4p = st[9];
        const R tk[5] = {st[10], st[11], st[11], st[11], st[12]};
        const R Na = t_shp<R>(TOPO, q, a);
        R Bm[5][5];
        bmat(sa, sa[0] * u[0] + sa[1] * u[1] + sa[2] * u[2], u, rho, drdp, drdT, e2p, e3p, e4p, Bm);
        R* o = sdc + kTanDC * ((size_t)(le * NEN + q) * NEN + a);
#pragma unroll
        for (int i = 0; i < 5; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k) o[5 * i + k] = w * (Bm[i][k] * tk[k] + (i == k ? Na : R(0)));
        const R fN = P.fct1 * Na;
        Bm[0][0] += fN * drdp;
        Bm[0][4] += fN * drdT;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Bm[1 + j][0] += fN * drdp * u[j];
            Bm[1 + j][1 + j] += fN * rho;
            Bm[1 + j][4] += fN * drdT * u[j];
            Bm[4][1 + j] += fN * rho * u[j];
        }
        Bm[4][0] += fN * e1p;
        Bm[4][4] += fN * e4p;
#pragma unroll
        for (int i = 0; i < 5; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k) o[25 + 5 * i + k] = Bm[i][k];
    }
    __syncthreads();
    const bool active = threadIdx.x < EPB * NB && e0 + (int)threadIdx.x / NB < ne;
    const int le = threadIdx.x / NB, ab = threadIdx.x % NB, a = ab / NEN, b = ab % NEN;
    const int e = e0 + le;
    R M[5][5];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
        for (int c = 0; c < 5; ++c) M[r][c] = R(0);
#pragma unroll 1
    for (int q = 0; q < (active ? NEN : 0); ++q) {
        // W (N_a I + B_a tau)(B_b + fct N_b A0), the factors from shared memory
        const R* Dq = sdc + kTanDC * ((size_t)(le * NEN + q) * NEN + a);
        const R* Cq = sdc + kTanDC * ((size_t)(le * NEN + q) * NEN + b) + 25;
        R Cm[5][5];
#pragma unroll
        for (int k = 0; k < 5; ++k)
#pragma unroll
            for (int c = 0; c < 5; ++c) Cm[k][c] = Cq[5 * k + c];
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            R D[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) D[k] = Dq[5 * r + k];
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                R acc = M[r][c];
#pragma unroll
                for (int k = 0; k < 5; ++k) acc += D[k] * Cm[k][c];
                M[r][c] = acc;
            }
        }
        const R* v = sqp + Q::kN * (NEN * le + q);
        const R w = v[Q::kW];
        if (P.navier) {
            // K_ab = sum_ij N_a,i K_ij N_b,j
            const R sa[3] = {v[Q::kShg + 3 * a], v[Q::kShg + 3 * a + 1], v[Q::kShg + 3 * a + 2]};
            const R sb[3] = {v[Q::kShg + 3 * b], v[Q::kShg + 3 * b + 1], v[Q::kShg + 3 * b + 2]};
            const R u[3] = {v[Q::kS], v[Q::kS + 1], v[Q::kS + 2]};
            const R Usa = sa[0] * u[0] + sa[1] * u[1] + sa[2] * u[2];
            const R Usb = sb[0] * u[0] + sb[1] * u[1] + sb[2] * u[2];
            const R sab = sa[0] * sb[0] + sa[1] * sb[1] + sa[2] * sb[2];
#pragma unroll
            for (int m = 0; m < 3; ++m) {
#pragma unroll
                for (int n = 0; n < 3; ++n)
                    M[1 + m][1 + n] += w * (P.rmu * sa[n] * sb[m] + P.rlm * sa[m] * sb[n] + (m == n ? P.rmu * sab : R(0)));
                M[4][1 + m] += w * (P.rmu * sa[m] * Usb + P.rlm * Usa * sb[m] + P.rmu * u[m] * sab);
            }
            M[4][4] += w * P.con * sab;
        }
    }
    if (active) {
        const int* ids = sid + NEN * le;
        const int na = ids[a], nb = ids[b];
        // the block diagonal is the tangent's diagonal blocks before bc3LHS (asigmr.f:92-103)
        if (bd && a == b) {
            R* ob = bd + 25 * (size_t)na;  // row-major BDiag(n, r, c)
#pragma unroll
            for (int r = 0; r < 5; ++r)
#pragma unroll
                for (int c = 0; c < 5; ++c) ob[5 * r + c] += M[r][c];
        }
        const int ia = iBC[na], ib = iBC[nb];
        if (ia | ib) bc3lhs_block(M, ia, BC + 6 * (size_t)na, ib, BC + 6 * (size_t)nb, a == b);
    }
    // Stage the blocks in shared memory (over the per-point factors, now read), then move
    // each block with 25 consecutive lanes of one warp: 4-5 sectors per block instead of one
    // sector per value.  With a block map: add into lhsK; without: element storage.
    __syncthreads();
    R* sblk = sdc;  // [EPB * NB][25], entry (f, g) at 5 g + f
    if (threadIdx.x < EPB * NB) {
        sk[threadIdx.x] = !active ? -1 : bmap ? bmap[(size_t)e * NB + ab] : e * NB + ab;
        if (active)
#pragma unroll
            for (int g = 0; g < 5; ++g)
#pragma unroll
                for (int f = 0; f < 5; ++f) sblk[25 * threadIdx.x + 5 * g + f] = M[f][g];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int j = warp; j < EPB * NB; j += nwarps) {
        const int k = sk[j];
        if (k < 0 || lane >= 25) continue;
        R* o = lhsK + 25 * (size_t)k + lane;
        const R v = sblk[25 * j + lane];
        if (bmap) *o = *o + v;
        else *o = v;
    }
}

template <typename R, int NEN, int TOPO>
void launch_one(Ctx& C, const int* d_ien, const int* d_map, const std::vector<int>& col, const R* x, const R* y,
                R* lhsK, R* bd) {
    const Phys<R> P = make_phys<R>(C.cfg);
    constexpr int EPB = tan_epb<NEN>();
    const size_t sm = tan_smem<R, NEN>();
    const int ncol = (int)col.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int e0 = col[c], ne = col[c + 1] - e0;
        if (ne <= 0) continue;
        // with no block map the output is element storage, offset by the colour's first element
        const int* map = d_map ? d_map + (size_t)NEN * NEN * e0 : nullptr;
        R* out = d_map ? lhsK : lhsK + 25 * (size_t)NEN * NEN * e0;
        k_tangent<R, NEN, TOPO><<<(ne + EPB - 1) / EPB, kTanThreads, sm, C.stream>>>(
            d_ien + (size_t)NEN * e0, map, ne, x, y, C.d_iBC, C.d_BC, out, bd, P);
        ++C.launches;
    }
}

}  // namespace

int upload_tangent_tables(Ctx& C) {
    std::vector<TopoTabD> td(3);
    std::vector<TopoTabF> tf(3);
    topo_tables_host(td.data());
    for (int k = 0; k < 3; ++k)
        for (int q = 0; q < 8; ++q) {
            tf[k].qwt[q] = (float)td[k].qwt[q];
            for (int a = 0; a < 8; ++a) {
                tf[k].shp[q][a] = (float)td[k].shp[q][a];
                for (int i = 0; i < 3; ++i) tf[k].shgl[q][i][a] = (float)td[k].shgl[q][i][a];
            }
        }
    int rc = check(C, cudaMemcpyToSymbolAsync(c_tt, td.data(), sizeof(TopoTabD) * 3, 0, cudaMemcpyHostToDevice,
                                              C.stream),
                   "tangent tables");
    if (rc == PHGPU_OK)
        rc = check(C, cudaMemcpyToSymbolAsync(c_ttf, tf.data(), sizeof(TopoTabF) * 3, 0, cudaMemcpyHostToDevice,
                                              C.stream),
                   "tangent tables");
    // the sources are this function's locals
    if (rc == PHGPU_OK) rc = check(C, cudaStreamSynchronize(C.stream), "tangent tables");
    return rc;
}

int configure_tangent_kernels(Ctx& C) {
    int rc = PHGPU_OK;
    auto T = [&](cudaError_t e) { if (rc == PHGPU_OK) rc = check(C, e, "cudaFuncSetAttribute"); };
    T(smem_attr(k_tangent<double, 4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tan_smem<double, 4>()));
    T(smem_attr(k_tangent<double, 8, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tan_smem<double, 8>()));
    T(smem_attr(k_tangent<double, 6, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tan_smem<double, 6>()));
    T(smem_attr(k_tangent<float, 4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tan_smem<float, 4>()));
    T(smem_attr(k_tangent<float, 8, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tan_smem<float, 8>()));
    T(smem_attr(k_tangent<float, 6, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tan_smem<float, 6>()));
    return rc;
}

// lhsK += the element tangents of every block (tets, hexes, wedges), colour by colour;
// bd (optional, device layout) += their diagonal blocks before the boundary conditions
template <typename R>
void launch_tangent(Ctx& C, const R* x, const R* y, R* lhsK, R* bd) {
    const SparseCtx& S = C.sp;
    if (C.E > 0) launch_one<R, 4, 2>(C, S.d_ient, S.d_tmap, S.tcol_start, x, y, lhsK, bd);
    if (C.nhex > 0) launch_one<R, 8, 0>(C, C.d_ienh, S.d_hmap, C.hcol_start, x, y, lhsK, bd);
    if (C.nwedge > 0) launch_one<R, 6, 1>(C, C.d_ienw, S.d_wmap, C.wcol_start, x, y, lhsK, bd);
}
template void launch_tangent<double>(Ctx&, const double*, const double*, double*, double*);
template void launch_tangent<float>(Ctx&, const float*, const float*, float*, float*);

// EG = the element tangents (after bc3LHS) stored per element; bd += their diagonal blocks
template <typename R>
void launch_tangent_ebe(Ctx& C, const R* x, const R* y, R* EG, R* bd) {
    const SparseCtx& S = C.sp;
    R* hex = EG + 25 * 16 * (size_t)C.E;
    R* wedge = hex + 25 * 64 * (size_t)C.nhex;
    if (C.E > 0) launch_one<R, 4, 2>(C, S.d_ient, nullptr, S.tcol_start, x, y, EG, bd);
    if (C.nhex > 0) launch_one<R, 8, 0>(C, C.d_ienh, nullptr, C.hcol_start, x, y, hex, bd);
    if (C.nwedge > 0) launch_one<R, 6, 1>(C, C.d_ienw, nullptr, C.wcol_start, x, y, wedge, bd);
}
template void launch_tangent_ebe<double>(Ctx&, const double*, const double*, double*, double*);
template void launch_tangent_ebe<float>(Ctx&, const float*, const float*, float*, float*);

}  // namespace phgpu
