// topo_ress.cu -- the outer residual (ires = 1) of hex and wedge blocks without FP64
// arithmetic, the counterpart of the tets' split residual (k_chunk_ress).
//
// The Euler flux at a quadrature point is split exactly as F(y_q) = F(y_r) + [F(y_q) -
// F(y_r)], y_r the state of the element's local node 0:
//   * F(y_r) is constant over the element, so its weighted sum over the points is
//     sum_i I_a,i F_i(y_r) with I_a,i = sum_q W_q N_a,i(q).  W_q dxi/dx at a point is
//     the point weight times the adjugate of the Jacobian, so I depends on the
//     coordinates alone: it is formed once in FP64 on the host (the mesh does not move)
//     and kept as hi/lo floats; the products with F(y_r) are double-float.
//   * the increment is written with the exact expansions of k_chunk_ress
//     (rho - rho_r = (dp T_r - p_r dT) / (R T T_r), m_i u_j - m_ri u_rj = dm_i u_j +
//     m_ri du_j, ...) of increments y_b - y_r formed from the hi/lo copies, in FP32.
// The metric, tau, the least-squares and viscous terms and the time term are FP32 (e3.f
// with the hex/wedge metric of e3tau.f:1408-1425).  One thread per (element, point) and
// per (element, node); each node's double-float sum is added to the FP64 output.  Elements
// of one colour share no node.
#include <vector>

#include "phgpu_impl.cuh"
#include "df64.cuh"
#include "qpoint.cuh"

namespace phgpu {
namespace {

__constant__ TopoTabF c_trf[2];  // 0 hex, 1 wedge

constexpr int kRsThreads = 128;
template <int NEN> constexpr int rs_epb() { return kRsThreads / NEN; }  // hex 16, wedge 21
template <bool WITH_Q> constexpr int rs_node() { return WITH_Q ? 30 : 18; }  // xh(3) yh(5) ylo(5) ac(5) q(12)
template <int NEN> constexpr int rs_qp() { return 21 + 3 * NEN; }  // W, F(15), A0 ac (5), shg

template <int NEN, bool WITH_Q>
constexpr size_t rs_smem() {
    return sizeof(float) * (size_t)rs_epb<NEN>() * NEN * (rs_node<WITH_Q>() + rs_qp<NEN>());
}

struct RsConst {
    float rRgas_hi, rRgas_lo, cv_hi, cv_lo;  // 1/R, R/(gamma-1)
};

template <int NEN, int TOPO, bool WITH_Q>
__global__ void __launch_bounds__(kRsThreads)
k_topo_ress(const int* __restrict__ ien, int ne, const float2* __restrict__ I, const float* __restrict__ xh,
            const float* __restrict__ yh, const float* __restrict__ ylo, const float* __restrict__ acf,
            const float* __restrict__ ql, double* __restrict__ out, Phys<float> P, RsConst K) {
    constexpr int EPB = rs_epb<NEN>(), ND = rs_node<WITH_Q>(), QD = rs_qp<NEN>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sn = reinterpret_cast<float*>(smem_raw);  // [EPB][NEN][ND]
    float* sq = sn + EPB * NEN * ND;                  // [EPB][NEN q][QD]
    const int le = threadIdx.x / NEN, a = threadIdx.x % NEN;
    const int e = blockIdx.x * EPB + le;
    const bool active = le < EPB && e < ne;
    float* nod = sn + (size_t)le * NEN * ND;
    int node = 0;
    if (active) {
        node = ien[(size_t)e * NEN + a];
        float* s = nod + ND * a;
#pragma unroll
        for (int d = 0; d < 3; ++d) s[d] = __ldg(xh + 3 * (size_t)node + d);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            s[3 + k] = __ldg(yh + 5 * (size_t)node + k);
            s[8 + k] = __ldg(ylo + 5 * (size_t)node + k);
            s[13 + k] = __ldg(acf + 5 * (size_t)node + k);
        }
        if (WITH_Q)
#pragma unroll
            for (int k = 0; k < 12; ++k) s[18 + k] = __ldg(ql + 13 * (size_t)node + k);
    }
    __syncthreads();
    if (active) {
        // ---- point q = a ----
        const int q = a;
        float dxdxi[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                float acc = 0.f;
#pragma unroll
                for (int b = 0; b < NEN; ++b) acc += nod[ND * b + i] * c_trf[TOPO].shgl[q][j][b];
                dxdxi[i][j] = acc;
            }
        float di[3][3];
        di[0][0] = dxdxi[1][1] * dxdxi[2][2] - dxdxi[2][1] * dxdxi[1][2];
        di[0][1] = dxdxi[2][1] * dxdxi[0][2] - dxdxi[0][1] * dxdxi[2][2];
        di[0][2] = dxdxi[0][1] * dxdxi[1][2] - dxdxi[0][2] * dxdxi[1][1];
        const float tmp = 1.f / (di[0][0] * dxdxi[0][0] + di[0][1] * dxdxi[1][0] + di[0][2] * dxdxi[2][0]);
        di[0][0] *= tmp;
        di[0][1] *= tmp;
        di[0][2] *= tmp;
        di[1][0] = (dxdxi[1][2] * dxdxi[2][0] - dxdxi[1][0] * dxdxi[2][2]) * tmp;
        di[1][1] = (dxdxi[0][0] * dxdxi[2][2] - dxdxi[2][0] * dxdxi[0][2]) * tmp;
        di[1][2] = (dxdxi[1][0] * dxdxi[0][2] - dxdxi[0][0] * dxdxi[1][2]) * tmp;
        di[2][0] = (dxdxi[1][0] * dxdxi[2][1] - dxdxi[1][1] * dxdxi[2][0]) * tmp;
        di[2][1] = (dxdxi[2][0] * dxdxi[0][1] - dxdxi[0][0] * dxdxi[2][1]) * tmp;
        di[2][2] = (dxdxi[0][0] * dxdxi[1][1] - dxdxi[0][1] * dxdxi[1][0]) * tmp;
        float* o = sq + (size_t)QD * (le * NEN + q);
        o[0] = c_trf[TOPO].qwt[q] / tmp;
        float* shg = o + 21;
        // increments from local node 0 (hi and lo parts), the point's state, gradients
        const float* r = nod;
        float bq[5], aq[5], dq[5], g[3][5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            bq[k] = aq[k] = dq[k] = 0.f;
#pragma unroll
            for (int i = 0; i < 3; ++i) g[i][k] = 0.f;
        }
        float divq[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int b = 0; b < NEN; ++b) {
            const float* s = nod + ND * b;
            float sh[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                sh[i] = c_trf[TOPO].shgl[q][0][b] * di[0][i] + c_trf[TOPO].shgl[q][1][b] * di[1][i] +
                        c_trf[TOPO].shgl[q][2][b] * di[2][i];
                shg[3 * b + i] = sh[i];
            }
            const float Nb = c_trf[TOPO].shp[q][b];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const float d = (s[3 + k] - r[3 + k]) + (s[8 + k] - r[8 + k]);
                dq[k] += Nb * d;
                bq[k] += Nb * s[3 + k];
                aq[k] += Nb * s[13 + k];
#pragma unroll
                for (int i = 0; i < 3; ++i) g[i][k] += sh[i] * d;  // sum_b N_b,i = 0
            }
            if (WITH_Q)
#pragma unroll
                for (int k = 0; k < 4; ++k) divq[k] += sh[0] * s[18 + k] + sh[1] * s[22 + k] + sh[2] * s[26 + k];
        }
        Qp<float> st;
        qp_state(P, bq[0], bq[1], bq[2], bq[3], bq[4], st);
        Geo<float> gm;
        {
            auto cij = [&](int i, int j) { return di[0][i] * di[0][j] + di[1][i] * di[1][j] + di[2][i] * di[2][j]; };
            gm.G[0] = cij(0, 0);
            gm.G[1] = cij(0, 1);
            gm.G[2] = cij(1, 1);
            gm.G[3] = cij(0, 2);
            gm.G[4] = cij(1, 2);
            gm.G[5] = cij(2, 2);
            gm.GG = gm.G[0] * gm.G[0] + gm.G[2] * gm.G[2] + gm.G[5] * gm.G[5] +
                    2.f * (gm.G[1] * gm.G[1] + gm.G[3] * gm.G[3] + gm.G[4] * gm.G[4]);
            gm.trG = gm.G[0] + gm.G[2] + gm.G[5];
        }
        qp_tau(P, gm, st);
        float aig[5], a0a[5];
        ai_gi(st, g, aig);
        a0_v(st, aq, a0a);
        float tl[5];
        tl[0] = st.tau[0] * (aig[0] + a0a[0]);
        tl[1] = st.tau[1] * (aig[1] + a0a[1] - divq[0]);
        tl[2] = st.tau[1] * (aig[2] + a0a[2] - divq[1]);
        tl[3] = st.tau[1] * (aig[3] + a0a[3] - divq[2]);
        tl[4] = st.tau[2] * (aig[4] + a0a[4] - divq[3]);
        // Euler-flux increment F(y_q) - F(y_r) (flux sign of e3conv.f:72-96)
        const float pr = r[3], Tr = r[7];
        const float ur[3] = {r[4], r[5], r[6]};
        const float rhor = pr * P.rRgas / Tr;
        const float mr[3] = {rhor * ur[0], rhor * ur[1], rhor * ur[2]};
        const float drho = (dq[0] * Tr - pr * dq[4]) * P.rRgas / (Tr * st.T);
        const float dek = P.cv * dq[4] + (ur[0] * dq[1] + ur[1] * dq[2] + ur[2] * dq[3]) +
                          0.5f * (dq[1] * dq[1] + dq[2] * dq[2] + dq[3] * dq[3]);
        const float ek = st.ei + st.rk;
        float F[3][5];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float dm = drho * st.u[i] + rhor * dq[1 + i];
            F[i][0] = -dm;
#pragma unroll
            for (int j = 0; j < 3; ++j) F[i][1 + j] = -(dm * st.u[j] + mr[i] * dq[1 + j]) - (i == j ? dq[0] : 0.f);
            F[i][4] = -(dm * ek + mr[i] * dek) - (dq[1 + i] * st.p + ur[i] * dq[0]);
        }
        if (P.navier) {
            Visc<float> vs;
            viscous(P, g, vs);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
#pragma unroll
                for (int j = 0; j < 3; ++j) F[i][1 + j] += vs.t[i][j];
                F[i][4] += st.u[0] * vs.t[i][0] + st.u[1] * vs.t[i][1] + st.u[2] * vs.t[i][2] + vs.q[i];
            }
        }
        add_ai_v(st, tl, F);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k) o[1 + 5 * i + k] = F[i][k];
#pragma unroll
        for (int k = 0; k < 5; ++k) o[16 + k] = a0a[k];
    }
    __syncthreads();
    if (!active) return;
    // ---- node a: the FP32 increments summed over the points, plus sum_i I_a,i F_i(y_r) ----
    float o32[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
    for (int q = 0; q < NEN; ++q) {
        const float* v = sq + (size_t)QD * (le * NEN + q);
        const float w = v[0];
        const float* sh = v + 21 + 3 * a;
        const float Na = c_trf[TOPO].shp[q][a];
#pragma unroll
        for (int k = 0; k < 5; ++k)
            o32[k] += w * (sh[0] * v[1 + k] + sh[1] * v[6 + k] + sh[2] * v[11 + k] + Na * v[16 + k]);
    }
    const float* r = nod;
    const df64 p = df_make(r[3], r[8]);
    const df64 u[3] = {df_make(r[4], r[9]), df_make(r[5], r[10]), df_make(r[6], r[11])};
    const df64 T = df_make(r[7], r[12]);
    const df64 rho = df_mul(p, df_mul(df_make(K.rRgas_hi, K.rRgas_lo), df_rcp(T)));
    df64 rk = df_add(df_add(df_mul(u[0], u[0]), df_mul(u[1], u[1])), df_mul(u[2], u[2]));
    rk.hi *= 0.5f;
    rk.lo *= 0.5f;
    const df64 ek = df_add(df_mul(df_make(K.cv_hi, K.cv_lo), T), rk);
    const float2* Ia = I + 3 * ((size_t)e * NEN + a);
    const df64 Iai[3] = {df_make(Ia[0].x, Ia[0].y), df_make(Ia[1].x, Ia[1].y), df_make(Ia[2].x, Ia[2].y)};
    df64 c[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) c[k] = df_make(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const df64 m = df_mul(rho, u[i]);
        df64 Fi[5];
        Fi[0] = df_neg(m);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Fi[1 + j] = df_neg(df_mul(m, u[j]));
            if (i == j) Fi[1 + j] = df_sub(Fi[1 + j], p);
        }
        Fi[4] = df_neg(df_add(df_mul(m, ek), df_mul(u[i], p)));
#pragma unroll
        for (int k = 0; k < 5; ++k) c[k] = df_add(c[k], df_mul(Iai[i], Fi[k]));
    }
    double* og = out + 5 * (size_t)node;
#pragma unroll
    for (int k = 0; k < 5; ++k) og[k] += df_to_double(df_add(c[k], o32[k]));
}

template <int NEN, int TOPO>
void launch_block(Ctx& C, const int* d_ien, const std::vector<int>& col, const float2* I, const float* yh,
                  const float* ylo, const float* acf, const float* ql, double* out, const Phys<float>& P,
                  const RsConst& K) {
    constexpr int EPB = rs_epb<NEN>();
    const int ncol = (int)col.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int e0 = col[c], ne = col[c + 1] - e0;
        if (ne <= 0) continue;
        const int grid = (ne + EPB - 1) / EPB;
        const int* ie = d_ien + (size_t)NEN * e0;
        const float2* Ie = I + 3 * (size_t)NEN * e0;
        if (ql)
            k_topo_ress<NEN, TOPO, true><<<grid, kRsThreads, rs_smem<NEN, true>(), C.stream>>>(
                ie, ne, Ie, C.d_xf, yh, ylo, acf, ql, out, P, K);
        else
            k_topo_ress<NEN, TOPO, false><<<grid, kRsThreads, rs_smem<NEN, false>(), C.stream>>>(
                ie, ne, Ie, C.d_xf, yh, ylo, acf, ql, out, P, K);
        ++C.launches;
    }
}

// I_a,i = sum_q qwt_q sum_j shgl_j,a(q) adj(J(q))_j,i in FP64 (adj = det J * dxi/dx), as hi/lo floats
void flux_integrals(const TopoTabD& t, int nen, const std::vector<double>& x, const std::vector<int>& ien, int ne,
                    std::vector<float2>& out) {
    out.resize(3 * (size_t)nen * ne);
    for (int e = 0; e < ne; ++e) {
        const int* nd = ien.data() + (size_t)nen * e;
        double I[8][3] = {};
        for (int q = 0; q < nen; ++q) {
            double J[3][3] = {};
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    for (int b = 0; b < nen; ++b) J[i][j] += x[3 * (size_t)nd[b] + i] * t.shgl[q][j][b];
            double A[3][3];
            A[0][0] = J[1][1] * J[2][2] - J[2][1] * J[1][2];
            A[0][1] = J[2][1] * J[0][2] - J[0][1] * J[2][2];
            A[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
            A[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            A[1][1] = J[0][0] * J[2][2] - J[2][0] * J[0][2];
            A[1][2] = J[1][0] * J[0][2] - J[0][0] * J[1][2];
            A[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            A[2][1] = J[2][0] * J[0][1] - J[0][0] * J[2][1];
            A[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
            for (int a = 0; a < nen; ++a)
                for (int i = 0; i < 3; ++i)
                    I[a][i] += t.qwt[q] * (t.shgl[q][0][a] * A[0][i] + t.shgl[q][1][a] * A[1][i] +
                                           t.shgl[q][2][a] * A[2][i]);
        }
        for (int a = 0; a < nen; ++a)
            for (int i = 0; i < 3; ++i) {
                const float hi = (float)I[a][i];
                out[3 * ((size_t)e * nen + a) + i] = make_float2(hi, (float)(I[a][i] - (double)hi));
            }
    }
}

}  // namespace

int configure_topo_ress(Ctx& C);

int topo_split_setup(Ctx& C) {
    if (C.split_ready || (C.nhex == 0 && C.nwedge == 0)) return PHGPU_OK;
    TopoTabD td[3];
    topo_tables_host(td);
    std::vector<TopoTabF> tf(2);
    for (int k = 0; k < 2; ++k)
        for (int q = 0; q < 8; ++q) {
            tf[k].qwt[q] = (float)td[k].qwt[q];
            for (int a = 0; a < 8; ++a) {
                tf[k].shp[q][a] = (float)td[k].shp[q][a];
                for (int i = 0; i < 3; ++i) tf[k].shgl[q][i][a] = (float)td[k].shgl[q][i][a];
            }
        }
    int rc = check(C, cudaMemcpyToSymbolAsync(c_trf, tf.data(), sizeof(TopoTabF) * 2, 0, cudaMemcpyHostToDevice,
                                              C.stream),
                   "split-residual tables");
    if (rc == PHGPU_OK) rc = check(C, cudaStreamSynchronize(C.stream), "split-residual tables");  // a local source
    if (rc != PHGPU_OK) return rc;
    std::vector<double> x(3 * (size_t)C.N);
    rc = d2h(C, x.data(), C.d_x, sizeof(double) * x.size(), "download x");
    if (rc != PHGPU_OK) return rc;
    std::vector<float2> Ih, Iw;
    if (C.nhex > 0) flux_integrals(td[0], 8, x, C.h_ienh, C.nhex, Ih);
    if (C.nwedge > 0) flux_integrals(td[1], 6, x, C.h_ienw, C.nwedge, Iw);
    for (auto* pr : {&Ih, &Iw}) {
        float2** d = pr == &Ih ? &C.d_Ih : &C.d_Iw;
        if (cudaMalloc((void**)d, sizeof(float2) * std::max<size_t>(pr->size(), 1)) != cudaSuccess) {
            C.err = "cudaMalloc (flux integrals)";
            return PHGPU_ERR_NOMEM;
        }
        if (!pr->empty()) {
            rc = h2d(C, *d, pr->data(), sizeof(float2) * pr->size(), "upload flux integrals");
            if (rc != PHGPU_OK) return rc;
        }
    }
    rc = configure_topo_ress(C);
    if (rc == PHGPU_OK) C.split_ready = true;
    return rc;
}

void launch_topo_ress(Ctx& C, const float* yh, const float* ylo, const float* acf, double* out, const float* ql) {
    const Phys<float> P = make_phys<float>(C.cfg);
    RsConst K;
    auto split = [](double v, float& hi, float& lo) {
        hi = (float)v;
        lo = (float)(v - (double)hi);
    };
    split(1.0 / C.cfg.Rgas, K.rRgas_hi, K.rRgas_lo);
    split(C.cfg.Rgas / C.cfg.gamma1, K.cv_hi, K.cv_lo);
    if (C.nhex > 0) launch_block<8, 0>(C, C.d_ienh, C.hcol_start, C.d_Ih, yh, ylo, acf, ql, out, P, K);
    if (C.nwedge > 0) launch_block<6, 1>(C, C.d_ienw, C.wcol_start, C.d_Iw, yh, ylo, acf, ql, out, P, K);
}

int configure_topo_ress(Ctx& C) {
    int rc = PHGPU_OK;
    auto T = [&](cudaError_t e) { if (rc == PHGPU_OK) rc = check(C, e, "cudaFuncSetAttribute"); };
    T(smem_attr(k_topo_ress<8, 0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs_smem<8, false>()));
    T(smem_attr(k_topo_ress<8, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs_smem<8, true>()));
    T(smem_attr(k_topo_ress<6, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs_smem<6, false>()));
    T(smem_attr(k_topo_ress<6, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs_smem<6, true>()));
    return rc;
}

}  // namespace phgpu
