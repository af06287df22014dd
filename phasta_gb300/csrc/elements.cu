// elements.cu -- interior and boundary element kernels for linear tets.
//
// Physics of e3.f (e3ivar, e3mtrx, e3conv, e3visc, e3LS/e3tau, e3massr, e3bdg,
// e3wmlt; phSolver/compressible) and e3b.f/e3bvar.f, written for the GPU:
//  * a linear tet has constant shape-function gradients and Jacobian, so the
//    metrics (e3metric), the gradients of Y (e3ivar.f:259-334), the viscous
//    stress (e3visc.f:278-368, momentum part) and the tau metric (e3gijd)
//    are computed once per element instead of once per quadrature point;
//  * products with the Euler Jacobians A0..A3 (e3mtrx.f:79-224) use their
//    closed forms (A_i Y,i, A_i v, A0 v) instead of explicit 5x5 matrices;
//  * the block-diagonal tangent of e3bdg.f for node a,
//      N_a B_a + fct N_a^2 A0 + fct N_a B_a tau A0 + sum_pq N_a,p N_a,q (A_p tau A_q + K_pq),
//    with B_a = sum_i N_a,i A_i, is evaluated as the product
//      (N_a I + B_a tau)(B_a + fct N_a A0) + K_a,
//    which is the same sum regrouped;
//  * the weights of e3wmlt.f are applied once per element after the
//    quadrature sum (WdetJ is the same at every point of a linear tet).
// Results agree with the statement-by-statement restatement to rounding.
#include <algorithm>
#include <type_traits>

#include "phgpu_impl.cuh"
#include "df64.cuh"
#include "qpoint.cuh"

// occupancy targets (resident CTAs per SM) of the FP32 chunk kernels
#ifndef PHGPU_RES32_MINB
#define PHGPU_RES32_MINB 4
#endif
#ifndef PHGPU_FULL32_MINB
#define PHGPU_FULL32_MINB 3
#endif
#ifndef PHGPU_FULL32BD_MINB
#define PHGPU_FULL32BD_MINB 4
#endif
#ifndef PHGPU_RESS_MINB
#define PHGPU_RESS_MINB 3
#endif
#ifndef PHGPU_LINPIPE_MINB
#define PHGPU_LINPIPE_MINB 4
#endif
#ifndef PHGPU_RES_QUNROLL
#define PHGPU_RES_QUNROLL 1
#endif
#define PH_STR(x) #x
#define PH_UNROLL(n) _Pragma(PH_STR(unroll n))

namespace phgpu {

__constant__ TetTables c_tab;
__constant__ float c_shpf[4][4];   // single-precision copies (no conversions in FP32 kernels)
__constant__ float c_qwtf;

int upload_topo_tables(Ctx& C);

// tet point weight: symtet.c's 1/4 scaled by 4/3 (genint.f:72)
constexpr double kTetQwt = (4.0 / 3.0) * 0.25;

int upload_tables(Ctx& C) {
    TetTables t;
    // symtet.c 4-point rule (barycentric (a,b,b,b) permutations), genint.f:72 Qwt *= 4/3
    const double a4 = 0.5854101966249685, b4 = 0.1381966011250150;
    const double pts[4][3] = {{a4, b4, b4}, {b4, a4, b4}, {b4, b4, a4}, {b4, b4, b4}};
    for (int q = 0; q < 4; ++q) {
        t.shp[q][0] = pts[q][0];
        t.shp[q][1] = pts[q][1];
        t.shp[q][2] = pts[q][2];
        t.shp[q][3] = 1.0 - pts[q][0] - pts[q][1] - pts[q][2];
        t.Qwt[q] = kTetQwt;
    }
    // symtri.c 3-point rule, genint.f:73 Qwtb *= 2
    const double A = 0.333333333333333, B = 0.666666666666667, Cc = 0.166666666666667;
    const double ptb[3][3] = {{B, Cc, Cc}, {Cc, B, Cc}, {Cc, Cc, B}};
    for (int q = 0; q < 3; ++q) {
        t.shpb[q][0] = ptb[q][0];
        t.shpb[q][1] = ptb[q][1];
        t.shpb[q][2] = ptb[q][2];
        t.shpb[q][3] = 1.0 - ptb[q][0] - ptb[q][1] - ptb[q][2];
        t.Qwtb[q] = 2.0 * A;
    }
    int rc = check(C, cudaMemcpyToSymbolAsync(c_tab, &t, sizeof(t), 0, cudaMemcpyHostToDevice, C.stream),
                   "upload tables");
    float sf[4][4];
    for (int q = 0; q < 4; ++q)
        for (int a = 0; a < 4; ++a) sf[q][a] = (float)t.shp[q][a];
    if (rc == PHGPU_OK)
        rc = check(C, cudaMemcpyToSymbolAsync(c_shpf, sf, sizeof(sf), 0, cudaMemcpyHostToDevice, C.stream),
                   "upload tables");
    const float qf = (float)t.Qwt[0];
    if (rc == PHGPU_OK)
        rc = check(C, cudaMemcpyToSymbolAsync(c_qwtf, &qf, sizeof(qf), 0, cudaMemcpyHostToDevice, C.stream),
                   "upload tables");
    if (rc == PHGPU_OK) rc = upload_topo_tables(C);
    // the sources are this function's locals
    if (rc == PHGPU_OK) rc = check(C, cudaStreamSynchronize(C.stream), "upload tables");
    return rc;
}

template <typename R>
Phys<R> make_phys(const phgpu_config& c) {
    Phys<R> p;
    const double cv = c.Rgas / c.gamma1, cp = c.Rgas * c.gamma / c.gamma1;
    const double rlm = -(2.0 / 3.0) * c.rmu;
    const double dts = c.iremoveStabTimeTerm ? 0.0 : c.dtsfct * c.Dtgl;
    p.Rgas = (R)c.Rgas;
    p.rRgas = (R)(1.0 / c.Rgas);
    p.cv = (R)cv;
    p.cp = (R)cp;
    p.rmu = (R)c.rmu;
    p.rlm = (R)rlm;
    p.rlm2mu = (R)(rlm + 2.0 * c.rmu);
    p.rlmpmu = (R)(rlm + c.rmu);
    p.con = (R)(c.rmu * cp / c.pr);
    p.fct1 = (R)(c.almi / c.gami / c.alfi * c.Dtgl);
    p.dts2 = (R)((2.0 * dts) * (2.0 * dts));
    p.fmu2 = (R)(36.0 * c.rmu * c.rmu);
    p.taucfct = (R)c.taucfct;
    p.rtempcv = (R)(c.temper / cv);
    p.navier = c.Navier;
    p.supg = c.ivart >= 2;
    p.epsM = (R)c.epsM;
    p.idc = c.iDC;
    p.itau = c.itau;
    p.rdts = (R)(1.0 / (c.Dtgl * c.dtsfct));
    p.celt = (R)(2.0 / 3.0);
    p.temper = (R)c.temper;
    return p;
}
template Phys<double> make_phys<double>(const phgpu_config&);
template Phys<float> make_phys<float>(const phgpu_config&);

namespace {

template <typename R> __device__ __forceinline__ R shp(int q, int a);
template <> __device__ __forceinline__ double shp<double>(int q, int a) { return c_tab.shp[q][a]; }
template <> __device__ __forceinline__ float shp<float>(int q, int a) { return c_shpf[q][a]; }
template <typename R> __device__ __forceinline__ R qwt();
template <> __device__ __forceinline__ double qwt<double>() { return c_tab.Qwt[0]; }
template <> __device__ __forceinline__ float qwt<float>() { return c_qwtf; }

template <typename R>
__device__ __forceinline__ void geometry(const R (&xl)[4][3], Geo<R>& g) {
    R d[3][3];  // dx_i / dxi_j with the halved tet gradients (genshp.f:32-35)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) d[i][j] = R(0.5) * (xl[j][i] - xl[3][i]);
    const R c00 = d[1][1] * d[2][2] - d[2][1] * d[1][2];
    const R c01 = d[2][1] * d[0][2] - d[0][1] * d[2][2];
    const R c02 = d[0][1] * d[1][2] - d[0][2] * d[1][1];
    const R det = c00 * d[0][0] + c01 * d[1][0] + c02 * d[2][0];
    const R rdet = R(1) / det;
    R di[3][3];
    di[0][0] = c00 * rdet;
    di[0][1] = c01 * rdet;
    di[0][2] = c02 * rdet;
    di[1][0] = (d[1][2] * d[2][0] - d[1][0] * d[2][2]) * rdet;
    di[1][1] = (d[0][0] * d[2][2] - d[2][0] * d[0][2]) * rdet;
    di[1][2] = (d[1][0] * d[0][2] - d[0][0] * d[1][2]) * rdet;
    di[2][0] = (d[1][0] * d[2][1] - d[1][1] * d[2][0]) * rdet;
    di[2][1] = (d[2][0] * d[0][1] - d[0][0] * d[2][1]) * rdet;
    di[2][2] = (d[0][0] * d[1][1] - d[0][1] * d[1][0]) * rdet;
    g.WdetJ = qwt<R>() * det;
    R s[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        g.shg[0][i] = R(0.5) * di[0][i];
        g.shg[1][i] = R(0.5) * di[1][i];
        g.shg[2][i] = R(0.5) * di[2][i];
        g.shg[3][i] = -(g.shg[0][i] + g.shg[1][i] + g.shg[2][i]);
        s[i] = di[0][i] + di[1][i] + di[2][i];
    }
    // e3tau.f:1440-1470: G = dxidx^T M dxidx with M = c2 * ones + (c1 - c2) I
    const R c2 = R(6.299605249474365e-01), cm = R(1.259921049894873e+00 - 6.299605249474365e-01);
    auto gij = [&](int i, int j) {
        return cm * (di[0][i] * di[0][j] + di[1][i] * di[1][j] + di[2][i] * di[2][j]) + c2 * s[i] * s[j];
    };
    g.G[0] = gij(0, 0);
    g.G[1] = gij(0, 1);
    g.G[2] = gij(1, 1);
    g.G[3] = gij(0, 2);
    g.G[4] = gij(1, 2);
    g.G[5] = gij(2, 2);
    g.GG = g.G[0] * g.G[0] + g.G[2] * g.G[2] + g.G[5] * g.G[5] +
           R(2) * (g.G[1] * g.G[1] + g.G[3] * g.G[3] + g.G[4] * g.G[4]);
    g.trG = g.G[0] + g.G[2] + g.G[5];
}

// gradients g[i][k] = sum_n N_n,i v_n,k
template <typename R>
__device__ __forceinline__ void gradients(const Geo<R>& geo, const R (&v)[4][5], R (&g)[3][5]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 5; ++k)
            g[i][k] = geo.shg[0][i] * v[0][k] + geo.shg[1][i] * v[1][k] + geo.shg[2][i] * v[2][k] +
                      geo.shg[3][i] * v[3][k];
}

template <typename R>
__device__ __forceinline__ void load5(const R* __restrict__ a, int n, R (&o)[5]) {
    const R* p = a + 5 * (size_t)n;
#pragma unroll
    for (int k = 0; k < 5; ++k) o[k] = ldg(p + k);
}

// --------------------------------------------------------------------------
// chunk kernels: one CTA per chunk of <= kChunk elements
//   phase 1  the chunk's nodes are staged in shared memory
//   phase 2  each element's contributions go to shared-memory slots
//   phase 3  each chunk node sums its slots (ascending (element, corner)
//            order) and adds the sum to the global array; chunks that run
//            concurrently share no node
// --------------------------------------------------------------------------
struct ChunkArgs {
    const int* elem;     // nchunk+1
    const int* node;     // nchunk+1
    const int* nodes;    // global node of each chunk-local node
    const int* cstart;   // slot-list offsets per chunk-local node (+1)
    const unsigned short* csr;  // slot = element*4 + corner
    const ushort4* lien; // local node indices per element
};

template <typename R>
__device__ __forceinline__ void lds5(const R* __restrict__ s, int l, R (&o)[5]) {
#pragma unroll
    for (int k = 0; k < 5; ++k) o[k] = s[5 * l + k];
}

// residual family for one element (node data already gathered):
//   RM_RES    : ires = 1 residual of state va with acceleration vb
//   RM_MODRES : ires = 2 modified residual of (va = perturbed, vb = base)
//   RM_LIN    : d/d eps of the modified residual at vb in direction va
// writes the four nodal contributions (already weighted) to o[a][k]
template <typename R, int MODE>
__device__ __forceinline__ void elem_res(const Phys<R>& P, const R (&xl)[4][3], const R (&va)[4][5],
                                         const R (&vb)[4][5], R (&o)[4][5], const R* divq = nullptr) {
    Geo<R> geo;
    geometry(xl, geo);
    const R (&base)[4][5] = (MODE == RM_RES) ? va : vb;
    R g[3][5];
    gradients(geo, va, g);
    Visc<R> vs;
    if (P.navier) viscous(P, g, vs);
    R S[3][5];
    R Tn[4][5];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 5; ++k) S[i][k] = R(0);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int k = 0; k < 5; ++k) Tn[a][k] = R(0);

    PH_UNROLL(PHGPU_RES_QUNROLL)
    for (int q = 0; q < 4; ++q) {
        R N[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) N[a] = shp<R>(q, a);
        R bq[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) bq[k] = N[0] * base[0][k] + N[1] * base[1][k] + N[2] * base[2][k] + N[3] * base[3][k];
        Qp<R> b;
        qp_state(P, bq[0], bq[1], bq[2], bq[3], bq[4], b);
        qp_tau(P, geo, b);
        R F[3][5];
        R r16[5];
        R aig[5];
        ai_gi(b, g, aig);
        R ly[5];  // the least-squares residual before tau (discontinuity capturing)
#pragma unroll
        for (int k = 0; k < 5; ++k) ly[k] = aig[k];
        if (MODE == RM_RES) {
            // Euler flux integrated by parts (e3conv.f:72-96)
            const R ek = b.ei + b.rk;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const R m = -b.u[i] * b.rho;
                F[i][0] = m;
#pragma unroll
                for (int j = 0; j < 3; ++j) F[i][1 + j] = m * b.u[j] - (i == j ? b.p : R(0));
                F[i][4] = m * ek - b.u[i] * b.p;
            }
            R acq[5], a0a[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) acq[k] = N[0] * vb[0][k] + N[1] * vb[1][k] + N[2] * vb[2][k] + N[3] * vb[3][k];
            a0_v(b, acq, a0a);
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                r16[k] = a0a[k];
                aig[k] = aig[k] + a0a[k];  // rLyi += A0 aci (e3ls.f:105-143)
            }
            if (divq) {  // idiff = 1: rLyi -= div q (e3ls.f:147-156)
#pragma unroll
                for (int k = 0; k < 4; ++k) aig[1 + k] -= divq[k];
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) ly[k] = aig[k];
        } else {
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 5; ++k) F[i][k] = R(0);
            R du[5];
            R pv[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) pv[k] = N[0] * va[0][k] + N[1] * va[1][k] + N[2] * va[2][k] + N[3] * va[3][k];
            if (MODE == RM_MODRES) {
                // conservative variables of the perturbed state (e3ivar.f:96-131)
                const R rho6 = pv[0] / (P.Rgas * pv[4]);
                const R rk6 = R(0.5) * (pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3]);
                du[0] = rho6;
                du[1] = rho6 * pv[1];
                du[2] = rho6 * pv[2];
                du[3] = rho6 * pv[3];
                du[4] = rho6 * (pv[4] * P.cv + rk6);
            } else {
                a0_v(b, pv, du);
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                aig[k] = aig[k] + P.fct1 * du[k];  // rLymi = rLyi + fct1 dui
                r16[k] = aig[k];                   // rmi(16:20) (e3conv.f:183, e3massr.f:74-88)
            }
        }
        if (P.navier) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
#pragma unroll
                for (int j = 0; j < 3; ++j) F[i][1 + j] += vs.t[i][j];
                F[i][4] += b.u[0] * vs.t[i][0] + b.u[1] * vs.t[i][1] + b.u[2] * vs.t[i][2] + vs.q[i];
            }
        }
        // tau L and the least-squares term A_i tau L (e3ls.f:231-459)
        R tl[5];
        tl[0] = b.tau[0] * aig[0];
        tl[1] = b.tau[1] * aig[1];
        tl[2] = b.tau[1] * aig[2];
        tl[3] = b.tau[1] * aig[3];
        tl[4] = b.tau[2] * aig[4];
        add_ai_v(b, tl, F);
        if constexpr (sizeof(R) == 8 && MODE != RM_LIN) {
            // discontinuity capturing (e3dc.f): the residual pairs rTLS with tau L, the
            // modified residual (ires = 2) with L itself (e3tau.f:185-205)
            if (P.idc) {
                R gA[3][5];
                const R dc = dc_point(P, geo.G, b, g, ly, MODE == RM_RES ? tl : ly, gA);
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 5; ++k) F[i][k] += dc * gA[i][k];
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k) S[i][k] += F[i][k];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k) Tn[a][k] += N[a] * r16[k];
    }
    // e3wmlt.f weights
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int k = 0; k < 5; ++k)
            o[a][k] = geo.WdetJ * (geo.shg[a][0] * S[0][k] + geo.shg[a][1] * S[1][k] + geo.shg[a][2] * S[2][k] + Tn[a][k]);
}

// div q of the reconstructed nodal diffusive flux (e3ivar.f:374-395): q staged as 12 values
// per chunk node (row-major 3 x 4: flux direction i, component k)
template <typename R>
__device__ __forceinline__ void tet_divq(const R (&xl)[4][3], const R* __restrict__ sq, const int (&nd)[4],
                                         R (&divq)[4]) {
    Geo<R> geo;
    geometry(xl, geo);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        R acc = R(0);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const R* q = sq + 12 * nd[a];
            acc += geo.shg[a][0] * q[k] + geo.shg[a][1] * q[4 + k] + geo.shg[a][2] * q[8 + k];
        }
        divq[k] = acc;
    }
}

template <typename R, int MODE>
__global__ void __launch_bounds__(kChunk, sizeof(R) == 4 ? PHGPU_RES32_MINB : 2)
k_chunk_res(ChunkArgs ca, int chunk0, const R* __restrict__ x, const R* __restrict__ ya,
            const R* __restrict__ yb, const R* __restrict__ ac, R* __restrict__ out, Phys<R> P, int iabres,
            const int* __restrict__ skip, const R* __restrict__ ql = nullptr) {
    if (skip && *skip) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sm = reinterpret_cast<R*>(smem_raw);
    const int c = chunk0 + blockIdx.x;
    const int e0 = ca.elem[c], ne = ca.elem[c + 1] - e0;
    const int n0 = ca.node[c], nn = ca.node[c + 1] - n0;
    const bool with_q = (MODE == RM_RES) && ql != nullptr;
    R* sx = sm;
    R* sa = sx + 3 * nn;
    R* sb = sa + 5 * nn;
    R* sq = sb + 5 * nn;                  // idiff = 1: reconstructed flux, 12 per node
    R* slot = sq + (with_q ? 12 * nn : 0);
    const R* bsrc = (MODE == RM_RES) ? ac : yb;
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        const int gn = ca.nodes[n0 + l];
#pragma unroll
        for (int d = 0; d < 3; ++d) sx[3 * l + d] = ldg(x + 3 * (size_t)gn + d);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            sa[5 * l + k] = ldg(ya + 5 * (size_t)gn + k);
            sb[5 * l + k] = ldg(bsrc + 5 * (size_t)gn + k);
        }
        if (with_q)
            for (int k = 0; k < 12; ++k) sq[12 * l + k] = ldg(ql + 13 * (size_t)gn + k);
    }
    __syncthreads();
    if ((int)threadIdx.x < ne) {
        const ushort4 ln = ca.lien[e0 + threadIdx.x];
        const int nd[4] = {ln.x, ln.y, ln.z, ln.w};
        R xl[4][3], va[4][5], vb[4][5];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
            for (int d = 0; d < 3; ++d) xl[a][d] = sx[3 * nd[a] + d];
            lds5(sa, nd[a], va[a]);
            lds5(sb, nd[a], vb[a]);
        }
        R o[4][5];
        if (with_q) {
            R divq[4];
            tet_divq(xl, sq, nd, divq);
            elem_res<R, MODE>(P, xl, va, vb, o, divq);
        } else {
            elem_res<R, MODE>(P, xl, va, vb, o);
        }
        R* sl = slot + 20 * threadIdx.x;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k) sl[5 * a + k] = iabres ? fabs(o[a][k]) : o[a][k];
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        R acc[5] = {R(0), R(0), R(0), R(0), R(0)};
        const int s0 = ca.cstart[n0 + l], s1 = ca.cstart[n0 + l + 1];
        for (int s = s0; s < s1; ++s) {
            const R* sl = slot + 5 * (int)ca.csr[s];
#pragma unroll
            for (int k = 0; k < 5; ++k) acc[k] += sl[k];
        }
        R* og = out + 5 * (size_t)ca.nodes[n0 + l];
#pragma unroll
        for (int k = 0; k < 5; ++k) og[k] += acc[k];
    }
}

// --------------------------------------------------------------------------
// persistent, software-pipelined sweeps over the chunks of one colour (cp.async staging)
// --------------------------------------------------------------------------
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// words of a node-id stage of the pipelined split residual: e0, ne, n0, nn, then the chunk's
// global node ids
__host__ __device__ constexpr int lin_id_words(int lmax) { return 4 + lmax; }

// --- bulk copies (cp.async.bulk, completion on an mbarrier) ---
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// makes the initialised mbarriers visible to the async proxy (the bulk-copy unit that completes
// them) before their first use
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// one contiguous copy global -> shared: both addresses 16-byte aligned, size a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// a wait that gives up: false after kMbarTries unsuccessful tries (each may suspend the thread
// for a short, hardware-chosen time), so that a copy that never completes cannot hang the GPU
constexpr int kMbarTries = kMbarTriesMax;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int tries = kMbarTries) {
    for (int i = 0; i < tries; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
// self-test of the bounded wait: an mbarrier that expects two arrivals and gets one never
// completes its phase, so mbar_wait gives up after `tries` tries; status[0] is then the bit a
// sweep sets when its bulk copy does not complete
__global__ void k_wait_limit_probe(int tries, int* status) {
    __shared__ unsigned long long bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 2);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive(&bar);
        status[0] = mbar_wait(&bar, 0, tries) ? 0 : kPipeCopyFailed;
    }
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}

// floats of one node-data stage of the pipelined linearized product: the packed base state
// and coordinates (8 per node, 16-byte aligned), the direction (5) and the product (5)
__host__ __device__ constexpr int lin_data_words(int lmax) { return (18 * lmax + 3) & ~3; }

// The FP32 linearized product over the chunks of one colour, software-pipelined: each CTA
// walks chunks chunk0 + blockIdx.x, + gridDim.x, ...  Per chunk, one thread moves the chunk's
// record (header, node ids, connectivity, slot lists, slot offsets: contiguous, 16-byte aligned,
// chunks.cu) into shared memory with one bulk copy two chunks ahead, completion signalled on an
// mbarrier; one chunk ahead every thread gathers the chunk's node data with cp.async (the packed
// base state and coordinates as two 16-byte copies, the direction and the product's current
// values as 4-byte ones) into the other half of a double buffer, while the current chunk is
// computed.  Chunks of one colour share no node, so prefetching the product's values of a later
// chunk is safe.  The arithmetic and the summation order are those of k_chunk_res<float, RM_LIN>.
// If a bulk copy does not complete within the wait limit, the CTA sets bit 8 of *err and returns.
template <int MINB>
__global__ void __launch_bounds__(kChunk, MINB)
k_chunk_lin_pipe(const uint4* __restrict__ rec, const int* __restrict__ rec_off, int chunk0, int nch,
                 const float4* __restrict__ xb, const float* __restrict__ ya, float* __restrict__ out, Phys<float> P,
                 int lmax, int rec_bytes, int* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* R = smem_raw;                                   // 3 record stages of rec_bytes
    float* D = reinterpret_cast<float*>(smem_raw + 3 * (size_t)rec_bytes);  // 2 node-data stages
    const int dw = lin_data_words(lmax);
    float* slot = D + 2 * dw;                                      // 20 per element
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(slot + 20 * kChunk);
    __shared__ int s_abort;
    const int cend = chunk0 + nch, G = gridDim.x;
    int c = chunk0 + blockIdx.x;
    if (c >= cend) return;
    auto issue = [&](int chunk, int st) {  // thread 0: the record of chunk into stage st
        const unsigned bytes = 16u * (unsigned)(rec_off[chunk + 1] - rec_off[chunk]);
        mbar_expect_tx(&bar[st], bytes);
        bulk_g2s(R + (size_t)st * rec_bytes, rec + rec_off[chunk], bytes, &bar[st]);
    };
    auto record = [&](int st) { return reinterpret_cast<const int*>(R + (size_t)st * rec_bytes); };
    // node data of the chunk whose record is in stage st, into data stage b
    auto stage_data = [&](int st, float* b) {
        const int* h = record(st);
        const int nn = h[3];
        const int* ids = h + rec_ids_off();
        float* sxb = b;
        float* sa = sxb + 8 * lmax;
        float* so = sa + 5 * lmax;
        for (int l = threadIdx.x; l < nn; l += blockDim.x) {
            const size_t gn = (size_t)ids[l];
            cp_async16(sxb + 8 * l, xb + 2 * gn);
            cp_async16(sxb + 8 * l + 4, xb + 2 * gn + 1);
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                cp_async4(sa + 5 * l + k, ya + 5 * gn + k);
                cp_async4(so + 5 * l + k, out + 5 * gn + k);
            }
        }
    };
    // every thread reaches this with the same ok: a failed wait ends the CTA after a second
    // bounded wait for the copy it was waiting on
    auto aborted = [&](bool ok, int st, unsigned parity) {
        if (!ok) s_abort = 1;
        __syncthreads();
        if (!s_abort) return false;
        if (threadIdx.x == 0) atomicOr(err, 8);
        (void)mbar_wait(&bar[st], parity);
        return true;
    };
    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int i = 0; i < 3; ++i) mbar_init(&bar[i], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        issue(c, 0);
        if (c + G < cend) issue(c + G, 1);
    }
    if (aborted(mbar_wait(&bar[0], 0), 0, 0)) {
        if (c + G < cend) (void)mbar_wait(&bar[1], 0);  // the other copy in flight
        return;
    }
    stage_data(0, D);
    cp_async_commit();
    for (int it = 0; c < cend; c += G, ++it) {
        const int cn = c + G;
        const int sn = (it + 1) % 3;
        const unsigned pn = (unsigned)(((it + 1) / 3) & 1);
        cp_async_wait<0>();  // node data of chunk c
        const bool ok = cn < cend ? mbar_wait(&bar[sn], pn) : true;  // record of chunk cn
        if (aborted(ok, sn, pn)) return;
        if (cn < cend) stage_data(sn, D + ((it + 1) & 1) * dw);
        if (threadIdx.x == 0 && cn + G < cend) {
            fence_proxy_async();  // the stage's last readers finished at the barrier above
            issue(cn + G, (it + 2) % 3);
        }
        cp_async_commit();
        const int* h = record(it % 3);
        const int ne = h[1], nn = h[3];
        const int* ids = h + rec_ids_off();
        const ushort4* slie = reinterpret_cast<const ushort4*>(h + rec_lien_off(nn));
        const unsigned short* scsr = reinterpret_cast<const unsigned short*>(h + rec_csr_off(ne, nn));
        const int* scst = h + rec_cst_off(ne, nn);
        const float* cur = D + (it & 1) * dw;
        const float* sxb = cur;
        const float* sa = sxb + 8 * lmax;
        const float* so = sa + 5 * lmax;
        if ((int)threadIdx.x < ne) {
            const ushort4 ln = slie[threadIdx.x];
            const int nd[4] = {ln.x, ln.y, ln.z, ln.w};
            float xl[4][3], va[4][5], vb[4][5];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float4 p0 = *reinterpret_cast<const float4*>(sxb + 8 * nd[a]);
                const float4 p1 = *reinterpret_cast<const float4*>(sxb + 8 * nd[a] + 4);
                vb[a][0] = p0.x;
                vb[a][1] = p0.y;
                vb[a][2] = p0.z;
                vb[a][3] = p0.w;
                vb[a][4] = p1.x;
                xl[a][0] = p1.y;
                xl[a][1] = p1.z;
                xl[a][2] = p1.w;
                lds5(sa, nd[a], va[a]);
            }
            float o[4][5];
            elem_res<float, RM_LIN>(P, xl, va, vb, o);
            float* sl = slot + 20 * threadIdx.x;
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int k = 0; k < 5; ++k) sl[5 * a + k] = o[a][k];
        }
        __syncthreads();
        for (int l = threadIdx.x; l < nn; l += blockDim.x) {
            float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
            const int s0 = scst[l], s1 = scst[l + 1];
            for (int s = s0; s < s1; ++s) {
                const float* sl = slot + 5 * (int)scsr[s];
#pragma unroll
                for (int k = 0; k < 5; ++k) acc[k] += sl[k];
            }
            float* og = out + 5 * (size_t)ids[l];
#pragma unroll
            for (int k = 0; k < 5; ++k) og[k] = so[5 * l + k] + acc[k];
        }
        // no barrier here: the next iteration's first barrier precedes every write of the slots,
        // of this data stage and of this record stage
    }
    cp_async_wait<0>();
}

// the FP32 base state and the coordinates packed per node: (yb0, yb1, yb2, yb3), (yb4, x0, x1, x2)
__global__ void k_pack_xb(const float* __restrict__ xf, const float* __restrict__ yf, float4* __restrict__ xb,
                          int N) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        const float* y = yf + 5 * (size_t)n;
        const float* x = xf + 3 * (size_t)n;
        xb[2 * (size_t)n] = make_float4(y[0], y[1], y[2], y[3]);
        xb[2 * (size_t)n + 1] = make_float4(y[4], x[0], x[1], x[2]);
    }
}

// --------------------------------------------------------------------------
// idiff = 1: lumped L2 reconstruction of the diffusive flux (AsIq/e3q.f:54-191).
// Per element and node a: sum_q N_a WdetJ qdi(q) (12 values, qdi the viscous
// flux of e3q.f at point q) and sum_q N_a WdetJ (lumped mass); out holds 13
// values per node (flux row-major (direction, component), then the mass).
// --------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void visc_flux12(const Phys<R>& P, const Visc<R>& vs, R u0, R u1, R u2, R (&q)[12]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        q[4 * i + 0] = vs.t[i][0];
        q[4 * i + 1] = vs.t[i][1];
        q[4 * i + 2] = vs.t[i][2];
        q[4 * i + 3] = u0 * vs.t[i][0] + u1 * vs.t[i][1] + u2 * vs.t[i][2] + vs.q[i];
    }
}

template <typename R>
__global__ void __launch_bounds__(kChunk)
k_chunk_qrec(ChunkArgs ca, int chunk0, const R* __restrict__ x, const R* __restrict__ y, R* __restrict__ out,
             Phys<R> P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sm = reinterpret_cast<R*>(smem_raw);
    const int c = chunk0 + blockIdx.x;
    const int e0 = ca.elem[c], ne = ca.elem[c + 1] - e0;
    const int n0 = ca.node[c], nn = ca.node[c + 1] - n0;
    R* sx = sm;
    R* sy = sx + 3 * nn;
    R* slot = sy + 5 * nn;  // 13 per (element, corner)
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        const int gn = ca.nodes[n0 + l];
#pragma unroll
        for (int d = 0; d < 3; ++d) sx[3 * l + d] = ldg(x + 3 * (size_t)gn + d);
#pragma unroll
        for (int k = 0; k < 5; ++k) sy[5 * l + k] = ldg(y + 5 * (size_t)gn + k);
    }
    __syncthreads();
    if ((int)threadIdx.x < ne) {
        const ushort4 ln = ca.lien[e0 + threadIdx.x];
        const int nd[4] = {ln.x, ln.y, ln.z, ln.w};
        R xl[4][3], yl[4][5];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
            for (int d = 0; d < 3; ++d) xl[a][d] = sx[3 * nd[a] + d];
            lds5(sy, nd[a], yl[a]);
        }
        Geo<R> geo;
        geometry(xl, geo);
        R g[3][5];
        gradients(geo, yl, g);
        Visc<R> vs;
        viscous(P, g, vs);
        R ql[4][13];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 13; ++k) ql[a][k] = R(0);
#pragma unroll 1
        for (int q = 0; q < 4; ++q) {
            R N[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) N[a] = shp<R>(q, a);
            const R u0 = N[0] * yl[0][1] + N[1] * yl[1][1] + N[2] * yl[2][1] + N[3] * yl[3][1];
            const R u1 = N[0] * yl[0][2] + N[1] * yl[1][2] + N[2] * yl[2][2] + N[3] * yl[3][2];
            const R u2 = N[0] * yl[0][3] + N[1] * yl[1][3] + N[2] * yl[2][3] + N[3] * yl[3][3];
            R qd[12];
            visc_flux12(P, vs, u0, u1, u2, qd);
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const R w = N[a] * geo.WdetJ;
#pragma unroll
                for (int k = 0; k < 12; ++k) ql[a][k] += w * qd[k];
                ql[a][12] += w;
            }
        }
        R* sl = slot + 52 * threadIdx.x;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 13; ++k) sl[13 * a + k] = ql[a][k];
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        R acc[13];
#pragma unroll
        for (int k = 0; k < 13; ++k) acc[k] = R(0);
        const int s0 = ca.cstart[n0 + l], s1 = ca.cstart[n0 + l + 1];
        for (int s = s0; s < s1; ++s) {
            const R* sl = slot + 13 * (int)ca.csr[s];
#pragma unroll
            for (int k = 0; k < 13; ++k) acc[k] += sl[k];
        }
        R* og = out + 13 * (size_t)ca.nodes[n0 + l];
#pragma unroll
        for (int k = 0; k < 13; ++k) og[k] += acc[k];
    }
}

// --------------------------------------------------------------------------
// outer residual (ires = 1) with FP64 Galerkin terms and FP32 stabilization:
// the element metrics and weights, the Euler flux (e3conv.f:72-96) and the
// time term N_a A0 Y,t (e3massr.f:26-58) -- the large terms that cancel
// between elements -- are FP64; the least-squares term A_i tau L (e3ls.f) and
// the viscous flux (e3visc.f), which are small in comparison, are FP32.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(kChunk, 2)
k_chunk_resh(ChunkArgs ca, int chunk0, const double* __restrict__ x, const double* __restrict__ y,
             const double* __restrict__ ac, const float* __restrict__ xf, const float* __restrict__ yf,
             const float* __restrict__ acf, double* __restrict__ out, Phys<double> P, Phys<float> Pf) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* sm = reinterpret_cast<double*>(smem_raw);
    const int c = chunk0 + blockIdx.x;
    const int e0 = ca.elem[c], ne = ca.elem[c + 1] - e0;
    const int n0 = ca.node[c], nn = ca.node[c + 1] - n0;
    double* sx = sm;
    double* sy = sx + 3 * nn;
    double* sa = sy + 5 * nn;
    double* slot = sa + 5 * nn;
    float* fsm = reinterpret_cast<float*>(slot + 20 * kChunk);
    float* fx = fsm;
    float* fy = fx + 3 * nn;
    float* fa = fy + 5 * nn;
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        const size_t gn = ca.nodes[n0 + l];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            sx[3 * l + d] = __ldg(x + 3 * gn + d);
            fx[3 * l + d] = __ldg(xf + 3 * gn + d);
        }
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            sy[5 * l + k] = __ldg(y + 5 * gn + k);
            sa[5 * l + k] = __ldg(ac + 5 * gn + k);
            fy[5 * l + k] = __ldg(yf + 5 * gn + k);
            fa[5 * l + k] = __ldg(acf + 5 * gn + k);
        }
    }
    __syncthreads();
    if ((int)threadIdx.x < ne) {
        const ushort4 ln = ca.lien[e0 + threadIdx.x];
        const int nd[4] = {ln.x, ln.y, ln.z, ln.w};
        // ---- FP32: viscous flux and least-squares term, summed over the points ----
        float S32[3][5];
        {
            float xl[4][3], yl[4][5], al[4][5];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
#pragma unroll
                for (int d = 0; d < 3; ++d) xl[a][d] = fx[3 * nd[a] + d];
                lds5(fy, nd[a], yl[a]);
                lds5(fa, nd[a], al[a]);
            }
            Geo<float> geo;
            geometry(xl, geo);
            float g[3][5];
            gradients(geo, yl, g);
            Visc<float> vs;
            if (Pf.navier) viscous(Pf, g, vs);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 5; ++k) S32[i][k] = 0.f;
#pragma unroll 1
            for (int q = 0; q < 4; ++q) {
                float N[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) N[a] = shp<float>(q, a);
                float bq[5], aq[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    bq[k] = N[0] * yl[0][k] + N[1] * yl[1][k] + N[2] * yl[2][k] + N[3] * yl[3][k];
                    aq[k] = N[0] * al[0][k] + N[1] * al[1][k] + N[2] * al[2][k] + N[3] * al[3][k];
                }
                Qp<float> b;
                qp_state(Pf, bq[0], bq[1], bq[2], bq[3], bq[4], b);
                qp_tau(Pf, geo, b);
                float aig[5], a0a[5];
                ai_gi(b, g, aig);
                a0_v(b, aq, a0a);
                float tl[5];
                tl[0] = b.tau[0] * (aig[0] + a0a[0]);
                tl[1] = b.tau[1] * (aig[1] + a0a[1]);
                tl[2] = b.tau[1] * (aig[2] + a0a[2]);
                tl[3] = b.tau[1] * (aig[3] + a0a[3]);
                tl[4] = b.tau[2] * (aig[4] + a0a[4]);
                float F[3][5];
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 5; ++k) F[i][k] = 0.f;
                if (Pf.navier) {
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
#pragma unroll
                        for (int j = 0; j < 3; ++j) F[i][1 + j] = vs.t[i][j];
                        F[i][4] = b.u[0] * vs.t[i][0] + b.u[1] * vs.t[i][1] + b.u[2] * vs.t[i][2] + vs.q[i];
                    }
                }
                add_ai_v(b, tl, F);
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 5; ++k) S32[i][k] += F[i][k];
            }
        }
        // ---- FP64: metrics, Euler flux and time term ----
        double xl[4][3], yl[4][5];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
            for (int d = 0; d < 3; ++d) xl[a][d] = sx[3 * nd[a] + d];
            lds5(sy, nd[a], yl[a]);
        }
        Geo<double> geo;
        geometry(xl, geo);
        double S[3][5], Tn[4][5];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k) S[i][k] = (double)S32[i][k];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k) Tn[a][k] = 0.0;
#pragma unroll 1
        for (int q = 0; q < 4; ++q) {
            double N[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) N[a] = shp<double>(q, a);
            double bq[5], aq[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                bq[k] = N[0] * yl[0][k] + N[1] * yl[1][k] + N[2] * yl[2][k] + N[3] * yl[3][k];
                aq[k] = N[0] * sa[5 * nd[0] + k] + N[1] * sa[5 * nd[1] + k] + N[2] * sa[5 * nd[2] + k] +
                        N[3] * sa[5 * nd[3] + k];
            }
            const double p = bq[0], u0 = bq[1], u1 = bq[2], u2 = bq[3], T = bq[4];
            const double rT = 1.0 / T;
            const double drdp = P.rRgas * rT;
            const double rho = p * drdp;
            const double drdT = -rho * rT;
            const double rk = 0.5 * (u0 * u0 + u1 * u1 + u2 * u2);
            const double hk = T * P.cp + rk;
            const double ek = T * P.cv + rk;
            const double e1p = drdp * hk - rT * T;
            const double e4p = drdT * hk + rho * P.cp;
            const double uu[3] = {u0, u1, u2};
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const double m = -uu[i] * rho;
                S[i][0] += m;
#pragma unroll
                for (int j = 0; j < 3; ++j) S[i][1 + j] += m * uu[j] - (i == j ? p : 0.0);
                S[i][4] += m * ek - uu[i] * p;
            }
            // A0 Y,t
            const double sA = drdp * aq[0] + drdT * aq[4];
            double a0a[5];
            a0a[0] = sA;
#pragma unroll
            for (int j = 0; j < 3; ++j) a0a[1 + j] = uu[j] * sA + rho * aq[1 + j];
            a0a[4] = e1p * aq[0] + rho * (u0 * aq[1] + u1 * aq[2] + u2 * aq[3]) + e4p * aq[4];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int k = 0; k < 5; ++k) Tn[a][k] += N[a] * a0a[k];
        }
        double* sl = slot + 20 * threadIdx.x;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k)
                sl[5 * a + k] = geo.WdetJ * (geo.shg[a][0] * S[0][k] + geo.shg[a][1] * S[1][k] +
                                             geo.shg[a][2] * S[2][k] + Tn[a][k]);
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        const int s0 = ca.cstart[n0 + l], s1 = ca.cstart[n0 + l + 1];
        for (int s = s0; s < s1; ++s) {
            const double* sl = slot + 5 * (int)ca.csr[s];
#pragma unroll
            for (int k = 0; k < 5; ++k) acc[k] += sl[k];
        }
        double* og = out + 5 * (size_t)ca.nodes[n0 + l];
#pragma unroll
        for (int k = 0; k < 5; ++k) og[k] += acc[k];
    }
}

// --------------------------------------------------------------------------
// outer residual (ires = 1) without FP64 arithmetic.  The Euler flux at a
// quadrature point is split exactly as F(y_q) = F(y_r) + [F(y_q) - F(y_r)],
// y_r the state of the element's local node 3:
//   * F(y_r) is constant over the element, so its weighted sum over the four
//     points is 4 F(y_r) WdetJ shg_a = (Qwt/2) cof'_a F(y_r), cof'_a the
//     cofactors of the edge matrix x_j - x_3.  These terms are large and cancel
//     between the elements around a node; they are formed in double-float
//     arithmetic (df64.cuh) from hi/lo float copies of x and y.
//   * the increment is written with the exact expansions
//       rho - rho_r = (dp T_r - p_r dT) / (R T T_r),  m_i - m_ri = drho u_i + rho_r du_i,
//       m_i u_j - m_ri u_rj = dm_i u_j + m_ri du_j, ...
//     of increments dy = y_q - y_r formed from the hi/lo copies, so FP32
//     evaluates it to FP32 accuracy relative to its own (small) size.
// The time term (e3massr.f:26-58), the least-squares term (e3ls.f) and the
// viscous flux (e3visc.f) are FP32, as in k_chunk_resh.  Slots and node sums
// are double-float; each node's sum is added to the FP64 output.
// --------------------------------------------------------------------------
struct DfConst {
    float rRgas_hi, rRgas_lo, cv_hi, cv_lo, wq_hi, wq_lo;  // 1/R, R/(gamma-1), Qwt/2
};

constexpr int kSplitSlot = 40;  // per element: 20 hi then 20 lo


// one element of the split outer residual: its four nodal contributions as double-float
// hi/lo pairs in its slot sl (kSplitSlot floats), from the chunk's staged node data
template <bool WITH_Q>
__device__ __forceinline__ void ress_element(const ushort4 ln, const float* __restrict__ sxh,
                                             const float* __restrict__ sxl, const float* __restrict__ syh,
                                             const float* __restrict__ syl, const float* __restrict__ sa,
                                             const float* __restrict__ sq, float* __restrict__ sl,
                                             const Phys<float>& Pf, const DfConst& K) {
    const int nd[4] = {ln.x, ln.y, ln.z, ln.w};
    float o32[4][5];
    {
        float xl[4][3], yl[4][5], al[4][5], dl[3][5];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
            for (int d = 0; d < 3; ++d) xl[a][d] = sxh[3 * nd[a] + d];
            lds5(syh, nd[a], yl[a]);
            lds5(sa, nd[a], al[a]);
        }
        // increments from local node 3, from the hi and lo parts
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k)
                dl[a][k] = (yl[a][k] - yl[3][k]) + (syl[5 * nd[a] + k] - syl[5 * nd[3] + k]);
        Geo<float> geo;
        geometry(xl, geo);
        // gradients from the increments (sum_a shg_a = 0): differences of nearby nodal
        // values keep their own FP32 accuracy instead of that of the values
        float g[3][5];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k)
                g[i][k] = geo.shg[0][i] * dl[0][k] + geo.shg[1][i] * dl[1][k] + geo.shg[2][i] * dl[2][k];
        Visc<float> vs;
        if (Pf.navier) viscous(Pf, g, vs);
        float divq[4] = {0.f, 0.f, 0.f, 0.f};  // idiff = 1 (e3ivar.f:374-395)
        if (WITH_Q) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float acc = 0.f;
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const float* q = sq + 12 * nd[a];
                    acc += geo.shg[a][0] * q[k] + geo.shg[a][1] * q[4 + k] + geo.shg[a][2] * q[8 + k];
                }
                divq[k] = acc;
            }
        }
        const float pr = yl[3][0], Tr = yl[3][4];
        const float ur[3] = {yl[3][1], yl[3][2], yl[3][3]};
        const float rhor = pr * Pf.rRgas / Tr;
        const float mr[3] = {rhor * ur[0], rhor * ur[1], rhor * ur[2]};
        float S32[3][5], T32[4][5];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k) S32[i][k] = 0.f;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k) T32[a][k] = 0.f;
#pragma unroll 1
        for (int q = 0; q < 4; ++q) {
            float N[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) N[a] = shp<float>(q, a);
            float bq[5], aq[5], dq[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                bq[k] = N[0] * yl[0][k] + N[1] * yl[1][k] + N[2] * yl[2][k] + N[3] * yl[3][k];
                aq[k] = N[0] * al[0][k] + N[1] * al[1][k] + N[2] * al[2][k] + N[3] * al[3][k];
                dq[k] = N[0] * dl[0][k] + N[1] * dl[1][k] + N[2] * dl[2][k];
            }
            Qp<float> b;
            qp_state(Pf, bq[0], bq[1], bq[2], bq[3], bq[4], b);
            qp_tau(Pf, geo, b);
            float aig[5], a0a[5];
            ai_gi(b, g, aig);
            a0_v(b, aq, a0a);
            float tl[5];
            tl[0] = b.tau[0] * (aig[0] + a0a[0]);
            tl[1] = b.tau[1] * (aig[1] + a0a[1] - divq[0]);
            tl[2] = b.tau[1] * (aig[2] + a0a[2] - divq[1]);
            tl[3] = b.tau[1] * (aig[3] + a0a[3] - divq[2]);
            tl[4] = b.tau[2] * (aig[4] + a0a[4] - divq[3]);
            float F[3][5];
            // Euler-flux increment F(y_q) - F(y_r) (flux sign of e3conv.f:72-96)
            const float drho = (dq[0] * Tr - pr * dq[4]) * Pf.rRgas / (Tr * b.T);
            const float dek = Pf.cv * dq[4] + (ur[0] * dq[1] + ur[1] * dq[2] + ur[2] * dq[3]) +
                              0.5f * (dq[1] * dq[1] + dq[2] * dq[2] + dq[3] * dq[3]);
            const float ek = b.ei + b.rk;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float dm = drho * b.u[i] + rhor * dq[1 + i];
                F[i][0] = -dm;
#pragma unroll
                for (int j = 0; j < 3; ++j) F[i][1 + j] = -(dm * b.u[j] + mr[i] * dq[1 + j]) - (i == j ? dq[0] : 0.f);
                F[i][4] = -(dm * ek + mr[i] * dek) - (dq[1 + i] * b.p + ur[i] * dq[0]);
            }
            if (Pf.navier) {
#pragma unroll
                for (int i = 0; i < 3; ++i) {
#pragma unroll
                    for (int j = 0; j < 3; ++j) F[i][1 + j] += vs.t[i][j];
                    F[i][4] += b.u[0] * vs.t[i][0] + b.u[1] * vs.t[i][1] + b.u[2] * vs.t[i][2] + vs.q[i];
                }
            }
            add_ai_v(b, tl, F);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 5; ++k) S32[i][k] += F[i][k];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int k = 0; k < 5; ++k) T32[a][k] += N[a] * a0a[k];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k)
                o32[a][k] = geo.WdetJ * (geo.shg[a][0] * S32[0][k] + geo.shg[a][1] * S32[1][k] +
                                         geo.shg[a][2] * S32[2][k] + T32[a][k]);
    }
    // ---- element-constant flux F(y_r) (double-float) ----
    const int r = nd[3];
    const df64 p = df_make(syh[5 * r + 0], syl[5 * r + 0]);
    const df64 u[3] = {df_make(syh[5 * r + 1], syl[5 * r + 1]), df_make(syh[5 * r + 2], syl[5 * r + 2]),
                       df_make(syh[5 * r + 3], syl[5 * r + 3])};
    const df64 T = df_make(syh[5 * r + 4], syl[5 * r + 4]);
    const df64 rho = df_mul(p, df_mul(df_make(K.rRgas_hi, K.rRgas_lo), df_rcp(T)));
    df64 rk = df_add(df_add(df_mul(u[0], u[0]), df_mul(u[1], u[1])), df_mul(u[2], u[2]));
    rk.hi *= 0.5f;
    rk.lo *= 0.5f;
    const df64 ek = df_add(df_mul(df_make(K.cv_hi, K.cv_lo), T), rk);
    df64 F[3][5];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const df64 m = df_mul(rho, u[i]);
        F[i][0] = df_neg(m);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            F[i][1 + j] = df_neg(df_mul(m, u[j]));
            if (i == j) F[i][1 + j] = df_sub(F[i][1 + j], p);
        }
        F[i][4] = df_neg(df_add(df_mul(m, ek), df_mul(u[i], p)));
    }
    // cofactors of the edge matrix d'[i][j] = x_j,i - x_3,i (the geometry() layout)
    df64 d[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            d[i][j] = df_diff(sxh[3 * nd[j] + i], sxl[3 * nd[j] + i], sxh[3 * r + i], sxl[3 * r + i]);
    auto minor2 = [](df64 a, df64 b, df64 c2, df64 e) { return df_sub(df_mul(a, b), df_mul(c2, e)); };
    df64 cof[3][3];
    cof[0][0] = minor2(d[1][1], d[2][2], d[2][1], d[1][2]);
    cof[0][1] = minor2(d[2][1], d[0][2], d[0][1], d[2][2]);
    cof[0][2] = minor2(d[0][1], d[1][2], d[0][2], d[1][1]);
    cof[1][0] = minor2(d[1][2], d[2][0], d[1][0], d[2][2]);
    cof[1][1] = minor2(d[0][0], d[2][2], d[2][0], d[0][2]);
    cof[1][2] = minor2(d[1][0], d[0][2], d[0][0], d[1][2]);
    cof[2][0] = minor2(d[1][0], d[2][1], d[1][1], d[2][0]);
    cof[2][1] = minor2(d[2][0], d[0][1], d[0][0], d[2][1]);
    cof[2][2] = minor2(d[0][0], d[1][1], d[0][1], d[1][0]);
    const df64 wq = df_make(K.wq_hi, K.wq_lo);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i) cof[a][i] = df_mul(cof[a][i], wq);
    df64 s3[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) s3[k] = df_make(0.f, 0.f);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const df64 g64 = df_add(df_add(df_mul(cof[a][0], F[0][k]), df_mul(cof[a][1], F[1][k])),
                                    df_mul(cof[a][2], F[2][k]));
            s3[k] = df_add(s3[k], g64);
            const df64 v = df_add(g64, o32[a][k]);
            sl[5 * a + k] = v.hi;
            sl[20 + 5 * a + k] = v.lo;
        }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const df64 v = df_add(df_neg(s3[k]), o32[3][k]);  // shg_3 = -(shg_0 + shg_1 + shg_2)
        sl[15 + k] = v.hi;
        sl[35 + k] = v.lo;
    }
}

template <bool WITH_Q>
__global__ void __launch_bounds__(kChunk, PHGPU_RESS_MINB)
k_chunk_ress(ChunkArgs ca, int chunk0, const float* __restrict__ xh, const float* __restrict__ xlo,
             const float* __restrict__ yh, const float* __restrict__ ylo, const float* __restrict__ acf,
             double* __restrict__ out, Phys<float> Pf, DfConst K, const float* __restrict__ ql) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sm = reinterpret_cast<float*>(smem_raw);
    const int c = chunk0 + blockIdx.x;
    const int e0 = ca.elem[c], ne = ca.elem[c + 1] - e0;
    const int n0 = ca.node[c], nn = ca.node[c + 1] - n0;
    float* sxh = sm;
    float* sxl = sxh + 3 * nn;
    float* syh = sxl + 3 * nn;
    float* syl = syh + 5 * nn;
    float* sa = syl + 5 * nn;
    float* sq = sa + 5 * nn;              // idiff = 1: reconstructed flux, 12 per node
    float* slot = sq + (WITH_Q ? 12 * nn : 0);
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        const size_t gn = ca.nodes[n0 + l];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            sxh[3 * l + d] = __ldg(xh + 3 * gn + d);
            sxl[3 * l + d] = __ldg(xlo + 3 * gn + d);
        }
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            syh[5 * l + k] = __ldg(yh + 5 * gn + k);
            syl[5 * l + k] = __ldg(ylo + 5 * gn + k);
            sa[5 * l + k] = __ldg(acf + 5 * gn + k);
        }
        if (WITH_Q)
            for (int k = 0; k < 12; ++k) sq[12 * l + k] = __ldg(ql + 13 * gn + k);
    }
    __syncthreads();
    if ((int)threadIdx.x < ne)
        ress_element<WITH_Q>(ca.lien[e0 + threadIdx.x], sxh, sxl, syh, syl, sa, sq, slot + kSplitSlot * threadIdx.x,
                             Pf, K);
    __syncthreads();
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        df64 acc[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) acc[k] = df_make(0.f, 0.f);
        const int s0 = ca.cstart[n0 + l], s1 = ca.cstart[n0 + l + 1];
        for (int s = s0; s < s1; ++s) {
            const int sid = (int)ca.csr[s];
            const float* sl = slot + kSplitSlot * (sid >> 2) + 5 * (sid & 3);
#pragma unroll
            for (int k = 0; k < 5; ++k) acc[k] = df_add(acc[k], df_make(sl[k], sl[20 + k]));
        }
        double* og = out + 5 * (size_t)ca.nodes[n0 + l];
#pragma unroll
        for (int k = 0; k < 5; ++k) og[k] += df_to_double(acc[k]);
    }
}

// The split outer residual over the chunks of one colour, pipelined like k_chunk_lin_pipe:
// node ids two chunks ahead, the nodal data (hi/lo coordinates and state, FP32 ac, the
// reconstructed flux, the residual's current FP64 values), connectivity and slot lists one
// chunk ahead, by cp.async; arithmetic and summation order of k_chunk_ress.
constexpr int kRessNode = 21;  // staged floats per node: x hi/lo (6), y hi/lo (10), ac (5)

__host__ __device__ constexpr int ress_stage_words(int lmax, bool with_q) {
    // FP64 product values first (8-byte aligned), then the float data, then the indices
    return ((((10 * lmax + kRessNode * lmax + (with_q ? 12 * lmax : 0) + 1) & ~1) + 4 * kChunk + lmax + 2) + 1) & ~1;
}

template <bool WITH_Q, int MINB>
__global__ void __launch_bounds__(kChunk, MINB)
k_chunk_ress_pipe(ChunkArgs ca, int chunk0, int nch, const float* __restrict__ xh, const float* __restrict__ xlo,
                  const float* __restrict__ yh, const float* __restrict__ ylo, const float* __restrict__ acf,
                  double* __restrict__ out, Phys<float> Pf, DfConst K, const float* __restrict__ ql, int lmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sm = reinterpret_cast<float*>(smem_raw);
    const int per = ress_stage_words(lmax, WITH_Q);
    const int fw = 10 * lmax;                                   // floats start after the doubles
    const int lie_off = (fw + kRessNode * lmax + (WITH_Q ? 12 * lmax : 0) + 1) & ~1;
    int* ids = reinterpret_cast<int*>(sm + 2 * per);
    const int idw = lin_id_words(lmax);
    float* slot = sm + 2 * per + 3 * idw;
    auto stage_ids = [&](int c, int ib) {
        int* h = ids + ib * idw;
        const int n0 = ca.node[c], nn = ca.node[c + 1] - n0;
        if (threadIdx.x == 0) {
            const int e0 = ca.elem[c];
            h[0] = e0;
            h[1] = ca.elem[c + 1] - e0;
            h[2] = n0;
            h[3] = nn;
        }
        for (int l = threadIdx.x; l < nn; l += blockDim.x) cp_async4(h + 4 + l, ca.nodes + n0 + l);
    };
    auto stage_data = [&](int ib, float* b) {
        const int* h = ids + ib * idw;
        const int e0 = h[0], ne = h[1], n0 = h[2], nn = h[3];
        double* so = reinterpret_cast<double*>(b);
        float* sxh = b + fw;
        float* sxl = sxh + 3 * lmax;
        float* syh = sxl + 3 * lmax;
        float* syl = syh + 5 * lmax;
        float* sa = syl + 5 * lmax;
        float* sq = sa + 5 * lmax;
        float* sl = b + lie_off;
        float* sc = sl + 2 * kChunk;
        float* st = sc + 2 * kChunk;
        const unsigned* csr_w = reinterpret_cast<const unsigned*>(ca.csr) + 2 * (size_t)e0;
        for (int i = threadIdx.x; i < ne; i += blockDim.x) {
            const unsigned s8 = (unsigned)__cvta_generic_to_shared(sl + 2 * i);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s8), "l"(ca.lien + e0 + i) : "memory");
        }
        for (int w = threadIdx.x; w < 2 * ne; w += blockDim.x) cp_async4(sc + w, csr_w + w);
        for (int l = threadIdx.x; l <= nn; l += blockDim.x) cp_async4(st + l, ca.cstart + n0 + l);
        for (int l = threadIdx.x; l < nn; l += blockDim.x) {
            const size_t gn = (size_t)h[4 + l];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                cp_async4(sxh + 3 * l + d, xh + 3 * gn + d);
                cp_async4(sxl + 3 * l + d, xlo + 3 * gn + d);
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                cp_async4(syh + 5 * l + k, yh + 5 * gn + k);
                cp_async4(syl + 5 * l + k, ylo + 5 * gn + k);
                cp_async4(sa + 5 * l + k, acf + 5 * gn + k);
                const unsigned s8 = (unsigned)__cvta_generic_to_shared(so + 5 * l + k);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s8), "l"(out + 5 * gn + k) : "memory");
            }
            if (WITH_Q)
                for (int k = 0; k < 12; ++k) cp_async4(sq + 12 * l + k, ql + 13 * gn + k);
        }
    };
    const int cend = chunk0 + nch, G = gridDim.x;
    int c = chunk0 + blockIdx.x;
    if (c >= cend) return;
    stage_ids(c, 0);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    stage_data(0, sm);
    if (c + G < cend) stage_ids(c + G, 1);
    cp_async_commit();
    for (int it = 0; c < cend; c += G, ++it) {
        cp_async_wait<0>();
        __syncthreads();
        const int cn = c + G;
        if (cn < cend) stage_data((it + 1) % 3, sm + ((it + 1) & 1) * per);
        if (cn + G < cend) stage_ids(cn + G, (it + 2) % 3);
        cp_async_commit();
        const float* cur = sm + (it & 1) * per;
        const int* h = ids + (it % 3) * idw;
        const int e0 = h[0], ne = h[1], nn = h[3];
        const double* so = reinterpret_cast<const double*>(cur);
        const float* sxh = cur + fw;
        const float* sxl = sxh + 3 * lmax;
        const float* syh = sxl + 3 * lmax;
        const float* syl = syh + 5 * lmax;
        const float* sa = syl + 5 * lmax;
        const float* sq = sa + 5 * lmax;
        const ushort4* slie = reinterpret_cast<const ushort4*>(cur + lie_off);
        const unsigned short* scsr = reinterpret_cast<const unsigned short*>(cur + lie_off + 2 * kChunk);
        const int* scst = reinterpret_cast<const int*>(cur + lie_off + 4 * kChunk);
        if ((int)threadIdx.x < ne)
            ress_element<WITH_Q>(slie[threadIdx.x], sxh, sxl, syh, syl, sa, sq, slot + kSplitSlot * threadIdx.x, Pf,
                                 K);
        __syncthreads();
        const int sbase = 4 * e0;
        // one thread per (chunk node, component), the node's slots in ascending order: the
        // double-float sums are spread over all four warps (one thread per node left three
        // quarters of the CTA waiting at the barrier)
        for (int p = threadIdx.x; p < 5 * nn; p += blockDim.x) {
            const int l = p / 5, k = p - 5 * l;
            df64 acc = df_make(0.f, 0.f);
            const int s0 = scst[l] - sbase, s1 = scst[l + 1] - sbase;
            for (int s = s0; s < s1; ++s) {
                const int sid = (int)scsr[s];
                const float* sl = slot + kSplitSlot * (sid >> 2) + 5 * (sid & 3) + k;
                acc = df_add(acc, df_make(sl[0], sl[20]));
            }
            out[5 * (size_t)h[4 + l] + k] = so[p] + df_to_double(acc);
        }
        // no barrier here: the next iteration's first barrier precedes every write of the slots,
        // of this data stage and of this id stage
    }
    cp_async_wait<0>();
}

// --------------------------------------------------------------------------
// ElmMFG interior (ires = 3, iprec = 1): res, rmes and BDiag of node a of one
// element; the quadrature-point state is evaluated by each of the four
// threads of an element.  35 outputs: res 0-4, rmes 5-9, BDiag 10-34.
// --------------------------------------------------------------------------
constexpr int kFullOutAll = 35;  // res 0-4, rmes 5-9, BDiag 10-34
constexpr int kFullSub = kChunk / 4;  // elements per sub-batch (4 threads each)
template <typename R> constexpr int full_nsub() { return sizeof(R) == 4 ? 4 : 1; }

// Lanes 4e..4e+3 of a warp hold one element; lane a evaluates quadrature
// point q = a once and the four lanes exchange the point data by shuffles.
constexpr int kQpVals = 25;  // u(3) p rho ek drdp drdT e1p e2p e3p e4p tau(3) A_i Y,i (5) A0 Y,t (5)

// BD_ONLY: BDiag alone (the mixed-precision preconditioner), 25 outputs: no gradients,
// viscous stress or residual terms, and 15 shuffled point values instead of 25
template <typename R, bool BD_ONLY = false>
__device__ __forceinline__ void elem_full_node(const Phys<R>& P, int a, const R (&xl)[4][3], const R (&yl)[4][5],
                                               const R (&al)[4][5], R* __restrict__ out35,
                                               const R* divq = nullptr) {
    constexpr int NV = BD_ONLY ? 15 : kQpVals;
    Geo<R> geo;
    geometry(xl, geo);
    R g[3][5];
    Visc<R> vs;
    if constexpr (!BD_ONLY) {
        gradients(geo, yl, g);
        if (P.navier) viscous(P, g, vs);
    }
    R s[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) s[i] = (a == 0) ? geo.shg[0][i] : (a == 1) ? geo.shg[1][i] : (a == 2) ? geo.shg[2][i] : geo.shg[3][i];
    const R ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    R sv[3] = {R(0), R(0), R(0)}, sq = R(0);
    if (!BD_ONLY && P.navier) {
#pragma unroll
        for (int j = 0; j < 3; ++j) sv[j] = s[0] * vs.t[0][j] + s[1] * vs.t[1][j] + s[2] * vs.t[2][j];
        sq = s[0] * vs.q[0] + s[1] * vs.q[1] + s[2] * vs.q[2];
    }
    // this lane's quadrature point (q = a)
    R own[NV];
    R odc[16];  // discontinuity capturing at this point: DC and g^ij A0 Y,j (FP64, iDC != 0)
    {
        R N[4];
#pragma unroll
        for (int n = 0; n < 4; ++n) N[n] = shp<R>(a, n);
        R yq[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) yq[k] = N[0] * yl[0][k] + N[1] * yl[1][k] + N[2] * yl[2][k] + N[3] * yl[3][k];
        Qp<R> b;
        qp_state(P, yq[0], yq[1], yq[2], yq[3], yq[4], b);
        qp_tau(P, geo, b);
        own[0] = b.u[0]; own[1] = b.u[1]; own[2] = b.u[2]; own[3] = b.p; own[4] = b.rho; own[5] = b.ei + b.rk;
        own[6] = b.drdp; own[7] = b.drdT; own[8] = b.e1p; own[9] = b.e2p; own[10] = b.e3p; own[11] = b.e4p;
        own[12] = b.tau[0]; own[13] = b.tau[1]; own[14] = b.tau[2];
        if constexpr (!BD_ONLY) {
            R aq[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) aq[k] = N[0] * al[0][k] + N[1] * al[1][k] + N[2] * al[2][k] + N[3] * al[3][k];
            R aig[5], a0a[5];
            ai_gi(b, g, aig);
            a0_v(b, aq, a0a);
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                own[15 + k] = aig[k];
                own[20 + k] = a0a[k];
            }
            if constexpr (sizeof(R) == 8) {
                if (P.idc) {
                    const R tkk[5] = {b.tau[0], b.tau[1], b.tau[1], b.tau[1], b.tau[2]};
                    R ly[5], lt[5], gA[3][5];
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        ly[k] = aig[k] + a0a[k] - ((divq && k > 0) ? divq[k - 1] : R(0));
                        lt[k] = tkk[k] * ly[k];
                    }
                    odc[0] = dc_point(P, geo.G, b, g, ly, lt, gA);
#pragma unroll
                    for (int i = 0; i < 3; ++i)
#pragma unroll
                        for (int k = 0; k < 5; ++k) odc[1 + 5 * i + k] = gA[i][k];
                }
            }
        }
    }
    R rl[5], rml[5], B_[5][5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        rl[k] = R(0);
        rml[k] = R(0);
#pragma unroll
        for (int j = 0; j < 5; ++j) B_[k][j] = R(0);
    }
    const int base_lane = (threadIdx.x & 31) & ~3;
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        R v[kQpVals];
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] = __shfl_sync(0xffffffffu, own[i], base_lane + q);
        const R Na = shp<R>(q, a);
        const R u0 = v[0], u1 = v[1], u2 = v[2], p = v[3], rho = v[4], ek = v[5];
        const R drdp = v[6], drdT = v[7], e1p = v[8], e2p = v[9], e3p = v[10], e4p = v[11];
        const R tk[5] = {v[12], v[13], v[13], v[13], v[14]};
        const R uu[3] = {u0, u1, u2};
        const R Us = s[0] * u0 + s[1] * u1 + s[2] * u2;
        R Bm[5][5];
        Bm[0][0] = drdp * Us;
        Bm[0][4] = drdT * Us;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Bm[0][1 + j] = rho * s[j];
            Bm[1 + j][0] = drdp * Us * uu[j] + s[j];
            Bm[1 + j][4] = drdT * Us * uu[j];
#pragma unroll
            for (int k = 0; k < 3; ++k) Bm[1 + j][1 + k] = rho * (uu[j] * s[k] + (j == k ? Us : R(0)));
            Bm[4][1 + j] = e3p * s[j] + rho * Us * uu[j];
        }
        Bm[4][0] = e2p * Us;
        Bm[4][4] = e4p * Us;
        if constexpr (!BD_ONLY) {
            R lt[5], lm[5], rm16[5];
            const R du[5] = {rho, rho * u0, rho * u1, rho * u2, rho * ek};
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                rm16[k] = v[15 + k] + P.fct1 * du[k];
                const R dq = (divq && k > 0) ? divq[k - 1] : R(0);  // idiff = 1 (e3ls.f:147-156)
                lt[k] = tk[k] * (v[15 + k] + v[20 + k] - dq);
                lm[k] = tk[k] * rm16[k];
            }
            if constexpr (sizeof(R) == 8) {
                // discontinuity capturing: both residuals gain s_a . DC gA; the modified
                // residual's z-flux of continuity is the reference's rmi(:,11) = rmi(:,12) +
                // DC gA(:,12) (e3dc.f:366), the z-flux of x-momentum plus its DC part
                if (P.idc) {
                    R dq[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) dq[i] = __shfl_sync(0xffffffffu, odc[i], base_lane + q);
                    const R dc = dq[0];
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        const R f = dc * (s[0] * dq[1 + k] + s[1] * dq[6 + k] + s[2] * dq[11 + k]);
                        rl[k] += f;
                        rml[k] += f;
                    }
                    const R sz = drdp * lm[0] + drdT * lm[4];
                    const R z0 = u2 * sz + rho * lm[3];
                    const R z1 = u0 * z0 + rho * u2 * lm[1] + (P.navier ? vs.t[2][0] : R(0));
                    rml[0] += s[2] * (z1 + dc * dq[12] - z0 - dc * dq[11]);
                }
            }
            R fe[5];
            const R m = -rho * Us;
            fe[0] = m;
#pragma unroll
            for (int j = 0; j < 3; ++j) fe[1 + j] = m * uu[j] - s[j] * p + sv[j];
            const R usv = u0 * sv[0] + u1 * sv[1] + u2 * sv[2] + sq;
            fe[4] = m * ek - Us * p + usv;
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                R bt = R(0), bm = R(0);
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    bt += Bm[r][k] * lt[k];
                    bm += Bm[r][k] * lm[k];
                }
                const R fm = (r == 0) ? R(0) : (r == 4) ? usv : sv[r - 1];
                rl[r] += fe[r] + bt + Na * v[20 + r];
                rml[r] += fm + bm + Na * rm16[r];
            }
        }
        // BDiag: (N_a I + B_a tau)(B_a + fct N_a A0) + K_a
        const R fN = P.fct1 * Na;
        R Cm[5][5];
#pragma unroll
        for (int r = 0; r < 5; ++r)
#pragma unroll
            for (int k = 0; k < 5; ++k) Cm[r][k] = Bm[r][k];
        Cm[0][0] += fN * drdp;
        Cm[0][4] += fN * drdT;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Cm[1 + j][0] += fN * drdp * uu[j];
            Cm[1 + j][1 + j] += fN * rho;
            Cm[1 + j][4] += fN * drdT * uu[j];
            Cm[4][1 + j] += fN * rho * uu[j];
        }
        Cm[4][0] += fN * e1p;
        Cm[4][4] += fN * e4p;
        if (P.supg) {
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                R D[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) D[k] = Bm[r][k] * tk[k] + (r == k ? Na : R(0));
#pragma unroll
                for (int cc = 0; cc < 5; ++cc) {
                    R acc = R(0);
#pragma unroll
                    for (int k = 0; k < 5; ++k) acc += D[k] * Cm[k][cc];
                    B_[r][cc] += acc;
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < 5; ++r)
#pragma unroll
                for (int cc = 0; cc < 5; ++cc) B_[r][cc] += Na * Cm[r][cc];
        }
        if (P.navier) {
            R km[3][3];
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) km[j][k] = P.rlmpmu * s[j] * s[k] + (j == k ? P.rmu * ss : R(0));
#pragma unroll
            for (int j = 0; j < 3; ++j) {
#pragma unroll
                for (int k = 0; k < 3; ++k) B_[1 + j][1 + k] += km[j][k];
                B_[4][1 + j] += km[j][0] * u0 + km[j][1] * u1 + km[j][2] * u2;
            }
            B_[4][4] += P.con * ss;
        }
    }
    const R w = geo.WdetJ;
    constexpr int o0 = BD_ONLY ? 0 : 10;
    if constexpr (!BD_ONLY) {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            out35[k] = w * rl[k];
            out35[5 + k] = w * rml[k];
        }
    }
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
        for (int cc = 0; cc < 5; ++cc) out35[o0 + 5 * r + cc] = w * B_[r][cc];
}

template <typename R, bool BD_ONLY>
__global__ void __launch_bounds__(kChunk, sizeof(R) == 4 ? (BD_ONLY ? PHGPU_FULL32BD_MINB : PHGPU_FULL32_MINB) : 2)
k_chunk_full(ChunkArgs ca, int chunk0, const R* __restrict__ x, const R* __restrict__ y, const R* __restrict__ ac,
             R* __restrict__ res, R* __restrict__ rmes, R* __restrict__ bd, Phys<R> P,
             const R* __restrict__ ql = nullptr, const float4* __restrict__ xb = nullptr) {
    constexpr int kFullOut = BD_ONLY ? 25 : kFullOutAll;  // values per slot: BDiag, or res rmes BDiag
    constexpr int kBd = BD_ONLY ? 0 : 10;                    // offset of BDiag in a slot
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sm = reinterpret_cast<R*>(smem_raw);
    const int c = chunk0 + blockIdx.x;
    const int e0 = ca.elem[c], ne = ca.elem[c + 1] - e0;
    const int n0 = ca.node[c], nn = ca.node[c + 1] - n0;
    const bool with_q = ql != nullptr && res != nullptr;
    R* sx = sm;
    R* sy = sx + 3 * nn;
    R* sa = sy + 5 * nn;
    R* sq = sa + 5 * nn;                          // idiff = 1: 12 per node
    constexpr bool single = kFullSub * full_nsub<R>() >= kChunk;
    R* acc = sq + (with_q ? 12 * nn : 0);         // nn x 35 (multi-round only)
    R* slot = acc + (single ? 0 : kFullOut * nn); // (kChunk * nsub) x 35
    // the connectivity of this thread's tet in each sub-batch of the first round, loaded
    // before the staging so that its latency overlaps it
    ushort4 lnp[4];
#pragma unroll
    for (int sb = 0; sb < 4; ++sb) {
        const int el = min(sb * kFullSub + (int)(threadIdx.x >> 2), ne - 1);
        if (sb < full_nsub<R>()) lnp[sb] = ca.lien[e0 + el];
    }
    // FP32 block diagonal alone: the state and coordinates packed per node (yb0..yb4, x0, x1,
    // x2) when given, two 16-byte loads per node
    bool packed = false;
    if constexpr (BD_ONLY && sizeof(R) == 4) {
        if (xb) {
            packed = true;
            for (int l = threadIdx.x; l < nn; l += blockDim.x) {
                const size_t gn = (size_t)ca.nodes[n0 + l];
                const float4 p0 = __ldg(xb + 2 * gn), p1 = __ldg(xb + 2 * gn + 1);
                sy[5 * l + 0] = p0.x;
                sy[5 * l + 1] = p0.y;
                sy[5 * l + 2] = p0.z;
                sy[5 * l + 3] = p0.w;
                sy[5 * l + 4] = p1.x;
                sx[3 * l + 0] = p1.y;
                sx[3 * l + 1] = p1.z;
                sx[3 * l + 2] = p1.w;
            }
        }
    }
    if (!packed)
        for (int l = threadIdx.x; l < nn; l += blockDim.x) {
            const int gn = ca.nodes[n0 + l];
#pragma unroll
            for (int d = 0; d < 3; ++d) sx[3 * l + d] = ldg(x + 3 * (size_t)gn + d);
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                sy[5 * l + k] = ldg(y + 5 * (size_t)gn + k);
                if (!BD_ONLY) sa[5 * l + k] = ldg(ac + 5 * (size_t)gn + k);  // the block diagonal needs no ac
            }
            if (with_q)
                for (int k = 0; k < 12; ++k) sq[12 * l + k] = ldg(ql + 13 * (size_t)gn + k);
        }
    if (!single)
        for (int i = threadIdx.x; i < kFullOut * nn; i += blockDim.x) acc[i] = R(0);
    // FP32: the whole chunk is computed before one accumulation round;
    // FP64: one sub-batch per round (bounded shared memory)
    constexpr int nsub = full_nsub<R>();
    for (int b0 = 0; b0 < ne; b0 += kFullSub * nsub) {
        __syncthreads();
#pragma unroll 1
        for (int sb = 0; sb < nsub; ++sb) {
            const int el_raw = b0 + sb * kFullSub + (threadIdx.x >> 2), a = threadIdx.x & 3;
            const bool valid = el_raw < ne;
            const int el = valid ? el_raw : ne - 1;  // every lane takes part in the shuffles
            const ushort4 ln = b0 > 0 ? ca.lien[e0 + el]
                               : sb == 0 ? lnp[0] : sb == 1 ? lnp[1] : sb == 2 ? lnp[2] : lnp[3];
            const int nd[4] = {ln.x, ln.y, ln.z, ln.w};
            R xl[4][3], yl[4][5], al[4][5];
#pragma unroll
            for (int n = 0; n < 4; ++n) {
#pragma unroll
                for (int d = 0; d < 3; ++d) xl[n][d] = sx[3 * nd[n] + d];
                lds5(sy, nd[n], yl[n]);
                if (BD_ONLY) {
#pragma unroll
                    for (int k = 0; k < 5; ++k) al[n][k] = R(0);
                } else {
                    lds5(sa, nd[n], al[n]);
                }
            }
            R o35[kFullOut];
            if (with_q) {
                R divq[4];
                tet_divq(xl, sq, nd, divq);
                elem_full_node<R, BD_ONLY>(P, a, xl, yl, al, o35, divq);
            } else {
                elem_full_node<R, BD_ONLY>(P, a, xl, yl, al, o35);
            }
            if (valid) {
                R* sl = slot + kFullOut * (sb * kChunk + threadIdx.x);
#pragma unroll
                for (int k = 0; k < kFullOut; ++k) sl[k] = o35[k];
            }
        }
        __syncthreads();
        const int lo = 4 * b0, hi = 4 * (b0 + kFullSub * nsub);
        if (kFullSub * nsub >= kChunk) {
            // single round: one thread per (chunk node, row of five slot values), the node's
            // slots in ascending order, straight into the global arrays (one thread per node left
            // most of the CTA waiting while 25 or 35 sums per node ran)
            constexpr int NR = kFullOut / 5;
            for (int p = threadIdx.x; p < NR * nn; p += blockDim.x) {
                const int l = p / NR, r = p - NR * l;
                const int s0 = ca.cstart[n0 + l], s1 = ca.cstart[n0 + l + 1];
                R t[5] = {R(0), R(0), R(0), R(0), R(0)};
                for (int s = s0; s < s1; ++s) {
                    const R* sl = slot + kFullOut * (int)ca.csr[s] + 5 * r;
#pragma unroll
                    for (int k = 0; k < 5; ++k) t[k] += sl[k];
                }
                const size_t gn = ca.nodes[n0 + l];
                R* dst;
                if (!BD_ONLY && r == 0) dst = res ? res + 5 * gn : nullptr;
                else if (!BD_ONLY && r == 1) dst = rmes ? rmes + 5 * gn : nullptr;
                else dst = bd ? bd + 25 * gn + 5 * (r - kBd / 5) : nullptr;
                if (dst) {
#pragma unroll
                    for (int k = 0; k < 5; ++k) dst[k] += t[k];
                }
            }
            return;
        }
        for (int l = threadIdx.x; l < nn; l += blockDim.x) {
            const int s0 = ca.cstart[n0 + l], s1 = ca.cstart[n0 + l + 1];
            R* ac_ = acc + kFullOut * l;
            for (int s = s0; s < s1; ++s) {
                const int j = ca.csr[s];
                if (j < lo || j >= hi) continue;
                const R* sl = slot + kFullOut * (j - lo);
#pragma unroll
                for (int k = 0; k < kFullOut; ++k) ac_[k] += sl[k];
            }
        }
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nn; l += blockDim.x) {
        const size_t gn = ca.nodes[n0 + l];
        const R* ac_ = acc + kFullOut * l;
        if (!BD_ONLY && res) {
#pragma unroll
            for (int k = 0; k < 5; ++k) res[5 * gn + k] += ac_[k];
        }
        if (!BD_ONLY && rmes) {
#pragma unroll
            for (int k = 0; k < 5; ++k) rmes[5 * gn + k] += ac_[5 + k];
        }
        if (bd) {
#pragma unroll
            for (int k = 0; k < 25; ++k) bd[25 * gn + k] += ac_[kBd + k];
        }
    }
}

// --------------------------------------------------------------------------
// boundary faces (e3b.f / e3bvar.f, ires = 3): one thread per boundary tet
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock)
k_boundary(const int4* __restrict__ ienb, const int* __restrict__ iBCB, const double* __restrict__ BCB,
           int ne, const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ res,
           Phys<double> P) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int4 nd4 = ienb[e];
    const int nd[4] = {nd4.x, nd4.y, nd4.z, nd4.w};
    double xl[4][3], yl[4][5];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int d = 0; d < 3; ++d) xl[a][d] = x[3 * (size_t)nd[a] + d];
        load5(y, nd[a], yl[a]);
    }
    const int flags = iBCB[e];
    Geo<double> geo;
    geometry(xl, geo);
    double g[3][5];
    gradients(geo, yl, g);
    Visc<double> vs;
    if (P.navier) viscous(P, g, vs);
    double v1[3], v2[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        v1[d] = xl[1][d] - xl[0][d];
        v2[d] = xl[2][d] - xl[0][d];
    }
    const double n0 = v1[1] * v2[2] - v2[1] * v1[2];
    const double n1 = v2[0] * v1[2] - v1[0] * v2[2];
    const double n2 = v1[0] * v2[1] - v2[0] * v1[1];
    const double area2 = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    const double rn = 1.0 / area2;
    const double bn[3] = {n0 * rn, n1 * rn, n2 * rn};
    double rl[3][5];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 5; ++k) rl[a][k] = 0.0;
    const double* bcb = BCB + 18 * (size_t)e;
#pragma unroll 1
    for (int q = 0; q < 3; ++q) {
        const double N0 = c_tab.shpb[q][0], N1 = c_tab.shpb[q][1], N2 = c_tab.shpb[q][2];
        double v[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] = N0 * yl[0][k] + N1 * yl[1][k] + N2 * yl[2][k];
        const double pres = v[0], u0 = v[1], u1 = v[2], u2 = v[3], T = v[4];
        const double rk = 0.5 * (u0 * u0 + u1 * u1 + u2 * u2);
        const double rho = pres / (P.Rgas * T);
        const double ei = T * P.cv;
        const double WdetJb = c_tab.Qwtb[q] * area2 * 0.25;
        double rou = N0 * bcb[0] + N1 * bcb[6] + N2 * bcb[12];
        double p = N0 * bcb[1] + N1 * bcb[7] + N2 * bcb[13];
        double Fv[3], Fh5;
        Fv[0] = N0 * bcb[2] + N1 * bcb[8] + N2 * bcb[14];
        Fv[1] = N0 * bcb[3] + N1 * bcb[9] + N2 * bcb[15];
        Fv[2] = N0 * bcb[4] + N1 * bcb[10] + N2 * bcb[16];
        Fh5 = N0 * bcb[5] + N1 * bcb[11] + N2 * bcb[17];
        double un;
        if (!(flags & 1)) {
            un = bn[0] * u0 + bn[1] * u1 + bn[2] * u2;
            rou = rho * un;
        } else {
            un = rou / rho;
        }
        if (!(flags & 2)) p = pres;
        double F[5];
        F[0] = rou;
        F[1] = rou * u0 + bn[0] * p;
        F[2] = rou * u1 + bn[1] * p;
        F[3] = rou * u2 + bn[2] * p;
        F[4] = rou * (ei + rk) + un * p;
        if (P.navier) {
            if (!(flags & 4)) {
#pragma unroll
                for (int j = 0; j < 3; ++j) Fv[j] = bn[0] * vs.t[0][j] + bn[1] * vs.t[1][j] + bn[2] * vs.t[2][j];
            }
            const double Fv5 = u0 * Fv[0] + u1 * Fv[1] + u2 * Fv[2];
            const double heat = -(bn[0] * vs.q[0] + bn[1] * vs.q[1] + bn[2] * vs.q[2]);
            if (!(flags & 8)) Fh5 = heat;
            F[1] -= Fv[0];
            F[2] -= Fv[1];
            F[3] -= Fv[2];
            F[4] = F[4] - Fv5 + Fh5;
        }
        const double Nq[3] = {N0, N1, N2};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k) rl[a][k] += WdetJb * Nq[a] * F[k];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double* o = res + 5 * (size_t)nd[a];
#pragma unroll
        for (int k = 0; k < 5; ++k) o[k] += rl[a][k];
    }
}

// --------------------------------------------------------------------------
// hex and wedge blocks (lcsyst 2 and 3, linear basis).  One thread per
// (element, node); the linear rules have as many points as nodes, so thread a
// of an element evaluates quadrature point q = a (metric e3metric.f, state
// e3ivar.f/getthm.f, tau e3tau.f with the dxidx^T dxidx metric of
// e3tau.f:1408-1425) and shares it in shared memory; then each thread sums
// its node's weighted terms over the points (e3wmlt.f, e3bdg.f) and adds
// them to the node.  Elements of one colour share no node.
// --------------------------------------------------------------------------
__constant__ TopoTabD c_topo[2];   // 0 hex, 1 wedge
__constant__ TopoTabF c_topof[2];

template <typename R> __device__ __forceinline__ R tshp(int t, int q, int a);
template <> __device__ __forceinline__ double tshp<double>(int t, int q, int a) { return c_topo[t].shp[q][a]; }
template <> __device__ __forceinline__ float tshp<float>(int t, int q, int a) { return c_topof[t].shp[q][a]; }
template <typename R> __device__ __forceinline__ R tshgl(int t, int q, int i, int a);
template <> __device__ __forceinline__ double tshgl<double>(int t, int q, int i, int a) { return c_topo[t].shgl[q][i][a]; }
template <> __device__ __forceinline__ float tshgl<float>(int t, int q, int i, int a) { return c_topof[t].shgl[q][i][a]; }
template <typename R> __device__ __forceinline__ R tqwt(int t, int q);
template <> __device__ __forceinline__ double tqwt<double>(int t, int q) { return c_topo[t].qwt[q]; }
template <> __device__ __forceinline__ float tqwt<float>(int t, int q) { return c_topof[t].qwt[q]; }

constexpr int kTopoThreads = 128;
enum TopoMode : int { TM_RES = RM_RES, TM_MODRES = RM_MODRES, TM_LIN = RM_LIN, TM_FULL = 4, TM_QREC = 5 };
constexpr int kTopoNode = 25;  // staged per node: x(3) ya(5) yb(5) reconstructed flux(12)
// the FP32 linearized and modified residuals read no reconstructed flux, no conservative
// variables and no DC terms: a lean layout (13 values per node, the point values up to kDu)
// lets a fifth CTA per SM fit in shared memory
template <typename R, int MODE>
constexpr bool topo_lean() { return sizeof(R) == 4 && (MODE == RM_LIN || MODE == RM_MODRES); }
template <typename R, int MODE>
constexpr int topo_node() { return topo_lean<R, MODE>() ? 13 : kTopoNode; }

// shared values of one quadrature point (FP64 also holds the discontinuity-capturing terms)
template <int NEN, bool DC = false, bool LEAN = false>
struct TopoQp {
    static constexpr int kShg = 0;                  // shg[b][i], NEN*3
    static constexpr int kW = NEN * 3;              // WdetJ
    static constexpr int kU = kW + 1;               // u(3) p rho ek drdp drdT e1p e2p e3p e4p tau(3) = 15
    static constexpr int kAig = kU + 15;            // A_i Y,i (5)
    static constexpr int kA0 = kAig + 5;            // A0 Y,t (res) / dU (modified, linear) (5)
    static constexpr int kVt = kA0 + 5;             // viscous stress t[i][j] (9)
    static constexpr int kVq = kVt + 9;             // heat flux (3)
    static constexpr int kDu = kVq + 3;             // conservative variables (full mode) (5)
    static constexpr int kDq = kDu + 5;             // div of the reconstructed flux (4)
    static constexpr int kDc = kDq + 4;             // DC and g^ij A0 Y,j (16, FP64)
    static constexpr int kN = LEAN ? kDu : kDc + (DC ? 16 : 0);
};

// resident CTAs per SM the lean variants are compiled for: their shared memory allows 6, which
// costs spills (80 registers); at 5 (96 registers, no spill) the mixed-topology Newton iteration
// takes 14.46 ms against 14.95 at 6, 15.06 uncapped (104 registers, 4 CTAs) and 14.78 with the
// full layout
#ifndef PHGPU_TOPO_LEAN_MINB
#define PHGPU_TOPO_LEAN_MINB 5
#endif
template <typename R, int MODE>
constexpr int topo_minb() { return topo_lean<R, MODE>() ? PHGPU_TOPO_LEAN_MINB : 1; }

template <typename R, int NEN, int TOPO, int MODE>
__global__ void __launch_bounds__(kTopoThreads, topo_minb<R, MODE>())
k_topo(const int* __restrict__ ien, int ne, const R* __restrict__ x, const R* __restrict__ ya,
       const R* __restrict__ yb, const R* __restrict__ ac, R* __restrict__ res, R* __restrict__ rmes,
       R* __restrict__ bd, Phys<R> P, int iabres, const int* __restrict__ skip, const R* __restrict__ ql,
       const float4* __restrict__ xbp = nullptr) {
    if (skip && *skip) return;
    constexpr bool LEAN = topo_lean<R, MODE>();
    constexpr int NS = topo_node<R, MODE>();  // staged values per node
    using Q = TopoQp<NEN, sizeof(R) == 8, LEAN>;
    constexpr int EPB = kTopoThreads / NEN;  // elements per CTA
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sm = reinterpret_cast<R*>(smem_raw);
    const int le = threadIdx.x / NEN, a = threadIdx.x % NEN;
    const int e = blockIdx.x * EPB + le;
    const bool active = le < EPB && e < ne;
    R* sx = sm + (size_t)le * NEN * NS;
    R* sq = sm + (size_t)EPB * NEN * NS + (size_t)le * NEN * Q::kN;
    const bool with_q = (MODE == TM_RES || MODE == TM_FULL) && ql != nullptr;
    int node = 0;
    if (active) {
        node = ien[(size_t)e * NEN + a];
        R* s = sx + NS * a;
        bool packed = false;
        if constexpr (LEAN) {
            if (xbp) {
                // the FP32 base state and coordinates packed per node: two 16-byte loads
                const float4 p0 = __ldg(xbp + 2 * (size_t)node), p1 = __ldg(xbp + 2 * (size_t)node + 1);
                s[8] = p0.x;
                s[9] = p0.y;
                s[10] = p0.z;
                s[11] = p0.w;
                s[12] = p1.x;
                s[0] = p1.y;
                s[1] = p1.z;
                s[2] = p1.w;
                packed = true;
            }
        }
        if (!packed) {
#pragma unroll
            for (int d = 0; d < 3; ++d) s[d] = ldg(x + 3 * (size_t)node + d);
        }
        const R* bsrc = (MODE == TM_RES || MODE == TM_FULL) ? ac : yb;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            s[3 + k] = ldg(ya + 5 * (size_t)node + k);
            if (MODE != TM_QREC && !packed) s[8 + k] = ldg(bsrc + 5 * (size_t)node + k);
        }
        if (with_q)
            for (int k = 0; k < 12; ++k) s[13 + k] = ldg(ql + 13 * (size_t)node + k);
    }
    __syncthreads();
    if (active) {
        // ---- quadrature point q = a: metric (e3metric.f:22-77) ----
        const int q = a;
        R dxdxi[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                R acc = R(0);
#pragma unroll
                for (int b = 0; b < NEN; ++b) acc += sx[NS * b + i] * tshgl<R>(TOPO, q, j, b);
                dxdxi[i][j] = acc;
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
        R* o = sq + Q::kN * q;
        o[Q::kW] = tqwt<R>(TOPO, q) / tmp;
        R g[3][5];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k) g[i][k] = R(0);
        R bq[5], pv[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) bq[k] = pv[k] = R(0);
        R aq[5] = {R(0), R(0), R(0), R(0), R(0)};
#pragma unroll
        for (int b = 0; b < NEN; ++b) {
            R sh[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                sh[i] = tshgl<R>(TOPO, q, 0, b) * di[0][i] + tshgl<R>(TOPO, q, 1, b) * di[1][i] +
                        tshgl<R>(TOPO, q, 2, b) * di[2][i];
                o[Q::kShg + 3 * b + i] = sh[i];
            }
            const R Nb = tshp<R>(TOPO, q, b);
            const R* s = sx + NS * b;
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const R va = s[3 + k];
#pragma unroll
                for (int i = 0; i < 3; ++i) g[i][k] += sh[i] * va;
                pv[k] += Nb * va;
                if (MODE == TM_RES || MODE == TM_FULL) aq[k] += Nb * s[8 + k];
                else if (MODE != TM_QREC) bq[k] += Nb * s[8 + k];
            }
            if (with_q)  // div q at this point (e3ivar.f:374-395)
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    o[Q::kDq + k] = (b == 0 ? R(0) : o[Q::kDq + k]) + sh[0] * s[13 + k] + sh[1] * s[17 + k] +
                                    sh[2] * s[21 + k];
        }
        if (MODE == TM_QREC) {
            // viscous flux of e3q.f at this point (the point's velocity enters the energy row)
            Visc<R> vq;
            viscous(P, g, vq);
            R qd[12];
            visc_flux12(P, vq, pv[1], pv[2], pv[3], qd);
#pragma unroll
            for (int k = 0; k < 12; ++k) o[Q::kVt + k] = qd[k];
        } else {
        if (MODE == TM_RES || MODE == TM_FULL) {
#pragma unroll
            for (int k = 0; k < 5; ++k) bq[k] = pv[k];
        }
        Qp<R> st;
        qp_state(P, bq[0], bq[1], bq[2], bq[3], bq[4], st);
        Geo<R> gm;  // only the metric of tau (e3tau.f:1408-1425)
        {
            auto gij = [&](int i, int j) { return di[0][i] * di[0][j] + di[1][i] * di[1][j] + di[2][i] * di[2][j]; };
            gm.G[0] = gij(0, 0);
            gm.G[1] = gij(0, 1);
            gm.G[2] = gij(1, 1);
            gm.G[3] = gij(0, 2);
            gm.G[4] = gij(1, 2);
            gm.G[5] = gij(2, 2);
            gm.GG = gm.G[0] * gm.G[0] + gm.G[2] * gm.G[2] + gm.G[5] * gm.G[5] +
                    R(2) * (gm.G[1] * gm.G[1] + gm.G[3] * gm.G[3] + gm.G[4] * gm.G[4]);
            gm.trG = gm.G[0] + gm.G[2] + gm.G[5];
        }
        qp_tau(P, gm, st);
        R aig[5], a0x[5];
        ai_gi(st, g, aig);
        if (MODE == TM_RES || MODE == TM_FULL) {
            a0_v(st, aq, a0x);
        } else if (MODE == TM_MODRES) {
            // conservative variables of the perturbed state (e3ivar.f:96-131)
            const R rho6 = pv[0] / (P.Rgas * pv[4]);
            const R rk6 = R(0.5) * (pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3]);
            a0x[0] = rho6;
            a0x[1] = rho6 * pv[1];
            a0x[2] = rho6 * pv[2];
            a0x[3] = rho6 * pv[3];
            a0x[4] = rho6 * (pv[4] * P.cv + rk6);
        } else {
            a0_v(st, pv, a0x);
        }
        Visc<R> vs;
        if (P.navier) viscous(P, g, vs);
        else {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                vs.q[i] = R(0);
#pragma unroll
                for (int j = 0; j < 3; ++j) vs.t[i][j] = R(0);
            }
        }
        R* ov = o + Q::kU;
        ov[0] = st.u[0];
        ov[1] = st.u[1];
        ov[2] = st.u[2];
        ov[3] = st.p;
        ov[4] = st.rho;
        ov[5] = st.ei + st.rk;
        ov[6] = st.drdp;
        ov[7] = st.drdT;
        ov[8] = st.e1p;
        ov[9] = st.e2p;
        ov[10] = st.e3p;
        ov[11] = st.e4p;
        ov[12] = st.tau[0];
        ov[13] = st.tau[1];
        ov[14] = st.tau[2];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            o[Q::kAig + k] = aig[k];
            o[Q::kA0 + k] = a0x[k];
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) {
#pragma unroll
            for (int j = 0; j < 3; ++j) o[Q::kVt + 3 * i + j] = vs.t[i][j];
            o[Q::kVq + i] = vs.q[i];
        }
        if constexpr (!LEAN) {
            const R du[5] = {st.rho, st.rho * st.u[0], st.rho * st.u[1], st.rho * st.u[2], st.rho * (st.ei + st.rk)};
#pragma unroll
            for (int k = 0; k < 5; ++k) o[Q::kDu + k] = du[k];
        }
        if constexpr (sizeof(R) == 8 && MODE != TM_LIN) {
            // discontinuity capturing (e3dc.f): rTLS pairs the least-squares residual with its
            // tau-scaled self for the residual, with itself for the modified residual
            if (P.idc) {
                R ly[5], lt[5], gA[3][5];
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    if (MODE == TM_MODRES) {
                        ly[k] = aig[k];
                        lt[k] = ly[k];
                    } else {
                        ly[k] = aig[k] + a0x[k] - ((with_q && k > 0) ? o[Q::kDq + k - 1] : R(0));
                        lt[k] = (k == 0 ? st.tau[0] : k == 4 ? st.tau[2] : st.tau[1]) * ly[k];
                    }
                }
                o[Q::kDc] = dc_point(P, gm.G, st, g, ly, lt, gA);
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 5; ++k) o[Q::kDc + 1 + 5 * i + k] = gA[i][k];
            }
        }
        }
    }
    __syncthreads();
    if (!active) return;
    if (MODE == TM_QREC) {
        // node a: sum_q N_a WdetJ qdi and the lumped mass (e3q.f:160-177)
        R qa[13];
#pragma unroll
        for (int k = 0; k < 13; ++k) qa[k] = R(0);
#pragma unroll 1
        for (int q = 0; q < NEN; ++q) {
            const R* v = sq + Q::kN * q;
            const R w = tshp<R>(TOPO, q, a) * v[Q::kW];
#pragma unroll
            for (int k = 0; k < 12; ++k) qa[k] += w * v[Q::kVt + k];
            qa[12] += w;
        }
        R* og = res + 13 * (size_t)node;
#pragma unroll
        for (int k = 0; k < 13; ++k) og[k] += qa[k];
        return;
    }
    // ---- node a: weighted terms summed over the points ----
    R rl[5], rml[5], B_[5][5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        rl[k] = rml[k] = R(0);
#pragma unroll
        for (int j = 0; j < 5; ++j) B_[k][j] = R(0);
    }
#pragma unroll 1
    for (int q = 0; q < NEN; ++q) {
        const R* v = sq + Q::kN * q;
        const R w = v[Q::kW];
        const R s[3] = {v[Q::kShg + 3 * a], v[Q::kShg + 3 * a + 1], v[Q::kShg + 3 * a + 2]};
        const R Na = tshp<R>(TOPO, q, a);
        const R* u = v + Q::kU;
        const R u0 = u[0], u1 = u[1], u2 = u[2], p = u[3], rho = u[4], ek = u[5];
        const R drdp = u[6], drdT = u[7], e1p = u[8], e2p = u[9], e3p = u[10], e4p = u[11];
        const R tk[5] = {u[12], u[13], u[13], u[13], u[14]};
        const R uu[3] = {u0, u1, u2};
        R sv[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) sv[j] = s[0] * v[Q::kVt + j] + s[1] * v[Q::kVt + 3 + j] + s[2] * v[Q::kVt + 6 + j];
        const R sqh = s[0] * v[Q::kVq] + s[1] * v[Q::kVq + 1] + s[2] * v[Q::kVq + 2];
        const R usv = u0 * sv[0] + u1 * sv[1] + u2 * sv[2] + sqh;
        const R Us = s[0] * u0 + s[1] * u1 + s[2] * u2;
        // B = sum_i s_i A_i (e3mtrx.f closed form)
        R Bm[5][5];
        Bm[0][0] = drdp * Us;
        Bm[0][4] = drdT * Us;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Bm[0][1 + j] = rho * s[j];
            Bm[1 + j][0] = drdp * Us * uu[j] + s[j];
            Bm[1 + j][4] = drdT * Us * uu[j];
#pragma unroll
            for (int k = 0; k < 3; ++k) Bm[1 + j][1 + k] = rho * (uu[j] * s[k] + (j == k ? Us : R(0)));
            Bm[4][1 + j] = e3p * s[j] + rho * Us * uu[j];
        }
        Bm[4][0] = e2p * Us;
        Bm[4][4] = e4p * Us;
        if (MODE == TM_RES || MODE == TM_FULL) {
            R lt[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const R dq = (with_q && k > 0) ? v[Q::kDq + k - 1] : R(0);  // e3ls.f:147-156
                lt[k] = tk[k] * (v[Q::kAig + k] + v[Q::kA0 + k] - dq);
            }
            R fe[5];
            const R m = -rho * Us;
            fe[0] = m;
#pragma unroll
            for (int j = 0; j < 3; ++j) fe[1 + j] = m * uu[j] - s[j] * p + sv[j];
            fe[4] = m * ek - Us * p + usv;
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                R bt = R(0);
#pragma unroll
                for (int k = 0; k < 5; ++k) bt += Bm[r][k] * lt[k];
                rl[r] += w * (fe[r] + bt + Na * v[Q::kA0 + r]);
            }
        }
        if (MODE != TM_RES) {
            R rm16[5], lm[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                const R dk = (MODE == TM_FULL) ? v[Q::kDu + k] : v[Q::kA0 + k];
                rm16[k] = v[Q::kAig + k] + P.fct1 * dk;
                lm[k] = tk[k] * rm16[k];
            }
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                R bm = R(0);
#pragma unroll
                for (int k = 0; k < 5; ++k) bm += Bm[r][k] * lm[k];
                const R fm = (r == 0) ? R(0) : (r == 4) ? usv : sv[r - 1];
                rml[r] += w * (fm + bm + Na * rm16[r]);
            }
            if constexpr (sizeof(R) == 8 && MODE == TM_FULL) {
                // the reference's rmi(:,11) = rmi(:,12) + DC gA(:,12) (e3dc.f:366)
                if (P.idc) {
                    const R* dq = v + Q::kDc;
                    const R sz = drdp * lm[0] + drdT * lm[4];
                    const R z0 = u2 * sz + rho * lm[3];
                    const R z1 = u0 * z0 + rho * u2 * lm[1] + v[Q::kVt + 6];
                    rml[0] += w * s[2] * (z1 + dq[0] * dq[12] - z0 - dq[0] * dq[11]);
                }
            }
        }
        if constexpr (sizeof(R) == 8 && MODE != TM_LIN) {
            if (P.idc) {
                const R* dq = v + Q::kDc;
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    const R f = w * dq[0] * (s[0] * dq[1 + k] + s[1] * dq[6 + k] + s[2] * dq[11 + k]);
                    if (MODE == TM_RES || MODE == TM_FULL) rl[k] += f;
                    if (MODE != TM_RES) rml[k] += f;
                }
            }
        }
        if (MODE == TM_FULL && bd) {
            // (N_a I + B tau)(B + fct N_a A0) + K_a (e3bdg.f)
            const R fN = P.fct1 * Na;
            R Cm[5][5];
#pragma unroll
            for (int r = 0; r < 5; ++r)
#pragma unroll
                for (int k = 0; k < 5; ++k) Cm[r][k] = Bm[r][k];
            Cm[0][0] += fN * drdp;
            Cm[0][4] += fN * drdT;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                Cm[1 + j][0] += fN * drdp * uu[j];
                Cm[1 + j][1 + j] += fN * rho;
                Cm[1 + j][4] += fN * drdT * uu[j];
                Cm[4][1 + j] += fN * rho * uu[j];
            }
            Cm[4][0] += fN * e1p;
            Cm[4][4] += fN * e4p;
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                R D[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) D[k] = (P.supg ? Bm[r][k] * tk[k] : R(0)) + (r == k ? Na : R(0));
#pragma unroll
                for (int cc = 0; cc < 5; ++cc) {
                    R acc = R(0);
#pragma unroll
                    for (int k = 0; k < 5; ++k) acc += D[k] * Cm[k][cc];
                    B_[r][cc] += w * acc;
                }
            }
            if (P.navier) {
                const R ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
                R km[3][3];
#pragma unroll
                for (int j = 0; j < 3; ++j)
#pragma unroll
                    for (int k = 0; k < 3; ++k) km[j][k] = P.rlmpmu * s[j] * s[k] + (j == k ? P.rmu * ss : R(0));
#pragma unroll
                for (int j = 0; j < 3; ++j) {
#pragma unroll
                    for (int k = 0; k < 3; ++k) B_[1 + j][1 + k] += w * km[j][k];
                    B_[4][1 + j] += w * (km[j][0] * u0 + km[j][1] * u1 + km[j][2] * u2);
                }
                B_[4][4] += w * P.con * ss;
            }
        }
    }
    if ((MODE == TM_RES || MODE == TM_FULL) && res) {
        R* og = res + 5 * (size_t)node;
#pragma unroll
        for (int k = 0; k < 5; ++k) og[k] += rl[k];
    }
    if (MODE != TM_RES && rmes) {
        R* og = rmes + 5 * (size_t)node;
#pragma unroll
        for (int k = 0; k < 5; ++k) og[k] += iabres ? fabs(rml[k]) : rml[k];
    }
    if (MODE == TM_FULL && bd) {
        R* ob = bd + 25 * (size_t)node;
#pragma unroll
        for (int r = 0; r < 5; ++r)
#pragma unroll
            for (int cc = 0; cc < 5; ++cc) ob[5 * r + cc] += B_[r][cc];
    }
}

}  // namespace

// hex and wedge tables: the rules and linear shapes of symhex.c/symwdg.c and
// HexShapeAndDrv/WedgeShapeAndDrv (wedge in-plane derivatives on the area-2 parent);
// tet: the 4-point rule of symtet.c with the halved vertex-mode gradients of genshp.f:32-35
void topo_tables_host(TopoTabD* t) {
    for (int k = 0; k < 3; ++k) t[k] = TopoTabD{};
    const double g = 0.577350269189626;
    const double sgn[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                              {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int q = 0; q < 8; ++q) {
        const double par[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, (q & 4) ? g : -g};
        t[0].qwt[q] = 1.0;
        for (int a = 0; a < 8; ++a) {
            const double f[3] = {(1.0 + sgn[a][0] * par[0]) / 2.0, (1.0 + sgn[a][1] * par[1]) / 2.0,
                                 (1.0 + sgn[a][2] * par[2]) / 2.0};
            t[0].shp[q][a] = f[0] * f[1] * f[2];
            t[0].shgl[q][0][a] = sgn[a][0] / 2.0 * f[1] * f[2];
            t[0].shgl[q][1][a] = f[0] * sgn[a][1] / 2.0 * f[2];
            t[0].shgl[q][2][a] = f[0] * f[1] * sgn[a][2] / 2.0;
        }
    }
    const double P3 = 0.166666666666667, P4 = 0.666666666666667, Qz = 0.577350269189626, W = 0.666666666666667;
    const double tri[3][2] = {{P3, P3}, {P4, P3}, {P3, P4}};
    const double dLr[3] = {-1.0, 1.0, 0.0}, dLs[3] = {-1.0, 0.0, 1.0};
    for (int q = 0; q < 6; ++q) {
        const double r = tri[q % 3][0], s2 = tri[q % 3][1], z = q < 3 ? -Qz : Qz;
        const double L[3] = {1.0 - r - s2, r, s2};
        t[1].qwt[q] = W;
        for (int a = 0; a < 6; ++a) {
            const int v = a % 3;
            const double zs = a < 3 ? -1.0 : 1.0;
            const double fz = (1.0 + zs * z) / 2.0;
            t[1].shp[q][a] = L[v] * fz;
            t[1].shgl[q][0][a] = dLr[v] * fz / 2.0;
            t[1].shgl[q][1][a] = dLs[v] * fz / 2.0;
            t[1].shgl[q][2][a] = L[v] * zs / 2.0;
        }
    }
    const double a4 = 0.5854101966249685, b4 = 0.1381966011250150;
    const double pts[4][3] = {{a4, b4, b4}, {b4, a4, b4}, {b4, b4, a4}, {b4, b4, b4}};
    for (int q = 0; q < 4; ++q) {
        t[2].qwt[q] = kTetQwt;
        for (int a = 0; a < 3; ++a) t[2].shp[q][a] = pts[q][a];
        t[2].shp[q][3] = 1.0 - pts[q][0] - pts[q][1] - pts[q][2];
        for (int i = 0; i < 3; ++i) {
            for (int a = 0; a < 3; ++a) t[2].shgl[q][i][a] = (i == a) ? 0.5 : 0.0;
            t[2].shgl[q][i][3] = -0.5;
        }
    }
}

int upload_topo_tables(Ctx& C) {
    TopoTabD t[3];
    topo_tables_host(t);
    std::vector<TopoTabD> td(2);
    std::vector<TopoTabF> tf(2);
    for (int k = 0; k < 2; ++k) {
        td[k] = t[k];
        for (int q = 0; q < 8; ++q) {
            tf[k].qwt[q] = (float)t[k].qwt[q];
            for (int a = 0; a < 8; ++a) {
                tf[k].shp[q][a] = (float)t[k].shp[q][a];
                for (int i = 0; i < 3; ++i) tf[k].shgl[q][i][a] = (float)t[k].shgl[q][i][a];
            }
        }
    }
    int rc = check(C, cudaMemcpyToSymbolAsync(c_topo, td.data(), sizeof(TopoTabD) * 2, 0, cudaMemcpyHostToDevice,
                                              C.stream),
                   "upload tables");
    if (rc == PHGPU_OK)
        rc = check(C, cudaMemcpyToSymbolAsync(c_topof, tf.data(), sizeof(TopoTabF) * 2, 0, cudaMemcpyHostToDevice,
                                              C.stream),
                   "upload tables");
    if (rc == PHGPU_OK) rc = check(C, cudaStreamSynchronize(C.stream), "upload tables");
    return rc;
}

template <typename R, int NEN, int MODE>
constexpr size_t topo_smem() {
    return sizeof(R) * (size_t)(kTopoThreads / NEN) * NEN *
           (topo_node<R, MODE>() + TopoQp<NEN, sizeof(R) == 8, topo_lean<R, MODE>()>::kN);
}

template <typename R, int NEN, int TOPO>
int configure_topo_kernels(Ctx& C) {
    int rc = PHGPU_OK;
    auto T = [&](cudaError_t e) { if (rc == PHGPU_OK) rc = check(C, e, "cudaFuncSetAttribute"); };
    T(smem_attr(k_topo<R, NEN, TOPO, TM_RES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)topo_smem<R, NEN, TM_RES>()));
    T(smem_attr(k_topo<R, NEN, TOPO, TM_MODRES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)topo_smem<R, NEN, TM_MODRES>()));
    T(smem_attr(k_topo<R, NEN, TOPO, TM_LIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)topo_smem<R, NEN, TM_LIN>()));
    T(smem_attr(k_topo<R, NEN, TOPO, TM_FULL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)topo_smem<R, NEN, TM_FULL>()));
    T(smem_attr(k_topo<R, NEN, TOPO, TM_QREC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)topo_smem<R, NEN, TM_QREC>()));
    return rc;
}

template <typename R, int NEN, int TOPO>
static void launch_topo_one(Ctx& C, int mode, const int* d_ien, const std::vector<int>& col, const R* x,
                            const R* ya, const R* yb, const R* ac, R* res, R* rmes, R* bd, int iabres,
                            const int* skip, const R* ql) {
    const Phys<R> P = make_phys<R>(C.cfg);
    constexpr int EPB = kTopoThreads / NEN;
    const int ncol = (int)col.size() - 1;
    // the packed FP32 node records hold exactly this x and base state
    const float4* xbp = (sizeof(R) == 4 && (const void*)x == (const void*)C.d_xf && (const void*)yb == (const void*)C.d_yf)
                            ? C.d_xbf : nullptr;
    for (int c = 0; c < ncol; ++c) {
        const int e0 = col[c], ne = col[c + 1] - e0;
        if (ne <= 0) continue;
        const int grid = (ne + EPB - 1) / EPB;
        const int* ie = d_ien + (size_t)NEN * e0;
        switch (mode) {
            case TM_RES:
                k_topo<R, NEN, TOPO, TM_RES><<<grid, kTopoThreads, topo_smem<R, NEN, TM_RES>(), C.stream>>>(ie, ne, x, ya, yb, ac, res, rmes, bd, P, iabres, skip, ql);
                break;
            case TM_MODRES:
                k_topo<R, NEN, TOPO, TM_MODRES><<<grid, kTopoThreads, topo_smem<R, NEN, TM_MODRES>(), C.stream>>>(ie, ne, x, ya, yb, ac, res, rmes, bd, P, iabres, skip, ql, xbp);
                break;
            case TM_LIN:
                k_topo<R, NEN, TOPO, TM_LIN><<<grid, kTopoThreads, topo_smem<R, NEN, TM_LIN>(), C.stream>>>(ie, ne, x, ya, yb, ac, res, rmes, bd, P, iabres, skip, ql, xbp);
                break;
            case TM_QREC:
                k_topo<R, NEN, TOPO, TM_QREC><<<grid, kTopoThreads, topo_smem<R, NEN, TM_QREC>(), C.stream>>>(ie, ne, x, ya, yb, ac, res, rmes, bd, P, iabres, skip, ql);
                break;
            default:
                k_topo<R, NEN, TOPO, TM_FULL><<<grid, kTopoThreads, topo_smem<R, NEN, TM_FULL>(), C.stream>>>(ie, ne, x, ya, yb, ac, res, rmes, bd, P, iabres, skip, ql);
                break;
        }
        ++C.launches;
    }
}

template <typename R>
void launch_topo(Ctx& C, int mode, const R* x, const R* ya, const R* yb, const R* ac, R* res, R* rmes, R* bd,
                 int iabres, const int* skip, const R* ql) {
    if (C.nhex > 0)
        launch_topo_one<R, 8, 0>(C, mode, C.d_ienh, C.hcol_start, x, ya, yb, ac, res, rmes, bd, iabres, skip, ql);
    if (C.nwedge > 0)
        launch_topo_one<R, 6, 1>(C, mode, C.d_ienw, C.wcol_start, x, ya, yb, ac, res, rmes, bd, iabres, skip, ql);
}
template void launch_topo<double>(Ctx&, int, const double*, const double*, const double*, const double*, double*,
                                  double*, double*, int, const int*, const double*);
template void launch_topo<float>(Ctx&, int, const float*, const float*, const float*, const float*, float*, float*,
                                 float*, int, const int*, const float*);

static ChunkArgs chunk_args(const Ctx& C) {
    return ChunkArgs{C.d_ch_elem, C.d_ch_node, C.d_ch_nodes, C.d_ch_cstart, C.d_ch_csr, C.d_ch_lien};
}

template <typename R>
size_t res_smem(const Ctx& C) { return sizeof(R) * ((size_t)C.chunk_lmax * 13 + (size_t)kChunk * 20); }
size_t ress_pipe_smem(const Ctx& C, bool with_q) {
    return sizeof(float) * (2 * (size_t)ress_stage_words(C.chunk_lmax, with_q) + 3 * (size_t)lin_id_words(C.chunk_lmax) +
                            (size_t)kChunk * kSplitSlot);
}
size_t lin_pipe_smem(const Ctx& C) {
    // 3 record stages, 2 node-data stages, the element slots, 3 mbarriers
    return 3 * (size_t)C.chunk_rec_max + sizeof(float) * (2 * (size_t)lin_data_words(C.chunk_lmax) + (size_t)kChunk * 20) +
           4 * sizeof(unsigned long long);
}
// extra shared memory of the reconstructed flux (idiff = 1): 12 per chunk node
template <typename R>
size_t q_smem(const Ctx& C) { return sizeof(R) * (size_t)C.chunk_lmax * 12; }
template <typename R>
size_t qrec_smem(const Ctx& C) { return sizeof(R) * ((size_t)C.chunk_lmax * 8 + (size_t)kChunk * 52); }
template <typename R, bool BD_ONLY = false>
size_t full_smem(const Ctx& C) {
    const bool single = kFullSub * full_nsub<R>() >= kChunk;
    const size_t out = BD_ONLY ? 25 : kFullOutAll;
    return sizeof(R) * ((size_t)C.chunk_lmax * (13 + (single ? 0 : out)) + (size_t)kChunk * full_nsub<R>() * out);
}

size_t resh_smem(const Ctx& C) {
    return sizeof(double) * ((size_t)C.chunk_lmax * 13 + (size_t)kChunk * 20) + sizeof(float) * (size_t)C.chunk_lmax * 13;
}
size_t ress_smem(const Ctx& C) { return sizeof(float) * ((size_t)C.chunk_lmax * 21 + (size_t)kChunk * kSplitSlot); }

static void split(double v, float& hi, float& lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

template <typename R>
int configure_chunk_kernels(Ctx& C) {
    const int rs = (int)res_smem<R>(C), fs = (int)full_smem<R>(C);
    int rc = PHGPU_OK;
    auto T = [&](cudaError_t e) { if (rc == PHGPU_OK) rc = check(C, e, "cudaFuncSetAttribute"); };
    T(smem_attr(k_chunk_res<R, RM_RES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           rs + (int)q_smem<R>(C)));
    T(smem_attr(k_chunk_qrec<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)qrec_smem<R>(C)));
    T(smem_attr(k_chunk_res<R, RM_MODRES>, cudaFuncAttributeMaxDynamicSharedMemorySize, rs));
    T(smem_attr(k_chunk_res<R, RM_LIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, rs));
    T(smem_attr(k_chunk_full<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, fs + (int)q_smem<R>(C)));
    T(smem_attr(k_chunk_full<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)full_smem<R, true>(C)));
    return rc;
}
int configure_element_kernels(Ctx& C) {
    if (full_smem<double>(C) + q_smem<double>(C) > 227 * 1024) {
        C.err = "a mesh chunk has too many distinct nodes for shared memory";
        return PHGPU_ERR_UNSUPPORTED;
    }
    int rc = configure_chunk_kernels<double>(C);
    if (rc == PHGPU_OK) rc = configure_chunk_kernels<float>(C);
    if (rc == PHGPU_OK)
        rc = check(C, smem_attr(k_chunk_resh, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)resh_smem(C)),
                   "cudaFuncSetAttribute");
    if (rc == PHGPU_OK)
        rc = check(C, smem_attr(k_chunk_ress<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)ress_smem(C)),
                   "cudaFuncSetAttribute");
    if (rc == PHGPU_OK)
        rc = check(C, smem_attr(k_chunk_ress<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(ress_smem(C) + q_smem<float>(C))),
                   "cudaFuncSetAttribute");
    if (rc == PHGPU_OK) {
        // persistent grids of the pipelined sweeps: every resident CTA slot of each variant
        int dev = 0, nsm = 0;
        rc = check(C, cudaGetDevice(&dev), "cudaGetDevice");
        if (rc == PHGPU_OK) rc = check(C, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
        auto grid_of = [&](const void* f, size_t smem, int* grid) {
            int per_sm = 0;
            if (rc == PHGPU_OK)
                rc = check(C, smem_attr(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                           "cudaFuncSetAttribute");
            if (rc == PHGPU_OK)
                rc = check(C, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, kChunk, smem), "occupancy");
            *grid = std::max(1, nsm * per_sm);
        };
        grid_of((const void*)k_chunk_lin_pipe<3>, lin_pipe_smem(C), &C.lin_grids[0]);
        grid_of((const void*)k_chunk_lin_pipe<4>, lin_pipe_smem(C), &C.lin_grids[1]);
        int g2 = 0;
        grid_of((const void*)k_chunk_ress_pipe<false, 2>, ress_pipe_smem(C, false), &C.ress_grids[0]);
        grid_of((const void*)k_chunk_ress_pipe<false, 3>, ress_pipe_smem(C, false), &C.ress_grids[1]);
        grid_of((const void*)k_chunk_ress_pipe<false, 4>, ress_pipe_smem(C, false), &C.ress_grids[2]);
        grid_of((const void*)k_chunk_ress_pipe<true, 2>, ress_pipe_smem(C, true), &g2);
        grid_of((const void*)k_chunk_ress_pipe<true, 3>, ress_pipe_smem(C, true), &g2);
        grid_of((const void*)k_chunk_ress_pipe<true, 4>, ress_pipe_smem(C, true), &g2);
        if (rc == PHGPU_OK) select_sweep_variants(C, PHGPU_LINPIPE_MINB, PHGPU_RESS_MINB);
    }
    if (rc == PHGPU_OK) rc = configure_topo_kernels<double, 8, 0>(C);
    if (rc == PHGPU_OK) rc = configure_topo_kernels<double, 6, 1>(C);
    if (rc == PHGPU_OK) rc = configure_topo_kernels<float, 8, 0>(C);
    if (rc == PHGPU_OK) rc = configure_topo_kernels<float, 6, 1>(C);
    return rc;
}

template <typename R>
void launch_elem_res(Ctx& C, int mode, const R* x, const R* ya, const R* yb, const R* ac, R* out,
                     int iabres, const int* skip, const R* ql) {
    const Phys<R> P = make_phys<R>(C.cfg);
    const ChunkArgs ca = chunk_args(C);
    const size_t sm = res_smem<R>(C) + ((mode == RM_RES && ql) ? q_smem<R>(C) : 0);
    const int ncol = (int)C.chunk_col_start.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int c0 = C.chunk_col_start[c], nc = C.chunk_col_start[c + 1] - c0;
        if (nc <= 0) continue;
        if (mode == RM_RES)
            k_chunk_res<R, RM_RES><<<nc, kChunk, sm, C.stream>>>(ca, c0, x, ya, yb, ac, out, P, iabres, skip, ql);
        else if (mode == RM_MODRES)
            k_chunk_res<R, RM_MODRES><<<nc, kChunk, sm, C.stream>>>(ca, c0, x, ya, yb, ac, out, P, iabres, skip);
        else if constexpr (std::is_same<R, float>::value) {
            // the pipelined kernel reads the base state from the packed records of d_yf
            if (!C.cfg.no_pipe && !skip && !iabres && (const void*)yb == (const void*)C.d_yf) {
                const int g = std::min(nc, C.lin_pipe_grid);
                const float4* xbp = C.d_xbf;
                int* err = C.d_flag + 1;
                if (C.lin_minb == 3)
                    k_chunk_lin_pipe<3><<<g, kChunk, lin_pipe_smem(C), C.stream>>>(
                        C.d_ch_rec, C.d_ch_rec_off, c0, nc, xbp, ya, out, P, C.chunk_lmax, C.chunk_rec_max, err);
                else
                    k_chunk_lin_pipe<4><<<g, kChunk, lin_pipe_smem(C), C.stream>>>(
                        C.d_ch_rec, C.d_ch_rec_off, c0, nc, xbp, ya, out, P, C.chunk_lmax, C.chunk_rec_max, err);
            } else
                k_chunk_res<R, RM_LIN><<<nc, kChunk, sm, C.stream>>>(ca, c0, x, ya, yb, ac, out, P, iabres, skip);
        } else
            k_chunk_res<R, RM_LIN><<<nc, kChunk, sm, C.stream>>>(ca, c0, x, ya, yb, ac, out, P, iabres, skip);
        ++C.launches;
    }
    // hex and wedge blocks: ires = 1 writes res, ires = 2 (and the linearized form) rmes
    if (mode == RM_RES) launch_topo<R>(C, TM_RES, x, ya, yb, ac, out, nullptr, nullptr, iabres, skip, ql);
    else launch_topo<R>(C, mode, x, ya, yb, ac, nullptr, out, nullptr, iabres, skip, nullptr);
}
template void launch_elem_res<double>(Ctx&, int, const double*, const double*, const double*, const double*,
                                      double*, int, const int*, const double*);
template void launch_elem_res<float>(Ctx&, int, const float*, const float*, const float*, const float*, float*,
                                     int, const int*, const float*);

// lumped L2 reconstruction of the diffusive flux into out (13 per node, zeroed by the caller)
template <typename R>
void launch_qrec(Ctx& C, const R* x, const R* y, R* out) {
    const Phys<R> P = make_phys<R>(C.cfg);
    const ChunkArgs ca = chunk_args(C);
    const size_t sm = qrec_smem<R>(C);
    const int ncol = (int)C.chunk_col_start.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int c0 = C.chunk_col_start[c], nc = C.chunk_col_start[c + 1] - c0;
        if (nc <= 0) continue;
        k_chunk_qrec<R><<<nc, kChunk, sm, C.stream>>>(ca, c0, x, y, out, P);
        ++C.launches;
    }
    launch_topo<R>(C, TM_QREC, x, y, nullptr, nullptr, out, nullptr, nullptr, 0, nullptr, nullptr);
}
template void launch_qrec<double>(Ctx&, const double*, const double*, double*);
template void launch_qrec<float>(Ctx&, const float*, const float*, float*);

void pack_xb(Ctx& C) {
    // every topology's FP32 products read the packed records, so pack on every mesh
    if (C.N == 0) return;
    const int blocks = (int)std::min<size_t>(((size_t)C.N + 255) / 256, 8192);
    k_pack_xb<<<blocks, 256, 0, C.stream>>>(C.d_xf, C.d_yf, C.d_xbf, C.N);
    ++C.launches;
}

// ---------------------------------------------------------------------------
// autotuner of the two pipelined sweeps' register/occupancy variants
// ---------------------------------------------------------------------------
// (0 selects the compiled-in default of each)
void select_sweep_variants(Ctx& C, int lin_minb, int ress_minb) {
    static_assert(PHGPU_LINPIPE_MINB >= 3 && PHGPU_LINPIPE_MINB <= 4, "linearized-product variants are 3 and 4");
    static_assert(PHGPU_RESS_MINB >= 2 && PHGPU_RESS_MINB <= 4, "split-residual variants are 2, 3 and 4");
    C.lin_minb = (lin_minb == 3 || lin_minb == 4) ? lin_minb : PHGPU_LINPIPE_MINB;
    C.ress_minb = (ress_minb >= 2 && ress_minb <= 4) ? ress_minb : PHGPU_RESS_MINB;
    C.lin_pipe_grid = C.lin_grids[C.lin_minb - 3];
    C.ress_pipe_grid = C.ress_grids[C.ress_minb - 2];
}

// Each candidate runs once to warm up, then three times between CUDA events, on the context's own
// mesh and state (the FP32 split of y and ac, which the next assembly writes again; direction =
// the state for the linearized product; outputs to scratch).  A variant replaces the compiled-in
// default only when it is more than kTuneGain faster: the variants are the same source under
// different register budgets, and the compiler may contract multiplies and adds differently
// under each, so their results agree to FP32 rounding but not bit for bit; the margin keeps
// the choice (and so the results) from flipping with timing noise.  On a mesh whose default
// linearized product takes less than kTuneMinMs the timings are mostly noise and the defaults
// stay (unless tuning is forced with phgpu_set_tuning(-1, -1)).  The choice holds for the
// context's lifetime.  The split residual is tuned only when it is the outer residual in use.
constexpr double kTuneGain = 0.05;
constexpr double kTuneMinMs = 0.5;
int autotune_sweeps(Ctx& C) {
    Range nv("phgpu: sweep autotuner");
    if (C.tuned || C.tune_forced || C.cfg.no_pipe || C.E == 0) return PHGPU_OK;
    const size_t n5 = 5 * (size_t)C.N;
    const long long l0 = C.launches;
    // flag[1] collects the sweeps' bulk-copy status over the timing runs (the assembly after
    // the tuner clears the flags again)
    if (check(C, cudaMemsetAsync(C.d_flag + 1, 0, sizeof(int), C.stream), "autotune") != PHGPU_OK)
        return PHGPU_ERR_CUDA;
    split_f32(C, C.d_y, C.d_yf, C.d_ylo, n5);
    pack_xb(C);
    to_f32(C, C.d_ac, C.d_acf, n5);
    cudaEvent_t e0 = C.ev[2], e1 = C.ev[3];
    auto time_it = [&](auto&& fn) {
        fn();
        cudaEventRecord(e0, C.stream);
        for (int r = 0; r < 3; ++r) fn();
        cudaEventRecord(e1, C.stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        return (double)ms / 3.0;
    };
    select_sweep_variants(C, 0, 0);
    const int def_l = C.lin_minb, def_r = C.ress_minb;
    // the fastest variant, or the default unless that one beats it by more than kTuneGain
    auto pick = [](const double* ms, int lo, int hi, int def) {
        int best = def;
        for (int m = lo; m <= hi; ++m)
            if (ms[m - lo] < ms[best - lo]) best = m;
        return ms[best - lo] < (1.0 - kTuneGain) * ms[def - lo] ? best : def;
    };
    auto time_lin = [&](int m) {
        select_sweep_variants(C, m, def_r);
        C.tune_ms[m - 3] = time_it([&] {
            launch_elem_res<float>(C, RM_LIN, C.d_xf, C.d_yf, C.d_yf, nullptr, C.d_t32, 0, nullptr);
        });
    };
    time_lin(def_l);
    if (!C.tune_always && C.tune_ms[def_l - 3] < kTuneMinMs) {
        C.launches = l0;
        select_sweep_variants(C, def_l, def_r);
        C.tuned = true;
        int f = 0;
        if (check(C, cudaMemcpyAsync(&f, C.d_flag + 1, sizeof(int), cudaMemcpyDeviceToHost, C.stream), "autotune") !=
                PHGPU_OK ||
            check(C, cudaStreamSynchronize(C.stream), "autotune") != PHGPU_OK)
            return PHGPU_ERR_CUDA;
        if (f & kPipeCopyFailed) return fail(C, PHGPU_ERR_CUDA, kPipeCopyMsg);
        return check(C, cudaGetLastError(), "autotune");
    }
    for (int m = 3; m <= 4; ++m)
        if (m != def_l) time_lin(m);
    const int best_l = pick(C.tune_ms, 3, 4, def_l);
    int best_r = def_r;
    if (C.cfg.outer_residual == PHGPU_RES_SPLITDF) {
        for (int m = 2; m <= 4; ++m) {
            select_sweep_variants(C, best_l, m);
            C.tune_ms[2 + m - 2] = time_it([&] { launch_elem_ress(C, C.d_yf, C.d_ylo, C.d_acf, C.d_t64, nullptr); });
        }
        best_r = pick(C.tune_ms + 2, 2, 4, def_r);
    }
    C.launches = l0;  // tuning launches are not part of the solve
    select_sweep_variants(C, best_l, best_r);
    C.tuned = true;
    int f = 0;
    if (check(C, cudaMemcpyAsync(&f, C.d_flag + 1, sizeof(int), cudaMemcpyDeviceToHost, C.stream), "autotune") !=
            PHGPU_OK ||
        check(C, cudaStreamSynchronize(C.stream), "autotune") != PHGPU_OK)
        return PHGPU_ERR_CUDA;
    if (f & kPipeCopyFailed) return fail(C, PHGPU_ERR_CUDA, kPipeCopyMsg);
    return check(C, cudaGetLastError(), "autotune");
}

void launch_elem_resh(Ctx& C, const double* y, const double* ac, const float* yf, const float* acf, double* out) {
    const Phys<double> P = make_phys<double>(C.cfg);
    const Phys<float> Pf = make_phys<float>(C.cfg);
    const ChunkArgs ca = chunk_args(C);
    const size_t sm = resh_smem(C);
    const int ncol = (int)C.chunk_col_start.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int c0 = C.chunk_col_start[c], nc = C.chunk_col_start[c + 1] - c0;
        if (nc <= 0) continue;
        k_chunk_resh<<<nc, kChunk, sm, C.stream>>>(ca, c0, C.d_x, y, ac, C.d_xf, yf, acf, out, P, Pf);
        ++C.launches;
    }
}

void launch_elem_ress(Ctx& C, const float* yh, const float* ylo, const float* acf, double* out, const float* ql) {
    const Phys<float> Pf = make_phys<float>(C.cfg);
    DfConst K;
    split(1.0 / C.cfg.Rgas, K.rRgas_hi, K.rRgas_lo);
    split(C.cfg.Rgas / C.cfg.gamma1, K.cv_hi, K.cv_lo);
    split(0.5 * kTetQwt, K.wq_hi, K.wq_lo);
    const ChunkArgs ca = chunk_args(C);
    const size_t sm = ress_smem(C) + (ql ? q_smem<float>(C) : 0);
    const int ncol = (int)C.chunk_col_start.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int c0 = C.chunk_col_start[c], nc = C.chunk_col_start[c + 1] - c0;
        if (nc <= 0) continue;
        if (!C.cfg.no_pipe) {
            const int g = std::min(nc, C.ress_pipe_grid);
            const size_t smp = ress_pipe_smem(C, ql != nullptr);
#define PH_RESS(Q, M) k_chunk_ress_pipe<Q, M><<<g, kChunk, smp, C.stream>>>(ca, c0, nc, C.d_xf, C.d_xlo, yh, ylo, \
                                                                          acf, out, Pf, K, ql, C.chunk_lmax)
            if (ql) {
                if (C.ress_minb == 2) PH_RESS(true, 2);
                else if (C.ress_minb == 4) PH_RESS(true, 4);
                else PH_RESS(true, 3);
            } else {
                if (C.ress_minb == 2) PH_RESS(false, 2);
                else if (C.ress_minb == 4) PH_RESS(false, 4);
                else PH_RESS(false, 3);
            }
#undef PH_RESS
        } else if (ql) {
            k_chunk_ress<true><<<nc, kChunk, sm, C.stream>>>(ca, c0, C.d_xf, C.d_xlo, yh, ylo, acf, out, Pf, K, ql);
        } else {
            k_chunk_ress<false><<<nc, kChunk, sm, C.stream>>>(ca, c0, C.d_xf, C.d_xlo, yh, ylo, acf, out, Pf, K, ql);
        }
        ++C.launches;
    }
}

template <typename R>
void launch_elem_full(Ctx& C, const R* x, const R* y, const R* ac, R* res, R* rmes, R* bd, const R* ql) {
    const Phys<R> P = make_phys<R>(C.cfg);
    const ChunkArgs ca = chunk_args(C);
    // BDiag alone (the mixed-precision preconditioner) runs the kernel without the residual terms
    const bool bd_only = !res && !rmes;
    const size_t sm = bd_only ? full_smem<R, true>(C) : full_smem<R>(C) + ((ql && res) ? q_smem<R>(C) : 0);
    // the packed FP32 node records hold exactly this x and y
    const float4* xb_packed = (sizeof(R) == 4 && (const void*)x == (const void*)C.d_xf &&
                               (const void*)y == (const void*)C.d_yf) ? C.d_xbf : nullptr;
    const int ncol = (int)C.chunk_col_start.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int c0 = C.chunk_col_start[c], nc = C.chunk_col_start[c + 1] - c0;
        if (nc <= 0) continue;
        if (bd_only)
            k_chunk_full<R, true><<<nc, kChunk, sm, C.stream>>>(ca, c0, x, y, ac, nullptr, nullptr, bd, P, nullptr,
                                                              xb_packed);
        else
            k_chunk_full<R, false><<<nc, kChunk, sm, C.stream>>>(ca, c0, x, y, ac, res, rmes, bd, P,
                                                               (ql && res) ? ql : nullptr);
        ++C.launches;
    }
    launch_topo<R>(C, TM_FULL, x, y, nullptr, ac, res, rmes, bd, 0, nullptr, (ql && res) ? ql : nullptr);
}
template void launch_elem_full<double>(Ctx&, const double*, const double*, const double*, double*, double*,
                                       double*, const double*);
template void launch_elem_full<float>(Ctx&, const float*, const float*, const float*, float*, float*, float*,
                                      const float*);

void launch_boundary(Ctx& C, const double* y, double* res) {
    const Phys<double> P = make_phys<double>(C.cfg);
    const int ncol = (int)C.bcol_start.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int e0 = C.bcol_start[c], ne = C.bcol_start[c + 1] - e0;
        if (ne <= 0) continue;
        const int grid = (ne + kBlock - 1) / kBlock;
        k_boundary<<<grid, kBlock, 0, C.stream>>>(C.d_ienb + e0, C.d_iBCB + e0, C.d_BCB + 18 * (size_t)e0, ne,
                                                   C.d_x, y, res, P);
        ++C.launches;
    }
    launch_bnd_blocks(C, y, res);
}

// the bounded mbarrier wait of the pipelined sweeps, made to run out (k_wait_limit_probe)
int selftest_wait_limit(int tries, int* status) {
    int* d = nullptr;
    cudaError_t e = cudaMalloc((void**)&d, sizeof(int));
    if (e != cudaSuccess) return PHGPU_ERR_NOMEM;
    e = cudaMemset(d, 0xff, sizeof(int));
    if (e == cudaSuccess) {
        k_wait_limit_probe<<<1, 32>>>(tries, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(status, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? PHGPU_OK : PHGPU_ERR_CUDA;
}

}  // namespace phgpu

extern "C" int phgpu_selftest_wait_limit(int tries, int* status) {
    if (!status || tries < 1 || tries > phgpu::kMbarTriesMax) return PHGPU_ERR_INVALID;
    return phgpu::selftest_wait_limit(tries, status);
}
