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
#include "phgpu_impl.cuh"

namespace phgpu {

__constant__ TetTables c_tab;

void upload_tables(Ctx& C) {
    TetTables t;
    // symtet.c 4-point rule (barycentric (a,b,b,b) permutations), genint.f:72 Qwt *= 4/3
    const double a4 = 0.5854101966249685, b4 = 0.1381966011250150;
    const double pts[4][3] = {{a4, b4, b4}, {b4, a4, b4}, {b4, b4, a4}, {b4, b4, b4}};
    for (int q = 0; q < 4; ++q) {
        t.shp[q][0] = pts[q][0];
        t.shp[q][1] = pts[q][1];
        t.shp[q][2] = pts[q][2];
        t.shp[q][3] = 1.0 - pts[q][0] - pts[q][1] - pts[q][2];
        t.Qwt[q] = (4.0 / 3.0) * 0.25;
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
    check(C, cudaMemcpyToSymbolAsync(c_tab, &t, sizeof(t), 0, cudaMemcpyHostToDevice, C.stream),
          "upload tables");
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
    return p;
}
template Phys<double> make_phys<double>(const phgpu_config&);
template Phys<float> make_phys<float>(const phgpu_config&);

namespace {

__device__ __forceinline__ float rsqrt_(float v) { return rsqrtf(v); }
__device__ __forceinline__ double rsqrt_(double v) { return rsqrt(v); }

template <typename R>
struct Geo {
    R WdetJ;
    R shg[4][3];
    R G[6];  // tet-invariant metric, order (11, 12, 22, 13, 23, 33)
    R GG, trG;
};

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
    g.WdetJ = R(c_tab.Qwt[0]) * det;
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

// viscous stress (symmetric) and heat flux of a gradient field (e3visc.f:278-368)
template <typename R>
struct Visc {
    R t[3][3];
    R q[3];
};
template <typename R>
__device__ __forceinline__ void viscous(const Phys<R>& P, const R (&g)[3][5], Visc<R>& v) {
    const R divu = g[0][1] + g[1][2] + g[2][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) v.t[i][j] = P.rmu * (g[i][1 + j] + g[j][1 + i]);
        v.t[i][i] = P.rlm * divu + R(2) * P.rmu * g[i][1 + i];
        v.q[i] = P.con * g[i][4];
    }
}

template <typename R>
struct Qp {
    R u[3], p, T;
    R rho, rk, ei, drdp, drdT, e1p, e2p, e3p, e4p;
    R tau[3];
};

// thermodynamics and the scalars that define A0..A3 (getthm.f ipress=0, e3mtrx.f)
template <typename R>
__device__ __forceinline__ void qp_state(const Phys<R>& P, R p, R u0, R u1, R u2, R T, Qp<R>& b) {
    b.p = p;
    b.u[0] = u0;
    b.u[1] = u1;
    b.u[2] = u2;
    b.T = T;
    const R rT = R(1) / T;
    b.drdp = P.rRgas * rT;            // rho * betaT = 1/(R T)
    b.rho = p * b.drdp;
    b.drdT = -b.rho * rT;             // -rho * alfap
    b.rk = R(0.5) * (u0 * u0 + u1 * u1 + u2 * u2);
    b.ei = T * P.cv;
    const R hk = T * P.cp + b.rk;
    b.e1p = b.drdp * hk - rT * T;
    b.e2p = b.e1p + R(1);
    b.e3p = b.rho * hk;
    b.e4p = b.drdT * hk + b.rho * P.cp;
}

// diagonal tau (e3tau.f:140-181, itau = 0)
template <typename R>
__device__ __forceinline__ void qp_tau(const Phys<R>& P, const Geo<R>& geo, Qp<R>& b) {
    const R* G = geo.G;
    const R u0 = b.u[0], u1 = b.u[1], u2 = b.u[2];
    const R uGu = u0 * (u0 * G[0] + R(2) * (u1 * G[1] + u2 * G[3])) + u1 * (u1 * G[2] + R(2) * u2 * G[4]) +
                  u2 * u2 * G[5];
    const R t2 = b.rho * b.rho * (P.dts2 + uGu) + P.fmu2 * geo.GG;
    const R rfact = rsqrt_(t2);
    const R fact = t2 * rfact;
    b.tau[0] = R(0.125) * fact / (b.rho * geo.trG) * P.taucfct;
    b.tau[1] = rfact;
    b.tau[2] = rfact * P.rtempcv;
}

// sum_i A_i Y,i (e3conv.f:100-179) in closed form
template <typename R>
__device__ __forceinline__ void ai_gi(const Qp<R>& b, const R (&g)[3][5], R (&o)[5]) {
    const R u0 = b.u[0], u1 = b.u[1], u2 = b.u[2];
    const R ugp = u0 * g[0][0] + u1 * g[1][0] + u2 * g[2][0];
    const R ugT = u0 * g[0][4] + u1 * g[1][4] + u2 * g[2][4];
    const R divu = g[0][1] + g[1][2] + g[2][3];
    const R c0 = b.drdp * ugp + b.rho * divu + b.drdT * ugT;
    R adv[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) adv[d] = u0 * g[0][1 + d] + u1 * g[1][1 + d] + u2 * g[2][1 + d];
    o[0] = c0;
#pragma unroll
    for (int d = 0; d < 3; ++d) o[1 + d] = b.u[d] * c0 + g[d][0] + b.rho * adv[d];
    o[4] = b.e2p * ugp + b.e3p * divu + b.rho * (u0 * adv[0] + u1 * adv[1] + u2 * adv[2]) + b.e4p * ugT;
}

// A0 v
template <typename R>
__device__ __forceinline__ void a0_v(const Qp<R>& b, const R (&v)[5], R (&o)[5]) {
    const R s = b.drdp * v[0] + b.drdT * v[4];
    o[0] = s;
#pragma unroll
    for (int j = 0; j < 3; ++j) o[1 + j] = b.u[j] * s + b.rho * v[1 + j];
    o[4] = b.e1p * v[0] + b.rho * (b.u[0] * v[1] + b.u[1] * v[2] + b.u[2] * v[3]) + b.e4p * v[4];
}

// F_i += A_i v for i = 0..2
template <typename R>
__device__ __forceinline__ void add_ai_v(const Qp<R>& b, const R (&v)[5], R (&F)[3][5]) {
    const R s = b.drdp * v[0] + b.drdT * v[4];
    const R t = b.e2p * v[0] + b.rho * (b.u[0] * v[1] + b.u[1] * v[2] + b.u[2] * v[3]) + b.e4p * v[4];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const R r0 = b.u[i] * s + b.rho * v[1 + i];
        F[i][0] += r0;
#pragma unroll
        for (int j = 0; j < 3; ++j) F[i][1 + j] += b.u[j] * r0 + b.rho * b.u[i] * v[1 + j] + (i == j ? v[0] : R(0));
        F[i][4] += b.u[i] * t + b.e3p * v[1 + i];
    }
}

template <typename R> __device__ __forceinline__ R ldg(const R* p) { return __ldg(p); }

template <typename R>
__device__ __forceinline__ void load5(const R* __restrict__ a, int n, R (&o)[5]) {
    const R* p = a + 5 * (size_t)n;
#pragma unroll
    for (int k = 0; k < 5; ++k) o[k] = ldg(p + k);
}

// --------------------------------------------------------------------------
// residual family, one thread per element
//   RM_RES    : ires = 1 residual (Euler + viscous + SUPG + time term)
//   RM_MODRES : ires = 2 modified residual of (ya = perturbed, yb = base)
//   RM_LIN    : d/d eps of the modified residual at yb in direction ya
// --------------------------------------------------------------------------
template <typename R, int MODE>
__global__ void __launch_bounds__(kBlock)
k_elem_res(const int4* __restrict__ ien, int ne, const R* __restrict__ x, const R* __restrict__ ya,
           const R* __restrict__ yb, const R* __restrict__ ac, R* __restrict__ out, Phys<R> P,
           int iabres, const int* __restrict__ skip) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    if (skip && *skip) return;
    const int4 nd4 = ien[e];
    const int nd[4] = {nd4.x, nd4.y, nd4.z, nd4.w};
    Geo<R> geo;
    {
        R xl[4][3];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d) xl[a][d] = ldg(x + 3 * (size_t)nd[a] + d);
        geometry(xl, geo);
    }
    // RM_RES: va = state, vb = acceleration; otherwise va = perturbed state or
    // direction and vb = base state
    R va[4][5], vb[4][5];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        load5(ya, nd[a], va[a]);
        load5(MODE == RM_RES ? ac : yb, nd[a], vb[a]);
    }
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

#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        R N[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) N[a] = R(c_tab.shp[q][a]);
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
        } else {
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 5; ++k) F[i][k] = R(0);
            R du[5];
            if (MODE == RM_MODRES) {
                // conservative variables of the perturbed state (e3ivar.f:96-131)
                R pv[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) pv[k] = N[0] * va[0][k] + N[1] * va[1][k] + N[2] * va[2][k] + N[3] * va[3][k];
                const R rho6 = pv[0] / (P.Rgas * pv[4]);
                const R rk6 = R(0.5) * (pv[1] * pv[1] + pv[2] * pv[2] + pv[3] * pv[3]);
                du[0] = rho6;
                du[1] = rho6 * pv[1];
                du[2] = rho6 * pv[2];
                du[3] = rho6 * pv[3];
                du[4] = rho6 * (pv[4] * P.cv + rk6);
            } else {
                R vq[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) vq[k] = N[0] * va[0][k] + N[1] * va[1][k] + N[2] * va[2][k] + N[3] * va[3][k];
                a0_v(b, vq, du);
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
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 5; ++k) S[i][k] += F[i][k];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int k = 0; k < 5; ++k) Tn[a][k] += N[a] * r16[k];
    }
    // e3wmlt.f + local.f scatter (colour-exclusive read-modify-write)
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        R* o = out + 5 * (size_t)nd[a];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            R v = geo.WdetJ * (geo.shg[a][0] * S[0][k] + geo.shg[a][1] * S[1][k] + geo.shg[a][2] * S[2][k] + Tn[a][k]);
            if (iabres) v = fabs(v);
            o[k] += v;
        }
    }
}

// --------------------------------------------------------------------------
// ElmMFG interior (ires = 3, iprec = 1): res, rmes and BDiag.
// One thread per (element, node a); the quadrature-point state is evaluated
// by each of the four threads of an element.
// --------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kBlock)
k_elem_full(const int4* __restrict__ ien, int ne, const R* __restrict__ x, const R* __restrict__ y,
            const R* __restrict__ ac, R* __restrict__ res, R* __restrict__ rmes, R* __restrict__ bd,
            Phys<R> P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int e = t >> 2, a = t & 3;
    if (e >= ne) return;
    const int4 nd4 = ien[e];
    const int nd[4] = {nd4.x, nd4.y, nd4.z, nd4.w};
    Geo<R> geo;
    {
        R xl[4][3];
#pragma unroll
        for (int n = 0; n < 4; ++n)
#pragma unroll
            for (int d = 0; d < 3; ++d) xl[n][d] = ldg(x + 3 * (size_t)nd[n] + d);
        geometry(xl, geo);
    }
    R yl[4][5], al[4][5];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        load5(y, nd[n], yl[n]);
        load5(ac, nd[n], al[n]);
    }
    R g[3][5];
    gradients(geo, yl, g);
    Visc<R> vs;
    if (P.navier) viscous(P, g, vs);
    R s[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) s[i] = geo.shg[a][i];
    const R ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    R rl[5], rml[5], B_[5][5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        rl[k] = R(0);
        rml[k] = R(0);
#pragma unroll
        for (int j = 0; j < 5; ++j) B_[k][j] = R(0);
    }
    // viscous part of the weighted flux sum_i s_i F_i (element constant momentum part)
    R sv[3] = {R(0), R(0), R(0)}, sq = R(0);
    if (P.navier) {
#pragma unroll
        for (int j = 0; j < 3; ++j) sv[j] = s[0] * vs.t[0][j] + s[1] * vs.t[1][j] + s[2] * vs.t[2][j];
        sq = s[0] * vs.q[0] + s[1] * vs.q[1] + s[2] * vs.q[2];
    }
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        R N[4];
#pragma unroll
        for (int n = 0; n < 4; ++n) N[n] = R(c_tab.shp[q][n]);
        const R Na = N[a];
        R yq[5], aq[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            yq[k] = N[0] * yl[0][k] + N[1] * yl[1][k] + N[2] * yl[2][k] + N[3] * yl[3][k];
            aq[k] = N[0] * al[0][k] + N[1] * al[1][k] + N[2] * al[2][k] + N[3] * al[3][k];
        }
        Qp<R> b;
        qp_state(P, yq[0], yq[1], yq[2], yq[3], yq[4], b);
        qp_tau(P, geo, b);
        const R u0 = b.u[0], u1 = b.u[1], u2 = b.u[2];
        R aig[5], a0a[5], du[5];
        ai_gi(b, g, aig);
        a0_v(b, aq, a0a);
        const R ek = b.ei + b.rk;
        du[0] = b.rho;
        du[1] = b.rho * u0;
        du[2] = b.rho * u1;
        du[3] = b.rho * u2;
        du[4] = b.rho * ek;
        R lt[5], lm[5];  // tau (A_i Y,i + A0 Y,t)  and  tau (A_i Y,i + fct U)
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            lt[k] = aig[k] + a0a[k];
            lm[k] = aig[k] + P.fct1 * du[k];
        }
        const R tk[5] = {b.tau[0], b.tau[1], b.tau[1], b.tau[1], b.tau[2]};
        R rm16[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            rm16[k] = lm[k];
            lt[k] *= tk[k];
            lm[k] *= tk[k];
        }
        // B_a = sum_i s_i A_i
        const R Us = s[0] * u0 + s[1] * u1 + s[2] * u2;
        R Bm[5][5];
        Bm[0][0] = b.drdp * Us;
        Bm[0][4] = b.drdT * Us;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Bm[0][1 + j] = b.rho * s[j];
            Bm[1 + j][0] = b.drdp * Us * b.u[j] + s[j];
            Bm[1 + j][4] = b.drdT * Us * b.u[j];
#pragma unroll
            for (int k = 0; k < 3; ++k) Bm[1 + j][1 + k] = b.rho * (b.u[j] * s[k] + (j == k ? Us : R(0)));
            Bm[4][1 + j] = b.e3p * s[j] + b.rho * Us * b.u[j];
        }
        Bm[4][0] = b.e2p * Us;
        Bm[4][4] = b.e4p * Us;
        // residual: sum_i s_i (Euler_i + visc_i) + B_a tau L + N_a A0 Y,t
        R fe[5];
        const R m = -b.rho * Us;
        fe[0] = m;
#pragma unroll
        for (int j = 0; j < 3; ++j) fe[1 + j] = m * b.u[j] - s[j] * b.p + sv[j];
        fe[4] = m * ek - Us * b.p + (u0 * sv[0] + u1 * sv[1] + u2 * sv[2]) + sq;
        R fm[5];
        fm[0] = R(0);
#pragma unroll
        for (int j = 0; j < 3; ++j) fm[1 + j] = sv[j];
        fm[4] = (u0 * sv[0] + u1 * sv[1] + u2 * sv[2]) + sq;
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            R bt = R(0), bm = R(0);
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                bt += Bm[r][k] * lt[k];
                bm += Bm[r][k] * lm[k];
            }
            rl[r] += fe[r] + bt + Na * a0a[r];
            rml[r] += fm[r] + bm + Na * rm16[r];
        }
        // BDiag: (N_a I + B_a tau)(B_a + fct N_a A0) + K_a
        R Cm[5][5];
#pragma unroll
        for (int r = 0; r < 5; ++r)
#pragma unroll
            for (int k = 0; k < 5; ++k) Cm[r][k] = Bm[r][k];
        const R fN = P.fct1 * Na;
        Cm[0][0] += fN * b.drdp;
        Cm[0][4] += fN * b.drdT;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Cm[1 + j][0] += fN * b.drdp * b.u[j];
            Cm[1 + j][1 + j] += fN * b.rho;
            Cm[1 + j][4] += fN * b.drdT * b.u[j];
            Cm[4][1 + j] += fN * b.rho * b.u[j];
        }
        Cm[4][0] += fN * b.e1p;
        Cm[4][4] += fN * b.e4p;
        if (P.supg) {
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                R D[5];
#pragma unroll
                for (int k = 0; k < 5; ++k) D[k] = Bm[r][k] * tk[k] + (r == k ? Na : R(0));
#pragma unroll
                for (int c = 0; c < 5; ++c) {
                    R acc = R(0);
#pragma unroll
                    for (int k = 0; k < 5; ++k) acc += D[k] * Cm[k][c];
                    B_[r][c] += acc;
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < 5; ++r)
#pragma unroll
                for (int c = 0; c < 5; ++c) B_[r][c] += Na * Cm[r][c];
        }
        if (P.navier) {
            // K_a = sum_pq s_p s_q K_pq: momentum rmu|s|^2 I + (lambda+mu) s s^T, energy row K u, con |s|^2
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
    if (res) {
        R* o = res + 5 * (size_t)nd[a];
#pragma unroll
        for (int k = 0; k < 5; ++k) o[k] += w * rl[k];
    }
    if (rmes) {
        R* o = rmes + 5 * (size_t)nd[a];
#pragma unroll
        for (int k = 0; k < 5; ++k) o[k] += w * rml[k];
    }
    if (bd) {
        R* o = bd + 25 * (size_t)nd[a];
#pragma unroll
        for (int r = 0; r < 5; ++r)
#pragma unroll
            for (int c = 0; c < 5; ++c) o[5 * r + c] += w * B_[r][c];
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

}  // namespace

template <typename R>
void launch_elem_res(Ctx& C, int mode, const R* x, const R* ya, const R* yb, const R* ac, R* out,
                     int iabres, const int* skip) {
    const Phys<R> P = make_phys<R>(C.cfg);
    const int ncol = (int)C.col_start.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int e0 = C.col_start[c], ne = C.col_start[c + 1] - e0;
        if (ne <= 0) continue;
        const int grid = (ne + kBlock - 1) / kBlock;
        const int4* ien = C.d_ien + e0;
        if (mode == RM_RES)
            k_elem_res<R, RM_RES><<<grid, kBlock, 0, C.stream>>>(ien, ne, x, ya, yb, ac, out, P, iabres, skip);
        else if (mode == RM_MODRES)
            k_elem_res<R, RM_MODRES><<<grid, kBlock, 0, C.stream>>>(ien, ne, x, ya, yb, ac, out, P, iabres, skip);
        else
            k_elem_res<R, RM_LIN><<<grid, kBlock, 0, C.stream>>>(ien, ne, x, ya, yb, ac, out, P, iabres, skip);
        ++C.launches;
    }
}
template void launch_elem_res<double>(Ctx&, int, const double*, const double*, const double*, const double*,
                                      double*, int, const int*);
template void launch_elem_res<float>(Ctx&, int, const float*, const float*, const float*, const float*, float*,
                                     int, const int*);

template <typename R>
void launch_elem_full(Ctx& C, const R* x, const R* y, const R* ac, R* res, R* rmes, R* bd) {
    const Phys<R> P = make_phys<R>(C.cfg);
    const int ncol = (int)C.col_start.size() - 1;
    for (int c = 0; c < ncol; ++c) {
        const int e0 = C.col_start[c], ne = C.col_start[c + 1] - e0;
        if (ne <= 0) continue;
        const int grid = (4 * ne + kBlock - 1) / kBlock;
        k_elem_full<R><<<grid, kBlock, 0, C.stream>>>(C.d_ien + e0, ne, x, y, ac, res, rmes, bd, P);
        ++C.launches;
    }
}
template void launch_elem_full<double>(Ctx&, const double*, const double*, const double*, double*, double*,
                                       double*);
template void launch_elem_full<float>(Ctx&, const float*, const float*, const float*, float*, float*, float*);

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
}

}  // namespace phgpu
