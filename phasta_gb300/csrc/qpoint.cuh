// qpoint.cuh -- quadrature-point state shared by the element kernels: the
// thermodynamic scalars that define the Euler Jacobians A0..A3 (getthm.f with
// ipress = 0, e3mtrx.f) and the diagonal stabilization tau (e3tau.f:140-181,
// itau = 0).  Included by each translation unit that evaluates element
// integrals; every function is inline device code.
#pragma once
#include "phgpu_impl.cuh"

namespace phgpu {
namespace {

__device__ __forceinline__ float rsqrt_(float v) { return rsqrtf(v); }
__device__ __forceinline__ double rsqrt_(double v) { return rsqrt(v); }

template <typename R> __device__ __forceinline__ R ldg(const R* p) { return __ldg(p); }

// element metric of a linear tet, and the metric of tau for every topology
template <typename R>
struct Geo {
    R WdetJ;
    R shg[4][3];
    R G[6];  // tau metric, order (11, 12, 22, 13, 23, 33)
    R GG, trG;
};

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

// diagonal tau: itau = 0 (Shakib, e3tau.f:140-181) or, in FP64, itau = 1 (Franca's tau with
// the cell Reynolds number and a diffusive limit, e3tau.f:54-139)
template <typename R>
__device__ __forceinline__ void qp_tau(const Phys<R>& P, const Geo<R>& geo, Qp<R>& b) {
    const R* G = geo.G;
    const R u0 = b.u[0], u1 = b.u[1], u2 = b.u[2];
    if constexpr (sizeof(R) == 8) {
        if (P.itau == 1) {
            const R det = G[0] * G[2] * G[5] - G[0] * G[4] * G[4] - G[2] * G[3] * G[3] - G[5] * G[1] * G[1] +
                          R(2) * G[1] * G[3] * G[4];
            const R uau = u0 * u0 * (G[2] * G[5] - G[4] * G[4]) + u1 * u1 * (G[0] * G[5] - G[3] * G[3]) +
                          u2 * u2 * (G[0] * G[2] - G[1] * G[1]) +
                          R(2) * (u0 * u1 * (G[3] * G[4] - G[1] * G[5]) + u0 * u2 * (G[1] * G[4] - G[3] * G[2]) +
                                  u1 * u2 * (G[3] * G[1] - G[0] * G[4]));
            const R uh1 = R(2) * sqrt(uau / det);  // |u| h_1
            const R h2o2u = R(1) / sqrt(u0 * u0 * G[0] + u1 * u1 * G[2] + u2 * u2 * G[5] +
                                        R(2) * (u0 * u1 * G[1] + u0 * u2 * G[3] + u1 * u2 * G[4]) + R(1e-15));
            const R reh = R(0.5) * b.rho * uh1 / P.rmu;  // cell Reynolds number
            b.tau[0] = R(0.5) * uh1 * fmin(R(1), reh) * P.taucfct;
            const R t1 = fmin(P.rdts, h2o2u) / b.rho;
            const R t2 = t1 / P.cv;
            const R fd = h2o2u * h2o2u * b.rk * P.celt / P.rmu;
            b.tau[1] = fmin(t1, fd);
            b.tau[2] = fmin(t2, fd * P.rmu / P.con) * P.temper;
            return;
        }
    }
    const R uGu = u0 * (u0 * G[0] + R(2) * (u1 * G[1] + u2 * G[3])) + u1 * (u1 * G[2] + R(2) * u2 * G[4]) +
                  u2 * u2 * G[5];
    const R t2 = b.rho * b.rho * (P.dts2 + uGu) + P.fmu2 * geo.GG;
    const R rfact = rsqrt_(t2);
    const R fact = t2 * rfact;
    b.tau[0] = R(0.125) * fact / (b.rho * geo.trG) * P.taucfct;
    b.tau[1] = rfact;
    b.tau[2] = rfact * P.rtempcv;
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

// Discontinuity capturing at one point (e3dc.f with e3mtrx.f:232-297 and e3tau.f:183-261):
// returns the factor DC and fills gA[i] = sum_j g^ij A0 Y,j, so the point's fluxes gain
// DC gA.  ly is the least-squares residual before tau and lt the vector rTLS pairs it with
// (ly scaled by tau for the residual, ly itself for the modified residual); G is the tau
// metric (11, 12, 22, 13, 23, 33).
template <typename R>
__device__ __forceinline__ R dc_point(const Phys<R>& P, const R (&G)[6], const Qp<R>& b, const R (&g)[3][5],
                                      const R (&ly)[5], const R (&lt)[5], R (&gA)[3][5]) {
    const R rho = b.rho, T = b.T, u0 = b.u[0], u1 = b.u[1], u2 = b.u[2];
    const R alfap = R(1) / T, betaT = R(1) / b.p;
    const R s1 = R(1) / (rho * rho * betaT * T);
    const R cvd = P.cp - alfap * alfap * T / rho / betaT;
    const R c0 = (rho * betaT) * (rho * betaT) * s1, c1 = -(rho * alfap * rho * betaT * s1), c2 = rho / T,
            c3 = (rho * alfap) * (rho * alfap) * s1 + rho * cvd / (T * T);
    const R h = T * P.cp, e1 = h - b.rk;
    const R f1 = R(1) / (rho * cvd * (T * T));
    const R dd = alfap * T / rho / betaT;
    const R e2 = e1 - dd, e3 = e2 - cvd * T;
    const R e5 = e1 * e1 - R(2) * e1 * dd + R(2) * b.rk * cvd * T + P.cp * T / rho / betaT;
    const R cvT = cvd * T;
    // A0^-1 (symmetric, 15 entries) and dV/dY (upper triangle, 15 entries) in e3mtrx's order
    const R ai[15] = {e5 * f1, (u0 * u0 + cvT) * f1, (u1 * u1 + cvT) * f1, (u2 * u2 + cvT) * f1, f1,
                      u0 * e3 * f1, u1 * e3 * f1, u2 * e3 * f1, -e2 * f1, u0 * u1 * f1,
                      u2 * u0 * f1, -u0 * f1, u1 * u2 * f1, -u1 * f1, -u2 * f1};
    const R t1 = R(1) / T, t2 = t1 / T;
    const R dv[15] = {t1 / rho, -t1 * u0, t1, -t1 * u1, R(0), t1, -t1 * u2, R(0), R(0), t1,
                      -e1 * t2, -t2 * u0, -t2 * u1, -t2 * u2, t2};
    const R* L = lt;
    const R* Y = ly;
    const R rTLS = Y[0] * (L[0] * dv[0] + dv[1] * L[1] + dv[3] * L[2] + L[3] * dv[6] + dv[10] * L[4]) +
                   Y[1] * (L[1] * dv[2] + L[2] * dv[4] + dv[7] * L[3] + L[4] * dv[11]) +
                   Y[2] * (L[2] * dv[5] + dv[8] * L[3] + dv[12] * L[4]) + Y[3] * (L[3] * dv[9] + dv[13] * L[4]) +
                   Y[4] * (dv[14] * L[4]);
    const R raLS = R(2) * (Y[3] * Y[4] * ai[14] + Y[2] * Y[4] * ai[13] + Y[0] * Y[1] * ai[5] + Y[1] * Y[2] * ai[9] +
                           Y[1] * Y[3] * ai[10] + Y[0] * Y[2] * ai[6] + Y[2] * Y[3] * ai[12] + Y[1] * Y[4] * ai[11] +
                           Y[0] * Y[3] * ai[7] + Y[0] * Y[4] * ai[8]) +
                   Y[0] * Y[0] * ai[0] + Y[1] * Y[1] * ai[1] + Y[2] * Y[2] * ai[2] + Y[3] * Y[3] * ai[3] +
                   Y[4] * Y[4] * ai[4];
    // inverse metric g^ij, order (11, 22, 33, 12, 13, 23)
    const R q0 = G[0], q1 = G[2], q2 = G[5], q3 = G[1], q4 = G[3], q5 = G[4];
    const R detI = R(1) / (q0 * q1 * q2 - q0 * q5 * q5 - q3 * q3 * q2 + R(2) * q3 * q4 * q5 - q4 * q4 * q1);
    const R gi[6] = {detI * (q1 * q2 - q5 * q5), detI * (q0 * q2 - q4 * q4), detI * (q0 * q1 - q3 * q3),
                     detI * (q4 * q5 - q3 * q2), detI * (q3 * q5 - q4 * q1), detI * (q3 * q4 - q0 * q5)};
    R A0g[3][5];
#pragma unroll
    for (int j = 0; j < 3; ++j) a0_v(b, g[j], A0g[j]);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        gA[0][k] = gi[0] * A0g[0][k] + gi[3] * A0g[1][k] + gi[4] * A0g[2][k];
        gA[1][k] = gi[3] * A0g[0][k] + gi[1] * A0g[1][k] + gi[5] * A0g[2][k];
        gA[2][k] = gi[4] * A0g[0][k] + gi[5] * A0g[1][k] + gi[2] * A0g[2][k];
    }
    auto yy = [&](const R (&a)[5], const R (&c)[5]) {
        return a[0] * c0 * c[0] + a[0] * c1 * c[4] + a[4] * c1 * c[0] + c2 * (a[1] * c[1] + a[2] * c[2] + a[3] * c[3]) +
               a[4] * c3 * c[4];
    };
    const R y11 = yy(g[0], g[0]), y22 = yy(g[1], g[1]), y33 = yy(g[2], g[2]);
    const R y12 = yy(g[0], g[1]), y13 = yy(g[0], g[2]), y23 = yy(g[1], g[2]);
    const R gnorm = R(1) / (gi[0] * y11 + R(2) * (gi[3] * y12 + gi[4] * y13 + gi[5] * y23) + gi[1] * y22 +
                            gi[2] * y33 + P.epsM);
    // ipord = 1: fact = 1 (e3dc.f:253-303)
    const R mallet = fmax(R(0), sqrt(raLS * gnorm) - rTLS * gnorm);
    const R quad = R(2) * rTLS * gnorm;
    return P.idc == 1 ? mallet : P.idc == 2 ? quad : fmin(mallet, quad);
}

}  // namespace
}  // namespace phgpu
