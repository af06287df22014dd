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

}  // namespace
}  // namespace phgpu
