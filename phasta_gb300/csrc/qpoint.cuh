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

}  // namespace
}  // namespace phgpu
