// phasta_oracle.cpp -- CPU restatement (FP64) of PHASTA's compressible
// matrix-free Newton-Krylov hot path.
//
// TEST INFRASTRUCTURE ONLY: the parity checker of the GB300 kernels and the
// timed CPU baseline of the benchmark.  Nothing in the product links it.
//
// Every routine below follows the reference routine it names statement by
// statement, in the same operation order (array statements over the npro
// element vector become per-element scalar statements, which evaluates the
// same arithmetic).  Compile with -ffp-contract=off so no multiply-add is
// fused behind the restatement's back.  Terms the reference leaves out
// because they multiply structural zeros of the Euler Jacobians are written
// here as dense sums; adding an exact zero leaves every partial sum unchanged.
//
// Pinned against the reference itself: tests/golden/ref_*.npz hold outputs of
// the reference's own Fortran routines (executed from its sources by
// tests/golden/make_ref_golden.py), and tests/test_ref_golden.py checks this
// file against them.
#include "phasta_oracle.h"

#include <cmath>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>
#include <cstdint>

namespace {

// numeric constants of common.h:281-296
const double zero = 0.0, one = 1.0, two = 2.0, three = 3.0, four = 4.0;
const double pt125 = 0.125, pt5 = 0.5;
const double pt66 = 0.6666666666666666666666666666667;

// ---------------------------------------------------------------------------
// quadrature and shape functions for linear tets
//   symtet.c (4-point rule, barycentric (a,b,b,b) permutations, weights 1/4)
//   genint.f:72-73 (Qwt *= 4/3, Qwtb *= 2)
//   uniformP.c TetShapeAndDrv (N = L, dN of the vertex modes)
//   genshp.f:32-35 / genshpb.f (shgl /= 2 for tets)
//   symtri.c (3-point rule (B,C,C) with weights A)
// ---------------------------------------------------------------------------
struct Tables {
    double shp[4][4];      // [q][a]
    double shgl[4][3][4];  // [q][i][a]
    double Qwt[4];
    double shpb[3][4];
    double shglb[3][3][4];
    double Qwtb[3];
};

void tet_shape(const double par[3], double N[4], double dN[4][3]) {
    // uniformP.c:8-30 vertex modes
    double L[4] = {par[0], par[1], par[2], 1.0 - par[0] - par[1] - par[2]};
    for (int i = 0; i < 4; ++i) {
        N[i] = L[i];
        for (int j = 0; j < 3; ++j)
            dN[i][j] = (i == 3) ? -1.0 : (i == j ? 1.0 : 0.0);
    }
}

Tables make_tables() {
    Tables t;
    const double a4 = 0.5854101966249685, b4 = 0.1381966011250150;  // symtet.c
    const double pts[4][4] = {{a4, b4, b4, b4}, {b4, a4, b4, b4}, {b4, b4, a4, b4}, {b4, b4, b4, a4}};
    for (int q = 0; q < 4; ++q) {
        double N[4], dN[4][3];
        tet_shape(pts[q], N, dN);
        for (int a = 0; a < 4; ++a) {
            t.shp[q][a] = N[a];
            for (int i = 0; i < 3; ++i) t.shgl[q][i][a] = dN[a][i] / two;
        }
        t.Qwt[q] = (four / three) * 0.25;
    }
    const double A = 0.3333333333333330000000000000000000, B = 0.666666666666667,
                 C = 0.166666666666667;  // symtri.c
    const double ptb[3][3] = {{B, C, C}, {C, B, C}, {C, C, B}};
    for (int q = 0; q < 3; ++q) {
        double N[4], dN[4][3];
        tet_shape(ptb[q], N, dN);
        for (int a = 0; a < 4; ++a) {
            t.shpb[q][a] = N[a];
            for (int i = 0; i < 3; ++i) t.shglb[q][i][a] = dN[a][i] / two;
        }
        t.Qwtb[q] = two * A;
    }
    return t;
}

const Tables& tables() {
    static const Tables t = make_tables();
    return t;
}

// interior element topologies (lcsyst 1 tet, 2 hex, 3 wedge), linear basis (ipord = 1)
struct Topo {
    int lcsyst, nshl, ngauss;
    double shp[8][8];      // [q][a]
    double shgl[8][3][8];  // [q][i][a]
    double Qwt[8];
};

Topo make_topo(int lcsyst) {
    Topo t{};
    t.lcsyst = lcsyst;
    if (lcsyst == 1) {
        const Tables& T = tables();
        t.nshl = 4;
        t.ngauss = 4;
        for (int q = 0; q < 4; ++q) {
            t.Qwt[q] = T.Qwt[q];
            for (int a = 0; a < 4; ++a) {
                t.shp[q][a] = T.shp[q][a];
                for (int i = 0; i < 3; ++i) t.shgl[q][i][a] = T.shgl[q][i][a];
            }
        }
    } else if (lcsyst == 2) {
        // symhex.c 2-point Gauss rule per direction (xi fastest), weights 1 (genint.f: no scaling);
        // HexShapeAndDrv (newshape.cc) p = 1: trilinear vertex modes, node order
        // (-,-,-), (+,-,-), (+,+,-), (-,+,-), then zeta = +1
        const double g = 0.577350269189626;
        const double sgn[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                  {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
        t.nshl = 8;
        t.ngauss = 8;
        for (int q = 0; q < 8; ++q) {
            const double par[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, (q & 4) ? g : -g};
            t.Qwt[q] = 1.0;
            for (int a = 0; a < 8; ++a) {
                const double f[3] = {(1.0 + sgn[a][0] * par[0]) / 2.0, (1.0 + sgn[a][1] * par[1]) / 2.0,
                                     (1.0 + sgn[a][2] * par[2]) / 2.0};
                t.shp[q][a] = f[0] * f[1] * f[2];
                t.shgl[q][0][a] = sgn[a][0] / 2.0 * f[1] * f[2];
                t.shgl[q][1][a] = f[0] * sgn[a][1] / 2.0 * f[2];
                t.shgl[q][2][a] = f[0] * f[1] * sgn[a][2] / 2.0;
            }
        }
    } else {
        // symwdg.c 2-point rule: triangle points (1/6,1/6), (2/3,1/6), (1/6,2/3) x zeta = -+1/sqrt(3),
        // weight 2/3 each; WedgeShapeAndDrv p = 1: N = L_a (1 -+ zeta)/2, L = (1-r-s, r, s), with the
        // in-plane derivatives taken on a parent triangle of area 2 (half of d/dr, d/ds; the weights
        // sum to 4)
        const double P3 = 0.166666666666667, P4 = 0.666666666666667, Q = 0.577350269189626;
        const double W = 0.666666666666667;
        const double tri[3][2] = {{P3, P3}, {P4, P3}, {P3, P4}};
        t.nshl = 6;
        t.ngauss = 6;
        for (int q = 0; q < 6; ++q) {
            const double r = tri[q % 3][0], s2 = tri[q % 3][1], z = q < 3 ? -Q : Q;
            const double L[3] = {1.0 - r - s2, r, s2};
            const double dLr[3] = {-1.0, 1.0, 0.0}, dLs[3] = {-1.0, 0.0, 1.0};
            t.Qwt[q] = W;
            for (int a = 0; a < 6; ++a) {
                const int v = a % 3;
                const double zs = a < 3 ? -1.0 : 1.0;
                const double fz = (1.0 + zs * z) / 2.0;
                t.shp[q][a] = L[v] * fz;
                t.shgl[q][0][a] = dLr[v] * fz / 2.0;
                t.shgl[q][1][a] = dLs[v] * fz / 2.0;
                t.shgl[q][2][a] = L[v] * zs / 2.0;
            }
        }
    }
    return t;
}

const Topo& topo(int lcsyst) {
    static const Topo t[3] = {make_topo(1), make_topo(2), make_topo(3)};
    return t[lcsyst - 1];
}

// boundary element topologies (genint.f, genshpb.f; elmmfg.f:171-188 turns a wedge block's
// lcsyst 3 into nenbl, so 3 is the triangle face and 4 the quadrilateral face), linear basis
struct BTopo {
    int lcsyst, nshl, nshlb, ngaussb;
    int lnode[4];          // face nodes, 0-based, getbnodes order (hierarchic.f:90-165)
    double shpb[4][8];     // [q][a]
    double shglb[4][3][8]; // [q][i][a]
    double Qwtb[4];
};

// the linear hex and wedge shapes of make_topo at one parent point
void hex_shape(const double par[3], double N[8], double dN[3][8]) {
    const double sgn[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                              {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int a = 0; a < 8; ++a) {
        const double f[3] = {(1.0 + sgn[a][0] * par[0]) / 2.0, (1.0 + sgn[a][1] * par[1]) / 2.0,
                             (1.0 + sgn[a][2] * par[2]) / 2.0};
        N[a] = f[0] * f[1] * f[2];
        dN[0][a] = sgn[a][0] / 2.0 * f[1] * f[2];
        dN[1][a] = f[0] * sgn[a][1] / 2.0 * f[2];
        dN[2][a] = f[0] * f[1] * sgn[a][2] / 2.0;
    }
}
void wedge_shape(double r, double s2, double z, double N[8], double dN[3][8]) {
    const double L[3] = {1.0 - r - s2, r, s2};
    const double dLr[3] = {-1.0, 1.0, 0.0}, dLs[3] = {-1.0, 0.0, 1.0};
    for (int a = 0; a < 6; ++a) {
        const int v = a % 3;
        const double zs = a < 3 ? -1.0 : 1.0;
        const double fz = (1.0 + zs * z) / 2.0;
        N[a] = L[v] * fz;
        dN[0][a] = dLr[v] * fz / 2.0;
        dN[1][a] = dLs[v] * fz / 2.0;
        dN[2][a] = L[v] * zs / 2.0;
    }
}

BTopo make_btopo(int lcsyst) {
    BTopo t{};
    t.lcsyst = lcsyst;
    if (lcsyst == 1) {
        // the tet's 3-point triangle rule on face (0,1,2) (genint.f:61-75, genshpb.f)
        const Tables& T = tables();
        t.nshl = 4;
        t.nshlb = 3;
        t.ngaussb = 3;
        for (int n = 0; n < 3; ++n) t.lnode[n] = n;
        for (int q = 0; q < 3; ++q) {
            t.Qwtb[q] = T.Qwtb[q];
            for (int a = 0; a < 4; ++a) {
                t.shpb[q][a] = T.shpb[q][a];
                for (int i = 0; i < 3; ++i) t.shglb[q][i][a] = T.shglb[q][i][a];
            }
        }
    } else if (lcsyst == 2) {
        // symquad.c rule 2: (xi, eta) = (-+1/sqrt(3)) with xi fastest on zeta = -1, weights 1
        // (genint.f:140-142, no scaling)
        const double g = 0.577350269189626;
        t.nshl = 8;
        t.nshlb = 4;
        t.ngaussb = 4;
        for (int n = 0; n < 4; ++n) t.lnode[n] = n;
        for (int q = 0; q < 4; ++q) {
            const double par[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, -1.0};
            t.Qwtb[q] = 1.0;
            hex_shape(par, t.shpb[q], t.shglb[q]);
        }
    } else if (lcsyst == 3) {
        // symtri.c 3-point rule with its last point moved first (genint.f:325-332): (1/6, 1/6),
        // (2/3, 1/6), (1/6, 2/3) on zeta = -1, weights 0.333333333333333
        const double P3 = 0.166666666666667, P4 = 0.666666666666667;
        const double tri[3][2] = {{P3, P3}, {P4, P3}, {P3, P4}};
        t.nshl = 6;
        t.nshlb = 3;
        t.ngaussb = 3;
        for (int n = 0; n < 3; ++n) t.lnode[n] = n;
        for (int q = 0; q < 3; ++q) {
            t.Qwtb[q] = 0.333333333333333;
            wedge_shape(tri[q][0], tri[q][1], -1.0, t.shpb[q], t.shglb[q]);
        }
    } else {
        // symquadw.c rule 2: r = 0.211324865405187, 0.788675134594813 (r fastest), s = 0,
        // zeta = -+0.577350269189626, weights 1 (genint.f:340-343); face nodes 1, 4, 5, 2
        const double r[2] = {0.211324865405187, 0.788675134594813}, g = 0.577350269189626;
        t.nshl = 6;
        t.nshlb = 4;
        t.ngaussb = 4;
        t.lnode[0] = 0;
        t.lnode[1] = 3;
        t.lnode[2] = 4;
        t.lnode[3] = 1;
        for (int q = 0; q < 4; ++q) {
            t.Qwtb[q] = 1.0;
            wedge_shape(r[q & 1], 0.0, (q & 2) ? g : -g, t.shpb[q], t.shglb[q]);
        }
    }
    return t;
}

const BTopo& btopo(int lcsyst) {
    static const BTopo t[4] = {make_btopo(1), make_btopo(2), make_btopo(3), make_btopo(4)};
    return t[lcsyst - 1];
}

// ---------------------------------------------------------------------------
// e3.f for one element (lhs = 0, idiff = 0, iLES = iRANS = iLSet = 0, iDC = 0,
// no body force, ipord = 1, itau = 0)
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// e3 (e3.f and the routines it calls) for one element, generic in the scalar type: R = double is
// the oracle; R = Flop counts the floating-point operations of the reference formulation
// (or_e3_flops).  sqrt, max and min go through these overloads.
// ---------------------------------------------------------------------------
inline double osqrt(double x) { return std::sqrt(x); }
inline double omax(double a, double b) { return std::max(a, b); }
inline double omin(double a, double b) { return std::min(a, b); }

// counting scalar: every +, -, *, / and sqrt of two operands counts one operation
struct Flop {
    double v = 0.0;
    Flop() = default;
    Flop(double x) : v(x) {}  // NOLINT: constants and table values enter the arithmetic
};
thread_local long long g_flops = 0;
inline Flop operator+(Flop a, Flop b) { ++g_flops; return Flop(a.v + b.v); }
inline Flop operator-(Flop a, Flop b) { ++g_flops; return Flop(a.v - b.v); }
inline Flop operator*(Flop a, Flop b) { ++g_flops; return Flop(a.v * b.v); }
inline Flop operator/(Flop a, Flop b) { ++g_flops; return Flop(a.v / b.v); }
inline Flop operator-(Flop a) { return Flop(-a.v); }
inline Flop& operator+=(Flop& a, Flop b) { a = a + b; return a; }
inline Flop& operator-=(Flop& a, Flop b) { a = a - b; return a; }
inline Flop& operator*=(Flop& a, Flop b) { a = a * b; return a; }
inline Flop& operator/=(Flop& a, Flop b) { a = a / b; return a; }
inline bool operator<(Flop a, Flop b) { return a.v < b.v; }
inline bool operator>(Flop a, Flop b) { return a.v > b.v; }
inline bool operator<=(Flop a, Flop b) { return a.v <= b.v; }
inline bool operator>=(Flop a, Flop b) { return a.v >= b.v; }
inline bool operator==(Flop a, Flop b) { return a.v == b.v; }
inline bool operator!=(Flop a, Flop b) { return a.v != b.v; }
inline Flop osqrt(Flop x) { ++g_flops; return Flop(std::sqrt(x.v)); }
inline Flop omax(Flop a, Flop b) { return Flop(std::max(a.v, b.v)); }
inline Flop omin(Flop a, Flop b) { return Flop(std::min(a.v, b.v)); }

template <class R>
void e3_element_t(const or_common& c, const Topo& tp, int ires, int iprec, const R (*yl)[5],
                const R (*ycl)[5], const R (*acl)[5], const R (*xl)[3],
                R (*rl)[5], R (*rml)[5], R (*bdl)[5][5], const R (*ql)[12],
                R* EG) {
    const int nshl = tp.nshl, nenl = tp.nshl, ngauss = tp.ngauss;
    const R Rgas = c.Rgas, gamma = c.gamma, gamma1 = c.gamma1;

    for (int intp = 0; intp < ngauss; ++intp) {
        if (tp.Qwt[intp] == zero) continue;  // e3.f:110
        const double* shape = tp.shp[intp];
        const double (*shgl)[8] = tp.shgl[intp];
        R ri[20] = {0}, rmi[20] = {0};

        // ---------------- e3ivar.f:96-156 ----------------
        R dui[5] = {0, 0, 0, 0, 0};
        for (int n = 0; n < nshl; ++n)
            for (int k = 0; k < 5; ++k) dui[k] = dui[k] + shape[n] * yl[n][k];
        R rk = pt5 * (dui[1] * dui[1] + dui[2] * dui[2] + dui[3] * dui[3]);
        {   // getthm ithm=6 (getthm.f:103-148): pres=dui(1), T=dui(5)
            R rho6 = dui[0] / (Rgas * dui[4]);
            R ei6 = dui[4] * (Rgas / gamma1);
            dui[0] = rho6;
            dui[1] = rho6 * dui[1];
            dui[2] = rho6 * dui[2];
            dui[3] = rho6 * dui[3];
            dui[4] = rho6 * (ei6 + rk);
        }
        R pres = 0, u1 = 0, u2 = 0, u3 = 0, Tq = 0;
        for (int n = 0; n < nshl; ++n) {
            pres = pres + shape[n] * ycl[n][0];
            u1 = u1 + shape[n] * ycl[n][1];
            u2 = u2 + shape[n] * ycl[n][2];
            u3 = u3 + shape[n] * ycl[n][3];
            Tq = Tq + shape[n] * ycl[n][4];
        }
        R aci[5] = {0, 0, 0, 0, 0};
        for (int n = 0; n < nshl; ++n)
            for (int k = 0; k < 5; ++k) aci[k] = aci[k] + shape[n] * acl[n][k];
        rk = pt5 * (u1 * u1 + u2 * u2 + u3 * u3);
        // getthm ithm=7 (getthm.f:111, 148, 157-171)
        const R rho = pres / (Rgas * Tq);
        const R ei = Tq * (Rgas / gamma1);
        const R h = Tq * (Rgas * gamma / gamma1);
        const R cv = Rgas / gamma1;
        const R cp = Rgas * gamma / gamma1;
        const R alfap = one / Tq;
        const R betaT = one / pres;
        // getDiff (getdiff.f:127, 164, 171, 258-261): constant mu, Stokes, no eddy viscosity
        R rmu = c.rmu;
        R rlm = -pt66 * rmu;
        R con = rmu * cp / c.pr;
        const R xmut = 0.0;
        rlm = rlm - pt66 * xmut;
        rmu = rmu + xmut;
        const R rlm2mu = rlm + two * rmu;
        con = con + xmut * cp / c.pr;
        // e3metric (e3metric.f:22-77)
        R dxdxi[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int n = 0; n < nenl; ++n)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) dxdxi[i][j] = dxdxi[i][j] + xl[n][i] * shgl[j][n];
        R dxidx[3][3];
        dxidx[0][0] = dxdxi[1][1] * dxdxi[2][2] - dxdxi[2][1] * dxdxi[1][2];
        dxidx[0][1] = dxdxi[2][1] * dxdxi[0][2] - dxdxi[0][1] * dxdxi[2][2];
        dxidx[0][2] = dxdxi[0][1] * dxdxi[1][2] - dxdxi[0][2] * dxdxi[1][1];
        const R tmp = one / (dxidx[0][0] * dxdxi[0][0] + dxidx[0][1] * dxdxi[1][0] +
                                  dxidx[0][2] * dxdxi[2][0]);
        dxidx[0][0] = dxidx[0][0] * tmp;
        dxidx[0][1] = dxidx[0][1] * tmp;
        dxidx[0][2] = dxidx[0][2] * tmp;
        dxidx[1][0] = (dxdxi[1][2] * dxdxi[2][0] - dxdxi[1][0] * dxdxi[2][2]) * tmp;
        dxidx[1][1] = (dxdxi[0][0] * dxdxi[2][2] - dxdxi[2][0] * dxdxi[0][2]) * tmp;
        dxidx[1][2] = (dxdxi[1][0] * dxdxi[0][2] - dxdxi[0][0] * dxdxi[1][2]) * tmp;
        dxidx[2][0] = (dxdxi[1][0] * dxdxi[2][1] - dxdxi[1][1] * dxdxi[2][0]) * tmp;
        dxidx[2][1] = (dxdxi[2][0] * dxdxi[0][1] - dxdxi[0][0] * dxdxi[2][1]) * tmp;
        dxidx[2][2] = (dxdxi[0][0] * dxdxi[1][1] - dxdxi[0][1] * dxdxi[1][0]) * tmp;
        const R WdetJ = tp.Qwt[intp] / tmp;
        R shg[8][3];
        for (int n = 0; n < nshl; ++n)
            for (int i = 0; i < 3; ++i)
                shg[n][i] = shgl[0][n] * dxidx[0][i] + shgl[1][n] * dxidx[1][i] +
                            shgl[2][n] * dxidx[2][i];
        // global gradients of the (perturbed) yl (e3ivar.f:259-334)
        R g[3][5] = {{0}};
        for (int n = 0; n < nshl; ++n)
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 5; ++k) g[i][k] = g[i][k] + shg[n][i] * yl[n][k];

        // ---------------- e3mtrx.f:79-224 ----------------
        R A0[5][5] = {{0}}, A[3][5][5] = {{{0}}};
        const R drdp = rho * betaT;
        const R drdT = -rho * alfap;
        A0[4][0] = drdp * (h + rk) - alfap * Tq;
        const R e2p = A0[4][0] + one;
        const R e3p = rho * (h + rk);
        const R e4p = drdT * (h + rk) + rho * cp;
        A0[0][0] = drdp;
        A0[0][4] = drdT;
        A0[1][0] = drdp * u1; A0[1][1] = rho; A0[1][4] = drdT * u1;
        A0[2][0] = drdp * u2; A0[2][2] = rho; A0[2][4] = drdT * u2;
        A0[3][0] = drdp * u3; A0[3][3] = rho; A0[3][4] = drdT * u3;
        A0[4][1] = rho * u1; A0[4][2] = rho * u2; A0[4][3] = rho * u3; A0[4][4] = e4p;
        R (*A1)[5] = A[0], (*A2)[5] = A[1], (*A3)[5] = A[2];
        A1[0][0] = drdp * u1; A1[0][1] = rho; A1[0][4] = drdT * u1;
        A1[1][0] = drdp * u1 * u1 + 1; A1[1][1] = two * rho * u1; A1[1][4] = drdT * u1 * u1;
        A1[2][0] = drdp * u1 * u2; A1[2][1] = rho * u2; A1[2][2] = rho * u1; A1[2][4] = drdT * u1 * u2;
        A1[3][0] = drdp * u1 * u3; A1[3][1] = rho * u3; A1[3][3] = rho * u1; A1[3][4] = drdT * u1 * u3;
        A1[4][0] = u1 * e2p; A1[4][1] = e3p + rho * u1 * u1; A1[4][2] = rho * u1 * u2;
        A1[4][3] = rho * u1 * u3; A1[4][4] = u1 * e4p;
        A2[0][0] = drdp * u2; A2[0][2] = rho; A2[0][4] = drdT * u2;
        A2[1][0] = drdp * u1 * u2; A2[1][1] = rho * u2; A2[1][2] = rho * u1; A2[1][4] = drdT * u1 * u2;
        A2[2][0] = drdp * u2 * u2 + 1; A2[2][2] = two * rho * u2; A2[2][4] = drdT * u2 * u2;
        A2[3][0] = drdp * u2 * u3; A2[3][2] = rho * u3; A2[3][3] = rho * u2; A2[3][4] = drdT * u2 * u3;
        A2[4][0] = u2 * e2p; A2[4][1] = rho * u1 * u2; A2[4][2] = e3p + rho * u2 * u2;
        A2[4][3] = rho * u2 * u3; A2[4][4] = u2 * e4p;
        A3[0][0] = drdp * u3; A3[0][3] = rho; A3[0][4] = drdT * u3;
        A3[1][0] = drdp * u1 * u3; A3[1][1] = rho * u3; A3[1][3] = rho * u1; A3[1][4] = drdT * u1 * u3;
        A3[2][0] = drdp * u3 * u2; A3[2][2] = rho * u3; A3[2][3] = rho * u2; A3[2][4] = drdT * u3 * u2;
        A3[3][0] = drdp * u3 * u3 + 1; A3[3][3] = two * rho * u3; A3[3][4] = drdT * u3 * u3;
        A3[4][0] = u3 * e2p; A3[4][1] = rho * u1 * u3; A3[4][2] = rho * u2 * u3;
        A3[4][3] = e3p + rho * u3 * u3; A3[4][4] = u3 * e4p;

        // ---------------- e3conv.f:72-184 ----------------
        if (ires == 1 || ires == 3) {
            ri[0] = (-u1) * rho;
            ri[1] = (-u1) * rho * u1 - pres;
            ri[2] = (-u1) * rho * u2;
            ri[3] = (-u1) * rho * u3;
            ri[4] = (-u1) * rho * (ei + rk) - u1 * pres;
            ri[5] = (-u2) * rho;
            ri[6] = (-u2) * rho * u1;
            ri[7] = (-u2) * rho * u2 - pres;
            ri[8] = (-u2) * rho * u3;
            ri[9] = (-u2) * rho * (ei + rk) - u2 * pres;
            ri[10] = (-u3) * rho;
            ri[11] = (-u3) * rho * u1;
            ri[12] = (-u3) * rho * u2;
            ri[13] = (-u3) * rho * u3 - pres;
            ri[14] = (-u3) * rho * (ei + rk) - u3 * pres;
        }
        R rLyi[5];
        for (int k = 0; k < 5; ++k) {
            R s = 0.0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 5; ++j) s = s + A[i][k][j] * g[i][j];
            rLyi[k] = s;
        }
        if (ires == 2 || ires == 3)
            for (int k = 0; k < 5; ++k) rmi[15 + k] = rLyi[k];

        // ---------------- e3visc.f:278-368 (Navier == 1, rlsli == 0) ----------------
        if (c.Navier == 1) {
            const R (*g1)[5] = &g[0], (*g2)[5] = &g[1], (*g3)[5] = &g[2];
            (void)g1; (void)g2; (void)g3;
            const R* G1 = g[0]; const R* G2 = g[1]; const R* G3 = g[2];
            rmi[1] = rlm2mu * G1[1] + rlm * G2[2] + rlm * G3[3] - 0.0;
            rmi[2] = rmu * G1[2] + rmu * G2[1] - 0.0;
            rmi[3] = rmu * G1[3] + rmu * G3[1] - 0.0;
            rmi[4] = rlm2mu * u1 * G1[1] + rmu * u2 * G1[2] + rmu * u3 * G1[3] +
                     rmu * u2 * G2[1] + rlm * u1 * G2[2] + rmu * u3 * G3[1] +
                     rlm * u1 * G3[3] + con * G1[4];
            for (int k = 1; k < 5; ++k) ri[k] = ri[k] + rmi[k];
            rmi[6] = rmu * G1[2] + rmu * G2[1] - 0.0;
            rmi[7] = rlm * G1[1] + rlm2mu * G2[2] + rlm * G3[3] - 0.0;
            rmi[8] = rmu * G2[3] + rmu * G3[2] - 0.0;
            rmi[9] = rlm * u2 * G1[1] + rmu * u1 * G1[2] + rmu * u1 * G2[1] +
                     rlm2mu * u2 * G2[2] + rmu * u3 * G2[3] + rmu * u3 * G3[2] +
                     rlm * u2 * G3[3] + con * G2[4];
            for (int k = 6; k < 10; ++k) ri[k] = ri[k] + rmi[k];
            rmi[11] = rmu * G1[3] + rmu * G3[1] - 0.0;
            rmi[12] = rmu * G2[3] + rmu * G3[2] - 0.0;
            rmi[13] = rlm * G1[1] + rlm * G2[2] + rlm2mu * G3[3] - 0.0;
            rmi[14] = rlm * u3 * G1[1] + rmu * u1 * G1[3] + rlm * u3 * G2[2] +
                      rmu * u2 * G2[3] + rmu * u1 * G3[1] + rmu * u2 * G3[2] +
                      rlm2mu * u3 * G3[3] + con * G3[4];
            for (int k = 11; k < 15; ++k) ri[k] = ri[k] + rmi[k];
        }

        // ---------------- e3ls.f:96-143 ----------------
        const R fct1 = c.almi / c.gami / c.alfi * c.Dtgl;
        R rLymi[5] = {0, 0, 0, 0, 0};
        if (ires != 1)
            for (int k = 0; k < 5; ++k) rLymi[k] = rLyi[k] + fct1 * dui[k];
        if (ires == 1 || ires == 3)
            for (int k = 0; k < 5; ++k) {
                R s = rLyi[k];
                for (int j = 0; j < 5; ++j) s = s + A0[k][j] * aci[j];
                rLyi[k] = s;
            }
        // idiff >= 1: divergence of the reconstructed diffusive flux (e3ivar.f:363-395),
        // subtracted from the least-squares term (e3ls.f:147-156)
        if (ql && c.idiff >= 1 && (ires == 1 || ires == 3)) {
            R divqi[4] = {0, 0, 0, 0};
            for (int n = 0; n < nshl; ++n)
                for (int k = 0; k < 4; ++k)
                    divqi[k] = divqi[k] + shg[n][0] * ql[n][k] + shg[n][1] * ql[n][4 + k] + shg[n][2] * ql[n][8 + k];
            for (int k = 0; k < 4; ++k) rLyi[1 + k] = rLyi[1 + k] - divqi[k];
        }

        // ---------------- e3tau.f:140-181 (itau = 0) + e3gijd (e3tau.f:1397-1508) ----------------
        R gijd[6];
        if (tp.lcsyst >= 2) {
            // hexes and wedges: dxidx^T dxidx (e3tau.f:1408-1425)
            auto col = [&](int i, int j) {
                return dxidx[0][i] * dxidx[0][j] + dxidx[1][i] * dxidx[1][j] + dxidx[2][i] * dxidx[2][j];
            };
            gijd[0] = col(0, 0);
            gijd[1] = col(0, 1);
            gijd[2] = col(1, 1);
            gijd[3] = col(0, 2);
            gijd[4] = col(1, 2);
            gijd[5] = col(2, 2);
        } else {
            const R c1 = 1.259921049894873e+00, c2 = 6.299605249474365e-01;
            R t1, t2, t3;
            t1 = c1 * dxidx[0][0] + c2 * (dxidx[1][0] + dxidx[2][0]);
            t2 = c1 * dxidx[1][0] + c2 * (dxidx[0][0] + dxidx[2][0]);
            t3 = c1 * dxidx[2][0] + c2 * (dxidx[0][0] + dxidx[1][0]);
            gijd[0] = dxidx[0][0] * t1 + dxidx[1][0] * t2 + dxidx[2][0] * t3;
            t1 = c1 * dxidx[0][1] + c2 * (dxidx[1][1] + dxidx[2][1]);
            t2 = c1 * dxidx[1][1] + c2 * (dxidx[0][1] + dxidx[2][1]);
            t3 = c1 * dxidx[2][1] + c2 * (dxidx[0][1] + dxidx[1][1]);
            gijd[1] = dxidx[0][0] * t1 + dxidx[1][0] * t2 + dxidx[2][0] * t3;
            gijd[2] = dxidx[0][1] * t1 + dxidx[1][1] * t2 + dxidx[2][1] * t3;
            t1 = c1 * dxidx[0][2] + c2 * (dxidx[1][2] + dxidx[2][2]);
            t2 = c1 * dxidx[1][2] + c2 * (dxidx[0][2] + dxidx[2][2]);
            t3 = c1 * dxidx[2][2] + c2 * (dxidx[0][2] + dxidx[1][2]);
            gijd[3] = dxidx[0][0] * t1 + dxidx[1][0] * t2 + dxidx[2][0] * t3;
            gijd[4] = dxidx[0][1] * t1 + dxidx[1][1] * t2 + dxidx[2][1] * t3;
            gijd[5] = dxidx[0][2] * t1 + dxidx[1][2] * t2 + dxidx[2][2] * t3;
        }
        R tau[3];
        if (c.itau == 1) {
            // Diagonal-Franca (e3tau.f:54-139), iremoveStabTimeTerm = 0, ipord = 1
            R fact = gijd[0] * gijd[2] * gijd[5] - gijd[0] * gijd[4] * gijd[4] - gijd[2] * gijd[3] * gijd[3] -
                          gijd[5] * gijd[1] * gijd[1] + gijd[1] * gijd[3] * gijd[4] * two;
            R uh1 = u1 * u1 * (gijd[2] * gijd[5] - gijd[4] * gijd[4]) +
                         u2 * u2 * (gijd[0] * gijd[5] - gijd[3] * gijd[3]) +
                         u3 * u3 * (gijd[0] * gijd[2] - gijd[1] * gijd[1]) +
                         two * (u1 * u2 * (gijd[3] * gijd[4] - gijd[1] * gijd[5]) +
                                u1 * u3 * (gijd[1] * gijd[4] - gijd[3] * gijd[2]) +
                                u2 * u3 * (gijd[3] * gijd[1] - gijd[0] * gijd[4]));
            uh1 = two * osqrt(uh1 / fact);
            R h2o2u = u1 * u1 * gijd[0] + u2 * u2 * gijd[2] + u3 * u3 * gijd[5] +
                           (u1 * u2 * gijd[1] + u1 * u3 * gijd[3] + u2 * u3 * gijd[4]) * two + 1.0e-15;
            h2o2u = one / osqrt(h2o2u);
            fact = pt5 * rho * uh1 / rmu;
            tau[0] = pt5 * uh1 * omin(one, fact) * c.taucfct;
            const R dts = one / (c.Dtgl * c.dtsfct);
            tau[1] = omin(dts, h2o2u);
            tau[1] = tau[1] / rho;
            tau[2] = tau[1] / cv;
            fact = h2o2u * h2o2u * rk * pt66 / rmu;
            tau[1] = omin(tau[1], fact);
            tau[2] = omin(tau[2], fact * rmu / con) * c.temper;
        } else {
            const R fff = 36.0;  // ipord == 1
            const R dts = (c.iremoveStabTimeTerm == 1) ? zero : c.dtsfct * c.Dtgl;
            R t2 = rho * rho * ((two * dts) * (two * dts) +
                                     (u1 * (u1 * gijd[0] + two * (u2 * gijd[1] + u3 * gijd[3])) +
                                      u2 * (u2 * gijd[2] + two * u3 * gijd[4]) + u3 * u3 * gijd[5])) +
                        fff * (rmu * rmu) *
                            (gijd[0] * gijd[0] + gijd[2] * gijd[2] + gijd[5] * gijd[5] +
                             two * (gijd[1] * gijd[1] + gijd[3] * gijd[3] + gijd[4] * gijd[4]));
            const R fact = osqrt(t2);
            tau[0] = pt125 * fact / (rho * (gijd[0] + gijd[2] + gijd[5])) * c.taucfct;
            tau[1] = one / fact;
            tau[2] = tau[1] / cv * c.temper;
        }
        const R tauk[5] = {tau[0], tau[1], tau[1], tau[1], tau[2]};
        R rLyt[5];  // the least-squares residual before tau, for the DC factor (e3tau.f:183)
        for (int k = 0; k < 5; ++k) rLyt[k] = rLyi[k];
        if (ires == 1 || ires == 3)
            for (int k = 0; k < 5; ++k) rLyi[k] = tauk[k] * rLyi[k];
        if (ires != 1)
            for (int k = 0; k < 5; ++k) rLymi[k] = tauk[k] * rLymi[k];

        // ---------------- e3ls.f:231-459: A_i (tau L) ----------------
        if (ires != 1)
            for (int r = 0; r < 15; ++r) {
                const int i = r / 5, row = r % 5;
                R s = 0.0;
                for (int j = 0; j < 5; ++j) s = s + A[i][row][j] * rLymi[j];
                rmi[r] = s + rmi[r];
            }
        if (ires == 1 || ires == 3)
            for (int r = 0; r < 15; ++r) {
                const int i = r / 5, row = r % 5;
                R s = 0.0;
                for (int j = 0; j < 5; ++j) s = s + A[i][row][j] * rLyi[j];
                ri[r] = s + ri[r];
            }

        // ---------------- discontinuity capturing (e3.f:217-222), iDC != 0 ----------------
        if (c.iDC != 0) {
            // A0DC, A0inv and dV/dY (e3mtrx.f:232-297); e3mtrx's local cv
            const R s1 = one / (rho * rho * betaT * Tq);
            const R cvd = cp - (alfap * alfap * Tq / rho / betaT);
            const R A0DC[4] = {(rho * betaT) * (rho * betaT) * s1, -(rho * alfap * rho * betaT * s1), rho / Tq,
                                    (-(rho * alfap)) * (-(rho * alfap)) * s1 + (rho * cvd / (Tq * Tq))};
            R A0inv[15];
            {
                const R fact1 = one / (rho * cvd * (Tq * Tq));
                const R d = alfap * Tq / rho / betaT;
                const R e1bar = h - rk;
                const R e2bar = e1bar - d;
                const R e3bar = e2bar - cvd * Tq;
                const R e5bar = e1bar * e1bar - 2 * e1bar * d + 2 * rk * cvd * Tq + cp * Tq / rho / betaT;
                const R c1bar = u1 * u1 + cvd * Tq, c2bar = u2 * u2 + cvd * Tq, c3bar = u3 * u3 + cvd * Tq;
                A0inv[0] = e5bar * fact1;
                A0inv[1] = c1bar * fact1;
                A0inv[2] = c2bar * fact1;
                A0inv[3] = c3bar * fact1;
                A0inv[4] = 1 * fact1;
                A0inv[5] = u1 * e3bar * fact1;
                A0inv[6] = u2 * e3bar * fact1;
                A0inv[7] = u3 * e3bar * fact1;
                A0inv[8] = -e2bar * fact1;
                A0inv[9] = u1 * u2 * fact1;
                A0inv[10] = u3 * u1 * fact1;
                A0inv[11] = -u1 * fact1;
                A0inv[12] = u2 * u3 * fact1;
                A0inv[13] = -u2 * fact1;
                A0inv[14] = -u3 * fact1;
            }
            R dV[15];
            {
                const R fact1 = 1 / Tq, fact2 = fact1 / Tq;
                dV[0] = fact1 / rho; dV[1] = -fact1 * u1; dV[2] = fact1; dV[3] = -fact1 * u2; dV[4] = zero;
                dV[5] = fact1; dV[6] = -fact1 * u3; dV[7] = zero; dV[8] = zero; dV[9] = fact1;
                dV[10] = -(h - rk) * fact2; dV[11] = -fact2 * u1; dV[12] = -fact2 * u2; dV[13] = -fact2 * u3;
                dV[14] = fact2;
            }
            // rTLS = (Ly - S) tau~ (Ly - S) with rLyi tau-scaled for ires 1, 3 and unscaled for
            // ires 2; raLS = (Ly - S) A0^-1 (Ly - S) (e3tau.f:193-237)
            const R* L = rLyi;
            const R* T0 = rLyt;
            const R rTLS = T0[0] * (L[0] * dV[0] + dV[1] * L[1] + dV[3] * L[2] + L[3] * dV[6] + dV[10] * L[4]) +
                                T0[1] * (L[1] * dV[2] + L[2] * dV[4] + dV[7] * L[3] + L[4] * dV[11]) +
                                T0[2] * (L[2] * dV[5] + dV[8] * L[3] + dV[12] * L[4]) +
                                T0[3] * (L[3] * dV[9] + dV[13] * L[4]) + T0[4] * (dV[14] * L[4]);
            const R raLS = two * T0[3] * T0[4] * A0inv[14] + two * T0[2] * T0[4] * A0inv[13] +
                                two * T0[0] * T0[1] * A0inv[5] + two * T0[1] * T0[2] * A0inv[9] +
                                two * T0[1] * T0[3] * A0inv[10] + two * T0[0] * T0[2] * A0inv[6] +
                                two * T0[2] * T0[3] * A0inv[12] + two * T0[1] * T0[4] * A0inv[11] +
                                two * T0[0] * T0[3] * A0inv[7] + two * T0[0] * T0[4] * A0inv[8] +
                                T0[0] * T0[0] * A0inv[0] + T0[1] * T0[1] * A0inv[1] + T0[2] * T0[2] * A0inv[2] +
                                T0[3] * T0[3] * A0inv[3] + T0[4] * T0[4] * A0inv[4];
            // inverse of the tau metric, order (11, 22, 33, 12, 13, 23) (e3tau.f:241-260)
            const R gu[6] = {gijd[0], gijd[2], gijd[5], gijd[1], gijd[3], gijd[4]};
            const R detI = one / (gu[0] * gu[1] * gu[2] - gu[0] * gu[5] * gu[5] - gu[3] * gu[3] * gu[2] +
                                       gu[3] * gu[4] * gu[5] * two - gu[4] * gu[4] * gu[1]);
            const R gi[6] = {detI * (gu[1] * gu[2] - gu[5] * gu[5]), detI * (gu[0] * gu[2] - gu[4] * gu[4]),
                                  detI * (gu[0] * gu[1] - gu[3] * gu[3]), detI * (gu[4] * gu[5] - gu[3] * gu[2]),
                                  detI * (gu[3] * gu[5] - gu[4] * gu[1]), detI * (gu[3] * gu[4] - gu[0] * gu[5])};
            // e3dc.f:55-240: A0 Y,j, g^ij A0 Y,j and Y,i A0DC Y,j
            R A0g[15];
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 5; ++k)
                    A0g[5 * j + k] = A0[k][0] * g[j][0] + A0[k][1] * g[j][1] + A0[k][2] * g[j][2] +
                                     A0[k][3] * g[j][3] + A0[k][4] * g[j][4];
            R gA[15];
            for (int k = 0; k < 5; ++k) {
                gA[k] = gi[0] * A0g[k] + gi[3] * A0g[5 + k] + gi[4] * A0g[10 + k];
                gA[5 + k] = gi[3] * A0g[k] + gi[1] * A0g[5 + k] + gi[5] * A0g[10 + k];
                gA[10 + k] = gi[4] * A0g[k] + gi[5] * A0g[5 + k] + gi[2] * A0g[10 + k];
            }
            auto yy = [&](const R* a) {
                return A0DC[0] * (a[0] * a[0]) + two * a[0] * A0DC[1] * a[4] + A0DC[2] * (a[1] * a[1]) +
                       A0DC[2] * (a[2] * a[2]) + A0DC[2] * (a[3] * a[3]) + A0DC[3] * (a[4] * a[4]);
            };
            auto yx = [&](const R* a, const R* b) {
                return a[0] * A0DC[0] * b[0] + a[0] * A0DC[1] * b[4] + a[1] * A0DC[2] * b[1] +
                       a[2] * A0DC[2] * b[2] + a[3] * A0DC[2] * b[3] + a[4] * A0DC[1] * b[0] + a[4] * A0DC[3] * b[4];
            };
            const R y1 = yy(g[0]), y2 = yy(g[1]), y3 = yy(g[2]);
            const R y4 = yx(g[0], g[1]), y5 = yx(g[0], g[2]), y6 = yx(g[1], g[2]);
            const R gnorm = one / (gi[0] * y1 + two * gi[3] * y4 + two * gi[4] * y5 + gi[1] * y2 +
                                        two * gi[5] * y6 + gi[2] * y3 + c.epsM);
            R DC = 0.0;  // ipord = 1: fact = 1
            if (c.iDC == 1) DC = omax(zero, osqrt(raLS * gnorm) - rTLS * gnorm);
            if (c.iDC == 2) DC = two * rTLS * gnorm;
            if (c.iDC == 3) DC = omin(omax(zero, osqrt(raLS * gnorm) - rTLS * gnorm), two * rTLS * gnorm);
            if (ires == 1 || ires == 3) {
                for (int r = 0; r < 15; ++r) {
                    ri[r] = ri[r] + DC * gA[r];
                    // the reference's update of rmi(:,11) reads rmi(:,12) (e3dc.f:366)
                    rmi[r] = (r == 10) ? rmi[11] + DC * gA[11] : rmi[r] + DC * gA[r];
                }
            } else if (ires == 2) {
                for (int r = 0; r < 15; ++r) rmi[r] = rmi[r] + DC * gA[r];
            }
        }

        // ---------------- e3massr.f:26-88 ----------------
        if (ires == 1 || ires == 3)
            for (int k = 0; k < 5; ++k) {
                R s = ri[15 + k];
                for (int j = 0; j < 5; ++j) s = s + A0[k][j] * aci[j];
                ri[15 + k] = s;
            }
        if (ires != 1)
            for (int k = 0; k < 5; ++k) rmi[15 + k] = rmi[15 + k] + fct1 * dui[k];

        // ---------------- lhs = 1: element tangent EG[nedof][nedof], nedof = 5 nshl ----------------
        if (EG) {
            const int nedof = 5 * nshl;
            auto E = [&](int r, int cc) -> R& { return EG[(size_t)r * nedof + cc]; };
            // e3conv.f:186-260: N_a (A_i N_b,i)
            for (int j = 0; j < nshl; ++j) {
                const R f1 = WdetJ * shg[j][0], f2 = WdetJ * shg[j][1], f3 = WdetJ * shg[j][2];
                R AiNbi[5][5];
                for (int r = 0; r < 5; ++r)
                    for (int cc = 0; cc < 5; ++cc) AiNbi[r][cc] = f1 * A1[r][cc] + f2 * A2[r][cc] + f3 * A3[r][cc];
                for (int i = 0; i < nshl; ++i)
                    for (int cc = 0; cc < 5; ++cc)
                        for (int r = 0; r < 5; ++r) E(5 * i + r, 5 * j + cc) = E(5 * i + r, 5 * j + cc) + shape[i] * AiNbi[r][cc];
            }
            // stiff(15,15): e3visc.f:65-127 (diffusivity K_ij), then e3ls.f:464-702 (A_i tau A_j)
            R stiff[15][15] = {{0}};
            if (c.Navier == 1) {
                const R uu[3] = {u1, u2, u3};
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        R (*K)[15] = stiff;
                        const int ri = 5 * i, cj = 5 * j;
                        for (int m = 0; m < 3; ++m)
                            for (int n = 0; n < 3; ++n) {
                                R v = 0.0;
                                if (i == j && m == n) v = (m == i) ? rlm2mu : rmu;
                                else if (i != j && m == i && n == j) v = rlm;
                                else if (i != j && m == j && n == i) v = rmu;
                                if (v != 0.0) K[ri + 1 + m][cj + 1 + n] = v;
                            }
                        // energy row: u_m times the momentum rows
                        for (int n = 0; n < 3; ++n) {
                            R v = 0.0;
                            if (i == j) v = ((n == i) ? rlm2mu : rmu) * uu[n];
                            else if (n == j) v = rlm * uu[i];
                            else if (n == i) v = rmu * uu[j];
                            if (i == j || n == j || n == i) K[ri + 4][cj + 1 + n] = v;
                        }
                        if (i == j) K[ri + 4][cj + 4] = con;
                    }
            }
            R AtA0[3][5][5];
            for (int i = 0; i < 3; ++i) {
                R Atau[5][5];
                for (int r = 0; r < 5; ++r)
                    for (int k = 0; k < 5; ++k) Atau[r][k] = A[i][r][k] * tauk[k];
                for (int cc = 0; cc < 5; ++cc)
                    for (int r = 0; r < 5; ++r)
                        AtA0[i][r][cc] = Atau[r][0] * A0[0][cc] + Atau[r][1] * A0[1][cc] + Atau[r][2] * A0[2][cc] +
                                         Atau[r][3] * A0[3][cc] + Atau[r][4] * A0[4][cc];
                for (int j = 0; j < 3; ++j)
                    for (int cc = 0; cc < 5; ++cc)
                        for (int r = 0; r < 5; ++r)
                            stiff[5 * i + r][5 * j + cc] =
                                stiff[5 * i + r][5 * j + cc] +
                                (Atau[r][0] * A[j][0][cc] + Atau[r][1] * A[j][1][cc] + Atau[r][2] * A[j][2][cc] +
                                 Atau[r][3] * A[j][3][cc] + Atau[r][4] * A[j][4][cc]);
            }
            // e3ls.f:703-766: least-squares time term N_a,i A_i tau A0 N_b
            for (int i = 0; i < nshl; ++i) {
                R At[5][5];
                for (int r = 0; r < 5; ++r)
                    for (int cc = 0; cc < 5; ++cc)
                        At[r][cc] = shg[i][0] * AtA0[0][r][cc] + shg[i][1] * AtA0[1][r][cc] + shg[i][2] * AtA0[2][r][cc];
                for (int j = 0; j < nshl; ++j) {
                    const R fact = shape[j] * WdetJ * c.almi / c.gami / c.alfi * c.Dtgl;
                    for (int r = 0; r < 5; ++r)
                        for (int cc = 0; cc < 5; ++cc) E(5 * i + r, 5 * j + cc) = E(5 * i + r, 5 * j + cc) + fact * At[r][cc];
                }
            }
            // e3massl.f:1-75 (bcool = 0): N_a N_b fct A0
            {
                const R temp = WdetJ * c.almi / c.gami / c.alfi * c.Dtgl;
                for (int j = 0; j < nshl; ++j)
                    for (int i = 0; i < nshl; ++i) {
                        const R f = (shape[i] * shape[j]) * (temp + 0.0);
                        for (int cc = 0; cc < 5; ++cc)
                            for (int r = 0; r < 5; ++r) E(5 * i + r, 5 * j + cc) = E(5 * i + r, 5 * j + cc) + f * A0[r][cc];
                    }
            }
            // e3wmlt.f (lhs part): N_a,i stiff_ij N_b,j
            for (int j = 0; j < nshl; ++j) {
                const R g1 = WdetJ * shg[j][0], g2 = WdetJ * shg[j][1], g3 = WdetJ * shg[j][2];
                R st[3][5][5];
                for (int cc = 0; cc < 5; ++cc)
                    for (int r = 0; r < 5; ++r)
                        for (int b = 0; b < 3; ++b)
                            st[b][r][cc] = g1 * stiff[5 * b + r][cc] + g2 * stiff[5 * b + r][5 + cc] +
                                           g3 * stiff[5 * b + r][10 + cc];
                for (int i = 0; i < nshl; ++i)
                    for (int cc = 0; cc < 5; ++cc)
                        for (int r = 0; r < 5; ++r)
                            E(5 * i + r, 5 * j + cc) = E(5 * i + r, 5 * j + cc) + shg[i][0] * st[0][r][cc] +
                                                       shg[i][1] * st[1][r][cc] + shg[i][2] * st[2][r][cc];
            }
        }

        // ---------------- e3bdg.f (iprec == 1, lhs != 1, itau < 10) ----------------
        if (iprec == 1 && bdl && !EG) {
            // convective, non-integrated-by-parts: N_b A_i N_b,i  (e3bdg.f:37-189)
            for (int j = 0; j < nshl; ++j) {
                const R t = shape[j] * WdetJ;
                for (int r = 0; r < 5; ++r)
                    for (int cc = 0; cc < 5; ++cc)
                        bdl[j][r][cc] = bdl[j][r][cc] +
                                        t * (shg[j][0] * A1[r][cc] + shg[j][1] * A2[r][cc] +
                                             shg[j][2] * A3[r][cc]);
            }
            // mass (e3bdg.f:219-246), bcool = 0
            {
                const R ff = c.almi / c.gami / c.alfi;
                const R t = WdetJ * (c.Dtgl * ff + 0.0);
                for (int j = 0; j < nshl; ++j) {
                    const R t2 = (shape[j] * shape[j]) * t;
                    for (int r = 0; r < 5; ++r)
                        for (int cc = 0; cc < 5; ++cc) bdl[j][r][cc] = bdl[j][r][cc] + t2 * A0[r][cc];
                }
            }
            // least-squares time term N_a,i A_i tau A0 (e3bdg.f:254-342)
            if (c.ivart >= 2) {
                R AtA0[3][5][5];
                for (int i = 0; i < 3; ++i) {
                    R Atau[5][5];
                    for (int r = 0; r < 5; ++r)
                        for (int k = 0; k < 5; ++k) Atau[r][k] = A[i][r][k] * tauk[k];
                    for (int cc = 0; cc < 5; ++cc)
                        for (int r = 0; r < 5; ++r)
                            AtA0[i][r][cc] = Atau[r][0] * A0[0][cc] + Atau[r][1] * A0[1][cc] +
                                             Atau[r][2] * A0[2][cc] + Atau[r][3] * A0[3][cc] +
                                             Atau[r][4] * A0[4][cc];
                }
                for (int a = 0; a < nshl; ++a) {
                    const R t1 = shape[a] * WdetJ * c.almi / c.gami / c.alfi * c.Dtgl;
                    for (int r = 0; r < 5; ++r)
                        for (int cc = 0; cc < 5; ++cc)
                            bdl[a][r][cc] = bdl[a][r][cc] +
                                            t1 * (shg[a][0] * AtA0[0][r][cc] + shg[a][1] * AtA0[1][r][cc] +
                                                  shg[a][2] * AtA0[2][r][cc]);
                }
            }
            // stiffness: N_a,p (A_p tau A_q + K_pq) N_a,q  (e3bdg.f:346-2590)
            const int blocks[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
            for (int b = 0; b < 6; ++b) {
                const int p = blocks[b][0], q = blocks[b][1];
                const R (*Ap)[5] = A[p];
                const R (*Aq)[5] = A[q];
                R M[5][5];
                if (c.ivart >= 2) {
                    for (int r = 0; r < 5; ++r)
                        for (int cc = 0; cc < 5; ++cc) {
                            if (p == q) {
                                M[r][cc] = tau[0] * Ap[r][0] * Ap[0][cc] +
                                           tau[1] * (Ap[r][1] * Ap[1][cc] + Ap[r][2] * Ap[2][cc] +
                                                     Ap[r][3] * Ap[3][cc]) +
                                           tau[2] * Ap[r][4] * Ap[4][cc];
                            } else {
                                M[r][cc] = tau[0] * (Ap[r][0] * Aq[0][cc] + Aq[r][0] * Ap[0][cc]) +
                                           tau[1] * (Ap[r][1] * Aq[1][cc] + Ap[r][2] * Aq[2][cc] +
                                                     Ap[r][3] * Aq[3][cc] + Aq[r][1] * Ap[1][cc] +
                                                     Aq[r][2] * Ap[2][cc] + Aq[r][3] * Ap[3][cc]) +
                                           tau[2] * (Ap[r][4] * Aq[4][cc] + Aq[r][4] * Ap[4][cc]);
                            }
                        }
                } else {
                    std::memset(M, 0, sizeof(M));
                }
                if (c.Navier == 1) {
                    const R uu[3] = {u1, u2, u3};
                    if (p == q) {
                        // diagonal: rlm2mu on the p-th momentum row, rmu on the others
                        for (int d = 0; d < 3; ++d) {
                            const R coef = (d == p) ? rlm2mu : rmu;
                            M[1 + d][1 + d] = M[1 + d][1 + d] + coef;
                        }
                        for (int d = 0; d < 3; ++d) {
                            const R coef = (d == p) ? rlm2mu : rmu;
                            M[4][1 + d] = M[4][1 + d] + coef * uu[d];
                        }
                        M[4][4] = M[4][4] + con;
                    } else {
                        // off-diagonal pair (p,q): rlm2mu - rmu = rlm + rmu
                        M[1 + p][1 + q] = M[1 + p][1 + q] + rlm2mu - rmu;
                        M[1 + q][1 + p] = M[1 + q][1 + p] + rlm2mu - rmu;
                        M[4][1 + p] = M[4][1 + p] + (rlm2mu - rmu) * uu[q];
                        M[4][1 + q] = M[4][1 + q] + (rlm2mu - rmu) * uu[p];
                    }
                }
                for (int j = 0; j < nshl; ++j) {
                    const R t = WdetJ * shg[j][p] * shg[j][q];
                    for (int r = 0; r < 5; ++r)
                        for (int cc = 0; cc < 5; ++cc) bdl[j][r][cc] = bdl[j][r][cc] + t * M[r][cc];
                }
            }
        }

        // ---------------- e3wmlt.f:72-145 ----------------
        if (ires == 1 || ires == 3)
            for (int i = 0; i < nshl; ++i)
                for (int k = 0; k < 5; ++k)
                    rl[i][k] = rl[i][k] + WdetJ * (shg[i][0] * ri[k] + shg[i][1] * ri[5 + k] +
                                                   shg[i][2] * ri[10 + k]);
        if (ires == 2 || ires == 3)
            for (int i = 0; i < nshl; ++i)
                for (int k = 0; k < 5; ++k)
                    rml[i][k] = rml[i][k] + WdetJ * (shg[i][0] * rmi[k] + shg[i][1] * rmi[5 + k] +
                                                     shg[i][2] * rmi[10 + k] + shape[i] * rmi[15 + k]);
        if (ires == 1 || ires == 3)  // temporal term (adds exact zeros when ires == 2)
            for (int i = 0; i < nshl; ++i)
                for (int k = 0; k < 5; ++k) rl[i][k] = rl[i][k] + shape[i] * WdetJ * ri[15 + k];
    }
}

void e3_element(const or_common& c, const Topo& tp, int ires, int iprec, const double (*yl)[5],
                const double (*ycl)[5], const double (*acl)[5], const double (*xl)[3],
                double (*rl)[5], double (*rml)[5], double (*bdl)[5][5], const double (*ql)[12] = nullptr,
                double* EG = nullptr) {
    e3_element_t<double>(c, tp, ires, iprec, yl, ycl, acl, xl, rl, rml, bdl, ql, EG);
}

// ---------------------------------------------------------------------------
// e3b.f + e3bvar.f for one boundary element of topology bt (ires 1/3): the state at a point
// from the face nodes, the metric and gradients from all nodes, the normal by e3bvar.f:156-176
// and the weight by e3bvar.f:184-197 for each boundary topology
// ---------------------------------------------------------------------------
void e3b_element(const or_common& c, const BTopo& bt, const double (*yl)[5], int iBCB, const double (*BCB)[6],
                 const double (*xlb)[3], double (*rl)[5]) {
    const double Rgas = c.Rgas, gamma = c.gamma, gamma1 = c.gamma1;
    const int nshlb = bt.nshlb, nshl = bt.nshl, nenl = bt.nshl;
    const int* lnode = bt.lnode;
    for (int intp = 0; intp < bt.ngaussb; ++intp) {
        if (bt.Qwtb[intp] == zero) continue;
        const double* shpb = bt.shpb[intp];
        const double (*shglb)[8] = bt.shglb[intp];
        // e3bvar.f:100-121
        double pres = 0, u1 = 0, u2 = 0, u3 = 0, Tq = 0;
        for (int n = 0; n < nshlb; ++n) {
            const int l = lnode[n];
            pres = pres + shpb[l] * yl[l][0];
            u1 = u1 + shpb[l] * yl[l][1];
            u2 = u2 + shpb[l] * yl[l][2];
            u3 = u3 + shpb[l] * yl[l][3];
            Tq = Tq + shpb[l] * yl[l][4];
        }
        const double rk = pt5 * (u1 * u1 + u2 * u2 + u3 * u3);
        const double rho = pres / (Rgas * Tq);
        const double ei = Tq * (Rgas / gamma1);
        const double cp = Rgas * gamma / gamma1;
        // metrics (e3bvar.f:139-199)
        double dx[3][3] = {{0}};
        for (int n = 0; n < nenl; ++n)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) dx[i][j] = dx[i][j] + xlb[n][i] * shglb[j][n];
        double t1, t2, t3;
        if (bt.lcsyst == 4) {
            t1 = dx[1][0] * dx[2][2] - dx[1][2] * dx[2][0];
            t2 = dx[2][0] * dx[0][2] - dx[2][2] * dx[0][0];
            t3 = dx[0][0] * dx[1][2] - dx[0][2] * dx[1][0];
        } else {
            double v1[3], v2[3];
            for (int i = 0; i < 3; ++i) { v1[i] = xlb[1][i] - xlb[0][i]; v2[i] = xlb[2][i] - xlb[0][i]; }
            if (bt.lcsyst == 1) {
                t1 = v1[1] * v2[2] - v2[1] * v1[2];
                t2 = v2[0] * v1[2] - v1[0] * v2[2];
                t3 = v1[0] * v2[1] - v2[0] * v1[1];
            } else {
                t1 = -v1[1] * v2[2] + v2[1] * v1[2];
                t2 = -v2[0] * v1[2] + v1[0] * v2[2];
                t3 = -v1[0] * v2[1] + v2[0] * v1[1];
            }
        }
        double temp = one / std::sqrt(t1 * t1 + t2 * t2 + t3 * t3);
        const double bn[3] = {t1 * temp, t2 * temp, t3 * temp};
        double WdetJb;
        if (bt.lcsyst == 3) WdetJb = (one - bt.Qwtb[intp]) / (four * temp);
        else if (bt.lcsyst == 4) WdetJb = bt.Qwtb[intp] / temp;
        else WdetJb = bt.Qwtb[intp] / (four * temp);
        double g[3][5] = {{0}};
        if (c.Navier == 1) {
            double di[3][3];
            di[0][0] = dx[1][1] * dx[2][2] - dx[2][1] * dx[1][2];
            di[0][1] = dx[2][1] * dx[0][2] - dx[0][1] * dx[2][2];
            di[0][2] = dx[0][1] * dx[1][2] - dx[0][2] * dx[1][1];
            temp = one / (di[0][0] * dx[0][0] + di[0][1] * dx[1][0] + di[0][2] * dx[2][0]);
            di[0][0] = di[0][0] * temp;
            di[0][1] = di[0][1] * temp;
            di[0][2] = di[0][2] * temp;
            di[1][0] = (dx[1][2] * dx[2][0] - dx[1][0] * dx[2][2]) * temp;
            di[1][1] = (dx[0][0] * dx[2][2] - dx[2][0] * dx[0][2]) * temp;
            di[1][2] = (dx[1][0] * dx[0][2] - dx[0][0] * dx[1][2]) * temp;
            di[2][0] = (dx[1][0] * dx[2][1] - dx[1][1] * dx[2][0]) * temp;
            di[2][1] = (dx[2][0] * dx[0][1] - dx[0][0] * dx[2][1]) * temp;
            di[2][2] = (dx[0][0] * dx[1][1] - dx[0][1] * dx[1][0]) * temp;
            double gl[3][5] = {{0}};
            for (int n = 0; n < nshl; ++n)
                for (int i = 0; i < 3; ++i)
                    for (int k = 0; k < 5; ++k) gl[i][k] = gl[i][k] + shglb[i][n] * yl[n][k];
            for (int k = 1; k < 5; ++k)
                for (int i = 0; i < 3; ++i)
                    g[i][k] = di[0][i] * gl[0][k] + di[1][i] * gl[1][k] + di[2][i] * gl[2][k];
        }
        double rou = 0, p = 0;
        for (int n = 0; n < nshlb; ++n) {
            rou = rou + shpb[lnode[n]] * BCB[n][0];
            p = p + shpb[lnode[n]] * BCB[n][1];
        }
        double Fv2 = 0, Fv3 = 0, Fv4 = 0, Fh5 = 0;
        if (c.Navier == 1)
            for (int n = 0; n < nshlb; ++n) {
                Fv2 = Fv2 + shpb[lnode[n]] * BCB[n][2];
                Fv3 = Fv3 + shpb[lnode[n]] * BCB[n][3];
                Fv4 = Fv4 + shpb[lnode[n]] * BCB[n][4];
                Fh5 = Fh5 + shpb[lnode[n]] * BCB[n][5];
            }
        // e3b.f:134-166
        double un;
        if (!(iBCB & 1)) {
            un = bn[0] * u1 + bn[1] * u2 + bn[2] * u3;
            rou = rho * (un);
        } else {
            un = (rou / rho);
        }
        if (!(iBCB & 2)) p = pres;
        double F1 = rou;
        double F2 = rou * u1 + bn[0] * p;
        double F3 = rou * u2 + bn[1] * p;
        double F4 = rou * u3 + bn[2] * p;
        double F5 = rou * (ei + rk) + un * p;
        if (c.Navier == 1) {
            // getDiff with the boundary T, cp
            double rmu = c.rmu;
            double rlm = -pt66 * rmu;
            double con = rmu * cp / c.pr;
            const double rlm2mu = rlm + two * rmu;
            const double* G1 = g[0]; const double* G2 = g[1]; const double* G3 = g[2];
            const double tau1n = bn[0] * (rlm2mu * G1[1] + rlm * G2[2] + rlm * G3[3]) +
                                 bn[1] * (rmu * (G2[1] + G1[2])) + bn[2] * (rmu * (G3[1] + G1[3]));
            const double tau2n = bn[0] * (rmu * (G2[1] + G1[2])) +
                                 bn[1] * (rlm * G1[1] + rlm2mu * G2[2] + rlm * G3[3]) +
                                 bn[2] * (rmu * (G3[2] + G2[3]));
            const double tau3n = bn[0] * (rmu * (G3[1] + G1[3])) + bn[1] * (rmu * (G3[2] + G2[3])) +
                                 bn[2] * (rlm * G1[1] + rlm * G2[2] + rlm2mu * G3[3]);
            if (!(iBCB & 4)) { Fv2 = tau1n; Fv3 = tau2n; Fv4 = tau3n; }
            const double Fv5 = u1 * Fv2 + u2 * Fv3 + u3 * Fv4;
            const double heat = -con * (bn[0] * G1[4] + bn[1] * G2[4] + bn[2] * G3[4]);
            if (!(iBCB & 8)) Fh5 = heat;
            F2 = F2 - Fv2;
            F3 = F3 - Fv3;
            F4 = F4 - Fv4;
            F5 = F5 - Fv5 + Fh5;
        }
        // e3b.f:224-241
        for (int n = 0; n < nshlb; ++n) {
            const int l = lnode[n];
            const double w = WdetJb * shpb[l];
            rl[l][0] = rl[l][0] + w * F1;
            rl[l][1] = rl[l][1] + w * F2;
            rl[l][2] = rl[l][2] + w * F3;
            rl[l][3] = rl[l][3] + w * F4;
            rl[l][4] = rl[l][4] + w * F5;
        }
    }
}

// localy gather (localy.f:48-73): global (u,v,w,p,T) -> local (p,u,v,w,T)
inline void gather_y(const double* y, int nshg, int node, double out[5]) {
    out[0] = y[3 * (size_t)nshg + node];
    out[1] = y[0 * (size_t)nshg + node];
    out[2] = y[1 * (size_t)nshg + node];
    out[3] = y[2 * (size_t)nshg + node];
    out[4] = y[4 * (size_t)nshg + node];
}
inline void gather_x(const double* x, int nshg, int node, double out[3]) {
    for (int d = 0; d < 3; ++d) out[d] = x[d * (size_t)nshg + node];
}

template <class F>
void parallel_for(int n, int nthreads, F&& f) {
    if (nthreads <= 1 || n < 2) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    nthreads = std::min(nthreads, n);
    std::vector<std::thread> th;
    th.reserve(nthreads);
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t]() {
            for (int i = t; i < n; i += nthreads) f(i);
        });
    for (auto& x : th) x.join();
}

// e3q.f:54-191 with e3qvar.f (idiff = 1) for one element: ql(a,1:12) += N_a WdetJ qdi,
// rmassl(a) += N_a WdetJ, qdi the viscous flux at the point
void e3q_element(const or_common& c, const Topo& tp, const double (*ycl)[5], const double (*xl)[3],
                 double (*ql)[12], double* rmassl) {
    const int nshl = tp.nshl, nenl = tp.nshl;
    for (int intp = 0; intp < tp.ngauss; ++intp) {
        if (tp.Qwt[intp] == zero) continue;
        const double* shape = tp.shp[intp];
        const double (*shgl)[8] = tp.shgl[intp];
        double u1 = 0, u2 = 0, u3 = 0;
        for (int n = 0; n < nshl; ++n) {
            u1 = u1 + shape[n] * ycl[n][1];
            u2 = u2 + shape[n] * ycl[n][2];
            u3 = u3 + shape[n] * ycl[n][3];
        }
        // getthm ithm = 7: cp; getDiff: constant mu, Stokes (getdiff.f:127,164,171)
        const double cp = c.Rgas * c.gamma / c.gamma1;
        const double rmu = c.rmu, rlm = -pt66 * rmu, rlm2mu = rlm + two * rmu, con = rmu * cp / c.pr;
        // e3metric.f:22-77
        double dxdxi[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int n = 0; n < nenl; ++n)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) dxdxi[i][j] = dxdxi[i][j] + xl[n][i] * shgl[j][n];
        double dxidx[3][3];
        dxidx[0][0] = dxdxi[1][1] * dxdxi[2][2] - dxdxi[2][1] * dxdxi[1][2];
        dxidx[0][1] = dxdxi[2][1] * dxdxi[0][2] - dxdxi[0][1] * dxdxi[2][2];
        dxidx[0][2] = dxdxi[0][1] * dxdxi[1][2] - dxdxi[0][2] * dxdxi[1][1];
        const double tmp = one / (dxidx[0][0] * dxdxi[0][0] + dxidx[0][1] * dxdxi[1][0] +
                                  dxidx[0][2] * dxdxi[2][0]);
        dxidx[0][0] = dxidx[0][0] * tmp;
        dxidx[0][1] = dxidx[0][1] * tmp;
        dxidx[0][2] = dxidx[0][2] * tmp;
        dxidx[1][0] = (dxdxi[1][2] * dxdxi[2][0] - dxdxi[1][0] * dxdxi[2][2]) * tmp;
        dxidx[1][1] = (dxdxi[0][0] * dxdxi[2][2] - dxdxi[2][0] * dxdxi[0][2]) * tmp;
        dxidx[1][2] = (dxdxi[1][0] * dxdxi[0][2] - dxdxi[0][0] * dxdxi[1][2]) * tmp;
        dxidx[2][0] = (dxdxi[1][0] * dxdxi[2][1] - dxdxi[1][1] * dxdxi[2][0]) * tmp;
        dxidx[2][1] = (dxdxi[2][0] * dxdxi[0][1] - dxdxi[0][0] * dxdxi[2][1]) * tmp;
        dxidx[2][2] = (dxdxi[0][0] * dxdxi[1][1] - dxdxi[0][1] * dxdxi[1][0]) * tmp;
        const double WdetJ = tp.Qwt[intp] / tmp;
        double shg[8][3];
        for (int n = 0; n < nshl; ++n)
            for (int i = 0; i < 3; ++i)
                shg[n][i] = shgl[0][n] * dxidx[0][i] + shgl[1][n] * dxidx[1][i] + shgl[2][n] * dxidx[2][i];
        double g[3][5] = {{0}};
        for (int n = 0; n < nshl; ++n)
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 5; ++k) g[i][k] = g[i][k] + shg[n][i] * ycl[n][k];
        const double* g1 = g[0];
        const double* g2 = g[1];
        const double* g3 = g[2];
        double qdi[12];
        qdi[0] = rlm2mu * g1[1] + rlm * g2[2] + rlm * g3[3];
        qdi[1] = rmu * g1[2] + rmu * g2[1];
        qdi[2] = rmu * g1[3] + rmu * g3[1];
        qdi[3] = rlm2mu * u1 * g1[1] + rmu * u2 * g1[2] + rmu * u3 * g1[3] + rmu * u2 * g2[1] +
                 rlm * u1 * g2[2] + rmu * u3 * g3[1] + rlm * u1 * g3[3] + con * g1[4];
        qdi[4] = rmu * g1[2] + rmu * g2[1];
        qdi[5] = rlm * g1[1] + rlm2mu * g2[2] + rlm * g3[3];
        qdi[6] = rmu * g2[3] + rmu * g3[2];
        qdi[7] = rlm * u2 * g1[1] + rmu * u1 * g1[2] + rmu * u1 * g2[1] + rlm2mu * u2 * g2[2] +
                 rmu * u3 * g2[3] + rmu * u3 * g3[2] + rlm * u2 * g3[3] + con * g2[4];
        qdi[8] = rmu * g1[3] + rmu * g3[1];
        qdi[9] = rmu * g2[3] + rmu * g3[2];
        qdi[10] = rlm * g1[1] + rlm * g2[2] + rlm2mu * g3[3];
        qdi[11] = rlm * u3 * g1[1] + rmu * u1 * g1[3] + rlm * u3 * g2[2] + rmu * u2 * g2[3] +
                  rmu * u1 * g3[1] + rmu * u2 * g3[2] + rlm2mu * u3 * g3[3] + con * g3[4];
        for (int i = 0; i < nshl; ++i)
            for (int k = 0; k < 12; ++k) ql[i][k] = ql[i][k] + shape[i] * WdetJ * qdi[k];
        for (int i = 0; i < nshl; ++i) rmassl[i] = rmassl[i] + shape[i] * WdetJ;
    }
}

// AsIq (asiq.f) over every block + qpbc (qpbc.f): the lumped L2 reconstruction of the
// diffusive flux, qres(nshg,12) column-major
void reconstruct_q(const or_common& c, const or_mesh& m, const double* y, double* qres) {
    const int nshg = m.nshg;
    std::vector<double> rmass(nshg, 0.0);
    std::fill(qres, qres + 12 * (size_t)nshg, 0.0);
    auto run = [&](const Topo& tp, const int* ie) {
        double ycl[8][5], xl[8][3], ql[8][12] = {{0}}, rm[8] = {0};
        for (int a = 0; a < tp.nshl; ++a) {
            gather_y(y, nshg, ie[a], ycl[a]);
            gather_x(m.x, nshg, ie[a], xl[a]);
        }
        e3q_element(c, tp, ycl, xl, ql, rm);
        for (int k = 0; k < 12; ++k)
            for (int a = 0; a < tp.nshl; ++a) qres[k * (size_t)nshg + ie[a]] += ql[a][k];
        for (int a = 0; a < tp.nshl; ++a) rmass[ie[a]] += rm[a];
    };
    for (int b = 0; b < m.nblk; ++b)
        for (int e = m.blk_start[b]; e < m.blk_start[b + 1]; ++e) run(topo(1), m.ien + 4 * (size_t)e);
    for (int e = 0; e < m.nhex; ++e) run(topo(2), m.ienh + 8 * (size_t)e);
    for (int e = 0; e < m.nwedge; ++e) run(topo(3), m.ienw + 6 * (size_t)e);
    // qpbc.f: periodic slaves summed into masters, then copied back; lumped mass inverted
    for (int j = 0; j < nshg; ++j)
        if ((m.iBC[j] >> 10) & 1) {
            const int i = m.iper[j];
            rmass[i] = rmass[i] + rmass[j];
            for (int k = 0; k < 12; ++k) qres[k * (size_t)nshg + i] += qres[k * (size_t)nshg + j];
        }
    for (int j = 0; j < nshg; ++j)
        if ((m.iBC[j] >> 10) & 1) {
            const int i = m.iper[j];
            rmass[j] = rmass[i];
            for (int k = 0; k < 12; ++k) qres[k * (size_t)nshg + j] = qres[k * (size_t)nshg + i];
        }
    for (int j = 0; j < nshg; ++j) rmass[j] = one / rmass[j];
    for (int k = 0; k < 12; ++k)
        for (int j = 0; j < nshg; ++j) qres[k * (size_t)nshg + j] = rmass[j] * qres[k * (size_t)nshg + j];
}

// gather (localy.f, localx.f), e3, scatter (local.f:66-80) of one interior element
void one_element(const or_common& c, const Topo& tp, const or_mesh& m, const int* ie, int ires, int iprec,
                 const double* yp, const double* yc, const double* ac, double* res, double* rmes, double* bd,
                 int iabres, const double* qres) {
    const int nshg = m.nshg, nen = tp.nshl;
    double yl[8][5], ycl[8][5], acl[8][5], xl[8][3], ql[8][12];
    for (int a = 0; a < nen; ++a) {
        gather_y(yp, nshg, ie[a], yl[a]);
        gather_y(yc, nshg, ie[a], ycl[a]);
        gather_y(ac, nshg, ie[a], acl[a]);
        gather_x(m.x, nshg, ie[a], xl[a]);
        if (qres)
            for (int k = 0; k < 12; ++k) ql[a][k] = qres[k * (size_t)nshg + ie[a]];
    }
    double rl[8][5] = {{0}}, rml[8][5] = {{0}}, bdl[8][5][5] = {{{0}}};
    e3_element(c, tp, ires, iprec, yl, ycl, acl, xl, rl, rml, iprec ? bdl : nullptr, qres ? ql : nullptr);
    if (iabres == 1)
        for (int a = 0; a < nen; ++a)
            for (int k = 0; k < 5; ++k) rml[a][k] = std::fabs(rml[a][k]);
    // res rows in equation order
    for (int k = 0; k < 5; ++k)
        for (int a = 0; a < nen; ++a) {
            if (res && (ires == 1 || ires == 3)) res[k * (size_t)nshg + ie[a]] += rl[a][k];
            if (rmes && (ires == 2 || ires == 3)) rmes[k * (size_t)nshg + ie[a]] += rml[a][k];
        }
    if (iprec && bd)
        for (int j = 0; j < 5; ++j)
            for (int i = 0; i < 5; ++i)
                for (int a = 0; a < nen; ++a) bd[(i + 5 * j) * (size_t)nshg + ie[a]] += bdl[a][i][j];
}

// Interior element loop shared by ElmMFG / ItrRes / residual-only.
// ires 3: res, rmes, (BDiag if iprec); ires 2: rmes from (yp, yc); ires 1: res.
void element_sweep(const or_common& c, const or_mesh& m, int ires, int iprec,
                   const double* yp, const double* yc, const double* ac,
                   double* res, double* rmes, double* bd, int iabres, int nthreads,
                   const double* qres = nullptr) {
    const int nshg = m.nshg;
    const int ngrp = m.ngrp > 0 ? m.ngrp : 1;
    for (int gI = 0; gI < ngrp; ++gI) {
        const int b0 = m.ngrp > 0 ? m.grp_start[gI] : 0;
        const int b1 = m.ngrp > 0 ? m.grp_start[gI + 1] : m.nblk;
        // blocks inside a group touch disjoint nodes, so they may run concurrently;
        // with one thread the block order is the reference's.
        const int nb = b1 - b0;
        auto run_block = [&](int bi) {
            const int blk = b0 + bi;
            for (int e = m.blk_start[blk]; e < m.blk_start[blk + 1]; ++e)
                one_element(c, topo(1), m, m.ien + 4 * (size_t)e, ires, iprec, yp, yc, ac, res, rmes, bd, iabres,
                            qres);
        };
        parallel_for(nb, nthreads, run_block);
    }
    // hex and wedge blocks (elmmfg.f:113-146 block loop), element by element
    for (int e = 0; e < m.nhex; ++e)
        one_element(c, topo(2), m, m.ienh + 8 * (size_t)e, ires, iprec, yp, yc, ac, res, rmes, bd, iabres, qres);
    for (int e = 0; e < m.nwedge; ++e)
        one_element(c, topo(3), m, m.ienw + 6 * (size_t)e, ires, iprec, yp, yc, ac, res, rmes, bd, iabres, qres);
}

void boundary_sweep(const or_common& c, const or_mesh& m, const double* y, double* res) {
    const int nshg = m.nshg;
    for (int e = 0; e < m.nbelem; ++e) {
        const int* ie = m.ienb + 4 * (size_t)e;
        double yl[4][5], xl[4][3];
        for (int a = 0; a < 4; ++a) {
            gather_y(y, nshg, ie[a], yl[a]);
            gather_x(m.x, nshg, ie[a], xl[a]);
        }
        double bcb[3][6];
        for (int n = 0; n < 3; ++n)
            for (int k = 0; k < 6; ++k) bcb[n][k] = m.BCB ? m.BCB[(e * 3 + n) * 6 + k] : 0.0;
        double rl[4][5] = {{0}};
        e3b_element(c, btopo(1), yl, m.iBCB ? m.iBCB[2 * e] : 0, bcb, xl, rl);
        for (int k = 0; k < 5; ++k)
            for (int a = 0; a < 4; ++a) res[k * (size_t)nshg + ie[a]] += rl[a][k];
    }
    // boundary hex and wedge blocks (elmmfg.f:171-211)
    for (int b = 0; b < m.nbblk; ++b) {
        const or_bnd_block& B = m.bblk[b];
        const BTopo& bt = btopo(B.lcsyst);
        for (int e = 0; e < B.nelem; ++e) {
            const int* ie = B.ien + (size_t)bt.nshl * e;
            double yl[8][5], xl[8][3];
            for (int a = 0; a < bt.nshl; ++a) {
                gather_y(y, nshg, ie[a], yl[a]);
                gather_x(m.x, nshg, ie[a], xl[a]);
            }
            double bcb[4][6];
            for (int n = 0; n < bt.nshlb; ++n)
                for (int k = 0; k < 6; ++k) bcb[n][k] = B.BCB ? B.BCB[((size_t)e * bt.nshlb + n) * 6 + k] : 0.0;
            double rl[8][5] = {{0}};
            e3b_element(c, bt, yl, B.iBCB ? B.iBCB[2 * e] : 0, bcb, xl, rl);
            for (int k = 0; k < 5; ++k)
                for (int a = 0; a < bt.nshl; ++a) res[k * (size_t)nshg + ie[a]] += rl[a][k];
        }
    }
}

inline int ibits3(int v) { return (v >> 3) & 7; }
inline bool btest(int v, int b) { return (v >> b) & 1; }

// bc3lhs.f:1-198 on one element tangent EG[nedof][nedof] (intpres = 0): per node with
// a Dirichlet bit, its rows and columns are combined, zeroed and given a unit diagonal
void bc3lhs_element(const or_mesh& m, const int* ie, int nshl, double* EG) {
    const int N = m.nshg, nedof = 5 * nshl;
    auto E = [&](int r, int cc) -> double& { return EG[(size_t)r * nedof + cc]; };
    auto zero_rc = [&](int d) {
        for (int i = 0; i < nedof; ++i) {
            E(i, d) = zero;
            E(d, i) = zero;
        }
    };
    for (int inod = 0; inod < nshl; ++inod) {
        const int in = ie[inod];
        const int ib = m.iBC[in];
        if (ib == 0) continue;
        const int i1 = 5 * inod, i2 = i1 + 1, i3 = i1 + 2, i4 = i1 + 3, i5 = i1 + 4;
        const double b4 = m.BC[3 * (size_t)N + in], b5 = m.BC[4 * (size_t)N + in], b6 = m.BC[5 * (size_t)N + in];
        if (btest(ib, 2)) {
            zero_rc(i1);
            E(i1, i1) = one;
        }
        // velocity: (target row/col t1 [, t2]) -= coefficient * source, then the source is constrained
        auto combine1 = [&](int src, int ta, double ca, int tb, double cb) {
            for (int i = 0; i < nedof; ++i) {
                E(ta, i) = E(ta, i) - ca * E(src, i);
                E(tb, i) = E(tb, i) - cb * E(src, i);
            }
            for (int i = 0; i < nedof; ++i) {
                E(i, ta) = E(i, ta) - ca * E(i, src);
                E(i, tb) = E(i, tb) - cb * E(i, src);
            }
            zero_rc(src);
            E(src, src) = one;
        };
        auto combine2 = [&](int s1, int s2, int t) {
            for (int i = 0; i < nedof; ++i) E(t, i) = E(t, i) - b4 * E(s1, i) - b6 * E(s2, i);
            for (int i = 0; i < nedof; ++i) E(i, t) = E(i, t) - b4 * E(i, s1) - b6 * E(i, s2);
            for (int i = 0; i < nedof; ++i) {
                E(i, s1) = zero;
                E(s1, i) = zero;
                E(i, s2) = zero;
                E(s2, i) = zero;
            }
            E(s1, s1) = one;
            E(s2, s2) = one;
        };
        switch (ibits3(ib)) {
            case 1: combine1(i2, i3, b4, i4, b5); break;
            case 2: combine1(i3, i2, b4, i4, b5); break;
            case 3: combine2(i2, i3, i4); break;
            case 4: combine1(i4, i2, b4, i3, b5); break;
            case 5: combine2(i2, i4, i3); break;
            case 6: combine2(i3, i4, i2); break;
            case 7:
                for (int i = 0; i < nedof; ++i) {
                    E(i, i2) = zero; E(i2, i) = zero;
                    E(i, i3) = zero; E(i3, i) = zero;
                    E(i, i4) = zero; E(i4, i) = zero;
                }
                E(i2, i2) = one;
                E(i3, i3) = one;
                E(i4, i4) = one;
                break;
            default: break;
        }
        if (btest(ib, 1)) {
            zero_rc(i5);
            E(i5, i5) = one;
        }
        if (btest(ib, 11)) {  // intpres = 0: the continuity row stays
            for (int i = 0; i < nedof; ++i) {
                E(i, i2) = zero; E(i2, i) = zero;
                E(i, i3) = zero; E(i3, i) = zero;
                E(i, i4) = zero; E(i4, i) = zero;
                E(i, i5) = zero; E(i5, i) = zero;
            }
            E(i2, i2) = one;
            E(i3, i3) = one;
            E(i4, i4) = one;
            E(i5, i5) = one;
        }
    }
}

// fillsparse.f:1-52 (fillsparseC): EG blocks added to lhsK(25, nnz_tot) at the block of
// (row ien(a), column ien(b)), found by sparseloc's search of the sorted row (1-based colm/rowp)
void fillsparse_element(const int* ie, int nshl, const double* EG, const int* colm, const int* rowp, double* lhsK) {
    const int nedof = 5 * nshl;
    for (int aa = 0; aa < nshl; ++aa) {
        const int i = ie[aa];
        const int c0 = colm[i] - 1, n = colm[i + 1] - colm[i];
        for (int b = 0; b < nshl; ++b) {
            const int want = ie[b] + 1;
            int lo = 0, hi = n - 1, k = -1;
            while (lo <= hi) {
                const int mid = (lo + hi) / 2;
                if (rowp[c0 + mid] == want) { k = c0 + mid; break; }
                if (rowp[c0 + mid] < want) lo = mid + 1;
                else hi = mid - 1;
            }
            if (k < 0) continue;  // cannot happen for an adjacency built from the same mesh
            double* blk = lhsK + 25 * (size_t)k;
            for (int g = 0; g < 5; ++g)
                for (int f = 0; f < 5; ++f)
                    blk[5 * g + f] = blk[5 * g + f] + EG[(size_t)(5 * aa + f) * nedof + 5 * b + g];
        }
    }
}

// AsIGMR (asigmr.f:1-105) + bc3LHS + fillsparseC for one interior element (elmgmr.f:429-466)
// EBE store (ElmGMRe, elmgmr.f:1-275): EGmass(numel, nedof, nedof) column-major, element eidx
struct EbeStore {
    double* EG;
    size_t numel;
    int nedof;
    size_t eidx;
};

void one_element_lhs(const or_common& c, const Topo& tp, const or_mesh& m, const int* ie, const double* y,
                     const double* ac, double* res, double* bd, const int* colm, const int* rowp, double* lhsK,
                     const double* qres, const EbeStore* ebe = nullptr) {
    const int nshg = m.nshg, nen = tp.nshl, nedof = 5 * nen;
    double yl[8][5], acl[8][5], xl[8][3], ql[8][12];
    for (int a = 0; a < nen; ++a) {
        gather_y(y, nshg, ie[a], yl[a]);
        gather_y(ac, nshg, ie[a], acl[a]);
        gather_x(m.x, nshg, ie[a], xl[a]);
        if (qres)
            for (int k = 0; k < 12; ++k) ql[a][k] = qres[k * (size_t)nshg + ie[a]];
    }
    double rl[8][5] = {{0}}, rml[8][5] = {{0}};
    std::vector<double> EG((size_t)nedof * nedof, 0.0);
    e3_element(c, tp, 3, 1, yl, yl, acl, xl, rl, rml, nullptr, qres ? ql : nullptr, EG.data());
    for (int k = 0; k < 5; ++k)
        for (int a = 0; a < nen; ++a) res[k * (size_t)nshg + ie[a]] += rl[a][k];
    // block diagonal from the tangent before its boundary conditions (asigmr.f:92-103)
    for (int j = 0; j < 5; ++j)
        for (int i = 0; i < 5; ++i)
            for (int a = 0; a < nen; ++a)
                bd[(i + 5 * j) * (size_t)nshg + ie[a]] += EG[(size_t)(5 * a + i) * nedof + 5 * a + j];
    bc3lhs_element(m, ie, nen, EG.data());
    if (ebe) {
        for (int j = 0; j < nedof; ++j)
            for (int i = 0; i < nedof; ++i)
                ebe->EG[ebe->eidx + ebe->numel * ((size_t)i + (size_t)ebe->nedof * j)] = EG[(size_t)i * nedof + j];
    } else {
        fillsparse_element(ie, nen, EG.data(), colm, rowp, lhsK);
    }
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {


// Element groups for the threaded sweep: greedy colouring (no two elements of
// a group share a node), each colour cut into blocks of at most bksiz
// elements.  perm[nelem] lists the element order, blk_start[nblk+1] and
// grp_start[ngrp+1] the blocks and groups; returns ngrp (or -1 on overflow).
int or_make_groups(int nshg, int nelem, const int* ien, int bksiz, int* perm, int* blk_start,
                   int* nblk_out, int* grp_start, int max_grp) {
    std::vector<uint64_t> m0(nshg, 0), m1(nshg, 0);
    std::vector<int> col(nelem);
    int ncol = 0;
    for (int e = 0; e < nelem; ++e) {
        const int* nd = ien + 4 * (size_t)e;
        uint64_t f0 = 0, f1 = 0;
        for (int a = 0; a < 4; ++a) { f0 |= m0[nd[a]]; f1 |= m1[nd[a]]; }
        int c;
        if (~f0) c = __builtin_ctzll(~f0);
        else if (~f1) c = 64 + __builtin_ctzll(~f1);
        else return -1;
        col[e] = c;
        ncol = std::max(ncol, c + 1);
        for (int a = 0; a < 4; ++a) {
            if (c < 64) m0[nd[a]] |= 1ull << c;
            else m1[nd[a]] |= 1ull << (c - 64);
        }
    }
    if (ncol > max_grp) return -1;
    std::vector<std::vector<int>> cls(ncol);
    for (int e = 0; e < nelem; ++e) cls[col[e]].push_back(e);
    int p = 0, nb = 0;
    grp_start[0] = 0;
    for (int c = 0; c < ncol; ++c) {
        for (size_t i = 0; i < cls[c].size(); ++i) {
            if (i % bksiz == 0) blk_start[nb++] = p;
            perm[p++] = cls[c][i];
        }
        grp_start[c + 1] = nb;
    }
    blk_start[nb] = p;
    *nblk_out = nb;
    return ncol;
}

void or_tet_tables(double shp[16], double shgl[48], double Qwt[4], double shpb[12],
                   double shglb[36], double Qwtb[3]) {
    const Tables& t = tables();
    for (int q = 0; q < 4; ++q) {
        Qwt[q] = t.Qwt[q];
        for (int a = 0; a < 4; ++a) {
            shp[q * 4 + a] = t.shp[q][a];
            for (int i = 0; i < 3; ++i) shgl[(q * 3 + i) * 4 + a] = t.shgl[q][i][a];
        }
    }
    for (int q = 0; q < 3; ++q) {
        Qwtb[q] = t.Qwtb[q];
        for (int a = 0; a < 4; ++a) {
            shpb[q * 4 + a] = t.shpb[q][a];
            for (int i = 0; i < 3; ++i) shglb[(q * 3 + i) * 4 + a] = t.shglb[q][i][a];
        }
    }
}

void or_e3(const or_common* c, int ires, int iprec, const double* yl, const double* ycl,
           const double* acl, const double* xl, double* rl, double* rml, double* bdl) {
    e3_element(*c, topo(1), ires, iprec, (const double (*)[5])yl, (const double (*)[5])ycl,
               (const double (*)[5])acl, (const double (*)[3])xl, (double (*)[5])rl,
               (double (*)[5])rml, iprec ? (double (*)[5][5])bdl : nullptr);
}

void or_topo_tables(int lcsyst, double shp[64], double shgl[192], double Qwt[8], int* nshl, int* ngauss) {
    const Topo& t = topo(lcsyst);
    *nshl = t.nshl;
    *ngauss = t.ngauss;
    for (int q = 0; q < t.ngauss; ++q) {
        Qwt[q] = t.Qwt[q];
        for (int a = 0; a < t.nshl; ++a) {
            shp[q * t.nshl + a] = t.shp[q][a];
            for (int i = 0; i < 3; ++i) shgl[(q * 3 + i) * t.nshl + a] = t.shgl[q][i][a];
        }
    }
}

void or_e3_topo(const or_common* c, int lcsyst, int ires, int iprec, const double* yl, const double* ycl,
                const double* acl, const double* xl, double* rl, double* rml, double* bdl) {
    e3_element(*c, topo(lcsyst), ires, iprec, (const double (*)[5])yl, (const double (*)[5])ycl,
               (const double (*)[5])acl, (const double (*)[3])xl, (double (*)[5])rl, (double (*)[5])rml,
               (double (*)[5][5])bdl);
}

void or_e3b(const or_common* c, int ires, const double* yl, const int* iBCB, const double* BCB,
            const double* xlb, double* rl) {
    if (ires == 1 || ires == 3)
        e3b_element(*c, btopo(1), (const double (*)[5])yl, iBCB ? iBCB[0] : 0, (const double (*)[6])BCB,
                    (const double (*)[3])xlb, (double (*)[5])rl);
}

void or_btopo_tables(int lcsyst, double shpb[32], double shglb[96], double Qwtb[4], int* nshl, int* nshlb,
                     int* ngaussb, int lnode[4]) {
    const BTopo& t = btopo(lcsyst);
    *nshl = t.nshl;
    *nshlb = t.nshlb;
    *ngaussb = t.ngaussb;
    for (int n = 0; n < 4; ++n) lnode[n] = n < t.nshlb ? t.lnode[n] : -1;
    for (int q = 0; q < t.ngaussb; ++q) {
        Qwtb[q] = t.Qwtb[q];
        for (int a = 0; a < t.nshl; ++a) {
            shpb[q * t.nshl + a] = t.shpb[q][a];
            for (int i = 0; i < 3; ++i) shglb[(q * 3 + i) * t.nshl + a] = t.shglb[q][i][a];
        }
    }
}

// bc3res.f:23-160 (single rank)
void or_bc3res(const or_mesh* m, const double* y, double* res, const or_common* c) {
    const int N = m->nshg;
    const int* iBC = m->iBC;
    const double* BC = m->BC;
    double* r[5];
    for (int k = 0; k < 5; ++k) r[k] = res + (size_t)k * N;
    auto bc = [&](int k, int n) { return BC[(size_t)(k - 1) * N + n]; };  // 1-based column
    for (int n = 0; n < N; ++n) {
        const int ib = iBC[n];
        if (btest(ib, 0)) {  // density
            r[4][n] = r[4][n] + bc(1, n) * c->Rgas * r[0][n];
            r[0][n] = zero;
        }
        if (btest(ib, 2)) {  // pressure
            if (c->EntropyPressure == 1) {
                const double* yy[5];
                for (int k = 0; k < 5; ++k) yy[k] = y + (size_t)k * N;
                r[1][n] = r[1][n] - yy[0][n] * r[0][n];
                r[2][n] = r[2][n] - yy[1][n] * r[0][n];
                r[3][n] = r[3][n] - yy[2][n] * r[0][n];
                r[4][n] = r[4][n] - (c->gamma * c->Rgas / c->gamma1 * yy[4][n] +
                                     pt5 * (yy[0][n] * yy[0][n] + yy[1][n] * yy[1][n] + yy[2][n] * yy[2][n])) *
                                        r[0][n];
            }
            r[0][n] = zero;
        }
        const int v = ibits3(ib);
        switch (v) {
            case 1:
                r[2][n] = r[2][n] - bc(4, n) * r[1][n];
                r[3][n] = r[3][n] - bc(5, n) * r[1][n];
                r[1][n] = zero;
                break;
            case 2:
                r[1][n] = r[1][n] - bc(4, n) * r[2][n];
                r[3][n] = r[3][n] - bc(5, n) * r[2][n];
                r[2][n] = zero;
                break;
            case 3:
                r[3][n] = r[3][n] - bc(4, n) * r[1][n] - bc(6, n) * r[2][n];
                r[1][n] = zero;
                r[2][n] = zero;
                break;
            case 4:
                r[1][n] = r[1][n] - bc(4, n) * r[3][n];
                r[2][n] = r[2][n] - bc(5, n) * r[3][n];
                r[3][n] = zero;
                break;
            case 5:
                r[2][n] = r[2][n] - bc(4, n) * r[1][n] - bc(6, n) * r[3][n];
                r[1][n] = zero;
                r[3][n] = zero;
                break;
            case 6:
                r[1][n] = r[1][n] - bc(4, n) * r[2][n] - bc(6, n) * r[3][n];
                r[2][n] = zero;
                r[3][n] = zero;
                break;
            case 7:
                r[1][n] = zero;
                r[2][n] = zero;
                r[3][n] = zero;
                break;
            default:
                break;
        }
        if (btest(ib, 1)) r[4][n] = zero;  // temperature
    }
    // local periodic (bc3res.f:155-160), sequential as in the reference
    for (int j = 0; j < N; ++j)
        if (btest(iBC[j], 10)) {
            const int i = m->iper[j];
            for (int k = 0; k < 5; ++k) {
                r[k][i] = r[k][i] + r[k][j];
                r[k][j] = zero;
            }
        }
}

// bc3bdg.f:23-322 (single rank)
void or_bc3bdg(const or_mesh* m, const double* y, double* bdiag, const or_common* c) {
    const int N = m->nshg;
    const int* iBC = m->iBC;
    const double* BC = m->BC;
    auto B = [&](int i, int j, int n) -> double& {  // 1-based (i,j)
        return bdiag[((size_t)(i - 1) + 5 * (size_t)(j - 1)) * N + n];
    };
    auto bc = [&](int k, int n) { return BC[(size_t)(k - 1) * N + n]; };
    for (int n = 0; n < N; ++n) {
        const int ib = iBC[n];
        const double a5 = -y[4 * (size_t)N + n] * (c->Rgas * c->gamma / c->gamma1);
        if (btest(ib, 0)) {
            B(5, 5, n) = B(5, 5, n) + a5 * a5 * B(1, 1, n) + a5 * B(1, 5, n) + a5 * B(5, 1, n);
            B(4, 5, n) = B(4, 5, n) + a5 * B(4, 1, n);
            B(3, 5, n) = B(3, 5, n) + a5 * B(3, 1, n);
            B(2, 5, n) = B(2, 5, n) + a5 * B(2, 1, n);
            B(5, 4, n) = B(5, 4, n) + a5 * B(1, 4, n);
            B(5, 3, n) = B(5, 3, n) + a5 * B(1, 3, n);
            B(5, 2, n) = B(5, 2, n) + a5 * B(1, 2, n);
            B(1, 2, n) = zero; B(1, 3, n) = zero; B(1, 4, n) = zero; B(1, 5, n) = zero;
            B(2, 1, n) = zero; B(3, 1, n) = zero; B(4, 1, n) = zero; B(5, 1, n) = zero;
            B(1, 1, n) = one;
        }
        if (btest(ib, 2)) {
            B(1, 2, n) = zero; B(1, 3, n) = zero; B(1, 4, n) = zero; B(1, 5, n) = zero;
            B(2, 1, n) = zero; B(3, 1, n) = zero; B(4, 1, n) = zero; B(5, 1, n) = zero;
            B(1, 1, n) = one;
        }
        const int v = ibits3(ib);
        // a single constrained velocity component d (1-based dof 1+d) with the
        // two coefficients of the others (bc3bdg.f:71-155)
        auto single = [&](int dc, int o1, int o2) {  // dc: constrained dof row, o1/o2: the others
            const double b4 = bc(4, n), b5 = bc(5, n);
            B(5, o2, n) = B(5, o2, n) - b5 * B(5, dc, n);
            B(5, o1, n) = B(5, o1, n) - b4 * B(5, dc, n);
            B(o2, 5, n) = B(o2, 5, n) - b5 * B(dc, 5, n);
            B(o1, 5, n) = B(o1, 5, n) - b4 * B(dc, 5, n);
            B(o2, 1, n) = B(o2, 1, n) - b5 * B(dc, 1, n);
            B(o1, 1, n) = B(o1, 1, n) - b4 * B(dc, 1, n);
            B(1, o2, n) = B(1, o2, n) - b5 * B(1, dc, n);
            B(1, o1, n) = B(1, o1, n) - b4 * B(1, dc, n);
            B(o2, o2, n) = B(o2, o2, n) + b5 * b5 * B(dc, dc, n) - b5 * B(dc, o2, n) - b5 * B(o2, dc, n);
            B(o1, o2, n) = B(o1, o2, n) + b4 * b5 * B(dc, dc, n) - b5 * B(o1, dc, n) - b4 * B(dc, o2, n);
            B(o2, o1, n) = B(o2, o1, n) + b4 * b5 * B(dc, dc, n) - b5 * B(dc, o1, n) - b4 * B(o2, dc, n);
            B(o1, o1, n) = B(o1, o1, n) + b4 * b4 * B(dc, dc, n) - b4 * B(dc, o1, n) - b4 * B(o1, dc, n);
            for (int k = 1; k <= 5; ++k)
                if (k != dc) { B(dc, k, n) = zero; B(k, dc, n) = zero; }
            B(dc, dc, n) = one;
        };
        auto dbl = [&](int d1, int d2, int o) {  // two constrained components, one free (o)
            const double b4 = bc(4, n), b6 = bc(6, n);
            B(o, o, n) = B(o, o, n) + b4 * b4 * B(d1, d1, n) + b6 * b6 * B(d2, d2, n) +
                         b4 * b6 * (B(d1, d2, n) + B(d2, d1, n)) - b4 * (B(d1, o, n) + B(o, d1, n)) -
                         b6 * (B(d2, o, n) + B(o, d2, n));
            B(o, 1, n) = B(o, 1, n) - b4 * B(d1, 1, n) - b6 * B(d2, 1, n);
            B(o, 5, n) = B(o, 5, n) - b4 * B(d1, 5, n) - b6 * B(d2, 5, n);
            B(1, o, n) = B(1, o, n) - b4 * B(1, d1, n) - b6 * B(1, d2, n);
            B(5, o, n) = B(5, o, n) - b4 * B(5, d1, n) - b6 * B(5, d2, n);
            for (int k = 1; k <= 5; ++k) {
                if (k != d1) { B(d1, k, n) = zero; B(k, d1, n) = zero; }
                if (k != d2) { B(d2, k, n) = zero; B(k, d2, n) = zero; }
            }
            B(d1, d1, n) = one;
            B(d2, d2, n) = one;
        };
        switch (v) {
            case 1: single(2, 3, 4); break;
            case 2: single(3, 2, 4); break;
            case 3: {  // bc3bdg.f:139-168, written with products of entries as in the reference
                const double b4 = bc(4, n), b6 = bc(6, n);
                B(4, 4, n) = B(4, 4, n) + b4 * b4 * B(2, 2, n) + b6 * b6 * B(3, 3, n) +
                             b4 * b6 * (B(2, 3, n) * B(3, 2, n)) - b6 * (B(4, 3, n) * B(3, 4, n)) -
                             b4 * (B(4, 2, n) * B(2, 4, n));
                B(1, 4, n) = B(1, 4, n) - b4 * B(1, 2, n) - b6 * B(1, 3, n);
                B(4, 1, n) = B(4, 1, n) - b4 * B(2, 1, n) - b6 * B(3, 1, n);
                B(5, 4, n) = B(5, 4, n) - b4 * B(5, 2, n) - b6 * B(5, 3, n);
                B(4, 5, n) = B(4, 5, n) - b4 * B(2, 5, n) - b6 * B(3, 5, n);
                for (int k = 1; k <= 5; ++k) {
                    if (k != 2) { B(2, k, n) = zero; B(k, 2, n) = zero; }
                    if (k != 3) { B(3, k, n) = zero; B(k, 3, n) = zero; }
                }
                B(3, 3, n) = one;
                B(2, 2, n) = one;
                break;
            }
            case 4: single(4, 2, 3); break;
            case 5: dbl(2, 4, 3); break;
            case 6: dbl(3, 4, 2); break;
            case 7:
                for (int a = 2; a <= 4; ++a)
                    for (int k = 1; k <= 5; ++k)
                        if (k != a) { B(a, k, n) = zero; B(k, a, n) = zero; }
                B(2, 2, n) = one; B(3, 3, n) = one; B(4, 4, n) = one;
                break;
            default: break;
        }
        if (btest(ib, 1)) {
            B(5, 5, n) = one;
            for (int k = 1; k <= 4; ++k) { B(k, 5, n) = zero; B(5, k, n) = zero; }
        }
    }
    for (int j = 0; j < N; ++j)
        if (btest(iBC[j], 10)) {
            const int i = m->iper[j];
            for (int a = 1; a <= 5; ++a)
                for (int b = 1; b <= 5; ++b) B(a, b, i) = B(a, b, i) + B(a, b, j);
        }
    for (int j = 0; j < N; ++j)
        if (btest(iBC[j], 10)) {
            const int i = m->iper[j];
            for (int a = 1; a <= 5; ++a)
                for (int b = 1; b <= 5; ++b) B(a, b, j) = B(a, b, i);
        }
}

// itrbc.f:54-176 (no limiting, single rank); y in global order (u,v,w,p,T)
void or_itrbc(const or_mesh* m, double* y, double* ac, int ires, double Rgas) {
    const int N = m->nshg;
    const int* iBC = m->iBC;
    const double* BC = m->BC;
    auto bc = [&](int k, int n) { return BC[(size_t)(k - 1) * N + n]; };
    auto Y = [&](int k, int n) -> double& { return y[(size_t)(k - 1) * N + n]; };
    for (int n = 0; n < N; ++n) {
        const int ib = iBC[n];
        if (btest(ib, 1)) Y(5, n) = bc(2, n);
        switch (ibits3(ib)) {
            case 1: Y(1, n) = bc(3, n) - bc(4, n) * Y(2, n) - bc(5, n) * Y(3, n); break;
            case 2: Y(2, n) = bc(3, n) - bc(4, n) * Y(1, n) - bc(5, n) * Y(3, n); break;
            case 3: Y(1, n) = bc(3, n) - bc(4, n) * Y(3, n); Y(2, n) = bc(5, n) - bc(6, n) * Y(3, n); break;
            case 4: Y(3, n) = bc(3, n) - bc(4, n) * Y(1, n) - bc(5, n) * Y(2, n); break;
            case 5: Y(1, n) = bc(3, n) - bc(4, n) * Y(2, n); Y(3, n) = bc(5, n) - bc(6, n) * Y(2, n); break;
            case 6: Y(2, n) = bc(3, n) - bc(4, n) * Y(1, n); Y(3, n) = bc(5, n) - bc(6, n) * Y(1, n); break;
            case 7: Y(1, n) = bc(3, n); Y(2, n) = bc(4, n); Y(3, n) = bc(5, n); break;
            default: break;
        }
    }
    // density (itrbc.f:124-143): getthm ithm=2 gives pres = Rgas*rho*T, which the
    // reference stores into y(:,1); pressure (itrbc.f:146-151) into y(:,4)
    for (int n = 0; n < N; ++n)
        if (btest(iBC[n], 0)) Y(1, n) = Rgas * bc(1, n) * Y(5, n);
    for (int n = 0; n < N; ++n)
        if (btest(iBC[n], 2)) Y(4, n) = bc(1, n);
    for (int k = 1; k <= 5; ++k) {
        for (int n = 0; n < N; ++n) Y(k, n) = Y(k, m->iper[n]);
        if (ires != 2 && ac)
            for (int n = 0; n < N; ++n) ac[(size_t)(k - 1) * N + n] = ac[(size_t)(k - 1) * N + m->iper[n]];
    }
}

// i3lu.f:39-171
void or_i3lu(int N, double* bd, double* r, int code) {
    auto D = [&](int i, int j, int n) -> double& { return bd[((size_t)(i - 1) + 5 * (size_t)(j - 1)) * N + n]; };
    auto R = [&](int k, int n) -> double& { return r[(size_t)(k - 1) * N + n]; };
    for (int n = 0; n < N; ++n) {
        if (code == 0) {
            D(1, 1, n) = one / D(1, 1, n);
            D(2, 1, n) = D(1, 1, n) * D(2, 1, n);
            D(3, 1, n) = D(1, 1, n) * D(3, 1, n);
            D(4, 1, n) = D(1, 1, n) * D(4, 1, n);
            D(5, 1, n) = D(1, 1, n) * D(5, 1, n);
            D(2, 2, n) = D(2, 2, n) - D(2, 1, n) * D(1, 2, n);
            D(2, 3, n) = D(2, 3, n) - D(2, 1, n) * D(1, 3, n);
            D(2, 4, n) = D(2, 4, n) - D(2, 1, n) * D(1, 4, n);
            D(2, 5, n) = D(2, 5, n) - D(2, 1, n) * D(1, 5, n);
            D(2, 2, n) = one / D(2, 2, n);
            D(3, 2, n) = D(2, 2, n) * (D(3, 2, n) - D(3, 1, n) * D(1, 2, n));
            D(4, 2, n) = D(2, 2, n) * (D(4, 2, n) - D(4, 1, n) * D(1, 2, n));
            D(5, 2, n) = D(2, 2, n) * (D(5, 2, n) - D(5, 1, n) * D(1, 2, n));
            D(3, 3, n) = D(3, 3, n) - D(3, 1, n) * D(1, 3, n) - D(3, 2, n) * D(2, 3, n);
            D(3, 4, n) = D(3, 4, n) - D(3, 1, n) * D(1, 4, n) - D(3, 2, n) * D(2, 4, n);
            D(3, 5, n) = D(3, 5, n) - D(3, 1, n) * D(1, 5, n) - D(3, 2, n) * D(2, 5, n);
            D(3, 3, n) = one / D(3, 3, n);
            D(4, 3, n) = D(3, 3, n) * (D(4, 3, n) - D(4, 1, n) * D(1, 3, n) - D(4, 2, n) * D(2, 3, n));
            D(5, 3, n) = D(3, 3, n) * (D(5, 3, n) - D(5, 1, n) * D(1, 3, n) - D(5, 2, n) * D(2, 3, n));
            D(4, 4, n) = D(4, 4, n) - D(4, 1, n) * D(1, 4, n) - D(4, 2, n) * D(2, 4, n) -
                         D(4, 3, n) * D(3, 4, n);
            D(4, 4, n) = one / D(4, 4, n);
            D(5, 4, n) = D(4, 4, n) * (D(5, 4, n) - D(5, 1, n) * D(1, 4, n) - D(5, 2, n) * D(2, 4, n) -
                                       D(5, 3, n) * D(3, 4, n));
            D(5, 5, n) = D(5, 5, n) - D(5, 1, n) * D(1, 5, n) - D(5, 2, n) * D(2, 5, n) -
                         D(5, 3, n) * D(3, 5, n) - D(5, 4, n) * D(4, 5, n);
            D(5, 5, n) = one / D(5, 5, n);
        } else if (code == 1) {
            R(2, n) = R(2, n) - D(2, 1, n) * R(1, n);
            R(3, n) = R(3, n) - D(3, 1, n) * R(1, n) - D(3, 2, n) * R(2, n);
            R(4, n) = R(4, n) - D(4, 1, n) * R(1, n) - D(4, 2, n) * R(2, n) - D(4, 3, n) * R(3, n);
            R(5, n) = R(5, n) - D(5, 1, n) * R(1, n) - D(5, 2, n) * R(2, n) - D(5, 3, n) * R(3, n) -
                      D(5, 4, n) * R(4, n);
        } else if (code == 2) {
            R(5, n) = D(5, 5, n) * R(5, n);
            R(4, n) = D(4, 4, n) * (R(4, n) - R(5, n) * D(4, 5, n));
            R(3, n) = D(3, 3, n) * (R(3, n) - R(5, n) * D(3, 5, n) - R(4, n) * D(3, 4, n));
            R(2, n) = D(2, 2, n) * (R(2, n) - R(5, n) * D(2, 5, n) - R(4, n) * D(2, 4, n) -
                                    R(3, n) * D(2, 3, n));
            R(1, n) = D(1, 1, n) * (R(1, n) - R(5, n) * D(1, 5, n) - R(4, n) * D(1, 4, n) -
                                    R(3, n) * D(1, 3, n) - R(2, n) * D(1, 2, n));
        } else if (code == 3) {
            R(1, n) = R(1, n) / D(1, 1, n) + R(2, n) * D(1, 2, n) + R(3, n) * D(1, 3, n) +
                      R(4, n) * D(1, 4, n) + R(5, n) * D(1, 5, n);
            R(2, n) = R(2, n) / D(2, 2, n) + R(3, n) * D(2, 3, n) + R(4, n) * D(2, 4, n) +
                      R(5, n) * D(2, 5, n);
            R(3, n) = R(3, n) / D(3, 3, n) + R(4, n) * D(3, 4, n) + R(5, n) * D(3, 5, n);
            R(4, n) = R(4, n) / D(4, 4, n) + R(5, n) * D(4, 5, n);
            R(5, n) = R(5, n) / D(5, 5, n);
        }
    }
}

// shuffle.f:11-29
void or_yshuffle(int N, double* r, int code) {
    std::vector<double> t((size_t)5 * N);
    std::memcpy(t.data(), r, sizeof(double) * 5 * (size_t)N);
    if (code == 0) {  // old2new: (p,u,v,w,T) -> (u,v,w,p,T)
        for (int k = 0; k < 3; ++k) std::memcpy(r + (size_t)k * N, t.data() + (size_t)(k + 1) * N, sizeof(double) * N);
        std::memcpy(r + (size_t)3 * N, t.data(), sizeof(double) * N);
    } else {  // new2old: (u,v,w,p,T) -> (p,u,v,w,T)
        for (int k = 0; k < 3; ++k) std::memcpy(r + (size_t)(k + 1) * N, t.data() + (size_t)k * N, sizeof(double) * N);
        std::memcpy(r, t.data() + (size_t)3 * N, sizeof(double) * N);
    }
}

void or_elmmfg(const or_common* c, const or_mesh* m, const double* y, const double* ac,
               double* res, double* rmes, double* bdiag, int iprec, int nthreads) {
    const size_t N = m->nshg;
    std::memset(res, 0, sizeof(double) * 5 * N);
    std::memset(rmes, 0, sizeof(double) * 5 * N);
    if (iprec) std::memset(bdiag, 0, sizeof(double) * 25 * N);
    std::vector<double> qres;
    if (c->idiff == 1) {
        qres.resize(12 * N);
        reconstruct_q(*c, *m, y, qres.data());
    }
    element_sweep(*c, *m, 3, iprec, y, y, ac, res, rmes, iprec ? bdiag : nullptr, 0, nthreads,
                  qres.empty() ? nullptr : qres.data());
    boundary_sweep(*c, *m, y, res);  // AsBMFG: rml is zero while Jactyp == 0 (e3b.f:244-246)
    or_bc3res(m, y, res, c);
    or_bc3res(m, y, rmes, c);
    if (iprec) or_bc3bdg(m, y, bdiag, c);
}

void or_itrres(const or_common* c, const or_mesh* m, const double* yp, const double* yc,
               const double* ac, double* rmes, int iabres, int nthreads) {
    element_sweep(*c, *m, 2, 0, yp, yc, ac, nullptr, rmes, nullptr, iabres, nthreads);
    // boundary elements are skipped while Jactyp == 0 (itrres.f:95)
    or_bc3res(m, yc, rmes, c);
}

void or_elmres(const or_common* c, const or_mesh* m, const double* y, const double* ac,
               double* res, int nthreads) {
    const size_t N = m->nshg;
    std::memset(res, 0, sizeof(double) * 5 * N);
    std::vector<double> qres;
    if (c->idiff == 1) {
        qres.resize(12 * N);
        reconstruct_q(*c, *m, y, qres.data());
    }
    element_sweep(*c, *m, 1, 0, y, y, ac, res, nullptr, nullptr, 0, nthreads, qres.empty() ? nullptr : qres.data());
    boundary_sweep(*c, *m, y, res);
    or_bc3res(m, y, res, c);
}

// au1mfg.f:57-83: uBrg <- (L^-1 Rmod(P U^-1 (ypre + eps u)) - rmes) / eps
static void au1mfg(const or_common& c, const or_mesh& m, const double* ypre, const double* y,
                   const double* ac, const double* rmes, const double* bd, double* u,
                   int nthreads) {
    const size_t n5 = 5 * (size_t)m.nshg;
    std::vector<double> ub(n5, 0.0), ut(n5);
    for (size_t i = 0; i < n5; ++i) ut[i] = ypre[i] + c.eGMRES * u[i];
    or_i3lu(m.nshg, const_cast<double*>(bd), ut.data(), 2);
    or_yshuffle(m.nshg, ut.data(), 0);
    or_itrbc(&m, ut.data(), ut.data(), 2, c.Rgas);
    or_itrres(&c, &m, ut.data(), y, ac, ub.data(), 0, nthreads);
    or_i3lu(m.nshg, const_cast<double*>(bd), ub.data(), 1);
    for (size_t i = 0; i < n5; ++i) u[i] = (ub[i] - rmes[i]) / c.eGMRES;
}

static double sumsq(const double* a, size_t n) {
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += a[i] * a[i];
    return s;
}

// au2mfg.f:55-108: restart residual R - J Dy by a central difference of ItrRes
// with eps = epsM^(2/3) / ||Dy||; u receives the new first Krylov vector
static void au2mfg(const or_common& c, const or_mesh& m, const double* ypre, const double* y,
                   const double* ac, const double* res, const double* Dy, const double* bd,
                   double* u, int nthreads) {
    const size_t n5 = 5 * (size_t)m.nshg;
    double* bdm = const_cast<double*>(bd);
    const double eps = std::pow(c.epsM, 2.0 / 3.0) / std::sqrt(sumsq(Dy, n5));
    std::vector<double> ub1(n5, 0.0), ub2(n5, 0.0), ut(n5);
    for (size_t i = 0; i < n5; ++i) ut[i] = ypre[i] + eps * Dy[i];
    or_i3lu(m.nshg, bdm, ut.data(), 2);
    or_yshuffle(m.nshg, ut.data(), 0);
    or_itrbc(&m, ut.data(), ut.data(), 2, c.Rgas);
    or_itrres(&c, &m, ut.data(), y, ac, ub1.data(), 0, nthreads);
    or_i3lu(m.nshg, bdm, ub1.data(), 1);
    for (size_t i = 0; i < n5; ++i) ut[i] = ypre[i] - eps * Dy[i];
    or_i3lu(m.nshg, bdm, ut.data(), 2);
    or_yshuffle(m.nshg, ut.data(), 0);
    or_itrbc(&m, ut.data(), ut.data(), 2, c.Rgas);
    or_itrres(&c, &m, ut.data(), y, ac, ub2.data(), 0, nthreads);
    or_i3lu(m.nshg, bdm, ub2.data(), 1);
    for (size_t i = 0; i < n5; ++i) u[i] = res[i] - (ub1[i] - ub2[i]) / (two * eps);
}
static double dot(const double* a, const double* b, size_t n) {
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

// itrfdi.f:45-139
static void itrfdi(or_common& c, const or_mesh& m, const double* ypre, const double* y,
                   const double* ac, const double* rmes, const double* ubrg, const double* bd,
                   int nthreads) {
    const size_t n5 = 5 * (size_t)m.nshg;
    double* bdm = const_cast<double*>(bd);
    std::vector<double> rtmp(n5, 0.0), ytmp(ypre, ypre + n5);
    or_i3lu(m.nshg, bdm, ytmp.data(), 2);
    or_yshuffle(m.nshg, ytmp.data(), 0);
    or_itrres(&c, &m, ytmp.data(), y, ac, rtmp.data(), 1, nthreads);
    or_i3lu(m.nshg, bdm, rtmp.data(), 1);
    const double epsA = (c.epsM * c.epsM) * std::sqrt(sumsq(rtmp.data(), n5));
    const double epsSD = std::sqrt(c.epsM);
    std::fill(rtmp.begin(), rtmp.end(), 0.0);
    for (size_t i = 0; i < n5; ++i) ytmp[i] = ypre[i] + epsSD * ubrg[i];
    or_i3lu(m.nshg, bdm, ytmp.data(), 2);
    or_yshuffle(m.nshg, ytmp.data(), 0);
    or_itrres(&c, &m, ytmp.data(), y, ac, rtmp.data(), 0, nthreads);
    for (size_t i = 0; i < n5; ++i) ytmp[i] = ypre[i] - epsSD * ubrg[i];
    or_i3lu(m.nshg, bdm, ytmp.data(), 2);
    or_yshuffle(m.nshg, ytmp.data(), 0);
    or_itrres(&c, &m, ytmp.data(), y, ac, rtmp.data(), 0, nthreads);
    or_i3lu(m.nshg, bdm, rtmp.data(), 1);
    for (size_t i = 0; i < n5; ++i) {
        const double d = (rtmp[i] - two * rmes[i]) / c.epsM;
        rtmp[i] = d * d;
    }
    double s = 0.0;
    for (size_t i = 0; i < n5; ++i) s += rtmp[i];
    const double SDnrm = std::sqrt(s);
    c.eGMRES = two * std::sqrt(epsA / SDnrm);
}

void or_solmfg(or_common* c, const or_mesh* m, const double* y, const double* ac, double* res,
               double* bdiag, double* Dy, or_solve_stats* st, int nthreads) {
    const int N = m->nshg;
    const size_t n5 = 5 * (size_t)N;
    const int K = c->Kspace;
    std::vector<double> rmes(n5), ypre(n5), temp(n5);
    std::vector<double> uB(n5 * (K + 1));
    std::vector<double> H((K + 1) * K, 0.0), eB(K + 1, 0.0), yB(K, 0.0), Rc(K, 0.0), Rs(K, 0.0);
    auto Hm = [&](int i, int j) -> double& { return H[(size_t)(i - 1) + (size_t)(K + 1) * (j - 1)]; };
    auto U = [&](int j) { return uB.data() + n5 * (size_t)(j - 1); };

    or_elmmfg(c, m, y, ac, res, rmes.data(), bdiag, 1, nthreads);
    or_i3lu(N, bdiag, nullptr, 0);
    or_i3lu(N, bdiag, res, 1);
    or_i3lu(N, bdiag, rmes.data(), 1);
    std::memcpy(U(1), res, sizeof(double) * n5);
    std::fill(Dy, Dy + n5, 0.0);
    std::memcpy(ypre.data(), y, sizeof(double) * n5);
    or_yshuffle(N, ypre.data(), 1);
    or_i3lu(N, bdiag, ypre.data(), 3);
    double unorm = std::sqrt(sumsq(res, n5));
    st->unorm0 = unorm;
    int iKs = 0, lGMRES = 0;
    double echeck = 0.0;
    if (!(unorm < 100. * c->epsM * c->epsM)) {
        const double epsnrm = c->etol * unorm;
        if (c->iter == 1 && (c->istep % 20) == 0)
            itrfdi(*c, *m, ypre.data(), y, ac, rmes.data(), res, bdiag, nthreads);
        for (int mG = 1; mG <= c->nGMRES; ++mG) {
            lGMRES = mG - 1;
            if (lGMRES > 0) {
                // solmfg.f:186-203: restart from R - J Dy (Au2MFG)
                au2mfg(*c, *m, ypre.data(), y, ac, res, Dy, bdiag, temp.data(), nthreads);
                std::memcpy(U(1), temp.data(), sizeof(double) * n5);
                unorm = std::sqrt(sumsq(temp.data(), n5));
            }
            std::fill(eB.begin(), eB.end(), 0.0);
            eB[0] = unorm;
            for (size_t i = 0; i < n5; ++i) U(1)[i] = U(1)[i] / unorm;
            for (int iK = 1; iK <= K; ++iK) {
                iKs = iK;
                std::memcpy(temp.data(), U(iKs), sizeof(double) * n5);
                au1mfg(*c, *m, ypre.data(), y, ac, rmes.data(), bdiag, temp.data(), nthreads);
                std::memcpy(U(iKs + 1), temp.data(), sizeof(double) * n5);
                double beta = 0.0;
                for (int jK = 1; jK <= iKs + 1; ++jK) {
                    double* w = U(iKs + 1);
                    if (jK == 1) {
                        beta = dot(w, U(1), n5);
                    } else {
                        const double* up = U(jK - 1);
                        for (size_t i = 0; i < n5; ++i) w[i] = w[i] - beta * up[i];
                        beta = dot(w, U(jK), n5);
                    }
                    Hm(jK, iKs) = beta;
                }
                unorm = std::sqrt(beta);
                Hm(iKs + 1, iKs) = unorm;
                for (size_t i = 0; i < n5; ++i) U(iKs + 1)[i] = U(iKs + 1)[i] / unorm;
                for (int jK = 1; jK <= iKs - 1; ++jK) {
                    const double t = Rc[jK - 1] * Hm(jK, iKs) + Rs[jK - 1] * Hm(jK + 1, iKs);
                    Hm(jK + 1, iKs) = -Rs[jK - 1] * Hm(jK, iKs) + Rc[jK - 1] * Hm(jK + 1, iKs);
                    Hm(jK, iKs) = t;
                }
                const double t = std::sqrt(Hm(iKs, iKs) * Hm(iKs, iKs) + Hm(iKs + 1, iKs) * Hm(iKs + 1, iKs));
                Rc[iKs - 1] = Hm(iKs, iKs) / t;
                Rs[iKs - 1] = Hm(iKs + 1, iKs) / t;
                Hm(iKs, iKs) = t;
                Hm(iKs + 1, iKs) = zero;
                const double te = Rc[iKs - 1] * eB[iKs - 1] + Rs[iKs - 1] * eB[iKs];
                eB[iKs] = -Rs[iKs - 1] * eB[iKs - 1] + Rc[iKs - 1] * eB[iKs];
                eB[iKs - 1] = te;
                st->ntotGM += 1;
                echeck = std::fabs(eB[iKs]);
                if (echeck <= epsnrm && iKs >= c->minIters) break;
            }
            for (int jK = iKs; jK >= 1; --jK) {
                yB[jK - 1] = eB[jK - 1] / Hm(jK, jK);
                for (int lK = 1; lK <= jK - 1; ++lK) eB[lK - 1] = eB[lK - 1] - yB[jK - 1] * Hm(lK, jK);
            }
            for (int jK = 1; jK <= iKs; ++jK) {
                const double* uj = U(jK);
                for (size_t i = 0; i < n5; ++i) Dy[i] = Dy[i] + yB[jK - 1] * uj[i];
            }
            if (std::fabs(eB[iKs]) <= epsnrm) break;
        }
    }
    or_i3lu(N, bdiag, Dy, 2);
    st->iKs = iKs;
    st->lGMRES = lGMRES;
    st->echeck = echeck;
    st->eGMRES = c->eGMRES;
    st->totres = std::sqrt(sumsq(res, n5)) / (double)N;
}

// genadj.f:1-76 with Asadj (asadj.f): every node's unique neighbours over all element blocks,
// listed in ascending order; colm (nshg+1) and rowp are 1-based.  -1 when a row would
// exceed 15*nnz entries or the total nnz*nshg (where the reference stops).
int or_genadj(const or_mesh* m, int nnz, int* colm, int* rowp, int* icnt) {
    const int N = m->nshg;
    std::vector<std::vector<int>> rows(N);
    auto add = [&](const int* ien, int nshl, int ne) {
        for (int e = 0; e < ne; ++e) {
            const int* nd = ien + (size_t)nshl * e;
            for (int j = 0; j < nshl; ++j) {
                std::vector<int>& r = rows[nd[j]];
                for (int k = 0; k < nshl; ++k)
                    if (std::find(r.begin(), r.end(), nd[k]) == r.end()) r.push_back(nd[k]);
            }
        }
    };
    add(m->ien, 4, m->nelem);
    add(m->ienh, 8, m->nhex);
    add(m->ienw, 6, m->nwedge);
    colm[0] = 1;
    int cnt = 0;
    for (int i = 0; i < N; ++i) {
        if ((int)rows[i].size() > 15 * nnz) return -1;
        colm[i + 1] = colm[i] + (int)rows[i].size();
        std::sort(rows[i].begin(), rows[i].end());
        for (int v : rows[i]) {
            if (cnt >= nnz * N) return -1;
            rowp[cnt++] = v + 1;
        }
    }
    *icnt = cnt;
    return 0;
}

// ElmGMRs (elmgmr.f:280-613) with lhs = 1, iprec = 1: res, BDiag and the assembled
// tangent lhsK(25, nnz_tot) (column-major 5x5 blocks, lhsK[25 k + 5 g + f] = (f, g))
void or_elmgmrs(const or_common* c, const or_mesh* m, const double* y, const double* ac, const int* colm,
                const int* rowp, int nnz_tot, double* res, double* bdiag, double* lhsK, int nthreads) {
    const size_t N = m->nshg;
    std::memset(res, 0, sizeof(double) * 5 * N);
    std::memset(bdiag, 0, sizeof(double) * 25 * N);
    std::memset(lhsK, 0, sizeof(double) * 25 * (size_t)nnz_tot);
    std::vector<double> qres;
    if (c->idiff == 1) {
        qres.resize(12 * N);
        reconstruct_q(*c, *m, y, qres.data());
    }
    const double* q = qres.empty() ? nullptr : qres.data();
    const int ngrp = m->ngrp > 0 ? m->ngrp : 1;
    for (int gI = 0; gI < ngrp; ++gI) {
        const int b0 = m->ngrp > 0 ? m->grp_start[gI] : 0;
        const int b1 = m->ngrp > 0 ? m->grp_start[gI + 1] : m->nblk;
        parallel_for(b1 - b0, nthreads, [&](int bi) {
            const int blk = b0 + bi;
            for (int e = m->blk_start[blk]; e < m->blk_start[blk + 1]; ++e)
                one_element_lhs(*c, topo(1), *m, m->ien + 4 * (size_t)e, y, ac, res, bdiag, colm, rowp, lhsK, q);
        });
    }
    for (int e = 0; e < m->nhex; ++e)
        one_element_lhs(*c, topo(2), *m, m->ienh + 8 * (size_t)e, y, ac, res, bdiag, colm, rowp, lhsK, q);
    for (int e = 0; e < m->nwedge; ++e)
        one_element_lhs(*c, topo(3), *m, m->ienw + 6 * (size_t)e, y, ac, res, bdiag, colm, rowp, lhsK, q);
    boundary_sweep(*c, *m, y, res);
    or_bc3res(m, y, res, c);
    or_bc3bdg(m, y, bdiag, c);
}

// Spsi3pre (spsi3pre.f:1-196): lhsK(i, j) <- L_i^-1 lhsK(i, j) U_j^-1 with the i3LU factors
// (unit lower L below the diagonal, U above it, reciprocal pivots on it)
void or_spsi3pre(int N, const int* colm, const int* rowp, const double* bd, double* lhsK) {
    auto B = [&](int n, int r, int cc) { return bd[(size_t)(r + 5 * cc) * N + n]; };
    for (int i = 0; i < N; ++i)
        for (int k = colm[i] - 1; k < colm[i + 1] - 1; ++k) {
            double* a = lhsK + 25 * (size_t)k;
            for (int r = 1; r < 5; ++r)
                for (int g = 0; g < 5; ++g) {
                    double v = a[5 * g + r];
                    for (int cc = 0; cc < r; ++cc) v = v - B(i, r, cc) * a[5 * g + cc];
                    a[5 * g + r] = v;
                }
        }
    for (int i = 0; i < N; ++i)
        for (int k = colm[i] - 1; k < colm[i + 1] - 1; ++k) {
            const int j = rowp[k] - 1;
            double* a = lhsK + 25 * (size_t)k;
            for (int g = 0; g < 5; ++g)
                for (int f = 0; f < 5; ++f) {
                    double v = a[5 * g + f];
                    for (int cc = 0; cc < g; ++cc) v = v - B(j, cc, g) * a[5 * cc + f];
                    a[5 * g + f] = B(j, g, g) * v;
                }
        }
}

// SparseAp (sparseap.f:1-104) then bc3per (bc3per.f:1-20): p <- lhsK p with the periodic
// gather p(:) = p(iper(:)) first and the slave rows summed into their masters after
void or_sparseap(const or_mesh* m, const int* colm, const int* rowp, const double* lhsK, double* p) {
    const int N = m->nshg;
    std::vector<double> pg(5 * (size_t)N), q(5 * (size_t)N, 0.0);
    for (int k = 0; k < 5; ++k)
        for (int n = 0; n < N; ++n) pg[(size_t)k * N + n] = p[(size_t)k * N + m->iper[n]];
    for (int i = 0; i < N; ++i) {
        double t[5] = {0, 0, 0, 0, 0};
        for (int k = colm[i] - 1; k < colm[i + 1] - 1; ++k) {
            const int j = rowp[k] - 1;
            const double* a = lhsK + 25 * (size_t)k;
            for (int f = 0; f < 5; ++f)
                t[f] = t[f] + a[f] * pg[j] + a[5 + f] * pg[(size_t)N + j] + a[10 + f] * pg[2 * (size_t)N + j] +
                       a[15 + f] * pg[3 * (size_t)N + j] + a[20 + f] * pg[4 * (size_t)N + j];
        }
        for (int f = 0; f < 5; ++f) q[(size_t)f * N + i] = q[(size_t)f * N + i] + t[f];
    }
    for (int j = 0; j < N; ++j)
        if (btest(m->iBC[j], 10)) {
            const int i = m->iper[j];
            for (int k = 0; k < 5; ++k) {
                q[(size_t)k * N + i] = q[(size_t)k * N + i] + q[(size_t)k * N + j];
                q[(size_t)k * N + j] = zero;
            }
        }
    std::memcpy(p, q.data(), sizeof(double) * 5 * N);
}

// SolGMRs (solgmr.f:480-700): ElmGMRs, i3LU, Spsi3pre and GMRES on the preconditioned
// assembled tangent.  st->lGMRES is read on entry as the COMMON lGMRES that the restart
// test of solgmr.f:528 reads (SolGMRs itself counts in lGMRESs); it returns lGMRESs.
void or_solgmrs(or_common* c, const or_mesh* m, const int* colm, const int* rowp, int nnz_tot, const double* y,
                const double* ac, double* res, double* bdiag, double* Dy, double* lhsK, or_solve_stats* st,
                int nthreads) {
    const int N = m->nshg;
    const size_t n5 = 5 * (size_t)N;
    const int K = c->Kspace;
    const int lGMRES_common = st->lGMRES;
    std::vector<double> temp(n5), uB(n5 * (K + 1));
    std::vector<double> H((K + 1) * K, 0.0), eB(K + 1, 0.0), yB(K, 0.0), Rc(K, 0.0), Rs(K, 0.0);
    auto Hm = [&](int i, int j) -> double& { return H[(size_t)(i - 1) + (size_t)(K + 1) * (j - 1)]; };
    auto U = [&](int j) { return uB.data() + n5 * (size_t)(j - 1); };
    or_elmgmrs(c, m, y, ac, colm, rowp, nnz_tot, res, bdiag, lhsK, nthreads);
    or_i3lu(N, bdiag, nullptr, 0);
    or_i3lu(N, bdiag, res, 1);
    std::fill(Dy, Dy + n5, 0.0);
    or_spsi3pre(N, colm, rowp, bdiag, lhsK);
    std::memcpy(U(1), res, sizeof(double) * n5);
    double unorm = std::sqrt(sumsq(res, n5));
    st->unorm0 = unorm;
    int iKs = 0, lGMRESs = 0;
    double echeck = 0.0;
    if (!(unorm < 100. * c->epsM * c->epsM)) {
        const double epsnrm = c->etol * unorm;
        for (int mG = 1; mG <= c->nGMRES; ++mG) {
            lGMRESs = mG - 1;
            if (lGMRES_common > 0) {
                std::memcpy(temp.data(), Dy, sizeof(double) * n5);
                or_sparseap(m, colm, rowp, lhsK, temp.data());
                for (size_t i = 0; i < n5; ++i) temp[i] = res[i] - temp[i];
                std::memcpy(U(1), temp.data(), sizeof(double) * n5);
                unorm = std::sqrt(sumsq(temp.data(), n5));
            }
            std::fill(eB.begin(), eB.end(), 0.0);
            eB[0] = unorm;
            for (size_t i = 0; i < n5; ++i) U(1)[i] = U(1)[i] / unorm;
            for (int iK = 1; iK <= K; ++iK) {
                iKs = iK;
                std::memcpy(U(iKs + 1), U(iKs), sizeof(double) * n5);
                or_sparseap(m, colm, rowp, lhsK, U(iKs + 1));
                double beta = 0.0;
                for (int jK = 1; jK <= iKs + 1; ++jK) {
                    double* w = U(iKs + 1);
                    if (jK == 1) {
                        beta = dot(w, U(1), n5);
                    } else {
                        const double* up = U(jK - 1);
                        for (size_t i = 0; i < n5; ++i) w[i] = w[i] - beta * up[i];
                        beta = dot(w, U(jK), n5);
                    }
                    Hm(jK, iKs) = beta;
                }
                unorm = std::sqrt(beta);
                Hm(iKs + 1, iKs) = unorm;
                for (size_t i = 0; i < n5; ++i) U(iKs + 1)[i] = U(iKs + 1)[i] / unorm;
                for (int jK = 1; jK <= iKs - 1; ++jK) {
                    const double t = Rc[jK - 1] * Hm(jK, iKs) + Rs[jK - 1] * Hm(jK + 1, iKs);
                    Hm(jK + 1, iKs) = -Rs[jK - 1] * Hm(jK, iKs) + Rc[jK - 1] * Hm(jK + 1, iKs);
                    Hm(jK, iKs) = t;
                }
                const double t = std::sqrt(Hm(iKs, iKs) * Hm(iKs, iKs) + Hm(iKs + 1, iKs) * Hm(iKs + 1, iKs));
                Rc[iKs - 1] = Hm(iKs, iKs) / t;
                Rs[iKs - 1] = Hm(iKs + 1, iKs) / t;
                Hm(iKs, iKs) = t;
                Hm(iKs + 1, iKs) = zero;
                const double te = Rc[iKs - 1] * eB[iKs - 1] + Rs[iKs - 1] * eB[iKs];
                eB[iKs] = -Rs[iKs - 1] * eB[iKs - 1] + Rc[iKs - 1] * eB[iKs];
                eB[iKs - 1] = te;
                st->ntotGM += 1;
                echeck = std::fabs(eB[iKs]);
                if (echeck <= epsnrm && iKs >= c->minIters) break;
            }
            for (int jK = iKs; jK >= 1; --jK) {
                yB[jK - 1] = eB[jK - 1] / Hm(jK, jK);
                for (int lK = 1; lK <= jK - 1; ++lK) eB[lK - 1] = eB[lK - 1] - yB[jK - 1] * Hm(lK, jK);
            }
            for (int jK = 1; jK <= iKs; ++jK) {
                const double* uj = U(jK);
                for (size_t i = 0; i < n5; ++i) Dy[i] = Dy[i] + yB[jK - 1] * uj[i];
            }
            echeck = std::fabs(eB[iKs]);
            if (echeck <= epsnrm) break;
        }
    }
    or_i3lu(N, bdiag, Dy, 2);
    st->iKs = iKs;
    st->lGMRES = lGMRESs;
    st->echeck = echeck;
    st->eGMRES = c->eGMRES;
    st->totres = std::sqrt(sumsq(res, n5)) / (double)N;
}

// ---- element-by-element solver (SolGMRe) on single-topology meshes ----
// element e of EGmass is the e-th element of the reference's block order: tets (input order,
// eid[] maps the oracle's grouped order back to it), then hexes, then wedges.
static int ebe_nedof(const or_mesh& m) { return m.nhex ? 40 : m.nwedge ? 30 : 20; }

// ElmGMRe (elmgmr.f:1-275): res, BDiag, and EGmass after bc3LHS
void or_elmgmre(const or_common* c, const or_mesh* m, const int* eid, const double* y, const double* ac,
                double* res, double* bdiag, double* EG, int nthreads) {
    const size_t N = m->nshg;
    const size_t numel = (size_t)m->nelem + m->nhex + m->nwedge;
    const int nedof = ebe_nedof(*m);
    std::memset(res, 0, sizeof(double) * 5 * N);
    std::memset(bdiag, 0, sizeof(double) * 25 * N);
    std::memset(EG, 0, sizeof(double) * numel * nedof * nedof);
    std::vector<double> qres;
    if (c->idiff == 1) {
        qres.resize(12 * N);
        reconstruct_q(*c, *m, y, qres.data());
    }
    const double* q = qres.empty() ? nullptr : qres.data();
    const int ngrp = m->ngrp > 0 ? m->ngrp : 1;
    for (int gI = 0; gI < ngrp; ++gI) {
        const int b0 = m->ngrp > 0 ? m->grp_start[gI] : 0;
        const int b1 = m->ngrp > 0 ? m->grp_start[gI + 1] : m->nblk;
        parallel_for(b1 - b0, nthreads, [&](int bi) {
            const int blk = b0 + bi;
            for (int e = m->blk_start[blk]; e < m->blk_start[blk + 1]; ++e) {
                const EbeStore st{EG, numel, nedof, (size_t)(eid ? eid[e] : e)};
                one_element_lhs(*c, topo(1), *m, m->ien + 4 * (size_t)e, y, ac, res, bdiag, nullptr, nullptr,
                                nullptr, q, &st);
            }
        });
    }
    for (int e = 0; e < m->nhex; ++e) {
        const EbeStore st{EG, numel, nedof, (size_t)m->nelem + e};
        one_element_lhs(*c, topo(2), *m, m->ienh + 8 * (size_t)e, y, ac, res, bdiag, nullptr, nullptr, nullptr, q,
                        &st);
    }
    for (int e = 0; e < m->nwedge; ++e) {
        const EbeStore st{EG, numel, nedof, (size_t)m->nelem + m->nhex + e};
        one_element_lhs(*c, topo(3), *m, m->ienw + 6 * (size_t)e, y, ac, res, bdiag, nullptr, nullptr, nullptr, q,
                        &st);
    }
    boundary_sweep(*c, *m, y, res);
    or_bc3res(m, y, res, c);
    or_bc3bdg(m, y, bdiag, c);
}

// the nodes of element e of the block order
static const int* ebe_nodes(const or_mesh& m, const std::vector<int>& pos, size_t e, int* nshl) {
    if (e < (size_t)m.nelem) { *nshl = 4; return m.ien + 4 * (size_t)pos[e]; }
    e -= m.nelem;
    if (e < (size_t)m.nhex) { *nshl = 8; return m.ienh + 8 * e; }
    *nshl = 6;
    return m.ienw + 6 * (e - m.nhex);
}
static std::vector<int> ebe_pos(const or_mesh& m, const int* eid) {
    std::vector<int> pos(m.nelem);
    for (int e = 0; e < m.nelem; ++e) pos[eid ? eid[e] : e] = e;
    return pos;
}

// i3pre (i3pre.f:1-105): EGmass rows of node a <- L_a^-1 rows, then columns of node b <- U_b^-1
void or_i3pre(const or_mesh* m, const int* eid, const double* bd, double* EG) {
    const size_t N = m->nshg, numel = (size_t)m->nelem + m->nhex + m->nwedge;
    const int nedof = ebe_nedof(*m);
    const std::vector<int> pos = ebe_pos(*m, eid);
    auto B = [&](int n, int r, int cc) { return bd[(size_t)(r + 5 * cc) * N + n]; };
    for (size_t e = 0; e < numel; ++e) {
        int nshl;
        const int* ie = ebe_nodes(*m, pos, e, &nshl);
        auto E = [&](int i, int j) -> double& { return EG[e + numel * ((size_t)i + (size_t)nedof * j)]; };
        for (int a = 0; a < nshl; ++a) {
            const int i = 5 * a, n = ie[a];
            for (int j = 0; j < nedof; ++j)
                for (int r = 1; r < 5; ++r) {
                    double v = E(i + r, j);
                    for (int cc = 0; cc < r; ++cc) v = v - B(n, r, cc) * E(i + cc, j);
                    E(i + r, j) = v;
                }
        }
        for (int a = 0; a < nshl; ++a) {
            const int i = 5 * a, n = ie[a];
            for (int j = 0; j < nedof; ++j)
                for (int g = 0; g < 5; ++g) {
                    double v = E(j, i + g);
                    for (int cc = 0; cc < g; ++cc) v = v - B(n, cc, g) * E(j, i + cc);
                    E(j, i + g) = B(n, g, g) * v;
                }
        }
    }
}

// Au1GMR (au1gmr.f:1-60) with AsAuGMR (asaugmr.f) and localt (localt.f), then bc3per:
// p <- sum_e EGmass_e p_e with the periodic gather p(iper) first
void or_au1gmr(const or_mesh* m, const int* eid, const double* EG, double* p) {
    const size_t N = m->nshg, numel = (size_t)m->nelem + m->nhex + m->nwedge;
    const int nedof = ebe_nedof(*m);
    const std::vector<int> pos = ebe_pos(*m, eid);
    std::vector<double> pg(5 * N), q(5 * N, 0.0);
    for (int k = 0; k < 5; ++k)
        for (size_t n = 0; n < N; ++n) pg[k * N + n] = p[k * N + m->iper[n]];
    for (size_t e = 0; e < numel; ++e) {
        int nshl;
        const int* ie = ebe_nodes(*m, pos, e, &nshl);
        auto E = [&](int i, int j) { return EG[e + numel * ((size_t)i + (size_t)nedof * j)]; };
        double ul[40], ub[40] = {0};
        for (int b = 0; b < nshl; ++b)
            for (int k = 0; k < 5; ++k) ul[5 * b + k] = pg[k * N + ie[b]];
        for (int i = 0; i < 5 * nshl; i += 5)
            for (int j = 0; j < 5 * nshl; j += 5)
                for (int r = 0; r < 5; ++r)
                    ub[i + r] = ub[i + r] + E(i + r, j) * ul[j] + E(i + r, j + 1) * ul[j + 1] +
                                E(i + r, j + 2) * ul[j + 2] + E(i + r, j + 3) * ul[j + 3] +
                                E(i + r, j + 4) * ul[j + 4];
        for (int a = 0; a < nshl; ++a)
            for (int k = 0; k < 5; ++k) q[k * N + ie[a]] = q[k * N + ie[a]] + ub[5 * a + k];
    }
    for (size_t j = 0; j < N; ++j)
        if (btest(m->iBC[j], 10)) {
            const int i = m->iper[j];
            for (int k = 0; k < 5; ++k) {
                q[k * N + i] = q[k * N + i] + q[k * N + j];
                q[k * N + j] = zero;
            }
        }
    std::memcpy(p, q.data(), sizeof(double) * 5 * N);
}

// SolGMRe (solgmr.f:1-245): ElmGMRe, i3LU, i3pre, GMRES with element-by-element products;
// restarts from the true residual, convergence without the minIters test
void or_solgmre(or_common* c, const or_mesh* m, const int* eid, const double* y, const double* ac, double* res,
                double* bdiag, double* Dy, double* EG, or_solve_stats* st, int nthreads) {
    const int N = m->nshg;
    const size_t n5 = 5 * (size_t)N;
    const int K = c->Kspace;
    std::vector<double> temp(n5), uB(n5 * (K + 1));
    std::vector<double> H((K + 1) * K, 0.0), eB(K + 1, 0.0), yB(K, 0.0), Rc(K, 0.0), Rs(K, 0.0);
    auto Hm = [&](int i, int j) -> double& { return H[(size_t)(i - 1) + (size_t)(K + 1) * (j - 1)]; };
    auto U = [&](int j) { return uB.data() + n5 * (size_t)(j - 1); };
    or_elmgmre(c, m, eid, y, ac, res, bdiag, EG, nthreads);
    or_i3lu(N, bdiag, nullptr, 0);
    or_i3lu(N, bdiag, res, 1);
    std::fill(Dy, Dy + n5, 0.0);
    or_i3pre(m, eid, bdiag, EG);
    std::memcpy(U(1), res, sizeof(double) * n5);
    double unorm = std::sqrt(sumsq(res, n5));
    st->unorm0 = unorm;
    int iKs = 0, lGMRES = 0;
    double echeck = 0.0;
    if (!(unorm < 100. * c->epsM * c->epsM)) {
        const double epsnrm = c->etol * unorm;
        for (int mG = 1; mG <= c->nGMRES; ++mG) {
            lGMRES = mG - 1;
            if (lGMRES > 0) {
                std::memcpy(temp.data(), Dy, sizeof(double) * n5);
                or_au1gmr(m, eid, EG, temp.data());
                for (size_t i = 0; i < n5; ++i) temp[i] = res[i] - temp[i];
                std::memcpy(U(1), temp.data(), sizeof(double) * n5);
                unorm = std::sqrt(sumsq(temp.data(), n5));
            }
            std::fill(eB.begin(), eB.end(), 0.0);
            eB[0] = unorm;
            for (size_t i = 0; i < n5; ++i) U(1)[i] = U(1)[i] / unorm;
            for (int iK = 1; iK <= K; ++iK) {
                iKs = iK;
                std::memcpy(U(iKs + 1), U(iKs), sizeof(double) * n5);
                or_au1gmr(m, eid, EG, U(iKs + 1));
                double beta = 0.0;
                for (int jK = 1; jK <= iKs + 1; ++jK) {
                    double* w = U(iKs + 1);
                    if (jK == 1) {
                        beta = dot(w, U(1), n5);
                    } else {
                        const double* up = U(jK - 1);
                        for (size_t i = 0; i < n5; ++i) w[i] = w[i] - beta * up[i];
                        beta = dot(w, U(jK), n5);
                    }
                    Hm(jK, iKs) = beta;
                }
                unorm = std::sqrt(beta);
                Hm(iKs + 1, iKs) = unorm;
                for (size_t i = 0; i < n5; ++i) U(iKs + 1)[i] = U(iKs + 1)[i] / unorm;
                for (int jK = 1; jK <= iKs - 1; ++jK) {
                    const double t = Rc[jK - 1] * Hm(jK, iKs) + Rs[jK - 1] * Hm(jK + 1, iKs);
                    Hm(jK + 1, iKs) = -Rs[jK - 1] * Hm(jK, iKs) + Rc[jK - 1] * Hm(jK + 1, iKs);
                    Hm(jK, iKs) = t;
                }
                const double t = std::sqrt(Hm(iKs, iKs) * Hm(iKs, iKs) + Hm(iKs + 1, iKs) * Hm(iKs + 1, iKs));
                Rc[iKs - 1] = Hm(iKs, iKs) / t;
                Rs[iKs - 1] = Hm(iKs + 1, iKs) / t;
                Hm(iKs, iKs) = t;
                Hm(iKs + 1, iKs) = zero;
                const double te = Rc[iKs - 1] * eB[iKs - 1] + Rs[iKs - 1] * eB[iKs];
                eB[iKs] = -Rs[iKs - 1] * eB[iKs - 1] + Rc[iKs - 1] * eB[iKs];
                eB[iKs - 1] = te;
                st->ntotGM += 1;
                echeck = std::fabs(eB[iKs]);
                if (echeck <= epsnrm) break;
            }
            for (int jK = iKs; jK >= 1; --jK) {
                yB[jK - 1] = eB[jK - 1] / Hm(jK, jK);
                for (int lK = 1; lK <= jK - 1; ++lK) eB[lK - 1] = eB[lK - 1] - yB[jK - 1] * Hm(lK, jK);
            }
            for (int jK = 1; jK <= iKs; ++jK) {
                const double* uj = U(jK);
                for (size_t i = 0; i < n5; ++i) Dy[i] = Dy[i] + yB[jK - 1] * uj[i];
            }
            echeck = std::fabs(eB[iKs]);
            if (echeck <= epsnrm) break;
        }
    }
    or_i3lu(N, bdiag, Dy, 2);
    st->iKs = iKs;
    st->lGMRES = lGMRES;
    st->echeck = echeck;
    st->eGMRES = c->eGMRES;
    st->totres = std::sqrt(sumsq(res, n5)) / (double)N;
}

void or_itrpredict(const or_common* c, int N, const double* yold, const double* acold, double* y,
                   double* ac) {
    const size_t n5 = 5 * (size_t)N;
    for (size_t i = 0; i < n5; ++i) {
        y[i] = yold[i];
        ac[i] = acold[i] * (one - c->almi / c->gami);
    }
}

void or_itrcorrect(const or_common* c, int N, double* y, double* ac, const double* yold,
                   const double* acold, const double* Dy) {
    auto Y = [&](int k, int n) -> double& { return y[(size_t)(k - 1) * N + n]; };
    auto D = [&](int k, int n) { return Dy[(size_t)(k - 1) * N + n]; };
    for (int n = 0; n < N; ++n) {
        Y(1, n) = Y(1, n) - D(2, n);
        Y(2, n) = Y(2, n) - D(3, n);
        Y(3, n) = Y(3, n) - D(4, n);
        Y(4, n) = Y(4, n) - D(1, n);
        Y(5, n) = Y(5, n) - D(5, n);
    }
    const double fct1 = (one - c->almi / c->gami);
    const double fct2 = c->almi * c->Dtgl / c->gami / c->alfi;
    for (size_t i = 0; i < 5 * (size_t)N; ++i) ac[i] = acold[i] * fct1 + (y[i] - yold[i]) * fct2;
}

void or_itrupdate(const or_common* c, int N, double* yold, double* acold, const double* y,
                  const double* ac) {
    const double fct2 = one / c->almi, fct3 = one / c->alfi;
    for (size_t i = 0; i < 5 * (size_t)N; ++i) {
        acold[i] = acold[i] + (ac[i] - acold[i]) * fct2;
        yold[i] = yold[i] + (y[i] - yold[i]) * fct3;
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// floating-point operations of the reference formulation of e3 for one element (the counting
// scalar through the same statements as the oracle), and the element's outputs for a check
// ---------------------------------------------------------------------------
extern "C" long long or_e3_flops(const or_common* c, int lcsyst, int ires, int iprec, const double* yl,
                                 const double* ycl, const double* acl, const double* xl, double* rl,
                                 double* rml, double* bdl) {
    const Topo& tp = topo(lcsyst);
    const int n = tp.nshl;
    std::vector<Flop> y(5 * n), yc(5 * n), a(5 * n), x(3 * n), r(5 * n), rm(5 * n), bd(25 * n);
    for (int i = 0; i < 5 * n; ++i) {
        y[i] = yl[i];
        yc[i] = ycl[i];
        a[i] = acl[i];
        r[i] = rl[i];
        rm[i] = rml[i];
    }
    for (int i = 0; i < 3 * n; ++i) x[i] = xl[i];
    for (int i = 0; i < 25 * n; ++i) bd[i] = bdl ? bdl[i] : 0.0;
    g_flops = 0;
    e3_element_t<Flop>(*c, tp, ires, iprec, (const Flop (*)[5])y.data(), (const Flop (*)[5])yc.data(),
                       (const Flop (*)[5])a.data(), (const Flop (*)[3])x.data(), (Flop (*)[5])r.data(),
                       (Flop (*)[5])rm.data(), iprec ? (Flop (*)[5][5])bd.data() : nullptr, nullptr, nullptr);
    const long long nf = g_flops;
    for (int i = 0; i < 5 * n; ++i) {
        rl[i] = r[i].v;
        rml[i] = rm[i].v;
    }
    if (bdl)
        for (int i = 0; i < 25 * n; ++i) bdl[i] = bd[i].v;
    return nf;
}
