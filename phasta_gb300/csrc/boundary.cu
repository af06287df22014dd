// boundary.cu -- boundary hexes and wedges (AsBMFG/e3b/e3bvar for the boundary element blocks
// of lcsyst 2, 3 and 4; phSolver/compressible/asbmfg.f:1-60, e3b.f:1-387, e3bvar.f:1-290;
// the block loop of elmmfg.f:171-211).
//
// The reference loops over boundary element blocks, gathers each element whole and
// integrates the face flux at the boundary rule's points.  Here each block keeps its elements
// in colour order on the device (no two elements of a colour share a node) and one FP64
// thread per element evaluates the face flux and adds it to its face nodes; boundary faces
// are O(E^(2/3)) of the mesh, so this is a small launch beside the interior sweeps.  The
// residual is the only output: BDiag and the Jacobian-vector products carry no face terms on
// the path (e3b.f adds EGmass only with iLHScond > 0 and the modified residual only with
// Jactyp = 1; ItrRes visits boundary blocks only with Jactyp != 0, itrres.f:94).
#include "phgpu_impl.cuh"

namespace phgpu {

// boundary rule and shapes of one boundary topology (genint.f, genshpb.f; linear basis)
struct BndTab {
    double shpb[4][8];      // [q][a]
    double shglb[4][3][8];  // [q][i][a] parent-coordinate derivatives
    double Qwtb[4];
    int lnode[4];           // face nodes, 0-based, in getbnodes order (hierarchic.f:90-165)
};
__constant__ BndTab c_btab[3];  // lcsyst 2, 3, 4

namespace {

// The rules and shapes, restated: lcsyst 2 the 2x2 Gauss rule of symquad.c on the hex's
// zeta = -1 face (weights 1, genint.f:140-142) with the trilinear hex shapes; lcsyst 3 the
// 3-point rule of symtri.c with its last point moved first on the wedge's zeta = -1 triangle
// (genint.f:325-334); lcsyst 4 the rule of symquadw.c on the wedge's s = 0 face (r mapped to
// [0, 1], genint.f:340-343).  Wedge in-plane derivatives are taken on the area-2 parent
// triangle, as for the interior wedge (WedgeShapeAndDrv).
void bnd_tables_host(BndTab t[3]) {
    for (int k = 0; k < 3; ++k) t[k] = BndTab{};
    auto hex = [](const double par[3], double* N, double (*dN)[8]) {
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
    };
    auto wedge = [](double r, double s2, double z, double* N, double (*dN)[8]) {
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
    };
    const double g = 0.577350269189626;
    for (int q = 0; q < 4; ++q) {
        const double par[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, -1.0};
        t[0].Qwtb[q] = 1.0;
        hex(par, t[0].shpb[q], t[0].shglb[q]);
        t[0].lnode[q] = q;
    }
    const double P3 = 0.166666666666667, P4 = 0.666666666666667;
    const double tri[3][2] = {{P3, P3}, {P4, P3}, {P3, P4}};
    for (int q = 0; q < 3; ++q) {
        t[1].Qwtb[q] = 0.333333333333333;
        wedge(tri[q][0], tri[q][1], -1.0, t[1].shpb[q], t[1].shglb[q]);
        t[1].lnode[q] = q;
    }
    t[1].lnode[3] = -1;
    const double r[2] = {0.211324865405187, 0.788675134594813};
    for (int q = 0; q < 4; ++q) {
        t[2].Qwtb[q] = 1.0;
        wedge(r[q & 1], 0.0, (q & 2) ? g : -g, t[2].shpb[q], t[2].shglb[q]);
    }
    t[2].lnode[0] = 0;
    t[2].lnode[1] = 3;
    t[2].lnode[2] = 4;
    t[2].lnode[3] = 1;
}

// face node n of topology LCSYST (the table's lnode, known at compile time)
template <int LCSYST>
__device__ __forceinline__ constexpr int face_node(int n) {
    return LCSYST == 4 ? (n == 0 ? 0 : n == 1 ? 3 : n == 2 ? 4 : 1) : n;
}

// One boundary element of topology LCSYST per thread: e3bvar (state at the point from the face
// nodes, deformation gradient and its inverse from all nodes, the normal of e3bvar.f:156-176 and
// the weight of e3bvar.f:184-197), the Euler and Navier-Stokes face flux of e3b.f:138-233 with the
// iBCB switches, and the face nodes' residual (e3b.f:261-280).
template <int LCSYST>
__global__ void __launch_bounds__(128)
k_bnd_block(const int* __restrict__ ien, const int* __restrict__ ibcb, const double* __restrict__ bcb, int ne,
            const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ res, Phys<double> P) {
    constexpr int NSHL = LCSYST == 2 ? 8 : 6;
    constexpr int NSHLB = LCSYST == 3 ? 3 : 4;
    constexpr int NQ = LCSYST == 3 ? 3 : 4;
    const BndTab& T = c_btab[LCSYST - 2];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int nd[NSHL];
    double xl[NSHL][3], yl[NSHL][5];
#pragma unroll
    for (int a = 0; a < NSHL; ++a) {
        nd[a] = ien[(size_t)NSHL * e + a];
#pragma unroll
        for (int d = 0; d < 3; ++d) xl[a][d] = x[3 * (size_t)nd[a] + d];
#pragma unroll
        for (int k = 0; k < 5; ++k) yl[a][k] = y[5 * (size_t)nd[a] + k];
    }
    const int flags = ibcb[2 * (size_t)e];
    const double* bc = bcb + (size_t)NSHLB * 6 * e;
    double rl[NSHLB][5];
#pragma unroll
    for (int n = 0; n < NSHLB; ++n)
#pragma unroll
        for (int k = 0; k < 5; ++k) rl[n][k] = 0.0;
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        const double* N = T.shpb[q];
        double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int n = 0; n < NSHLB; ++n) {
            const int l = face_node<LCSYST>(n);
#pragma unroll
            for (int k = 0; k < 5; ++k) v[k] += N[l] * yl[l][k];
        }
        const double pres = v[0], u0 = v[1], u1 = v[2], u2 = v[3], Tq = v[4];
        const double rk = 0.5 * (u0 * u0 + u1 * u1 + u2 * u2);
        const double rho = pres / (P.Rgas * Tq);
        const double ei = Tq * P.cv;
        double dx[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
        for (int a = 0; a < NSHL; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) dx[i][j] += xl[a][i] * T.shglb[q][j][a];
        double t1, t2, t3;
        if (LCSYST == 4) {
            t1 = dx[1][0] * dx[2][2] - dx[1][2] * dx[2][0];
            t2 = dx[2][0] * dx[0][2] - dx[2][2] * dx[0][0];
            t3 = dx[0][0] * dx[1][2] - dx[0][2] * dx[1][0];
        } else {
            double v1[3], v2[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                v1[i] = xl[1][i] - xl[0][i];
                v2[i] = xl[2][i] - xl[0][i];
            }
            t1 = -v1[1] * v2[2] + v2[1] * v1[2];
            t2 = -v2[0] * v1[2] + v1[0] * v2[2];
            t3 = -v1[0] * v2[1] + v2[0] * v1[1];
        }
        const double rn = 1.0 / sqrt(t1 * t1 + t2 * t2 + t3 * t3);
        const double bn[3] = {t1 * rn, t2 * rn, t3 * rn};
        const double WdetJb = LCSYST == 3 ? (1.0 - T.Qwtb[q]) / (4.0 * rn)
                            : LCSYST == 4 ? T.Qwtb[q] / rn : T.Qwtb[q] / (4.0 * rn);
        double rou = 0.0, p = 0.0, Fv[3] = {0.0, 0.0, 0.0}, Fh5 = 0.0;
#pragma unroll
        for (int n = 0; n < NSHLB; ++n) {
            const double w = N[face_node<LCSYST>(n)];
            rou += w * bc[6 * n + 0];
            p += w * bc[6 * n + 1];
            Fv[0] += w * bc[6 * n + 2];
            Fv[1] += w * bc[6 * n + 3];
            Fv[2] += w * bc[6 * n + 4];
            Fh5 += w * bc[6 * n + 5];
        }
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
            // grad-V: the inverse deformation gradient (e3bvar.f:202-227), local gradients over
            // all nodes, velocity and temperature gradients (dof 1..4)
            double di[3][3];
            di[0][0] = dx[1][1] * dx[2][2] - dx[2][1] * dx[1][2];
            di[0][1] = dx[2][1] * dx[0][2] - dx[0][1] * dx[2][2];
            di[0][2] = dx[0][1] * dx[1][2] - dx[0][2] * dx[1][1];
            const double rd = 1.0 / (di[0][0] * dx[0][0] + di[0][1] * dx[1][0] + di[0][2] * dx[2][0]);
            di[0][0] *= rd;
            di[0][1] *= rd;
            di[0][2] *= rd;
            di[1][0] = (dx[1][2] * dx[2][0] - dx[1][0] * dx[2][2]) * rd;
            di[1][1] = (dx[0][0] * dx[2][2] - dx[2][0] * dx[0][2]) * rd;
            di[1][2] = (dx[1][0] * dx[0][2] - dx[0][0] * dx[1][2]) * rd;
            di[2][0] = (dx[1][0] * dx[2][1] - dx[1][1] * dx[2][0]) * rd;
            di[2][1] = (dx[2][0] * dx[0][1] - dx[0][0] * dx[2][1]) * rd;
            di[2][2] = (dx[0][0] * dx[1][1] - dx[0][1] * dx[1][0]) * rd;
            double gl[3][5] = {{0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0}};
#pragma unroll
            for (int a = 0; a < NSHL; ++a)
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 1; k < 5; ++k) gl[i][k] += T.shglb[q][i][a] * yl[a][k];
            double G[3][5];
#pragma unroll
            for (int k = 1; k < 5; ++k)
#pragma unroll
                for (int i = 0; i < 3; ++i) G[i][k] = di[0][i] * gl[0][k] + di[1][i] * gl[1][k] + di[2][i] * gl[2][k];
            const double tau1n = bn[0] * (P.rlm2mu * G[0][1] + P.rlm * G[1][2] + P.rlm * G[2][3]) +
                                 bn[1] * (P.rmu * (G[1][1] + G[0][2])) + bn[2] * (P.rmu * (G[2][1] + G[0][3]));
            const double tau2n = bn[0] * (P.rmu * (G[1][1] + G[0][2])) +
                                 bn[1] * (P.rlm * G[0][1] + P.rlm2mu * G[1][2] + P.rlm * G[2][3]) +
                                 bn[2] * (P.rmu * (G[2][2] + G[1][3]));
            const double tau3n = bn[0] * (P.rmu * (G[2][1] + G[0][3])) + bn[1] * (P.rmu * (G[2][2] + G[1][3])) +
                                 bn[2] * (P.rlm * G[0][1] + P.rlm * G[1][2] + P.rlm2mu * G[2][3]);
            if (!(flags & 4)) {
                Fv[0] = tau1n;
                Fv[1] = tau2n;
                Fv[2] = tau3n;
            }
            const double Fv5 = u0 * Fv[0] + u1 * Fv[1] + u2 * Fv[2];
            const double heat = -P.con * (bn[0] * G[0][4] + bn[1] * G[1][4] + bn[2] * G[2][4]);
            if (!(flags & 8)) Fh5 = heat;
            F[1] -= Fv[0];
            F[2] -= Fv[1];
            F[3] -= Fv[2];
            F[4] = F[4] - Fv5 + Fh5;
        }
#pragma unroll
        for (int n = 0; n < NSHLB; ++n) {
            const double w = WdetJb * N[face_node<LCSYST>(n)];
#pragma unroll
            for (int k = 0; k < 5; ++k) rl[n][k] += w * F[k];
        }
    }
#pragma unroll
    for (int n = 0; n < NSHLB; ++n) {
        double* o = res + 5 * (size_t)nd[face_node<LCSYST>(n)];
#pragma unroll
        for (int k = 0; k < 5; ++k) o[k] += rl[n][k];
    }
}

#define BD_TRY(x)                      \
    do {                               \
        const int _s = (x);            \
        if (_s != PHGPU_OK) return _s; \
    } while (0)

template <typename T>
int balloc(Ctx& C, T** p, size_t n) {
    *p = nullptr;
    const cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (n ? n : 1));
    if (e != cudaSuccess) return fail(C, PHGPU_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return PHGPU_OK;
}

}  // namespace

int bnd_setup(Ctx& C, const phgpu_mesh* m) {
    if (m->nbblk <= 0) return PHGPU_OK;
    if (!m->bblk) return fail(C, PHGPU_ERR_INVALID, "nbblk > 0 with no boundary blocks");
    std::vector<BndTab> host(3);
    bnd_tables_host(host.data());
    BD_TRY(check(C, cudaMemcpyToSymbolAsync(c_btab, host.data(), sizeof(BndTab) * 3, 0, cudaMemcpyHostToDevice,
                                            C.stream),
                 "boundary tables"));
    BD_TRY(check(C, cudaStreamSynchronize(C.stream), "boundary tables"));  // the source is a local
    for (int b = 0; b < m->nbblk; ++b) {
        const phgpu_bnd_block& B = m->bblk[b];
        if (B.lcsyst < 2 || B.lcsyst > 4 || B.nelem < 0 || (B.nelem > 0 && (!B.ien || !B.iBCB || !B.BCB)))
            return fail(C, PHGPU_ERR_INVALID, "boundary block: lcsyst 2, 3 or 4 with ien, iBCB and BCB");
        BndBlockDev D;
        D.lcsyst = B.lcsyst;
        D.nelem = B.nelem;
        D.nshl = B.lcsyst == 2 ? 8 : 6;
        D.nshlb = B.lcsyst == 3 ? 3 : 4;
        for (size_t i = 0; i < (size_t)D.nshl * B.nelem; ++i)
            if (B.ien[i] < 0 || B.ien[i] >= C.N) return fail(C, PHGPU_ERR_INVALID, "boundary block connectivity");
        if (B.nelem == 0) continue;
        std::vector<int> order;
        BD_TRY(colour(C, C.N, B.ien, D.nshl, B.nelem, order, D.col_start));
        std::vector<int> ien((size_t)D.nshl * B.nelem), ibcb(2 * (size_t)B.nelem);
        std::vector<double> bcb((size_t)D.nshlb * 6 * B.nelem);
        for (int i = 0; i < B.nelem; ++i) {
            const size_t e = order[i];
            for (int a = 0; a < D.nshl; ++a) ien[(size_t)D.nshl * i + a] = B.ien[(size_t)D.nshl * e + a];
            ibcb[2 * (size_t)i] = B.iBCB[2 * e];
            ibcb[2 * (size_t)i + 1] = B.iBCB[2 * e + 1];
            for (int k = 0; k < D.nshlb * 6; ++k) bcb[(size_t)D.nshlb * 6 * i + k] = B.BCB[(size_t)D.nshlb * 6 * e + k];
        }
        C.bblk.push_back(D);
        BndBlockDev& d = C.bblk.back();
        BD_TRY(balloc(C, &d.d_ien, ien.size()));
        BD_TRY(balloc(C, &d.d_ibcb, ibcb.size()));
        BD_TRY(balloc(C, &d.d_bcb, bcb.size()));
        BD_TRY(check(C, cudaMemcpyAsync(d.d_ien, ien.data(), sizeof(int) * ien.size(), cudaMemcpyHostToDevice,
                                        C.stream), "boundary block"));
        BD_TRY(check(C, cudaMemcpyAsync(d.d_ibcb, ibcb.data(), sizeof(int) * ibcb.size(), cudaMemcpyHostToDevice,
                                        C.stream), "boundary block"));
        BD_TRY(check(C, cudaMemcpyAsync(d.d_bcb, bcb.data(), sizeof(double) * bcb.size(), cudaMemcpyHostToDevice,
                                        C.stream), "boundary block"));
        // the host vectors go out of scope
        BD_TRY(check(C, cudaStreamSynchronize(C.stream), "boundary block"));
    }
    return PHGPU_OK;
}

void bnd_free(Ctx& C) {
    for (BndBlockDev& d : C.bblk) {
        cudaFree(d.d_ien);
        cudaFree(d.d_ibcb);
        cudaFree(d.d_bcb);
    }
    C.bblk.clear();
}

void launch_bnd_blocks(Ctx& C, const double* y, double* res) {
    if (C.bblk.empty()) return;
    const Phys<double> P = make_phys<double>(C.cfg);
    for (const BndBlockDev& d : C.bblk) {
        const int ncol = (int)d.col_start.size() - 1;
        for (int c = 0; c < ncol; ++c) {
            const int e0 = d.col_start[c], ne = d.col_start[c + 1] - e0;
            if (ne <= 0) continue;
            const int grid = (ne + 127) / 128;
            const int* ien = d.d_ien + (size_t)d.nshl * e0;
            const int* ibcb = d.d_ibcb + 2 * (size_t)e0;
            const double* bcb = d.d_bcb + (size_t)d.nshlb * 6 * e0;
            if (d.lcsyst == 2)
                k_bnd_block<2><<<grid, 128, 0, C.stream>>>(ien, ibcb, bcb, ne, C.d_x, y, res, P);
            else if (d.lcsyst == 3)
                k_bnd_block<3><<<grid, 128, 0, C.stream>>>(ien, ibcb, bcb, ne, C.d_x, y, res, P);
            else
                k_bnd_block<4><<<grid, 128, 0, C.stream>>>(ien, ibcb, bcb, ne, C.d_x, y, res, P);
            ++C.launches;
        }
    }
}

}  // namespace phgpu
