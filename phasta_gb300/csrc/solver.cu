// solver.cu -- set-up (colouring, device mirrors) and the drivers of the hot
// path: ElmMFG (elmmfg.f), ItrRes (itrres.f), SolMFG (solmfg.f: block-LU
// preconditioning, finite-difference or linearized Au1MFG, MGS Arnoldi,
// Givens least squares), itrFDI (itrfdi.f), itrCorrect/itrBC/itrUpdate
// (itrPC.f, itrbc.f) and the C ABI of include/phgpu.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <type_traits>

#include "phgpu_impl.cuh"
#include "df64.cuh"

namespace phgpu {

int check(Ctx& C, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return PHGPU_OK;
    if (C.err.empty()) C.err = std::string(what) + ": " + cudaGetErrorString(e);
    return PHGPU_ERR_CUDA;
}

int fail(Ctx& C, int code, const std::string& msg) {
    C.err = msg;
    return code;
}

namespace {
// a synchronous copy cannot be part of a graph: every host set-up runs before a capture starts
int not_capturing(Ctx& C, const char* what) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(C.stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
        return fail(C, PHGPU_ERR_CUDA, std::string(what) + ": host copy while the stream is captured");
    return PHGPU_OK;
}
}  // namespace

int h2d(Ctx& C, void* dst, const void* src, size_t bytes, const char* what) {
    if (bytes == 0) return PHGPU_OK;
    int rc = not_capturing(C, what);
    if (rc == PHGPU_OK) rc = check(C, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, C.stream), what);
    return rc != PHGPU_OK ? rc : check(C, cudaStreamSynchronize(C.stream), what);
}

int d2h(Ctx& C, void* dst, const void* src, size_t bytes, const char* what) {
    if (bytes == 0) return PHGPU_OK;
    int rc = not_capturing(C, what);
    if (rc == PHGPU_OK) rc = check(C, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, C.stream), what);
    return rc != PHGPU_OK ? rc : check(C, cudaStreamSynchronize(C.stream), what);
}

int dzero(Ctx& C, void* dst, size_t bytes, const char* what) {
    return bytes == 0 ? PHGPU_OK : check(C, cudaMemsetAsync(dst, 0, bytes, C.stream), what);
}

namespace {

#define PH_TRY(x)                          \
    do {                                   \
        int _s = (x);                      \
        if (_s != PHGPU_OK) return _s;     \
    } while (0)

template <typename T>
int dalloc(Ctx& C, T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
    if (e != cudaSuccess) {
        C.err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return PHGPU_ERR_NOMEM;
    }
    return PHGPU_OK;
}

int sync(Ctx& C) {
    PH_TRY(check(C, cudaGetLastError(), "kernel launch"));
    return check(C, cudaStreamSynchronize(C.stream), "stream synchronize");
}

}  // namespace

// greedy first-fit colouring: no two elements of a colour share a node
int colour(Ctx& C, int n_nodes, const int* ien, int nen, int ne, std::vector<int>& order, std::vector<int>& start) {
    std::vector<uint64_t> m0(n_nodes, 0), m1(n_nodes, 0);
    std::vector<int> col(ne);
    int ncol = 0;
    for (int e = 0; e < ne; ++e) {
        const int* nd = ien + nen * (size_t)e;
        uint64_t f0 = 0, f1 = 0;
        for (int a = 0; a < nen; ++a) {
            f0 |= m0[nd[a]];
            f1 |= m1[nd[a]];
        }
        int c;
        if (~f0) c = __builtin_ctzll(~f0);
        else if (~f1) c = 64 + __builtin_ctzll(~f1);
        else return fail(C, PHGPU_ERR_UNSUPPORTED, "element colouring needs more than 128 colours");
        col[e] = c;
        ncol = std::max(ncol, c + 1);
        for (int a = 0; a < nen; ++a) {
            if (c < 64) m0[nd[a]] |= (1ull << c);
            else m1[nd[a]] |= (1ull << (c - 64));
        }
    }
    start.assign(ncol + 1, 0);
    for (int e = 0; e < ne; ++e) start[col[e] + 1]++;
    for (int c = 0; c < ncol; ++c) start[c + 1] += start[c];
    std::vector<int> pos(start.begin(), start.end() - 1);
    order.resize(ne);
    for (int e = 0; e < ne; ++e) order[pos[col[e]]++] = e;
    return PHGPU_OK;
}

namespace {

// ------------------------------------------------------------------------
// small device kernels of the driver
// ------------------------------------------------------------------------
template <typename V>
__global__ void k_axpy_pre(const double* __restrict__ ypre, const V* __restrict__ u, double e, V* __restrict__ t,
                           size_t n, const int* skip) {
    if (skip && *skip) return;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        t[i] = (V)(ypre[i] + e * (double)u[i]);
}
template <typename V>
__global__ void k_fd_diff(const V* __restrict__ ub, const V* __restrict__ rmes, double e, V* __restrict__ u,
                          size_t n, const int* skip) {
    if (skip && *skip) return;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        u[i] = (ub[i] - rmes[i]) / (V)e;
}
// u = res - (ub1 - ub2) / (2 eps)  (au2mfg.f:104)
__global__ void k_cd_diff(const double* __restrict__ res, const double* ub1, const double* __restrict__ ub2,
                          double two_eps, double* u, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        u[i] = res[i] - (ub1[i] - ub2[i]) / two_eps;
}
template <typename V>
__global__ void k_copy(const V* __restrict__ a, V* __restrict__ b, size_t n, const int* skip) {
    if (skip && *skip) return;
    // 16-byte vectors when both arrays allow them, then the elements the vectors leave
    const bool vec = (((uintptr_t)a | (uintptr_t)b) & 15) == 0;
    const size_t W = 16 / sizeof(V), nv = vec ? n / W : 0;
    const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = t0; i < nv; i += stride) reinterpret_cast<float4*>(b)[i] = reinterpret_cast<const float4*>(a)[i];
    for (size_t i = W * nv + t0; i < n; i += stride) b[i] = a[i];
}
__global__ void k_fdi_combine(double* __restrict__ r, const double* __restrict__ rmes, double epsM, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double d = (r[i] - 2.0 * rmes[i]) / epsM;
        r[i] = d;
    }
}
__global__ void k_axpby(const double* __restrict__ a, double alpha, const double* __restrict__ b, double beta,
                        double* __restrict__ o, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        o[i] = alpha * a[i] + beta * b[i];
}

// Givens update of column iKs (solmfg.f:274-317); also sets H(iKs+1,iKs) = sqrt(beta).
// Inside a captured cycle (open_next) it opens the next iteration's conditional node
// unless the cycle has converged or failed.
__global__ void k_givens(double* __restrict__ s, int K, int iKs, int minIters, int* __restrict__ flag,
                         cudaGraphConditionalHandle next, int open_next, int capped) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (flag[0]) return;
    auto H = [&](int i, int j) -> double& { return s[S_H + (i - 1) + (K + 1) * (j - 1)]; };
    double* eB = s + S_EB;
    double* Rc = s + S_RC;
    double* Rs = s + S_RS;
    const double unorm = sqrt(H(iKs + 1, iKs));
    H(iKs + 1, iKs) = unorm;
    s[S_TMP2] = unorm;  // the last norm of the cycle (a sparse-solver restart without a new residual)
    for (int jK = 1; jK <= iKs - 1; ++jK) {
        const double t = Rc[jK - 1] * H(jK, iKs) + Rs[jK - 1] * H(jK + 1, iKs);
        H(jK + 1, iKs) = -Rs[jK - 1] * H(jK, iKs) + Rc[jK - 1] * H(jK + 1, iKs);
        H(jK, iKs) = t;
    }
    const double t = sqrt(H(iKs, iKs) * H(iKs, iKs) + H(iKs + 1, iKs) * H(iKs + 1, iKs));
    Rc[iKs - 1] = H(iKs, iKs) / t;
    Rs[iKs - 1] = H(iKs + 1, iKs) / t;
    H(iKs, iKs) = t;
    H(iKs + 1, iKs) = 0.0;
    const double te = Rc[iKs - 1] * eB[iKs - 1] + Rs[iKs - 1] * eB[iKs];
    eB[iKs] = -Rs[iKs - 1] * eB[iKs - 1] + Rc[iKs - 1] * eB[iKs];
    eB[iKs - 1] = te;
    const double echeck = fabs(eB[iKs]);
    s[S_ECHECK] = echeck;
    if (!(echeck == echeck)) flag[1] |= 2;
    if (echeck <= s[S_EPSNRM] && iKs >= minIters) flag[0] = 1;
    flag[2] = iKs;
    // capped: a learned flexible-GMRES cycle stops at flag[3] iterations (then block-diagonal
    // cycles take over)
    const bool stop = (flag[0] | flag[1]) || (capped && iKs >= flag[3]);
    if (open_next) cudaGraphSetConditional(next, stop ? 0u : 1u);
}

// back substitution H y = e (solmfg.f:329-334)
// (iks_dev: the iteration count a captured cycle left on the device, read in place of iKs)
__global__ void k_backsolve(double* __restrict__ s, int K, int iKs, const int* __restrict__ iks_dev) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (iks_dev) iKs = min(max(*iks_dev, 0), K);
    auto H = [&](int i, int j) -> double { return s[S_H + (i - 1) + (K + 1) * (j - 1)]; };
    double* eB = s + S_EB;
    double* yB = s + S_YB;
    for (int jK = iKs; jK >= 1; --jK) {
        yB[jK - 1] = eB[jK - 1] / H(jK, jK);
        for (int lK = 1; lK <= jK - 1; ++lK) eB[lK - 1] = eB[lK - 1] - yB[jK - 1] * H(lK, jK);
    }
}

// Dy = Dy + sum_j yBrg(j) u_j (solmfg.f:338-340).  FP32 Krylov vectors: the sum over j
// runs in double-float (coefficients split once per block), then one FP64 add per entry.
template <typename V>
__global__ void k_update_dy(double* __restrict__ Dy, const V* __restrict__ U, size_t ld, int iKs, int K,
                            const double* __restrict__ s, size_t n, const int* __restrict__ iks_dev) {
    if (iks_dev) iKs = min(max(*iks_dev, 0), K);
    const double* yB = s + S_YB;
    if constexpr (std::is_same<V, float>::value) {
        __shared__ float ch[kMaxK], cl[kMaxK];
        for (int j = threadIdx.x; j < iKs; j += blockDim.x) {
            ch[j] = (float)yB[j];
            cl[j] = (float)(yB[j] - (double)ch[j]);
        }
        __syncthreads();
        const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
        // four entries per thread and pass: 16-byte loads of every basis row and of Dy (the rows
        // start on 256-byte boundaries); each entry's sum over j in the same order as one at a time
        const size_t n4 = ((reinterpret_cast<uintptr_t>(U) & 15) == 0 && ld % 4 == 0 &&
                           (reinterpret_cast<uintptr_t>(Dy) & 15) == 0)
                              ? n / 4
                              : 0;
        for (size_t i4 = t0; i4 < n4; i4 += stride) {
            df64 acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
            for (int j = 0; j < iKs; ++j) {
                const float4 u = *reinterpret_cast<const float4*>(U + (size_t)j * ld + 4 * i4);
                const df64 c = df_make(ch[j], cl[j]);
                acc[0] = df_add(acc[0], df_mul(c, u.x));
                acc[1] = df_add(acc[1], df_mul(c, u.y));
                acc[2] = df_add(acc[2], df_mul(c, u.z));
                acc[3] = df_add(acc[3], df_mul(c, u.w));
            }
            double2* d = reinterpret_cast<double2*>(Dy + 4 * i4);
            double2 d0 = d[0], d1 = d[1];
            d0.x = d0.x + df_to_double(acc[0]);
            d0.y = d0.y + df_to_double(acc[1]);
            d1.x = d1.x + df_to_double(acc[2]);
            d1.y = d1.y + df_to_double(acc[3]);
            d[0] = d0;
            d[1] = d1;
        }
        for (size_t i = 4 * n4 + t0; i < n; i += stride) {
            df64 acc{0.f, 0.f};
            for (int j = 0; j < iKs; ++j) acc = df_add(acc, df_mul(df_make(ch[j], cl[j]), U[(size_t)j * ld + i]));
            Dy[i] = Dy[i] + df_to_double(acc);
        }
    } else {
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
            double d = Dy[i];
            for (int j = 0; j < iKs; ++j) d = d + yB[j] * (double)U[(size_t)j * ld + i];
            Dy[i] = d;
        }
    }
}

__global__ void k_init_cycle(double* __restrict__ s, int K, double unorm, double epsnrm, int* flag, int cap) {
    const int t = threadIdx.x;
    for (int i = t; i < K + 1; i += blockDim.x) s[S_EB + i] = 0.0;
    for (int i = t; i < (K + 1) * K; i += blockDim.x) s[S_H + i] = 0.0;
    if (t == 0) {
        s[S_EB] = unorm;
        s[S_UNORM] = unorm;
        s[S_EPSNRM] = epsnrm;
        s[S_ECHECK] = 0.0;
        flag[0] = 0;
        flag[2] = 0;
        flag[3] = cap;
    }
}

// k_init_cycle with the norm on the device: unorm = ||L^-1 R|| from S_TMP0, epsnrm = etol unorm
// (solmfg.f:161); opens the cycle's first Krylov iteration unless the norm is below the
// early-exit bound (solmfg.f:158), not finite, or the LU reported a pivot failure
__global__ void k_init_cycle_dev(double* __restrict__ s, int K, double etol, double tiny, int* flag,
                                 cudaGraphConditionalHandle first) {
    const int t = threadIdx.x;
    const double unorm = sqrt(s[S_TMP0]);
    for (int i = t; i < K + 1; i += blockDim.x) s[S_EB + i] = 0.0;
    for (int i = t; i < (K + 1) * K; i += blockDim.x) s[S_H + i] = 0.0;
    if (t == 0) {
        s[S_EB] = unorm;
        s[S_UNORM] = unorm;
        s[S_EPSNRM] = etol * unorm;
        s[S_ECHECK] = 0.0;
        flag[0] = 0;
        flag[2] = 0;
        flag[3] = K;
        const bool finite = unorm == unorm && unorm <= 1.7976931348623157e308;
        if (!finite) flag[1] |= 2;
        cudaGraphSetConditional(first, (finite && !(unorm < tiny) && flag[1] == 0) ? 1u : 0u);
    }
}

// statistics of one Newton iteration of the step graph: [0] ||R||^2, [1] ||L^-1 R||^2, [2] the
// final |eBrg| of the cycle, [3] its Krylov iterations, [4] the LU status, [5] the error bits
// after the cycle
__global__ void k_step_record(const double* __restrict__ s, const int* __restrict__ flag, double* out, int phase) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (phase == 0) {
        out[0] = s[S_TMP3];
        out[1] = s[S_TMP0];
        out[4] = flag[1];
    } else {
        out[2] = s[S_ECHECK];
        out[3] = flag[2];
        out[5] = flag[1];
    }
}

// itrCorrect (itrPC.f:128-148) in the device's local dof order
__global__ void k_correct(double* __restrict__ y, double* __restrict__ ac, const double* __restrict__ yold,
                          const double* __restrict__ acold, const double* __restrict__ Dy, double fct1,
                          double fct2, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double yi = y[i] - Dy[i];
        y[i] = yi;
        ac[i] = acold[i] * fct1 + (yi - yold[i]) * fct2;
    }
}
__global__ void k_predict(const double* __restrict__ yold, const double* __restrict__ acold, double* __restrict__ y,
                          double* __restrict__ ac, double f, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        y[i] = yold[i];
        ac[i] = acold[i] * f;
    }
}
__global__ void k_update(double* __restrict__ yold, double* __restrict__ acold, const double* __restrict__ y,
                         const double* __restrict__ ac, double fct2, double fct3, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        acold[i] = acold[i] + (ac[i] - acold[i]) * fct2;
        yold[i] = yold[i] + (y[i] - yold[i]) * fct3;
    }
}

constexpr int kVG = kRedBlocks, kVT = 256;

// ------------------------------------------------------------------------
// ElmMFG / residual drivers on resident device data
// ------------------------------------------------------------------------
// idiff = 1: the reconstructed diffusive flux of state y in d_qres (elmmfg.f:56-111)
const double* reconstruct_q(Ctx& C, const double* y) {
    if (C.cfg.idiff != 1) return nullptr;
    fill0(C, C.d_qres, sizeof(double) * 13 * (size_t)C.N);
    launch_qrec<double>(C, C.d_x, y, C.d_qres);
    qpbc<double>(C, C.d_qres);
    return C.d_qres;
}

int elmres64(Ctx& C, const double* y, const double* ac, double* res) {
    const double* ql = reconstruct_q(C, y);
    fill0(C, res, sizeof(double) * 5 * (size_t)C.N);
    launch_elem_res<double>(C, RM_RES, C.d_x, y, nullptr, ac, res, 0, nullptr, ql);
    if (has_boundary(C)) launch_boundary(C, y, res);
    bc3res<double>(C, res);
    return check(C, cudaGetLastError(), "elmres");
}

int elmmfg64(Ctx& C, const double* y, const double* ac, double* res, double* rmes, double* bd, int iprec) {
    const size_t N = C.N;
    const double* ql = reconstruct_q(C, y);
    fill0(C, res, sizeof(double) * 5 * N);
    fill0(C, rmes, sizeof(double) * 5 * N);
    if (iprec) {
        fill0(C, bd, sizeof(double) * 25 * N);
        launch_elem_full<double>(C, C.d_x, y, ac, res, rmes, bd, ql);
    } else {
        launch_elem_res<double>(C, RM_RES, C.d_x, y, nullptr, ac, res, 0, nullptr, ql);
        launch_elem_res<double>(C, RM_MODRES, C.d_x, y, y, ac, rmes, 0, nullptr);
    }
    if (has_boundary(C)) launch_boundary(C, y, res);
    bc3res<double>(C, res);
    bc3res<double>(C, rmes);
    if (iprec) bc3bdg<double>(C, y, bd);
    return check(C, cudaGetLastError(), "elmmfg");
}

// the FP64 tangent of ElmGMRs (lhs = 1: lhsK) or ElmGMRe (ebe: element storage), and BDiag
// from its diagonal blocks + bc3BDg
int tangent64(Ctx& C, const double* y, double* out, double* bd, bool ebe = false) {
    fill0(C, bd, sizeof(double) * 25 * (size_t)C.N);
    if (ebe) {
        launch_tangent_ebe<double>(C, C.d_x, y, out, bd);
    } else {
        fill0(C, out, sizeof(double) * 25 * (size_t)C.sp.nnzb);
        launch_tangent<double>(C, C.d_x, y, out, bd);
    }
    bc3bdg<double>(C, y, bd);
    return check(C, cudaGetLastError(), "tangent");
}

// rmes += Rmod(yp; yc) then bc3Res (itrres.f)
template <typename R>
int itrres_dev(Ctx& C, const R* x, const R* yp, const R* yc, R* rmes, int iabres, const int* skip) {
    launch_elem_res<R>(C, RM_MODRES, x, yp, yc, nullptr, rmes, iabres, skip);
    bc3res<R>(C, rmes);
    return PHGPU_OK;
}

// ------------------------------------------------------------------------
// SolMFG
// ------------------------------------------------------------------------
template <typename V>
struct KrylovOps;

// Jacobian-vector product u <- L^-1 J U^-1 u (Au1MFG, au1mfg.f:57-83)
int ap_fd64(Ctx& C, double* u, const double* rmes, const int* skip) {
    const size_t n5 = 5 * (size_t)C.N;
    double* t = C.d_t64;
    double* ub = C.d_t64b;
    k_axpy_pre<double><<<kVG, kVT, 0, C.stream>>>(C.d_ypre, u, C.cfg.eGMRES, t, n5, skip);
    ++C.launches;
    lu_apply<double, double>(C, C.d_bd, t, PHGPU_LU_BACKWARD);
    itrbc_pert<double>(C, t, false);
    fill0(C, ub, sizeof(double) * n5);
    itrres_dev<double>(C, C.d_x, t, C.d_y, ub, 0, skip);
    lu_apply<double, double>(C, C.d_bd, ub, PHGPU_LU_FORWARD);
    k_fd_diff<double><<<kVG, kVT, 0, C.stream>>>(ub, rmes, C.cfg.eGMRES, u, n5, skip);
    ++C.launches;
    return PHGPU_OK;
}

// restart vector R - J Dy by a central difference of ItrRes (Au2MFG, au2mfg.f:55-104):
// eps = epsM^(2/3) / ||Dy||, out = res - (R(ypre + eps Dy) - R(ypre - eps Dy)) / (2 eps)
int au2_fd64(Ctx& C, double* out) {
    const size_t n5 = 5 * (size_t)C.N;
    dot<double>(C, C.d_Dy, C.d_Dy, n5, S_TMP0, nullptr);
    PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, C.d_scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream),
                 "Au2MFG norm"));
    PH_TRY(sync(C));
    const double eps = std::pow(C.cfg.epsM, 2.0 / 3.0) / std::sqrt(C.h_scal[S_TMP0]);
    if (!std::isfinite(eps)) return fail(C, PHGPU_ERR_NONFINITE, "Au2MFG: zero or non-finite restart step");
    double* t = C.d_t64;
    double* ub2 = C.d_t64b;
    for (int side = 0; side < 2; ++side) {
        double* ub = side == 0 ? out : ub2;
        k_axpy_pre<double><<<kVG, kVT, 0, C.stream>>>(C.d_ypre, C.d_Dy, side == 0 ? eps : -eps, t, n5, nullptr);
        ++C.launches;
        lu_apply<double, double>(C, C.d_bd, t, PHGPU_LU_BACKWARD);
        itrbc_pert<double>(C, t, false);
        fill0(C, ub, sizeof(double) * n5);
        itrres_dev<double>(C, C.d_x, t, C.d_y, ub, 0, nullptr);
        lu_apply<double, double>(C, C.d_bd, ub, PHGPU_LU_FORWARD);
    }
    k_cd_diff<<<kVG, kVT, 0, C.stream>>>(C.d_res, out, ub2, 2.0 * eps, out, n5);
    ++C.launches;
    return PHGPU_OK;
}

// u_out = L^-1 J U^-1 u_in (u_in may be u_out)
template <typename V>
int ap_lin(Ctx& C, const V* u_in, V* u, const int* skip);

template <>
int ap_lin<double>(Ctx& C, const double* u_in, double* u, const int* skip) {
    const size_t n5 = 5 * (size_t)C.N;
    double* v = C.d_t64;
    lu_apply<double, double>(C, C.d_bd, u_in, v, PHGPU_LU_BACKWARD);
    itrbc_pert<double>(C, v, true);
    fill0(C, u, sizeof(double) * n5);
    launch_elem_res<double>(C, RM_LIN, C.d_x, v, C.d_y, nullptr, u, 0, skip);
    bc3res<double>(C, u);
    lu_apply<double, double>(C, C.d_bd, u, PHGPU_LU_FORWARD);
    return PHGPU_OK;
}

template <>
int ap_lin<float>(Ctx& C, const float* u_in, float* u, const int* skip) {
    const size_t n5 = 5 * (size_t)C.N;
    float* v = C.d_t32;
    lu_apply<float, float>(C, C.d_bdf, u_in, v, PHGPU_LU_BACKWARD);
    itrbc_pert<float>(C, v, true);
    fill0(C, u, sizeof(float) * n5);
    launch_elem_res<float>(C, RM_LIN, C.d_xf, v, C.d_yf, nullptr, u, 0, skip);
    bc3res<float>(C, u);
    lu_apply<float, float>(C, C.d_bdf, u, PHGPU_LU_FORWARD);
    return PHGPU_OK;
}

// itrFDI (itrfdi.f:45-139), FP64
int itrfdi_dev(Ctx& C, const double* rmes, const double* ubrg) {
    const size_t n5 = 5 * (size_t)C.N;
    double* rt = C.d_t64b;
    double* yt = C.d_t64;
    // cancellation error epsA
    fill0(C, rt, sizeof(double) * n5);
    k_copy<double><<<kVG, kVT, 0, C.stream>>>(C.d_ypre, yt, n5, nullptr);
    ++C.launches;
    lu_apply<double, double>(C, C.d_bd, yt, PHGPU_LU_BACKWARD);
    itrres_dev<double>(C, C.d_x, yt, C.d_y, rt, 1, nullptr);
    lu_apply<double, double>(C, C.d_bd, rt, PHGPU_LU_FORWARD);
    dot<double>(C, rt, rt, n5, S_TMP0, nullptr);
    // second derivative
    const double epsSD = std::sqrt(C.cfg.epsM);
    fill0(C, rt, sizeof(double) * n5);
    k_axpy_pre<double><<<kVG, kVT, 0, C.stream>>>(C.d_ypre, ubrg, epsSD, yt, n5, nullptr);
    ++C.launches;
    lu_apply<double, double>(C, C.d_bd, yt, PHGPU_LU_BACKWARD);
    itrres_dev<double>(C, C.d_x, yt, C.d_y, rt, 0, nullptr);
    k_axpy_pre<double><<<kVG, kVT, 0, C.stream>>>(C.d_ypre, ubrg, -epsSD, yt, n5, nullptr);
    ++C.launches;
    lu_apply<double, double>(C, C.d_bd, yt, PHGPU_LU_BACKWARD);
    itrres_dev<double>(C, C.d_x, yt, C.d_y, rt, 0, nullptr);
    lu_apply<double, double>(C, C.d_bd, rt, PHGPU_LU_FORWARD);
    k_fdi_combine<<<kVG, kVT, 0, C.stream>>>(rt, rmes, C.cfg.epsM, n5);
    ++C.launches;
    dot<double>(C, rt, rt, n5, S_TMP1, nullptr);
    PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, C.d_scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream), "fdi"));
    PH_TRY(sync(C));
    const double epsA = (C.cfg.epsM * C.cfg.epsM) * std::sqrt(C.h_scal[S_TMP0]);
    const double SDnrm = std::sqrt(C.h_scal[S_TMP1]);
    C.cfg.eGMRES = 2.0 * std::sqrt(epsA / SDnrm);
    if (!std::isfinite(C.cfg.eGMRES) || C.cfg.eGMRES <= 0.0)
        return fail(C, PHGPU_ERR_NONFINITE, "itrFDI produced a non-finite finite-difference interval");
    return PHGPU_OK;
}

template <typename V> V* sparse_lhs(Ctx& C);
template <> double* sparse_lhs<double>(Ctx& C) { return C.sp.d_lhsK; }
template <> float* sparse_lhs<float>(Ctx& C) { return C.sp.d_lhsKf; }
template <typename V> V* ebe_lhs(Ctx& C);
template <> double* ebe_lhs<double>(Ctx& C) { return C.sp.d_EG; }
template <> float* ebe_lhs<float>(Ctx& C) { return C.sp.d_EGf; }

// q = A p for the assembled (SparseAp) or element-by-element (Au1GMR) operator, then bc3per
template <typename V>
void assembled_ap(Ctx& C, bool ebe, const V* p, V* q) {
    if (ebe) ebe_ap<V, V>(C, ebe_lhs<V>(C), p, q);
    else sparse_ap<V, V>(C, sparse_lhs<V>(C), p, q);
}

// Krylov iteration iK of a cycle (solmfg.f:230-317): the product into u_{iK+1}, modified
// Gram-Schmidt against u_1..u_iK, the new vector's norm and the Givens update
template <typename V>
int krylov_step(Ctx& C, int iK, int min_iters, bool sparse, bool ebe, cudaGraphConditionalHandle next,
                int open_next, bool learned = false) {
    const size_t n5 = 5 * (size_t)C.N;
    const int K = C.cfg.Kspace;
    V* U = (V*)C.d_U;
    auto Uj = [&](int j) { return U + (size_t)(j - 1) * C.ldU; };  // 1-based
    double* s = C.d_scal;
    V* w = Uj(iK + 1);
    if constexpr (std::is_same<V, float>::value) {
        if (learned) {
            // flexible GMRES: z_iK = P(u_iK) kept for the solution, w = A~ z_iK
            float* z = C.net.d_Z + (size_t)(iK - 1) * C.ldU;
            net_apply(C, Uj(iK), z);
            PH_TRY(ap_lin<V>(C, z, w, nullptr));
        }
    }
    if (learned) {
    } else if (sparse) {
        assembled_ap<V>(C, ebe, Uj(iK), w);
    } else if constexpr (std::is_same<V, double>::value) {
        if (C.cfg.ap_mode == PHGPU_AP_FD) {
            k_copy<V><<<kVG, kVT, 0, C.stream>>>(Uj(iK), w, n5, nullptr);
            ++C.launches;
            PH_TRY(ap_fd64(C, w, C.d_rmes, nullptr));
        } else {
            PH_TRY(ap_lin<V>(C, Uj(iK), w, nullptr));
        }
    } else {
        PH_TRY(ap_lin<V>(C, Uj(iK), w, nullptr));
    }
    // modified Gram-Schmidt (solmfg.f:247-267)
    double* Hcol = s + S_H + (size_t)(K + 1) * (iK - 1);
    for (int jK = 1; jK <= iK + 1; ++jK) {
        const V* up = (jK == 1) ? nullptr : Uj(jK - 1);
        const double* bprev = (jK == 1) ? nullptr : Hcol + (jK - 2);
        mgs_step<V>(C, w, up, bprev, Uj(jK), n5, Hcol + (jK - 1), nullptr);
    }
    scale_by<V>(C, w, Hcol + iK, 1, n5, nullptr);
    k_givens<<<1, 1, 0, C.stream>>>(s, K, iK, min_iters, C.d_flag, next, open_next, learned ? 1 : 0);
    ++C.launches;
    return check(C, cudaGetLastError(), "krylov step");
}

}  // namespace

void cycle_graph_free(CycleGraph& G) {
    if (G.exec) cudaGraphExecDestroy(G.exec);
    if (G.graph) cudaGraphDestroy(G.graph);
    G.exec = nullptr;
    G.graph = nullptr;
}
void cycle_graph_free(Ctx& C) {
    cycle_graph_free(C.cyc);
    cycle_graph_free(C.cyc_net);
}

namespace {

// Capture the Krylov iterations of a cycle as a graph of conditional nodes (or reuse the
// last one): false when it cannot be built, and cycles are then launched kernel by kernel
template <typename V>
bool cycle_graph(Ctx& C, int min_iters, bool sparse, bool ebe, bool learned = false) {
    CycleGraph& G = learned ? C.cyc_net : C.cyc;
    if (G.disabled) return false;
    phgpu_config key = C.cfg;  // the fields the captured kernels do not read
    key.iter = 0;
    key.istep = 0;
    key.eGMRES = 0.0;
    const void* lhs = !sparse ? nullptr : ebe ? (const void*)ebe_lhs<V>(C) : (const void*)sparse_lhs<V>(C);
    if (G.exec && G.vsize == (int)sizeof(V) && G.min_iters == min_iters && G.lhs == lhs && G.lin_minb == C.lin_minb &&
        std::memcmp(&G.key, &key, sizeof key) == 0)
        return true;
    phgpu::cycle_graph_free(G);
    const int K = C.cfg.Kspace;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    std::vector<cudaGraphConditionalHandle> h(K + 2, 0);
    for (int i = 1; i <= K && e == cudaSuccess; ++i)
        e = cudaGraphConditionalHandleCreate(&h[i], g, i == 1 ? 1u : 0u, cudaGraphCondAssignDefault);
    const long long l0 = C.launches;
    G.launches.assign(K + 1, 0);
    cudaGraphNode_t prev = nullptr;
    for (int i = 1; i <= K && e == cudaSuccess; ++i) {
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h[i];
        p.conditional.type = cudaGraphCondTypeIf;
        p.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        e = cudaGraphAddNode(&node, g, prev ? &prev : nullptr, nullptr, prev ? 1 : 0, &p);
        if (e != cudaSuccess) break;
        cudaGraph_t body = p.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(C.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) break;
        const long long li = C.launches;
        const int rc = krylov_step<V>(C, i, min_iters, sparse, ebe, h[i + 1], i < K ? 1 : 0, learned);
        cudaGraph_t captured = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(C.stream, &captured);
        G.launches[i] = C.launches - li;
        e = rc != PHGPU_OK ? cudaErrorUnknown : e2;
        prev = node;
    }
    C.launches = l0;
    G.graph = g;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&G.exec, g, 0);
    if (e != cudaSuccess) {
        G.why = std::string("cycle graph: ") + cudaGetErrorString(e);
        (void)cudaGetLastError();
        cycle_graph_free(G);
        G.disabled = true;
        return false;
    }
    G.key = key;
    G.vsize = (int)sizeof(V);
    G.min_iters = min_iters;
    G.lin_minb = C.lin_minb;
    G.lhs = lhs;
    return true;
}

// GMRES cycles on V-typed Krylov vectors; b (= L^-1 R, FP64) in d_res, output Dy (FP64, before U^-1).
// ap_mode PHGPU_AP_SPARSE: the product is SparseAp + bc3per on the preconditioned tangent, and a
// new cycle recomputes R - A Dy only when lgmres_common > 0 (SolGMRs, solgmr.f:526-537)
template <typename V>
int gmres(Ctx& C, phgpu_stats* st, int lgmres_common = 0, bool unorm_ready = false) {
    Range nv("phgpu: GMRES cycles");
    // SolGMRe restarts from the true residual and stops without the minIters test (solgmr.f:130-210)
    const bool ebe = C.cfg.ap_mode == PHGPU_AP_EBE;
    const bool sparse = C.cfg.ap_mode == PHGPU_AP_SPARSE || ebe;
    if (ebe) lgmres_common = 1;
    const int min_iters = ebe ? 0 : C.cfg.minIters;
    const size_t n5 = 5 * (size_t)C.N;
    const int K = C.cfg.Kspace;
    V* U = (V*)C.d_U;
    auto Uj = [&](int j) { return U + (size_t)(j - 1) * C.ldU; };  // 1-based
    double* s = C.d_scal;
    const int* done = C.d_flag;
    // ||b|| (already read with the assembly's status when unorm_ready)
    if (!unorm_ready) {
        dot<double>(C, C.d_res, C.d_res, n5, S_TMP0, nullptr);
        PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, s, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream), "unorm"));
        PH_TRY(sync(C));
    }
    double unorm = std::sqrt(C.h_scal[S_TMP0]);
    st->unorm0 = unorm;
    st->totres = unorm / (double)C.N;
    fill0(C, C.d_Dy, sizeof(double) * n5);
    st->iKs = 0;
    st->lGMRES = 0;
    st->net_its = 0;
    st->net_fallback = PHGPU_NET_PLAIN;
    if (!std::isfinite(unorm)) return fail(C, PHGPU_ERR_NONFINITE, "non-finite residual (tnanq)");
    if (unorm < 100. * C.cfg.epsM * C.cfg.epsM) return PHGPU_OK;
    const double epsnrm = C.cfg.etol * unorm;
    if (C.cfg.ap_mode == PHGPU_AP_FD && C.cfg.iter == 1 && (C.cfg.istep % 20) == 0) PH_TRY(itrfdi_dev(C, C.d_rmes, C.d_res));
    st->eGMRES = C.cfg.eGMRES;
    if constexpr (std::is_same<V, double>::value) {
        k_copy<double><<<kVG, kVT, 0, C.stream>>>(C.d_res, Uj(1), n5, nullptr);
        ++C.launches;
    } else {
        to_f32(C, C.d_res, Uj(1), n5);
    }
    // learned preconditioner: the first cycle is flexible GMRES with the network, capped one
    // iteration below the last block-diagonal solve; if it does not converge, nGMRES
    // block-diagonal cycles continue from its solution
    const bool want_net = std::is_same<V, float>::value && C.cfg.precond == PHGPU_PRECOND_LEARNED && !sparse;
    bool use_net = false;
    int cap = K;
    if (want_net && net_usable(C) && !C.net.disabled && C.net.its_ref >= 2) {
        use_net = true;
        cap = std::min(K, C.net.its_ref - 1);
        PH_TRY(net_prepare(C));
    }
    const int ncycles = C.cfg.nGMRES + (use_net ? 1 : 0);
    int its_plain = 0;
    bool net_ok = false;
    // device time of the cycles: a learned cycle must beat the block-diagonal iterations it replaces
    const bool timed = want_net && C.net.ev0;
    if (timed) cudaEventRecord(C.net.ev0, C.stream);
    int iKs = 0;
    for (int mG = 1; mG <= ncycles; ++mG) {
        const bool learned = use_net && mG == 1;
        st->lGMRES = mG - 1;
        if (mG > 1 && sparse && lgmres_common <= 0) {
            // SolGMRs tests the COMMON lGMRES, which it never sets (solgmr.f:528): the cycle
            // starts again from its first vector, scaled by the last norm of the previous cycle
            unorm = C.h_scal[S_TMP2];
        } else if (mG > 1 && sparse) {
            V* t = Uj(1);
            if constexpr (std::is_same<V, double>::value) {
                assembled_ap<double>(C, ebe, C.d_Dy, t);
                k_axpby<<<kVG, kVT, 0, C.stream>>>(C.d_res, 1.0, t, -1.0, t, n5);
                ++C.launches;
            } else {
                to_f32(C, C.d_Dy, C.d_t32b, n5);
                assembled_ap<float>(C, ebe, C.d_t32b, C.d_t32);
                to_f64(C, C.d_t32, C.d_t64b, n5);
                k_axpby<<<kVG, kVT, 0, C.stream>>>(C.d_res, 1.0, C.d_t64b, -1.0, C.d_t64b, n5);
                ++C.launches;
                to_f32(C, C.d_t64b, t, n5);
            }
            dot<V>(C, t, t, n5, S_TMP0, nullptr);
            PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, s, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream), "unorm"));
            PH_TRY(sync(C));
            unorm = std::sqrt(C.h_scal[S_TMP0]);
        } else if (mG > 1) {
            // restart: uBrg(1) = R - A Dy, by Au2MFG's central difference when the
            // product is finite-differenced, else with the linearized product
            V* t = Uj(1);
            if constexpr (std::is_same<V, double>::value) {
                if (C.cfg.ap_mode == PHGPU_AP_FD) {
                    PH_TRY(au2_fd64(C, t));
                } else {
                    PH_TRY(ap_lin<V>(C, C.d_Dy, t, nullptr));
                    k_axpby<<<kVG, kVT, 0, C.stream>>>(C.d_res, 1.0, t, -1.0, t, n5);  // t = b - A Dy
                    ++C.launches;
                }
            } else {
                to_f32(C, C.d_Dy, t, n5);
                PH_TRY(ap_lin<V>(C, t, t, nullptr));
                to_f64(C, t, C.d_t64b, n5);
                k_axpby<<<kVG, kVT, 0, C.stream>>>(C.d_res, 1.0, C.d_t64b, -1.0, C.d_t64b, n5);
                ++C.launches;
                to_f32(C, C.d_t64b, t, n5);
            }
            dot<V>(C, t, t, n5, S_TMP0, nullptr);
            PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, s, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream), "unorm"));
            PH_TRY(sync(C));
            unorm = std::sqrt(C.h_scal[S_TMP0]);
        }
        k_init_cycle<<<1, 256, 0, C.stream>>>(s, K, unorm, epsnrm, C.d_flag, cap);
        ++C.launches;
        // uBrg(1) /= unorm
        scale_by<V>(C, Uj(1), s + S_UNORM, 0, n5, nullptr);
        // the solution is sum_j y_j u_j, or sum_j y_j z_j in a learned (flexible) cycle
        const V* basis = U;
        if constexpr (std::is_same<V, float>::value)
            if (learned) basis = C.net.d_Z;
        bool nonfinite = false;
        // the finite-difference product reads eGMRES (changed by itrFDI) as a launch value
        if (!C.cfg.no_graph && C.cfg.ap_mode != PHGPU_AP_FD && cycle_graph<V>(C, min_iters, sparse, ebe, learned)) {
            CycleGraph& G = learned ? C.cyc_net : C.cyc;
            PH_TRY(check(C, cudaGraphLaunch(G.exec, C.stream), "cycle graph launch"));
            ++G.runs;
            // back substitution and update with the iteration count the graph left in flag[2],
            // then one host read of the flags and the final residual estimate
            k_backsolve<<<1, 1, 0, C.stream>>>(s, K, 0, C.d_flag + 2);
            k_update_dy<V><<<kVG, kVT, 0, C.stream>>>(C.d_Dy, basis, C.ldU, 0, K, s, n5, C.d_flag + 2);
            C.launches += 2;
            PH_TRY(check(C, cudaMemcpyAsync(C.h_flag, C.d_flag, sizeof(int) * 3, cudaMemcpyDeviceToHost, C.stream), "flag"));
            PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, s, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream), "echeck"));
            PH_TRY(sync(C));
            iKs = C.h_flag[2];
            if (iKs < 1 || iKs > K) return fail(C, PHGPU_ERR_CUDA, "cycle graph ran no Krylov iteration");
            for (int i = 1; i <= iKs; ++i) C.launches += G.launches[i];
            st->ntotGM += iKs;
            if (C.h_flag[1] & kPipeCopyFailed) return fail(C, PHGPU_ERR_CUDA, kPipeCopyMsg);
            nonfinite = C.h_flag[1] != 0;
        } else {
            for (int iK = 1; iK <= K; ++iK) {
                iKs = iK;
                PH_TRY(krylov_step<V>(C, iK, min_iters, sparse, ebe, 0, 0, learned));
                st->ntotGM += 1;
                PH_TRY(check(C, cudaMemcpyAsync(C.h_flag, C.d_flag, sizeof(int) * 2, cudaMemcpyDeviceToHost, C.stream), "flag"));
                PH_TRY(sync(C));
                if (C.h_flag[1] & kPipeCopyFailed) return fail(C, PHGPU_ERR_CUDA, kPipeCopyMsg);
                if (C.h_flag[1]) {
                    nonfinite = true;
                    break;
                }
                if (C.h_flag[0] || (learned && iK >= cap)) break;
            }
            if (!nonfinite) {
                k_backsolve<<<1, 1, 0, C.stream>>>(s, K, iKs, nullptr);
                k_update_dy<V><<<kVG, kVT, 0, C.stream>>>(C.d_Dy, basis, C.ldU, iKs, K, s, n5, nullptr);
                C.launches += 2;
                PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, s, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream), "echeck"));
                PH_TRY(sync(C));
            }
        }
        if (nonfinite) {
            if (!learned) return fail(C, PHGPU_ERR_NONFINITE, "non-finite Hessenberg entry in GMRES");
            // the network gave a non-finite direction: drop the cycle, block-diagonal GMRES from Dy = 0
            fill0(C, C.d_Dy, sizeof(double) * n5);
            fill0(C, C.d_flag + 1, sizeof(int));
            st->net_its = iKs;
            continue;
        }
        st->echeck = C.h_scal[S_ECHECK];
        const bool converged = C.h_scal[S_ECHECK] <= epsnrm;
        if (learned) {
            st->net_its = iKs;
            float ms = 0.f;
            if (timed) {
                cudaEventRecord(C.net.ev1, C.stream);
                cudaEventSynchronize(C.net.ev1);
                cudaEventElapsedTime(&ms, C.net.ev0, C.net.ev1);
            }
            C.net.ms_last = ms;
            // converged, and faster than the block-diagonal iterations it replaces
            net_ok = converged && (!timed || C.net.ms_ref_iter <= 0.0 || ms < C.net.its_ref * C.net.ms_ref_iter);
        } else {
            its_plain += iKs;
        }
        if (converged) break;
    }
    st->iKs = iKs;
    if (want_net) ++(use_net ? (net_ok ? C.net.n_used : C.net.n_fell_back) : C.net.n_plain);
    if (use_net) {
        st->net_fallback = net_ok ? PHGPU_NET_USED : PHGPU_NET_FELL_BACK;
        // off after two failed learned cycles in a row, or at once after one that took more
        // than twice the time of the block-diagonal iterations it was to replace
        const bool much_slower = timed && C.net.ms_ref_iter > 0.0 &&
                                 C.net.ms_last > 2.0 * C.net.its_ref * C.net.ms_ref_iter;
        if (net_ok) {
            C.net.fails = 0;
        } else if (much_slower || ++C.net.fails >= 2) {
            C.net.disabled = true;
        }
    } else if (want_net) {
        // a block-diagonal solve with the learned preconditioner selected: its count and its time
        // per iteration are the reference
        C.net.its_ref = its_plain;
        float ms = 0.f;
        if (timed) {
            cudaEventRecord(C.net.ev1, C.stream);
            cudaEventSynchronize(C.net.ev1);
            cudaEventElapsedTime(&ms, C.net.ev0, C.net.ev1);
        }
        C.net.ms_ref_iter = its_plain > 0 ? ms / its_plain : 0.0;
    }
    (void)done;
    return PHGPU_OK;
}

// The assembly part of SolMFG / SolGMRs / SolGMRe on resident data, launches only (no host
// round trip): residual R (d_res), ||R||^2 (S_TMP3), BDiag and its LU factors (status in flag[1]),
// L^-1 R in d_res and ||L^-1 R||^2 (S_TMP0); for the matrix-free solver also ypre = U y.
int assemble_and_factor(Ctx& C, int lhs, bool asm_bd, bool sparse, bool ebe) {
    Range nv("phgpu: assembly and block LU");
    const size_t N = C.N, n5 = 5 * N;
    if (C.cfg.precision == PHGPU_FP64) {
        if (sparse) {
            // ElmGMRs / ElmGMRe: the residual, and BDiag from the tangent's diagonal blocks
            PH_TRY(elmres64(C, C.d_y, C.d_ac, C.d_res));
            if (lhs) PH_TRY(tangent64(C, C.d_y, ebe ? C.sp.d_EG : C.sp.d_lhsK, C.d_bd, ebe));
        } else {
            PH_TRY(elmmfg64(C, C.d_y, C.d_ac, C.d_res, C.d_rmes, C.d_bd, 1));
        }
    } else {
        if (C.cfg.ap_mode == PHGPU_AP_FD)
            return fail(C, PHGPU_ERR_UNSUPPORTED, "mixed precision needs the linearized or the assembled product");
        // outer residual (FP64, or FP64 Galerkin + FP32 stabilization); FP32 block-diagonal tangent
        if (C.cfg.outer_residual == PHGPU_RES_SPLITDF) split_f32(C, C.d_y, C.d_yf, C.d_ylo, n5);
        else to_f32(C, C.d_y, C.d_yf, n5);
        pack_xb(C);
        to_f32(C, C.d_ac, C.d_acf, n5);
        if (C.cfg.outer_residual == PHGPU_RES_GALERKIN64 || C.cfg.outer_residual == PHGPU_RES_SPLITDF) {
            if (C.cfg.idiff == 1 && C.cfg.outer_residual == PHGPU_RES_GALERKIN64)
                return fail(C, PHGPU_ERR_UNSUPPORTED, "idiff = 1 needs the FP64 or the double-float outer residual");
            const double* ql = reconstruct_q(C, C.d_y);
            if (ql) to_f32(C, C.d_qres, C.d_qresf, 13 * N);
            fill0(C, C.d_res, sizeof(double) * n5);
            if (C.cfg.outer_residual == PHGPU_RES_SPLITDF)
                launch_elem_ress(C, C.d_yf, C.d_ylo, C.d_acf, C.d_res, ql ? C.d_qresf : nullptr);
            else launch_elem_resh(C, C.d_y, C.d_ac, C.d_yf, C.d_acf, C.d_res);
            // hex and wedge blocks: the same split residual, or FP64 with the Galerkin64 option
            if (C.cfg.outer_residual == PHGPU_RES_SPLITDF && (C.nhex > 0 || C.nwedge > 0)) {
                PH_TRY(topo_split_setup(C));
                launch_topo_ress(C, C.d_yf, C.d_ylo, C.d_acf, C.d_res, ql ? C.d_qresf : nullptr);
            } else {
                launch_topo<double>(C, RM_RES, C.d_x, C.d_y, nullptr, C.d_ac, C.d_res, nullptr, nullptr, 0, nullptr,
                                    ql);
            }
            if (has_boundary(C)) launch_boundary(C, C.d_y, C.d_res);
            bc3res<double>(C, C.d_res);
        } else {
            PH_TRY(elmres64(C, C.d_y, C.d_ac, C.d_res));
        }
        if (asm_bd) {
            fill0(C, C.d_bdf, sizeof(float) * 25 * N);
            if (ebe) {
                launch_tangent_ebe<float>(C, C.d_xf, C.d_yf, C.sp.d_EGf, C.d_bdf);
            } else if (sparse) {
                // FP32 tangent; its diagonal blocks are the block diagonal
                fill0(C, C.sp.d_lhsKf, sizeof(float) * 25 * (size_t)C.sp.nnzb);
                launch_tangent<float>(C, C.d_xf, C.d_yf, C.sp.d_lhsKf, C.d_bdf);
            } else {
                launch_elem_full<float>(C, C.d_xf, C.d_yf, C.d_acf, nullptr, nullptr, C.d_bdf);
            }
            bc3bdg<float>(C, C.d_y, C.d_bdf);
        }
    }
    // nonlinear residual ||R|| (FP64, unpreconditioned)
    dot<double>(C, C.d_res, C.d_res, n5, S_TMP3, nullptr);
    fill0(C, C.d_flag, sizeof(int) * 2);
    if (asm_bd) {
        if (C.cfg.precision == PHGPU_MIXED) lu_fact_f32(C, C.d_bdf, C.d_bd, C.d_flag);
        else lu_fact<double>(C, C.d_bd, C.d_flag);
    }
    lu_apply<double, double>(C, C.d_bd, C.d_res, PHGPU_LU_FORWARD);
    if (sparse) {
        if (ebe) {
            if (C.cfg.precision == PHGPU_FP64) i3pre<double>(C, C.d_bd, C.sp.d_EG);
            else i3pre<float>(C, C.d_bdf, C.sp.d_EGf);
        } else if (lhs) {
            if (C.cfg.precision == PHGPU_FP64) spsi3pre<double>(C, C.d_bd, C.sp.d_lhsK);
            else spsi3pre<float>(C, C.d_bdf, C.sp.d_lhsKf);
            C.sp.have = C.cfg.precision;
        }
    } else {
        if (C.cfg.precision == PHGPU_FP64) lu_apply<double, double>(C, C.d_bd, C.d_rmes, PHGPU_LU_FORWARD);
        // ypre = U . y (local order is already the "old" order)
        k_copy<double><<<kVG, kVT, 0, C.stream>>>(C.d_y, C.d_ypre, n5, nullptr);
        ++C.launches;
        lu_apply<double, double>(C, C.d_bd, C.d_ypre, PHGPU_LU_PRODUCT);
    }
    // ||L^-1 R|| for GMRES
    dot<double>(C, C.d_res, C.d_res, n5, S_TMP0, nullptr);
    return PHGPU_OK;
}

// SolMFG (solmfg.f) or, with ap_mode PHGPU_AP_SPARSE, SolGMRs (solgmr.f:480): lhs = 1 forms
// BDiag and the tangent (iprec = lhs, itrdrv.f:456-457); lhs = 0 reuses the factored BDiag
// and the preconditioned tangent of the last lhs = 1 solve
int solve_dev(Ctx& C, phgpu_stats* st, int lhs, int lgmres_common) {
    Range nv("phgpu: flow solve");
    const size_t N = C.N, n5 = 5 * N;
    const bool ebe = C.cfg.ap_mode == PHGPU_AP_EBE;
    const bool sparse = C.cfg.ap_mode == PHGPU_AP_SPARSE || ebe;
    if (ebe) {
        if (!lhs) return fail(C, PHGPU_ERR_UNSUPPORTED, "the element-by-element solver assembles on every call");
        PH_TRY(ebe_setup(C));
    } else if (sparse) {
        PH_TRY(sparse_setup(C));
        if (!lhs && C.sp.have != C.cfg.precision)
            return fail(C, PHGPU_ERR_INVALID, "lhs = 0 needs the tangent of an earlier lhs = 1 solve");
    }
    // discontinuity capturing is in the FP64 residual kernels; the linearized and assembled
    // products do not carry it
    if (C.cfg.iDC != 0 && (C.cfg.precision != PHGPU_FP64 || C.cfg.ap_mode != PHGPU_AP_FD))
        return fail(C, PHGPU_ERR_UNSUPPORTED, "iDC != 0 needs FP64 with the finite-difference product");
    if (C.cfg.precond == PHGPU_PRECOND_LEARNED && (C.cfg.precision != PHGPU_MIXED || C.cfg.ap_mode != PHGPU_AP_LINEAR))
        return fail(C, PHGPU_ERR_UNSUPPORTED, "the learned preconditioner needs mixed precision with the linearized product");
    const bool asm_bd = !sparse || lhs;
    if (C.cfg.precision == PHGPU_MIXED && C.cfg.ap_mode == PHGPU_AP_LINEAR) PH_TRY(autotune_sweeps(C));
    cudaEventRecord(C.ev[0], C.stream);
    PH_TRY(assemble_and_factor(C, lhs, asm_bd, sparse, ebe));
    PH_TRY(check(C, cudaMemcpyAsync(C.h_flag, C.d_flag, sizeof(int) * 2, cudaMemcpyDeviceToHost, C.stream), "flag"));
    PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, C.d_scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream), "rn"));
    PH_TRY(sync(C));
    st->rnorm = std::sqrt(C.h_scal[S_TMP3]);
    if (C.h_flag[1]) return fail(C, PHGPU_ERR_SINGULAR, "zero or non-finite pivot in the block-diagonal LU");
    cudaEventRecord(C.ev[1], C.stream);
    int rc;
    if (C.cfg.precision == PHGPU_FP64) rc = gmres<double>(C, st, lgmres_common, true);
    else rc = gmres<float>(C, st, lgmres_common, true);
    if (rc != PHGPU_OK) return rc;
    lu_apply<double, double>(C, C.d_bd, C.d_Dy, PHGPU_LU_BACKWARD);
    cudaEventRecord(C.ev[2], C.stream);
    PH_TRY(sync(C));
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, C.ev[0], C.ev[1]);
    cudaEventElapsedTime(&b, C.ev[1], C.ev[2]);
    st->t_assembly_ms = a;
    st->t_gmres_ms = b;
    st->status = PHGPU_OK;
    return PHGPU_OK;
}

int solmfg_dev(Ctx& C, phgpu_stats* st) { return solve_dev(C, st, 1, 0); }

// element-by-element storage (device order, [element][a][b][25]) <-> the reference's
// EGmass(numel, nedof, nedof), column-major, elements in input order (one topology)
void ebe_shape(const Ctx& C, int* nen, size_t* numel, const std::vector<int>** order) {
    if (C.E > 0) { *nen = 4; *numel = C.E; *order = &C.sp.torder; }
    else if (C.nhex > 0) { *nen = 8; *numel = C.nhex; *order = &C.horder; }
    else { *nen = 6; *numel = C.nwedge; *order = &C.worder; }
}
int ebe_download(Ctx& C, const double* d_eg, double* ref) {
    int nen;
    size_t numel;
    const std::vector<int>* order;
    ebe_shape(C, &nen, &numel, &order);
    const int nedof = 5 * nen, NB = nen * nen;
    std::vector<double> h(25 * C.sp.eg_blocks);
    PH_TRY(check(C, cudaMemcpyAsync(h.data(), d_eg, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, C.stream),
                 "download EGmass"));
    PH_TRY(sync(C));
    for (size_t p = 0; p < numel; ++p) {
        const size_t e = (*order)[p];
        for (int a = 0; a < nen; ++a)
            for (int b = 0; b < nen; ++b)
                for (int g = 0; g < 5; ++g)
                    for (int f = 0; f < 5; ++f)
                        ref[e + numel * ((size_t)(5 * a + f) + (size_t)nedof * (5 * b + g))] =
                            h[25 * (p * NB + (size_t)a * nen + b) + 5 * g + f];
    }
    return PHGPU_OK;
}
int ebe_upload(Ctx& C, const double* ref, double* d_eg) {
    int nen;
    size_t numel;
    const std::vector<int>* order;
    ebe_shape(C, &nen, &numel, &order);
    const int nedof = 5 * nen, NB = nen * nen;
    std::vector<double> h(25 * C.sp.eg_blocks);
    for (size_t p = 0; p < numel; ++p) {
        const size_t e = (*order)[p];
        for (int a = 0; a < nen; ++a)
            for (int b = 0; b < nen; ++b)
                for (int g = 0; g < 5; ++g)
                    for (int f = 0; f < 5; ++f)
                        h[25 * (p * NB + (size_t)a * nen + b) + 5 * g + f] =
                            ref[e + numel * ((size_t)(5 * a + f) + (size_t)nedof * (5 * b + g))];
    }
    PH_TRY(check(C, cudaMemcpyAsync(d_eg, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, C.stream),
                 "upload EGmass"));
    return sync(C);
}

int correct_dev(Ctx& C) {
    const size_t n5 = 5 * (size_t)C.N;
    const phgpu_config& c = C.cfg;
    k_correct<<<kVG, kVT, 0, C.stream>>>(C.d_y, C.d_ac, C.d_yold, C.d_acold, C.d_Dy, 1.0 - c.almi / c.gami,
                                         c.almi * c.Dtgl / c.gami / c.alfi, n5);
    ++C.launches;
    itrbc_state(C, C.d_y, C.d_ac, true);
    return check(C, cudaGetLastError(), "itrCorrect");
}

int newton_dev(Ctx& C, phgpu_stats* st) {
    PH_TRY(solmfg_dev(C, st));
    PH_TRY(correct_dev(C));
    return PHGPU_OK;
}

// ---------------------------------------------------------------------------
// the whole time step as one CUDA graph (StepGraph)
// ---------------------------------------------------------------------------
// (with the learned preconditioner selected, once it is switched off -- or has no weights --
// every solve is block-diagonal, and the step graph applies as well)
bool step_graph_eligible(const Ctx& C, int nitr) {
    const phgpu_config& c = C.cfg;
    const bool plain = c.precond == PHGPU_PRECOND_BDIAG ||
                       (c.precond == PHGPU_PRECOND_LEARNED && (C.net.disabled || !net_usable(C)));
    return !c.no_graph && c.precision == PHGPU_MIXED && c.ap_mode == PHGPU_AP_LINEAR && plain &&
           c.nGMRES == 1 && c.iDC == 0 && nitr >= 1 && nitr <= kStepGraphMaxNitr && !C.stepg.disabled;
}

void step_graph_free(StepGraph& G) {
    if (G.exec) cudaGraphExecDestroy(G.exec);
    if (G.graph) cudaGraphDestroy(G.graph);
    G.exec = nullptr;
    G.graph = nullptr;
}

// Capture itrPredict + itrBC, nitr Newton iterations (assembly and LU, one GMRES cycle whose Krylov
// iterations are conditional nodes, back substitution, update, U^-1, itrCorrect + itrBC) and
// itrUpdate + itrBC: the kernels of time_step_dev in the same order with the same arguments,
// the cycle's norms read on the device instead of on the host.
int step_graph_build(Ctx& C, int nitr) {
    Range nv("phgpu: step graph capture");
    StepGraph& G = C.stepg;
    const size_t n5 = 5 * (size_t)C.N;
    const int K = C.cfg.Kspace;
    if (!G.d_stats && cudaMalloc((void**)&G.d_stats, sizeof(double) * 8 * kStepGraphMaxNitr) != cudaSuccess)
        return fail(C, PHGPU_ERR_NOMEM, "step graph statistics");
    if (!G.aux) PH_TRY(check(C, cudaStreamCreateWithFlags(&G.aux, cudaStreamNonBlocking), "step graph stream"));
    // host set-up the assembly does on its first call, outside the capture
    if (C.cfg.outer_residual == PHGPU_RES_SPLITDF && (C.nhex > 0 || C.nwedge > 0)) PH_TRY(topo_split_setup(C));
    PH_TRY(sync(C));
    step_graph_free(G);
    float* U = (float*)C.d_U;
    auto Uj = [&](int j) { return U + (size_t)(j - 1) * C.ldU; };
    double* s = C.d_scal;
    const phgpu_config c = C.cfg;
    const double tiny = 100. * c.epsM * c.epsM;
    cudaStream_t st0 = C.stream;
    const long long l0 = C.launches;
    std::vector<long long> body(K + 1, 0);
    int rc = PHGPU_OK;
    cudaError_t e = cudaStreamBeginCapture(st0, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
        k_predict<<<kVG, kVT, 0, st0>>>(C.d_yold, C.d_acold, C.d_y, C.d_ac, 1.0 - c.almi / c.gami, n5);
        ++C.launches;
        itrbc_state(C, C.d_y, C.d_ac, true);
        for (int it = 1; it <= nitr && rc == PHGPU_OK && e == cudaSuccess; ++it) {
            double* out = G.d_stats + 8 * (it - 1);
            rc = assemble_and_factor(C, 1, true, false, false);
            if (rc != PHGPU_OK) break;
            k_step_record<<<1, 1, 0, st0>>>(s, C.d_flag, out, 0);
            ++C.launches;
            fill0(C, C.d_Dy, sizeof(double) * n5);
            to_f32(C, C.d_res, Uj(1), n5);
            cudaStreamCaptureStatus cs;
            cudaGraph_t g = nullptr;
            const cudaGraphNode_t* deps = nullptr;
            size_t nd = 0;
            e = cudaStreamGetCaptureInfo(st0, &cs, nullptr, &g, &deps, nullptr, &nd);
            std::vector<cudaGraphConditionalHandle> h(K + 2, 0);
            for (int i = 1; i <= K && e == cudaSuccess; ++i)
                e = cudaGraphConditionalHandleCreate(&h[i], g, 0u, cudaGraphCondAssignDefault);
            if (e != cudaSuccess) break;
            k_init_cycle_dev<<<1, 256, 0, st0>>>(s, K, c.etol, tiny, C.d_flag, h[1]);
            ++C.launches;
            scale_by<float>(C, Uj(1), s + S_UNORM, 0, n5, nullptr);
            e = cudaStreamGetCaptureInfo(st0, &cs, nullptr, &g, &deps, nullptr, &nd);
            if (e != cudaSuccess) break;
            std::vector<cudaGraphNode_t> prev(deps, deps + nd);
            cudaGraphNode_t node = nullptr;
            for (int i = 1; i <= K && e == cudaSuccess && rc == PHGPU_OK; ++i) {
                cudaGraphNodeParams p{};
                p.type = cudaGraphNodeTypeConditional;
                p.conditional.handle = h[i];
                p.conditional.type = cudaGraphCondTypeIf;
                p.conditional.size = 1;
                e = cudaGraphAddNode(&node, g, prev.data(), nullptr, prev.size(), &p);
                if (e != cudaSuccess) break;
                cudaGraph_t bodyg = p.conditional.phGraph_out[0];
                e = cudaStreamBeginCaptureToGraph(G.aux, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
                if (e != cudaSuccess) break;
                C.stream = G.aux;
                const long long lb = C.launches;
                rc = krylov_step<float>(C, i, c.minIters, false, false, h[i + 1], i < K ? 1 : 0, false);
                C.stream = st0;
                body[i] = C.launches - lb;
                C.launches = lb;
                cudaGraph_t captured = nullptr;
                const cudaError_t e2 = cudaStreamEndCapture(G.aux, &captured);
                if (e2 != cudaSuccess) e = e2;
                prev.assign(1, node);
            }
            if (e != cudaSuccess || rc != PHGPU_OK) break;
            e = cudaStreamUpdateCaptureDependencies(st0, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
            if (e != cudaSuccess) break;
            k_backsolve<<<1, 1, 0, st0>>>(s, K, 0, C.d_flag + 2);
            k_update_dy<float><<<kVG, kVT, 0, st0>>>(C.d_Dy, U, C.ldU, 0, K, s, n5, C.d_flag + 2);
            k_step_record<<<1, 1, 0, st0>>>(s, C.d_flag, out, 1);
            C.launches += 3;
            lu_apply<double, double>(C, C.d_bd, C.d_Dy, PHGPU_LU_BACKWARD);
            rc = correct_dev(C);
        }
        if (e == cudaSuccess && rc == PHGPU_OK) {
            k_update<<<kVG, kVT, 0, st0>>>(C.d_yold, C.d_acold, C.d_y, C.d_ac, 1.0 / c.almi, 1.0 / c.alfi, n5);
            ++C.launches;
            itrbc_state(C, C.d_yold, C.d_acold, true);
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t e3 = cudaStreamEndCapture(st0, &graph);
        if (e == cudaSuccess) e = e3;
        G.graph = graph;
    }
    C.stream = st0;
    G.fixed_launches = C.launches - l0;
    G.body_launches = body;
    C.launches = l0;
    if (e == cudaSuccess && rc == PHGPU_OK) e = cudaGraphInstantiate(&G.exec, G.graph, 0);
    // fixed part: everything but the Krylov iteration bodies (they were taken out as captured)
    if (e != cudaSuccess || rc != PHGPU_OK) {
        (void)cudaGetLastError();
        step_graph_free(G);
        if (rc != PHGPU_OK) return rc;
        G.why = std::string("step graph: ") + cudaGetErrorString(e);
        G.disabled = true;
        return PHGPU_ERR_CUDA;
    }
    G.key = c;
    G.key.iter = G.key.istep = 0;
    G.key.eGMRES = 0.0;
    G.nitr = nitr;
    G.lin_minb = C.lin_minb;
    G.ress_minb = C.ress_minb;
    return PHGPU_OK;
}

// one time step through the graph; *used = false when the graph could not be built (the caller
// then launches the step kernel by kernel)
int step_graph_run(Ctx& C, int nitr, phgpu_stats* st, bool* used) {
    Range nv("phgpu: time step (graph)");
    StepGraph& G = C.stepg;
    *used = false;
    phgpu_config key = C.cfg;
    key.iter = key.istep = 0;
    key.eGMRES = 0.0;
    if (!G.exec || G.nitr != nitr || G.lin_minb != C.lin_minb || G.ress_minb != C.ress_minb ||
        std::memcmp(&G.key, &key, sizeof key) != 0) {
        const int rc = step_graph_build(C, nitr);
        if (rc != PHGPU_OK) {
            if (G.disabled) {
                C.err.clear();
                return PHGPU_OK;
            }
            return rc;
        }
    }
    PH_TRY(check(C, cudaGraphLaunch(G.exec, C.stream), "step graph launch"));
    *used = true;
    ++G.runs;
    double out[8 * kStepGraphMaxNitr];
    PH_TRY(check(C, cudaMemcpyAsync(out, G.d_stats, sizeof(double) * 8 * nitr, cudaMemcpyDeviceToHost, C.stream),
                 "step statistics"));
    PH_TRY(sync(C));
    long long iks_tot = 0, body = 0;
    for (int it = 0; it < nitr; ++it) {
        const double* o = out + 8 * it;
        if (o[4] != 0.0) return fail(C, PHGPU_ERR_SINGULAR, "zero or non-finite pivot in the block-diagonal LU");
        if (((int)o[5]) & kPipeCopyFailed) return fail(C, PHGPU_ERR_CUDA, kPipeCopyMsg);
        if (((int)o[5]) & 2) return fail(C, PHGPU_ERR_NONFINITE, "non-finite value in GMRES");
        const int iks = (int)o[3];
        iks_tot += iks;
        for (int i = 1; i <= iks && i < (int)G.body_launches.size(); ++i) body += G.body_launches[i];
    }
    const double* o = out + 8 * (nitr - 1);
    st->iKs = (int)o[3];
    st->lGMRES = 0;
    st->ntotGM += (int)iks_tot;
    st->unorm0 = std::sqrt(o[1]);
    st->totres = st->unorm0 / (double)C.N;
    st->echeck = o[2];
    st->rnorm = std::sqrt(o[0]);
    st->eGMRES = C.cfg.eGMRES;
    st->t_assembly_ms = st->t_gmres_ms = 0.0;
    st->net_its = 0;
    st->net_fallback = PHGPU_NET_PLAIN;
    st->status = PHGPU_OK;
    C.launches += G.fixed_launches + body;
    C.cyc.runs += nitr;  // each Newton iteration's GMRES cycle ran as (part of) a graph
    if (C.cfg.precond == PHGPU_PRECOND_LEARNED) C.net.n_plain += nitr;
    C.cfg.iter = nitr;
    C.cfg.istep += 1;
    return PHGPU_OK;
}

int time_step_dev(Ctx& C, int nitr, phgpu_stats* st) {
    Range nv("phgpu: time step");
    if (step_graph_eligible(C, nitr)) {
        bool used = false;
        PH_TRY(autotune_sweeps(C));  // before the kernels are fixed in the graph
        PH_TRY(step_graph_run(C, nitr, st, &used));
        if (used) return PHGPU_OK;
    }
    const size_t n5 = 5 * (size_t)C.N;
    const phgpu_config& c = C.cfg;
    k_predict<<<kVG, kVT, 0, C.stream>>>(C.d_yold, C.d_acold, C.d_y, C.d_ac, 1.0 - c.almi / c.gami, n5);
    ++C.launches;
    itrbc_state(C, C.d_y, C.d_ac, true);
    for (int it = 1; it <= nitr; ++it) {
        C.cfg.iter = it;
        PH_TRY(newton_dev(C, st));
    }
    k_update<<<kVG, kVT, 0, C.stream>>>(C.d_yold, C.d_acold, C.d_y, C.d_ac, 1.0 / c.almi, 1.0 / c.alfi, n5);
    ++C.launches;
    itrbc_state(C, C.d_yold, C.d_acold, true);
    C.cfg.istep += 1;
    return sync(C);
}

}  // namespace
}  // namespace phgpu

// ============================================================================
// C ABI
// ============================================================================
using phgpu::Ctx;

extern "C" {

int phgpu_create(const phgpu_mesh* m, const phgpu_config* cfg, phgpu_ctx** out) {
    using namespace phgpu;
    if (!out) return PHGPU_ERR_INVALID;
    *out = nullptr;
    if (!m || !cfg || m->nshg <= 0 || m->nelem < 0 || !m->x || !m->iBC || !m->BC || !m->iper)
        return PHGPU_ERR_INVALID;
    if (m->nhex < 0 || m->nwedge < 0 || (m->nelem > 0 && !m->ien) || (m->nhex > 0 && !m->ienh) ||
        (m->nwedge > 0 && !m->ienw) || m->nelem + m->nhex + m->nwedge <= 0)
        return PHGPU_ERR_INVALID;
    if (m->nbelem < 0 || (m->nbelem > 0 && !m->ienb)) return PHGPU_ERR_INVALID;
    if (cfg->Kspace < 1 || cfg->Kspace > kMaxK || cfg->nGMRES < 1) return PHGPU_ERR_INVALID;
    if ((cfg->itau != 0 && cfg->itau != 1) || cfg->ipord != 1 || cfg->EntropyPressure != 0) return PHGPU_ERR_UNSUPPORTED;
    // itau = 1 (Diagonal-Franca) is in the FP64 kernels; the reference leaves its momentum tau
    // unset when the stabilization time term is removed (e3tau.f:107-111)
    if (cfg->itau == 1 && (cfg->precision != PHGPU_FP64 || cfg->iremoveStabTimeTerm != 0 || !(cfg->rmu > 0.0)))
        return PHGPU_ERR_UNSUPPORTED;
    if (cfg->idiff != 0 && cfg->idiff != 1) return PHGPU_ERR_UNSUPPORTED;
    if (cfg->iDC < 0 || cfg->iDC > 3) return PHGPU_ERR_INVALID;
    if (cfg->precond != PHGPU_PRECOND_BDIAG && cfg->precond != PHGPU_PRECOND_LEARNED) return PHGPU_ERR_INVALID;
    phgpu_ctx* h = new (std::nothrow) phgpu_ctx();
    if (!h) return PHGPU_ERR_NOMEM;
    Ctx& C = h->c;
    C.N = m->nshg;
    C.E = m->nelem;
    C.Eb = m->nbelem;
    C.cfg = *cfg;
    const int N = C.N;
    // validate connectivity and periodic masters
    for (size_t i = 0; i < 4 * (size_t)C.E; ++i)
        if (m->ien[i] < 0 || m->ien[i] >= N) { delete h; return PHGPU_ERR_INVALID; }
    for (size_t i = 0; i < 4 * (size_t)C.Eb; ++i)
        if (m->ienb[i] < 0 || m->ienb[i] >= N) { delete h; return PHGPU_ERR_INVALID; }
    for (size_t i = 0; i < 8 * (size_t)m->nhex; ++i)
        if (m->ienh[i] < 0 || m->ienh[i] >= N) { delete h; return PHGPU_ERR_INVALID; }
    for (size_t i = 0; i < 6 * (size_t)m->nwedge; ++i)
        if (m->ienw[i] < 0 || m->ienw[i] >= N) { delete h; return PHGPU_ERR_INVALID; }
    C.nhex = m->nhex;
    C.nwedge = m->nwedge;
    for (int n = 0; n < N; ++n) {
        const int p = m->iper[n];
        if (p < 0 || p >= N) { delete h; return PHGPU_ERR_INVALID; }
        if (p != n && m->iper[p] != p) { delete h; return PHGPU_ERR_UNSUPPORTED; }  // chains
        if (((m->iBC[n] >> 10) & 1) != (p != n ? 1 : 0)) { delete h; return PHGPU_ERR_INVALID; }
        if ((m->iBC[n] >> 11) & 1) { delete h; return PHGPU_ERR_UNSUPPORTED; }  // scaled-plane extraction (irscale)
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { delete h; return PHGPU_ERR_CUDA; }
    C.device = dev;
    if (cudaStreamCreateWithFlags(&C.stream, cudaStreamNonBlocking) != cudaSuccess) { delete h; return PHGPU_ERR_CUDA; }
    for (auto& e : C.ev) cudaEventCreate(&e);
    int rc = PHGPU_OK;
    auto T = [&](int s) { if (rc == PHGPU_OK) rc = s; };
    // colouring
    std::vector<int> border;
    std::vector<int>& horder = C.horder;
    std::vector<int>& worder = C.worder;
    if (C.Eb > 0) T(colour(C, N, m->ienb, 4, C.Eb, border, C.bcol_start));
    if (C.nhex > 0) T(colour(C, N, m->ienh, 8, C.nhex, horder, C.hcol_start));
    if (C.nwedge > 0) T(colour(C, N, m->ienw, 6, C.nwedge, worder, C.wcol_start));
    if (rc != PHGPU_OK) { phgpu_destroy(h); return rc; }
    T(bnd_setup(C, m));
    if (rc != PHGPU_OK) { phgpu_destroy(h); return rc; }
    if (C.E > 0) T(build_chunks(C, m->ien, m->x));
    C.h_ien.assign(m->ien, m->ien + 4 * (size_t)C.E);
    if (rc == PHGPU_OK) T(configure_element_kernels(C));
    if (rc != PHGPU_OK) { phgpu_destroy(h); return rc; }
    std::vector<int4> ienb(std::max(C.Eb, 1));
    std::vector<int> ibcb(std::max(C.Eb, 1), 0);
    std::vector<double> bcb(18 * (size_t)std::max(C.Eb, 1), 0.0);
    for (int i = 0; i < C.Eb; ++i) {
        const int e = border[i];
        const int* p = m->ienb + 4 * (size_t)e;
        ienb[i] = make_int4(p[0], p[1], p[2], p[3]);
        ibcb[i] = m->iBCB ? m->iBCB[2 * (size_t)e] : 0;
        if (m->BCB)
            for (int k = 0; k < 18; ++k) bcb[18 * (size_t)i + k] = m->BCB[18 * (size_t)e + k];
    }
    // node arrays
    std::vector<double> x(3 * (size_t)N), bc(6 * (size_t)N);
    std::vector<float> xf(3 * (size_t)N), xlo(3 * (size_t)N);
    for (int n = 0; n < N; ++n) {
        for (int d = 0; d < 3; ++d) {
            const size_t i = 3 * (size_t)n + d;
            x[i] = m->x[(size_t)d * N + n];
            xf[i] = (float)x[i];
            xlo[i] = (float)(x[i] - (double)xf[i]);
        }
        for (int k = 0; k < 6; ++k) bc[6 * (size_t)n + k] = m->BC[(size_t)k * N + n];
    }
    std::vector<int> bcn, slaves, mst, sstart, slv;
    for (int n = 0; n < N; ++n) {
        if (m->iBC[n] & 0x3F) bcn.push_back(n);
        if (m->iper[n] != n) slaves.push_back(n);
    }
    {
        std::vector<int> cnt(N, 0);
        for (int s : slaves) cnt[m->iper[s]]++;
        std::vector<int> pos(N, -1);
        sstart.push_back(0);
        for (int n = 0; n < N; ++n)
            if (cnt[n] > 0) {
                pos[n] = (int)mst.size();
                mst.push_back(n);
                sstart.push_back(sstart.back() + cnt[n]);
            }
        slv.assign(slaves.size(), 0);
        std::vector<int> fillp(sstart.begin(), sstart.end() - 1);
        for (int s : slaves) slv[fillp[pos[m->iper[s]]]++] = s;  // ascending slave order
    }
    C.nbcn = (int)bcn.size();
    C.nslave = (int)slaves.size();
    C.nmaster = (int)mst.size();
    const size_t n5 = 5 * (size_t)N;
    const int K = cfg->Kspace;
    T(dalloc(C, &C.d_ienb, std::max(C.Eb, 1)));
    T(dalloc(C, &C.d_iBCB, std::max(C.Eb, 1)));
    T(dalloc(C, &C.d_BCB, 18 * (size_t)std::max(C.Eb, 1)));
    T(dalloc(C, &C.d_ienh, 8 * (size_t)std::max(C.nhex, 1)));
    T(dalloc(C, &C.d_ienw, 6 * (size_t)std::max(C.nwedge, 1)));
    T(dalloc(C, &C.d_x, 3 * (size_t)N));
    T(dalloc(C, &C.d_xf, 3 * (size_t)N));
    T(dalloc(C, &C.d_xbf, 2 * (size_t)N));
    T(dalloc(C, &C.d_xlo, 3 * (size_t)N));
    T(dalloc(C, &C.d_iBC, N));
    T(dalloc(C, &C.d_BC, 6 * (size_t)N));
    T(dalloc(C, &C.d_iper, N));
    T(dalloc(C, &C.d_bcn, std::max(C.nbcn, 1)));
    T(dalloc(C, &C.d_slaves, std::max(C.nslave, 1)));
    T(dalloc(C, &C.d_mst, std::max(C.nmaster, 1)));
    T(dalloc(C, &C.d_slv_start, C.nmaster + 1));
    T(dalloc(C, &C.d_slv, std::max(C.nslave, 1)));
    for (double** p : {&C.d_y, &C.d_ac, &C.d_yold, &C.d_acold, &C.d_res, &C.d_rmes, &C.d_Dy, &C.d_ypre, &C.d_t64, &C.d_t64b})
        T(dalloc(C, p, n5));
    T(dalloc(C, &C.d_bd, 25 * (size_t)N));
    T(dalloc(C, &C.d_bdstage, 25 * (size_t)N));
    for (float** p : {&C.d_yf, &C.d_ylo, &C.d_acf, &C.d_resf, &C.d_rmesf, &C.d_t32, &C.d_t32b}) T(dalloc(C, p, n5));
    T(dalloc(C, &C.d_bdf, 25 * (size_t)N));
    T(dalloc(C, &C.d_qres, 13 * (size_t)N));
    T(dalloc(C, &C.d_qresf, 13 * (size_t)N));
    {
        const size_t vb = (cfg->precision == PHGPU_FP64) ? sizeof(double) : sizeof(float);
        char* p = nullptr;
        C.ldU = (n5 + 63) / 64 * 64;
        T(dalloc(C, &p, vb * C.ldU * (size_t)(K + 1)));
        C.d_U = p;
        C.Ucap = K;
    }
    T(dalloc(C, &C.d_scal, S_TOTAL));
    T(dalloc(C, &C.d_part, kRedBlocks));
    T(dalloc(C, &C.d_count, 1));
    T(dalloc(C, &C.d_flag, 4));
    if (rc == PHGPU_OK) T(check(C, cudaMemsetAsync(C.d_flag, 0, sizeof(int) * 4, C.stream), "clear flags"));
    if (rc == PHGPU_OK && cudaMallocHost((void**)&C.h_scal, sizeof(double) * 16) != cudaSuccess) rc = PHGPU_ERR_NOMEM;
    if (rc == PHGPU_OK && cudaMallocHost((void**)&C.h_flag, sizeof(int) * 4) != cudaSuccess) rc = PHGPU_ERR_NOMEM;
    if (rc != PHGPU_OK) {
        phgpu_destroy(h);
        return rc;
    }
    // on the context's stream; the host vectors stay alive until the stream synchronisation below
    auto up = [&](void* d, const void* s, size_t bytes) {
        if (bytes) T(check(C, cudaMemcpyAsync(d, s, bytes, cudaMemcpyHostToDevice, C.stream), "upload mesh"));
    };
    up(C.d_ienb, ienb.data(), sizeof(int4) * ienb.size());
    if (C.nhex > 0) {
        std::vector<int> v(8 * (size_t)C.nhex);
        for (int i = 0; i < C.nhex; ++i)
            for (int a = 0; a < 8; ++a) v[8 * (size_t)i + a] = m->ienh[8 * (size_t)horder[i] + a];
        up(C.d_ienh, v.data(), sizeof(int) * v.size());
        C.h_ienh = v;
    }
    if (C.nwedge > 0) {
        std::vector<int> v(6 * (size_t)C.nwedge);
        for (int i = 0; i < C.nwedge; ++i)
            for (int a = 0; a < 6; ++a) v[6 * (size_t)i + a] = m->ienw[6 * (size_t)worder[i] + a];
        up(C.d_ienw, v.data(), sizeof(int) * v.size());
        C.h_ienw = v;
    }
    up(C.d_iBCB, ibcb.data(), sizeof(int) * ibcb.size());
    up(C.d_BCB, bcb.data(), sizeof(double) * bcb.size());
    up(C.d_x, x.data(), sizeof(double) * x.size());
    up(C.d_xf, xf.data(), sizeof(float) * xf.size());
    up(C.d_xlo, xlo.data(), sizeof(float) * xlo.size());
    up(C.d_iBC, m->iBC, sizeof(int) * N);
    up(C.d_BC, bc.data(), sizeof(double) * bc.size());
    up(C.d_iper, m->iper, sizeof(int) * N);
    if (C.nbcn) up(C.d_bcn, bcn.data(), sizeof(int) * C.nbcn);
    if (C.nslave) up(C.d_slaves, slaves.data(), sizeof(int) * C.nslave);
    if (C.nmaster) up(C.d_mst, mst.data(), sizeof(int) * C.nmaster);
    up(C.d_slv_start, sstart.data(), sizeof(int) * sstart.size());
    if (C.nslave) up(C.d_slv, slv.data(), sizeof(int) * C.nslave);
    T(check(C, cudaStreamSynchronize(C.stream), "upload mesh"));
    T(check(C, cudaMemsetAsync(C.d_count, 0, sizeof(unsigned int), C.stream), "memset"));
    T(check(C, cudaMemsetAsync(C.d_scal, 0, sizeof(double) * S_TOTAL, C.stream), "memset"));
    for (double* p : {C.d_y, C.d_ac, C.d_yold, C.d_acold})
        T(check(C, cudaMemsetAsync(p, 0, sizeof(double) * n5, C.stream), "memset"));
    T(upload_tables(C));
    T(sync(C));
    if (rc != PHGPU_OK) {
        phgpu_destroy(h);
        return rc;
    }
    *out = h;
    return PHGPU_OK;
}

int phgpu_destroy(phgpu_ctx* h) {
    if (!h) return PHGPU_OK;
    Ctx& C = h->c;
    if (C.stream) cudaStreamSynchronize(C.stream);
    phgpu::cycle_graph_free(C);
    phgpu::net_free(C);
    phgpu::bnd_free(C);
    if (C.stepg.exec) cudaGraphExecDestroy(C.stepg.exec);
    if (C.stepg.graph) cudaGraphDestroy(C.stepg.graph);
    if (C.stepg.d_stats) cudaFree(C.stepg.d_stats);
    if (C.stepg.aux) cudaStreamDestroy(C.stepg.aux);
    void* ptrs[] = {C.d_ch_elem, C.d_ch_node, C.d_ch_nodes, C.d_ch_cstart, C.d_ch_csr, C.d_ch_lien,
                    C.d_ch_rec, C.d_ch_rec_off, C.d_xbf,
                    C.d_bdstage, C.d_ien, C.d_ienh, C.d_ienw, C.d_ienb, C.d_iBCB, C.d_BCB, C.d_x, C.d_xf, C.d_xlo, C.d_iBC, C.d_BC, C.d_iper, C.d_bcn,
                    C.d_slaves, C.d_mst, C.d_slv_start, C.d_slv, C.d_y, C.d_ac, C.d_yold, C.d_acold, C.d_res,
                    C.d_rmes, C.d_Dy, C.d_ypre, C.d_t64, C.d_t64b, C.d_bd, C.d_yf, C.d_ylo, C.d_acf, C.d_resf, C.d_rmesf,
                    C.d_t32, C.d_t32b, C.d_bdf, C.d_qres, C.d_qresf, C.d_U, C.d_scal, C.d_part, C.d_count, C.d_flag,
                    C.sp.d_rs, C.sp.d_bcol, C.sp.d_bcolp, C.sp.d_brow, C.sp.d_ient, C.sp.d_tmap, C.sp.d_hmap,
                    C.sp.d_wmap, C.sp.d_lhsK, C.sp.d_lhsKf, C.sp.d_EG, C.sp.d_EGf, C.d_Ih, C.d_Iw};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (C.h_scal) cudaFreeHost(C.h_scal);
    if (C.h_flag) cudaFreeHost(C.h_flag);
    for (auto& e : C.ev)
        if (e) cudaEventDestroy(e);
    if (C.stream) cudaStreamDestroy(C.stream);
    delete h;
    return PHGPU_OK;
}

int phgpu_set_config(phgpu_ctx* h, const phgpu_config* cfg) {
    if (!h || !cfg) return PHGPU_ERR_INVALID;
    if (cfg->Kspace < 1 || cfg->Kspace > h->c.Ucap || cfg->nGMRES < 1) return PHGPU_ERR_INVALID;
    if ((cfg->itau != 0 && cfg->itau != 1) || cfg->ipord != 1 || cfg->EntropyPressure != 0) return PHGPU_ERR_UNSUPPORTED;
    // itau = 1 (Diagonal-Franca) is in the FP64 kernels; the reference leaves its momentum tau
    // unset when the stabilization time term is removed (e3tau.f:107-111)
    if (cfg->itau == 1 && (cfg->precision != PHGPU_FP64 || cfg->iremoveStabTimeTerm != 0 || !(cfg->rmu > 0.0)))
        return PHGPU_ERR_UNSUPPORTED;
    if (cfg->idiff != 0 && cfg->idiff != 1) return PHGPU_ERR_UNSUPPORTED;
    if (cfg->iDC < 0 || cfg->iDC > 3) return PHGPU_ERR_INVALID;
    if (cfg->precond != PHGPU_PRECOND_BDIAG && cfg->precond != PHGPU_PRECOND_LEARNED) return PHGPU_ERR_INVALID;
    const bool was64 = h->c.cfg.precision == PHGPU_FP64;
    const bool is64 = cfg->precision == PHGPU_FP64;
    if (was64 != is64 && !was64) return PHGPU_ERR_UNSUPPORTED;  // basis was allocated as FP32
    h->c.cfg = *cfg;
    return PHGPU_OK;
}
int phgpu_get_config(phgpu_ctx* h, phgpu_config* cfg) {
    if (!h || !cfg) return PHGPU_ERR_INVALID;
    *cfg = h->c.cfg;
    return PHGPU_OK;
}
const char* phgpu_last_error(phgpu_ctx* h) { return h ? h->c.err.c_str() : "null context"; }
void* phgpu_stream(phgpu_ctx* h) { return h ? (void*)h->c.stream : nullptr; }
int phgpu_num_colors(phgpu_ctx* h) { return h ? (int)h->c.chunk_col_start.size() - 1 : 0; }
long long phgpu_kernel_launches(phgpu_ctx* h) { return h ? h->c.launches : 0; }

int phgpu_set_tuning(phgpu_ctx* h, int lin_minb, int ress_minb) {
    if (!h) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    if ((lin_minb == 0 && ress_minb == 0) || (lin_minb == -1 && ress_minb == -1)) {
        C.tune_forced = false;
        C.tuned = false;
        C.tune_always = lin_minb == -1;
        for (double& t : C.tune_ms) t = -1.0;
        phgpu::select_sweep_variants(C, 0, 0);
        return PHGPU_OK;
    }
    if (lin_minb < 3 || lin_minb > 4 || ress_minb < 2 || ress_minb > 4)
        return phgpu::fail(C, PHGPU_ERR_INVALID, "sweep variants: lin_minb 3 or 4, ress_minb 2, 3 or 4");
    C.tune_forced = true;
    phgpu::select_sweep_variants(C, lin_minb, ress_minb);
    return PHGPU_OK;
}

int phgpu_tuning(phgpu_ctx* h, int* lin_minb, int* ress_minb, double* ms) {
    if (!h) return PHGPU_ERR_INVALID;
    const Ctx& C = h->c;
    if (lin_minb) *lin_minb = C.lin_minb;
    if (ress_minb) *ress_minb = C.ress_minb;
    if (ms) for (int i = 0; i < 5; ++i) ms[i] = C.tune_ms[i];
    return C.tune_forced ? 2 : C.tuned ? 1 : 0;
}

long long phgpu_step_graphs(phgpu_ctx* h) {
    if (!h) return 0;
    if (h->c.stepg.disabled) {
        h->c.err = h->c.stepg.why;
        return -1;
    }
    return h->c.stepg.runs;
}

long long phgpu_graph_cycles(phgpu_ctx* h) {
    if (!h) return 0;
    if (h->c.cyc.disabled) {
        h->c.err = h->c.cyc.why;
        return -1;
    }
    return h->c.cyc.runs;
}

int phgpu_elmmfg(phgpu_ctx* h, const double* y, const double* ac, double* res, double* rmes, double* bdiag,
                 int iprec) {
    using namespace phgpu;
    if (!h || !y || !ac || !res || !rmes || (iprec && !bdiag)) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    ref_to_dev_state(C, y, C.d_t64, C.d_y);
    ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(elmmfg64(C, C.d_y, C.d_ac, C.d_res, C.d_rmes, C.d_bd, iprec));
    dev_to_ref_res(C, C.d_res, C.d_t64, res);
    dev_to_ref_res(C, C.d_rmes, C.d_t64b, rmes);
    if (iprec) {
        dev_to_ref_bd(C, C.d_bd, C.d_bdstage, bdiag);
        return sync(C);
    }
    return sync(C);
}

int phgpu_elmres(phgpu_ctx* h, const double* y, const double* ac, double* res) {
    using namespace phgpu;
    if (!h || !y || !ac || !res) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    ref_to_dev_state(C, y, C.d_t64, C.d_y);
    ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(elmres64(C, C.d_y, C.d_ac, C.d_res));
    dev_to_ref_res(C, C.d_res, C.d_t64, res);
    return sync(C);
}

int phgpu_itrres(phgpu_ctx* h, const double* yp, const double* yc, const double* ac, double* rmes) {
    using namespace phgpu;
    if (!h || !yp || !yc || !rmes) return PHGPU_ERR_INVALID;
    (void)ac;  // the modified residual (ires = 2) does not read the acceleration
    Ctx& C = h->c;
    C.err.clear();
    ref_to_dev_state(C, yp, C.d_t64, C.d_ypre);
    ref_to_dev_state(C, yc, C.d_t64b, C.d_y);
    ref_to_dev_res(C, rmes, C.d_t64, C.d_rmes);
    PH_TRY(itrres_dev<double>(C, C.d_x, C.d_ypre, C.d_y, C.d_rmes, 0, nullptr));
    dev_to_ref_res(C, C.d_rmes, C.d_t64b, rmes);
    return sync(C);
}

int phgpu_i3lu(phgpu_ctx* h, double* bdiag, double* r, int code) {
    using namespace phgpu;
    if (!h || !bdiag || (code != PHGPU_LU_FACT && !r) || code < 0 || code > 3) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    double* tmp = C.d_bdstage;
    ref_to_dev_bd(C, bdiag, tmp, C.d_bd);
    int rc = PHGPU_OK;
    if (code == PHGPU_LU_FACT) {
        fill0(C, C.d_flag, sizeof(int) * 2);
        lu_fact<double>(C, C.d_bd, C.d_flag);
        dev_to_ref_bd(C, C.d_bd, tmp, bdiag);
        cudaMemcpyAsync(C.h_flag, C.d_flag, sizeof(int) * 2, cudaMemcpyDeviceToHost, C.stream);
        rc = sync(C);
        if (rc == PHGPU_OK && C.h_flag[1]) rc = fail(C, PHGPU_ERR_SINGULAR, "zero pivot in i3LU");
    } else {
        ref_to_dev_res(C, r, C.d_t64, C.d_res);
        lu_apply<double, double>(C, C.d_bd, C.d_res, code);
        dev_to_ref_res(C, C.d_res, C.d_t64, r);
        rc = sync(C);
    }
    return rc;
}

int phgpu_upload_state(phgpu_ctx* h, const double* y, const double* ac, const double* yold, const double* acold) {
    using namespace phgpu;
    if (!h) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    if (y) ref_to_dev_state(C, y, C.d_t64, C.d_y);
    if (ac) ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(sync(C));
    if (yold) ref_to_dev_state(C, yold, C.d_t64, C.d_yold);
    if (acold) ref_to_dev_state(C, acold, C.d_t64b, C.d_acold);
    return sync(C);
}

int phgpu_download_state(phgpu_ctx* h, double* y, double* ac, double* yold, double* acold) {
    using namespace phgpu;
    if (!h) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    if (y) dev_to_ref_state(C, C.d_y, C.d_t64, y);
    if (ac) dev_to_ref_state(C, C.d_ac, C.d_t64b, ac);
    PH_TRY(sync(C));
    if (yold) dev_to_ref_state(C, C.d_yold, C.d_t64, yold);
    if (acold) dev_to_ref_state(C, C.d_acold, C.d_t64b, acold);
    return sync(C);
}

int phgpu_solmfg(phgpu_ctx* h, const double* y, const double* ac, double* res, double* bdiag, double* Dy,
                 phgpu_stats* st) {
    using namespace phgpu;
    if (!h || !y || !ac || !st) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    ref_to_dev_state(C, y, C.d_t64, C.d_y);
    ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(sync(C));
    int ntot = st->ntotGM;
    *st = phgpu_stats{};
    st->ntotGM = ntot;
    PH_TRY(solmfg_dev(C, st));
    if (res) dev_to_ref_res(C, C.d_res, C.d_t64, res);
    if (Dy) dev_to_ref_res(C, C.d_Dy, C.d_t64b, Dy);
    PH_TRY(sync(C));
    if (bdiag) {
        dev_to_ref_bd(C, C.d_bd, C.d_bdstage, bdiag);
        return sync(C);
    }
    return PHGPU_OK;
}

int phgpu_set_bc(phgpu_ctx* h, const double* BC) {
    using namespace phgpu;
    if (!h || !BC) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    const int N = C.N;
    std::vector<double> bc(6 * (size_t)N);
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < 6; ++k) bc[6 * (size_t)n + k] = BC[(size_t)k * N + n];
    PH_TRY(check(C, cudaMemcpyAsync(C.d_BC, bc.data(), sizeof(double) * bc.size(), cudaMemcpyHostToDevice, C.stream), "BC"));
    return sync(C);
}

int phgpu_net_collect(phgpu_ctx* h, int slot, int which) {
    using namespace phgpu;
    if (!h) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    if (C.cfg.precision != PHGPU_MIXED || C.cfg.ap_mode != PHGPU_AP_LINEAR)
        return fail(C, PHGPU_ERR_UNSUPPORTED, "training pairs come from a mixed-precision solve with the linearized product");
    if (slot < 0 || slot >= C.net.tr.cap) return fail(C, PHGPU_ERR_INVALID, "pair slot outside the allocated training set");
    if (which < 0 || which > C.cfg.Kspace) return fail(C, PHGPU_ERR_INVALID, "which: 0 (solution) or a Krylov vector 1..Kspace");
    const size_t n5 = 5 * (size_t)C.N;
    // features of the solve's state and factors
    PH_TRY(net_setup(C));
    PH_TRY(net_prepare(C));
    float* u = C.d_t32b;
    if (which == 0) {
        // w = U Dy, the Krylov-space solution
        k_copy<double><<<kVG, kVT, 0, C.stream>>>(C.d_Dy, C.d_t64, n5, nullptr);
        ++C.launches;
        lu_apply<double, double>(C, C.d_bd, C.d_t64, PHGPU_LU_PRODUCT);
        to_f32(C, C.d_t64, u, n5);
    } else {
        // Krylov vector u_which of the solve's last cycle
        k_copy<float><<<kVG, kVT, 0, C.stream>>>((const float*)C.d_U + (size_t)(which - 1) * C.ldU, u, n5, nullptr);
        ++C.launches;
    }
    // A~ u with the operator the Krylov loop multiplies by
    float* Au = C.net.d_Z;
    PH_TRY(ap_lin<float>(C, u, Au, nullptr));
    dot<float>(C, Au, Au, n5, S_TMP0, nullptr);
    PH_TRY(net_store_pair(C, slot, Au, u, C.d_scal + S_TMP0));
    return sync(C);
}

int phgpu_genadj(const phgpu_mesh* m, int nnz, int* colm, int* rowp, int* icnt) {
    using namespace phgpu;
    if (!m || !colm || !rowp || !icnt || nnz <= 0 || m->nshg <= 0 || m->nelem < 0 || m->nhex < 0 || m->nwedge < 0)
        return PHGPU_ERR_INVALID;
    if ((m->nelem > 0 && !m->ien) || (m->nhex > 0 && !m->ienh) || (m->nwedge > 0 && !m->ienw)) return PHGPU_ERR_INVALID;
    const int N = m->nshg;
    const int* blk[3] = {m->ien, m->ienh, m->ienw};
    const size_t len[3] = {4 * (size_t)m->nelem, 8 * (size_t)m->nhex, 6 * (size_t)m->nwedge};
    for (int b = 0; b < 3; ++b)
        for (size_t i = 0; i < len[b]; ++i)
            if (blk[b][i] < 0 || blk[b][i] >= N) return PHGPU_ERR_INVALID;
    std::vector<int> cm, rp;
    block_adjacency(N, m->ien, m->nelem, m->ienh, m->nhex, m->ienw, m->nwedge, cm, rp);
    for (int n = 0; n < N; ++n)
        if (cm[n + 1] - cm[n] > 15 * nnz) return PHGPU_ERR_TOO_LARGE;  // genadj.f: "increase overflow factor"
    if (rp.size() > (size_t)nnz * N) return PHGPU_ERR_TOO_LARGE;        // genadj.f: "increase nnz"
    std::copy(cm.begin(), cm.end(), colm);
    std::copy(rp.begin(), rp.end(), rowp);
    *icnt = (int)rp.size();
    return PHGPU_OK;
}

int phgpu_nnz_tot(phgpu_ctx* h, int* nnz_tot) {
    using namespace phgpu;
    if (!h || !nnz_tot) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    PH_TRY(sparse_setup(C));
    *nnz_tot = C.sp.nnzb;
    return PHGPU_OK;
}

int phgpu_elmgmrs(phgpu_ctx* h, const double* y, const double* ac, double* res, double* bdiag, double* lhsK) {
    using namespace phgpu;
    if (!h || !y || !ac || !res || !bdiag || !lhsK) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    PH_TRY(sparse_setup(C));
    C.sp.have = -1;
    ref_to_dev_state(C, y, C.d_t64, C.d_y);
    ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(elmres64(C, C.d_y, C.d_ac, C.d_res));
    PH_TRY(tangent64(C, C.d_y, C.sp.d_lhsK, C.d_bd));
    dev_to_ref_res(C, C.d_res, C.d_t64, res);
    dev_to_ref_bd(C, C.d_bd, C.d_bdstage, bdiag);
    PH_TRY(check(C, cudaMemcpyAsync(lhsK, C.sp.d_lhsK, sizeof(double) * 25 * (size_t)C.sp.nnzb,
                                    cudaMemcpyDeviceToHost, C.stream), "download lhsK"));
    return sync(C);
}

int phgpu_spsi3pre(phgpu_ctx* h, const double* bdiag, double* lhsK) {
    using namespace phgpu;
    if (!h || !bdiag || !lhsK) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    PH_TRY(sparse_setup(C));
    C.sp.have = -1;
    const size_t nb = 25 * (size_t)C.sp.nnzb;
    ref_to_dev_bd(C, bdiag, C.d_bdstage, C.d_bd);
    PH_TRY(check(C, cudaMemcpyAsync(C.sp.d_lhsK, lhsK, sizeof(double) * nb, cudaMemcpyHostToDevice, C.stream), "upload lhsK"));
    spsi3pre<double>(C, C.d_bd, C.sp.d_lhsK);
    PH_TRY(check(C, cudaMemcpyAsync(lhsK, C.sp.d_lhsK, sizeof(double) * nb, cudaMemcpyDeviceToHost, C.stream), "download lhsK"));
    return sync(C);
}

int phgpu_sparseap(phgpu_ctx* h, const double* lhsK, double* p) {
    using namespace phgpu;
    if (!h || !lhsK || !p) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    PH_TRY(sparse_setup(C));
    C.sp.have = -1;
    const size_t nb = 25 * (size_t)C.sp.nnzb;
    PH_TRY(check(C, cudaMemcpyAsync(C.sp.d_lhsK, lhsK, sizeof(double) * nb, cudaMemcpyHostToDevice, C.stream), "upload lhsK"));
    ref_to_dev_res(C, p, C.d_t64, C.d_t64b);
    sparse_ap<double, double>(C, C.sp.d_lhsK, C.d_t64b, C.d_Dy);
    dev_to_ref_res(C, C.d_Dy, C.d_t64, p);
    return sync(C);
}

int phgpu_solgmrs(phgpu_ctx* h, const double* y, const double* ac, int lhs, double* res, double* bdiag, double* Dy,
                  double* lhsK, phgpu_stats* st) {
    using namespace phgpu;
    if (!h || !y || !ac || !st || (lhs != 0 && lhs != 1)) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    ref_to_dev_state(C, y, C.d_t64, C.d_y);
    ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(sync(C));
    const int ntot = st->ntotGM, lg = st->lGMRES;
    *st = phgpu_stats{};
    st->ntotGM = ntot;
    const int ap = C.cfg.ap_mode;
    C.cfg.ap_mode = PHGPU_AP_SPARSE;
    const int rc = solve_dev(C, st, lhs, lg);
    C.cfg.ap_mode = ap;
    PH_TRY(rc);
    if (res) dev_to_ref_res(C, C.d_res, C.d_t64, res);
    if (Dy) dev_to_ref_res(C, C.d_Dy, C.d_t64b, Dy);
    if (bdiag) dev_to_ref_bd(C, C.d_bd, C.d_bdstage, bdiag);
    if (lhsK && C.cfg.precision == PHGPU_FP64)
        PH_TRY(check(C, cudaMemcpyAsync(lhsK, C.sp.d_lhsK, sizeof(double) * 25 * (size_t)C.sp.nnzb,
                                        cudaMemcpyDeviceToHost, C.stream), "download lhsK"));
    return sync(C);
}

// the element-by-element entry points work in FP64 on the context's FP64 element storage
static int ebe_fp64(phgpu::Ctx& C) {
    const int prec = C.cfg.precision;
    C.cfg.precision = PHGPU_FP64;
    const int rc = phgpu::ebe_setup(C);
    C.cfg.precision = prec;
    return rc;
}

int phgpu_elmgmre(phgpu_ctx* h, const double* y, const double* ac, double* res, double* bdiag, double* EGmass) {
    using namespace phgpu;
    if (!h || !y || !ac || !res || !bdiag || !EGmass) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    PH_TRY(ebe_fp64(C));
    ref_to_dev_state(C, y, C.d_t64, C.d_y);
    ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(elmres64(C, C.d_y, C.d_ac, C.d_res));
    PH_TRY(tangent64(C, C.d_y, C.sp.d_EG, C.d_bd, true));
    dev_to_ref_res(C, C.d_res, C.d_t64, res);
    dev_to_ref_bd(C, C.d_bd, C.d_bdstage, bdiag);
    return ebe_download(C, C.sp.d_EG, EGmass);
}

int phgpu_i3pre(phgpu_ctx* h, const double* bdiag, double* EGmass) {
    using namespace phgpu;
    if (!h || !bdiag || !EGmass) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    PH_TRY(ebe_fp64(C));
    ref_to_dev_bd(C, bdiag, C.d_bdstage, C.d_bd);
    PH_TRY(ebe_upload(C, EGmass, C.sp.d_EG));
    i3pre<double>(C, C.d_bd, C.sp.d_EG);
    return ebe_download(C, C.sp.d_EG, EGmass);
}

int phgpu_au1gmr(phgpu_ctx* h, const double* EGmass, double* p) {
    using namespace phgpu;
    if (!h || !EGmass || !p) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    PH_TRY(ebe_fp64(C));
    PH_TRY(ebe_upload(C, EGmass, C.sp.d_EG));
    ref_to_dev_res(C, p, C.d_t64, C.d_t64b);
    ebe_ap<double, double>(C, C.sp.d_EG, C.d_t64b, C.d_Dy);
    dev_to_ref_res(C, C.d_Dy, C.d_t64, p);
    return sync(C);
}

int phgpu_solgmre(phgpu_ctx* h, const double* y, const double* ac, double* res, double* bdiag, double* Dy,
                  double* EGmass, phgpu_stats* st) {
    using namespace phgpu;
    if (!h || !y || !ac || !st) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    ref_to_dev_state(C, y, C.d_t64, C.d_y);
    ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(sync(C));
    const int ntot = st->ntotGM;
    *st = phgpu_stats{};
    st->ntotGM = ntot;
    const int ap = C.cfg.ap_mode;
    C.cfg.ap_mode = PHGPU_AP_EBE;
    const int rc = solve_dev(C, st, 1, 0);
    C.cfg.ap_mode = ap;
    PH_TRY(rc);
    if (res) dev_to_ref_res(C, C.d_res, C.d_t64, res);
    if (Dy) dev_to_ref_res(C, C.d_Dy, C.d_t64b, Dy);
    if (bdiag) dev_to_ref_bd(C, C.d_bd, C.d_bdstage, bdiag);
    PH_TRY(sync(C));
    if (EGmass && C.cfg.precision == PHGPU_FP64) return ebe_download(C, C.sp.d_EG, EGmass);
    return PHGPU_OK;
}

int phgpu_itrcorrect(phgpu_ctx* h, double* y, double* ac, const double* yold, const double* acold, const double* Dy) {
    using namespace phgpu;
    if (!h || !y || !ac || !yold || !acold || !Dy) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    C.err.clear();
    ref_to_dev_state(C, y, C.d_t64, C.d_y);
    ref_to_dev_state(C, ac, C.d_t64b, C.d_ac);
    PH_TRY(sync(C));
    ref_to_dev_state(C, yold, C.d_t64, C.d_yold);
    ref_to_dev_state(C, acold, C.d_t64b, C.d_acold);
    PH_TRY(sync(C));
    ref_to_dev_res(C, Dy, C.d_t64, C.d_Dy);
    PH_TRY(correct_dev(C));
    dev_to_ref_state(C, C.d_y, C.d_t64, y);
    dev_to_ref_state(C, C.d_ac, C.d_t64b, ac);
    return sync(C);
}

int phgpu_newton_dev(phgpu_ctx* h, phgpu_stats* st) {
    if (!h || !st) return PHGPU_ERR_INVALID;
    h->c.err.clear();
    int ntot = st->ntotGM;
    *st = phgpu_stats{};
    st->ntotGM = ntot;
    int rc = phgpu::newton_dev(h->c, st);
    st->status = rc;
    return rc;
}

int phgpu_newton(phgpu_ctx* h, double* y, double* ac, const double* yold, const double* acold, phgpu_stats* st) {
    if (!h || !y || !ac || !yold || !acold || !st) return PHGPU_ERR_INVALID;
    int rc = phgpu_upload_state(h, y, ac, yold, acold);
    if (rc != PHGPU_OK) return rc;
    rc = phgpu_newton_dev(h, st);
    if (rc != PHGPU_OK) return rc;
    return phgpu_download_state(h, y, ac, nullptr, nullptr);
}

int phgpu_time_step_dev(phgpu_ctx* h, int nitr, phgpu_stats* st) {
    if (!h || !st || nitr < 1) return PHGPU_ERR_INVALID;
    h->c.err.clear();
    int ntot = st->ntotGM;
    *st = phgpu_stats{};
    st->ntotGM = ntot;
    int rc = phgpu::time_step_dev(h->c, nitr, st);
    st->status = rc;
    return rc;
}

int phgpu_time_step(phgpu_ctx* h, double* yold, double* acold, double* y, double* ac, int nitr, phgpu_stats* st) {
    if (!h || !yold || !acold || !y || !ac || !st) return PHGPU_ERR_INVALID;
    int rc = phgpu_upload_state(h, nullptr, nullptr, yold, acold);
    if (rc != PHGPU_OK) return rc;
    rc = phgpu_time_step_dev(h, nitr, st);
    if (rc != PHGPU_OK) return rc;
    return phgpu_download_state(h, y, ac, yold, acold);
}

int phgpu_residual_norm_dev(phgpu_ctx* h, double* rnorm) {
    using namespace phgpu;
    if (!h || !rnorm) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    PH_TRY(elmres64(C, C.d_y, C.d_ac, C.d_res));
    dot<double>(C, C.d_res, C.d_res, 5 * (size_t)C.N, S_TMP2, nullptr);
    PH_TRY(check(C, cudaMemcpyAsync(C.h_scal, C.d_scal, sizeof(double) * 8, cudaMemcpyDeviceToHost, C.stream), "rnorm"));
    PH_TRY(sync(C));
    *rnorm = std::sqrt(C.h_scal[S_TMP2]);
    return PHGPU_OK;
}

int phgpu_sweep_dev(phgpu_ctx* h, int which) {
    using namespace phgpu;
    if (!h) return PHGPU_ERR_INVALID;
    Ctx& C = h->c;
    const size_t n5 = 5 * (size_t)C.N;
    switch (which) {
        case 0:  // FP64 residual
            launch_elem_res<double>(C, RM_RES, C.d_x, C.d_y, nullptr, C.d_ac, C.d_res, 0, nullptr);
            break;
        case 1:  // FP64 modified residual
            launch_elem_res<double>(C, RM_MODRES, C.d_x, C.d_y, C.d_y, nullptr, C.d_rmes, 0, nullptr);
            break;
        case 2:  // FP32 linearized product in direction y
            launch_elem_res<float>(C, RM_LIN, C.d_xf, C.d_yf, C.d_yf, nullptr, C.d_t32, 0, nullptr);
            break;
        case 15: {  // the same product with one CTA per chunk (no cp.async pipeline)
            const int keep = C.cfg.no_pipe;
            C.cfg.no_pipe = 1;
            launch_elem_res<float>(C, RM_LIN, C.d_xf, C.d_yf, C.d_yf, nullptr, C.d_t32, 0, nullptr);
            C.cfg.no_pipe = keep;
            break;
        }
        case 3:  // FP32 block diagonal
            launch_elem_full<float>(C, C.d_xf, C.d_yf, C.d_acf, nullptr, nullptr, C.d_bdf);
            break;
        case 4:  // FP64 block diagonal + residuals
            launch_elem_full<double>(C, C.d_x, C.d_y, C.d_ac, C.d_res, C.d_rmes, C.d_bd);
            break;
        case 5:
            to_f32(C, C.d_y, C.d_yf, n5);
            pack_xb(C);
            to_f32(C, C.d_ac, C.d_acf, n5);
            break;
        case 17:  // one application of the learned preconditioner (needs weights and a solve's features)
            if (!net_usable(C) || !C.net.d_Z) return fail(C, PHGPU_ERR_INVALID, "no network weights or features");
            net_apply(C, C.d_yf, C.net.d_Z);
            break;
        case 18:  // the learned preconditioner's context features
            if (!C.net.d_ctx) return fail(C, PHGPU_ERR_INVALID, "network not set up");
            PH_TRY(net_prepare(C));
            break;
        case 6:  // FP64-Galerkin / FP32-stabilization residual
            launch_elem_resh(C, C.d_y, C.d_ac, C.d_yf, C.d_acf, C.d_res);
            break;
        case 16: {  // the tets' split residual with one CTA per chunk (no cp.async pipeline)
            const int keep = C.cfg.no_pipe;
            C.cfg.no_pipe = 1;
            launch_elem_ress(C, C.d_yf, C.d_ylo, C.d_acf, C.d_res);
            C.cfg.no_pipe = keep;
            break;
        }
        case 7:  // double-float constant flux + FP32 increments (needs the hi/lo split of case 8)
            launch_elem_ress(C, C.d_yf, C.d_ylo, C.d_acf, C.d_res);
            if (C.nhex > 0 || C.nwedge > 0) {
                PH_TRY(topo_split_setup(C));
                launch_topo_ress(C, C.d_yf, C.d_ylo, C.d_acf, C.d_res, nullptr);
            }
            break;
        case 8:
            split_f32(C, C.d_y, C.d_yf, C.d_ylo, n5);
            pack_xb(C);
            to_f32(C, C.d_ac, C.d_acf, n5);
            break;
        case 9:   // FP32 assembled tangent (zero fill + element sweep)
        case 11:  // FP64 assembled tangent
            PH_TRY(sparse_setup(C));
            C.sp.have = -1;
            if (which == 9) {
                fill0(C, C.sp.d_lhsKf, sizeof(float) * 25 * (size_t)C.sp.nnzb);
                launch_tangent<float>(C, C.d_xf, C.d_yf, C.sp.d_lhsKf);
            } else {
                fill0(C, C.sp.d_lhsK, sizeof(double) * 25 * (size_t)C.sp.nnzb);
                launch_tangent<double>(C, C.d_x, C.d_y, C.sp.d_lhsK);
            }
            break;
        case 10:  // FP32 block-sparse product (SparseAp + bc3per) of the state
            PH_TRY(sparse_setup(C));
            sparse_ap<float, float>(C, C.sp.d_lhsKf, C.d_yf, C.d_t32);
            break;
        case 12:  // FP64 block-sparse product
            PH_TRY(sparse_setup(C));
            sparse_ap<double, double>(C, C.sp.d_lhsK, C.d_y, C.d_t64);
            break;
        case 13:  // FP32 element tangents stored per element (element-by-element solver)
            PH_TRY(ebe_setup(C));
            launch_tangent_ebe<float>(C, C.d_xf, C.d_yf, C.sp.d_EGf, nullptr);
            break;
        case 14:  // FP32 element-by-element product (Au1GMR + bc3per)
            PH_TRY(ebe_setup(C));
            ebe_ap<float, float>(C, C.sp.d_EGf, C.d_yf, C.d_t32);
            break;
        default:
            return PHGPU_ERR_INVALID;
    }
    return check(C, cudaGetLastError(), "sweep");
}

}  // extern "C"
