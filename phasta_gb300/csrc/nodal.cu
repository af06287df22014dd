// nodal.cu -- per-node kernels: boundary conditions (bc3res.f, bc3bdg.f,
// itrbc.f), 5x5 block LU (i3lu.f), layout conversion between the reference's
// column-major arrays and the device's node-major arrays, and deterministic
// reductions with FP64 accumulation (sumgat, mpitools.f:104-140).
#include "phgpu_impl.cuh"
#include "df64.cuh"

namespace phgpu {

namespace {

constexpr int kT = 256;
inline int nblocks(size_t n) { return (int)((n + kT - 1) / kT); }

__device__ __forceinline__ int vbits(int ib) { return (ib >> 3) & 7; }

// ---------------- bc3Res (local part, bc3res.f:23-152) ----------------
template <typename R>
__global__ void k_bc3res(const int* __restrict__ nodes, int nn, const int* __restrict__ iBC,
                         const double* __restrict__ BC, R* __restrict__ r, double Rgas) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn) return;
    const int n = nodes[t];
    const int ib = iBC[n];
    R* v = r + 5 * (size_t)n;
    const double* bc = BC + 6 * (size_t)n;
    if (ib & 1) {  // density
        v[4] = v[4] + (R)bc[0] * (R)Rgas * v[0];
        v[0] = R(0);
    }
    if (ib & 4) v[0] = R(0);  // pressure (EntropyPressure = 0 form)
    const R b4 = (R)bc[3], b5 = (R)bc[4], b6 = (R)bc[5];
    switch (vbits(ib)) {
        case 1: v[2] = v[2] - b4 * v[1]; v[3] = v[3] - b5 * v[1]; v[1] = R(0); break;
        case 2: v[1] = v[1] - b4 * v[2]; v[3] = v[3] - b5 * v[2]; v[2] = R(0); break;
        case 3: v[3] = v[3] - b4 * v[1] - b6 * v[2]; v[1] = R(0); v[2] = R(0); break;
        case 4: v[1] = v[1] - b4 * v[3]; v[2] = v[2] - b5 * v[3]; v[3] = R(0); break;
        case 5: v[2] = v[2] - b4 * v[1] - b6 * v[3]; v[1] = R(0); v[3] = R(0); break;
        case 6: v[1] = v[1] - b4 * v[2] - b6 * v[3]; v[2] = R(0); v[3] = R(0); break;
        case 7: v[1] = R(0); v[2] = R(0); v[3] = R(0); break;
        default: break;
    }
    if (ib & 2) v[4] = R(0);  // temperature
}

// periodic: master += slaves (ascending slave order, bc3res.f:155-160), slaves = 0
template <typename R, int W>
__global__ void k_periodic_sum(const int* __restrict__ mst, const int* __restrict__ ss,
                               const int* __restrict__ slv, int nm, R* __restrict__ r, int copyback) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nm) return;
    const int m = mst[t];
    R acc[W];
#pragma unroll
    for (int k = 0; k < W; ++k) acc[k] = r[(size_t)W * m + k];
    for (int j = ss[t]; j < ss[t + 1]; ++j) {
        const int s = slv[j];
#pragma unroll
        for (int k = 0; k < W; ++k) acc[k] = acc[k] + r[(size_t)W * s + k];
    }
#pragma unroll
    for (int k = 0; k < W; ++k) r[(size_t)W * m + k] = acc[k];
    for (int j = ss[t]; j < ss[t + 1]; ++j) {
        const int s = slv[j];
#pragma unroll
        for (int k = 0; k < W; ++k) r[(size_t)W * s + k] = copyback ? acc[k] : R(0);
    }
}

// ---------------- bc3BDg (local part, bc3bdg.f:23-305) ----------------
template <typename R>
__global__ void k_bc3bdg(const int* __restrict__ nodes, int nn, const int* __restrict__ iBC,
                         const double* __restrict__ BC, const double* __restrict__ y, R* __restrict__ bd,
                         double a5c) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn) return;
    const int n = nodes[t];
    const int ib = iBC[n];
    R* D = bd + 25 * (size_t)n;
    auto B = [&](int i, int j) -> R& { return D[5 * (i - 1) + (j - 1)]; };  // 1-based
    const double* bc = BC + 6 * (size_t)n;
    auto zero_rc = [&](int d) {
        for (int k = 1; k <= 5; ++k)
            if (k != d) { B(d, k) = R(0); B(k, d) = R(0); }
        B(d, d) = R(1);
    };
    if (ib & 1) {
        const R a5 = (R)(-y[5 * (size_t)n + 4] * a5c);
        B(5, 5) = B(5, 5) + a5 * a5 * B(1, 1) + a5 * B(1, 5) + a5 * B(5, 1);
        B(4, 5) = B(4, 5) + a5 * B(4, 1);
        B(3, 5) = B(3, 5) + a5 * B(3, 1);
        B(2, 5) = B(2, 5) + a5 * B(2, 1);
        B(5, 4) = B(5, 4) + a5 * B(1, 4);
        B(5, 3) = B(5, 3) + a5 * B(1, 3);
        B(5, 2) = B(5, 2) + a5 * B(1, 2);
        zero_rc(1);
    }
    if (ib & 4) zero_rc(1);
    const R b4 = (R)bc[3], b5 = (R)bc[4], b6 = (R)bc[5];
    auto single = [&](int dc, int o1, int o2) {
        B(5, o2) = B(5, o2) - b5 * B(5, dc);
        B(5, o1) = B(5, o1) - b4 * B(5, dc);
        B(o2, 5) = B(o2, 5) - b5 * B(dc, 5);
        B(o1, 5) = B(o1, 5) - b4 * B(dc, 5);
        B(o2, 1) = B(o2, 1) - b5 * B(dc, 1);
        B(o1, 1) = B(o1, 1) - b4 * B(dc, 1);
        B(1, o2) = B(1, o2) - b5 * B(1, dc);
        B(1, o1) = B(1, o1) - b4 * B(1, dc);
        B(o2, o2) = B(o2, o2) + b5 * b5 * B(dc, dc) - b5 * B(dc, o2) - b5 * B(o2, dc);
        B(o1, o2) = B(o1, o2) + b4 * b5 * B(dc, dc) - b5 * B(o1, dc) - b4 * B(dc, o2);
        B(o2, o1) = B(o2, o1) + b4 * b5 * B(dc, dc) - b5 * B(dc, o1) - b4 * B(o2, dc);
        B(o1, o1) = B(o1, o1) + b4 * b4 * B(dc, dc) - b4 * B(dc, o1) - b4 * B(o1, dc);
        zero_rc(dc);
    };
    auto dbl = [&](int d1, int d2, int o) {
        B(o, o) = B(o, o) + b4 * b4 * B(d1, d1) + b6 * b6 * B(d2, d2) + b4 * b6 * (B(d1, d2) + B(d2, d1)) -
                  b4 * (B(d1, o) + B(o, d1)) - b6 * (B(d2, o) + B(o, d2));
        B(1, o) = B(1, o) - b4 * B(1, d1) - b6 * B(1, d2);
        B(o, 1) = B(o, 1) - b4 * B(d1, 1) - b6 * B(d2, 1);
        B(5, o) = B(5, o) - b4 * B(5, d1) - b6 * B(5, d2);
        B(o, 5) = B(o, 5) - b4 * B(d1, 5) - b6 * B(d2, 5);
        zero_rc(d1);
        zero_rc(d2);
    };
    switch (vbits(ib)) {
        case 1: single(2, 3, 4); break;
        case 2: single(3, 2, 4); break;
        case 3:  // bc3bdg.f:139-168 (the reference multiplies entries in this case)
            B(4, 4) = B(4, 4) + b4 * b4 * B(2, 2) + b6 * b6 * B(3, 3) + b4 * b6 * (B(2, 3) * B(3, 2)) -
                      b6 * (B(4, 3) * B(3, 4)) - b4 * (B(4, 2) * B(2, 4));
            B(1, 4) = B(1, 4) - b4 * B(1, 2) - b6 * B(1, 3);
            B(4, 1) = B(4, 1) - b4 * B(2, 1) - b6 * B(3, 1);
            B(5, 4) = B(5, 4) - b4 * B(5, 2) - b6 * B(5, 3);
            B(4, 5) = B(4, 5) - b4 * B(2, 5) - b6 * B(3, 5);
            zero_rc(2);
            zero_rc(3);
            break;
        case 4: single(4, 2, 3); break;
        case 5: dbl(2, 4, 3); break;
        case 6: dbl(3, 4, 2); break;
        case 7: zero_rc(2); zero_rc(3); zero_rc(4); break;
        default: break;
    }
    if (ib & 2) zero_rc(5);
}

// ---------------- itrBC (itrbc.f:54-176) on a state or a perturbation ----------------
// mode 0: state (affine, sets BC values); mode 1: linear part only (zero constants)
template <typename R>
__global__ void k_itrbc(const int* __restrict__ nodes, int nn, const int* __restrict__ iBC,
                        const double* __restrict__ BC, R* __restrict__ y, int lin, double Rgas) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn) return;
    const int n = nodes[t];
    const int ib = iBC[n];
    R* v = y + 5 * (size_t)n;  // local order p, u, v, w, T
    const double* bc = BC + 6 * (size_t)n;
    const R c2 = lin ? R(0) : (R)bc[1], c3 = lin ? R(0) : (R)bc[2], c5 = lin ? R(0) : (R)bc[4];
    const R b4 = (R)bc[3], b5 = (R)bc[4], b6 = (R)bc[5];
    if (ib & 2) v[4] = c2;
    switch (vbits(ib)) {
        case 1: v[1] = c3 - b4 * v[2] - b5 * v[3]; break;
        case 2: v[2] = c3 - b4 * v[1] - b5 * v[3]; break;
        case 3: v[1] = c3 - b4 * v[3]; v[2] = c5 - b6 * v[3]; break;
        case 4: v[3] = c3 - b4 * v[1] - b5 * v[2]; break;
        case 5: v[1] = c3 - b4 * v[2]; v[3] = c5 - b6 * v[2]; break;
        case 6: v[2] = c3 - b4 * v[1]; v[3] = c5 - b6 * v[1]; break;
        case 7:
            v[1] = c3;
            v[2] = lin ? R(0) : (R)bc[3];
            v[3] = c5;
            break;
        default: break;
    }
    if (ib & 1) v[1] = (R)Rgas * (R)bc[0] * v[4];  // itrbc.f:124-143 stores into y(:,1)
    if (ib & 4) v[0] = lin ? R(0) : (R)bc[0];
}

// slave <- master copy (itrbc.f:170-174)
template <typename R>
__global__ void k_periodic_copy(const int* __restrict__ slaves, int ns, const int* __restrict__ iper,
                                R* __restrict__ y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns) return;
    const int s = slaves[t];
    const int m = iper[s];
#pragma unroll
    for (int k = 0; k < 5; ++k) y[5 * (size_t)s + k] = y[5 * (size_t)m + k];
}

// ---------------- i3LU (i3lu.f:39-171) ----------------
// The factorization follows i3lu.f:41-97 statement by statement, including
// that U(4,5) is left at its input value (the reference updates every other
// upper entry of rows 2-5 but not that one).
// The factors of the blocks in `in` (type I) are written to bd (type R) and, when given, to bdf
// as floats; in may be bd or bdf.  The block's 25 x kLuT values are staged through one shared
// buffer in both directions (read in, factored in registers, written back), so the global reads
// and writes are contiguous (one thread per node would read and write at a stride of 25
// values); the arithmetic per node is unchanged.
constexpr int kLuT = 128;
template <typename R, typename I>
__global__ void __launch_bounds__(kLuT) k_lu_fact(const I* in, R* bd, float* bdf, int N, int* __restrict__ flag) {
    __shared__ __align__(16) unsigned char s_buf[25 * kLuT * 8];
    I* s_in = reinterpret_cast<I*>(s_buf);
    R* s_out = reinterpret_cast<R*>(s_buf);
    const int n0 = blockIdx.x * kLuT, t = threadIdx.x;
    const int nb = min(kLuT, N - n0);
    const size_t base = 25 * (size_t)n0;
    for (int k = t; k < 25 * nb; k += kLuT) s_in[k] = in[base + k];
    __syncthreads();
    const int n = n0 + t;
    R a[5][5];
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) a[i][j] = t < nb ? (R)s_in[25 * t + 5 * i + j] : (i == j ? R(1) : R(0));
    __syncthreads();
    bool bad = false;
    auto inv = [&](R v) {
        if (!(v == v) || v == R(0) || isinf(v)) bad = true;
        return R(1) / v;
    };
    a[0][0] = inv(a[0][0]);
    a[1][0] = a[0][0] * a[1][0];
    a[2][0] = a[0][0] * a[2][0];
    a[3][0] = a[0][0] * a[3][0];
    a[4][0] = a[0][0] * a[4][0];
    a[1][1] = a[1][1] - a[1][0] * a[0][1];
    a[1][2] = a[1][2] - a[1][0] * a[0][2];
    a[1][3] = a[1][3] - a[1][0] * a[0][3];
    a[1][4] = a[1][4] - a[1][0] * a[0][4];
    a[1][1] = inv(a[1][1]);
    a[2][1] = a[1][1] * (a[2][1] - a[2][0] * a[0][1]);
    a[3][1] = a[1][1] * (a[3][1] - a[3][0] * a[0][1]);
    a[4][1] = a[1][1] * (a[4][1] - a[4][0] * a[0][1]);
    a[2][2] = a[2][2] - a[2][0] * a[0][2] - a[2][1] * a[1][2];
    a[2][3] = a[2][3] - a[2][0] * a[0][3] - a[2][1] * a[1][3];
    a[2][4] = a[2][4] - a[2][0] * a[0][4] - a[2][1] * a[1][4];
    a[2][2] = inv(a[2][2]);
    a[3][2] = a[2][2] * (a[3][2] - a[3][0] * a[0][2] - a[3][1] * a[1][2]);
    a[4][2] = a[2][2] * (a[4][2] - a[4][0] * a[0][2] - a[4][1] * a[1][2]);
    a[3][3] = a[3][3] - a[3][0] * a[0][3] - a[3][1] * a[1][3] - a[3][2] * a[2][3];
    a[3][3] = inv(a[3][3]);
    a[4][3] = a[3][3] * (a[4][3] - a[4][0] * a[0][3] - a[4][1] * a[1][3] - a[4][2] * a[2][3]);
    a[4][4] = a[4][4] - a[4][0] * a[0][4] - a[4][1] * a[1][4] - a[4][2] * a[2][4] - a[4][3] * a[3][4];
    a[4][4] = inv(a[4][4]);
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) s_out[25 * t + 5 * i + j] = a[i][j];
    __syncthreads();
    for (int k = t; k < 25 * nb; k += kLuT) {
        const R v = s_out[k];
        bd[base + k] = v;
        if (bdf) bdf[base + k] = (float)v;
    }
    if (bad && flag && n < N) atomicOr(flag + 1, 1);
}

// in and out may be the same array (each thread reads its node's five values before writing them)
template <typename R, typename V>
__global__ void k_lu_apply(const R* __restrict__ bd, const V* in, V* out, int N, int code,
                           const int* __restrict__ skip) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    if (skip && *skip) return;
    const R* D = bd + 25 * (size_t)n;
    const V* vi = in + 5 * (size_t)n;
    V* v = out + 5 * (size_t)n;
    R x[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) x[k] = (R)vi[k];
    auto A = [&](int i, int j) { return D[5 * i + j]; };
    if (code == PHGPU_LU_FORWARD) {
        x[1] = x[1] - A(1, 0) * x[0];
        x[2] = x[2] - A(2, 0) * x[0] - A(2, 1) * x[1];
        x[3] = x[3] - A(3, 0) * x[0] - A(3, 1) * x[1] - A(3, 2) * x[2];
        x[4] = x[4] - A(4, 0) * x[0] - A(4, 1) * x[1] - A(4, 2) * x[2] - A(4, 3) * x[3];
    } else if (code == PHGPU_LU_BACKWARD) {
        x[4] = A(4, 4) * x[4];
        x[3] = A(3, 3) * (x[3] - x[4] * A(3, 4));
        x[2] = A(2, 2) * (x[2] - x[4] * A(2, 4) - x[3] * A(2, 3));
        x[1] = A(1, 1) * (x[1] - x[4] * A(1, 4) - x[3] * A(1, 3) - x[2] * A(1, 2));
        x[0] = A(0, 0) * (x[0] - x[4] * A(0, 4) - x[3] * A(0, 3) - x[2] * A(0, 2) - x[1] * A(0, 1));
    } else {  // product U.r
        x[0] = x[0] / A(0, 0) + x[1] * A(0, 1) + x[2] * A(0, 2) + x[3] * A(0, 3) + x[4] * A(0, 4);
        x[1] = x[1] / A(1, 1) + x[2] * A(1, 2) + x[3] * A(1, 3) + x[4] * A(1, 4);
        x[2] = x[2] / A(2, 2) + x[3] * A(2, 3) + x[4] * A(2, 4);
        x[3] = x[3] / A(3, 3) + x[4] * A(3, 4);
        x[4] = x[4] / A(4, 4);
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = (V)x[k];
}

// ---------------- layout conversion ----------------
// reference (nshg, 5) column-major, global order (u,v,w,p,T) <-> device [n][5] (p,u,v,w,T)
__global__ void k_state_in(const double* __restrict__ a, double* __restrict__ b, int N) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    double* o = b + 5 * (size_t)n;
    o[0] = a[3 * (size_t)N + n];
    o[1] = a[n];
    o[2] = a[(size_t)N + n];
    o[3] = a[2 * (size_t)N + n];
    o[4] = a[4 * (size_t)N + n];
}
__global__ void k_state_out(const double* __restrict__ b, double* __restrict__ a, int N) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const double* o = b + 5 * (size_t)n;
    a[3 * (size_t)N + n] = o[0];
    a[n] = o[1];
    a[(size_t)N + n] = o[2];
    a[2 * (size_t)N + n] = o[3];
    a[4 * (size_t)N + n] = o[4];
}
template <int W>
__global__ void k_soa_to_aos(const double* __restrict__ a, double* __restrict__ b, int N) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
#pragma unroll
    for (int k = 0; k < W; ++k) b[(size_t)W * n + k] = a[(size_t)k * N + n];
}
template <int W>
__global__ void k_aos_to_soa(const double* __restrict__ b, double* __restrict__ a, int N) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
#pragma unroll
    for (int k = 0; k < W; ++k) a[(size_t)k * N + n] = b[(size_t)W * n + k];
}
// BDiag (nshg,5,5) column-major bd[(i+5j)N+n] <-> [n][5i+j]
__global__ void k_bd_in(const double* __restrict__ a, double* __restrict__ b, int N) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) b[25 * (size_t)n + 5 * i + j] = a[(size_t)(i + 5 * j) * N + n];
}
__global__ void k_bd_out(const double* __restrict__ b, double* __restrict__ a, int N) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int j = 0; j < 5; ++j) a[(size_t)(i + 5 * j) * N + n] = b[25 * (size_t)n + 5 * i + j];
}
// four entries per thread and pass when both arrays start on 16-byte boundaries (16-byte
// loads or stores on each side), element by element for the rest
template <typename A, typename B>
__global__ void k_convert(const A* __restrict__ a, B* __restrict__ b, size_t n) {
    const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    const size_t n4 = (((uintptr_t)a | (uintptr_t)b) & 15) == 0 ? n / 4 : 0;
    for (size_t i = t0; i < n4; i += stride) {
        A v[4];
        if constexpr (sizeof(A) == 8) {
            const double2 p = reinterpret_cast<const double2*>(a)[2 * i], q = reinterpret_cast<const double2*>(a)[2 * i + 1];
            v[0] = p.x; v[1] = p.y; v[2] = q.x; v[3] = q.y;
        } else {
            const float4 p = reinterpret_cast<const float4*>(a)[i];
            v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = p.w;
        }
        if constexpr (sizeof(B) == 8) {
            reinterpret_cast<double2*>(b)[2 * i] = make_double2((B)v[0], (B)v[1]);
            reinterpret_cast<double2*>(b)[2 * i + 1] = make_double2((B)v[2], (B)v[3]);
        } else {
            reinterpret_cast<float4*>(b)[i] = make_float4((B)v[0], (B)v[1], (B)v[2], (B)v[3]);
        }
    }
    for (size_t i = 4 * n4 + t0; i < n; i += stride) b[i] = (B)a[i];
}

// ---------------- reductions (FP64 accumulation, fixed grid => deterministic) ----------------
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    return s;  // valid in thread 0
}

// the last block to finish sums the per-block partials in block order
__device__ __forceinline__ void finish_reduce(double bsum, double* part, unsigned int* count, double* out,
                                              double* sh) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = bsum;
        __threadfence();
        const unsigned int prev = atomicAdd(count, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double v = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) v += ((volatile double*)part)[i];
    __syncthreads();
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) {
        *out = s;
        *count = 0u;
    }
}

// Per-thread accumulation of a dot product.  FP64 vectors: FP64 fused multiply-adds.
// FP32 vectors: each product is split exactly into p + e (two_prod) and summed in
// double-float, which is at least as accurate as FP64 products of the float values
// and keeps the FP64 pipe (1/64 of the FP32 rate on this part) out of the loop.
template <typename V>
struct DotAcc;
template <>
struct DotAcc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
};
template <>
struct DotAcc<float> {
    df64 s{0.f, 0.f};
    __device__ __forceinline__ void add(float a, float b) {
        const float p = __fmul_rn(a, b);
        s = df_add(s, df_make(p, __fmaf_rn(a, b, -p)));
    }
    __device__ __forceinline__ double value() const { return df_to_double(s); }
};

// 16-byte vectors of the streaming kernels (every vector of the Krylov loop starts on a
// 256-byte boundary); the n % W tail is handled element by element
__device__ __forceinline__ bool al16(const void* p) { return ((uintptr_t)p & 15) == 0; }
template <typename V> struct Vec16;
template <> struct Vec16<float> {
    using T = float4;
    static constexpr int W = 4;
    __device__ static float at(const T& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
    __device__ static void set(T& v, int k, float x) {
        if (k == 0) v.x = x; else if (k == 1) v.y = x; else if (k == 2) v.z = x; else v.w = x;
    }
};
template <> struct Vec16<double> {
    using T = double2;
    static constexpr int W = 2;
    __device__ static double at(const T& v, int k) { return k == 0 ? v.x : v.y; }
    __device__ static void set(T& v, int k, double x) {
        if (k == 0) v.x = x; else v.y = x;
    }
};

template <typename V>
__global__ void __launch_bounds__(kRedThreads)
k_dot(const V* __restrict__ a, const V* __restrict__ b, size_t n, double* part, unsigned int* count,
      double* out, const int* __restrict__ skip) {
    using X = Vec16<V>;
    __shared__ double sh[32];
    if (skip && *skip) return;
    DotAcc<V> acc;
    const size_t nv = (al16(a) && al16(b)) ? n / X::W : 0, t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const typename X::T* av = reinterpret_cast<const typename X::T*>(a);
    const typename X::T* bv = reinterpret_cast<const typename X::T*>(b);
    for (size_t i = t0; i < nv; i += stride) {
        const typename X::T x = av[i], y = bv[i];
#pragma unroll
        for (int k = 0; k < X::W; ++k) acc.add(X::at(x, k), X::at(y, k));
    }
    for (size_t i = X::W * nv + t0; i < n; i += stride) acc.add(a[i], b[i]);
    const double bs = block_sum(acc.value(), sh);
    __syncthreads();
    finish_reduce(bs, part, count, out, sh);
}

// MGS step of solmfg.f:247-267: if up: w = w - beta_prev * up;  out = w . uj
template <typename V>
__global__ void __launch_bounds__(kRedThreads)
k_mgs(V* w, const V* __restrict__ up, const double* __restrict__ beta_prev, const V* uj, int self,
      size_t n, double* part, unsigned int* count, double* out, const int* __restrict__ skip) {
    // self != 0 when uj is w itself (the last step of solmfg.f:247-267 forms w.w)
    __shared__ double sh[32];
    if (skip && *skip) return;
    using X = Vec16<V>;
    using T = typename X::T;
    const double bp = up ? *beta_prev : 0.0;
    const V bv = (V)bp;
    DotAcc<V> acc;
    const bool vec = al16(w) && al16(up) && al16(uj);
    const size_t nv = vec ? n / X::W : 0, t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    T* wv = reinterpret_cast<T*>(w);
    const T* upv = reinterpret_cast<const T*>(up);
    const T* ujv = reinterpret_cast<const T*>(uj);
    // one element of this thread's stride: update w, add its product to the dot
    auto step = [&](size_t i, T wi, const T& ui, const T& ji) {
        if (up) {
#pragma unroll
            for (int k = 0; k < X::W; ++k) X::set(wi, k, X::at(wi, k) - bv * X::at(ui, k));
            wv[i] = wi;
        }
        const T u2 = self ? wi : ji;
#pragma unroll
        for (int k = 0; k < X::W; ++k) acc.add(X::at(wi, k), X::at(u2, k));
    };
    // two strides per pass, every load of both issued before the first store (the store to w
    // would otherwise hold back the next loads); the order of the updates and of the dot's
    // additions is the one-stride loop's
    size_t i = t0;
    for (; i + stride < nv; i += 2 * stride) {
        const T wa = wv[i], wb = wv[i + stride];
        T ua{}, ub{}, ja{}, jb{};
        if (up) {
            ua = upv[i];
            ub = upv[i + stride];
        }
        if (!self) {
            ja = ujv[i];
            jb = ujv[i + stride];
        }
        step(i, wa, ua, ja);
        step(i + stride, wb, ub, jb);
    }
    for (; i < nv; i += stride) {
        T ui{}, ji{};
        if (up) ui = upv[i];
        if (!self) ji = ujv[i];
        step(i, wv[i], ui, ji);
    }
    for (size_t i = X::W * nv + t0; i < n; i += stride) {
        V wi = w[i];
        if (up) {
            wi = wi - bv * up[i];
            w[i] = wi;
        }
        const V ui = self ? wi : uj[i];
        acc.add(wi, ui);
    }
    const double bs = block_sum(acc.value(), sh);
    __syncthreads();
    finish_reduce(bs, part, count, out, sh);
}

// mode 0: w *= 1/s ; mode 1: w *= 1/sqrt(s)
template <typename V>
__global__ void k_scale(V* __restrict__ w, const double* __restrict__ s, int mode, size_t n,
                        const int* __restrict__ skip) {
    if (skip && *skip) return;
    using X = Vec16<V>;
    using T = typename X::T;
    const double d = mode ? sqrt(*s) : *s;
    const V f = (V)(1.0 / d);
    const size_t nv = al16(w) ? n / X::W : 0, t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    T* wv = reinterpret_cast<T*>(w);
    for (size_t i = t0; i < nv; i += stride) {
        T x = wv[i];
#pragma unroll
        for (int k = 0; k < X::W; ++k) X::set(x, k, X::at(x, k) * f);
        wv[i] = x;
    }
    for (size_t i = X::W * nv + t0; i < n; i += stride) w[i] = w[i] * f;
}

}  // namespace

// ============================ host wrappers ============================
template <typename R>
void bc3res(Ctx& C, R* r) {
    if (C.nbcn > 0) {
        k_bc3res<R><<<nblocks(C.nbcn), kT, 0, C.stream>>>(C.d_bcn, C.nbcn, C.d_iBC, C.d_BC, r, C.cfg.Rgas);
        ++C.launches;
    }
    if (C.nmaster > 0) {
        k_periodic_sum<R, 5><<<nblocks(C.nmaster), kT, 0, C.stream>>>(C.d_mst, C.d_slv_start, C.d_slv, C.nmaster, r, 0);
        ++C.launches;
    }
}
template void bc3res<double>(Ctx&, double*);
template void bc3res<float>(Ctx&, float*);

// bc3per (bc3per.f:1-20): the periodic part of bc3Res alone
template <typename R>
void bc3per(Ctx& C, R* r) {
    if (C.nmaster > 0) {
        k_periodic_sum<R, 5><<<nblocks(C.nmaster), kT, 0, C.stream>>>(C.d_mst, C.d_slv_start, C.d_slv, C.nmaster, r, 0);
        ++C.launches;
    }
}
template void bc3per<double>(Ctx&, double*);
template void bc3per<float>(Ctx&, float*);

template <typename R>
void bc3bdg(Ctx& C, const double* y, R* bd) {
    if (C.nbcn > 0) {
        k_bc3bdg<R><<<nblocks(C.nbcn), kT, 0, C.stream>>>(C.d_bcn, C.nbcn, C.d_iBC, C.d_BC, y, bd,
                                                           C.cfg.Rgas * C.cfg.gamma / C.cfg.gamma1);
        ++C.launches;
    }
    if (C.nmaster > 0) {
        k_periodic_sum<R, 25><<<nblocks(C.nmaster), kT, 0, C.stream>>>(C.d_mst, C.d_slv_start, C.d_slv, C.nmaster, bd, 1);
        ++C.launches;
    }
}
template void bc3bdg<double>(Ctx&, const double*, double*);
template void bc3bdg<float>(Ctx&, const double*, float*);

template <typename R>
void itrbc_pert(Ctx& C, R* v, bool linear) {
    if (C.nbcn > 0) {
        k_itrbc<R><<<nblocks(C.nbcn), kT, 0, C.stream>>>(C.d_bcn, C.nbcn, C.d_iBC, C.d_BC, v, linear ? 1 : 0, C.cfg.Rgas);
        ++C.launches;
    }
    if (C.nslave > 0) {
        k_periodic_copy<R><<<nblocks(C.nslave), kT, 0, C.stream>>>(C.d_slaves, C.nslave, C.d_iper, v);
        ++C.launches;
    }
}
template void itrbc_pert<double>(Ctx&, double*, bool);
template void itrbc_pert<float>(Ctx&, float*, bool);

void itrbc_state(Ctx& C, double* y, double* ac, bool with_ac) {
    itrbc_pert<double>(C, y, false);
    if (with_ac && ac && C.nslave > 0) {
        k_periodic_copy<double><<<nblocks(C.nslave), kT, 0, C.stream>>>(C.d_slaves, C.nslave, C.d_iper, ac);
        ++C.launches;
    }
}

template <typename R>
void lu_fact(Ctx& C, R* bd, int* flag) {
    k_lu_fact<R, R><<<(C.N + kLuT - 1) / kLuT, kLuT, 0, C.stream>>>(bd, bd, nullptr, C.N, flag);
    ++C.launches;
}
template void lu_fact<double>(Ctx&, double*, int*);
template void lu_fact<float>(Ctx&, float*, int*);

void lu_fact_f32(Ctx& C, float* bdf, double* bd, int* flag) {
    k_lu_fact<double, float><<<(C.N + kLuT - 1) / kLuT, kLuT, 0, C.stream>>>(bdf, bd, bdf, C.N, flag);
    ++C.launches;
}

template <typename R, typename V>
void lu_apply(Ctx& C, const R* bd, V* r, int code) {
    k_lu_apply<R, V><<<nblocks(C.N), kT, 0, C.stream>>>(bd, r, r, C.N, code, nullptr);
    ++C.launches;
}
template <typename R, typename V>
void lu_apply(Ctx& C, const R* bd, const V* in, V* out, int code) {
    k_lu_apply<R, V><<<nblocks(C.N), kT, 0, C.stream>>>(bd, in, out, C.N, code, nullptr);
    ++C.launches;
}
template void lu_apply<double, double>(Ctx&, const double*, const double*, double*, int);
template void lu_apply<float, float>(Ctx&, const float*, const float*, float*, int);
template void lu_apply<double, double>(Ctx&, const double*, double*, int);
template void lu_apply<double, float>(Ctx&, const double*, float*, int);
template void lu_apply<float, float>(Ctx&, const float*, float*, int);

void ref_to_dev_state(Ctx& C, const double* h, double* d_tmp, double* d_out) {
    check(C, cudaMemcpyAsync(d_tmp, h, sizeof(double) * 5 * (size_t)C.N, cudaMemcpyHostToDevice, C.stream), "H2D state");
    k_state_in<<<nblocks(C.N), kT, 0, C.stream>>>(d_tmp, d_out, C.N);
    ++C.launches;
}
void dev_to_ref_state(Ctx& C, const double* d_in, double* d_tmp, double* h) {
    k_state_out<<<nblocks(C.N), kT, 0, C.stream>>>(d_in, d_tmp, C.N);
    ++C.launches;
    check(C, cudaMemcpyAsync(h, d_tmp, sizeof(double) * 5 * (size_t)C.N, cudaMemcpyDeviceToHost, C.stream), "D2H state");
}
void ref_to_dev_res(Ctx& C, const double* h, double* d_tmp, double* d_out) {
    check(C, cudaMemcpyAsync(d_tmp, h, sizeof(double) * 5 * (size_t)C.N, cudaMemcpyHostToDevice, C.stream), "H2D vec");
    k_soa_to_aos<5><<<nblocks(C.N), kT, 0, C.stream>>>(d_tmp, d_out, C.N);
    ++C.launches;
}
void dev_to_ref_res(Ctx& C, const double* d_in, double* d_tmp, double* h) {
    k_aos_to_soa<5><<<nblocks(C.N), kT, 0, C.stream>>>(d_in, d_tmp, C.N);
    ++C.launches;
    check(C, cudaMemcpyAsync(h, d_tmp, sizeof(double) * 5 * (size_t)C.N, cudaMemcpyDeviceToHost, C.stream), "D2H vec");
}
void ref_to_dev_bd(Ctx& C, const double* h, double* d_tmp, double* d_out) {
    check(C, cudaMemcpyAsync(d_tmp, h, sizeof(double) * 25 * (size_t)C.N, cudaMemcpyHostToDevice, C.stream), "H2D bd");
    k_bd_in<<<nblocks(C.N), kT, 0, C.stream>>>(d_tmp, d_out, C.N);
    ++C.launches;
}
void dev_to_ref_bd(Ctx& C, const double* d_in, double* d_tmp, double* h) {
    k_bd_out<<<nblocks(C.N), kT, 0, C.stream>>>(d_in, d_tmp, C.N);
    ++C.launches;
    check(C, cudaMemcpyAsync(h, d_tmp, sizeof(double) * 25 * (size_t)C.N, cudaMemcpyDeviceToHost, C.stream), "D2H bd");
}
void to_f32(Ctx& C, const double* a, float* b, size_t n) {
    k_convert<double, float><<<kRedBlocks, kT, 0, C.stream>>>(a, b, n);
    ++C.launches;
}
__global__ void k_split(const double* __restrict__ a, float* __restrict__ hi, float* __restrict__ lo, size_t n) {
    const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    // four entries per thread and pass with 16-byte loads and stores when all three arrays allow
    const size_t n4 = (((uintptr_t)a | (uintptr_t)hi | (uintptr_t)lo) & 15) == 0 ? n / 4 : 0;
    for (size_t i = t0; i < n4; i += stride) {
        const double2 p = reinterpret_cast<const double2*>(a)[2 * i], q = reinterpret_cast<const double2*>(a)[2 * i + 1];
        const double v[4] = {p.x, p.y, q.x, q.y};
        float h[4], l[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            h[k] = (float)v[k];
            l[k] = (float)(v[k] - (double)h[k]);
        }
        reinterpret_cast<float4*>(hi)[i] = make_float4(h[0], h[1], h[2], h[3]);
        reinterpret_cast<float4*>(lo)[i] = make_float4(l[0], l[1], l[2], l[3]);
    }
    for (size_t i = 4 * n4 + t0; i < n; i += stride) {
        const double v = a[i];
        const float h = (float)v;
        hi[i] = h;
        lo[i] = (float)(v - (double)h);
    }
}
// qpbc.f: 1/rmass scaling of the 12 flux values of each node (the 13th value is the mass)
template <typename R>
__global__ void k_qscale(R* __restrict__ q, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    R* v = q + 13 * (size_t)i;
    const R r = R(1) / v[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) v[k] = r * v[k];
}
template <typename R>
void qpbc(Ctx& C, R* q13) {
    // periodic slaves summed into their master, the master's values copied back (qpbc.f)
    if (C.nmaster > 0) {
        k_periodic_sum<R, 13><<<nblocks(C.nmaster), kT, 0, C.stream>>>(C.d_mst, C.d_slv_start, C.d_slv, C.nmaster,
                                                                       q13, 1);
        ++C.launches;
    }
    k_qscale<R><<<nblocks(C.N), kT, 0, C.stream>>>(q13, C.N);
    ++C.launches;
}
template void qpbc<double>(Ctx&, double*);
template void qpbc<float>(Ctx&, float*);

void split_f32(Ctx& C, const double* a, float* hi, float* lo, size_t n) {
    k_split<<<kRedBlocks, kT, 0, C.stream>>>(a, hi, lo, n);
    ++C.launches;
}
void to_f64(Ctx& C, const float* a, double* b, size_t n) {
    k_convert<float, double><<<kRedBlocks, kT, 0, C.stream>>>(a, b, n);
    ++C.launches;
}
void fill0(Ctx& C, void* p, size_t bytes) {
    check(C, cudaMemsetAsync(p, 0, bytes, C.stream), "memset");
}

template <typename V>
void dot(Ctx& C, const V* a, const V* b, size_t n, int slot, const int* skip) {
    k_dot<V><<<kRedBlocks, kRedThreads, 0, C.stream>>>(a, b, n, C.d_part, C.d_count, C.d_scal + slot, skip);
    ++C.launches;
}
template void dot<double>(Ctx&, const double*, const double*, size_t, int, const int*);
template void dot<float>(Ctx&, const float*, const float*, size_t, int, const int*);

template <typename V>
void mgs_step(Ctx& C, V* w, const V* uprev, const double* beta_prev, const V* uj, size_t n, double* beta_out,
              const int* skip) {
    k_mgs<V><<<kRedBlocks, kRedThreads, 0, C.stream>>>(w, uprev, beta_prev, uj, uj == w ? 1 : 0, n, C.d_part,
                                                        C.d_count, beta_out, skip);
    ++C.launches;
}
template void mgs_step<double>(Ctx&, double*, const double*, const double*, const double*, size_t, double*, const int*);
template void mgs_step<float>(Ctx&, float*, const float*, const double*, const float*, size_t, double*, const int*);

template <typename V>
void scale_by(Ctx& C, V* w, const double* s, int mode, size_t n, const int* skip) {
    k_scale<V><<<kRedBlocks, kT, 0, C.stream>>>(w, s, mode, n, skip);
    ++C.launches;
}
template void scale_by<double>(Ctx&, double*, const double*, int, size_t, const int*);
template void scale_by<float>(Ctx&, float*, const double*, int, size_t, const int*);

}  // namespace phgpu
