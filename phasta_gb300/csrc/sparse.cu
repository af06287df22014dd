// sparse.cu -- the block-sparse side of the sparse solver (impl = 1x, lhs = 1):
//   * the node adjacency of genadj.f/asadj.f (host; rows sorted ascending),
//   * per-element block maps replacing fillsparseC's sparseloc search
//     (fillsparse.f) by one host-side search at set-up,
//   * Spsi3pre (spsi3pre.f): lhsK(i,j) <- L_i^-1 lhsK(i,j) U_j^-1,
//   * SparseAp (sparseap.f) with the periodic gather and bc3per (bc3per.f).
//
// lhsK lives in the reference's layout, lhsK(25, nnz_tot) column-major: block
// k is 25 contiguous values with entry (f, g) at 5 g + f, blocks of a row are
// contiguous and ordered by column node.  The product gives each (row,
// equation) pair one thread, which reads its five entries of every block of the
// row and gathers p through the iper-mapped column list.
#include <algorithm>

#include "phgpu_impl.cuh"

namespace phgpu {

void block_adjacency(int N, const int* ien, int ne, const int* ienh, int nh, const int* ienw, int nw,
                     std::vector<int>& colm, std::vector<int>& rowp) {
    // node -> incident elements (all blocks), then each row = sorted unique nodes of those elements
    struct Blk { const int* ien; int nen, ne; };
    const Blk blks[3] = {{ien, 4, ne}, {ienh, 8, nh}, {ienw, 6, nw}};
    std::vector<int> deg(N + 1, 0);
    for (const Blk& b : blks)
        for (size_t i = 0; i < (size_t)b.nen * b.ne; ++i) deg[b.ien[i] + 1]++;
    for (int n = 0; n < N; ++n) deg[n + 1] += deg[n];
    std::vector<long long> inc(deg[N]);  // (block << 40) | element
    std::vector<int> fillp(deg.begin(), deg.end() - 1);
    for (int bi = 0; bi < 3; ++bi) {
        const Blk& b = blks[bi];
        for (int e = 0; e < b.ne; ++e)
            for (int a = 0; a < b.nen; ++a) inc[fillp[b.ien[(size_t)b.nen * e + a]]++] = ((long long)bi << 40) | e;
    }
    colm.assign(N + 1, 1);
    rowp.clear();
    std::vector<int> row;
    for (int n = 0; n < N; ++n) {
        row.clear();
        for (int t = deg[n]; t < deg[n + 1]; ++t) {
            const Blk& b = blks[inc[t] >> 40];
            const int e = (int)(inc[t] & ((1ll << 40) - 1));
            for (int a = 0; a < b.nen; ++a) row.push_back(b.ien[(size_t)b.nen * e + a]);
        }
        std::sort(row.begin(), row.end());
        row.erase(std::unique(row.begin(), row.end()), row.end());
        for (int v : row) rowp.push_back(v + 1);
        colm[n + 1] = colm[n] + (int)row.size();
    }
}

namespace {

template <typename T>
int dcopy(Ctx& C, T** d, const T* h, size_t n) {
    if (cudaMalloc((void**)d, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
        C.err = "cudaMalloc (sparse tangent)";
        return PHGPU_ERR_NOMEM;
    }
    if (n == 0) return PHGPU_OK;
    return h2d(C, *d, h, sizeof(T) * n, "upload sparse structure");
}

// block index of (element, a, b) for every element of a block (element-major, a-major)
void block_map(const std::vector<int>& colm, const std::vector<int>& rowp, const int* ien, int nen, int ne,
               std::vector<int>& map) {
    map.resize((size_t)nen * nen * ne);
    for (int e = 0; e < ne; ++e)
        for (int a = 0; a < nen; ++a) {
            const int i = ien[(size_t)nen * e + a];
            const int* r0 = rowp.data() + (colm[i] - 1);
            const int* r1 = rowp.data() + (colm[i + 1] - 1);
            for (int b = 0; b < nen; ++b) {
                const int* f = std::lower_bound(r0, r1, ien[(size_t)nen * e + b] + 1);
                map[((size_t)e * nen + a) * nen + b] = (int)(f - rowp.data());
            }
        }
}

// L_i^-1 a U_j^-1 for one 5x5 block a (a[5 g + f] = entry (f, g)) with the i3LU factors of
// its row node (Li) and column node (Uj), row-major: Li[5 r + c] = BDiag(i, r, c)
template <typename R>
__device__ __forceinline__ void precondition_block(R* __restrict__ a, const R* __restrict__ Li,
                                                   const R* __restrict__ Uj) {
    R m[5][5];
#pragma unroll
    for (int g = 0; g < 5; ++g)
#pragma unroll
        for (int f = 0; f < 5; ++f) m[f][g] = a[5 * g + f];
    // forward substitution with the unit lower factor of row node i, column by column
#pragma unroll
    for (int r = 1; r < 5; ++r)
#pragma unroll
        for (int g = 0; g < 5; ++g) {
            R v = m[r][g];
#pragma unroll
            for (int c = 0; c < r; ++c) v = v - Li[5 * r + c] * m[c][g];
            m[r][g] = v;
        }
    // right solve with the upper factor of column node j (reciprocal pivots on its diagonal)
#pragma unroll
    for (int g = 0; g < 5; ++g)
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            R v = m[f][g];
#pragma unroll
            for (int c = 0; c < g; ++c) v = v - Uj[5 * c + g] * m[f][c];
            m[f][g] = Uj[5 * g + g] * v;
        }
#pragma unroll
    for (int g = 0; g < 5; ++g)
#pragma unroll
        for (int f = 0; f < 5; ++f) a[5 * g + f] = m[f][g];
}

// ---- Spsi3pre: one thread per block ----
template <typename R>
__global__ void k_spsi3pre(const int* __restrict__ brow, const int* __restrict__ bcol, const R* __restrict__ bd,
                           R* __restrict__ A, int nnzb) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnzb) return;
    precondition_block(A + 25 * (size_t)k, bd + 25 * (size_t)brow[k], bd + 25 * (size_t)bcol[k]);
}

// ---- i3pre (i3pre.f): the same transform on every block (a, b) of the stored element tangents ----
template <typename R, int NEN>
__global__ void k_i3pre(const int* __restrict__ ien, const R* __restrict__ bd, R* __restrict__ EG, int ne) {
    constexpr int NB = NEN * NEN;
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)ne * NB) return;
    const size_t e = t / NB;
    const int ab = (int)(t - e * NB), a = ab / NEN, b = ab - NEN * (ab / NEN);
    const int* nd = ien + (size_t)NEN * e;
    precondition_block(EG + 25 * t, bd + 25 * (size_t)nd[a], bd + 25 * (size_t)nd[b]);
}

// ---- Au1GMR (au1gmr.f, asaugmr.f): one thread per (element, node a, equation f) ----
// q(node a, f) += sum_b sum_g EG_e(a, b)(f, g) p(iper(node b), g); elements of one colour share no node
template <typename M, typename V, int NEN>
__global__ void k_ebe_ap(const int* __restrict__ ien, const M* __restrict__ EG, const int* __restrict__ iper,
                         const V* __restrict__ p, V* __restrict__ q, int ne) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)ne * 5 * NEN) return;
    const size_t e = t / (5 * NEN);
    const int r = (int)(t - e * 5 * NEN), a = r / 5, f = r - 5 * (r / 5);
    const int* nd = ien + (size_t)NEN * e;
    const M* blk = EG + 25 * ((size_t)e * NEN + a) * NEN + f;
    V acc = V(0);
#pragma unroll
    for (int b = 0; b < NEN; ++b) {
        const V* pb = p + 5 * (size_t)iper[nd[b]];
        const M* m = blk + 25 * b;
        acc += (V)m[0] * pb[0] + (V)m[5] * pb[1] + (V)m[10] * pb[2] + (V)m[15] * pb[3] + (V)m[20] * pb[4];
    }
    V* o = q + 5 * (size_t)nd[a] + f;
    *o = *o + acc;
}

// ---- SparseAp: one thread per (block row, equation) ----
// Thread (i, f) forms q(i, f) = sum_k sum_g lhsK(k)(f, g) p(iper(col k), g) over the blocks
// of row i: five strided values of each block (the row's segment is read in full by its
// five threads), one gathered node of p, and no reduction across threads.
constexpr int kSpThreads = 160;  // 32 block rows

template <typename M, typename V>
__global__ void __launch_bounds__(kSpThreads)
k_bsr_spmv(const int* __restrict__ rs, const int* __restrict__ bcolp, const M* __restrict__ A,
           const V* __restrict__ p, V* __restrict__ q, int N) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = t / 5, f = t - 5 * (t / 5);
    if (row >= N) return;
    const int k0 = rs[row], k1 = rs[row + 1];
    V acc = V(0);
#pragma unroll 2
    for (int k = k0; k < k1; ++k) {
        const M* a = A + 25 * (size_t)k + f;
        const V* pj = p + 5 * (size_t)bcolp[k];
        acc += (V)a[0] * pj[0] + (V)a[5] * pj[1] + (V)a[10] * pj[2] + (V)a[15] * pj[3] + (V)a[20] * pj[4];
    }
    q[5 * (size_t)row + f] = acc;
}

}  // namespace

// the element colouring of the tet tangent, the tables and kernel attributes (both solvers)
static int tangent_setup(Ctx& C) {
    SparseCtx& S = C.sp;
    if (S.tan_ready) return PHGPU_OK;
    std::vector<int> tien(4 * (size_t)C.E);
    if (C.E > 0) {
        // tets: their own colouring (the chunk order of the residual kernels groups elements that share nodes)
        const int rcc = colour(C, C.N, C.h_ien.data(), 4, C.E, S.torder, S.tcol_start);
        if (rcc != PHGPU_OK) return rcc;
        for (int i = 0; i < C.E; ++i)
            for (int a = 0; a < 4; ++a) tien[4 * (size_t)i + a] = C.h_ien[4 * (size_t)S.torder[i] + a];
    }
    S.h_ient = tien;
    int rc = dcopy(C, &S.d_ient, tien.data(), tien.size());
    if (rc == PHGPU_OK) rc = upload_tangent_tables(C);
    if (rc == PHGPU_OK) rc = configure_tangent_kernels(C);
    if (rc == PHGPU_OK) S.tan_ready = true;
    return rc;
}

// the FP32 tangent is allocated the first time a mixed-precision solve needs it
static int ensure_f32(Ctx& C) {
    SparseCtx& S = C.sp;
    if (C.cfg.precision != PHGPU_MIXED || S.d_lhsKf) return PHGPU_OK;
    if (cudaMalloc((void**)&S.d_lhsKf, sizeof(float) * 25 * (size_t)std::max(S.nnzb, 1)) != cudaSuccess) {
        C.err = "cudaMalloc (FP32 sparse tangent)";
        return PHGPU_ERR_NOMEM;
    }
    return PHGPU_OK;
}

int sparse_setup(Ctx& C) {
    SparseCtx& S = C.sp;
    if (S.ready) return ensure_f32(C);
    const int N = C.N;
    {
        const int rct = tangent_setup(C);
        if (rct != PHGPU_OK) return rct;
    }
    block_adjacency(N, C.h_ien.data(), C.E, C.h_ienh.data(), C.nhex, C.h_ienw.data(), C.nwedge, S.colm, S.rowp);
    S.nnzb = (int)S.rowp.size();
    std::vector<int> rs(N + 1), bcol(S.nnzb), bcolp(S.nnzb), brow(S.nnzb);
    std::vector<int> iper(N);
    {
        const int rci = d2h(C, iper.data(), C.d_iper, sizeof(int) * N, "download iper");
        if (rci != PHGPU_OK) return rci;
    }
    for (int n = 0; n <= N; ++n) rs[n] = S.colm[n] - 1;
    for (int n = 0; n < N; ++n)
        for (int k = rs[n]; k < rs[n + 1]; ++k) {
            brow[k] = n;
            bcol[k] = S.rowp[k] - 1;
            bcolp[k] = iper[bcol[k]];
        }
    std::vector<int> tmap, hmap, wmap;
    if (C.E > 0) block_map(S.colm, S.rowp, S.h_ient.data(), 4, C.E, tmap);
    if (C.nhex > 0) block_map(S.colm, S.rowp, C.h_ienh.data(), 8, C.nhex, hmap);
    if (C.nwedge > 0) block_map(S.colm, S.rowp, C.h_ienw.data(), 6, C.nwedge, wmap);
    int rc = PHGPU_OK;
    auto T = [&](int s) { if (rc == PHGPU_OK) rc = s; };
    T(dcopy(C, &S.d_rs, rs.data(), rs.size()));
    T(dcopy(C, &S.d_bcol, bcol.data(), bcol.size()));
    T(dcopy(C, &S.d_bcolp, bcolp.data(), bcolp.size()));
    T(dcopy(C, &S.d_brow, brow.data(), brow.size()));
    T(dcopy(C, &S.d_tmap, tmap.data(), tmap.size()));
    T(dcopy(C, &S.d_hmap, hmap.data(), hmap.size()));
    T(dcopy(C, &S.d_wmap, wmap.data(), wmap.size()));
    if (rc == PHGPU_OK && cudaMalloc((void**)&S.d_lhsK, sizeof(double) * 25 * (size_t)std::max(S.nnzb, 1)) != cudaSuccess)
        rc = PHGPU_ERR_NOMEM;
    if (rc == PHGPU_OK) rc = ensure_f32(C);
    if (rc == PHGPU_OK) rc = check(C, cudaStreamSynchronize(C.stream), "sparse set-up");
    if (rc != PHGPU_OK) {
        if (C.err.empty()) C.err = "sparse set-up failed";
        return rc;
    }
    S.ready = true;
    return PHGPU_OK;
}

int ebe_setup(Ctx& C) {
    SparseCtx& S = C.sp;
    if ((C.E > 0) + (C.nhex > 0) + (C.nwedge > 0) != 1) {
        C.err = "the element-by-element solver needs a mesh of one element topology (i3pre.f gathers the block "
                "diagonal through a section of the largest element's size)";
        return PHGPU_ERR_UNSUPPORTED;
    }
    const int rct = tangent_setup(C);
    if (rct != PHGPU_OK) return rct;
    S.eg_blocks = 16 * (size_t)C.E + 64 * (size_t)C.nhex + 36 * (size_t)C.nwedge;
    const bool f64 = C.cfg.precision == PHGPU_FP64;
    if (f64 && !S.d_EG && cudaMalloc((void**)&S.d_EG, sizeof(double) * 25 * S.eg_blocks) != cudaSuccess) {
        C.err = "cudaMalloc (element tangents)";
        return PHGPU_ERR_NOMEM;
    }
    if (!f64 && !S.d_EGf && cudaMalloc((void**)&S.d_EGf, sizeof(float) * 25 * S.eg_blocks) != cudaSuccess) {
        C.err = "cudaMalloc (FP32 element tangents)";
        return PHGPU_ERR_NOMEM;
    }
    return check(C, cudaStreamSynchronize(C.stream), "element-by-element set-up");
}

template <typename R>
void spsi3pre(Ctx& C, const R* bd, R* lhsK) {
    const int n = C.sp.nnzb;
    if (n == 0) return;
    k_spsi3pre<R><<<(n + 127) / 128, 128, 0, C.stream>>>(C.sp.d_brow, C.sp.d_bcol, bd, lhsK, n);
    ++C.launches;
}
template void spsi3pre<double>(Ctx&, const double*, double*);
template void spsi3pre<float>(Ctx&, const float*, float*);

template <typename M, typename V>
void sparse_ap(Ctx& C, const M* lhsK, const V* p, V* q) {
    const int N = C.N;
    const size_t threads = 5 * (size_t)N;
    k_bsr_spmv<M, V><<<(unsigned)((threads + kSpThreads - 1) / kSpThreads), kSpThreads, 0, C.stream>>>(
        C.sp.d_rs, C.sp.d_bcolp, lhsK, p, q, N);
    ++C.launches;
    bc3per<V>(C, q);
}
template void sparse_ap<double, double>(Ctx&, const double*, const double*, double*);
template void sparse_ap<float, float>(Ctx&, const float*, const float*, float*);

// the element blocks of the element-by-element storage: connectivity, colours, first block
struct EbeBlock {
    const int* ien;
    const std::vector<int>* col;
    int nen, ne;
    size_t blk0;
};
static int ebe_blocks(const Ctx& C, EbeBlock* out) {
    int n = 0;
    if (C.E > 0) out[n++] = {C.sp.d_ient, &C.sp.tcol_start, 4, C.E, 0};
    if (C.nhex > 0) out[n++] = {C.d_ienh, &C.hcol_start, 8, C.nhex, 16 * (size_t)C.E};
    if (C.nwedge > 0) out[n++] = {C.d_ienw, &C.wcol_start, 6, C.nwedge, 16 * (size_t)C.E + 64 * (size_t)C.nhex};
    return n;
}

template <typename R>
void i3pre(Ctx& C, const R* bd, R* EG) {
    EbeBlock b[3];
    const int nb = ebe_blocks(C, b);
    for (int i = 0; i < nb; ++i) {
        const size_t nt = (size_t)b[i].ne * b[i].nen * b[i].nen;
        const unsigned grid = (unsigned)((nt + 127) / 128);
        R* eg = EG + 25 * b[i].blk0;
        if (b[i].nen == 4) k_i3pre<R, 4><<<grid, 128, 0, C.stream>>>(b[i].ien, bd, eg, b[i].ne);
        else if (b[i].nen == 8) k_i3pre<R, 8><<<grid, 128, 0, C.stream>>>(b[i].ien, bd, eg, b[i].ne);
        else k_i3pre<R, 6><<<grid, 128, 0, C.stream>>>(b[i].ien, bd, eg, b[i].ne);
        ++C.launches;
    }
}
template void i3pre<double>(Ctx&, const double*, double*);
template void i3pre<float>(Ctx&, const float*, float*);

template <typename M, typename V>
void ebe_ap(Ctx& C, const M* EG, const V* p, V* q) {
    fill0(C, q, sizeof(V) * 5 * (size_t)C.N);
    EbeBlock b[3];
    const int nb = ebe_blocks(C, b);
    for (int i = 0; i < nb; ++i) {
        const int NEN = b[i].nen;
        const std::vector<int>& col = *b[i].col;
        for (size_t c = 0; c + 1 < col.size(); ++c) {
            const int e0 = col[c], ne = col[c + 1] - e0;
            if (ne <= 0) continue;
            const size_t nt = (size_t)ne * 5 * NEN;
            const unsigned grid = (unsigned)((nt + 159) / 160);
            const int* ie = b[i].ien + (size_t)NEN * e0;
            const M* eg = EG + 25 * (b[i].blk0 + (size_t)NEN * NEN * e0);
            if (NEN == 4) k_ebe_ap<M, V, 4><<<grid, 160, 0, C.stream>>>(ie, eg, C.d_iper, p, q, ne);
            else if (NEN == 8) k_ebe_ap<M, V, 8><<<grid, 160, 0, C.stream>>>(ie, eg, C.d_iper, p, q, ne);
            else k_ebe_ap<M, V, 6><<<grid, 160, 0, C.stream>>>(ie, eg, C.d_iper, p, q, ne);
            ++C.launches;
        }
    }
    bc3per<V>(C, q);
}
template void ebe_ap<double, double>(Ctx&, const double*, const double*, double*);
template void ebe_ap<float, float>(Ctx&, const float*, const float*, float*);

}  // namespace phgpu
