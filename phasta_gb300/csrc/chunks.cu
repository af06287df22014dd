// chunks.cu -- host preprocessing of the element loop.
//
// Elements are ordered along a Morton (Z-order) curve of their centroids and
// cut into chunks of at most kChunk consecutive elements, so a chunk is a
// compact piece of the mesh.  For every chunk we store
//   * its distinct nodes (ascending global ids)              -> staged in shared memory
//   * each element's four local node indices (uint16)         -> gathers from shared memory
//   * for every local node, the (element, corner) slots that
//     touch it, in ascending order                            -> deterministic per-node sums
// Chunks sharing a node get different colours (greedy first fit over the
// chunk order); chunks of one colour run concurrently, colours run in
// sequence, so the global read-modify-write of a node is never concurrent.
// This replaces the per-element colouring of the reference's serial scatter
// (local.f:66-80) with one launch per chunk colour.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <queue>
#include <tuple>
#include <type_traits>

#include "phgpu_impl.cuh"

namespace phgpu {

namespace {
inline uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}
}  // namespace

int build_chunks(Ctx& C, const int* ien, const double* x_ref) {
    const int N = C.N, E = C.E;
    // Morton keys of element centroids
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int n = 0; n < N; ++n)
        for (int d = 0; d < 3; ++d) {
            const double v = x_ref[(size_t)d * N + n];
            lo[d] = std::min(lo[d], v);
            hi[d] = std::max(hi[d], v);
        }
    std::vector<std::pair<uint64_t, int>> key(E);
    const double scale = (double)((1u << 21) - 1);
    for (int e = 0; e < E; ++e) {
        uint64_t k = 0;
        for (int d = 0; d < 3; ++d) {
            double c = 0.0;
            for (int a = 0; a < 4; ++a) c += x_ref[(size_t)d * N + ien[4 * (size_t)e + a]];
            c *= 0.25;
            const double span = hi[d] - lo[d];
            const double t = span > 0 ? (c - lo[d]) / span : 0.0;
            const uint64_t q = (uint64_t)std::min(scale, std::max(0.0, t * scale));
            k |= spread3(q) << d;
        }
        key[e] = {k, e};
    }
    std::sort(key.begin(), key.end());
    const int nch = (E + kChunk - 1) / kChunk;
    // nodes and slots of every chunk
    std::vector<int> cnode_start(nch + 1, 0), cnodes;
    cnodes.reserve((size_t)E);  // typical: ~0.5 node per element
    std::vector<int> local(N, -1);
    std::vector<ushort4> lien_m(E);  // in Morton order
    std::vector<int> csr_start_m;    // per chunk-local node (global running index)
    std::vector<uint16_t> csr_m;
    csr_start_m.reserve((size_t)E + 1);
    csr_m.reserve(4 * (size_t)E);
    csr_start_m.push_back(0);
    std::vector<int> tmp;
    int lmax = 0;
    for (int c = 0; c < nch; ++c) {
        const int e0 = c * kChunk, e1 = std::min(E, e0 + kChunk);
        tmp.clear();
        for (int i = e0; i < e1; ++i)
            for (int a = 0; a < 4; ++a) tmp.push_back(ien[4 * (size_t)key[i].second + a]);
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
        const int nn = (int)tmp.size();
        lmax = std::max(lmax, nn);
        for (int l = 0; l < nn; ++l) local[tmp[l]] = l;
        cnode_start[c] = (int)cnodes.size();
        cnodes.insert(cnodes.end(), tmp.begin(), tmp.end());
        std::vector<int> cnt(nn + 1, 0);
        for (int i = e0; i < e1; ++i) {
            const int* nd = ien + 4 * (size_t)key[i].second;
            ushort4 u;
            u.x = (unsigned short)local[nd[0]];
            u.y = (unsigned short)local[nd[1]];
            u.z = (unsigned short)local[nd[2]];
            u.w = (unsigned short)local[nd[3]];
            lien_m[i] = u;
            for (int a = 0; a < 4; ++a) cnt[local[nd[a]] + 1]++;
        }
        for (int l = 0; l < nn; ++l) cnt[l + 1] += cnt[l];
        const size_t base = csr_m.size();
        csr_m.resize(base + cnt[nn]);
        std::vector<int> pos(cnt.begin(), cnt.end() - 1);
        for (int i = e0; i < e1; ++i) {  // ascending (element, corner) order
            const int* nd = ien + 4 * (size_t)key[i].second;
            for (int a = 0; a < 4; ++a) csr_m[base + pos[local[nd[a]]]++] = (uint16_t)((i - e0) * 4 + a);
        }
        for (int l = 0; l < nn; ++l) csr_start_m.push_back((int)base + cnt[l + 1]);
        for (int l = 0; l < nn; ++l) local[tmp[l]] = -1;
    }
    cnode_start[nch] = (int)cnodes.size();
    // DSatur colouring of the chunks (chunks that share a node conflict; Brelaz 1979): the chunk
    // with the most distinct colours among its neighbours next, ties by degree, then by chunk
    // number; each takes the smallest free colour.  Fewer and more even colours than first fit
    // in Morton order (13 against 17 at 64^3 x 6, the smallest colour 74 chunks against 1), so
    // fewer launches and tails per sweep; deterministic.
    std::vector<int> nch_start(N + 1, 0);
    for (int j = 0; j < cnode_start[nch]; ++j) nch_start[cnodes[j] + 1]++;
    for (int n = 0; n < N; ++n) nch_start[n + 1] += nch_start[n];
    std::vector<int> nch_list(cnode_start[nch]);
    {
        std::vector<int> pos(nch_start.begin(), nch_start.end() - 1);
        for (int c = 0; c < nch; ++c)
            for (int j = cnode_start[c]; j < cnode_start[c + 1]; ++j) nch_list[pos[cnodes[j]]++] = c;
    }
    std::vector<int64_t> adj_start(nch + 1, 0);
    std::vector<int> adj;
    adj.reserve((size_t)nch * 32);
    for (int c = 0; c < nch; ++c) {
        const size_t b0 = adj.size();
        for (int j = cnode_start[c]; j < cnode_start[c + 1]; ++j) {
            const int n = cnodes[j];
            for (int k = nch_start[n]; k < nch_start[n + 1]; ++k)
                if (nch_list[k] != c) adj.push_back(nch_list[k]);
        }
        std::sort(adj.begin() + b0, adj.end());
        adj.erase(std::unique(adj.begin() + b0, adj.end()), adj.end());
        adj_start[c + 1] = (int64_t)adj.size();
    }
    std::vector<int> ccol(nch, -1), sat(nch, 0);
    std::vector<uint64_t> u0(nch, 0), u1(nch, 0);  // colours taken by a chunk's neighbours
    // (saturation, degree, -chunk): the largest first
    std::priority_queue<std::tuple<int, int, int>> pq;
    for (int c = 0; c < nch; ++c) pq.emplace(0, (int)(adj_start[c + 1] - adj_start[c]), -c);
    int ncol = 0;
    while (!pq.empty()) {
        const auto [sc, dc, nc] = pq.top();
        pq.pop();
        const int c = -nc;
        if (ccol[c] >= 0 || sc != sat[c]) continue;  // done, or an outdated entry
        int col;
        if (~u0[c]) col = __builtin_ctzll(~u0[c]);
        else if (~u1[c]) col = 64 + __builtin_ctzll(~u1[c]);
        else {
            C.err = "chunk colouring needs more than 128 colours";
            return PHGPU_ERR_UNSUPPORTED;
        }
        ccol[c] = col;
        ncol = std::max(ncol, col + 1);
        for (int64_t k = adj_start[c]; k < adj_start[c + 1]; ++k) {
            const int o = adj[k];
            if (ccol[o] >= 0) continue;
            uint64_t& w = col < 64 ? u0[o] : u1[o];
            const uint64_t bit = 1ull << (col & 63);
            if (w & bit) continue;
            w |= bit;
            ++sat[o];
            pq.emplace(sat[o], (int)(adj_start[o + 1] - adj_start[o]), -o);
        }
        (void)dc;
    }
    // no two chunks of a colour share a node: their node sums run concurrently without atomics
    {
        std::vector<int> last(N, -1);
        std::vector<int> by_col(nch);
        std::iota(by_col.begin(), by_col.end(), 0);
        std::stable_sort(by_col.begin(), by_col.end(), [&](int x, int y) { return ccol[x] < ccol[y]; });
        for (int c : by_col)
            for (int j = cnode_start[c]; j < cnode_start[c + 1]; ++j) {
                const int n = cnodes[j];
                if (last[n] == ccol[c]) {
                    C.err = "chunk colouring put two chunks that share a node in one colour";
                    return PHGPU_ERR_INVALID;
                }
                last[n] = ccol[c];
            }
    }
    // chunks sorted by colour (stable), elements follow their chunk
    std::vector<int> corder(nch);
    std::iota(corder.begin(), corder.end(), 0);
    std::stable_sort(corder.begin(), corder.end(), [&](int a, int b) { return ccol[a] < ccol[b]; });
    C.chunk_col_start.assign(ncol + 1, 0);
    for (int c = 0; c < nch; ++c) C.chunk_col_start[ccol[c] + 1]++;
    for (int k = 0; k < ncol; ++k) C.chunk_col_start[k + 1] += C.chunk_col_start[k];
    std::vector<int> elem_start(nch + 1, 0), node_start(nch + 1, 0), nodes, cstart;
    std::vector<ushort4> lien(E);
    std::vector<uint16_t> csr;
    std::vector<int4> ien_c(E);
    std::vector<int> perm(E);
    nodes.reserve(cnodes.size());
    csr.reserve(csr_m.size());
    cstart.reserve(cnodes.size() + 1);
    cstart.push_back(0);
    int ep = 0;
    for (int k = 0; k < nch; ++k) {
        const int c = corder[k];
        const int e0 = c * kChunk, e1 = std::min(E, e0 + kChunk);
        elem_start[k] = ep;
        for (int i = e0; i < e1; ++i) {
            lien[ep] = lien_m[i];
            const int* nd = ien + 4 * (size_t)key[i].second;
            ien_c[ep] = make_int4(nd[0], nd[1], nd[2], nd[3]);
            perm[ep] = key[i].second;
            ++ep;
        }
        node_start[k] = (int)nodes.size();
        for (int j = cnode_start[c]; j < cnode_start[c + 1]; ++j) {
            nodes.push_back(cnodes[j]);
            const int lo_ = csr_start_m[j], hi_ = csr_start_m[j + 1];
            csr.insert(csr.end(), csr_m.begin() + lo_, csr_m.begin() + hi_);
            cstart.push_back((int)csr.size());
        }
    }
    elem_start[nch] = ep;
    node_start[nch] = (int)nodes.size();
    // every shared-memory index the kernels form must be in range
    for (int k = 0; k < nch; ++k) {
        const int ne = elem_start[k + 1] - elem_start[k], nn = node_start[k + 1] - node_start[k];
        if (ne <= 0 || ne > kChunk || nn <= 0 || nn > lmax) {
            C.err = "chunk construction produced an out-of-range chunk";
            return PHGPU_ERR_INVALID;
        }
        // each element corner is in one slot list: chunk k's lists start at 4 * elem_start[k]
        // (the pipelined linearized product copies them from there)
        if (cstart[node_start[k]] != 4 * elem_start[k] || cstart[node_start[k + 1]] != 4 * elem_start[k + 1]) {
            C.err = "chunk construction produced misplaced slot lists";
            return PHGPU_ERR_INVALID;
        }
        for (int i = elem_start[k]; i < elem_start[k + 1]; ++i) {
            const ushort4 u = lien[i];
            if (u.x >= nn || u.y >= nn || u.z >= nn || u.w >= nn) {
                C.err = "chunk construction produced an out-of-range local node";
                return PHGPU_ERR_INVALID;
            }
        }
        for (int l = node_start[k]; l < node_start[k + 1]; ++l)
            for (int s = cstart[l]; s < cstart[l + 1]; ++s)
                if (csr[s] >= 4 * ne) {
                    C.err = "chunk construction produced an out-of-range slot";
                    return PHGPU_ERR_INVALID;
                }
    }
    C.nchunk = nch;
    C.chunk_lmax = lmax;
    C.perm_e = perm;
    auto up = [&](auto** d, const auto& v) -> int {
        using T = typename std::remove_reference<decltype(v)>::type::value_type;
        cudaError_t e = cudaMalloc((void**)d, sizeof(T) * std::max<size_t>(v.size(), 1));
        if (e != cudaSuccess) return check(C, e, "cudaMalloc chunks");
        return h2d(C, *d, v.data(), sizeof(T) * v.size(), "upload chunks");
    };
    int rc = PHGPU_OK;
    auto T = [&](int s) { if (rc == PHGPU_OK) rc = s; };
    T(up(&C.d_ch_elem, elem_start));
    T(up(&C.d_ch_node, node_start));
    T(up(&C.d_ch_nodes, nodes));
    T(up(&C.d_ch_cstart, cstart));
    T(up(&C.d_ch_csr, csr));
    T(up(&C.d_ch_lien, lien));
    T(up(&C.d_ien, ien_c));
    // per-chunk records for the bulk copies (16-byte aligned parts, sizes multiples of 16 bytes)
    std::vector<int> rec_off(nch + 1, 0);
    size_t words = 0;
    int rec_max = 0;
    for (int k = 0; k < nch; ++k) {
        const int ne = elem_start[k + 1] - elem_start[k], nn = node_start[k + 1] - node_start[k];
        const int w = chunk_record_words(ne, nn);
        rec_max = std::max(rec_max, 4 * w);
        words += (size_t)w;
        if (words / 4 > (size_t)INT32_MAX) {
            C.err = "chunk records exceed 2^31 16-byte units";
            return PHGPU_ERR_TOO_LARGE;
        }
        rec_off[k + 1] = (int)(words / 4);
    }
    std::vector<uint32_t> rec(std::max<size_t>(words, 4), 0u);
    for (int k = 0; k < nch; ++k) {
        const int e0 = elem_start[k], ne = elem_start[k + 1] - e0;
        const int n0 = node_start[k], nn = node_start[k + 1] - n0;
        uint32_t* r = rec.data() + 4 * (size_t)rec_off[k];
        r[0] = (uint32_t)e0;
        r[1] = (uint32_t)ne;
        r[2] = (uint32_t)n0;
        r[3] = (uint32_t)nn;
        for (int l = 0; l < nn; ++l) r[rec_ids_off() + l] = (uint32_t)nodes[n0 + l];
        std::memcpy(r + rec_lien_off(nn), lien.data() + e0, sizeof(ushort4) * ne);
        std::memcpy(r + rec_csr_off(ne, nn), csr.data() + 4 * (size_t)e0, sizeof(uint16_t) * 4 * ne);
        for (int l = 0; l <= nn; ++l) r[rec_cst_off(ne, nn) + l] = (uint32_t)(cstart[n0 + l] - 4 * e0);
    }
    C.chunk_rec_max = rec_max;
    std::vector<uint4> rec4(rec.size() / 4);
    std::memcpy(rec4.data(), rec.data(), sizeof(uint4) * rec4.size());
    T(up(&C.d_ch_rec, rec4));
    T(up(&C.d_ch_rec_off, rec_off));
    return rc;
}

}  // namespace phgpu
