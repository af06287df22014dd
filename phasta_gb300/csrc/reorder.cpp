// reorder.cpp -- reverse Cuthill-McKee node order of a PHASTA mesh (host code).
//
// PHASTA's solver takes its node numbering from the pre-processor, which renumbers the
// nodes for locality before the partitioned mesh is written (the solver itself never
// renumbers: the arrays of phSolver/compressible/elmmfg.f:1-5 arrive in file order).  A
// mesh whose nodes come in an arbitrary order makes every chunk of elements gather its
// nodes from all over the state vectors; phgpu_rcm_order gives the caller the reverse
// Cuthill-McKee order (Cuthill & McKee 1969; George's reversal, 1971; the pseudo-peripheral
// start node of Gibbs, Poole & Stockmeyer 1976 as simplified by George & Liu 1979) to apply
// before phgpu_create.
//
// Graph: two nodes are adjacent when they share an interior element (tet, hex or wedge);
// a periodic slave is adjacent to its master, so that both land close in the new order.
// Ties are broken by the old node number: the order is a deterministic function of the mesh.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "../../include/phgpu.h"

namespace {

struct Graph {
    std::vector<int64_t> start;  // nshg + 1
    std::vector<int> adj;
    int degree(int n) const { return (int)(start[n + 1] - start[n]); }
};

// unique neighbours of every node (CSR, each row sorted by node number)
Graph build_graph(const phgpu_mesh& m) {
    const int N = m.nshg;
    std::vector<int64_t> cnt(N + 1, 0);
    auto each_block = [&](auto&& fn) {
        if (m.nelem > 0) fn(m.ien, (int64_t)m.nelem, 4);
        if (m.nhex > 0) fn(m.ienh, (int64_t)m.nhex, 8);
        if (m.nwedge > 0) fn(m.ienw, (int64_t)m.nwedge, 6);
    };
    // pass 1: an upper bound of each row (nen - 1 entries per element and node, 1 per periodic pair)
    each_block([&](const int* ien, int64_t ne, int nen) {
        for (int64_t e = 0; e < ne; ++e)
            for (int a = 0; a < nen; ++a) cnt[ien[nen * e + a] + 1] += nen - 1;
    });
    if (m.iper)
        for (int n = 0; n < N; ++n)
            if (m.iper[n] != n) {
                ++cnt[n + 1];
                ++cnt[m.iper[n] + 1];
            }
    std::vector<int64_t> fill(N + 1, 0);
    for (int n = 0; n < N; ++n) fill[n + 1] = fill[n] + cnt[n + 1];
    std::vector<int> raw(fill[N]);
    std::vector<int64_t> pos(fill.begin(), fill.end() - 1);
    each_block([&](const int* ien, int64_t ne, int nen) {
        for (int64_t e = 0; e < ne; ++e)
            for (int a = 0; a < nen; ++a)
                for (int b = 0; b < nen; ++b)
                    if (a != b) raw[pos[ien[nen * e + a]]++] = ien[nen * e + b];
    });
    if (m.iper)
        for (int n = 0; n < N; ++n)
            if (m.iper[n] != n) {
                raw[pos[n]++] = m.iper[n];
                raw[pos[m.iper[n]]++] = n;
            }
    // pass 2: sort and deduplicate each row in place, then compact
    Graph g;
    g.start.assign(N + 1, 0);
    int64_t out = 0;
    for (int n = 0; n < N; ++n) {
        auto b = raw.begin() + fill[n], e = raw.begin() + pos[n];
        std::sort(b, e);
        e = std::unique(b, e);
        g.start[n] = out;
        for (auto it = b; it != e; ++it)
            if (*it != n) raw[out++] = *it;
    }
    g.start[N] = out;
    raw.resize(out);
    g.adj.swap(raw);
    return g;
}

// breadth-first level structure from root over the unvisited part; returns the nodes in
// visiting order and the level of the last node; mark[] == stamp marks visited nodes
int bfs_levels(const Graph& g, int root, std::vector<int>& mark, int stamp, std::vector<int>& order,
               std::vector<int>& level) {
    order.clear();
    order.push_back(root);
    mark[root] = stamp;
    level[root] = 0;
    for (size_t h = 0; h < order.size(); ++h) {
        const int n = order[h];
        for (int64_t k = g.start[n]; k < g.start[n + 1]; ++k) {
            const int j = g.adj[k];
            if (mark[j] != stamp && mark[j] >= 0) {
                mark[j] = stamp;
                level[j] = level[n] + 1;
                order.push_back(j);
            }
        }
    }
    return level[order.back()];
}

}  // namespace

extern "C" {

int phgpu_rcm_order(const phgpu_mesh* m, int* new_of_old, long long* bandwidth_before, long long* bandwidth_after) {
    if (!m || !new_of_old || m->nshg <= 0 || m->nelem < 0 || m->nhex < 0 || m->nwedge < 0 ||
        (m->nelem > 0 && !m->ien) || (m->nhex > 0 && !m->ienh) || (m->nwedge > 0 && !m->ienw))
        return PHGPU_ERR_INVALID;
    const int N = m->nshg;
    auto bad = [&](const int* ien, int64_t n) {
        for (int64_t i = 0; i < n; ++i)
            if (ien[i] < 0 || ien[i] >= N) return true;
        return false;
    };
    if (bad(m->ien, 4 * (int64_t)m->nelem) || bad(m->ienh, 8 * (int64_t)m->nhex) ||
        bad(m->ienw, 6 * (int64_t)m->nwedge) || (m->iper && bad(m->iper, N)))
        return PHGPU_ERR_INVALID;
    const Graph g = build_graph(*m);
    // mark: 0 unvisited, -1 numbered, > 0 visited by the BFS of that stamp
    std::vector<int> mark(N, 0), level(N, 0), tmp, order;
    order.reserve(N);
    std::vector<int> by_degree(N);
    for (int n = 0; n < N; ++n) by_degree[n] = n;
    std::stable_sort(by_degree.begin(), by_degree.end(),
                     [&](int a, int b) { return g.degree(a) < g.degree(b); });
    int stamp = 0;
    std::vector<int> nb;
    for (int seed : by_degree) {
        if (mark[seed] < 0) continue;
        // pseudo-peripheral root: restart from the lowest-degree node of the last level while
        // the eccentricity grows
        int root = seed;
        int ecc = bfs_levels(g, root, mark, ++stamp, tmp, level);
        for (int pass = 0; pass < 16; ++pass) {
            int best = -1;
            for (size_t i = tmp.size(); i-- > 0;) {
                const int n = tmp[i];
                if (level[n] != ecc) break;
                if (best < 0 || g.degree(n) < g.degree(best) || (g.degree(n) == g.degree(best) && n < best)) best = n;
            }
            const int e2 = bfs_levels(g, best, mark, ++stamp, tmp, level);
            if (e2 <= ecc) break;
            root = best;
            ecc = e2;
        }
        // Cuthill-McKee from root: neighbours by increasing degree, then node number
        const size_t first = order.size();
        order.push_back(root);
        mark[root] = -1;
        for (size_t h = first; h < order.size(); ++h) {
            const int n = order[h];
            nb.clear();
            for (int64_t k = g.start[n]; k < g.start[n + 1]; ++k)
                if (mark[g.adj[k]] >= 0) nb.push_back(g.adj[k]);
            std::sort(nb.begin(), nb.end(), [&](int a, int b) {
                return g.degree(a) != g.degree(b) ? g.degree(a) < g.degree(b) : a < b;
            });
            for (int j : nb) {
                mark[j] = -1;
                order.push_back(j);
            }
        }
    }
    if ((int)order.size() != N) return PHGPU_ERR_INVALID;
    for (int i = 0; i < N; ++i) new_of_old[order[i]] = N - 1 - i;  // reversed
    auto bandwidth = [&](const int* perm) {
        long long bw = 0;
        for (int n = 0; n < N; ++n)
            for (int64_t k = g.start[n]; k < g.start[n + 1]; ++k) {
                const long long d = (long long)(perm ? perm[n] - perm[g.adj[k]] : n - g.adj[k]);
                bw = std::max(bw, d < 0 ? -d : d);
            }
        return bw;
    };
    if (bandwidth_before) *bandwidth_before = bandwidth(nullptr);
    if (bandwidth_after) *bandwidth_after = bandwidth(new_of_old);
    return PHGPU_OK;
}

}  // extern "C"
