// ridge_host.cu -- host-side helpers of the sign adjustment, in C++ behind the
// same C ABI (no device code).
//
// m16_compose_signs: the sign propagation of
// AdvancedAdjuster._adjust_ridge_directions (src/processing/adjust_directions.py:382-415)
// visits the tree from its root and keeps or negates each child's direction
// by the sign of its dot product with the parent's adjusted direction.  The
// dot products' signs (against the parent's unadjusted direction) are
// computed beforehand; what remains is one pass in visiting order composing
// them with the parent's final sign.
#include <stdint.h>

#include <vector>

#include "../../include/miccai2016_gb300.h"

// m16_tree_order: the visiting order and parents of that propagation over an
// undirected forest: breadth first from the root, then every other tree from
// its lowest-index point (the reference hangs the rest of a forest off the
// root that way).  In a tree each point's parent -- its neighbour on the
// path to the tree's start -- does not depend on the order neighbours are
// taken in.
extern "C" int m16_tree_order(int64_t n, const int32_t *ea, const int32_t *eb, int64_t n_edges, int32_t root,
                              int32_t *order, int32_t *pred)
{
    if (n < 1 || n > INT32_MAX || n_edges < 0 || (n_edges > 0 && (!ea || !eb)) || !order || !pred || root < 0 ||
        root >= n)
        return M16_ERR_BAD_ARG;
    std::vector<int64_t> start(n + 1, 0);
    for (int64_t k = 0; k < n_edges; ++k) {
        if (ea[k] < 0 || ea[k] >= n || eb[k] < 0 || eb[k] >= n) return M16_ERR_BAD_ARG;
        ++start[ea[k] + 1];
        ++start[eb[k] + 1];
    }
    for (int64_t i = 0; i < n; ++i) start[i + 1] += start[i];
    std::vector<int32_t> adj(2 * n_edges);
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t k = 0; k < n_edges; ++k) {
        adj[fill[ea[k]]++] = eb[k];
        adj[fill[eb[k]]++] = ea[k];
    }
    std::vector<char> seen(n, 0);
    int64_t head = 0, tail = 0;
    auto visit_from = [&](int32_t s) {
        seen[s] = 1;
        pred[s] = -1;
        order[tail++] = s;
        while (head < tail) {
            const int32_t c = order[head++];
            for (int64_t k = start[c]; k < start[c + 1]; ++k) {
                const int32_t d = adj[k];
                if (seen[d]) continue;
                seen[d] = 1;
                pred[d] = c;
                order[tail++] = d;
            }
        }
    };
    visit_from(root);
    for (int32_t i = 0; i < (int32_t)n; ++i)
        if (!seen[i]) visit_from(i);
    return tail == n ? M16_OK : M16_ERR_BAD_ARG;
}

extern "C" int m16_compose_signs(int64_t n, const int32_t *order, int64_t n_order, const int32_t *pred,
                                 const int8_t *e, int8_t *s)
{
    if (n < 1 || n_order < 0 || n_order > n || !order || !pred || !e || !s) return M16_ERR_BAD_ARG;
    for (int64_t k = 0; k < n_order; ++k) {
        const int32_t c = order[k];
        if (c < 0 || c >= n) return M16_ERR_BAD_ARG;
        const int8_t ek = e[c];
        if (ek == 0) { s[c] = 1; continue; }      // a restart: the root, a new tree, a zero dot
        if (ek == 2) { s[c] = -1; continue; }     // NaN dot: negated whatever the parent
        const int32_t p = pred[c];
        if (p < 0 || p >= n) return M16_ERR_BAD_ARG;
        s[c] = (int8_t)(s[p] * ek);               // the parent precedes the child in the visiting order
    }
    return M16_OK;
}
