// ridge_signs.cu -- the sign propagation of the ridge directions on the GPU.
//
// AdvancedAdjuster._adjust_ridge_directions (src/processing/adjust_directions.py:382-415)
// walks the minimum spanning tree of the ridge points from point 0 and keeps
// or negates each child's direction by the sign of np.dot(child, adjusted
// parent).  With s the sign a point's direction ends up with, np.dot(d_c,
// s_p d_p) = s_p np.dot(d_c, d_p) bit for bit, so every decision reduces to
// the sign of the edge's own dot product e = sign(np.dot(d_a, d_b)), which
// does not depend on the edge's orientation:
//   e = +1 or -1: s_child = s_parent * e;
//   e = 0 (a zero dot, either sign of zero passes ">= 0"): s_child = +1;
//   e = NaN: s_child = -1 ("np.dot(...) >= 0" fails whatever the parent).
// Over the edges with e = +-1 the signs are a parity: s_v = s_top * (-1)^(the
// number of negative edges between v and the top of its piece), where a
// piece is a component of those edges.  The parities come from a union-find
// whose parent links carry the parity of the link (one 32-bit word: parity
// bit and parent index, linked from the higher root to the lower, path
// halving by compare-and-swap).  The pieces' tops follow from the few
// remaining edges on the host: a tree's first piece starts at the tree's
// lowest point (point 0 for the reference's root; every other tree of a
// forest from its lowest-index point, as the reference's loop hangs them),
// and a piece entered through a zero or NaN edge starts at that edge's
// endpoint inside it with sign +1 or -1.
//
// Edge signs whose float32 rounding could differ from the exact dot's sign
// (|exact| within the rounding error bound of zero) are marked 3; the caller
// evaluates those few with np.dot itself and passes the codes back in.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace m16 {
namespace {

constexpr int kRsBlock = 256;
constexpr uint32_t kParityBit = 0x80000000u;
constexpr uint32_t kIndexMask = 0x7fffffffu;
constexpr int kRsWalkLimit = 1 << 24;

// sign code of the dot product of directions a and b (float32 x 3)
// (4: an endpoint outside [0, R), which m16_ridge_signs rejects)
__global__ void rs_edge_codes_kernel(const float *__restrict__ dirs, int64_t R, const int32_t *__restrict__ ea,
                                     const int32_t *__restrict__ eb, int64_t n, int8_t *__restrict__ codes)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        if (ea[k] < 0 || ea[k] >= R || eb[k] < 0 || eb[k] >= R) {
            codes[k] = 4;
            continue;
        }
        const float *u = dirs + 3 * (int64_t)ea[k];
        const float *v = dirs + 3 * (int64_t)eb[k];
        // the products of float32 values are exact in double
        const double p0 = __dmul_rn((double)u[0], (double)v[0]);
        const double p1 = __dmul_rn((double)u[1], (double)v[1]);
        const double p2 = __dmul_rn((double)u[2], (double)v[2]);
        const double exact = __dadd_rn(__dadd_rn(p0, p1), p2);
        int8_t c;
        if (isnan(exact)) {
            c = 2;
        } else {
            // a float32 sum of three products (in any order, with or without
            // fused multiply-adds) is within 3 * 2^-23 * sum |products| of the
            // exact value; the margin is generous
            const double bound = 8.0 * 1.1920928955078125e-07 * (fabs(p0) + fabs(p1) + fabs(p2));
            c = fabs(exact) <= bound ? 3 : (exact > 0.0 ? 1 : (exact < 0.0 ? -1 : 0));
        }
        codes[k] = c;
    }
}

__global__ void rs_init_kernel(uint32_t *parent, int64_t R)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < R; v += (int64_t)gridDim.x * blockDim.x)
        parent[v] = (uint32_t)v;
}

// root of v and the parity of the path to it; halves the path on the way
__device__ __forceinline__ uint32_t rs_find(uint32_t *parent, uint32_t v, uint32_t *parity, unsigned long long *err)
{
    uint32_t acc = 0, x = v;
    for (int steps = 0; steps < kRsWalkLimit; ++steps) {
        const uint32_t w = parent[x];
        const uint32_t px = w & kIndexMask;
        if (px == x) {
            *parity = acc;
            return x;
        }
        const uint32_t g = parent[px];
        const uint32_t gx = g & kIndexMask;
        if (gx != px) {
            // link x to its grandparent: the parity of the two links combined
            const uint32_t nw = ((w ^ g) & kParityBit) | gx;
            atomicCAS(parent + x, w, nw);   // a failed swap means another thread moved x up already
        }
        acc ^= w & kParityBit;
        x = px;
    }
    atomicAdd(err, 1ull);
    *parity = acc;
    return x;
}

// union of the endpoints of every +-1 edge, with the edge's parity
__global__ void rs_union_kernel(const int32_t *__restrict__ ea, const int32_t *__restrict__ eb,
                                const int8_t *__restrict__ codes, int64_t n, int64_t R, uint32_t *parent,
                                unsigned long long *err, unsigned long long *bad)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int8_t c = codes[k];
        if (c != 1 && c != -1) continue;
        if (ea[k] < 0 || ea[k] >= R || eb[k] < 0 || eb[k] >= R) {
            atomicAdd(bad, 1ull);
            continue;
        }
        const uint32_t e = c < 0 ? kParityBit : 0u;
        int tries = 0;
        for (; tries < kRsWalkLimit; ++tries) {
            uint32_t pa, pb;
            const uint32_t ra = rs_find(parent, (uint32_t)ea[k], &pa, err);
            const uint32_t rb = rs_find(parent, (uint32_t)eb[k], &pb, err);
            if (ra == rb) break;   // not a forest edge: ignored
            const uint32_t hi = ra > rb ? ra : rb, lo = ra > rb ? rb : ra;
            // hi becomes a child of lo: parity(hi -> lo) = pa ^ pb ^ e
            if (atomicCAS(parent + hi, hi, ((pa ^ pb ^ e) & kParityBit) | lo) == hi) break;
        }
        if (tries >= kRsWalkLimit) atomicAdd(err, 1ull);
    }
}

// root, parity to the root, and the lowest point of each piece
__global__ void rs_flatten_kernel(uint32_t *parent, int64_t R, uint32_t *root, uint8_t *par, int32_t *piece_min,
                                  unsigned long long *err)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < R; v += (int64_t)gridDim.x * blockDim.x) {
        uint32_t p;
        const uint32_t r = rs_find(parent, (uint32_t)v, &p, err);
        root[v] = r;
        par[v] = p ? 1 : 0;
        atomicMin(piece_min + r, (int32_t)v);
    }
}

// the zero and NaN edges, compacted with their endpoints' pieces and the
// pieces' lowest points: (a, b, code, root a, root b, min a, min b)
__global__ void rs_cut_kernel(const int32_t *__restrict__ ea, const int32_t *__restrict__ eb,
                              const int8_t *__restrict__ codes, int64_t n, int64_t R,
                              const uint32_t *__restrict__ root, const int32_t *__restrict__ piece_min, int32_t *cut,
                              unsigned long long *count, unsigned long long *bad)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int8_t c = codes[k];
        if (c == 1 || c == -1) continue;
        if ((c != 0 && c != 2) || ea[k] < 0 || ea[k] >= R || eb[k] < 0 || eb[k] >= R) {
            atomicAdd(bad, 1ull);   // an unresolved or unknown code, or an endpoint outside [0, R)
            continue;
        }
        const unsigned long long slot = atomicAdd(count, 1ull);
        int32_t *o = cut + 7 * slot;
        const uint32_t ra = root[ea[k]], rb = root[eb[k]];
        o[0] = ea[k];
        o[1] = eb[k];
        o[2] = c;
        o[3] = (int32_t)ra;
        o[4] = (int32_t)rb;
        o[5] = piece_min[ra];
        o[6] = piece_min[rb];
    }
}

// the tops the host set for the pieces joined by zero / NaN edges: (root, top, sign)
__global__ void rs_set_tops_kernel(const int32_t *__restrict__ set, int64_t n, int32_t *top, int8_t *top_sign)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        top[set[3 * k]] = set[3 * k + 1];
        top_sign[set[3 * k]] = (int8_t)set[3 * k + 2];
    }
}

// top of every other piece: its lowest point, with sign +1
__global__ void rs_tops_kernel(const uint32_t *__restrict__ root, int64_t R, const int32_t *__restrict__ piece_min,
                               int32_t *top, int8_t *top_sign)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < R; v += (int64_t)gridDim.x * blockDim.x) {
        if (root[v] == (uint32_t)v && top[v] < 0) {
            top[v] = piece_min[v];
            top_sign[v] = 1;
        }
    }
}

__global__ void rs_signs_kernel(const uint32_t *__restrict__ root, const uint8_t *__restrict__ par, int64_t R,
                                const int32_t *__restrict__ top, const int8_t *__restrict__ top_sign,
                                int8_t *__restrict__ signs)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < R; v += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t r = root[v];
        const int32_t t = top[r];
        const int8_t s = top_sign[r];
        signs[v] = (par[v] ^ par[t]) ? (int8_t)-s : s;
    }
}

struct RsLayout {
    size_t parent, root, par, pmin, top, tsign, cut, set, ctrl, total;
};

RsLayout rs_layout(int64_t R, int64_t n_edges)
{
    RsLayout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    L.parent = take(4 * (size_t)R);
    L.root = take(4 * (size_t)R);
    L.par = take((size_t)R);
    L.pmin = take(4 * (size_t)R);
    L.top = take(4 * (size_t)R);
    L.tsign = take((size_t)R);
    L.cut = take(28 * (size_t)std::max<int64_t>(n_edges, 1));
    L.set = take(24 * (size_t)std::max<int64_t>(n_edges, 1));
    L.ctrl = take(32);
    L.total = off;
    return L;
}

int rs_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(div_up(n, kRsBlock), 8 * kSMs)); }

}  // namespace
}  // namespace m16

using namespace m16;

extern "C" size_t m16_ridge_signs_workspace_bytes(int64_t num_points, int64_t num_edges)
{
    if (num_points < 1 || num_points > (int64_t)kIndexMask || num_edges < 0 || num_edges >= num_points) return 0;
    return rs_layout(num_points, num_edges).total;
}

extern "C" int m16_ridge_edge_codes(const float *dirs3, int64_t num_points, const int32_t *edges_a,
                                    const int32_t *edges_b, int64_t num_edges, int8_t *codes, void *stream)
{
    if (num_points < 1 || num_edges < 0 || num_edges >= num_points || !dirs3 || !codes ||
        (num_edges > 0 && (!edges_a || !edges_b)))
        return M16_ERR_BAD_ARG;
    if (num_edges == 0) return M16_OK;
    cudaStream_t st = (cudaStream_t)stream;
    rs_edge_codes_kernel<<<rs_grid(num_edges), kRsBlock, 0, st>>>(dirs3, num_points, edges_a, edges_b, num_edges,
                                                                  codes);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" int m16_ridge_signs(int64_t num_points, const int32_t *edges_a, const int32_t *edges_b,
                               const int8_t *codes, int64_t num_edges, int8_t *signs, void *workspace,
                               size_t workspace_bytes, void *stream)
{
    if (num_points < 1 || num_points > (int64_t)kIndexMask || num_edges < 0 || num_edges >= num_points || !signs ||
        (num_edges > 0 && (!edges_a || !edges_b || !codes)))
        return M16_ERR_BAD_ARG;
    const RsLayout Ly = rs_layout(num_points, num_edges);
    if (!workspace || workspace_bytes < Ly.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    uint32_t *parent = (uint32_t *)(ws + Ly.parent);
    uint32_t *root = (uint32_t *)(ws + Ly.root);
    uint8_t *par = (uint8_t *)(ws + Ly.par);
    int32_t *pmin = (int32_t *)(ws + Ly.pmin);
    int32_t *top = (int32_t *)(ws + Ly.top);
    int8_t *tsign = (int8_t *)(ws + Ly.tsign);
    int32_t *cut = (int32_t *)(ws + Ly.cut);
    int32_t *set = (int32_t *)(ws + Ly.set);
    // [0] walks at the limit, [1] cut edges, [2] edges with a code other than -1, 0, 1, 2 or out of range
    unsigned long long *ctrl = (unsigned long long *)(ws + Ly.ctrl);
    const int64_t R = num_points;
    const int gr = rs_grid(R), ge = rs_grid(std::max<int64_t>(num_edges, 1));
    M16_CUDA_TRY(cudaMemsetAsync(ctrl, 0, 32, st));
    M16_CUDA_TRY(cudaMemsetAsync(pmin, 0x7f, 4 * (size_t)R, st));   // 0x7f7f7f7f > every index
    M16_CUDA_TRY(cudaMemsetAsync(top, 0xff, 4 * (size_t)R, st));    // -1: not set
    rs_init_kernel<<<gr, kRsBlock, 0, st>>>(parent, R);
    if (num_edges > 0)
        rs_union_kernel<<<ge, kRsBlock, 0, st>>>(edges_a, edges_b, codes, num_edges, R, parent, ctrl, ctrl + 2);
    rs_flatten_kernel<<<gr, kRsBlock, 0, st>>>(parent, R, root, par, pmin, ctrl);
    if (num_edges > 0)
        rs_cut_kernel<<<ge, kRsBlock, 0, st>>>(edges_a, edges_b, codes, num_edges, R, root, pmin, cut, ctrl + 1,
                                               ctrl + 2);
    M16_CUDA_TRY(cudaGetLastError());
    unsigned long long hc[3];
    M16_CUDA_TRY(cudaMemcpyAsync(hc, ctrl, 24, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    if (hc[2] != 0) return M16_ERR_BAD_ARG;
    if (hc[0] != 0) return M16_ERR_TIMEOUT;
    const int64_t n_cut = (int64_t)hc[1];
    if (n_cut > 0) {
        // the pieces joined by zero / NaN edges: each tree of pieces starts at
        // the piece of its lowest point; every other piece at the endpoint of
        // the edge it is entered by
        std::vector<int32_t> hcut(7 * n_cut);
        M16_CUDA_TRY(cudaMemcpyAsync(hcut.data(), cut, 28 * (size_t)n_cut, cudaMemcpyDeviceToHost, st));
        M16_CUDA_TRY(cudaStreamSynchronize(st));
        std::vector<int32_t> pieces;
        pieces.reserve(2 * n_cut);
        for (int64_t k = 0; k < n_cut; ++k) {
            pieces.push_back(hcut[7 * k + 3]);
            pieces.push_back(hcut[7 * k + 4]);
        }
        std::sort(pieces.begin(), pieces.end());
        pieces.erase(std::unique(pieces.begin(), pieces.end()), pieces.end());
        const int64_t P = (int64_t)pieces.size();
        auto local = [&](int32_t r) {
            return (int64_t)(std::lower_bound(pieces.begin(), pieces.end(), r) - pieces.begin());
        };
        std::vector<int32_t> pmin_local(P);
        std::vector<int64_t> start(P + 1, 0);
        for (int64_t k = 0; k < n_cut; ++k) {
            const int64_t la = local(hcut[7 * k + 3]), lb = local(hcut[7 * k + 4]);
            pmin_local[la] = hcut[7 * k + 5];
            pmin_local[lb] = hcut[7 * k + 6];
            ++start[la + 1];
            ++start[lb + 1];
        }
        for (int64_t i = 0; i < P; ++i) start[i + 1] += start[i];
        std::vector<int64_t> adj(2 * n_cut), fill(start.begin(), start.end() - 1);
        for (int64_t k = 0; k < n_cut; ++k) {
            adj[fill[local(hcut[7 * k + 3])]++] = k;
            adj[fill[local(hcut[7 * k + 4])]++] = k;
        }
        std::vector<int64_t> by_min(P);
        for (int64_t i = 0; i < P; ++i) by_min[i] = i;
        std::sort(by_min.begin(), by_min.end(), [&](int64_t a, int64_t b) { return pmin_local[a] < pmin_local[b]; });
        std::vector<char> seen(P, 0);
        std::vector<int32_t> hset(3 * P);
        std::vector<int64_t> queue;
        queue.reserve(P);
        for (int64_t s0 : by_min) {
            if (seen[s0]) continue;
            seen[s0] = 1;
            hset[3 * s0] = pieces[s0];
            hset[3 * s0 + 1] = pmin_local[s0];
            hset[3 * s0 + 2] = 1;
            queue.clear();
            queue.push_back(s0);
            for (size_t h = 0; h < queue.size(); ++h) {
                const int64_t c = queue[h];
                for (int64_t j = start[c]; j < start[c + 1]; ++j) {
                    const int32_t *e = &hcut[7 * adj[j]];
                    const int64_t la = local(e[3]), lb = local(e[4]);
                    const int64_t d = la == c ? lb : la;
                    if (seen[d]) continue;   // the piece it came from (or, not a forest, one reached already)
                    seen[d] = 1;
                    // the edge's endpoint inside d starts it: +1 after a zero dot, -1 after NaN
                    hset[3 * d] = pieces[d];
                    hset[3 * d + 1] = la == c ? e[1] : e[0];
                    hset[3 * d + 2] = e[2] == 2 ? -1 : 1;
                    queue.push_back(d);
                }
            }
        }
        M16_CUDA_TRY(cudaMemcpyAsync(set, hset.data(), 12 * (size_t)P, cudaMemcpyHostToDevice, st));
        rs_set_tops_kernel<<<rs_grid(P), kRsBlock, 0, st>>>(set, P, top, tsign);
        M16_CUDA_TRY(cudaStreamSynchronize(st));   // hset goes out of scope
    }
    rs_tops_kernel<<<gr, kRsBlock, 0, st>>>(root, R, pmin, top, tsign);
    rs_signs_kernel<<<gr, kRsBlock, 0, st>>>(root, par, R, top, tsign, signs);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}
