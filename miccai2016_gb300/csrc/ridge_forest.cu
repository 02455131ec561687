// ridge_forest.cu -- the forest steps of the sign adjustment on the GPU: the
// sign propagation of the ridge directions along the minimum spanning tree,
// and the joins of the local trees of that tree (m16_ridge_forest_joins,
// below the propagation).
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
        const int8_t c = codes ? codes[k] : (int8_t)1;   // no codes: every edge joins with parity 0
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

// root and parity to the root of every point.  A piece's root is also its
// lowest point: a union links the higher root under the lower, so every
// root is the least index of its tree (path halving moves no root).
__global__ void rs_flatten_kernel(uint32_t *parent, int64_t R, uint32_t *root, uint8_t *par, unsigned long long *err)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < R; v += (int64_t)gridDim.x * blockDim.x) {
        uint32_t p;
        const uint32_t r = rs_find(parent, (uint32_t)v, &p, err);
        root[v] = r;
        par[v] = p ? 1 : 0;
    }
}

// the zero and NaN edges, compacted with their endpoints' pieces and the
// pieces' lowest points: (a, b, code, root a, root b, min a, min b)
__global__ void rs_cut_kernel(const int32_t *__restrict__ ea, const int32_t *__restrict__ eb,
                              const int8_t *__restrict__ codes, int64_t n, int64_t R,
                              const uint32_t *__restrict__ root, int32_t *cut,
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
        o[5] = (int32_t)ra;   // the pieces' lowest points are their roots
        o[6] = (int32_t)rb;
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
__global__ void rs_tops_kernel(const uint32_t *__restrict__ root, int64_t R, int32_t *top, int8_t *top_sign)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < R; v += (int64_t)gridDim.x * blockDim.x) {
        if (root[v] == (uint32_t)v && top[v] < 0) {
            top[v] = (int32_t)v;   // a root is its piece's lowest point
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
    size_t parent, root, par, top, tsign, cut, set, ctrl, total;
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
    int32_t *top = (int32_t *)(ws + Ly.top);
    int8_t *tsign = (int8_t *)(ws + Ly.tsign);
    int32_t *cut = (int32_t *)(ws + Ly.cut);
    int32_t *set = (int32_t *)(ws + Ly.set);
    // [0] walks at the limit, [1] cut edges, [2] edges with a code other than -1, 0, 1, 2 or out of range
    unsigned long long *ctrl = (unsigned long long *)(ws + Ly.ctrl);
    const int64_t R = num_points;
    const int gr = rs_grid(R), ge = rs_grid(std::max<int64_t>(num_edges, 1));
    M16_CUDA_TRY(cudaMemsetAsync(ctrl, 0, 32, st));
    M16_CUDA_TRY(cudaMemsetAsync(top, 0xff, 4 * (size_t)R, st));    // -1: not set
    rs_init_kernel<<<gr, kRsBlock, 0, st>>>(parent, R);
    if (num_edges > 0)
        rs_union_kernel<<<ge, kRsBlock, 0, st>>>(edges_a, edges_b, codes, num_edges, R, parent, ctrl, ctrl + 2);
    rs_flatten_kernel<<<gr, kRsBlock, 0, st>>>(parent, R, root, par, ctrl);
    if (num_edges > 0)
        rs_cut_kernel<<<ge, kRsBlock, 0, st>>>(edges_a, edges_b, codes, num_edges, R, root, cut, ctrl + 1,
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
    rs_tops_kernel<<<gr, kRsBlock, 0, st>>>(root, R, top, tsign);
    rs_signs_kernel<<<gr, kRsBlock, 0, st>>>(root, par, R, top, tsign, signs);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

// ---- joins of the local trees -----------------------------------------------------
//
// The ridge-point tree is SciPy's Kruskal over all pairs in (weight, i, j)
// order (adjust_directions.py:374-379).  Its local phase (m16_ridge_mst_local)
// reproduces it up to weight r; what remains is to join the local trees as
// the full Kruskal would: Kruskal over the components, each pair of
// components weighted by its least point pair in (weight, i, j) order.  With
// unit voxel size every squared distance is an integer and the weights
// sqrt(d^2) order like d^2 (distinct integers below 2^32 have distinct
// double square roots), so the least pair of two components is the least
// (d^2, lo, hi), found exactly in integer arithmetic: the components are
// ranked by size, and the points of each rank are compared with every point
// of the lower-ranked (smaller) components, keeping per query point its
// nearest target point with the lowest index.  A ridge of one large segment
// and a few small ones costs |large| x |small| integer distance evaluations.

namespace m16 {
namespace {

constexpr int kFjChunk = 2048;          // target points per block, staged in shared memory
constexpr int kFjScanItems = 1024;      // points per block of the component numbering
constexpr int64_t kFjMaxCoord = 32767;  // |dz|^2 + |dy|^2 + |dx|^2 < 2^32

// roots per block of kFjScanItems points (a root is its component's lowest
// point); 4 consecutive points per thread, as fj_root_id_kernel takes them
__global__ void __launch_bounds__(256) fj_root_count_kernel(const uint32_t *__restrict__ root, int64_t R,
                                                            unsigned *__restrict__ bcount)
{
    __shared__ unsigned tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kFjScanItems + 4 * threadIdx.x;
    unsigned c = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int64_t v = base + j;
        c += (v < R && root[v] == (uint32_t)v) ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&tot, c);
    __syncthreads();
    if (threadIdx.x == 0) bcount[blockIdx.x] = tot;
}

// number of each root in index order: boff[block] + roots before it in the block
__global__ void __launch_bounds__(256) fj_root_id_kernel(const uint32_t *__restrict__ root, int64_t R,
                                                         const unsigned *__restrict__ boff, int32_t *__restrict__ cid)
{
    __shared__ unsigned warp_tot[8];
    const int64_t base = (int64_t)blockIdx.x * kFjScanItems + 4 * threadIdx.x;   // 4 consecutive points per thread
    unsigned flags = 0, cnt = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int64_t v = base + j;
        const unsigned f = (v < R && root[v] == (uint32_t)v) ? 1u : 0u;
        flags |= f << j;
        cnt += f;
    }
    // exclusive scan of cnt over the block's 256 threads
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    unsigned before = 0;
    for (int k = 0; k < w; ++k) before += warp_tot[k];
    unsigned id = boff[blockIdx.x] + before + x - cnt;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (flags & (1u << j)) cid[base + j] = (int32_t)id++;
}

// component of every point, the component sizes, coordinates in range
__global__ void fj_comp_kernel(const uint32_t *__restrict__ root, const int32_t *__restrict__ cid,
                               const int32_t *__restrict__ pts, int64_t R, int32_t *__restrict__ comp,
                               unsigned *__restrict__ size, unsigned long long *bad)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < R; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = cid[root[v]];
        comp[v] = c;
        atomicAdd(size + c, 1u);
        const int32_t a = pts[3 * v], b = pts[3 * v + 1], d = pts[3 * v + 2];
        if (a < 0 || a > kFjMaxCoord || b < 0 || b > kFjMaxCoord || d < 0 || d > kFjMaxCoord) atomicAdd(bad, 1ull);
    }
}

// points grouped by their component's rank (any order inside a group)
__global__ void fj_scatter_kernel(const int32_t *__restrict__ comp, int64_t R, const int32_t *__restrict__ rank_of,
                                  const unsigned *__restrict__ start, unsigned *__restrict__ fill,
                                  int32_t *__restrict__ perm)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < R; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = rank_of[comp[v]];
        perm[start[r] + atomicAdd(fill + r, 1u)] = (int32_t)v;
    }
}

struct FjChunk {
    int32_t rank, begin, end;   // target positions [begin, end) of perm, all of one rank
};

// every query point q of a rank above the chunk's against the chunk's points:
// key[chunk rank][q - qbase] = min over targets p of (d^2 << 32 | p)
__global__ void __launch_bounds__(256) fj_nearest_kernel(const int32_t *__restrict__ pts,
                                                         const int32_t *__restrict__ perm,
                                                         const unsigned *__restrict__ start,
                                                         const FjChunk *__restrict__ chunks, int64_t R, int64_t qbase,
                                                         unsigned long long *__restrict__ key)
{
    __shared__ int4 tp[kFjChunk];
    const FjChunk ch = chunks[blockIdx.x];
    const int nt = ch.end - ch.begin;
    for (int k = threadIdx.x; k < nt; k += blockDim.x) {
        const int32_t p = perm[ch.begin + k];
        tp[k] = make_int4(pts[3 * p], pts[3 * p + 1], pts[3 * p + 2], p);
    }
    __syncthreads();
    const int64_t q0 = start[ch.rank + 1];
    unsigned long long *krow = key + (int64_t)ch.rank * (R - qbase);
    for (int64_t qi = q0 + threadIdx.x; qi < R; qi += blockDim.x) {
        const int32_t q = perm[qi];
        const int a = pts[3 * q], b = pts[3 * q + 1], c = pts[3 * q + 2];
        unsigned long long best = ~0ull;
        for (int k = 0; k < nt; ++k) {
            const int4 t = tp[k];
            const int da = t.x - a, db = t.y - b, dc = t.z - c;
            const unsigned d2 = (unsigned)(da * da) + (unsigned)(db * db) + (unsigned)(dc * dc);
            const unsigned long long kk = ((unsigned long long)d2 << 32) | (unsigned)t.w;
            best = kk < best ? kk : best;
        }
        atomicMin(krow + (qi - qbase), best);
    }
}

__global__ void fj_fill_kernel(unsigned long long *p, int64_t n)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        p[k] = ~0ull;
}

struct FjLayout {
    size_t parent, root, par, cid, comp, size, rank, start, fill, perm, bcount, chunks, key, ctrl, total;
    int64_t max_keys, max_chunks;
};

FjLayout fj_layout(int64_t R)
{
    FjLayout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    const int64_t nb = div_up(R, kFjScanItems);
    L.max_keys = 4 * R;
    L.max_chunks = R / kFjChunk + R + 1;
    L.parent = take(4 * (size_t)R);
    L.root = take(4 * (size_t)R);
    L.par = take((size_t)R);
    L.cid = take(4 * (size_t)R);
    L.comp = take(4 * (size_t)R);
    L.size = take(4 * (size_t)R);
    L.rank = take(4 * (size_t)R);
    L.start = take(4 * (size_t)(R + 1));
    L.fill = take(4 * (size_t)R);
    L.perm = take(4 * (size_t)R);
    L.bcount = take(4 * (size_t)nb);
    L.chunks = take(sizeof(FjChunk) * (size_t)L.max_chunks);
    L.key = take(8 * (size_t)L.max_keys);
    L.ctrl = take(32);
    L.total = off;
    return L;
}

}  // namespace
}  // namespace m16

extern "C" size_t m16_ridge_forest_joins_workspace_bytes(int64_t num_points)
{
    if (num_points < 1 || num_points > (int64_t)kIndexMask) return 0;
    return fj_layout(num_points).total;
}

extern "C" int m16_ridge_forest_joins(const int32_t *pts3, int64_t num_points, const int32_t *edges_a,
                                      const int32_t *edges_b, int64_t num_edges, int64_t max_pair_evaluations,
                                      int32_t *join_a, int32_t *join_b, int64_t *num_joins, void *workspace,
                                      size_t workspace_bytes, void *stream)
{
    const int64_t R = num_points;
    if (R < 1 || R > (int64_t)kIndexMask || num_edges < 0 || num_edges >= R || !pts3 || !join_a || !join_b ||
        !num_joins || (num_edges > 0 && (!edges_a || !edges_b)))
        return M16_ERR_BAD_ARG;
    const FjLayout Ly = fj_layout(R);
    if (!workspace || workspace_bytes < Ly.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    *num_joins = 0;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    uint32_t *parent = (uint32_t *)(ws + Ly.parent);
    uint32_t *root = (uint32_t *)(ws + Ly.root);
    uint8_t *par = (uint8_t *)(ws + Ly.par);
    int32_t *cid = (int32_t *)(ws + Ly.cid);
    int32_t *comp = (int32_t *)(ws + Ly.comp);
    unsigned *size = (unsigned *)(ws + Ly.size);
    int32_t *rank_of = (int32_t *)(ws + Ly.rank);
    unsigned *start = (unsigned *)(ws + Ly.start);
    unsigned *fill = (unsigned *)(ws + Ly.fill);
    int32_t *perm = (int32_t *)(ws + Ly.perm);
    unsigned *bcount = (unsigned *)(ws + Ly.bcount);
    FjChunk *chunks = (FjChunk *)(ws + Ly.chunks);
    unsigned long long *key = (unsigned long long *)(ws + Ly.key);
    unsigned long long *ctrl = (unsigned long long *)(ws + Ly.ctrl);   // [0] walks at the limit, [1] bad edges, [2] bad coordinates
    const int gr = rs_grid(R), ge = rs_grid(std::max<int64_t>(num_edges, 1));
    const int64_t nb = div_up(R, kFjScanItems);
    // components of the forest: union-find, each root its component's lowest point
    M16_CUDA_TRY(cudaMemsetAsync(ctrl, 0, 32, st));
    rs_init_kernel<<<gr, kRsBlock, 0, st>>>(parent, R);
    if (num_edges > 0)
        rs_union_kernel<<<ge, kRsBlock, 0, st>>>(edges_a, edges_b, nullptr, num_edges, R, parent, ctrl, ctrl + 1);
    rs_flatten_kernel<<<gr, kRsBlock, 0, st>>>(parent, R, root, par, ctrl);
    fj_root_count_kernel<<<(unsigned)nb, 256, 0, st>>>(root, R, bcount);
    M16_CUDA_TRY(cudaGetLastError());
    std::vector<unsigned> hb(nb);
    M16_CUDA_TRY(cudaMemcpyAsync(hb.data(), bcount, 4 * (size_t)nb, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    unsigned C = 0;
    for (int64_t b = 0; b < nb; ++b) {
        const unsigned c = hb[b];
        hb[b] = C;
        C += c;
    }
    if (C <= 1) return M16_OK;   // one tree already
    M16_CUDA_TRY(cudaMemcpyAsync(bcount, hb.data(), 4 * (size_t)nb, cudaMemcpyHostToDevice, st));
    fj_root_id_kernel<<<(unsigned)nb, 256, 0, st>>>(root, R, bcount, cid);
    M16_CUDA_TRY(cudaMemsetAsync(size, 0, 4 * (size_t)C, st));
    fj_comp_kernel<<<gr, kRsBlock, 0, st>>>(root, cid, pts3, R, comp, size, ctrl + 2);
    M16_CUDA_TRY(cudaGetLastError());
    std::vector<unsigned> hsize(C);
    unsigned long long hc[3];
    M16_CUDA_TRY(cudaMemcpyAsync(hsize.data(), size, 4 * (size_t)C, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaMemcpyAsync(hc, ctrl, 24, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    if (hc[1] != 0 || hc[2] != 0) return M16_ERR_BAD_ARG;
    if (hc[0] != 0) return M16_ERR_TIMEOUT;
    // ranks: components by size, largest first (ties by number)
    std::vector<int32_t> order(C), rank_h(C);
    for (unsigned c = 0; c < C; ++c) order[c] = (int32_t)c;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return hsize[a] > hsize[b]; });
    std::vector<unsigned> hstart(C + 1, 0);
    for (unsigned t = 0; t < C; ++t) {
        rank_h[order[t]] = (int32_t)t;
        hstart[t + 1] = hstart[t] + hsize[order[t]];
    }
    // the work and memory of the search: every rank against the ranks after it
    const int64_t qbase = hstart[1];
    double work = 0.0;
    std::vector<FjChunk> hch;
    for (unsigned t = 0; t + 1 < C; ++t) {
        work += (double)hsize[order[t]] * (double)(R - hstart[t + 1]);
        for (int64_t b0 = hstart[t]; b0 < (int64_t)hstart[t + 1]; b0 += kFjChunk)
            hch.push_back(FjChunk{(int32_t)t, (int32_t)b0, (int32_t)std::min<int64_t>(b0 + kFjChunk, hstart[t + 1])});
    }
    const int64_t nkeys = (int64_t)(C - 1) * (R - qbase);
    if (work > (double)max_pair_evaluations || nkeys > Ly.max_keys || (int64_t)hch.size() > Ly.max_chunks ||
        (int64_t)hch.size() > INT32_MAX)
        return M16_ERR_TOO_LARGE;
    M16_CUDA_TRY(cudaMemcpyAsync(rank_of, rank_h.data(), 4 * (size_t)C, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(start, hstart.data(), 4 * (size_t)(C + 1), cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(chunks, hch.data(), sizeof(FjChunk) * hch.size(), cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemsetAsync(fill, 0, 4 * (size_t)C, st));
    fj_scatter_kernel<<<gr, kRsBlock, 0, st>>>(comp, R, rank_of, start, fill, perm);
    fj_fill_kernel<<<rs_grid(nkeys), kRsBlock, 0, st>>>(key, nkeys);
    fj_nearest_kernel<<<(unsigned)hch.size(), 256, 0, st>>>(pts3, perm, start, chunks, R, qbase, key);
    M16_CUDA_TRY(cudaGetLastError());
    std::vector<unsigned long long> hkey(nkeys);
    std::vector<int32_t> hperm(R - qbase);
    M16_CUDA_TRY(cudaMemcpyAsync(hkey.data(), key, 8 * (size_t)nkeys, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaMemcpyAsync(hperm.data(), perm + qbase, 4 * (size_t)(R - qbase), cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    // least (d^2, lo, hi) of every pair of ranks (s > t)
    struct Cand {
        uint64_t d2;
        int32_t lo, hi, s, t;
    };
    std::vector<Cand> cand;
    cand.reserve((size_t)C * (C - 1) / 2);
    for (unsigned t = 0; t + 1 < C; ++t) {
        const unsigned long long *krow = hkey.data() + (int64_t)t * (R - qbase);
        for (unsigned s = t + 1; s < C; ++s) {
            Cand best{~0ull, INT32_MAX, INT32_MAX, (int32_t)s, (int32_t)t};
            for (int64_t qi = hstart[s]; qi < (int64_t)hstart[s + 1]; ++qi) {
                const unsigned long long k = krow[qi - qbase];
                const int32_t q = hperm[qi - qbase], p = (int32_t)(k & 0xffffffffu);
                const uint64_t d2 = k >> 32;
                const int32_t lo = std::min(q, p), hi = std::max(q, p);
                if (d2 < best.d2 || (d2 == best.d2 && (lo < best.lo || (lo == best.lo && hi < best.hi))))
                    best = Cand{d2, lo, hi, (int32_t)s, (int32_t)t};
            }
            cand.push_back(best);
        }
    }
    // Kruskal over the components in (weight, lo, hi) order
    std::sort(cand.begin(), cand.end(), [](const Cand &a, const Cand &b) {
        if (a.d2 != b.d2) return a.d2 < b.d2;
        if (a.lo != b.lo) return a.lo < b.lo;
        return a.hi < b.hi;
    });
    std::vector<int32_t> uf(C);
    for (unsigned c = 0; c < C; ++c) uf[c] = (int32_t)c;
    auto find = [&](int32_t x) {
        while (uf[x] != x) {
            uf[x] = uf[uf[x]];
            x = uf[x];
        }
        return x;
    };
    int64_t nj = 0;
    for (const Cand &c : cand) {
        const int32_t a = find(c.s), b = find(c.t);
        if (a == b) continue;
        uf[std::max(a, b)] = std::min(a, b);
        join_a[nj] = c.lo;
        join_b[nj] = c.hi;
        if (++nj == (int64_t)C - 1) break;
    }
    *num_joins = nj;
    return M16_OK;
}
