// ridge_mst.cu -- the local phase of the ridge-point minimum spanning tree on
// the GPU.
//
// The reference builds the tree of all R ridge points with SciPy's Kruskal over
// the dense distance matrix (src/processing/adjust_directions.py:374-379).  The
// host restatement (ridge_mst.py) defines the order of equal distances as
// (weight, i, j) and splits the tree into a local phase -- Kruskal over every
// pair of points whose offset is not longer than r = |voxel size| -- and a
// global phase that joins the local trees.  This file computes the local
// phase with Boruvka's algorithm: in every round each component picks its
// least outgoing candidate edge in the total order (weight, i, j), and the
// picked edges are added and their components merged.  With every key
// distinct the minimum spanning forest is unique, so the edge set equals the
// one Kruskal's algorithm gives in that order.
//
// Weights are computed exactly as the host does (numpy, float64, no
// contraction): u = point * voxel_size per axis, d = u_i - u_j,
// w = sqrt((d0 d0 + d1 d1) + d2 d2); an edge is a candidate when w <= r.
// A component's least edge is found in two passes: the least weight (an
// atomic minimum on the bits of a positive double, which order like the
// values), then among the edges of that weight the least (i, j) packed into
// 64 bits.
//
// Where every product point * voxel size is exact in double (unit voxel
// size, or any size whose significand ends in at least as many zero bits as
// the coordinates have bits), each difference u_i - u_j is exactly the offset
// times the voxel size, so the weight depends on the offset alone (its sign
// drops out in the squares): it is computed once per offset, with the same
// operations, instead of once per candidate pair and pass -- the double
// square root per pair was most of the local phase's time.
#include <cuda_runtime.h>
#include <math.h>
#include <float.h>
#include <stdlib.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace m16 {
namespace {

struct MstArgs {
    const int *pts;        // R x 3 (axis order 0, 1, 2)
    int64_t R;
    int lo0, lo1, lo2;     // bounding box of the points
    int b0, b1, b2;
    double vs0, vs1, vs2;
    double r;
    const int *offs;       // n_off x 3, the candidate offsets (lexicographically positive)
    int n_off;
    const double *offw;    // n_off: each offset's weight where it does not depend on the points, else null
    const int *grid;       // b0 x b1 x b2: point index or -1
    int *comp;             // R: component of each point (a root index)
    int *parent;           // R: for roots, the component hooked to
    unsigned long long *minw, *minij;   // R: per root
    int *edges;            // 2 x (R - 1)
    unsigned long long *ctrl;   // [0] edges so far, [1] walks at the limit or edge overflow, [2] bad points
};

constexpr unsigned long long kNone = ~0ull;
constexpr int kWalkLimit = 1 << 24;

__device__ __forceinline__ double edge_weight(const MstArgs &a, int i, int j)
{
    const double d0 = __dsub_rn(__dmul_rn((double)a.pts[3 * i], a.vs0), __dmul_rn((double)a.pts[3 * j], a.vs0));
    const double d1 = __dsub_rn(__dmul_rn((double)a.pts[3 * i + 1], a.vs1), __dmul_rn((double)a.pts[3 * j + 1], a.vs1));
    const double d2 = __dsub_rn(__dmul_rn((double)a.pts[3 * i + 2], a.vs2), __dmul_rn((double)a.pts[3 * j + 2], a.vs2));
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
}

// the weight of every offset (edge_weight's operations on the offset times
// the voxel size): where the products are exact this is every pair's weight
__global__ void mst_offset_weights_kernel(MstArgs a, double *offw)
{
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < a.n_off; o += gridDim.x * blockDim.x) {
        const double d0 = __dmul_rn((double)a.offs[3 * o], a.vs0);
        const double d1 = __dmul_rn((double)a.offs[3 * o + 1], a.vs1);
        const double d2 = __dmul_rn((double)a.offs[3 * o + 2], a.vs2);
        offw[o] = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
    }
}

// the point grid; a point outside the box or a second point on one cell is
// counted in ctrl[2] (the call then fails) instead of being written
__global__ void mst_grid_kernel(MstArgs a, int *grid)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.R; i += (int64_t)gridDim.x * blockDim.x) {
        const int q0 = a.pts[3 * i] - a.lo0, q1 = a.pts[3 * i + 1] - a.lo1, q2 = a.pts[3 * i + 2] - a.lo2;
        a.comp[i] = (int)i;
        if (q0 < 0 || q1 < 0 || q2 < 0 || q0 >= a.b0 || q1 >= a.b1 || q2 >= a.b2) {
            atomicAdd(a.ctrl + 2, 1ull);
            continue;
        }
        if (atomicCAS(grid + ((int64_t)q0 * a.b1 + q1) * a.b2 + q2, -1, (int)i) != -1) atomicAdd(a.ctrl + 2, 1ull);
    }
}

// pass 0: least weight of each component's outgoing candidate edges;
// pass 1: least (i, j) among the edges of that weight
template <int PASS>
__global__ void mst_min_kernel(MstArgs a)
{
    const int64_t total = a.R * a.n_off;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / a.n_off), o = (int)(t % a.n_off);
        const int q0 = a.pts[3 * i] - a.lo0 + a.offs[3 * o];
        const int q1 = a.pts[3 * i + 1] - a.lo1 + a.offs[3 * o + 1];
        const int q2 = a.pts[3 * i + 2] - a.lo2 + a.offs[3 * o + 2];
        if (q0 < 0 || q1 < 0 || q2 < 0 || q0 >= a.b0 || q1 >= a.b1 || q2 >= a.b2) continue;
        const int j = a.grid[((int64_t)q0 * a.b1 + q1) * a.b2 + q2];
        if (j < 0) continue;
        const int lo = min(i, j), hi = max(i, j);
        const int ca = a.comp[lo], cb = a.comp[hi];
        if (ca == cb) continue;
        const double w = a.offw ? a.offw[o] : edge_weight(a, lo, hi);
        if (!(w <= a.r)) continue;
        const unsigned long long wb = (unsigned long long)__double_as_longlong(w);
        if (PASS == 0) {
            atomicMin(a.minw + ca, wb);
            atomicMin(a.minw + cb, wb);
        } else {
            const unsigned long long key = ((unsigned long long)(unsigned)lo << 32) | (unsigned)hi;
            if (a.minw[ca] == wb) atomicMin(a.minij + ca, key);
            if (a.minw[cb] == wb) atomicMin(a.minij + cb, key);
        }
    }
}

// every root with a picked edge hooks onto the component across it (of two
// components that picked the same edge, the larger index hooks) and records
// the edge
__global__ void mst_hook_kernel(MstArgs a)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.R; c += (int64_t)gridDim.x * blockDim.x) {
        if (a.comp[c] != (int)c) continue;
        const unsigned long long key = a.minij[c];
        if (key == kNone) continue;
        const int lo = (int)(key >> 32), hi = (int)(key & 0xffffffffu);
        const int ca = a.comp[lo], cb = a.comp[hi];
        const int other = ca == (int)c ? cb : ca;
        if (a.minij[other] == key && (int)c < other) continue;
        a.parent[c] = other;
        const unsigned long long e = atomicAdd(a.ctrl, 1ull);
        if (e >= (unsigned long long)(a.R - 1)) {   // a forest has at most R - 1 edges: never expected
            atomicAdd(a.ctrl + 1, 1ull);
            continue;
        }
        a.edges[2 * e] = lo;
        a.edges[2 * e + 1] = hi;
    }
}

// each point's component becomes the root its old root's hooks lead to (the
// hooks form trees: of two components that picked the same edge one hooked)
__global__ void mst_relabel_kernel(MstArgs a)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.R; i += (int64_t)gridDim.x * blockDim.x) {
        int p = a.comp[i];
        int steps = 0;
        while (a.parent[p] != p && steps < kWalkLimit) {
            p = a.parent[p];
            ++steps;
        }
        if (steps >= kWalkLimit) atomicAdd(a.ctrl + 1, 1ull);
        a.comp[i] = p;
    }
}

// new roots: reset their hook and their picks for the next round
__global__ void mst_reset_kernel(MstArgs a)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.R; c += (int64_t)gridDim.x * blockDim.x) {
        a.parent[c] = (int)c;
        a.minw[c] = kNone;
        a.minij[c] = kNone;
    }
}

struct MstLayout {
    size_t grid, comp, parent, minw, minij, offs, offw, ctrl, total;
};

inline MstLayout mst_layout(int64_t R, int64_t cells, int n_off)
{
    MstLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.grid = take((size_t)cells * 4);
    L.comp = take((size_t)R * 4);
    L.parent = take((size_t)R * 4);
    L.minw = take((size_t)R * 8);
    L.minij = take((size_t)R * 8);
    L.offs = take((size_t)std::max(n_off, 1) * 12);
    L.offw = take((size_t)std::max(n_off, 1) * 8);
    L.ctrl = take(24);
    L.total = off;
    return L;
}

inline int blocks_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(16 * kSMs, div_up(n, 256))); }

// whether p * v is exact in double for every integer |p| <= maxabs: v's
// significand (53 bits) ends in at least as many zero bits as maxabs has
inline bool products_exact(double v, int64_t maxabs)
{
    if (!(v >= DBL_MIN) || !isfinite(v)) return false;
    int e = 0;
    const double m = frexp(v, &e);                        // v = m * 2^e, m in [0.5, 1)
    const uint64_t sig = (uint64_t)ldexp(m, 53);          // the 53-bit significand, exactly
    int tz = 0;
    while (tz < 53 && !((sig >> tz) & 1u)) ++tz;
    int bits = 0;
    while (bits < 63 && (maxabs >> bits) != 0) ++bits;
    return bits <= tz;
}

}  // namespace
}  // namespace m16

using namespace m16;

extern "C" size_t m16_ridge_mst_workspace_bytes(int64_t num_points, const int32_t *box_dims3, int32_t n_offsets)
{
    if (num_points < 1 || num_points > (int64_t)INT32_MAX || !box_dims3 || n_offsets < 0) return 0;
    if (box_dims3[0] < 1 || box_dims3[1] < 1 || box_dims3[2] < 1) return 0;
    return mst_layout(num_points, (int64_t)box_dims3[0] * box_dims3[1] * box_dims3[2], n_offsets).total;
}

extern "C" int m16_ridge_mst_local(const int32_t *pts3, int64_t num_points, const int32_t *box_lo3,
                                   const int32_t *box_dims3, const double *voxel_size3, const int32_t *offsets3,
                                   int32_t n_offsets, double r, int32_t *edges, int64_t *n_edges, void *workspace,
                                   size_t workspace_bytes, void *stream)
{
    if (num_points < 1 || num_points > (int64_t)INT32_MAX) return M16_ERR_BAD_SHAPE;
    if (!pts3 || !box_lo3 || !box_dims3 || !voxel_size3 || !edges || !n_edges || n_offsets < 0 ||
        (n_offsets > 0 && !offsets3) || !(r > 0.0))
        return M16_ERR_BAD_ARG;
    for (int k = 0; k < 3; ++k) {
        if (box_dims3[k] < 1) return M16_ERR_BAD_SHAPE;
        if (!(voxel_size3[k] > 0.0) || !isfinite(voxel_size3[k])) return M16_ERR_BAD_ARG;
    }
    const int64_t cells = (int64_t)box_dims3[0] * box_dims3[1] * box_dims3[2];
    const MstLayout L = mst_layout(num_points, cells, n_offsets);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    *n_edges = 0;
    if (num_points < 2) return M16_OK;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    MstArgs a;
    a.pts = pts3;
    a.R = num_points;
    a.lo0 = box_lo3[0]; a.lo1 = box_lo3[1]; a.lo2 = box_lo3[2];
    a.b0 = box_dims3[0]; a.b1 = box_dims3[1]; a.b2 = box_dims3[2];
    a.vs0 = voxel_size3[0]; a.vs1 = voxel_size3[1]; a.vs2 = voxel_size3[2];
    a.r = r;
    a.offs = (const int *)(ws + L.offs);
    a.n_off = n_offsets;
    a.offw = nullptr;
    a.grid = (const int *)(ws + L.grid);
    a.comp = (int *)(ws + L.comp);
    a.parent = (int *)(ws + L.parent);
    a.minw = (unsigned long long *)(ws + L.minw);
    a.minij = (unsigned long long *)(ws + L.minij);
    a.edges = edges;
    a.ctrl = (unsigned long long *)(ws + L.ctrl);
    if (n_offsets > 0)
        M16_CUDA_TRY(cudaMemcpyAsync(ws + L.offs, offsets3, (size_t)n_offsets * 12, cudaMemcpyHostToDevice, st));
    // the largest coordinate magnitude in the box and in the offsets
    int64_t maxabs = 0;
    for (int k = 0; k < 3; ++k) {
        maxabs = std::max<int64_t>(maxabs, std::llabs((int64_t)box_lo3[k]));
        maxabs = std::max<int64_t>(maxabs, std::llabs((int64_t)box_lo3[k] + box_dims3[k] - 1));
    }
    for (int64_t o = 0; o < 3 * (int64_t)n_offsets; ++o) maxabs = std::max<int64_t>(maxabs, std::llabs((int64_t)offsets3[o]));
    if (n_offsets > 0 && products_exact(voxel_size3[0], maxabs) && products_exact(voxel_size3[1], maxabs) &&
        products_exact(voxel_size3[2], maxabs)) {
        mst_offset_weights_kernel<<<1, 256, 0, st>>>(a, (double *)(ws + L.offw));
        a.offw = (const double *)(ws + L.offw);
    }
    M16_CUDA_TRY(cudaMemsetAsync(ws + L.grid, 0xff, (size_t)cells * 4, st));
    M16_CUDA_TRY(cudaMemsetAsync(a.ctrl, 0, 24, st));
    mst_grid_kernel<<<blocks_for(num_points), 256, 0, st>>>(a, (int *)(ws + L.grid));
    unsigned long long bad = 0;
    M16_CUDA_TRY(cudaMemcpyAsync(&bad, a.ctrl + 2, 8, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    if (bad != 0) return M16_ERR_BAD_ARG;   // points outside the box, or two points on one cell
    const int64_t total = num_points * (int64_t)n_offsets;
    unsigned long long h[2] = {0, 0}, before = 0;
    // every round at least halves the number of components that still have
    // an outgoing candidate edge, so 64 rounds are never reached
    for (int round = 0; round < 64 && n_offsets > 0; ++round) {
        mst_reset_kernel<<<blocks_for(num_points), 256, 0, st>>>(a);
        mst_min_kernel<0><<<blocks_for(total), 256, 0, st>>>(a);
        mst_min_kernel<1><<<blocks_for(total), 256, 0, st>>>(a);
        mst_hook_kernel<<<blocks_for(num_points), 256, 0, st>>>(a);
        mst_relabel_kernel<<<blocks_for(num_points), 256, 0, st>>>(a);
        M16_CUDA_TRY(cudaGetLastError());
        M16_CUDA_TRY(cudaMemcpyAsync(h, a.ctrl, 16, cudaMemcpyDeviceToHost, st));
        M16_CUDA_TRY(cudaStreamSynchronize(st));
        if (h[1] != 0) return M16_ERR_TIMEOUT;   // a walk did not end or the edges overflowed: never expected
        if (h[0] == before) break;
        before = h[0];
    }
    *n_edges = (int64_t)h[0];
    return M16_OK;
}
