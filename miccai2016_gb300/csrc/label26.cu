// label26.cu -- connected components of a binary volume on the GPU under 26-
// or 6-connectivity, numbered exactly as scipy.ndimage.label numbers them
// (with a 3 x 3 x 3 structure of ones, or its default cross).  The sign
// adjustment labels its ridge with 26-connectivity twice: the hysteresis
// (src/processing/ridge_detection.py:80-131: the union of the 26-connected
// candidate components holding a sure voxel) and the ridge cleaning
// (src/processing/adjust_directions.py:290-339).  The experiment's Dice of
// the largest component (src/phantom_experiment.py:52-103, select_largest +
// dice_for) labels the thresholded segmentation with the default
// 6-connectivity: m16_dice_largest below.
//
// Union-find over voxel indices: every foreground voxel starts as its own
// root; for each of its 13 forward neighbours a lock-free union hooks the
// larger of the two roots onto the smaller, so every component
// ends with the smallest linear index of its voxels as root (a root is
// hooked only while it is still a root, by compare-and-swap).  SciPy numbers
// components 1, 2, ... in the raster order of their first voxel, which is the
// order of those smallest indices: a component's label is one plus the number
// of roots before its root, an exclusive scan of the root flags.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "common.cuh"

namespace m16 {
namespace {

constexpr int kFindLimit = 1 << 26;   // pointer walks never get this long: a bound, not a wait

__device__ __forceinline__ int find_root(const int *parent, int i, unsigned long long *err)
{
    int steps = 0;
    int p = parent[i];
    while (p != i) {
        i = p;
        p = parent[i];
        if (++steps > kFindLimit) { atomicAdd(err, 1ull); break; }
    }
    return i;
}

__global__ void lb_init_kernel(const uint8_t *__restrict__ mask, int64_t n, int *__restrict__ parent)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        parent[i] = mask[i] ? (int)i : -1;
}

// union of each foreground voxel with its forward neighbours: the forward
// half of the 26-neighbourhood ((dz, dy, dx) > (0, 0, 0) in offsets k = 14..26
// of the 3 x 3 x 3 cube, k = 9 (dz + 1) + 3 (dy + 1) + dx + 1), or of the
// 6-neighbourhood (k = 14, 16, 22: +x, +y, +z)
template <int CONN>
__global__ void lb_union_kernel(const uint8_t *__restrict__ mask, int d0, int d1, int d2, int *parent,
                                unsigned long long *err)
{
    const int64_t s0 = (int64_t)d1 * d2, n = s0 * d0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!mask[i]) continue;
        const int z = (int)(i / s0), y = (int)((i / d2) % d1), x = (int)(i % d2);
        for (int t = 0; t < (CONN == 26 ? 13 : 3); ++t) {
            const int k = CONN == 26 ? 14 + t : (t == 0 ? 14 : t == 1 ? 16 : 22);
            const int dz = k / 9 - 1, dy = (k / 3) % 3 - 1, dx = k % 3 - 1;
            const int zz = z + dz, yy = y + dy, xx = x + dx;
            if (zz >= d0 || yy < 0 || yy >= d1 || xx < 0 || xx >= d2) continue;
            const int64_t j = i + (int64_t)dz * s0 + (int64_t)dy * d2 + dx;
            if (!mask[j]) continue;
            int a = find_root(parent, (int)i, err), b = find_root(parent, (int)j, err);
            int tries = 0;
            while (a != b && tries++ < kFindLimit) {
                if (a < b) { const int t = a; a = b; b = t; }   // hook the larger root a onto b
                // only while a is still a root: re-pointing a hooked node
                // would cut its subtree off its set
                const int old = atomicCAS(parent + a, a, b);
                if (old == a) break;
                a = find_root(parent, old, err);               // a was hooked meanwhile: retry from the roots
                b = find_root(parent, b, err);
            }
            if (tries >= kFindLimit) atomicAdd(err, 1ull);
        }
    }
}

// every voxel points at its root; roots are flagged for the numbering
__global__ void lb_compress_kernel(int64_t n, int *parent, unsigned *__restrict__ is_root, unsigned long long *err)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = parent[i];
        if (p < 0) { is_root[i] = 0u; continue; }
        const int r = find_root(parent, (int)i, err);
        parent[i] = r;
        is_root[i] = r == (int)i ? 1u : 0u;
    }
}

// exclusive scan of the root flags in blocks of 1024, then of the block sums
constexpr int kScan = 1024;

__global__ void __launch_bounds__(256) lb_scan_local_kernel(const unsigned *__restrict__ flag, int64_t n,
                                                            unsigned *__restrict__ rank, unsigned *__restrict__ bsum)
{
    __shared__ unsigned s[256];
    const int64_t base = blockIdx.x * (int64_t)kScan + 4 * threadIdx.x;
    unsigned v[4], t = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < n ? flag[base + k] : 0u;
        t += v[k];
    }
    s[threadIdx.x] = t;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
        const unsigned add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
        __syncthreads();
        s[threadIdx.x] += add;
        __syncthreads();
    }
    unsigned run = s[threadIdx.x] - t;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) rank[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 255) bsum[blockIdx.x] = s[255];
}

// sequential exclusive scan of the block sums by one block, 1024 per pass
__global__ void __launch_bounds__(1024) lb_scan_blocks_kernel(unsigned *bsum, int64_t nblocks, unsigned *total)
{
    __shared__ unsigned s[1024];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (int64_t base = 0; base < nblocks; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const unsigned v = i < nblocks ? bsum[i] : 0u;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const unsigned add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
            __syncthreads();
            s[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < nblocks) bsum[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += s[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// labels = 1 + rank of the voxel's root (0 on the background)
__global__ void lb_number_kernel(const int *__restrict__ parent, const unsigned *__restrict__ rank,
                                 const unsigned *__restrict__ bsum, int64_t n, int32_t *__restrict__ labels)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = parent[i];
        labels[i] = r < 0 ? 0 : (int32_t)(rank[r] + bsum[r / kScan] + 1u);
    }
}

struct LbLayout {
    size_t parent, flag, rank, bsum, ctrl, total;
    int64_t nblocks;
};

inline LbLayout lb_layout(int64_t n)
{
    LbLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.nblocks = div_up(n, kScan);
    L.parent = take((size_t)n * 4);
    L.flag = take((size_t)n * 4);
    L.rank = take((size_t)n * 4);
    L.bsum = take((size_t)(L.nblocks + 1) * 4);
    L.ctrl = take(16);
    L.total = off;
    return L;
}

inline int lb_blocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(16 * kSMs, div_up(n, 256))); }

// the labelling's launches on a laid-out workspace; ctrl[0] counts walk-limit
// errors, the component count lands at ctrl + 1 (as unsigned)
inline int label_launch(const uint8_t *mask, int32_t d0, int32_t d1, int32_t d2, int conn, int32_t *labels,
                        char *ws, const LbLayout &L, cudaStream_t st)
{
    const int64_t n = (int64_t)d0 * d1 * d2;
    int *parent = (int *)(ws + L.parent);
    unsigned *flag = (unsigned *)(ws + L.flag), *rank = (unsigned *)(ws + L.rank), *bsum = (unsigned *)(ws + L.bsum);
    unsigned long long *ctrl = (unsigned long long *)(ws + L.ctrl);
    M16_CUDA_TRY(cudaMemsetAsync(ctrl, 0, 16, st));
    lb_init_kernel<<<lb_blocks(n), 256, 0, st>>>(mask, n, parent);
    if (conn == 26) lb_union_kernel<26><<<lb_blocks(n), 256, 0, st>>>(mask, d0, d1, d2, parent, ctrl);
    else lb_union_kernel<6><<<lb_blocks(n), 256, 0, st>>>(mask, d0, d1, d2, parent, ctrl);
    lb_compress_kernel<<<lb_blocks(n), 256, 0, st>>>(n, parent, flag, ctrl);
    lb_scan_local_kernel<<<(unsigned)L.nblocks, 256, 0, st>>>(flag, n, rank, bsum);
    lb_scan_blocks_kernel<<<1, 1024, 0, st>>>(bsum, L.nblocks, (unsigned *)(ctrl + 1));
    lb_number_kernel<<<lb_blocks(n), 256, 0, st>>>(parent, rank, bsum, n, labels);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

// ---- Dice of the largest 6-connected component ------------------------------

// mask = seg >= threshold (NaN is background, as numpy's comparison); the
// ground truth's voxel count (nonzero = 1) into *truth_count
__global__ void dl_binarize_kernel(const float *__restrict__ seg, const uint8_t *__restrict__ truth, int64_t n,
                                   float threshold, uint8_t *__restrict__ mask, unsigned long long *truth_count)
{
    unsigned c = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        mask[i] = seg[i] >= threshold ? 1 : 0;
        c += truth[i] != 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(truth_count, (unsigned long long)c);
}

// voxels per label; the lanes of a warp with the same label add once
__global__ void dl_sizes_kernel(const int32_t *__restrict__ labels, int64_t n, unsigned *__restrict__ sizes)
{
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const int32_t l = i < n ? labels[i] : 0;
        const unsigned same = __match_any_sync(0xffffffffu, l);
        const int leader = __ffs(same) - 1;
        if (l > 0 && (int)(threadIdx.x & 31) == leader) atomicAdd(sizes + l, (unsigned)__popc(same));
    }
}

// the largest component, the lowest label among equal sizes (select_largest
// keeps the first label whose size is strictly larger): max of
// size * 2^32 + (2^32 - 1 - label)
__global__ void dl_argmax_kernel(const unsigned *__restrict__ sizes, const unsigned *__restrict__ n_labels,
                                 unsigned long long *best)
{
    const unsigned nl = *n_labels;
    unsigned long long m = 0;
    for (unsigned l = 1 + blockIdx.x * blockDim.x + threadIdx.x; l <= nl; l += gridDim.x * blockDim.x)
        m = max(m, ((unsigned long long)sizes[l] << 32) | (unsigned long long)(0xffffffffu - l));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(best, m);
}

// voxels of the largest component inside the ground truth
__global__ void dl_intersect_kernel(const int32_t *__restrict__ labels, const uint8_t *__restrict__ truth, int64_t n,
                                    const unsigned long long *best, unsigned long long *inter)
{
    const unsigned long long b = *best;
    if (!b) return;
    const int32_t want = (int32_t)(0xffffffffu - (unsigned)(b & 0xffffffffu));
    unsigned c = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        c += labels[i] == want && truth[i] != 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(inter, (unsigned long long)c);
}

// ---- hysteresis: the candidate components that hold a sure voxel -------------

__global__ void hy_union_mask_kernel(const uint8_t *__restrict__ cand, const uint8_t *__restrict__ sure, int64_t n,
                                     uint8_t *__restrict__ both)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        both[i] = (cand[i] | sure[i]) ? 1 : 0;
}

// flag[label] = 1 for every label holding a sure voxel
__global__ void hy_flag_kernel(const int32_t *__restrict__ labels, const uint8_t *__restrict__ sure, int64_t n,
                               uint8_t *__restrict__ flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (sure[i]) flag[labels[i]] = 1;   // every writer stores 1: no atomics needed
}

__global__ void hy_select_kernel(const int32_t *__restrict__ labels, const uint8_t *__restrict__ flag, int64_t n,
                                 uint8_t *__restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = labels[i];
        out[i] = l > 0 && flag[l] ? 1 : 0;
    }
}

struct DlLayout {
    LbLayout lb;
    size_t mask, labels, sizes, ctrl, total;
};

inline DlLayout dl_layout(int64_t n)
{
    DlLayout D;
    D.lb = lb_layout(n);
    size_t off = D.lb.total;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    D.mask = take((size_t)n);
    D.labels = take((size_t)n * 4);
    D.sizes = take((size_t)(n + 1) * 4);
    D.ctrl = take(64);   // truth count, best key, intersection
    D.total = off;
    return D;
}

inline bool label_shape_ok(int32_t d0, int32_t d1, int32_t d2)
{
    return d0 >= 1 && d1 >= 1 && d2 >= 1 && (int64_t)d0 * d1 * d2 <= (int64_t)INT32_MAX - 1;
}

}  // namespace
}  // namespace m16

using namespace m16;

extern "C" size_t m16_label26_workspace_bytes(int32_t d0, int32_t d1, int32_t d2)
{
    if (!label_shape_ok(d0, d1, d2)) return 0;
    return lb_layout((int64_t)d0 * d1 * d2).total;
}

extern "C" size_t m16_label_workspace_bytes(int32_t d0, int32_t d1, int32_t d2)
{
    return m16_label26_workspace_bytes(d0, d1, d2);
}

extern "C" int m16_label(const uint8_t *mask, int32_t d0, int32_t d1, int32_t d2, int32_t connectivity,
                         int32_t *labels, int32_t *n_labels, void *workspace, size_t workspace_bytes, void *stream)
{
    if (!label_shape_ok(d0, d1, d2)) return M16_ERR_BAD_SHAPE;
    if (!mask || !labels || !n_labels || (connectivity != 6 && connectivity != 26)) return M16_ERR_BAD_ARG;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const LbLayout L = lb_layout(n);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    const int r = label_launch(mask, d0, d1, d2, connectivity, labels, ws, L, st);
    if (r != M16_OK) return r;
    unsigned long long h[2] = {0, 0};
    M16_CUDA_TRY(cudaMemcpyAsync(h, ws + L.ctrl, 16, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    if (h[0] != 0) return M16_ERR_TIMEOUT;   // a root walk hit its bound: never expected
    *n_labels = (int32_t)(h[1] & 0xffffffffu);
    return M16_OK;
}

extern "C" int m16_label26(const uint8_t *mask, int32_t d0, int32_t d1, int32_t d2, int32_t *labels,
                           int32_t *n_labels, void *workspace, size_t workspace_bytes, void *stream)
{
    return m16_label(mask, d0, d1, d2, 26, labels, n_labels, workspace, workspace_bytes, stream);
}

extern "C" size_t m16_dice_largest_workspace_bytes(int32_t d0, int32_t d1, int32_t d2)
{
    if (!label_shape_ok(d0, d1, d2)) return 0;
    return dl_layout((int64_t)d0 * d1 * d2).total;
}

extern "C" int m16_dice_largest(const float *seg, const uint8_t *truth, int32_t d0, int32_t d1, int32_t d2,
                                float threshold, double *dice, int64_t *largest_size, int32_t *n_components,
                                void *workspace, size_t workspace_bytes, void *stream)
{
    if (!label_shape_ok(d0, d1, d2)) return M16_ERR_BAD_SHAPE;
    if (!seg || !truth || !dice) return M16_ERR_BAD_ARG;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const DlLayout D = dl_layout(n);
    if (!workspace || workspace_bytes < D.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    uint8_t *mask = (uint8_t *)(ws + D.mask);
    int32_t *labels = (int32_t *)(ws + D.labels);
    unsigned *sizes = (unsigned *)(ws + D.sizes);
    unsigned long long *ctrl = (unsigned long long *)(ws + D.ctrl);   // [0] truth count, [1] best, [2] intersection
    M16_CUDA_TRY(cudaMemsetAsync(ctrl, 0, 64, st));
    M16_CUDA_TRY(cudaMemsetAsync(sizes, 0, (size_t)(n + 1) * 4, st));
    dl_binarize_kernel<<<lb_blocks(n), 256, 0, st>>>(seg, truth, n, threshold, mask, ctrl);
    const int r = label_launch(mask, d0, d1, d2, 6, labels, ws, D.lb, st);
    if (r != M16_OK) return r;
    const unsigned *nl = (const unsigned *)(ws + D.lb.ctrl + 8);
    dl_sizes_kernel<<<lb_blocks(n), 256, 0, st>>>(labels, n, sizes);
    dl_argmax_kernel<<<lb_blocks(n), 256, 0, st>>>(sizes, nl, ctrl + 1);
    dl_intersect_kernel<<<lb_blocks(n), 256, 0, st>>>(labels, truth, n, ctrl + 1, ctrl + 2);
    M16_CUDA_TRY(cudaGetLastError());
    unsigned long long h[3] = {0, 0, 0}, lh[2] = {0, 0};
    M16_CUDA_TRY(cudaMemcpyAsync(h, ctrl, 24, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaMemcpyAsync(lh, ws + D.lb.ctrl, 16, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    if (lh[0] != 0) return M16_ERR_TIMEOUT;
    const unsigned long long size = h[1] >> 32;
    if (n_components) *n_components = (int32_t)(lh[1] & 0xffffffffu);
    if (largest_size) *largest_size = (int64_t)size;
    // 2 |largest & truth| / (|largest| + |truth|) in double; no foreground gives 0
    // (the reference's select_largest returns None there and dice_for fails)
    const double den = (double)size + (double)h[0];
    *dice = size == 0 || den == 0.0 ? 0.0 : 2.0 * (double)h[2] / den;
    return M16_OK;
}

// The hysteresis of the sign adjustment (ridge_detection.py:80-131): the
// voxels of the 26-connected components of (cand | sure) that hold a sure
// voxel.  The workspace is m16_dice_largest's (mask, labels, per-label flags).
extern "C" size_t m16_hysteresis_workspace_bytes(int32_t d0, int32_t d1, int32_t d2)
{
    return m16_dice_largest_workspace_bytes(d0, d1, d2);
}

extern "C" int m16_hysteresis(const uint8_t *cand, const uint8_t *sure, int32_t d0, int32_t d1, int32_t d2,
                              uint8_t *out, void *workspace, size_t workspace_bytes, void *stream)
{
    if (!label_shape_ok(d0, d1, d2)) return M16_ERR_BAD_SHAPE;
    if (!cand || !sure || !out) return M16_ERR_BAD_ARG;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const DlLayout D = dl_layout(n);
    if (!workspace || workspace_bytes < D.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    uint8_t *both = (uint8_t *)(ws + D.mask);
    int32_t *labels = (int32_t *)(ws + D.labels);
    uint8_t *flag = (uint8_t *)(ws + D.sizes);   // n + 1 bytes of the (n + 1) * 4 size area
    hy_union_mask_kernel<<<lb_blocks(n), 256, 0, st>>>(cand, sure, n, both);
    const int r = label_launch(both, d0, d1, d2, 26, labels, ws, D.lb, st);
    if (r != M16_OK) return r;
    M16_CUDA_TRY(cudaMemsetAsync(flag, 0, (size_t)(n + 1), st));
    hy_flag_kernel<<<lb_blocks(n), 256, 0, st>>>(labels, sure, n, flag);
    hy_select_kernel<<<lb_blocks(n), 256, 0, st>>>(labels, flag, n, out);
    M16_CUDA_TRY(cudaGetLastError());
    unsigned long long h = 0;
    M16_CUDA_TRY(cudaMemcpyAsync(&h, ws + D.lb.ctrl, 8, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    return h != 0 ? M16_ERR_TIMEOUT : M16_OK;
}
