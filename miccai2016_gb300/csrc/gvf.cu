// gvf.cu -- gradient vector flow (Xu & Prince), the GB300 replacement of the
// reference's gvfDelta / gvfUpdate / magDelta / gvfNormalize / response
// kernels (src/clcode/gvf.cl:44-253) and of the loop in GvfGpu._execute
// (src/processing/gradient_vector_flow.py:179-232).
//
// One fused sweep per iteration: g_out = g - dt * (r * (g - v) - mu * lap(g))
// with the 7-point mirror-boundary Laplacian, reading g from one planar
// buffer and writing the other (ping-pong), r = |v|^2 recomputed from v (or
// read when the caller gives a response).  On check iterations the sweep
// also sums |delta| per block for the convergence criterion.
//
// Workspace: v0, v1, v2 (planar copies of the interleaved field), r (only
// with a caller response), g_a[3], g_b[3], block partials, control word,
// magnitude log.  Per voxel-iteration the sweep moves g 12 + v 12 (+ r 4)
// read and g 12 written.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "common.cuh"

namespace m16 {
namespace {

struct GvfCtrl {
    int stopped;
    int iterations;
    int n_checks;
    int pad;
};

struct GvfArgs {
    int d0, d1, d2, zc;
    float mu, dt, rss0, rss1, rss2;
    const float *v0, *v1, *v2, *r;
    const float *gi0, *gi1, *gi2;
    float *go0, *go1, *go2;
    float *partials;
    GvfCtrl *ctrl;
};

constexpr int kBX = 32, kBY = 8;

__global__ void gvf_init_kernel(const float *__restrict__ v3, const float *__restrict__ resp, int64_t n,
                                float *v0, float *v1, float *v2, float *r, float *g0, float *g1, float *g2,
                                GvfCtrl *ctrl)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        v0[i] = v3[3 * i];
        v1[i] = v3[3 * i + 1];
        v2[i] = v3[3 * i + 2];
        if (resp) r[i] = resp[i];
        g0[i] = 0.f;
        g1[i] = 0.f;
        g2[i] = 0.f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctrl->stopped = 0;
        ctrl->iterations = 0;
        ctrl->n_checks = 0;
    }
}

// gvfDelta + gvfUpdate (+ magDelta partial sums), gvf.cl:44-99, 162-202.
// Each thread walks a z-column chunk; the loads of kGvfZB slices (the next
// slice, the four in-plane neighbours and v) are issued together before any
// of them is used, so each thread keeps several slices of loads in flight.
#ifndef M16_GVF_ZB
#define M16_GVF_ZB 2
#endif
#ifndef M16_GVF_MINB
#define M16_GVF_MINB 4   // 4 blocks per SM caps the sweep at 64 registers: measured fastest on GB300
#endif
constexpr int kGvfZB = M16_GVF_ZB;
// 1: the x neighbours come from the adjacent lanes (warp shuffles) instead of
// loads, except at the warp's ends.  Measured slower on GB300 (256^3, 100
// iterations: 12.64 ms against 12.27 ms with the loads, which hit L1), so off.
#ifndef M16_GVF_XSHFL
#define M16_GVF_XSHFL 0
#endif

template <bool RESP, bool CHECK>
__global__ void __launch_bounds__(kBX * kBY, M16_GVF_MINB) gvf_sweep_kernel(GvfArgs a)
{
    __shared__ float red[32];
    pdl_wait();          // programmatic dependent launch (common.cuh)
    pdl_launch_next();
    if (__ldcg(&a.ctrl->stopped)) return;
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    float acc = 0.f;
#if M16_GVF_XSHFL
    const int lane = threadIdx.x;   // a warp is one 32-wide row of x (kBX = 32)
    const unsigned active = __ballot_sync(0xffffffffu, x < a.d2 && y < a.d1);
#endif
    if (x < a.d2 && y < a.d1) {
        const int z0 = blockIdx.z * a.zc;
        const int z1 = min(z0 + a.zc, a.d0);
        const int64_t s0 = (int64_t)a.d1 * a.d2;
        // mirror neighbours along y and x (an axis of length 1 has none)
        const int64_t yb = a.d1 > 1 ? (y > 0 ? -(int64_t)a.d2 : (int64_t)a.d2) : 0;
        const int64_t ya = a.d1 > 1 ? (y < a.d1 - 1 ? (int64_t)a.d2 : -(int64_t)a.d2) : 0;
        const int64_t xb = a.d2 > 1 ? (x > 0 ? -1 : 1) : 0;
        const int64_t xa = a.d2 > 1 ? (x < a.d2 - 1 ? 1 : -1) : 0;
        int64_t i = ((int64_t)z0 * a.d1 + y) * a.d2 + x;
        auto ld3 = [&](int64_t j, float &p, float &q, float &s) {
            p = __ldg(a.gi0 + j); q = __ldg(a.gi1 + j); s = __ldg(a.gi2 + j);
        };
        // carried along z: previous and current slice
        float c0, c1, c2, p0, p1, p2;
        ld3(i, c0, c1, c2);
        if (a.d0 == 1) { p0 = c0; p1 = c1; p2 = c2; }
        else if (z0 > 0) ld3(i - s0, p0, p1, p2);
        else ld3(i + s0, p0, p1, p2);   // mirror at z = 0
        for (int zb = z0; zb < z1; zb += kGvfZB, i += kGvfZB * s0) {
            float nx[kGvfZB][3], nyb[kGvfZB][3], nya[kGvfZB][3], nxb[kGvfZB][3], nxa[kGvfZB][3], w[kGvfZB][3],
                rr[kGvfZB];
#pragma unroll
            for (int k = 0; k < kGvfZB; ++k) {
                const int z = zb + k;
                if (z < z1) {
                    const int64_t j = i + k * s0;
                    if (z < a.d0 - 1) ld3(j + s0, nx[k][0], nx[k][1], nx[k][2]);   // z + 1
                    ld3(j + yb, nyb[k][0], nyb[k][1], nyb[k][2]);
                    ld3(j + ya, nya[k][0], nya[k][1], nya[k][2]);
#if M16_GVF_XSHFL
                    // only the warp's end lanes load their outer x neighbour
                    if (lane == 0 && x > 0) ld3(j - 1, nxb[k][0], nxb[k][1], nxb[k][2]);
                    if (lane == 31 && x < a.d2 - 1) ld3(j + 1, nxa[k][0], nxa[k][1], nxa[k][2]);
#else
                    ld3(j + xb, nxb[k][0], nxb[k][1], nxb[k][2]);
                    ld3(j + xa, nxa[k][0], nxa[k][1], nxa[k][2]);
#endif
                    w[k][0] = __ldg(a.v0 + j); w[k][1] = __ldg(a.v1 + j); w[k][2] = __ldg(a.v2 + j);
                    if (RESP) rr[k] = __ldg(a.r + j);
                }
            }
#pragma unroll
            for (int k = 0; k < kGvfZB; ++k) {
                const int z = zb + k;
                if (z < z1) {
                    const int64_t j = i + k * s0;
                    float n0, n1, n2;   // z + 1 (mirror at the last slice)
                    if (a.d0 == 1) { n0 = c0; n1 = c1; n2 = c2; }
                    else if (z < a.d0 - 1) { n0 = nx[k][0]; n1 = nx[k][1]; n2 = nx[k][2]; }
                    else { n0 = p0; n1 = p1; n2 = p2; }
#if M16_GVF_XSHFL
                    {
                        // x - 1 and x + 1 from the neighbouring lanes (the active
                        // lanes of a warp are 0 .. last, all in this branch)
                        const float cc[3] = {c0, c1, c2};
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            const float up = __shfl_up_sync(active, cc[q], 1);     // x - 1
                            const float dn = __shfl_down_sync(active, cc[q], 1);   // x + 1 (unused past the end)
                            float xbv, xav;
                            if (a.d2 == 1) { xbv = cc[q]; xav = cc[q]; }
                            else {
                                xbv = x == 0 ? dn : (lane == 0 ? nxb[k][q] : up);          // mirror at x = 0
                                xav = x == a.d2 - 1 ? (lane == 0 ? nxb[k][q] : up)          // mirror at the end
                                                    : (lane == 31 ? nxa[k][q] : dn);
                            }
                            nxb[k][q] = xbv;
                            nxa[k][q] = xav;
                        }
                    }
#endif
                    const float l0 = ((p0 + n0 - 2.f * c0) * a.rss0 + (nyb[k][0] + nya[k][0] - 2.f * c0) * a.rss1) +
                                     (nxb[k][0] + nxa[k][0] - 2.f * c0) * a.rss2;
                    const float l1 = ((p1 + n1 - 2.f * c1) * a.rss0 + (nyb[k][1] + nya[k][1] - 2.f * c1) * a.rss1) +
                                     (nxb[k][1] + nxa[k][1] - 2.f * c1) * a.rss2;
                    const float l2 = ((p2 + n2 - 2.f * c2) * a.rss0 + (nyb[k][2] + nya[k][2] - 2.f * c2) * a.rss1) +
                                     (nxb[k][2] + nxa[k][2] - 2.f * c2) * a.rss2;
                    const float w0 = w[k][0], w1 = w[k][1], w2 = w[k][2];
                    const float r = RESP ? rr[k] : w0 * w0 + w1 * w1 + w2 * w2;
                    const float e0 = r * (c0 - w0) - a.mu * l0;
                    const float e1 = r * (c1 - w1) - a.mu * l1;
                    const float e2 = r * (c2 - w2) - a.mu * l2;
                    a.go0[j] = c0 - a.dt * e0;
                    a.go1[j] = c1 - a.dt * e1;
                    a.go2[j] = c2 - a.dt * e2;
                    if (CHECK) acc += sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
                    p0 = c0; p1 = c1; p2 = c2;
                    c0 = n0; c1 = n1; c2 = n2;
                }
            }
        }
    }
    if (CHECK) {
        const float s = block_sum(acc, red);
        if (threadIdx.x == 0 && threadIdx.y == 0)
            a.partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
    }
}

// mean |delta| and the tolerance test (gradient_vector_flow.py:459-478)
__global__ void gvf_check_kernel(const float *__restrict__ part, int nparts, double inv_n, double tol, int iter,
                                 int check_idx, int cap, GvfCtrl *ctrl, double *mags)
{
    __shared__ double s[256];
    pdl_wait();
    pdl_launch_next();
    if (__ldcg(&ctrl->stopped)) return;
    double acc = 0.0;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) acc += (double)part[k];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double mag = s[0] * inv_n;
        if (check_idx < cap) mags[check_idx] = mag;
        ctrl->n_checks = check_idx + 1;
        if (mag < tol) {
            ctrl->stopped = 1;
            ctrl->iterations = iter + 1;
        }
    }
}

// interleave (and optionally normalise, gvf.cl:215-232) the current field
__global__ void gvf_output_kernel(const float *__restrict__ g0, const float *__restrict__ g1,
                                  const float *__restrict__ g2, int64_t n, int normalize, float *__restrict__ g3)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float a = g0[i], b = g1[i], c = g2[i];
        if (normalize) {
            float nrm = sqrtf(a * a + b * b + c * c);
            if (nrm != 0.f) {
                nrm = 1.f / nrm;
                a *= nrm; b *= nrm; c *= nrm;
            }
        }
        g3[3 * i] = a;
        g3[3 * i + 1] = b;
        g3[3 * i + 2] = c;
    }
}

struct GvfLayout {
    size_t v, r, ga, gb, partials, ctrl, mags, total;
    int nparts, cap;
};

inline int gvf_zc(int d0, int d1, int d2)
{
    const int64_t cols = div_up(d2, kBX) * div_up(d1, kBY);
    int64_t zc = (int64_t)d0 * cols / (8 * kSMs);
    zc = std::max<int64_t>(1, std::min<int64_t>(16, zc));
    if (zc >= kGvfZB) zc = zc / kGvfZB * kGvfZB;   // whole load batches
    return (int)zc;
}

inline GvfLayout gvf_layout(int d0, int d1, int d2, int has_response, int mags_cap)
{
    GvfLayout L;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const int zc = gvf_zc(d0, d1, d2);
    L.nparts = (int)(div_up(d2, kBX) * div_up(d1, kBY) * div_up(d0, zc));
    L.cap = std::max(mags_cap, 1);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.v = take(3 * n * 4);
    L.r = has_response ? take(n * 4) : 0;
    L.ga = take(3 * n * 4);
    L.gb = take(3 * n * 4);
    L.partials = take((size_t)L.nparts * 4);
    L.ctrl = take(sizeof(GvfCtrl));
    L.mags = take((size_t)L.cap * 8);
    L.total = off;
    return L;
}

}  // namespace
}  // namespace m16

using namespace m16;

extern "C" size_t m16_gvf_workspace_bytes(int32_t d0, int32_t d1, int32_t d2, int32_t has_response,
                                          int32_t mags_cap)
{
    if (d0 < 1 || d1 < 1 || d2 < 1) return 0;
    return gvf_layout(d0, d1, d2, has_response, mags_cap).total;
}

extern "C" int m16_gvf_run(const float *v3, const float *response, int32_t d0, int32_t d1, int32_t d2,
                           const double *voxel_size, double mu, double dt, int32_t first_iter, int32_t n_iters,
                           int32_t update, double tol, int32_t normalize, float *g3, int32_t *iterations,
                           int32_t *stopped, double *mags, int32_t mags_cap, int32_t *n_mags, void *workspace,
                           size_t workspace_bytes, void *stream)
{
    if (d0 < 1 || d1 < 1 || d2 < 1) return M16_ERR_BAD_SHAPE;
    if ((int64_t)d0 * d1 * d2 > ((int64_t)1 << 34)) return M16_ERR_BAD_SHAPE;
    if (!v3 || !g3 || !voxel_size) return M16_ERR_BAD_ARG;
    if (update < 1 || first_iter < 0 || n_iters < 0 || !(dt > 0.0) || !(mu >= 0.0)) return M16_ERR_BAD_ARG;
    for (int k = 0; k < 3; ++k)
        if (!(voxel_size[k] > 0.0)) return M16_ERR_BAD_ARG;
    const GvfLayout L = gvf_layout(d0, d1, d2, response != nullptr, mags_cap);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    const int64_t n = (int64_t)d0 * d1 * d2;
    float *v = (float *)(ws + L.v);
    float *ga = (float *)(ws + L.ga);
    float *gb = (float *)(ws + L.gb);
    float *r = response ? (float *)(ws + L.r) : nullptr;
    GvfCtrl *ctrl = (GvfCtrl *)(ws + L.ctrl);
    double *mlog = (double *)(ws + L.mags);
    const int blocks1d = (int)std::min<int64_t>(4 * kSMs, div_up(n, 256));
    if (first_iter == 0) {
        gvf_init_kernel<<<blocks1d, 256, 0, st>>>(v3, response, n, v, v + n, v + 2 * n, r, ga, ga + n, ga + 2 * n,
                                                  ctrl);
        M16_CUDA_TRY(cudaGetLastError());
    }
    GvfArgs a;
    a.d0 = d0; a.d1 = d1; a.d2 = d2; a.zc = gvf_zc(d0, d1, d2);
    a.mu = (float)mu; a.dt = (float)dt;
    a.rss0 = (float)(1.0 / (voxel_size[0] * voxel_size[0]));
    a.rss1 = (float)(1.0 / (voxel_size[1] * voxel_size[1]));
    a.rss2 = (float)(1.0 / (voxel_size[2] * voxel_size[2]));
    a.v0 = v; a.v1 = v + n; a.v2 = v + 2 * n; a.r = r;
    a.partials = (float *)(ws + L.partials);
    a.ctrl = ctrl;
    const dim3 block(kBX, kBY, 1);
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)div_up(d0, a.zc));
    const double inv_n = 1.0 / (double)n;
    for (int k = 0; k < n_iters; ++k) {
        const int it = first_iter + k;
        float *in = (it & 1) ? gb : ga;
        float *out = (it & 1) ? ga : gb;
        a.gi0 = in; a.gi1 = in + n; a.gi2 = in + 2 * n;
        a.go0 = out; a.go1 = out + n; a.go2 = out + 2 * n;
        const bool check = (it % update) == 0;
        // programmatic dependent launch: each sweep waits on the device for
        // the previous one (which reads the buffer it writes) before any access
        if (check) {
            if (response) M16_CUDA_TRY(launch_pdl(gvf_sweep_kernel<true, true>, grid, block, st, true, a));
            else M16_CUDA_TRY(launch_pdl(gvf_sweep_kernel<false, true>, grid, block, st, true, a));
            M16_CUDA_TRY(launch_pdl(gvf_check_kernel, dim3(1), dim3(256), st, true, (const float *)a.partials,
                                    L.nparts, inv_n, tol, it, it / update, L.cap, ctrl, mlog));
        } else {
            if (response) M16_CUDA_TRY(launch_pdl(gvf_sweep_kernel<true, false>, grid, block, st, true, a));
            else M16_CUDA_TRY(launch_pdl(gvf_sweep_kernel<false, false>, grid, block, st, true, a));
        }
    }
    M16_CUDA_TRY(cudaGetLastError());
    GvfCtrl h;
    M16_CUDA_TRY(cudaMemcpyAsync(&h, ctrl, sizeof(h), cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    const int done = h.stopped ? h.iterations : first_iter + n_iters;   // total iterations so far
    const float *cur = (done & 1) ? gb : ga;
    gvf_output_kernel<<<blocks1d, 256, 0, st>>>(cur, cur + n, cur + 2 * n, n, normalize, g3);
    M16_CUDA_TRY(cudaGetLastError());
    if (iterations) *iterations = done;
    if (stopped) *stopped = h.stopped;
    if (n_mags) *n_mags = h.n_checks;
    if (mags && mags_cap > 0) {
        const int cnt = std::min(std::min(h.n_checks, mags_cap), L.cap);
        if (cnt > 0) M16_CUDA_TRY(cudaMemcpyAsync(mags, mlog, (size_t)cnt * 8, cudaMemcpyDeviceToHost, st));
    }
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    return M16_OK;
}
