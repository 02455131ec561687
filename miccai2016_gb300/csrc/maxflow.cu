// maxflow.cu -- continuous max-flow with anisotropic total variation (ATV),
// the GB300 replacement of the reference's update_p / update_u / update_tmp
// kernels (src/clcode-anisotropic/update_qp.cl:150-316) and of the solve loop
// in CmfCutQAnisotropicGpu._execute
// (src/processing/continuous_cut_anisotropic_gpu.py:198-344).
//
// Data layout in HBM (one solve, N voxels, all fp32, C order z-y-x):
//   caller:    img, quat3 (N x 3), alpha (N or scalar), cs, ct, labels (u8), u (output/state)
//   workspace: hp0, hp1, hp2, pt, tmp (N each), q4 (N x float4, the expanded
//              quaternion), block partials, control word, residual log.
//
// Per iteration two kernels run:
//   P: hp <- project_alpha(H^-1 hp + steps * H^T grad(tmp)), hp <- H p
//   U: div(hp), p_s, p_t, u and tmp = err - u / cc (update_tmp fused), and on
//      check iterations the |err| partial sums of the residual.
// Each thread marches along z through a column of the volume; x/y neighbours
// come from L1, the z neighbour is carried in a register.  The quaternion is
// expanded once per solve so the iterations need no trigonometry.
#include <cuda_runtime.h>
#include <math.h>
#include <float.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <vector>

#include "common.cuh"
#include "sweeps.cuh"

namespace m16 {
namespace {

struct MfCtrl {
    int stopped;      // 1 once a check stopped the solve
    int iterations;   // iterations executed
    int n_checks;     // residual checks done
    int pad0;
    float denom;      // max(img) + FLT_MIN
    float pad1[3];
};

struct MfArgs {
    int d0, d1, d2, zc;
    float rcc, rs0, rs1, rs2, ss0, ss1, ss2;
    float sq0, sq1, sq2, isq0, isq1, isq2;
    float alpha_scalar;
    float *hp0, *hp1, *hp2, *tmp, *pt, *u;
    const float4 *q4;
    const float *alpha, *sqeigs, *cs, *ct;
    const uint8_t *labels;
    float *partials;
    MfCtrl *ctrl;
};

constexpr int kBX = 32, kBY = 8;

// ---- initialisation ------------------------------------------------------

__global__ void mf_max_kernel(const float *__restrict__ img, int64_t n, float *__restrict__ part)
{
    __shared__ float sm[32];
    __shared__ int snan;
    if (threadIdx.x == 0) snan = 0;
    __syncthreads();
    float m = -INFINITY;
    int nan = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = img[i];
        if (v != v) nan = 1; else m = fmaxf(m, v);
    }
    if (nan) snan = 1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = sm[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, sm[w]);
        part[blockIdx.x] = snan ? NAN : r;
    }
}

__global__ void mf_init_ctrl_kernel(const float *__restrict__ part, int nparts, int num_iter, MfCtrl *ctrl)
{
    if (threadIdx.x != 0) return;
    float m = -INFINITY;
    bool nan = false;
    for (int k = 0; k < nparts; ++k) {
        const float v = part[k];
        if (v != v) nan = true; else m = fmaxf(m, v);
    }
    ctrl->denom = (nan ? NAN : m) + FLT_MIN;   // np.max(img) + np.finfo(float32).tiny
    ctrl->stopped = 0;
    ctrl->iterations = num_iter;
    ctrl->n_checks = 0;
}

// hp = 0, p_t = fmin(cs, ct), u = img / denom, tmp = -u * rcc, q4 = qexpand(quat3)
// (continuous_cut_anisotropic_gpu.py:276-289)
__global__ void mf_init_kernel(MfArgs a, const float *__restrict__ img, const float *__restrict__ quat3, int64_t n)
{
    const float denom = a.ctrl->denom;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        a.hp0[i] = 0.f;
        a.hp1[i] = 0.f;
        a.hp2[i] = 0.f;
        a.pt[i] = fminf(a.cs[i], a.ct[i]);
        const float ui = img[i] / denom;
        a.u[i] = ui;
        a.tmp[i] = -(ui * a.rcc);
        const float *s = quat3 + 3 * i;
        const_cast<float4 *>(a.q4)[i] = qexpand(s[0], s[1], s[2]);
    }
}

// ---- P and U sweeps (bodies in sweeps.cuh, shared with the batched engine) --

// resident blocks per SM the sweeps are compiled for: 4 caps them at 64
// registers (the flow sweep needs 69 uncapped, which allows 3); measured on
// GB300 at 256^3 the capped flow sweep runs 0.861 of the HBM copy rate
// against 0.794 uncapped, the label sweep is unchanged
#ifndef M16_MF_MINB
#define M16_MF_MINB 4
#endif
constexpr int kZB = kMfZB > kMfUZB ? kMfZB : kMfUZB;   // z-chunks are whole load batches of both sweeps

__device__ __forceinline__ FlowView flow_view(const MfArgs &a)
{
    FlowView f;
    f.d0 = a.d0; f.d1 = a.d1; f.d2 = a.d2;
    f.ss0 = a.ss0; f.ss1 = a.ss1; f.ss2 = a.ss2;
    f.sq0 = a.sq0; f.sq1 = a.sq1; f.sq2 = a.sq2; f.isq0 = a.isq0; f.isq1 = a.isq1; f.isq2 = a.isq2;
    f.alpha_scalar = a.alpha_scalar; f.alpha = a.alpha; f.grad2 = nullptr; f.w = 0.f; f.neg_inv_decay2 = 0.f;
    f.sqeigs = a.sqeigs; f.q4 = a.q4; f.tmp = a.tmp; f.hp0 = a.hp0; f.hp1 = a.hp1; f.hp2 = a.hp2;
    return f;
}

__device__ __forceinline__ LabelView label_view(const MfArgs &a)
{
    LabelView l;
    l.d0 = a.d0; l.d1 = a.d1; l.d2 = a.d2;
    l.rcc = a.rcc; l.rs0 = a.rs0; l.rs1 = a.rs1; l.rs2 = a.rs2;
    l.hp0 = a.hp0; l.hp1 = a.hp1; l.hp2 = a.hp2; l.cs = a.cs; l.ct = a.ct; l.labels = a.labels;
    l.pt = a.pt; l.u = a.u; l.tmp = a.tmp;
    return l;
}

template <bool POINTWISE, bool ALPHA_ARR>
__global__ void __launch_bounds__(kBX * kBY, M16_MF_MINB) mf_update_p_kernel(MfArgs a)
{
    pdl_wait();
    pdl_launch_next();
    if (__ldcg(&a.ctrl->stopped)) return;
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    if (x >= a.d2 || y >= a.d1) return;
    const int z0 = blockIdx.z * a.zc;
    flow_column<POINTWISE, ALPHA_ARR ? kAlphaArray : kAlphaScalar>(flow_view(a), x, y, z0, min(z0 + a.zc, a.d0));
}

template <bool SUPERVISED, bool CHECK>
__global__ void __launch_bounds__(kBX * kBY, M16_MF_MINB) mf_update_u_kernel(MfArgs a)
{
    __shared__ float red[32];
    pdl_wait();
    pdl_launch_next();
    if (__ldcg(&a.ctrl->stopped)) return;
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    float acc = 0.f;
    if (x < a.d2 && y < a.d1) {
        const int z0 = blockIdx.z * a.zc;
        acc = label_column<SUPERVISED>(label_view(a), x, y, z0, min(z0 + a.zc, a.d0));
    }
    if (CHECK) {
        const float s = block_sum(acc, red);
        if (threadIdx.x == 0 && threadIdx.y == 0)
            a.partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
    }
}

// residual = sum(partials) / (N * rcc); stop on NaN or below the bound
// (continuous_cut_anisotropic_gpu.py:321-337)
__global__ void mf_check_kernel(const float *__restrict__ part, int nparts, double inv_norm, double bound,
                                int iter, int check_idx, int resid_cap, MfCtrl *ctrl, double *resid)
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
        const double err = s[0] * inv_norm;
        if (check_idx < resid_cap) resid[check_idx] = err;
        ctrl->n_checks = check_idx + 1;
        if (isnan(err) || err < bound) {
            ctrl->stopped = 1;
            ctrl->iterations = iter + 1;
        }
    }
}

// ---- host side --------------------------------------------------------------

struct MfLayout {
    size_t hp0, hp1, hp2, pt, tmp, q4, partials, maxpart, ctrl, resid, total;
    int nparts, resid_cap;
};

constexpr int kMaxBlocks = 4 * kSMs;

// z-slices per thread: enough blocks for 8 per SM, at most 16, a multiple of
// the load batch once it reaches it
inline int choose_zc(int d0, int d1, int d2)
{
    const int64_t cols = div_up(d2, kBX) * div_up(d1, kBY);
    int64_t zc = (int64_t)d0 * cols / (8 * kSMs);
    if (zc < 1) zc = 1;
    if (zc > 16) zc = 16;
    if (zc >= kZB) zc = zc / kZB * kZB;
    return (int)zc;
}

// the two-sweep state, the expanded quaternions, the block partials and the
// residual log
inline MfLayout mf_layout(int d0, int d1, int d2, int num_iter, int update)
{
    MfLayout L;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const int zc = choose_zc(d0, d1, d2);
    L.nparts = (int)(div_up(d2, kBX) * div_up(d1, kBY) * div_up(d0, zc));
    L.resid_cap = num_iter / (update > 0 ? update : 1) + 2;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.hp0 = take(n * 4); L.hp1 = take(n * 4); L.hp2 = take(n * 4);
    L.pt = take(n * 4); L.tmp = take(n * 4);
    L.q4 = take(n * 16);
    L.partials = take((size_t)L.nparts * 4);
    L.maxpart = take(kMaxBlocks * 4);
    L.ctrl = take(sizeof(MfCtrl));
    L.resid = take((size_t)L.resid_cap * 8);
    L.total = off;
    return L;
}

inline bool finite_pos(double v) { return v > 0.0 && v < 1e300; }

}  // namespace
}  // namespace m16

using namespace m16;

extern "C" size_t m16_maxflow_workspace_bytes(int32_t d0, int32_t d1, int32_t d2, const m16_cut_params *params)
{
    if (d0 < 1 || d1 < 1 || d2 < 1 || !params) return 0;
    return mf_layout(d0, d1, d2, params->num_iter, params->update).total;
}

extern "C" int m16_maxflow_solve(const float *img, const float *quat3, const double *sqevals3,
                                 const float *sqeigs, const float *alpha, float alpha_scalar,
                                 const float *cs, const float *ct, const uint8_t *labels,
                                 int32_t d0, int32_t d1, int32_t d2, const m16_cut_params *params,
                                 float *u, int32_t *iterations, double *residuals, int32_t residuals_cap,
                                 int32_t *n_residuals, void *workspace, size_t workspace_bytes, void *stream)
{
    return m16_maxflow_solve_ex(img, quat3, sqevals3, sqeigs, alpha, alpha_scalar, cs, ct, labels, d0, d1, d2,
                                params, u, iterations, residuals, residuals_cap, n_residuals, workspace,
                                workspace_bytes, stream, nullptr);
}

namespace {
// A pool of CUDA events bracketing the P/U launches of one chunk of iterations.
struct EventPool {
    std::vector<cudaEvent_t> ev;
    int used = 0;
    bool ok = true;
    explicit EventPool(int n) : ev(n, nullptr)
    {
        for (auto &e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) { ok = false; e = nullptr; }
    }
    ~EventPool()
    {
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
};
}  // namespace

// The solve: every iteration a flow and a label launch.
static int maxflow_solve_impl(const float *img, const float *quat3, const double *sqevals3, const float *sqeigs,
                              const float *alpha, float alpha_scalar, const float *cs, const float *ct,
                              const uint8_t *labels, int32_t d0, int32_t d1, int32_t d2,
                              const m16_cut_params *params, float *u, int32_t *iterations, double *residuals,
                              int32_t residuals_cap, int32_t *n_residuals, void *workspace, size_t workspace_bytes,
                              void *stream, m16_solve_stats *stats)
{
    if (d0 < 1 || d1 < 1 || d2 < 1) return M16_ERR_BAD_SHAPE;
    if ((int64_t)d0 * d1 * d2 > ((int64_t)1 << 34)) return M16_ERR_BAD_SHAPE;
    if (!params || !img || !quat3 || !cs || !ct || !u || !iterations) return M16_ERR_BAD_ARG;
    if (!sqevals3 && !sqeigs) return M16_ERR_BAD_ARG;
    if (params->update < 1 || params->num_iter < 0) return M16_ERR_BAD_ARG;
    if (!(params->cc > 0.0) || !(params->steps >= 0.0)) return M16_ERR_BAD_ARG;
    for (int k = 0; k < 3; ++k)
        if (!finite_pos(params->scaling[k])) return M16_ERR_BAD_ARG;
    if (sqevals3)
        for (int k = 0; k < 3; ++k)
            if (!finite_pos(sqevals3[k])) return M16_ERR_BAD_ARG;
    const MfLayout L = mf_layout(d0, d1, d2, params->num_iter, params->update);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    const int64_t n = (int64_t)d0 * d1 * d2;

    // constants as _reinit_clprograms derives them (continuous_cut_anisotropic_gpu.py:104-129)
    const double *sc = params->scaling;
    const double smin = fmin(sc[0], fmin(sc[1], sc[2]));
    const double rcc = 1.0 / (params->cc * (smin * smin));
    MfArgs a;
    a.d0 = d0; a.d1 = d1; a.d2 = d2; a.zc = choose_zc(d0, d1, d2);
    a.rcc = (float)rcc;
    a.rs0 = (float)(1.0 / sc[0]); a.rs1 = (float)(1.0 / sc[1]); a.rs2 = (float)(1.0 / sc[2]);
    a.ss0 = (float)(params->steps / sc[0] * (smin * smin));
    a.ss1 = (float)(params->steps / sc[1] * (smin * smin));
    a.ss2 = (float)(params->steps / sc[2] * (smin * smin));
    const double sqd[3] = {sqevals3 ? sqevals3[0] : 1.0, sqevals3 ? sqevals3[1] : 1.0, sqevals3 ? sqevals3[2] : 1.0};
    a.sq0 = (float)sqd[0]; a.sq1 = (float)sqd[1]; a.sq2 = (float)sqd[2];
    a.isq0 = (float)(1.0 / sqd[0]); a.isq1 = (float)(1.0 / sqd[1]); a.isq2 = (float)(1.0 / sqd[2]);
    a.alpha_scalar = alpha_scalar;
    a.hp0 = (float *)(ws + L.hp0); a.hp1 = (float *)(ws + L.hp1); a.hp2 = (float *)(ws + L.hp2);
    a.pt = (float *)(ws + L.pt); a.tmp = (float *)(ws + L.tmp); a.u = u;
    a.q4 = (const float4 *)(ws + L.q4);
    a.alpha = alpha; a.sqeigs = sqeigs; a.cs = cs; a.ct = ct; a.labels = labels;
    a.partials = (float *)(ws + L.partials);
    a.ctrl = (MfCtrl *)(ws + L.ctrl);
    double *resid = (double *)(ws + L.resid);

    const int init_blocks = (int)std::min<int64_t>(kMaxBlocks, div_up(n, 256));
    mf_max_kernel<<<init_blocks, 256, 0, st>>>(img, n, (float *)(ws + L.maxpart));
    mf_init_ctrl_kernel<<<1, 32, 0, st>>>((float *)(ws + L.maxpart), init_blocks, params->num_iter, a.ctrl);
    mf_init_kernel<<<init_blocks, 256, 0, st>>>(a, img, quat3, n);
    M16_CUDA_TRY(cudaGetLastError());

    const dim3 block(kBX, kBY, 1);
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)div_up(d0, a.zc));
    const int nparts_sweep = (int)(grid.x * grid.y * grid.z);
    const bool pointwise = sqevals3 == nullptr;
    const bool alpha_arr = alpha != nullptr;
    const bool sup = labels != nullptr;
    const double inv_norm = 1.0 / ((double)n * rcc);
    const int update = params->update;
    const int chunk = update * std::max(1, 64 / update);

    const bool timing = stats && stats->time_kernels;
    const bool pdl = !(stats && (stats->flags & M16_SOLVE_NO_PDL));
    std::unique_ptr<EventPool> pool;
    if (timing) {
        pool.reset(new EventPool(3 * chunk));
        if (!pool->ok) return M16_ERR_CUDA;
    }
    int launches = 3, p_launches = 0, u_launches = 0;
    double p_ms = 0.0, u_ms = 0.0;

    MfCtrl hctrl;
    hctrl.stopped = 0;
    int it = 0;
    while (it < params->num_iter) {
        const int end = std::min(params->num_iter, it + chunk);
        // per launch slot: its iteration, for the timing
        std::vector<int> slot_it;
        while (it < end) {
            const int j = (int)slot_it.size();
            if (timing) cudaEventRecord(pool->ev[3 * j], st);
            slot_it.push_back(it);
            const MfArgs &s = a;
            if (pointwise) {
                if (alpha_arr) M16_CUDA_TRY(launch_pdl(mf_update_p_kernel<true, true>, grid, block, st, pdl, s));
                else M16_CUDA_TRY(launch_pdl(mf_update_p_kernel<true, false>, grid, block, st, pdl, s));
            } else {
                if (alpha_arr) M16_CUDA_TRY(launch_pdl(mf_update_p_kernel<false, true>, grid, block, st, pdl, s));
                else M16_CUDA_TRY(launch_pdl(mf_update_p_kernel<false, false>, grid, block, st, pdl, s));
            }
            if (timing) cudaEventRecord(pool->ev[3 * j + 1], st);
            const bool check = (it % update) == 0;
            if (check) {
                if (sup) M16_CUDA_TRY(launch_pdl(mf_update_u_kernel<true, true>, grid, block, st, pdl, s));
                else M16_CUDA_TRY(launch_pdl(mf_update_u_kernel<false, true>, grid, block, st, pdl, s));
                if (timing) cudaEventRecord(pool->ev[3 * j + 2], st);
                M16_CUDA_TRY(launch_pdl(mf_check_kernel, dim3(1), dim3(256), st, pdl, (const float *)a.partials,
                                          nparts_sweep, inv_norm, params->error_bound, it, it / update, L.resid_cap,
                                          a.ctrl, resid));
                ++launches;
            } else {
                if (sup) M16_CUDA_TRY(launch_pdl(mf_update_u_kernel<true, false>, grid, block, st, pdl, s));
                else M16_CUDA_TRY(launch_pdl(mf_update_u_kernel<false, false>, grid, block, st, pdl, s));
                if (timing) cudaEventRecord(pool->ev[3 * j + 2], st);
            }
            launches += 2;
            ++it;
        }
        M16_CUDA_TRY(cudaGetLastError());
        M16_CUDA_TRY(cudaMemcpyAsync(&hctrl, a.ctrl, sizeof(MfCtrl), cudaMemcpyDeviceToHost, st));
        M16_CUDA_TRY(cudaStreamSynchronize(st));
        if (timing) {
            // only launches that ran (not the no-op launches after a stop) count
            const int ran_end = hctrl.stopped ? std::min(end, hctrl.iterations) : end;
            for (size_t j = 0; j < slot_it.size(); ++j) {
                if (slot_it[j] >= ran_end) break;
                float a_ms = 0.f, b_ms = 0.f;
                M16_CUDA_TRY(cudaEventElapsedTime(&a_ms, pool->ev[3 * j], pool->ev[3 * j + 1]));
                M16_CUDA_TRY(cudaEventElapsedTime(&b_ms, pool->ev[3 * j + 1], pool->ev[3 * j + 2]));
                p_ms += a_ms;
                u_ms += b_ms;
                ++p_launches;
                ++u_launches;
            }
        }
        if (hctrl.stopped) break;
    }
    M16_CUDA_TRY(cudaMemcpyAsync(&hctrl, a.ctrl, sizeof(MfCtrl), cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    const int ran = hctrl.stopped ? hctrl.iterations : it;
    if (stats) {
        stats->launches = launches;
        if (!timing) p_launches = u_launches = ran;
        stats->p_launches = p_launches;
        stats->u_launches = u_launches;
        stats->p_ms = p_ms;
        stats->u_ms = u_ms;
        stats->pair_launches = 0;
        stats->pair_ms = 0.0;
        stats->pair_zc = 0;
    }
    *iterations = hctrl.iterations;
    if (n_residuals) *n_residuals = hctrl.n_checks;
    if (residuals && residuals_cap > 0) {
        const int cnt = std::min(std::min(hctrl.n_checks, residuals_cap), L.resid_cap);
        if (cnt > 0) {
            M16_CUDA_TRY(cudaMemcpyAsync(residuals, resid, (size_t)cnt * 8, cudaMemcpyDeviceToHost, st));
            M16_CUDA_TRY(cudaStreamSynchronize(st));
        }
    }
    return M16_OK;
}

extern "C" int m16_maxflow_solve_ex(const float *img, const float *quat3, const double *sqevals3,
                                    const float *sqeigs, const float *alpha, float alpha_scalar,
                                    const float *cs, const float *ct, const uint8_t *labels,
                                    int32_t d0, int32_t d1, int32_t d2, const m16_cut_params *params,
                                    float *u, int32_t *iterations, double *residuals, int32_t residuals_cap,
                                    int32_t *n_residuals, void *workspace, size_t workspace_bytes, void *stream,
                                    m16_solve_stats *stats)
{
    // the two sweeps are the only iteration path (the fused iteration and two
    // iterations per launch measured slower at every size and were removed)
    if (stats && stats->path != M16_PATH_DEFAULT && stats->path != M16_PATH_TWO_SWEEPS) return M16_ERR_BAD_ARG;
    return maxflow_solve_impl(img, quat3, sqevals3, sqeigs, alpha, alpha_scalar, cs, ct, labels, d0, d1, d2, params,
                              u, iterations, residuals, residuals_cap, n_residuals, workspace, workspace_bytes,
                              stream, stats);
}

// ---- fixed-footprint variant: no allocation by anyone --------------------------
//
// m16_maxflow_solve takes its scratch from a workspace the caller allocates.
// Some callers cannot allocate device memory at all: a plugin whose host owns
// every byte of device memory through its own pool and hands it no allocator,
// a language binding (Go, Java, ...) that wants a fixed device footprint known
// at load time, or a service that must not allocate once it is serving.  For
// them m16_maxflow_solve_static runs the same solve with its scratch in the
// file-scope array below, which the CUDA module reserves on every device that
// loads this library and which stays reserved until the process exits.
//
// Limits: at most kStaticMaxVoxels voxels (e.g. 64 x 64 x 64) and at most
// kStaticMaxChecks residual checks (num_iter / update + 2 <= kStaticMaxChecks).

namespace m16 {
namespace {
constexpr int64_t kStaticMaxVoxels = 262144;
constexpr int kStaticMaxChecks = 4096;
// hp0, hp1, hp2, pt, tmp (4 B each) + q4 (16 B) + block partials (<= 4 B per voxel,
// every block covers at least one voxel) + max partials + control + residual log,
// each region rounded up to 256 B
constexpr size_t kStaticBytes = 11u << 20;   // 11 MiB >= 10,521,344 B needed at the limits

}  // namespace
}  // namespace m16

static __device__ __align__(256) unsigned char m16_static_scratch[m16::kStaticBytes];

namespace m16 {
namespace {
// Device address of the scratch array on the current device.  Host code cannot
// use the array's name as a device address, so every call asks the runtime for
// it, with the calling device current.  The lookup is cheap once the module is
// loaded, and it is never stale: a device reset, or any teardown and
// re-creation of the context, reloads the module and may move the array, and
// the next lookup returns the new address.
int static_scratch_on_current_device(void **out)
{
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, m16_static_scratch) != cudaSuccess || !p) return M16_ERR_CUDA;
    *out = p;
    return M16_OK;
}
}  // namespace
}  // namespace m16

extern "C" int m16_maxflow_solve_static(const float *img, const float *quat3, const double *sqevals3,
                                        const float *sqeigs, const float *alpha, float alpha_scalar,
                                        const float *cs, const float *ct, const uint8_t *labels,
                                        int32_t d0, int32_t d1, int32_t d2, const m16_cut_params *params,
                                        float *u, int32_t *iterations, double *residuals, int32_t residuals_cap,
                                        int32_t *n_residuals, void *stream)
{
    // size checks first: nothing touches the GPU for a request that cannot fit
    if (d0 < 1 || d1 < 1 || d2 < 1 || !params) return d0 < 1 || d1 < 1 || d2 < 1 ? M16_ERR_BAD_SHAPE : M16_ERR_BAD_ARG;
    if (params->update < 1 || params->num_iter < 0) return M16_ERR_BAD_ARG;
    if ((int64_t)d0 * d1 * d2 > kStaticMaxVoxels) return M16_ERR_TOO_LARGE;
    if (params->num_iter / params->update + 2 > kStaticMaxChecks) return M16_ERR_TOO_LARGE;
    const MfLayout L = mf_layout(d0, d1, d2, params->num_iter, params->update);
    if (L.total > kStaticBytes) return M16_ERR_TOO_LARGE;
    void *scratch = nullptr;
    const int st = static_scratch_on_current_device(&scratch);
    if (st != M16_OK) return st;
    // The solve's initialisation kernels write every scratch word before it is
    // read (flow state, control word, partial sums), so nothing of the previous
    // call's contents leaks into this one.
    // the two-sweep iteration: its workspace fits the fixed array
    return maxflow_solve_impl(img, quat3, sqevals3, sqeigs, alpha, alpha_scalar, cs, ct, labels, d0, d1, d2, params,
                              u, iterations, residuals, residuals_cap, n_residuals, scratch, kStaticBytes, stream,
                              nullptr);
}
