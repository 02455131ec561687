// capacities.cu -- the per-volume inputs of the cut and the fast Dice score on
// the GPU, replacing the host steps of the reference experiment:
//
//   source / sink capacities   PhantomExperiment._calculate_bgfg_weights_for
//                              (src/phantom_experiment.py:280-301): Gaussian
//                              log-likelihood ratio of foreground 1 against
//                              background 0 at the volume's noise level
//   |grad I|^2                 np.linalg.norm(np.gradient(img), axis=0) ** 2
//                              (src/phantom_experiment.py:345)
//   fast Dice                  fast_dice_for (src/phantom_experiment.py:38-49)
//
// The capacities and |grad I|^2 are evaluated in float64 with the host
// code's operation order (central differences (f[i+1] - f[i-1]) / 2 inside,
// one-sided differences at the two ends of each axis, the squared norm as
// sqrt((g0^2 + g1^2) + g2^2)^2) and rounded to float32 at the end, which is
// what the cut reads.  The per-instance nonterminal weight
// w * exp(-|grad I|^2 / decay^2) (:359) is never stored: the flow sweeps
// evaluate it from |grad I|^2.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "common.cuh"

namespace m16 {
namespace {

constexpr int kBX = 32, kBY = 8;

// normpdf (phantom_experiment.py:29-35): exp((x - mean)^2 * (1 / (-2 var))) * (1 / sqrt(2 pi var))
__device__ __forceinline__ double normpdf(double x, double mean, double inv_m2var, double norm)
{
    const double d = __dsub_rn(x, mean);
    return __dmul_rn(exp(__dmul_rn(__dmul_rn(d, d), inv_m2var)), norm);
}

__global__ void __launch_bounds__(kBX * kBY) cap_kernel(const float *__restrict__ img, int d0, int d1, int d2,
                                                        double inv_m2var, double norm, double eps, double rq,
                                                        float *__restrict__ cs, float *__restrict__ ct,
                                                        float *__restrict__ grad2)
{
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= d2 || y >= d1) return;
    const int64_t s1 = d2, s0 = (int64_t)d1 * d2;
    const int64_t i = (int64_t)z * s0 + (int64_t)y * s1 + x;
    const double v = (double)__ldg(img + i);
    if (cs || ct) {
        const double bgp = normpdf(v, 0.0, inv_m2var, norm);
        const double fgp = normpdf(v, 1.0, inv_m2var, norm);
        const double r = log(__ddiv_rn(__dadd_rn(fgp, eps), __dadd_rn(bgp, eps)));
        if (ct) ct[i] = (float)__dmul_rn(rq, fmax(-r, 0.0));   // background weights: the sink
        if (cs) cs[i] = (float)__dmul_rn(rq, fmax(r, 0.0));    // foreground weights: the source
    }
    if (grad2) {
        // np.gradient, edge_order 1, unit spacing
        auto diff = [&](int p, int n, int64_t st) -> double {
            if (p == 0) return __dsub_rn((double)__ldg(img + i + st), v);
            if (p == n - 1) return __dsub_rn(v, (double)__ldg(img + i - st));
            return __ddiv_rn(__dsub_rn((double)__ldg(img + i + st), (double)__ldg(img + i - st)), 2.0);
        };
        const double g0 = diff(z, d0, s0), g1 = diff(y, d1, s1), g2 = diff(x, d2, 1);
        const double ss = __dadd_rn(__dadd_rn(__dmul_rn(g0, g0), __dmul_rn(g1, g1)), __dmul_rn(g2, g2));
        const double nrm = __dsqrt_rn(ss);
        grad2[i] = (float)__dmul_rn(nrm, nrm);
    }
}

// Fast Dice of many segmentations against one ground truth: per block and
// instance the sums of (u >= 0.5) and (u >= 0.5) * truth, and the truth's sum
constexpr int kDiceBlocks = 2 * kSMs;

__global__ void __launch_bounds__(256) dice_partial_kernel(const float *const *__restrict__ us, int ninst,
                                                           const float *__restrict__ truth, int64_t n,
                                                           double *__restrict__ part)
{
    __shared__ double red[3][8];
    const int inst = blockIdx.y;
    const float *u = us[inst];
    double seg = 0.0, inter = 0.0, tru = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float t = __ldg(truth + i);
        const bool s = __ldg(u + i) >= 0.5f;
        seg += s ? 1.0 : 0.0;
        inter += s ? (double)t : 0.0;
        if (inst == 0) tru += (double)t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        seg += __shfl_down_sync(0xffffffffu, seg, o);
        inter += __shfl_down_sync(0xffffffffu, inter, o);
        tru += __shfl_down_sync(0xffffffffu, tru, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = seg;
        red[1][threadIdx.x >> 5] = inter;
        red[2][threadIdx.x >> 5] = tru;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0, c = 0.0;
        for (int w = 0; w < 8; ++w) { a += red[0][w]; b += red[1][w]; c += red[2][w]; }
        double *p = part + 3 * ((int64_t)inst * gridDim.x + blockIdx.x);
        p[0] = a; p[1] = b; p[2] = c;
    }
}

// dice[i] = 2 inter / (seg + truth), block partials summed in a fixed order
__global__ void dice_final_kernel(const double *__restrict__ part, int nblocks, int ninst, double *__restrict__ dice)
{
    const int inst = blockIdx.x * blockDim.x + threadIdx.x;
    if (inst >= ninst) return;
    double tru = 0.0, seg = 0.0, inter = 0.0;
    for (int b = 0; b < nblocks; ++b) {
        tru += part[3 * b + 2];   // instance 0's blocks hold the truth sums
        seg += part[3 * ((int64_t)inst * nblocks + b)];
        inter += part[3 * ((int64_t)inst * nblocks + b) + 1];
    }
    dice[inst] = 2.0 * inter / (seg + tru);
}

struct DiceLayout {
    size_t ptrs, part, dice, total;
};

inline DiceLayout dice_layout(int ninst)
{
    DiceLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.ptrs = take(sizeof(float *) * (size_t)ninst);
    L.part = take((size_t)3 * 8 * kDiceBlocks * ninst);
    L.dice = take((size_t)8 * ninst);
    L.total = off;
    return L;
}

}  // namespace
}  // namespace m16

using namespace m16;

extern "C" int m16_capacities(const float *img, int32_t d0, int32_t d1, int32_t d2, double noise_level,
                              double eps, float *cs, float *ct, float *grad2, void *stream)
{
    if (d0 < 1 || d1 < 1 || d2 < 1 || d0 > 65535) return M16_ERR_BAD_SHAPE;
    if (grad2 && (d0 < 2 || d1 < 2 || d2 < 2)) return M16_ERR_BAD_SHAPE;   // np.gradient needs 2 points per axis
    if (!img || (!cs && !ct && !grad2)) return M16_ERR_BAD_ARG;
    if ((cs || ct) && (!(noise_level > 0.0) || !isfinite(noise_level) || !(eps > 0.0))) return M16_ERR_BAD_ARG;
    // the host code's constants, in float64
    const double var = noise_level * noise_level;
    const double inv_m2var = 1.0 / (-2.0 * var);
    const double norm = 1.0 / sqrt(2.0 * M_PI * var);
    const double p_hat = norm;                      // normpdf(0, 0, var) == normpdf(1, 1, var)
    const double rq = 1.0 / log((p_hat + eps) / eps);
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)d0);
    cap_kernel<<<grid, dim3(kBX, kBY, 1), 0, (cudaStream_t)stream>>>(img, d0, d1, d2, inv_m2var, norm, eps, rq, cs,
                                                                     ct, grad2);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" size_t m16_fast_dice_workspace_bytes(int32_t ninst)
{
    if (ninst < 1) return 0;
    return dice_layout(ninst).total;
}

extern "C" int m16_fast_dice(const float *const *u, int32_t ninst, int64_t n, const float *truth, double *dice,
                             void *workspace, size_t workspace_bytes, void *stream)
{
    if (ninst < 1 || n < 1 || ninst > 65535) return M16_ERR_BAD_ARG;
    if (!u || !truth || !dice) return M16_ERR_BAD_ARG;
    for (int k = 0; k < ninst; ++k)
        if (!u[k]) return M16_ERR_BAD_ARG;
    const DiceLayout L = dice_layout(ninst);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    const float **dptr = (const float **)(ws + L.ptrs);
    double *part = (double *)(ws + L.part);
    double *ddice = (double *)(ws + L.dice);
    const int nblocks = (int)std::min<int64_t>(kDiceBlocks, div_up(n, 256));
    M16_CUDA_TRY(cudaMemcpyAsync(dptr, u, sizeof(float *) * (size_t)ninst, cudaMemcpyHostToDevice, st));
    dice_partial_kernel<<<dim3((unsigned)nblocks, (unsigned)ninst, 1), 256, 0, st>>>(dptr, ninst, truth, n, part);
    dice_final_kernel<<<(unsigned)div_up(ninst, 128), 128, 0, st>>>(part, nblocks, ninst, ddice);
    M16_CUDA_TRY(cudaGetLastError());
    M16_CUDA_TRY(cudaMemcpyAsync(dice, ddice, 8 * (size_t)ninst, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    return M16_OK;
}
