// frangi.cu -- Frangi vesselness on GB300: Gaussian-derivative Hessian per
// scale, 3x3 Jacobi eigendecomposition, vesselness and running maximum over
// scales.  Replaces the reference's GaussianFilter3D/Hessian/Eigendecomposition/
// VesselnessUpdate/VesselnessCalculation (src/processing/qfrangi_gpu.py:30-631)
// and the kernels axis0/1/2 (src/clcode/convolve_naive.cl), eigs
// (src/clcode/qeigs.cl), updateVesselness/calculateNorm (src/clcode/frangi.cl)
// and redMax (src/clcode/max.cl).
//
// The six Hessian entries share their separable factors, so one scale costs
// 15 one-dimensional passes instead of the reference's 18 (and no host round
// trip): z-pass of orders 0/1/2 -> Z0, Z1, Z2; y-pass -> the six products
//   A = y0 Z2 (-> 00), B = y2 Z0 (-> 11), C = y0 Z0 (-> 22),
//   D = y1 Z1 (-> 01), E = y0 Z1 (-> 02), F = y1 Z0 (-> 12);
// x-pass fused with the eigensolve: 00 = x0 A, 11 = x0 B, 22 = x2 C,
// 01 = x0 D, 02 = x1 E, 12 = x1 F.  Every pass is a true convolution (taps
// read reversed) with the reference's mirror boundary (period 2(n-1)).
#include <cuda_runtime.h>
#include <math.h>
#include <float.h>

#include <algorithm>

#include "common.cuh"

namespace m16 {
namespace {

constexpr int kMaxTaps = M16_MAX_TAPS;   // 2 * radius + 1 <= kMaxTaps
constexpr int kBX = 32, kBY = 8;

// taps of one axis, orders 0, 1, 2 (already scaled by sigma ** order)
struct AxisTaps {
    float t[3][kMaxTaps];
    int radius;
};

// mirror-completed index with period 2 (n - 1) (convolve_naive.cl:25-63)
__device__ __forceinline__ int mirror(int p, int n)
{
    if (n == 1) return 0;
    const int period = 2 * (n - 1);
    p %= period;
    if (p < 0) p += period;
    return p < n ? p : period - p;
}

inline int fr_zc(int d0, int d1, int d2)
{
    const int64_t cols = div_up(d2, kBX) * div_up(d1, kBY);
    int64_t zc = (int64_t)d0 * cols / (8 * kSMs);
    return (int)std::max<int64_t>(1, std::min<int64_t>(8, zc));
}

// ---- pass 1: z (axis 0), orders 0, 1, 2 ------------------------------------
__global__ void __launch_bounds__(kBX * kBY) fr_conv_z_kernel(const float *__restrict__ img, float *__restrict__ z0,
                                                              float *__restrict__ z1, float *__restrict__ z2, int d0,
                                                              int d1, int d2, int zc, AxisTaps tp)
{
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    if (x >= d2 || y >= d1) return;
    const int za = blockIdx.z * zc, zb = min(za + zc, d0);
    const int64_t s0 = (int64_t)d1 * d2;
    const int64_t col = (int64_t)y * d2 + x;
    const int r = tp.radius, K = 2 * r + 1;
    for (int z = za; z < zb; ++z) {
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
        const bool inner = z - r >= 0 && z + r < d0;
        for (int j = 0; j < K; ++j) {
            const int m = inner ? z - r + j : mirror(z - r + j, d0);
            const float v = __ldg(img + col + m * s0);
            const int k = K - 1 - j;
            a0 = fmaf(tp.t[0][k], v, a0);
            a1 = fmaf(tp.t[1][k], v, a1);
            a2 = fmaf(tp.t[2][k], v, a2);
        }
        const int64_t i = col + z * s0;
        z0[i] = a0;
        z1[i] = a1;
        z2[i] = a2;
    }
}

// ---- pass 2: y (axis 1), the six products ----------------------------------
__global__ void __launch_bounds__(kBX * kBY) fr_conv_y_kernel(const float *__restrict__ z0, const float *__restrict__ z1,
                                                              const float *__restrict__ z2, float *__restrict__ six,
                                                              int d0, int d1, int d2, int zc, AxisTaps tp)
{
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    if (x >= d2 || y >= d1) return;
    const int za = blockIdx.z * zc, zb = min(za + zc, d0);
    const int64_t s0 = (int64_t)d1 * d2, n = s0 * d0;
    const int r = tp.radius, K = 2 * r + 1;
    const bool inner = y - r >= 0 && y + r < d1;
    for (int z = za; z < zb; ++z) {
        const int64_t plane = (int64_t)z * s0 + x;
        float A = 0.f, B = 0.f, C = 0.f, D = 0.f, E = 0.f, F = 0.f;
        for (int j = 0; j < K; ++j) {
            const int m = inner ? y - r + j : mirror(y - r + j, d1);
            const int64_t idx = plane + (int64_t)m * d2;
            const float v0 = __ldg(z0 + idx), v1 = __ldg(z1 + idx), v2 = __ldg(z2 + idx);
            const int k = K - 1 - j;
            const float t0 = tp.t[0][k], t1 = tp.t[1][k], t2 = tp.t[2][k];
            A = fmaf(t0, v2, A);
            B = fmaf(t2, v0, B);
            C = fmaf(t0, v0, C);
            D = fmaf(t1, v1, D);
            E = fmaf(t0, v1, E);
            F = fmaf(t1, v0, F);
        }
        const int64_t i = plane + (int64_t)y * d2;
        six[i] = A;
        six[n + i] = B;
        six[2 * n + i] = C;
        six[3 * n + i] = D;
        six[4 * n + i] = E;
        six[5 * n + i] = F;
    }
}

// ---- Jacobi eigensolve (qeigs.cl:35-256), eigenvalues ascending by |lambda| -

__constant__ float kSorterQuat[6][4] = {{0.f, 0.f, 0.f, 1.f},
                                        {0.f, -0.70710678118654752f, 0.70710678118654752f, 0.f},
                                        {-0.70710678118654752f, 0.70710678118654752f, 0.f, 0.f},
                                        {-0.5f, -0.5f, -0.5f, 0.5f},
                                        {0.5f, 0.5f, 0.5f, 0.5f},
                                        {-0.70710678118654752f, 0.f, 0.70710678118654752f, 0.f}};

__device__ __forceinline__ bool eigcmp(float a, float b) { return fabsf(a) < fabsf(b); }

// squeezed quaternion of q (scalar part last), qsqueezeLast (quaternion_math.h:45-69)
__device__ __forceinline__ void squeeze_last(const float q[4], float v[3])
{
    const float q1 = q[0], q2 = q[1], q3 = q[2], q0 = q[3];
    const float q1spq2s = q1 * q1 + q2 * q2;
    const bool c1 = q1spq2s < FLT_EPSILON;
    const bool c2 = c1 || (1.f - q1spq2s) < FLT_EPSILON;
    const float q1q3 = q1 * q3, q2q0 = q2 * q0, q1q0 = q1 * q0, q2q3 = q2 * q3;
    auto satan2 = [](float a, float b) { return (a == 0.f && b == 0.f) ? 0.f : atan2f(a, b); };
    v[0] = satan2(q1q3 + q2q0, q1q0 - q2q3);
    v[1] = c2 ? (c1 ? 0.f : 3.14159265358979323846f) : acosf(fminf(fmaxf(1.f - 2.f * q1spq2s, -1.f), 1.f));
    float at2 = c2 ? (q1 * q2 - q0 * q3) : (q1q3 - q2q0);
    at2 = satan2(at2, c2 ? (0.5f - (q2 * q2 + q3 * q3)) : (q1q0 + q2q3));
    v[2] = c2 ? (-at2 + v[0] * (c1 ? -1.f : 1.f)) : at2;
}

// state of one eigensolve between its sweeps and its sort
struct Jacobi {
    float on[3], off[3], oq[4];
    bool converged;
};

// the cyclic sweeps, up to 50, until the off-diagonal sum is at most
// max |h| * FLT_EPSILON (qeigs.cl:146-256)
__device__ __forceinline__ void jacobi_sweeps(const float h[6], Jacobi &J)
{
    const float GAMMA = 5.8284271247461900976f, C_STAR = 0.9238795325112867561f, S_STAR = 0.3826834323650897717f;
    float on[3] = {h[0], h[1], h[2]};
    float off[3] = {h[5], h[4], h[3]};
    float oq[4] = {0.f, 0.f, 0.f, 1.f};
    const float tol = fmaxf(fmaxf(fmaxf(fabsf(on[0]), fabsf(on[1])), fmaxf(fabsf(on[2]), fabsf(off[0]))),
                            fmaxf(fabsf(off[1]), fabsf(off[2]))) * FLT_EPSILON;
    bool converged = false;
    for (int it = 0; it < 50; ++it) {
        if (fabsf(off[0]) + fabsf(off[1]) + fabsf(off[2]) <= tol) {
            converged = true;
            break;
        }
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq < 2 ? 0 : 1;
            const int q = pq == 0 ? 1 : 2;
            const int r = 3 ^ (p | q);
            // approximate Givens rotation (McAdams et al.)
            float c = 2.f * (on[q] - on[p]);
            float s = off[r];
            float t1 = s * s, t2 = c * c;
            const bool cond = GAMMA * t1 < t2;
            t1 = rsqrtf(t1 + t2);
            c = cond ? t1 * c : C_STAR;
            s = cond ? t1 * s : S_STAR;
            // accumulate the quaternion (scalar part last)
            t1 = c * oq[p] - s * oq[q];
            t2 = c * oq[q] + s * oq[p];
            oq[p] = t1; oq[q] = t2;
            const float sr = (r == 1) ? s : -s;
            t1 = c * oq[3] + sr * oq[r];
            t2 = c * oq[r] - sr * oq[3];
            oq[3] = t1; oq[r] = t2;
            // rotate the matrix
            t1 = 1.f - 2.f * s * s;
            s = 2.f * c * s;
            c = t1;
            t1 = off[r] * c + on[p] * s;
            t2 = on[q] * c + off[r] * s;
            on[p] = c * (on[p] * c - off[r] * s) - s * (off[r] * c - on[q] * s);
            on[q] = c * t2 + s * t1;
            off[r] = c * t1 - s * t2;
            t2 = off[q];
            off[q] = c * t2 - s * off[p];
            off[p] = c * off[p] + s * t2;
        }
    }
    for (int k = 0; k < 3; ++k) {
        J.on[k] = on[k];
        J.off[k] = off[k];
    }
    for (int k = 0; k < 4; ++k) J.oq[k] = oq[k];
    J.converged = converged;
}

// eigenvalues ascending by |lambda| and the squeezed quaternion of the
// eigenvectors (sortEigs, qeigs.cl:60-92, and the quaternion's squeeze);
// NaN where the sweeps did not converge
__device__ __forceinline__ void jacobi_finish(const Jacobi &J, float out[6])
{
    if (!J.converged) {
        for (int k = 0; k < 6; ++k) out[k] = NAN;
        return;
    }
    float on[3] = {J.on[0], J.on[1], J.on[2]};
    const float *oq = J.oq;
    int o0, o1, o2, ot;
    float vt;
    bool c = eigcmp(on[0], on[1]);
    vt = on[0]; on[0] = c ? on[0] : on[1]; o0 = c ? 0 : 1; on[1] = c ? on[1] : vt; o1 = c ? 1 : 0;
    c = eigcmp(on[1], on[2]);
    vt = on[1]; ot = o1; on[1] = c ? on[1] : on[2]; o1 = c ? o1 : 2; on[2] = c ? on[2] : vt; o2 = c ? 2 : ot;
    c = eigcmp(on[0], on[1]);
    vt = on[0]; ot = o0; on[0] = c ? on[0] : on[1]; o0 = c ? o0 : o1; on[1] = c ? on[1] : vt; o1 = c ? o1 : ot;
    const int sk = (o0 << 1) | (o1 > o2 ? 1 : 0);
    const float l0 = kSorterQuat[sk][0], l1 = kSorterQuat[sk][1], l2 = kSorterQuat[sk][2], l3 = kSorterQuat[sk][3];
    float q[4];
    q[3] = l3 * oq[3] - (l0 * oq[0] + l1 * oq[1] + l2 * oq[2]);
    q[0] = l3 * oq[0] + l0 * oq[3] + l1 * oq[2] - l2 * oq[1];
    q[1] = l3 * oq[1] - l0 * oq[2] + l1 * oq[3] + l2 * oq[0];
    q[2] = l3 * oq[2] + l0 * oq[1] - l1 * oq[0] + l2 * oq[3];
    q[3] = -q[3];   // eigenvectors in columns
    float sq[3];
    squeeze_last(q, sq);
    out[0] = on[0]; out[1] = on[1]; out[2] = on[2];
    out[3] = sq[0]; out[4] = sq[1]; out[5] = sq[2];
}

__device__ __forceinline__ void eig3(const float h[6], float out[6])
{
    Jacobi J;
    jacobi_sweeps(h, J);
    jacobi_finish(J, out);
}

// Frangi response of one eigen-triple (frangi.cl:46-92)
__device__ __forceinline__ float vesselness(const float e[6], float alpha, float beta, float c, bool bright)
{
    const float l1 = fabsf(e[0]);
    float l2 = bright ? e[1] : -e[1];
    float l3 = bright ? e[2] : -e[2];
    const bool valid = l2 < 0.f && l3 < 0.f;
    l2 = fabsf(l2);
    l3 = fabsf(l3);
    const float rb = l1 / (sqrtf(l2 * l3) + FLT_MIN);
    const float ra = l2 / (l3 + FLT_MIN);
    const float ss = l1 * l1 + l2 * l2 + l3 * l3;
    const float ta = ra / alpha, tb = rb / beta;
    return (valid ? 1.f : 0.f) * ((1.f - expf(-0.5f * ta * ta)) * expf(-0.5f * tb * tb) *
                                  (1.f - expf(-0.5f * ss / (c * c))));
}

struct FrArgs {
    int d0, d1, d2, zc;
    float alpha, beta, c;   // c < 0: read the per-scale c from *c_dev
    int bright;
    const float *six;
    float *eig6;            // N x 6, or null when the update is fused
    float *val, *quat3;
    float *partials;        // per-block max Hessian norm
    const float *c_dev;     // the update kernel's scale's c
    // c of the previous scale when its update rides along in this x pass
    // (read from eig6 just before this scale's triple replaces it), else null
    const float *c_prev;
    int first;              // the update done here is the first one: it writes
                            // val and quat without reading them
};

// one scale's update of the running maximum (updateVesselness,
// frangi.cl:46-92).  The first update writes what the maximum over
// (-inf, zero quaternion) and this scale gives: v where v is a number, the
// initial values where it is NaN.
__device__ __forceinline__ void update_max(const FrArgs &a, const float e[6], float c, bool first, int64_t i)
{
    const float v = vesselness(e, a.alpha, a.beta, c, a.bright != 0);
    if (first) {
        const bool take = v > -INFINITY;
        a.val[i] = take ? v : -INFINITY;
        a.quat3[3 * i] = take ? e[3] : 0.f;
        a.quat3[3 * i + 1] = take ? e[4] : 0.f;
        a.quat3[3 * i + 2] = take ? e[5] : 0.f;
    } else if (v > a.val[i]) {
        a.val[i] = v;
        a.quat3[3 * i] = e[3];
        a.quat3[3 * i + 1] = e[4];
        a.quat3[3 * i + 2] = e[5];
    }
}

// output of one eigensolve: the running maximum update when c is given,
// else the eigen-triple stored for the update after c is known (first the
// previous scale's triple there goes through its update, when c_prev is
// set), its norm folded into mx (calculateNorm, frangi.cl)
template <bool FUSED_UPDATE>
__device__ __forceinline__ void x_output(const FrArgs &a, const float e[6], int64_t i, float c_prev, float &mx)
{
    if (FUSED_UPDATE) {
        update_max(a, e, a.c, a.first != 0, i);
    } else {
        float2 *o = reinterpret_cast<float2 *>(a.eig6 + 6 * i);
        if (a.c_prev) {
            const float2 p01 = o[0], p23 = o[1], p45 = o[2];
            const float ep[6] = {p01.x, p01.y, p23.x, p23.y, p45.x, p45.y};
            update_max(a, ep, c_prev, a.first != 0, i);
        }
        o[0] = make_float2(e[0], e[1]);
        o[1] = make_float2(e[2], e[3]);
        o[2] = make_float2(e[4], e[5]);
        // calculateNorm + redMax (NaN-neutral)
        mx = fmaxf(mx, sqrtf(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]));
    }
}

template <bool FUSED_UPDATE>
__device__ __forceinline__ void x_epilogue(const FrArgs &a, const float h[6], int64_t i, float c_prev, float &mx)
{
    float e[6];
    eig3(h, e);
    x_output<FUSED_UPDATE>(a, e, i, c_prev, mx);
}

// block maximum of the norms into the block's partial (redMax, max.cl);
// fmaxf ignores NaN as the reference's fmax does
__device__ __forceinline__ void block_max_to_partial(float mx, float *red, float *partials)
{
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
        float m = red[0];
        for (int w = 1; w < (kBX * kBY) / 32; ++w) m = fmaxf(m, red[w]);
        partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = m;
    }
}

// ---- pass 3: x (axis 2) fused with the eigensolve ----------------------------
// One lane per voxel.  The Jacobi's data-dependent sweep count makes a warp
// wait for its slowest voxel (21 of 32 lanes active on average).  Handing
// each lane the next matrix of a per-warp pool as its own converges raised
// that to 25 of 32 but added as many instructions as it saved (895 M -> 910
// M warp instructions at 256^3, sigma 1, still issue-bound): no faster.
// This is the kernel for any radius; radii up to kRunMaxR take the
// specialised fr_conv_x_eig_run_kernel below.
template <bool FUSED_UPDATE>
__global__ void __launch_bounds__(kBX * kBY) fr_conv_x_eig_kernel(FrArgs a, AxisTaps tp)
{
    __shared__ float red[32];
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    const float c_prev = (!FUSED_UPDATE && a.c_prev) ? *a.c_prev : 0.f;
    float mx = -INFINITY;
    if (x < a.d2 && y < a.d1) {
        const int za = blockIdx.z * a.zc, zb = min(za + a.zc, a.d0);
        const int64_t s0 = (int64_t)a.d1 * a.d2, n = s0 * a.d0;
        const int r = tp.radius, K = 2 * r + 1;
        const bool inner = x - r >= 0 && x + r < a.d2;
        for (int z = za; z < zb; ++z) {
            const int64_t row = (int64_t)z * s0 + (int64_t)y * a.d2;
            float h[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int j = 0; j < K; ++j) {
                const int m = inner ? x - r + j : mirror(x - r + j, a.d2);
                const int64_t idx = row + m;
                const int k = K - 1 - j;
                const float t0 = tp.t[0][k], t1 = tp.t[1][k], t2 = tp.t[2][k];
                h[0] = fmaf(t0, __ldg(a.six + idx), h[0]);
                h[1] = fmaf(t0, __ldg(a.six + n + idx), h[1]);
                h[2] = fmaf(t2, __ldg(a.six + 2 * n + idx), h[2]);
                h[3] = fmaf(t0, __ldg(a.six + 3 * n + idx), h[3]);
                h[4] = fmaf(t1, __ldg(a.six + 4 * n + idx), h[4]);
                h[5] = fmaf(t1, __ldg(a.six + 5 * n + idx), h[5]);
            }
            x_epilogue<FUSED_UPDATE>(a, h, row + x, c_prev, mx);
        }
    }
    if (!FUSED_UPDATE) block_max_to_partial(mx, red, a.partials);
}

// ---- radius-specialised passes ------------------------------------------------
// For radii 1..kRunMaxR every pass is instantiated per radius: the tap loops
// unroll and the taps become constant operands.  The z and y passes keep a
// run of outputs per thread and read each input once for the whole run
// (kRun + 2R loads instead of kRun * (2R + 1)); the x pass stages each row
// of the six products, with its halo, in the warp's own shared memory and
// convolves from there.  Every output still accumulates its taps in the
// same order (j = 0..K-1, tap K-1-j) with the same fused multiply-adds, so
// the results equal the kernels above bit for bit.
constexpr int kRunMaxR = 16;
constexpr int kRun = 8;   // outputs per thread along z (z pass) or y (y pass)
static_assert(2 * kRunMaxR <= kBX, "the x pass stages each row in two 32-column steps");

template <int R, bool INNER>
__device__ __forceinline__ void z_run(const float *__restrict__ col, int64_t s0, int za, int d0, const AxisTaps &tp,
                                      float (&acc)[kRun][3])
{
    constexpr int K = 2 * R + 1;
#pragma unroll
    for (int p = 0; p < kRun + 2 * R; ++p) {
        const int m = INNER ? za - R + p : mirror(za - R + p, d0);
        const float v = __ldg(col + (int64_t)m * s0);
#pragma unroll
        for (int o = 0; o < kRun; ++o) {
            const int j = p - o;
            if (j >= 0 && j < K) {
                acc[o][0] = fmaf(tp.t[0][K - 1 - j], v, acc[o][0]);
                acc[o][1] = fmaf(tp.t[1][K - 1 - j], v, acc[o][1]);
                acc[o][2] = fmaf(tp.t[2][K - 1 - j], v, acc[o][2]);
            }
        }
    }
}

template <int R>
__global__ void __launch_bounds__(kBX * kBY) fr_conv_z_run_kernel(const float *__restrict__ img, float *__restrict__ z0,
                                                                  float *__restrict__ z1, float *__restrict__ z2,
                                                                  int d0, int d1, int d2, AxisTaps tp)
{
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    if (x >= d2 || y >= d1) return;
    const int za = blockIdx.z * kRun;
    const int64_t s0 = (int64_t)d1 * d2;
    const int64_t col = (int64_t)y * d2 + x;
    float acc[kRun][3];
#pragma unroll
    for (int o = 0; o < kRun; ++o) acc[o][0] = acc[o][1] = acc[o][2] = 0.f;
    if (za - R >= 0 && za + kRun - 1 + R < d0)
        z_run<R, true>(img + col, s0, za, d0, tp, acc);
    else
        z_run<R, false>(img + col, s0, za, d0, tp, acc);
#pragma unroll
    for (int o = 0; o < kRun; ++o) {
        if (za + o < d0) {
            const int64_t i = col + (int64_t)(za + o) * s0;
            z0[i] = acc[o][0];
            z1[i] = acc[o][1];
            z2[i] = acc[o][2];
        }
    }
}

template <int R, bool INNER>
__device__ __forceinline__ void y_run(const float *__restrict__ z0, const float *__restrict__ z1,
                                      const float *__restrict__ z2, int64_t plane, int d2, int ya, int d1,
                                      const AxisTaps &tp, float (&acc)[kRun][6])
{
    constexpr int K = 2 * R + 1;
#pragma unroll
    for (int p = 0; p < kRun + 2 * R; ++p) {
        const int m = INNER ? ya - R + p : mirror(ya - R + p, d1);
        const int64_t idx = plane + (int64_t)m * d2;
        const float v0 = __ldg(z0 + idx), v1 = __ldg(z1 + idx), v2 = __ldg(z2 + idx);
#pragma unroll
        for (int o = 0; o < kRun; ++o) {
            const int j = p - o;
            if (j >= 0 && j < K) {
                const int k = K - 1 - j;
                acc[o][0] = fmaf(tp.t[0][k], v2, acc[o][0]);   // A = y0 Z2
                acc[o][1] = fmaf(tp.t[2][k], v0, acc[o][1]);   // B = y2 Z0
                acc[o][2] = fmaf(tp.t[0][k], v0, acc[o][2]);   // C = y0 Z0
                acc[o][3] = fmaf(tp.t[1][k], v1, acc[o][3]);   // D = y1 Z1
                acc[o][4] = fmaf(tp.t[0][k], v1, acc[o][4]);   // E = y0 Z1
                acc[o][5] = fmaf(tp.t[1][k], v0, acc[o][5]);   // F = y1 Z0
            }
        }
    }
}

// grid (x blocks, y blocks of kBY runs of kRun rows, one z plane per block)
template <int R>
__global__ void __launch_bounds__(kBX * kBY) fr_conv_y_run_kernel(const float *__restrict__ z0,
                                                                  const float *__restrict__ z1,
                                                                  const float *__restrict__ z2,
                                                                  float *__restrict__ six, int d0, int d1, int d2,
                                                                  AxisTaps tp)
{
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int ya = (blockIdx.y * kBY + threadIdx.y) * kRun;
    if (x >= d2 || ya >= d1) return;
    const int64_t s0 = (int64_t)d1 * d2, n = s0 * d0;
    const int64_t plane = (int64_t)blockIdx.z * s0 + x;
    float acc[kRun][6];
#pragma unroll
    for (int o = 0; o < kRun; ++o)
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[o][c] = 0.f;
    if (ya - R >= 0 && ya + kRun - 1 + R < d1)
        y_run<R, true>(z0, z1, z2, plane, d2, ya, d1, tp, acc);
    else
        y_run<R, false>(z0, z1, z2, plane, d2, ya, d1, tp, acc);
#pragma unroll
    for (int o = 0; o < kRun; ++o) {
        if (ya + o < d1) {
            const int64_t i = plane + (int64_t)(ya + o) * d2;
#pragma unroll
            for (int c = 0; c < 6; ++c) six[c * n + i] = acc[o][c];
        }
    }
}

// x pass fused with the eigensolve; warp w of the block works on row
// y = blockIdx.y * kBY + w and stages its 32 + 2R columns of the six
// products in shared memory (only __syncwarp between staging and reads)
template <bool FUSED_UPDATE, int R>
__global__ void __launch_bounds__(kBX * kBY) fr_conv_x_eig_run_kernel(FrArgs a, AxisTaps tp)
{
    constexpr int K = 2 * R + 1, W = kBX + 2 * R;
    __shared__ float red[32];
    __shared__ float rows[kBY][6][W];
    const int lane = threadIdx.x;
    const int x0 = blockIdx.x * kBX, x = x0 + lane;
    const int y = blockIdx.y * kBY + threadIdx.y;
    const float c_prev = (!FUSED_UPDATE && a.c_prev) ? *a.c_prev : 0.f;
    float mx = -INFINITY;
    if (y < a.d1) {   // uniform over the warp
        float (*buf)[W] = rows[threadIdx.y];
        const int za = blockIdx.z * a.zc, zb = min(za + a.zc, a.d0);
        const int64_t s0 = (int64_t)a.d1 * a.d2, n = s0 * a.d0;
        const bool inner = x0 - R >= 0 && x0 + kBX - 1 + R < a.d2;
        for (int z = za; z < zb; ++z) {
            const int64_t row = (int64_t)z * s0 + (int64_t)y * a.d2;
#pragma unroll
            for (int i0 = 0; i0 < W; i0 += kBX) {
                const int i = i0 + lane;
                if (i < W) {
                    const int m = inner ? x0 - R + i : mirror(x0 - R + i, a.d2);
                    const float *src = a.six + row + m;
#pragma unroll
                    for (int c = 0; c < 6; ++c) buf[c][i] = __ldg(src + c * n);
                }
            }
            __syncwarp();
            float h[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const int k = K - 1 - j;
                h[0] = fmaf(tp.t[0][k], buf[0][lane + j], h[0]);
                h[1] = fmaf(tp.t[0][k], buf[1][lane + j], h[1]);
                h[2] = fmaf(tp.t[2][k], buf[2][lane + j], h[2]);
                h[3] = fmaf(tp.t[0][k], buf[3][lane + j], h[3]);
                h[4] = fmaf(tp.t[1][k], buf[4][lane + j], h[4]);
                h[5] = fmaf(tp.t[1][k], buf[5][lane + j], h[5]);
            }
            __syncwarp();
            // Every lane solves (a zero matrix past the volume's edge), and the
            // warp meets again before the sort and squeeze: without that, lanes
            // that finish their sweeps at different counts run the squeeze's
            // atan2/acos in as many separate groups (about 3x its instructions).
            if (x >= a.d2)
                for (int c = 0; c < 6; ++c) h[c] = 0.f;
            Jacobi J;
            jacobi_sweeps(h, J);
            __syncwarp();
            float e[6];
            jacobi_finish(J, e);
            if (x < a.d2) x_output<FUSED_UPDATE>(a, e, row + x, c_prev, mx);
        }
    }
    if (!FUSED_UPDATE) block_max_to_partial(mx, red, a.partials);
}

#define FR_RADIUS_CASES(CALL)                                                                                   \
    case 1: CALL(1); break;   case 2: CALL(2); break;   case 3: CALL(3); break;   case 4: CALL(4); break;     \
    case 5: CALL(5); break;   case 6: CALL(6); break;   case 7: CALL(7); break;   case 8: CALL(8); break;     \
    case 9: CALL(9); break;   case 10: CALL(10); break; case 11: CALL(11); break; case 12: CALL(12); break;   \
    case 13: CALL(13); break; case 14: CALL(14); break; case 15: CALL(15); break; case 16: CALL(16); break;

// the x pass for one scale: the specialised kernel for radii 1..kRunMaxR,
// else the kernel for any radius (same grid)
template <bool FUSED_UPDATE>
void launch_x_eig(const FrArgs &a, const AxisTaps &tpx, dim3 grid, cudaStream_t st)
{
    const dim3 block(kBX, kBY, 1);
#define FR_X_CALL(R) fr_conv_x_eig_run_kernel<FUSED_UPDATE, R><<<grid, block, 0, st>>>(a, tpx)
    switch (tpx.radius) {
        FR_RADIUS_CASES(FR_X_CALL)
        default: fr_conv_x_eig_kernel<FUSED_UPDATE><<<grid, block, 0, st>>>(a, tpx); break;
    }
#undef FR_X_CALL
}

// c = 0.5 * max norm of one scale (qfrangi_gpu.py:429-433)
__global__ void fr_c_kernel(const float *__restrict__ part, int nparts, float *c_out)
{
    __shared__ float s[256];
    float m = -INFINITY;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) m = fmaxf(m, part[k]);
    s[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] = fmaxf(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *c_out = 0.5f * (s[0] == -INFINITY ? NAN : s[0]);
}

// updateVesselness (frangi.cl:46-92) of the last scale from its stored
// eigendecompositions (the earlier scales' updates ride along in the next
// scale's x pass)
__global__ void fr_update_kernel(FrArgs a, int64_t n)
{
    const float c = *a.c_dev;
    const bool first = a.first != 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 *p = reinterpret_cast<const float2 *>(a.eig6 + 6 * i);
        const float2 e01 = p[0], e23 = p[1], e45 = p[2];
        const float e[6] = {e01.x, e01.y, e23.x, e23.y, e45.x, e45.y};
        update_max(a, e, c, first, i);
    }
}

__global__ void fr_eigs_kernel(const float *__restrict__ in6, float *__restrict__ out6, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float h[6], e[6];
        for (int k = 0; k < 6; ++k) h[k] = in6[6 * i + k];
        eig3(h, e);
        for (int k = 0; k < 6; ++k) out6[6 * i + k] = e[k];
    }
}

// interleave the x-pass of the six products into an N x 6 Hessian (tests)
__global__ void fr_conv_x_hessian_kernel(const float *__restrict__ six, float *__restrict__ h6, int d0, int d1, int d2,
                                         int zc, AxisTaps tp)
{
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    if (x >= d2 || y >= d1) return;
    const int za = blockIdx.z * zc, zb = min(za + zc, d0);
    const int64_t s0 = (int64_t)d1 * d2, n = s0 * d0;
    const int r = tp.radius, K = 2 * r + 1;
    for (int z = za; z < zb; ++z) {
        const int64_t row = (int64_t)z * s0 + (int64_t)y * d2;
        float h[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int j = 0; j < K; ++j) {
            const int64_t idx = row + mirror(x - r + j, d2);
            const int k = K - 1 - j;
            h[0] = fmaf(tp.t[0][k], __ldg(six + idx), h[0]);
            h[1] = fmaf(tp.t[0][k], __ldg(six + n + idx), h[1]);
            h[2] = fmaf(tp.t[2][k], __ldg(six + 2 * n + idx), h[2]);
            h[3] = fmaf(tp.t[0][k], __ldg(six + 3 * n + idx), h[3]);
            h[4] = fmaf(tp.t[1][k], __ldg(six + 4 * n + idx), h[4]);
            h[5] = fmaf(tp.t[1][k], __ldg(six + 5 * n + idx), h[5]);
        }
        for (int k = 0; k < 6; ++k) h6[6 * (row + x) + k] = h[k];
    }
}

struct FrLayout {
    size_t z, six, eig, part, cdev, total;
    int nparts;
};

inline FrLayout fr_layout(int d0, int d1, int d2, int nscales)
{
    FrLayout L;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const int zc = fr_zc(d0, d1, d2);
    L.nparts = (int)(div_up(d2, kBX) * div_up(d1, kBY) * div_up(d0, zc));
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.z = take(3 * n * 4);
    L.six = take(6 * n * 4);
    L.eig = take(6 * n * 4);
    L.part = take((size_t)L.nparts * 4);
    L.cdev = take((size_t)std::max(nscales, 1) * 4);
    L.total = off;
    return L;
}

bool fill_taps(AxisTaps &tp, const float *taps_axis, int radius)
{
    if (radius < 0 || 2 * radius + 1 > kMaxTaps) return false;
    tp.radius = radius;
    for (int o = 0; o < 3; ++o)
        for (int k = 0; k < kMaxTaps; ++k) tp.t[o][k] = k < 2 * radius + 1 ? taps_axis[o * kMaxTaps + k] : 0.f;
    return true;
}

int hessian_passes(const float *img, int d0, int d1, int d2, const float *taps, const int *radius, char *ws,
                   const FrLayout &L, cudaStream_t st, AxisTaps *tpx)
{
    AxisTaps tpz, tpy;
    if (!fill_taps(tpz, taps, radius[0]) || !fill_taps(tpy, taps + 3 * kMaxTaps, radius[1]) ||
        !fill_taps(*tpx, taps + 6 * kMaxTaps, radius[2]))
        return M16_ERR_BAD_ARG;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const int zc = fr_zc(d0, d1, d2);
    const dim3 block(kBX, kBY, 1);
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)div_up(d0, zc));
    float *z = (float *)(ws + L.z);
    float *six = (float *)(ws + L.six);
    const dim3 grid_z((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)div_up(d0, kRun));
#define FR_Z_CALL(R) fr_conv_z_run_kernel<R><<<grid_z, block, 0, st>>>(img, z, z + n, z + 2 * n, d0, d1, d2, tpz)
    switch (tpz.radius) {
        FR_RADIUS_CASES(FR_Z_CALL)
        default: fr_conv_z_kernel<<<grid, block, 0, st>>>(img, z, z + n, z + 2 * n, d0, d1, d2, zc, tpz); break;
    }
#undef FR_Z_CALL
    // one z plane per block of the specialised y pass (grid z limit 65535)
    const dim3 grid_y((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY * kRun), (unsigned)d0);
    const int ry = d0 <= 65535 ? tpy.radius : 0;
#define FR_Y_CALL(R) fr_conv_y_run_kernel<R><<<grid_y, block, 0, st>>>(z, z + n, z + 2 * n, six, d0, d1, d2, tpy)
    switch (ry) {
        FR_RADIUS_CASES(FR_Y_CALL)
        default: fr_conv_y_kernel<<<grid, block, 0, st>>>(z, z + n, z + 2 * n, six, d0, d1, d2, zc, tpy); break;
    }
#undef FR_Y_CALL
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

}  // namespace
}  // namespace m16

using namespace m16;

extern "C" size_t m16_frangi_workspace_bytes(int32_t d0, int32_t d1, int32_t d2, int32_t nscales)
{
    if (d0 < 1 || d1 < 1 || d2 < 1) return 0;
    return fr_layout(d0, d1, d2, nscales).total;
}

extern "C" int m16_frangi(const float *img, int32_t d0, int32_t d1, int32_t d2, int32_t nscales, const float *taps,
                          const int32_t *radius, float alpha, float beta, float c, int32_t bright, float *val,
                          float *quat3, float *c_used, void *workspace, size_t workspace_bytes, void *stream)
{
    if (d0 < 1 || d1 < 1 || d2 < 1 || (int64_t)d0 * d1 * d2 > ((int64_t)1 << 33)) return M16_ERR_BAD_SHAPE;
    if (!img || !taps || !radius || !val || !quat3 || nscales < 1) return M16_ERR_BAD_ARG;
    const FrLayout L = fr_layout(d0, d1, d2, nscales);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const int blocks1d = (int)std::min<int64_t>(8 * kSMs, div_up(n, 256));
    FrArgs a;
    a.d0 = d0; a.d1 = d1; a.d2 = d2; a.zc = fr_zc(d0, d1, d2);
    a.alpha = alpha; a.beta = beta; a.c = c; a.bright = bright;
    a.six = (const float *)(ws + L.six);
    a.eig6 = (float *)(ws + L.eig);
    a.val = val; a.quat3 = quat3;
    a.partials = (float *)(ws + L.part);
    a.c_dev = nullptr;
    a.c_prev = nullptr;
    a.first = 0;
    float *cdev = (float *)(ws + L.cdev);
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)div_up(d0, a.zc));
    for (int s = 0; s < nscales; ++s) {
        AxisTaps tpx;
        const int rc = hessian_passes(img, d0, d1, d2, taps + (size_t)s * 9 * kMaxTaps, radius + 3 * s, ws, L, st, &tpx);
        if (rc != M16_OK) return rc;
        if (c >= 0.f) {
            a.first = s == 0;
            launch_x_eig<true>(a, tpx, grid, st);
        } else {
            // scale s - 1's update rides along: its triple is read at each
            // voxel just before scale s's replaces it
            a.c_prev = s > 0 ? cdev + s - 1 : nullptr;
            a.first = s == 1;
            launch_x_eig<false>(a, tpx, grid, st);
            fr_c_kernel<<<1, 256, 0, st>>>(a.partials, L.nparts, cdev + s);
        }
        M16_CUDA_TRY(cudaGetLastError());
    }
    if (c < 0.f) {
        a.c_dev = cdev + nscales - 1;
        a.c_prev = nullptr;
        a.first = nscales == 1;
        fr_update_kernel<<<blocks1d, 256, 0, st>>>(a, n);
        M16_CUDA_TRY(cudaGetLastError());
    }
    if (c_used) {
        if (c >= 0.f) {
            for (int s = 0; s < nscales; ++s) c_used[s] = c;
        } else {
            M16_CUDA_TRY(cudaMemcpyAsync(c_used, cdev, (size_t)nscales * 4, cudaMemcpyDeviceToHost, st));
            M16_CUDA_TRY(cudaStreamSynchronize(st));
        }
    }
    return M16_OK;
}

extern "C" int m16_hessian(const float *img, int32_t d0, int32_t d1, int32_t d2, const float *taps,
                           const int32_t *radius, float *h6, void *workspace, size_t workspace_bytes, void *stream)
{
    if (d0 < 1 || d1 < 1 || d2 < 1) return M16_ERR_BAD_SHAPE;
    if (!img || !taps || !radius || !h6) return M16_ERR_BAD_ARG;
    const FrLayout L = fr_layout(d0, d1, d2, 1);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    AxisTaps tpx;
    const int rc = hessian_passes(img, d0, d1, d2, taps, radius, (char *)workspace, L, st, &tpx);
    if (rc != M16_OK) return rc;
    const int zc = fr_zc(d0, d1, d2);
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)div_up(d0, zc));
    fr_conv_x_hessian_kernel<<<grid, dim3(kBX, kBY, 1), 0, st>>>((const float *)((char *)workspace + L.six), h6, d0,
                                                                 d1, d2, zc, tpx);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" int m16_eigs(const float *h6, int64_t n, float *out6, void *stream)
{
    if (n < 0 || (n > 0 && (!h6 || !out6))) return M16_ERR_BAD_ARG;
    if (n == 0) return M16_OK;
    const int blocks = (int)std::min<int64_t>(8 * kSMs, div_up(n, 256));
    fr_eigs_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(h6, out6, n);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}
