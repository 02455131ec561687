// directions.cu -- the direction kernels of the sign adjustment and the
// transformation completion: detectRidges (src/clcode/detect_ridges.cl:34-102),
// extractMainDirections, completeTransformations and adjustNonRidgeSigns
// (src/clcode/adjust_directions.cl:29-246).
//
// These decide discrete outcomes (ridge or not, nearest ridge point, sign), so
// their arithmetic follows the reference's rounding sequence: explicit _rn
// intrinsics instead of contracted multiply-adds, and the quaternion
// expansion's trigonometry as the float nearest to the exact value (the
// reference's OpenCL C promotes `* 0.5` to double and rounds cos/sin to
// float).  That float comes from a double-float evaluation in single
// precision (ffsincos.cuh) and, where its error bound reaches a rounding
// boundary or the argument lies outside [-4, 4], from double precision.
#include <cuda_runtime.h>
#include <math.h>
#include <float.h>

#include <algorithm>
#include <climits>

#include "common.cuh"
#include "ffsincos.cuh"

namespace m16 {
namespace {

constexpr int kBX = 32, kBY = 8;

// float(sin(x)) and float(cos(x)) of x = (double)v * scale (scale 1 or 0.5):
// single precision where certain, double precision otherwise.  The double
// argument is formed only on the fallback path, so the common path issues no
// FP64 instruction (FP64 runs at a small fraction of the FP32 rate).
__device__ __forceinline__ void sincos_ref(float v, float scale, float *s, float *c)
{
    if (ff::sincos_rn(__fmul_rn(v, scale), s, c)) return;
    double sd, cd;
    sincos((double)v * (double)scale, &sd, &cd);
    *s = (float)sd;
    *c = (float)cd;
}

// qexpand with the reference's precision: half angles rounded to float, the
// cosines and sines rounded to float from their exact values.  theta / 2 is
// exact in float except for subnormal theta, where the rounded half still
// gives the same floats (|x| < 2^-12: sin rounds to the rounded x, cos to 1).
__device__ __forceinline__ void qexpand_ref(float phi, float theta, float psi, float q[4])
{
    const float pp = __fmul_rn(__fadd_rn(phi, psi), 0.5f);
    const float pm = __fmul_rn(__fsub_rn(phi, psi), 0.5f);
    float ct, st, cpp, spp, cpm, spm;
    sincos_ref(theta, 0.5f, &st, &ct);
    sincos_ref(pp, 1.0f, &spp, &cpp);
    sincos_ref(pm, 1.0f, &spm, &cpm);
    q[0] = __fmul_rn(cpp, ct);
    q[1] = __fmul_rn(cpm, st);
    q[2] = __fmul_rn(spm, st);
    q[3] = __fmul_rn(spp, ct);
}

__device__ __forceinline__ float sq_rn(float x) { return __fmul_rn(x, x); }

// columns of quat2matFloat3 (quaternion_math.h:257-289), no contraction
__device__ __forceinline__ void quat_cols(const float q[4], float c0[3], float c1[3], float c2[3])
{
    const float qx2 = sq_rn(q[1]), qy2 = sq_rn(q[2]), qz2 = sq_rn(q[3]);
    const float qwqx = __fmul_rn(q[0], q[1]), qwqy = __fmul_rn(q[0], q[2]), qwqz = __fmul_rn(q[0], q[3]);
    const float qxqy = __fmul_rn(q[1], q[2]), qxqz = __fmul_rn(q[1], q[3]), qyqz = __fmul_rn(q[2], q[3]);
    if (c0) {
        c0[0] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(qy2, qz2)));
        c0[1] = __fmul_rn(2.f, __fadd_rn(qxqy, qwqz));
        c0[2] = __fmul_rn(2.f, __fsub_rn(qxqz, qwqy));
    }
    if (c1) {
        c1[0] = __fmul_rn(2.f, __fsub_rn(qxqy, qwqz));
        c1[1] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(qx2, qz2)));
        c1[2] = __fmul_rn(2.f, __fadd_rn(qyqz, qwqx));
    }
    if (c2) {
        c2[0] = __fmul_rn(2.f, __fadd_rn(qxqz, qwqy));
        c2[1] = __fmul_rn(2.f, __fsub_rn(qyqz, qwqx));
        c2[2] = __fsub_rn(1.f, __fmul_rn(2.f, __fadd_rn(qx2, qy2)));
    }
}

// ---- detectRidges -----------------------------------------------------------
// dirs3 (optional): the main direction (first column) of the same expansion,
// what extractMainDirections computes, written in the same pass
__global__ void __launch_bounds__(kBX * kBY) dr_detect_ridges_kernel(const float *__restrict__ resp,
                                                                     const float *__restrict__ quat3,
                                                                     float *__restrict__ ridge, int d0, int d1,
                                                                     int d2, float threshold,
                                                                     float *__restrict__ dirs3)
{
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y * kBY + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= d2 || y >= d1) return;
    const int64_t i = ((int64_t)z * d1 + y) * d2 + x;
    float q[4], c0[3], c1[3], c2[3];
    qexpand_ref(quat3[3 * i], quat3[3 * i + 1], quat3[3 * i + 2], q);
    quat_cols(q, dirs3 ? c0 : nullptr, c1, c2);
    if (dirs3) {
        dirs3[3 * i] = c0[0];
        dirs3[3 * i + 1] = c0[1];
        dirs3[3 * i + 2] = c0[2];
    }
    const float pos[3] = {(float)z, (float)y, (float)x};
    const int dims[3] = {d0, d1, d2};
    const int64_t s0 = (int64_t)d1 * d2;
    float maxv = -INFINITY;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float a = (float)((-1) * (j < 3) + (j > 4));
        const float b = (float)((j % 3) - 1 + (j == 4));
        float p[3];
        int o[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            p[k] = __fadd_rn(__fadd_rn(pos[k], __fmul_rn(a, c1[k])), __fmul_rn(b, c2[k]));
            o[k] = (int)p[k];   // toward zero, as convert_int3
            p[k] = __fsub_rn(p[k], (float)o[k]);
        }
        const float u[3] = {__fsub_rn(1.f, p[0]), __fsub_rn(1.f, p[1]), __fsub_rn(1.f, p[2])};
        float v = 0.f;
        // all eight corners inside the volume (one test per sample instead of
        // one per corner; o < dims - 1 also holds off a saturated conversion)
        if (o[0] >= 0 && o[1] >= 0 && o[2] >= 0 && o[0] < d0 - 1 && o[1] < d1 - 1 && o[2] < d2 - 1) {
            const float *base = resp + ((int64_t)o[0] * d1 + o[1]) * d2 + o[2];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int r0 = k >> 2, r1 = (k >> 1) & 1, r2 = k & 1;
                const float w0 = r0 ? p[0] : u[0];
                const float w1 = r1 ? p[1] : u[1];
                const float w2 = r2 ? p[2] : u[2];
                const float s = __ldg(base + (r0 ? s0 : 0) + (r1 ? d2 : 0) + r2);
                v = __fadd_rn(v, __fmul_rn(__fmul_rn(__fmul_rn(s, w0), w1), w2));
            }
        } else {
            // corners outside the volume read -1 (detect_ridges.cl)
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int r0 = k >> 2, r1 = (k >> 1) & 1, r2 = k & 1;
                const int a0 = o[0] + r0, a1 = o[1] + r1, a2 = o[2] + r2;
                const float w0 = r0 ? p[0] : u[0];
                const float w1 = r1 ? p[1] : u[1];
                const float w2 = r2 ? p[2] : u[2];
                const bool out = a0 < 0 || a1 < 0 || a2 < 0 || a0 >= dims[0] || a1 >= dims[1] || a2 >= dims[2];
                const float s = out ? -1.f : __ldg(resp + ((int64_t)a0 * d1 + a1) * d2 + a2);
                v = __fadd_rn(v, __fmul_rn(__fmul_rn(__fmul_rn(s, w0), w1), w2));
            }
        }
        maxv = v > maxv ? v : maxv;
    }
    const float r = resp[i];
    // threshold: the largest float not above the reference's double
    // threshold, so r > threshold exactly when (double)r exceeds it
    ridge[i] = (r > threshold && r > maxv) ? 1.f : 0.f;
}

// ---- extractMainDirections ----------------------------------------------------
__global__ void dr_extract_kernel(const float *in3, float *out3, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float q[4], c0[3];
        qexpand_ref(in3[3 * i], in3[3 * i + 1], in3[3 * i + 2], q);
        quat_cols(q, c0, nullptr, nullptr);
        out3[3 * i] = c0[0];
        out3[3 * i + 1] = c0[1];
        out3[3 * i + 2] = c0[2];
    }
}

// ---- completeTransformations ----------------------------------------------------
__device__ __forceinline__ void normalize3(const float v[3], float o[3])
{
    const float l2 = __fadd_rn(__fadd_rn(sq_rn(v[0]), sq_rn(v[1])), sq_rn(v[2]));
    if (l2 == 0.f) { o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; return; }
    const float l = __fsqrt_rn(l2);
    o[0] = __fdiv_rn(v[0], l); o[1] = __fdiv_rn(v[1], l); o[2] = __fdiv_rn(v[2], l);
}

__device__ __forceinline__ float rsqrt_ref(float x) { return __fdiv_rn(1.f, __fsqrt_rn(x)); }

// (float)(1.0 + (double)a - (double)b - (double)c), the reference's rounding
// of mat2quat's diagonal sums.  When every nonzero term is finite with
// 2^-27 <= |t| < 2, each term is a multiple of 2^-50 and every partial sum
// is below 8 in magnitude, so all three double additions are exact and the
// result is the correctly rounded float of the exact sum: here in 64-bit
// integers scaled by 2^50, rounded once by the integer-to-float conversion.
// Other terms (tiny, NaN, infinite) take the double path.
__device__ __forceinline__ float one_plus_minus_minus(float a, float b, float c)
{
    const float lo = 7.450580596923828125e-9f;   // 2^-27
    auto exact = [lo](float t) { return t == 0.f || (fabsf(t) >= lo && fabsf(t) < 2.f); };
    if (exact(a) && exact(b) && exact(c)) {
        const float up = 1125899906842624.f;           // 2^50
        const float down = 8.8817841970012523e-16f;    // 2^-50
        const long long sum = (1LL << 50) + __float2ll_rn(__fmul_rn(a, up)) - __float2ll_rn(__fmul_rn(b, up)) -
                              __float2ll_rn(__fmul_rn(c, up));
        return __fmul_rn(__ll2float_rn(sum), down);
    }
    return (float)(1.0 + (double)a - (double)b - (double)c);
}

// qsqueeze (quaternion_math.h:20-39), scalar part first, written literally
// (products with the 0/1 conditions included: they decide the sign of zero
// that atan2 sees).  The reference forms v[1] and atan2's denominator in
// double: (pi or 0) * f2 + ac * nf2 and (0.5 - x) * f2 + y * nf2.  One of
// f2, nf2 is zero, so one term is +-0 (or NaN) and the sum is the other
// term, with the same sign-of-zero rules in float; 0.5 - x rounded from
// double is the float difference (Figueroa 1995).  Float gives the same bits.
__device__ __forceinline__ void qsqueeze_ref(const float q[4], float v[3])
{
    const float q1spq2s = __fadd_rn(sq_rn(q[1]), sq_rn(q[2]));
    const bool c1 = q1spq2s < FLT_EPSILON;
    const bool c2 = c1 || __fsub_rn(1.f, q1spq2s) < FLT_EPSILON;
    const float f2 = c2 ? 1.f : 0.f, nf2 = c2 ? 0.f : 1.f;
    const float q1q3 = __fmul_rn(q[1], q[3]), q2q0 = __fmul_rn(q[2], q[0]);
    const float q1q0 = __fmul_rn(q[1], q[0]), q2q3 = __fmul_rn(q[2], q[3]);
    auto satan2 = [](float a, float b) { return (a == 0.f && b == 0.f) ? 0.f : atan2f(a, b); };
    v[0] = satan2(__fadd_rn(q1q3, q2q0), __fsub_rn(q1q0, q2q3));
    const float ac = acosf(fminf(fmaxf(__fsub_rn(1.f, __fmul_rn(2.f, q1spq2s)), -1.f), 1.f));
    const float pi_f = 3.14159265358979323846f;   // float nearest to pi, as (float) of the double
    v[1] = __fadd_rn(__fmul_rn(c1 ? 0.f : pi_f, f2), __fmul_rn(ac, nf2));
    float at2 = __fadd_rn(__fmul_rn(__fsub_rn(__fmul_rn(q[1], q[2]), __fmul_rn(q[0], q[3])), f2),
                          __fmul_rn(__fsub_rn(q1q3, q2q0), nf2));
    const float den = __fadd_rn(__fmul_rn(__fsub_rn(0.5f, __fadd_rn(sq_rn(q[2]), sq_rn(q[3]))), f2),
                                __fmul_rn(__fadd_rn(q1q0, q2q3), nf2));
    at2 = satan2(at2, den);
    v[2] = __fadd_rn(__fmul_rn(__fadd_rn(-at2, __fmul_rn(v[0], c1 ? -1.f : 1.f)), f2), __fmul_rn(at2, nf2));
}

__global__ void dr_complete_kernel(const float *in3, float *out3, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v[3] = {in3[3 * i], in3[3 * i + 1], in3[3 * i + 2]};
        float e0[3], e1[3], e2[3], t[3];
        normalize3(v, e0);
        if (fabsf(e0[0]) > fabsf(e0[1])) { t[0] = -e0[2]; t[1] = 0.f; t[2] = e0[0]; }
        else { t[0] = 0.f; t[1] = e0[2]; t[2] = -e0[1]; }
        normalize3(t, e1);
        e2[0] = __fsub_rn(__fmul_rn(e0[1], e1[2]), __fmul_rn(e0[2], e1[1]));
        e2[1] = __fsub_rn(__fmul_rn(e0[2], e1[0]), __fmul_rn(e0[0], e1[2]));
        e2[2] = __fsub_rn(__fmul_rn(e0[0], e1[1]), __fmul_rn(e0[1], e1[0]));
        // mat2quat (quaternion_math.h:301-340), m[row][col] with columns e0, e1, e2
        const float m00 = e0[0], m01 = e1[0], m02 = e2[0];
        const float m10 = e0[1], m11 = e1[1], m12 = e2[1];
        const float m20 = e0[2], m21 = e1[2], m22 = e2[2];
        // The reference rounds s + 1, r * 0.5 and 0.25 / s from double.  Each
        // is one operation on floats, and a double result rounded to float is
        // the correctly rounded float result (53 >= 2 * 24 + 2 bits, Figueroa
        // 1995), so the float operations below give the same bits; the
        // diagonal sums go through one_plus_minus_minus.
        float q[4];
        float s = __fadd_rn(__fadd_rn(m00, m11), m22);
        if (s > 0.f) {
            s = __fmul_rn(rsqrt_ref(__fadd_rn(s, 1.f)), 0.5f);
            q[0] = __fdiv_rn(0.25f, s);
            q[1] = __fmul_rn(__fsub_rn(m21, m12), s);
            q[2] = __fmul_rn(__fsub_rn(m02, m20), s);
            q[3] = __fmul_rn(__fsub_rn(m10, m01), s);
        } else if (m00 > m11 && m00 > m22) {
            s = __fmul_rn(rsqrt_ref(one_plus_minus_minus(m00, m11, m22)), 0.5f);
            q[0] = __fmul_rn(__fsub_rn(m21, m12), s);
            q[1] = __fdiv_rn(0.25f, s);
            q[2] = __fmul_rn(__fadd_rn(m01, m10), s);
            q[3] = __fmul_rn(__fadd_rn(m02, m20), s);
        } else if (m11 > m22) {
            s = __fmul_rn(rsqrt_ref(one_plus_minus_minus(m11, m00, m22)), 0.5f);
            q[0] = __fmul_rn(__fsub_rn(m02, m20), s);
            q[1] = __fmul_rn(__fadd_rn(m01, m10), s);
            q[2] = __fdiv_rn(0.25f, s);
            q[3] = __fmul_rn(__fadd_rn(m12, m21), s);
        } else {
            s = __fmul_rn(rsqrt_ref(one_plus_minus_minus(m22, m00, m11)), 0.5f);
            q[0] = __fmul_rn(__fsub_rn(m10, m01), s);
            q[1] = __fmul_rn(__fadd_rn(m02, m20), s);
            q[2] = __fmul_rn(__fadd_rn(m12, m21), s);
            q[3] = __fdiv_rn(0.25f, s);
        }
        float sq[3];
        qsqueeze_ref(q, sq);
        out3[3 * i] = sq[0];
        out3[3 * i + 1] = sq[1];
        out3[3 * i + 2] = sq[2];
    }
}

// ---- adjustNonRidgeSigns ----------------------------------------------------------
// Brute-force nearest ridge point per voxel: ridge points are staged through
// shared memory in tiles; every thread scans them in ascending index order with
// a strict <, so the lowest index wins ties exactly as in the reference.
constexpr int kTile = 1024;

__global__ void __launch_bounds__(256) dr_adjust_kernel(float *__restrict__ dirs3, const uint16_t *__restrict__ coords,
                                                        const float *__restrict__ rdirs, int64_t R, int d0, int d1,
                                                        int d2, float s0, float s1, float s2)
{
    __shared__ float sc[3][kTile];
    const int64_t n = (int64_t)d0 * d1 * d2;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool act = i < n;
    float p0 = 0.f, p1 = 0.f, p2 = 0.f;
    if (act) {
        p2 = (float)(i % d2);
        p1 = (float)((i / d2) % d1);
        p0 = (float)(i / ((int64_t)d1 * d2));
    }
    float best = INFINITY;
    int64_t bj = 0;
    for (int64_t t0 = 0; t0 < R; t0 += kTile) {
        const int cnt = (int)(R - t0 < kTile ? R - t0 : kTile);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
            sc[0][k] = (float)coords[3 * (t0 + k)];
            sc[1][k] = (float)coords[3 * (t0 + k) + 1];
            sc[2][k] = (float)coords[3 * (t0 + k) + 2];
        }
        __syncthreads();
        if (act) {
            for (int k = 0; k < cnt; ++k) {
                const float f0 = __fmul_rn(fabsf(__fsub_rn(p0, sc[0][k])), s0);
                const float f1 = __fmul_rn(fabsf(__fsub_rn(p1, sc[1][k])), s1);
                const float f2 = __fmul_rn(fabsf(__fsub_rn(p2, sc[2][k])), s2);
                const float d = __fadd_rn(__fadd_rn(__fmul_rn(f0, f0), __fmul_rn(f1, f1)), __fmul_rn(f2, f2));
                if (d < best) { best = d; bj = t0 + k; }
            }
        }
    }
    if (!act || R == 0) return;
    float *v = dirs3 + 3 * i;
    const float w0 = rdirs[3 * bj], w1 = rdirs[3 * bj + 1], w2 = rdirs[3 * bj + 2];
    const float dot = __fadd_rn(__fadd_rn(__fmul_rn(v[0], w0), __fmul_rn(v[1], w1)), __fmul_rn(v[2], w2));
    if (dot < 0.f) {
        v[0] = -v[0];
        v[1] = -v[1];
        v[2] = -v[2];
    }
}

// ---- adjustNonRidgeSigns over a cell index ----------------------------------------
// The same nearest ridge point (smallest distance, then smallest index) found
// without visiting every point: the ridge points are bucketed into cubic cells
// of c voxels a side, and each voxel scans Chebyshev shells of cells around
// its own cell.  A cell is skipped only when a lower bound of every distance
// in it exceeds the best distance so far, and the scan ends when the bound of
// everything outside the scanned block does; both bounds are evaluated with
// the distance's own rounded operations on the smallest possible per-axis
// offsets, and every rounded operation involved is monotone, so no point
// that could win (ties included) is ever skipped.  Equal distances resolve
// by comparing indices, so the order of the points inside a cell is free.
struct CellGrid {
    int c;                 // cell side in voxels
    int g0, g1, g2;        // cells per axis
    int d0, d1, d2;        // the volume (coordinates beyond it are clamped into its last cells)
    int64_t ncells;
};

constexpr int64_t kMaxCells = (int64_t)1 << 22;   // the two-level scan covers 4096 x 1024 cells

inline CellGrid make_cell_grid(int d0, int d1, int d2, int64_t R)
{
    const double n = (double)d0 * d1 * d2;
    // about four ridge points per cell on average
    int c = (int)ceil(cbrt(4.0 * n / (double)std::max<int64_t>(R, 1)));
    c = std::max(2, std::min(c, 1 << 16));
    CellGrid g;
    g.d0 = d0; g.d1 = d1; g.d2 = d2;
    for (;; ++c) {
        g.c = c;
        g.g0 = (int)div_up(d0, c); g.g1 = (int)div_up(d1, c); g.g2 = (int)div_up(d2, c);
        g.ncells = (int64_t)g.g0 * g.g1 * g.g2;
        if (g.ncells <= kMaxCells) break;
    }
    return g;
}

constexpr int kScanItems = 1024;   // cells per scan block (256 threads x 4)

struct NrLayout {
    size_t count, start, bsum, pts, total;
    int64_t nblocks;
};

inline NrLayout nr_layout(const CellGrid &g, int64_t R)
{
    NrLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L.nblocks = div_up(g.ncells, kScanItems);
    L.count = take((size_t)g.ncells * 4);
    L.start = take((size_t)(g.ncells + 1) * 4);
    L.bsum = take((size_t)(L.nblocks + 1) * 4);
    L.pts = take((size_t)R * 16);
    L.total = off;
    return L;
}

// cell of a ridge point; a coordinate beyond the volume goes to the last cell
// of its axis (its distances only grow, so every bound stays a bound)
__device__ __forceinline__ int64_t cell_of(int a0, int a1, int a2, CellGrid g)
{
    a0 = min(a0, g.d0 - 1); a1 = min(a1, g.d1 - 1); a2 = min(a2, g.d2 - 1);
    return ((int64_t)(a0 / g.c) * g.g1 + a1 / g.c) * g.g2 + a2 / g.c;
}

__global__ void nr_count_kernel(const uint16_t *__restrict__ coords, int64_t R, CellGrid g,
                                unsigned *__restrict__ count)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < R; j += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(count + cell_of(coords[3 * j], coords[3 * j + 1], coords[3 * j + 2], g), 1u);
}

// exclusive scan of the counts, in blocks of kScanItems: local scan + block sums
__global__ void __launch_bounds__(256) nr_scan_local_kernel(const unsigned *__restrict__ count, int64_t ncells,
                                                            unsigned *__restrict__ start, unsigned *__restrict__ bsum)
{
    __shared__ unsigned s[256];
    const int64_t base = blockIdx.x * (int64_t)kScanItems + 4 * threadIdx.x;
    unsigned v[4], t = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < ncells ? count[base + k] : 0u;
        t += v[k];
    }
    s[threadIdx.x] = t;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {   // inclusive Hillis-Steele over the thread totals
        const unsigned add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
        __syncthreads();
        s[threadIdx.x] += add;
        __syncthreads();
    }
    unsigned run = s[threadIdx.x] - t;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < ncells) start[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 255) bsum[blockIdx.x] = s[255];
}

// exclusive scan of the block sums in place (one block; nblocks <= 4096)
__global__ void __launch_bounds__(1024) nr_scan_blocks_kernel(unsigned *bsum, int64_t nblocks)
{
    __shared__ unsigned s[1024];
    unsigned v[4], t = 0;
    const int64_t base = 4 * (int64_t)threadIdx.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < nblocks ? bsum[base + k] : 0u;
        t += v[k];
    }
    s[threadIdx.x] = t;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
        __syncthreads();
        s[threadIdx.x] += add;
        __syncthreads();
    }
    unsigned run = s[threadIdx.x] - t;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < nblocks) bsum[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 1023) bsum[nblocks] = s[1023];
}

// start[i] += offset of its block; start[ncells] = R; counts reset to 0 (the
// scatter reuses them as fill counters)
__global__ void nr_scan_add_kernel(unsigned *__restrict__ start, unsigned *__restrict__ count,
                                   const unsigned *__restrict__ bsum, int64_t ncells, int64_t nblocks)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= ncells; i += (int64_t)gridDim.x * blockDim.x) {
        if (i == ncells) { start[i] = bsum[nblocks]; continue; }
        start[i] += bsum[i / kScanItems];
        count[i] = 0u;
    }
}

__global__ void nr_scatter_kernel(const uint16_t *__restrict__ coords, int64_t R, CellGrid g,
                                  const unsigned *__restrict__ start, unsigned *__restrict__ fill,
                                  float4 *__restrict__ pts)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < R; j += (int64_t)gridDim.x * blockDim.x) {
        const int a0 = coords[3 * j], a1 = coords[3 * j + 1], a2 = coords[3 * j + 2];
        const int64_t c = cell_of(a0, a1, a2, g);
        const unsigned pos = start[c] + atomicAdd(fill + c, 1u);
        pts[pos] = make_float4((float)a0, (float)a1, (float)a2, __int_as_float((int)j));
    }
}

// the reference's distance: ((|dp0| s0)^2 + (|dp1| s1)^2) + (|dp2| s2)^2, each step rounded
__device__ __forceinline__ float ref_dist(float f0, float f1, float f2)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(f0, f0), __fmul_rn(f1, f1)), __fmul_rn(f2, f2));
}

// lower bound of the rounded squared term of an axis for every point outside
// cells [clo, chi] of that axis (infinite when the block reaches both ends)
__device__ __forceinline__ float block_gap(int p, int clo, int chi, int ncell, int c, float s)
{
    float o = INFINITY;
    if (clo > 0) o = fminf(o, __fmul_rn((float)(p - clo * c + 1), s));
    if (chi < ncell - 1) o = fminf(o, __fmul_rn((float)((chi + 1) * c - p), s));
    return o == INFINITY ? INFINITY : __fmul_rn(o, o);
}

// smallest |p - c| over integer c in [lo, hi] (0 inside), times s, rounded
__device__ __forceinline__ float axis_gap(int p, int lo, int hi, float s)
{
    const int m = p < lo ? lo - p : (p > hi ? p - hi : 0);
    return __fmul_rn((float)m, s);
}

// Each warp takes a kNrPX x kNrPY patch of the block's 32 x 8 tile (x, y),
// so that its voxels fall into fewer cells and walk the same cells' point
// lists together.  Measured on GB300 (256^3 helix, R = 1.9 M, 4^3 cells):
// 32 x 1 2.28 ms, 16 x 2 2.19 ms, 8 x 4 2.29 ms, 4 x 8 2.30 ms.
#ifndef M16_NR_PATCH
#define M16_NR_PATCH 16
#endif
constexpr int kNrPX = M16_NR_PATCH, kNrPY = 32 / kNrPX;
static_assert(kBX % kNrPX == 0 && kBY % kNrPY == 0 && (kBX / kNrPX) * (kBY / kNrPY) == kBY,
              "a warp per patch, the block's 8 warps tiling 32 x 8");

__global__ void __launch_bounds__(kBX * kBY) dr_adjust_indexed_kernel(
    float *__restrict__ dirs3, const float4 *__restrict__ pts, const unsigned *__restrict__ start,
    const float *__restrict__ rdirs, CellGrid g, int d0, int d1, int d2, float s0, float s1, float s2)
{
    const int w = threadIdx.y, lane = threadIdx.x;
    const int x = blockIdx.x * kBX + (w % (kBX / kNrPX)) * kNrPX + lane % kNrPX;
    const int y = blockIdx.y * kBY + (w / (kBX / kNrPX)) * kNrPY + lane / kNrPX;
    const int z = blockIdx.z;
    if (x >= d2 || y >= d1) return;
    const float p0 = (float)z, p1 = (float)y, p2 = (float)x;
    const int cz = z / g.c, cy = y / g.c, cx = x / g.c;
    float best = INFINITY;
    int bj = INT_MAX;
    const int rmax = max(max(max(cz, g.g0 - 1 - cz), max(cy, g.g1 - 1 - cy)), max(cx, g.g2 - 1 - cx));
    for (int r = 0; r <= rmax; ++r) {
        for (int dz = -r; dz <= r; ++dz) {
            const int qz = cz + dz;
            if (qz < 0 || qz >= g.g0) continue;
            const float gz = axis_gap(z, qz * g.c, qz * g.c + g.c - 1, s0);
            for (int dy = -r; dy <= r; ++dy) {
                const int qy = cy + dy;
                if (qy < 0 || qy >= g.g1) continue;
                const float gy = axis_gap(y, qy * g.c, qy * g.c + g.c - 1, s1);
                const bool face = dz == -r || dz == r || dy == -r || dy == r;
                const int step = face ? 1 : 2 * r;   // off the faces only dx = -r and dx = r lie on the shell
                for (int dx = -r; dx <= r; dx += step) {
                    const int qx = cx + dx;
                    if (qx >= 0 && qx < g.g2) {
                        const float gx = axis_gap(x, qx * g.c, qx * g.c + g.c - 1, s2);
                        if (!(ref_dist(gz, gy, gx) > best)) {
                            const int64_t cell = ((int64_t)qz * g.g1 + qy) * g.g2 + qx;
                            const unsigned e = __ldg(start + cell + 1);
                            for (unsigned k = __ldg(start + cell); k < e; ++k) {
                                const float4 q = __ldg(pts + k);
                                const float f0 = __fmul_rn(fabsf(__fsub_rn(p0, q.x)), s0);
                                const float f1 = __fmul_rn(fabsf(__fsub_rn(p1, q.y)), s1);
                                const float f2 = __fmul_rn(fabsf(__fsub_rn(p2, q.z)), s2);
                                const float d = ref_dist(f0, f1, f2);
                                const int j = __float_as_int(q.w);
                                if (d < best || (d == best && j < bj)) { best = d; bj = j; }
                            }
                        }
                    }
                    if (r == 0) break;
                }
            }
        }
        // everything outside the scanned block differs on some axis by more
        // than the block reaches on that axis (no points lie beyond the grid)
        const float oz = fminf(block_gap(z, cz - r, cz + r, g.g0, g.c, s0), block_gap(y, cy - r, cy + r, g.g1, g.c, s1));
        const float lo = fminf(oz, block_gap(x, cx - r, cx + r, g.g2, g.c, s2));
        if (lo > best) break;
    }
    if (bj == INT_MAX) return;
    float *v = dirs3 + 3 * (((int64_t)z * d1 + y) * d2 + x);
    const float w0 = __ldg(rdirs + 3 * (int64_t)bj), w1 = __ldg(rdirs + 3 * (int64_t)bj + 1),
                w2 = __ldg(rdirs + 3 * (int64_t)bj + 2);
    const float dot = __fadd_rn(__fadd_rn(__fmul_rn(v[0], w0), __fmul_rn(v[1], w1)), __fmul_rn(v[2], w2));
    if (dot < 0.f) {
        v[0] = -v[0];
        v[1] = -v[1];
        v[2] = -v[2];
    }
}

inline int blocks1d(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(16 * kSMs, div_up(n, 256))); }

}  // namespace
}  // namespace m16

using namespace m16;

namespace {
// the largest float not above t (NaN for NaN): for every float r,
// r > float_at_or_below(t) exactly when (double)r > t
float float_at_or_below(double t)
{
    if (t != t) return NAN;
    float f = (float)t;
    if ((double)f > t) f = nextafterf(f, -INFINITY);
    return f;
}
}  // namespace

extern "C" int m16_detect_ridges(const float *resp, const float *quat3, int32_t d0, int32_t d1, int32_t d2,
                                 double threshold, float *ridge, void *stream)
{
    if (d0 < 1 || d1 < 1 || d2 < 1 || d0 > 65535) return M16_ERR_BAD_SHAPE;
    if (!resp || !quat3 || !ridge) return M16_ERR_BAD_ARG;
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)d0);
    dr_detect_ridges_kernel<<<grid, dim3(kBX, kBY, 1), 0, (cudaStream_t)stream>>>(resp, quat3, ridge, d0, d1, d2,
                                                                                 float_at_or_below(threshold),
                                                                                 nullptr);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" int m16_detect_ridges_main_directions(const float *resp, const float *quat3, int32_t d0, int32_t d1,
                                                 int32_t d2, double threshold, float *ridge, float *dirs3, void *stream)
{
    if (d0 < 1 || d1 < 1 || d2 < 1 || d0 > 65535) return M16_ERR_BAD_SHAPE;
    if (!resp || !quat3 || !ridge || !dirs3) return M16_ERR_BAD_ARG;
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)d0);
    dr_detect_ridges_kernel<<<grid, dim3(kBX, kBY, 1), 0, (cudaStream_t)stream>>>(resp, quat3, ridge, d0, d1, d2,
                                                                                 float_at_or_below(threshold),
                                                                                 dirs3);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" int m16_extract_main_directions(const float *quat3, int64_t n, float *dirs3, void *stream)
{
    if (n < 0 || (n > 0 && (!quat3 || !dirs3))) return M16_ERR_BAD_ARG;
    if (n == 0) return M16_OK;
    dr_extract_kernel<<<blocks1d(n), 256, 0, (cudaStream_t)stream>>>(quat3, dirs3, n);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" int m16_complete_transformations(const float *dirs3, int64_t n, float *quat3, void *stream)
{
    if (n < 0 || (n > 0 && (!quat3 || !dirs3))) return M16_ERR_BAD_ARG;
    if (n == 0) return M16_OK;
    dr_complete_kernel<<<blocks1d(n), 256, 0, (cudaStream_t)stream>>>(dirs3, quat3, n);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" int m16_adjust_nonridge_signs(float *dirs3, int32_t d0, int32_t d1, int32_t d2, const uint16_t *coords,
                                         const float *rdirs, int64_t num_ridge, const double *scaling3,
                                         void *stream)
{
    if (d0 < 1 || d1 < 1 || d2 < 1) return M16_ERR_BAD_SHAPE;
    if (!dirs3 || !scaling3 || num_ridge < 1 || !coords || !rdirs) return M16_ERR_BAD_ARG;
    const int64_t n = (int64_t)d0 * d1 * d2;
    const int blocks = (int)div_up(n, 256);
    dr_adjust_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(dirs3, coords, rdirs, num_ridge, d0, d1, d2,
                                                               (float)scaling3[0], (float)scaling3[1],
                                                               (float)scaling3[2]);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" size_t m16_adjust_nonridge_signs_workspace_bytes(int32_t d0, int32_t d1, int32_t d2, int64_t num_ridge)
{
    if (d0 < 1 || d1 < 1 || d2 < 1 || num_ridge < 1) return 0;
    return nr_layout(make_cell_grid(d0, d1, d2, num_ridge), num_ridge).total;
}

extern "C" int m16_adjust_nonridge_signs_indexed(float *dirs3, int32_t d0, int32_t d1, int32_t d2,
                                                 const uint16_t *coords, const float *rdirs, int64_t num_ridge,
                                                 const double *scaling3, void *workspace, size_t workspace_bytes,
                                                 void *stream)
{
    if (d0 < 1 || d1 < 1 || d2 < 1 || d0 > 65535) return M16_ERR_BAD_SHAPE;
    if (!dirs3 || !scaling3 || num_ridge < 1 || num_ridge > (int64_t)INT32_MAX || !coords || !rdirs)
        return M16_ERR_BAD_ARG;
    for (int k = 0; k < 3; ++k)
        if (!(scaling3[k] > 0.0) || !isfinite(scaling3[k])) return M16_ERR_BAD_ARG;
    const CellGrid g = make_cell_grid(d0, d1, d2, num_ridge);
    const NrLayout L = nr_layout(g, num_ridge);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    unsigned *count = (unsigned *)(ws + L.count), *start = (unsigned *)(ws + L.start), *bsum = (unsigned *)(ws + L.bsum);
    float4 *pts = (float4 *)(ws + L.pts);
    M16_CUDA_TRY(cudaMemsetAsync(count, 0, (size_t)g.ncells * 4, st));
    nr_count_kernel<<<blocks1d(num_ridge), 256, 0, st>>>(coords, num_ridge, g, count);
    nr_scan_local_kernel<<<(unsigned)L.nblocks, 256, 0, st>>>(count, g.ncells, start, bsum);
    nr_scan_blocks_kernel<<<1, 1024, 0, st>>>(bsum, L.nblocks);
    nr_scan_add_kernel<<<blocks1d(g.ncells + 1), 256, 0, st>>>(start, count, bsum, g.ncells, L.nblocks);
    nr_scatter_kernel<<<blocks1d(num_ridge), 256, 0, st>>>(coords, num_ridge, g, start, count, pts);
    const dim3 grid((unsigned)div_up(d2, kBX), (unsigned)div_up(d1, kBY), (unsigned)d0);
    dr_adjust_indexed_kernel<<<grid, dim3(kBX, kBY, 1), 0, st>>>(dirs3, pts, start, rdirs, g, d0, d1, d2,
                                                                (float)scaling3[0], (float)scaling3[1],
                                                                (float)scaling3[2]);
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}
