// sweeps.cuh -- the two per-iteration sweeps of the ATV continuous max-flow,
// shared by the single-solve path (maxflow.cu) and the batched engine
// (batched.cu).  One thread walks one (y, x) column from z0 to z1; see
// maxflow.cu for the reference equations (src/clcode-anisotropic/update_qp.cl).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"

#ifndef M16_MF_ZB
#define M16_MF_ZB 2
#endif
// z-slices whose loads the label sweep issues together: 4 measured fastest on
// GB300 (the label sweep holds fewer values per slice than the flow sweep)
#ifndef M16_MF_UZB
#define M16_MF_UZB 4
#endif

namespace m16 {

constexpr int kMfZB = M16_MF_ZB;    // z-slices whose loads the flow sweep issues together
constexpr int kMfUZB = M16_MF_UZB;  // the same for the label sweep

// where the projection radius alpha comes from
// kAlphaSource: read `alpha` and, when exp_alpha is set, use w * exp(neg_inv_decay2 * value)
// (one code path for instances with an alpha field and with (weighting, decay))
enum AlphaMode { kAlphaScalar = 0, kAlphaArray = 1, kAlphaFromGrad2 = 2, kAlphaSource = 3 };

// Everything one instance's flow sweep reads and writes.
struct FlowView {
    int d0, d1, d2;
    float ss0, ss1, ss2;                       // steps / voxel size, scaled (SS0-2)
    float sq0, sq1, sq2, isq0, isq1, isq2;     // sqrt of the constant eigenvalues and reciprocals
    float alpha_scalar;                        // kAlphaScalar
    const float *alpha;                        // kAlphaArray
    const float *grad2;                        // kAlphaFromGrad2: alpha = w * exp(-grad2 / decay^2)
    float w, neg_inv_decay2;
    const float *sqeigs;                       // per-voxel sqrt eigenvalues (POINTWISE)
    const float4 *q4;                          // expanded quaternions
    const float *tmp;
    float *hp0, *hp1, *hp2;
};

// Everything one instance's label sweep reads and writes.
struct LabelView {
    int d0, d1, d2;
    float rcc, rs0, rs1, rs2;
    const float *hp0, *hp1, *hp2;
    const float *cs, *ct;
    const uint8_t *labels;
    float *pt, *u, *tmp;
};

// P at one voxel (update_qp.cl:150-232): g = steps * grad tmp from the
// voxel's tmp (tc) and its forward neighbours (tz, ty, tx; each used only
// where its flag says the neighbour exists), p = H^-1 hp + H^T g projected
// onto |p| <= rad, returns hp = H p.  (s0v, s1v, s2v) = sqrt of the
// eigenvalues, (i0v, i1v, i2v) their reciprocals.
__device__ __forceinline__ float3 flow_point(float ss0, float ss1, float ss2, float tc, float tz, float ty, float tx,
                                             bool zin, bool yin, bool xin, float4 q, float rad, float h0, float h1,
                                             float h2, float s0v, float s1v, float s2v, float i0v, float i1v,
                                             float i2v)
{
    const float3 g = make_float3(zin ? (tz - tc) * ss0 : 0.f, yin ? (ty - tc) * ss1 : 0.f,
                                 xin ? (tx - tc) * ss2 : 0.f);
    const Rot R = quat2rot(q);
    const float3 rg = rot_t(R, g);
    const float3 rh = rot_t(R, make_float3(h0, h1, h2));
    float3 p = make_float3(rh.x * i0v + rg.x * s0v, rh.y * i1v + rg.y * s1v, rh.z * i2v + rg.z * s2v);
    const float nrm = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
    const float sc = nrm > rad ? rad / nrm : 1.f;
    p = make_float3(p.x * sc * s0v, p.y * sc * s1v, p.z * sc * s2v);
    return rot(R, p);
}

// U at one voxel (update_qp.cl:241-300 with update_tmp :311-316 fused):
// div(hp) from the voxel's hp (h0, h1, h2) and its backward neighbours'
// (h0m, h1m, h2m; z only where zlo, the own component only where the forward
// flag is set), then p_s, p_t, u and tmp = err - u / cc.  Returns err.
// p_s = min(div + p_t - (u - s_off)/cc, C_s); p_t = min(-div + p_s + (u - t_off)/cc, C_t)
// with (s_off, t_off) = (1, 0) unsupervised and (!(l & 2), l & 1) with seeds l.
template <bool SUPERVISED>
__device__ __forceinline__ float label_point(float rcc, float rs0, float rs1, float rs2, float h0, float h1, float h2,
                                             float h0m, float h1m, float h2m, bool zlo, bool zhi, bool yhi, bool xhi,
                                             float uo, float ptv, float csv, float ctv, uint8_t lab, float &ptn,
                                             float &un, float &tmpv)
{
    const float a0 = (zhi ? h0 : 0.f) - (zlo ? h0m : 0.f);
    const float a1 = (yhi ? h1 : 0.f) - h1m;
    const float a2 = (xhi ? h2 : 0.f) - h2m;
    const float div = a0 * rs0 + a1 * rs1 + a2 * rs2;
    float s_off = 1.f, t_off = 0.f;
    if (SUPERVISED) {
        s_off = (float)(!(lab & 2));
        t_off = (float)(lab & 1);
    }
    const float psx = div + ptv - rcc * (uo - s_off);
    const float ps = csv < psx ? csv : psx;
    const float ptx = -div + ps + rcc * (uo - t_off);
    ptn = ctv < ptx ? ctv : ptx;
    const float err = div - ps + ptn;
    un = uo - err / rcc;
    tmpv = err - un * rcc;
    return err;
}

// P: p = H^-1 hp + H^T (steps grad tmp), projected onto |p| <= alpha, hp = H p
// (update_qp.cl:150-232) for voxels (z0..z1, y, x).
template <bool POINTWISE, int ALPHA, int kFZB = kMfZB>
__device__ __forceinline__ void flow_column(const FlowView &a, int x, int y, int z0, int z1)
{
    const int64_t s0 = (int64_t)a.d1 * a.d2;
    int64_t i = ((int64_t)z0 * a.d1 + y) * a.d2 + x;
    const bool yin = y < a.d1 - 1, xin = x < a.d2 - 1;
    float t = __ldg(a.tmp + i);
    for (int zb = z0; zb < z1; zb += kFZB, i += kFZB * s0) {
        float tz[kFZB], ty[kFZB], tx[kFZB], al[kFZB], h0[kFZB], h1[kFZB], h2[kFZB];
        float4 q[kFZB];
        float se0[kFZB], se1[kFZB], se2[kFZB];
#pragma unroll
        for (int k = 0; k < kFZB; ++k) {
            if (zb + k < z1) {
                const int64_t j = i + k * s0;
                tz[k] = (zb + k < a.d0 - 1) ? __ldg(a.tmp + j + s0) : 0.f;
                ty[k] = yin ? __ldg(a.tmp + j + a.d2) : 0.f;
                tx[k] = xin ? __ldg(a.tmp + j + 1) : 0.f;
                q[k] = __ldg(a.q4 + j);
                if (ALPHA == kAlphaArray) al[k] = __ldg(a.alpha + j);
                else if (ALPHA == kAlphaFromGrad2) al[k] = __ldg(a.grad2 + j);
                else al[k] = a.alpha_scalar;
                h0[k] = a.hp0[j];
                h1[k] = a.hp1[j];
                h2[k] = a.hp2[j];
                if (POINTWISE) {
                    se0[k] = __ldg(a.sqeigs + 3 * j);
                    se1[k] = __ldg(a.sqeigs + 3 * j + 1);
                    se2[k] = __ldg(a.sqeigs + 3 * j + 2);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kFZB; ++k) {
            if (zb + k < z1) {
                const int64_t j = i + k * s0;
                const float tc = k == 0 ? t : tz[k - 1];
                const bool zin = zb + k < a.d0 - 1;
                float s0v = a.sq0, s1v = a.sq1, s2v = a.sq2, i0v = a.isq0, i1v = a.isq1, i2v = a.isq2;
                if (POINTWISE) {
                    s0v = se0[k]; s1v = se1[k]; s2v = se2[k];
                    i0v = 1.f / s0v; i1v = 1.f / s1v; i2v = 1.f / s2v;
                }
                const float rad = ALPHA == kAlphaFromGrad2 ? a.w * expf(a.neg_inv_decay2 * al[k]) : al[k];
                const float3 h = flow_point(a.ss0, a.ss1, a.ss2, tc, tz[k], ty[k], tx[k], zin, yin, xin, q[k], rad,
                                            h0[k], h1[k], h2[k], s0v, s1v, s2v, i0v, i1v, i2v);
                a.hp0[j] = h.x;
                a.hp1[j] = h.y;
                a.hp2[j] = h.z;
            }
        }
        t = tz[kFZB - 1];
    }
}

// U: div(hp), p_s, p_t, u, and tmp = err - u / cc (update_qp.cl:241-300 with
// update_tmp :311-316 fused) for voxels (z0..z1, y, x); returns sum |err|.
template <bool SUPERVISED, int ZB = kMfUZB>
__device__ __forceinline__ float label_column(const LabelView &a, int x, int y, int z0, int z1)
{
    float acc = 0.f;
    const int64_t s0 = (int64_t)a.d1 * a.d2;
    int64_t i = ((int64_t)z0 * a.d1 + y) * a.d2 + x;
    const bool ylo = y > 0, xlo = x > 0, yhi = y < a.d1 - 1, xhi = x < a.d2 - 1;
    float h0m = z0 > 0 ? __ldg(a.hp0 + i - s0) : 0.f;
    for (int zb = z0; zb < z1; zb += ZB, i += ZB * s0) {
        float h0[ZB], h1[ZB], h2[ZB], h1m[ZB], h2m[ZB], uo[ZB], ptv[ZB], csv[ZB],
            ctv[ZB];
        uint8_t lab[ZB];
#pragma unroll
        for (int k = 0; k < ZB; ++k) {
            if (zb + k < z1) {
                const int64_t j = i + k * s0;
                h0[k] = __ldg(a.hp0 + j);
                h1[k] = __ldg(a.hp1 + j);
                h2[k] = __ldg(a.hp2 + j);
                h1m[k] = ylo ? __ldg(a.hp1 + j - a.d2) : 0.f;
                h2m[k] = xlo ? __ldg(a.hp2 + j - 1) : 0.f;
                uo[k] = a.u[j];
                ptv[k] = a.pt[j];
                csv[k] = __ldg(a.cs + j);
                ctv[k] = __ldg(a.ct + j);
                if (SUPERVISED) lab[k] = __ldg(a.labels + j);
            }
        }
#pragma unroll
        for (int k = 0; k < ZB; ++k) {
            if (zb + k < z1) {
                const int64_t j = i + k * s0;
                const int z = zb + k;
                const float prev0 = k == 0 ? h0m : h0[k - 1];
                float ptn, un, tmpv;
                const float err = label_point<SUPERVISED>(a.rcc, a.rs0, a.rs1, a.rs2, h0[k], h1[k], h2[k], prev0,
                                                          h1m[k], h2m[k], z > 0, z < a.d0 - 1, yhi, xhi, uo[k],
                                                          ptv[k], csv[k], ctv[k], SUPERVISED ? lab[k] : (uint8_t)0,
                                                          ptn, un, tmpv);
                a.pt[j] = ptn;
                a.u[j] = un;
                a.tmp[j] = tmpv;
                acc += fabsf(err);
            }
        }
        h0m = h0[ZB - 1];
    }
    return acc;
}

}  // namespace m16
