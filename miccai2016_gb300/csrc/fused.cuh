// fused.cuh -- one kernel per max-flow iteration: the flow sweep (P) and the
// label sweep (U) of the same iteration fused, for the single-solve path and
// the batched engine.
//
// U at voxel v needs the new flow field at v and at its three backward
// neighbours, which belong to P of the same iteration.  A block owns a 32 x 8
// (x, y) tile and walks a z-chunk; per slice its 33 x 9 threads compute P on
// the tile plus the row and column in front of it (the halo, 16 % extra P),
// keep the y and x components in shared memory for the backward differences,
// carry the z component of the previous slice in a register, then run U on
// the tile.  P of the halo reads the flow field and tmp of neighbouring tiles,
// which other blocks overwrite in the same launch, so hp and tmp are
// ping-pong buffers (read *_in, write *_out); p_t and u are only touched at
// their own voxel and stay in place.  Per voxel and iteration this moves
// tmp 4 + hp 12 + quaternion 16 + alpha 4 + cs 4 + ct 4 + pt 4 + u 4 read and
// hp 12 + pt 4 + u 4 + tmp 4 written = 76 B, against 88 B for the two
// separate sweeps (the hp field is read once instead of twice).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"
#include "sweeps.cuh"

namespace m16 {

constexpr int kFX = 33, kFY = 9;   // block: the 32 x 8 tile plus one halo column and row

struct FusedView {
    int d0, d1, d2;
    float ss0, ss1, ss2, rcc, rs0, rs1, rs2;
    float sq0, sq1, sq2, isq0, isq1, isq2;
    float alpha_scalar;
    const float *alpha, *grad2;
    float w, neg_inv_decay2;
    int exp_alpha;   // kAlphaSource: 1 when alpha holds |grad I|^2
    const float *sqeigs;
    const float4 *q4;
    const float *tmp_in, *hp0_in, *hp1_in, *hp2_in;
    float *tmp_out, *hp0_out, *hp1_out, *hp2_out;
    const float *cs, *ct;
    const uint8_t *labels;
    float *pt, *u;
};

// Everything one thread reads for one slice: the flow sweep's inputs (all
// in-volume threads) and the label sweep's (tile threads).
struct SliceIn {
    float tc, tz, ty, tx, al, h0, h1, h2;
    float4 q;
    float se0, se1, se2;
    float uo, ptv, csv, ctv;
    uint8_t lab;
};

template <bool POINTWISE, int ALPHA, bool SUPERVISED>
__device__ __forceinline__ void fused_load(const FusedView &a, int z, int y, int x, int64_t i, bool valid,
                                           bool inner, SliceIn &s)
{
    if (!valid) return;
    const int64_t s0 = (int64_t)a.d1 * a.d2;
    s.tc = __ldg(a.tmp_in + i);
    s.tz = z < a.d0 - 1 ? __ldg(a.tmp_in + i + s0) : 0.f;
    s.ty = y < a.d1 - 1 ? __ldg(a.tmp_in + i + a.d2) : 0.f;
    s.tx = x < a.d2 - 1 ? __ldg(a.tmp_in + i + 1) : 0.f;
    s.q = __ldg(a.q4 + i);
    if (ALPHA == kAlphaArray || ALPHA == kAlphaSource) s.al = __ldg(a.alpha + i);
    else if (ALPHA == kAlphaFromGrad2) s.al = __ldg(a.grad2 + i);
    else s.al = a.alpha_scalar;
    s.h0 = __ldg(a.hp0_in + i);
    s.h1 = __ldg(a.hp1_in + i);
    s.h2 = __ldg(a.hp2_in + i);
    if (POINTWISE) {
        s.se0 = __ldg(a.sqeigs + 3 * i);
        s.se1 = __ldg(a.sqeigs + 3 * i + 1);
        s.se2 = __ldg(a.sqeigs + 3 * i + 2);
    }
    if (inner) {
        s.uo = a.u[i];
        s.ptv = a.pt[i];
        s.csv = __ldg(a.cs + i);
        s.ctv = __ldg(a.ct + i);
        if (SUPERVISED) s.lab = __ldg(a.labels + i);
    }
}

// P at one voxel (update_qp.cl:150-232) from its loaded inputs
template <bool POINTWISE, int ALPHA>
__device__ __forceinline__ float3 fused_flow(const FusedView &a, int z, int y, int x, const SliceIn &s)
{
    const bool zin = z < a.d0 - 1, yin = y < a.d1 - 1, xin = x < a.d2 - 1;
    float s0v = a.sq0, s1v = a.sq1, s2v = a.sq2, i0v = a.isq0, i1v = a.isq1, i2v = a.isq2;
    if (POINTWISE) {
        s0v = s.se0; s1v = s.se1; s2v = s.se2;
        i0v = 1.f / s0v; i1v = 1.f / s1v; i2v = 1.f / s2v;
    }
    const float3 g = make_float3(zin ? (s.tz - s.tc) * a.ss0 : 0.f, yin ? (s.ty - s.tc) * a.ss1 : 0.f,
                                 xin ? (s.tx - s.tc) * a.ss2 : 0.f);
    const Rot R = quat2rot(s.q);
    float rad = s.al;
    if (ALPHA == kAlphaFromGrad2 || (ALPHA == kAlphaSource && a.exp_alpha)) rad = a.w * expf(a.neg_inv_decay2 * s.al);
    const float3 rg = rot_t(R, g);
    const float3 rh = rot_t(R, make_float3(s.h0, s.h1, s.h2));
    float3 p = make_float3(rh.x * i0v + rg.x * s0v, rh.y * i1v + rg.y * s1v, rh.z * i2v + rg.z * s2v);
    const float nrm = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
    const float sc = nrm > rad ? rad / nrm : 1.f;
    p = make_float3(p.x * sc * s0v, p.y * sc * s1v, p.z * sc * s2v);
    return rot(R, p);
}

// One block, one tile (bx, by), slices z0..z1.  blockDim = (kFX, kFY); the
// thread at (rx, ry) handles x = 32 bx - 1 + rx, y = 8 by - 1 + ry; rx = 0 and
// ry = 0 are the halo.  The inputs of slice z + 1 are loaded before slice z is
// computed, so every thread keeps one slice of loads in flight across the
// barrier.  Returns this thread's sum of |err| (0 for halo threads).
// sm: 2 buffers x 2 components x kFY x kFX floats of shared memory.
template <bool POINTWISE, int ALPHA, bool SUPERVISED>
__device__ __forceinline__ float fused_tile(const FusedView &a, int bx, int by, int z0, int z1,
                                            float (*sm)[2][kFY][kFX])
{
    const int rx = threadIdx.x, ry = threadIdx.y;
    const int x = bx * 32 - 1 + rx, y = by * 8 - 1 + ry;
    const bool valid = x >= 0 && y >= 0 && x < a.d2 && y < a.d1;
    const bool inner = valid && rx > 0 && ry > 0;
    const int64_t s0 = (int64_t)a.d1 * a.d2;
    const int64_t col = valid ? (int64_t)y * a.d2 + x : 0;
    float acc = 0.f;
    // z component of the new flow one slice back (for the backward z difference)
    float h0prev = 0.f;
    SliceIn cur, nxt;
    if (inner && z0 > 0) {
        fused_load<POINTWISE, ALPHA, false>(a, z0 - 1, y, x, col + (z0 - 1) * s0, true, false, cur);
        h0prev = fused_flow<POINTWISE, ALPHA>(a, z0 - 1, y, x, cur).x;
    }
    if (z0 < z1) fused_load<POINTWISE, ALPHA, SUPERVISED>(a, z0, y, x, col + z0 * s0, valid, inner, cur);
    for (int z = z0; z < z1; ++z) {
        const int buf = z & 1;
        const int64_t i = col + z * s0;
        if (z + 1 < z1) fused_load<POINTWISE, ALPHA, SUPERVISED>(a, z + 1, y, x, i + s0, valid, inner, nxt);
        float3 h = make_float3(0.f, 0.f, 0.f);
        if (valid) h = fused_flow<POINTWISE, ALPHA>(a, z, y, x, cur);
        sm[buf][0][ry][rx] = h.y;
        sm[buf][1][ry][rx] = h.z;
        if (inner) {
            a.hp0_out[i] = h.x;
            a.hp1_out[i] = h.y;
            a.hp2_out[i] = h.z;
        }
        __syncthreads();
        if (inner) {
            // U (update_qp.cl:241-300) with update_tmp (:311-316) fused
            const float a0 = (z < a.d0 - 1 ? h.x : 0.f) - (z > 0 ? h0prev : 0.f);
            const float a1 = (y < a.d1 - 1 ? h.y : 0.f) - (y > 0 ? sm[buf][0][ry - 1][rx] : 0.f);
            const float a2 = (x < a.d2 - 1 ? h.z : 0.f) - (x > 0 ? sm[buf][1][ry][rx - 1] : 0.f);
            const float div = a0 * a.rs0 + a1 * a.rs1 + a2 * a.rs2;
            float s_off = 1.f, t_off = 0.f;
            if (SUPERVISED) {
                s_off = (float)(!(cur.lab & 2));
                t_off = (float)(cur.lab & 1);
            }
            const float psx = div + cur.ptv - a.rcc * (cur.uo - s_off);
            const float ps = cur.csv < psx ? cur.csv : psx;
            const float ptx = -div + ps + a.rcc * (cur.uo - t_off);
            const float ptn = cur.ctv < ptx ? cur.ctv : ptx;
            const float err = div - ps + ptn;
            const float un = cur.uo - err / a.rcc;
            a.pt[i] = ptn;
            a.u[i] = un;
            a.tmp_out[i] = err - un * a.rcc;
            acc += fabsf(err);
        }
        h0prev = h.x;
        cur = nxt;
    }
    return acc;
}

// Block-wide sum for the (kFX, kFY) block (its last warp is partial, so the
// values go through shared memory); valid in thread (0, 0).  vals holds
// kFX * kFY floats.  Fixed summation order.
__device__ __forceinline__ float fused_block_sum(float v, float *vals)
{
    const int tid = threadIdx.x + kFX * threadIdx.y;
    constexpr int nthreads = kFX * kFY;
    vals[tid] = v;
    __syncthreads();
    float r = 0.f;
    if (tid < 32) {
        for (int k = tid; k < nthreads; k += 32) r += vals[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;
}

}  // namespace m16
