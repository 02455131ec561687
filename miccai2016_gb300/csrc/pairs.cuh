// pairs.cuh -- two iterations of the ATV max-flow in one launch (temporal
// blocking of the flow and label sweeps; the per-voxel arithmetic is
// flow_point / label_point of sweeps.cuh, the reference's update_p / update_u
// / update_tmp, src/clcode-anisotropic/update_qp.cl:150-316).
//
// Why: one iteration moves 84 B per voxel through HBM in the two sweeps (the
// flow state, tmp, the quaternion, alpha and the capacities), and both sweeps
// already run near the copy rate.  Two iterations in one pass read the state
// and the inputs once and write the state once: 52 B read (tmp 4, q4 16,
// alpha 4, hp 12, cs 4, ct 4, pt 4, u 4) and 24 B written per voxel for two
// iterations, 38 B per voxel-iteration plus the halo's share.
//
// Tiling.  A block owns 32 x 16 (x, y) positions, one warp per row, and
// marches along z.  The dependence cone of one iteration reaches one voxel
// forward (the flow sweep's gradient) and one backward (the label sweep's
// divergence) in each axis, so two iterations need two halo voxels on each
// side: the block's outputs are its inner 28 x 12 positions.  Along z the
// block computes the first iteration at plane v and the second at plane
// v - 1 in the same step, and starts two planes before its z-chunk so the
// second iteration's z-neighbours exist at the chunk's first plane.
//
// Staging.  The inputs of plane v + 2 are copied into shared memory with
// cp.async while planes v and v + 1 are computed on (three stages of 29 KB);
// the first iteration's flow and label results of a plane live in shared
// memory for the x/y neighbours, the z-neighbours are carried in registers.
//
// The state is double-buffered between launches: a launch reads one set
// (hp, pt, u, tmp) and writes the other, because neighbouring blocks read
// the halo of the set being replaced.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sweeps.cuh"

namespace m16 {

constexpr int kPX = 32, kPY = 16;                // positions of a block (one warp per row)
constexpr int kPH = 2;                           // halo width on each side in x and y
constexpr int kPIX = kPX - 2 * kPH;              // 28 output columns
constexpr int kPIY = kPY - 2 * kPH;              // 12 output rows
constexpr int kPN = kPX * kPY;                   // 512 threads
constexpr int kPPad = 32;                        // padding around the arrays read at neighbours
constexpr int kPA = kPN + 2 * kPPad;             // length of a padded plane array

// One staged plane of the inputs.
struct PairStage {
    float4 q[kPN];             // expanded quaternion
    float tmp[kPA];            // read at x+1 and y+1: padded
    float al[kPN];
    float h0[kPN], h1[kPN], h2[kPN];
    float cs[kPN], ct[kPN], pt[kPN], u[kPN];
};

constexpr int kPStages = 3;
// dynamic shared memory of the pair kernel: the stages, then the first
// iteration's flow plane (3 arrays), its tmp planes (2, alternating by plane
// parity) and the second iteration's flow plane (3)
constexpr size_t kPairSmem = kPStages * sizeof(PairStage) + 8 * kPA * sizeof(float);

// Everything the pair kernel reads and writes: the state is read from the
// *_in set and written to the *_out set.
struct PairView {
    int d0, d1, d2, zc;
    float rcc, rs0, rs1, rs2, ss0, ss1, ss2;
    float sq0, sq1, sq2, isq0, isq1, isq2;
    float alpha_scalar;
    const float4 *q4;
    const float *alpha, *cs, *ct;
    const uint8_t *labels;
    const float *hp0_in, *hp1_in, *hp2_in, *pt_in, *u_in, *tmp_in;
    float *hp0_out, *hp1_out, *hp2_out, *pt_out, *u_out, *tmp_out;
};

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// 4- and 16-byte asynchronous global -> shared copies; src_bytes 0 fills zeros
// and reads nothing (the address is still a valid one)
__device__ __forceinline__ void cp_async4(void *dst, const void *src, int src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(smem_addr(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src, int src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Two iterations over the block's tile; returns the block's share of
// sum |err| of the second iteration (its output voxels) when CHECK.
template <bool ALPHA_ARR, bool SUPERVISED, bool CHECK>
__device__ __forceinline__ float pair_tile(const PairView &a, unsigned char *smem)
{
    PairStage *stage = reinterpret_cast<PairStage *>(smem);
    float *s_hp1 = reinterpret_cast<float *>(stage + kPStages);   // 3 arrays of kPA
    float *s_tmp1 = s_hp1 + 3 * kPA;                                // 2 arrays (plane parity)
    float *s_hp2 = s_tmp1 + 2 * kPA;                                // 3 arrays

    const int lx = threadIdx.x, ly = threadIdx.y, pos = ly * kPX + lx;
    const int x = (int)blockIdx.x * kPIX - kPH + lx;
    const int y = (int)blockIdx.y * kPIY - kPH + ly;
    const bool inside = x >= 0 && x < a.d2 && y >= 0 && y < a.d1;
    const bool output = inside && lx >= kPH && lx < kPX - kPH && ly >= kPH && ly < kPY - kPH;
    const bool xin = x < a.d2 - 1, yin = y < a.d1 - 1;   // forward neighbours (flow); also the label's own terms
    const bool xlo = x > 0, ylo = y > 0;                 // backward neighbours (label)
    const int za = (int)blockIdx.z * a.zc, zb = min(za + a.zc, a.d0);
    const int v0 = max(za - 2, 0);          // first plane of the first iteration
    const int vlast = min(zb, a.d0 - 1);    // last plane of the first iteration
    const int64_t s0 = (int64_t)a.d1 * a.d2;
    const int64_t col = inside ? (int64_t)y * a.d2 + x : 0;
    const int cb = inside ? 4 : 0;

    auto issue = [&](int v) {
        if (v == vlast + 1 && v < a.d0) {
            // the first iteration's flow at plane vlast reads tmp one plane further
            cp_async4(&stage[v % kPStages].tmp[kPPad + pos], a.tmp_in + (int64_t)v * s0 + col, cb);
        } else if (v <= vlast) {
            PairStage &S = stage[v % kPStages];
            const int64_t i = (int64_t)v * s0 + col;   // in bounds also outside the volume (col 0)
            cp_async4(&S.tmp[kPPad + pos], a.tmp_in + i, cb);
            cp_async16(&S.q[pos], a.q4 + i, inside ? 16 : 0);
            if (ALPHA_ARR) cp_async4(&S.al[pos], a.alpha + i, cb);
            cp_async4(&S.h0[pos], a.hp0_in + i, cb);
            cp_async4(&S.h1[pos], a.hp1_in + i, cb);
            cp_async4(&S.h2[pos], a.hp2_in + i, cb);
            cp_async4(&S.cs[pos], a.cs + i, cb);
            cp_async4(&S.ct[pos], a.ct + i, cb);
            cp_async4(&S.pt[pos], a.pt_in + i, cb);
            cp_async4(&S.u[pos], a.u_in + i, cb);
        }
        cp_async_commit();
    };

    issue(v0);
    issue(v0 + 1);

    // carried between steps: the first iteration's results at plane v - 1
    // (inputs of the second iteration there) and the z-neighbours of the divergences
    float4 q_p = make_float4(0.f, 0.f, 0.f, 1.f);
    float al_p = a.alpha_scalar, cs_p = 0.f, ct_p = 0.f;
    float g0_p = 0.f, g1_p = 0.f, g2_p = 0.f;   // first-iteration hp at v - 1
    float pt_p = 0.f, u_p = 0.f;                // first-iteration pt, u at v - 1
    uint8_t lab_p = 0;
    float c2 = 0.f;                             // second-iteration hp0 at w - 1
    float acc = 0.f;

    // v runs to zb: the second iteration's last plane is zb - 1 (at zb <= d0 - 1
    // the first iteration still computes plane zb, its z-neighbour)
    for (int v = v0; v <= zb; ++v) {
        const bool first = v <= vlast;   // the first iteration has a plane v
        const bool second = v > v0;      // the second iteration runs at plane w = v - 1
        cp_async_wait_all();
        __syncthreads();                 // plane v and v + 1 staged; last step's readers done
        issue(v + 2);
        const PairStage &S = stage[v % kPStages];
        const PairStage &Sn = stage[(v + 1) % kPStages];

        // first iteration, flow at plane v
        float4 q = q_p;
        float al = al_p, g0 = 0.f, g1 = 0.f, g2 = 0.f;
        if (first) {
            q = S.q[pos];
            al = ALPHA_ARR ? S.al[pos] : a.alpha_scalar;
            const bool zin = v < a.d0 - 1;
            const float tc = S.tmp[kPPad + pos];
            const float tz = zin ? Sn.tmp[kPPad + pos] : 0.f;
            const float ty = yin ? S.tmp[kPPad + pos + kPX] : 0.f;
            const float tx = xin ? S.tmp[kPPad + pos + 1] : 0.f;
            const float3 h = flow_point(a.ss0, a.ss1, a.ss2, tc, tz, ty, tx, zin, yin, xin, q, al, S.h0[pos],
                                        S.h1[pos], S.h2[pos], a.sq0, a.sq1, a.sq2, a.isq0, a.isq1, a.isq2);
            g0 = h.x; g1 = h.y; g2 = h.z;
            s_hp1[kPPad + pos] = g0;
            s_hp1[kPA + kPPad + pos] = g1;
            s_hp1[2 * kPA + kPPad + pos] = g2;
        }
        __syncthreads();

        // first iteration, labels at plane v
        float pt1 = 0.f, u1 = 0.f, tmp1 = 0.f;
        uint8_t lab = 0;
        if (first) {
            if (SUPERVISED && inside) lab = __ldg(a.labels + (int64_t)v * s0 + col);
            const float h1m = ylo ? s_hp1[kPA + kPPad + pos - kPX] : 0.f;
            const float h2m = xlo ? s_hp1[2 * kPA + kPPad + pos - 1] : 0.f;
            label_point<SUPERVISED>(a.rcc, a.rs0, a.rs1, a.rs2, g0, g1, g2, g0_p, h1m, h2m, v > 0, v < a.d0 - 1, yin,
                                    xin, S.u[pos], S.pt[pos], S.cs[pos], S.ct[pos], lab, pt1, u1, tmp1);
            s_tmp1[(v & 1) * kPA + kPPad + pos] = tmp1;
        }

        // second iteration, flow at plane w = v - 1: tmp of the first
        // iteration at w (x/y neighbours from the previous step) and at v
        float3 f = make_float3(0.f, 0.f, 0.f);
        const int w = v - 1;
        if (second) {
            const float *tw = s_tmp1 + (w & 1) * kPA + kPPad;
            const bool zin = w < a.d0 - 1;
            const float tc = tw[pos];
            const float tz = zin ? tmp1 : 0.f;
            const float ty = yin ? tw[pos + kPX] : 0.f;
            const float tx = xin ? tw[pos + 1] : 0.f;
            f = flow_point(a.ss0, a.ss1, a.ss2, tc, tz, ty, tx, zin, yin, xin, q_p, al_p, g0_p, g1_p, g2_p, a.sq0,
                           a.sq1, a.sq2, a.isq0, a.isq1, a.isq2);
            s_hp2[kPPad + pos] = f.x;
            s_hp2[kPA + kPPad + pos] = f.y;
            s_hp2[2 * kPA + kPPad + pos] = f.z;
        }
        __syncthreads();

        // second iteration, labels at plane w; the chunk's planes are written
        if (second) {
            const float h1m = ylo ? s_hp2[kPA + kPPad + pos - kPX] : 0.f;
            const float h2m = xlo ? s_hp2[2 * kPA + kPPad + pos - 1] : 0.f;
            float pt2, u2, tmp2;
            const float err = label_point<SUPERVISED>(a.rcc, a.rs0, a.rs1, a.rs2, f.x, f.y, f.z, c2, h1m, h2m, w > 0,
                                                      w < a.d0 - 1, yin, xin, u_p, pt_p, cs_p, ct_p, lab_p, pt2, u2,
                                                      tmp2);
            c2 = f.x;
            if (output && w >= za) {   // w <= zb - 1 by the loop bound
                const int64_t i = (int64_t)w * s0 + col;
                a.hp0_out[i] = f.x;
                a.hp1_out[i] = f.y;
                a.hp2_out[i] = f.z;
                a.pt_out[i] = pt2;
                a.u_out[i] = u2;
                a.tmp_out[i] = tmp2;
                if (CHECK) acc += fabsf(err);
            }
        }

        // the first iteration's plane v becomes the second iteration's input
        if (first) {
            q_p = q;
            al_p = al;
            cs_p = S.cs[pos];
            ct_p = S.ct[pos];
            g0_p = g0; g1_p = g1; g2_p = g2;
            pt_p = pt1;
            u_p = u1;
            lab_p = lab;
        }
    }
    cp_async_wait_all();
    return acc;
}

}  // namespace m16
