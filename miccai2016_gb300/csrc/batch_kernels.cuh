// batch_kernels.cuh -- device side of the batched ATV max-flow: descriptors,
// set-up kernels, the flow / label sweeps over a work list of (group, tile)
// items, the per-instance residual check and the scatter of u.  Included by
// batched.cu (m16_batch_solve: a fixed batch run to completion) and serve.cu
// (m16_server_*: requests admitted and retired while others iterate).
//
// The reference runs its (weighting, decay) grid search as one
// CmfCutQAnisotropicGpu.execute() per grid point and cut type
// (src/phantom_experiment.py:350-368), each with three launches per iteration
// and a blocking residual read every `update` iterations.  Here a batch of
// instances -- any mix of volumes, weightings, decays and eigenvalue sets --
// advances together: every flow (P) and label (U) launch covers all active
// instances, the residual check of every instance is one block of one launch,
// and an instance stops on its own at its threshold.
//
// Layout.  Instances of one volume with the same eigenvalues (and the same
// kind of alpha) form groups of kLanes = 4; a group's state is interleaved,
// one float4 per voxel and field (lane = instance), so one 16-byte load or
// store serves four solves and a warp moves 512 contiguous bytes per field.
// The volume's quaternions, |grad I|^2 and capacities are read once per voxel
// for the whole group and the rotation is built once.  The projection radius
// of a lane is its alpha field (gathered into an interleaved field at set-up)
// or w * exp(-|grad I|^2 / decay^2) (phantom_experiment.py:359) computed in
// the flow sweep, so per voxel and instance only the state streams from HBM:
// flow reads tmp 4 + hp 12 and writes hp 12, labels read hp 12 + p_t 4 + u 4
// and write p_t 4 + u 4 + tmp 4 -- 60 B per voxel-iteration.
//
// Instances whose volume is shared by fewer than three others of the same
// kind (ragged batches, served requests) form one-lane groups instead: plain
// float fields and the single solve's z-batched sweep bodies (sweeps.cuh),
// so no padding lanes stream.
//
// Stopping.  The check kernel sets a lane's bit in its group's stop mask; the
// label sweep then keeps that lane's u (the solve's result) unchanged, blocks
// of a group whose lanes have all stopped return at once, and the work list
// drops finished groups.  At the end u is scattered out of the interleaved
// field into each instance's output array.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <float.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "sweeps.cuh"

namespace m16 {
namespace {

constexpr int kBX = 32, kBY = 8, kTile = kBX * kBY;
constexpr int kLanes = 4;     // instances per group: one float4 per voxel and field
constexpr int kFields = 6;    // hp0 hp1 hp2 pt tmp u (+ alpha for groups with alpha fields)
constexpr unsigned kAllLanes = (1u << kLanes) - 1u;

struct InstCtrl {
    int stopped;
    int iterations;
    int n_checks;
    int pad;
    double resid;   // last checked residual
};

struct VolDev {
    int d0, d1, d2, zc, tx, ty, tz, pad;
    float rcc, rs0, rs1, rs2, ss0, ss1, ss2, denom;
    const float4 *q4;
    const float *grad2, *cs, *ct;
    int64_t n;
};

struct GroupDev {
    int64_t part_off;        // float4 index of the group's first partial sum
    int vol, nparts, has_alpha;
    int lanes, pad0, pad1, pad2;   // 4: interleaved float4 fields; 1: plain float fields
    float4 w, nid2;          // per lane: alpha = w * exp(nid2 * |grad I|^2), nid2 = -1 / decay^2
    float sq0, sq1, sq2, isq0, isq1, isq2;
    void *state;             // kFields (+1 for 4-lane alpha groups) slabs of `slab` elements
    int64_t slab;            // elements (float4 or float) per slab
    const float *alpha1;     // one-lane groups: the instance's own alpha field, or NULL
};

struct InstDev {
    int group, lane;
    float *u_out;
    const float *alpha;
};

// z-slices per block: enough blocks for `blocks_per_sm` (by default
// M16_BATCH_BLOCKS_PER_SM) per SM over the volume's groups (many short blocks
// keep the last wave short), at most 32
#ifndef M16_BATCH_BLOCKS_PER_SM
#define M16_BATCH_BLOCKS_PER_SM 16
#endif
// resident blocks per SM of the four-lane sweeps: 4 caps them at 64
// registers (a few bytes spill to L1); measured on GB300 (424 instances at
// 128^3) one iteration takes 8.64 ms against 9.09 ms at 3 and 10.21 ms at 2
#ifndef M16_BATCH_MINB
#define M16_BATCH_MINB 4
#endif
inline int batch_zc(int d0, int d1, int d2, int ngroups_of_volume, int blocks_per_sm = M16_BATCH_BLOCKS_PER_SM)
{
    const int64_t cols = div_up(d2, kBX) * div_up(d1, kBY);
    int64_t zc = (int64_t)d0 * cols * std::max(ngroups_of_volume, 1) / ((int64_t)blocks_per_sm * kSMs);
    zc = std::max<int64_t>(1, std::min<int64_t>(32, zc));
    return (int)zc;
}

// One z-chunk for every volume of a launch: the launch covers the tiles of
// all its groups, so the target number of blocks applies to their sum
// (total_column_slices = sum over groups of d0 x the volume's 32 x 8 columns).
#ifndef M16_BATCH_ZC_ROUND
#define M16_BATCH_ZC_ROUND 4
#endif
inline int batch_zc_total(int64_t total_column_slices, int blocks_per_sm = M16_BATCH_BLOCKS_PER_SM)
{
    int64_t zc = total_column_slices / ((int64_t)blocks_per_sm * kSMs);
    zc = std::max<int64_t>(1, std::min<int64_t>(32, zc));
    if (zc >= M16_BATCH_ZC_ROUND) zc = zc / M16_BATCH_ZC_ROUND * M16_BATCH_ZC_ROUND;
    return (int)zc;
}

inline int64_t column_slices(int d0, int d1, int d2) { return (int64_t)d0 * div_up(d2, kBX) * div_up(d1, kBY); }

__device__ __forceinline__ float lane_of(const float4 &v, int l)
{
    return l == 0 ? v.x : (l == 1 ? v.y : (l == 2 ? v.z : v.w));
}

// ---- initialisation ---------------------------------------------------------

__global__ void bt_max_kernel(const float *__restrict__ img, int64_t n, float *__restrict__ part)
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

__global__ void bt_denom_kernel(const float *__restrict__ part, int nparts, VolDev *vol)
{
    if (threadIdx.x != 0) return;
    float m = -INFINITY;
    bool nan = false;
    for (int k = 0; k < nparts; ++k) {
        const float v = part[k];
        if (v != v) nan = true; else m = fmaxf(m, v);
    }
    vol->denom = (nan ? NAN : m) + FLT_MIN;   // np.max(img) + np.finfo(float32).tiny
}

__global__ void bt_expand_kernel(const float *__restrict__ quat3, float4 *__restrict__ q4, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        q4[i] = qexpand(quat3[3 * i], quat3[3 * i + 1], quat3[3 * i + 2]);
}

// every lane of a group: hp = 0, p_t = fmin(cs, ct), u = img / denom,
// tmp = -u * rcc (continuous_cut_anisotropic_gpu.py:276-289)
__global__ void bt_init_group_kernel(const float *__restrict__ img, const VolDev *vols, const GroupDev *groups, int g)
{
    const GroupDev &G = groups[g];
    const VolDev &V = vols[G.vol];
    const float denom = V.denom;
    const int64_t S = G.slab;
    if (G.lanes == 1) {
        float *st1 = (float *)G.state;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < V.n;
             i += (int64_t)gridDim.x * blockDim.x) {
            const float ui = img[i] / denom;
            st1[i] = 0.f;
            st1[S + i] = 0.f;
            st1[2 * S + i] = 0.f;
            st1[3 * S + i] = fminf(V.cs[i], V.ct[i]);
            st1[4 * S + i] = -(ui * V.rcc);
            st1[5 * S + i] = ui;
        }
        return;
    }
    float4 *st = (float4 *)G.state;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < V.n; i += (int64_t)gridDim.x * blockDim.x) {
        const float ptv = fminf(V.cs[i], V.ct[i]);
        const float ui = img[i] / denom;
        const float ti = -(ui * V.rcc);
        st[i] = zero;
        st[S + i] = zero;
        st[2 * S + i] = zero;
        st[3 * S + i] = make_float4(ptv, ptv, ptv, ptv);
        st[4 * S + i] = make_float4(ti, ti, ti, ti);
        st[5 * S + i] = make_float4(ui, ui, ui, ui);
    }
}

// interleave the lanes' alpha fields (absent lanes: 0)
__global__ void bt_gather_alpha_kernel(const GroupDev *groups, int g, const float *a0, const float *a1,
                                       const float *a2, const float *a3, int64_t n)
{
    const GroupDev &G = groups[g];
    float4 *al = (float4 *)G.state + kFields * G.slab;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        al[i] = make_float4(a0 ? a0[i] : 0.f, a1 ? a1[i] : 0.f, a2 ? a2[i] : 0.f, a3 ? a3[i] : 0.f);
}

// u of one instance out of its group's interleaved field
__global__ void bt_scatter_u_kernel(const GroupDev *groups, const InstDev *insts, int inst, int64_t n)
{
    const InstDev &I = insts[inst];
    const GroupDev &G = groups[I.group];
    const int L = G.lanes;
    const float *u = (const float *)G.state + 5 * G.slab * L;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        I.u_out[i] = u[L * i + I.lane];
}

// ---- the sweeps ---------------------------------------------------------------
// A work item is (group, tile); a block of 32 x 8 threads walks the tile's
// z-chunk, one (y, x) column per thread, all four lanes of the group per voxel.

__device__ __forceinline__ void decode_tile(const VolDev &V, int tile, int &bx, int &by, int &bz)
{
    bx = tile % V.tx;
    by = (tile / V.tx) % V.ty;
    bz = tile / (V.tx * V.ty);
}

// P (update_qp.cl:150-232) for the four lanes of a group
template <bool ALPHA_ARR>
__global__ void __launch_bounds__(kTile, M16_BATCH_MINB) bt_flow_kernel(const int2 *__restrict__ work,
                                                                       const VolDev *vols, const GroupDev *groups,
                                                                       const unsigned *__restrict__ gmask)
{
    pdl_wait();
    pdl_launch_next();
    const int2 wk = work[blockIdx.x];
    if (__ldcg(gmask + wk.x) == kAllLanes) return;
    const GroupDev &G = groups[wk.x];
    const VolDev &V = vols[G.vol];
    int bx, by, bz;
    decode_tile(V, wk.y, bx, by, bz);
    const int d0 = V.d0, d1 = V.d1, d2 = V.d2;
    const int x = bx * kBX + threadIdx.x, y = by * kBY + threadIdx.y;
    const int z0 = bz * V.zc, z1 = min(z0 + V.zc, d0);
    if (x >= d2 || y >= d1) return;
    const int s0 = d1 * d2;
    const bool yin = y < d1 - 1, xin = x < d2 - 1;
    const float ss0 = V.ss0, ss1 = V.ss1, ss2 = V.ss2;
    const float sq[3] = {G.sq0, G.sq1, G.sq2};
    const float isq[3] = {G.isq0, G.isq1, G.isq2};
    const float4 w4 = G.w, n4 = G.nid2;
    const int64_t S = G.slab;
    float4 *__restrict__ hp0 = (float4 *)G.state;
    float4 *__restrict__ hp1 = hp0 + S;
    float4 *__restrict__ hp2 = hp1 + S;
    const float4 *__restrict__ tmp = hp0 + 4 * S;
    const float4 *__restrict__ al4 = hp0 + kFields * S;
    const float4 *__restrict__ q4 = V.q4;
    const float *__restrict__ grad2 = V.grad2;
    for (int z = z0; z < z1; ++z) {
        const int i = (z * d1 + y) * d2 + x;
        const bool zin = z < d0 - 1;
        const float4 q = __ldg(q4 + i);
        float4 a4;
        float g2 = 0.f;
        if (ALPHA_ARR) a4 = __ldg(al4 + i);
        else g2 = __ldg(grad2 + i);
        const float4 tc = __ldg(tmp + i);
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 tz = zin ? __ldg(tmp + i + s0) : zero;
        const float4 ty = yin ? __ldg(tmp + i + d2) : zero;
        const float4 tx = xin ? __ldg(tmp + i + 1) : zero;
        const float4 h0 = hp0[i], h1 = hp1[i], h2 = hp2[i];
        const Rot R = quat2rot(q);
        float o0[kLanes], o1[kLanes], o2[kLanes];
#pragma unroll
        for (int l = 0; l < kLanes; ++l) {
            const float c = lane_of(tc, l);
            const float3 gr = make_float3(zin ? (lane_of(tz, l) - c) * ss0 : 0.f,
                                          yin ? (lane_of(ty, l) - c) * ss1 : 0.f,
                                          xin ? (lane_of(tx, l) - c) * ss2 : 0.f);
            const float rad = ALPHA_ARR ? lane_of(a4, l) : lane_of(w4, l) * expf(lane_of(n4, l) * g2);
            const float3 rg = rot_t(R, gr);
            const float3 rh = rot_t(R, make_float3(lane_of(h0, l), lane_of(h1, l), lane_of(h2, l)));
            float3 p = make_float3(rh.x * isq[0] + rg.x * sq[0], rh.y * isq[1] + rg.y * sq[1],
                                   rh.z * isq[2] + rg.z * sq[2]);
            const float nrm = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
            const float sc = nrm > rad ? rad / nrm : 1.f;
            p = make_float3(p.x * sc * sq[0], p.y * sc * sq[1], p.z * sc * sq[2]);
            const float3 h = rot(R, p);
            o0[l] = h.x;
            o1[l] = h.y;
            o2[l] = h.z;
        }
        hp0[i] = make_float4(o0[0], o0[1], o0[2], o0[3]);
        hp1[i] = make_float4(o1[0], o1[1], o1[2], o1[3]);
        hp2[i] = make_float4(o2[0], o2[1], o2[2], o2[3]);
    }
}

// U with update_tmp fused (update_qp.cl:241-300, :311-316) for the four lanes
// of a group; a stopped lane keeps its u.  On check iterations the block's
// per-lane sum of |err| goes to partials[part_off + tile] (fixed order).
template <bool CHECK>
__global__ void __launch_bounds__(kTile, M16_BATCH_MINB) bt_label_kernel(const int2 *__restrict__ work,
                                                                        const VolDev *vols, const GroupDev *groups,
                                                                        const unsigned *__restrict__ gmask,
                                                                        float4 *__restrict__ partials)
{
    pdl_wait();
    pdl_launch_next();
    __shared__ float4 red[kTile / 32];
    const int2 wk = work[blockIdx.x];
    const unsigned stopped = __ldcg(gmask + wk.x);
    if (stopped == kAllLanes) return;   // uniform over the block
    const GroupDev &G = groups[wk.x];
    const VolDev &V = vols[G.vol];
    int bx, by, bz;
    decode_tile(V, wk.y, bx, by, bz);
    const int d0 = V.d0, d1 = V.d1, d2 = V.d2;
    const int x = bx * kBX + threadIdx.x, y = by * kBY + threadIdx.y;
    const int z0 = bz * V.zc, z1 = min(z0 + V.zc, d0);
    float acc[kLanes] = {0.f, 0.f, 0.f, 0.f};
    if (x < d2 && y < d1) {
        const int s0 = d1 * d2;
        const bool ylo = y > 0, xlo = x > 0, yhi = y < d1 - 1, xhi = x < d2 - 1;
        const float rcc = V.rcc, rs0 = V.rs0, rs1 = V.rs1, rs2 = V.rs2;
        const int64_t S = G.slab;
        float4 *const st = (float4 *)G.state;
        const float4 *__restrict__ hp0 = st;
        const float4 *__restrict__ hp1 = hp0 + S;
        const float4 *__restrict__ hp2 = hp1 + S;
        float4 *__restrict__ ptp = st + 3 * S;
        float4 *__restrict__ tmp = st + 4 * S;
        float4 *__restrict__ up = st + 5 * S;
        const float *__restrict__ csp = V.cs;
        const float *__restrict__ ctp = V.ct;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int z = z0; z < z1; ++z) {
            const int i = (z * d1 + y) * d2 + x;
            const float4 h0 = __ldg(hp0 + i), h1 = __ldg(hp1 + i), h2 = __ldg(hp2 + i);
            const float4 h0m = z > 0 ? __ldg(hp0 + i - s0) : zero;
            const float4 h1m = ylo ? __ldg(hp1 + i - d2) : zero;
            const float4 h2m = xlo ? __ldg(hp2 + i - 1) : zero;
            const float4 uo = up[i], pto = ptp[i];
            const float csv = __ldg(csp + i), ctv = __ldg(ctp + i);
            const bool zhi = z < d0 - 1;
            float on[kLanes], op[kLanes], ot[kLanes];
#pragma unroll
            for (int l = 0; l < kLanes; ++l) {
                const float div = ((zhi ? lane_of(h0, l) : 0.f) - lane_of(h0m, l)) * rs0 +
                                  ((yhi ? lane_of(h1, l) : 0.f) - lane_of(h1m, l)) * rs1 +
                                  ((xhi ? lane_of(h2, l) : 0.f) - lane_of(h2m, l)) * rs2;
                const float u0 = lane_of(uo, l);
                const float psx = div + lane_of(pto, l) - rcc * (u0 - 1.f);
                const float ps = csv < psx ? csv : psx;
                const float ptx = -div + ps + rcc * u0;
                const float ptn = ctv < ptx ? ctv : ptx;
                const float err = div - ps + ptn;
                const float un = u0 - err / rcc;
                op[l] = ptn;
                on[l] = (stopped >> l) & 1u ? u0 : un;
                ot[l] = err - un * rcc;
                if (CHECK) acc[l] += fabsf(err);
            }
            ptp[i] = make_float4(op[0], op[1], op[2], op[3]);
            up[i] = make_float4(on[0], on[1], on[2], on[3]);
            tmp[i] = make_float4(ot[0], ot[1], ot[2], ot[3]);
        }
    }
    if (CHECK) {
        const int tid = threadIdx.x + kBX * threadIdx.y;
#pragma unroll
        for (int l = 0; l < kLanes; ++l)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[l] += __shfl_down_sync(0xffffffffu, acc[l], o);
        if ((tid & 31) == 0) red[tid >> 5] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        __syncthreads();
        if (tid == 0) {
            float4 s = red[0];
            for (int w = 1; w < kTile / 32; ++w) {
                s.x += red[w].x; s.y += red[w].y; s.z += red[w].z; s.w += red[w].w;
            }
            partials[G.part_off + wk.y] = s;
        }
    }
}

// ---- one-lane groups: the single solve's sweep bodies over the work list ----
// resident blocks per SM of the one-lane sweeps: 4 (64 registers) measured
// fastest on GB300 (the 12-volume ragged batch: 0.91x -> 1.01x its plain solves)
#ifndef M16_BATCH1_MINB
#define M16_BATCH1_MINB 4
#endif
// z-slices whose loads the one-lane flow / label sweeps issue together, and
// whether the flow sweep reads its view (the descriptor values) from shared
// memory.  Measured on GB300 for one 256^3 instance of 1000 iterations (with
// an alpha field in brackets), the single solve's own sweeps taking 232 ms:
//   view in registers: flow 1 / label 4 259 (257) ms, flow 2 / label 4 264
//   (285), flow 1 / label 2 293 (291), flow 2 / label 2 297 (319);
//   flow view in shared memory, flow 2 / label 4: 245 (243) ms; both views in
//   shared memory, flow 2 / label 2: 258 (256).
#ifndef M16_BATCH1_FZB
#define M16_BATCH1_FZB 2
#endif
#ifndef M16_BATCH1_UZB
#define M16_BATCH1_UZB M16_MF_UZB
#endif
// bit 1: the one-lane flow sweep reads its view from shared memory, bit 2:
// the label sweep does
#ifndef M16_BATCH1_SMEM_VIEW
#define M16_BATCH1_SMEM_VIEW 1
#endif

template <int ALPHA>
__global__ void __launch_bounds__(kTile, M16_BATCH1_MINB) bt1_flow_kernel(const int2 *__restrict__ work,
                                                                         const VolDev *vols, const GroupDev *groups,
                                                                         const unsigned *__restrict__ gmask)
{
    pdl_wait();
    pdl_launch_next();
    const int2 wk = work[blockIdx.x];
    if (__ldcg(gmask + wk.x) & 1u) return;
    const GroupDev &G = groups[wk.x];
    const VolDev &V = vols[G.vol];
    int bx, by, bz;
    decode_tile(V, wk.y, bx, by, bz);
    const int x = bx * kBX + threadIdx.x, y = by * kBY + threadIdx.y;
#if (M16_BATCH1_SMEM_VIEW & 1)
    // the view in shared memory: its fields are read where used instead of
    // held in registers for the whole column
    __shared__ FlowView sf;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        float *st = (float *)G.state;
        const int64_t S = G.slab;
        sf.d0 = V.d0; sf.d1 = V.d1; sf.d2 = V.d2;
        sf.ss0 = V.ss0; sf.ss1 = V.ss1; sf.ss2 = V.ss2;
        sf.sq0 = G.sq0; sf.sq1 = G.sq1; sf.sq2 = G.sq2; sf.isq0 = G.isq0; sf.isq1 = G.isq1; sf.isq2 = G.isq2;
        sf.alpha_scalar = 0.f;
        sf.alpha = G.alpha1;
        sf.grad2 = V.grad2;
        sf.w = G.w.x;
        sf.neg_inv_decay2 = G.nid2.x;
        sf.sqeigs = nullptr;
        sf.q4 = V.q4;
        sf.tmp = st + 4 * S;
        sf.hp0 = st; sf.hp1 = st + S; sf.hp2 = st + 2 * S;
    }
    __syncthreads();
    if (x >= sf.d2 || y >= sf.d1) return;
    const int zc = V.zc;
    const int z0 = bz * zc, z1 = min(z0 + zc, sf.d0);
    flow_column<false, ALPHA, M16_BATCH1_FZB>(sf, x, y, z0, z1);
#else
    if (x >= V.d2 || y >= V.d1) return;
    const int z0 = bz * V.zc, z1 = min(z0 + V.zc, V.d0);
    float *st = (float *)G.state;
    const int64_t S = G.slab;
    FlowView f;
    f.d0 = V.d0; f.d1 = V.d1; f.d2 = V.d2;
    f.ss0 = V.ss0; f.ss1 = V.ss1; f.ss2 = V.ss2;
    f.sq0 = G.sq0; f.sq1 = G.sq1; f.sq2 = G.sq2; f.isq0 = G.isq0; f.isq1 = G.isq1; f.isq2 = G.isq2;
    f.alpha_scalar = 0.f;
    f.alpha = G.alpha1;
    f.grad2 = V.grad2;
    f.w = G.w.x;
    f.neg_inv_decay2 = G.nid2.x;
    f.sqeigs = nullptr;
    f.q4 = V.q4;
    f.tmp = st + 4 * S;
    f.hp0 = st; f.hp1 = st + S; f.hp2 = st + 2 * S;
    flow_column<false, ALPHA, M16_BATCH1_FZB>(f, x, y, z0, z1);
#endif
}

template <bool CHECK>
__global__ void __launch_bounds__(kTile, M16_BATCH1_MINB) bt1_label_kernel(const int2 *__restrict__ work,
                                                                          const VolDev *vols, const GroupDev *groups,
                                                                          const unsigned *__restrict__ gmask,
                                                                          float4 *__restrict__ partials)
{
    pdl_wait();
    pdl_launch_next();
    __shared__ float red[kTile / 32];
    const int2 wk = work[blockIdx.x];
    if (__ldcg(gmask + wk.x) & 1u) return;   // uniform over the block
    const GroupDev &G = groups[wk.x];
    const VolDev &V = vols[G.vol];
    int bx, by, bz;
    decode_tile(V, wk.y, bx, by, bz);
    const int x = bx * kBX + threadIdx.x, y = by * kBY + threadIdx.y;
    const int z0 = bz * V.zc, z1 = min(z0 + V.zc, V.d0);
    float acc = 0.f;
#if (M16_BATCH1_SMEM_VIEW & 2)
    __shared__ LabelView sl;   // read where used, not held in registers
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        float *st = (float *)G.state;
        const int64_t S = G.slab;
        sl.d0 = V.d0; sl.d1 = V.d1; sl.d2 = V.d2;
        sl.rcc = V.rcc; sl.rs0 = V.rs0; sl.rs1 = V.rs1; sl.rs2 = V.rs2;
        sl.hp0 = st; sl.hp1 = st + S; sl.hp2 = st + 2 * S;
        sl.cs = V.cs; sl.ct = V.ct; sl.labels = nullptr;
        sl.pt = st + 3 * S; sl.tmp = st + 4 * S; sl.u = st + 5 * S;
    }
    __syncthreads();
    if (x < sl.d2 && y < sl.d1) acc = label_column<false, M16_BATCH1_UZB>(sl, x, y, z0, z1);
#else
    if (x < V.d2 && y < V.d1) {
        float *st = (float *)G.state;
        const int64_t S = G.slab;
        LabelView l;
        l.d0 = V.d0; l.d1 = V.d1; l.d2 = V.d2;
        l.rcc = V.rcc; l.rs0 = V.rs0; l.rs1 = V.rs1; l.rs2 = V.rs2;
        l.hp0 = st; l.hp1 = st + S; l.hp2 = st + 2 * S;
        l.cs = V.cs; l.ct = V.ct; l.labels = nullptr;
        l.pt = st + 3 * S; l.tmp = st + 4 * S; l.u = st + 5 * S;
        acc = label_column<false, M16_BATCH1_UZB>(l, x, y, z0, z1);
    }
#endif
    if (CHECK) {
        const int tid = threadIdx.x + kBX * threadIdx.y;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if ((tid & 31) == 0) red[tid >> 5] = acc;
        __syncthreads();
        if (tid == 0) {
            float s = red[0];
            for (int w = 1; w < kTile / 32; ++w) s += red[w];
            partials[G.part_off + wk.y] = make_float4(s, 0.f, 0.f, 0.f);
        }
    }
}

// one block per instance: residual = sum over the tiles of its lane's partial
// sums / (N * rcc); below the bound (or NaN) the instance stops.  Every
// instance is checked at its own iterations 0, update, 2 update, ..., so the
// n-th check (from 0) follows iteration n * update and a stop there counts
// n * update + 1 iterations, wherever the instance joined the batch.
__global__ void bt_check_kernel(const VolDev *vols, const GroupDev *groups, const InstDev *insts,
                                InstCtrl *ctrl, unsigned *gmask, const float4 *__restrict__ partials, double bound,
                                int update, const int *__restrict__ list)
{
    pdl_wait();
    pdl_launch_next();
    __shared__ double s[256];
    const int inst = list ? list[blockIdx.x] : (int)blockIdx.x;   // list: the instances to check
    const InstDev &I = insts[inst];
    InstCtrl &C = ctrl[inst];
    if (__ldcg(&C.stopped)) return;
    const GroupDev &G = groups[I.group];
    const VolDev &V = vols[G.vol];
    const float *p = (const float *)(partials + G.part_off) + I.lane;
    double acc = 0.0;
    for (int k = threadIdx.x; k < G.nparts; k += blockDim.x) acc += (double)p[4 * k];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double err = s[0] / ((double)V.n * (double)V.rcc);
        C.resid = err;
        const int n = C.n_checks;
        C.n_checks = n + 1;
        if (isnan(err) || err < bound) {
            C.stopped = 1;
            C.iterations = n * update + 1;
            atomicOr(gmask + I.group, 1u << I.lane);
        }
    }
}

}  // namespace
}  // namespace m16
