// batched.cu -- many ATV max-flow solves in one launch per sweep.
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
// Stopping.  The check kernel sets a lane's bit in its group's stop mask; the
// label sweep then keeps that lane's u (the solve's result) unchanged, blocks
// of a group whose lanes have all stopped return at once, and the work list
// drops finished groups.  At the end u is scattered out of the interleaved
// field into each instance's output array.
#include <cuda_runtime.h>
#include <math.h>
#include <float.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"

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
    int vol, part_off, nparts, has_alpha;
    float4 w, nid2;          // per lane: alpha = w * exp(nid2 * |grad I|^2), nid2 = -1 / decay^2
    float sq0, sq1, sq2, isq0, isq1, isq2;
    float4 *state;           // kFields (+1) slabs of `slab` float4
    int64_t slab;
};

struct InstDev {
    int group, lane;
    float *u_out;
    const float *alpha;
};

// z-slices per block: enough blocks for M16_BATCH_BLOCKS_PER_SM per SM over
// the volume's groups (many short blocks keep the last wave short), at most 32
#ifndef M16_BATCH_BLOCKS_PER_SM
#define M16_BATCH_BLOCKS_PER_SM 16
#endif
#ifndef M16_BATCH_MINB
#define M16_BATCH_MINB 3
#endif
inline int batch_zc(int d0, int d1, int d2, int ngroups_of_volume)
{
    const int64_t cols = div_up(d2, kBX) * div_up(d1, kBY);
    int64_t zc = (int64_t)d0 * cols * std::max(ngroups_of_volume, 1) /
                 ((int64_t)M16_BATCH_BLOCKS_PER_SM * kSMs);
    zc = std::max<int64_t>(1, std::min<int64_t>(32, zc));
    return (int)zc;
}

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
    float4 *st = G.state;
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
    float4 *al = G.state + kFields * G.slab;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        al[i] = make_float4(a0 ? a0[i] : 0.f, a1 ? a1[i] : 0.f, a2 ? a2[i] : 0.f, a3 ? a3[i] : 0.f);
}

// u of one instance out of its group's interleaved field
__global__ void bt_scatter_u_kernel(const GroupDev *groups, const InstDev *insts, int inst, int64_t n)
{
    const InstDev &I = insts[inst];
    const GroupDev &G = groups[I.group];
    const float *u4 = (const float *)(G.state + 5 * G.slab);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        I.u_out[i] = u4[4 * i + I.lane];
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
    float4 *__restrict__ hp0 = G.state;
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
        const float4 *__restrict__ hp0 = G.state;
        const float4 *__restrict__ hp1 = hp0 + S;
        const float4 *__restrict__ hp2 = hp1 + S;
        float4 *__restrict__ ptp = G.state + 3 * S;
        float4 *__restrict__ tmp = G.state + 4 * S;
        float4 *__restrict__ up = G.state + 5 * S;
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

// one block per instance: residual = sum over the tiles of its lane's partial
// sums / (N * rcc); below the bound (or NaN) the instance stops
__global__ void bt_check_kernel(const VolDev *vols, const GroupDev *groups, const InstDev *insts,
                                InstCtrl *ctrl, unsigned *gmask, const float4 *__restrict__ partials, double bound,
                                int iter)
{
    __shared__ double s[256];
    const InstDev &I = insts[blockIdx.x];
    InstCtrl &C = ctrl[blockIdx.x];
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
        C.n_checks += 1;
        if (isnan(err) || err < bound) {
            C.stopped = 1;
            C.iterations = iter + 1;
            atomicOr(gmask + I.group, 1u << I.lane);
        }
    }
}

// ---- host side --------------------------------------------------------------

struct Plan {
    std::vector<int> inst_group, inst_lane;       // per instance
    std::vector<std::vector<int>> group_insts;    // per group: instance per lane (-1 padding)
    std::vector<int> group_vol;
    std::vector<int> ngroups_of_vol;
};

// groups: instances of one volume with the same eigenvalues and the same kind
// of alpha, in instance order, four to a group
inline Plan make_plan(int nvol, const m16_batch_instance *inst, int ninst)
{
    Plan P;
    P.inst_group.assign(ninst, -1);
    P.inst_lane.assign(ninst, -1);
    P.ngroups_of_vol.assign(nvol, 0);
    std::map<std::tuple<int, double, double, double, int>, int> open;   // key -> group with free lanes
    for (int i = 0; i < ninst; ++i) {
        const m16_batch_instance &I = inst[i];
        const auto key = std::make_tuple(I.volume, I.sqevals[0], I.sqevals[1], I.sqevals[2], I.alpha ? 1 : 0);
        auto it = open.find(key);
        int g;
        if (it == open.end()) {
            g = (int)P.group_insts.size();
            P.group_insts.push_back(std::vector<int>(kLanes, -1));
            P.group_vol.push_back(I.volume);
            P.ngroups_of_vol[I.volume] += 1;
            open[key] = g;
        } else {
            g = it->second;
        }
        int lane = 0;
        while (P.group_insts[g][lane] >= 0) ++lane;
        P.group_insts[g][lane] = i;
        P.inst_group[i] = g;
        P.inst_lane[i] = lane;
        if (lane == kLanes - 1) open.erase(key);
    }
    return P;
}

struct BatchLayout {
    std::vector<size_t> q4, maxpart;        // per volume
    std::vector<size_t> state;              // per group
    std::vector<int> part_off, nparts;      // per group (float4 units)
    size_t ctrl, gmask, vols, groups, insts, work, partials, total;
    int64_t total_blocks, total_parts;
};

constexpr int kMaxBlocks = 4 * kSMs;

inline BatchLayout batch_layout(const m16_batch_volume *vols, int nvol, const m16_batch_instance *inst, int ninst,
                                const Plan &P)
{
    BatchLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    std::vector<int64_t> tiles(nvol);
    for (int v = 0; v < nvol; ++v) {
        const int64_t n = (int64_t)vols[v].d0 * vols[v].d1 * vols[v].d2;
        L.q4.push_back(take(n * 16));
        L.maxpart.push_back(take(kMaxBlocks * 4));
        const int zc = batch_zc(vols[v].d0, vols[v].d1, vols[v].d2, P.ngroups_of_vol[v]);
        tiles[v] = div_up(vols[v].d2, kBX) * div_up(vols[v].d1, kBY) * div_up(vols[v].d0, zc);
    }
    L.total_blocks = 0;
    L.total_parts = 0;
    const int ngroups = (int)P.group_insts.size();
    for (int g = 0; g < ngroups; ++g) {
        const m16_batch_volume &V = vols[P.group_vol[g]];
        const int64_t n = (int64_t)V.d0 * V.d1 * V.d2;
        const bool has_alpha = inst[P.group_insts[g][0]].alpha != nullptr;
        L.state.push_back(take((kFields + (has_alpha ? 1 : 0)) * align_up(n * 16, 256)));
        L.part_off.push_back((int)L.total_parts);
        L.nparts.push_back((int)tiles[P.group_vol[g]]);
        L.total_parts += tiles[P.group_vol[g]];
        L.total_blocks += tiles[P.group_vol[g]];
    }
    L.ctrl = take(sizeof(InstCtrl) * std::max(ninst, 1));
    L.gmask = take(sizeof(unsigned) * std::max(ngroups, 1));
    L.vols = take(sizeof(VolDev) * std::max(nvol, 1));
    L.groups = take(sizeof(GroupDev) * std::max(ngroups, 1));
    L.insts = take(sizeof(InstDev) * std::max(ninst, 1));
    L.work = take(sizeof(int2) * std::max<int64_t>(L.total_blocks, 1));
    L.partials = take(16 * std::max<int64_t>(L.total_parts, 1));
    L.total = off;
    return L;
}

bool batch_args_ok(const m16_batch_volume *vols, int nvol, const m16_batch_instance *inst, int ninst)
{
    if (!vols || !inst || nvol < 1 || ninst < 1) return false;
    for (int v = 0; v < nvol; ++v) {
        const m16_batch_volume &V = vols[v];
        if (V.d0 < 1 || V.d1 < 1 || V.d2 < 1 || !V.img || !V.quat3 || !V.cs || !V.ct) return false;
        // the sweeps index a volume with 32-bit voxel offsets
        if ((int64_t)V.d0 * V.d1 * V.d2 > (int64_t)INT32_MAX) return false;
        for (int k = 0; k < 3; ++k)
            if (!(V.scaling[k] > 0.0)) return false;
    }
    for (int i = 0; i < ninst; ++i) {
        const m16_batch_instance &I = inst[i];
        if (I.volume < 0 || I.volume >= nvol || !I.u) return false;
        if (!I.alpha && (!vols[I.volume].grad2 || !(I.decay != 0.0))) return false;
        for (int k = 0; k < 3; ++k)
            if (!(I.sqevals[k] > 0.0)) return false;
    }
    return true;
}

}  // namespace
}  // namespace m16

using namespace m16;

extern "C" size_t m16_batch_workspace_bytes(const m16_batch_volume *vols, int32_t nvol,
                                            const m16_batch_instance *inst, int32_t ninst)
{
    if (!batch_args_ok(vols, nvol, inst, ninst)) return 0;
    return batch_layout(vols, nvol, inst, ninst, make_plan(nvol, inst, ninst)).total;
}

extern "C" int m16_batch_solve(const m16_batch_volume *vols, int32_t nvol, const m16_batch_instance *inst,
                               int32_t ninst, const m16_cut_params *params, int32_t *iterations, double *residuals,
                               void *workspace, size_t workspace_bytes, void *stream, m16_solve_stats *stats)
{
    if (!params || params->update < 1 || params->num_iter < 0 || !(params->cc > 0.0)) return M16_ERR_BAD_ARG;
    if (!batch_args_ok(vols, nvol, inst, ninst)) return M16_ERR_BAD_ARG;
    if (stats && (stats->path < M16_PATH_DEFAULT || stats->path > M16_PATH_FUSED)) return M16_ERR_BAD_ARG;
    const Plan P = make_plan(nvol, inst, ninst);
    const BatchLayout L = batch_layout(vols, nvol, inst, ninst, P);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    const int ngroups = (int)P.group_insts.size();

    // device descriptors
    std::vector<VolDev> hv(nvol);
    for (int v = 0; v < nvol; ++v) {
        const m16_batch_volume &V = vols[v];
        VolDev &d = hv[v];
        d.d0 = V.d0; d.d1 = V.d1; d.d2 = V.d2;
        d.zc = batch_zc(V.d0, V.d1, V.d2, P.ngroups_of_vol[v]);
        d.tx = (int)div_up(V.d2, kBX); d.ty = (int)div_up(V.d1, kBY); d.tz = (int)div_up(V.d0, d.zc);
        const double *sc = V.scaling;
        const double smin = fmin(sc[0], fmin(sc[1], sc[2]));
        d.rcc = (float)(1.0 / (params->cc * (smin * smin)));
        d.rs0 = (float)(1.0 / sc[0]); d.rs1 = (float)(1.0 / sc[1]); d.rs2 = (float)(1.0 / sc[2]);
        d.ss0 = (float)(params->steps / sc[0] * (smin * smin));
        d.ss1 = (float)(params->steps / sc[1] * (smin * smin));
        d.ss2 = (float)(params->steps / sc[2] * (smin * smin));
        d.denom = 1.f;
        d.q4 = (const float4 *)(ws + L.q4[v]);
        d.grad2 = V.grad2; d.cs = V.cs; d.ct = V.ct;
        d.n = (int64_t)V.d0 * V.d1 * V.d2;
    }
    std::vector<GroupDev> hg(ngroups);
    std::vector<unsigned> hmask(ngroups, 0u);
    for (int g = 0; g < ngroups; ++g) {
        GroupDev &d = hg[g];
        const std::vector<int> &lanes = P.group_insts[g];
        const m16_batch_instance &I0 = inst[lanes[0]];
        d.vol = P.group_vol[g];
        d.part_off = L.part_off[g];
        d.nparts = L.nparts[g];
        d.has_alpha = I0.alpha ? 1 : 0;
        float w[kLanes], nid2[kLanes];
        for (int l = 0; l < kLanes; ++l) {
            const int i = lanes[l];
            if (i < 0) {   // padding lane: alpha 0, counted as stopped
                w[l] = 0.f;
                nid2[l] = 0.f;
                hmask[g] |= 1u << l;
                continue;
            }
            w[l] = (float)inst[i].weighting;
            nid2[l] = inst[i].alpha ? 0.f : (float)(-1.0 / (inst[i].decay * inst[i].decay));
        }
        d.w = make_float4(w[0], w[1], w[2], w[3]);
        d.nid2 = make_float4(nid2[0], nid2[1], nid2[2], nid2[3]);
        d.sq0 = (float)I0.sqevals[0]; d.sq1 = (float)I0.sqevals[1]; d.sq2 = (float)I0.sqevals[2];
        d.isq0 = (float)(1.0 / I0.sqevals[0]); d.isq1 = (float)(1.0 / I0.sqevals[1]);
        d.isq2 = (float)(1.0 / I0.sqevals[2]);
        d.state = (float4 *)(ws + L.state[g]);
        d.slab = (int64_t)(align_up(hv[d.vol].n * 16, 256) / 16);
    }
    std::vector<InstDev> hi(ninst);
    for (int i = 0; i < ninst; ++i) {
        hi[i].group = P.inst_group[i];
        hi[i].lane = P.inst_lane[i];
        hi[i].u_out = inst[i].u;
        hi[i].alpha = inst[i].alpha;
    }
    std::vector<InstCtrl> hctrl(ninst);
    for (int i = 0; i < ninst; ++i) {
        hctrl[i].stopped = 0;
        hctrl[i].iterations = params->num_iter;
        hctrl[i].n_checks = 0;
        hctrl[i].pad = 0;
        hctrl[i].resid = NAN;
    }
    VolDev *dvols = (VolDev *)(ws + L.vols);
    GroupDev *dgroups = (GroupDev *)(ws + L.groups);
    InstDev *dinsts = (InstDev *)(ws + L.insts);
    InstCtrl *dctrl = (InstCtrl *)(ws + L.ctrl);
    unsigned *dmask = (unsigned *)(ws + L.gmask);
    int2 *dwork = (int2 *)(ws + L.work);
    float4 *dpart = (float4 *)(ws + L.partials);
    M16_CUDA_TRY(cudaMemcpyAsync(dvols, hv.data(), sizeof(VolDev) * nvol, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dgroups, hg.data(), sizeof(GroupDev) * ngroups, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dinsts, hi.data(), sizeof(InstDev) * ninst, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dctrl, hctrl.data(), sizeof(InstCtrl) * ninst, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dmask, hmask.data(), sizeof(unsigned) * ngroups, cudaMemcpyHostToDevice, st));

    // per-volume set-up, then per-group state
    int launches = 0;
    for (int v = 0; v < nvol; ++v) {
        const int blocks = (int)std::min<int64_t>(kMaxBlocks, div_up(hv[v].n, 256));
        float *mp = (float *)(ws + L.maxpart[v]);
        bt_max_kernel<<<blocks, 256, 0, st>>>(vols[v].img, hv[v].n, mp);
        bt_denom_kernel<<<1, 32, 0, st>>>(mp, blocks, dvols + v);
        bt_expand_kernel<<<blocks, 256, 0, st>>>(vols[v].quat3, (float4 *)(ws + L.q4[v]), hv[v].n);
        launches += 3;
    }
    for (int g = 0; g < ngroups; ++g) {
        const int64_t n = hv[hg[g].vol].n;
        const int blocks = (int)std::min<int64_t>(kMaxBlocks, div_up(n, 256));
        bt_init_group_kernel<<<blocks, 256, 0, st>>>(vols[hg[g].vol].img, dvols, dgroups, g);
        ++launches;
        if (hg[g].has_alpha) {
            const float *a[kLanes];
            for (int l = 0; l < kLanes; ++l)
                a[l] = P.group_insts[g][l] >= 0 ? inst[P.group_insts[g][l]].alpha : nullptr;
            bt_gather_alpha_kernel<<<blocks, 256, 0, st>>>(dgroups, g, a[0], a[1], a[2], a[3], n);
            ++launches;
        }
    }
    M16_CUDA_TRY(cudaGetLastError());

    // the work list: per group and tile, groups with an active lane only;
    // alpha-field groups first (the flow sweep is compiled per alpha kind)
    std::vector<char> gactive(ngroups, 1);
    for (int g = 0; g < ngroups; ++g) gactive[g] = hmask[g] != kAllLanes;
    int n_alpha_items = 0;
    auto build_work = [&](std::vector<int2> &w) {
        w.clear();
        for (int pass = 0; pass < 2; ++pass) {
            for (int g = 0; g < ngroups; ++g) {
                if (!gactive[g] || (hg[g].has_alpha != 0) != (pass == 0)) continue;
                const VolDev &V = hv[hg[g].vol];
                const int ntiles = V.tx * V.ty * V.tz;
                for (int t = 0; t < ntiles; ++t) w.push_back(make_int2(g, t));
            }
            if (pass == 0) n_alpha_items = (int)w.size();
        }
    };
    std::vector<int2> work;
    build_work(work);
    M16_CUDA_TRY(cudaMemcpyAsync(dwork, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, st));

    const int update = params->update;
    const int chunk = update * std::max(1, 64 / update);
    const bool timing = stats && stats->time_kernels;
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    if (timing) {
        M16_CUDA_TRY(cudaEventCreate(&e0));
        M16_CUDA_TRY(cudaEventCreate(&e1));
        M16_CUDA_TRY(cudaEventCreate(&e2));
    }
    double p_ms = 0.0, u_ms = 0.0;
    int p_n = 0, u_n = 0;
    int it = 0;
    int n_groups_active = ngroups;
    int listed = ngroups;   // groups in the current work list
    const dim3 block(kBX, kBY, 1);
    while (it < params->num_iter && n_groups_active > 0 && !work.empty()) {
        const int end = std::min(params->num_iter, it + chunk);
        const int nb_alpha = n_alpha_items;
        const int nb_exp = (int)work.size() - n_alpha_items;
        for (; it < end; ++it) {
            if (timing) cudaEventRecord(e0, st);
            const bool check = (it % update) == 0;
            if (nb_alpha > 0) bt_flow_kernel<true><<<nb_alpha, block, 0, st>>>(dwork, dvols, dgroups, dmask);
            if (nb_exp > 0) bt_flow_kernel<false><<<nb_exp, block, 0, st>>>(dwork + nb_alpha, dvols, dgroups, dmask);
            if (timing) cudaEventRecord(e1, st);
            if (check)
                bt_label_kernel<true><<<(unsigned)work.size(), block, 0, st>>>(dwork, dvols, dgroups, dmask, dpart);
            else
                bt_label_kernel<false><<<(unsigned)work.size(), block, 0, st>>>(dwork, dvols, dgroups, dmask, dpart);
            if (timing) {
                cudaEventRecord(e2, st);
                M16_CUDA_TRY(cudaEventSynchronize(e2));
                float a = 0.f, b = 0.f;
                cudaEventElapsedTime(&a, e0, e1);
                cudaEventElapsedTime(&b, e1, e2);
                p_ms += a; ++p_n;
                u_ms += b; ++u_n;
            }
            launches += (nb_alpha > 0) + (nb_exp > 0) + 1;
            if (check) {
                bt_check_kernel<<<ninst, 256, 0, st>>>(dvols, dgroups, dinsts, dctrl, dmask, dpart,
                                                       params->error_bound, it);
                ++launches;
            }
        }
        M16_CUDA_TRY(cudaGetLastError());
        M16_CUDA_TRY(cudaMemcpyAsync(hmask.data(), dmask, sizeof(unsigned) * ngroups, cudaMemcpyDeviceToHost, st));
        M16_CUDA_TRY(cudaStreamSynchronize(st));
        n_groups_active = 0;
        for (int g = 0; g < ngroups; ++g) {
            gactive[g] = hmask[g] != kAllLanes;
            n_groups_active += gactive[g];
        }
        // drop finished groups from the work list once they are a quarter of it
        if (n_groups_active > 0 && n_groups_active * 4 <= listed * 3) {
            build_work(work);
            listed = n_groups_active;
            M16_CUDA_TRY(cudaMemcpyAsync(dwork, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, st));
        }
    }
    if (timing) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(e2);
    }
    for (int i = 0; i < ninst; ++i) {
        const int64_t n = hv[inst[i].volume].n;
        const int blocks = (int)std::min<int64_t>(kMaxBlocks, div_up(n, 256));
        bt_scatter_u_kernel<<<blocks, 256, 0, st>>>(dgroups, dinsts, i, n);
        ++launches;
    }
    M16_CUDA_TRY(cudaGetLastError());
    M16_CUDA_TRY(cudaMemcpyAsync(hctrl.data(), dctrl, sizeof(InstCtrl) * ninst, cudaMemcpyDeviceToHost, st));
    M16_CUDA_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < ninst; ++i) {
        if (iterations) iterations[i] = hctrl[i].iterations;
        if (residuals) residuals[i] = hctrl[i].resid;
    }
    if (stats) {
        stats->launches = launches;
        stats->p_launches = p_n;
        stats->u_launches = u_n;
        stats->p_ms = p_ms;
        stats->u_ms = u_ms;
    }
    return M16_OK;
}
