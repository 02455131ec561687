// batched.cu -- m16_batch_solve: a fixed batch of ATV max-flow instances
// run to completion, every flow / label launch covering all active instances
// (device side and layout in batch_kernels.cuh).
#include <cuda_runtime.h>
#include <math.h>
#include <float.h>

#include <algorithm>
#include <cstddef>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "batch_kernels.cuh"

namespace m16 {
namespace {

// ---- host side --------------------------------------------------------------

struct Plan {
    std::vector<int> inst_group, inst_lane;       // per instance
    std::vector<std::vector<int>> group_insts;    // per group: instance per lane (-1 padding)
    std::vector<int> group_vol, group_lanes;
    std::vector<int> ngroups_of_vol;
};

// groups: instances of one volume with the same eigenvalues and the same kind
// of alpha, in instance order, four to a group; a group that would hold fewer
// than three instances becomes one-lane groups (padding lanes would stream
// more than the shared volume data saves)
inline Plan make_plan(int nvol, const m16_batch_instance *inst, int ninst)
{
    Plan Q;   // four-lane grouping first
    Q.inst_group.assign(ninst, -1);
    Q.inst_lane.assign(ninst, -1);
    {
        std::map<std::tuple<int, double, double, double, int>, int> open;
        for (int i = 0; i < ninst; ++i) {
            const m16_batch_instance &I = inst[i];
            const auto key = std::make_tuple(I.volume, I.sqevals[0], I.sqevals[1], I.sqevals[2], I.alpha ? 1 : 0);
            auto it = open.find(key);
            int g;
            if (it == open.end()) {
                g = (int)Q.group_insts.size();
                Q.group_insts.push_back(std::vector<int>(kLanes, -1));
                open[key] = g;
            } else {
                g = it->second;
            }
            int lane = 0;
            while (Q.group_insts[g][lane] >= 0) ++lane;
            Q.group_insts[g][lane] = i;
            if (lane == kLanes - 1) open.erase(key);
        }
    }
    Plan P;
    P.inst_group.assign(ninst, -1);
    P.inst_lane.assign(ninst, -1);
    P.ngroups_of_vol.assign(nvol, 0);
    for (const std::vector<int> &lanes : Q.group_insts) {
        int real = 0;
        for (int i : lanes) real += i >= 0;
        const int vol = inst[lanes[0]].volume;
        if (real >= 3) {
            const int g = (int)P.group_insts.size();
            P.group_insts.push_back(lanes);
            P.group_vol.push_back(vol);
            P.group_lanes.push_back(kLanes);
            P.ngroups_of_vol[vol] += 1;
            for (int l = 0; l < kLanes; ++l)
                if (lanes[l] >= 0) { P.inst_group[lanes[l]] = g; P.inst_lane[lanes[l]] = l; }
        } else {
            for (int i : lanes) {
                if (i < 0) continue;
                const int g = (int)P.group_insts.size();
                std::vector<int> one(kLanes, -1);
                one[0] = i;
                P.group_insts.push_back(one);
                P.group_vol.push_back(vol);
                P.group_lanes.push_back(1);
                P.ngroups_of_vol[vol] += 1;
                P.inst_group[i] = g;
                P.inst_lane[i] = 0;
            }
        }
    }
    return P;
}

struct BatchLayout {
    std::vector<size_t> q4, maxpart;        // per volume
    std::vector<size_t> state;              // per group
    std::vector<int64_t> part_off;          // per group (float4 units)
    std::vector<int> nparts;                // per group
    size_t ctrl, gmask, vols, groups, insts, work, partials, total;
    int64_t total_blocks, total_parts;
};

constexpr int kMaxBlocks = 4 * kSMs;

// Autotuner of the sweeps' tile shape: the z-chunk of a (32 x 8 x zc) tile
// follows from a target number of blocks per SM; the candidates are timed on
// one check interval each of the solve itself and the fastest is kept for the
// rest of it and for later batches of the same shape (a process-wide cache).
constexpr int kTuneBps[3] = {8, 16, 32};
constexpr int kTuneMinItems = kSMs;   // smaller work lists are launch-bound: keep the default

std::mutex g_tune_mu;
std::map<std::vector<int64_t>, int> g_tuned;   // batch shape -> blocks per SM

inline BatchLayout batch_layout(const m16_batch_volume *vols, int nvol, const m16_batch_instance *inst, int ninst,
                                const Plan &P)
{
    BatchLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    std::vector<int64_t> tiles(nvol);
    int64_t total_cs = 0;
    for (int v = 0; v < nvol; ++v)
        total_cs += column_slices(vols[v].d0, vols[v].d1, vols[v].d2) * P.ngroups_of_vol[v];
    for (int v = 0; v < nvol; ++v) {
        const int64_t n = (int64_t)vols[v].d0 * vols[v].d1 * vols[v].d2;
        L.q4.push_back(take(n * 16));
        L.maxpart.push_back(take(kMaxBlocks * 4));
        // sized for the candidate with the most (smallest) tiles
        int zc = 32;
        for (int c : kTuneBps) zc = std::min(zc, batch_zc_total(total_cs, c));
        tiles[v] = div_up(vols[v].d2, kBX) * div_up(vols[v].d1, kBY) * div_up(vols[v].d0, zc);
    }
    L.total_blocks = 0;
    L.total_parts = 0;
    const int ngroups = (int)P.group_insts.size();
    for (int g = 0; g < ngroups; ++g) {
        const m16_batch_volume &V = vols[P.group_vol[g]];
        const int64_t n = (int64_t)V.d0 * V.d1 * V.d2;
        const bool has_alpha = inst[P.group_insts[g][0]].alpha != nullptr;
        if (P.group_lanes[g] == kLanes)
            L.state.push_back(take((kFields + (has_alpha ? 1 : 0)) * align_up(n * 16, 256)));
        else
            L.state.push_back(take(kFields * align_up(n * 4, 256)));
        L.part_off.push_back(L.total_parts);
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

// The host copies of a batch's descriptors and the device addresses of its
// tables, filled by batch_prepare (which also uploads the descriptors and runs
// the per-volume and per-group set-up kernels on the stream).
struct BatchRun {
    Plan P;
    BatchLayout L;
    int ngroups = 0;
    std::vector<VolDev> hv;
    std::vector<GroupDev> hg;
    std::vector<unsigned> hmask;
    std::vector<InstDev> hi;
    std::vector<InstCtrl> hctrl;
    VolDev *dvols = nullptr;
    GroupDev *dgroups = nullptr;
    InstDev *dinsts = nullptr;
    InstCtrl *dctrl = nullptr;
    unsigned *dmask = nullptr;
    int2 *dwork = nullptr;
    float4 *dpart = nullptr;
};

int batch_prepare(const m16_batch_volume *vols, int nvol, const m16_batch_instance *inst, int ninst,
                  const m16_cut_params *params, char *ws, cudaStream_t st, BatchRun &B, int &launches)
{
    const Plan &P = B.P;
    const BatchLayout &L = B.L;
    const int ngroups = B.ngroups;
    std::vector<VolDev> &hv = B.hv;
    std::vector<GroupDev> &hg = B.hg;
    std::vector<unsigned> &hmask = B.hmask;
    std::vector<InstDev> &hi = B.hi;
    std::vector<InstCtrl> &hctrl = B.hctrl;
    hv.assign(nvol, VolDev());
    hg.assign(ngroups, GroupDev());
    hmask.assign(ngroups, 0u);
    hi.assign(ninst, InstDev());
    hctrl.assign(ninst, InstCtrl());
    // device descriptors
    for (int v = 0; v < nvol; ++v) {
        const m16_batch_volume &V = vols[v];
        VolDev &d = hv[v];
        d.d0 = V.d0; d.d1 = V.d1; d.d2 = V.d2;
        d.zc = 1;   // set by configure()
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
    for (int g = 0; g < ngroups; ++g) {
        GroupDev &d = hg[g];
        const std::vector<int> &lanes = P.group_insts[g];
        const m16_batch_instance &I0 = inst[lanes[0]];
        d.vol = P.group_vol[g];
        d.part_off = L.part_off[g];
        d.nparts = L.nparts[g];
        d.has_alpha = I0.alpha ? 1 : 0;
        d.lanes = P.group_lanes[g];
        d.pad0 = d.pad1 = d.pad2 = 0;
        d.alpha1 = d.lanes == 1 ? I0.alpha : nullptr;
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
        d.state = ws + L.state[g];
        const size_t esz = d.lanes == kLanes ? 16 : 4;
        d.slab = (int64_t)(align_up(hv[d.vol].n * esz, 256) / esz);
    }
    for (int i = 0; i < ninst; ++i) {
        hi[i].group = P.inst_group[i];
        hi[i].lane = P.inst_lane[i];
        hi[i].u_out = inst[i].u;
        hi[i].alpha = inst[i].alpha;
    }
    for (int i = 0; i < ninst; ++i) {
        hctrl[i].stopped = 0;
        hctrl[i].iterations = params->num_iter;
        hctrl[i].n_checks = 0;
        hctrl[i].pad = 0;
        hctrl[i].resid = NAN;
    }
    VolDev *dvols = B.dvols = (VolDev *)(ws + L.vols);
    GroupDev *dgroups = B.dgroups = (GroupDev *)(ws + L.groups);
    InstDev *dinsts = B.dinsts = (InstDev *)(ws + L.insts);
    InstCtrl *dctrl = B.dctrl = (InstCtrl *)(ws + L.ctrl);
    unsigned *dmask = B.dmask = (unsigned *)(ws + L.gmask);
    B.dwork = (int2 *)(ws + L.work);
    B.dpart = (float4 *)(ws + L.partials);
    M16_CUDA_TRY(cudaMemcpyAsync(dvols, hv.data(), sizeof(VolDev) * nvol, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dgroups, hg.data(), sizeof(GroupDev) * ngroups, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dinsts, hi.data(), sizeof(InstDev) * ninst, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dctrl, hctrl.data(), sizeof(InstCtrl) * ninst, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dmask, hmask.data(), sizeof(unsigned) * ngroups, cudaMemcpyHostToDevice, st));

    // per-volume set-up, then per-group state
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
        if (hg[g].has_alpha && hg[g].lanes == kLanes) {
            const float *a[kLanes];
            for (int l = 0; l < kLanes; ++l)
                a[l] = P.group_insts[g][l] >= 0 ? inst[P.group_insts[g][l]].alpha : nullptr;
            bt_gather_alpha_kernel<<<blocks, 256, 0, st>>>(dgroups, g, a[0], a[1], a[2], a[3], n);
            ++launches;
        }
    }
    M16_CUDA_TRY(cudaGetLastError());

    return M16_OK;
}

// one iteration's launches on stream s: the flow sweeps of the four
// work-list segments, the label sweeps, and on check iterations the residual
// check; e0..e2 (optional) bracket the flow and the label launches.  Returns
// the number of launches.
int launch_iteration(const BatchRun &B, const int *seg, int ninst, const m16_cut_params *params, cudaStream_t s,
                     bool check, cudaEvent_t e0, cudaEvent_t e1, cudaEvent_t e2)
{
    const dim3 block(kBX, kBY, 1);
    int n = 0;
    if (e0) cudaEventRecord(e0, s);
    const int n4 = seg[2], n1 = seg[4] - seg[2];
    cudaError_t e = cudaSuccess;
    auto keep = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
    if (seg[1] > seg[0])
        keep(launch_pdl(bt_flow_kernel<true>, dim3(seg[1] - seg[0]), block, s, true, B.dwork + seg[0], B.dvols,
                        B.dgroups, B.dmask));
    if (seg[2] > seg[1])
        keep(launch_pdl(bt_flow_kernel<false>, dim3(seg[2] - seg[1]), block, s, true, B.dwork + seg[1], B.dvols,
                        B.dgroups, B.dmask));
    if (seg[3] > seg[2])
        keep(launch_pdl(bt1_flow_kernel<kAlphaArray>, dim3(seg[3] - seg[2]), block, s, true, B.dwork + seg[2],
                        B.dvols, B.dgroups, B.dmask));
    if (seg[4] > seg[3])
        keep(launch_pdl(bt1_flow_kernel<kAlphaFromGrad2>, dim3(seg[4] - seg[3]), block, s, true, B.dwork + seg[3],
                        B.dvols, B.dgroups, B.dmask));
    if (e1) cudaEventRecord(e1, s);
    if (n4 > 0) {
        if (check)
            keep(launch_pdl(bt_label_kernel<true>, dim3(n4), block, s, true, B.dwork, B.dvols, B.dgroups, B.dmask,
                            B.dpart));
        else
            keep(launch_pdl(bt_label_kernel<false>, dim3(n4), block, s, true, B.dwork, B.dvols, B.dgroups, B.dmask,
                            B.dpart));
    }
    if (n1 > 0) {
        if (check)
            keep(launch_pdl(bt1_label_kernel<true>, dim3(n1), block, s, true, B.dwork + seg[2], B.dvols, B.dgroups,
                            B.dmask, B.dpart));
        else
            keep(launch_pdl(bt1_label_kernel<false>, dim3(n1), block, s, true, B.dwork + seg[2], B.dvols, B.dgroups,
                            B.dmask, B.dpart));
    }
    if (e2) cudaEventRecord(e2, s);
    for (int k = 0; k < 4; ++k) n += seg[k + 1] > seg[k];
    n += (n4 > 0) + (n1 > 0);
    if (check) {
        keep(launch_pdl(bt_check_kernel, dim3(ninst), dim3(256), s, true, (const VolDev *)B.dvols,
                        (const GroupDev *)B.dgroups, (const InstDev *)B.dinsts, B.dctrl, B.dmask,
                        (const float4 *)B.dpart, params->error_bound, params->update, (const int *)nullptr));
        ++n;
    }
    if (e != cudaSuccess) return -1;
    return n;
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
    if (stats && stats->path != M16_PATH_DEFAULT && stats->path != M16_PATH_TWO_SWEEPS) return M16_ERR_BAD_ARG;
    const Plan P = make_plan(nvol, inst, ninst);
    const BatchLayout L = batch_layout(vols, nvol, inst, ninst, P);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    const int ngroups = (int)P.group_insts.size();

    BatchRun B;
    B.P = P;
    B.L = L;
    B.ngroups = ngroups;
    int launches = 0;
    {
        const int r = batch_prepare(vols, nvol, inst, ninst, params, ws, st, B, launches);
        if (r != M16_OK) return r;
    }
    std::vector<VolDev> &hv = B.hv;
    std::vector<GroupDev> &hg = B.hg;
    std::vector<unsigned> &hmask = B.hmask;
    std::vector<InstCtrl> &hctrl = B.hctrl;
    VolDev *dvols = B.dvols;
    GroupDev *dgroups = B.dgroups;
    InstDev *dinsts = B.dinsts;
    InstCtrl *dctrl = B.dctrl;
    unsigned *dmask = B.dmask;
    int2 *dwork = B.dwork;

    // the work list: per group and tile, groups with an active lane only, in
    // four segments (the sweeps are compiled per group kind): four-lane with
    // alpha fields, four-lane with (w, decay), one-lane with alpha fields,
    // one-lane with (w, decay)
    std::vector<char> gactive(ngroups, 1);
    for (int g = 0; g < ngroups; ++g) gactive[g] = hmask[g] != kAllLanes;
    int seg[5] = {0, 0, 0, 0, 0};   // segment k: items seg[k] .. seg[k + 1] - 1
    auto kind_of = [&](int g) { return (hg[g].lanes == kLanes ? 0 : 2) + (hg[g].has_alpha ? 0 : 1); };
    int work_version = 0;   // bumped whenever the work list (and its segments) is rebuilt
    auto build_work = [&](std::vector<int2> &w) {
        ++work_version;
        w.clear();
        for (int k = 0; k < 4; ++k) {
            seg[k] = (int)w.size();
            for (int g = 0; g < ngroups; ++g) {
                if (!gactive[g] || kind_of(g) != k) continue;
                const VolDev &V = hv[hg[g].vol];
                const int ntiles = V.tx * V.ty * V.tz;
                for (int t = 0; t < ntiles; ++t) w.push_back(make_int2(g, t));
            }
        }
        seg[4] = (int)w.size();
    };
    std::vector<int2> work;

    // tile shape: z-chunks for `bps` blocks per SM, the groups' partial-sum
    // slots, the work list (the volumes' max / denominator fields written by
    // the set-up kernels are left alone: only zc..tz are copied)
    int cur_bps = 0;
    int64_t total_cs = 0;
    for (int v = 0; v < nvol; ++v) total_cs += column_slices(hv[v].d0, hv[v].d1, hv[v].d2) * P.ngroups_of_vol[v];
    auto configure = [&](int bps) -> cudaError_t {
        for (int v = 0; v < nvol; ++v) {
            VolDev &d = hv[v];
            d.zc = batch_zc_total(total_cs, bps);
            d.tz = (int)div_up(d.d0, d.zc);
            cudaError_t e = cudaMemcpyAsync((char *)(dvols + v) + offsetof(VolDev, zc), &d.zc, 4 * sizeof(int),
                                            cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) return e;
        }
        int64_t off = 0;
        for (int g = 0; g < ngroups; ++g) {
            const VolDev &V = hv[hg[g].vol];
            hg[g].part_off = off;
            hg[g].nparts = V.tx * V.ty * V.tz;
            off += hg[g].nparts;
        }
        cudaError_t e = cudaMemcpyAsync(dgroups, hg.data(), sizeof(GroupDev) * ngroups, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return e;
        build_work(work);
        cur_bps = bps;
        // the host vectors must stay unchanged until the copies ran
        e = cudaMemcpyAsync(dwork, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return e;
        return cudaStreamSynchronize(st);
    };
    std::vector<int64_t> tune_key;
    for (int v = 0; v < nvol; ++v) {
        tune_key.push_back(vols[v].d0); tune_key.push_back(vols[v].d1); tune_key.push_back(vols[v].d2);
        tune_key.push_back(P.ngroups_of_vol[v]);
    }
    for (int g = 0; g < ngroups; ++g) tune_key.push_back(hg[g].lanes * 2 + hg[g].has_alpha);
    tune_key.push_back(params->update);
    int start_bps = M16_BATCH_BLOCKS_PER_SM;
    bool tune = false;
    if (stats && (stats->flags & M16_BATCH_NO_TUNE) && stats->blocks_per_sm > 0) {
        // a fixed tile shape: one of the tuner's candidates (the workspace is
        // sized for them)
        bool known = false;
        for (int c : kTuneBps) known = known || c == stats->blocks_per_sm;
        if (!known) return M16_ERR_BAD_ARG;
        start_bps = stats->blocks_per_sm;
    }
    if (!(stats && (stats->flags & M16_BATCH_NO_TUNE))) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto f = g_tuned.find(tune_key);
        if (f != g_tuned.end()) start_bps = f->second;
        else tune = true;
    }
    M16_CUDA_TRY(configure(start_bps));
    const bool timed_solve = stats && stats->time_kernels;
    // one-lane groups (ragged batches) run the single solve's sweep bodies,
    // whose tile shape is already tuned; only four-lane groups are tuned
    bool any4 = false;
    for (int g = 0; g < ngroups; ++g) any4 = any4 || hg[g].lanes == kLanes;
    if (timed_solve || !any4 || (int64_t)work.size() < kTuneMinItems || params->num_iter < 4 * params->update)
        tune = false;

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

    // one iteration's launches on stream `s`: the flow sweeps of the four
    // work-list segments, the label sweeps, and on check iterations the
    // residual check; returns the number of launches
    auto enqueue_iteration = [&](cudaStream_t s, bool check, bool time_it) -> int {
        return launch_iteration(B, seg, ninst, params, s, check, time_it ? e0 : nullptr, time_it ? e1 : nullptr,
                                time_it ? e2 : nullptr);
    };

    // Full chunks (chunk iterations starting at a multiple of `update`, so
    // the check pattern is the same in every one) are captured once per work
    // list into a CUDA graph on a private stream and replayed on `st`; the
    // last partial chunk and timed solves launch directly.
    const bool use_graph = !timing && !(stats && (stats->flags & M16_BATCH_NO_GRAPH));
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int graph_launches = 0;
    int graph_version = -1;   // the work list the graph was captured from
    auto drop_graph = [&]() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        gexec = nullptr;
        graph = nullptr;
    };
    cudaEvent_t *tune_events[2] = {nullptr, nullptr};
    auto release = [&]() {
        drop_graph();
        if (cap) cudaStreamDestroy(cap);
        cap = nullptr;
        for (cudaEvent_t *e : tune_events)
            if (e && *e) { cudaEventDestroy(*e); *e = nullptr; }
        if (timing) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaEventDestroy(e2);
        }
    };
#define M16_BT_TRY(expr)                                           \
    do {                                                           \
        cudaError_t e__ = (expr);                                  \
        if (e__ != cudaSuccess) { release(); return M16_ERR_CUDA; } \
    } while (0)
    if (use_graph) M16_BT_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));

    // tuning: check intervals [k update, (k + 1) update) run candidate k,
    // timed from after their check iteration to their end
    int tune_stage = tune ? 0 : -1;
    double tune_ms[3] = {0.0, 0.0, 0.0};
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    tune_events[0] = &t0;
    tune_events[1] = &t1;
    if (tune) {
        M16_BT_TRY(cudaEventCreate(&t0));
        M16_BT_TRY(cudaEventCreate(&t1));
        if (cur_bps != kTuneBps[0]) M16_BT_TRY(configure(kTuneBps[0]));
    }
    while (it < params->num_iter && n_groups_active > 0 && !work.empty()) {
        if (tune_stage >= 0) {
            const int end = std::min(params->num_iter, it + update);
            int64_t vox = 0;   // voxels of the active groups: the work this interval does
            for (int g = 0; g < ngroups; ++g)
                if (gactive[g]) vox += hv[hg[g].vol].n * hg[g].lanes;
            for (; it < end; ++it) {
                launches += enqueue_iteration(st, (it % update) == 0, false);
                if (it % update == 0) M16_BT_TRY(cudaEventRecord(t0, st));
            }
            M16_BT_TRY(cudaEventRecord(t1, st));
            M16_BT_TRY(cudaEventSynchronize(t1));
            float ms = 0.f;
            M16_BT_TRY(cudaEventElapsedTime(&ms, t0, t1));
            tune_ms[tune_stage] = vox > 0 ? (double)ms / (double)vox : 0.0;
            ++tune_stage;
            if (tune_stage == 3) {
                int best = 0;
                for (int k = 1; k < 3; ++k)
                    if (tune_ms[k] < tune_ms[best]) best = k;
                {
                    std::lock_guard<std::mutex> lk(g_tune_mu);
                    g_tuned[tune_key] = kTuneBps[best];
                }
                tune_stage = -1;
                if (cur_bps != kTuneBps[best]) M16_BT_TRY(configure(kTuneBps[best]));
            } else {
                M16_BT_TRY(configure(kTuneBps[tune_stage]));
            }
        }
        const int end = std::min(params->num_iter, it + chunk);
        if (it >= params->num_iter) {
            // tuning ran the last iterations
        } else if (use_graph && end - it == chunk && it % update == 0) {
            // a graph holds the launch sizes and work-list segments it was
            // captured with: replay it only for the same work list
            if (gexec && graph_version != work_version) drop_graph();
            if (!gexec) {
                graph_version = work_version;
                M16_BT_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
                graph_launches = 0;
                for (int k = 0; k < chunk; ++k) graph_launches += enqueue_iteration(cap, (k % update) == 0, false);
                const cudaError_t ce = cudaStreamEndCapture(cap, &graph);
                if (ce != cudaSuccess) { release(); return M16_ERR_CUDA; }
                M16_BT_TRY(cudaGraphInstantiate(&gexec, graph, 0));
            }
            M16_BT_TRY(cudaGraphLaunch(gexec, st));
            launches += graph_launches;
            it = end;
        } else {
            for (; it < end; ++it) {
                const bool check = (it % update) == 0;
                launches += enqueue_iteration(st, check, timing);
                if (timing) {
                    M16_BT_TRY(cudaEventSynchronize(e2));
                    float a = 0.f, b = 0.f;
                    cudaEventElapsedTime(&a, e0, e1);
                    cudaEventElapsedTime(&b, e1, e2);
                    p_ms += a; ++p_n;
                    u_ms += b; ++u_n;
                }
            }
        }
        M16_BT_TRY(cudaGetLastError());
        M16_BT_TRY(cudaMemcpyAsync(hmask.data(), dmask, sizeof(unsigned) * ngroups, cudaMemcpyDeviceToHost, st));
        M16_BT_TRY(cudaStreamSynchronize(st));
        n_groups_active = 0;
        for (int g = 0; g < ngroups; ++g) {
            gactive[g] = hmask[g] != kAllLanes;
            n_groups_active += gactive[g];
        }
        // drop finished groups from the work list once they are a quarter of it
        if (n_groups_active > 0 && n_groups_active * 4 <= listed * 3) {
            build_work(work);
            listed = n_groups_active;
            M16_BT_TRY(cudaMemcpyAsync(dwork, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, st));
            drop_graph();   // the segments changed: capture again
        }
    }
    release();
#undef M16_BT_TRY
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
        stats->blocks_per_sm = cur_bps;
        stats->launches = launches;
        stats->p_launches = p_n;
        stats->u_launches = u_n;
        stats->p_ms = p_ms;
        stats->u_ms = u_ms;
    }
    return M16_OK;
}

// ---- the batch as a sequence of capture-safe steps ------------------------------
//
// m16_batch_begin prepares a batch on the stream (descriptors, set-up
// kernels, the default tile shape and a work list over every group) and
// returns a handle; m16_batch_iterate enqueues iterations and does nothing
// else -- no synchronisation, no allocation, no copies -- so a caller may
// capture it into a CUDA graph of its own; m16_batch_end scatters every
// instance's u to its output, reads the iteration counts and residuals and
// frees the handle.  Instances stop on the device at their residual bound
// (their lanes are masked); the work list is not shrunk between steps.

struct m16_batch {
    BatchRun B;
    std::vector<m16_batch_instance> inst;
    std::vector<int64_t> inst_n;    // voxels of each instance's volume
    m16_cut_params params;
    std::vector<int2> work;
    int seg[5] = {0, 0, 0, 0, 0};
    int ninst = 0;
    int iterations_run = 0;          // iterations enqueued by m16_batch_iterate
};

extern "C" int m16_batch_begin(const m16_batch_volume *vols, int32_t nvol, const m16_batch_instance *inst,
                               int32_t ninst, const m16_cut_params *params, void *workspace, size_t workspace_bytes,
                               void *stream, m16_batch **out)
{
    if (!out) return M16_ERR_BAD_ARG;
    *out = nullptr;
    if (!params || params->update < 1 || params->num_iter < 0 || !(params->cc > 0.0)) return M16_ERR_BAD_ARG;
    if (!batch_args_ok(vols, nvol, inst, ninst)) return M16_ERR_BAD_ARG;
    m16_batch *b = new m16_batch();
    b->B.P = make_plan(nvol, inst, ninst);
    b->B.L = batch_layout(vols, nvol, inst, ninst, b->B.P);
    if (!workspace || workspace_bytes < b->B.L.total || ((uintptr_t)workspace & 255)) {
        delete b;
        return M16_ERR_WORKSPACE;
    }
    b->B.ngroups = (int)b->B.P.group_insts.size();
    b->params = *params;
    b->ninst = ninst;
    b->inst.assign(inst, inst + ninst);
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    int launches = 0;
    const int r = batch_prepare(vols, nvol, inst, ninst, params, ws, st, b->B, launches);
    if (r != M16_OK) {
        delete b;
        return r;
    }
    BatchRun &B = b->B;
    for (int i = 0; i < ninst; ++i) b->inst_n.push_back(B.hv[inst[i].volume].n);
    // the default tile shape (one z-chunk over the whole launch's work)
    int64_t total_cs = 0;
    for (int v = 0; v < nvol; ++v)
        total_cs += column_slices(B.hv[v].d0, B.hv[v].d1, B.hv[v].d2) * B.P.ngroups_of_vol[v];
    const int zc = batch_zc_total(total_cs, M16_BATCH_BLOCKS_PER_SM);
    for (int v = 0; v < nvol; ++v) {
        VolDev &d = B.hv[v];
        d.zc = zc;
        d.tz = (int)div_up(d.d0, d.zc);
        // only zc..tz: the set-up kernels write the denominator on the device
        if (cudaMemcpyAsync((char *)(B.dvols + v) + offsetof(VolDev, zc), &d.zc, 4 * sizeof(int),
                            cudaMemcpyHostToDevice, st) != cudaSuccess) {
            delete b;
            return M16_ERR_CUDA;
        }
    }
    int64_t off = 0;
    for (int g = 0; g < B.ngroups; ++g) {
        const VolDev &V = B.hv[B.hg[g].vol];
        B.hg[g].part_off = off;
        B.hg[g].nparts = V.tx * V.ty * V.tz;
        off += B.hg[g].nparts;
    }
    // work list: groups with an active lane, four segments by group kind
    auto kind_of = [&](int g) { return (B.hg[g].lanes == kLanes ? 0 : 2) + (B.hg[g].has_alpha ? 0 : 1); };
    for (int k = 0; k < 4; ++k) {
        b->seg[k] = (int)b->work.size();
        for (int g = 0; g < B.ngroups; ++g) {
            if (B.hmask[g] == kAllLanes || kind_of(g) != k) continue;
            const VolDev &V = B.hv[B.hg[g].vol];
            const int ntiles = V.tx * V.ty * V.tz;
            for (int t = 0; t < ntiles; ++t) b->work.push_back(make_int2(g, t));
        }
    }
    b->seg[4] = (int)b->work.size();
    // the handle owns the host sources until the copies have run
    if (cudaMemcpyAsync(B.dgroups, B.hg.data(), sizeof(GroupDev) * B.ngroups, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        (!b->work.empty() && cudaMemcpyAsync(B.dwork, b->work.data(), sizeof(int2) * b->work.size(),
                                             cudaMemcpyHostToDevice, st) != cudaSuccess) ||
        cudaGetLastError() != cudaSuccess) {
        cudaStreamSynchronize(st);
        delete b;
        return M16_ERR_CUDA;
    }
    *out = b;
    return M16_OK;
}

extern "C" int m16_batch_iterate(m16_batch *b, int32_t count, void *stream)
{
    if (!b || count < 0) return M16_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    for (int k = 0; k < count && b->iterations_run < b->params.num_iter; ++k) {
        const bool check = (b->iterations_run % b->params.update) == 0;
        launch_iteration(b->B, b->seg, b->ninst, &b->params, st, check, nullptr, nullptr, nullptr);
        ++b->iterations_run;
    }
    M16_CUDA_TRY(cudaGetLastError());
    return M16_OK;
}

extern "C" int m16_batch_end(m16_batch *b, int32_t *iterations, double *residuals, void *stream)
{
    if (!b) return M16_ERR_BAD_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = M16_OK;
    for (int i = 0; i < b->ninst && rc == M16_OK; ++i) {
        const int blocks = (int)std::min<int64_t>(kMaxBlocks, div_up(b->inst_n[i], 256));
        bt_scatter_u_kernel<<<blocks, 256, 0, st>>>(b->B.dgroups, b->B.dinsts, i, b->inst_n[i]);
        if (cudaGetLastError() != cudaSuccess) rc = M16_ERR_CUDA;
    }
    if (rc == M16_OK &&
        (cudaMemcpyAsync(b->B.hctrl.data(), b->B.dctrl, sizeof(InstCtrl) * b->ninst, cudaMemcpyDeviceToHost, st) !=
             cudaSuccess ||
         cudaStreamSynchronize(st) != cudaSuccess))
        rc = M16_ERR_CUDA;
    if (rc == M16_OK) {
        for (int i = 0; i < b->ninst; ++i) {
            const InstCtrl &c = b->B.hctrl[i];
            // an instance that never stopped ran every iteration enqueued
            // directly or, replayed from graphs of whole check intervals, one
            // check interval per check
            const int ran = std::min(b->params.num_iter, std::max(b->iterations_run, c.n_checks * b->params.update));
            if (iterations) iterations[i] = c.stopped ? c.iterations : ran;
            if (residuals) residuals[i] = c.resid;
        }
    }
    delete b;
    return rc;
}
