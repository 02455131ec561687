// batched.cu -- many ATV max-flow solves in one launch per sweep.
//
// The reference runs its (weighting, decay) grid search as one
// CmfCutQAnisotropicGpu.execute() per grid point and cut type
// (src/phantom_experiment.py:350-368), each with three launches per iteration
// and a blocking residual read every `update` iterations.  Here a batch of
// instances -- any mix of volumes, weightings, decays and eigenvalue sets --
// advances together: every flow (P) and label (U) launch covers all active
// instances, the residual check of every instance is one block of one launch,
// and an instance stops on its own at its threshold (its later blocks return
// at once).  Instances of one volume share its quaternions, |grad I|^2 and
// capacities; the work list orders blocks tile-major so those shared tiles are
// read from L2 by every instance that uses them.  The projection radius of an
// instance is computed in the flow sweep as w * exp(-|grad I|^2 / decay^2)
// (phantom_experiment.py:359), so the per-instance state is all that streams
// from HBM: hp (3 floats), p_t, u, tmp.
#include <cuda_runtime.h>
#include <math.h>
#include <float.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "sweeps.cuh"

namespace m16 {
namespace {

constexpr int kBX = 32, kBY = 8;

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

struct InstDev {
    int vol, part_off, nparts, pad;
    float w, neg_inv_decay2;
    float sq0, sq1, sq2, isq0, isq1, isq2;
    const float *alpha;
    float *hp0, *hp1, *hp2, *pt, *tmp, *u;
    InstCtrl *ctrl;
};

inline int batch_zc(int d0, int d1, int d2)
{
    const int64_t cols = div_up(d2, kBX) * div_up(d1, kBY);
    int64_t zc = (int64_t)d0 * cols / (8 * kSMs);
    zc = std::max<int64_t>(1, std::min<int64_t>(16, zc));
    if (zc >= kMfZB) zc = zc / kMfZB * kMfZB;
    return (int)zc;
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

// hp = 0, p_t = fmin(cs, ct), u = img / denom, tmp = -u * rcc (continuous_cut_anisotropic_gpu.py:276-289)
__global__ void bt_init_inst_kernel(const float *__restrict__ img, const VolDev *vols, const InstDev *insts, int inst,
                                    int num_iter)
{
    const InstDev I = insts[inst];
    const VolDev &V = vols[I.vol];
    const float denom = V.denom;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < V.n; i += (int64_t)gridDim.x * blockDim.x) {
        I.hp0[i] = 0.f;
        I.hp1[i] = 0.f;
        I.hp2[i] = 0.f;
        I.pt[i] = fminf(V.cs[i], V.ct[i]);
        const float ui = img[i] / denom;
        I.u[i] = ui;
        I.tmp[i] = -(ui * V.rcc);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        I.ctrl->stopped = 0;
        I.ctrl->iterations = num_iter;
        I.ctrl->n_checks = 0;
        I.ctrl->resid = NAN;
    }
}

// ---- sweeps over the work list ----------------------------------------------------

__device__ __forceinline__ void decode_tile(const VolDev &V, int tile, int &bx, int &by, int &bz)
{
    bx = tile % V.tx;
    by = (tile / V.tx) % V.ty;
    bz = tile / (V.tx * V.ty);
}

__global__ void __launch_bounds__(kBX * kBY) bt_flow_kernel(const int2 *__restrict__ work, const VolDev *vols,
                                                            const InstDev *insts)
{
    const int2 wk = work[blockIdx.x];
    const InstDev &I = insts[wk.x];
    if (__ldcg(&I.ctrl->stopped)) return;
    const VolDev &V = vols[I.vol];
    int bx, by, bz;
    decode_tile(V, wk.y, bx, by, bz);
    const int x = bx * kBX + threadIdx.x, y = by * kBY + threadIdx.y;
    if (x >= V.d2 || y >= V.d1) return;
    const int z0 = bz * V.zc, z1 = min(z0 + V.zc, V.d0);
    FlowView f;
    f.d0 = V.d0; f.d1 = V.d1; f.d2 = V.d2;
    f.ss0 = V.ss0; f.ss1 = V.ss1; f.ss2 = V.ss2;
    f.sq0 = I.sq0; f.sq1 = I.sq1; f.sq2 = I.sq2; f.isq0 = I.isq0; f.isq1 = I.isq1; f.isq2 = I.isq2;
    f.alpha_scalar = 0.f; f.alpha = I.alpha; f.grad2 = V.grad2; f.w = I.w; f.neg_inv_decay2 = I.neg_inv_decay2;
    f.sqeigs = nullptr; f.q4 = V.q4; f.tmp = I.tmp; f.hp0 = I.hp0; f.hp1 = I.hp1; f.hp2 = I.hp2;
    if (I.alpha) flow_column<false, kAlphaArray>(f, x, y, z0, z1);
    else flow_column<false, kAlphaFromGrad2>(f, x, y, z0, z1);
}

template <bool CHECK>
__global__ void __launch_bounds__(kBX * kBY) bt_label_kernel(const int2 *__restrict__ work, const VolDev *vols,
                                                             const InstDev *insts, float *__restrict__ partials)
{
    __shared__ float red[32];
    const int2 wk = work[blockIdx.x];
    const InstDev &I = insts[wk.x];
    if (__ldcg(&I.ctrl->stopped)) return;
    const VolDev &V = vols[I.vol];
    int bx, by, bz;
    decode_tile(V, wk.y, bx, by, bz);
    const int x = bx * kBX + threadIdx.x, y = by * kBY + threadIdx.y;
    float acc = 0.f;
    if (x < V.d2 && y < V.d1) {
        LabelView l;
        l.d0 = V.d0; l.d1 = V.d1; l.d2 = V.d2;
        l.rcc = V.rcc; l.rs0 = V.rs0; l.rs1 = V.rs1; l.rs2 = V.rs2;
        l.hp0 = I.hp0; l.hp1 = I.hp1; l.hp2 = I.hp2; l.cs = V.cs; l.ct = V.ct; l.labels = nullptr;
        l.pt = I.pt; l.u = I.u; l.tmp = I.tmp;
        const int z0 = bz * V.zc;
        acc = label_column<false>(l, x, y, z0, min(z0 + V.zc, V.d0));
    }
    if (CHECK) {
        const float s = block_sum(acc, red);
        if (threadIdx.x == 0 && threadIdx.y == 0) partials[I.part_off + wk.y] = s;
    }
}

// one block per instance: residual = sum(partials) / (N * rcc)
__global__ void bt_check_kernel(const VolDev *vols, const InstDev *insts, const float *__restrict__ partials,
                                double bound, int iter)
{
    __shared__ double s[256];
    const InstDev &I = insts[blockIdx.x];
    if (__ldcg(&I.ctrl->stopped)) return;
    const VolDev &V = vols[I.vol];
    double acc = 0.0;
    for (int k = threadIdx.x; k < I.nparts; k += blockDim.x) acc += (double)partials[I.part_off + k];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double err = s[0] / ((double)V.n * (double)V.rcc);
        I.ctrl->resid = err;
        I.ctrl->n_checks += 1;
        if (isnan(err) || err < bound) {
            I.ctrl->stopped = 1;
            I.ctrl->iterations = iter + 1;
        }
    }
}

struct BatchLayout {
    std::vector<size_t> q4, maxpart;        // per volume
    std::vector<size_t> state;              // per instance: hp0 hp1 hp2 pt tmp
    size_t ctrl;                            // InstCtrl[ninst], contiguous
    std::vector<int> part_off, nparts;      // per instance
    size_t vols, insts, work, partials, total;
    int64_t total_blocks, total_parts;
};

constexpr int kMaxBlocks = 4 * kSMs;

inline BatchLayout batch_layout(const m16_batch_volume *vols, int nvol, const m16_batch_instance *inst, int ninst)
{
    BatchLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    std::vector<int64_t> tiles(nvol);
    for (int v = 0; v < nvol; ++v) {
        const int64_t n = (int64_t)vols[v].d0 * vols[v].d1 * vols[v].d2;
        L.q4.push_back(take(n * 16));
        L.maxpart.push_back(take(kMaxBlocks * 4));
        const int zc = batch_zc(vols[v].d0, vols[v].d1, vols[v].d2);
        tiles[v] = div_up(vols[v].d2, kBX) * div_up(vols[v].d1, kBY) * div_up(vols[v].d0, zc);
    }
    L.total_blocks = 0;
    L.total_parts = 0;
    for (int i = 0; i < ninst; ++i) {
        const m16_batch_volume &V = vols[inst[i].volume];
        const int64_t n = (int64_t)V.d0 * V.d1 * V.d2;
        L.state.push_back(take(5 * align_up(n * 4, 256)));
        L.part_off.push_back((int)L.total_parts);
        L.nparts.push_back((int)tiles[inst[i].volume]);
        L.total_parts += tiles[inst[i].volume];
        L.total_blocks += tiles[inst[i].volume];
    }
    L.ctrl = take(sizeof(InstCtrl) * std::max(ninst, 1));
    L.vols = take(sizeof(VolDev) * std::max(nvol, 1));
    L.insts = take(sizeof(InstDev) * std::max(ninst, 1));
    L.work = take(sizeof(int2) * std::max<int64_t>(L.total_blocks, 1));
    L.partials = take(4 * std::max<int64_t>(L.total_parts, 1));
    L.total = off;
    return L;
}

bool batch_args_ok(const m16_batch_volume *vols, int nvol, const m16_batch_instance *inst, int ninst)
{
    if (!vols || !inst || nvol < 1 || ninst < 1) return false;
    for (int v = 0; v < nvol; ++v) {
        const m16_batch_volume &V = vols[v];
        if (V.d0 < 1 || V.d1 < 1 || V.d2 < 1 || !V.img || !V.quat3 || !V.cs || !V.ct) return false;
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
    return batch_layout(vols, nvol, inst, ninst).total;
}

extern "C" int m16_batch_solve(const m16_batch_volume *vols, int32_t nvol, const m16_batch_instance *inst,
                               int32_t ninst, const m16_cut_params *params, int32_t *iterations, double *residuals,
                               void *workspace, size_t workspace_bytes, void *stream, m16_solve_stats *stats)
{
    if (!params || params->update < 1 || params->num_iter < 0 || !(params->cc > 0.0)) return M16_ERR_BAD_ARG;
    if (!batch_args_ok(vols, nvol, inst, ninst)) return M16_ERR_BAD_ARG;
    const BatchLayout L = batch_layout(vols, nvol, inst, ninst);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255)) return M16_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;

    // device descriptors
    std::vector<VolDev> hv(nvol);
    for (int v = 0; v < nvol; ++v) {
        const m16_batch_volume &V = vols[v];
        VolDev &d = hv[v];
        d.d0 = V.d0; d.d1 = V.d1; d.d2 = V.d2;
        d.zc = batch_zc(V.d0, V.d1, V.d2);
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
    std::vector<InstDev> hi(ninst);
    for (int i = 0; i < ninst; ++i) {
        const m16_batch_instance &I = inst[i];
        InstDev &d = hi[i];
        const int64_t n = hv[I.volume].n;
        const size_t slab = align_up(n * 4, 256);
        d.vol = I.volume;
        d.part_off = L.part_off[i];
        d.nparts = L.nparts[i];
        d.w = (float)I.weighting;
        d.neg_inv_decay2 = I.alpha ? 0.f : (float)(-1.0 / (I.decay * I.decay));
        d.sq0 = (float)I.sqevals[0]; d.sq1 = (float)I.sqevals[1]; d.sq2 = (float)I.sqevals[2];
        d.isq0 = (float)(1.0 / I.sqevals[0]); d.isq1 = (float)(1.0 / I.sqevals[1]);
        d.isq2 = (float)(1.0 / I.sqevals[2]);
        d.alpha = I.alpha;
        char *base = ws + L.state[i];
        d.hp0 = (float *)base; d.hp1 = (float *)(base + slab); d.hp2 = (float *)(base + 2 * slab);
        d.pt = (float *)(base + 3 * slab); d.tmp = (float *)(base + 4 * slab);
        d.u = I.u;
        d.ctrl = (InstCtrl *)(ws + L.ctrl) + i;
    }
    VolDev *dvols = (VolDev *)(ws + L.vols);
    InstDev *dinsts = (InstDev *)(ws + L.insts);
    int2 *dwork = (int2 *)(ws + L.work);
    float *dpart = (float *)(ws + L.partials);
    M16_CUDA_TRY(cudaMemcpyAsync(dvols, hv.data(), sizeof(VolDev) * nvol, cudaMemcpyHostToDevice, st));
    M16_CUDA_TRY(cudaMemcpyAsync(dinsts, hi.data(), sizeof(InstDev) * ninst, cudaMemcpyHostToDevice, st));

    // per-volume set-up, then per-instance state
    int launches = 0;
    for (int v = 0; v < nvol; ++v) {
        const int blocks = (int)std::min<int64_t>(kMaxBlocks, div_up(hv[v].n, 256));
        float *mp = (float *)(ws + L.maxpart[v]);
        bt_max_kernel<<<blocks, 256, 0, st>>>(vols[v].img, hv[v].n, mp);
        bt_denom_kernel<<<1, 32, 0, st>>>(mp, blocks, dvols + v);
        bt_expand_kernel<<<blocks, 256, 0, st>>>(vols[v].quat3, (float4 *)(ws + L.q4[v]), hv[v].n);
        launches += 3;
    }
    for (int i = 0; i < ninst; ++i) {
        const int blocks = (int)std::min<int64_t>(kMaxBlocks, div_up(hv[hi[i].vol].n, 256));
        bt_init_inst_kernel<<<blocks, 256, 0, st>>>(vols[hi[i].vol].img, dvols, dinsts, i, params->num_iter);
        ++launches;
    }
    M16_CUDA_TRY(cudaGetLastError());

    // the work list: per volume, per tile, every instance of that volume
    std::vector<std::vector<int>> by_vol(nvol);
    std::vector<char> active(ninst, 1);
    int listed = 0;   // instances in the current work list
    auto build_work = [&](std::vector<int2> &w) {
        w.clear();
        for (auto &b : by_vol) b.clear();
        listed = 0;
        for (int i = 0; i < ninst; ++i)
            if (active[i]) { by_vol[hi[i].vol].push_back(i); ++listed; }
        for (int v = 0; v < nvol; ++v) {
            const int ntiles = hv[v].tx * hv[v].ty * hv[v].tz;
            for (int t = 0; t < ntiles; ++t)
                for (int i : by_vol[v]) w.push_back(make_int2(i, t));
        }
    };
    std::vector<int2> work;
    build_work(work);
    M16_CUDA_TRY(cudaMemcpyAsync(dwork, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, st));

    const int update = params->update;
    const int chunk = update * std::max(1, 64 / update);
    std::vector<InstCtrl> hctrl(ninst);
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
    int n_active = ninst;
    while (it < params->num_iter && n_active > 0) {
        const int end = std::min(params->num_iter, it + chunk);
        const unsigned nblocks = (unsigned)work.size();
        for (; it < end; ++it) {
            if (timing) cudaEventRecord(e0, st);
            bt_flow_kernel<<<nblocks, dim3(kBX, kBY, 1), 0, st>>>(dwork, dvols, dinsts);
            if (timing) cudaEventRecord(e1, st);
            const bool check = (it % update) == 0;
            if (check) bt_label_kernel<true><<<nblocks, dim3(kBX, kBY, 1), 0, st>>>(dwork, dvols, dinsts, dpart);
            else bt_label_kernel<false><<<nblocks, dim3(kBX, kBY, 1), 0, st>>>(dwork, dvols, dinsts, dpart);
            if (timing) {
                cudaEventRecord(e2, st);
                M16_CUDA_TRY(cudaEventSynchronize(e2));
                float a = 0.f, b = 0.f;
                cudaEventElapsedTime(&a, e0, e1);
                cudaEventElapsedTime(&b, e1, e2);
                p_ms += a; u_ms += b; ++p_n; ++u_n;
            }
            if (check) {
                bt_check_kernel<<<ninst, 256, 0, st>>>(dvols, dinsts, dpart, params->error_bound, it);
                ++launches;
            }
            launches += 2;
        }
        M16_CUDA_TRY(cudaGetLastError());
        InstCtrl *dctrl = (InstCtrl *)(ws + L.ctrl);
        M16_CUDA_TRY(cudaMemcpyAsync(hctrl.data(), dctrl, sizeof(InstCtrl) * ninst, cudaMemcpyDeviceToHost, st));
        M16_CUDA_TRY(cudaStreamSynchronize(st));
        n_active = 0;
        for (int i = 0; i < ninst; ++i) {
            active[i] = hctrl[i].stopped ? 0 : 1;
            n_active += active[i];
        }
        // drop finished instances from the work list once they are a quarter of it
        if (n_active > 0 && n_active * 4 <= listed * 3) {
            build_work(work);
            M16_CUDA_TRY(cudaMemcpyAsync(dwork, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, st));
        }
    }
    if (timing) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(e2);
    }
    M16_CUDA_TRY(cudaMemcpyAsync(hctrl.data(), (InstCtrl *)(ws + L.ctrl), sizeof(InstCtrl) * ninst,
                                 cudaMemcpyDeviceToHost, st));
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
