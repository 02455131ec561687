// serve.cu -- continuous batching of ATV max-flow requests (m16_server_*).
//
// A request is one volume with its own solve (a one-lane group of the batched
// engine, batch_kernels.cuh).  The server holds one caller workspace: its
// tables (descriptors, control words, work list) at the front and an arena for
// the requests behind them.  Admission allocates a request's inputs, state and
// partial sums in one arena block; the inputs are uploaded on the server's copy
// stream and the set-up kernels run on the compute stream behind an event, so
// uploads overlap the iterations of resident requests.  A step runs
// params->update iterations of every resident request (one residual check, at
// the first), reads the stop mask, retires requests at the bound or at
// num_iter, and starts their u downloads on the copy stream; poll() hands out
// requests whose download has finished and returns their memory.
//
// Steps are pipelined by one: a step call enqueues the next step first and
// only then waits for the previous step's stop mask, so the device runs while
// the host retires, admits and polls.  A request that stopped in step k is
// still listed (masked, no work) in step k + 1; its slot and memory are
// reused only after the last step that lists it has been processed.
#include <cuda_runtime.h>
#include <math.h>
#include <float.h>

#include <algorithm>
#include <iterator>
#include <map>
#include <vector>

#include "batch_kernels.cuh"

namespace m16 {
namespace {

constexpr size_t kAlign = 256;
constexpr int kSetupBlocks = 4 * kSMs;

// first-fit allocator over [0, size) in 256-byte granules; adjacent free
// ranges are merged on release
class Arena {
public:
    void init(size_t size) {
        free_.clear();
        used_.clear();
        if (size >= kAlign) free_[0] = size / kAlign * kAlign;
    }
    bool alloc(size_t bytes, size_t *off) {
        bytes = align_up(std::max<size_t>(bytes, 1), kAlign);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t o = it->first, sz = it->second;
            free_.erase(it);
            if (sz > bytes) free_[o + bytes] = sz - bytes;
            used_[o] = bytes;
            *off = o;
            return true;
        }
        return false;
    }
    void release(size_t off) {
        auto u = used_.find(off);
        if (u == used_.end()) return;
        const size_t o = u->first;
        size_t sz = u->second;
        used_.erase(u);
        auto nx = free_.lower_bound(o);
        if (nx != free_.end() && o + sz == nx->first) {   // merge with the next range
            sz += nx->second;
            nx = free_.erase(nx);
        }
        if (nx != free_.begin()) {                          // and with the previous one
            auto pv = std::prev(nx);
            if (pv->first + pv->second == o) {
                pv->second += sz;
                return;
            }
        }
        free_[o] = sz;
    }
    size_t free_bytes() const {
        size_t t = 0;
        for (const auto &f : free_) t += f.second;
        return t;
    }
    size_t largest() const {
        size_t m = 0;
        for (const auto &f : free_) m = std::max(m, f.second);
        return m;
    }

private:
    std::map<size_t, size_t> free_, used_;   // offset -> size
};

// z-chunk of a request's tiles: about M16_SERVE_BLOCKS_PER_SM blocks per SM
// for the request alone, at least two slices (the sweeps load two slices at a
// time)
#ifndef M16_SERVE_BLOCKS_PER_SM
#define M16_SERVE_BLOCKS_PER_SM 4
#endif
#ifndef M16_SERVE_MIN_ZC
#define M16_SERVE_MIN_ZC 2
#endif
inline int serve_zc(int d0, int d1, int d2)
{
    const int64_t cols = div_up(d2, kBX) * div_up(d1, kBY);
    const int64_t zc = (int64_t)d0 * cols / (M16_SERVE_BLOCKS_PER_SM * kSMs);
    return (int)std::max<int64_t>(std::min<int64_t>(M16_SERVE_MIN_ZC, d0), std::min<int64_t>(32, zc));
}

// where a request's fields sit in its arena block
struct ReqLayout {
    size_t img, quat3, alpha, cs, ct, q4, state, partials, maxpart, total;
    int zc, tx, ty, tz;
    int64_t n, slab;
};

inline ReqLayout req_layout(int d0, int d1, int d2)
{
    ReqLayout R;
    const int64_t n = (int64_t)d0 * d1 * d2;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, kAlign); return o; };
    R.n = n;
    R.img = take(n * 4);
    R.quat3 = take(n * 12);
    R.alpha = take(n * 4);   // |grad I|^2, or the per-voxel alpha
    R.cs = take(n * 4);
    R.ct = take(n * 4);
    R.q4 = take(n * 16);
    R.slab = (int64_t)(align_up(n * 4, kAlign) / 4);
    R.state = take(kFields * R.slab * 4);
    R.zc = serve_zc(d0, d1, d2);
    R.tx = (int)div_up(d2, kBX);
    R.ty = (int)div_up(d1, kBY);
    R.tz = (int)div_up(d0, R.zc);
    R.partials = take((size_t)R.tx * R.ty * R.tz * 16);
    R.maxpart = take(kSetupBlocks * 4);
    R.total = off;
    return R;
}

struct Tables {
    size_t vols, groups, insts, ctrl, gmask, work, list, total;
};

inline Tables tables(int max_slots, int max_work)
{
    Tables T;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, kAlign); return o; };
    T.vols = take(sizeof(VolDev) * max_slots);
    T.groups = take(sizeof(GroupDev) * max_slots);
    T.insts = take(sizeof(InstDev) * max_slots);
    T.ctrl = take(sizeof(InstCtrl) * max_slots);
    T.gmask = take(sizeof(unsigned) * max_slots);
    T.work = take(sizeof(int2) * (size_t)max_work);
    T.list = take(sizeof(int) * max_slots);
    T.total = off;
    return T;
}

enum SlotState { kFree = 0, kResident = 1, kDraining = 2 };

struct Slot {
    int state = kFree;
    int iters_planned = 0;   // iterations of the steps enqueued so far (before any stop is known)
    int64_t last_listed = -1;   // the last step whose work list holds the slot
    int64_t tag = 0;
    size_t block = 0;        // arena offset (from the arena's base)
    size_t u_off = 0;        // workspace offset of u
    int64_t n = 0;
    int tiles = 0;
    bool alpha = false;
    int iters_done = 0;      // iterations run so far
    int iterations = 0;      // at retirement
    double resid = NAN;
    float *u_host = nullptr;
    cudaEvent_t ev = nullptr;   // draining: the u download
};

// pinned host copies of one slot's descriptors, uploaded at admission
struct Staging {
    VolDev vol;
    GroupDev group;
    InstDev inst;
    InstCtrl ctrl;
    unsigned mask;
};

}  // namespace
}  // namespace m16

using namespace m16;

struct m16_server {
    m16_cut_params params;
    cudaStream_t stream = nullptr, copy = nullptr;
    // per step parity (steps k and k + 1 are in flight together): the end of
    // the step's kernels, its stop-mask copy, and timed events around its kernels
    cudaEvent_t step_end[2] = {nullptr, nullptr}, ctrl_ev[2] = {nullptr, nullptr};
    cudaEvent_t t_start[2] = {nullptr, nullptr}, t_end[2] = {nullptr, nullptr};
    char *ws = nullptr;
    size_t ws_bytes = 0;
    int max_slots = 0, max_work = 0;
    Tables T;
    size_t arena_base = 0;
    Arena arena;
    std::vector<Slot> slots;
    std::vector<int> free_slots;
    bool dirty = true;
    // pinned host buffers
    Staging *stage = nullptr;        // max_slots
    int2 *work_h[2] = {nullptr, nullptr};   // max_work each, by rebuild parity
    int *list_h[2] = {nullptr, nullptr};    // max_slots each, by rebuild parity
    unsigned *mask_h = nullptr;      // max_slots
    InstCtrl *ctrl_h[2] = {nullptr, nullptr};   // max_slots each, by step parity
    int seg_alpha = 0, n_items = 0;  // work items: [0, seg_alpha) alpha fields, [seg_alpha, n_items) (w, decay)
    int n_list = 0;                  // slots in the current list
    int64_t rebuilds = 0;
    std::vector<int> list_cur;       // the current list (host copy)
    std::vector<int> step_list[2];   // the list of each step in flight, by step parity
    int64_t steps = 0;               // steps enqueued
    int64_t processed = 0;           // steps whose stop masks have been read (all steps < processed)
    int64_t voxel_iterations = 0;    // iterations that ran, times each request's voxels
    double gpu_ms = 0.0;             // device time of the steps' kernels
    struct Done {
        int64_t tag;
        int iterations;
        double resid;
    };
    std::vector<Done> done;          // downloaded, not yet polled (by value: the slot may be reused)
};

namespace {

void release_host(m16_server *s)
{
    if (s->stage) cudaFreeHost(s->stage);
    for (int b = 0; b < 2; ++b) {
        if (s->work_h[b]) cudaFreeHost(s->work_h[b]);
        if (s->list_h[b]) cudaFreeHost(s->list_h[b]);
        if (s->ctrl_h[b]) cudaFreeHost(s->ctrl_h[b]);
        if (s->step_end[b]) cudaEventDestroy(s->step_end[b]);
        if (s->ctrl_ev[b]) cudaEventDestroy(s->ctrl_ev[b]);
        if (s->t_start[b]) cudaEventDestroy(s->t_start[b]);
        if (s->t_end[b]) cudaEventDestroy(s->t_end[b]);
    }
    if (s->mask_h) cudaFreeHost(s->mask_h);
    for (Slot &sl : s->slots)
        if (sl.ev) cudaEventDestroy(sl.ev);
    if (s->copy) cudaStreamDestroy(s->copy);
}

// rebuild the work list and the check list over the resident slots that
// still have iterations to run.  The host sources alternate by rebuild: the
// copy from a buffer is ordered before the step enqueued after it, which has
// been processed (its stop mask read) before the buffer's next rebuild.
int rebuild(m16_server *s)
{
    const int rb = (int)(s->rebuilds & 1);
    int2 *work = s->work_h[rb];
    int *list = s->list_h[rb];
    int nw = 0, nl = 0;
    s->list_cur.clear();
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) s->seg_alpha = nw;
        for (int k = 0; k < s->max_slots; ++k) {
            const Slot &sl = s->slots[k];
            if (sl.state != kResident || sl.alpha != (pass == 0)) continue;
            if (sl.iters_planned >= s->params.num_iter) continue;   // its last step is enqueued
            if (nw + sl.tiles > s->max_work) return M16_ERR_TOO_LARGE;
            for (int t = 0; t < sl.tiles; ++t) work[nw++] = make_int2(k, t);
            list[nl++] = k;
            s->list_cur.push_back(k);
        }
    }
    s->n_items = nw;
    s->n_list = nl;
    if (nw > 0)
        M16_CUDA_TRY(cudaMemcpyAsync(s->ws + s->T.work, work, sizeof(int2) * nw, cudaMemcpyHostToDevice, s->stream));
    if (nl > 0)
        M16_CUDA_TRY(cudaMemcpyAsync(s->ws + s->T.list, list, sizeof(int) * nl, cudaMemcpyHostToDevice, s->stream));
    s->rebuilds += 1;
    s->dirty = false;
    return M16_OK;
}

// the retired slot's u goes to the host on the copy stream, after the step
// (of parity b) in which it became final
int start_download(m16_server *s, int k, int b)
{
    Slot &sl = s->slots[k];
    sl.state = kDraining;
    M16_CUDA_TRY(cudaStreamWaitEvent(s->copy, s->step_end[b], 0));
    M16_CUDA_TRY(cudaMemcpyAsync(sl.u_host, s->ws + sl.u_off, sl.n * 4, cudaMemcpyDeviceToHost, s->copy));
    M16_CUDA_TRY(cudaEventRecord(sl.ev, s->copy));
    s->dirty = true;
    return M16_OK;
}

int process_step(m16_server *s, int64_t idx);

// hand out downloaded slots and return their memory: once the download has
// finished and every step that lists the slot has been processed.  Steps
// whose stop masks have arrived are processed first (without waiting), so the
// last requests come back without another step call.
void collect(m16_server *s)
{
    while (s->processed < s->steps && cudaEventQuery(s->ctrl_ev[s->processed & 1]) == cudaSuccess)
        if (process_step(s, s->processed) != M16_OK) break;
    for (int k = 0; k < s->max_slots; ++k) {
        Slot &sl = s->slots[k];
        if (sl.state != kDraining || sl.last_listed >= s->processed) continue;
        if (cudaEventQuery(sl.ev) != cudaSuccess) continue;
        s->arena.release(sl.block);
        sl.state = kFree;
        s->free_slots.push_back(k);
        s->done.push_back({sl.tag, sl.iterations, sl.resid});
    }
}

}  // namespace

extern "C" size_t m16_server_request_bytes(int32_t d0, int32_t d1, int32_t d2, int32_t has_alpha)
{
    (void)has_alpha;   // the alpha field takes the place of |grad I|^2
    if (d0 < 1 || d1 < 1 || d2 < 1 || (int64_t)d0 * d1 * d2 > (int64_t)INT32_MAX) return 0;
    return req_layout(d0, d1, d2).total;
}

extern "C" size_t m16_server_table_bytes(int32_t max_slots, int32_t max_work_items)
{
    if (max_slots < 1 || max_work_items < 1) return 0;
    return tables(max_slots, max_work_items).total;
}

extern "C" int m16_server_create(const m16_cut_params *params, int32_t max_slots, int32_t max_work_items,
                                 void *workspace, size_t workspace_bytes, void *stream, m16_server **out)
{
    if (!out) return M16_ERR_BAD_ARG;
    *out = nullptr;
    if (!params || params->update < 1 || params->num_iter < 1 || params->num_iter % params->update != 0 ||
        !(params->cc > 0.0) || max_slots < 1 || max_work_items < 1)
        return M16_ERR_BAD_ARG;
    const Tables T = tables(max_slots, max_work_items);
    if (!workspace || ((uintptr_t)workspace & (kAlign - 1)) || workspace_bytes < T.total + kAlign)
        return M16_ERR_WORKSPACE;
    m16_server *s = new m16_server();
    s->params = *params;
    s->stream = (cudaStream_t)stream;
    s->ws = (char *)workspace;
    s->ws_bytes = workspace_bytes;
    s->max_slots = max_slots;
    s->max_work = max_work_items;
    s->T = T;
    s->arena_base = T.total;
    s->arena.init(workspace_bytes - T.total);
    s->slots.resize(max_slots);
    for (int k = max_slots - 1; k >= 0; --k) s->free_slots.push_back(k);
    bool ok = cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMallocHost((void **)&s->stage, sizeof(Staging) * max_slots) == cudaSuccess &&
              cudaMallocHost((void **)&s->mask_h, sizeof(unsigned) * max_slots) == cudaSuccess;
    for (int b = 0; ok && b < 2; ++b)
        ok = cudaEventCreateWithFlags(&s->step_end[b], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&s->ctrl_ev[b], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreate(&s->t_start[b]) == cudaSuccess && cudaEventCreate(&s->t_end[b]) == cudaSuccess &&
             cudaMallocHost((void **)&s->work_h[b], sizeof(int2) * (size_t)max_work_items) == cudaSuccess &&
             cudaMallocHost((void **)&s->list_h[b], sizeof(int) * max_slots) == cudaSuccess &&
             cudaMallocHost((void **)&s->ctrl_h[b], sizeof(InstCtrl) * max_slots) == cudaSuccess;
    for (int k = 0; ok && k < max_slots; ++k)
        ok = cudaEventCreateWithFlags(&s->slots[k].ev, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        release_host(s);
        delete s;
        return M16_ERR_CUDA;
    }
    *out = s;
    return M16_OK;
}

extern "C" int m16_server_admit(m16_server *s, const m16_serve_request *req, int32_t *admitted)
{
    if (!s || !req || !admitted) return M16_ERR_BAD_ARG;
    *admitted = 0;
    if (req->d0 < 1 || req->d1 < 1 || req->d2 < 1) return M16_ERR_BAD_SHAPE;
    if ((int64_t)req->d0 * req->d1 * req->d2 > (int64_t)INT32_MAX) return M16_ERR_BAD_SHAPE;
    if (!req->img || !req->quat3 || !req->cs || !req->ct || !req->u) return M16_ERR_BAD_ARG;
    if (!req->alpha && (!req->grad2 || !(req->decay != 0.0))) return M16_ERR_BAD_ARG;
    for (int k = 0; k < 3; ++k)
        if (!(req->scaling[k] > 0.0) || !(req->sqevals[k] > 0.0)) return M16_ERR_BAD_ARG;
    collect(s);
    if (s->free_slots.empty()) return M16_OK;
    const ReqLayout R = req_layout(req->d0, req->d1, req->d2);
    if (R.tx * R.ty * R.tz > s->max_work) return M16_ERR_TOO_LARGE;
    size_t block;
    if (!s->arena.alloc(R.total, &block)) return M16_OK;
    const int k = s->free_slots.back();
    s->free_slots.pop_back();
    Slot &sl = s->slots[k];
    char *base = s->ws + s->arena_base + block;
    const int64_t n = R.n;
    cudaStream_t cp = s->copy, st = s->stream;

    // inputs on the copy stream
    M16_CUDA_TRY(cudaMemcpyAsync(base + R.img, req->img, n * 4, cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaMemcpyAsync(base + R.quat3, req->quat3, n * 12, cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaMemcpyAsync(base + R.alpha, req->alpha ? req->alpha : req->grad2, n * 4,
                                 cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaMemcpyAsync(base + R.cs, req->cs, n * 4, cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaMemcpyAsync(base + R.ct, req->ct, n * 4, cudaMemcpyHostToDevice, cp));

    // descriptors (staged in pinned memory, uploaded on the copy stream too)
    Staging &S = s->stage[k];
    VolDev &v = S.vol;
    const double *sc = req->scaling;
    const double smin = fmin(sc[0], fmin(sc[1], sc[2]));
    const m16_cut_params &p = s->params;
    v.d0 = req->d0; v.d1 = req->d1; v.d2 = req->d2;
    v.zc = R.zc; v.tx = R.tx; v.ty = R.ty; v.tz = R.tz; v.pad = 0;
    v.rcc = (float)(1.0 / (p.cc * (smin * smin)));
    v.rs0 = (float)(1.0 / sc[0]); v.rs1 = (float)(1.0 / sc[1]); v.rs2 = (float)(1.0 / sc[2]);
    v.ss0 = (float)(p.steps / sc[0] * (smin * smin));
    v.ss1 = (float)(p.steps / sc[1] * (smin * smin));
    v.ss2 = (float)(p.steps / sc[2] * (smin * smin));
    v.denom = 1.f;
    v.q4 = (const float4 *)(base + R.q4);
    v.grad2 = req->alpha ? nullptr : (const float *)(base + R.alpha);
    v.cs = (const float *)(base + R.cs);
    v.ct = (const float *)(base + R.ct);
    v.n = n;
    GroupDev &g = S.group;
    g.part_off = (int64_t)((s->arena_base + block + R.partials) / 16);
    g.vol = k;
    g.nparts = R.tx * R.ty * R.tz;
    g.has_alpha = req->alpha ? 1 : 0;
    g.lanes = 1;
    g.pad0 = g.pad1 = g.pad2 = 0;
    g.w = make_float4((float)req->weighting, 0.f, 0.f, 0.f);
    g.nid2 = make_float4(req->alpha ? 0.f : (float)(-1.0 / (req->decay * req->decay)), 0.f, 0.f, 0.f);
    g.sq0 = (float)req->sqevals[0]; g.sq1 = (float)req->sqevals[1]; g.sq2 = (float)req->sqevals[2];
    g.isq0 = (float)(1.0 / req->sqevals[0]); g.isq1 = (float)(1.0 / req->sqevals[1]);
    g.isq2 = (float)(1.0 / req->sqevals[2]);
    g.state = base + R.state;
    g.slab = R.slab;
    g.alpha1 = req->alpha ? (const float *)(base + R.alpha) : nullptr;
    S.inst.group = k;
    S.inst.lane = 0;
    S.inst.u_out = nullptr;
    S.inst.alpha = g.alpha1;
    S.ctrl.stopped = 0;
    S.ctrl.iterations = p.num_iter;
    S.ctrl.n_checks = 0;
    S.ctrl.pad = 0;
    S.ctrl.resid = NAN;
    S.mask = kAllLanes & ~1u;   // lanes 1..3 do not exist
    M16_CUDA_TRY(cudaMemcpyAsync(s->ws + s->T.vols + sizeof(VolDev) * k, &S.vol, sizeof(VolDev),
                                 cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaMemcpyAsync(s->ws + s->T.groups + sizeof(GroupDev) * k, &S.group, sizeof(GroupDev),
                                 cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaMemcpyAsync(s->ws + s->T.insts + sizeof(InstDev) * k, &S.inst, sizeof(InstDev),
                                 cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaMemcpyAsync(s->ws + s->T.ctrl + sizeof(InstCtrl) * k, &S.ctrl, sizeof(InstCtrl),
                                 cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaMemcpyAsync(s->ws + s->T.gmask + sizeof(unsigned) * k, &S.mask, sizeof(unsigned),
                                 cudaMemcpyHostToDevice, cp));
    M16_CUDA_TRY(cudaEventRecord(sl.ev, cp));

    // set-up on the compute stream once the uploads are in
    M16_CUDA_TRY(cudaStreamWaitEvent(st, sl.ev, 0));
    VolDev *dvols = (VolDev *)(s->ws + s->T.vols);
    const GroupDev *dgroups = (const GroupDev *)(s->ws + s->T.groups);
    const int blocks = (int)std::min<int64_t>(kSetupBlocks, div_up(n, 256));
    float *mp = (float *)(base + R.maxpart);
    bt_max_kernel<<<blocks, 256, 0, st>>>((const float *)(base + R.img), n, mp);
    bt_denom_kernel<<<1, 32, 0, st>>>(mp, blocks, dvols + k);
    bt_expand_kernel<<<blocks, 256, 0, st>>>((const float *)(base + R.quat3), (float4 *)(base + R.q4), n);
    bt_init_group_kernel<<<blocks, 256, 0, st>>>((const float *)(base + R.img), dvols, dgroups, k);
    M16_CUDA_TRY(cudaGetLastError());

    sl.state = kResident;
    sl.tag = req->tag;
    sl.block = block;
    sl.u_off = s->arena_base + block + R.state + (size_t)5 * R.slab * 4;
    sl.n = n;
    sl.tiles = R.tx * R.ty * R.tz;
    sl.alpha = req->alpha != nullptr;
    sl.iters_done = 0;
    sl.iters_planned = 0;
    sl.last_listed = -1;
    sl.iterations = 0;
    sl.resid = NAN;
    sl.u_host = req->u;
    s->dirty = true;
    *admitted = 1;
    return M16_OK;
}

namespace {

// read the stop mask of step idx (enqueued, not yet processed) and retire the
// requests that stopped in it or ran their last iteration in it
int process_step(m16_server *s, int64_t idx)
{
    if (idx != s->processed) return M16_ERR_BAD_ARG;   // in order only
    const int b = (int)(idx & 1);
    M16_CUDA_TRY(cudaEventSynchronize(s->ctrl_ev[b]));
    float step_ms = 0.f;
    M16_CUDA_TRY(cudaEventElapsedTime(&step_ms, s->t_start[b], s->t_end[b]));
    s->gpu_ms += step_ms;
    for (int k : s->step_list[b]) {
        Slot &sl = s->slots[k];
        if (sl.state != kResident) continue;   // retired after an earlier step: masked here
        const InstCtrl &c = s->ctrl_h[b][k];
        sl.resid = c.resid;
        // a request that stopped at this step's check ran that one iteration
        s->voxel_iterations += sl.n * (c.stopped ? std::max(0, c.iterations - sl.iters_done) : s->params.update);
        if (c.stopped) {
            sl.iterations = c.iterations;
        } else {
            sl.iters_done += s->params.update;
            if (sl.iters_done < s->params.num_iter) continue;
            sl.iterations = s->params.num_iter;
        }
        const int r = start_download(s, k, b);
        if (r != M16_OK) return r;
    }
    s->processed = idx + 1;
    return M16_OK;
}

}  // namespace

extern "C" int m16_server_step(m16_server *s)
{
    if (!s) return M16_ERR_BAD_ARG;
    collect(s);
    if (s->dirty) {
        const int r = rebuild(s);
        if (r != M16_OK) return r;
    }
    const bool enqueue = s->n_list > 0;
    if (enqueue) {
        cudaStream_t st = s->stream;
        const int64_t c = s->steps;
        const int b = (int)(c & 1);   // step c - 2 of this parity has been processed
        const VolDev *dvols = (const VolDev *)(s->ws + s->T.vols);
        const GroupDev *dgroups = (const GroupDev *)(s->ws + s->T.groups);
        const InstDev *dinsts = (const InstDev *)(s->ws + s->T.insts);
        InstCtrl *dctrl = (InstCtrl *)(s->ws + s->T.ctrl);
        unsigned *dmask = (unsigned *)(s->ws + s->T.gmask);
        const int2 *dwork = (const int2 *)(s->ws + s->T.work);
        const int *dlist = (const int *)(s->ws + s->T.list);
        float4 *dpart = (float4 *)s->ws;   // part_off counts float4 from the workspace start
        const dim3 block(kBX, kBY, 1);
        const int na = s->seg_alpha, ne = s->n_items - s->seg_alpha;
        M16_CUDA_TRY(cudaEventRecord(s->t_start[b], st));
        // programmatic dependent launch between the sweeps (common.cuh); the
        // first sweep follows an event record and launches in stream order
        for (int i = 0; i < s->params.update; ++i) {
            if (na > 0) M16_CUDA_TRY(launch_pdl(bt1_flow_kernel<kAlphaArray>, dim3(na), block, st, true, dwork, dvols,
                                                dgroups, (const unsigned *)dmask));
            if (ne > 0) M16_CUDA_TRY(launch_pdl(bt1_flow_kernel<kAlphaFromGrad2>, dim3(ne), block, st, true,
                                                dwork + na, dvols, dgroups, (const unsigned *)dmask));
            if (i == 0) {
                M16_CUDA_TRY(launch_pdl(bt1_label_kernel<true>, dim3(s->n_items), block, st, true, dwork, dvols,
                                        dgroups, (const unsigned *)dmask, dpart));
                M16_CUDA_TRY(launch_pdl(bt_check_kernel, dim3(s->n_list), dim3(256), st, true, dvols, dgroups,
                                        dinsts, dctrl, dmask, (const float4 *)dpart, s->params.error_bound,
                                        s->params.update, dlist));
            } else {
                M16_CUDA_TRY(launch_pdl(bt1_label_kernel<false>, dim3(s->n_items), block, st, true, dwork, dvols,
                                        dgroups, (const unsigned *)dmask, dpart));
            }
        }
        M16_CUDA_TRY(cudaGetLastError());
        M16_CUDA_TRY(cudaEventRecord(s->t_end[b], st));
        M16_CUDA_TRY(cudaEventRecord(s->step_end[b], st));
        M16_CUDA_TRY(cudaMemcpyAsync(s->ctrl_h[b], dctrl, sizeof(InstCtrl) * s->max_slots, cudaMemcpyDeviceToHost,
                                     st));
        M16_CUDA_TRY(cudaEventRecord(s->ctrl_ev[b], st));
        s->step_list[b] = s->list_cur;
        for (int k : s->list_cur) {
            Slot &sl = s->slots[k];
            sl.iters_planned += s->params.update;
            sl.last_listed = c;
            if (sl.iters_planned >= s->params.num_iter) s->dirty = true;   // out of the next list
        }
        s->steps = c + 1;
    }
    // the steps before the one just enqueued (all of them when none was)
    const int64_t upto = enqueue ? s->steps - 1 : s->steps;
    while (s->processed < upto) {
        const int r = process_step(s, s->processed);
        if (r != M16_OK) return r;
    }
    return M16_OK;
}

extern "C" int m16_server_poll(m16_server *s, int64_t *tags, int32_t *iterations, double *residuals, int32_t cap,
                               int32_t *n)
{
    if (!s || !n || cap < 0 || (cap > 0 && !tags)) return M16_ERR_BAD_ARG;
    collect(s);
    const int cnt = std::min<int>(cap, (int)s->done.size());
    for (int j = 0; j < cnt; ++j) {
        tags[j] = s->done[j].tag;
        if (iterations) iterations[j] = s->done[j].iterations;
        if (residuals) residuals[j] = s->done[j].resid;
    }
    s->done.erase(s->done.begin(), s->done.begin() + cnt);
    *n = cnt;
    return M16_OK;
}

extern "C" int m16_server_get_info(const m16_server *s, m16_server_info *info)
{
    if (!s || !info) return M16_ERR_BAD_ARG;
    int res = 0, dr = 0;
    for (const Slot &sl : s->slots) {
        res += sl.state == kResident;
        dr += sl.state == kDraining;
    }
    info->resident = res;
    info->draining = dr;
    info->free_slots = (int32_t)s->free_slots.size();
    info->reserved = 0;
    info->free_bytes = (int64_t)s->arena.free_bytes();
    info->largest_free = (int64_t)s->arena.largest();
    info->steps = s->steps;
    info->voxel_iterations = s->voxel_iterations;
    info->gpu_ms = s->gpu_ms;
    return M16_OK;
}

extern "C" int m16_server_destroy(m16_server *s)
{
    if (!s) return M16_ERR_BAD_ARG;
    cudaError_t e1 = cudaStreamSynchronize(s->stream);
    cudaError_t e2 = s->copy ? cudaStreamSynchronize(s->copy) : cudaSuccess;
    release_host(s);
    delete s;
    return (e1 == cudaSuccess && e2 == cudaSuccess) ? M16_OK : M16_ERR_CUDA;
}
