// Request server: single-step requests against resident cloths, continuous
// batching on one GPU.
//
// The reference steps one cloth per call on the host thread
// (cBaseCloth::Update -> cBaraffClothGpu::UpdatePos, src/sim/cloth/BaseCloth.cpp,
// src/sim/cloth/BaraffClothGpu.cpp:203-262).  Here a worker thread keeps the
// GPU busy with chunks.  One chunk is one CUDA graph launch:
//
//   k_srv_admit   descriptors of the requests admitted for this chunk (their
//                 per-solve arrays now point into the pool)
//   k_pins, k_tri, k_row         assembly and PCG start of those requests only
//   k_srv_begin   admitted-and-iterating count, chunk iteration budget
//   while (any iterating && budget left) { 1, 2 or 4 x (k_spmv; k_reduce; k_update; k_reduce) }   over every
//                 request on the GPU (finished ones skip their tiles)
//   k_advance     x_pre = x, x += dx for requests whose solve ended
//   k_srv_status  one record per request on the GPU; ended ones are closed
//
// Up to two chunks are in flight: while chunk k runs, the host reads the
// status of chunk k-1, retires the requests that ended (their pool memory is
// free again, the cloth's next request becomes ready) and admits ready
// requests in arrival order into chunk k+1 while a slot and pool memory are
// free.  A request that ended in chunk k-1 is still in chunk k's lists but
// inactive there: no kernel touches its per-solve arrays, so its pool range
// may be handed to a request of chunk k+1 (stream order keeps them apart).
//
// Per-instance arithmetic is the graph-loop solver's (exact fixed-point sums
// per instance), so a request's result does not depend on what else is in the
// chunk: it is bit-identical to stepping the cloth alone.
#include "internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <set>
#include <thread>

using namespace cloth;
using namespace cloth::detail;

namespace {

int sfail(int code, const std::string &msg)
{
    set_last_error(msg);
    return code;
}

#define SCK(call)                                                              \
    do                                                                         \
    {                                                                          \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                 \
            return sfail(CLOTH_ERR_CUDA,                                       \
                         std::string(#call) + ": " + cudaGetErrorString(e_));  \
    } while (0)

// Control words of one chunk; the host writes the first eight, the device
// keeps iters_left.
struct SrvCtl
{
    int n_admit;     // admission records
    int n_new;       // cloths assembled in this chunk (= n_admit)
    int n_inflight;  // cloths on the GPU (status records)
    int chunk_iters;
    int n_new_rt, n_new_tt, n_act_rt, pad;
    int iters_left;
    int pad2[3];
};
constexpr size_t kSrvHostBytes = 8 * sizeof(int);

struct __align__(16) AdmitRec
{
    int id;
    int pad[3];
    InstDesc desc;
};

struct SrvStatus
{
    int id;
    int done;
    int status;
    int iter;
    double rr, bb;
};

__global__ void k_srv_admit(const AdmitRec *recs, const SrvCtl *sc, InstDesc *table,
                            BatchCtl *ctl_new, BatchCtl *ctl_act)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        ctl_new->n_tiles_rows = sc->n_new_rt;
        ctl_new->n_tiles_tris = sc->n_new_tt;
        ctl_act->n_tiles_rows = sc->n_act_rt;
    }
    constexpr int W = int(sizeof(InstDesc) / sizeof(unsigned));
    static_assert(sizeof(InstDesc) % sizeof(unsigned) == 0, "descriptor size");
    const int n = sc->n_admit;
    for (int i = blockIdx.x; i < n; i += gridDim.x)
    {
        const unsigned *src = reinterpret_cast<const unsigned *>(&recs[i].desc);
        unsigned *dst = reinterpret_cast<unsigned *>(&table[recs[i].id]);
        for (int k = threadIdx.x; k < W; k += blockDim.x)
            dst[k] = src[k];
    }
}

__global__ void k_srv_begin(BatchCtl *ctl_new, BatchCtl *ctl_act, SrvCtl *sc,
                            cudaGraphConditionalHandle h)
{
    ctl_act->n_active += ctl_new->n_active;
    ctl_new->n_active = 0;
    sc->iters_left = sc->chunk_iters;
    cudaGraphSetConditional(h, (ctl_act->n_active > 0 && sc->chunk_iters > 0) ? 1u : 0u);
}

__global__ void k_srv_status(InstDesc *const *descs, const int *ids, const SrvCtl *sc,
                             SrvStatus *out)
{
    const int n = sc->n_inflight;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int id = ids[i];
        InstState *st = descs[id]->st;
        const int done = (!st->active && st->open) ? 1 : 0;
        SrvStatus o;
        o.id = id;
        o.done = done;
        o.status = st->status;
        o.iter = st->iter;
        o.rr = st->rr;
        o.bb = st->bb;
        out[i] = o;
        if (done)
            st->open = 0;
    }
}

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over [0, size) in 256-byte units.
struct PoolAlloc
{
    std::map<size_t, size_t> free_; // offset -> bytes
    size_t size = 0, used = 0, peak = 0;
    void reset(size_t n)
    {
        free_.clear();
        size = n;
        used = peak = 0;
        if (n)
            free_[0] = n;
    }
    bool take(size_t n, size_t *off)
    {
        n = align_up(n, 256);
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= n)
            {
                *off = it->first;
                size_t rest = it->second - n, o = it->first + n;
                free_.erase(it);
                if (rest)
                    free_[o] = rest;
                used += n;
                peak = std::max(peak, used);
                return true;
            }
        return false;
    }
    void give(size_t off, size_t n)
    {
        n = align_up(n, 256);
        used -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first)
        {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin())
        {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first)
            {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct Req
{
    long long tag;
    long long seq;
    double t_arrival;
};

struct SrvCloth
{
    cloth_s *c = nullptr;
    int ntr = 0, ntt = 0;
    size_t scratch = 0;
    std::deque<Req> queue;
    bool running = false;
    long long admit_chunk = -1;
    size_t off = 0;
    Req cur{};
    double t_admit = 0;
};

// Pinned host staging of one chunk (two of them alternate).
struct Stage
{
    char *mem = nullptr;
    SrvCtl *sc = nullptr;
    AdmitRec *admit = nullptr;
    int *new_ids = nullptr, *inflight = nullptr;
    Tile *new_tt = nullptr, *new_rt = nullptr, *act_rt = nullptr;
    SrvStatus *status = nullptr;
    int n_inflight = 0;
    long long chunk = -1;
    cudaEvent_t ev = nullptr;
};

} // namespace

struct cloth_server_s
{
    cloth_ctx *ctx = nullptr;
    cloth_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<SrvCloth> cl;
    std::set<std::pair<long long, int>> ready; // (seq of the head request, cloth)
    std::vector<int> inflight;                 // cloths admitted and not yet retired
    std::deque<cloth_server_result> results;
    long long seq = 0, submitted = 0, completed = 0, chunks = 0, waits = 0;
    int max_inflight_seen = 0;
    bool started = false, stopping = false, failed = false;
    std::string fail_msg;
    std::thread worker;
    // device
    char *dmem = nullptr;
    size_t own_bytes = 0;
    char *pool = nullptr;
    PoolAlloc alloc;
    size_t resident = 0;
    InstDesc *d_table = nullptr;
    InstDesc **d_ptrs = nullptr;
    SrvCtl *d_sc = nullptr;
    BatchCtl *d_ctl_new = nullptr, *d_ctl_act = nullptr;
    AdmitRec *d_admit = nullptr;
    int *d_new_ids = nullptr, *d_inflight = nullptr;
    Tile *d_new_tt = nullptr, *d_new_rt = nullptr, *d_act_rt = nullptr;
    SrvStatus *d_status = nullptr;
    Stage st[2];
    cudaGraphExec_t exec = nullptr;
    int total_rt = 0, total_tt = 0;
};

namespace {

size_t own_bytes_for(int n, int total_rt, int total_tt, Layout *L = nullptr,
                     size_t *offs = nullptr)
{
    Layout l;
    size_t o[11];
    o[0] = l.take<InstDesc>(n);
    o[1] = l.take<InstDesc *>(n);
    o[2] = l.take<SrvCtl>(1);
    o[3] = l.take<BatchCtl>(1);
    o[4] = l.take<BatchCtl>(1);
    o[5] = l.take<AdmitRec>(n);
    o[6] = l.take<int>(n);
    o[7] = l.take<int>(n);
    o[8] = l.take<Tile>(total_tt);
    o[9] = l.take<Tile>(total_rt);
    o[10] = l.take<Tile>(total_rt);
    size_t o_status = l.take<SrvStatus>(n);
    if (offs)
    {
        for (int k = 0; k < 11; k++)
            offs[k] = o[k];
        offs[11] = o_status;
    }
    if (L)
        *L = l;
    return l.off;
}

int add_node(cudaGraph_t g, cudaGraphNode_t *node, cudaGraphNode_t *last, void *func,
             int grid, int block, void **args, unsigned smem = 0)
{
    cudaKernelNodeParams p;
    std::memset(&p, 0, sizeof(p));
    p.func = func;
    p.gridDim = dim3(std::max(1, grid));
    p.blockDim = dim3(block);
    p.sharedMemBytes = smem;
    p.kernelParams = args;
    SCK(cudaGraphAddKernelNode(node, g, *last ? last : nullptr, *last ? 1 : 0, &p));
    *last = *node;
    return CLOTH_OK;
}

int build_chunk_graph(cloth_server_s *s)
{
    cloth_ctx *ctx = s->ctx;
    const int n = int(s->cl.size());
    const int one_wave_tri = ctx->num_sms * std::max(1, ctx->occ_tri);
    const int one_wave_row = ctx->num_sms * std::max(1, ctx->occ_row);
    // SpMV variants that apply skew block parts when a dihedral-bending cloth
    // is registered
    bool skew = false;
    for (const SrvCloth &sc : s->cl)
        skew = skew || sc.c->h.Aw != nullptr || sc.c->mat.bending_model == 1;
    const GraphLoopVariant *table = skew ? kSpmvSkewVariants : kSpmvVariants;
    int sv_i = ctx->tune_spmv;
    if (table[sv_i].bulk_stages)
    {
        // The bulk-staged SpMV stages p over every tile's column range; the
        // served cloths (up to 256 vertices a side) make that range five
        // tiles wide, and the served chunks were measured slower with it.
        // Take the fastest register variant of the context's last tuning.
        sv_i = kDefaultSpmvVariant;
        float best = 1e30f;
        for (int v = 0; v < kNumSpmvVariants && v < int(ctx->tune_ms_spmv.size()); v++)
            if (!table[v].bulk_stages && ctx->tune_ms_spmv[v] > 0.f &&
                ctx->tune_ms_spmv[v] < best)
            {
                best = ctx->tune_ms_spmv[v];
                sv_i = v;
            }
    }
    const int occ_sv = (skew ? ctx->occ_spmv_skew : ctx->occ_spmv)[sv_i];
    const unsigned smem_sv = 0;
    const GraphLoopVariant &sv = table[sv_i];
    const GraphLoopVariant &uv = kUpdateVariants[ctx->tune_update];
    const int one_wave_spmv = ctx->num_sms * std::max(1, occ_sv);
    const int one_wave_upd = ctx->num_sms * std::max(1, ctx->occ_update[ctx->tune_update]);
    cudaGraph_t g = nullptr;
    SCK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle hnd = 0;
    int rc = CLOTH_OK;
    if (cudaGraphConditionalHandleCreate(&hnd, g, 0, cudaGraphCondAssignDefault) !=
        cudaSuccess)
    {
        cudaGraphDestroy(g);
        return sfail(CLOTH_ERR_CUDA, "server: cudaGraphConditionalHandleCreate failed");
    }
    int zero = 0, one = 1;
    int *left = &s->d_sc->iters_left;
    const int *n_new = &s->d_sc->n_new;
    void *a_admit[] = {&s->d_admit, &s->d_sc, &s->d_table, &s->d_ctl_new, &s->d_ctl_act};
    void *a_pins[] = {&s->d_ptrs, &s->d_new_ids, &zero, &n_new};
    void *a_tri[] = {&s->d_ptrs, &s->d_new_tt, &s->d_ctl_new};
    void *a_row[] = {&s->d_ptrs, &s->d_new_rt, &s->d_ctl_new};
    void *a_begin[] = {&s->d_ctl_new, &s->d_ctl_act, &s->d_sc, &hnd};
    void *a_spmv[] = {&s->d_ptrs, &s->d_act_rt, &s->d_ctl_act, &one, &hnd};
    const int *n_inflight = &s->d_sc->n_inflight;
    void *a_red[] = {&s->d_ptrs, &s->d_inflight, &zero, &n_inflight, &s->d_ctl_act, &one, &hnd};
    void *a_upd[] = {&s->d_ptrs, &s->d_act_rt, &s->d_ctl_act, &one, &hnd, &left};
    void *a_adv[] = {&s->d_ptrs, &s->d_act_rt, &s->d_ctl_act, &one};
    void *a_stat[] = {&s->d_ptrs, &s->d_inflight, &s->d_sc, &s->d_status};
    cudaGraphNode_t last = nullptr, nd = nullptr;
    const int gsmall = std::max(1, std::min(n, 1024));
    if (rc == CLOTH_OK)
        rc = add_node(g, &nd, &last, (void *)k_srv_admit, std::min(n, 256), 128, a_admit);
    if (rc == CLOTH_OK)
        rc = add_node(g, &nd, &last, (void *)k_pins, gsmall, kTile, a_pins);
    if (rc == CLOTH_OK)
        rc = add_node(g, &nd, &last, (void *)k_tri, one_wave_tri, kTile, a_tri);
    if (rc == CLOTH_OK)
        rc = add_node(g, &nd, &last, (void *)k_row, one_wave_row, kTile, a_row);
    if (rc == CLOTH_OK)
        rc = add_node(g, &nd, &last, (void *)k_srv_begin, 1, 1, a_begin);
    if (rc == CLOTH_OK)
    {
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = hnd;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cn;
        if (cudaGraphAddNode(&cn, g, &last, nullptr, 1, &cp) != cudaSuccess)
            rc = sfail(CLOTH_ERR_CUDA, "server: cudaGraphAddNode(conditional) failed");
        else
        {
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            cudaGraphNode_t bl = nullptr, bn = nullptr;
            // several iterations per evaluation of the condition, as many as
            // divide the chunk's iteration budget (the update of the budget's
            // last iteration clears the condition)
            const int ci = s->cfg.chunk_iters;
            const int per_body = ci % 4 == 0 ? std::min(4, kLoopBodyIters)
                                 : ci % 2 == 0 ? std::min(2, kLoopBodyIters) : 1;
            for (int u = 0; u < per_body && rc == CLOTH_OK; u++)
            {
                rc = add_node(body, &bn, &bl, const_cast<void *>(sv.func), one_wave_spmv,
                              spmv_block(sv), a_spmv, smem_sv);
                if (rc == CLOTH_OK)
                    rc = add_node(body, &bn, &bl, (void *)k_reduce_pq, reduce_grid(n), kTile,
                                  a_red);
                if (rc == CLOTH_OK)
                    rc = add_node(body, &bn, &bl, const_cast<void *>(uv.func), one_wave_upd,
                                  kTile / uv.rows_per_thread, a_upd);
                if (rc == CLOTH_OK)
                    rc = add_node(body, &bn, &bl, (void *)k_reduce_rz, reduce_grid(n), kTile,
                                  a_red);
            }
            last = cn;
        }
    }
    if (rc == CLOTH_OK)
        rc = add_node(g, &nd, &last, (void *)k_advance, one_wave_row, kTile, a_adv);
    if (rc == CLOTH_OK)
        rc = add_node(g, &nd, &last, (void *)k_srv_status, std::max(1, (n + 127) / 128), 128,
                      a_stat);
    if (rc == CLOTH_OK && cudaGraphInstantiate(&s->exec, g, 0) != cudaSuccess)
        rc = sfail(CLOTH_ERR_CUDA, "server: cudaGraphInstantiate failed");
    cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
}

// Results of one finished chunk: retire requests whose step ended.
void retire_chunk(cloth_server_s *s, Stage &sg)
{
    const double t = now_s();
    std::lock_guard<std::mutex> lk(s->mu);
    bool any = false;
    for (int i = 0; i < sg.n_inflight; i++)
    {
        const SrvStatus &r = sg.status[i];
        if (!r.done || r.id < 0 || r.id >= int(s->cl.size()))
            continue;
        SrvCloth &cr = s->cl[r.id];
        if (!cr.running || cr.admit_chunk > sg.chunk)
            continue;
        cloth_server_result o;
        std::memset(&o, 0, sizeof(o));
        o.tag = cr.cur.tag;
        o.cloth = r.id;
        o.status = r.status;
        o.iters = r.iter;
        const double rn = std::sqrt(std::max(0.0, r.rr)), bn = std::sqrt(std::max(0.0, r.bb));
        o.rel_residual = bn > 0 ? rn / bn : rn;
        o.t_arrival = cr.cur.t_arrival;
        o.t_admit = cr.t_admit;
        o.t_done = t;
        cr.running = false;
        s->alloc.give(cr.off, cr.scratch);
        s->inflight.erase(std::find(s->inflight.begin(), s->inflight.end(), r.id));
        if (!cr.queue.empty())
            s->ready.insert({cr.queue.front().seq, r.id});
        s->results.push_back(o);
        s->completed++;
        any = true;
    }
    if (any)
        s->cv_done.notify_all();
}

// Build chunk lists into sg and launch the chunk. Returns false when there
// was nothing to run.
int launch_chunk(cloth_server_s *s, Stage &sg, long long chunk_no, bool *launched)
{
    *launched = false;
    int n_admit = 0, n_new_tt = 0, n_new_rt = 0, n_act_rt = 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        const double t = now_s();
        const int cap = s->cfg.max_inflight > 0 ? s->cfg.max_inflight : 1 << 30;
        while (!s->stopping && !s->ready.empty())
        {
            auto it = s->ready.begin();
            const int id = it->second;
            SrvCloth &cr = s->cl[id];
            size_t off = 0;
            if (int(s->inflight.size()) >= cap || !s->alloc.take(cr.scratch, &off))
            {
                s->waits++;
                break;
            }
            s->ready.erase(it);
            cr.running = true;
            cr.cur = cr.queue.front();
            cr.queue.pop_front();
            cr.admit_chunk = chunk_no;
            cr.t_admit = t;
            cr.off = off;
            AdmitRec &ar = sg.admit[n_admit];
            ar.id = id;
            ar.desc = cr.c->h;
            ar.desc.hold_maxiter = 0; // served solves always advance
            bind_scratch(cr.c, ar.desc, s->pool + off);
            sg.new_ids[n_admit] = id;
            n_admit++;
            for (int k = 0; k < cr.ntt; k++)
                sg.new_tt[n_new_tt++] = Tile{id, k * kTile, s->d_table + id, cr.c->d_state};
            for (int k = 0; k < cr.ntr; k++)
                sg.new_rt[n_new_rt++] = Tile{id, k * kTile, s->d_table + id, cr.c->d_state};
            s->inflight.push_back(id);
        }
        s->max_inflight_seen = std::max(s->max_inflight_seen, int(s->inflight.size()));
        for (size_t i = 0; i < s->inflight.size(); i++)
        {
            const int id = s->inflight[i];
            sg.inflight[i] = id;
            for (int k = 0; k < s->cl[id].ntr; k++)
                sg.act_rt[n_act_rt++] =
                    Tile{id, k * kTile, s->d_table + id, s->cl[id].c->d_state};
        }
        sg.n_inflight = int(s->inflight.size());
    }
    if (sg.n_inflight == 0)
        return CLOTH_OK;
    SrvCtl &h = *sg.sc;
    h.n_admit = n_admit;
    h.n_new = n_admit;
    h.n_inflight = sg.n_inflight;
    h.chunk_iters = s->cfg.chunk_iters;
    h.n_new_rt = n_new_rt;
    h.n_new_tt = n_new_tt;
    h.n_act_rt = n_act_rt;
    h.pad = 0;
    sg.chunk = chunk_no;
    cloth_ctx *ctx = s->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    cudaStream_t st = ctx->stream;
    auto h2d = [&](void *dst, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st)
                     : cudaSuccess;
    };
    SCK(h2d(s->d_sc, sg.sc, kSrvHostBytes));
    SCK(h2d(s->d_admit, sg.admit, size_t(n_admit) * sizeof(AdmitRec)));
    SCK(h2d(s->d_new_ids, sg.new_ids, size_t(n_admit) * sizeof(int)));
    SCK(h2d(s->d_new_tt, sg.new_tt, size_t(n_new_tt) * sizeof(Tile)));
    SCK(h2d(s->d_new_rt, sg.new_rt, size_t(n_new_rt) * sizeof(Tile)));
    SCK(h2d(s->d_act_rt, sg.act_rt, size_t(n_act_rt) * sizeof(Tile)));
    SCK(h2d(s->d_inflight, sg.inflight, size_t(sg.n_inflight) * sizeof(int)));
    SCK(cudaGraphLaunch(s->exec, st));
    SCK(cudaMemcpyAsync(sg.status, s->d_status, size_t(sg.n_inflight) * sizeof(SrvStatus),
                        cudaMemcpyDeviceToHost, st));
    SCK(cudaEventRecord(sg.ev, st));
    *launched = true;
    {
        std::lock_guard<std::mutex> lk2(s->mu);
        s->chunks++;
    }
    return CLOTH_OK;
}

void fail_all(cloth_server_s *s, const std::string &msg)
{
    std::lock_guard<std::mutex> lk(s->mu);
    s->failed = true;
    s->fail_msg = msg;
    const double t = now_s();
    for (size_t id = 0; id < s->cl.size(); id++)
    {
        SrvCloth &cr = s->cl[id];
        auto emit = [&](const Req &q) {
            cloth_server_result o;
            std::memset(&o, 0, sizeof(o));
            o.tag = q.tag;
            o.cloth = int(id);
            o.status = CLOTH_ERR_CUDA;
            o.t_arrival = q.t_arrival;
            o.t_done = t;
            s->results.push_back(o);
            s->completed++;
        };
        if (cr.running)
            emit(cr.cur);
        for (auto &q : cr.queue)
            emit(q);
        cr.queue.clear();
        cr.running = false;
    }
    s->ready.clear();
    s->inflight.clear();
    s->cv_done.notify_all();
}

void worker_main(cloth_server_s *s)
{
    cudaSetDevice(s->ctx->device);
    std::deque<int> outstanding; // stage indices, launch order
    int next = 0;
    long long chunk_no = 0;
    for (;;)
    {
        bool work;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            work = !s->inflight.empty() || (!s->ready.empty() && !s->stopping);
            if (!work && outstanding.empty())
            {
                if (s->stopping)
                    break;
                s->cv_work.wait_for(lk, std::chrono::milliseconds(20));
                continue;
            }
        }
        if (outstanding.size() == 2 || (!work && !outstanding.empty()))
        {
            Stage &sg = s->st[outstanding.front()];
            outstanding.pop_front();
            if (cudaEventSynchronize(sg.ev) != cudaSuccess)
            {
                fail_all(s, std::string("server: chunk failed: ") +
                                cudaGetErrorString(cudaGetLastError()));
                return;
            }
            retire_chunk(s, sg);
            continue;
        }
        bool launched = false;
        if (launch_chunk(s, s->st[next], chunk_no, &launched) != CLOTH_OK)
        {
            fail_all(s, "server: chunk launch failed");
            return;
        }
        if (launched)
        {
            outstanding.push_back(next);
            next ^= 1;
            chunk_no++;
        }
        else if (!outstanding.empty())
        {
            Stage &sg = s->st[outstanding.front()];
            outstanding.pop_front();
            if (cudaEventSynchronize(sg.ev) != cudaSuccess)
            {
                fail_all(s, "server: chunk failed");
                return;
            }
            retire_chunk(s, sg);
        }
    }
}

void release_device(cloth_server_s *s)
{
    if (s->exec)
        cudaGraphExecDestroy(s->exec);
    s->exec = nullptr;
    for (auto &sg : s->st)
    {
        if (sg.ev)
            cudaEventDestroy(sg.ev);
        if (sg.mem)
            cudaFreeHost(sg.mem);
        sg = Stage{};
    }
    if (s->pool)
        cudaFree(s->pool);
    s->pool = nullptr;
    if (s->dmem)
        cudaFree(s->dmem);
    s->dmem = nullptr;
    s->ctx->bytes -= std::min(s->ctx->bytes, s->own_bytes + s->alloc.size);
    s->own_bytes = 0;
    s->alloc.reset(0);
}

void stop_worker(cloth_server_s *s)
{
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        for (auto &cr : s->cl)
            cr.queue.clear();
        s->ready.clear();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable())
        s->worker.join();
}

} // namespace

bool cloth::detail::server_busy(const cloth_server_s *s, const cloth_s *c)
{
    auto *sv = const_cast<cloth_server_s *>(s);
    std::lock_guard<std::mutex> lk(sv->mu);
    for (const auto &cr : sv->cl)
        if (cr.c == c)
            return cr.running || !cr.queue.empty();
    return false;
}

void cloth::detail::server_teardown(cloth_server_s *s)
{
    stop_worker(s);
    cudaStreamSynchronize(s->ctx->stream);
    for (auto &cr : s->cl)
    {
        cr.c->server = nullptr;
        alloc_own_scratch(cr.c);
    }
    release_device(s);
    delete s;
}

extern "C" {

double cloth_server_now(void) { return now_s(); }

int cloth_server_create(cloth_ctx *ctx, const cloth_server_config *cfg, cloth_server **out)
{
    if (!ctx || !cfg || !out)
        return sfail(CLOTH_ERR_INVALID, "cloth_server_create: NULL argument");
    *out = nullptr;
    if (cfg->chunk_iters <= 0 || cfg->budget_bytes == 0)
        return sfail(CLOTH_ERR_INVALID, "cloth_server_create: chunk_iters and budget must be > 0");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    auto *s = new cloth_server_s();
    s->ctx = ctx;
    s->cfg = *cfg;
    ctx->servers.push_back(s);
    *out = s;
    return CLOTH_OK;
}

int cloth_server_add(cloth_server *s, cloth_t *c, double dt, const cloth_solve_params *params,
                     int *index)
{
    if (!s || !c)
        return sfail(CLOTH_ERR_INVALID, "cloth_server_add: NULL argument");
    if (c->ctx != s->ctx)
        return sfail(CLOTH_ERR_INVALID, "cloth_server_add: cloth belongs to another context");
    if (params && (params->max_iters < 0 || params->check_every < 0))
        return sfail(CLOTH_ERR_INVALID, "cloth_server_add: bad solve parameters");
    std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
    if (s->started)
        return sfail(CLOTH_ERR_STATE, "cloth_server_add: the server is running");
    if (c->server)
        return sfail(CLOTH_ERR_STATE, "cloth_server_add: the cloth is held by a server");
    if (!c->bodies.empty())
        return sfail(CLOTH_ERR_UNSUPPORTED, "cloth_server_add: a cloth with kinematic bodies "
                                            "is stepped alone");
    const int n = int(s->cl.size()) + 1;
    const int ntr = (c->tab.nv + kTile - 1) / kTile, ntt = (c->tab.nt + c->tab.n_dih + kTile - 1) / kTile;
    size_t max_scratch = c->sl.bytes;
    for (auto &cr : s->cl)
        max_scratch = std::max(max_scratch, cr.scratch);
    const size_t need = s->resident + c->arena_bytes +
                        own_bytes_for(n, s->total_rt + ntr, s->total_tt + ntt) +
                        align_up(max_scratch, 256);
    if (need > s->cfg.budget_bytes)
        return sfail(CLOTH_ERR_BUDGET, "cloth_server_add: resident state (" +
                                           std::to_string(need) + " bytes with the largest "
                                           "request's work memory) exceeds the budget");
    SCK(cudaSetDevice(s->ctx->device));
    set_params(c, params);
    set_dt(c, dt);
    if (c->drag_vid >= 0)
    {
        c->drag_vid = -1; // the drag point lasts one step (BaraffClothGpu.cpp:260-262)
        c->pins_dirty = true;
    }
    int rc = sync_pins(c);
    if (rc != CLOTH_OK)
        return rc;
    free_own_scratch(c);
    rc = sync_desc(c);
    if (rc != CLOTH_OK)
        return rc;
    c->server = s;
    SrvCloth cr;
    cr.c = c;
    cr.ntr = ntr;
    cr.ntt = ntt;
    cr.scratch = c->sl.bytes;
    s->cl.push_back(cr);
    s->resident += c->arena_bytes;
    s->total_rt += ntr;
    s->total_tt += ntt;
    if (index)
        *index = n - 1;
    return CLOTH_OK;
}

int cloth_server_start(cloth_server *s)
{
    if (!s)
        return sfail(CLOTH_ERR_INVALID, "cloth_server_start: NULL server");
    cloth_ctx *ctx = s->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (s->started)
        return sfail(CLOTH_ERR_STATE, "cloth_server_start: already started");
    if (s->cl.empty())
        return sfail(CLOTH_ERR_STATE, "cloth_server_start: no cloth registered");
    SCK(cudaSetDevice(ctx->device));
    const int n = int(s->cl.size());
    size_t offs[12];
    const size_t own = own_bytes_for(n, s->total_rt, s->total_tt, nullptr, offs);
    size_t max_scratch = 0;
    for (auto &cr : s->cl)
        max_scratch = std::max(max_scratch, align_up(cr.scratch, 256));
    if (s->resident + own + max_scratch > s->cfg.budget_bytes)
        return sfail(CLOTH_ERR_BUDGET, "cloth_server_start: budget leaves no room for the "
                                       "largest request's work memory");
    size_t pool = s->cfg.budget_bytes - s->resident - own;
    pool = pool / 256 * 256;
    // never more than all requests together could use
    size_t all = 0;
    for (auto &cr : s->cl)
        all += align_up(cr.scratch, 256);
    pool = std::min(pool, all);
    size_t free_b = 0, total_b = 0;
    SCK(cudaMemGetInfo(&free_b, &total_b));
    const size_t margin = size_t(256) << 20;
    if (own + pool + margin > free_b)
    {
        if (own + max_scratch + margin > free_b)
            return sfail(CLOTH_ERR_OOM, "cloth_server_start: not enough free device memory");
        pool = (free_b - own - margin) / 256 * 256;
    }
    if (cudaMalloc(&s->dmem, own) != cudaSuccess)
    {
        cudaGetLastError();
        s->dmem = nullptr;
        return sfail(CLOTH_ERR_OOM, "cloth_server_start: device allocation failed");
    }
    if (cudaMalloc(&s->pool, pool) != cudaSuccess)
    {
        cudaGetLastError();
        s->pool = nullptr;
        release_device(s);
        return sfail(CLOTH_ERR_OOM, "cloth_server_start: pool allocation failed");
    }
    s->own_bytes = own;
    s->alloc.reset(pool);
    ctx->bytes += own + pool;
    char *b = s->dmem;
    s->d_table = reinterpret_cast<InstDesc *>(b + offs[0]);
    s->d_ptrs = reinterpret_cast<InstDesc **>(b + offs[1]);
    s->d_sc = reinterpret_cast<SrvCtl *>(b + offs[2]);
    s->d_ctl_new = reinterpret_cast<BatchCtl *>(b + offs[3]);
    s->d_ctl_act = reinterpret_cast<BatchCtl *>(b + offs[4]);
    s->d_admit = reinterpret_cast<AdmitRec *>(b + offs[5]);
    s->d_new_ids = reinterpret_cast<int *>(b + offs[6]);
    s->d_inflight = reinterpret_cast<int *>(b + offs[7]);
    s->d_new_tt = reinterpret_cast<Tile *>(b + offs[8]);
    s->d_new_rt = reinterpret_cast<Tile *>(b + offs[9]);
    s->d_act_rt = reinterpret_cast<Tile *>(b + offs[10]);
    s->d_status = reinterpret_cast<SrvStatus *>(b + offs[11]);
    cudaStream_t st = ctx->stream;
    int rc = CLOTH_OK;
    auto fail_rel = [&](int code, const std::string &m) {
        release_device(s);
        return sfail(code, m);
    };
    if (cudaMemsetAsync(s->dmem, 0, own, st) != cudaSuccess)
        return fail_rel(CLOTH_ERR_CUDA, "cloth_server_start: memset failed");
    std::vector<InstDesc *> ptrs(n);
    for (int i = 0; i < n; i++)
        ptrs[i] = s->d_table + i;
    if (cudaMemcpy(s->d_ptrs, ptrs.data(), n * sizeof(InstDesc *), cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return fail_rel(CLOTH_ERR_CUDA, "cloth_server_start: upload failed");
    // pinned staging, two sets
    for (auto &sg : s->st)
    {
        Layout L;
        size_t o_sc = L.take<SrvCtl>(1), o_ad = L.take<AdmitRec>(n), o_ni = L.take<int>(n),
               o_in = L.take<int>(n), o_tt = L.take<Tile>(s->total_tt),
               o_nr = L.take<Tile>(s->total_rt), o_ar = L.take<Tile>(s->total_rt),
               o_st = L.take<SrvStatus>(n);
        if (cudaHostAlloc(&sg.mem, L.off, cudaHostAllocDefault) != cudaSuccess)
        {
            cudaGetLastError();
            sg.mem = nullptr;
            return fail_rel(CLOTH_ERR_OOM, "cloth_server_start: pinned allocation failed");
        }
        std::memset(sg.mem, 0, L.off);
        sg.sc = reinterpret_cast<SrvCtl *>(sg.mem + o_sc);
        sg.admit = reinterpret_cast<AdmitRec *>(sg.mem + o_ad);
        sg.new_ids = reinterpret_cast<int *>(sg.mem + o_ni);
        sg.inflight = reinterpret_cast<int *>(sg.mem + o_in);
        sg.new_tt = reinterpret_cast<Tile *>(sg.mem + o_tt);
        sg.new_rt = reinterpret_cast<Tile *>(sg.mem + o_nr);
        sg.act_rt = reinterpret_cast<Tile *>(sg.mem + o_ar);
        sg.status = reinterpret_cast<SrvStatus *>(sg.mem + o_st);
        if (cudaEventCreateWithFlags(&sg.ev, cudaEventDisableTiming) != cudaSuccess)
            return fail_rel(CLOTH_ERR_CUDA, "cloth_server_start: event creation failed");
    }
    rc = build_chunk_graph(s);
    if (rc != CLOTH_OK)
    {
        release_device(s);
        return rc;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess)
        return fail_rel(CLOTH_ERR_CUDA, "cloth_server_start: synchronize failed");
    s->started = true;
    s->worker = std::thread(worker_main, s);
    return CLOTH_OK;
}

int cloth_server_submit(cloth_server *s, int index, long long tag, double t_arrival)
{
    if (!s)
        return sfail(CLOTH_ERR_INVALID, "cloth_server_submit: NULL server");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (!s->started || s->stopping || s->failed)
            return sfail(CLOTH_ERR_STATE, s->failed ? s->fail_msg
                                                    : "cloth_server_submit: server not running");
        if (index < 0 || index >= int(s->cl.size()))
            return sfail(CLOTH_ERR_INVALID, "cloth_server_submit: bad cloth index");
        SrvCloth &cr = s->cl[index];
        Req q{tag, s->seq++, t_arrival >= 0 ? t_arrival : now_s()};
        const bool head = cr.queue.empty() && !cr.running;
        cr.queue.push_back(q);
        if (head)
            s->ready.insert({q.seq, index});
        s->submitted++;
    }
    s->cv_work.notify_one();
    return CLOTH_OK;
}

int cloth_server_poll(cloth_server *s, cloth_server_result *out, int cap, int *n, double wait_s)
{
    if (!s || !n || (cap > 0 && !out))
        return sfail(CLOTH_ERR_INVALID, "cloth_server_poll: bad argument");
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->results.empty() && wait_s > 0)
        s->cv_done.wait_for(lk, std::chrono::duration<double>(wait_s),
                            [&] { return !s->results.empty(); });
    int k = 0;
    while (k < cap && !s->results.empty())
    {
        out[k++] = s->results.front();
        s->results.pop_front();
    }
    *n = k;
    return CLOTH_OK;
}

int cloth_server_drain(cloth_server *s, double wait_s)
{
    if (!s)
        return sfail(CLOTH_ERR_INVALID, "cloth_server_drain: NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto done = [&] { return s->completed >= s->submitted || s->failed; };
    if (wait_s < 0)
        s->cv_done.wait(lk, done);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(wait_s), done))
        return sfail(CLOTH_ERR_TIMEOUT, "cloth_server_drain: requests still running");
    if (s->failed)
        return sfail(CLOTH_ERR_CUDA, s->fail_msg);
    return CLOTH_OK;
}

int cloth_server_get_stats(cloth_server *s, cloth_server_stats *o)
{
    if (!s || !o)
        return sfail(CLOTH_ERR_INVALID, "cloth_server_get_stats: NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(o, 0, sizeof(*o));
    o->submitted = s->submitted;
    o->completed = s->completed;
    o->chunks = s->chunks;
    o->admitted_waits = s->waits;
    o->max_inflight_seen = s->max_inflight_seen;
    o->registered = int(s->cl.size());
    o->resident_bytes = s->resident;
    o->pool_bytes = s->alloc.size;
    o->pool_peak_bytes = s->alloc.peak;
    o->own_bytes = s->own_bytes ? s->own_bytes
                                : own_bytes_for(int(s->cl.size()), s->total_rt, s->total_tt);
    for (auto &cr : s->cl)
        o->max_request_bytes = std::max(o->max_request_bytes, align_up(cr.scratch, 256));
    return CLOTH_OK;
}

int cloth_server_destroy(cloth_server *s)
{
    if (!s)
        return CLOTH_OK;
    cloth_ctx *ctx = s->ctx;
    stop_worker(s);
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    ctx->servers.erase(std::remove(ctx->servers.begin(), ctx->servers.end(), s),
                       ctx->servers.end());
    cudaStreamSynchronize(ctx->stream);
    int rc = CLOTH_OK;
    for (auto &cr : s->cl)
    {
        cr.c->server = nullptr;
        int r = alloc_own_scratch(cr.c);
        if (r != CLOTH_OK)
            rc = r;
    }
    release_device(s);
    delete s;
    return rc;
}

} // extern "C"
