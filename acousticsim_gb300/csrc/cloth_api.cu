// C ABI of the GB300 implicit cloth step: contexts, cloth instances, the
// step driver (one CUDA graph per launch set, PCG as a device-side while loop),
// batches and exports.  Declarations and reference mapping: include/cloth_gb300.h.
#include <map>
#include "internal.h"

#include <algorithm>
#include <cmath>

using namespace cloth;
using namespace cloth::detail;


namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

#define CK(call)                                                               \
    do                                                                         \
    {                                                                          \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                 \
            return fail(CLOTH_ERR_CUDA,                                        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));   \
    } while (0)

enum Phase
{
    PH_PINS = 0,
    PH_TRI,
    PH_ROW,
    PH_SPMV,
    PH_UPDATE,
    PH_ADVANCE,
    PH_COLLIDE,
    PH_REPULSE,
    PH_REDUCE
};

} // namespace

cloth_ctx_s::~cloth_ctx_s() = default;

cloth_s::~cloth_s()
{
    if (plain)
        cloth::plain_free(plain);
}

namespace cloth {
namespace detail {

struct Batch
{
    cloth_ctx *ctx = nullptr;
    std::vector<cloth_s *> members;
    char *mem = nullptr;
    InstDesc **d_descs = nullptr;
    int *d_inst = nullptr;
    Tile *d_rt = nullptr, *d_tt = nullptr;
    BatchCtl *d_ctl = nullptr;
    // the members' solve states gathered after a step, read back in one copy
    InstState *d_states = nullptr;
    BatchCtl *d_ctl_copy = nullptr;
    char *h_pinned = nullptr; // pinned: the members' states, then the set's control word
    int n_rt = 0, n_tt = 0;
    int grid_tri = 1, grid_row = 1;
    // graph-loop kernel variants (autotuned on the first step) and their grids
    int spmv_v = kDefaultSpmvVariant, upd_v = kDefaultUpdateVariant;
    bool tuned = false;
    int grid_spmv = 1, grid_update = 1;
    unsigned smem_spmv = 0; // dynamic shared memory of the chosen SpMV variant
    int spmv_waves = 8, upd_waves = 8;
    // a member carries skew block parts (dihedral bending): the SpMV variants
    // that apply them
    bool skew = false;
    // the (single) member collides with kinematic bodies
    bool collide = false;
    const GraphLoopVariant &spmv_variant(int v) const
    {
        return (skew ? kSpmvSkewVariants : kSpmvVariants)[v];
    }
    // stage bytes of the bulk-staged SpMV variants for these members, without
    // and with the halo of p
    unsigned bulk_stage[2] = {0, 0};
    unsigned stage_of(const GraphLoopVariant &sv) const { return bulk_stage[sv.bulk_halo ? 1 : 0]; }
    int spmv_occ(int v) const
    {
        const GraphLoopVariant &sv = spmv_variant(v);
        if (sv.bulk_stages)
            return bulk_occupancy(sv, stage_of(sv), ctx->max_smem_optin);
        return (skew ? ctx->occ_spmv_skew : ctx->occ_spmv)[v];
    }
    unsigned spmv_smem_of(int v) const
    {
        return bulk_smem(spmv_variant(v), stage_of(spmv_variant(v)));
    }
    bool spmv_usable(int v) const { return !spmv_variant(v).bulk_stages || spmv_occ(v) > 0; }
    void set_variants(int sv, int uv, int sw = 8, int uw = 8)
    {
        if (!spmv_usable(sv))
            sv = kDefaultSpmvVariant;
        spmv_v = sv;
        upd_v = uv;
        spmv_waves = sw;
        upd_waves = uw;
        grid_spmv = grid_for(spmv_variant(sv), spmv_occ(sv), sw);
        smem_spmv = spmv_smem_of(sv);
        grid_update = grid_for(kUpdateVariants[uv], ctx->occ_update[uv], uw);
    }
    // one block per group of TPB tiles, at most `waves` full waves of resident
    // blocks (fewer waves: each block walks more tiles, grid-stride); the
    // bulk-staged SpMV runs one wave of resident blocks, each walking its tiles
    int grid_for(const GraphLoopVariant &v, int occ, int waves = 8) const
    {
        if (v.bulk_stages)
            return std::max(1, std::min(n_rt, ctx->num_sms * std::max(occ, 1)));
        const int groups = (n_rt + v.tiles_per_block - 1) / v.tiles_per_block;
        return std::max(1, std::min(groups, ctx->num_sms * occ * waves));
    }
    // persistent solver plan
    bool persist_ok = false;
    bool persist_sm = false; // own-row state in shared memory
    bool persist_1b = false; // single-barrier variant (shared memory, every halo staged)
    TeamBlock *d_work = nullptr;
    int grid_persist = 0;
    int halo_cap = 0, rows_cap = 0;
    size_t smem_persist = 0;
    SpinCfg spin = {kSpinLimitDefault, 0u}; // the context's setting when the set was built
    // graph loop: the active count at which the loop stops and the persistent
    // kernel finishes the rest (0: the loop runs to the end), and the launch
    // sets of those rests, by member indices
    int hand_off = 0;
    std::map<std::vector<int>, std::unique_ptr<Batch>> tails;
    cudaGraphExec_t step_exec = nullptr;
    cudaGraphExec_t solve_exec = nullptr;
    ~Batch()
    {
        if (step_exec)
            cudaGraphExecDestroy(step_exec);
        if (solve_exec)
            cudaGraphExecDestroy(solve_exec);
        if (mem)
            cudaFree(mem);
        if (h_pinned)
            cudaFreeHost(h_pinned);
        if (d_work)
            cudaFree(d_work);
    }
};

} // namespace detail
} // namespace cloth

namespace {

cloth_solve_params default_params()
{
    cloth_solve_params p;
    p.max_iters = 1000;
    p.rel_tol = 1e-6;
    p.abs_tol = 0.0;
    p.check_every = 1;
    p.warm_start = 1;
    return p;
}

// ------------------------------------------------------------ profiling
cudaEvent_t take_event(cloth_ctx *c)
{
    if (c->ev_pool.empty())
    {
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
}

struct PhaseTimer
{
    cloth_ctx *c;
    int ph;
    cudaEvent_t a = nullptr;
    PhaseTimer(cloth_ctx *c_, int ph_) : c(c_), ph(ph_)
    {
        if (c->prof)
        {
            a = take_event(c);
            cudaEventRecord(a, c->stream);
        }
    }
    ~PhaseTimer()
    {
        if (c->prof)
        {
            cudaEvent_t b = take_event(c);
            cudaEventRecord(b, c->stream);
            c->ev_pending.push_back({ph, {a, b}});
        }
    }
};

void drain_profile(cloth_ctx *c)
{
    if (c->ev_pending.empty())
        return;
    cudaStreamSynchronize(c->stream);
    for (auto &p : c->ev_pending)
    {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        c->prof_ms[p.first] += ms;
        c->prof_n[p.first] += 1;
        c->ev_pool.push_back(p.second.first);
        c->ev_pool.push_back(p.second.second);
    }
    c->ev_pending.clear();
}

// ------------------------------------------------------------ cloth upload
int upload_tables(cloth_s *c)
{
    const Tables &t = c->tab;
    const int n = t.nv, T = t.nt, W = t.width;
    if (n >= kMaxClothVertices)
        return fail(CLOTH_ERR_MESH, "cloth_create: more than 2^24 vertices in one cloth");
    const int S = int(align_up(size_t(n), 32));
    // the triangle pass also runs the dihedral edges (indices nt .. nt + n_dih)
    const int ntr = (n + kTile - 1) / kTile, ntt = (T + t.n_dih + kTile - 1) / kTile;
    const size_t WS = size_t(W) * S;
    // planes of the stored (diagonal + upper) blocks and of the lower slots
    int Wu = 1, Wl = 0;
    for (int v = 0; v < n; v++)
    {
        const int len = t.rowptr[v + 1] - t.rowptr[v];
        Wu = std::max(Wu, len - t.diag_slot[v]);
        Wl = std::max(Wl, t.diag_slot[v]);
    }
    // tile-major planes (up_idx / lo_idx): whole 128-row tiles
    const size_t WuS = size_t(Wu) * ntr * kTile, WlS = size_t(std::max(Wl, 1)) * ntr * kTile;
    c->width_up = Wu;
    Layout L;
    size_t o_tri = L.take<int4>(T), o_tcoef = L.take<float4>(3 * size_t(T)),
           o_tdest = L.take<int4>(3 * size_t(T));
    size_t o_col = L.take<int>(WS), o_hsrc = L.take<uint32_t>(WS), o_kb = L.take<float>(WS),
           o_lref = L.take<uint32_t>(WlS), o_colu = L.take<int>(WuS);
    const int nd = t.n_dih;
    const bool dih = c->mat.bending_model == 1;
    size_t o_dvid = 0, o_dfac = 0, o_dsrc = 0, o_dent = 0;
    if (dih)
    {
        o_dvid = L.take<int4>(std::max(nd, 1));
        o_dfac = L.take<double>(std::max(nd, 1));
        o_dsrc = L.take<uint32_t>(WS);
        o_dent = L.take<uint32_t>(std::max<size_t>(t.dih_ent.size(), 1));
    }
    size_t o_thalo = L.take<int2>(ntr);
    size_t o_rowinfo = L.take<int>(n), o_fptr = L.take<int>(n + 1),
           o_mass = L.take<float>(n), o_grav = L.take<float>(n);
    size_t o_pv = L.take<int>(n + 1), o_pt = L.take<float4>(n + 1);
    size_t o_x64 = L.take<double>(3 * size_t(n)), o_xp64 = L.take<double>(3 * size_t(n));
    size_t o_x32 = L.take<float4>(n), o_dx = L.take<float4>(n);
    size_t o_st = L.take<InstState>(1), o_desc = L.take<InstDesc>(1);
    const size_t bytes = L.off;
    // per-solve work arrays, a separate allocation (a server hands these out)
    Layout W2;
    ScratchLayout &sl = c->sl;
    sl.hrec = W2.take<HRec>(9 * size_t(T));
    sl.frec = W2.take<float4>(3 * size_t(T));
    sl.A0 = W2.take<float4>(WuS);
    sl.A1 = W2.take<float2>(WuS);
    sl.M0 = W2.take<float4>(n);
    sl.M1 = W2.take<float2>(n);
    sl.b = W2.take<float4>(n);
    sl.r = W2.take<float4>(n);
    sl.z = W2.take<float4>(n);
    sl.p0 = W2.take<float4>(n);
    sl.p1 = W2.take<float4>(n);
    sl.q = W2.take<float4>(n);
    sl.w1 = W2.take<float4>(n);
    sl.part = W2.take<double>(3 * size_t(ntr));
    if (dih)
    {
        sl.drec = W2.take<float4>(4 * size_t(std::max(nd, 1)));
        sl.dfb = W2.take<float>(std::max(nd, 1));
        sl.Aw = W2.take<float4>(WuS);
    }
    sl.bytes = W2.off;

    char *base = nullptr;
    if (cudaMalloc(&base, bytes) != cudaSuccess)
    {
        cudaGetLastError();
        return fail(CLOTH_ERR_OOM, "cloth_create: device allocation of " +
                                       std::to_string(bytes) + " bytes failed");
    }
    c->arena = base;
    c->arena_bytes = bytes;
    if (cudaMalloc(&c->scratch, sl.bytes) != cudaSuccess)
    {
        cudaGetLastError();
        c->scratch = nullptr;
        return fail(CLOTH_ERR_OOM, "cloth_create: device allocation of " +
                                       std::to_string(sl.bytes) + " bytes failed");
    }
    c->scratch_bytes = sl.bytes;
    cudaStream_t s = c->ctx->stream;
    CK(cudaMemsetAsync(base, 0, bytes, s));
    CK(cudaMemsetAsync(c->scratch, 0, sl.bytes, s));

    // host staging in device layout
    std::vector<int4> tri(T);
    std::vector<float4> tcoef(3 * size_t(T));
    std::vector<int4> tdest(3 * size_t(T));
    for (int i = 0; i < T; i++)
    {
        const int *v = &c->mesh.tris[size_t(i) * 3];
        int a;
        std::memcpy(&a, &t.area[i], 4);
        tri[i] = make_int4(v[0], v[1], v[2], a);
        const float *cf = &t.coef[size_t(i) * 12];
        tcoef[3 * i + 0] = make_float4(cf[0], cf[1], cf[2], cf[3]);
        tcoef[3 * i + 1] = make_float4(cf[4], cf[5], cf[6], cf[7]);
        tcoef[3 * i + 2] = make_float4(cf[8], cf[9], cf[10], cf[11]);
        const int *hd = &t.h_dest[size_t(i) * 9];
        const int *fd = &t.f_dest[size_t(i) * 3];
        tdest[3 * i + 0] = make_int4(hd[0], hd[1], hd[2], hd[3]);
        tdest[3 * i + 1] = make_int4(hd[4], hd[5], hd[6], hd[7]);
        tdest[3 * i + 2] = make_int4(hd[8], fd[0], fd[1], fd[2]);
    }
    std::vector<int> col(WS, 0), colu(WuS, 0), rowinfo(n);
    std::vector<uint32_t> hsrc(WS, 0u), lref(WlS, 0u);
    std::vector<float> kb(WS, 0.f), mass(n), grav(n);
    for (int v = 0; v < n; v++)
    {
        int len = t.rowptr[v + 1] - t.rowptr[v];
        rowinfo[v] = len | (t.diag_slot[v] << 8);
        for (int sl = 0; sl < len; sl++)
        {
            size_t k = size_t(t.rowptr[v]) + sl;
            size_t o = size_t(sl) * S + v;
            col[o] = t.cols[k];
            hsrc[o] = (uint32_t(t.h_start[k]) << 5) | uint32_t(t.h_count[k]);
            kb[o] = t.kbend[k];
            if (sl >= t.diag_slot[v])
                colu[up_idx(sl - t.diag_slot[v], v, Wu)] = t.cols[k];
            if (sl < t.diag_slot[v])
            {
                // transposed block: row cols[k], the slot holding column v
                const int cr = t.cols[k];
                const int *b0 = &t.cols[t.rowptr[cr]], *b1 = &t.cols[t.rowptr[cr + 1]];
                const int s2 = int(std::lower_bound(b0, b1, v) - b0);
                lref[lo_idx(sl, v, Wl)] = (uint32_t(s2 - t.diag_slot[cr]) << 24) | uint32_t(cr);
            }
        }
        mass[v] = float(t.mass[v]);
        grav[v] = float(c->mat.gravity * t.mass[v]);
    }
    // column range of each 128-row tile (the bulk SpMV stages p over it)
    std::vector<int2> thalo(ntr);
    c->max_halo = 0;
    for (int tt = 0; tt < ntr; tt++)
    {
        int lo = n, hi = 0;
        for (int v = tt * kTile; v < std::min(n, (tt + 1) * kTile); v++)
            for (int k = t.rowptr[v]; k < t.rowptr[v + 1]; k++)
            {
                lo = std::min(lo, t.cols[k]);
                hi = std::max(hi, t.cols[k] + 1);
            }
        thalo[tt] = make_int2(lo, std::max(lo, hi));
        c->max_halo = std::max(c->max_halo, hi - lo);
    }
    std::vector<double> x64(c->mesh.pos);
    std::vector<float4> x32(n);
    for (int v = 0; v < n; v++)
        x32[v] = make_float4(float(x64[3 * v]), float(x64[3 * v + 1]),
                             float(x64[3 * v + 2]), 0.f);

    CK(cudaMemcpyAsync(base + o_tri, tri.data(), tri.size() * sizeof(int4),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_tcoef, tcoef.data(), tcoef.size() * sizeof(float4),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_tdest, tdest.data(), tdest.size() * sizeof(int4),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_col, col.data(), WS * sizeof(int),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_hsrc, hsrc.data(), WS * sizeof(uint32_t),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_kb, kb.data(), WS * sizeof(float),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_lref, lref.data(), WlS * sizeof(uint32_t),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_colu, colu.data(), WuS * sizeof(int),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_rowinfo, rowinfo.data(), n * sizeof(int),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_thalo, thalo.data(), ntr * sizeof(int2),
                       cudaMemcpyHostToDevice, s));
    std::vector<int4> dvid;
    std::vector<uint32_t> dsrc;
    if (dih)
    {
        dvid.resize(nd);
        for (int q = 0; q < nd; q++)
        {
            const int *st4 = &t.stencil[size_t(t.dih_edge[q]) * 4];
            dvid[q] = make_int4(st4[0], st4[1], st4[2], st4[3]);
        }
        dsrc.assign(WS, 0u);
        for (int v = 0; v < n; v++)
            for (int sl = 0; sl < t.rowptr[v + 1] - t.rowptr[v]; sl++)
            {
                const size_t k = size_t(t.rowptr[v]) + sl;
                dsrc[size_t(sl) * S + v] =
                    (uint32_t(t.dih_start[k]) << 5) | uint32_t(t.dih_count[k]);
            }
        if (nd > 0)
        {
            CK(cudaMemcpyAsync(base + o_dvid, dvid.data(), nd * sizeof(int4),
                               cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(base + o_dfac, t.dih_factor.data(), nd * sizeof(double),
                               cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(base + o_dent, t.dih_ent.data(),
                               t.dih_ent.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        }
        CK(cudaMemcpyAsync(base + o_dsrc, dsrc.data(), WS * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(base + o_fptr, t.f_rowptr.data(), (n + 1) * sizeof(int),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_mass, mass.data(), n * sizeof(float),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_grav, grav.data(), n * sizeof(float),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_x64, x64.data(), x64.size() * sizeof(double),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_xp64, x64.data(), x64.size() * sizeof(double),
                       cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(base + o_x32, x32.data(), x32.size() * sizeof(float4),
                       cudaMemcpyHostToDevice, s));

    InstDesc &h = c->h;
    std::memset(&h, 0, sizeof(h));
    h.nv = n;
    h.nt = T;
    h.width = W;
    h.stride = S;
    h.width_lo = Wl;
    h.width_up = Wu;
    h.ntile_rows = ntr;
    h.ntile_tris = ntt;
    h.tri = reinterpret_cast<const int4 *>(base + o_tri);
    h.tcoef = reinterpret_cast<const float4 *>(base + o_tcoef);
    h.tdest = reinterpret_cast<const int4 *>(base + o_tdest);
    h.col = reinterpret_cast<const int *>(base + o_col);
    h.hsrc = reinterpret_cast<const uint32_t *>(base + o_hsrc);
    h.kb = reinterpret_cast<const float *>(base + o_kb);
    h.lref = reinterpret_cast<const uint32_t *>(base + o_lref);
    h.colu = reinterpret_cast<const int *>(base + o_colu);
    if (dih)
    {
        h.n_dih = nd;
        h.dvid = reinterpret_cast<const int4 *>(base + o_dvid);
        h.dfac = reinterpret_cast<const double *>(base + o_dfac);
        h.dsrc = reinterpret_cast<const uint32_t *>(base + o_dsrc);
        h.dent = reinterpret_cast<const uint32_t *>(base + o_dent);
    }
    h.rowinfo = reinterpret_cast<const int *>(base + o_rowinfo);
    h.thalo = reinterpret_cast<const int2 *>(base + o_thalo);
    h.fptr = reinterpret_cast<const int *>(base + o_fptr);
    h.mass = reinterpret_cast<const float *>(base + o_mass);
    h.grav = reinterpret_cast<const float *>(base + o_grav);
    h.pin_vid = reinterpret_cast<const int *>(base + o_pv);
    h.pin_tgt = reinterpret_cast<const float4 *>(base + o_pt);
    h.npins = 0;
    h.x64 = reinterpret_cast<double *>(base + o_x64);
    h.xp64 = reinterpret_cast<double *>(base + o_xp64);
    h.x32 = reinterpret_cast<float4 *>(base + o_x32);
    h.dx = reinterpret_cast<float4 *>(base + o_dx);
    bind_scratch(c, h, c->scratch);
    h.st = reinterpret_cast<InstState *>(base + o_st);
    c->d_state = h.st;
    c->d_desc = reinterpret_cast<InstDesc *>(base + o_desc);
    CK(cudaStreamSynchronize(s));
    return CLOTH_OK;
}

} // namespace

void cloth::detail::drop_launch_sets(cloth_s *c)
{
    c->self.reset();
    if (c->ctx->last_batch)
        for (auto *m : c->ctx->last_batch->members)
            if (m == c)
            {
                c->ctx->last_batch.reset();
                break;
            }
}

void cloth::detail::bind_scratch(const cloth_s *c, InstDesc &h, char *base)
{
    const ScratchLayout &sl = c->sl;
    auto at = [&](size_t o) {
        return (base && o != ScratchLayout::kAbsent) ? base + o : nullptr;
    };
    h.hrec = reinterpret_cast<HRec *>(at(sl.hrec));
    h.drec = reinterpret_cast<float4 *>(at(sl.drec));
    h.dfb = reinterpret_cast<float *>(at(sl.dfb));
    h.Aw = reinterpret_cast<float4 *>(at(sl.Aw));
    h.frec = reinterpret_cast<float4 *>(at(sl.frec));
    h.A0 = reinterpret_cast<float4 *>(at(sl.A0));
    h.A1 = reinterpret_cast<float2 *>(at(sl.A1));
    h.M0 = reinterpret_cast<float4 *>(at(sl.M0));
    h.M1 = reinterpret_cast<float2 *>(at(sl.M1));
    h.b = reinterpret_cast<float4 *>(at(sl.b));
    h.r = reinterpret_cast<float4 *>(at(sl.r));
    h.z = reinterpret_cast<float4 *>(at(sl.z));
    h.p0 = reinterpret_cast<float4 *>(at(sl.p0));
    h.p1 = reinterpret_cast<float4 *>(at(sl.p1));
    h.q = reinterpret_cast<float4 *>(at(sl.q));
    h.w1 = reinterpret_cast<float4 *>(at(sl.w1));
    h.part = reinterpret_cast<double *>(at(sl.part));
}

int cloth::detail::alloc_own_scratch(cloth_s *c)
{
    if (c->scratch)
        return CLOTH_OK;
    if (cudaMalloc(&c->scratch, c->sl.bytes) != cudaSuccess)
    {
        cudaGetLastError();
        c->scratch = nullptr;
        return fail(CLOTH_ERR_OOM, "device allocation of " + std::to_string(c->sl.bytes) +
                                       " bytes failed");
    }
    c->scratch_bytes = c->sl.bytes;
    c->ctx->bytes += c->scratch_bytes;
    CK(cudaMemsetAsync(c->scratch, 0, c->sl.bytes, c->ctx->stream));
    bind_scratch(c, c->h, c->scratch);
    c->desc_dirty = true;
    c->assembled = false;
    return sync_desc(c);
}

void cloth::detail::free_own_scratch(cloth_s *c)
{
    if (!c->scratch)
        return;
    cudaStreamSynchronize(c->ctx->stream);
    c->self.reset();
    cloth_ctx *ctx = c->ctx;
    if (ctx->last_batch)
        for (auto *m : ctx->last_batch->members)
            if (m == c)
            {
                ctx->last_batch.reset();
                break;
            }
    cudaFree(c->scratch);
    c->scratch = nullptr;
    c->ctx->bytes -= c->scratch_bytes;
    c->scratch_bytes = 0;
    bind_scratch(c, c->h, nullptr);
    c->desc_dirty = true;
    c->assembled = false;
}

namespace {

void set_material_fields(cloth_s *c)
{
    c->h.k_warp = c->mat.stretch_k[0];
    c->h.k_weft = c->mat.stretch_k[1];
    c->h.k_bias = c->mat.stretch_k[2];
    c->h.fix_fv_norm = c->mat.fix_fv_norm;
    c->desc_dirty = true;
}

} // namespace

void cloth::detail::set_params(cloth_s *c, const cloth_solve_params *p, int hold_maxiter)
{
    cloth_solve_params q = p ? *p : default_params();
    InstDesc &h = c->h;
    int mi = std::max(0, q.max_iters);
    int ce = std::max(1, q.check_every);
    double rt = q.rel_tol > 0 ? q.rel_tol * q.rel_tol : 0.0;
    double at = q.abs_tol > 0 ? q.abs_tol * q.abs_tol : 0.0;
    int ws = q.warm_start ? 1 : 0;
    const int hm = hold_maxiter ? 1 : 0;
    if (h.max_iters != mi || h.check_every != ce || h.rel_tol2 != rt ||
        h.abs_tol2 != at || h.warm_start != ws || h.hold_maxiter != hm)
    {
        h.max_iters = mi;
        h.check_every = ce;
        h.rel_tol2 = rt;
        h.abs_tol2 = at;
        h.warm_start = ws;
        h.hold_maxiter = hm;
        c->desc_dirty = true;
    }
}

namespace {

} // namespace

void cloth::detail::set_dt(cloth_s *c, double dt)
{
    if (!(dt > 0))
        dt = c->mat.default_timestep;
    if (dt == c->dt_set)
        return;
    c->dt_set = dt;
    // float arithmetic as AssembleSystemMatrixKernel / AssembleSystemRHSKernel
    // evaluate it (BaraffClothGpu.cu:264, 270, 316)
    float h = float(dt);
    c->h.h2 = h * h;
    c->h.c_mass = 1 + h * c->mat.rayleigh_a;
    c->h.c_stiff = h * c->mat.rayleigh_b - h * h;
    c->desc_dirty = true;
}

namespace {

// Static points plus the drag point of this step; targets are float.
} // namespace

int cloth::detail::sync_pins(cloth_s *c)
{
    if (!c->pins_dirty)
        return CLOTH_OK;
    std::vector<int> vid;
    std::vector<float4> tgt;
    for (int v : c->static_pins)
    {
        vid.push_back(v);
        const double *p = &c->mesh.pos[size_t(v) * 3];
        tgt.push_back(make_float4(float(p[0]), float(p[1]), float(p[2]), 0.f));
    }
    if (c->drag_vid >= 0)
    {
        vid.push_back(c->drag_vid);
        tgt.push_back(make_float4(c->drag_tgt[0], c->drag_tgt[1], c->drag_tgt[2], 0.f));
    }
    if (int(vid.size()) > c->tab.nv + 1)
        return fail(CLOTH_ERR_INVALID, "too many pinned vertices");
    cudaStream_t s = c->ctx->stream;
    if (!vid.empty())
    {
        CK(cudaMemcpyAsync(const_cast<int *>(c->h.pin_vid), vid.data(),
                           vid.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(const_cast<float4 *>(c->h.pin_tgt), tgt.data(),
                           tgt.size() * sizeof(float4), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
    }
    if (c->h.npins != int(vid.size()))
    {
        c->h.npins = int(vid.size());
        c->desc_dirty = true;
    }
    c->pins_dirty = false;
    return CLOTH_OK;
}

namespace {

} // namespace

int cloth::detail::sync_desc(cloth_s *c)
{
    if (!c->desc_dirty)
        return CLOTH_OK;
    CK(cudaMemcpy(c->d_desc, &c->h, sizeof(InstDesc), cudaMemcpyHostToDevice));
    c->desc_dirty = false;
    return CLOTH_OK;
}

namespace {

// ------------------------------------------------------------ batches
int plan_persistent(cloth_ctx *ctx, Batch *b);

} // namespace

// room left for the bulk SpMV's static shared memory (barriers, stage headers)
constexpr unsigned kBulkStaticReserve = 2048;

unsigned cloth::detail::bulk_stage_bytes(const std::vector<cloth_s *> &cloths, bool skew,
                                         bool halo)
{
    unsigned best = 0;
    for (const cloth_s *c : cloths)
    {
        const unsigned wl = unsigned(c->h.width_lo), wu = unsigned(c->h.width_up);
        const bool sk = skew && (c->h.Aw != nullptr || c->mat.bending_model == 1);
        unsigned b = kTile * 4u + wl * kTile * 4u + wu * kTile * (28u + (sk ? 16u : 0u));
        if (halo)
            b += 32u * unsigned(std::min(c->max_halo, kBulkHaloCap));
        best = std::max(best, (b + 127u) & ~127u);
    }
    return best;
}

unsigned cloth::detail::bulk_smem(const GraphLoopVariant &v, unsigned stage_bytes)
{
    return v.bulk_stages ? unsigned(v.bulk_stages) * stage_bytes : 0u;
}

int cloth::detail::bulk_occupancy(const GraphLoopVariant &v, unsigned stage_bytes, int max_smem)
{
    const unsigned sm = bulk_smem(v, stage_bytes);
    // the kernels' dynamic shared memory limit is set to max_smem - kBulkStaticReserve
    if (!v.bulk_stages || sm == 0 || sm + kBulkStaticReserve > unsigned(max_smem))
        return 0;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, v.func, kBulkThreads, sm) !=
        cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    return occ;
}

namespace {

int make_batch(cloth_ctx *ctx, const std::vector<cloth_s *> &members,
               std::unique_ptr<Batch> &out)
{
    for (auto *c : members)
        if (!c->scratch)
            return fail(CLOTH_ERR_STATE, "the cloth is held by a server; step it through "
                                         "the server");
    auto b = std::make_unique<Batch>();
    b->ctx = ctx;
    b->members = members;
    std::vector<Tile> rt, tt;
    std::vector<InstDesc *> descs;
    std::vector<int> inst;
    for (size_t i = 0; i < members.size(); i++)
    {
        cloth_s *c = members[i];
        descs.push_back(c->d_desc);
        inst.push_back(int(i));
        for (int s = 0; s < c->tab.nv; s += kTile)
            rt.push_back(Tile{int(i), s, c->d_desc, c->d_state});
        // the triangle pass also covers the dihedral edges (after the triangles)
        for (int s = 0; s < c->tab.nt + c->tab.n_dih; s += kTile)
            tt.push_back(Tile{int(i), s, c->d_desc, c->d_state});
        b->skew = b->skew || c->h.Aw != nullptr;
        b->collide = b->collide || !c->bodies.empty();
    }
    if (b->collide && members.size() > 1)
        return fail(CLOTH_ERR_UNSUPPORTED, "a cloth with kinematic bodies is stepped alone "
                                           "(not in a batch)");
    b->n_rt = int(rt.size());
    b->n_tt = int(tt.size());
    Layout L;
    size_t o_d = L.take<InstDesc *>(descs.size()), o_i = L.take<int>(inst.size()),
           o_rt = L.take<Tile>(rt.size()), o_tt = L.take<Tile>(tt.size()),
           o_c = L.take<BatchCtl>(1), o_st = L.take<InstState>(members.size()),
           o_cc = L.take<BatchCtl>(1);
    CK(cudaMalloc(&b->mem, L.off));
    b->d_states = reinterpret_cast<InstState *>(b->mem + o_st);
    b->d_ctl_copy = reinterpret_cast<BatchCtl *>(b->mem + o_cc);
    CK(cudaMallocHost(&b->h_pinned, members.size() * sizeof(InstState) + sizeof(BatchCtl)));
    b->d_descs = reinterpret_cast<InstDesc **>(b->mem + o_d);
    b->d_inst = reinterpret_cast<int *>(b->mem + o_i);
    b->d_rt = reinterpret_cast<Tile *>(b->mem + o_rt);
    b->d_tt = reinterpret_cast<Tile *>(b->mem + o_tt);
    b->d_ctl = reinterpret_cast<BatchCtl *>(b->mem + o_c);
    BatchCtl ctl = {0, b->n_rt, b->n_tt, 0, 0, {0, 0, 0}};
    CK(cudaMemcpy(b->d_descs, descs.data(), descs.size() * sizeof(InstDesc *),
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b->d_inst, inst.data(), inst.size() * sizeof(int),
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b->d_rt, rt.data(), rt.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b->d_tt, tt.data(), tt.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b->d_ctl, &ctl, sizeof(ctl), cudaMemcpyHostToDevice));
    // one tile per block while that fits in a few waves; grid-stride beyond
    auto cap = [&](int occ) { return std::max(1, ctx->num_sms * occ * 8); };
    b->grid_tri = std::max(1, std::min(b->n_tt, cap(ctx->occ_tri)));
    b->grid_row = std::max(1, std::min(b->n_rt, cap(ctx->occ_row)));
    b->bulk_stage[0] = bulk_stage_bytes(members, b->skew, false);
    b->bulk_stage[1] = bulk_stage_bytes(members, b->skew, true);
    b->set_variants(ctx->tune_spmv, ctx->tune_update);
    int rc = plan_persistent(ctx, b.get());
    if (rc != CLOTH_OK)
        return rc;
    // a graph-loop set whose drivers agree bit for bit (the persistent solver,
    // two barriers) hands its last few iterating cloths to the persistent
    // kernel: the graph loop's iterations cost about the same however few
    // cloths remain
    const int ho = ctx->tail_hand_off < 0 ? std::max(1, ctx->num_sms / 16) : ctx->tail_hand_off;
    if (!b->persist_ok && !b->collide && ho > 0 && int(members.size()) > ho &&
        (ctx->solver == CLOTH_SOLVER_PERSISTENT || ctx->solver == CLOTH_SOLVER_PERSISTENT_2B))
    {
        b->hand_off = ho;
        CK(cudaMemcpy(&b->d_ctl->hand_off, &ho, sizeof(int), cudaMemcpyHostToDevice));
    }
    out = std::move(b);
    return CLOTH_OK;
}

// The persistent kernel a plan launches.
const void *persistent_kernel(const Batch *b)
{
    if (b->persist_1b)
        return (const void *)k_pcg1_persistent;
    if (b->skew)
        return b->persist_sm ? (const void *)k_pcg_persistent_sm_skew
                             : (const void *)k_pcg_persistent_gm_skew;
    return b->persist_sm ? (const void *)k_pcg_persistent_sm : (const void *)k_pcg_persistent_gm;
}

// Team plan of the persistent solver: every instance gets blocks in
// proportion to its rows (at least one), rows split in 32-aligned chunks, and
// each block's staged range covers the columns of its rows.
int plan_persistent(cloth_ctx *ctx, Batch *b)
{
    b->persist_ok = false;
    b->persist_1b = false;
    if (ctx->solver != CLOTH_SOLVER_PERSISTENT && ctx->solver != CLOTH_SOLVER_PERSISTENT_1B &&
        ctx->solver != CLOTH_SOLVER_PERSISTENT_2B)
        return CLOTH_OK;
    const size_t smem_cap_bytes =
        std::min<size_t>(size_t(std::max(ctx->max_smem_optin, 48 * 1024)) - 4096,
                         200 * 1024);
    // per-chunk partial sums (3 floats per 32-row chunk) follow the staged state
    const size_t part_max = 3 * size_t(kMaxBlockRows / kRedRows) * sizeof(float);
    const int cap_entries = int((smem_cap_bytes - part_max) / sizeof(float4));
    // occupancy at the largest staging size we may request
    int occ = 0;
    if (cudaFuncSetAttribute(k_pcg_persistent_sm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem_cap_bytes)) != cudaSuccess ||
        cudaFuncSetAttribute(k_pcg_persistent_gm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem_cap_bytes)) != cudaSuccess ||
        cudaFuncSetAttribute(k_pcg1_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem_cap_bytes)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_pcg_persistent_gm, kPBlock,
                                                      smem_cap_bytes) != cudaSuccess ||
        occ <= 0)
    {
        cudaGetLastError();
        return CLOTH_OK;
    }
    const int G = ctx->num_sms * occ;
    const int n = int(b->members.size());
    if (n > G)
        return CLOTH_OK;
    long long total = 0;
    for (auto *c : b->members)
        total += c->tab.nv;
    std::vector<int> nb(n);
    int used = 0;
    for (int i = 0; i < n; i++)
    {
        const Tables &t = b->members[i]->tab;
        const int maxb = std::max(1, (t.nv + kRedRows - 1) / kRedRows);
        long long want = (long long)G * t.nv / std::max(1ll, total);
        nb[i] = int(std::max(1ll, std::min<long long>(want, maxb)));
        used += nb[i];
    }
    // hand spare blocks to the instances with the most rows per block
    while (used < G)
    {
        int best = -1;
        double best_load = 0;
        for (int i = 0; i < n; i++)
        {
            const Tables &t = b->members[i]->tab;
            const int maxb = std::max(1, (t.nv + kRedRows - 1) / kRedRows);
            if (nb[i] >= maxb)
                continue;
            double load = double(t.nv) / nb[i];
            if (load > best_load)
            {
                best_load = load;
                best = i;
            }
        }
        if (best < 0)
            break;
        nb[best]++;
        used++;
    }
    while (used > G)
    {
        int worst = -1;
        double lo = 1e300;
        for (int i = 0; i < n; i++)
            if (nb[i] > 1 && double(b->members[i]->tab.nv) / nb[i] < lo)
            {
                lo = double(b->members[i]->tab.nv) / nb[i];
                worst = i;
            }
        if (worst < 0)
            return CLOTH_OK;
        nb[worst]--;
        used--;
    }
    std::vector<TeamBlock> work;
    int max_entries = 0, max_rows = 0;
    bool all_staged = true;
    for (int i = 0; i < n; i++)
    {
        const Tables &t = b->members[i]->tab;
        // ranges aligned to the reduction units keep an instance's sums the
        // same whatever the team size
        const int chunk = ((t.nv + nb[i] - 1) / nb[i] + kRedRows - 1) / kRedRows * kRedRows;
        if (chunk > kMaxBlockRows)
            return CLOTH_OK;
        int rank = 0;
        std::vector<TeamBlock> team;
        for (int r0 = 0; r0 < t.nv; r0 += chunk)
        {
            TeamBlock w;
            w.inst = i;
            w.rank = rank++;
            w.row0 = r0;
            w.row1 = std::min(t.nv, r0 + chunk);
            int lo = w.row0, hi = w.row1 - 1;
            for (int v = w.row0; v < w.row1; v++)
            {
                lo = std::min(lo, t.cols[t.rowptr[v]]);
                hi = std::max(hi, t.cols[t.rowptr[v + 1] - 1]);
            }
            w.halo0 = lo;
            w.halo1 = hi + 1;
            w.p_global = 0;
            team.push_back(w);
        }
        bool team_staged = true;
        for (auto &w : team)
        {
            w.nblk = int(team.size());
            max_rows = std::max(max_rows, w.row1 - w.row0);
            if (w.halo1 - w.halo0 > cap_entries)
            {
                w.halo0 = w.halo1 = -1;
                all_staged = false;
                team_staged = false;
            }
            else
                max_entries = std::max(max_entries, w.halo1 - w.halo0);
        }
        // staged blocks keep p over their halo in shared memory from one
        // iteration to the next; a block that reads p from global memory needs
        // its neighbours to write it there
        for (auto &w : team)
        {
            w.p_global = team_staged ? 0 : 1;
            work.push_back(w);
        }
    }
    while (int(work.size()) < G)
        work.push_back(TeamBlock{-1, 0, 0, 0, 0, -1, -1, 0});
    // own-row state (dx, r, q, M^-1: 72 bytes per row) in shared memory when
    // it fits next to the staged p.  (Keeping z there as well was measured
    // slower: at 512^2 it pushes the block past the 196 KB shared-memory
    // carve-out, and the L1 left for the matrix and gathers halves.)
    b->halo_cap = max_entries;
    b->rows_cap = max_rows;
    const size_t part_bytes =
        align_up(3 * size_t((max_rows + kRedRows - 1) / kRedRows) * sizeof(float), 16);
    const size_t sm_bytes = size_t(max_entries) * sizeof(float4) +
                            size_t(max_rows) * (kPersistMShared ? 72 : 48) + part_bytes;
    b->persist_sm = sm_bytes <= smem_cap_bytes;
    b->smem_persist =
        b->persist_sm ? sm_bytes : size_t(max_entries) * sizeof(float4) + part_bytes;
    // the single-barrier variant keeps dx, p and M^-1 per own row (56 bytes)
    // next to u over the halo: it fits wherever the two-barrier one does
    // (it has no skew block parts: launch sets with a dihedral-bending
    // instance take the two-barrier kernel)
    b->persist_1b = b->persist_sm && all_staged && ctx->solver == CLOTH_SOLVER_PERSISTENT_1B &&
                    !b->skew;
    int occ2 = 0;
    if (cudaFuncSetAttribute(k_pcg_persistent_sm_skew, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem_cap_bytes)) != cudaSuccess ||
        cudaFuncSetAttribute(k_pcg_persistent_gm_skew, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem_cap_bytes)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, persistent_kernel(b), kPBlock,
                                                      b->smem_persist) != cudaSuccess ||
        occ2 * ctx->num_sms < int(work.size()))
    {
        cudaGetLastError();
        return CLOTH_OK;
    }
    // the work list, then one arrival count per block slot (the team barrier
    // of the two-barrier kernels), zeroed before every launch
    CK(cudaMalloc(&b->d_work, work.size() * (sizeof(TeamBlock) + sizeof(unsigned long long))));
    CK(cudaMemcpy(b->d_work, work.data(), work.size() * sizeof(TeamBlock),
                  cudaMemcpyHostToDevice));
    b->grid_persist = int(work.size());
    b->persist_ok = true;
    return CLOTH_OK;
}

int add_kernel(cudaGraph_t g, cudaGraphNode_t *node, const cudaGraphNode_t *deps,
               size_t ndeps, void *func, int grid, int block, void **args, unsigned smem = 0)
{
    cudaKernelNodeParams p;
    std::memset(&p, 0, sizeof(p));
    p.func = func;
    p.gridDim = dim3(grid);
    p.blockDim = dim3(block);
    p.sharedMemBytes = smem;
    p.kernelParams = args;
    CK(cudaGraphAddKernelNode(node, g, deps, ndeps, &p));
    return CLOTH_OK;
}

// Graph of the PCG loop: k_cond, then while (any active) { kLoopBodyIters x
// (spmv; reduce p.q; update; reduce r.z) }.
// With full = true the assembly in front and the position update behind are
// part of the graph too (one launch per step).
int build_graph(Batch *b, bool full, cudaGraphExec_t *exec)
{
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    int rc = CLOTH_OK;
    cudaGraphConditionalHandle hnd = 0;
    cudaGraphNode_t last = nullptr, n = nullptr;
    int one = 1, zero = 0;
    int ninst = int(b->members.size());
    int gpins = std::max(1, std::min(ninst, 1024));
    const int *no_count = nullptr;
    int all_rows = 0;
    void *a_pins[] = {&b->d_descs, &b->d_inst, &ninst, &no_count};
    void *a_tri[] = {&b->d_descs, &b->d_tt, &b->d_ctl};
    void *a_row[] = {&b->d_descs, &b->d_rt, &b->d_ctl};
    void *a_cond[] = {&b->d_ctl, &hnd};
    void *a_spmv[] = {&b->d_descs, &b->d_rt, &b->d_ctl, &one, &hnd};
    void *a_red[] = {&b->d_descs, &b->d_inst, &ninst, &no_count, &b->d_ctl, &one, &hnd};
    int *no_left = nullptr;
    void *a_upd[] = {&b->d_descs, &b->d_rt, &b->d_ctl, &one, &hnd, &no_left};
    void *a_adv[] = {&b->d_descs, &b->d_rt, &b->d_ctl, &all_rows};
    (void)zero;
    auto chain = [&](void *f, int grid, void **args) {
        if (rc != CLOTH_OK)
            return;
        rc = add_kernel(g, &n, last ? &last : nullptr, last ? 1 : 0, f, grid,
                        f == (void *)k_cond ? 1 : kTile, args);
        last = n;
    };
    if (!b->persist_ok &&
        cudaGraphConditionalHandleCreate(&hnd, g, 1, cudaGraphCondAssignDefault) !=
            cudaSuccess)
    {
        cudaGraphDestroy(g);
        return fail(CLOTH_ERR_CUDA, "cudaGraphConditionalHandleCreate failed");
    }
    if (full)
    {
        cudaMemsetParams mp;
        std::memset(&mp, 0, sizeof(mp));
        mp.dst = &b->d_ctl->n_active;
        mp.value = 0;
        mp.elementSize = 4;
        mp.width = 1;
        mp.height = 1;
        if (cudaGraphAddMemsetNode(&n, g, nullptr, 0, &mp) != cudaSuccess)
            rc = fail(CLOTH_ERR_CUDA, "cudaGraphAddMemsetNode failed");
        last = n;
        chain((void *)k_pins, gpins, a_pins);
        chain((void *)k_tri, b->grid_tri, a_tri);
        chain((void *)k_row, b->grid_row, a_row);
    }
    if (b->persist_ok)
    {
        b->spin = b->ctx->spin;
        void *a_per[] = {&b->d_descs, &b->d_work, &b->halo_cap, &b->rows_cap, &b->spin};
        if (rc == CLOTH_OK)
        {
            // the team barriers' arrival counts start at zero
            cudaMemsetParams mp;
            std::memset(&mp, 0, sizeof(mp));
            mp.dst = b->d_work + b->grid_persist;
            mp.value = 0;
            mp.elementSize = 4;
            mp.width = size_t(b->grid_persist) * 2;
            mp.height = 1;
            if (cudaGraphAddMemsetNode(&n, g, last ? &last : nullptr, last ? 1 : 0, &mp) !=
                cudaSuccess)
                rc = fail(CLOTH_ERR_CUDA, "cudaGraphAddMemsetNode failed");
            else
                last = n;
        }
        if (rc == CLOTH_OK)
        {
            cudaKernelNodeParams p;
            std::memset(&p, 0, sizeof(p));
            p.func = const_cast<void *>(persistent_kernel(b));
            p.gridDim = dim3(b->grid_persist);
            p.blockDim = dim3(kPBlock);
            p.sharedMemBytes = unsigned(b->smem_persist);
            p.kernelParams = a_per;
            if (cudaGraphAddKernelNode(&n, g, last ? &last : nullptr, last ? 1 : 0, &p) !=
                cudaSuccess)
                rc = fail(CLOTH_ERR_CUDA, "cudaGraphAddKernelNode(persistent) failed");
            else
            {
                cudaLaunchAttributeValue v;
                std::memset(&v, 0, sizeof(v));
                v.cooperative = 1;
                if (cudaGraphKernelNodeSetAttribute(n, cudaLaunchAttributeCooperative, &v) !=
                    cudaSuccess)
                    rc = fail(CLOTH_ERR_CUDA, "cooperative attribute on graph node failed");
                last = n;
            }
        }
    }
    else
        chain((void *)k_cond, 1, a_cond);
    if (rc == CLOTH_OK && !b->persist_ok)
    {
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = hnd;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cn;
        if (cudaGraphAddNode(&cn, g, &last, nullptr, 1, &cp) != cudaSuccess)
            rc = fail(CLOTH_ERR_CUDA, "cudaGraphAddNode(conditional) failed");
        else
        {
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            cudaGraphNode_t k1, k2;
            const GraphLoopVariant &sv = b->spmv_variant(b->spmv_v);
            const GraphLoopVariant &uv = kUpdateVariants[b->upd_v];
            cudaGraphNode_t k3, k4, prev = nullptr;
            const int gred = reduce_grid(ninst);
            // kLoopBodyIters PCG iterations per evaluation of the while
            // condition (each evaluation costs about as much as a small
            // kernel); an instance that ends inside the body skips its tiles
            for (int u = 0; u < kLoopBodyIters && rc == CLOTH_OK; u++)
            {
                rc = add_kernel(body, &k1, prev ? &prev : nullptr, prev ? 1 : 0,
                                const_cast<void *>(sv.func), b->grid_spmv, spmv_block(sv),
                                a_spmv, b->smem_spmv);
                if (rc == CLOTH_OK)
                    rc = add_kernel(body, &k3, &k1, 1, (void *)k_reduce_pq, gred, kTile, a_red);
                if (rc == CLOTH_OK)
                    rc = add_kernel(body, &k2, &k3, 1, const_cast<void *>(uv.func),
                                    b->grid_update, kTile / uv.rows_per_thread, a_upd);
                if (rc == CLOTH_OK)
                    rc = add_kernel(body, &k4, &k2, 1, (void *)k_reduce_rz, gred, kTile, a_red);
                prev = k4;
            }
            last = cn;
        }
    }
    // (a set that hands its last cloths over advances after they finish)
    if (full && b->hand_off == 0)
        chain((void *)k_advance, b->grid_row, a_adv);
    if (rc == CLOTH_OK && cudaGraphInstantiate(exec, g, 0) != cudaSuccess)
        rc = fail(CLOTH_ERR_CUDA, "cudaGraphInstantiate failed");
    cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
}

// Host-driven launches of the same kernels (used when profiling, so every
// phase gets its own CUDA events; the arithmetic is identical).
int launch_assemble(Batch *b)
{
    cloth_ctx *ctx = b->ctx;
    cudaStream_t s = ctx->stream;
    int ninst = int(b->members.size());
    CK(cudaMemsetAsync(&b->d_ctl->n_active, 0, sizeof(int), s));
    {
        PhaseTimer t(ctx, PH_PINS);
        k_pins<<<std::max(1, std::min(ninst, 1024)), kTile, 0, s>>>(b->d_descs,
                                                                  b->d_inst, ninst, nullptr);
    }
    if (b->collide)
    {
        PhaseTimer t(ctx, PH_COLLIDE);
        int rc = collide_detect(b->members[0]);
        if (rc != CLOTH_OK)
            return rc;
    }
    {
        PhaseTimer t(ctx, PH_TRI);
        k_tri<<<b->grid_tri, kTile, 0, s>>>(b->d_descs, b->d_tt, b->d_ctl);
    }
    {
        PhaseTimer t(ctx, PH_ROW);
        k_row<<<b->grid_row, kTile, 0, s>>>(b->d_descs, b->d_rt, b->d_ctl);
    }
    CK(cudaGetLastError());
    return CLOTH_OK;
}

int launch_persistent(Batch *b)
{
    cloth_ctx *ctx = b->ctx;
    PhaseTimer t(ctx, PH_SPMV);
    b->spin = ctx->spin;
    void *args[] = {&b->d_descs, &b->d_work, &b->halo_cap, &b->rows_cap, &b->spin};
    CK(cudaMemsetAsync(b->d_work + b->grid_persist, 0,
                       size_t(b->grid_persist) * sizeof(unsigned long long), ctx->stream));
    CK(cudaLaunchCooperativeKernel(persistent_kernel(b),
                                   dim3(b->grid_persist), dim3(kPBlock), args,
                                   b->smem_persist, ctx->stream));
    return CLOTH_OK;
}

int launch_solve_host(Batch *b, int max_iters)
{
    cloth_ctx *ctx = b->ctx;
    cudaStream_t s = ctx->stream;
    if (b->persist_ok)
        return launch_persistent(b);
    cudaGraphConditionalHandle none = 0;
    int zero = 0;
    int *no_left = nullptr;
    void *a_spmv[] = {&b->d_descs, &b->d_rt, &b->d_ctl, &zero, &none};
    void *a_upd[] = {&b->d_descs, &b->d_rt, &b->d_ctl, &zero, &none, &no_left};
    int ninst = int(b->members.size());
    const int *no_count = nullptr;
    void *a_red[] = {&b->d_descs, &b->d_inst, &ninst, &no_count, &b->d_ctl, &zero, &none};
    const int gred = reduce_grid(ninst);
    const GraphLoopVariant &sv = b->spmv_variant(b->spmv_v);
    const GraphLoopVariant &uv = kUpdateVariants[b->upd_v];
    int *h_active = nullptr;
    CK(cudaMallocHost(&h_active, sizeof(int)));
    int rc = CLOTH_OK;
    const int chunk = 8;
    for (int it = 0; it < max_iters + chunk; it += chunk)
    {
        for (int k = 0; k < chunk; k++)
        {
            {
                PhaseTimer t(ctx, PH_SPMV);
                cudaLaunchKernel(sv.func, dim3(b->grid_spmv), dim3(spmv_block(sv)), a_spmv,
                                 b->smem_spmv, s);
            }
            {
                PhaseTimer t(ctx, PH_REDUCE);
                cudaLaunchKernel((const void *)k_reduce_pq, dim3(gred), dim3(kTile), a_red, 0, s);
            }
            {
                PhaseTimer t(ctx, PH_UPDATE);
                cudaLaunchKernel(uv.func, dim3(b->grid_update),
                                 dim3(kTile / uv.rows_per_thread), a_upd, 0, s);
            }
            {
                PhaseTimer t(ctx, PH_REDUCE);
                cudaLaunchKernel((const void *)k_reduce_rz, dim3(gred), dim3(kTile), a_red, 0, s);
            }
        }
        if (cudaMemcpyAsync(h_active, &b->d_ctl->n_active, sizeof(int),
                            cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
        {
            rc = fail(CLOTH_ERR_CUDA, "solve: readback failed");
            break;
        }
        if (*h_active <= 0)
            break;
    }
    cudaFreeHost(h_active);
    return rc;
}

int launch_advance(Batch *b)
{
    if (b->collide)
    {
        PhaseTimer t(b->ctx, PH_REPULSE);
        int rc = collide_repulse(b->members[0]);
        if (rc != CLOTH_OK)
            return rc;
    }
    PhaseTimer t(b->ctx, PH_ADVANCE);
    k_advance<<<b->grid_row, kTile, 0, b->ctx->stream>>>(b->d_descs, b->d_rt, b->d_ctl, 0);
    CK(cudaGetLastError());
    return CLOTH_OK;
}

int read_stats(Batch *b, cloth_solve_stats *stats)
{
    if (!stats)
        return CLOTH_OK;
    // every member's state and the set's control word: gathered on the
    // device, one copy back
    cudaStream_t s = b->ctx->stream;
    const int n = int(b->members.size());
    InstState *h_st = reinterpret_cast<InstState *>(b->h_pinned);
    BatchCtl *h_ctl = reinterpret_cast<BatchCtl *>(b->h_pinned + n * sizeof(InstState));
    k_snap_state<<<std::min(n, 1024), 64, 0, s>>>(b->d_descs, b->d_inst, n, b->d_states,
                                                   b->d_ctl, b->d_ctl_copy, 0);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h_st, b->d_states, n * sizeof(InstState), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h_ctl, b->d_ctl_copy, sizeof(BatchCtl), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    // a bounded wait of the graph-loop kernels that gave up (sticky: cleared here)
    const int ctl_err = h_ctl->err;
    if (ctl_err)
        CK(cudaMemset(&b->d_ctl->err, 0, sizeof(int)));
    for (int i = 0; i < n; i++)
    {
        const InstState &st = h_st[i];
        cloth_solve_stats &o = stats[i];
        o.iters = st.iter;
        // a bounded device wait that gave up flags the team (bar_err) or the set
        o.status = (st.bar_err || ctl_err) ? CLOTH_ERR_TIMEOUT : st.status;
        o.res_norm = std::sqrt(std::max(0.0, st.rr));
        o.rhs_norm = std::sqrt(std::max(0.0, st.bb));
        o.rel_residual = o.rhs_norm > 0 ? o.res_norm / o.rhs_norm : o.res_norm;
        o.solver = !b->persist_ok  ? CLOTH_SOLVER_GRAPH_LOOP
                   : b->persist_1b ? CLOTH_SOLVER_PERSISTENT_1B
                                   : CLOTH_SOLVER_PERSISTENT;
        if (b->collide && o.status == CLOTH_OK)
        {
            cloth_contact_stats cs;
            int rc = cloth_get_contacts(b->members[i], &cs, nullptr, nullptr, nullptr, nullptr);
            if (rc != CLOTH_OK)
                return rc;
            if (cs.overflow)
                o.status = CLOTH_ERR_CONTACTS;
        }
    }
    return CLOTH_OK;
}

int max_iters_of(const Batch *b)
{
    int m = 0;
    for (auto *c : b->members)
        m = std::max(m, c->h.max_iters);
    return m;
}

// Prepare every member for a step with dt and params.
int prepare(const std::vector<cloth_s *> &members, double dt,
            const cloth_solve_params *params, int hold_maxiter = 0)
{
    for (auto *c : members)
    {
        set_params(c, params, hold_maxiter);
        set_dt(c, dt);
        int rc = sync_pins(c);
        if (rc != CLOTH_OK)
            return rc;
        rc = sync_desc(c);
        if (rc != CLOTH_OK)
            return rc;
    }
    return CLOTH_OK;
}

// After a step the drag point is dropped (BaraffClothGpu.cpp:260-262).
void end_step(const std::vector<cloth_s *> &members)
{
    for (auto *c : members)
    {
        if (c->drag_vid >= 0)
        {
            c->drag_vid = -1;
            c->pins_dirty = true;
        }
        c->assembled = false;
        c->dx64_valid = false;
    }
}

// Autotuner of the graph-loop kernels: right after the assembly of a launch
// set's first step (PCG at iteration 0) every SpMV variant is timed on the
// real data - at iteration 0 the SpMV writes p = z and q = A z, the same every
// time, and adds its tile sums to the instance states, restored before each
// run - and every update variant is timed from a snapshot of the state it
// changes (dx, r, z, the instance states, the active count), restored after
// each run; the loop then starts from the states before the first SpMV. All variants compute bit-identical results, so the choice only moves
// the time. The fastest pair is kept for the launch set and becomes the
// context's default (the request server builds its chunks with it).
int autotune_graph_loop(Batch *b)
{
    cloth_ctx *ctx = b->ctx;
    cudaStream_t s = ctx->stream;
    const int ninst = int(b->members.size());
    float4 *rows = nullptr;
    InstState *sts = nullptr, *sts0 = nullptr;
    BatchCtl *ctl_buf = nullptr, *ctl0 = nullptr;
    CK(cudaMalloc(&rows, size_t(b->n_rt) * kTile * 3 * sizeof(float4)));
    CK(cudaMalloc(&sts, size_t(ninst) * sizeof(InstState)));
    CK(cudaMalloc(&sts0, size_t(ninst) * sizeof(InstState)));
    CK(cudaMalloc(&ctl_buf, sizeof(BatchCtl)));
    CK(cudaMalloc(&ctl0, sizeof(BatchCtl)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaGraphConditionalHandle none = 0;
    int zero = 0;
    int *no_left = nullptr;
    void *a_spmv[] = {&b->d_descs, &b->d_rt, &b->d_ctl, &zero, &none};
    void *a_upd[] = {&b->d_descs, &b->d_rt, &b->d_ctl, &zero, &none, &no_left};
    const int gsnap = std::max(1, std::min(b->n_rt, ctx->num_sms * 16));
    auto snap = [&](int restore) {
        k_snap_rows<<<gsnap, kTile, 0, s>>>(b->d_descs, b->d_rt, b->d_ctl, rows, restore);
        k_snap_state<<<std::max(1, std::min(ninst, 1024)), 64, 0, s>>>(
            b->d_descs, b->d_inst, ninst, sts, b->d_ctl, ctl_buf, restore);
    };
    // the instance states before the first SpMV (the SpMV adds its tile sums
    // to them, so every timed run starts from this copy)
    auto snap0 = [&](int restore) {
        k_snap_state<<<std::max(1, std::min(ninst, 1024)), 64, 0, s>>>(
            b->d_descs, b->d_inst, ninst, sts0, b->d_ctl, ctl0, restore);
    };
    snap0(0);
    auto time_launch = [&](const GraphLoopVariant &v, int grid, void **args,
                           unsigned smem = 0) -> float {
        cudaEventRecord(e0, s);
        cudaLaunchKernel(v.func, dim3(grid), dim3(spmv_block(v)), args, smem, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms;
    };
    const int kWaves[2] = {1, 8};
    int best_s = b->spmv_v, best_u = b->upd_v;
    float t_best = 1e30f;
    ctx->tune_ms_spmv.assign(kNumSpmvVariants, 0.f);
    ctx->tune_ms_update.assign(kNumUpdateVariants, 0.f);
    int best_sw = 8, best_uw = 8;
    for (int v = 0; v < kNumSpmvVariants; v++)
    {
        float tv = 1e30f;
        if (!b->spmv_usable(v))
        {
            ctx->tune_ms_spmv[v] = 0.f; // its stages do not fit in shared memory
            continue;
        }
        for (int wv : kWaves)
        {
            const int g = b->grid_for(b->spmv_variant(v), b->spmv_occ(v), wv);
            float t = 1e30f;
            for (int rep = 0; rep < 4; rep++)
            {
                snap0(1);
                const float ms = time_launch(b->spmv_variant(v), g, a_spmv, b->spmv_smem_of(v));
                if (rep > 0)
                    t = std::min(t, ms);
            }
            tv = std::min(tv, t);
            if (t < t_best)
            {
                t_best = t;
                best_s = v;
                best_sw = wv;
            }
        }
        ctx->tune_ms_spmv[v] = tv;
    }
    // the update variants run from the state after the first SpMV and p.q
    snap0(1);
    cudaLaunchKernel(b->spmv_variant(best_s).func,
                     dim3(b->grid_for(b->spmv_variant(best_s), b->spmv_occ(best_s), best_sw)),
                     dim3(spmv_block(b->spmv_variant(best_s))), a_spmv,
                     b->spmv_smem_of(best_s), s);
    {
        const int *no_count = nullptr;
        int ni = ninst;
        void *a_red[] = {&b->d_descs, &b->d_inst, &ni, &no_count, &b->d_ctl, &zero, &none};
        cudaLaunchKernel((const void *)k_reduce_pq, dim3(reduce_grid(ninst)), dim3(kTile), a_red,
                         0, s);
    }
    snap(0);
    t_best = 1e30f;
    for (int v = 0; v < kNumUpdateVariants; v++)
    {
        float tv = 1e30f;
        for (int wv : kWaves)
        {
            const int g = b->grid_for(kUpdateVariants[v], ctx->occ_update[v], wv);
            float t = 1e30f;
            for (int rep = 0; rep < 4; rep++)
            {
                snap(1);
                const float ms = time_launch(kUpdateVariants[v], g, a_upd);
                if (rep > 0)
                    t = std::min(t, ms);
            }
            tv = std::min(tv, t);
            if (t < t_best)
            {
                t_best = t;
                best_u = v;
                best_uw = wv;
            }
        }
        ctx->tune_ms_update[v] = tv;
    }
    // back to the state the loop starts from: the rows the SpMV leaves as they
    // are, the instance states before it
    snap(1);
    snap0(1);
    cudaError_t err = cudaStreamSynchronize(s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(rows);
    cudaFree(sts);
    cudaFree(sts0);
    cudaFree(ctl_buf);
    cudaFree(ctl0);
    if (err != cudaSuccess)
        return fail(CLOTH_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(err));
    b->set_variants(best_s, best_u, best_sw, best_uw);
    b->tuned = true;
    ctx->tune_spmv = best_s;
    ctx->tune_update = best_u;
    return CLOTH_OK;
}

// The end of a hand-off set's solve: the graph loop stopped once
// b->hand_off cloths or fewer still iterated; the persistent kernel (whose
// arithmetic is the graph loop's, bit for bit) finishes them from where they
// are.  Where those cloths do not fit one persistent launch, the graph loop
// runs on to the end instead.
int finish_tail(Batch *b)
{
    cloth_ctx *ctx = b->ctx;
    cudaStream_t s = ctx->stream;
    const int n = int(b->members.size());
    InstState *h_st = reinterpret_cast<InstState *>(b->h_pinned);
    k_snap_state<<<std::min(n, 1024), 64, 0, s>>>(b->d_descs, b->d_inst, n, b->d_states,
                                                   b->d_ctl, b->d_ctl_copy, 0);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h_st, b->d_states, n * sizeof(InstState), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<int> rest;
    for (int i = 0; i < n; i++)
        if (h_st[i].active)
            rest.push_back(i);
    if (rest.empty())
        return CLOTH_OK;
    // (a simulation whose slowest cloths keep changing would grow the cache
    // of tail launch sets without end: it is dropped past a few dozen)
    if (b->tails.size() >= 32 && b->tails.find(rest) == b->tails.end())
        b->tails.clear();
    std::unique_ptr<Batch> &tb = b->tails[rest];
    if (!tb)
    {
        std::vector<cloth_s *> sub;
        for (int i : rest)
            sub.push_back(b->members[size_t(i)]);
        int rc = make_batch(ctx, sub, tb);
        if (rc != CLOTH_OK)
            return rc;
    }
    if (tb->persist_ok && !tb->persist_1b)
        return launch_persistent(tb.get());
    // the loop to the end
    const int zero = 0;
    CK(cudaMemcpyAsync(&b->d_ctl->hand_off, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
    int rc = CLOTH_OK;
    if (!b->solve_exec)
        rc = build_graph(b, false, &b->solve_exec);
    if (rc == CLOTH_OK && cudaGraphLaunch(b->solve_exec, s) != cudaSuccess)
        rc = fail(CLOTH_ERR_CUDA, "cudaGraphLaunch failed");
    CK(cudaMemcpyAsync(&b->d_ctl->hand_off, &b->hand_off, sizeof(int), cudaMemcpyHostToDevice,
                       s));
    CK(cudaStreamSynchronize(s));
    return rc;
}

int run_step(Batch *b, double dt, const cloth_solve_params *params,
             cloth_solve_stats *stats)
{
    cloth_ctx *ctx = b->ctx;
    for (auto *c : b->members)
    {
        c->plain_host_valid = false;
        c->escalated_valid = false;
    }
    // a step that escalates solves ending at max_iters keeps their state
    const bool escalating = stats && ctx->escalate > 0 && !b->collide;
    int rc = prepare(b->members, dt, params, escalating && ctx->escalate >= 2 ? 1 : 0);
    if (rc != CLOTH_OK)
        return rc;
    if (ctx->prof)
    {
        rc = launch_assemble(b);
        if (rc == CLOTH_OK)
            rc = launch_solve_host(b, max_iters_of(b));
        if (rc == CLOTH_OK)
            rc = launch_advance(b);
    }
    else if (b->collide)
    {
        // contacts and repulsion around the solve: host-driven launches on
        // the stream (the counts stay on the device)
        rc = launch_assemble(b);
        if (rc == CLOTH_OK && b->persist_ok)
            rc = launch_persistent(b);
        else if (rc == CLOTH_OK)
        {
            if (!b->solve_exec)
                rc = build_graph(b, false, &b->solve_exec);
            if (rc == CLOTH_OK && cudaGraphLaunch(b->solve_exec, ctx->stream) != cudaSuccess)
                rc = fail(CLOTH_ERR_CUDA, "cudaGraphLaunch failed");
        }
        if (rc == CLOTH_OK)
            rc = launch_advance(b);
    }
    else if (!b->persist_ok && !b->tuned && ctx->autotune)
    {
        // first step of a graph-loop launch set: assemble, tune on the real
        // system, then solve and advance with the chosen kernels
        rc = launch_assemble(b);
        if (rc == CLOTH_OK)
            rc = autotune_graph_loop(b);
        if (rc == CLOTH_OK && !b->solve_exec)
            rc = build_graph(b, false, &b->solve_exec);
        if (rc == CLOTH_OK && cudaGraphLaunch(b->solve_exec, ctx->stream) != cudaSuccess)
            rc = fail(CLOTH_ERR_CUDA, "cudaGraphLaunch failed");
        if (rc == CLOTH_OK && b->hand_off > 0)
            rc = finish_tail(b);
        if (rc == CLOTH_OK)
            rc = launch_advance(b);
    }
    else
    {
        if (!b->step_exec)
        {
            rc = build_graph(b, true, &b->step_exec);
            if (rc != CLOTH_OK)
                return rc;
        }
        CK(cudaGraphLaunch(b->step_exec, ctx->stream));
        // (a hand-off set's graph ends with the loop)
        if (b->hand_off > 0)
        {
            rc = finish_tail(b);
            if (rc == CLOTH_OK)
                rc = launch_advance(b);
        }
    }
    if (rc != CLOTH_OK)
        return rc;
    if (!stats)
    {
        // asynchronous step: no escalation (a failed solve leaves the state)
        end_step(b->members);
        return CLOTH_OK;
    }
    rc = read_stats(b, stats);
    // precision escalation: a member whose FP32 PCG ended in NaN or breakdown
    // kept its pre-step state and assembled system (the advance skipped it);
    // re-solve it in FP64 and advance
    if (rc == CLOTH_OK && escalating)
    {
        const cloth_solve_params p = params ? *params : default_params();
        for (size_t i = 0; i < b->members.size() && rc == CLOTH_OK; i++)
            if (stats[i].status == CLOTH_ERR_NAN || stats[i].status == CLOTH_ERR_BREAKDOWN ||
                (ctx->escalate >= 2 && stats[i].status == CLOTH_ERR_MAXITER))
            {
                cloth_s *c = b->members[i];
                c->assembled = true; // this step's system is still in its work arrays
                rc = escalate_step(c, &p, &stats[i]);
                if (rc == CLOTH_OK)
                {
                    c->escalated = stats[i];
                    c->escalated_valid = true;
                }
            }
    }
    end_step(b->members);
    return rc;
}

Batch *self_batch(cloth_s *c, int *rc)
{
    *rc = CLOTH_OK;
    if (!c->self)
        *rc = make_batch(c->ctx, {c}, c->self);
    return c->self.get();
}

} // namespace

int cloth::detail::inner_solve(cloth_s *c, const double *rhs64, const cloth_solve_params *p,
                               cloth_solve_stats *stats)
{
    int rc;
    Batch *b = self_batch(c, &rc);
    if (rc != CLOTH_OK)
        return rc;
    set_params(c, p);
    rc = sync_desc(c);
    if (rc != CLOTH_OK)
        return rc;
    cudaStream_t s = c->ctx->stream;
    CK(cudaMemsetAsync(&b->d_ctl->n_active, 0, sizeof(int), s));
    k_ir_start<<<b->grid_row, kTile, 0, s>>>(b->d_descs, b->d_rt, b->d_ctl, rhs64);
    CK(cudaGetLastError());
    if (c->ctx->prof)
        rc = launch_solve_host(b, c->h.max_iters);
    else
    {
        if (!b->solve_exec)
            rc = build_graph(b, false, &b->solve_exec);
        if (rc == CLOTH_OK && cudaGraphLaunch(b->solve_exec, s) != cudaSuccess)
            rc = fail(CLOTH_ERR_CUDA, "cudaGraphLaunch failed");
    }
    if (rc != CLOTH_OK)
        return rc;
    return read_stats(b, stats);
}

namespace {

bool valid_params(const cloth_solve_params *p)
{
    return !p || (p->max_iters >= 0 && p->max_iters <= 100000000 &&
                  p->rel_tol >= 0 && p->abs_tol >= 0);
}

} // namespace

namespace cloth {
// Lets other translation units of the library report through cloth_last_error().
void set_last_error(const std::string &msg) { g_err = msg; }
} // namespace cloth

// ====================================================================== ABI
extern "C" {

int cloth_abi_version(void) { return CLOTH_ABI_VERSION; }

const char *cloth_last_error(void) { return g_err.c_str(); }

const char *cloth_status_string(int s)
{
    switch (s)
    {
    case CLOTH_OK: return "ok";
    case CLOTH_ERR_INVALID: return "invalid argument";
    case CLOTH_ERR_CUDA: return "CUDA error";
    case CLOTH_ERR_OOM: return "out of device memory";
    case CLOTH_ERR_BUDGET: return "device-memory budget exceeded";
    case CLOTH_ERR_MESH: return "unsupported mesh";
    case CLOTH_ERR_NAN: return "NaN or Inf in the solve";
    case CLOTH_ERR_BREAKDOWN: return "PCG breakdown (zero denominator)";
    case CLOTH_ERR_MAXITER: return "PCG stopped at max_iters";
    case CLOTH_ERR_TIMEOUT: return "device wait timed out";
    case CLOTH_ERR_UNSUPPORTED: return "unsupported";
    case CLOTH_ERR_STATE: return "call out of order";
    case CLOTH_ERR_CONTACTS: return "contact lists exceeded their capacity";
    default: return "unknown status";
    }
}

int cloth_ctx_create(int device, cloth_ctx **out)
{
    if (!out)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_create: out is NULL");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    {
        cudaGetLastError();
        return fail(CLOTH_ERR_CUDA, "cloth_ctx_create: no CUDA device");
    }
    if (device < 0 || device >= ndev)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_create: bad device index");
    CK(cudaSetDevice(device));
    auto c = std::make_unique<cloth_ctx>();
    c->device = device;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
    CK(cudaDeviceGetAttribute(&c->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                              device));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c->occ_tri, k_tri, kTile, 0));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c->occ_row, k_row, kTile, 0));
    c->occ_spmv.assign(kNumSpmvVariants, 1);
    c->occ_update.assign(kNumUpdateVariants, 1);
    c->occ_spmv_skew.assign(kNumSpmvVariants, 1);
    for (int v = 0; v < kNumSpmvVariants; v++)
    {
        for (const GraphLoopVariant *tab : {kSpmvVariants, kSpmvSkewVariants})
            if (tab[v].bulk_stages)
                CK(cudaFuncSetAttribute(tab[v].func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        c->max_smem_optin - int(kBulkStaticReserve)));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &c->occ_spmv[v], kSpmvVariants[v].func, spmv_block(kSpmvVariants[v]), 0));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &c->occ_spmv_skew[v], kSpmvSkewVariants[v].func, spmv_block(kSpmvSkewVariants[v]),
            0));
    }
    for (int v = 0; v < kNumUpdateVariants; v++)
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &c->occ_update[v], kUpdateVariants[v].func,
            kTile / kUpdateVariants[v].rows_per_thread, 0));
    *out = c.release();
    return CLOTH_OK;
}

int cloth_ctx_destroy(cloth_ctx *ctx)
{
    if (!ctx)
        return CLOTH_OK;
    // servers first, without the context lock: their worker threads take it
    cudaSetDevice(ctx->device);
    for (auto *sv : std::vector<cloth_server_s *>(ctx->servers))
        server_teardown(sv);
    ctx->servers.clear();
    {
        std::lock_guard<std::recursive_mutex> lk(ctx->mu);
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        ctx->last_batch.reset();
        for (auto *c : std::vector<cloth_s *>(ctx->cloths))
        {
            c->self.reset();
            f64_free(c);
            collide_free(c);
            if (c->arena)
                cudaFree(c->arena);
            if (c->scratch)
                cudaFree(c->scratch);
            delete c;
        }
        ctx->cloths.clear();
        body_release_all(ctx);
        for (auto &p : ctx->ev_pending)
        {
            cudaEventDestroy(p.second.first);
            cudaEventDestroy(p.second.second);
        }
        for (auto e : ctx->ev_pool)
            cudaEventDestroy(e);
        cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
    return CLOTH_OK;
}

int cloth_ctx_synchronize(cloth_ctx *ctx)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "ctx is NULL");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    CK(cudaStreamSynchronize(ctx->stream));
    return CLOTH_OK;
}

int cloth_ctx_set_profiling(cloth_ctx *ctx, int enable)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "ctx is NULL");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    drain_profile(ctx);
    ctx->prof = enable != 0;
    return CLOTH_OK;
}

int cloth_ctx_get_profile(cloth_ctx *ctx, double *ms_total, long long *launches)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "ctx is NULL");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    drain_profile(ctx);
    for (int k = 0; k < CLOTH_NUM_PHASES; k++)
    {
        if (ms_total)
            ms_total[k] = ctx->prof_ms[k];
        if (launches)
            launches[k] = ctx->prof_n[k];
    }
    return CLOTH_OK;
}

int cloth_ctx_reset_profile(cloth_ctx *ctx)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "ctx is NULL");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    drain_profile(ctx);
    for (int k = 0; k < CLOTH_NUM_PHASES; k++)
    {
        ctx->prof_ms[k] = 0;
        ctx->prof_n[k] = 0;
    }
    return CLOTH_OK;
}

int cloth_ctx_set_tail_hand_off(cloth_ctx *ctx, int max_instances)
{
    if (!ctx || max_instances < -1)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_set_tail_hand_off: bad argument");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    ctx->tail_hand_off = max_instances;
    ctx->last_batch.reset();
    return CLOTH_OK;
}

int cloth_ctx_set_solver(cloth_ctx *ctx, int solver)
{
    if (!ctx || (solver != CLOTH_SOLVER_PERSISTENT && solver != CLOTH_SOLVER_GRAPH_LOOP &&
                 solver != CLOTH_SOLVER_PERSISTENT_1B && solver != CLOTH_SOLVER_PERSISTENT_2B))
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_set_solver: bad argument");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    cudaStreamSynchronize(ctx->stream);
    ctx->solver = solver;
    ctx->last_batch.reset();
    for (auto *c : ctx->cloths)
        c->self.reset();
    return CLOTH_OK;
}

int cloth_ctx_set_escalation(cloth_ctx *ctx, int enable)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_set_escalation: NULL context");
    if (enable < 0 || enable > 2)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_set_escalation: level must be 0, 1 or 2");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    ctx->escalate = enable;
    return CLOTH_OK;
}

int cloth_ctx_set_spin_limit(cloth_ctx *ctx, unsigned polls, unsigned extra_arrivals)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_set_spin_limit: NULL context");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    cudaStreamSynchronize(ctx->stream);
    ctx->spin.limit = polls ? polls : kSpinLimitDefault;
    ctx->spin.extra = extra_arrivals;
    // launch sets carry the setting in their kernel arguments: rebuild them
    ctx->last_batch.reset();
    for (auto *c : ctx->cloths)
        c->self.reset();
    return CLOTH_OK;
}

int cloth_ctx_set_kernel_variant(cloth_ctx *ctx, int spmv_r, int spmv_u, int spmv_tpb,
                                 int upd_r, int upd_tpb, int autotune)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_set_kernel_variant: NULL context");
    int sv = -1, uv = -1;
    for (int v = 0; v < kNumSpmvVariants; v++)
        if (kSpmvVariants[v].rows_per_thread == spmv_r && kSpmvVariants[v].slot_unroll == spmv_u &&
            kSpmvVariants[v].tiles_per_block == spmv_tpb)
            sv = v;
    for (int v = 0; v < kNumUpdateVariants; v++)
        if (kUpdateVariants[v].rows_per_thread == upd_r &&
            kUpdateVariants[v].tiles_per_block == upd_tpb)
            uv = v;
    if (sv < 0 || uv < 0)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_set_kernel_variant: no such variant");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    ctx->tune_spmv = sv;
    ctx->tune_update = uv;
    ctx->autotune = autotune != 0;
    ctx->last_batch.reset();
    for (auto *c : ctx->cloths)
        c->self.reset();
    return CLOTH_OK;
}

int cloth_ctx_get_kernel_variant(cloth_ctx *ctx, int *spmv_r, int *spmv_u, int *spmv_tpb,
                                 int *upd_r, int *upd_tpb, int *autotune)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_get_kernel_variant: NULL context");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (spmv_r)
        *spmv_r = kSpmvVariants[ctx->tune_spmv].rows_per_thread;
    if (spmv_u)
        *spmv_u = kSpmvVariants[ctx->tune_spmv].slot_unroll;
    if (spmv_tpb)
        *spmv_tpb = kSpmvVariants[ctx->tune_spmv].tiles_per_block;
    if (upd_r)
        *upd_r = kUpdateVariants[ctx->tune_update].rows_per_thread;
    if (upd_tpb)
        *upd_tpb = kUpdateVariants[ctx->tune_update].tiles_per_block;
    if (autotune)
        *autotune = ctx->autotune ? 1 : 0;
    return CLOTH_OK;
}

int cloth_ctx_get_tuning_times(cloth_ctx *ctx, float *spmv_ms, int n_spmv, float *update_ms,
                               int n_update)
{
    if (!ctx)
        return fail(CLOTH_ERR_INVALID, "cloth_ctx_get_tuning_times: NULL context");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    for (int v = 0; v < n_spmv && spmv_ms; v++)
        spmv_ms[v] = v < int(ctx->tune_ms_spmv.size()) ? ctx->tune_ms_spmv[v] : 0.f;
    for (int v = 0; v < n_update && update_ms; v++)
        update_ms[v] = v < int(ctx->tune_ms_update.size()) ? ctx->tune_ms_update[v] : 0.f;
    return CLOTH_OK;
}

int cloth_ctx_device_bytes(cloth_ctx *ctx, size_t *bytes)
{
    if (!ctx || !bytes)
        return fail(CLOTH_ERR_INVALID, "NULL argument");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    *bytes = ctx->bytes;
    return CLOTH_OK;
}

int cloth_ctx_get_stream(cloth_ctx *ctx, void **stream)
{
    if (!ctx || !stream)
        return fail(CLOTH_ERR_INVALID, "NULL argument");
    *stream = reinterpret_cast<void *>(ctx->stream);
    return CLOTH_OK;
}

static void copy_out_mesh(const Mesh &m, int *nv, int *nt, int *ne, double *pos, float *uv,
                          int *tris, int *edges)
{
    if (nv)
        *nv = m.nv;
    if (nt)
        *nt = m.nt;
    if (ne)
        *ne = m.ne;
    if (pos)
        std::memcpy(pos, m.pos.data(), m.pos.size() * sizeof(double));
    if (uv)
        std::memcpy(uv, m.uv.data(), m.uv.size() * sizeof(float));
    if (tris)
        std::memcpy(tris, m.tris.data(), m.tris.size() * sizeof(int));
    if (edges)
        std::memcpy(edges, m.edges.data(), m.edges.size() * sizeof(int));
}

int cloth_mesh_from_obj(const char *path, const double *translation, int relocate, int *nv,
                        int *nt, int *ne, double *pos, float *uv, int *tris, int *edges)
{
    if (!path)
        return fail(CLOTH_ERR_INVALID, "cloth_mesh_from_obj: path is NULL");
    const double zero[3] = {0.0, 0.0, 0.0};
    Mesh m;
    std::string err;
    if (!load_obj_cloth(path, translation ? translation : zero, relocate != 0, m, err))
        return fail(CLOTH_ERR_MESH, err);
    copy_out_mesh(m, nv, nt, ne, pos, uv, tris, edges);
    return CLOTH_OK;
}

int cloth_grid_build(const cloth_grid_desc *grid, int *nv, int *nt, int *ne,
                     double *pos, float *uv, int *tris, int *edges)
{
    if (!grid)
        return fail(CLOTH_ERR_INVALID, "grid is NULL");
    GridDesc g;
    std::memcpy(g.size, grid->cloth_size, sizeof(g.size));
    std::memcpy(g.subdiv, grid->subdivision, sizeof(g.subdiv));
    std::memcpy(g.init_pos, grid->init_pos, sizeof(g.init_pos));
    g.uv_rotation_deg = grid->uv_rotation_deg;
    Mesh m;
    std::string err;
    if (!build_grid(g, m, err))
        return fail(CLOTH_ERR_INVALID, err);
    copy_out_mesh(m, nv, nt, ne, pos, uv, tris, edges);
    return CLOTH_OK;
}

int cloth_geometry_build(const cloth_grid_desc *grid, const char *geometry_type,
                         unsigned long long seed, int *nv, int *nt, int *ne, double *pos,
                         float *uv, int *tris, int *edges)
{
    if (!grid || !geometry_type)
        return fail(CLOTH_ERR_INVALID, "cloth_geometry_build: NULL argument");
    GridDesc g;
    std::memcpy(g.size, grid->cloth_size, sizeof(g.size));
    std::memcpy(g.subdiv, grid->subdivision, sizeof(g.subdiv));
    std::memcpy(g.init_pos, grid->init_pos, sizeof(g.init_pos));
    g.uv_rotation_deg = grid->uv_rotation_deg;
    const std::string type(geometry_type);
    Mesh m;
    std::string err;
    bool ok;
    if (type == "regular_triangle")
        ok = build_grid(g, m, err);
    else if (type == "regular_triangle_perturb")
        ok = perturb_grid(g, seed, m, err);
    else if (type == "delaunay")
        ok = delaunay_cloth(g, seed, m, err);
    else
        return fail(CLOTH_ERR_UNSUPPORTED, "cloth_geometry_build: unknown geometry_type '" +
                                               type + "'");
    if (!ok)
        return fail(CLOTH_ERR_INVALID, err);
    copy_out_mesh(m, nv, nt, ne, pos, uv, tris, edges);
    return CLOTH_OK;
}

static bool copy_mesh(const cloth_mesh_desc *mesh, Mesh &m, std::string &err)
{
    if (!mesh || mesh->nv <= 0 || mesh->nt <= 0 || !mesh->pos || !mesh->uv ||
        !mesh->tris || mesh->ne < 0 || (mesh->ne > 0 && !mesh->edges))
    {
        err = "bad mesh description";
        return false;
    }
    m.nv = mesh->nv;
    m.nt = mesh->nt;
    m.pos.assign(mesh->pos, mesh->pos + size_t(m.nv) * 3);
    m.uv.assign(mesh->uv, mesh->uv + size_t(m.nv) * 2);
    m.tris.assign(mesh->tris, mesh->tris + size_t(m.nt) * 3);
    if (mesh->ne > 0)
    {
        m.ne = mesh->ne;
        m.edges.assign(mesh->edges, mesh->edges + size_t(m.ne) * 4);
        return true;
    }
    return derive_edges(m, err);
}

static void copy_material(const cloth_material *mat, Material &mt)
{
    std::memcpy(mt.stretch_k, mat->stretch_k, sizeof(mt.stretch_k));
    std::memcpy(mt.bending_k, mat->bending_k, sizeof(mt.bending_k));
    mt.density = mat->density;
    mt.rayleigh_a = mat->rayleigh_a;
    mt.rayleigh_b = mat->rayleigh_b;
    mt.default_timestep = mat->default_timestep;
    mt.gravity = mat->gravity;
    mt.fix_fv_norm = mat->fix_fv_norm;
    mt.bending_model = mat->bending_model;
}

int cloth_host_tables(const cloth_mesh_desc *mesh, const cloth_material *mat,
                      int *ne, int *width, int *ell, int *stencil, float *coef,
                      float *area, double *mass, float *kbend, int *tri_slot)
{
    if (!mesh || !mat)
        return fail(CLOTH_ERR_INVALID, "cloth_host_tables: NULL argument");
    Mesh m;
    Material mt;
    Tables t;
    std::string err;
    if (!copy_mesh(mesh, m, err))
        return fail(CLOTH_ERR_MESH, err);
    copy_material(mat, mt);
    if (!build_tables(m, mt, t, err))
        return fail(CLOTH_ERR_MESH, err);
    const int R = CLOTH_ELL_REF_WIDTH;
    if (ne)
        *ne = m.ne;
    if (width)
        *width = t.width;
    for (int v = 0; v < t.nv; v++)
    {
        const int len = t.rowptr[v + 1] - t.rowptr[v];
        for (int s = 0; s < R; s++)
        {
            const size_t k = size_t(t.rowptr[v]) + s;
            if (ell)
                ell[size_t(v) * R + s] = s < len ? t.cols[k] : -1;
            if (kbend)
                kbend[size_t(v) * R + s] = s < len ? t.kbend[k] : 0.f;
        }
    }
    if (stencil)
        std::memcpy(stencil, t.stencil.data(), t.stencil.size() * sizeof(int));
    if (coef)
        std::memcpy(coef, t.coef.data(), t.coef.size() * sizeof(float));
    if (area)
        std::memcpy(area, t.area.data(), t.area.size() * sizeof(float));
    if (mass)
        std::memcpy(mass, t.mass.data(), t.mass.size() * sizeof(double));
    if (tri_slot)
        std::memcpy(tri_slot, t.tri_slot.data(), t.tri_slot.size() * sizeof(int));
    return CLOTH_OK;
}

int cloth_create(cloth_ctx *ctx, const cloth_mesh_desc *mesh,
                 const cloth_material *mat, cloth_t **out)
{
    if (!ctx || !mesh || !mat || !out)
        return fail(CLOTH_ERR_INVALID, "cloth_create: NULL argument");
    *out = nullptr;
    if (mesh->nv <= 0 || mesh->nt <= 0 || !mesh->pos || !mesh->uv || !mesh->tris ||
        (mesh->ne > 0 && !mesh->edges) || mesh->ne < 0)
        return fail(CLOTH_ERR_INVALID, "cloth_create: bad mesh description");
    if (!(mat->density > 0) || !(mat->default_timestep > 0))
        return fail(CLOTH_ERR_INVALID, "cloth_create: density and timestep must be > 0");
    auto c = std::make_unique<cloth_s>();
    c->ctx = ctx;
    Mesh &m = c->mesh;
    std::string err;
    if (!copy_mesh(mesh, m, err))
        return fail(CLOTH_ERR_MESH, err);
    Material &mt = c->mat;
    copy_material(mat, mt);
    // host tables outside the context lock: threads may create cloths in parallel
    if (!build_tables(m, mt, c->tab, err))
        return fail(CLOTH_ERR_MESH, err);
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    CK(cudaSetDevice(ctx->device));
    int rc = upload_tables(c.get());
    if (rc != CLOTH_OK)
    {
        if (c->arena)
            cudaFree(c->arena);
        if (c->scratch)
            cudaFree(c->scratch);
        return rc;
    }
    set_material_fields(c.get());
    set_params(c.get(), nullptr);
    set_dt(c.get(), mt.default_timestep);
    rc = sync_desc(c.get());
    if (rc != CLOTH_OK)
    {
        cudaFree(c->arena);
        cudaFree(c->scratch);
        return rc;
    }
    ctx->bytes += c->arena_bytes + c->scratch_bytes;
    ctx->cloths.push_back(c.get());
    *out = c.release();
    return CLOTH_OK;
}

int cloth_destroy(cloth_t *c)
{
    if (!c)
        return CLOTH_OK;
    cloth_ctx *ctx = c->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (c->server)
        return fail(CLOTH_ERR_STATE, "cloth_destroy: the cloth is held by a server "
                                     "(destroy the server first)");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->last_batch)
        for (auto *m : ctx->last_batch->members)
            if (m == c)
            {
                ctx->last_batch.reset();
                break;
            }
    c->self.reset();
    f64_free(c);
    collide_free(c);
    if (c->arena)
        cudaFree(c->arena);
    if (c->scratch)
        cudaFree(c->scratch);
    ctx->bytes -= c->arena_bytes + c->scratch_bytes;
    ctx->cloths.erase(std::remove(ctx->cloths.begin(), ctx->cloths.end(), c),
                      ctx->cloths.end());
    delete c;
    return CLOTH_OK;
}

int cloth_matrix_info(const cloth_t *c, long long *nnzb, int *width, size_t *resident_bytes,
                      size_t *solve_bytes)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    if (nnzb)
        *nnzb = (long long)c->tab.cols.size();
    if (width)
        *width = c->tab.width;
    if (resident_bytes)
        *resident_bytes = c->arena_bytes;
    if (solve_bytes)
        *solve_bytes = c->sl.bytes;
    return CLOTH_OK;
}

int cloth_num_vertices(const cloth_t *c, int *nv, int *nt, int *ne)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    if (nv)
        *nv = c->mesh.nv;
    if (nt)
        *nt = c->mesh.nt;
    if (ne)
        *ne = c->mesh.ne;
    return CLOTH_OK;
}

int cloth_set_material(cloth_t *c, const cloth_material *mat)
{
    if (!c || !mat)
        return fail(CLOTH_ERR_INVALID, "NULL argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    CK(cudaSetDevice(c->ctx->device));
    Material &mt = c->mat;
    if (mat->bending_model != mt.bending_model)
        return fail(CLOTH_ERR_INVALID,
                    "cloth_set_material: the bending model is fixed when the cloth is created");
    bool bend = mt.bending_k[0] != mat->bending_k[0] || mt.bending_k[1] != mat->bending_k[1];
    std::memcpy(mt.stretch_k, mat->stretch_k, sizeof(mt.stretch_k));
    std::memcpy(mt.bending_k, mat->bending_k, sizeof(mt.bending_k));
    mt.rayleigh_a = mat->rayleigh_a;
    mt.rayleigh_b = mat->rayleigh_b;
    mt.fix_fv_norm = mat->fix_fv_norm;
    if (mat->default_timestep > 0)
        mt.default_timestep = mat->default_timestep;
    if (bend)
    {
        rebuild_bending(c->mesh, mt, c->tab);
        const Tables &t = c->tab;
        std::vector<float> kb(size_t(t.width) * c->h.stride, 0.f);
        for (int v = 0; v < t.nv; v++)
            for (int s = 0; s < t.rowptr[v + 1] - t.rowptr[v]; s++)
                kb[size_t(s) * c->h.stride + v] = t.kbend[size_t(t.rowptr[v]) + s];
        CK(cudaMemcpy(const_cast<float *>(c->h.kb), kb.data(), kb.size() * sizeof(float),
                      cudaMemcpyHostToDevice));
        if (mt.bending_model == 1 && c->tab.n_dih > 0)
        {
            rebuild_dihedral_factor(c->mesh, mt, c->tab);
            CK(cudaMemcpy(const_cast<double *>(c->h.dfac), c->tab.dih_factor.data(),
                          c->tab.dih_factor.size() * sizeof(double), cudaMemcpyHostToDevice));
        }
    }
    set_material_fields(c);
    c->dt_set = -1.0; // damping may have changed
    return CLOTH_OK;
}

int cloth_find_vertices_from_uv(const cloth_t *c, const float *uv, int n, int *vids)
{
    if (!c || (n > 0 && (!uv || !vids)) || n < 0)
        return fail(CLOTH_ERR_INVALID, "bad argument");
    find_vertices_from_uv(c->mesh, uv, n, vids);
    return CLOTH_OK;
}

int cloth_add_static_vertices(cloth_t *c, const int *vids, int n)
{
    if (!c || n < 0 || (n > 0 && !vids))
        return fail(CLOTH_ERR_INVALID, "bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    for (int k = 0; k < n; k++)
        if (vids[k] < 0 || vids[k] >= c->mesh.nv)
            return fail(CLOTH_ERR_INVALID, "static vertex id out of range");
    for (int k = 0; k < n; k++)
        if (std::find(c->static_pins.begin(), c->static_pins.end(), vids[k]) ==
            c->static_pins.end())
            c->static_pins.push_back(vids[k]);
    c->pins_dirty = true;
    return CLOTH_OK;
}

int cloth_clear_static_vertices(cloth_t *c)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    c->static_pins.clear();
    c->pins_dirty = true;
    return CLOTH_OK;
}

int cloth_get_static_vertices(const cloth_t *c, int *vids, int cap, int *n)
{
    if (!c || !n)
        return fail(CLOTH_ERR_INVALID, "bad argument");
    *n = int(c->static_pins.size());
    for (int k = 0; k < std::min(cap, *n) && vids; k++)
        vids[k] = c->static_pins[k];
    return CLOTH_OK;
}

int cloth_set_drag_point(cloth_t *c, int vid, const float target[3])
{
    if (!c || !target || vid < 0 || vid >= c->mesh.nv)
        return fail(CLOTH_ERR_INVALID, "bad drag point");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    c->drag_vid = vid;
    std::memcpy(c->drag_tgt, target, sizeof(c->drag_tgt));
    c->pins_dirty = true;
    return CLOTH_OK;
}

static int set_state(cloth_t *c, const double *x, int nv, bool pre)
{
    if (!c || !x || nv != c->mesh.nv)
        return fail(CLOTH_ERR_INVALID, "set_pos: bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    if (c->server && server_busy(c->server, c))
        return fail(CLOTH_ERR_STATE, "set_pos: the cloth has server requests in flight");
    CK(cudaSetDevice(c->ctx->device));
    cudaStream_t s = c->ctx->stream;
    CK(cudaMemcpyAsync(pre ? c->h.xp64 : c->h.x64, x, size_t(nv) * 3 * sizeof(double),
                       cudaMemcpyHostToDevice, s));
    if (!pre)
        k_sync_x32<<<std::min(1024, (nv + 255) / 256), 256, 0, s>>>(c->d_desc);
    CK(cudaGetLastError());
    c->assembled = false;
    c->plain_host_valid = false;
    return CLOTH_OK;
}

int cloth_set_pos(cloth_t *c, const double *x, int nv) { return set_state(c, x, nv, false); }
int cloth_set_pre_pos(cloth_t *c, const double *x, int nv) { return set_state(c, x, nv, true); }

static int get_state(cloth_t *c, double *x, int nv, bool pre)
{
    if (!c || !x || nv != c->mesh.nv)
        return fail(CLOTH_ERR_INVALID, "get_pos: bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    if (c->server && server_busy(c->server, c))
        return fail(CLOTH_ERR_STATE, "get_pos: the cloth has server requests in flight");
    CK(cudaSetDevice(c->ctx->device));
    cudaStream_t s = c->ctx->stream;
    CK(cudaMemcpyAsync(x, pre ? c->h.xp64 : c->h.x64, size_t(nv) * 3 * sizeof(double),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return CLOTH_OK;
}

int cloth_get_pos(cloth_t *c, double *x, int nv) { return get_state(c, x, nv, false); }
int cloth_get_pre_pos(cloth_t *c, double *x, int nv) { return get_state(c, x, nv, true); }

int cloth_reset(cloth_t *c)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    int rc = cloth_set_pos(c, c->mesh.pos.data(), c->mesh.nv);
    if (rc == CLOTH_OK)
        rc = cloth_set_pre_pos(c, c->mesh.pos.data(), c->mesh.nv);
    if (rc != CLOTH_OK)
        return rc;
    CK(cudaMemsetAsync(c->h.dx, 0, size_t(c->mesh.nv) * sizeof(float4), c->ctx->stream));
    CK(cudaStreamSynchronize(c->ctx->stream));
    return CLOTH_OK;
}

int cloth_step(cloth_t *c, double dt, const cloth_solve_params *params,
               cloth_solve_stats *stats)
{
    if (!c || !valid_params(params))
        return fail(CLOTH_ERR_INVALID, "cloth_step: bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    CK(cudaSetDevice(c->ctx->device));
    int rc;
    Batch *b = self_batch(c, &rc);
    if (rc != CLOTH_OK)
        return rc;
    return run_step(b, dt, params, stats);
}

int cloth_step_host(cloth_t *c, double dt, const cloth_solve_params *params,
                    const double *x_in, const double *x_pre_in, double *x_out,
                    cloth_solve_stats *stats)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    int rc = CLOTH_OK;
    if (x_in)
        rc = cloth_set_pos(c, x_in, c->mesh.nv);
    if (rc == CLOTH_OK && x_pre_in)
        rc = cloth_set_pre_pos(c, x_pre_in, c->mesh.nv);
    if (rc == CLOTH_OK)
        rc = cloth_step(c, dt, params, stats);
    if (rc == CLOTH_OK && x_out)
        rc = cloth_get_pos(c, x_out, c->mesh.nv);
    return rc;
}

int cloth_assemble(cloth_t *c, double dt)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    CK(cudaSetDevice(c->ctx->device));
    int rc;
    Batch *b = self_batch(c, &rc);
    if (rc != CLOTH_OK)
        return rc;
    set_dt(c, dt);
    rc = sync_pins(c);
    if (rc == CLOTH_OK)
        rc = sync_desc(c);
    if (rc == CLOTH_OK)
        rc = launch_assemble(b);
    if (rc == CLOTH_OK)
    {
        c->assembled = true;
        c->dx64_valid = false;
        c->pcg_stale = false;
    }
    return rc;
}

int cloth_solve(cloth_t *c, const cloth_solve_params *params, cloth_solve_stats *stats)
{
    if (!c || !valid_params(params))
        return fail(CLOTH_ERR_INVALID, "cloth_solve: bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    if (!c->assembled)
        return fail(CLOTH_ERR_STATE, "cloth_solve: call cloth_assemble first");
    if (c->pcg_stale)
        return fail(CLOTH_ERR_STATE, "cloth_solve: a refined or FP64 solve replaced the PCG "
                                     "start; call cloth_assemble again");
    CK(cudaSetDevice(c->ctx->device));
    int rc;
    Batch *b = self_batch(c, &rc);
    if (rc != CLOTH_OK)
        return rc;
    // The PCG start (r0, z0, rho0) was formed by the assembly with the
    // parameters current then; max_iters / tolerances apply from here on.
    set_params(c, params);
    rc = sync_desc(c);
    if (rc != CLOTH_OK)
        return rc;
    c->dx64_valid = false;
    if (c->ctx->prof)
        rc = launch_solve_host(b, c->h.max_iters);
    else
    {
        if (!b->solve_exec)
            rc = build_graph(b, false, &b->solve_exec);
        if (rc == CLOTH_OK && cudaGraphLaunch(b->solve_exec, c->ctx->stream) != cudaSuccess)
            rc = fail(CLOTH_ERR_CUDA, "cudaGraphLaunch failed");
    }
    if (rc != CLOTH_OK)
        return rc;
    return read_stats(b, stats);
}

int cloth_advance(cloth_t *c)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    CK(cudaSetDevice(c->ctx->device));
    int rc;
    Batch *b = self_batch(c, &rc);
    if (rc != CLOTH_OK)
        return rc;
    // the FP64 result of a refined or FP64 solve, else the FP32 dx
    rc = c->dx64_valid ? f64_advance(c) : launch_advance(b);
    end_step({c});
    return rc;
}

int cloth_get_stats(cloth_t *c, cloth_solve_stats *stats)
{
    if (!c || !stats)
        return fail(CLOTH_ERR_INVALID, "NULL argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    CK(cudaSetDevice(c->ctx->device));
    CK(cudaStreamSynchronize(c->ctx->stream));
    InstState st;
    CK(cudaMemcpy(&st, c->d_state, sizeof(st), cudaMemcpyDeviceToHost));
    if (c->escalated_valid)
    {
        *stats = c->escalated; // the last step was re-solved in FP64
        return CLOTH_OK;
    }
    stats->iters = st.iter;
    stats->status = st.bar_err ? CLOTH_ERR_TIMEOUT : st.status;
    stats->res_norm = std::sqrt(std::max(0.0, st.rr));
    stats->rhs_norm = std::sqrt(std::max(0.0, st.bb));
    stats->rel_residual = stats->rhs_norm > 0 ? stats->res_norm / stats->rhs_norm
                                              : stats->res_norm;
    stats->solver = !(c->self && c->self->persist_ok) ? CLOTH_SOLVER_GRAPH_LOOP
                    : c->self->persist_1b             ? CLOTH_SOLVER_PERSISTENT_1B
                                                      : CLOTH_SOLVER_PERSISTENT;
    return CLOTH_OK;
}

int cloth_get_dx(cloth_t *c, double *dx, int nv)
{
    if (!c || !dx || nv != c->mesh.nv)
        return fail(CLOTH_ERR_INVALID, "bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    CK(cudaSetDevice(c->ctx->device));
    if (c->dx64_valid)
        return f64_get_dx(c, dx, nv);
    std::vector<float4> v(nv);
    CK(cudaStreamSynchronize(c->ctx->stream));
    CK(cudaMemcpy(v.data(), c->h.dx, size_t(nv) * sizeof(float4), cudaMemcpyDeviceToHost));
    for (int i = 0; i < nv; i++)
    {
        dx[3 * i] = v[i].x;
        dx[3 * i + 1] = v[i].y;
        dx[3 * i + 2] = v[i].z;
    }
    return CLOTH_OK;
}

int cloth_export_system(cloth_t *c, int *ell, float *A, float *b, float *fint,
                        float *kbend)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    if (!c->scratch)
        return fail(CLOTH_ERR_STATE, "export: the cloth is held by a server");
    CK(cudaSetDevice(c->ctx->device));
    CK(cudaStreamSynchronize(c->ctx->stream));
    const Tables &t = c->tab;
    const int n = t.nv, S = c->h.stride, W = t.width, R = CLOTH_ELL_REF_WIDTH;
    const size_t WS = size_t(W) * S;
    if (ell)
        for (int v = 0; v < n; v++)
            for (int s = 0; s < R; s++)
            {
                int len = t.rowptr[v + 1] - t.rowptr[v];
                ell[size_t(v) * R + s] = s < len ? t.cols[size_t(t.rowptr[v]) + s] : -1;
            }
    if (A)
    {
        // stored diagonal + upper blocks; a lower block is its transposed
        // upper block (the same symmetric 6 floats)
        const size_t WuS = size_t(c->width_up) * c->h.ntile_rows * kTile;
        std::vector<float4> a0(WuS), aw(c->h.Aw ? WuS : 0);
        std::vector<float2> a1(WuS);
        CK(cudaMemcpy(a0.data(), c->h.A0, WuS * sizeof(float4), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(a1.data(), c->h.A1, WuS * sizeof(float2), cudaMemcpyDeviceToHost));
        if (c->h.Aw)
            CK(cudaMemcpy(aw.data(), c->h.Aw, WuS * sizeof(float4), cudaMemcpyDeviceToHost));
        std::fill(A, A + size_t(n) * R * 9, 0.f);
        for (int v = 0; v < n; v++)
            for (int s = 0; s < t.rowptr[v + 1] - t.rowptr[v]; s++)
            {
                const int ds = t.diag_slot[v];
                size_t o;
                if (s >= ds)
                    o = up_idx(s - ds, v, c->width_up);
                else
                {
                    const int cr = t.cols[size_t(t.rowptr[v]) + s];
                    const int *b0 = &t.cols[t.rowptr[cr]], *b1 = &t.cols[t.rowptr[cr + 1]];
                    const int s2 = int(std::lower_bound(b0, b1, v) - b0);
                    o = up_idx(s2 - t.diag_slot[cr], cr, c->width_up);
                }
                float e[6] = {a0[o].x, a0[o].y, a0[o].z, a0[o].w, a1[o].x, a1[o].y};
                float full[9] = {e[0], e[1], e[2], e[1], e[3], e[4], e[2], e[4], e[5]};
                if (c->h.Aw)
                {
                    // skew part: block p = S p + w x p; the lower block is
                    // the transposed upper one, S p - w x p
                    const float sg = s >= ds ? 1.f : -1.f;
                    const float wx = sg * aw[o].x, wy = sg * aw[o].y, wz = sg * aw[o].z;
                    full[1] -= wz;
                    full[2] += wy;
                    full[3] += wz;
                    full[5] -= wx;
                    full[6] -= wy;
                    full[7] += wx;
                }
                std::memcpy(A + (size_t(v) * R + s) * 9, full, sizeof(full));
            }
    }
    if (b)
    {
        std::vector<float4> bv(n);
        CK(cudaMemcpy(bv.data(), c->h.b, size_t(n) * sizeof(float4), cudaMemcpyDeviceToHost));
        for (int v = 0; v < n; v++)
        {
            b[3 * v] = bv[v].x;
            b[3 * v + 1] = bv[v].y;
            b[3 * v + 2] = bv[v].z;
        }
    }
    if (fint)
    {
        // stretch part from the force records, bending part -K_b x or the
        // dihedral records' (c beta / 2) dbeta/dx
        std::vector<float4> fr(size_t(t.nt) * 3), x32(n), dr(c->h.drec ? 4 * size_t(t.n_dih) : 0);
        std::vector<float> dfb(c->h.drec ? t.n_dih : 0);
        CK(cudaMemcpy(fr.data(), c->h.frec, fr.size() * sizeof(float4), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(x32.data(), c->h.x32, x32.size() * sizeof(float4), cudaMemcpyDeviceToHost));
        if (!dr.empty())
        {
            CK(cudaMemcpy(dr.data(), c->h.drec, dr.size() * sizeof(float4),
                          cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(dfb.data(), c->h.dfb, dfb.size() * sizeof(float),
                          cudaMemcpyDeviceToHost));
        }
        for (int v = 0; v < n; v++)
        {
            float f[3] = {0, 0, 0};
            for (int k = t.f_rowptr[v]; k < t.f_rowptr[v + 1]; k++)
            {
                f[0] += fr[k].x;
                f[1] += fr[k].y;
                f[2] += fr[k].z;
            }
            for (int s = 0; s < t.rowptr[v + 1] - t.rowptr[v]; s++)
            {
                size_t k = size_t(t.rowptr[v]) + s;
                const float4 xc = x32[t.cols[k]];
                f[0] -= t.kbend[k] * xc.x;
                f[1] -= t.kbend[k] * xc.y;
                f[2] -= t.kbend[k] * xc.z;
            }
            if (!dr.empty())
            {
                const size_t k = size_t(t.rowptr[v]) + t.diag_slot[v];
                for (int j = 0; j < t.dih_count[k]; j++)
                {
                    const uint32_t en = t.dih_ent[size_t(t.dih_start[k]) + j];
                    const float4 g = dr[4 * size_t(en >> 4) + ((en >> 2) & 3u)];
                    const float fb = dfb[en >> 4];
                    f[0] += fb * g.x;
                    f[1] += fb * g.y;
                    f[2] += fb * g.z;
                }
            }
            std::memcpy(fint + 3 * size_t(v), f, sizeof(f));
        }
    }
    if (kbend)
    {
        std::fill(kbend, kbend + size_t(n) * R, 0.f);
        for (int v = 0; v < n; v++)
            for (int s = 0; s < t.rowptr[v + 1] - t.rowptr[v]; s++)
                kbend[size_t(v) * R + s] = t.kbend[size_t(t.rowptr[v]) + s];
    }
    return CLOTH_OK;
}

int cloth_export_dihedral(cloth_t *c, int *n_edges, int *edge_ids, float *grad, float *coef)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    const Tables &t = c->tab;
    if (n_edges)
        *n_edges = t.n_dih;
    if (edge_ids && t.n_dih > 0)
        std::memcpy(edge_ids, t.dih_edge.data(), t.dih_edge.size() * sizeof(int));
    if ((!grad && !coef) || t.n_dih == 0)
        return CLOTH_OK;
    if (!c->scratch)
        return fail(CLOTH_ERR_STATE, "export: the cloth is held by a server");
    CK(cudaSetDevice(c->ctx->device));
    CK(cudaStreamSynchronize(c->ctx->stream));
    std::vector<float4> dr(4 * size_t(t.n_dih));
    std::vector<float> dfb(t.n_dih);
    CK(cudaMemcpy(dr.data(), c->h.drec, dr.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dfb.data(), c->h.dfb, dfb.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (int q = 0; q < t.n_dih; q++)
    {
        for (int a = 0; a < 4 && grad; a++)
        {
            const float4 g = dr[4 * size_t(q) + a];
            grad[size_t(q) * 12 + 3 * a + 0] = g.x;
            grad[size_t(q) * 12 + 3 * a + 1] = g.y;
            grad[size_t(q) * 12 + 3 * a + 2] = g.z;
        }
        if (coef)
        {
            coef[2 * size_t(q)] = dr[4 * size_t(q)].w;
            coef[2 * size_t(q) + 1] = dfb[q];
        }
    }
    return CLOTH_OK;
}

int cloth_export_triangles(cloth_t *c, float *fint, float *hess)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    if (!c->scratch)
        return fail(CLOTH_ERR_STATE, "export: the cloth is held by a server");
    CK(cudaSetDevice(c->ctx->device));
    CK(cudaStreamSynchronize(c->ctx->stream));
    const Tables &t = c->tab;
    if (fint)
    {
        std::vector<float4> fr(size_t(t.nt) * 3);
        CK(cudaMemcpy(fr.data(), c->h.frec, fr.size() * sizeof(float4), cudaMemcpyDeviceToHost));
        for (int i = 0; i < t.nt; i++)
            for (int a = 0; a < 3; a++)
            {
                const float4 v = fr[t.f_dest[size_t(i) * 3 + a]];
                float *o = fint + size_t(i) * 9 + a * 3;
                o[0] = v.x;
                o[1] = v.y;
                o[2] = v.z;
            }
    }
    if (hess)
    {
        std::vector<HRec> hr(size_t(t.nt) * 9);
        CK(cudaMemcpy(hr.data(), c->h.hrec, hr.size() * sizeof(HRec), cudaMemcpyDeviceToHost));
        for (int i = 0; i < t.nt; i++)
            for (int ab = 0; ab < 9; ab++)
            {
                const HRec &r = hr[t.h_dest[size_t(i) * 9 + ab]];
                float e[6] = {r.h0.x, r.h0.y, r.h0.z, r.h0.w, r.h1.x, r.h1.y};
                float full[9] = {e[0], e[1], e[2], e[1], e[3], e[4], e[2], e[4], e[5]};
                std::memcpy(hess + (size_t(i) * 9 + ab) * 9, full, sizeof(full));
            }
    }
    return CLOTH_OK;
}

int cloth_export_tables(const cloth_t *c, int *stencil, float *coef, float *area,
                        float *mass, int *tri_slot)
{
    if (!c)
        return fail(CLOTH_ERR_INVALID, "cloth is NULL");
    const Tables &t = c->tab;
    if (stencil)
        std::memcpy(stencil, t.stencil.data(), t.stencil.size() * sizeof(int));
    if (coef)
        std::memcpy(coef, t.coef.data(), t.coef.size() * sizeof(float));
    if (area)
        std::memcpy(area, t.area.data(), t.area.size() * sizeof(float));
    if (mass)
        for (int v = 0; v < t.nv; v++)
            mass[v] = float(t.mass[v]);
    if (tri_slot)
        std::memcpy(tri_slot, t.tri_slot.data(), t.tri_slot.size() * sizeof(int));
    return CLOTH_OK;
}

int cloth_step_plain(cloth_t *c, double dt, const cloth_solve_params *params,
                     cloth_solve_stats *stats)
{
    if (!c || !valid_params(params) || (params && params->max_iters > 100000))
        return fail(CLOTH_ERR_INVALID, "cloth_step_plain: bad argument");
    if (c->mat.bending_model != 0)
        return fail(CLOTH_ERR_INVALID, "cloth_step_plain: the reference-structured path has "
                                       "the GPU cloth's quadratic bending only");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    CK(cudaSetDevice(c->ctx->device));
    CK(cudaStreamSynchronize(c->ctx->stream));
    const Tables &t = c->tab;
    const int n = t.nv, R = CLOTH_ELL_REF_WIDTH;
    if (!c->plain)
    {
        std::vector<int> ell(size_t(n) * R, -1);
        std::vector<float> kb(size_t(n) * R, 0.f), mass(n), grav(n);
        for (int v = 0; v < n; v++)
        {
            for (int s = 0; s < t.rowptr[v + 1] - t.rowptr[v]; s++)
            {
                ell[size_t(v) * R + s] = t.cols[size_t(t.rowptr[v]) + s];
                kb[size_t(v) * R + s] = t.kbend[size_t(t.rowptr[v]) + s];
            }
            mass[v] = float(t.mass[v]);
            grav[v] = float(c->mat.gravity * t.mass[v]);
        }
        PlainInit in{n, t.nt, ell.data(), kb.data(), mass.data(), grav.data(), c->h.tri, c->h.tcoef};
        int rc = plain_create(in, &c->plain);
        if (rc != CLOTH_OK)
            return rc;
        c->ctx->bytes += plain_bytes(c->plain);
    }
    if (!c->plain_host_valid)
    {
        c->plain_x.resize(size_t(n) * 3);
        c->plain_xp.resize(size_t(n) * 3);
        CK(cudaMemcpy(c->plain_x.data(), c->h.x64, c->plain_x.size() * 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(c->plain_xp.data(), c->h.xp64, c->plain_xp.size() * 8, cudaMemcpyDeviceToHost));
        c->plain_host_valid = true;
    }
    std::vector<int> pins(c->static_pins);
    std::vector<float> tgt;
    for (int v : c->static_pins)
        for (int k = 0; k < 4; k++)
            tgt.push_back(k < 3 ? float(c->mesh.pos[size_t(v) * 3 + k]) : 0.f);
    if (c->drag_vid >= 0)
    {
        pins.push_back(c->drag_vid);
        for (int k = 0; k < 4; k++)
            tgt.push_back(k < 3 ? c->drag_tgt[k] : 0.f);
    }
    if (!(dt > 0))
        dt = c->mat.default_timestep;
    int rc = plain_step(c->plain, c->plain_x.data(), c->plain_xp.data(), pins.data(), tgt.data(),
                        int(pins.size()), float(dt), c->mat.stretch_k[0], c->mat.stretch_k[1],
                        c->mat.stretch_k[2], c->mat.fix_fv_norm, c->mat.rayleigh_a,
                        c->mat.rayleigh_b, params, stats);
    if (rc != CLOTH_OK)
        return rc;
    // keep the library's device state in step, so GetPos and the fast path see it
    CK(cudaMemcpy(c->h.x64, c->plain_x.data(), c->plain_x.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->h.xp64, c->plain_xp.data(), c->plain_xp.size() * 8, cudaMemcpyHostToDevice));
    k_sync_x32<<<std::min(1024, (n + 255) / 256), 256, 0, c->ctx->stream>>>(c->d_desc);
    CK(cudaGetLastError());
    if (c->drag_vid >= 0)
    {
        c->drag_vid = -1;
        c->pins_dirty = true;
    }
    return CLOTH_OK;
}

int cloth_batch_step(cloth_ctx *ctx, cloth_t *const *cloths, int n, double dt,
                     const cloth_solve_params *params, cloth_solve_stats *stats)
{
    if (!ctx || !cloths || n <= 0 || !valid_params(params))
        return fail(CLOTH_ERR_INVALID, "cloth_batch_step: bad argument");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    std::vector<cloth_s *> members(cloths, cloths + n);
    for (auto *c : members)
        if (!c || c->ctx != ctx)
            return fail(CLOTH_ERR_INVALID, "cloth_batch_step: cloth of another context");
    {
        std::vector<cloth_s *> sorted(members);
        std::sort(sorted.begin(), sorted.end());
        if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
            return fail(CLOTH_ERR_INVALID, "cloth_batch_step: cloth listed twice");
    }
    CK(cudaSetDevice(ctx->device));
    if (!ctx->last_batch || ctx->last_batch->members != members)
    {
        ctx->last_batch.reset();
        int rc = make_batch(ctx, members, ctx->last_batch);
        if (rc != CLOTH_OK)
            return rc;
    }
    return run_step(ctx->last_batch.get(), dt, params, stats);
}

} // extern "C"
