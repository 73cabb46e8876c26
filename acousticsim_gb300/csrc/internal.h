// Host-side objects shared by the translation units of the library: the
// context, the cloth instance with its device memory, and the helpers the
// step driver (cloth_api.cu) and the request server (server.cu) both use.
// Not part of the C ABI.
#pragma once
#include "../../include/cloth_gb300.h"
#include "device.cuh"
#include "topology.h"

#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

namespace cloth {

// ---------------------------------------------------------------- kernels
__global__ void k_pins(InstDesc *const *descs, const int *inst_list, int ninst,
                       const int *ninst_dev);
__global__ void k_tri(InstDesc *const *descs, const Tile *tiles, const BatchCtl *ctl);
__global__ void k_row(InstDesc *const *descs, const Tile *tiles, BatchCtl *ctl);
__global__ void k_cond(const BatchCtl *ctl, cudaGraphConditionalHandle h);
// instance totals after the graph-loop SpMV (p.q -> alpha) and update (r.z,
// r.r -> beta, convergence): one block per instance of inst_list (ninst of
// them, or *ninst_dev when that is not null)
__global__ void k_reduce_pq(InstDesc *const *descs, const int *inst_list, int ninst,
                            const int *ninst_dev, BatchCtl *ctl, int use_cond,
                            cudaGraphConditionalHandle h);
__global__ void k_reduce_rz(InstDesc *const *descs, const int *inst_list, int ninst,
                            const int *ninst_dev, BatchCtl *ctl, int use_cond,
                            cudaGraphConditionalHandle h);
// one thread per instance, blocks of kTile threads
inline int reduce_grid(int ninst) { return ninst < 1 ? 1 : (ninst + 127) / 128; }
// graph-loop kernel variants (k_spmv_t<R, U>, k_update_t<R>); arguments:
//   spmv  (descs, tiles, ctl, use_cond, handle)
//   update(descs, tiles, ctl, use_cond, handle, iters_left)
extern const GraphLoopVariant kSpmvVariants[];
extern const GraphLoopVariant kSpmvSkewVariants[]; // same variants, skew block parts applied
extern const GraphLoopVariant kUpdateVariants[];
extern const int kNumSpmvVariants;
extern const int kNumUpdateVariants;
constexpr int kDefaultSpmvVariant = 3;   // R = 2, U = 1, TPB = 1 until a tuner says otherwise
// threads per block of an SpMV variant
inline int spmv_block(const GraphLoopVariant &v)
{
    return v.bulk_stages ? kBulkThreads : kTile / v.rows_per_thread;
}
constexpr int kDefaultUpdateVariant = 1; // R = 2, TPB = 1
__global__ void k_snap_rows(InstDesc *const *descs, const Tile *tiles, const BatchCtl *ctl,
                            float4 *buf, int restore);
__global__ void k_snap_state(InstDesc *const *descs, const int *inst, int ninst,
                             InstState *buf, BatchCtl *ctl, BatchCtl *ctl_buf, int restore);
__global__ void k_advance(InstDesc *const *descs, const Tile *tiles,
                          const BatchCtl *ctl, int finished_only);
__global__ void k_sync_x32(InstDesc *d);
__global__ void k_ir_start(InstDesc *const *descs, const Tile *tiles, BatchCtl *ctl,
                           const double *rhs64);
__global__ void k_pcg_persistent_sm(InstDesc *const *descs, const TeamBlock *work,
                                    int halo_cap, int rows_cap, SpinCfg sc);
__global__ void k_pcg_persistent_gm(InstDesc *const *descs, const TeamBlock *work,
                                    int halo_cap, int rows_cap, SpinCfg sc);
__global__ void k_pcg_persistent_sm_skew(InstDesc *const *descs, const TeamBlock *work,
                                         int halo_cap, int rows_cap, SpinCfg sc);
__global__ void k_pcg_persistent_gm_skew(InstDesc *const *descs, const TeamBlock *work,
                                         int halo_cap, int rows_cap, SpinCfg sc);
__global__ void k_pcg1_persistent(InstDesc *const *descs, const TeamBlock *work, int halo_cap,
                                  int rows_cap, SpinCfg sc);

// ---------------------------------------------------------------- plain path
struct PlainState;
struct PlainInit
{
    int nv, nt;
    const int *ell_host;
    const float *kb_scalar_host;
    const float *mass_host, *grav_host;
    const int4 *tri_dev;
    const float4 *coef_dev;
};
int plain_create(const PlainInit &in, PlainState **out);
void plain_free(PlainState *p);
size_t plain_bytes(const PlainState *p);
int plain_step(PlainState *p, double *x, double *xp, const int *pins, const float *pin_tgt,
               int npins, float dt, float kw, float kwe, float kb, int fix_fv, float ra,
               float rb, const cloth_solve_params *prm, cloth_solve_stats *stats);

void set_last_error(const std::string &msg);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Sub-allocations of one device allocation, 256-byte aligned.
struct Layout
{
    size_t off = 0;
    template <class T> size_t take(size_t n)
    {
        size_t o = off;
        off = align_up(off + n * sizeof(T), 256);
        return o;
    }
};

// Offsets of the per-solve work arrays inside one scratch allocation: the
// triangle records, the assembled system and preconditioner, and the PCG
// vectors.  Everything else of a cloth (mesh tables, ELL map, positions, the
// warm-start dx, pins, PCG scalars) is resident state.
struct ScratchLayout
{
    size_t hrec = 0, frec = 0, A0 = 0, A1 = 0, M0 = 0, M1 = 0, b = 0;
    size_t r = 0, z = 0, p0 = 0, p1 = 0, q = 0, w1 = 0, part = 0;
    // dihedral bending only (kAbsent otherwise)
    static constexpr size_t kAbsent = ~size_t(0);
    size_t drec = kAbsent, dfb = kAbsent, Aw = kAbsent;
    size_t bytes = 0;
};

namespace detail {
struct Batch;
}

} // namespace cloth

struct cloth_server_s;
struct cloth_f64_s;
struct cloth_body_s;
struct cloth_collide_s;

struct cloth_ctx_s
{
    int device = 0;
    cudaStream_t stream = nullptr;
    std::recursive_mutex mu;
    int num_sms = 0;
    int occ_tri = 1, occ_row = 1;
    std::vector<int> occ_spmv, occ_update; // resident blocks per SM of each variant
    std::vector<int> occ_spmv_skew;         // the same for kSpmvSkewVariants
    bool autotune = true;                  // tune graph-loop batches on their first step
    int tune_spmv = cloth::kDefaultSpmvVariant, tune_update = cloth::kDefaultUpdateVariant;
    std::vector<float> tune_ms_spmv, tune_ms_update; // the last tuning's timings
    int max_smem_optin = 0;
    // bounded waits of the persistent solvers (cloth_ctx_set_spin_limit; the
    // extra arrivals are the timeout test's hook, 0 otherwise)
    cloth::SpinCfg spin = {cloth::kSpinLimitDefault, 0u};
    int solver = 0; // 0: persistent cooperative PCG when the set fits, 1: graph loop
    // graph-loop launch sets of more cloths than this hand their last this-many
    // iterating cloths to the persistent kernel (-1: num_sms / 16; 0: never)
    int tail_hand_off = -1;
    // precision escalation of stepped solves: 0 off, 1 an FP32 PCG ending in
    // NaN / breakdown is re-solved in FP64, 2 one ending at max_iters too
    int escalate = 1;
    bool prof = false;
    double prof_ms[CLOTH_NUM_PHASES] = {};
    long long prof_n[CLOTH_NUM_PHASES] = {};
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    size_t bytes = 0;
    std::vector<cloth_s *> cloths;
    std::vector<cloth_server_s *> servers;
    std::vector<cloth_body_s *> bodies;
    std::unique_ptr<cloth::detail::Batch> last_batch;
    ~cloth_ctx_s();
};

struct cloth_s
{
    cloth_ctx *ctx = nullptr;
    cloth::Mesh mesh;
    cloth::Tables tab;
    cloth::Material mat;
    std::vector<int> static_pins;
    int drag_vid = -1;
    float drag_tgt[3] = {0, 0, 0};
    bool pins_dirty = true;
    int npins_uploaded = 0;
    char *arena = nullptr;    // resident state
    size_t arena_bytes = 0;
    char *scratch = nullptr;  // own per-solve work arrays; null while a server holds the cloth
    size_t scratch_bytes = 0;
    cloth::ScratchLayout sl;
    int width_up = 1;         // planes of the stored (diagonal + upper) blocks
    int max_halo = 0;         // widest column range of a 128-row tile
    cloth_server_s *server = nullptr;
    cloth_f64_s *f64 = nullptr; // FP64 work arrays (refinement, FP64 PCG), on first use
    bool dx64_valid = false;    // the last solve left an FP64 dx (refined or FP64 PCG)
    bool pcg_stale = false;     // the FP32 PCG start of the assembly was overwritten
    bool escalated_valid = false; // the last step was re-solved in FP64 (its stats)
    cloth_solve_stats escalated = {};
    cloth::InstDesc h;        // host copy of the descriptor
    cloth::InstDesc *d_desc = nullptr;
    cloth::InstState *d_state = nullptr;
    bool desc_dirty = true;
    bool assembled = false;
    double dt_set = -1.0;
    std::unique_ptr<cloth::detail::Batch> self;
    // plain (reference-structured) path: host positions and its device state
    cloth::PlainState *plain = nullptr;
    std::vector<double> plain_x, plain_xp;
    bool plain_host_valid = false;
    // kinematic bodies this cloth collides with, and the collision work arrays
    std::vector<cloth_body_s *> bodies;
    cloth_collide_s *col = nullptr;
    ~cloth_s();
};

namespace cloth {
namespace detail {

// Shared memory of one stage of the bulk-staged SpMV for a set of cloths:
// the widest cloth's row info, lower-slot columns and transposed-block
// indices, upper-slot columns and stored blocks (skew parts with `skew`) for
// 128 rows, plus p_old and z over its widest tile halo (at most kBulkHaloCap
// rows), rounded to 128 bytes.
unsigned bulk_stage_bytes(const std::vector<cloth_s *> &cloths, bool skew, bool halo);
// Dynamic shared memory and resident blocks per SM of a bulk SpMV variant
// with that stage size (0 blocks: it does not fit).
unsigned bulk_smem(const GraphLoopVariant &v, unsigned stage_bytes);
int bulk_occupancy(const GraphLoopVariant &v, unsigned stage_bytes, int max_smem);

// Points the scratch fields of h at base (null: clears them).
void bind_scratch(const cloth_s *c, InstDesc &h, char *base);
// Own scratch of a cloth: allocate (and bind, upload the descriptor) / free.
int alloc_own_scratch(cloth_s *c);
void free_own_scratch(cloth_s *c);
// Parameters, time step and pins of the next step, as the step driver sets them.
// hold_maxiter: the step escalates a solve that ends at max_iters, so the
// advance must leave that cloth's state (only the escalating step driver)
void set_params(cloth_s *c, const cloth_solve_params *p, int hold_maxiter = 0);
void set_dt(cloth_s *c, double dt);
int sync_pins(cloth_s *c);
int sync_desc(cloth_s *c);
// FP32 PCG solve of A e = float(rhs64) from e = 0 on the cloth's own launch set
// (the correction step of iterative refinement); e is left in dx.
int inner_solve(cloth_s *c, const double *rhs64, const cloth_solve_params *p,
                cloth_solve_stats *stats);
// FP64 result handling (precision.cu)
void f64_free(cloth_s *c);
int f64_advance(cloth_s *c);
int f64_get_dx(cloth_s *c, double *dx, int nv);
// Re-solve an assembled step whose FP32 PCG ended in NaN or breakdown with
// the FP64 flexible CG, then advance in FP64; fills the step's stats.
int escalate_step(cloth_s *c, const cloth_solve_params *p, cloth_solve_stats *out);
// A server's view of one of its cloths: true while requests are queued or running.
bool server_busy(const cloth_server_s *s, const cloth_s *c);
// Detach every cloth of a server and free it (context teardown).
void server_teardown(cloth_server_s *s);
// Collisions with kinematic bodies (collide.cu): contacts of the current
// positions (after the pins, before the row pass), and the repulsion of dx
// after the solve; both enqueue on the context's stream.
int collide_detect(cloth_s *c);
// Drops the launch sets (own and the context's last batch) built with c.
void drop_launch_sets(cloth_s *c);
int collide_repulse(cloth_s *c);
void collide_free(cloth_s *c);
void body_release_all(cloth_ctx *ctx);

} // namespace detail
} // namespace cloth
