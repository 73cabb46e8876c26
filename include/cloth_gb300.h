/*
 * cloth_gb300.h - C ABI of the GB300 (sm_103a) Baraff-Witkin implicit cloth step.
 *
 * This library is a drop-in for AcousticSim's GPU cloth path
 * (cloth_type "fem_gpu", class cBaraffClothGpu).  Every entry point below names
 * the reference interface it replaces (paths are relative to the reference
 * project root).  Conventions:
 *   - every call returns an int status (CLOTH_OK = 0) and never throws;
 *     cloth_last_error() gives a one-line message for the calling thread;
 *   - all pointers are HOST pointers unless the name ends in _dev;
 *   - arrays are packed row-major: positions nv*3, uv nv*2, triangles nt*3;
 *   - 3x3 blocks exported to the caller are row-major: (i,j) -> [3*i+j];
 *   - the library owns all device memory of a cloth; a context owns one CUDA
 *     stream, and calls on one context are serialised by an internal mutex.
 */
#ifndef CLOTH_GB300_H
#define CLOTH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLOTH_ABI_VERSION 2
#define CLOTH_ELL_REF_WIDTH 32 /* tCudaVector32i, src/sim/cloth/BaraffClothGpu.h:19 */

enum cloth_status {
    CLOTH_OK = 0,
    CLOTH_ERR_INVALID = 1,     /* bad argument or size */
    CLOTH_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    CLOTH_ERR_OOM = 3,         /* device allocation failed */
    CLOTH_ERR_BUDGET = 4,      /* admission refused: device-memory budget */
    CLOTH_ERR_MESH = 5,        /* mesh unsupported (non-manifold edge, row wider than 32) */
    CLOTH_ERR_NAN = 6,         /* NaN/Inf met in the solve (per-instance status) */
    CLOTH_ERR_BREAKDOWN = 7,   /* PCG denominator was zero (alpha or beta clamped) */
    CLOTH_ERR_MAXITER = 8,     /* solve stopped at max_iters above tolerance (per-instance status) */
    CLOTH_ERR_TIMEOUT = 9,     /* a bounded device wait gave up */
    CLOTH_ERR_UNSUPPORTED = 10,
    CLOTH_ERR_STATE = 11,      /* call out of order (e.g. solve before assemble) */
    CLOTH_ERR_CONTACTS = 12    /* contact lists exceeded their capacity (cloth_set_contact_capacity) */
};

typedef struct cloth_ctx_s cloth_ctx;
typedef struct cloth_s cloth_t;

/* Regular grid as cTriangulator::BuildGeometry_UniformTriangle builds it
 * (src/geometries/Triangulator.cpp:141-457, 621-658). JSON keys in quotes. */
typedef struct {
    double cloth_size[2];   /* "cloth_size": [height, width] in metres */
    int subdivision[2];     /* "subdivision": [height_div, width_div] */
    double init_pos[3];     /* "cloth_init_pos" (orientation must be zero) */
    float uv_rotation_deg;  /* "cloth_uv_rotation": 0, 45 or 90 */
} cloth_grid_desc;

/* Triangle mesh handed to cloth_create (cBaseCloth::InitGeometry,
 * src/sim/cloth/BaseCloth.cpp:292-416). */
typedef struct {
    int nv, nt, ne;        /* ne = 0 with edges = NULL: edges are derived (cObjUtil::BuildEdge order) */
    const double *pos;     /* nv*3 rest positions; also the initial state */
    const float *uv;       /* nv*2 material coordinates (tVertex::muv) */
    const int *tris;       /* nt*3 vertex ids */
    const int *edges;      /* ne*4: v0, v1, tri0, tri1 (tri1 = -1: boundary) */
} cloth_mesh_desc;

/* Material and step parameters (cBaraffClothGpu::Init,
 * src/sim/cloth/BaraffClothGpu.cpp:24-49; JSON keys in quotes). */
typedef struct {
    float stretch_k[3];       /* "cloth_stretch_stiffness": warp, weft, bias (shear) */
    float bending_k[2];       /* "cloth_bending_stiffness": u, v */
    float density;            /* "cloth_density" (kg/m^2) */
    float rayleigh_a;         /* "rayleigh_damping_a" */
    float rayleigh_b;         /* "rayleigh_damping_b" */
    double default_timestep;  /* "default_timestep" */
    double gravity;           /* -9.8 (BaraffClothGpu.cpp:561) */
    int fix_fv_norm;          /* 0: reference Hessian, whose weft term uses |Fu|
                                 (BaraffClothGpu.cu:55); 1: use |Fv| */
    int bending_model;        /* "cloth_bending_model": CLOTH_BENDING_QUADRATIC (the
                                 GPU cloth's constant Q-bending) or CLOTH_BENDING_DIHEDRAL */
} cloth_material;

/* Bending models.  QUADRATIC: cBaraffClothGpu's constant Q-bending matrix
 * (BaraffClothGpu.cpp:573-680).  DIHEDRAL: the CPU cloth's nonlinear
 * dihedral-angle bending, cDihedralMaterial (src/sim/cloth/DihedralBending.cpp:
 * 23-91, 382-488): per interior edge, force (c beta / 2) dbeta/dx and the
 * Gauss-Newton stiffness c dbeta/dx dbeta/dx^T with c = -K e / (h0 + h1), both
 * rebuilt from the current positions every step; stiffness K = bending_k[0]. */
#define CLOTH_BENDING_QUADRATIC 0
#define CLOTH_BENDING_DIHEDRAL 1

/* PCG controls (PCGSolver::Solve, src/sim/cloth/gpu_solvers/PCGSolver.cu:332-481).
 * The reference runs at most 100 iterations and stops when the absolute
 * residual norm drops below 1e-10, tested every 10th iteration. */
typedef struct {
    int max_iters;
    double rel_tol;      /* stop when ||r|| <= rel_tol * ||b||  (0 disables) */
    double abs_tol;      /* stop when ||r|| <= abs_tol          (0 disables) */
    int check_every;     /* test after iterations 1, 1+k, 1+2k, ... and at max_iters */
    int warm_start;      /* 1: start from the previous dx (reference); 0: from zero */
} cloth_solve_params;

typedef struct {
    int iters;            /* PCG iterations run */
    int status;           /* CLOTH_OK, CLOTH_ERR_MAXITER, CLOTH_ERR_NAN, CLOTH_ERR_BREAKDOWN */
    double res_norm;      /* ||r|| of the recurrence residual at exit (FP64 reduction) */
    double rhs_norm;      /* ||b|| */
    double rel_residual;  /* res_norm / rhs_norm */
    int solver;           /* CLOTH_SOLVER_PERSISTENT or CLOTH_SOLVER_GRAPH_LOOP */
} cloth_solve_stats;

/* PCG drivers. PERSISTENT: one cooperative launch runs all iterations of every
 * instance (team barriers between the SpMV and update phases); used whenever
 * the launch set fits in the resident blocks, else GRAPH_LOOP: two kernels per
 * iteration inside a CUDA-graph while loop with a device-side condition. */
#define CLOTH_SOLVER_PERSISTENT 0
#define CLOTH_SOLVER_GRAPH_LOOP 1
#define CLOTH_SOLVER_FP64 2       /* cloth_solve_fp64 */
/* PERSISTENT_1B: the persistent launch with one team barrier per iteration
 * (the same PCG in the Chronopoulos-Gear arrangement: r.u, w.u and r.r summed
 * together), used where every block's halo fits in shared memory; stats report
 * which one ran. PERSISTENT_2B: only the two-barrier persistent kernel. */
#define CLOTH_SOLVER_PERSISTENT_1B 3
#define CLOTH_SOLVER_PERSISTENT_2B 4
/* ESCALATED: the step's FP32 PCG ended in NaN or breakdown (a system beyond
 * FP32, e.g. stiff dihedral bending on a fine mesh), or at max_iters at
 * escalation level 2; the step was re-solved by
 * the all-FP64 PCG (cloth_solve_fp64) from zero and advanced in FP64; iters
 * and rel_residual are that solve's. See cloth_ctx_set_escalation. */
#define CLOTH_SOLVER_ESCALATED 5

/* ---------------------------------------------------------------- library */
int cloth_abi_version(void);
const char *cloth_last_error(void);
const char *cloth_status_string(int status);

/* ---------------------------------------------------------------- context */
/* New: one device + one CUDA stream + kernel timers. */
int cloth_ctx_create(int device, cloth_ctx **out);
int cloth_ctx_destroy(cloth_ctx *ctx);
int cloth_ctx_synchronize(cloth_ctx *ctx);
/* Per-phase CUDA-event timers (cTimeUtil::Begin/End, src/utils/TimeUtil.hpp:7-32).
 * Phases: 0 pins, 1 triangle assembly, 2 row assembly + PCG init,
 * 3 SpMV + p.Ap, 4 update + residual, 5 position update, 6 contact detection,
 * 7 contact repulsion, 8 instance totals of the graph-loop PCG (k_reduce_*). */
#define CLOTH_NUM_PHASES 9
int cloth_ctx_set_profiling(cloth_ctx *ctx, int enable);
int cloth_ctx_get_profile(cloth_ctx *ctx, double *ms_total, long long *launches);
int cloth_ctx_reset_profile(cloth_ctx *ctx);
/* Preferred PCG driver for launch sets built after the call. */
int cloth_ctx_set_solver(cloth_ctx *ctx, int solver);
/* Launch sets of more cloths than fit one persistent launch run the graph
 * loop; with the persistent solver (two barriers) chosen, such a set hands
 * its last max_instances iterating cloths to the persistent kernel, whose
 * arithmetic is the graph loop's bit for bit (results do not change; the few
 * slowest cloths' iterations stop paying the graph loop's per-iteration
 * latency).  -1 (the default): the GPU's SM count / 16; 0: never.  For launch
 * sets built after the call. */
int cloth_ctx_set_tail_hand_off(cloth_ctx *ctx, int max_instances);
/* Bounded waits of the persistent PCG drivers (no counterpart in the
 * reference, whose solver never waits on the device). A team barrier gives up
 * after `polls` polls (0: the default, 2^25, seconds); the solve then ends
 * with stats status CLOTH_ERR_TIMEOUT and the context stays usable.
 * `extra_arrivals` is a test hook: every barrier waits for that many arrivals
 * that no block makes, so the waits run out on purpose (0 in normal use).
 * Applies to launch sets built afterwards (cached ones are dropped). */
int cloth_ctx_set_spin_limit(cloth_ctx *ctx, unsigned polls, unsigned extra_arrivals);
/* Precision escalation of cloth_step / cloth_batch_step (level 1 by default;
 * no counterpart in the reference, whose FP32 solver simply returns). Level 1:
 * a cloth whose FP32 PCG ends in NaN or breakdown keeps its pre-step state, is
 * re-solved in FP64 (CLOTH_SOLVER_ESCALATED) and advanced. Level 2: the same
 * for a cloth whose FP32 PCG ends at max_iters (CLOTH_ERR_MAXITER; a system
 * the FP32 PCG stalls on, e.g. stiff dihedral bending); at level 1 such a step
 * is advanced with the dx it reached, as the reference does. Level 0: a step
 * ending in NaN or breakdown reports the status and leaves the cloth's state
 * unchanged. Steps made without stats, and cloths with bodies, are not
 * escalated. Other levels: CLOTH_ERR_INVALID. */
int cloth_ctx_set_escalation(cloth_ctx *ctx, int enable);
/* Graph-loop kernel variants (the batched and served PCG): rows per thread R
 * of the SpMV and update kernels, the SpMV's slot unroll U and the tiles a
 * block takes at a time (TPB). With autotune on (the default) every graph-loop
 * launch set times all variants on its first step and keeps the fastest; the
 * choice becomes the context's default, which the request server uses. Every
 * variant computes bit-identical results. Variants (SpMV R,U,TPB): 1,1,1
 * 1,2,1 1,3,1 2,1,1 2,2,1 4,1,1 1,1,4 1,2,4 2,1,4 2,2,4 4,1,4 2,1,8, and
 * 1,0,2 1,0,3: the bulk-staged SpMV (a producer warp streams each tile's
 * matrix planes and p over its column range into a ring of 2 or 3
 * shared-memory stages with bulk asynchronous copies; used when the stages
 * fit in shared memory); (update R,TPB): 1,1 2,1 4,1 1,4 2,4 1,8 2,8.
 * Others: CLOTH_ERR_INVALID.
 * Applies to launch sets built afterwards. */
int cloth_ctx_set_kernel_variant(cloth_ctx *ctx, int spmv_rows_per_thread,
                                 int spmv_slot_unroll, int spmv_tiles_per_block,
                                 int update_rows_per_thread, int update_tiles_per_block,
                                 int autotune);
int cloth_ctx_get_kernel_variant(cloth_ctx *ctx, int *spmv_rows_per_thread,
                                 int *spmv_slot_unroll, int *spmv_tiles_per_block,
                                 int *update_rows_per_thread, int *update_tiles_per_block,
                                 int *autotune);
/* Kernel times (ms, best of three) of the last tuning, per variant in the
 * order listed above. Zero when nothing was tuned. */
int cloth_ctx_get_tuning_times(cloth_ctx *ctx, float *spmv_ms, int n_spmv, float *update_ms,
                               int n_update);
/* Device bytes held by all cloths of the context. */
int cloth_ctx_device_bytes(cloth_ctx *ctx, size_t *bytes);
/* The context's cudaStream_t, so callers can order their own work and CUDA
 * events with the library's launches. */
int cloth_ctx_get_stream(cloth_ctx *ctx, void **stream);

/* ---------------------------------------------------------------- topology */
/* cTriangulator::BuildGeometry (Triangulator.cpp:32-139) for "regular_triangle".
 * Query sizes with all output pointers NULL, then fill. edges: ne*4 (v0, v1,
 * tri0, tri1); boundary edges have tri1 = -1. */
int cloth_grid_build(const cloth_grid_desc *grid, int *nv, int *nt, int *ne,
                     double *pos, float *uv, int *tris, int *edges);
/* cTriangulator::BuildGeometry (Triangulator.cpp:32-139) for geometry_type
 * "regular_triangle", "regular_triangle_perturb" (the grid with its interior
 * vertices jittered by up to a fifth of an edge, BuildRectVertices :395-457) or
 * "delaunay" (subdivision[0] * subdivision[1] points: the rectangle boundary,
 * then random points farther apart than sqrt(area / (n pi)), Delaunay-
 * triangulated counter-clockwise; TriangulatorDelaunay.cpp:41-216).  The two
 * random geometries draw from the reference's generator (std::default_random_
 * engine, uniform doubles) seeded with `seed` (the reference's main seeds it
 * with 0), so the points match the reference's bit for bit; the Delaunay
 * triangles are the same set, in this library's order (edges numbered by first
 * appearance over them).  Sizes and fill as cloth_grid_build; an unknown type
 * is CLOTH_ERR_UNSUPPORTED. */
int cloth_geometry_build(const cloth_grid_desc *grid, const char *geometry_type,
                         unsigned long long seed, int *nv, int *nt, int *ne, double *pos,
                         float *uv, int *tris, int *edges);

/* A cloth mesh from an OBJ file, as cBaseCloth::InitGeometry builds it with
 * "enable_cloth_from_obj": true (src/sim/cloth/BaseCloth.cpp:292-356 over
 * cObjUtil::LoadObj and cObjUtil::BuildEdge, src/utils/ObjUtil.cpp:10-240):
 * "cloth_obj_path" = path, "cloth_obj_translation" = translation (may be NULL
 * for zero), "enable_relocate_obj" = relocate.  Vertex i is OBJ vertex i (all
 * must be used by faces), coordinates read as float, y + 0.2, uv from the face
 * corners' texture coordinates times 10/3; faces are triangles or quads (split
 * along the shorter diagonal, as the reference's tinyobjloader does); edges
 * numbered in ascending vertex-pair order.  Sizes and fill as cloth_grid_build. */
int cloth_mesh_from_obj(const char *path, const double *translation, int relocate, int *nv,
                        int *nt, int *ne, double *pos, float *uv, int *tris, int *edges);

/* Host-only (no device needed): the init-time tables cloth_create builds, in
 * the reference's layout. Call with all outputs NULL to get *ne and *width.
 * ell nv*32 (-1 padded, as InitELLMatrix), stencil ne*4, coef nt*12, area nt,
 * mass nv, kbend nv*32 (+K_b scalar per block), tri_slot nt*9. */
int cloth_host_tables(const cloth_mesh_desc *mesh, const cloth_material *mat,
                      int *ne, int *width, int *ell, int *stencil, float *coef,
                      float *area, double *mass, float *kbend, int *tri_slot);

/* ---------------------------------------------------------------- cloth */
/* cBaraffClothGpu::Init (BaraffClothGpu.cpp:24-49): builds the edge stencils,
 * the vertex-sorted ELL pattern, the triangle->slot map, stretch coefficients
 * (InitStretchCoef, :517-553), the constant Q-bending matrix
 * (InitBendingMatrix/UpdateBendingMatrix, :573-680), lumped masses and gravity,
 * and uploads everything. The initial state is x = x_pre = mesh->pos. */
int cloth_create(cloth_ctx *ctx, const cloth_mesh_desc *mesh,
                 const cloth_material *mat, cloth_t **out);
int cloth_destroy(cloth_t *cloth);
int cloth_num_vertices(const cloth_t *cloth, int *nv, int *nt, int *ne);
/* Sparsity of the system matrix: nonzero 3x3 blocks (all of them, as the
 * reference's ELL holds them), the widest row, and the bytes of device memory
 * the cloth holds resident and per solve. */
int cloth_matrix_info(const cloth_t *cloth, long long *nnzb, int *width,
                      size_t *resident_bytes, size_t *solve_bytes);
/* Changes stretch/bending stiffness and damping (the reference's ImGui sliders,
 * BaraffClothGpu.cpp:282-291, and UpdateBendingMatrix). */
int cloth_set_material(cloth_t *cloth, const cloth_material *mat);

/* Static points: cBaseCloth::InitConstraint / FindVerticesIdFromUV
 * (BaseCloth.cpp:151-235), AddConstraintStaticVertices /
 * ClearConstraintStaticVertices (BaseCloth.cpp:553-563). Targets are the rest
 * positions, as cBaraffClothGpu::InitConstraint sets (BaraffClothGpu.cpp:372-384). */
int cloth_find_vertices_from_uv(const cloth_t *cloth, const float *uv, int n,
                                int *vids);
int cloth_add_static_vertices(cloth_t *cloth, const int *vids, int n);
int cloth_clear_static_vertices(cloth_t *cloth);
int cloth_get_static_vertices(const cloth_t *cloth, int *vids, int cap, int *n);
/* Drag point for the next step only (ApplyUserPerturbForceOnce,
 * BaraffClothGpu.cpp:266-281). */
int cloth_set_drag_point(cloth_t *cloth, int vid, const float target[3]);

/* State (cBaseCloth::SetPos/SetPrePos/GetPos, BaseCloth.cpp:97-112;
 * UpdatePosToCuda/UpdatePosToCpu, BaraffClothGpu.cpp:304-335). Positions are
 * kept in FP64 on the device, as the reference keeps them on the host. */
int cloth_set_pos(cloth_t *cloth, const double *x, int nv);
int cloth_set_pre_pos(cloth_t *cloth, const double *x, int nv);
int cloth_get_pos(cloth_t *cloth, double *x, int nv);
int cloth_get_pre_pos(cloth_t *cloth, double *x, int nv);
/* cBaraffClothGpu::Reset (BaraffClothGpu.cpp:293-299): x = x_pre = rest, dx = 0. */
int cloth_reset(cloth_t *cloth);

/* One implicit step (cBaraffClothGpu::UpdatePos, BaraffClothGpu.cpp:152-265):
 * snap pins, assemble A and b, PCG, x_pre = x, x += dx; all on the device.
 * dt <= 0 uses default_timestep. params NULL = library defaults
 * (rel_tol 1e-6, max_iters 1000, check every iteration, warm start).
 * stats may be NULL; when given, the call waits for the step to finish. */
int cloth_step(cloth_t *cloth, double dt, const cloth_solve_params *params,
               cloth_solve_stats *stats);
/* The same step with host buffers, as the reference's UpdatePos exchanges them:
 * upload x and x_pre, step, download x (any of the pointers may be NULL). */
int cloth_step_host(cloth_t *cloth, double dt, const cloth_solve_params *params,
                    const double *x_in, const double *x_pre_in, double *x_out,
                    cloth_solve_stats *stats);

/* ---------------------------------------------------------------- seam */
/* Assembled system: replaces BaraffClothGpu::UpdateStretchStiffnessMatrixAndFint,
 * AddBendingHessianAndIntForce, AssembleSystemRHS and AssembleSystemMatrix
 * (BaraffClothGpu.cpp:52-82, BaraffClothGpu.cu:127-483). Snaps pins first,
 * then builds A (pin-projected), b, the block-Jacobi inverse and the PCG start. */
int cloth_assemble(cloth_t *cloth, double dt);
/* Replaces PCGSolver::Solve (PCGSolver.cu:332-481) on the assembled system;
 * the solution stays on the device as dx (cloth_get_dx). */
int cloth_solve(cloth_t *cloth, const cloth_solve_params *params,
                cloth_solve_stats *stats);
/* x_pre = x; x += dx (BaraffClothGpu.cpp:246-258). */
int cloth_advance(cloth_t *cloth);
/* Statistics of the cloth's last solve (waits for the context's stream). */
int cloth_get_stats(cloth_t *cloth, cloth_solve_stats *stats);
int cloth_get_dx(cloth_t *cloth, double *dx, int nv);

/* Exports in the reference's layout for parity checks: ell (nv*32, -1 padded,
 * as mELLVidToGlobalVid), A (nv*32*9, row-major blocks, pinned rows/columns
 * zeroed off the diagonal), b (nv*3), fint (nv*3: stretch + bending force),
 * kbend (nv*32: bending scalar per block, the +K_b of mBendingStiffnessMatrixCuda).
 * Any output pointer may be NULL. */
int cloth_export_system(cloth_t *cloth, int *ell, float *A, float *b,
                        float *fint, float *kbend);
/* Per-triangle results of the last assembly: fint nt*9 (force on local vertex
 * a at [3a+k]) and hess nt*81 (block (a,b) at [9*(3a+b)], row-major). */
int cloth_export_triangles(cloth_t *cloth, float *fint, float *hess);
/* Per-interior-edge results of the last assembly of a dihedral-bending cloth
 * (cDihedralMaterial::Update, src/sim/cloth/DihedralBending.cpp:382-450):
 * n_edges, edge_ids (n_edges: edge index of each interior edge), grad
 * (n_edges*12: dbeta/dx of stencil vertices v0 v1 v2 v3) and coef (n_edges*2:
 * the factor c = -K e / (h0 + h1) and c beta / 2).  Zero edges for the
 * quadratic model.  Any output pointer may be NULL. */
int cloth_export_dihedral(cloth_t *cloth, int *n_edges, int *edge_ids, float *grad,
                          float *coef);
/* Init-time tables: stencil ne*4 (mEdgeAffectVertexId, -1 on the boundary),
 * coef nt*12 (Fu/Fv warp-weft, Fu/Fv diagonal), area nt, mass nv,
 * tri_slot nt*9 (ELL slot of vertex b in row of vertex a). */
int cloth_export_tables(const cloth_t *cloth, int *stencil, float *coef,
                        float *area, float *mass, int *tri_slot);

/* The reference GPU path's structure, re-expressed, as the comparison
 * baseline ("plain GPU PCG"): cBaraffClothGpu::UpdatePos
 * (BaraffClothGpu.cpp:152-265) with its host round trips (pins snapped and
 * positions kept in double on the host, float copies uploaded, dx downloaded
 * and added on the host), its assembly kernels (float atomics, 32-wide slot
 * search, BaraffClothGpu.cu:111-483) and PCGSolver::Solve (PCGSolver.cu:332-481:
 * four launches per iteration, float single-address atomic dot products, the
 * residual downloaded and its norm taken on the host every check_every-th
 * iteration). params NULL = the reference's settings (100 iterations,
 * ||r|| < 1e-10 absolute, checked every 10). The cloth's state is updated. */
int cloth_step_plain(cloth_t *cloth, double dt, const cloth_solve_params *params,
                     cloth_solve_stats *stats);

/* ---------------------------------------------------------------- precision */
/* FP64 checks and solvers on the assembled system (after cloth_assemble). The
 * system is the assembled one: FP32 blocks and right-hand side, exact in FP64.
 * The reference solves it in FP32 only (PCGSolver::Solve,
 * src/sim/cloth/gpu_solvers/PCGSolver.cu:332-481); its FP64 counterparts are
 * the CPU path's Eigen solvers (src/utils/SparseUtil.h). */
typedef struct {
    int outer;                     /* refinement steps (FP32 corrections) */
    int inner_iters;               /* FP32 PCG iterations over all corrections */
    int status;                    /* CLOTH_OK: reached rel_tol; MAXITER; NAN; BREAKDOWN */
    int solver;                    /* driver of the FP32 corrections */
    double initial_rel_residual;   /* ||b|| relative residual of dx = 0 (= 1) */
    double rel_residual;           /* final ||b - A dx|| / ||b||, FP64 */
    double last_inner_rel_residual;
    int rejected;                  /* corrections undone (failed, or raised the residual) */
    int pad;
} cloth_refine_stats;

/* ||b - A dx|| / ||b|| with the residual formed in FP64 (dx: the FP64 result
 * of the last refined or FP64 solve, else the FP32 dx). */
int cloth_residual_fp64(cloth_t *cloth, double *rel_residual);
/* Mixed-precision iterative refinement: dx = 0; repeat r = b - A dx in FP64;
 * stop when ||r|| <= rel_tol ||b||; solve A e = float(r) with the FP32 PCG
 * (inner: its iteration cap and relative tolerance); dx += e in FP64. At most
 * max_outer corrections. A correction whose FP32 solve fails (NaN, p.Ap = 0)
 * or that does not lower the FP64 residual is undone and retried with half
 * the inner iterations. The FP64 dx is what cloth_get_dx and cloth_advance
 * use afterwards. */
int cloth_solve_refined(cloth_t *cloth, const cloth_solve_params *inner, double rel_tol,
                        int max_outer, cloth_refine_stats *stats);
/* All-FP64 block-Jacobi PCG (FP64 vectors, FP64 inverse diagonal blocks, FP64
 * reductions) from dx = 0, for comparison; recurrence residual in stats.
 * The FP64 paths allocate their work arrays on a cloth's first FP64 call and
 * keep them (cloth_ctx_device_bytes counts them): FP64 vectors, and an FP64
 * copy of the stored blocks that each solve refreshes (48 B per stored block,
 * 80 B with dihedral bending), since GB300's FP64 pipe, not memory, bounds the
 * FP64 SpMV. */
int cloth_solve_fp64(cloth_t *cloth, const cloth_solve_params *params,
                     cloth_solve_stats *stats);
/* Flexible CG in FP64 (Notay's FCG(1): each direction A-orthogonalised
 * against the last) preconditioned by inner->max_iters FP32 PCG iterations
 * from zero on the same assembled system; FP64 vectors and SpMV, stop at
 * ||r|| <= rel_tol ||b|| (FP64), at most max_outer FP64 iterations.  Meant
 * for systems too ill-conditioned for the FP32 corrections of
 * cloth_solve_refined.  stats: outer = FP64 iterations, inner_iters = FP32
 * iterations, rejected = inner solves that failed (NaN, breakdown) and were
 * replaced by the FP64 block-Jacobi step; rel_residual is the FP64 residual of
 * the result.  The FP64 dx is what cloth_get_dx and cloth_advance use. */
int cloth_solve_flexible(cloth_t *cloth, const cloth_solve_params *inner, double rel_tol,
                         int max_outer, cloth_refine_stats *stats);

/* ---------------------------------------------------------------- collisions */
/* Static kinematic bodies (cKinematicBody after Init, src/sim/kinematic/
 * KinematicBody.cpp:27-121): a world-space triangle mesh; edges numbered as
 * cObjUtil::BuildEdge numbers them, triangle normals (v1-v0)x(v2-v1)
 * normalised, vertex normals the init-area-weighted sum of theirs. */
typedef struct cloth_body_s cloth_body;
int cloth_body_create(cloth_ctx *ctx, int nv, int nt, const double *pos, const int *tris,
                      cloth_body **out);
/* Fails while a cloth still collides with the body. */
int cloth_body_destroy(cloth_body *body);
/* Moving bodies (cKinematicBody with "is_static": false, KinematicBody.cpp:
 * Update, UpdateCurWorldTransformByTime, SetMeshPos). A body's normals stay
 * those its Init computed, as the reference's moving body keeps them; the
 * broad-phase boxes and grid are rebuilt for the new positions, and the next
 * step of a cloth colliding with the body detects contacts against them.
 * set_pos: any new world-space vertex positions (nv*3, same triangles). */
int cloth_body_set_pos(cloth_body *body, const double *pos);
/* The reference's time-driven motion: the body's vertices are the local mesh
 * (nv*3; the scaled OBJ vertices) posed by a translation and XYZ Euler angles
 * (Rz Ry Rx) interpolated linearly from init to target over elapsed_sec of
 * body time, then held. set_motion places the body at the initial pose (body
 * time 0) and recomputes its normals there (Init); update adds dt to the
 * body clock (a float, as mCurTime) and moves the body to its pose. */
int cloth_body_set_motion(cloth_body *body, const double *local, const double *init_pos,
                          const double *init_ori, const double *target_pos,
                          const double *target_ori, double elapsed_sec);
int cloth_body_update(cloth_body *body, float dt);
int cloth_body_get_pos(cloth_body *body, double *pos);
/* The same pose on the host, no device needed: world = pose(time) * local. */
int cloth_kinematic_pose(int nv, const double *local, const double *init_pos,
                         const double *init_ori, const double *target_pos,
                         const double *target_ori, double elapsed_sec, float time,
                         double *world);

/* The CPU cloth's collision handling (cSimScene::PerformCollisionDetection
 * with cBVHCollisionDetecter, src/sim/collision/BVHCollisionDetecter.cpp, and
 * cBaraffCloth::PrepareCollisionHessian / Repulsion, src/sim/cloth/
 * BaraffCloth.cpp:614-990) in this cloth's step, against the bodies in order
 * (the cloth being the first object of the scene).  Each step: contacts of
 * the positions the step starts from (triangle pairs whose 5 mm boxes meet;
 * cloth points and body triangles, body points and cloth triangles, cloth and
 * body edges closer than 3 mm, in the detecter's order); 1e-2 dC/dx dC/dx^T
 * per point-triangle contact added to the system matrix; after the solve the
 * contacts' impulses on dx (edge-edge contacts first, each seeing dx as the
 * earlier ones left it).  n = 0 turns collisions off.  A cloth with bodies is
 * stepped alone (not in a batch or by the request server). */
int cloth_set_bodies(cloth_t *cloth, cloth_body *const *bodies, int n);
/* Capacities of the triangle-pair, point-triangle and edge-edge lists (0:
 * the default for the cloth's size).  A step whose contacts do not fit
 * reports CLOTH_ERR_CONTACTS. */
int cloth_set_contact_capacity(cloth_t *cloth, int pairs, int point_triangle, int edge_edge);
typedef struct {
    int n_pt, n_ee;          /* contacts of the last step */
    int overflow;            /* a list ran out of capacity */
    int repulsion_rounds;    /* rounds of the ordered repulsion */
} cloth_contact_stats;
/* Contacts of the last step in the detecter's order: pt_i (cloth point?,
 * point id, triangle id) n_pt*3, pt_d (normal xyz, depth, barycentric xyz)
 * n_pt*7, ee_i (1, cloth edge, body edge) n_ee*3, ee_d (normal xyz, depth,
 * s, t) n_ee*6.  Any pointer may be NULL. */
int cloth_get_contacts(cloth_t *cloth, cloth_contact_stats *stats, int *pt_i, double *pt_d,
                       int *ee_i, double *ee_d);
/* dx after the last step's repulsion (nv*3, FP64). */
int cloth_get_repulsed_dx(cloth_t *cloth, double *dx, int nv);

/* ---------------------------------------------------------------- batch */
/* Many cloths of uneven sizes stepped together: one launch per phase covers
 * every instance (a packed tile list over all of them), each instance keeps its
 * own FP64 scalars, convergence test and iteration count, and the PCG loop is a
 * CUDA graph with a device-side while condition. All cloths must share ctx.
 * Each instance's result is bit-identical to stepping it alone. */
int cloth_batch_step(cloth_ctx *ctx, cloth_t *const *cloths, int n, double dt,
                     const cloth_solve_params *params, cloth_solve_stats *stats);

/* ---------------------------------------------------------------- serving */
/* Request server with continuous batching. The reference steps one cloth per
 * call on the host thread (cBaseCloth::Update -> UpdatePos,
 * src/sim/cloth/BaseCloth.cpp, src/sim/cloth/BaraffClothGpu.cpp:203-262);
 * this is the batch/serve variant over handle arrays.
 *
 * Registered cloths stay resident (mesh tables, ELL map, positions, the
 * warm-start dx, pins); a step request needs per-solve work memory (triangle
 * records, the assembled system, PCG vectors: about 1.1 KB per vertex) that
 * the server hands out from one pool. The pool is the device-memory budget
 * minus the resident bytes of the registered cloths and the server's own
 * buffers. A worker thread runs the device in chunks of chunk_iters PCG
 * iterations; between chunks it admits ready requests in arrival order while
 * a slot (max_inflight) and pool memory are free, so their assembly and PCG
 * run on the GPU beside requests already iterating, and it retires requests
 * whose solve ended (the position update runs on the device). Requests for
 * one cloth run one after another, in submission order. Every request's
 * arithmetic is per instance and fixed-order, so its result is bit-identical
 * to stepping that cloth alone with the graph-loop solver. */
typedef struct cloth_server_s cloth_server;

typedef struct {
    size_t budget_bytes;   /* device bytes the server may hold (resident + pool + own) */
    int max_inflight;      /* requests on the GPU at once (<= 0: no limit but memory) */
    int chunk_iters;       /* PCG iterations per chunk between admissions (> 0) */
} cloth_server_config;

typedef struct {
    long long tag;         /* caller's tag from cloth_server_submit */
    int cloth;             /* index from cloth_server_add */
    int status;            /* CLOTH_OK or the solve's per-instance status */
    int iters;             /* PCG iterations of this step */
    int pad;
    double rel_residual;   /* ||r|| / ||b|| at exit (FP64 recurrence) */
    double t_arrival;      /* cloth_server_now() clock, seconds */
    double t_admit;        /* when the request joined a chunk */
    double t_done;         /* when the worker saw the step finished */
} cloth_server_result;

typedef struct {
    long long submitted, completed, chunks;
    long long admitted_waits;   /* admissions deferred for lack of pool memory or slots */
    int max_inflight_seen;
    int registered;
    size_t resident_bytes;      /* registered cloths' resident state */
    size_t pool_bytes;          /* per-solve pool */
    size_t pool_peak_bytes;     /* largest pool use seen */
    size_t own_bytes;           /* the server's lists and descriptors */
    size_t max_request_bytes;   /* work memory of the largest registered cloth's request */
} cloth_server_stats;

/* Monotonic clock of the server (seconds), for arrival times. */
double cloth_server_now(void);
int cloth_server_create(cloth_ctx *ctx, const cloth_server_config *cfg, cloth_server **out);
/* Register a cloth (same ctx) with the dt and solve parameters its requests
 * use (dt <= 0: the material's default timestep; params NULL: defaults). The
 * cloth's own work memory is released; until the server is destroyed the
 * cloth is stepped only through the server (get/set_pos work while it has no
 * request queued or running). CLOTH_ERR_BUDGET when its resident bytes do not
 * fit the budget. Only before cloth_server_start. */
int cloth_server_add(cloth_server *srv, cloth_t *cloth, double dt,
                     const cloth_solve_params *params, int *index);
/* Allocate the pool (CLOTH_ERR_BUDGET when the largest registered cloth's
 * work memory does not fit) and start the worker thread. */
int cloth_server_start(cloth_server *srv);
/* Queue one step of cloth `index`. t_arrival < 0: now. Thread-safe. */
int cloth_server_submit(cloth_server *srv, int index, long long tag, double t_arrival);
/* Completed requests, oldest first: waits up to wait_s seconds for at least
 * one, returns at most cap in out and their count in *n. Thread-safe. */
int cloth_server_poll(cloth_server *srv, cloth_server_result *out, int cap, int *n,
                      double wait_s);
/* Wait until every submitted request has completed (wait_s < 0: no limit);
 * CLOTH_ERR_TIMEOUT when the time ran out. */
int cloth_server_drain(cloth_server *srv, double wait_s);
int cloth_server_get_stats(cloth_server *srv, cloth_server_stats *stats);
/* Stop the worker (requests still queued are dropped), hand every cloth its
 * own work memory back and free the server. */
int cloth_server_destroy(cloth_server *srv);

/* ---------------------------------------------------------------- no allocation */
/* Allocation-free PCG solve. No counterpart in the reference: this entry point
 * exists for callers that cannot allocate device memory when they solve - a
 * render or physics loop that must not stall on cudaMalloc or fail for lack of
 * memory in the middle of a frame, or a host whose device memory belongs to
 * another allocator or budget. It solves A x = b (block-Jacobi PCG, FP32
 * vectors, FP64 reductions) on a system the caller has assembled in the
 * reference's layout: ell_dev nv*32 vertex ids (-1 padded, sorted, as
 * mELLVidToGlobalVid), A_dev nv*32 3x3 blocks of 9 floats, column-major
 * (tCudaMatrix3f), b_dev and x_dev nv*3 floats; x_dev is the start and the
 * result. Rows and columns of the fixed_dev vertices are left out, and their
 * x entries are set to zero. All pointers are device pointers on the current
 * device; the work runs on `stream` (a cudaStream_t, NULL = default stream).
 * Nothing is allocated: the solver's scratch (4 MiB) is a static array that
 * every GPU loading this library holds until the process exits, which limits
 * nv to 32768; larger systems are rejected with CLOTH_ERR_INVALID, and so is
 * an ELL column id >= nv (found before any SpMV runs). Every call looks up the
 * array's device address on the current device and reuses the same array:
 * calls that may overlap on the GPU race and must be serialised by the caller.
 * The call blocks the host: it waits on `stream` for the solver state every
 * eight iterations, so it can never be stream-captured; on a capturing stream
 * it returns CLOTH_ERR_STATE and leaves the stream alone. Returns the solve's
 * own status: CLOTH_OK only when the tolerance was reached, else
 * CLOTH_ERR_MAXITER, CLOTH_ERR_NAN or CLOTH_ERR_BREAKDOWN (stats, when given,
 * say the same). */
int cloth_pcg_solve_ell32_noalloc(int nv, const int *ell_dev, const float *A_dev,
                                  const float *b_dev, float *x_dev, const int *fixed_dev,
                                  int nfixed, const cloth_solve_params *params,
                                  cloth_solve_stats *stats, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CLOTH_GB300_H */
