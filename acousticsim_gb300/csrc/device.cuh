// Device-side data layout of the implicit cloth step (sm_103a).
//
// One cloth instance = one InstDesc (pointers into its device arena) plus one
// InstState (its FP64 PCG scalars and convergence bookkeeping).  Kernels walk a
// list of 128-row (or 128-triangle) tiles; a tile never straddles instances,
// so every reduction is per instance and a cloth's arithmetic does not depend
// on which other cloths share the launch.
//
// Block ELL, slot-major: entry (row, slot) of an array with per-slot planes is
// at [slot * stride + row], so a warp's 32 rows read 32 consecutive elements of
// each plane.  A 3x3 block is symmetric (stretch, shear, bending, mass and the
// Rayleigh terms all are), so it is stored as 6 floats:
//   A0 = (a00, a01, a02, a11)  as float4,   A1 = (a12, a22) as float2.
// The matrix is block-symmetric bit for bit (block (i,j) and block (j,i) sum
// the same triangle records in the same order, the bending scalars are
// symmetric, the pin projection zeroes both), so only the diagonal and upper
// blocks (column >= row) are stored: row i's slots are sorted by column, the
// first diag_slot(i) of them are lower, and upper slot s lives in plane
// u = s - diag_slot(i) (u = 0: the diagonal block).  A lower slot keeps a
// reference to its transposed block (lref: that block's plane and column);
// the SpMV fetches the block, which another row of the same launch has just
// streamed, from L2.  The SpMV walks the lower slots by s and the upper ones
// by u, with the upper columns in planes of their own (colu), so that at
// every step the 32 rows of a warp read one plane of each array: coalesced,
// whatever the rows' diag_slot.  The stored blocks, colu and lref are kept
// tile-major (up_idx / lo_idx below).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cloth {

constexpr int kTile = 128;     // rows or triangles per tile = threads per block
constexpr int kMaxWidth = 32;  // ELL width limit (tCudaVector32i in the reference)

// Triangle record of the assembly pass: one per (triangle, a, b), 32 bytes.
// h = upper triangle of the 3x3 block (00 01 02 11 12 22), pad = 0.
struct __align__(16) HRec
{
    float4 h0; // 00 01 02 11
    float4 h1; // 12 22 pad pad
};

// Contacts of a cloth with kinematic bodies (the CPU cloth's collision
// handling, src/sim/collision/BVHCollisionDetecter.cpp and
// src/sim/cloth/BaraffCloth.cpp:614-990).
struct PtContact
{
    int cloth_point;  // 1: cloth point p against body triangle t; 0: body point p against cloth triangle t
    int p, t;
    float depth;      // (distance vector).normal, kept as float as the reference does
    double n[3];      // outer normal
    float bary[3];    // barycentric coordinates of the closest point on t
    int pad;
};
struct EeContact
{
    int e0, e1;       // cloth edge, body edge
    float s, t;       // closest-point parameters on e0 and e1
    double n[3];
    float depth;
    int pad;
};
// Entries of the per-vertex contact lists: an edge-edge contact index, or a
// point-triangle index with this bit set (so a sorted list runs in the
// reference's repulsion order: edge-edge contacts first).
constexpr int kPtTag = 0x40000000;
struct CollideCounts
{
    int n_pt, n_ee;   // contacts so far
    int overflow;     // a list exceeded its capacity (contacts lost)
    int rounds;       // repulsion rounds run
    int cap_inc;      // capacity of the per-vertex contact lists
    int pad[3];
};

struct InstState
{
    // FP64 PCG scalars
    double rho;     // r.z of the current iterate
    double pq;      // p.Ap of the current iteration
    double alpha, beta;
    double rr;      // ||r||^2
    double bb;      // ||b||^2
    double rr0;     // ||r0||^2
    // control
    int iter;
    int active;
    int status;
    unsigned ticket;
    // team barrier of the persistent solver (reset by the assembly)
    unsigned bar_count;
    unsigned bar_gen;
    int bar_err;
    int open;       // step assembled and not yet advanced (request server)
    // exact fixed-point team sums of the persistent solver, triple-buffered by
    // iteration: [buffer][quantity: p.q, r.z, r.r][limb: units of 2^32, units]
    unsigned long long acc[3][3][2];
    float acc_chk[3][3];  // FP32 magnitude check of the same sums
    float pad2[3];
};

struct InstDesc
{
    int nv, nt, width, stride;   // stride: padded row count of slot-major planes
    int width_lo, width_up;      // planes of lower slots (lref) and of stored blocks
    int ntile_rows, ntile_tris;
    int warm_start;
    int fix_fv_norm;
    int max_iters;
    int check_every;
    int hold_maxiter; // a solve ending at max_iters keeps the state too (to be escalated)
    int pad_hold;
    double rel_tol2; // rel_tol^2 (0 = off)
    double abs_tol2; // abs_tol^2 (0 = off)
    float k_warp, k_weft, k_bias;
    float h2;        // dt^2
    float c_mass;    // 1 + dt * rayleigh_a
    float c_stiff;   // dt * rayleigh_b - dt^2
    // triangles
    const int4 *tri;      // (v0, v1, v2, float_as_int(rest area))
    const float4 *tcoef;  // 3 per triangle: FuWW FvWW FuD FvD (12 floats)
    const int4 *tdest;    // 3 per triangle: h_dest[9], f_dest[3]
    // rows
    const int *col;       // [slot][stride] column (vertex) ids
    const uint32_t *lref; // lower slots, tile-major (lo_idx): u << 24 | column, the
                          // transposed block being upper plane u of that column's row
    const int *colu;      // upper slots, tile-major (up_idx): columns
    const uint32_t *hsrc; // [slot][stride] first record << 5 | record count
    const float *kb;      // [slot][stride] bending scalar (+K_b)
    const int *rowinfo;   // len | diag_slot << 8
    const int2 *thalo;    // per 128-row tile: the column range [x, y) its rows touch
    const int *fptr;      // nv+1 force-record ranges
    const float *mass;    // nv
    const float *grav;    // nv: gravity force (y component)
    // pins
    const int *pin_vid;     // npins
    const float4 *pin_tgt;  // npins
    int npins;
    // dihedral bending (all null, n_dih = 0, with the quadratic model)
    int n_dih;               // interior edges
    const int4 *dvid;        // n_dih stencils (v0 v1 v2 v3)
    const double *dfac;      // n_dih rest factors -K e / (h0 + h1)
    const uint32_t *dsrc;    // [slot][stride] first entry << 5 | entry count
    const uint32_t *dent;    // entries q << 4 | a << 2 | b
    // records written by the triangle pass
    HRec *hrec;
    float4 *frec;
    float4 *drec;            // 4 per interior edge: dbeta/dx_a (xyz), factor (w)
    float *dfb;              // per interior edge: factor * beta / 2
    // assembled system
    float4 *A0;          // diagonal and upper blocks, tile-major (up_idx)
    float2 *A1;
    float4 *Aw;          // skew part w of those blocks (block p = S p + w x p), or null
    // contacts with kinematic bodies (all null without bodies)
    const PtContact *cpt;
    const int *cinc_off;  // nv+1 per-vertex contact list ranges
    const int *cinc;      // per-vertex contact lists (sorted)
    const CollideCounts *ccount;
    double *dxr;          // nv*3: dx after the repulsion (FP64), used by the advance
    float4 *M0; // block-Jacobi inverse, symmetric: (00 01 02 11)
    float2 *M1; // (12 22)
    float4 *b;
    // state and PCG vectors (nv float4 each; .w unused except x32.w)
    double *x64, *xp64;  // nv*3
    float4 *x32;         // float copy of x; .w = 1 on pinned vertices
    float4 *dx, *r, *z, *p0, *p1, *q;
    float4 *w1;          // second buffer of w (single-barrier persistent PCG)
    double *part;        // 3 * ntile_rows reduction partials
    InstState *st;
};

// Tile-major planes.  The arrays of the stored (diagonal and upper) blocks
// and of the lower-slot references are kept per 128-row tile: entry (row,
// plane u) of an array with w planes is at ((row / 128) * w + u) * 128 +
// row % 128.  A warp's 32 rows still read 32 consecutive entries of one
// plane, and one tile's planes of an array are contiguous (a single bulk
// copy).  A lower-slot reference packs the transposed block's plane and
// column: u << 24 | c (meshes of up to 2^24 vertices).
static_assert(kTile == 128, "tile-major plane indexing assumes 128-row tiles");
constexpr uint32_t kLrefColMask = 0xFFFFFFu;
constexpr int kMaxClothVertices = 1 << 24;
__host__ __device__ __forceinline__ uint32_t up_idx(int u, int row, int width_up)
{
    return (uint32_t(row >> 7) * uint32_t(width_up) + uint32_t(u)) * uint32_t(kTile) +
           uint32_t(row & (kTile - 1));
}
__host__ __device__ __forceinline__ uint32_t lo_idx(int s, int row, int width_lo)
{
    return (uint32_t(row >> 7) * uint32_t(width_lo) + uint32_t(s)) * uint32_t(kTile) +
           uint32_t(row & (kTile - 1));
}
__host__ __device__ __forceinline__ int lref_col(uint32_t ref) { return int(ref & kLrefColMask); }
__host__ __device__ __forceinline__ uint32_t lref_block(uint32_t ref, int width_up)
{
    return up_idx(int(ref >> 24), int(ref & kLrefColMask), width_up);
}

// A tile carries its instance's descriptor and state addresses, so the PCG
// kernels reach both with one dependent load instead of walking the
// descriptor table and then the descriptor.
struct Tile
{
    int inst;
    int start;
    InstDesc *d;
    InstState *st;
};

// One block of the persistent PCG grid: a contiguous row range of one
// instance.  The instance's blocks form its team and meet at team barriers;
// p is staged in shared memory over [halo0, halo1), which covers every column
// the block's rows touch (halo0 = -1: the range did not fit, gather from L2).
struct TeamBlock
{
    int inst;   // index in the launch set, -1 = idle block
    int rank;   // rank in the team
    int nblk;   // team size
    int row0, row1;
    int halo0, halo1;
    int p_global; // the team keeps p in global memory (a block of it is not staged)
};

// Fixed-point scale: sums are carried as round(v * 2^s) with s chosen from
// the previous value of the same quantity so that it maps to about 2^kFxTop.
constexpr int kFxTop = 70;

constexpr int kPBlock = 1024;                // threads per persistent block
// The persistent block's own-row M^-1 in shared memory (true) or read from
// L2 each iteration (false): shared memory and L1 share one array per SM, so
// less shared memory leaves more L1 for the matrix stream.
constexpr bool kPersistMShared = true; // measured: false is 3 % slower at 512^2
constexpr int kRedRows = 32;                 // team ranges align to 32-row chunks (the FP32 warp sums)
constexpr int kSlotUnroll = 2;               // ELL slots whose loads are issued together
constexpr int kStageUnroll = 2;              // staged z rows per thread loaded together
constexpr int kMaxBlockRows = 16384;         // rows one persistent block may own
constexpr unsigned kSpinLimitDefault = 1u << 25; // bounded barrier wait (~seconds)

// Bounded waits of the persistent solvers' team barriers: a wait gives up
// after `limit` polls (the team's error flag is set and the solve ends with
// CLOTH_ERR_TIMEOUT).  `extra` arrivals are added to every barrier's target:
// 0 in normal use; a test sets it to make the waits run out (arrivals that no
// block makes), which exercises the timeout path without any device fault.
struct SpinCfg
{
    unsigned limit;
    unsigned extra;
};

// One variant of a graph-loop kernel: R rows per thread (blocks of kTile / R
// threads), U ELL slots whose loads are issued together (SpMV only), TPB
// consecutive tiles taken by a block at a time.
struct GraphLoopVariant
{
    int rows_per_thread;
    int slot_unroll;
    int tiles_per_block;
    const void *func;
    int bulk_stages; // > 0: bulk-staged SpMV with a ring of this many stages
    int bulk_halo;   // the bulk SpMV also stages p over each tile's column range
};

// PCG iterations per body of the graph loop's conditional while node
// (measured on 256 cloths: 1, 2, 4 iterations per body give 38.1, 36.7 and
// 35.8 ms per batched step)
constexpr int kLoopBodyIters = 4;

// Bulk-staged SpMV (k_spmv_bulk): kTile consumer threads plus one producer
// warp per block; a tile's staged column range (halo) holds at most
// kBulkHaloCap rows, wider tiles gather p from global memory.
constexpr int kBulkThreads = kTile + 32;
constexpr int kBulkHaloCap = 2048;

// Batch-wide control words (one per launch set).
struct BatchCtl
{
    int n_active;    // instances still iterating
    int n_tiles_rows;
    int n_tiles_tris;
    int err;         // a bounded wait of the graph-loop kernels gave up (sticky until read)
    int hand_off;    // the graph loop ends once this many instances or fewer iterate
                     // (the host finishes them with the persistent kernel); 0: to the end
    int pad[3];
};

} // namespace cloth
