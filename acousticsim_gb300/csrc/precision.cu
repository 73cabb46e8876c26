// FP64 paths of the solve: the true residual r = b - A dx in FP64, mixed
// precision iterative refinement (FP32 PCG corrections inside an FP64
// residual loop), and an all-FP64 block-Jacobi PCG for comparison.
//
// The system is the assembled one (FP32 blocks and right-hand side from the
// assembly kernels, exact in FP64): both solvers answer the same question, so
// their difference is the solver's precision alone.  The reference's solver
// is PCGSolver::Solve (src/sim/cloth/gpu_solvers/PCGSolver.cu:332-481, FP32
// throughout); its FP64 counterpart on the CPU side is Eigen's solvers on the
// same matrix (src/utils/SparseUtil.h).
//
// Kernels walk the rows of one cloth with a grid-stride loop; sums go through
// per-block FP64 partials that the last block (ticket) adds in block order,
// so every result is deterministic.
#include "internal.h"

#include <algorithm>
#include <cmath>

using namespace cloth;
using namespace cloth::detail;

namespace {

int pfail(int code, const std::string &msg)
{
    set_last_error(msg);
    return code;
}

#define PCK(call)                                                              \
    do                                                                         \
    {                                                                          \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                 \
            return pfail(CLOTH_ERR_CUDA,                                       \
                         std::string(#call) + ": " + cudaGetErrorString(e_));  \
    } while (0)

constexpr int kB64 = 256; // threads per block of the FP64 kernels

struct F64State
{
    double rho, pq, alpha, beta, rr, bb;
    double res2, bnorm2;  // true residual of the last k64_resid
    double rel_tol2, abs_tol2;
    int iter, active, status, max_iters;
    unsigned ticket;
    int fallbacks; // flexible CG: inner solves replaced by the FP64 block-Jacobi step
    int pad[2];
};

struct F64Ptr
{
    double *dx, *r, *z, *p, *q, *M;   // nv*3 each; M: nv*6 (symmetric inverse)
    double *part;                     // 3 * nblk partials
    F64State *st;
    int nblk;
    // the stored blocks in FP64 (the assembled FP32 planes converted, exactly,
    // by k64_mat before each solve): GB300's FP64 pipe is narrow, and the
    // conversions would otherwise run in the SpMV's inner loop every iteration
    double4_32a *B0;
    double2 *B1;
    double4_32a *Bw; // skew parts (dihedral bending), else null
};

__device__ __forceinline__ double sumw(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sums of N values, then the grid's last block adds the per-block
// partials in block order. Returns true in every thread of the last block,
// with the totals in tot.
template <int N>
__device__ bool grid_reduce(double (&v)[N], double *part, int nblk, unsigned *ticket,
                            double (&tot)[N])
{
    __shared__ double sh[N][kB64 / 32];
    __shared__ int last;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < N; k++)
    {
        const double s = sumw(v[k]);
        if (l == 0)
            sh[k][w] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < N; k++)
        {
            double s = 0.0;
            for (int j = 0; j < kB64 / 32; j++)
                s += sh[k][j];
            part[k * nblk + blockIdx.x] = s;
        }
        __threadfence();
        last = (atomicAdd(ticket, 1u) == unsigned(nblk - 1));
    }
    __syncthreads();
    if (!last)
        return false;
    __threadfence();
    // the last block adds the partials: thread t takes partials t, t + B, ...
    // (fixed order), then the block sum as above
#pragma unroll
    for (int k = 0; k < N; k++)
    {
        double s = 0.0;
        for (int j = threadIdx.x; j < nblk; j += kB64)
            s += __ldcg(&part[k * nblk + j]);
        s = sumw(s);
        __syncthreads();
        if (l == 0)
            sh[k][w] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < N; k++)
        {
            double s = 0.0;
            for (int j = 0; j < kB64 / 32; j++)
                s += sh[k][j];
            tot[k] = s;
        }
        *ticket = 0u;
    }
    return true;
}

// The fields of the assembled system the FP64 kernels read, loaded once per
// thread (the descriptor lives in global memory; held in registers here the
// slot loop does not reload them).
struct Mat64
{
    int nv, wl, wu;
    const int *__restrict__ rowinfo;
    const int *__restrict__ colu;
    const uint32_t *__restrict__ lref;
    const float4 *__restrict__ A0;
    const float2 *__restrict__ A1;
    const float4 *__restrict__ Aw;
    const float4 *__restrict__ dx;
    __device__ explicit Mat64(const InstDesc &d)
        : nv(d.nv), wl(d.width_lo), wu(d.width_up), rowinfo(d.rowinfo), colu(d.colu),
          lref(d.lref), A0(d.A0), A1(d.A1), Aw(d.Aw), dx(d.dx)
    {
    }
};

// The stored blocks' entries as FP64 values: the assembled FP32 planes
// (converted as they are read) or their FP64 copy; both give the same values.
struct F32Blocks
{
    const float4 *__restrict__ A0;
    const float2 *__restrict__ A1;
    const float4 *__restrict__ Aw;
    __device__ explicit F32Blocks(const Mat64 &m) : A0(m.A0), A1(m.A1), Aw(m.Aw) {}
    __device__ bool skew() const { return Aw != nullptr; }
    __device__ void sym(uint32_t o, double a[6]) const
    {
        const float4 u = A0[o];
        const float2 w = A1[o];
        a[0] = u.x, a[1] = u.y, a[2] = u.z, a[3] = u.w, a[4] = w.x, a[5] = w.y;
    }
    __device__ void w3(uint32_t o, double w[3]) const
    {
        const float4 u = Aw[o];
        w[0] = u.x, w[1] = u.y, w[2] = u.z;
    }
};
struct F64Blocks
{
    const double4_32a *__restrict__ B0;
    const double2 *__restrict__ B1;
    const double4_32a *__restrict__ Bw;
    __device__ explicit F64Blocks(const F64Ptr &f) : B0(f.B0), B1(f.B1), Bw(f.Bw) {}
    __device__ bool skew() const { return Bw != nullptr; }
    __device__ void sym(uint32_t o, double a[6]) const
    {
        const double4_32a u = B0[o];
        const double2 w = B1[o];
        a[0] = u.x, a[1] = u.y, a[2] = u.z, a[3] = u.w, a[4] = w.x, a[5] = w.y;
    }
    __device__ void w3(uint32_t o, double w[3]) const
    {
        const double4_32a u = Bw[o];
        w[0] = u.x, w[1] = u.y, w[2] = u.z;
    }
};

// y = A v on one row in FP64, slots in column order: the lower ones (block at
// the transposed position), then the diagonal and upper ones. v: nv*3
// doubles, or the FP32 dx when v64 is null.
template <class Blocks>
__device__ __forceinline__ void row_mul64(const Mat64 &d, const Blocks &B, int row,
                                          const double *__restrict__ v64, double *y)
{
    const int info = d.rowinfo[row];
    const int len = info & 255, ds = (info >> 8) & 255;
    y[0] = y[1] = y[2] = 0.0;
    for (int s = 0; s < len; s++)
    {
        const bool lower = s < ds;
        int c;
        uint32_t oa;
        if (lower)
        {
            const uint32_t ref = d.lref[lo_idx(s, row, d.wl)];
            c = lref_col(ref);
            oa = lref_block(ref, d.wu);
        }
        else
        {
            oa = up_idx(s - ds, row, d.wu);
            c = d.colu[oa];
        }
        double a[6];
        B.sym(oa, a);
        double x0, x1, x2;
        if (v64)
        {
            x0 = v64[3 * c];
            x1 = v64[3 * c + 1];
            x2 = v64[3 * c + 2];
        }
        else
        {
            const float4 f = d.dx[c];
            x0 = f.x;
            x1 = f.y;
            x2 = f.z;
        }
        // fused multiply-adds written out (device code is built without
        // contraction); GB300's FP64 pipe is narrow, so halving the FP64
        // instructions is what this loop is about
        y[0] = fma(a[2], x2, fma(a[1], x1, fma(a[0], x0, y[0])));
        y[1] = fma(a[4], x2, fma(a[3], x1, fma(a[1], x0, y[1])));
        y[2] = fma(a[5], x2, fma(a[4], x1, fma(a[2], x0, y[2])));
        if (B.skew())
        {
            // skew part (dihedral bending): + w x v on stored blocks, - on
            // the transposed ones (a sign flip, exact)
            double w[3];
            B.w3(oa, w);
            const double wx = lower ? -w[0] : w[0], wy = lower ? -w[1] : w[1],
                         wz = lower ? -w[2] : w[2];
            y[0] += wy * x2 - wz * x1;
            y[1] += wz * x0 - wx * x2;
            y[2] += wx * x1 - wy * x0;
        }
    }
}

// r = b - A dx in FP64 (dx: dx64, or the FP32 dx when dx64 is null);
// st.res2 = ||r||^2, st.bnorm2 = ||b||^2.
__global__ void __launch_bounds__(kB64) k64_resid(const InstDesc *dp, const double *dx64,
                                                  double *r64, F64Ptr f)
{
    const InstDesc &d = *dp;
    const Mat64 m(d);
    double v[2] = {0.0, 0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < m.nv;
         row += gridDim.x * blockDim.x)
    {
        double y[3];
        row_mul64(m, F32Blocks(m), row, dx64, y);
        const float4 b = d.b[row];
        const double r0 = double(b.x) - y[0], r1 = double(b.y) - y[1], r2 = double(b.z) - y[2];
        r64[3 * row] = r0;
        r64[3 * row + 1] = r1;
        r64[3 * row + 2] = r2;
        v[0] += r0 * r0 + r1 * r1 + r2 * r2;
        v[1] += double(b.x) * b.x + double(b.y) * b.y + double(b.z) * b.z;
    }
    double tot[2];
    if (grid_reduce<2>(v, f.part, f.nblk, &f.st->ticket, tot) && threadIdx.x == 0)
    {
        f.st->res2 = tot[0];
        f.st->bnorm2 = tot[1];
    }
}

// dx64 += dx32 (one refinement correction)
__global__ void k64_accum(const InstDesc *dp, double *dx64)
{
    const InstDesc &d = *dp;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
    {
        const float4 e = d.dx[row];
        dx64[3 * row] += double(e.x);
        dx64[3 * row + 1] += double(e.y);
        dx64[3 * row + 2] += double(e.z);
    }
}

// dx32 = float(dx64): the FP32 copy the next step warm-starts from
__global__ void k64_to32(const InstDesc *dp, const double *dx64)
{
    const InstDesc &d = *dp;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
        d.dx[row] = make_float4(float(dx64[3 * row]), float(dx64[3 * row + 1]),
                                float(dx64[3 * row + 2]), 0.f);
}

// x_pre = x, x += dx64 (FP64 result of the refinement or of the FP64 PCG)
__global__ void k64_advance(const InstDesc *dp, const double *dx64)
{
    const InstDesc &d = *dp;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
    {
        double x[3];
#pragma unroll
        for (int k = 0; k < 3; k++)
        {
            const double xo = d.x64[3 * row + k];
            d.xp64[3 * row + k] = xo;
            x[k] = xo + dx64[3 * row + k];
            d.x64[3 * row + k] = x[k];
        }
        d.x32[row] = make_float4(float(x[0]), float(x[1]), float(x[2]), 0.f);
    }
}

__device__ __forceinline__ void symv64(const double *m, const double *v, double *y)
{
    y[0] = fma(m[2], v[2], fma(m[1], v[1], m[0] * v[0]));
    y[1] = fma(m[4], v[2], fma(m[3], v[1], m[1] * v[0]));
    y[2] = fma(m[5], v[2], fma(m[4], v[1], m[2] * v[0]));
}

// FP64 PCG start: M = inverse of the FP64 diagonal block (adjugate), dx = 0,
// r = b, z = M r; rho = r.z, rr = r.r, bb = b.b.
__global__ void __launch_bounds__(kB64) k64_init(const InstDesc *dp, F64Ptr f)
{
    const InstDesc &d = *dp;
    double v[3] = {0.0, 0.0, 0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
    {
        // plane 0 holds the diagonal block
        const float4 u = d.A0[up_idx(0, row, d.width_up)];
        const float2 uw = d.A1[up_idx(0, row, d.width_up)];
        const double a[6] = {u.x, u.y, u.z, u.w, uw.x, uw.y};
        const double c00 = a[3] * a[5] - a[4] * a[4], c01 = a[2] * a[4] - a[1] * a[5],
                     c02 = a[1] * a[4] - a[2] * a[3], c11 = a[0] * a[5] - a[2] * a[2],
                     c12 = a[2] * a[1] - a[0] * a[4], c22 = a[0] * a[3] - a[1] * a[1];
        const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
        const double inv = 1.0 / det;
        double m[6] = {c00 * inv, c01 * inv, c02 * inv, c11 * inv, c12 * inv, c22 * inv};
#pragma unroll
        for (int k = 0; k < 6; k++)
            f.M[6 * row + k] = m[k];
        const float4 b = d.b[row];
        const double r[3] = {b.x, b.y, b.z};
        double z[3];
        symv64(m, r, z);
#pragma unroll
        for (int k = 0; k < 3; k++)
        {
            f.dx[3 * row + k] = 0.0;
            f.r[3 * row + k] = r[k];
            f.z[3 * row + k] = z[k];
            f.p[3 * row + k] = 0.0;
        }
        v[0] = fma(r[2], z[2], fma(r[1], z[1], fma(r[0], z[0], v[0])));
        v[1] = fma(r[2], r[2], fma(r[1], r[1], fma(r[0], r[0], v[1])));
    }
    v[2] = v[1];
    double tot[3];
    if (grid_reduce<3>(v, f.part, f.nblk, &f.st->ticket, tot) && threadIdx.x == 0)
    {
        F64State &s = *f.st;
        s.rho = tot[0];
        s.rr = tot[1];
        s.bb = tot[2];
        s.beta = 0.0;
        s.alpha = 0.0;
        s.iter = 0;
        s.status = 0;
        const bool conv = (s.rel_tol2 > 0.0 && s.rr <= s.rel_tol2 * s.bb) ||
                          (s.abs_tol2 > 0.0 && s.rr <= s.abs_tol2);
        s.active = (s.max_iters > 0 && !conv && isfinite(tot[0])) ? 1 : 0;
        if (!isfinite(tot[0]))
            s.status = CLOTH_ERR_NAN;
    }
}

__global__ void k64_cond(const F64State *st, cudaGraphConditionalHandle h)
{
    cudaGraphSetConditional(h, st->active ? 1u : 0u);
}

// p = z + beta p
__global__ void k64_p(const InstDesc *dp, F64Ptr f)
{
    const InstDesc &d = *dp;
    if (!f.st->active)
        return;
    const double beta = f.st->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * d.nv;
         i += gridDim.x * blockDim.x)
        f.p[i] = fma(beta, f.p[i], f.z[i]);
}

// The stored blocks in FP64 (every plane entry, padding included), before a
// solve that runs k64_spmv.
__global__ void __launch_bounds__(kB64) k64_mat(const InstDesc *dp, F64Ptr f)
{
    const InstDesc &d = *dp;
    const size_t n = size_t(d.width_up) * size_t(d.ntile_rows) * kTile;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += size_t(gridDim.x) * blockDim.x)
    {
        const float4 a = d.A0[i];
        const float2 b = d.A1[i];
        f.B0[i] = make_double4_32a(a.x, a.y, a.z, a.w);
        f.B1[i] = make_double2(b.x, b.y);
        if (f.Bw && d.Aw)
        {
            const float4 w = d.Aw[i];
            f.Bw[i] = make_double4_32a(w.x, w.y, w.z, 0.0);
        }
    }
}

// q = A p, pq = p.q -> alpha
__global__ void __launch_bounds__(kB64) k64_spmv(const InstDesc *dp, F64Ptr f,
                                                 cudaGraphConditionalHandle h, int use_cond)
{
    const InstDesc &d = *dp;
    if (!f.st->active)
        return;
    double v[1] = {0.0};
    const Mat64 m(d);
    const F64Blocks B(f);
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < m.nv;
         row += gridDim.x * blockDim.x)
    {
        double y[3];
        row_mul64(m, B, row, f.p, y);
#pragma unroll
        for (int k = 0; k < 3; k++)
            f.q[3 * row + k] = y[k];
        v[0] = fma(f.p[3 * row + 2], y[2], fma(f.p[3 * row + 1], y[1], fma(f.p[3 * row], y[0], v[0])));
    }
    double tot[1];
    if (grid_reduce<1>(v, f.part, f.nblk, &f.st->ticket, tot) && threadIdx.x == 0)
    {
        F64State &s = *f.st;
        s.pq = tot[0];
        if (!isfinite(tot[0]))
        {
            s.status = CLOTH_ERR_NAN;
            s.active = 0;
        }
        else if (tot[0] == 0.0)
        {
            s.status = CLOTH_ERR_BREAKDOWN;
            s.active = 0;
        }
        else
            s.alpha = s.rho / tot[0];
        if (!s.active && use_cond)
            cudaGraphSetConditional(h, 0u);
    }
}

// dx += alpha p, r -= alpha q, z = M r; r.z, r.r -> beta, convergence
__global__ void __launch_bounds__(kB64) k64_update(const InstDesc *dp, F64Ptr f,
                                                   cudaGraphConditionalHandle h)
{
    const InstDesc &d = *dp;
    if (!f.st->active)
        return;
    const double alpha = f.st->alpha;
    double v[2] = {0.0, 0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
    {
        double r[3], z[3], m[6];
#pragma unroll
        for (int k = 0; k < 3; k++)
        {
            f.dx[3 * row + k] = fma(alpha, f.p[3 * row + k], f.dx[3 * row + k]);
            r[k] = fma(-alpha, f.q[3 * row + k], f.r[3 * row + k]);
            f.r[3 * row + k] = r[k];
        }
#pragma unroll
        for (int k = 0; k < 6; k++)
            m[k] = f.M[6 * row + k];
        symv64(m, r, z);
#pragma unroll
        for (int k = 0; k < 3; k++)
            f.z[3 * row + k] = z[k];
        v[0] += r[0] * z[0] + r[1] * z[1] + r[2] * z[2];
        v[1] += r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    }
    double tot[2];
    if (grid_reduce<2>(v, f.part, f.nblk, &f.st->ticket, tot) && threadIdx.x == 0)
    {
        F64State &s = *f.st;
        s.beta = (s.rho == 0.0) ? 0.0 : tot[0] / s.rho;
        s.rho = tot[0];
        s.rr = tot[1];
        s.iter++;
        const bool conv = (s.rel_tol2 > 0.0 && s.rr <= s.rel_tol2 * s.bb) ||
                          (s.abs_tol2 > 0.0 && s.rr <= s.abs_tol2);
        if (!isfinite(tot[0]) || !isfinite(tot[1]))
        {
            s.status = CLOTH_ERR_NAN;
            s.active = 0;
        }
        else if (conv)
            s.active = 0;
        else if (s.iter >= s.max_iters)
        {
            s.status = CLOTH_ERR_MAXITER;
            s.active = 0;
        }
        if (!s.active)
            cudaGraphSetConditional(h, 0u);
    }
}

// ---- flexible CG with FP32 PCG inner solves (cloth_solve_flexible)
// z = the FP32 inner solve's dx (or M r in FP64 when the inner solve failed:
// NaN or breakdown); rho = z.r and zq = z.q (q = A p of the last outer step);
// then beta = -zq / pq (Notay's FCG(1): p orthogonalised against the last
// direction in the A inner product), 0 at the first step.
__global__ void __launch_bounds__(kB64) k64_fcg_z(const InstDesc *dp, F64Ptr f, int first)
{
    const InstDesc &d = *dp;
    const int st = d.st->status;
    const bool use_inner = (st == CLOTH_OK || st == CLOTH_ERR_MAXITER);
    double v[2] = {0.0, 0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
    {
        double z[3], r[3];
#pragma unroll
        for (int k = 0; k < 3; k++)
            r[k] = f.r[3 * row + k];
        if (use_inner)
        {
            const float4 e = d.dx[row];
            z[0] = e.x;
            z[1] = e.y;
            z[2] = e.z;
        }
        else
        {
            double m[6];
#pragma unroll
            for (int k = 0; k < 6; k++)
                m[k] = f.M[6 * row + k];
            symv64(m, r, z);
        }
#pragma unroll
        for (int k = 0; k < 3; k++)
            f.z[3 * row + k] = z[k];
        v[0] = fma(z[2], r[2], fma(z[1], r[1], fma(z[0], r[0], v[0])));
        if (!first)
            v[1] = fma(z[2], f.q[3 * row + 2],
                       fma(z[1], f.q[3 * row + 1], fma(z[0], f.q[3 * row], v[1])));
    }
    double tot[2];
    if (grid_reduce<2>(v, f.part, f.nblk, &f.st->ticket, tot) && threadIdx.x == 0)
    {
        F64State &s = *f.st;
        s.rho = tot[0];
        s.beta = first ? 0.0 : -tot[1] / s.pq;
        if (!use_inner)
            s.fallbacks++;
    }
}

// dx += alpha p, r -= alpha q; rr = r.r
__global__ void __launch_bounds__(kB64) k64_fcg_update(const InstDesc *dp, F64Ptr f)
{
    const InstDesc &d = *dp;
    if (!f.st->active)
        return;
    const double alpha = f.st->alpha;
    double v[1] = {0.0};
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
    {
#pragma unroll
        for (int k = 0; k < 3; k++)
        {
            f.dx[3 * row + k] = fma(alpha, f.p[3 * row + k], f.dx[3 * row + k]);
            const double r = fma(-alpha, f.q[3 * row + k], f.r[3 * row + k]);
            f.r[3 * row + k] = r;
            v[0] = fma(r, r, v[0]);
        }
    }
    double tot[1];
    if (grid_reduce<1>(v, f.part, f.nblk, &f.st->ticket, tot) && threadIdx.x == 0)
        f.st->rr = tot[0];
}

struct F64Work
{
    char *mem = nullptr;
    size_t bytes = 0;
    F64Ptr f{};
    double *dx64 = nullptr; // refinement result (also the FP64 PCG result)
    double *dx64_prev = nullptr;
    double *r64 = nullptr;
    cudaGraphExec_t pcg = nullptr;
    int grid = 0;
};

} // namespace

struct cloth_f64_s
{
    F64Work w;
};

namespace {

// FP64 work arrays of a cloth, allocated on first use.
int f64_work(cloth_s *c, F64Work **out)
{
    if (!c->f64)
    {
        auto *p = new cloth_f64_s();
        const int n = c->tab.nv;
        const int grid = std::max(1, c->ctx->num_sms * 8);
        Layout L;
        size_t o_dx = L.take<double>(3 * size_t(n)), o_r = L.take<double>(3 * size_t(n)),
               o_z = L.take<double>(3 * size_t(n)), o_p = L.take<double>(3 * size_t(n)),
               o_q = L.take<double>(3 * size_t(n)), o_M = L.take<double>(6 * size_t(n)),
               o_dx64 = L.take<double>(3 * size_t(n)), o_r64 = L.take<double>(3 * size_t(n)),
               o_prev = L.take<double>(3 * size_t(n)),
               o_part = L.take<double>(3 * size_t(grid)), o_st = L.take<F64State>(1);
        // FP64 copies of the stored blocks (every plane entry of whole tiles)
        const size_t nb = size_t(c->h.width_up) * size_t(c->h.ntile_rows) * kTile;
        const bool dih = c->mat.bending_model == 1;
        const size_t o_B0 = L.take<double4_32a>(nb), o_B1 = L.take<double2>(nb),
                     o_Bw = dih ? L.take<double4_32a>(nb) : 0;
        if (cudaMalloc(&p->w.mem, L.off) != cudaSuccess)
        {
            cudaGetLastError();
            delete p;
            return pfail(CLOTH_ERR_OOM, "FP64 work arrays: device allocation failed");
        }
        p->w.bytes = L.off;
        char *b = p->w.mem;
        p->w.f.dx = reinterpret_cast<double *>(b + o_dx);
        p->w.f.r = reinterpret_cast<double *>(b + o_r);
        p->w.f.z = reinterpret_cast<double *>(b + o_z);
        p->w.f.p = reinterpret_cast<double *>(b + o_p);
        p->w.f.q = reinterpret_cast<double *>(b + o_q);
        p->w.f.M = reinterpret_cast<double *>(b + o_M);
        p->w.f.part = reinterpret_cast<double *>(b + o_part);
        p->w.f.st = reinterpret_cast<F64State *>(b + o_st);
        p->w.f.nblk = grid;
        p->w.f.B0 = reinterpret_cast<double4_32a *>(b + o_B0);
        p->w.f.B1 = reinterpret_cast<double2 *>(b + o_B1);
        p->w.f.Bw = dih ? reinterpret_cast<double4_32a *>(b + o_Bw) : nullptr;
        p->w.dx64 = reinterpret_cast<double *>(b + o_dx64);
        p->w.r64 = reinterpret_cast<double *>(b + o_r64);
        p->w.dx64_prev = reinterpret_cast<double *>(b + o_prev);
        p->w.grid = grid;
        if (cudaMemsetAsync(b, 0, L.off, c->ctx->stream) != cudaSuccess)
        {
            cudaFree(p->w.mem);
            delete p;
            return pfail(CLOTH_ERR_CUDA, "FP64 work arrays: memset failed");
        }
        c->f64 = p;
        c->ctx->bytes += L.off;
    }
    *out = &c->f64->w;
    return CLOTH_OK;
}

int add_k(cudaGraph_t g, cudaGraphNode_t *last, void *fn, int grid, int block, void **args)
{
    cudaKernelNodeParams p;
    std::memset(&p, 0, sizeof(p));
    p.func = fn;
    p.gridDim = dim3(grid);
    p.blockDim = dim3(block);
    p.kernelParams = args;
    cudaGraphNode_t n;
    PCK(cudaGraphAddKernelNode(&n, g, *last ? last : nullptr, *last ? 1 : 0, &p));
    *last = n;
    return CLOTH_OK;
}

// Graph of the FP64 PCG: init, then while (active) { p; spmv; update }.
int build_f64_graph(cloth_s *c, F64Work *w)
{
    cudaGraph_t g = nullptr;
    PCK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h = 0;
    int rc = CLOTH_OK;
    if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess)
    {
        cudaGraphDestroy(g);
        return pfail(CLOTH_ERR_CUDA, "FP64 PCG: conditional handle");
    }
    const InstDesc *dp = c->d_desc;
    F64Ptr f = w->f;
    const F64State *stc = f.st;
    void *a_init[] = {&dp, &f};
    void *a_cond[] = {&stc, &h};
    void *a_p[] = {&dp, &f};
    int one = 1;
    void *a_spmv[] = {&dp, &f, &h, &one};
    void *a_upd[] = {&dp, &f, &h};
    cudaGraphNode_t last = nullptr;
    rc = add_k(g, &last, (void *)k64_init, w->grid, kB64, a_init);
    if (rc == CLOTH_OK)
        rc = add_k(g, &last, (void *)k64_cond, 1, 1, a_cond);
    if (rc == CLOTH_OK)
    {
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cn;
        if (cudaGraphAddNode(&cn, g, &last, nullptr, 1, &cp) != cudaSuccess)
            rc = pfail(CLOTH_ERR_CUDA, "FP64 PCG: conditional node");
        else
        {
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            cudaGraphNode_t bl = nullptr;
            rc = add_k(body, &bl, (void *)k64_p, w->grid, kB64, a_p);
            if (rc == CLOTH_OK)
                rc = add_k(body, &bl, (void *)k64_spmv, w->grid, kB64, a_spmv);
            if (rc == CLOTH_OK)
                rc = add_k(body, &bl, (void *)k64_update, w->grid, kB64, a_upd);
        }
    }
    if (rc == CLOTH_OK && cudaGraphInstantiate(&w->pcg, g, 0) != cudaSuccess)
        rc = pfail(CLOTH_ERR_CUDA, "FP64 PCG: cudaGraphInstantiate failed");
    cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
}

int sync_read_state(cloth_s *c, F64Work *w, F64State *out)
{
    PCK(cudaMemcpyAsync(out, w->f.st, sizeof(F64State), cudaMemcpyDeviceToHost,
                        c->ctx->stream));
    PCK(cudaStreamSynchronize(c->ctx->stream));
    return CLOTH_OK;
}

int check_solvable(cloth_s *c, const char *who)
{
    if (!c)
        return pfail(CLOTH_ERR_INVALID, std::string(who) + ": cloth is NULL");
    if (!c->scratch)
        return pfail(CLOTH_ERR_STATE, std::string(who) + ": the cloth is held by a server");
    if (!c->assembled)
        return pfail(CLOTH_ERR_STATE, std::string(who) + ": call cloth_assemble first");
    return CLOTH_OK;
}

int resid(cloth_s *c, F64Work *w, const double *dx64, double *rel)
{
    k64_resid<<<w->grid, kB64, 0, c->ctx->stream>>>(c->d_desc, dx64, w->r64, w->f);
    PCK(cudaGetLastError());
    F64State st;
    int rc = sync_read_state(c, w, &st);
    if (rc != CLOTH_OK)
        return rc;
    *rel = st.bnorm2 > 0 ? std::sqrt(st.res2 / st.bnorm2) : std::sqrt(st.res2);
    return CLOTH_OK;
}

} // namespace

void cloth::detail::f64_free(cloth_s *c)
{
    if (!c->f64)
        return;
    if (c->f64->w.pcg)
        cudaGraphExecDestroy(c->f64->w.pcg);
    if (c->f64->w.mem)
    {
        cudaFree(c->f64->w.mem);
        c->ctx->bytes -= std::min(c->ctx->bytes, c->f64->w.bytes);
    }
    delete c->f64;
    c->f64 = nullptr;
    c->dx64_valid = false;
}

int cloth::detail::f64_advance(cloth_s *c)
{
    F64Work *w = nullptr;
    int rc = f64_work(c, &w);
    if (rc != CLOTH_OK)
        return rc;
    const int grid = std::max(1, std::min(c->ctx->num_sms * 8, (c->tab.nv + 255) / 256));
    k64_advance<<<grid, 256, 0, c->ctx->stream>>>(c->d_desc, w->dx64);
    PCK(cudaGetLastError());
    return CLOTH_OK;
}

// FP32 copy of the FP64 solution (the next step's warm start)
__global__ void k64_dx32(const InstDesc *dp, const double *dx64)
{
    const InstDesc &d = *dp;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
        d.dx[row] = make_float4(float(dx64[3 * row]), float(dx64[3 * row + 1]),
                                float(dx64[3 * row + 2]), 0.f);
}

int cloth::detail::escalate_step(cloth_s *c, const cloth_solve_params *p,
                                 cloth_solve_stats *out)
{
    // the FP32 PCG ended in NaN or breakdown (or, at escalation level 2, at
    // max_iters) on the assembled system (the advance left the state alone):
    // the system is beyond FP32 there, so the step is re-solved by the
    // all-FP64 block-Jacobi PCG from zero to the step's tolerance, then
    // x += dx in FP64
    cloth_solve_params q = *p;
    q.warm_start = 0;
    if (!(q.rel_tol > 0) && !(q.abs_tol > 0))
        q.rel_tol = 1e-6;
    q.max_iters = std::max(q.max_iters, 100000);
    const double rhs = out->rhs_norm;
    int rc = cloth_solve_fp64(c, &q, out);
    if (rc != CLOTH_OK)
        return rc;
    out->solver = CLOTH_SOLVER_ESCALATED;
    if (!(out->rhs_norm > 0))
        out->rhs_norm = rhs;
    if (out->status != CLOTH_OK)
        return CLOTH_OK;
    F64Work *w = nullptr;
    rc = f64_work(c, &w);
    if (rc != CLOTH_OK)
        return rc;
    rc = f64_advance(c);
    if (rc != CLOTH_OK)
        return rc;
    const int grid = std::max(1, std::min(c->ctx->num_sms * 8, (c->tab.nv + 255) / 256));
    k64_dx32<<<grid, 256, 0, c->ctx->stream>>>(c->d_desc, w->dx64);
    PCK(cudaGetLastError());
    return CLOTH_OK;
}

int cloth::detail::f64_get_dx(cloth_s *c, double *dx, int nv)
{
    F64Work *w = nullptr;
    int rc = f64_work(c, &w);
    if (rc != CLOTH_OK)
        return rc;
    PCK(cudaMemcpyAsync(dx, w->dx64, size_t(nv) * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                        c->ctx->stream));
    PCK(cudaStreamSynchronize(c->ctx->stream));
    return CLOTH_OK;
}

extern "C" {

int cloth_residual_fp64(cloth_t *c, double *rel_residual)
{
    int rc = check_solvable(c, "cloth_residual_fp64");
    if (rc != CLOTH_OK)
        return rc;
    if (!rel_residual)
        return pfail(CLOTH_ERR_INVALID, "cloth_residual_fp64: NULL output");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    PCK(cudaSetDevice(c->ctx->device));
    F64Work *w = nullptr;
    rc = f64_work(c, &w);
    if (rc != CLOTH_OK)
        return rc;
    return resid(c, w, c->dx64_valid ? w->dx64 : nullptr, rel_residual);
}

int cloth_solve_fp64(cloth_t *c, const cloth_solve_params *params, cloth_solve_stats *stats)
{
    int rc = check_solvable(c, "cloth_solve_fp64");
    if (rc != CLOTH_OK)
        return rc;
    if (!params || params->max_iters < 0)
        return pfail(CLOTH_ERR_INVALID, "cloth_solve_fp64: bad parameters");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    PCK(cudaSetDevice(c->ctx->device));
    F64Work *w = nullptr;
    rc = f64_work(c, &w);
    if (rc != CLOTH_OK)
        return rc;
    if (!w->pcg && (rc = build_f64_graph(c, w)) != CLOTH_OK)
        return rc;
    F64State st0;
    std::memset(&st0, 0, sizeof(st0));
    st0.rel_tol2 = params->rel_tol > 0 ? params->rel_tol * params->rel_tol : 0.0;
    st0.abs_tol2 = params->abs_tol > 0 ? params->abs_tol * params->abs_tol : 0.0;
    st0.max_iters = params->max_iters;
    PCK(cudaMemcpyAsync(w->f.st, &st0, sizeof(st0), cudaMemcpyHostToDevice, c->ctx->stream));
    k64_mat<<<w->grid, kB64, 0, c->ctx->stream>>>(c->d_desc, w->f);
    PCK(cudaGetLastError());
    PCK(cudaGraphLaunch(w->pcg, c->ctx->stream));
    PCK(cudaMemcpyAsync(w->dx64, w->f.dx, size_t(c->tab.nv) * 3 * sizeof(double),
                        cudaMemcpyDeviceToDevice, c->ctx->stream));
    const int grid = std::max(1, std::min(c->ctx->num_sms * 8, (c->tab.nv + 255) / 256));
    k64_to32<<<grid, 256, 0, c->ctx->stream>>>(c->d_desc, w->dx64);
    PCK(cudaGetLastError());
    F64State st;
    rc = sync_read_state(c, w, &st);
    if (rc != CLOTH_OK)
        return rc;
    c->dx64_valid = true;
    c->pcg_stale = true;
    if (stats)
    {
        stats->iters = st.iter;
        stats->status = st.status;
        stats->res_norm = std::sqrt(std::max(0.0, st.rr));
        stats->rhs_norm = std::sqrt(std::max(0.0, st.bb));
        stats->rel_residual =
            stats->rhs_norm > 0 ? stats->res_norm / stats->rhs_norm : stats->res_norm;
        stats->solver = CLOTH_SOLVER_FP64;
    }
    return CLOTH_OK;
}

int cloth_solve_refined(cloth_t *c, const cloth_solve_params *inner, double rel_tol,
                        int max_outer, cloth_refine_stats *stats)
{
    int rc = check_solvable(c, "cloth_solve_refined");
    if (rc != CLOTH_OK)
        return rc;
    if (!inner || inner->max_iters < 0 || !(rel_tol > 0) || max_outer <= 0)
        return pfail(CLOTH_ERR_INVALID, "cloth_solve_refined: bad parameters");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    PCK(cudaSetDevice(c->ctx->device));
    F64Work *w = nullptr;
    rc = f64_work(c, &w);
    if (rc != CLOTH_OK)
        return rc;
    cudaStream_t s = c->ctx->stream;
    const size_t vbytes = size_t(c->tab.nv) * 3 * sizeof(double);
    PCK(cudaMemsetAsync(w->dx64, 0, vbytes, s));
    cloth_refine_stats out;
    std::memset(&out, 0, sizeof(out));
    out.status = CLOTH_ERR_MAXITER;
    const int grid = std::max(1, std::min(c->ctx->num_sms * 8, (c->tab.nv + 255) / 256));
    // Safeguard: FP32 PCG on a matrix this ill-conditioned can lose its way
    // (p.Ap of the wrong sign, a growing residual). A correction that fails or
    // that raises the FP64 residual is rejected (dx64 restored) and the step
    // is retried with half as many inner iterations as the failed one ran.
    cloth_solve_params ip = *inner;
    double rel = 0.0, best = 0.0;
    bool have_prev = false, restored = false;
    for (int k = 0;; k++)
    {
        rc = resid(c, w, w->dx64, &rel);
        if (rc != CLOTH_OK)
            return rc;
        if (k == 0)
        {
            out.initial_rel_residual = rel;
            best = rel;
        }
        else if (have_prev && !(rel < best))
        {
            // the last correction did not help: undo it
            PCK(cudaMemcpyAsync(w->dx64, w->dx64_prev, vbytes, cudaMemcpyDeviceToDevice, s));
            out.rejected++;
            rel = best;
            ip.max_iters = std::max(8, ip.max_iters / 2);
            restored = true;
        }
        else
            best = rel;
        have_prev = false;
        if (!std::isfinite(rel))
        {
            out.status = CLOTH_ERR_NAN;
            break;
        }
        if (rel <= rel_tol)
        {
            out.status = CLOTH_OK;
            break;
        }
        if (out.outer >= max_outer || out.rejected > 6)
            break;
        // FP32 correction: A e = float(r), then dx64 += e
        if (restored)
        {
            // the residual of the restored dx64 (r64 holds the rejected one's)
            rc = resid(c, w, w->dx64, &rel);
            if (rc != CLOTH_OK)
                return rc;
            restored = false;
        }
        cloth_solve_stats is;
        rc = inner_solve(c, w->r64, &ip, &is);
        if (rc != CLOTH_OK)
            return rc;
        out.outer++;
        out.inner_iters += is.iters;
        out.last_inner_rel_residual = is.rel_residual;
        out.solver = is.solver;
        if (is.status != CLOTH_OK && is.status != CLOTH_ERR_MAXITER)
        {
            // NaN or breakdown inside the correction: retry shorter
            out.rejected++;
            ip.max_iters = std::max(8, std::min(ip.max_iters, is.iters) / 2);
            continue;
        }
        PCK(cudaMemcpyAsync(w->dx64_prev, w->dx64, vbytes, cudaMemcpyDeviceToDevice, s));
        have_prev = true;
        k64_accum<<<grid, 256, 0, s>>>(c->d_desc, w->dx64);
        PCK(cudaGetLastError());
    }
    out.rel_residual = rel;
    k64_to32<<<grid, 256, 0, s>>>(c->d_desc, w->dx64);
    PCK(cudaGetLastError());
    PCK(cudaStreamSynchronize(s));
    c->dx64_valid = true;
    c->pcg_stale = true;
    if (stats)
        *stats = out;
    return CLOTH_OK;
}

int cloth_solve_flexible(cloth_t *c, const cloth_solve_params *inner, double rel_tol,
                         int max_outer, cloth_refine_stats *stats)
{
    int rc = check_solvable(c, "cloth_solve_flexible");
    if (rc != CLOTH_OK)
        return rc;
    if (!inner || inner->max_iters <= 0 || !(rel_tol > 0) || max_outer <= 0)
        return pfail(CLOTH_ERR_INVALID, "cloth_solve_flexible: bad parameters");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    PCK(cudaSetDevice(c->ctx->device));
    F64Work *w = nullptr;
    rc = f64_work(c, &w);
    if (rc != CLOTH_OK)
        return rc;
    cudaStream_t s = c->ctx->stream;
    const int grid = w->grid;
    const InstDesc *dp = c->d_desc;
    F64Ptr f = w->f;
    // FP64 start: dx = 0, r = b, the FP64 block-Jacobi inverse (fallback
    // preconditioner), bb = b.b
    F64State st0;
    std::memset(&st0, 0, sizeof(st0));
    st0.max_iters = 1; // k64_init marks the state active
    PCK(cudaMemcpyAsync(f.st, &st0, sizeof(st0), cudaMemcpyHostToDevice, s));
    k64_mat<<<grid, kB64, 0, s>>>(dp, f);
    k64_init<<<grid, kB64, 0, s>>>(dp, f);
    PCK(cudaGetLastError());
    F64State hs;
    rc = sync_read_state(c, w, &hs);
    if (rc != CLOTH_OK)
        return rc;
    const double bb = hs.bb;
    cloth_refine_stats out;
    std::memset(&out, 0, sizeof(out));
    out.status = CLOTH_ERR_MAXITER;
    out.initial_rel_residual = 1.0;
    double rel = bb > 0 ? std::sqrt(hs.rr / bb) : 0.0;
    cudaGraphConditionalHandle none = 0;
    for (int k = 0; k < max_outer; k++)
    {
        if (!std::isfinite(rel))
        {
            out.status = CLOTH_ERR_NAN;
            break;
        }
        if (rel <= rel_tol)
        {
            out.status = CLOTH_OK;
            break;
        }
        // z ~ A^-1 r by max_iters FP32 PCG iterations from zero
        cloth_solve_stats is;
        rc = inner_solve(c, f.r, inner, &is);
        if (rc != CLOTH_OK)
            return rc;
        out.inner_iters += is.iters;
        out.last_inner_rel_residual = is.rel_residual;
        k64_fcg_z<<<grid, kB64, 0, s>>>(dp, f, k == 0 ? 1 : 0);
        k64_p<<<grid, kB64, 0, s>>>(dp, f);
        k64_spmv<<<grid, kB64, 0, s>>>(dp, f, none, 0);
        k64_fcg_update<<<grid, kB64, 0, s>>>(dp, f);
        PCK(cudaGetLastError());
        rc = sync_read_state(c, w, &hs);
        if (rc != CLOTH_OK)
            return rc;
        out.outer++;
        rel = bb > 0 ? std::sqrt(hs.rr / bb) : 0.0;
        out.rejected = hs.fallbacks;
        if (!hs.active)
        {
            // p.Ap zero or not finite in the outer step
            out.status = hs.status ? hs.status : CLOTH_ERR_BREAKDOWN;
            break;
        }
    }
    if (out.status == CLOTH_ERR_MAXITER && rel <= rel_tol)
        out.status = CLOTH_OK;
    // the recurrence residual agrees with the FP64 one to rounding; report
    // the FP64 residual of the result
    PCK(cudaMemcpyAsync(w->dx64, f.dx, size_t(c->tab.nv) * 3 * sizeof(double),
                        cudaMemcpyDeviceToDevice, s));
    double relt = 0.0;
    rc = resid(c, w, w->dx64, &relt);
    if (rc != CLOTH_OK)
        return rc;
    out.rel_residual = relt;
    out.solver = CLOTH_SOLVER_FP64;
    k64_to32<<<grid, 256, 0, s>>>(c->d_desc, w->dx64);
    PCK(cudaGetLastError());
    PCK(cudaStreamSynchronize(s));
    c->dx64_valid = true;
    c->pcg_stale = true;
    if (stats)
        *stats = out;
    return CLOTH_OK;
}

} // extern "C"
