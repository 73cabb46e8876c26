// Allocation-free PCG solve (cloth_pcg_solve_ell32_noalloc).
//
// Some callers cannot allocate device memory when they need a solve: a
// render or physics loop that must not stall on cudaMalloc (it synchronises
// the device) or risk an out-of-memory failure mid-frame, a host process whose
// device memory is owned by another allocator or budget, or a plugin that is
// only handed buffers.  This entry point takes the caller's assembled system
// and solution buffer and keeps every other byte it needs (residual,
// search directions, preconditioner, reduction partials, solver scalars) in
// one static device array that the library image carries.
//
// The array is file-scope, 4 MiB, and every GPU that loads the library keeps
// it until the process exits.  It bounds the system to kNaMaxVertices
// vertices.  Every call uses the same array: calls that overlap on the GPU
// (other streams, other host threads) race and must be serialised by the
// caller; the solver clears what has to start at zero on each call.
#include "../../include/cloth_gb300.h"

#include <cuda_runtime.h>

#include <string>

namespace cloth {
void set_last_error(const std::string &msg); // cloth_api.cu: message for cloth_last_error()
}

#include <cmath>
#include <cstdint>

namespace {

constexpr int kNaMaxVertices = 32768;
constexpr int kNaTile = 128;
constexpr int kNaMaxTiles = kNaMaxVertices / kNaTile;
constexpr int kNaWidth = CLOTH_ELL_REF_WIDTH;

struct NaState
{
    double rho, pq, alpha, beta, rr, bb;
    int iter, active, status;
    unsigned ticket;
    int bad_col; // set by k_na_init when an ELL column id is >= nv
    int max_iters, check_every;
    double rel_tol2, abs_tol2;
};

// byte offsets inside the scratch array (all 256-byte aligned)
constexpr size_t kVec = size_t(kNaMaxVertices) * sizeof(float4);
constexpr size_t kOffR = 0;
constexpr size_t kOffZ = kOffR + kVec;
constexpr size_t kOffP0 = kOffZ + kVec;
constexpr size_t kOffP1 = kOffP0 + kVec;
constexpr size_t kOffQ = kOffP1 + kVec;
constexpr size_t kOffMinv = kOffQ + kVec;                               // 9 floats per row
constexpr size_t kOffFixed = kOffMinv + size_t(kNaMaxVertices) * 9 * sizeof(float);
constexpr size_t kOffPart = kOffFixed + size_t(kNaMaxVertices) * sizeof(int);
constexpr size_t kOffState = kOffPart + 3 * size_t(kNaMaxTiles) * sizeof(double);
constexpr size_t kNaBytes = (kOffState + sizeof(NaState) + 255) / 256 * 256;
static_assert(kNaBytes <= (4u << 20), "scratch exceeds 4 MiB");

} // namespace

// The scratch.  In host code this name is only a stand-in for the device
// symbol; its device address comes from cudaGetSymbolAddress (na_scratch()).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

namespace {

struct NaView
{
    float4 *r, *z, *p0, *p1, *q;
    float *minv;
    int *fixed;
    double *part;
    NaState *st;
};

__host__ __device__ inline NaView na_view(unsigned char *base)
{
    NaView v;
    v.r = reinterpret_cast<float4 *>(base + kOffR);
    v.z = reinterpret_cast<float4 *>(base + kOffZ);
    v.p0 = reinterpret_cast<float4 *>(base + kOffP0);
    v.p1 = reinterpret_cast<float4 *>(base + kOffP1);
    v.q = reinterpret_cast<float4 *>(base + kOffQ);
    v.minv = reinterpret_cast<float *>(base + kOffMinv);
    v.fixed = reinterpret_cast<int *>(base + kOffFixed);
    v.part = reinterpret_cast<double *>(base + kOffPart);
    v.st = reinterpret_cast<NaState *>(base + kOffState);
    return v;
}

// ---- device helpers ------------------------------------------------------
// Blocks are the reference's tCudaMatrix3f: column-major, (i,j) at [3*j+i].
__device__ inline void blk_mul(const float *a, const float *x, float *y)
{
    for (int i = 0; i < 3; i++)
        y[i] = a[i] * x[0] + a[3 + i] * x[1] + a[6 + i] * x[2];
}

__device__ inline float warp_sum(float v)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Tile partials (FP32 within a warp, FP64 across warps) and the last tile's
// fixed-order FP64 total; returns true in the last tile (all threads).
template <int N>
__device__ bool na_reduce(const NaView &v, int ntiles, const float (&x)[N], double (&tot)[N])
{
    __shared__ double sh[N][kNaTile / 32];
    __shared__ int last;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int k = 0; k < N; k++)
    {
        const float s = warp_sum(x[k]);
        if (l == 0)
            sh[k][w] = double(s);
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        for (int k = 0; k < N; k++)
        {
            double s = sh[k][0];
            for (int j = 1; j < kNaTile / 32; j++)
                s += sh[k][j];
            v.part[k * kNaMaxTiles + blockIdx.x] = s;
        }
        __threadfence();
        last = atomicAdd(&v.st->ticket, 1u) == unsigned(ntiles - 1);
    }
    __syncthreads();
    if (!last)
        return false;
    __threadfence();
    if (threadIdx.x == 0)
    {
        for (int k = 0; k < N; k++)
        {
            double s = 0.0;
            for (int t = 0; t < ntiles; t++)
                s += __ldcg(&v.part[k * kNaMaxTiles + t]);
            tot[k] = s;
        }
        v.st->ticket = 0u;
    }
    return true;
}

__device__ inline bool na_converged(const NaState &s, double rr)
{
    return (s.rel_tol2 > 0.0 && rr <= s.rel_tol2 * s.bb) || (s.abs_tol2 > 0.0 && rr <= s.abs_tol2);
}

// ---- kernels --------------------------------------------------------------
__global__ void k_na_flags(unsigned char *base, int nv, const int *fixed_ids, int nfixed)
{
    NaView v = na_view(base);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x)
        v.fixed[i] = 0;
    __syncthreads();
    if (blockIdx.x == 0)
        for (int k = threadIdx.x; k < nfixed; k += blockDim.x)
        {
            const int id = fixed_ids[k];
            if (id >= 0 && id < nv)
                v.fixed[id] = 1;
        }
}

// Block-Jacobi inverse, r0 = b - A x0 over free rows and columns, z0, dots.
__global__ void __launch_bounds__(kNaTile) k_na_init(unsigned char *base, const int *ell,
                                                     const float *A, const float *b, float *x,
                                                     int nv, int ntiles)
{
    NaView v = na_view(base);
    const int row = blockIdx.x * kNaTile + threadIdx.x;
    float part[3] = {0.f, 0.f, 0.f};
    if (row < nv)
    {
        const bool fx = v.fixed[row] != 0;
        float acc[3] = {0.f, 0.f, 0.f}, diag[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (fx)
            x[3 * row] = x[3 * row + 1] = x[3 * row + 2] = 0.f;
        for (int s = 0; s < kNaWidth; s++)
        {
            const int c = ell[row * kNaWidth + s];
            if (c < 0)
                break;
            if (c >= nv)
            {
                // a column id outside the system: record it, touch nothing;
                // the solve then ends with CLOTH_ERR_INVALID before any SpMV
                atomicExch(&v.st->bad_col, 1);
                break;
            }
            const float *a = A + (size_t(row) * kNaWidth + s) * 9;
            if (c == row)
                for (int k = 0; k < 9; k++)
                    diag[k] = a[k];
            if (fx || v.fixed[c])
                continue;
            const float xc[3] = {x[3 * c], x[3 * c + 1], x[3 * c + 2]};
            float y[3];
            blk_mul(a, xc, y);
            for (int k = 0; k < 3; k++)
                acc[k] += y[k];
        }
        // adjugate / determinant as tCudaMatrix::inverse (CudaMatrix.h:362-398)
        const float a0 = diag[0], b0 = diag[3], c0 = diag[6], d0 = diag[1], e0 = diag[4],
                    f0 = diag[7], g0 = diag[2], h0 = diag[5], i0 = diag[8];
        float m[9];
        m[0] = e0 * i0 - f0 * h0;
        m[3] = c0 * h0 - b0 * i0;
        m[6] = b0 * f0 - c0 * e0;
        m[1] = f0 * g0 - d0 * i0;
        m[4] = a0 * i0 - c0 * g0;
        m[7] = c0 * d0 - a0 * f0;
        m[2] = d0 * h0 - e0 * g0;
        m[5] = b0 * g0 - a0 * h0;
        m[8] = a0 * e0 - b0 * d0;
        const float inv = float(1.0 / double(a0 * m[0] + b0 * m[1] + c0 * m[2]));
        for (int k = 0; k < 9; k++)
        {
            m[k] *= inv;
            v.minv[size_t(row) * 9 + k] = m[k];
        }
        float r[3] = {0.f, 0.f, 0.f};
        if (!fx)
            for (int k = 0; k < 3; k++)
                r[k] = b[3 * row + k] - acc[k];
        float z[3];
        blk_mul(m, r, z);
        v.r[row] = make_float4(r[0], r[1], r[2], 0.f);
        v.z[row] = make_float4(z[0], z[1], z[2], 0.f);
        v.p0[row] = make_float4(0.f, 0.f, 0.f, 0.f);
        v.p1[row] = make_float4(0.f, 0.f, 0.f, 0.f);
        const float bb[3] = {fx ? 0.f : b[3 * row], fx ? 0.f : b[3 * row + 1],
                             fx ? 0.f : b[3 * row + 2]};
        part[0] = r[0] * z[0] + r[1] * z[1] + r[2] * z[2];
        part[1] = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        part[2] = bb[0] * bb[0] + bb[1] * bb[1] + bb[2] * bb[2];
    }
    double tot[3];
    if (na_reduce<3>(v, ntiles, part, tot) && threadIdx.x == 0)
    {
        NaState &s = *v.st;
        s.rho = tot[0];
        s.rr = tot[1];
        s.bb = tot[2];
        s.beta = 0.0;
        s.iter = 0;
        s.status = CLOTH_OK;
        s.active = (s.max_iters > 0 && !na_converged(s, tot[1])) ? 1 : 0;
        if (!isfinite(tot[0]) || !isfinite(tot[1]) || !isfinite(tot[2]))
        {
            s.status = CLOTH_ERR_NAN;
            s.active = 0;
        }
        if (atomicAdd(&s.bad_col, 0) != 0)
        {
            s.status = CLOTH_ERR_INVALID;
            s.active = 0;
        }
    }
}

// p = z + beta p_old; q = A p over free rows and columns; p.q.
__global__ void __launch_bounds__(kNaTile) k_na_spmv(unsigned char *base, const int *ell,
                                                     const float *A, int nv, int ntiles)
{
    NaView v = na_view(base);
    NaState *st = v.st;
    if (!st->active)
        return;
    const int it = st->iter;
    const float beta = float(st->beta);
    const float4 *pold = (it & 1) ? v.p1 : v.p0;
    float4 *pnew = (it & 1) ? v.p0 : v.p1;
    const int row = blockIdx.x * kNaTile + threadIdx.x;
    float part[1] = {0.f};
    if (row < nv)
    {
        const float4 zr = v.z[row], pr = pold[row];
        const float pv[3] = {zr.x + beta * pr.x, zr.y + beta * pr.y, zr.z + beta * pr.z};
        pnew[row] = make_float4(pv[0], pv[1], pv[2], 0.f);
        float q[3] = {0.f, 0.f, 0.f};
        if (!v.fixed[row])
            for (int s = 0; s < kNaWidth; s++)
            {
                const int c = ell[row * kNaWidth + s];
                if (c < 0 || c >= nv)
                    break;
                if (v.fixed[c])
                    continue;
                const float4 zc = v.z[c], pc = pold[c];
                const float pcv[3] = {zc.x + beta * pc.x, zc.y + beta * pc.y, zc.z + beta * pc.z};
                float y[3];
                blk_mul(A + (size_t(row) * kNaWidth + s) * 9, pcv, y);
                for (int k = 0; k < 3; k++)
                    q[k] += y[k];
            }
        v.q[row] = make_float4(q[0], q[1], q[2], 0.f);
        part[0] = pv[0] * q[0] + pv[1] * q[1] + pv[2] * q[2];
    }
    double tot[1];
    if (na_reduce<1>(v, ntiles, part, tot) && threadIdx.x == 0)
    {
        st->pq = tot[0];
        if (!isfinite(tot[0]))
        {
            st->status = CLOTH_ERR_NAN;
            st->active = 0;
        }
        else if (tot[0] == 0.0)
        {
            st->status = CLOTH_ERR_BREAKDOWN;
            st->active = 0;
        }
        else
            st->alpha = st->rho / tot[0];
    }
}

// x += alpha p; r -= alpha q; z = M^-1 r; r.z and r.r; convergence test.
__global__ void __launch_bounds__(kNaTile) k_na_update(unsigned char *base, float *x, int nv,
                                                       int ntiles)
{
    NaView v = na_view(base);
    NaState *st = v.st;
    if (!st->active)
        return;
    const int it = st->iter;
    const float alpha = float(st->alpha);
    const float4 *pnew = (it & 1) ? v.p0 : v.p1;
    const int row = blockIdx.x * kNaTile + threadIdx.x;
    float part[2] = {0.f, 0.f};
    if (row < nv)
    {
        const float4 p = pnew[row], q = v.q[row];
        float4 r = v.r[row];
        x[3 * row] += alpha * p.x;
        x[3 * row + 1] += alpha * p.y;
        x[3 * row + 2] += alpha * p.z;
        r.x -= alpha * q.x;
        r.y -= alpha * q.y;
        r.z -= alpha * q.z;
        const float rv[3] = {r.x, r.y, r.z};
        float z[3];
        blk_mul(v.minv + size_t(row) * 9, rv, z);
        v.r[row] = r;
        v.z[row] = make_float4(z[0], z[1], z[2], 0.f);
        part[0] = rv[0] * z[0] + rv[1] * z[1] + rv[2] * z[2];
        part[1] = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
    }
    double tot[2];
    if (na_reduce<2>(v, ntiles, part, tot) && threadIdx.x == 0)
    {
        NaState &s = *st;
        s.beta = (s.rho == 0.0) ? 0.0 : tot[0] / s.rho;
        s.rho = tot[0];
        s.rr = tot[1];
        s.iter = it + 1;
        const int n = s.iter;
        if (!isfinite(tot[0]) || !isfinite(tot[1]))
        {
            s.status = CLOTH_ERR_NAN;
            s.active = 0;
        }
        else if ((((n - 1) % s.check_every) == 0 || n >= s.max_iters) && na_converged(s, tot[1]))
            s.active = 0;
        else if (n >= s.max_iters)
        {
            s.status = CLOTH_ERR_MAXITER;
            s.active = 0;
        }
    }
}

int na_fail(int code, const std::string &m)
{
    cloth::set_last_error(m);
    return code;
}

// Device address of the scratch on the current device, looked up on every
// call with that device current (a lookup costs about a microsecond, and a
// cached address would go stale after cudaDeviceReset reloads the module).
int na_scratch(unsigned char **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
    {
        cudaGetLastError();
        return na_fail(CLOTH_ERR_CUDA, std::string("cloth_pcg_solve_ell32_noalloc: "
                                                   "cudaGetSymbolAddress: ") +
                                           cudaGetErrorString(e));
    }
    *out = static_cast<unsigned char *>(p);
    return CLOTH_OK;
}

} // namespace

extern "C" int cloth_pcg_solve_ell32_noalloc(int nv, const int *ell_dev, const float *A_dev,
                                             const float *b_dev, float *x_dev,
                                             const int *fixed_dev, int nfixed,
                                             const cloth_solve_params *params,
                                             cloth_solve_stats *stats, void *stream)
{
    if (nv <= 0 || !ell_dev || !A_dev || !b_dev || !x_dev || nfixed < 0 ||
        (nfixed > 0 && !fixed_dev))
        return na_fail(CLOTH_ERR_INVALID, "cloth_pcg_solve_ell32_noalloc: bad argument");
    if (nv > kNaMaxVertices)
        return na_fail(CLOTH_ERR_INVALID,
                       "cloth_pcg_solve_ell32_noalloc: " + std::to_string(nv) +
                           " vertices exceed the static scratch limit of " +
                           std::to_string(kNaMaxVertices));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The call waits on the host for the solver state every few iterations,
    // which a stream under capture cannot do: refuse before touching it.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess)
    {
        cudaGetLastError();
        return na_fail(CLOTH_ERR_CUDA, "cloth_pcg_solve_ell32_noalloc: cudaStreamIsCapturing failed");
    }
    if (cap != cudaStreamCaptureStatusNone)
        return na_fail(CLOTH_ERR_STATE,
                       "cloth_pcg_solve_ell32_noalloc: the stream is being captured; this call "
                       "synchronises with the host and cannot be captured");
    unsigned char *base = nullptr;
    int rc = na_scratch(&base);
    if (rc != CLOTH_OK)
        return rc;
    NaState init{};
    const int max_iters = params ? params->max_iters : 1000;
    const double rel = params ? params->rel_tol : 1e-6, abs = params ? params->abs_tol : 0.0;
    init.max_iters = max_iters < 0 ? 0 : max_iters;
    init.check_every = (params && params->check_every > 0) ? params->check_every : 1;
    init.rel_tol2 = rel > 0 ? rel * rel : 0.0;
    init.abs_tol2 = abs > 0 ? abs * abs : 0.0;
    const NaView v = na_view(base);
    const int ntiles = (nv + kNaTile - 1) / kNaTile;
#define NA_CK(call)                                                                  \
    do                                                                               \
    {                                                                                \
        const cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                       \
            return na_fail(CLOTH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
    // the solver state (including the reduction ticket) starts from zero
    NA_CK(cudaMemcpyAsync(v.st, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    k_na_flags<<<1, 256, 0, s>>>(base, nv, fixed_dev, nfixed);
    k_na_init<<<ntiles, kNaTile, 0, s>>>(base, ell_dev, A_dev, b_dev, x_dev, nv, ntiles);
    NA_CK(cudaGetLastError());
    NaState h{};
    const int chunk = 8;
    // the device stops at max_iters; the host bound (in 64-bit) only guards
    // against a state that never reports inactive
    const long long limit = static_cast<long long>(init.max_iters) + 2 * chunk;
    for (long long done = 0;; done += chunk)
    {
        NA_CK(cudaMemcpyAsync(&h, v.st, sizeof(h), cudaMemcpyDeviceToHost, s));
        NA_CK(cudaStreamSynchronize(s));
        if (!h.active || h.bad_col || done > limit)
            break;
        for (int k = 0; k < chunk; k++)
        {
            k_na_spmv<<<ntiles, kNaTile, 0, s>>>(base, ell_dev, A_dev, nv, ntiles);
            k_na_update<<<ntiles, kNaTile, 0, s>>>(base, x_dev, nv, ntiles);
        }
        NA_CK(cudaGetLastError());
    }
#undef NA_CK
    if (h.active && h.status == CLOTH_OK)
        h.status = CLOTH_ERR_MAXITER;
    if (h.bad_col)
        h.status = CLOTH_ERR_INVALID;
    if (stats)
    {
        stats->iters = h.iter;
        stats->status = h.status;
        stats->res_norm = std::sqrt(h.rr > 0 ? h.rr : 0.0);
        stats->rhs_norm = std::sqrt(h.bb > 0 ? h.bb : 0.0);
        stats->rel_residual = stats->rhs_norm > 0 ? stats->res_norm / stats->rhs_norm : stats->res_norm;
        stats->solver = CLOTH_SOLVER_GRAPH_LOOP;
    }
    // no stats object outlives the call, so the return value carries the
    // solve's own outcome: CLOTH_OK only when it reached the tolerance
    if (h.status == CLOTH_ERR_INVALID)
        return na_fail(CLOTH_ERR_INVALID,
                       "cloth_pcg_solve_ell32_noalloc: an ELL column id is >= nv");
    return h.status;
}
