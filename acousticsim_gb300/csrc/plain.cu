// The "plain" implicit cloth step: the reference GPU path's structure,
// re-expressed, as the comparison baseline for the batched and served solvers.
//
// Per step (cBaraffClothGpu::UpdatePos, src/sim/cloth/BaraffClothGpu.cpp:152-265):
//   host: snap pins in x / x_pre (double), upload float copies
//   memset K, f; one thread per triangle accumulates force and the nine
//   Hessian blocks with float atomics, finding each block's ELL slot by a
//   32-wide search (BaraffClothGpu.cu:111-194); bending add (:445-483); RHS
//   (:301-344); system matrix (:240-281); every wrapper synchronises
//   PCG (PCGSolver.cu:332-481): block-Jacobi inverse, r0/d0 with a float atomic
//   dot, then per iteration memset + three kernels with float atomic dots, the
//   residual downloaded and its norm computed on the host every 10th iteration
//   host: download dx, x_pre = x, x += dx in double, upload x and x_pre
//
// Layouts are the reference's: ELL rows of 32 vertex ids (-1 padded) and 3x3
// blocks of 9 floats, column-major, row-major over [row][slot].
#include "../../include/cloth_gb300.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace cloth {
void set_last_error(const std::string &msg);
}

namespace {

constexpr int PW = CLOTH_ELL_REF_WIDTH;
constexpr int PB = 128; // block size of the reference's CUDA_at launches

__device__ inline void atomic_add3(float *dst, const float *v)
{
    for (int k = 0; k < 3; k++)
        atomicAdd(dst + k, v[k]);
}

__device__ inline float norm3(const float *a)
{
    float s = 0.f;
    for (int k = 0; k < 3; k++)
        s += a[k] * a[k];
    return sqrtf(s);
}

// one stretch component: UpdateComponent (BaraffClothGpu.cu:88-109)
__device__ void plain_component(float Ku, float Kv, const float *cu, const float *cv,
                                const float *x0, const float *x1, const float *x2, float S,
                                int fix_fv, float *fint /*3 cols x3*/, float *H /*9 blocks x9*/)
{
    float Fu[3], Fv[3];
    for (int k = 0; k < 3; k++)
    {
        Fu[k] = cu[0] * x0[k] + cu[1] * x1[k] + cu[2] * x2[k];
        Fv[k] = cv[0] * x0[k] + cv[1] * x1[k] + cv[2] * x2[k];
    }
    const float nu = norm3(Fu), nv = norm3(Fv);
    const float Cu = nu - 1.f, Cv = nv - 1.f;
    float un[3], vn[3];
    for (int k = 0; k < 3; k++)
    {
        un[k] = Fu[k] / nu;
        vn[k] = Fv[k] / nv;
    }
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++)
            fint[3 * i + k] += (-S * Ku * Cu * un[k]) * cu[i] + (-S * Kv * Cv * vn[k]) * cv[i];
    const float nvh = fix_fv ? nv : nu;
    float Du[9], Dv[9];
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++)
        {
            Du[3 * c + r] = float(1.0 / nu) * un[r] * un[c] + ((r == c && nu > 1.f) ? float(1.0 - 1.0 / nu) : 0.f);
            Dv[3 * c + r] = float(1.0 / nvh) * vn[r] * vn[c] + ((r == c && nvh > 1.f) ? float(1.0 - 1.0 / nvh) : 0.f);
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 9; k++)
                H[9 * (3 * i + j) + k] += -S * (Ku * cu[i] * cu[j] * Du[k] + Kv * cv[i] * cv[j] * Dv[k]);
}

__device__ inline int slot_search(const int *row, int id)
{
    int res = -1;
    for (int i = 0; i < PW; i++)
        if (row[i] == id)
            res = i;
    return res;
}

__global__ void kp_stretch(int nt, const int4 *tri, const float4 *coef, const float *x,
                           float kw, float kwe, float kb, int fix_fv, const int *ell, float *f,
                           float *K)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt)
        return;
    const int4 tv = tri[t];
    const float S = __int_as_float(tv.w);
    const float4 c0 = coef[3 * t], c1 = coef[3 * t + 1], c2 = coef[3 * t + 2];
    const float cuw[3] = {c0.x, c0.y, c0.z}, cvw[3] = {c0.w, c1.x, c1.y};
    const float cud[3] = {c1.z, c1.w, c2.x}, cvd[3] = {c2.y, c2.z, c2.w};
    const int v[3] = {tv.x, tv.y, tv.z};
    const float *x0 = x + 3 * v[0], *x1 = x + 3 * v[1], *x2 = x + 3 * v[2];
    float fint[9] = {0}, H[81] = {0};
    plain_component(kw, kwe, cuw, cvw, x0, x1, x2, S, fix_fv, fint, H);
    plain_component(kb, kb, cud, cvd, x0, x1, x2, S, fix_fv, fint, H);
    for (int i = 0; i < 3; i++)
        atomic_add3(f + 3 * v[i], fint + 3 * i);
    for (int i = 0; i < 3; i++)
    {
        int row[PW];
        for (int s = 0; s < PW; s++)
            row[s] = ell[v[i] * PW + s];
        for (int j = 0; j < 3; j++)
        {
            const int s = slot_search(row, v[j]);
            float *dst = K + (size_t(v[i]) * PW + s) * 9;
            for (int k = 0; k < 9; k++)
                atomicAdd(dst + k, H[9 * (3 * i + j) + k]);
        }
    }
}

__global__ void kp_bending(int nv, const int *ell, const float *Kb, const float *x, float *f, float *K)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    for (int s = 0; s < PW; s++)
        for (int k = 0; k < 9; k++)
            K[(size_t(v) * PW + s) * 9 + k] -= Kb[(size_t(v) * PW + s) * 9 + k];
    float fi[3] = {0, 0, 0};
    for (int s = 0; s < PW; s++)
    {
        const int c = ell[v * PW + s];
        if (c < 0)
            break;
        const float *kb = Kb + (size_t(v) * PW + s) * 9;
        for (int r = 0; r < 3; r++)
            fi[r] += -(kb[r] * x[3 * c] + kb[3 + r] * x[3 * c + 1] + kb[6 + r] * x[3 * c + 2]);
    }
    for (int k = 0; k < 3; k++)
        f[3 * v + k] += fi[k];
}

__global__ void kp_rhs(int nv, float dt, const float *grav, const float *f, const int *ell,
                       const float *mass, const float *x, const float *xp, float *b)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    const float g[3] = {0.f, grav[v], 0.f};
    float out[3];
    for (int k = 0; k < 3; k++)
        out[k] = dt * dt * (g[k] + f[3 * v + k]);
    float sum[3] = {0, 0, 0};
    for (int s = 0; s < PW; s++)
        if (ell[v * PW + s] == v)
            for (int k = 0; k < 3; k++)
                sum[k] = (x[3 * v + k] - xp[3 * v + k]) * mass[v];
    for (int k = 0; k < 3; k++)
        b[3 * v + k] = out[k] + sum[k];
}

__global__ void kp_matrix(int nv, float dt, float ra, float rb, const int *ell, const float *K,
                          const float *mass, float *A)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    for (int s = 0; s < PW; s++)
    {
        const int c = ell[v * PW + s];
        if (c == -1)
            break;
        for (int k = 0; k < 9; k++)
            A[(size_t(v) * PW + s) * 9 + k] = (dt * rb - dt * dt) * K[(size_t(v) * PW + s) * 9 + k];
        if (c == v)
            for (int k = 0; k < 3; k++)
                A[(size_t(v) * PW + s) * 9 + 4 * k] += mass[v] * (1 + dt * ra);
    }
}

__device__ inline void mat3_mul(const float *a, const float *x, float *y)
{
    for (int r = 0; r < 3; r++)
        y[r] = a[r] * x[0] + a[3 + r] * x[1] + a[6 + r] * x[2];
}

__global__ void kp_precond(int nv, const int *ell, const float *A, float *Minv)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    for (int s = 0; s < PW; s++)
        if (ell[v * PW + s] == v)
        {
            const float *m = A + (size_t(v) * PW + s) * 9;
            const float a = m[0], bq = m[3], c = m[6], d = m[1], e = m[4], f = m[7],
                        g = m[2], h = m[5], i = m[8];
            float *o = Minv + size_t(v) * 9;
            o[0] = e * i - f * h;
            o[3] = c * h - bq * i;
            o[6] = bq * f - c * e;
            o[1] = f * g - d * i;
            o[4] = a * i - c * g;
            o[7] = c * d - a * f;
            o[2] = d * h - e * g;
            o[5] = bq * g - a * h;
            o[8] = a * e - bq * d;
            const float pre = 1.0 / (a * (e * i - f * h) - bq * (d * i - f * g) + c * (d * h - e * g));
            for (int k = 0; k < 9; k++)
                o[k] *= pre;
            return;
        }
}

__device__ inline bool is_fixed(int v, int nfix, const int *fix)
{
    for (int i = 0; i < nfix; i++)
        if (fix[i] == v)
            return true;
    return false;
}

__global__ void kp_r0(int nv, const float *x0, const float *b, float *r, float *d, float *rMr,
                      const float *Minv, const int *ell, const float *A, int nfix, const int *fix)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    if (is_fixed(v, nfix, fix))
    {
        for (int k = 0; k < 3; k++)
            r[3 * v + k] = d[3 * v + k] = 0.f;
        return;
    }
    float acc[3] = {0, 0, 0};
    for (int s = 0; s < PW; s++)
    {
        const int c = ell[v * PW + s];
        if (c == -1)
            break;
        // the reference's loop over the fixed list here only "continue"s that
        // inner loop, so fixed columns are not skipped (PCGSolver.cu:151-157)
        float y[3];
        mat3_mul(A + (size_t(v) * PW + s) * 9, x0 + 3 * c, y);
        for (int k = 0; k < 3; k++)
            acc[k] += y[k];
    }
    float rr[3], dd[3];
    for (int k = 0; k < 3; k++)
        rr[k] = b[3 * v + k] - acc[k];
    mat3_mul(Minv + size_t(v) * 9, rr, dd);
    for (int k = 0; k < 3; k++)
    {
        r[3 * v + k] = rr[k];
        d[3 * v + k] = dd[k];
    }
    atomicAdd(rMr, rr[0] * dd[0] + rr[1] * dd[1] + rr[2] * dd[2]);
}

__global__ void kp_dAd(int nv, const float *d, const int *ell, const float *A, float *z,
                       float *dAd, int nfix, const int *fix)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    if (is_fixed(v, nfix, fix))
    {
        for (int k = 0; k < 3; k++)
            z[3 * v + k] = 0.f;
        return;
    }
    float acc[3] = {0, 0, 0};
    for (int s = 0; s < PW; s++)
    {
        const int c = ell[v * PW + s];
        if (c == -1)
            break;
        if (is_fixed(c, nfix, fix))
            continue;
        float y[3];
        mat3_mul(A + (size_t(v) * PW + s) * 9, d + 3 * c, y);
        for (int k = 0; k < 3; k++)
            acc[k] += y[k];
    }
    for (int k = 0; k < 3; k++)
        z[3 * v + k] = acc[k];
    atomicAdd(dAd, d[3 * v] * acc[0] + d[3 * v + 1] * acc[1] + d[3 * v + 2] * acc[2]);
}

__global__ void kp_rnext(int nv, const float *rMr, const float *dAd, const float *z, float *r,
                         const float *Minv, float *rMr_next, const float *d, float *x)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    float alpha = rMr[0] / dAd[0];
    if (dAd[0] == 0.0f)
        alpha = 0.f;
    float rv[3], mr[3];
    for (int k = 0; k < 3; k++)
        rv[k] = r[3 * v + k] -= alpha * z[3 * v + k];
    mat3_mul(Minv + size_t(v) * 9, rv, mr);
    atomicAdd(rMr_next, rv[0] * mr[0] + rv[1] * mr[1] + rv[2] * mr[2]);
    for (int k = 0; k < 3; k++)
        x[3 * v + k] += alpha * d[3 * v + k];
}

__global__ void kp_direction(int nv, const float *rMr_next, const float *rMr, const float *Minv,
                             const float *r, float *d)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    float beta = rMr_next[0] / rMr[0];
    if (rMr[0] == 0.0f)
        beta = 0.f;
    float mr[3];
    mat3_mul(Minv + size_t(v) * 9, r + 3 * v, mr);
    for (int k = 0; k < 3; k++)
        d[3 * v + k] = mr[k] + beta * d[3 * v + k];
}

int pfail(int code, const std::string &m)
{
    cloth::set_last_error(m);
    return code;
}

} // namespace

namespace cloth {

// Device and host state of the plain path for one cloth (built on first use).
struct PlainState
{
    int nv = 0, nt = 0;
    std::vector<double> x, xp;      // host positions (the reference keeps them on the host)
    std::vector<float> xf, dxf;
    std::vector<int> pins;
    std::vector<float> pin_tgt;
    char *mem = nullptr;
    int *ell = nullptr, *fix = nullptr;
    float *Kb = nullptr, *K = nullptr, *A = nullptr, *f = nullptr, *b = nullptr, *x32 = nullptr,
          *xp32 = nullptr, *dx = nullptr, *r = nullptr, *d = nullptr, *z = nullptr,
          *Minv = nullptr, *rMr = nullptr, *dAd = nullptr, *mass = nullptr, *grav = nullptr;
    const int4 *tri = nullptr;
    const float4 *coef = nullptr;
    size_t bytes = 0;
    ~PlainState()
    {
        if (mem)
            cudaFree(mem);
    }
};

void plain_free(PlainState *p) { delete p; }

struct PlainInit
{
    int nv, nt;
    const int *ell_host;          // nv*32
    const float *kb_scalar_host;  // nv*32 bending scalars (+K_b per block)
    const float *mass_host, *grav_host;
    const int4 *tri_dev;
    const float4 *coef_dev;
};

int plain_create(const PlainInit &in, PlainState **out)
{
    auto p = new PlainState();
    p->nv = in.nv;
    p->nt = in.nt;
    const size_t n = size_t(in.nv);
    const size_t blk = n * PW * 9 * sizeof(float);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += (bytes + 255) / 256 * 256;
        return o;
    };
    const size_t o_ell = take(n * PW * sizeof(int)), o_fix = take((n + 1) * sizeof(int)),
                 o_Kb = take(blk), o_K = take(blk), o_A = take(blk),
                 o_f = take(n * 3 * 4), o_b = take(n * 3 * 4), o_x = take(n * 3 * 4),
                 o_xp = take(n * 3 * 4), o_dx = take(n * 3 * 4), o_r = take(n * 3 * 4),
                 o_d = take(n * 3 * 4), o_z = take(n * 3 * 4), o_M = take(n * 9 * 4),
                 o_rMr = take(100001 * 4), o_dAd = take(4), o_mass = take(n * 4),
                 o_grav = take(n * 4);
    if (cudaMalloc(&p->mem, off) != cudaSuccess)
    {
        cudaGetLastError();
        delete p;
        return pfail(CLOTH_ERR_OOM, "plain path: device allocation failed");
    }
    p->bytes = off;
    char *m = p->mem;
    p->ell = reinterpret_cast<int *>(m + o_ell);
    p->fix = reinterpret_cast<int *>(m + o_fix);
    p->Kb = reinterpret_cast<float *>(m + o_Kb);
    p->K = reinterpret_cast<float *>(m + o_K);
    p->A = reinterpret_cast<float *>(m + o_A);
    p->f = reinterpret_cast<float *>(m + o_f);
    p->b = reinterpret_cast<float *>(m + o_b);
    p->x32 = reinterpret_cast<float *>(m + o_x);
    p->xp32 = reinterpret_cast<float *>(m + o_xp);
    p->dx = reinterpret_cast<float *>(m + o_dx);
    p->r = reinterpret_cast<float *>(m + o_r);
    p->d = reinterpret_cast<float *>(m + o_d);
    p->z = reinterpret_cast<float *>(m + o_z);
    p->Minv = reinterpret_cast<float *>(m + o_M);
    p->rMr = reinterpret_cast<float *>(m + o_rMr);
    p->dAd = reinterpret_cast<float *>(m + o_dAd);
    p->mass = reinterpret_cast<float *>(m + o_mass);
    p->grav = reinterpret_cast<float *>(m + o_grav);
    p->tri = in.tri_dev;
    p->coef = in.coef_dev;
    // bending matrix as the reference stores it: value * I3 in 9-float blocks
    std::vector<float> kb(n * PW * 9, 0.f);
    for (size_t i = 0; i < n * PW; i++)
        for (int k = 0; k < 3; k++)
            kb[i * 9 + 4 * k] = in.kb_scalar_host[i];
    bool ok = cudaMemcpy(p->ell, in.ell_host, n * PW * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(p->Kb, kb.data(), kb.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(p->mass, in.mass_host, n * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(p->grav, in.grav_host, n * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemset(p->dx, 0, n * 3 * 4) == cudaSuccess;
    if (!ok)
    {
        cudaGetLastError();
        delete p;
        return pfail(CLOTH_ERR_CUDA, "plain path: upload failed");
    }
    *out = p;
    return CLOTH_OK;
}

size_t plain_bytes(const PlainState *p) { return p ? p->bytes : 0; }

// One plain step on the host state x, xp (double, updated in place).
int plain_step(PlainState *p, double *x, double *xp, const int *pins, const float *pin_tgt,
               int npins, float dt, float kw, float kwe, float kb, int fix_fv, float ra,
               float rb, const cloth_solve_params *prm, cloth_solve_stats *stats)
{
    const int nv = p->nv, nt = p->nt;
    const size_t n3 = size_t(nv) * 3;
#define PCK(call)                                                                   \
    do                                                                              \
    {                                                                               \
        const cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess)                                                      \
            return pfail(CLOTH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
    // UpdateConstraintVertexPos + UpdateConstraintVid: snap on the host, upload
    for (int k = 0; k < npins; k++)
        for (int c = 0; c < 3; c++)
            x[3 * pins[k] + c] = xp[3 * pins[k] + c] = double(pin_tgt[4 * k + c]);
    p->xf.resize(n3);
    for (size_t i = 0; i < n3; i++)
        p->xf[i] = float(x[i]);
    PCK(cudaMemcpy(p->x32, p->xf.data(), n3 * 4, cudaMemcpyHostToDevice));
    for (size_t i = 0; i < n3; i++)
        p->xf[i] = float(xp[i]);
    PCK(cudaMemcpy(p->xp32, p->xf.data(), n3 * 4, cudaMemcpyHostToDevice));
    if (npins > 0)
        PCK(cudaMemcpy(p->fix, pins, npins * sizeof(int), cudaMemcpyHostToDevice));
    const int gv = (nv + PB - 1) / PB, gt = (nt + PB - 1) / PB;
    const size_t blk = size_t(nv) * PW * 9 * 4;
    // UpdateStretchStiffnessMatrixAndFint
    PCK(cudaMemset(p->K, 0, blk));
    PCK(cudaMemset(p->f, 0, n3 * 4));
    kp_stretch<<<gt, PB>>>(nt, p->tri, p->coef, p->x32, kw, kwe, kb, fix_fv, p->ell, p->f, p->K);
    PCK(cudaDeviceSynchronize());
    // AddBendingHessianAndIntForce
    kp_bending<<<gv, PB>>>(nv, p->ell, p->Kb, p->x32, p->f, p->K);
    PCK(cudaDeviceSynchronize());
    // AssembleSystemRHS
    PCK(cudaMemset(p->b, 0, n3 * 4));
    kp_rhs<<<gv, PB>>>(nv, dt, p->grav, p->f, p->ell, p->mass, p->x32, p->xp32, p->b);
    PCK(cudaDeviceSynchronize());
    // AssembleSystemMatrix
    PCK(cudaMemset(p->A, 0, blk));
    kp_matrix<<<gv, PB>>>(nv, dt, ra, rb, p->ell, p->K, p->mass, p->A);
    PCK(cudaDeviceSynchronize());
    // PCGSolver::Solve
    const int max_iters = prm ? prm->max_iters : 100;
    const int check_every = (prm && prm->check_every > 0) ? prm->check_every : 10;
    const double rel = prm ? prm->rel_tol : 0.0, abs = prm ? prm->abs_tol : 1e-10;
    kp_precond<<<gv, PB>>>(nv, p->ell, p->A, p->Minv);
    PCK(cudaMemsetAsync(p->dAd, 0, 4));
    PCK(cudaMemsetAsync(p->r, 0, n3 * 4));
    PCK(cudaMemsetAsync(p->d, 0, n3 * 4));
    PCK(cudaMemsetAsync(p->z, 0, n3 * 4));
    PCK(cudaMemsetAsync(p->rMr, 0, size_t(max_iters + 1) * 4));
    kp_r0<<<gv, PB>>>(nv, p->dx, p->b, p->r, p->d, p->rMr, p->Minv, p->ell, p->A, npins, p->fix);
    double bnorm = 1.0;
    if (rel > 0)
    {
        std::vector<float> bh(n3);
        PCK(cudaMemcpy(bh.data(), p->b, n3 * 4, cudaMemcpyDeviceToHost));
        double s = 0;
        for (int v = 0; v < nv; v++)
        {
            bool fx = false;
            for (int k = 0; k < npins; k++)
                fx |= pins[k] == v;
            if (!fx)
                for (int c = 0; c < 3; c++)
                    s += double(bh[3 * v + c]) * bh[3 * v + c];
        }
        bnorm = std::sqrt(s);
    }
    std::vector<float> rh(n3);
    int it = 0, status = CLOTH_ERR_MAXITER;
    double res = 0;
    for (int cur = 0; cur < max_iters; cur++)
    {
        PCK(cudaMemsetAsync(p->dAd, 0, 4));
        kp_dAd<<<gv, PB>>>(nv, p->d, p->ell, p->A, p->z, p->dAd, npins, p->fix);
        kp_rnext<<<gv, PB>>>(nv, p->rMr + cur, p->dAd, p->z, p->r, p->Minv, p->rMr + cur + 1,
                             p->d, p->dx);
        kp_direction<<<gv, PB>>>(nv, p->rMr + cur + 1, p->rMr + cur, p->Minv, p->r, p->d);
        it = cur + 1;
        if (cur % check_every == 0 || cur == max_iters - 1)
        {
            PCK(cudaMemcpy(rh.data(), p->r, n3 * 4, cudaMemcpyDeviceToHost));
            float s = 0.f;
            for (int v = 0; v < nv; v++)
            {
                const float nrm = std::sqrt(rh[3 * v] * rh[3 * v] + rh[3 * v + 1] * rh[3 * v + 1] +
                                            rh[3 * v + 2] * rh[3 * v + 2]);
                s += nrm * nrm;
            }
            res = std::sqrt(double(s));
            if ((abs > 0 && res < abs) || (rel > 0 && res <= rel * bnorm))
            {
                status = CLOTH_OK;
                break;
            }
            if (!std::isfinite(res))
            {
                status = CLOTH_ERR_NAN;
                break;
            }
        }
    }
    PCK(cudaGetLastError());
    // post-solve: download dx, update on the host in double
    p->dxf.resize(n3);
    PCK(cudaMemcpy(p->dxf.data(), p->dx, n3 * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n3; i++)
    {
        xp[i] = x[i];
        x[i] += double(p->dxf[i]);
    }
    for (size_t i = 0; i < n3; i++)
        p->xf[i] = float(x[i]);
    PCK(cudaMemcpy(p->x32, p->xf.data(), n3 * 4, cudaMemcpyHostToDevice));
    for (size_t i = 0; i < n3; i++)
        p->xf[i] = float(xp[i]);
    PCK(cudaMemcpy(p->xp32, p->xf.data(), n3 * 4, cudaMemcpyHostToDevice));
#undef PCK
    if (stats)
    {
        stats->iters = it;
        stats->status = status;
        stats->res_norm = res;
        stats->rhs_norm = bnorm;
        stats->rel_residual = rel > 0 && bnorm > 0 ? res / bnorm : res;
        stats->solver = -1;
    }
    return CLOTH_OK;
}

} // namespace cloth
