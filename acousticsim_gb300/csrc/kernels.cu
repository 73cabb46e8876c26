// Kernels of the implicit cloth step (sm_103a).
//
//   k_pins         snap pinned vertices to their targets      (UpdateConstraintVertexPos)
//   k_tri          triangle-parallel stretch/shear force and 3x3 Hessian blocks,
//                  written without atomics through the precomputed
//                  triangle -> record map                     (UpdateStretch_K_fint)
//   k_row          row-parallel reduction of the records in fixed order, bending
//                  (K -= K_b, f -= K_b x), A = (h b - h^2) K + (1 + h a) M, RHS,
//                  pin projection, block-Jacobi inverse and the PCG start
//                  r = b - A dx0, z = M^-1 r                  (AddBendingHessianAndIntForce,
//                                                              AssembleSystemRHS/Matrix,
//                                                              BlockJacobPreconditioner,
//                                                              Calc_r0_d0_r0Minvr0)
//   k_spmv         p = z + beta p (recomputed at the gathered columns), q = A p,
//                  p.q as exact fixed-point sums              (Calc_dTAd_zi, UpdateDirection)
//   k_update       dx += alpha p, r -= alpha q, z = M^-1 r, r.z and r.r as exact
//                  fixed-point sums                           (Calc_rnext_rnextMinvrnext_xnext)
//   k_reduce_*     per-instance totals, alpha / beta, the convergence test
//   k_advance      x_pre = x, x += dx in FP64                 (BaraffClothGpu.cpp:246-258)
//
// Reference kernels: src/sim/cloth/BaraffClothGpu.cu, src/sim/cloth/gpu_solvers/PCGSolver.cu.
#include "device.cuh"

#include <type_traits>

namespace cloth {

namespace {

__device__ __forceinline__ float3 operator+(float3 a, float3 b)
{
    return make_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
__device__ __forceinline__ float3 operator-(float3 a, float3 b)
{
    return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float3 operator*(float s, float3 a)
{
    return make_float3(s * a.x, s * a.y, s * a.z);
}
__device__ __forceinline__ float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 f4(float3 v, float w = 0.f)
{
    return make_float4(v.x, v.y, v.z, w);
}
// Row-level products stay in FP32; sums from 32 rows upward are FP64 (GB300's
// FP64 pipe is narrow, so FP64 work is kept per warp, not per row).
__device__ __forceinline__ float fdot(float3 a, float3 b)
{
    return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x));
}
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// sum of squares in component order, as tCudaMatrix::norm (CudaMatrix.h:314-320)
__device__ __forceinline__ float norm3(float3 a)
{
    float s = a.x * a.x;
    s = s + a.y * a.y;
    s = s + a.z * a.z;
    return sqrtf(s);
}
// symmetric 3x3 (00 01 02 11 12 22) times vector
// (explicit fused multiply-adds: device code is built without implicit
// contraction, so every kernel variant rounds the same way)
__device__ __forceinline__ float3 symv(const float *s, float3 v)
{
    return make_float3(fmaf(s[2], v.z, fmaf(s[1], v.y, s[0] * v.x)),
                       fmaf(s[4], v.z, fmaf(s[3], v.y, s[1] * v.x)),
                       fmaf(s[5], v.z, fmaf(s[4], v.y, s[2] * v.x)));
}
// p = z + beta p_old with one rounding per component (the persistent
// kernels' form, so every PCG driver forms the same p)
__device__ __forceinline__ float3 pform(float3 z, float beta, float3 po)
{
    return make_float3(fmaf(beta, po.x, z.x), fmaf(beta, po.y, z.y), fmaf(beta, po.z, z.z));
}
// w x p: the skew part of a block of the dihedral-bending model (an upper
// block is S p + w x p, its transposed lower block S p - w x p)
__device__ __forceinline__ float3 skewv(float4 w, float3 p)
{
    return make_float3(fmaf(w.y, p.z, -(w.z * p.y)), fmaf(w.z, p.x, -(w.x * p.z)),
                       fmaf(w.x, p.y, -(w.y * p.x)));
}
__device__ __forceinline__ void load_sym(const float4 *a0, const float2 *a1,
                                         size_t o, float *s)
{
    float4 u = a0[o];
    float2 w = a1[o];
    s[0] = u.x;
    s[1] = u.y;
    s[2] = u.z;
    s[3] = u.w;
    s[4] = w.x;
    s[5] = w.y;
}

// Symmetric 3x3 inverse by the adjugate, as tCudaMatrix::inverse
// (CudaMatrix.h:362-398) evaluates it for a symmetric block.
__device__ __forceinline__ void sym_inverse(const float *a, float *m)
{
    // a = [[a0 a1 a2] [a1 a3 a4] [a2 a4 a5]]
    float c00 = a[3] * a[5] - a[4] * a[4];
    float c01 = a[2] * a[4] - a[1] * a[5];
    float c02 = a[1] * a[4] - a[2] * a[3];
    float c11 = a[0] * a[5] - a[2] * a[2];
    float c12 = a[2] * a[1] - a[0] * a[4];
    float c22 = a[0] * a[3] - a[1] * a[1];
    float det = a[0] * c00 + a[1] * c01 + a[2] * c02;
    float inv = float(1.0 / double(det));
    m[0] = c00 * inv;
    m[1] = c01 * inv;
    m[2] = c02 * inv;
    m[3] = c11 * inv;
    m[4] = c12 * inv;
    m[5] = c22 * inv;
}

// Sum N values over the block (FP32 within a warp, FP64 across warps);
// thread 0 gets the totals. Fixed order.
template <int N>
__device__ __forceinline__ void block_sum(const float (&vf)[N], double (&v)[N],
                                          double (*sh)[kTile / 32])
{
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    float t[N];
#pragma unroll
    for (int k = 0; k < N; k++)
        t[k] = warp_sum(vf[k]);
    if (l == 0)
#pragma unroll
        for (int k = 0; k < N; k++)
            sh[k][w] = double(t[k]);
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < N; k++)
        {
            double s = sh[k][0];
#pragma unroll
            for (int j = 1; j < kTile / 32; j++)
                s += sh[k][j];
            v[k] = s;
        }
    __syncthreads();
}

// FP64 block sum (last-tile stage only); thread 0 gets the totals.
template <int N>
__device__ __forceinline__ void block_sum_d(double (&v)[N], double (*sh)[kTile / 32])
{
#pragma unroll
    for (int k = 0; k < N; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0)
#pragma unroll
        for (int k = 0; k < N; k++)
            sh[k][w] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < N; k++)
        {
            double s = sh[k][0];
#pragma unroll
            for (int j = 1; j < kTile / 32; j++)
                s += sh[k][j];
            v[k] = s;
        }
    __syncthreads();
}

// s[k] += part[k * nt + i] for i = v, v + kTile, v + 2 kTile, ... in that
// order; eight loads in flight at a time (the additions keep their order).
template <int N>
__device__ __forceinline__ void sum_strided(const double *part, int nt, int v,
                                            double (&s)[N])
{
    constexpr int B = 8;
    for (int i0 = v; i0 < nt; i0 += B * kTile)
    {
        double x[B][N];
#pragma unroll
        for (int j = 0; j < B; j++)
        {
            const int i = i0 + j * kTile;
#pragma unroll
            for (int k = 0; k < N; k++)
                x[j][k] = i < nt ? __ldcg(&part[k * nt + i]) : 0.0;
        }
#pragma unroll
        for (int j = 0; j < B; j++)
            if (i0 + j * kTile < nt)
#pragma unroll
                for (int k = 0; k < N; k++)
                    s[k] += x[j][k];
    }
}

// Publish this tile's N partials and find out whether it is the instance's
// last tile. When it is, every thread of the block returns true and totals
// holds the instance sums (summed in tile order, deterministic).
template <int N>
__device__ bool tile_reduce(const InstDesc &d, int tile_idx, const float (&vf)[N],
                            double (&totals)[N], double (*sh)[kTile / 32],
                            int *flag)
{
    double v[N];
    block_sum<N>(vf, v, sh);
    const int nt = d.ntile_rows;
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < N; k++)
            d.part[k * nt + tile_idx] = v[k];
        __threadfence();
        unsigned prev = atomicAdd(&d.st->ticket, 1u);
        *flag = (prev == unsigned(nt - 1));
    }
    __syncthreads();
    if (!*flag)
        return false;
    __threadfence();
    double s[N];
#pragma unroll
    for (int k = 0; k < N; k++)
        s[k] = 0.0;
    // fixed thread -> tile assignment, then a fixed-order block sum
    sum_strided<N>(d.part, nt, threadIdx.x, s);
    block_sum_d<N>(s, sh);
#pragma unroll
    for (int k = 0; k < N; k++)
        totals[k] = s[k];
    return true;
}

__device__ __forceinline__ bool test_converged(const InstDesc &d,
                                               const InstState &s, double rr)
{
    bool ok = false;
    if (d.rel_tol2 > 0.0 && rr <= d.rel_tol2 * s.bb)
        ok = true;
    if (d.abs_tol2 > 0.0 && rr <= d.abs_tol2)
        ok = true;
    return ok;
}

// PCG start bookkeeping of one instance (thread 0 of its last tile): FP64
// scalars from the start sums tot = (r.z, r.r, b.b), counters, the team
// barrier and team-sum buffers of the persistent solver, the active flag.
__device__ __forceinline__ void begin_solve(const InstDesc &d, const double (&tot)[3],
                                            BatchCtl *ctl)
{
    InstState &st = *d.st;
    st.ticket = 0u;
    st.rho = tot[0];
    st.rr = tot[1];
    st.rr0 = tot[1];
    st.bb = tot[2];
    st.beta = 0.0;
    st.alpha = 0.0;
    st.pq = tot[0]; // the estimate the first p.q's fixed-point scale comes from
    st.iter = 0;
    st.status = 0;
    st.bar_count = 0u;
    st.bar_err = 0;
    st.open = 1;
    for (int bq = 0; bq < 3; bq++)
        for (int q = 0; q < 3; q++)
        {
            st.acc[bq][q][0] = 0ull;
            st.acc[bq][q][1] = 0ull;
            st.acc_chk[bq][q] = 0.f;
        }
    if (!isfinite(tot[0]) || !isfinite(tot[1]) || !isfinite(tot[2]))
    {
        st.status = 6; // CLOTH_ERR_NAN
        st.active = 0;
    }
    else if (d.max_iters <= 0 || test_converged(d, st, tot[1]))
    {
        st.active = 0;
    }
    else
    {
        st.active = 1;
        atomicAdd(&ctl->n_active, 1);
    }
}

// round(v * 2^s) as a signed 128-bit integer, returned as H * 2^32 + L with
// 0 <= L < 2^32 (integer operations only).  Exact addition of these limbs
// makes a team sum independent of how the rows are split over blocks.
__device__ __forceinline__ void fx_split(float v, int s, long long &H,
                                         unsigned long long &L)
{
    const unsigned bits = __float_as_uint(v);
    const int e = int((bits >> 23) & 0xffu);
    H = 0;
    L = 0;
    if (e == 0 || e == 255)
        return; // zero, subnormal (below any scale in use) or Inf/NaN (check sum)
    const unsigned long long m = (bits & 0x7fffffu) | 0x800000u;
    const int sh = e - 150 + s; // |v| = m * 2^(e - 150)
    unsigned long long fh = 0ull, fl = 0ull;
    if (sh >= 104)
    {
        fh = 0x3fffffffffffffffull; // saturate; the check sum flags it
        fl = ~0ull;
    }
    else if (sh >= 64)
        fh = m << (sh - 64);
    else if (sh > 0)
    {
        fl = m << sh;
        fh = m >> (64 - sh);
    }
    else if (sh == 0)
        fl = m;
    else if (sh > -25)
        fl = (m + (1ull << (-sh - 1))) >> (-sh);
    if (bits & 0x80000000u)
    {
        fl = ~fl + 1ull;
        fh = ~fh + (fl == 0ull ? 1ull : 0ull);
    }
    L = fl & 0xffffffffull;
    H = (long long)((fh << 32) | (fl >> 32));
}

// Scale exponent for an estimate of a sum (from the double's exponent bits).
__device__ __forceinline__ int fx_scale(double est)
{
    const long long b = __double_as_longlong(est);
    const int e = int((b >> 52) & 0x7ff);
    if (e == 0 || e == 0x7ff)
        return 100;
    const int s = kFxTop - (e - 1023);
    return max(-900, min(900, s));
}

// 2^e for |e| < 1000, built from the exponent field
__device__ __forceinline__ double pow2(int e)
{
    return __longlong_as_double((long long)(1023 + e) << 52);
}

__device__ __forceinline__ double fx_value(unsigned long long H, unsigned long long L,
                                           int s)
{
    return double((long long)H) * pow2(32 - s) + double(L) * pow2(-s);
}

// An instance leaves the loop: the thread that brings the active count down
// to the launch set's hand-off count (0: the last active instance) clears the
// graph's while condition.
__device__ __forceinline__ void retire(BatchCtl *ctl, bool use_cond,
                                       cudaGraphConditionalHandle h)
{
    int prev = atomicSub(&ctl->n_active, 1);
    if (use_cond && prev - 1 == ctl->hand_off)
        cudaGraphSetConditional(h, 0u);
}

// One stretch component (warp/weft or the 45-degree bias frame) of one
// triangle: UpdateComponent / CalcFint / CalcHessian (BaraffClothGpu.cu:7-109).
// Adds the force columns to f and -S*(Ku cu cu^T Du + Kv cv cv^T Dv) to the six
// unique blocks hb[pair][6] (pairs 00 01 02 11 12 22).
// F = c0 x0 + c1 x1 + c2 x2 is evaluated as c1 e1 + c2 e2 + (c0+c1+c2) x0 with
// the edge vectors e1 = x1 - x0, e2 = x2 - x0 formed from the FP64 positions:
// the same value, without the cancellation of three O(|c| |x|) terms in FP32.
__device__ __forceinline__ float3 deformation(const float *c, float3 e1, float3 e2,
                                              float3 x0)
{
    const float s = float((double(c[0]) + double(c[1])) + double(c[2]));
    return c[1] * e1 + c[2] * e2 + s * x0;
}

__device__ __forceinline__ void stretch_component(
    float Ku, float Kv, float S, const float *cu, const float *cv, float3 e1,
    float3 e2, float3 x0, bool fix_fv, float3 *f, float (*hb)[6])
{
    float3 Fu = deformation(cu, e1, e2, x0);
    float3 Fv = deformation(cv, e1, e2, x0);
    float nu = norm3(Fu), nv = norm3(Fv);
    float Cu = nu - 1.f, Cv = nv - 1.f;
    float3 uh = make_float3(Fu.x / nu, Fu.y / nu, Fu.z / nu);
    float3 vh = make_float3(Fv.x / nv, Fv.y / nv, Fv.z / nv);
    // CalcFint: u_base = -S Ku Cu Fu/|Fu|, v_base likewise
    float su = -S * Ku * Cu, sv = -S * Kv * Cv;
    float3 ub = su * uh, vb = sv * vh;
#pragma unroll
    for (int i = 0; i < 3; i++)
        f[i] = f[i] + (cu[i] * ub + cv[i] * vb);
    // CalcHessian: D = n n^T / |F| + [|F| > 1] (1 - 1/|F|) I. The reference
    // uses |Fu| for the weft term as well (BaraffClothGpu.cu:54-55).
    float nvh = fix_fv ? nv : nu;
    float iu = float(1.0 / double(nu)), iv = float(1.0 / double(nvh));
    float eu = (nu > 1.f) ? float(1.0 - 1.0 / double(nu)) : 0.f;
    float ev = (nvh > 1.f) ? float(1.0 - 1.0 / double(nvh)) : 0.f;
    float Du[6] = {iu * uh.x * uh.x + eu, iu * uh.x * uh.y, iu * uh.x * uh.z,
                   iu * uh.y * uh.y + eu, iu * uh.y * uh.z, iu * uh.z * uh.z + eu};
    float Dv[6] = {iv * vh.x * vh.x + ev, iv * vh.x * vh.y, iv * vh.x * vh.z,
                   iv * vh.y * vh.y + ev, iv * vh.y * vh.z, iv * vh.z * vh.z + ev};
    const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int p = 0; p < 6; p++)
    {
        float wu = -S * (Ku * cu[pa[p]] * cu[pb[p]]);
        float wv = -S * (Kv * cv[pa[p]] * cv[pb[p]]);
#pragma unroll
        for (int k = 0; k < 6; k++)
            hb[p][k] += wu * Du[k] + wv * Dv[k];
    }
}

// ---- dihedral bending (cDihedralMaterial, DihedralBending.cpp:120-270, 382-450)
struct D3
{
    double x, y, z;
};
__device__ __forceinline__ D3 d3sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 d3add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 d3scale(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double d3dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 d3cross(D3 a, D3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ D3 d3load(const double *p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ float4 d3f4(D3 a, float w)
{
    return make_float4(float(a.x), float(a.y), float(a.z), w);
}

// One interior edge with stencil (v0 v1 v2 v3), in FP64 from the FP64
// positions: n0 = (v1 - v0) x (v2 - v1), n1 = (v0 - v1) x (v3 - v0),
// e = v1 - v0, beta = atan2(e^.(n0^ x n1^), n0^.n1^).  dbeta/dn0 and
// dbeta/dn1 are the closed forms -(e x n0) / (|e| |n0|^2) and
// (e x n1) / (|e| |n1|^2): the values the reference's
// -sign(sin beta) / sqrt(1 - (n0^.n1^)^2) (I - n^ n^T) / |n| n'^ expressions
// take, without their cancellation as beta -> 0.  The vertex gradients follow
// the reference's chain rule (DihedralBending.cpp:225-268).  Writes the four
// gradients with the factor c in .w, and c beta / 2 (force = (c beta / 2)
// dbeta/dx, Hessian c dbeta/dx dbeta/dx^T, DihedralBending.cpp:420-427).
__device__ __forceinline__ void dihedral_edge(const InstDesc &d, int q)
{
    const int4 s = d.dvid[q];
    const D3 v0 = d3load(d.x64 + 3 * size_t(s.x)), v1 = d3load(d.x64 + 3 * size_t(s.y)),
             v2 = d3load(d.x64 + 3 * size_t(s.z)), v3 = d3load(d.x64 + 3 * size_t(s.w));
    const D3 e = d3sub(v1, v0);
    const D3 n0 = d3cross(e, d3sub(v2, v1));
    const D3 n1 = d3cross(d3sub(v0, v1), d3sub(v3, v0));
    const double nn0 = d3dot(n0, n0), nn1 = d3dot(n1, n1), le = sqrt(d3dot(e, e));
    const double i0 = 1.0 / sqrt(nn0), i1 = 1.0 / sqrt(nn1), ie = 1.0 / le;
    const D3 n0h = d3scale(n0, i0), n1h = d3scale(n1, i1), eh = d3scale(e, ie);
    const double beta = atan2(d3dot(eh, d3cross(n0h, n1h)), d3dot(n0h, n1h));
    const D3 g0 = d3scale(d3cross(e, n0), -1.0 / (le * nn0));
    const D3 g1 = d3scale(d3cross(e, n1), 1.0 / (le * nn1));
    const D3 gv0 = d3add(d3cross(d3sub(v1, v2), g0), d3cross(d3sub(v3, v1), g1));
    const D3 gv1 = d3add(d3cross(d3sub(v2, v0), g0), d3cross(d3sub(v0, v3), g1));
    const D3 gv2 = d3cross(d3sub(v0, v1), g0);
    const D3 gv3 = d3cross(d3sub(v1, v0), g1);
    const double c = d.dfac[q];
    const float cf = float(c);
    float4 *rec = d.drec + 4 * size_t(q);
    rec[0] = d3f4(gv0, cf);
    rec[1] = d3f4(gv1, cf);
    rec[2] = d3f4(gv2, cf);
    rec[3] = d3f4(gv3, cf);
    d.dfb[q] = float(c * beta / 2);
}

// Block (a, b) of one dihedral edge, c g_a g_b^T, added as its symmetric part
// S and skew vector w (S p + w x p = c g_a (g_b . p)).  S is formed
// symmetrically in a and b and w changes sign with them, bit for bit, so the
// row-a and row-b copies of a block pair are exact transposes.
__device__ __forceinline__ void dihedral_block(float4 ga, float4 gb, float *K, float *w)
{
    const float c = ga.w, h = 0.5f * c;
    K[0] += c * (ga.x * gb.x);
    K[1] += h * (ga.x * gb.y + ga.y * gb.x);
    K[2] += h * (ga.x * gb.z + ga.z * gb.x);
    K[3] += c * (ga.y * gb.y);
    K[4] += h * (ga.y * gb.z + ga.z * gb.y);
    K[5] += c * (ga.z * gb.z);
    // c/2 (g_a g_b^T - g_b g_a^T) p = c/2 (g_b x g_a) x p
    w[0] += h * (gb.y * ga.z - gb.z * ga.y);
    w[1] += h * (gb.z * ga.x - gb.x * ga.z);
    w[2] += h * (gb.x * ga.y - gb.y * ga.x);
}

} // namespace

// ------------------------------------------------------------------ pins
// UpdateConstraintVertexPos (BaraffClothGpu.cpp:411-436): pinned vertices are
// put at their target in x and x_pre; x32.w marks them for the row pass.
__global__ void k_pins(InstDesc *const *descs, const int *inst_list, int ninst,
                       const int *ninst_dev)
{
    if (ninst_dev)
        ninst = *ninst_dev;
    for (int i = blockIdx.x; i < ninst; i += gridDim.x)
    {
        const InstDesc &d = *descs[inst_list[i]];
        for (int k = threadIdx.x; k < d.npins; k += blockDim.x)
        {
            int v = d.pin_vid[k];
            float4 t = d.pin_tgt[k];
            double tx = t.x, ty = t.y, tz = t.z;
            d.x64[3 * v + 0] = tx;
            d.x64[3 * v + 1] = ty;
            d.x64[3 * v + 2] = tz;
            d.xp64[3 * v + 0] = tx;
            d.xp64[3 * v + 1] = ty;
            d.xp64[3 * v + 2] = tz;
            d.x32[v] = make_float4(t.x, t.y, t.z, 1.f);
        }
    }
}

// ------------------------------------------------------------------ triangles
__global__ void __launch_bounds__(kTile) k_tri(InstDesc *const *descs,
                                               const Tile *tiles,
                                               const BatchCtl *ctl)
{
    const int ntiles = ctl->n_tiles_tris;
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x)
    {
        const Tile tl = tiles[ti];
        const InstDesc &d = *descs[tl.inst];
        const int t = tl.start + threadIdx.x;
        if (t >= d.nt)
        {
            // the dihedral edges follow the triangles in the tile list
            if (t - d.nt < d.n_dih)
                dihedral_edge(d, t - d.nt);
            continue;
        }
        const int4 tv = d.tri[t];
        const float S = __int_as_float(tv.w);
        const float4 c0 = d.tcoef[3 * t + 0], c1 = d.tcoef[3 * t + 1],
                     c2 = d.tcoef[3 * t + 2];
        const float cuw[3] = {c0.x, c0.y, c0.z}, cvw[3] = {c0.w, c1.x, c1.y};
        const float cud[3] = {c1.z, c1.w, c2.x}, cvd[3] = {c2.y, c2.z, c2.w};
        const double *p0 = d.x64 + 3 * tv.x, *p1 = d.x64 + 3 * tv.y,
                     *p2 = d.x64 + 3 * tv.z;
        const double a0 = p0[0], a1 = p0[1], a2 = p0[2];
        const float3 x0 = make_float3(float(a0), float(a1), float(a2));
        const float3 e1 = make_float3(float(p1[0] - a0), float(p1[1] - a1),
                                      float(p1[2] - a2));
        const float3 e2 = make_float3(float(p2[0] - a0), float(p2[1] - a1),
                                      float(p2[2] - a2));
        float3 f[3] = {make_float3(0, 0, 0), make_float3(0, 0, 0),
                       make_float3(0, 0, 0)};
        float hb[6][6];
#pragma unroll
        for (int p = 0; p < 6; p++)
#pragma unroll
            for (int k = 0; k < 6; k++)
                hb[p][k] = 0.f;
        const bool fix = d.fix_fv_norm != 0;
        stretch_component(d.k_warp, d.k_weft, S, cuw, cvw, e1, e2, x0, fix, f, hb);
        stretch_component(d.k_bias, d.k_bias, S, cud, cvd, e1, e2, x0, fix, f, hb);

        const int4 g0 = d.tdest[3 * t + 0], g1 = d.tdest[3 * t + 1],
                   g2 = d.tdest[3 * t + 2];
        // h_dest[a*3+b] for a,b in 0..2, then f_dest[0..2]
        const int hd[9] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w, g2.x};
        const int fd[3] = {g2.y, g2.z, g2.w};
        const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
        for (int p = 0; p < 6; p++)
        {
            HRec r;
            r.h0 = make_float4(hb[p][0], hb[p][1], hb[p][2], hb[p][3]);
            r.h1 = make_float4(hb[p][4], hb[p][5], 0.f, 0.f);
            d.hrec[hd[pa[p] * 3 + pb[p]]] = r;
            if (pa[p] != pb[p])
                d.hrec[hd[pb[p] * 3 + pa[p]]] = r;
        }
#pragma unroll
        for (int a = 0; a < 3; a++)
            d.frec[fd[a]] = f4(f[a]);
    }
}

// ------------------------------------------------------------------ rows
__global__ void __launch_bounds__(kTile) k_row(InstDesc *const *descs,
                                               const Tile *tiles, BatchCtl *ctl)
{
    __shared__ double sh[3][kTile / 32];
    __shared__ int flag;
    const int ntiles = ctl->n_tiles_rows;
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x)
    {
        const Tile tl = tiles[ti];
        const InstDesc &d = *descs[tl.inst];
        const int row = tl.start + threadIdx.x;
        float part[3] = {0.f, 0.f, 0.f};
        if (row < d.nv)
        {
            const int info = d.rowinfo[row];
            const int len = info & 255, ds = (info >> 8) & 255;
            const float4 xv = d.x32[row];
            const bool fixv = xv.w != 0.f;
            const int ncinc = d.ccount ? d.ccount->cap_inc : 0;
            const float m = d.mass[row];
            float3 f = make_float3(0, 0, 0);
            for (int k = d.fptr[row]; k < d.fptr[row + 1]; k++)
                f = f + xyz(d.frec[k]);
            float3 acc = make_float3(0, 0, 0);
            float ad[6] = {0, 0, 0, 0, 0, 0};
            for (int s = 0; s < len; s++)
            {
                const size_t o = size_t(s) * d.stride + row;
                const int c = d.col[o];
                const uint32_t hs = d.hsrc[o];
                const float kbv = d.kb[o];
                float K[6] = {0, 0, 0, 0, 0, 0};
                const uint32_t r0 = hs >> 5, cnt = hs & 31u;
                for (uint32_t k = 0; k < cnt; k++)
                {
                    const HRec h = d.hrec[r0 + k];
                    K[0] += h.h0.x;
                    K[1] += h.h0.y;
                    K[2] += h.h0.z;
                    K[3] += h.h0.w;
                    K[4] += h.h1.x;
                    K[5] += h.h1.y;
                }
                const float4 xc = (c == row) ? xv : d.x32[c];
                // bending: K -= K_b (K_b = kb I), f += -K_b x
                f = f - kbv * xyz(xc);
                K[0] -= kbv;
                K[3] -= kbv;
                K[5] -= kbv;
                // dihedral bending: K += c g_a g_b^T over the stencils holding
                // (row, c) in edge order; f += (c beta / 2) g_a at the diagonal
                float wv[3] = {0.f, 0.f, 0.f};
                if (d.dsrc)
                {
                    const uint32_t de = d.dsrc[o];
                    const uint32_t e0 = de >> 5, ne = de & 31u;
                    for (uint32_t k = 0; k < ne; k++)
                    {
                        const uint32_t en = d.dent[e0 + k];
                        const float4 *rec = d.drec + 4 * size_t(en >> 4);
                        const float4 ga = rec[(en >> 2) & 3u], gb = rec[en & 3u];
                        dihedral_block(ga, gb, K, wv);
                        if (s == ds)
                            f = f + d.dfb[en >> 4] * xyz(ga);
                    }
                }
                float A[6];
#pragma unroll
                for (int k = 0; k < 6; k++)
                    A[k] = d.c_stiff * K[k];
                float4 Aw = make_float4(d.c_stiff * wv[0], d.c_stiff * wv[1], d.c_stiff * wv[2],
                                        0.f);
                // contact Hessian (PrepareCollisionHessian, BaraffCloth.cpp:928-990):
                // 1e-2 (w_i N)(w_j N)^T per point-triangle contact holding row
                // and c, w = 1 at a cloth point, -b at a cloth triangle's
                // vertices; added to the system matrix unscaled, formed
                // symmetrically so both rows of a pair hold the same block
                float Hc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if (d.cinc_off)
                    for (int k = d.cinc_off[row]; k < min(d.cinc_off[row + 1], ncinc); k++)
                    {
                        const int tag = d.cinc[k];
                        if (!(tag & kPtTag))
                            continue;
                        const PtContact &pc = d.cpt[tag & ~kPtTag];
                        double wi = 0.0, wj = 0.0;
                        bool hit = false;
                        if (pc.cloth_point)
                        {
                            if (c == row)
                            {
                                wi = wj = 1.0;
                                hit = true;
                            }
                        }
                        else
                        {
                            const int4 tv = d.tri[pc.t];
                            const int vv[3] = {tv.x, tv.y, tv.z};
#pragma unroll
                            for (int q = 0; q < 3; q++)
                            {
                                if (vv[q] == row)
                                    wi = -double(pc.bary[q]);
                                if (vv[q] == c)
                                {
                                    wj = -double(pc.bary[q]);
                                    hit = true;
                                }
                            }
                        }
                        if (!hit)
                            continue;
                        const double N[3] = {pc.n[0], pc.n[1], pc.n[2]};
                        const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
                        for (int q = 0; q < 6; q++)
                        {
                            const double u = (wi * N[pa[q]]) * (wj * N[pb[q]]);
                            const double v = (wi * N[pb[q]]) * (wj * N[pa[q]]);
                            Hc[q] += float(1e-2 * (0.5 * (u + v)));
                        }
                    }
                bool zero = false;
                if (s == ds)
                {
                    const float md = m * d.c_mass;
                    A[0] += md;
                    A[3] += md;
                    A[5] += md;
#pragma unroll
                    for (int k = 0; k < 6; k++)
                    {
                        A[k] += Hc[k];
                        ad[k] = A[k];
                    }
                }
                else if (fixv || xc.w != 0.f)
                {
                    zero = true;
#pragma unroll
                    for (int k = 0; k < 6; k++)
                        A[k] = 0.f;
                    Aw = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                else
                {
#pragma unroll
                    for (int k = 0; k < 6; k++)
                        A[k] += Hc[k];
                }
                if (s >= ds)
                {
                    // stored: diagonal and upper blocks (the lower ones are
                    // the same values, held by the transposed position)
                    const size_t ou = up_idx(s - ds, row, d.width_up);
                    d.A0[ou] = make_float4(A[0], A[1], A[2], A[3]);
                    d.A1[ou] = make_float2(A[4], A[5]);
                    if (d.Aw)
                        d.Aw[ou] = Aw;
                }
                if (d.warm_start && !zero && !fixv)
                {
                    const float3 xd = xyz(d.dx[c]);
                    acc = acc + symv(A, xd);
                    if (d.Aw)
                        acc = acc + skewv(Aw, xd);
                }
            }
            // AssembleSystemRHSKernel (BaraffClothGpu.cu:301-344)
            const float3 g = make_float3(0.f, d.grav[row], 0.f);
            const float3 xc = make_float3(float(d.x64[3 * row + 0]),
                                          float(d.x64[3 * row + 1]),
                                          float(d.x64[3 * row + 2]));
            const float3 xp = make_float3(float(d.xp64[3 * row + 0]),
                                          float(d.xp64[3 * row + 1]),
                                          float(d.xp64[3 * row + 2]));
            float3 b = d.h2 * (g + f) + m * (xc - xp);
            if (fixv)
                b = make_float3(0, 0, 0);
            float M[6];
            sym_inverse(ad, M);
            float3 r = b - acc;
            if (fixv || !d.warm_start)
                d.dx[row] = make_float4(0, 0, 0, 0);
            if (fixv)
                r = make_float3(0, 0, 0);
            const float3 z = symv(M, r);
            d.b[row] = f4(b);
            d.r[row] = f4(r);
            d.z[row] = f4(z);
            d.M0[row] = make_float4(M[0], M[1], M[2], M[3]);
            d.M1[row] = make_float2(M[4], M[5]);
            part[0] = fdot(r, z);
            part[1] = fdot(r, r);
            part[2] = fdot(b, b);
        }
        double tot[3];
        if (tile_reduce<3>(d, tl.start / kTile, part, tot, sh, &flag) &&
            threadIdx.x == 0)
            begin_solve(d, tot, ctl);
    }
}

// PCG start of an iterative-refinement correction: the system is the
// assembled A with right-hand side float(rhs64) (zero on pinned rows), from
// dx = 0.  Same bookkeeping as the start k_row makes.
__global__ void __launch_bounds__(kTile) k_ir_start(InstDesc *const *descs,
                                                    const Tile *tiles, BatchCtl *ctl,
                                                    const double *rhs64)
{
    __shared__ double sh[3][kTile / 32];
    __shared__ int flag;
    const int ntiles = ctl->n_tiles_rows;
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x)
    {
        const Tile tl = tiles[ti];
        const InstDesc &d = *descs[tl.inst];
        const int row = tl.start + threadIdx.x;
        float part[3] = {0.f, 0.f, 0.f};
        if (row < d.nv)
        {
            const bool fixv = d.x32[row].w != 0.f;
            float3 r = make_float3(float(rhs64[3 * row + 0]), float(rhs64[3 * row + 1]),
                                   float(rhs64[3 * row + 2]));
            if (fixv)
                r = make_float3(0, 0, 0);
            float M[6];
            load_sym(d.M0, d.M1, row, M);
            const float3 z = symv(M, r);
            d.dx[row] = make_float4(0, 0, 0, 0);
            d.r[row] = f4(r);
            d.z[row] = f4(z);
            part[0] = fdot(r, z);
            part[1] = fdot(r, r);
            part[2] = part[1];
        }
        double tot[3];
        if (tile_reduce<3>(d, tl.start / kTile, part, tot, sh, &flag) &&
            threadIdx.x == 0)
            begin_solve(d, tot, ctl);
    }
}

// Sets the while condition from the active count (one thread).
__global__ void k_cond(const BatchCtl *ctl, cudaGraphConditionalHandle h)
{
    cudaGraphSetConditional(h, ctl->n_active > ctl->hand_off ? 1u : 0u);
}

// ------------------------------------------------------------------ PCG
// The graph-loop kernels come in variants: R rows per thread (blocks of
// kTile / R threads; thread t of a tile owns rows t, t + kTile/R, ...) and U
// ELL slots whose loads are issued together.  Every variant reproduces the
// arithmetic and the summation order of R = 1 exactly - the per-row work is
// the same code, and the tile sums go through 32-row groups summed in group
// order, whichever thread held the group - so the variant an autotuner picks
// does not change any result.
namespace {

// A tile's N sums (rows held R per thread) into quantities q0.. of the
// instance's team-sum buffer bq: the FP32 butterfly of each 32-row group (the
// persistent kernels' chunks: their team ranges are aligned to 32 rows), each
// group sum as fixed-point limbs at scale sc[k] (fx_split; lane r N + k
// converts group (r, k), side by side), the limbs of a warp's groups added
// with shuffles and sent with one reduction per limb by lanes 0 .. N-1.  The
// totals are exact, so every kernel variant and every PCG driver gets the
// same ones.  R and N are powers of two.
template <int R, int N>
__device__ __forceinline__ void tile_fx_add(const float (&vf)[R][N], InstState *st, int bq,
                                            int q0, const int (&sc)[N])
{
    constexpr unsigned FULLM = 0xffffffffu;
    const int l = threadIdx.x & 31;
    float tsum[R][N];
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int k = 0; k < N; k++)
            tsum[r][k] = warp_sum(vf[r][k]);
    long long hh = 0;
    unsigned long long ll = 0ull;
    float c = 0.f;
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int k = 0; k < N; k++)
            if (l == r * N + k)
            {
                fx_split(tsum[r][k], sc[k], hh, ll);
                c = tsum[r][k];
            }
#pragma unroll
    for (int o = (R / 2) * N; o >= N && o > 0; o >>= 1)
    {
        hh += __shfl_xor_sync(FULLM, hh, o);
        ll += __shfl_xor_sync(FULLM, ll, o);
        c += __shfl_xor_sync(FULLM, c, o);
    }
    if (l < N)
    {
        atomicAdd(&st->acc[bq][q0 + l][0], (unsigned long long)hh);
        atomicAdd(&st->acc[bq][q0 + l][1], ll);
        atomicAdd(&st->acc_chk[bq][q0 + l], c);
    }
}

// Read-only load of a pointer field (the descriptor is constant during a kernel).
template <class T> __device__ __forceinline__ T *ldg_ptr(T *const *addr)
{
    return reinterpret_cast<T *>(
        __ldg(reinterpret_cast<const unsigned long long *>(addr)));
}

// What the SpMV kernel needs of one instance, loaded once per run of
// consecutive tiles of that instance (descriptor fields are read-only during
// the kernel; the scalars are the ones the previous kernel left).
struct SpmvHdr
{
    int inst, nv, wu, nt, active, wl;
    int it, s_pq; // iteration (team-sum buffer it % 3) and the p.q scale
    float beta;
    const int *rowinfo, *colu;
    const uint32_t *lref;
    const float4 *A0;
    const float2 *A1;
    const float4 *Aw; // skew parts (dihedral bending), or null
    const float4 *z, *pold;
    float4 *pnew, *q;
    double *part;
    InstState *st;
};

__device__ __forceinline__ void load_hdr(SpmvHdr &h, const Tile &tl)
{
    const InstDesc *dp = tl.d;
    const int inst = tl.inst;
    InstState *st = tl.st;
    h.inst = inst;
    h.active = st->active;
    const int it = st->iter;
    h.it = it;
    h.s_pq = fx_scale(st->pq);
    h.beta = float(st->beta);
    h.nv = __ldg(&dp->nv);
    h.wu = __ldg(&dp->width_up);
    h.wl = __ldg(&dp->width_lo);
    h.nt = __ldg(&dp->ntile_rows);
    h.rowinfo = ldg_ptr(&dp->rowinfo);
    h.lref = ldg_ptr(&dp->lref);
    h.colu = ldg_ptr(&dp->colu);
    h.A0 = ldg_ptr(reinterpret_cast<float4 *const *>(&dp->A0));
    h.A1 = ldg_ptr(reinterpret_cast<float2 *const *>(&dp->A1));
    h.Aw = ldg_ptr(reinterpret_cast<float4 *const *>(&dp->Aw));
    h.z = ldg_ptr(reinterpret_cast<float4 *const *>(&dp->z));
    float4 *p0 = ldg_ptr(&dp->p0), *p1 = ldg_ptr(&dp->p1);
    h.pold = (it & 1) ? p1 : p0;
    h.pnew = (it & 1) ? p0 : p1;
    h.q = ldg_ptr(&dp->q);
    h.part = ldg_ptr(&dp->part);
    h.st = st;
}

// R rows of q = A p (rows row0 + r * T) with p = z + beta p_old recomputed
// at the gathered columns; writes p_new and q, leaves p.q per row in pq.
// Slots in column order: the lower ones by s (block at the transposed
// position), then the diagonal and upper ones by plane u. Step k covers lower
// plane k for k < wl and upper plane k - wl after (wl, the instance's lower
// plane count, is uniform), so every load instruction of a warp reads one
// plane; at each step the loads of all R rows and U steps are in flight
// together.  SKEW: the instance may carry skew block parts (dihedral
// bending); they are read and applied when its header has them.
template <int R, int U, int T, bool SKEW>
__device__ __forceinline__ void spmv_rows(const SpmvHdr &d, int row0, float (&pq)[R][1])
{
    const float beta = d.beta;
    const int wl = d.wl;
    int len[R], ds[R], kend[R];
    float3 pv[R], q[R];
    bool ok[R];
    int kmax = 0;
#pragma unroll
    for (int r = 0; r < R; r++)
    {
        const int row = row0 + r * T;
        ok[r] = row < d.nv;
        len[r] = ds[r] = 0;
        pv[r] = q[r] = make_float3(0, 0, 0);
        if (ok[r])
        {
            const int info = d.rowinfo[row];
            len[r] = info & 255;
            ds[r] = (info >> 8) & 255;
            pv[r] = xyz(d.z[row]);
            if (beta != 0.f)
                pv[r] = pform(pv[r], beta, xyz(d.pold[row]));
            d.pnew[row] = f4(pv[r]);
        }
        kend[r] = wl + (len[r] - ds[r]);
        kmax = max(kmax, ok[r] ? kend[r] : 0);
    }
    for (int k0 = 0; k0 < kmax; k0 += U)
    {
        int cc[R][U];
        float4 a0[R][U];
        float2 a1[R][U];
        float4 aw[R][U];
        bool on[R][U];
#pragma unroll
        for (int k = 0; k < U; k++)
        {
            const int kk = k0 + k;
            const bool lower = kk < wl;
#pragma unroll
            for (int r = 0; r < R; r++)
            {
                const int row = row0 + r * T;
                on[r][k] = ok[r] && (lower ? kk < ds[r] : kk < kend[r]);
                if (on[r][k])
                {
                    uint32_t oa;
                    if (lower)
                    {
                        const uint32_t ref = d.lref[lo_idx(kk, row, wl)];
                        cc[r][k] = lref_col(ref);
                        oa = lref_block(ref, d.wu);
                    }
                    else
                    {
                        oa = up_idx(kk - wl, row, d.wu);
                        cc[r][k] = d.colu[oa];
                    }
                    a0[r][k] = d.A0[oa];
                    a1[r][k] = d.A1[oa];
                    if (SKEW && d.Aw)
                        aw[r][k] = d.Aw[oa];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < U; k++)
#pragma unroll
            for (int r = 0; r < R; r++)
                if (on[r][k])
                {
                    const int row = row0 + r * T;
                    const int c = cc[r][k];
                    const float A[6] = {a0[r][k].x, a0[r][k].y, a0[r][k].z, a0[r][k].w,
                                        a1[r][k].x, a1[r][k].y};
                    float3 pc;
                    if (c == row)
                        pc = pv[r];
                    else
                    {
                        pc = xyz(d.z[c]);
                        if (beta != 0.f)
                            pc = pform(pc, beta, xyz(d.pold[c]));
                    }
                    q[r] = q[r] + symv(A, pc);
                    if (SKEW && d.Aw)
                    {
                        const float3 cw = skewv(aw[r][k], pc);
                        q[r] = (k0 + k < wl) ? q[r] - cw : q[r] + cw;
                    }
                }
    }
#pragma unroll
    for (int r = 0; r < R; r++)
    {
        pq[r][0] = 0.f;
        if (ok[r])
        {
            d.q[row0 + r * T] = f4(q[r]);
            pq[r][0] = fdot(pv[r], q[r]);
        }
    }
}

struct UpdHdr
{
    int inst, nv, nt, active, iter;
    int s_rz, s_rr; // scales of the new r.z and r.r
    float alpha;
    const float4 *pnew, *q;
    float4 *dx, *r, *z;
    const float4 *M0;
    const float2 *M1;
    double *part;
    InstState *st;
};

__device__ __forceinline__ void load_hdr(UpdHdr &h, const Tile &tl)
{
    const InstDesc *dp = tl.d;
    const int inst = tl.inst;
    InstState *st = tl.st;
    h.inst = inst;
    h.active = st->active;
    h.iter = st->iter;
    h.s_rz = fx_scale(st->rho);
    h.s_rr = fx_scale(st->rr);
    h.alpha = float(st->alpha);
    h.nv = __ldg(&dp->nv);
    h.nt = __ldg(&dp->ntile_rows);
    float4 *p0 = ldg_ptr(&dp->p0), *p1 = ldg_ptr(&dp->p1);
    h.pnew = (h.iter & 1) ? p0 : p1;
    h.q = ldg_ptr(&dp->q);
    h.dx = ldg_ptr(&dp->dx);
    h.r = ldg_ptr(&dp->r);
    h.z = ldg_ptr(&dp->z);
    h.M0 = ldg_ptr(reinterpret_cast<float4 *const *>(&dp->M0));
    h.M1 = ldg_ptr(reinterpret_cast<float2 *const *>(&dp->M1));
    h.part = ldg_ptr(&dp->part);
    h.st = st;
}

} // namespace

// Blocks take TPB consecutive tile-list entries at a time (grid-stride over
// those groups); the instance header is reloaded only when the instance
// changes, so its dependent loads are paid once per run of tiles.
template <int R, int U, int TPB, bool SKEW>
__global__ void __launch_bounds__(kTile / R) k_spmv_t(InstDesc *const *descs,
                                                      const Tile *tiles, BatchCtl *ctl,
                                                      int use_cond,
                                                      cudaGraphConditionalHandle h)
{
    constexpr int T = kTile / R;
    __shared__ SpmvHdr d; // the current instance's header (thread 0 loads it)
    const int ntiles = ctl->n_tiles_rows;
    int cur = -1;
    for (int t0 = blockIdx.x * TPB; t0 < ntiles; t0 += gridDim.x * TPB)
    {
        const int t1 = min(t0 + TPB, ntiles);
        for (int ti = t0; ti < t1; ti++)
        {
            const Tile tl = tiles[ti];
            if (tl.inst != cur)
            {
                __syncthreads();
                if (threadIdx.x == 0)
                    load_hdr(d, tl);
                __syncthreads();
                cur = tl.inst;
            }
            if (!d.active)
                continue;
            float part[R][1];
            spmv_rows<R, U, T, SKEW>(d, tl.start + threadIdx.x, part);
            const int sc[1] = {d.s_pq};
            tile_fx_add<R, 1>(part, d.st, d.it % 3, 0, sc);
        }
    }
}

template <int R, int TPB>
__global__ void __launch_bounds__(kTile / R) k_update_t(InstDesc *const *descs,
                                                        const Tile *tiles, BatchCtl *ctl,
                                                        int use_cond,
                                                        cudaGraphConditionalHandle h,
                                                        int *iters_left)
{
    constexpr int T = kTile / R;
    // chunked loops (the request server): the last iteration of a chunk ends
    // the while loop; the condition is read after the body completes
    if (iters_left && blockIdx.x == 0 && threadIdx.x == 0)
    {
        const int left = *iters_left - 1;
        *iters_left = left;
        if (use_cond && left <= 0)
            cudaGraphSetConditional(h, 0u);
    }
    __shared__ UpdHdr d; // the current instance's header (thread 0 loads it)
    const int ntiles = ctl->n_tiles_rows;
    int cur = -1;
    for (int t0 = blockIdx.x * TPB; t0 < ntiles; t0 += gridDim.x * TPB)
    {
        const int t1 = min(t0 + TPB, ntiles);
        for (int ti = t0; ti < t1; ti++)
        {
            const Tile tl = tiles[ti];
            if (tl.inst != cur)
            {
                __syncthreads();
                if (threadIdx.x == 0)
                    load_hdr(d, tl);
                __syncthreads();
                cur = tl.inst;
            }
            if (!d.active)
                continue;
            const float alpha = d.alpha;
            float part[R][2];
#pragma unroll
            for (int r = 0; r < R; r++)
            {
                const int row = tl.start + r * T + threadIdx.x;
                part[r][0] = part[r][1] = 0.f;
                if (row < d.nv)
                {
                    const float3 p = xyz(d.pnew[row]);
                    const float3 qv = xyz(d.q[row]);
                    float3 x = xyz(d.dx[row]);
                    float3 rr = xyz(d.r[row]);
                    x = make_float3(fmaf(alpha, p.x, x.x), fmaf(alpha, p.y, x.y),
                                    fmaf(alpha, p.z, x.z));
                    rr = make_float3(fmaf(-alpha, qv.x, rr.x), fmaf(-alpha, qv.y, rr.y),
                                     fmaf(-alpha, qv.z, rr.z));
                    float M[6];
                    load_sym(d.M0, d.M1, row, M);
                    const float3 z = symv(M, rr);
                    d.dx[row] = f4(x);
                    d.r[row] = f4(rr);
                    d.z[row] = f4(z);
                    part[r][0] = fdot(rr, z);
                    part[r][1] = fdot(rr, rr);
                }
            }
            const int sc[2] = {d.s_rz, d.s_rr};
            tile_fx_add<R, 2>(part, d.st, d.iter % 3, 1, sc);
        }
    }
}

// ------------------------------------------------------------------ bulk-staged SpMV
// The same SpMV as k_spmv_t (R = 1: one row per thread, the same slot order
// and arithmetic, so the results are bit-identical), with the streamed data
// moved by the copy engine instead of by dependent loads.  For every tile, one
// thread issues bulk asynchronous copies (cp.async.bulk, completion counted
// on an mbarrier) of the tile's row info, lower-slot columns and
// transposed-block indices, upper-slot columns and stored blocks, and the z
// and p_old rows of the tile's column range (its halo); a ring of NST stages
// in shared memory keeps NST - 1 tiles in flight while the block computes one.
// The compute then reads everything from shared memory except the lower
// slots' transposed blocks, gathered from L2 (a neighbouring tile streamed
// them moments before).  p = z + beta p_old is formed once per halo row in
// shared memory.  A tile whose halo does not fit in its stage gathers z and
// p_old from global memory instead.
namespace {

struct BulkHdr
{
    int go;                 // instance active: the stage is (being) filled
    int start, nrows;       // first row, rows of the tile in the instance
    int h0, nh;             // halo rows [h0, h0 + nh) staged (nh = 0: not staged)
    int skew;               // the stage holds skew block parts
    int tile_idx, nt;       // partial-sum slot
    int wu;                 // upper planes (transposed-block indexing)
    float beta;
    unsigned o_lr, o_cu, o_a0, o_a1, o_aw, o_z, o_p; // byte offsets in the stage
    const float4 *A0;       // transposed-block gathers
    const float2 *A1;
    const float4 *Aw;
    const float4 *z, *pold; // halo fallback gathers
    float4 *pnew, *q;
    double *part;
    InstState *st;
    int it, s_pq; // iteration (team-sum buffer it % 3) and the p.q scale
};

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                     smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], "
                 "%2, [%3];" ::"r"(smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ unsigned dynamic_smem_bytes()
{
    unsigned r;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
    return r;
}

// A stage's wait gives up after this long (each try_wait may suspend the
// thread for a while, so the bound is on the global timer, not on polls).
constexpr unsigned long long kBulkWaitNs = 2000000000ull;
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// What the producer warp needs of one tile: its lane k resolves tile
// j + k's dependent loads (tile list -> descriptor -> halo table, and the
// instance state) for 32 tiles at once, ahead of their copies.
struct BulkMeta
{
    int go, start, nv, wl, wu, nt, it, s_pq;
    int hx, hy;
    float beta;
    const int *rowinfo, *colu;
    const uint32_t *lref;
    const float4 *A0, *Aw, *z;
    const float2 *A1;
    float4 *p0, *p1, *q;
    double *part;
    InstState *st;
};

__device__ __forceinline__ void bulk_meta(const Tile *tiles, int ti, BulkMeta &m)
{
    const Tile tl = tiles[ti];
    const InstDesc *dp = tl.d;
    m.st = tl.st;
    m.start = tl.start;
    m.go = __ldcg(&tl.st->active);
    m.it = __ldcg(&tl.st->iter);
    m.s_pq = fx_scale(__ldcg(&tl.st->pq));
    m.beta = float(__ldcg(&tl.st->beta));
    m.nv = __ldg(&dp->nv);
    m.wl = __ldg(&dp->width_lo);
    m.wu = __ldg(&dp->width_up);
    m.nt = __ldg(&dp->ntile_rows);
    m.rowinfo = ldg_ptr(&dp->rowinfo);
    m.colu = ldg_ptr(&dp->colu);
    m.lref = ldg_ptr(&dp->lref);
    m.A0 = ldg_ptr(reinterpret_cast<float4 *const *>(&dp->A0));
    m.A1 = ldg_ptr(reinterpret_cast<float2 *const *>(&dp->A1));
    m.Aw = ldg_ptr(reinterpret_cast<float4 *const *>(&dp->Aw));
    m.z = ldg_ptr(reinterpret_cast<float4 *const *>(&dp->z));
    m.p0 = ldg_ptr(&dp->p0);
    m.p1 = ldg_ptr(&dp->p1);
    m.q = ldg_ptr(&dp->q);
    m.part = ldg_ptr(&dp->part);
    const int2 hh = __ldg(ldg_ptr(&dp->thalo) + tl.start / kTile);
    m.hx = hh.x;
    m.hy = hh.y;
}

template <class T> __device__ __forceinline__ T *shfl_ptr(T *p, int src)
{
    return reinterpret_cast<T *>(
        __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(p), src));
}

// The producer warp fills one stage with the tile whose metadata lane `src`
// holds (nothing but the phase when its instance is done): lane 0 writes the
// header and arrives with the stage's byte count, then the lanes share the
// copies (row info, each plane, the halo of z and p_old).
template <bool SKEW, bool HALO>
__device__ __forceinline__ void bulk_issue_warp(const BulkMeta &m, int src, BulkHdr &h,
                                                unsigned char *stage, unsigned stage_bytes,
                                                uint64_t *bar, int lane)
{
    constexpr unsigned FULLM = 0xffffffffu;
    const int go = __shfl_sync(FULLM, m.go, src);
    if (!go)
    {
        if (lane == 0)
        {
            h.go = 0;
            mbar_arrive(bar); // nothing to copy: complete the phase now
        }
        __syncwarp();
        return;
    }
    const int start = __shfl_sync(FULLM, m.start, src), nv = __shfl_sync(FULLM, m.nv, src);
    const int wl = __shfl_sync(FULLM, m.wl, src);
    const int wu = __shfl_sync(FULLM, m.wu, src), it = __shfl_sync(FULLM, m.it, src);
    const int hx = __shfl_sync(FULLM, m.hx, src), hy = __shfl_sync(FULLM, m.hy, src);
    const float beta = __shfl_sync(FULLM, m.beta, src);
    const float4 *A0 = shfl_ptr(m.A0, src), *Aw = shfl_ptr(m.Aw, src), *z = shfl_ptr(m.z, src);
    const float2 *A1 = shfl_ptr(m.A1, src);
    float4 *p0 = shfl_ptr(m.p0, src), *p1 = shfl_ptr(m.p1, src);
    const float4 *pold = (it & 1) ? p1 : p0;
    const int nrows = min(kTile, nv - start);
    const bool skew = SKEW && Aw != nullptr;
    const unsigned o_lr = kTile * 4;
    const unsigned o_cu = o_lr + unsigned(wl) * kTile * 4;
    const unsigned o_a0 = o_cu + unsigned(wu) * kTile * 4;
    const unsigned o_a1 = o_a0 + unsigned(wu) * kTile * 16;
    const unsigned o_aw = o_a1 + unsigned(wu) * kTile * 8;
    const unsigned o_z = o_aw + (skew ? unsigned(wu) * kTile * 16 : 0u);
    int nh = hy - hx;
    const bool two = beta != 0.f;
    unsigned halo = unsigned(nh) * 16u * (two ? 2u : 1u);
    if (!HALO || nh <= 0 || o_z + halo > stage_bytes)
    {
        nh = 0;
        halo = 0;
    }
    const unsigned o_p = o_z + unsigned(nh) * 16u;
    const unsigned ri_bytes = unsigned((nrows + 3) & ~3) * 4u;
    const unsigned pb = kTile * 4u; // one plane of 4-byte entries (tile-major, whole tiles)
    if (lane == 0)
    {
        // the whole header before the arrival: its release publishes the
        // header to the consumers that acquire the completed phase
        h.go = 1;
        h.start = start;
        h.nrows = nrows;
        h.h0 = hx;
        h.nh = nh;
        h.skew = skew ? 1 : 0;
        h.tile_idx = start / kTile;
        h.nt = m.nt;
        h.wu = wu;
        h.beta = beta;
        h.o_lr = o_lr;
        h.o_cu = o_cu;
        h.o_a0 = o_a0;
        h.o_a1 = o_a1;
        h.o_aw = o_aw;
        h.o_z = o_z;
        h.o_p = o_p;
        h.A0 = A0;
        h.A1 = A1;
        h.Aw = Aw;
        h.z = z;
        h.pold = pold;
        h.pnew = (it & 1) ? p0 : p1;
        h.q = m.q;
        h.part = m.part;
        h.st = m.st;
        h.it = it;
    }
    // lane 0 holds nt, q, part and st of its own tile only: broadcast them
    // above when src != 0
    const int s_pq = __shfl_sync(FULLM, m.s_pq, src);
    if (lane == 0)
        h.s_pq = s_pq;
    if (src != 0)
    {
        const int nt = __shfl_sync(FULLM, m.nt, src);
        float4 *q = shfl_ptr(m.q, src);
        double *part = shfl_ptr(m.part, src);
        InstState *st = shfl_ptr(m.st, src);
        if (lane == 0)
        {
            h.nt = nt;
            h.q = q;
            h.part = part;
            h.st = st;
        }
    }
    const unsigned tx = ri_bytes + unsigned(wl) * pb +
                        unsigned(wu) * (pb + 4u * pb + 2u * pb + (skew ? 4u * pb : 0u)) + halo;
    if (lane == 0)
        mbar_arrive_expect_tx(bar, tx);
    __syncwarp();
    const int *rowinfo = shfl_ptr(m.rowinfo, src), *colu = shfl_ptr(m.colu, src);
    const uint32_t *lref = shfl_ptr(m.lref, src);
    // one copy per array: a tile's planes are contiguous (tile-major)
    const size_t tl = size_t(start / kTile);
    const int ncopy = 5 + (skew ? 1 : 0) + (nh ? (two ? 2 : 1) : 0);
    for (int c = lane; c < ncopy; c += 32)
    {
        const int k = (c >= 5 && !skew) ? c + 1 : c; // 5: Aw, 6: z, 7: p_old
        switch (k)
        {
        case 0:
            bulk_g2s(stage, rowinfo + start, ri_bytes, bar);
            break;
        case 1:
            if (wl)
                bulk_g2s(stage + o_lr, lref + tl * wl * kTile, unsigned(wl) * pb, bar);
            break;
        case 2:
            bulk_g2s(stage + o_cu, colu + tl * wu * kTile, unsigned(wu) * pb, bar);
            break;
        case 3:
            bulk_g2s(stage + o_a0, A0 + tl * wu * kTile, unsigned(wu) * 4u * pb, bar);
            break;
        case 4:
            bulk_g2s(stage + o_a1, A1 + tl * wu * kTile, unsigned(wu) * 2u * pb, bar);
            break;
        case 5:
            bulk_g2s(stage + o_aw, Aw + tl * wu * kTile, unsigned(wu) * 4u * pb, bar);
            break;
        case 6:
            bulk_g2s(stage + o_z, z + hx, unsigned(nh) * 16u, bar);
            break;
        default:
            bulk_g2s(stage + o_p, pold + hx, unsigned(nh) * 16u, bar);
            break;
        }
    }
}

// What a consumer thread needs of a stage, copied from its header into
// registers once per tile (the header sits in shared memory, and stores
// through generic pointers would otherwise force it to be re-read).
struct BulkRegs
{
    int start, h0;
    float beta;
    bool skew;
    const unsigned char *stage;
    int wu;
    unsigned o_lr, o_cu, o_a0, o_a1, o_aw, o_z;
    const float4 *A0;
    const float2 *A1;
    const float4 *Aw;
    const float4 *z, *pold;
    float4 *pnew, *q;
};

__device__ __forceinline__ BulkRegs bulk_regs(const BulkHdr &h, const unsigned char *stage)
{
    BulkRegs r;
    r.start = h.start;
    r.h0 = h.h0;
    r.beta = h.beta;
    r.skew = h.skew != 0;
    r.stage = stage;
    r.wu = h.wu;
    r.o_lr = h.o_lr;
    r.o_cu = h.o_cu;
    r.o_a0 = h.o_a0;
    r.o_a1 = h.o_a1;
    r.o_aw = h.o_aw;
    r.o_z = h.o_z;
    r.A0 = h.A0;
    r.A1 = h.A1;
    r.Aw = h.Aw;
    r.z = h.z;
    r.pold = h.pold;
    r.pnew = h.pnew;
    r.q = h.q;
    return r;
}

// The lower slots' transposed blocks of one row, gathered from global memory
// (L2) before the stage's p is formed, so that their latency overlaps the
// halo pass: the first PF lower slots.
template <bool SKEW>
struct BulkLower
{
    static constexpr int PF = 6;
    float4 a0[PF];
    float2 a1[PF];
    float4 aw[SKEW ? PF : 1];
    uint32_t ref[PF];
};

template <bool SKEW>
__device__ __forceinline__ void bulk_lower_issue(const BulkHdr &h, const unsigned char *stage,
                                                 int t, int ds, BulkLower<SKEW> &L)
{
    const uint32_t *__restrict__ lr = reinterpret_cast<const uint32_t *>(stage + h.o_lr) + t;
    const bool sk = SKEW && h.skew;
    const int wu = h.wu;
    const float4 *__restrict__ A0 = h.A0;
    const float2 *__restrict__ A1 = h.A1;
#pragma unroll
    for (int k = 0; k < BulkLower<SKEW>::PF; k++)
        if (k < ds)
        {
            const uint32_t ref = lr[k * kTile];
            const uint32_t o = lref_block(ref, wu);
            L.ref[k] = ref;
            L.a0[k] = __ldcg(A0 + o);
            L.a1[k] = __ldcg(A1 + o);
            if (sk)
                L.aw[k] = __ldcg(h.Aw + o);
        }
}

// One row of q = A p from a filled stage (thread t = row start + t, `info`
// its row info, L its first lower slots' blocks); returns p.q.  STAGED: p over
// the tile's column range is in the stage (formed there); otherwise
// p = z + beta p_old is gathered from global memory at each column.  The sum
// runs in the one order of every SpMV: lower slots in column order, then the
// diagonal and upper slots.
template <bool SKEW, bool STAGED>
__device__ __forceinline__ float bulk_row(const BulkRegs &r, int t, int info,
                                          const BulkLower<SKEW> &L)
{
    constexpr int CH = 4; // lower slots past the prefetched ones: gathers in flight together
    const unsigned char *__restrict__ stage = r.stage;
    const int row = r.start + t;
    const int len = info & 255, ds = (info >> 8) & 255;
    const float4 *__restrict__ P = reinterpret_cast<const float4 *>(stage + r.o_z);
    const float beta = r.beta;
    auto pcol = [&](int c) -> float3 {
        if (STAGED)
            return xyz(P[c - r.h0]);
        float3 pc = xyz(__ldg(r.z + c));
        if (beta != 0.f)
            pc = pform(pc, beta, xyz(__ldg(r.pold + c)));
        return pc;
    };
    const float3 pv = pcol(row);
    const bool sk = SKEW && r.skew;
    const int *__restrict__ cu = reinterpret_cast<const int *>(stage + r.o_cu) + t;
    const float4 *__restrict__ a0s = reinterpret_cast<const float4 *>(stage + r.o_a0) + t;
    const float2 *__restrict__ a1s = reinterpret_cast<const float2 *>(stage + r.o_a1) + t;
    const float4 *__restrict__ aws = reinterpret_cast<const float4 *>(stage + r.o_aw) + t;
    const int nu = len - ds;
    float3 q = make_float3(0.f, 0.f, 0.f);
    // lower slots, column order: the prefetched transposed blocks ...
#pragma unroll
    for (int k = 0; k < BulkLower<SKEW>::PF; k++)
        if (k < ds)
        {
            const float3 pc = pcol(lref_col(L.ref[k]));
            const float A[6] = {L.a0[k].x, L.a0[k].y, L.a0[k].z, L.a0[k].w, L.a1[k].x, L.a1[k].y};
            q = q + symv(A, pc);
            if (sk)
                q = q - skewv(L.aw[SKEW ? k : 0], pc);
        }
    // ... and any further ones, gathered here (L2)
    const uint32_t *__restrict__ lr = reinterpret_cast<const uint32_t *>(stage + r.o_lr) + t;
#pragma unroll 1
    for (int s0 = BulkLower<SKEW>::PF; s0 < ds; s0 += CH)
    {
        float4 a0[CH], aw[CH];
        float2 a1[CH];
        float3 pc[CH];
#pragma unroll
        for (int k = 0; k < CH; k++)
            if (s0 + k < ds)
            {
                const uint32_t ref = lr[(s0 + k) * kTile];
                const uint32_t o = lref_block(ref, r.wu);
                a0[k] = __ldcg(r.A0 + o);
                a1[k] = __ldcg(r.A1 + o);
                if (sk)
                    aw[k] = __ldcg(r.Aw + o);
                pc[k] = pcol(lref_col(ref));
            }
#pragma unroll
        for (int k = 0; k < CH; k++)
            if (s0 + k < ds)
            {
                const float A[6] = {a0[k].x, a0[k].y, a0[k].z, a0[k].w, a1[k].x, a1[k].y};
                q = q + symv(A, pc[k]);
                if (sk)
                    q = q - skewv(aw[k], pc[k]);
            }
    }
    // diagonal and upper slots in slot order (all staged), software-pipelined:
    // the next slot's column is read while this slot's product is formed
    int cn = nu > 0 ? cu[0] : 0;
#pragma unroll 1
    for (int u = 0; u < nu; u++)
    {
        const int c = cn;
        if (u + 1 < nu)
            cn = cu[(u + 1) * kTile];
        const float4 a0 = a0s[u * kTile];
        const float2 a1 = a1s[u * kTile];
        const float3 pc = pcol(c);
        const float A[6] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y};
        q = q + symv(A, pc);
        if (sk)
            q = q + skewv(aws[u * kTile], pc);
    }
    r.pnew[row] = f4(pv);
    r.q[row] = f4(q);
    return fdot(pv, q);
}

} // namespace

// Block: kTile consumer threads (one row each) and one producer warp.  The
// producer walks the block's tiles (blockIdx.x, + gridDim.x, ...), waits for a
// stage to be released (empty barrier: one arrival per consumer warp), and
// fills it (full barrier: its arrival plus the copies' bytes); a done
// instance's tile is announced with go = 0 and no copies.  Consumers sync
// among themselves on named barrier 1 (the producer never joins it).
namespace {
__device__ __forceinline__ void consumer_sync()
{
    asm volatile("bar.sync 1, %0;" ::"n"(kTile) : "memory");
}
__device__ __forceinline__ bool consumer_all(bool v)
{
    unsigned r;
    asm volatile("{\n\t.reg .pred p, q;\n\t"
                 "setp.ne.u32 p, %1, 0;\n\t"
                 "bar.red.and.pred q, 1, %2, p;\n\t"
                 "selp.u32 %0, 1, 0, q;\n\t}"
                 : "=r"(r)
                 : "r"(v ? 1u : 0u), "n"(kTile)
                 : "memory");
    return r != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > kBulkWaitNs)
            return false;
    return true;
}
} // namespace

template <int NST, bool SKEW, bool HALO>
__global__ void __launch_bounds__(kBulkThreads, SKEW ? 1 : 2) k_spmv_bulk(InstDesc *const *descs,
                                                            const Tile *tiles, BatchCtl *ctl,
                                                            int use_cond,
                                                            cudaGraphConditionalHandle hcond)
{
    extern __shared__ __align__(128) unsigned char bulk_smem[];
    __shared__ __align__(8) uint64_t full[NST], empty[NST];
    __shared__ BulkHdr hdr[NST];
    // the p.q of a stage's tile per consumer warp; the producer turns them
    // into the instance's fixed-point total when it takes the stage back
    __shared__ float wsumf[NST][kTile / 32];
    const unsigned stage_bytes = (dynamic_smem_bytes() / NST) & ~127u;
    const int ntiles = ctl->n_tiles_rows;
    const int G = gridDim.x;
    const int nmine = int(blockIdx.x) < ntiles ? (ntiles - 1 - int(blockIdx.x)) / G + 1 : 0;
    const int tid = threadIdx.x;
    if (tid == 0)
    {
        for (int k = 0; k < NST; k++)
        {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], kTile / 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid >= kTile)
    {
        // ---- producer warp: lane k resolves tile j + k's metadata for 32
        // tiles at a time; tiles of instances that are done are skipped
        // without a stage; the lanes share each tile's copies; after the last
        // tile a header with go = -1 tells the consumers to stop
        const int lane = tid - kTile;
        BulkMeta m;
        int used = 0; // stages filled so far
        auto acquire = [&](int stg) -> bool {
            if (used < NST)
                return true;
            const bool ok = mbar_wait_bounded(&empty[stg], ((used / NST) - 1) & 1);
            return __all_sync(0xffffffffu, ok);
        };
        // the released stage's tile p.q into its instance's team-sum buffer,
        // in two halves around the stage's refill (so the refill does not
        // wait): grab reads the tile's consumer-warp sums and its header
        // before they are overwritten, send (lane k converts warp k's FP32
        // sum to fixed-point limbs, tile_fx_add's arithmetic; the limbs are
        // added exactly; lane 0 sends one reduction per limb) runs after
        struct Grab
        {
            int go, it, s;
            InstState *st;
            float v;
        };
        auto grab = [&](int stg) -> Grab {
            const BulkHdr &o = hdr[stg];
            Grab g{o.go, o.it, o.s_pq, o.st, 0.f};
            if (lane < kTile / 32)
                g.v = wsumf[stg][lane];
            __syncwarp();
            return g;
        };
        auto send = [&](const Grab &g) {
            if (g.go != 1)
                return;
            constexpr unsigned M4 = (1u << (kTile / 32)) - 1u;
            if (lane < kTile / 32)
            {
                long long hh;
                unsigned long long ll;
                fx_split(g.v, g.s, hh, ll);
                float c = g.v;
#pragma unroll
                for (int k = (kTile / 32) / 2; k > 0; k >>= 1)
                {
                    hh += __shfl_xor_sync(M4, hh, k);
                    ll += __shfl_xor_sync(M4, ll, k);
                    c += __shfl_xor_sync(M4, c, k);
                }
                if (lane == 0)
                {
                    const int bq = g.it % 3;
                    atomicAdd(&g.st->acc[bq][0][0], (unsigned long long)hh);
                    atomicAdd(&g.st->acc[bq][0][1], ll);
                    atomicAdd(&g.st->acc_chk[bq][0], c);
                }
            }
            __syncwarp();
        };
        auto flush = [&](int stg) { send(grab(stg)); };
        for (int j = 0; j < nmine; j++)
        {
            if ((j & 31) == 0)
            {
                m.go = 0;
                if (j + lane < nmine)
                    bulk_meta(tiles, blockIdx.x + (j + lane) * G, m);
            }
            if (!__shfl_sync(0xffffffffu, m.go, j & 31))
                continue;
            const int stg = used % NST;
            if (!acquire(stg))
                return; // consumers stuck: they give up on their own bounded waits
            Grab g{0, 0, 0, nullptr, 0.f};
            if (used >= NST)
                g = grab(stg);
            bulk_issue_warp<SKEW, HALO>(m, j & 31, hdr[stg], bulk_smem + stg * stage_bytes,
                                        stage_bytes, &full[stg], lane);
            send(g);
            used++;
        }
        const int stg = used % NST;
        if (!acquire(stg))
            return;
        if (used >= NST)
            flush(stg);
        if (lane == 0)
        {
            hdr[stg].go = -1;
            mbar_arrive(&full[stg]);
        }
        __syncwarp();
        // the other stages' last tiles: fill f = used - NST + k went to stage
        // f % NST, and its release completes phase f / NST of that stage's
        // empty barrier
        for (int k = 1; k < NST; k++)
        {
            const int f = used - NST + k;
            if (f < 0)
                continue;
            const bool ok = __all_sync(0xffffffffu,
                                       mbar_wait_bounded(&empty[f % NST], (f / NST) & 1));
            if (!ok)
            {
                if (lane == 0)
                    atomicExch(&ctl->err, 1);
                return;
            }
            flush(f % NST);
        }
        return;
    }
    // ---- consumers: one row per thread, one stage after the other until
    // the producer's end marker
    const int lane = tid & 31, warp = tid >> 5;
    for (int j = 0;; j++)
    {
        const int stg = j % NST;
        unsigned char *stage = bulk_smem + stg * stage_bytes;
        const bool got = mbar_wait_bounded(&full[stg], (j / NST) & 1);
        if (!consumer_all(got))
        {
            // the stage never completed: record it for the launch set (the
            // host reports the solve as timed out) and stop
            if (tid == 0)
                atomicExch(&ctl->err, 1);
            return;
        }
        if (hdr[stg].go < 0)
            break;
        const BulkHdr &hd = hdr[stg];
        if (hd.go)
        {
            const bool act = tid < hd.nrows;
            const int info = act ? reinterpret_cast<const int *>(stage)[tid] : 0;
            // the lower slots' gathers go out first, ahead of the halo pass
            BulkLower<SKEW> L;
            if (act)
                bulk_lower_issue<SKEW>(hd, stage, tid, (info >> 8) & 255, L);
            if (hd.nh && hd.beta != 0.f)
            {
                // p = z + beta p_old over the halo, in place of z
                float4 *Z = reinterpret_cast<float4 *>(stage + hd.o_z);
                const float4 *Po = reinterpret_cast<const float4 *>(stage + hd.o_p);
                for (int k = tid; k < hd.nh; k += kTile)
                    Z[k] = f4(pform(xyz(Z[k]), hd.beta, xyz(Po[k])));
                consumer_sync();
            }
            float pq = 0.f;
            if (act)
            {
                const BulkRegs r = bulk_regs(hd, stage);
                pq = hd.nh ? bulk_row<SKEW, true>(r, tid, info, L)
                           : bulk_row<SKEW, false>(r, tid, info, L);
            }
            // the tile's p.q: FP32 sums of its 32-row groups (one per consumer
            // warp), which the producer adds to the instance's fixed-point
            // total when it takes the stage back
            const float t = warp_sum(pq);
            if (lane == 0)
                wsumf[stg][warp] = t;
            // generic writes to the stage (the halo's p) are ordered before
            // the copy engine refills it
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            consumer_sync();
            if (lane == 0)
                mbar_arrive(&empty[stg]);
        }
        else
        {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            consumer_sync();
            if (lane == 0)
                mbar_arrive(&empty[stg]);
        }
    }
}

// Instance totals of a graph-loop half-iteration (k_reduce_pq, k_reduce_rz),
// one thread per instance of the list: the exact fixed-point totals the tiles
// added (decoded at the scales the tiles used: the previous p.q, the current
// r.z and r.r, as the persistent kernels take them), then the scalar step.
// KIND 0 (after the SpMV): p.q -> alpha, or the end of the solve when p.q is
// zero or not finite.  KIND 1 (after the update): r.z, r.r -> beta, the
// iteration count and the convergence test; the next iteration's buffer
// (last used two iterations ago) is cleared.
namespace {
__device__ __forceinline__ double loop_total(const InstState *st, int bq, int q, int s,
                                             int *bad)
{
    const double v = fx_value(__ldcg(&st->acc[bq][q][0]), __ldcg(&st->acc[bq][q][1]), s);
    const float chk = __ldcg(&st->acc_chk[bq][q]);
    if (!isfinite(chk) || fabs(v - double(chk)) > 1e-3 * fabs(double(chk)) + 1e-30)
        *bad = 1;
    return v;
}

template <int KIND>
__device__ __forceinline__ void reduce_body(InstDesc *const *descs, const int *inst_list,
                                            int ninst, const int *ninst_dev, BatchCtl *ctl,
                                            int use_cond, cudaGraphConditionalHandle h)
{
    if (ninst_dev)
        ninst = *ninst_dev;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < ninst;
         b += gridDim.x * blockDim.x)
    {
        const InstDesc *dp = descs[inst_list[b]];
        InstState *stp = ldg_ptr(&dp->st);
        if (!__ldcg(&stp->active))
            continue;
        InstState &st = *stp;
        const int it0 = st.iter;
        const int bq = it0 % 3;
        int bad = 0;
        if (KIND == 0)
        {
            const double pq = loop_total(stp, bq, 0, fx_scale(st.pq), &bad);
            st.pq = pq;
            if (bad || !isfinite(pq))
            {
                st.status = 6;
                st.active = 0;
                retire(ctl, use_cond, h);
            }
            else if (pq == 0.0)
            {
                // PCGSolver.cu:259-263 clamps alpha to zero; nothing moves
                // afterwards, so the loop ends here. (p.Ap < 0 goes on with a
                // negative alpha, as the reference does.)
                st.status = 7;
                st.active = 0;
                retire(ctl, use_cond, h);
            }
            else
                st.alpha = st.rho / pq;
        }
        else
        {
            const double rho0 = st.rho;
            const double rho_new = loop_total(stp, bq, 1, fx_scale(rho0), &bad);
            const double rr = loop_total(stp, bq, 2, fx_scale(st.rr), &bad);
            const int nb = (it0 + 1) % 3;
            for (int q = 0; q < 3; q++)
            {
                st.acc[nb][q][0] = 0ull;
                st.acc[nb][q][1] = 0ull;
                st.acc_chk[nb][q] = 0.f;
            }
            st.beta = (rho0 == 0.0) ? 0.0 : rho_new / rho0;
            st.rho = rho_new;
            st.rr = rr;
            const int n = it0 + 1;
            st.iter = n;
            bool stop = false;
            if (bad || !isfinite(rho_new) || !isfinite(rr))
            {
                st.status = 6;
                stop = true;
            }
            else
            {
                const int check_every = __ldg(&dp->check_every);
                const int max_iters = __ldg(&dp->max_iters);
                const double rel_tol2 = __ldg(&dp->rel_tol2), abs_tol2 = __ldg(&dp->abs_tol2);
                const bool check = ((n - 1) % check_every) == 0 || n >= max_iters;
                const bool conv = (rel_tol2 > 0.0 && rr <= rel_tol2 * st.bb) ||
                                  (abs_tol2 > 0.0 && rr <= abs_tol2);
                if (check && conv)
                {
                    st.status = 0;
                    stop = true;
                }
                else if (n >= max_iters)
                {
                    st.status = 8; // CLOTH_ERR_MAXITER
                    stop = true;
                }
            }
            if (stop)
            {
                st.active = 0;
                retire(ctl, use_cond, h);
            }
        }
    }
}
} // namespace

__global__ void __launch_bounds__(kTile)
    k_reduce_pq(InstDesc *const *descs, const int *inst_list, int ninst, const int *ninst_dev,
                BatchCtl *ctl, int use_cond, cudaGraphConditionalHandle h)
{
    reduce_body<0>(descs, inst_list, ninst, ninst_dev, ctl, use_cond, h);
}

__global__ void __launch_bounds__(kTile)
    k_reduce_rz(InstDesc *const *descs, const int *inst_list, int ninst, const int *ninst_dev,
                BatchCtl *ctl, int use_cond, cudaGraphConditionalHandle h)
{
    reduce_body<1>(descs, inst_list, ninst, ninst_dev, ctl, use_cond, h);
}

// Variant table of the graph-loop kernels (the autotuner's search space).
#define SPMV_VARIANTS(SK)                                                                     \
    {1, 1, 1, (const void *)k_spmv_t<1, 1, 1, SK>}, {1, 2, 1, (const void *)k_spmv_t<1, 2, 1, SK>}, \
    {1, 3, 1, (const void *)k_spmv_t<1, 3, 1, SK>}, {2, 1, 1, (const void *)k_spmv_t<2, 1, 1, SK>}, \
    {2, 2, 1, (const void *)k_spmv_t<2, 2, 1, SK>}, {4, 1, 1, (const void *)k_spmv_t<4, 1, 1, SK>}, \
    {1, 1, 4, (const void *)k_spmv_t<1, 1, 4, SK>}, {1, 2, 4, (const void *)k_spmv_t<1, 2, 4, SK>}, \
    {2, 1, 4, (const void *)k_spmv_t<2, 1, 4, SK>}, {2, 2, 4, (const void *)k_spmv_t<2, 2, 4, SK>}, \
    {4, 1, 4, (const void *)k_spmv_t<4, 1, 4, SK>}, {2, 1, 8, (const void *)k_spmv_t<2, 1, 8, SK>}, \
    {1, 0, 2, (const void *)k_spmv_bulk<2, SK, true>, 2, 1},                                  \
    {1, 0, 3, (const void *)k_spmv_bulk<3, SK, true>, 3, 1},                                  \
    {0, 0, 2, (const void *)k_spmv_bulk<2, SK, false>, 2, 0},                                 \
    {0, 0, 3, (const void *)k_spmv_bulk<3, SK, false>, 3, 0},                                 \
    {0, 0, 4, (const void *)k_spmv_bulk<4, SK, false>, 4, 0}
extern const GraphLoopVariant kSpmvVariants[] = {SPMV_VARIANTS(false)};
// the same variants for launch sets holding a dihedral-bending instance
extern const GraphLoopVariant kSpmvSkewVariants[] = {SPMV_VARIANTS(true)};
#undef SPMV_VARIANTS
extern const GraphLoopVariant kUpdateVariants[] = {
    {1, 0, 1, (const void *)k_update_t<1, 1>}, {2, 0, 1, (const void *)k_update_t<2, 1>},
    {4, 0, 1, (const void *)k_update_t<4, 1>}, {1, 0, 4, (const void *)k_update_t<1, 4>},
    {2, 0, 4, (const void *)k_update_t<2, 4>}, {1, 0, 8, (const void *)k_update_t<1, 8>},
    {2, 0, 8, (const void *)k_update_t<2, 8>},
};
extern const int kNumSpmvVariants = 17;
extern const int kNumUpdateVariants = 7;
static_assert(sizeof(kSpmvVariants) / sizeof(kSpmvVariants[0]) == 17, "variant count");
static_assert(sizeof(kSpmvSkewVariants) / sizeof(kSpmvSkewVariants[0]) == 17, "variant count");
static_assert(sizeof(kUpdateVariants) / sizeof(kUpdateVariants[0]) == 7, "variant count");

// Copies of the PCG state the autotuner disturbs (dx, r, z per row, the
// instance scalars), so that timing k_update candidates leaves no trace.
__global__ void __launch_bounds__(kTile) k_snap_rows(InstDesc *const *descs, const Tile *tiles,
                                                     const BatchCtl *ctl, float4 *buf,
                                                     int restore)
{
    const int ntiles = ctl->n_tiles_rows;
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x)
    {
        const Tile tl = tiles[ti];
        const InstDesc &d = *descs[tl.inst];
        const int row = tl.start + threadIdx.x;
        if (row >= d.nv)
            continue;
        float4 *b = buf + 3 * (size_t(ti) * kTile + threadIdx.x);
        if (restore)
        {
            d.dx[row] = b[0];
            d.r[row] = b[1];
            d.z[row] = b[2];
        }
        else
        {
            b[0] = d.dx[row];
            b[1] = d.r[row];
            b[2] = d.z[row];
        }
    }
}

__global__ void k_snap_state(InstDesc *const *descs, const int *inst, int ninst,
                             InstState *buf, BatchCtl *ctl, BatchCtl *ctl_buf, int restore)
{
    constexpr int W = int(sizeof(InstState) / sizeof(unsigned));
    for (int i = blockIdx.x; i < ninst; i += gridDim.x)
    {
        unsigned *a = reinterpret_cast<unsigned *>(descs[inst[i]]->st);
        unsigned *b = reinterpret_cast<unsigned *>(buf + i);
        for (int k = threadIdx.x; k < W; k += blockDim.x)
        {
            if (restore)
                a[k] = b[k];
            else
                b[k] = a[k];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        if (restore)
            *ctl = *ctl_buf;
        else
            *ctl_buf = *ctl;
    }
}

// ------------------------------------------------------------------ persistent PCG
// One cooperative launch runs every PCG iteration of every instance in the
// launch set.  Each block owns a contiguous row range of one instance; the
// instance's blocks (its team) meet at two barriers per iteration, after
// which every block sums the team's per-block partials in the same fixed
// order, so all of them derive bit-identical alpha, beta and stop decisions
// without a third synchronisation.  Data written by other blocks inside the
// kernel (z, p, partials) is read through L2 (ld.global.cg); A is read-only.
namespace {

// Barrier of the nblk blocks of one team: one thread per block arrives with
// an acquire-release atomic (its release covers the writes the block's CTA
// barrier ordered before it) and polls the generation word with acquire
// loads. Returns false when the bounded wait gave up; the team's error flag
// is set then and the solve stops.
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *a, unsigned v)
{
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.u32 %0, [%1], %2;" : "=r"(old) : "l"(a), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void red_add_release(unsigned *a, unsigned v)
{
    asm volatile("red.add.release.gpu.u32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned *a)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
    return v;
}

__device__ __forceinline__ bool team_barrier(InstState *st, int nblk, const SpinCfg &sc)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        ok = 1;
        if (nblk > 1)
        {
            const unsigned g = ld_acquire(&st->bar_gen);
            if (atom_add_acq_rel(&st->bar_count, 1u) == unsigned(nblk - 1) + sc.extra)
            {
                st->bar_count = 0u;
                red_add_release(&st->bar_gen, 1u);
            }
            else
            {
                unsigned n = 0;
                while (ld_acquire(&st->bar_gen) == g)
                {
                    if (++n > sc.limit)
                    {
                        atomicExch(&st->bar_err, 1);
                        ok = 0;
                        break;
                    }
                    if (n > 256)
                        __nanosleep(32);
                }
            }
        }
    }
    __syncthreads();
    return ok != 0;
}

// Barrier of the two-barrier persistent kernels: a monotonic arrival count
// per team (zeroed before every launch); barrier k of a launch waits for
// k * nblk arrivals. One thread per block arrives with a release reduction
// (it covers the writes the CTA barrier ordered before it, the partial sums
// included) and polls with acquire loads; no thread waits for its own
// arrival to return. Returns false when the bounded wait gave up (the team's
// error flag is set then).
__device__ __forceinline__ bool team_barrier_count(unsigned long long *count,
                                                   unsigned long long target, InstState *st,
                                                   int nblk, const SpinCfg &sc)
{
    target += sc.extra;
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        ok = 1;
        if (nblk > 1)
        {
            asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(count) : "memory");
            unsigned n = 0;
            for (;;)
            {
                unsigned long long v;
                asm volatile("ld.acquire.gpu.global.u64 %0, [%1];"
                             : "=l"(v)
                             : "l"(count)
                             : "memory");
                if (v >= target)
                    break;
                if (++n > sc.limit)
                {
                    atomicExch(&st->bar_err, 1);
                    ok = 0;
                    break;
                }
                if (n > 256)
                    __nanosleep(32);
            }
        }
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ float4 ldcg4(const float4 *p) { return __ldcg(p); }

// Loads of the matrix carry an L2 evict_last policy: A is re-read every PCG
// iteration and should outlive the streamed vectors in L2.
__device__ __forceinline__ unsigned long long l2_keep_policy()
{
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ float4 ld_keep(const float4 *ptr, unsigned long long pol)
{
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(ptr), "l"(pol));
    return v;
}
__device__ __forceinline__ float2 ld_keep(const float2 *ptr, unsigned long long pol)
{
    float2 v;
    asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
        : "=f"(v.x), "=f"(v.y)
        : "l"(ptr), "l"(pol));
    return v;
}
__device__ __forceinline__ int ld_keep(const int *ptr, unsigned long long pol)
{
    int v;
    asm("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(ptr), "l"(pol));
    return v;
}

} // namespace

namespace {

// Per-warp fixed-point accumulator of NQ chunk sums (held by lane 0).
template <int NQ> struct WarpFx
{
    long long H[NQ];
    unsigned long long L[NQ];
    float chk[NQ];
    __device__ __forceinline__ void clear()
    {
#pragma unroll
        for (int q = 0; q < NQ; q++)
        {
            H[q] = 0;
            L[q] = 0ull;
            chk[q] = 0.f;
        }
    }
    __device__ __forceinline__ void add(int q, float v, int s)
    {
        long long h;
        unsigned long long l;
        fx_split(v, s, h, l);
        H[q] += h;
        L[q] += l;
        chk[q] += v;
    }
};

} // namespace

// State of the block's own rows lives in shared memory (SM = true) or in
// global memory (SM = false, for row ranges too long for shared memory).
// SKEW: the launch set holds a dihedral-bending instance; skew block parts
// are read and applied where an instance has them.
template <bool SM, bool SKEW>
__device__ __forceinline__ void pcg_persistent_body(InstDesc *const *descs,
                                                    const TeamBlock *work, int halo_cap,
                                                    int rows_cap, SpinCfg sc)
{
    constexpr int NW = kPBlock / 32;
    extern __shared__ float4 sm_dyn[];
    __shared__ InstDesc d;
    // FP64 PCG scalars: owned by thread 0, the block reads the FP32 copies
    __shared__ double s_rho, s_beta, s_alpha, s_pq, s_rr;
    __shared__ float bc_af, bc_bf;
    __shared__ int bc_stop, bc_s[3];
    const TeamBlock w = work[blockIdx.x];
    if (w.inst < 0)
        return;
    if (threadIdx.x == 0)
        d = *descs[w.inst];
    __syncthreads();
    InstState *st = d.st;
    if (!__ldcg(&st->active))
        return;
    // dynamic shared memory: staged p, then the own-row state (SM only)
    float4 *sp = sm_dyn;
    float4 *sdx = sp + halo_cap;
    float4 *sr = sdx + rows_cap;
    float4 *sq = sr + rows_cap;
    float4 *sm0 = sq + rows_cap;
    float2 *sm1 = reinterpret_cast<float2 *>(sm0 + rows_cap);
    // FP32 sums of the 32-row chunks, one array per quantity (p.q, r.z, r.r):
    // kept in shared memory rather than in per-thread accumulators, which
    // leaves the SpMV loop its registers
    const int cps = (rows_cap + 31) / 32;
    float *cpart = reinterpret_cast<float *>(
        SM ? (kPersistMShared ? reinterpret_cast<float4 *>(sm1 + rows_cap) : sm0) : sdx);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned long long keep = l2_keep_policy();
    const int nrow = w.row1 - w.row0;
    const int nch = (nrow + 31) / 32;
    const bool staged = w.halo0 >= 0;
    if (SM)
        for (int i = tid; i < nrow; i += kPBlock)
        {
            const int row = w.row0 + i;
            sdx[i] = d.dx[row];
            sr[i] = d.r[row];
            if (kPersistMShared)
            {
                sm0[i] = d.M0[row];
                sm1[i] = d.M1[row];
            }
        }
    // the solve's state: at its start (PCG start bookkeeping: no iteration,
    // beta = 0, p.q estimate = r.z) or where a graph loop handed it over
    // (its iteration count, scalars and p_old in global memory)
    __shared__ int s_it0;
    if (tid == 0)
    {
        s_it0 = __ldcg(&st->iter);
        s_rho = __ldcg(&st->rho);
        s_rr = __ldcg(&st->rr);
        s_pq = __ldcg(&st->pq);
        s_beta = __ldcg(&st->beta);
        s_alpha = __ldcg(&st->alpha);
        bc_bf = float(s_beta);
    }
    __syncthreads();
    const int it0 = s_it0;
    int it = it0, status = 0;
    // the team's arrival count: after the work list, one word per block slot,
    // the team using its first block's
    __shared__ unsigned long long s_nbar; // arrivals barrier k waits for (thread 0)
    if (tid == 0)
        s_nbar = 0ull;
    auto team_count = [&]() {
        return reinterpret_cast<unsigned long long *>(const_cast<TeamBlock *>(work) + gridDim.x) +
               (blockIdx.x - w.rank);
    };

    // Team sum of nq quantities (q0.. of the chunk sums): warp q turns every
    // chunk sum of quantity q0 + q into fixed point (scale sc[q]) and folds
    // them (exact integer adds: any order gives the same limbs), its lane 0
    // sends one reduction per limb to the team buffer, then the team barrier.
    // Returns false when the barrier gave up.
    auto team_sum = [&](int nq, int q0, int bq, int sc0, int sc1) -> bool {
        __syncthreads();
        if (warp < nq)
        {
            const int q = warp;
            const int sq = q == 0 ? sc0 : sc1;
            {
                unsigned long long h = 0ull, l = 0ull;
                float c = 0.f;
                for (int ch = lane; ch < nch; ch += 32)
                {
                    const float v = cpart[(q0 + q) * cps + ch];
                    long long hh;
                    unsigned long long ll;
                    fx_split(v, sq, hh, ll);
                    h += (unsigned long long)hh;
                    l += ll;
                    c += v;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                {
                    h += __shfl_xor_sync(0xffffffffu, h, o);
                    l += __shfl_xor_sync(0xffffffffu, l, o);
                    c += __shfl_xor_sync(0xffffffffu, c, o);
                }
                if (lane == 0)
                {
                    atomicAdd(&st->acc[bq][q0 + q][0], h);
                    atomicAdd(&st->acc[bq][q0 + q][1], l);
                    atomicAdd(&st->acc_chk[bq][q0 + q], c);
                }
            }
        }
        if (tid == 0)
            s_nbar += (unsigned long long)w.nblk;
        return team_barrier_count(team_count(), s_nbar, st, w.nblk, sc);
    };
    // Reads a team sum after the barrier; flags a fixed-point overflow when it
    // disagrees with the FP32 magnitude check.
    auto team_value = [&](int q, int bq, int s, int *bad) -> double {
        const double v = fx_value(__ldcg(&st->acc[bq][q][0]), __ldcg(&st->acc[bq][q][1]), s);
        const float chk = __ldcg(&st->acc_chk[bq][q]);
        if (!isfinite(chk) || fabs(v - double(chk)) > 1e-3 * fabs(double(chk)) + 1e-30)
            *bad = 1;
        return v;
    };

    for (;;)
    {
        const int bq = it % 3;
        const float4 *pold = (it & 1) ? d.p1 : d.p0;
        float4 *pnew = (it & 1) ? d.p0 : d.p1;
        __syncthreads();
        const float bf = bc_bf;
        const bool first = (bf == 0.f);
        if (tid == 0)
        {
            // scales of this iteration, identical in every block of the team
            bc_s[0] = fx_scale(s_pq);
            bc_s[1] = fx_scale(s_rho);
            bc_s[2] = fx_scale(s_rr);
            if (w.rank == 0)
            {
                // the buffer of iteration it+1 was last read in iteration it-2
                const int nb = (it + 1) % 3;
                for (int q = 0; q < 3; q++)
                {
                    st->acc[nb][q][0] = 0ull;
                    st->acc[nb][q][1] = 0ull;
                    st->acc_chk[nb][q] = 0.f;
                }
            }
        }
        // ---- p = z + beta p_old over the staged range. The staged p of the
        // last iteration is still in shared memory (every block computes p of
        // a row with the same operation on the same values as its owner), so
        // only z is read; kStageUnroll rows per thread have their loads in
        // flight together.
        if (staged)
        {
            const int nh = w.halo1 - w.halo0;
            // (the skew kernels, one more plane in the SpMV, have no registers
            // for a second row)
            constexpr int SU = SKEW ? 1 : kStageUnroll;
            for (int i0 = tid; i0 < nh; i0 += SU * kPBlock)
            {
                float4 zz[SU];
#pragma unroll
                for (int u = 0; u < SU; u++)
                    if (i0 + u * kPBlock < nh)
                        zz[u] = ldcg4(d.z + w.halo0 + i0 + u * kPBlock);
#pragma unroll
                for (int u = 0; u < SU; u++)
                {
                    const int i = i0 + u * kPBlock;
                    if (i < nh)
                    {
                        float4 pn = zz[u];
                        if (!first)
                        {
                            // the previous p: staged by the last iteration,
                            // or in global memory on the first one after a
                            // hand-over
                            const float4 po = (it == it0 && it0 > 0)
                                                  ? ldcg4(pold + w.halo0 + i)
                                                  : sp[i];
                            pn.x = fmaf(bf, po.x, pn.x);
                            pn.y = fmaf(bf, po.y, pn.y);
                            pn.z = fmaf(bf, po.z, pn.z);
                        }
                        sp[i] = pn;
                    }
                }
            }
        }
        __syncthreads();
        const int s0q = bc_s[0], s1q = bc_s[1], s2q = bc_s[2];
        // ---- q = A p on own rows; p.q per 32-row chunk
        for (int ch = warp; ch < nch; ch += NW)
        {
            const int li = ch * 32 + lane;
            const int row = w.row0 + li;
            float part = 0.f;
            if (li < nrow)
            {
                float3 pv;
                if (staged)
                    pv = xyz(sp[row - w.halo0]);
                else
                {
                    const float4 zz = ldcg4(d.z + row);
                    pv = xyz(zz);
                    if (!first)
                    {
                        const float4 po = ldcg4(pold + row);
                        pv = make_float3(fmaf(bf, po.x, zz.x), fmaf(bf, po.y, zz.y),
                                         fmaf(bf, po.z, zz.z));
                    }
                }
                if (!staged || w.p_global)
                    pnew[row] = f4(pv);
                const int info = ld_keep(d.rowinfo + row, keep);
                const int len = info & 255, ds = (info >> 8) & 255;
                float3 q = make_float3(0, 0, 0);
                // Slots in column order: the lower ones by s (block at the
                // transposed position), then the diagonal and upper ones by
                // plane u. Step k covers lower plane k for k < wl and upper
                // plane k - wl after, so every load instruction of a warp reads
                // one plane (wl, the instance's lower plane count, is uniform).
                // kSlotUnroll steps' loads are in flight together.
                const int wl = d.width_lo, kend = wl + (len - ds);
                for (int k0 = 0; k0 < kend; k0 += kSlotUnroll)
                {
                    int cc[kSlotUnroll];
                    float4 a0[kSlotUnroll];
                    float2 a1[kSlotUnroll];
                    float4 aw[kSlotUnroll];
                    bool on[kSlotUnroll];
#pragma unroll
                    for (int k = 0; k < kSlotUnroll; k++)
                    {
                        const int kk = k0 + k;
                        const bool lower = kk < wl;
                        on[k] = lower ? kk < ds : kk < kend;
                        if (on[k])
                        {
                            uint32_t oa;
                            if (lower)
                            {
                                const uint32_t ref = uint32_t(ld_keep(
                                    reinterpret_cast<const int *>(d.lref) + lo_idx(kk, row, wl),
                                    keep));
                                cc[k] = lref_col(ref);
                                oa = lref_block(ref, d.width_up);
                            }
                            else
                            {
                                oa = up_idx(kk - wl, row, d.width_up);
                                cc[k] = ld_keep(d.colu + oa, keep);
                            }
                            a0[k] = ld_keep(d.A0 + oa, keep);
                            a1[k] = ld_keep(d.A1 + oa, keep);
                            if (SKEW && d.Aw)
                                aw[k] = ld_keep(d.Aw + oa, keep);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < kSlotUnroll; k++)
                        if (on[k])
                        {
                            const int c = cc[k];
                            const float A[6] = {a0[k].x, a0[k].y, a0[k].z, a0[k].w,
                                                a1[k].x, a1[k].y};
                            float3 pc;
                            if (staged)
                                pc = xyz(sp[c - w.halo0]);
                            else if (c == row)
                                pc = pv;
                            else
                            {
                                const float4 zz = ldcg4(d.z + c);
                                pc = xyz(zz);
                                if (!first)
                                {
                                    const float4 po = ldcg4(pold + c);
                                    pc = make_float3(fmaf(bf, po.x, zz.x),
                                                     fmaf(bf, po.y, zz.y),
                                                     fmaf(bf, po.z, zz.z));
                                }
                            }
                            q = q + symv(A, pc);
                            if (SKEW && d.Aw)
                            {
                                const float3 cw = skewv(aw[k], pc);
                                q = (k0 + k < wl) ? q - cw : q + cw;
                            }
                        }
                }
                if (SM)
                    sq[li] = f4(q);
                else
                    d.q[row] = f4(q);
                part = fdot(pv, q);
            }
            part = warp_sum(part);
            if (lane == 0)
                cpart[ch] = part;
        }
        if (!team_sum(1, 0, bq, s0q, s0q))
        {
            status = 9; // CLOTH_ERR_TIMEOUT
            break;
        }
        if (tid == 0)
        {
            int bad = 0;
            const double pq = team_value(0, bq, s0q, &bad);
            s_pq = pq;
            int stop = 0;
            if (bad || !isfinite(pq))
                stop = 6;
            else if (pq == 0.0)
                stop = 7;
            else
                s_alpha = s_rho / pq;
            bc_af = float(s_alpha);
            bc_stop = stop;
        }
        __syncthreads();
        if (bc_stop)
        {
            status = bc_stop;
            break;
        }
        const float af = bc_af;
        // ---- dx += alpha p, r -= alpha q, z = M^-1 r; r.z and r.r per chunk
        for (int ch = warp; ch < nch; ch += NW)
        {
            const int li = ch * 32 + lane;
            const int row = w.row0 + li;
            float pr = 0.f, prr = 0.f;
            if (li < nrow)
            {
                const float3 p = staged ? xyz(sp[row - w.halo0]) : xyz(pnew[row]);
                const float3 qv = SM ? xyz(sq[li]) : xyz(d.q[row]);
                float3 x = SM ? xyz(sdx[li]) : xyz(d.dx[row]);
                float3 r = SM ? xyz(sr[li]) : xyz(d.r[row]);
                x = make_float3(fmaf(af, p.x, x.x), fmaf(af, p.y, x.y), fmaf(af, p.z, x.z));
                r = make_float3(fmaf(-af, qv.x, r.x), fmaf(-af, qv.y, r.y),
                                fmaf(-af, qv.z, r.z));
                float M[6];
                if (SM && kPersistMShared)
                {
                    const float4 u = sm0[li];
                    const float2 v = sm1[li];
                    M[0] = u.x;
                    M[1] = u.y;
                    M[2] = u.z;
                    M[3] = u.w;
                    M[4] = v.x;
                    M[5] = v.y;
                }
                else
                    load_sym(d.M0, d.M1, row, M);
                const float3 z = symv(M, r);
                if (SM)
                {
                    sdx[li] = f4(x);
                    sr[li] = f4(r);
                }
                else
                {
                    d.dx[row] = f4(x);
                    d.r[row] = f4(r);
                }
                d.z[row] = f4(z);
                pr = fdot(r, z);
                prr = fdot(r, r);
            }
            pr = warp_sum(pr);
            prr = warp_sum(prr);
            if (lane == 0)
            {
                cpart[cps + ch] = pr;
                cpart[2 * cps + ch] = prr;
            }
        }
        if (!team_sum(2, 1, bq, s1q, s2q))
        {
            status = 9;
            break;
        }
        it++;
        if (tid == 0)
        {
            int bad = 0;
            const double rho_new = team_value(1, bq, s1q, &bad);
            const double rr = team_value(2, bq, s2q, &bad);
            s_beta = (s_rho == 0.0) ? 0.0 : rho_new / s_rho;
            s_rho = rho_new;
            s_rr = rr;
            int stop = 0; // 0 go on, 1 converged, else a status code
            if (bad || !isfinite(rho_new) || !isfinite(rr))
                stop = 6;
            else
            {
                const bool check = ((it - 1) % d.check_every) == 0 || it >= d.max_iters;
                if (check && test_converged(d, *st, rr))
                    stop = 1;
                else if (it >= d.max_iters)
                    stop = 8;
            }
            bc_bf = float(s_beta);
            bc_stop = stop;
        }
        __syncthreads();
        const int stop = bc_stop;
        if (stop)
        {
            status = (stop == 1) ? 0 : stop;
            break;
        }
    }
    if (SM)
    {
        __syncthreads();
        for (int i = tid; i < nrow; i += kPBlock)
        {
            const int row = w.row0 + i;
            d.dx[row] = sdx[i];
            d.r[row] = sr[i];
        }
    }
    if (w.rank == 0 && tid == 0)
    {
        st->iter = it;
        st->status = status;
        st->rho = s_rho;
        st->rr = s_rr;
        st->pq = s_pq;
        st->alpha = s_alpha;
        st->beta = s_beta;
        st->active = 0;
    }
}

__global__ void __launch_bounds__(kPBlock, 1)
    k_pcg_persistent_sm(InstDesc *const *descs, const TeamBlock *work, int halo_cap,
                        int rows_cap, SpinCfg sc)
{
    pcg_persistent_body<true, false>(descs, work, halo_cap, rows_cap, sc);
}

__global__ void __launch_bounds__(kPBlock, 1)
    k_pcg_persistent_gm(InstDesc *const *descs, const TeamBlock *work, int halo_cap,
                        int rows_cap, SpinCfg sc)
{
    pcg_persistent_body<false, false>(descs, work, halo_cap, rows_cap, sc);
}

// launch sets holding a dihedral-bending instance
__global__ void __launch_bounds__(kPBlock, 1)
    k_pcg_persistent_sm_skew(InstDesc *const *descs, const TeamBlock *work, int halo_cap,
                             int rows_cap, SpinCfg sc)
{
    pcg_persistent_body<true, true>(descs, work, halo_cap, rows_cap, sc);
}

__global__ void __launch_bounds__(kPBlock, 1)
    k_pcg_persistent_gm_skew(InstDesc *const *descs, const TeamBlock *work, int halo_cap,
                             int rows_cap, SpinCfg sc)
{
    pcg_persistent_body<false, true>(descs, work, halo_cap, rows_cap, sc);
}

// ------------------------------------------------------------------ single-barrier persistent PCG
// The same block-Jacobi PCG in the Chronopoulos-Gear arrangement: with
// u = M^-1 r and w = A u, the scalars come from gamma = r.u, delta = w.u
// and r.r, all three summed at ONE team barrier per iteration:
//   beta = gamma / gamma_prev,  alpha = gamma / (delta - beta gamma / alpha_prev)
//   p = u + beta p,  s = w + beta s,  dx += alpha p,  r -= alpha s,
//   u = M^-1 r,  w = A u.
// The SpMV needs u over the block's halo.  A block recomputes u for the halo
// rows it does not own from the previous iteration's r, w and s, which their
// owners wrote to global memory before the barrier (two buffers each,
// alternating by iteration, so no row is overwritten while another block may
// still read it), with the same code the owners run, so the values agree bit
// for bit.  Requires the shared-memory plan with every block's halo staged.
// Team sums are the exact fixed-point sums of the two-barrier solver, so an
// instance's result does not depend on the launch set.
namespace {

// r_new = r - alpha (w + beta s) and s_new = w + beta s (s absent at the
// first iteration); the owner and every block staging the row run this.
__device__ __forceinline__ float3 cg1_residual(float3 r, float3 w, float3 s, float af,
                                               float bf, bool first, float3 &s_new)
{
    s_new = first ? w
                  : make_float3(fmaf(bf, s.x, w.x), fmaf(bf, s.y, w.y), fmaf(bf, s.z, w.z));
    return make_float3(fmaf(-af, s_new.x, r.x), fmaf(-af, s_new.y, r.y),
                       fmaf(-af, s_new.z, r.z));
}

} // namespace

__global__ void __launch_bounds__(kPBlock, 1)
    k_pcg1_persistent(InstDesc *const *descs, const TeamBlock *work, int halo_cap,
                      int rows_cap, SpinCfg sc)
{
    constexpr int NW = kPBlock / 32;
    extern __shared__ float4 sm_dyn[];
    __shared__ InstDesc d;
    __shared__ unsigned long long wsum_h[3][NW], wsum_l[3][NW];
    __shared__ float wsum_c[3][NW];
    // FP64 scalars: owned by thread 0, the block reads the FP32 copies
    __shared__ double s_gam, s_del, s_rr, s_alpha, s_beta;
    __shared__ float bc_af, bc_bf;
    __shared__ int bc_stop, bc_s[3];
    const TeamBlock w = work[blockIdx.x];
    if (w.inst < 0)
        return;
    if (threadIdx.x == 0)
        d = *descs[w.inst];
    __syncthreads();
    InstState *st = d.st;
    if (!__ldcg(&st->active))
        return;
    // dynamic shared memory: u over the halo, then own rows' dx, p, M^-1
    float4 *su = sm_dyn;
    float4 *sx = su + halo_cap;
    float4 *sp = sx + rows_cap;
    float4 *sm0 = sp + rows_cap;
    float2 *sm1 = reinterpret_cast<float2 *>(sm0 + rows_cap);
    float4 *const rb[2] = {d.r, d.z};
    float4 *const sb[2] = {d.p0, d.p1};
    float4 *const wb[2] = {d.q, d.w1};

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned long long keep = l2_keep_policy();
    const int nrow = w.row1 - w.row0;
    const int nch = (nrow + 31) / 32;
    const int h0 = w.halo0, nh = w.halo1 - w.halo0;
    for (int i = tid; i < nrow; i += kPBlock)
    {
        const int row = w.row0 + i;
        sx[i] = d.dx[row];
        sm0[i] = d.M0[row];
        sm1[i] = d.M1[row];
    }
    // u0 = z0 of the assembly over the halo
    for (int i = tid; i < nh; i += kPBlock)
        su[i] = ldcg4(d.z + h0 + i);
    if (tid == 0)
    {
        s_gam = __ldcg(&st->rho);
        s_rr = __ldcg(&st->rr);
        s_del = s_gam; // scale estimate for the first delta
        s_alpha = 0.0;
        s_beta = 0.0;
        bc_s[0] = fx_scale(s_gam);
        bc_s[1] = fx_scale(s_del);
        bc_s[2] = fx_scale(s_rr);
    }
    // (the three sum buffers start at zero: the PCG start cleared them)
    __syncthreads();

    auto team_sum = [&](WarpFx<3> &wfx, int bq) -> bool {
        if (lane == 0)
            for (int q = 0; q < 3; q++)
            {
                wsum_h[q][warp] = (unsigned long long)wfx.H[q];
                wsum_l[q][warp] = wfx.L[q];
                wsum_c[q][warp] = wfx.chk[q];
            }
        __syncthreads();
        if (tid == 0)
            for (int q = 0; q < 3; q++)
            {
                unsigned long long hh = 0ull, ll = 0ull;
                float c = 0.f;
                for (int j = 0; j < NW; j++)
                {
                    hh += wsum_h[q][j];
                    ll += wsum_l[q][j];
                    c += wsum_c[q][j];
                }
                atomicAdd(&st->acc[bq][q][0], hh);
                atomicAdd(&st->acc[bq][q][1], ll);
                atomicAdd(&st->acc_chk[bq][q], c);
            }
        return team_barrier(st, w.nblk, sc);
    };
    auto team_value = [&](int q, int bq, int s, int *bad) -> double {
        const double v = fx_value(__ldcg(&st->acc[bq][q][0]), __ldcg(&st->acc[bq][q][1]), s);
        const float chk = __ldcg(&st->acc_chk[bq][q]);
        if (!isfinite(chk) || fabs(v - double(chk)) > 1e-3 * fabs(double(chk)) + 1e-30)
            *bad = 1;
        return v;
    };
    // w = A u on an own row from the staged u; writes wbuf, returns w.u
    auto spmv_row = [&](int row, float3 uv, float4 *wbuf) -> float {
        const int info = ld_keep(d.rowinfo + row, keep);
        const int len = info & 255, ds = (info >> 8) & 255;
        const int wl = d.width_lo, kend = wl + (len - ds);
        float3 q = make_float3(0, 0, 0);
        for (int k0 = 0; k0 < kend; k0 += kSlotUnroll)
        {
            int cc[kSlotUnroll];
            float4 a0[kSlotUnroll];
            float2 a1[kSlotUnroll];
            bool on[kSlotUnroll];
#pragma unroll
            for (int k = 0; k < kSlotUnroll; k++)
            {
                const int kk = k0 + k;
                const bool lower = kk < wl;
                on[k] = lower ? kk < ds : kk < kend;
                if (on[k])
                {
                    uint32_t oa;
                    if (lower)
                    {
                        const uint32_t ref = uint32_t(ld_keep(
                            reinterpret_cast<const int *>(d.lref) + lo_idx(kk, row, wl), keep));
                        cc[k] = lref_col(ref);
                        oa = lref_block(ref, d.width_up);
                    }
                    else
                    {
                        oa = up_idx(kk - wl, row, d.width_up);
                        cc[k] = ld_keep(d.colu + oa, keep);
                    }
                    a0[k] = ld_keep(d.A0 + oa, keep);
                    a1[k] = ld_keep(d.A1 + oa, keep);
                }
            }
#pragma unroll
            for (int k = 0; k < kSlotUnroll; k++)
                if (on[k])
                {
                    const float A[6] = {a0[k].x, a0[k].y, a0[k].z, a0[k].w, a1[k].x, a1[k].y};
                    q = q + symv(A, xyz(su[cc[k] - h0]));
                }
        }
        wbuf[row] = f4(q);
        return fdot(q, uv);
    };

    int it = 0, status = 0, bq = 1;
    // ---- setup: w0 = A u0; gamma0 = r0.u0, delta0 = w0.u0, r0.r0
    {
        const int s0q = bc_s[0], s1q = bc_s[1], s2q = bc_s[2];
        WarpFx<3> f;
        f.clear();
        for (int ch = warp; ch < nch; ch += NW)
        {
            const int li = ch * 32 + lane;
            const int row = w.row0 + li;
            float pg = 0.f, pd = 0.f, pr = 0.f;
            if (li < nrow)
            {
                const float3 uv = xyz(su[row - h0]);
                const float3 rv = xyz(ldcg4(rb[0] + row));
                pd = spmv_row(row, uv, wb[0]);
                pg = fdot(rv, uv);
                pr = fdot(rv, rv);
            }
            pg = warp_sum(pg);
            pd = warp_sum(pd);
            pr = warp_sum(pr);
            if (lane == 0)
            {
                f.add(0, pg, s0q);
                f.add(1, pd, s1q);
                f.add(2, pr, s2q);
            }
        }
        if (!team_sum(f, bq))
            status = 9;
    }
    while (status == 0)
    {
        // ---- scalars from the sums of this iteration
        if (tid == 0)
        {
            int bad = 0;
            const double gam = team_value(0, bq, bc_s[0], &bad);
            const double del = team_value(1, bq, bc_s[1], &bad);
            const double rr = team_value(2, bq, bc_s[2], &bad);
            int stop = 0; // 0 go on, 1 converged, else a status code
            double beta = 0.0, alpha = s_alpha;
            if (bad || !isfinite(gam) || !isfinite(del) || !isfinite(rr))
                stop = 6;
            else if (it > 0)
            {
                const bool check = ((it - 1) % d.check_every) == 0 || it >= d.max_iters;
                if (check && test_converged(d, *st, rr))
                    stop = 1;
                else if (it >= d.max_iters)
                    stop = 8;
            }
            if (!stop)
            {
                beta = (it == 0 || s_gam == 0.0) ? 0.0 : gam / s_gam;
                const double den = (it == 0) ? del : del - beta * gam / s_alpha;
                if (den == 0.0)
                    stop = 7;
                else
                    alpha = gam / den;
            }
            s_gam = gam;
            s_del = del;
            s_rr = rr;
            s_beta = beta;
            s_alpha = alpha;
            bc_af = float(alpha);
            bc_bf = float(beta);
            bc_stop = stop;
            bc_s[0] = fx_scale(gam);
            bc_s[1] = fx_scale(del);
            bc_s[2] = fx_scale(rr);
            if (w.rank == 0)
            {
                // the buffer of the next sums was last read two iterations ago
                const int nb = (bq + 1) % 3;
                for (int q = 0; q < 3; q++)
                {
                    st->acc[nb][q][0] = 0ull;
                    st->acc[nb][q][1] = 0ull;
                    st->acc_chk[nb][q] = 0.f;
                }
            }
        }
        __syncthreads();
        if (bc_stop)
        {
            status = (bc_stop == 1) ? 0 : bc_stop;
            break;
        }
        const float af = bc_af, bf = bc_bf;
        const bool first = (it == 0);
        const int cur = it & 1, nxt = cur ^ 1;
        const int s0q = bc_s[0], s1q = bc_s[1], s2q = bc_s[2];
        WarpFx<3> f;
        f.clear();
        // ---- own rows: p, s, dx, r, u; gamma and r.r of the new r
        for (int ch = warp; ch < nch; ch += NW)
        {
            const int li = ch * 32 + lane;
            const int row = w.row0 + li;
            float pg = 0.f, pr = 0.f;
            if (li < nrow)
            {
                const float3 uv = xyz(su[row - h0]);
                const float3 wv = xyz(ldcg4(wb[cur] + row));
                const float3 sv = first ? make_float3(0, 0, 0) : xyz(ldcg4(sb[cur] + row));
                const float3 rv = xyz(ldcg4(rb[cur] + row));
                float3 pv = uv;
                if (!first)
                {
                    const float3 po = xyz(sp[li]);
                    pv = make_float3(fmaf(bf, po.x, uv.x), fmaf(bf, po.y, uv.y),
                                     fmaf(bf, po.z, uv.z));
                }
                float3 s_new;
                const float3 r_new = cg1_residual(rv, wv, sv, af, bf, first, s_new);
                float3 x = xyz(sx[li]);
                x = make_float3(fmaf(af, pv.x, x.x), fmaf(af, pv.y, x.y), fmaf(af, pv.z, x.z));
                const float4 m0 = sm0[li];
                const float2 m1 = sm1[li];
                const float M[6] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y};
                const float3 u_new = symv(M, r_new);
                sp[li] = f4(pv);
                sx[li] = f4(x);
                sb[nxt][row] = f4(s_new);
                rb[nxt][row] = f4(r_new);
                su[row - h0] = f4(u_new);
                pg = fdot(r_new, u_new);
                pr = fdot(r_new, r_new);
            }
            pg = warp_sum(pg);
            pr = warp_sum(pr);
            if (lane == 0)
            {
                f.add(0, pg, s0q);
                f.add(2, pr, s2q);
            }
        }
        // ---- halo rows owned by other blocks: the same u from their r, w, s
        for (int i = tid; i < nh; i += kPBlock)
        {
            const int row = h0 + i;
            if (row >= w.row0 && row < w.row1)
                continue;
            const float3 wv = xyz(ldcg4(wb[cur] + row));
            const float3 sv = first ? make_float3(0, 0, 0) : xyz(ldcg4(sb[cur] + row));
            const float3 rv = xyz(ldcg4(rb[cur] + row));
            float3 s_new;
            const float3 r_new = cg1_residual(rv, wv, sv, af, bf, first, s_new);
            float M[6];
            load_sym(d.M0, d.M1, row, M);
            su[i] = f4(symv(M, r_new));
        }
        __syncthreads();
        // ---- w = A u on own rows; delta = w.u
        for (int ch = warp; ch < nch; ch += NW)
        {
            const int li = ch * 32 + lane;
            const int row = w.row0 + li;
            float pd = 0.f;
            if (li < nrow)
                pd = spmv_row(row, xyz(su[row - h0]), wb[nxt]);
            pd = warp_sum(pd);
            if (lane == 0)
                f.add(1, pd, s1q);
        }
        bq = (bq + 1) % 3;
        it++;
        if (!team_sum(f, bq))
        {
            status = 9; // CLOTH_ERR_TIMEOUT
            break;
        }
    }
    // ---- own rows back to the standard buffers: dx, and r into d.r
    __syncthreads();
    for (int i = tid; i < nrow; i += kPBlock)
    {
        const int row = w.row0 + i;
        d.dx[row] = sx[i];
        if (it & 1)
            d.r[row] = ldcg4(rb[1] + row);
    }
    if (w.rank == 0 && tid == 0)
    {
        st->iter = it;
        st->status = status;
        st->rho = s_gam;
        st->rr = s_rr;
        st->pq = s_del;
        st->alpha = s_alpha;
        st->beta = s_beta;
        st->active = 0;
    }
}

// ------------------------------------------------------------------ advance
__global__ void __launch_bounds__(kTile) k_advance(InstDesc *const *descs,
                                                   const Tile *tiles,
                                                   const BatchCtl *ctl,
                                                   int finished_only)
{
    const int ntiles = ctl->n_tiles_rows;
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x)
    {
        const Tile tl = tiles[ti];
        const InstDesc &d = *descs[tl.inst];
        // finished_only: instances whose solve ended and whose step is still
        // open (the request server's tile list holds running ones too)
        if (finished_only && (d.st->active || !d.st->open))
            continue;
        // a solve that ended in NaN, breakdown or a timed-out wait leaves the
        // state as it was (the step driver may re-solve it in FP64), and so
        // does one that ended at max_iters in a step that escalates those
        const int status = d.st->status;
        if (status == 6 || status == 7 || status == 9 || (status == 8 && d.hold_maxiter))
            continue;
        const int row = tl.start + threadIdx.x;
        if (row >= d.nv)
            continue;
        const float4 dxv = d.dx[row];
        double x[3];
        double dd[3] = {double(dxv.x), double(dxv.y), double(dxv.z)};
        if (d.dxr)
        {
            // dx after the contacts' repulsion (FP64)
            dd[0] = d.dxr[3 * size_t(row)];
            dd[1] = d.dxr[3 * size_t(row) + 1];
            dd[2] = d.dxr[3 * size_t(row) + 2];
        }
#pragma unroll
        for (int k = 0; k < 3; k++)
        {
            const double xo = d.x64[3 * row + k];
            d.xp64[3 * row + k] = xo;
            x[k] = xo + dd[k];
            d.x64[3 * row + k] = x[k];
        }
        d.x32[row] = make_float4(float(x[0]), float(x[1]), float(x[2]), 0.f);
    }
}

// x32 from x64 after a host upload; clears the pin marks (k_pins sets them).
__global__ void k_sync_x32(InstDesc *d_ptr)
{
    const InstDesc &d = *d_ptr;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < d.nv;
         row += gridDim.x * blockDim.x)
        d.x32[row] = make_float4(float(d.x64[3 * row]), float(d.x64[3 * row + 1]),
                                 float(d.x64[3 * row + 2]), 0.f);
}

} // namespace cloth
