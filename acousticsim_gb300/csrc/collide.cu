// Collisions of a cloth with static kinematic bodies: the CPU cloth's contact
// handling (cSimScene::PerformCollisionDetection with cBVHCollisionDetecter,
// src/sim/collision/BVHCollisionDetecter.cpp; cBaraffCloth::
// PrepareCollisionHessian and Repulsion, src/sim/cloth/BaraffCloth.cpp:614-990)
// run on the device as part of a cloth's step.
//
// Per step, on the positions the step starts from (after the pins):
//   1. grown boxes (5 mm) and normals of the cloth triangles;
//   2. triangle pairs whose boxes meet (a uniform grid over each body's
//      triangles; every pair is reported by exactly one cell) - the leaf pairs
//      the reference's BVH walk reaches;
//   3. candidate lists sorted as the reference's std::sets sort them:
//      (cloth point, body triangle), (body point, cloth triangle) and
//      (cloth edge, body edge), each built per point / edge from the pairs of
//      its triangles, and the narrow phase (distance under 3 mm) in that order;
//   4. per-vertex lists of the contacts touching each cloth vertex.
// The row pass adds the contact Hessian (1e-2 dC/dx dC/dx^T per
// point-triangle contact) to the assembled blocks.  After the solve, the
// repulsion applies the contacts' impulses to dx in the reference's order
// (edge-edge contacts, then point-triangle ones, each reading dx as the earlier
// ones left it): a contact runs once every earlier contact on its vertices has
// run, so contacts on disjoint vertices run together and the result is the
// sequential one.  Every list has a capacity; a contact that does not fit is
// dropped and the step reports CLOTH_ERR_CONTACTS.
#include "internal.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>

using namespace cloth;
using namespace cloth::detail;

namespace {

constexpr int kColBlock = 256;
constexpr int kLocalCand = 128;  // candidates one point or edge may gather
constexpr int kRepBlock = 1024;

struct BodyView
{
    int nv, nt, ne;
    const double *pos;    // nv*3
    const int *tris;      // nt*3
    const int *tedge;     // nt*3: edges (v0 v1), (v1 v2), (v2 v0)
    const int *edges;     // ne*4: v0 v1 tri0 tri1 (-1: boundary)
    const double *tn;     // nt*3
    const double *vn;     // nv*3
    const double *blo, *bhi; // nt*3 grown boxes
    const int *vt_off, *vt; // vertex -> triangles
    const int *cell_off, *cell_tris;
    double g0[3];
    double cell;
    int gdim[3];
};

} // namespace

struct cloth_body_s
{
    cloth_ctx *ctx = nullptr;
    int nv = 0, nt = 0, ne = 0;
    char *mem = nullptr;
    size_t bytes = 0;
    BodyView v{};
    // host copies: the triangles and the normals the body's Init left (a
    // moving body keeps them, as cKinematicBody::Update does)
    std::vector<int> tris;
    std::vector<double> tn, vn;
    // time-driven motion (cloth_body_set_motion); unused for other bodies
    bool moving = false;
    std::vector<double> local;
    double ip[3] = {0, 0, 0}, io[3] = {0, 0, 0}, tp[3] = {0, 0, 0}, to[3] = {0, 0, 0};
    double elapsed = 0.0;
    float time = 0.f;
};

struct cloth_collide_s
{
    int cap_pairs = 0, cap_pt = 0, cap_ee = 0, cap_inc = 0;
    int max_bnt = 0, max_bnv = 0;
    char *mem = nullptr;
    size_t bytes = 0;
    double *ctlo = nullptr, *cthi = nullptr, *ctn = nullptr;
    int *tp_off = nullptr, *tp = nullptr;
    int *bt_off = nullptr, *bt_cur = nullptr, *bt = nullptr;
    int *lst = nullptr;      // per point / edge counts, then offsets
    PtContact *pt = nullptr;
    EeContact *ee = nullptr;
    int *inc_off = nullptr, *inc_cur = nullptr, *inc = nullptr;
    int *rptr = nullptr, *cstate = nullptr, *wa = nullptr, *wb = nullptr;
    int *tile_sum = nullptr;
    int4 *cverts = nullptr;   // cloth vertices of every contact (and their count)
    int4 *clpos = nullptr, *csucc = nullptr; // place in, and successor on, each vertex's list
    double *dxr = nullptr;
    CollideCounts *cnt = nullptr;
    int *vt_off = nullptr, *vt = nullptr; // cloth vertex -> triangles
    int *edges = nullptr;                 // ne*4 cloth edges
    double *mass64 = nullptr;             // nv vertex masses (FP64, as the repulsion uses them)
    int cap_request[3] = {0, 0, 0};       // pairs, point-triangle, edge-edge (0: default)
};

namespace {

// ------------------------------------------------------------------ helpers
struct V3
{
    double x, y, z;
};
__device__ __forceinline__ V3 ld3(const double *p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross3(V3 a, V3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ V3 nrm3(V3 a)
{
    const double n = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return {a.x / n, a.y / n, a.z / n};
}
__device__ __forceinline__ float clampf01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }

// ClosestPtPointTriangle (BVHCollisionDetecter.cpp:17-86), dot products
// rounded to float as the reference keeps them.
__device__ V3 closest_pt_tri(V3 p, V3 a, V3 b, V3 c, float *bary)
{
    const V3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
    bary[0] = bary[1] = bary[2] = 0.f;
    const float d1 = float(dot3(ab, ap)), d2 = float(dot3(ac, ap));
    if (d1 <= 0.0f && d2 <= 0.0f)
    {
        bary[0] = 1;
        return a;
    }
    const V3 bp = sub3(p, b);
    const float d3 = float(dot3(ab, bp)), d4 = float(dot3(ac, bp));
    if (d3 >= 0.0f && d4 <= d3)
    {
        bary[1] = 1;
        return b;
    }
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f)
    {
        const float v = d1 / (d1 - d3);
        bary[0] = 1 - v;
        bary[1] = v;
        return {a.x + double(v) * ab.x, a.y + double(v) * ab.y, a.z + double(v) * ab.z};
    }
    const V3 cp = sub3(p, c);
    const float d5 = float(dot3(ab, cp)), d6 = float(dot3(ac, cp));
    if (d6 >= 0.0f && d5 <= d6)
    {
        bary[2] = 1;
        return c;
    }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f)
    {
        const float w = d2 / (d2 - d6);
        bary[0] = 1 - w;
        bary[2] = w;
        return {a.x + double(w) * ac.x, a.y + double(w) * ac.y, a.z + double(w) * ac.z};
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
    {
        const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary[1] = 1 - w;
        bary[2] = w;
        const V3 cb = sub3(c, b);
        return {b.x + double(w) * cb.x, b.y + double(w) * cb.y, b.z + double(w) * cb.z};
    }
    const float denom = 1.0f / (va + vb + vc);
    const float v = vb * denom, w = vc * denom;
    bary[0] = 1 - v - w;
    bary[1] = v;
    bary[2] = w;
    return {a.x + ab.x * double(v) + ac.x * double(w), a.y + ab.y * double(v) + ac.y * double(w),
            a.z + ab.z * double(v) + ac.z * double(w)};
}

// EdgeEdgeDist (BVHCollisionDetecter.cpp:100-175): Ericson's closest points of
// two segments with float scalars.
__device__ void edge_edge(V3 p1, V3 q1, V3 p2, V3 q2, float &s, float &t)
{
    const V3 d1 = sub3(q1, p1), d2 = sub3(q2, p2), r = sub3(p1, p2);
    const float a = float(dot3(d1, d1)), e = float(dot3(d2, d2)), f = float(dot3(d2, r));
    const float EPS = 1e-10f;
    s = 0.f;
    t = 0.f;
    if (a <= EPS)
    {
        s = 0.0f;
        t = clampf01(f / e);
    }
    else
    {
        const float c = float(dot3(d1, r));
        if (e <= EPS)
        {
            t = 0.0f;
            s = clampf01(-c / a);
        }
        else
        {
            const float b = float(dot3(d1, d2));
            const float denom = a * e - b * b;
            s = denom != 0.0f ? clampf01((b * f - c * e) / denom) : 0.0f;
            t = (b * s + f) / e;
            if (t < 0.0f)
            {
                t = 0.0f;
                s = clampf01(-c / a);
            }
            else if (t > 1.0f)
            {
                t = 1.0f;
                s = clampf01((b - c) / a);
            }
        }
    }
}

__device__ __forceinline__ bool boxes_meet(const double *al, const double *ah, const double *bl,
                                           const double *bh)
{
    return al[0] <= bh[0] && ah[0] >= bl[0] && al[1] <= bh[1] && ah[1] >= bl[1] &&
           al[2] <= bh[2] && ah[2] >= bl[2];
}

__device__ __forceinline__ int cell_of(const BodyView &b, double v, int k)
{
    const double q = floor((v - b.g0[k]) / b.cell);
    return q < 0.0 ? 0 : (q >= double(b.gdim[k]) ? b.gdim[k] - 1 : int(q));
}

// sorted unique insert into a bounded local list; false when full
__device__ __forceinline__ bool insert_sorted(int *a, int &n, int v)
{
    int k = n;
    while (k > 0 && a[k - 1] > v)
        k--;
    if (k > 0 && a[k - 1] == v)
        return true;
    if (n >= kLocalCand)
        return false;
    for (int j = n; j > k; j--)
        a[j] = a[j - 1];
    a[k] = v;
    n++;
    return true;
}

// ------------------------------------------------------------------ kernels
__global__ void k_col_begin(CollideCounts *cnt, int cap_inc)
{
    if (threadIdx.x == 0)
    {
        *cnt = CollideCounts{};
        cnt->cap_inc = cap_inc;
    }
}

// 1. grown boxes and normals of the cloth triangles (cObjBVH::UpdateAABB,
//    cBaseObject::UpdateTriangleNormal)
__global__ void k_col_tri_boxes(int nt, const int4 *tri, const double *x, double *lo, double *hi,
                                double *tn)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x)
    {
        const int4 v = tri[t];
        const V3 a = ld3(x + 3 * size_t(v.x)), b = ld3(x + 3 * size_t(v.y)),
                 c = ld3(x + 3 * size_t(v.z));
        const double av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z}, cv[3] = {c.x, c.y, c.z};
        for (int k = 0; k < 3; k++)
        {
            const double mn = fmin(fmin(av[k], bv[k]), cv[k]);
            const double mx = fmax(fmax(av[k], bv[k]), cv[k]);
            lo[3 * size_t(t) + k] = mn - 5e-3;
            hi[3 * size_t(t) + k] = mx + 5e-3;
        }
        const V3 n = nrm3(cross3(sub3(b, a), sub3(c, b)));
        tn[3 * size_t(t) + 0] = n.x;
        tn[3 * size_t(t) + 1] = n.y;
        tn[3 * size_t(t) + 2] = n.z;
    }
}

// 2. body triangles whose boxes meet cloth triangle T's.  fill = 0 counts
//    into off[T]; fill = 1 writes them at off[T] (exclusive offsets) sorted.
__global__ void k_col_pairs(BodyView b, int nt, const double *lo, const double *hi, int *off,
                            int *tp, int cap, int fill, CollideCounts *cnt)
{
    for (int T = blockIdx.x * blockDim.x + threadIdx.x; T < nt; T += gridDim.x * blockDim.x)
    {
        const double *al = lo + 3 * size_t(T), *ah = hi + 3 * size_t(T);
        int i0[3], i1[3];
        bool outside = false;
        for (int k = 0; k < 3; k++)
        {
            const double gmax = b.g0[k] + b.cell * b.gdim[k];
            if (ah[k] < b.g0[k] || al[k] > gmax)
                outside = true;
            i0[k] = cell_of(b, al[k], k);
            i1[k] = cell_of(b, ah[k], k);
        }
        int n = 0;
        const int base = fill ? off[T] : 0;
        if (!outside)
            for (int iz = i0[2]; iz <= i1[2]; iz++)
                for (int iy = i0[1]; iy <= i1[1]; iy++)
                    for (int ix = i0[0]; ix <= i1[0]; ix++)
                    {
                        const int cell = (iz * b.gdim[1] + iy) * b.gdim[0] + ix;
                        for (int k = b.cell_off[cell]; k < b.cell_off[cell + 1]; k++)
                        {
                            const int t = b.cell_tris[k];
                            const double *bl = b.blo + 3 * size_t(t), *bh = b.bhi + 3 * size_t(t);
                            if (!boxes_meet(al, ah, bl, bh))
                                continue;
                            // the pair belongs to the cell of its overlap's low corner
                            if (cell_of(b, fmax(al[0], bl[0]), 0) != ix ||
                                cell_of(b, fmax(al[1], bl[1]), 1) != iy ||
                                cell_of(b, fmax(al[2], bl[2]), 2) != iz)
                                continue;
                            if (fill)
                            {
                                if (base + n < cap)
                                    tp[base + n] = t;
                                else
                                    atomicExch(&cnt->overflow, 1);
                            }
                            n++;
                        }
                    }
        if (!fill)
            off[T] = n;
        else
        {
            // ascending body triangle ids
            const int m = min(n, max(0, cap - base));
            for (int i = 1; i < m; i++)
            {
                const int v = tp[base + i];
                int j = i;
                while (j > 0 && tp[base + j - 1] > v)
                {
                    tp[base + j] = tp[base + j - 1];
                    j--;
                }
                tp[base + j] = v;
            }
        }
    }
}

// Exclusive scan of a[0..n) in place, a[n] = total, *total = total: blocks
// of kScanTile elements scan their tiles and leave their sums; one block
// scans the sums; the blocks add their tile's offset.
constexpr int kScanTile = 4096;
constexpr int kScanMaxTiles = 4096; // n up to 16 M

__global__ void __launch_bounds__(1024) k_col_scan_tiles(int *a, int n, int *tile_sum)
{
    __shared__ int part[1024];
    const int base = blockIdx.x * kScanTile, tid = threadIdx.x;
    const int i0 = min(n, base + tid * 4), i1 = min(n, i0 + 4);
    int v[4] = {0, 0, 0, 0}, s = 0;
    for (int i = i0; i < i1; i++)
    {
        v[i - i0] = a[i];
        s += v[i - i0];
    }
    part[tid] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        const int u = tid >= o ? part[tid - o] : 0;
        __syncthreads();
        part[tid] += u;
        __syncthreads();
    }
    int run = part[tid] - s;
    for (int i = i0; i < i1; i++)
    {
        a[i] = run;
        run += v[i - i0];
    }
    if (tid == 1023)
        tile_sum[blockIdx.x] = part[1023];
}

__global__ void __launch_bounds__(1024) k_col_scan_top(int *tile_sum, int ntiles, int *a, int n,
                                                       int *total)
{
    __shared__ int part[1024];
    const int tid = threadIdx.x;
    const int per = (ntiles + 1023) / 1024;
    const int t0 = min(ntiles, tid * per), t1 = min(ntiles, t0 + per);
    int s = 0;
    for (int t = t0; t < t1; t++)
        s += tile_sum[t];
    part[tid] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        const int u = tid >= o ? part[tid - o] : 0;
        __syncthreads();
        part[tid] += u;
        __syncthreads();
    }
    int run = part[tid] - s;
    for (int t = t0; t < t1; t++)
    {
        const int v = tile_sum[t];
        tile_sum[t] = run;
        run += v;
    }
    if (tid == 1023)
    {
        a[n] = part[1023];
        if (total)
            *total = part[1023];
    }
}

__global__ void k_col_scan_add(int *a, int n, const int *tile_sum)
{
    const int off = tile_sum[blockIdx.x];
    const int base = blockIdx.x * kScanTile;
    if (off)
        for (int i = base + threadIdx.x; i < min(n, base + kScanTile); i += blockDim.x)
            a[i] += off;
}

// pairs grouped by body triangle: counts, then ids at atomic cursors, then
// each group sorted by cloth triangle
__global__ void k_col_bt_count(int nt, const int *tp_off, const int *tp, int cap, int *bt_off)
{
    for (int T = blockIdx.x * blockDim.x + threadIdx.x; T < nt; T += gridDim.x * blockDim.x)
        for (int k = tp_off[T]; k < min(tp_off[T + 1], cap); k++)
            atomicAdd(&bt_off[tp[k]], 1);
}
__global__ void k_col_bt_fill(int nt, const int *tp_off, const int *tp, int cap, const int *bt_off,
                              int *bt_cur, int *bt)
{
    for (int T = blockIdx.x * blockDim.x + threadIdx.x; T < nt; T += gridDim.x * blockDim.x)
        for (int k = tp_off[T]; k < min(tp_off[T + 1], cap); k++)
        {
            const int t = tp[k];
            const int pos = bt_off[t] + atomicAdd(&bt_cur[t], 1);
            if (pos < cap)
                bt[pos] = T;
        }
}
// Ascending unique values of a union of sorted segments [b_i, e_i) of one
// array (a k-way merge; no copy of the candidates is kept).
constexpr int kMaxLists = 64;
struct MergeIter
{
    const int *a;
    int cur[kMaxLists], end[kMaxLists];
    int n;
    __device__ void init(const int *arr)
    {
        a = arr;
        n = 0;
    }
    __device__ bool add(int b, int e)
    {
        if (b >= e)
            return true;
        if (n >= kMaxLists)
            return false;
        cur[n] = b;
        end[n] = e;
        n++;
        return true;
    }
    __device__ bool next(int &v)
    {
        int m = INT_MAX;
        for (int i = 0; i < n; i++)
            if (cur[i] < end[i] && a[cur[i]] < m)
                m = a[cur[i]];
        if (m == INT_MAX)
            return false;
        for (int i = 0; i < n; i++)
            while (cur[i] < end[i] && a[cur[i]] == m)
                cur[i]++;
        v = m;
        return true;
    }
};

constexpr int kSortCap = 8192;   // candidates a block sorts in shared memory
constexpr int kSortBlock = 256;

// ascending bitonic sort of s[0..P) (P a power of two) by one block
__device__ void block_bitonic(int *s, int P)
{
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1)
        {
            for (int i = threadIdx.x; i < P; i += blockDim.x)
            {
                const int ixj = i ^ j;
                if (ixj > i)
                {
                    const bool up = (i & k) == 0;
                    const int a = s[i], b = s[ixj];
                    if ((a > b) == up)
                    {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
}

// each body triangle's list of cloth triangles, ascending: one block per
// list, sorted in shared memory (by one thread beyond kSortCap)
__global__ void __launch_bounds__(kSortBlock) k_col_bt_sort(int bnt, const int *bt_off, int *bt,
                                                            int cap)
{
    __shared__ int sv[kSortCap];
    for (int t = blockIdx.x; t < bnt; t += gridDim.x)
    {
        const int b0 = min(bt_off[t], cap), b1 = min(bt_off[t + 1], cap);
        const int n = b1 - b0;
        if (n <= 1)
            continue;
        if (n <= kSortCap)
        {
            int P = 1;
            while (P < n)
                P <<= 1;
            for (int i = threadIdx.x; i < P; i += blockDim.x)
                sv[i] = i < n ? bt[b0 + i] : INT_MAX;
            __syncthreads();
            block_bitonic(sv, P);
            for (int i = threadIdx.x; i < n; i += blockDim.x)
                bt[b0 + i] = sv[i];
            __syncthreads();
        }
        else if (threadIdx.x == 0)
            for (int i = b0 + 1; i < b1; i++)
            {
                const int v = bt[i];
                int j = i;
                while (j > b0 && bt[j - 1] > v)
                {
                    bt[j] = bt[j - 1];
                    j--;
                }
                bt[j] = v;
            }
        __syncthreads();
    }
}

// 3a. cloth point p against body triangles (BVHCollisionDetecter.cpp:420-500,
//     obj0 = cloth).  write = 0 counts into cntv[p]; write = 1 stores the
//     contacts at cnt->n_pt + cntv[p] (exclusive offsets).
__global__ void k_col_pt_cloth(BodyView b, int nv, const double *x, const int *vt_off,
                               const int *vt, const int *tp_off, const int *tp, int cap_pairs,
                               int *cntv, PtContact *out, int cap, int write, CollideCounts *cnt)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nv; p += gridDim.x * blockDim.x)
    {
        MergeIter it;
        it.init(tp);
        bool ok = true;
        for (int k = vt_off[p]; k < vt_off[p + 1]; k++)
        {
            const int T = vt[k];
            ok &= it.add(min(tp_off[T], cap_pairs), min(tp_off[T + 1], cap_pairs));
        }
        if (!ok)
            atomicExch(&cnt->overflow, 1);
        const V3 pt = ld3(x + 3 * size_t(p));
        int n = 0;
        const int base = write ? cnt->n_pt + cntv[p] : 0;
        int t;
        while (it.next(t))
        {
            const int *tv = b.tris + 3 * size_t(t);
            float bary[3];
            const V3 q = closest_pt_tri(pt, ld3(b.pos + 3 * size_t(tv[0])),
                                        ld3(b.pos + 3 * size_t(tv[1])),
                                        ld3(b.pos + 3 * size_t(tv[2])), bary);
            const V3 nn = ld3(b.tn + 3 * size_t(t));
            const V3 dv = sub3(pt, q);
            if (!(sqrt(dot3(dv, dv)) < 3e-3))
                continue;
            if (write)
            {
                if (base + n < cap)
                {
                    PtContact c;
                    c.cloth_point = 1;
                    c.p = p;
                    c.t = t;
                    c.depth = float(dot3(dv, nn));
                    c.n[0] = nn.x;
                    c.n[1] = nn.y;
                    c.n[2] = nn.z;
                    c.bary[0] = bary[0];
                    c.bary[1] = bary[1];
                    c.bary[2] = bary[2];
                    c.pad = 0;
                    out[base + n] = c;
                }
                else
                    atomicExch(&cnt->overflow, 1);
            }
            n++;
        }
        if (!write)
            cntv[p] = n;
    }
}

// 3b. body point q against cloth triangles (obj0 = body): the cloth
//     triangle's normal, turned to the body point's normal side.
__device__ __forceinline__ bool pt_body_hit(const BodyView &b, const double *x, const int4 *tri,
                                            const double *ctn, int q, int T, PtContact *o)
{
    const V3 pt = ld3(b.pos + 3 * size_t(q));
    const int4 tv = tri[T];
    float bary[3];
    const V3 c = closest_pt_tri(pt, ld3(x + 3 * size_t(tv.x)), ld3(x + 3 * size_t(tv.y)),
                                ld3(x + 3 * size_t(tv.z)), bary);
    V3 nn = ld3(ctn + 3 * size_t(T));
    if (dot3(nn, ld3(b.vn + 3 * size_t(q))) < 0)
        nn = {-nn.x, -nn.y, -nn.z};
    const V3 dv = sub3(c, pt);
    if (!(sqrt(dot3(dv, dv)) < 3e-3))
        return false;
    if (o)
    {
        o->cloth_point = 0;
        o->p = q;
        o->t = T;
        o->depth = float(dot3(dv, nn));
        o->n[0] = nn.x;
        o->n[1] = nn.y;
        o->n[2] = nn.z;
        o->bary[0] = bary[0];
        o->bary[1] = bary[1];
        o->bary[2] = bary[2];
        o->pad = 0;
    }
    return true;
}

// One block per body point: its candidate cloth triangles (the union of its
// triangles' sorted lists) sorted in shared memory; each thread takes a
// contiguous run of the sorted candidates, so a block prefix sum over the
// threads' hit counts gives every contact its place in the detecter's
// order.  Beyond kSortCap candidates one thread merges the lists instead.
__global__ void __launch_bounds__(kSortBlock) k_col_pt_body(
    BodyView b, const double *x, const int4 *tri, const double *ctn, const int *bt_off,
    const int *bt, int cap_pairs, int *cntv, PtContact *out, int cap, int write,
    CollideCounts *cnt)
{
    __shared__ int sv[kSortCap];
    __shared__ int s_part[kSortBlock];
    __shared__ int s_n;
    for (int q = blockIdx.x; q < b.nv; q += gridDim.x)
    {
        if (threadIdx.x == 0)
        {
            int n = 0;
            for (int k = b.vt_off[q]; k < b.vt_off[q + 1]; k++)
            {
                const int t = b.vt[k];
                n += min(bt_off[t + 1], cap_pairs) - min(bt_off[t], cap_pairs);
            }
            s_n = n;
        }
        __syncthreads();
        const int n = s_n;
        const int base = write ? cnt->n_pt + cntv[q] : 0;
        if (n > kSortCap)
        {
            // serial merge of the lists
            if (threadIdx.x == 0)
            {
                MergeIter it;
                it.init(bt);
                bool ok = true;
                for (int k = b.vt_off[q]; k < b.vt_off[q + 1]; k++)
                {
                    const int t = b.vt[k];
                    ok &= it.add(min(bt_off[t], cap_pairs), min(bt_off[t + 1], cap_pairs));
                }
                if (!ok)
                    atomicExch(&cnt->overflow, 1);
                int h = 0, T;
                while (it.next(T))
                {
                    PtContact o;
                    if (!pt_body_hit(b, x, tri, ctn, q, T, write ? &o : nullptr))
                        continue;
                    if (write)
                    {
                        if (base + h < cap)
                            out[base + h] = o;
                        else
                            atomicExch(&cnt->overflow, 1);
                    }
                    h++;
                }
                if (!write)
                    cntv[q] = h;
            }
            __syncthreads();
            continue;
        }
        if (n == 0)
        {
            if (!write && threadIdx.x == 0)
                cntv[q] = 0;
            __syncthreads();
            continue;
        }
        int P = 1;
        while (P < n)
            P <<= 1;
        // gather the lists: list k starts at s_part[k] of the candidates
        const int nl = b.vt_off[q + 1] - b.vt_off[q];
        if (threadIdx.x == 0)
        {
            int o = 0;
            for (int k = 0; k < nl && k < kSortBlock; k++)
            {
                const int t = b.vt[b.vt_off[q] + k];
                s_part[k] = o;
                o += min(bt_off[t + 1], cap_pairs) - min(bt_off[t], cap_pairs);
            }
        }
        __syncthreads();
        if (nl <= kSortBlock)
            for (int k = 0; k < nl; k++)
            {
                const int t = b.vt[b.vt_off[q] + k];
                const int b0 = min(bt_off[t], cap_pairs), b1 = min(bt_off[t + 1], cap_pairs);
                for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x)
                    sv[s_part[k] + (i - b0)] = bt[i];
            }
        else if (threadIdx.x == 0)
        {
            int o = 0;
            for (int k = b.vt_off[q]; k < b.vt_off[q + 1]; k++)
            {
                const int t = b.vt[k];
                for (int i = min(bt_off[t], cap_pairs); i < min(bt_off[t + 1], cap_pairs); i++)
                    sv[o++] = bt[i];
            }
        }
        for (int i = n + threadIdx.x; i < P; i += blockDim.x)
            sv[i] = INT_MAX;
        __syncthreads();
        block_bitonic(sv, P);
        // contiguous runs of the sorted candidates, duplicates skipped
        const int per = (n + blockDim.x - 1) / blockDim.x;
        const int i0 = min(n, int(threadIdx.x) * per), i1 = min(n, i0 + per);
        int h = 0;
        for (int i = i0; i < i1; i++)
            if ((i == 0 || sv[i] != sv[i - 1]) && pt_body_hit(b, x, tri, ctn, q, sv[i], nullptr))
                h++;
        s_part[threadIdx.x] = h;
        __syncthreads();
        for (int o = 1; o < int(blockDim.x); o <<= 1)
        {
            const int v = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0;
            __syncthreads();
            s_part[threadIdx.x] += v;
            __syncthreads();
        }
        if (write)
        {
            int pos = base + s_part[threadIdx.x] - h;
            for (int i = i0; i < i1; i++)
            {
                PtContact o;
                if ((i == 0 || sv[i] != sv[i - 1]) && pt_body_hit(b, x, tri, ctn, q, sv[i], &o))
                {
                    if (pos < cap)
                        out[pos] = o;
                    else
                        atomicExch(&cnt->overflow, 1);
                    pos++;
                }
            }
        }
        else if (threadIdx.x == blockDim.x - 1)
            cntv[q] = s_part[threadIdx.x];
        __syncthreads();
    }
}

// The body edges of the body triangles paired with a cloth edge's (at most
// two) triangles, ascending: from a sorted local list when they fit, else by
// repeated minimum search (no bound, slower).
struct EdgeCands
{
    int buf[kLocalCand];
    int nbuf;
    bool spilled;
    int last;
    int pos;
    MergeIter m;
    const int *tedge;
    int seg_b[2], seg_e[2], nseg;
    const int *tp;
    __device__ void init(const int *tp_, const int *tedge_, int b0, int e0, int b1, int e1)
    {
        tp = tp_;
        tedge = tedge_;
        nseg = 0;
        if (b0 < e0)
        {
            seg_b[nseg] = b0;
            seg_e[nseg] = e0;
            nseg++;
        }
        if (b1 < e1)
        {
            seg_b[nseg] = b1;
            seg_e[nseg] = e1;
            nseg++;
        }
        nbuf = 0;
        spilled = false;
        m.init(tp);
        for (int i = 0; i < nseg; i++)
            m.add(seg_b[i], seg_e[i]);
        int t;
        while (!spilled && m.next(t))
            for (int k = 0; k < 3 && !spilled; k++)
                spilled = !insert_sorted(buf, nbuf, tedge[3 * size_t(t) + k]);
        pos = 0;
        last = -1;
    }
    __device__ bool next(int &f)
    {
        if (!spilled)
        {
            if (pos >= nbuf)
                return false;
            f = buf[pos++];
            return true;
        }
        int best = INT_MAX;
        MergeIter mm;
        mm.init(tp);
        for (int i = 0; i < nseg; i++)
            mm.add(seg_b[i], seg_e[i]);
        int t;
        while (mm.next(t))
            for (int k = 0; k < 3; k++)
            {
                const int e = tedge[3 * size_t(t) + k];
                if (e > last && e < best)
                    best = e;
            }
        if (best == INT_MAX)
            return false;
        last = best;
        f = best;
        return true;
    }
};

// 3c. cloth edge e against body edges (BVHCollisionDetecter.cpp:507-630,
//     obj0 = cloth): the cross product of the edges, turned to the side of
//     the body edge's triangle normals
__global__ void k_col_ee(BodyView b, int ne, const int *edges, const double *x,
                         const int *tp_off, const int *tp, int cap_pairs, int *cntv,
                         EeContact *out, int cap, int write, CollideCounts *cnt)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x)
    {
        const int v0 = edges[4 * size_t(e)], v1 = edges[4 * size_t(e) + 1];
        const int T0 = edges[4 * size_t(e) + 2], T1 = edges[4 * size_t(e) + 3];
        EdgeCands ec;
        ec.init(tp, b.tedge, T0 >= 0 ? min(tp_off[T0], cap_pairs) : 0,
                T0 >= 0 ? min(tp_off[T0 + 1], cap_pairs) : 0,
                T1 >= 0 ? min(tp_off[T1], cap_pairs) : 0,
                T1 >= 0 ? min(tp_off[T1 + 1], cap_pairs) : 0);
        const V3 p0 = ld3(x + 3 * size_t(v0)), p1 = ld3(x + 3 * size_t(v1));
        int n = 0;
        const int base = write ? cnt->n_ee + cntv[e] : 0;
        int f;
        while (ec.next(f))
        {
            const int *fe = b.edges + 4 * size_t(f);
            const V3 p2 = ld3(b.pos + 3 * size_t(fe[0])), p3 = ld3(b.pos + 3 * size_t(fe[1]));
            float s, t;
            edge_edge(p0, p1, p2, p3, s, t);
            const float s1 = 1 - s, t1 = 1 - t;
            const V3 c0 = {double(s1) * p0.x + double(s) * p1.x, double(s1) * p0.y + double(s) * p1.y,
                           double(s1) * p0.z + double(s) * p1.z};
            const V3 c1 = {double(t1) * p2.x + double(t) * p3.x, double(t1) * p2.y + double(t) * p3.y,
                           double(t1) * p2.z + double(t) * p3.z};
            V3 nn = nrm3(cross3(sub3(p1, p0), sub3(p3, p2)));
            V3 on = ld3(b.tn + 3 * size_t(fe[2]));
            if (fe[3] != -1)
            {
                const V3 o2 = ld3(b.tn + 3 * size_t(fe[3]));
                on = {on.x + o2.x, on.y + o2.y, on.z + o2.z};
            }
            if (dot3(nrm3(on), nn) < 0)
                nn = {-nn.x, -nn.y, -nn.z};
            const V3 dv = sub3(c0, c1);
            if (!(sqrt(dot3(dv, dv)) < 3e-3))
                continue;
            if (write)
            {
                if (base + n < cap)
                {
                    EeContact o;
                    o.e0 = e;
                    o.e1 = f;
                    o.s = s;
                    o.t = t;
                    o.n[0] = nn.x;
                    o.n[1] = nn.y;
                    o.n[2] = nn.z;
                    o.depth = float(dot3(dv, nn));
                    o.pad = 0;
                    out[base + n] = o;
                }
                else
                    atomicExch(&cnt->overflow, 1);
            }
            n++;
        }
        if (!write)
            cntv[e] = n;
    }
}

__global__ void k_col_advance(CollideCounts *cnt, int which, const int *total)
{
    if (threadIdx.x == 0)
    {
        if (which == 0)
            cnt->n_pt += *total;
        else
            cnt->n_ee += *total;
    }
}

// 4. per-vertex lists of the contacts touching each cloth vertex
__device__ __forceinline__ int contact_vertices(const CollideCounts *cnt, const PtContact *pt,
                                                const EeContact *ee, const int *edges,
                                                const int4 *tri, int i, int *v, int *tag)
{
    if (i < cnt->n_ee)
    {
        const EeContact &c = ee[i];
        v[0] = edges[4 * size_t(c.e0)];
        v[1] = edges[4 * size_t(c.e0) + 1];
        *tag = i;
        return 2;
    }
    const int k = i - cnt->n_ee;
    const PtContact &c = pt[k];
    *tag = k | kPtTag;
    if (c.cloth_point)
    {
        v[0] = c.p;
        return 1;
    }
    const int4 t = tri[c.t];
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    return 3;
}

__global__ void k_col_inc(const CollideCounts *cnt, int cap_pt, int cap_ee, const PtContact *pt,
                          const EeContact *ee, const int *edges, const int4 *tri, int *inc_off,
                          int *inc_cur, int *inc, int cap_inc, int fill, CollideCounts *cw,
                          int4 *cverts)
{
    CollideCounts c = *cnt;
    c.n_pt = min(c.n_pt, cap_pt);
    c.n_ee = min(c.n_ee, cap_ee);
    const int n = c.n_pt + c.n_ee;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        int v[3] = {-1, -1, -1}, tag;
        const int m = contact_vertices(&c, pt, ee, edges, tri, i, v, &tag);
        if (fill)
            cverts[i] = make_int4(v[0], v[1], v[2], m);
        for (int k = 0; k < m; k++)
        {
            if (!fill)
                atomicAdd(&inc_off[v[k]], 1);
            else
            {
                const int pos = inc_off[v[k]] + atomicAdd(&inc_cur[v[k]], 1);
                if (pos < cap_inc)
                    inc[pos] = tag;
                else
                    atomicExch(&cw->overflow, 1);
            }
        }
    }
}

__global__ void k_col_inc_sort(int nv, const int *inc_off, int *inc, int cap_inc)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
    {
        const int b0 = min(inc_off[v], cap_inc), b1 = min(inc_off[v + 1], cap_inc);
        for (int i = b0 + 1; i < b1; i++)
        {
            const int x = inc[i];
            int j = i;
            while (j > b0 && inc[j - 1] > x)
            {
                inc[j] = inc[j - 1];
                j--;
            }
            inc[j] = x;
        }
    }
}

// For every contact and each of its vertices: its place in that vertex's
// list (clpos) and the contact after it there (csucc, -1 at the end).
__global__ void k_col_links(int nv, const CollideCounts *cnt, int cap_pt, int cap_ee,
                            const int *inc_off, const int *inc, int cap_inc, const int4 *cverts,
                            int4 *clpos, int4 *csucc)
{
    const int n_ee = min(cnt->n_ee, cap_ee);
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
    {
        const int b0 = min(inc_off[v], cap_inc), b1 = min(inc_off[v + 1], cap_inc);
        for (int j = b0; j < b1; j++)
        {
            const int tg = inc[j];
            const int i = (tg & kPtTag) ? n_ee + (tg & ~kPtTag) : tg;
            int nx = -1;
            if (j + 1 < b1)
            {
                const int t2 = inc[j + 1];
                nx = (t2 & kPtTag) ? n_ee + (t2 & ~kPtTag) : t2;
            }
            const int4 cv = cverts[i];
            int *lp = reinterpret_cast<int *>(&clpos[i]);
            int *sc = reinterpret_cast<int *>(&csucc[i]);
            if (cv.x == v)
            {
                lp[0] = j - b0;
                sc[0] = nx;
            }
            else if (cv.y == v)
            {
                lp[1] = j - b0;
                sc[1] = nx;
            }
            else if (cv.z == v)
            {
                lp[2] = j - b0;
                sc[2] = nx;
            }
        }
    }
    (void)cap_pt;
}

__global__ void k_col_dxr(int nv, const float4 *dx, double *dxr, int *rptr, int ncs,
                          int *cstate)
{
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += stride)
    {
        const float4 d = dx[v];
        dxr[3 * size_t(v)] = d.x;
        dxr[3 * size_t(v) + 1] = d.y;
        dxr[3 * size_t(v) + 2] = d.z;
        rptr[v] = 0;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncs; i += stride)
        cstate[i] = 0;
}

// One contact's impulse on dxr (BaraffCloth.cpp:636-925), v: its cloth vertices.
__device__ void repulse_one(const CollideCounts &c, const PtContact *pt, const EeContact *ee,
                            int i, const int *v, const double *mass, double *dxr, double dt,
                            double K)
{
    const double v_thre = 0.01, scale = double(0.1f);
    if (i < c.n_ee)
    {
        const EeContact &e = ee[i];
        const float a = e.s, b = e.t, a1 = 1 - a;
        const int v0 = v[0], v1 = v[1];
        double vrel[3];
        for (int k = 0; k < 3; k++)
            vrel[k] = (double(a1) * dxr[3 * size_t(v0) + k] + double(a) * dxr[3 * size_t(v1) + k]) /
                      dt;
        const double ms = mass[v0] + mass[v1];
        const double vn = vrel[0] * e.n[0] + vrel[1] * e.n[1] + vrel[2] * e.n[2];
        const double Ic = vn > v_thre ? 0 : ms * fabs(vn) / 2;
        const double d = 3e-3 - double(e.depth);
        double Ir = 0;
        if (!(vn > double(0.1f) * d / dt))
        {
            const double Ir0 = dt * K * d, Ir1 = ms * (double(0.1f) * d / dt - vn);
            Ir = Ir0 < Ir1 ? Ir0 : Ir1;
        }
        const double I = Ic + Ir;
        const float den = 1 + a * a + (1 - a) * (1 - a) + b * b + (1 - b) * (1 - b);
        const double It = 2 * I / double(den);
        for (int k = 0; k < 3; k++)
        {
            dxr[3 * size_t(v0) + k] += scale * dt * double(a1) * It / ms * e.n[k];
            dxr[3 * size_t(v1) + k] += scale * dt * double(a) * It / ms * e.n[k];
        }
        return;
    }
    const PtContact &p = pt[i - c.n_ee];
    double vrel[3], ms;
    const double bw[3] = {p.bary[0], p.bary[1], p.bary[2]};
    if (p.cloth_point)
    {
        for (int k = 0; k < 3; k++)
            vrel[k] = dxr[3 * size_t(v[0]) + k] / dt;
        ms = mass[v[0]];
    }
    else
    {
        for (int k = 0; k < 3; k++)
            vrel[k] = (dxr[3 * size_t(v[0]) + k] * bw[0] + dxr[3 * size_t(v[1]) + k] * bw[1] +
                       dxr[3 * size_t(v[2]) + k] * bw[2]) /
                      dt;
        ms = mass[v[0]] + mass[v[1]] + mass[v[2]];
    }
    const double vn = vrel[0] * p.n[0] + vrel[1] * p.n[1] + vrel[2] * p.n[2];
    const double Ic = vn > v_thre ? 0 : ms * fabs(vn) / 2;
    const double d = 3e-3 - double(p.depth);
    double Ir = 0;
    if (!(vn > 0.1 * d / dt))
    {
        const double Ir0 = dt * K * d, Ir1 = ms * (0.1 * d / dt - vn);
        Ir = Ir0 < Ir1 ? Ir0 : Ir1;
    }
    const double I = Ic + Ir;
    const double It = 2 * I / (1 + (bw[0] * bw[0] + bw[1] * bw[1] + bw[2] * bw[2]));
    if (p.cloth_point)
        for (int k = 0; k < 3; k++)
            dxr[3 * size_t(v[0]) + k] += scale * (dt * It / ms * p.n[k]);
    else
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                dxr[3 * size_t(v[j]) + k] += scale * (dt * bw[j] * It / ms * p.n[k]);
}



// Repulsion (BaraffCloth.cpp:626-926) in rounds: a contact runs when it heads
// the list of every vertex it touches (every earlier contact there has run),
// so the contacts of one round share no vertex and the result is that of the
// sequential loop.  The first round's contacts come from a scan of all; after
// that only the new heads of the vertices a round touched can become ready,
// so each round visits just those (work lists wa / wb, a queued flag per
// contact).
__global__ void __launch_bounds__(kRepBlock) k_col_repulse(
    const CollideCounts *cnt_in, int cap_pt, int cap_ee, const PtContact *pt, const EeContact *ee,
    const int4 *cverts, const int4 *clpos, const int4 *csucc, const double *mass, int *rptr,
    int *queued, int *wa, int *wb, double *dxr, double dt, double K, CollideCounts *cw)
{
    __shared__ int s_na, s_nb, s_done;
    CollideCounts c = *cnt_in;
    c.n_pt = min(c.n_pt, cap_pt);
    c.n_ee = min(c.n_ee, cap_ee);
    const int n = c.n_pt + c.n_ee;
    // contact i heads all its lists when every vertex has run exactly the
    // contacts before it there
    auto ready = [&](int i) {
        const int4 cv = cverts[i], lp = clpos[i];
        bool r = rptr[cv.x] == lp.x;
        if (cv.w > 1)
            r = r && rptr[cv.y] == lp.y;
        if (cv.w > 2)
            r = r && rptr[cv.z] == lp.z;
        return r;
    };
    if (threadIdx.x == 0)
    {
        s_na = 0;
        s_nb = 0;
        s_done = 0;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (ready(i))
        {
            queued[i] = 1;
            wa[atomicAdd(&s_na, 1)] = i;
        }
    __syncthreads();
    int rounds = 0;
    int *cur = wa, *nxt = wb;
    while (s_na > 0 && rounds <= n)
    {
        const int na = s_na;
        // run this round's contacts (vertex-disjoint), then move their
        // vertices past them
        for (int k = threadIdx.x; k < na; k += blockDim.x)
        {
            const int i = cur[k];
            const int4 cv = cverts[i];
            const int v[3] = {cv.x, cv.y, cv.z};
            repulse_one(c, pt, ee, i, v, mass, dxr, dt, K);
            for (int q = 0; q < cv.w; q++)
                rptr[v[q]]++;
        }
        if (threadIdx.x == 0)
        {
            s_done += na;
            s_nb = 0;
        }
        __syncthreads();
        // their successors that now head all their lists
        for (int k = threadIdx.x; k < na; k += blockDim.x)
        {
            const int i = cur[k];
            const int4 sc = csucc[i];
            const int m = cverts[i].w;
            const int su[3] = {sc.x, sc.y, sc.z};
            for (int q = 0; q < m; q++)
            {
                const int h = su[q];
                if (h >= 0 && ready(h) && atomicExch(&queued[h], 1) == 0)
                    nxt[atomicAdd(&s_nb, 1)] = h;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0)
            s_na = s_nb;
        int *t = cur;
        cur = nxt;
        nxt = t;
        rounds++;
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        cw->rounds = rounds;
        if (s_done != n)
            cw->overflow = 1; // a contact never headed its lists (a lost list entry)
    }
}

} // namespace

// ------------------------------------------------------------------ host
namespace {

int col_fail(int code, const std::string &msg)
{
    set_last_error(msg);
    return code;
}

#define CCK(call)                                                              \
    do                                                                         \
    {                                                                          \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess)                                                 \
            return col_fail(CLOTH_ERR_CUDA,                                    \
                            std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int grid_blocks(const cloth_ctx *ctx, long long n)
{
    const long long b = (n + kColBlock - 1) / kColBlock;
    return int(std::max(1LL, std::min(b, (long long)ctx->num_sms * 16)));
}

void body_free(cloth_body_s *b)
{
    if (b->mem)
        cudaFree(b->mem);
    b->mem = nullptr;
}

// (Re)allocates the collision work arrays of a cloth for its bodies.
int collide_alloc(cloth_s *c)
{
    cloth_collide_s *w = c->col;
    const int nv = c->tab.nv, nt = c->tab.nt, ne = c->tab.ne;
    int max_bnt = 1, max_bnv = 1;
    long long sum_bnv = 0;
    for (auto *b : c->bodies)
    {
        max_bnt = std::max(max_bnt, b->nt);
        max_bnv = std::max(max_bnv, b->nv);
        sum_bnv += b->nv;
    }
    const long long cap_pairs = w->cap_request[0] > 0 ? w->cap_request[0] : 16LL * nt + 65536;
    const long long cap_pt =
        w->cap_request[1] > 0 ? w->cap_request[1] : 4LL * nv + 4 * sum_bnv + 4096;
    const long long cap_ee = w->cap_request[2] > 0 ? w->cap_request[2] : 8LL * nv + 4096;
    const long long cap_inc = 3 * cap_pt + 2 * cap_ee;
    if (cap_pairs > (1LL << 30) || cap_inc > (1LL << 30))
        return col_fail(CLOTH_ERR_INVALID, "collisions: contact capacities too large");
    if (std::max({(long long)nt, (long long)ne, (long long)max_bnt, (long long)max_bnv}) >=
        (long long)kScanTile * kScanMaxTiles)
        return col_fail(CLOTH_ERR_INVALID, "collisions: mesh too large for the contact lists");
    if (w->mem)
    {
        cudaFree(w->mem);
        c->ctx->bytes -= w->bytes;
        w->mem = nullptr;
    }
    const int nlist = std::max(std::max(nv, ne), max_bnv);
    Layout L;
    const size_t o_ctlo = L.take<double>(3 * size_t(nt)), o_cthi = L.take<double>(3 * size_t(nt)),
                 o_ctn = L.take<double>(3 * size_t(nt)), o_tpoff = L.take<int>(size_t(nt) + 1),
                 o_tp = L.take<int>(size_t(cap_pairs)), o_btoff = L.take<int>(size_t(max_bnt) + 1),
                 o_btcur = L.take<int>(size_t(max_bnt)), o_bt = L.take<int>(size_t(cap_pairs)),
                 o_lst = L.take<int>(size_t(nlist) + 1), o_pt = L.take<PtContact>(size_t(cap_pt)),
                 o_ee = L.take<EeContact>(size_t(cap_ee)),
                 o_incoff = L.take<int>(size_t(nv) + 1), o_inccur = L.take<int>(size_t(nv)),
                 o_inc = L.take<int>(size_t(cap_inc)), o_rptr = L.take<int>(size_t(nv)),
                 o_cst = L.take<int>(size_t(cap_pt + cap_ee)),
                 o_wa = L.take<int>(size_t(cap_pt + cap_ee)), o_wb = L.take<int>(size_t(cap_pt + cap_ee)),
                 o_dxr = L.take<double>(3 * size_t(nv)),
                 o_cnt = L.take<CollideCounts>(2), o_vtoff = L.take<int>(size_t(nv) + 1),
                 o_tsum = L.take<int>(kScanMaxTiles),
                 o_cvert = L.take<int4>(size_t(cap_pt + cap_ee)),
                 o_clpos = L.take<int4>(size_t(cap_pt + cap_ee)),
                 o_csucc = L.take<int4>(size_t(cap_pt + cap_ee)),
                 o_vt = L.take<int>(3 * size_t(nt)), o_edges = L.take<int>(4 * size_t(ne)),
                 o_mass = L.take<double>(size_t(nv));
    char *base = nullptr;
    if (cudaMalloc(&base, L.off) != cudaSuccess)
    {
        cudaGetLastError();
        return col_fail(CLOTH_ERR_OOM, "collisions: device allocation of " +
                                           std::to_string(L.off) + " bytes failed");
    }
    w->mem = base;
    w->bytes = L.off;
    c->ctx->bytes += w->bytes;
    w->ctlo = reinterpret_cast<double *>(base + o_ctlo);
    w->cthi = reinterpret_cast<double *>(base + o_cthi);
    w->ctn = reinterpret_cast<double *>(base + o_ctn);
    w->tp_off = reinterpret_cast<int *>(base + o_tpoff);
    w->tp = reinterpret_cast<int *>(base + o_tp);
    w->bt_off = reinterpret_cast<int *>(base + o_btoff);
    w->bt_cur = reinterpret_cast<int *>(base + o_btcur);
    w->bt = reinterpret_cast<int *>(base + o_bt);
    w->lst = reinterpret_cast<int *>(base + o_lst);
    w->pt = reinterpret_cast<PtContact *>(base + o_pt);
    w->ee = reinterpret_cast<EeContact *>(base + o_ee);
    w->inc_off = reinterpret_cast<int *>(base + o_incoff);
    w->inc_cur = reinterpret_cast<int *>(base + o_inccur);
    w->inc = reinterpret_cast<int *>(base + o_inc);
    w->rptr = reinterpret_cast<int *>(base + o_rptr);
    w->cstate = reinterpret_cast<int *>(base + o_cst);
    w->wa = reinterpret_cast<int *>(base + o_wa);
    w->wb = reinterpret_cast<int *>(base + o_wb);
    w->dxr = reinterpret_cast<double *>(base + o_dxr);
    w->cnt = reinterpret_cast<CollideCounts *>(base + o_cnt);
    w->tile_sum = reinterpret_cast<int *>(base + o_tsum);
    w->cverts = reinterpret_cast<int4 *>(base + o_cvert);
    w->clpos = reinterpret_cast<int4 *>(base + o_clpos);
    w->csucc = reinterpret_cast<int4 *>(base + o_csucc);
    w->vt_off = reinterpret_cast<int *>(base + o_vtoff);
    w->vt = reinterpret_cast<int *>(base + o_vt);
    w->edges = reinterpret_cast<int *>(base + o_edges);
    w->mass64 = reinterpret_cast<double *>(base + o_mass);
    w->cap_pairs = int(cap_pairs);
    w->cap_pt = int(cap_pt);
    w->cap_ee = int(cap_ee);
    w->cap_inc = int(cap_inc);
    w->max_bnt = max_bnt;
    w->max_bnv = max_bnv;
    // cloth vertex -> triangles, edges, masses (static)
    std::vector<int> vo(size_t(nv) + 1, 0), vl(3 * size_t(nt));
    for (int k = 0; k < 3 * nt; k++)
        vo[c->mesh.tris[k] + 1]++;
    for (int v = 0; v < nv; v++)
        vo[v + 1] += vo[v];
    std::vector<int> fillc(nv, 0);
    for (int t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++)
        {
            const int v = c->mesh.tris[3 * size_t(t) + k];
            vl[vo[v] + fillc[v]++] = t;
        }
    CCK(cudaMemcpy(w->vt_off, vo.data(), vo.size() * sizeof(int), cudaMemcpyHostToDevice));
    CCK(cudaMemcpy(w->vt, vl.data(), vl.size() * sizeof(int), cudaMemcpyHostToDevice));
    CCK(cudaMemcpy(w->edges, c->mesh.edges.data(), c->mesh.edges.size() * sizeof(int),
                   cudaMemcpyHostToDevice));
    CCK(cudaMemcpy(w->mass64, c->tab.mass.data(), size_t(nv) * sizeof(double),
                   cudaMemcpyHostToDevice));
    CCK(cudaMemset(w->cnt, 0, 2 * sizeof(CollideCounts)));
    // descriptor fields the row pass and the advance read
    c->h.cpt = w->pt;
    c->h.cinc_off = w->inc_off;
    c->h.cinc = w->inc;
    c->h.ccount = w->cnt;
    c->h.dxr = w->dxr;
    c->desc_dirty = true;
    return CLOTH_OK;
}

} // namespace

namespace {

void col_scan(cloth_collide_s *w, int *a, int n, int *total, cudaStream_t s)
{
    const int tiles = std::max(1, (n + kScanTile - 1) / kScanTile);
    k_col_scan_tiles<<<tiles, 1024, 0, s>>>(a, n, w->tile_sum);
    k_col_scan_top<<<1, 1024, 0, s>>>(w->tile_sum, tiles, a, n, total);
    k_col_scan_add<<<tiles, 256, 0, s>>>(a, n, w->tile_sum);
}

} // namespace

int cloth::detail::collide_detect(cloth_s *c)
{
    cloth_collide_s *w = c->col;
    if (!w || c->bodies.empty())
        return CLOTH_OK;
    cloth_ctx *ctx = c->ctx;
    cudaStream_t s = ctx->stream;
    const int nv = c->tab.nv, nt = c->tab.nt, ne = c->tab.ne;
    const int4 *tri = c->h.tri;
    const double *x = c->h.x64;
    int *total = reinterpret_cast<int *>(&w->cnt[1]); // scratch word for scan totals
    k_col_begin<<<1, 32, 0, s>>>(w->cnt, w->cap_inc);
    k_col_tri_boxes<<<grid_blocks(ctx, nt), kColBlock, 0, s>>>(nt, tri, x, w->ctlo, w->cthi,
                                                               w->ctn);
    for (auto *b : c->bodies)
    {
        const BodyView &bv = b->v;
        // triangle pairs
        k_col_pairs<<<grid_blocks(ctx, nt), kColBlock, 0, s>>>(bv, nt, w->ctlo, w->cthi,
                                                               w->tp_off, w->tp, w->cap_pairs,
                                                               0, w->cnt);
        col_scan(w, w->tp_off, nt, total, s);
        k_col_pairs<<<grid_blocks(ctx, nt), kColBlock, 0, s>>>(bv, nt, w->ctlo, w->cthi,
                                                               w->tp_off, w->tp, w->cap_pairs,
                                                               1, w->cnt);
        // grouped by body triangle
        CCK(cudaMemsetAsync(w->bt_off, 0, (size_t(bv.nt) + 1) * sizeof(int), s));
        CCK(cudaMemsetAsync(w->bt_cur, 0, size_t(bv.nt) * sizeof(int), s));
        k_col_bt_count<<<grid_blocks(ctx, nt), kColBlock, 0, s>>>(nt, w->tp_off, w->tp,
                                                                  w->cap_pairs, w->bt_off);
        col_scan(w, w->bt_off, bv.nt, total, s);
        k_col_bt_fill<<<grid_blocks(ctx, nt), kColBlock, 0, s>>>(
            nt, w->tp_off, w->tp, w->cap_pairs, w->bt_off, w->bt_cur, w->bt);
        k_col_bt_sort<<<std::max(1, std::min(bv.nt, ctx->num_sms * 16)), kSortBlock, 0, s>>>(
            bv.nt, w->bt_off, w->bt, w->cap_pairs);
        // cloth points against body triangles
        for (int pass = 0; pass < 2; pass++)
        {
            k_col_pt_cloth<<<grid_blocks(ctx, nv), kColBlock, 0, s>>>(
                bv, nv, x, w->vt_off, w->vt, w->tp_off, w->tp, w->cap_pairs, w->lst, w->pt,
                w->cap_pt, pass, w->cnt);
            if (pass == 0)
                col_scan(w, w->lst, nv, total, s);
        }
        k_col_advance<<<1, 32, 0, s>>>(w->cnt, 0, total);
        // body points against cloth triangles
        for (int pass = 0; pass < 2; pass++)
        {
            k_col_pt_body<<<std::max(1, std::min(bv.nv, ctx->num_sms * 16)), kSortBlock, 0, s>>>(
                bv, x, tri, w->ctn, w->bt_off, w->bt, w->cap_pairs, w->lst, w->pt, w->cap_pt,
                pass, w->cnt);
            if (pass == 0)
                col_scan(w, w->lst, bv.nv, total, s);
        }
        k_col_advance<<<1, 32, 0, s>>>(w->cnt, 0, total);
        // cloth edges against body edges
        for (int pass = 0; pass < 2; pass++)
        {
            k_col_ee<<<grid_blocks(ctx, ne), kColBlock, 0, s>>>(bv, ne, w->edges, x,
                                                                w->tp_off, w->tp, w->cap_pairs,
                                                                w->lst, w->ee, w->cap_ee, pass,
                                                                w->cnt);
            if (pass == 0)
                col_scan(w, w->lst, ne, total, s);
        }
        k_col_advance<<<1, 32, 0, s>>>(w->cnt, 1, total);
    }
    // per-vertex contact lists
    CCK(cudaMemsetAsync(w->inc_off, 0, (size_t(nv) + 1) * sizeof(int), s));
    CCK(cudaMemsetAsync(w->inc_cur, 0, size_t(nv) * sizeof(int), s));
    const int gc = grid_blocks(ctx, std::max(w->cap_pt, w->cap_ee));
    k_col_inc<<<gc, kColBlock, 0, s>>>(w->cnt, w->cap_pt, w->cap_ee, w->pt, w->ee, w->edges,
                                       tri, w->inc_off, w->inc_cur, w->inc, w->cap_inc, 0,
                                       w->cnt, w->cverts);
    col_scan(w, w->inc_off, nv, total, s);
    k_col_inc<<<gc, kColBlock, 0, s>>>(w->cnt, w->cap_pt, w->cap_ee, w->pt, w->ee, w->edges,
                                       tri, w->inc_off, w->inc_cur, w->inc, w->cap_inc, 1,
                                       w->cnt, w->cverts);
    k_col_inc_sort<<<grid_blocks(ctx, nv), kColBlock, 0, s>>>(nv, w->inc_off, w->inc,
                                                              w->cap_inc);
    k_col_links<<<grid_blocks(ctx, nv), kColBlock, 0, s>>>(nv, w->cnt, w->cap_pt, w->cap_ee,
                                                           w->inc_off, w->inc, w->cap_inc,
                                                           w->cverts, w->clpos, w->csucc);
    CCK(cudaGetLastError());
    return CLOTH_OK;
}

int cloth::detail::collide_repulse(cloth_s *c)
{
    cloth_collide_s *w = c->col;
    if (!w || c->bodies.empty())
        return CLOTH_OK;
    cloth_ctx *ctx = c->ctx;
    cudaStream_t s = ctx->stream;
    const int nv = c->tab.nv;
    const float kmean = ((c->mat.stretch_k[0] + c->mat.stretch_k[1]) + c->mat.stretch_k[2]) / 3.0f;
    const double K = double(kmean) * 1;
    k_col_dxr<<<grid_blocks(ctx, std::max(nv, w->cap_pt + w->cap_ee)), kColBlock, 0, s>>>(
        nv, c->h.dx, w->dxr, w->rptr, w->cap_pt + w->cap_ee, w->cstate);
    k_col_repulse<<<1, kRepBlock, 0, s>>>(w->cnt, w->cap_pt, w->cap_ee, w->pt, w->ee,
                                          w->cverts, w->clpos, w->csucc, w->mass64, w->rptr,
                                          w->cstate, w->wa, w->wb, w->dxr, c->dt_set, K, w->cnt);
    CCK(cudaGetLastError());
    return CLOTH_OK;
}

void cloth::detail::collide_free(cloth_s *c)
{
    if (!c->col)
        return;
    if (c->col->mem)
    {
        cudaFree(c->col->mem);
        c->ctx->bytes -= c->col->bytes;
    }
    delete c->col;
    c->col = nullptr;
    c->h.cpt = nullptr;
    c->h.cinc_off = nullptr;
    c->h.cinc = nullptr;
    c->h.ccount = nullptr;
    c->h.dxr = nullptr;
    c->desc_dirty = true;
}

void cloth::detail::body_release_all(cloth_ctx *ctx)
{
    for (auto *b : ctx->bodies)
    {
        body_free(b);
        delete b;
    }
    ctx->bodies.clear();
}

// ------------------------------------------------------------------ ABI
namespace {

// A body's device arrays from world-space positions: edges, normals (those
// given, else computed as the body's Init computes them), grown boxes,
// vertex -> triangle lists and the uniform grid, in a fresh allocation that
// b->mem / b->bytes / b->v then describe (the caller owns any older one).
// Called with the context's lock held and its device current.
int body_build(cloth_ctx *ctx, int nv, int nt, const double *pos, const int *tris,
               const double *keep_tn, const double *keep_vn, cloth_body_s *b)
{
    Mesh m;
    m.nv = nv;
    m.nt = nt;
    m.pos.assign(pos, pos + 3 * size_t(nv));
    m.tris.assign(tris, tris + 3 * size_t(nt));
    std::string err;
    if (!derive_edges(m, err))
        return col_fail(CLOTH_ERR_MESH, err);
    const int ne = m.ne;
    // triangle edges (v0 v1), (v1 v2), (v2 v0)
    std::map<std::pair<int, int>, int> eid;
    for (int e = 0; e < ne; e++)
        eid[{m.edges[4 * size_t(e)], m.edges[4 * size_t(e) + 1]}] = e;
    std::vector<int> tedge(3 * size_t(nt));
    for (int t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++)
        {
            const int a = tris[3 * size_t(t) + k], b = tris[3 * size_t(t) + (k + 1) % 3];
            tedge[3 * size_t(t) + k] = eid.at({std::min(a, b), std::max(a, b)});
        }
    // normals as the body's Init leaves them (cKinematicBody::Init:
    // CalcTriangleInitArea, UpdateTriangleNormal, UpdateVertexNormalFromTriangleNormal)
    std::vector<double> tn(3 * size_t(nt)), vn(3 * size_t(nv), 0.0);
    for (int t = 0; t < nt && !keep_tn; t++)
    {
        const double *p0 = pos + 3 * size_t(tris[3 * t]), *p1 = pos + 3 * size_t(tris[3 * t + 1]),
                     *p2 = pos + 3 * size_t(tris[3 * t + 2]);
        const double a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        const double b[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
        const double cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                              a[0] * b[1] - a[1] * b[0]};
        const double l = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        for (int k = 0; k < 3; k++)
            tn[3 * size_t(t) + k] = cr[k] / l;
        const double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        const double e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
        const double c2[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                              e1[0] * e2[1] - e1[1] * e2[0]};
        const double area =
            double(float(0.5 * std::sqrt(c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2])));
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++)
                vn[3 * size_t(tris[3 * t + i]) + k] += tn[3 * size_t(t) + k] * area;
    }
    for (int v = 0; v < nv && !keep_tn; v++)
    {
        double *n = &vn[3 * size_t(v)];
        const double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (l > 0)
            for (int k = 0; k < 3; k++)
                n[k] /= l;
    }
    if (keep_tn)
    {
        tn.assign(keep_tn, keep_tn + 3 * size_t(nt));
        vn.assign(keep_vn, keep_vn + 3 * size_t(nv));
    }
    // grown boxes, vertex -> triangles, uniform grid over the boxes
    std::vector<double> blo(3 * size_t(nt)), bhi(3 * size_t(nt));
    double g0[3] = {1e300, 1e300, 1e300}, g1[3] = {-1e300, -1e300, -1e300}, cell = 0.0;
    for (int t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++)
        {
            double mn = pos[3 * size_t(tris[3 * t]) + k], mx = mn;
            for (int i = 1; i < 3; i++)
            {
                const double v = pos[3 * size_t(tris[3 * t + i]) + k];
                mn = std::min(mn, v);
                mx = std::max(mx, v);
            }
            blo[3 * size_t(t) + k] = mn - 5e-3;
            bhi[3 * size_t(t) + k] = mx + 5e-3;
            g0[k] = std::min(g0[k], mn - 5e-3);
            g1[k] = std::max(g1[k], mx + 5e-3);
            cell = std::max(cell, (mx - mn) + 1e-2);
        }
    int gdim[3];
    for (;;)
    {
        long long total = 1;
        for (int k = 0; k < 3; k++)
        {
            gdim[k] = std::max(1, int(std::ceil((g1[k] - g0[k]) / cell)));
            total *= gdim[k];
        }
        if (total <= (1LL << 22))
            break;
        cell *= 1.5;
    }
    auto cell_of = [&](double v, int k) {
        const double q = std::floor((v - g0[k]) / cell);
        return q < 0.0 ? 0 : (q >= double(gdim[k]) ? gdim[k] - 1 : int(q));
    };
    const long long ncell = (long long)gdim[0] * gdim[1] * gdim[2];
    std::vector<int> coff(size_t(ncell) + 1, 0);
    std::vector<std::pair<int, int>> reg; // (cell, triangle)
    for (int t = 0; t < nt; t++)
    {
        int i0[3], i1[3];
        for (int k = 0; k < 3; k++)
        {
            i0[k] = cell_of(blo[3 * size_t(t) + k], k);
            i1[k] = cell_of(bhi[3 * size_t(t) + k], k);
        }
        for (int iz = i0[2]; iz <= i1[2]; iz++)
            for (int iy = i0[1]; iy <= i1[1]; iy++)
                for (int ix = i0[0]; ix <= i1[0]; ix++)
                    reg.push_back({(iz * gdim[1] + iy) * gdim[0] + ix, t});
    }
    std::sort(reg.begin(), reg.end());
    std::vector<int> ctris(reg.size());
    for (size_t k = 0; k < reg.size(); k++)
    {
        coff[reg[k].first + 1]++;
        ctris[k] = reg[k].second;
    }
    for (long long k = 0; k < ncell; k++)
        coff[k + 1] += coff[k];
    std::vector<int> vo(size_t(nv) + 1, 0), vl(3 * size_t(nt));
    for (int k = 0; k < 3 * nt; k++)
        vo[tris[k] + 1]++;
    for (int v = 0; v < nv; v++)
        vo[v + 1] += vo[v];
    {
        std::vector<int> f(nv, 0);
        for (int t = 0; t < nt; t++)
            for (int k = 0; k < 3; k++)
            {
                const int v = tris[3 * t + k];
                vl[vo[v] + f[v]++] = t;
            }
    }
    Layout L;
    const size_t o_pos = L.take<double>(3 * size_t(nv)), o_tris = L.take<int>(3 * size_t(nt)),
                 o_te = L.take<int>(3 * size_t(nt)), o_e = L.take<int>(4 * size_t(ne)),
                 o_tn = L.take<double>(3 * size_t(nt)), o_vn = L.take<double>(3 * size_t(nv)),
                 o_lo = L.take<double>(3 * size_t(nt)), o_hi = L.take<double>(3 * size_t(nt)),
                 o_vo = L.take<int>(size_t(nv) + 1), o_vl = L.take<int>(3 * size_t(nt)),
                 o_co = L.take<int>(size_t(ncell) + 1), o_ct = L.take<int>(std::max<size_t>(reg.size(), 1));
    b->ne = ne;
    b->mem = nullptr;
    if (cudaMalloc(&b->mem, L.off) != cudaSuccess)
    {
        cudaGetLastError();
        b->mem = nullptr;
        return col_fail(CLOTH_ERR_OOM, "cloth body: device allocation failed");
    }
    b->bytes = L.off;
    char *base = b->mem;
    auto up = [&](size_t o, const void *src, size_t bytes) {
        return cudaMemcpy(base + o, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    bool ok = up(o_pos, pos, 3 * size_t(nv) * 8) && up(o_tris, tris, 3 * size_t(nt) * 4) &&
              up(o_te, tedge.data(), tedge.size() * 4) && up(o_e, m.edges.data(), m.edges.size() * 4) &&
              up(o_tn, tn.data(), tn.size() * 8) && up(o_vn, vn.data(), vn.size() * 8) &&
              up(o_lo, blo.data(), blo.size() * 8) && up(o_hi, bhi.data(), bhi.size() * 8) &&
              up(o_vo, vo.data(), vo.size() * 4) && up(o_vl, vl.data(), vl.size() * 4) &&
              up(o_co, coff.data(), coff.size() * 4) &&
              (ctris.empty() || up(o_ct, ctris.data(), ctris.size() * 4));
    if (!ok)
    {
        cudaFree(b->mem);
        b->mem = nullptr;
        return col_fail(CLOTH_ERR_CUDA, "cloth body: upload failed");
    }
    BodyView &v = b->v;
    v.nv = nv;
    v.nt = nt;
    v.ne = ne;
    v.pos = reinterpret_cast<const double *>(base + o_pos);
    v.tris = reinterpret_cast<const int *>(base + o_tris);
    v.tedge = reinterpret_cast<const int *>(base + o_te);
    v.edges = reinterpret_cast<const int *>(base + o_e);
    v.tn = reinterpret_cast<const double *>(base + o_tn);
    v.vn = reinterpret_cast<const double *>(base + o_vn);
    v.blo = reinterpret_cast<const double *>(base + o_lo);
    v.bhi = reinterpret_cast<const double *>(base + o_hi);
    v.vt_off = reinterpret_cast<const int *>(base + o_vo);
    v.vt = reinterpret_cast<const int *>(base + o_vl);
    v.cell_off = reinterpret_cast<const int *>(base + o_co);
    v.cell_tris = reinterpret_cast<const int *>(base + o_ct);
    for (int k = 0; k < 3; k++)
    {
        v.g0[k] = g0[k];
        v.gdim[k] = gdim[k];
    }
    v.cell = cell;
    b->tn = std::move(tn);
    b->vn = std::move(vn);
    (void)ctx;
    return CLOTH_OK;
}

// cKinematicBody's world transform at body time t (KinematicBody.cpp
// UpdateCurWorldTransformByTime, GetWorldTransform; RotUtil.cpp
// EulerAnglesToRotMat, XYZ order: Rz * Ry * Rx) applied to the local mesh.
// Products are summed term by term in index order, as the reference's 4x4
// products evaluate them.
void kinematic_pose(int nv, const double *local, const double *ip, const double *io,
                    const double *tp, const double *to, double elapsed, float time,
                    double *world)
{
    float ct = time;
    if (ct > elapsed)
        ct = float(elapsed);
    const double a = (elapsed - double(ct)) / elapsed, c = double(ct) / elapsed;
    double pos[3], ori[3];
    for (int k = 0; k < 3; k++)
    {
        pos[k] = a * ip[k] + c * tp[k];
        ori[k] = a * io[k] + c * to[k];
    }
    auto rot = [](int axis, double ang, double m[4][4]) {
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                m[i][j] = i == j ? 1.0 : 0.0;
        const double cs = std::cos(ang), sn = std::sin(ang);
        const int p = axis == 0 ? 1 : 0, q = axis == 2 ? 1 : 2;
        m[p][p] = cs;
        m[q][q] = cs;
        if (axis == 1) // about y: (0 2) = sin, (2 0) = -sin
        {
            m[p][q] = sn;
            m[q][p] = -sn;
        }
        else
        {
            m[p][q] = -sn;
            m[q][p] = sn;
        }
    };
    auto mul = [](const double l[4][4], const double r[4][4], double o[4][4]) {
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
            {
                double s = l[i][0] * r[0][j];
                for (int k = 1; k < 4; k++)
                    s = l[i][k] * r[k][j] + s;
                o[i][j] = s;
            }
    };
    double rx[4][4], ry[4][4], rz[4][4], zy[4][4], r[4][4];
    rot(0, ori[0], rx);
    rot(1, ori[1], ry);
    rot(2, ori[2], rz);
    mul(rz, ry, zy);
    mul(zy, rx, r);
    double tr[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            tr[i][j] = (i < 3 && j < 3) ? r[i][j] : (i == j ? 1.0 : 0.0);
    for (int i = 0; i < 3; i++)
        tr[i][3] = pos[i];
    for (int v = 0; v < nv; v++)
    {
        const double x[4] = {local[3 * size_t(v)], local[3 * size_t(v) + 1],
                             local[3 * size_t(v) + 2], 1.0};
        for (int i = 0; i < 3; i++)
        {
            double s = tr[i][0] * x[0];
            for (int k = 1; k < 4; k++)
                s = tr[i][k] * x[k] + s;
            world[3 * size_t(v) + i] = s;
        }
    }
}

// New device arrays for new positions; keep_normals: the body's current ones
int body_move(cloth_body_s *b, const double *pos, bool keep_normals)
{
    cloth_ctx *ctx = b->ctx;
    CCK(cudaSetDevice(ctx->device));
    CCK(cudaStreamSynchronize(ctx->stream)); // no detection still reads the old arrays
    cloth_body_s nb;
    nb.ctx = ctx;
    nb.nv = b->nv;
    nb.nt = b->nt;
    const int rc = body_build(ctx, b->nv, b->nt, pos, b->tris.data(),
                              keep_normals ? b->tn.data() : nullptr,
                              keep_normals ? b->vn.data() : nullptr, &nb);
    if (rc != CLOTH_OK)
        return rc;
    cudaFree(b->mem);
    ctx->bytes = ctx->bytes - b->bytes + nb.bytes;
    b->mem = nb.mem;
    b->bytes = nb.bytes;
    b->v = nb.v;
    b->tn = std::move(nb.tn);
    b->vn = std::move(nb.vn);
    return CLOTH_OK;
}

} // namespace

int cloth_body_create(cloth_ctx *ctx, int nv, int nt, const double *pos, const int *tris,
                      cloth_body **out)
{
    if (!ctx || !pos || !tris || !out || nv < 3 || nt < 1)
        return col_fail(CLOTH_ERR_INVALID, "cloth_body_create: bad argument");
    *out = nullptr;
    for (int k = 0; k < 3 * nt; k++)
        if (tris[k] < 0 || tris[k] >= nv)
            return col_fail(CLOTH_ERR_MESH, "cloth_body_create: triangle vertex id out of range");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    CCK(cudaSetDevice(ctx->device));
    auto b = new cloth_body_s();
    b->ctx = ctx;
    b->nv = nv;
    b->nt = nt;
    b->tris.assign(tris, tris + 3 * size_t(nt));
    const int rc = body_build(ctx, nv, nt, pos, tris, nullptr, nullptr, b);
    if (rc != CLOTH_OK)
    {
        delete b;
        return rc;
    }
    ctx->bodies.push_back(b);
    ctx->bytes += b->bytes;
    *out = b;
    return CLOTH_OK;
}

int cloth_kinematic_pose(int nv, const double *local, const double *init_pos,
                         const double *init_ori, const double *target_pos,
                         const double *target_ori, double elapsed_sec, float time,
                         double *world)
{
    if (nv < 1 || !local || !init_pos || !init_ori || !target_pos || !target_ori || !world ||
        !(elapsed_sec > 0))
        return col_fail(CLOTH_ERR_INVALID, "cloth_kinematic_pose: bad argument");
    kinematic_pose(nv, local, init_pos, init_ori, target_pos, target_ori, elapsed_sec, time,
                   world);
    return CLOTH_OK;
}

int cloth_body_set_pos(cloth_body *b, const double *pos)
{
    if (!b || !pos)
        return col_fail(CLOTH_ERR_INVALID, "cloth_body_set_pos: bad argument");
    std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
    return body_move(b, pos, true);
}

int cloth_body_set_motion(cloth_body *b, const double *local, const double *init_pos,
                          const double *init_ori, const double *target_pos,
                          const double *target_ori, double elapsed_sec)
{
    if (!b || !local || !init_pos || !init_ori || !target_pos || !target_ori ||
        !(elapsed_sec > 0))
        return col_fail(CLOTH_ERR_INVALID, "cloth_body_set_motion: bad argument");
    std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
    b->local.assign(local, local + 3 * size_t(b->nv));
    for (int k = 0; k < 3; k++)
    {
        b->ip[k] = init_pos[k];
        b->io[k] = init_ori[k];
        b->tp[k] = target_pos[k];
        b->to[k] = target_ori[k];
    }
    b->elapsed = elapsed_sec;
    b->time = 0.f;
    b->moving = true;
    // placed at the initial pose, normals from there (the body's Init)
    std::vector<double> w(3 * size_t(b->nv));
    kinematic_pose(b->nv, b->local.data(), b->ip, b->io, b->tp, b->to, b->elapsed, b->time,
                   w.data());
    return body_move(b, w.data(), false);
}

int cloth_body_update(cloth_body *b, float dt)
{
    if (!b)
        return col_fail(CLOTH_ERR_INVALID, "cloth_body_update: NULL body");
    std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
    b->time += dt; // the body clock is a float, as mCurTime is
    if (!b->moving)
        return CLOTH_OK;
    std::vector<double> w(3 * size_t(b->nv));
    kinematic_pose(b->nv, b->local.data(), b->ip, b->io, b->tp, b->to, b->elapsed, b->time,
                   w.data());
    return body_move(b, w.data(), true);
}

int cloth_body_get_pos(cloth_body *b, double *pos)
{
    if (!b || !pos)
        return col_fail(CLOTH_ERR_INVALID, "cloth_body_get_pos: bad argument");
    std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
    CCK(cudaSetDevice(b->ctx->device));
    CCK(cudaStreamSynchronize(b->ctx->stream));
    CCK(cudaMemcpy(pos, b->v.pos, 3 * size_t(b->nv) * sizeof(double), cudaMemcpyDeviceToHost));
    return CLOTH_OK;
}

int cloth_body_destroy(cloth_body *b)
{
    if (!b)
        return CLOTH_OK;
    cloth_ctx *ctx = b->ctx;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    for (auto *c : ctx->cloths)
        if (std::find(c->bodies.begin(), c->bodies.end(), b) != c->bodies.end())
            return col_fail(CLOTH_ERR_STATE, "cloth_body_destroy: a cloth still collides with "
                                             "this body (cloth_set_bodies first)");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->bytes -= b->bytes;
    body_free(b);
    ctx->bodies.erase(std::remove(ctx->bodies.begin(), ctx->bodies.end(), b), ctx->bodies.end());
    delete b;
    return CLOTH_OK;
}

int cloth_set_bodies(cloth_t *c, cloth_body *const *bodies, int n)
{
    if (!c || n < 0 || (n > 0 && !bodies))
        return col_fail(CLOTH_ERR_INVALID, "cloth_set_bodies: bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    if (c->server)
        return col_fail(CLOTH_ERR_STATE, "cloth_set_bodies: the cloth is held by a server");
    for (int i = 0; i < n; i++)
        if (!bodies[i] || bodies[i]->ctx != c->ctx)
            return col_fail(CLOTH_ERR_INVALID, "cloth_set_bodies: body of another context");
    CCK(cudaSetDevice(c->ctx->device));
    CCK(cudaStreamSynchronize(c->ctx->stream));
    c->bodies.assign(bodies, bodies + n);
    drop_launch_sets(c); // rebuilt for the new collision state
    if (n == 0)
    {
        collide_free(c);
        return sync_desc(c);
    }
    if (!c->col)
        c->col = new cloth_collide_s();
    int rc = collide_alloc(c);
    if (rc != CLOTH_OK)
    {
        collide_free(c);
        c->bodies.clear();
        return rc;
    }
    return sync_desc(c);
}

int cloth_set_contact_capacity(cloth_t *c, int pairs, int point_triangle, int edge_edge)
{
    if (!c || pairs < 0 || point_triangle < 0 || edge_edge < 0)
        return col_fail(CLOTH_ERR_INVALID, "cloth_set_contact_capacity: bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    if (!c->col)
        c->col = new cloth_collide_s();
    c->col->cap_request[0] = pairs;
    c->col->cap_request[1] = point_triangle;
    c->col->cap_request[2] = edge_edge;
    if (c->bodies.empty())
        return CLOTH_OK;
    CCK(cudaSetDevice(c->ctx->device));
    CCK(cudaStreamSynchronize(c->ctx->stream));
    int rc = collide_alloc(c);
    if (rc != CLOTH_OK)
        return rc;
    return sync_desc(c);
}

int cloth_get_contacts(cloth_t *c, cloth_contact_stats *st, int *pt_i, double *pt_d, int *ee_i,
                       double *ee_d)
{
    if (!c)
        return col_fail(CLOTH_ERR_INVALID, "cloth is NULL");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    cloth_contact_stats s{};
    cloth_collide_s *w = c->col;
    if (!w || !w->mem || c->bodies.empty())
    {
        if (st)
            *st = s;
        return CLOTH_OK;
    }
    CCK(cudaSetDevice(c->ctx->device));
    CCK(cudaStreamSynchronize(c->ctx->stream));
    CollideCounts cc;
    CCK(cudaMemcpy(&cc, w->cnt, sizeof(cc), cudaMemcpyDeviceToHost));
    s.n_pt = std::min(cc.n_pt, w->cap_pt);
    s.n_ee = std::min(cc.n_ee, w->cap_ee);
    s.overflow = cc.overflow;
    s.repulsion_rounds = cc.rounds;
    if (st)
        *st = s;
    if (pt_i || pt_d)
    {
        std::vector<PtContact> v(size_t(s.n_pt));
        if (s.n_pt)
            CCK(cudaMemcpy(v.data(), w->pt, v.size() * sizeof(PtContact), cudaMemcpyDeviceToHost));
        for (int i = 0; i < s.n_pt; i++)
        {
            if (pt_i)
            {
                pt_i[3 * i] = v[i].cloth_point;
                pt_i[3 * i + 1] = v[i].p;
                pt_i[3 * i + 2] = v[i].t;
            }
            if (pt_d)
            {
                for (int k = 0; k < 3; k++)
                    pt_d[7 * size_t(i) + k] = v[i].n[k];
                pt_d[7 * size_t(i) + 3] = double(v[i].depth);
                for (int k = 0; k < 3; k++)
                    pt_d[7 * size_t(i) + 4 + k] = double(v[i].bary[k]);
            }
        }
    }
    if (ee_i || ee_d)
    {
        std::vector<EeContact> v(size_t(s.n_ee));
        if (s.n_ee)
            CCK(cudaMemcpy(v.data(), w->ee, v.size() * sizeof(EeContact), cudaMemcpyDeviceToHost));
        for (int i = 0; i < s.n_ee; i++)
        {
            if (ee_i)
            {
                ee_i[3 * i] = 1;
                ee_i[3 * i + 1] = v[i].e0;
                ee_i[3 * i + 2] = v[i].e1;
            }
            if (ee_d)
            {
                for (int k = 0; k < 3; k++)
                    ee_d[6 * size_t(i) + k] = v[i].n[k];
                ee_d[6 * size_t(i) + 3] = double(v[i].depth);
                ee_d[6 * size_t(i) + 4] = double(v[i].s);
                ee_d[6 * size_t(i) + 5] = double(v[i].t);
            }
        }
    }
    return CLOTH_OK;
}

int cloth_get_repulsed_dx(cloth_t *c, double *dx, int nv)
{
    if (!c || !dx || nv != c->tab.nv)
        return col_fail(CLOTH_ERR_INVALID, "cloth_get_repulsed_dx: bad argument");
    std::lock_guard<std::recursive_mutex> lk(c->ctx->mu);
    if (!c->col || !c->col->mem || c->bodies.empty())
        return col_fail(CLOTH_ERR_STATE, "cloth_get_repulsed_dx: the cloth has no bodies");
    CCK(cudaSetDevice(c->ctx->device));
    CCK(cudaStreamSynchronize(c->ctx->stream));
    CCK(cudaMemcpy(dx, c->col->dxr, 3 * size_t(nv) * sizeof(double), cudaMemcpyDeviceToHost));
    return CLOTH_OK;
}
