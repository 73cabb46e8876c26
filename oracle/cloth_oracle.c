/*
 * cloth_oracle.c - CPU restatement of AcousticSim's implicit cloth step.
 * TEST INFRASTRUCTURE ONLY (see cloth_oracle.h): the checker of the GPU path,
 * never part of it.  Each function cites the reference lines it restates.
 * Built with -ffp-contract=off so x86 and Arm hosts round identically.
 */
#include "cloth_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define W CLOTH_ORC_W

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ grid */
int orc_grid(const double size[2], const int subdiv[2], const double init_pos[3],
             float uv_rotation_deg, int *nv_out, int *nt_out, int *ne_out,
             double *pos, float *uv, int *tris, int *edges)
{
    const int hd = subdiv[0], wd = subdiv[1];
    if (hd < 1 || wd < 1)
        return -1;
    const int lines_h = hd + 1; /* vertices per column strip */
    const int nv = (wd + 1) * lines_h, nt = 2 * wd * hd;
    const int ne = (wd + 1) * hd + lines_h * wd + hd * wd;
    if (nv_out)
        *nv_out = nv;
    if (nt_out)
        *nt_out = nt;
    if (ne_out)
        *ne_out = ne;
    if (!pos && !uv && !tris && !edges)
        return 0;
    /* Triangulator.cpp:417-455: vertex (i, j) at (i*w_unit, j*h_unit) minus the
     * centre, i over the width divisions (outer), j over the height ones. */
    const double h_unit = size[0] / hd, w_unit = size[1] / wd;
    /* RotateMaterialCoordsAfterReset (:621-658): the angle is rounded to float
     * and the 2x2 rotation is applied in float. */
    const float ang = (float)(uv_rotation_deg / 180.0 * M_PI);
    const float cr = (float)cos((double)ang), sr = (float)sin((double)ang);
    for (int i = 0; i <= wd; i++)
        for (int j = 0; j <= hd; j++)
        {
            const int v = i * lines_h + j;
            double p[3];
            p[0] = i * w_unit - size[1] / 2;
            p[1] = j * h_unit - size[0] / 2;
            p[2] = 0.0;
            for (int k = 0; k < 3; k++)
                p[k] += init_pos[k];
            if (pos)
                for (int k = 0; k < 3; k++)
                    pos[3 * v + k] = p[k];
            if (uv)
            {
                const float mx = (float)(p[0] + (-init_pos[0]));
                const float my = (float)(p[1] + (-init_pos[1]));
                uv[2 * v] = cr * mx + (-sr) * my;
                uv[2 * v + 1] = sr * mx + cr * my;
            }
        }
    /* Triangulator.cpp:192-389: two triangles per cell, diagonal direction by
     * the parity of (row + col); edges numbered by row strips. */
    const int per_row = 2 * hd + lines_h;
    int t = 0;
    for (int row = 0; row < wd; row++)
        for (int col = 0; col < hd; col++)
        {
            const int a = row * lines_h + col; /* upper-left  */
            const int bq = a + 1;              /* upper-right */
            const int cq = a + lines_h;        /* lower-left  */
            const int d = cq + 1;              /* lower-right */
            const int even = ((row + col) & 1) == 0;
            const int e_top = row * per_row + col;
            const int e_left = row * per_row + hd + 2 * col;
            const int e_skew = e_left + 1, e_right = e_left + 2;
            const int e_bottom = e_top + per_row;
            const int t0 = t, t1 = t + 1;
            if (tris)
            {
                int *o = tris + 3 * t;
                if (even)
                {
                    o[0] = a; o[1] = cq; o[2] = d;
                    o[3] = a; o[4] = d;  o[5] = bq;
                }
                else
                {
                    o[0] = a;  o[1] = cq; o[2] = bq;
                    o[3] = cq; o[4] = d;  o[5] = bq;
                }
            }
            t += 2;
            if (!edges)
                continue;
#define SETE(id, v0, v1, ta, tb)                                               \
    do                                                                         \
    {                                                                          \
        edges[4 * (id) + 0] = (v0);                                            \
        edges[4 * (id) + 1] = (v1);                                            \
        edges[4 * (id) + 2] = (ta);                                            \
        edges[4 * (id) + 3] = (tb);                                            \
    } while (0)
            if (even)
                SETE(e_skew, a, d, t0, t1);
            else
                SETE(e_skew, bq, cq, t0, t1);
            {
                const int ta = even ? t0 : t1;
                SETE(e_bottom, cq, d, ta, row == wd - 1 ? -1 : ta + 2 * hd);
            }
            SETE(e_right, bq, d, t1, col == hd - 1 ? -1 : t1 + 1);
            if (row == 0)
                SETE(e_top, a, bq, even ? t1 : t0, -1);
            if (col == 0)
                SETE(e_left, a, cq, t0, -1);
#undef SETE
        }
    return 0;
}

/* ------------------------------------------------------------------ tables */
static double cot_ref(const double *A, const double *B, const double *C)
{
    /* CalcCotangent (QBendingMaterial.cpp:11-19): dots rounded to float. */
    double ab[3], ac[3];
    for (int k = 0; k < 3; k++)
    {
        ab[k] = B[k] - A[k];
        ac[k] = C[k] - A[k];
    }
    const float d_bc = (float)((ab[0] * ac[0] + ab[1] * ac[1]) + ab[2] * ac[2]);
    const float d_bb = (float)((ab[0] * ab[0] + ab[1] * ab[1]) + ab[2] * ab[2]);
    const float d_cc = (float)((ac[0] * ac[0] + ac[1] * ac[1]) + ac[2] * ac[2]);
    const float den = d_bb * d_cc - d_bc * d_bc;
    return (double)(d_bc / sqrtf(den));
}

static int row_insert(int *row, int *len, int v)
{
    int k = 0;
    while (k < *len && row[k] < v)
        k++;
    if (k < *len && row[k] == v)
        return 0;
    if (*len >= W)
        return -1;
    memmove(row + k + 1, row + k, sizeof(int) * (size_t)(*len - k));
    row[k] = v;
    (*len)++;
    return 0;
}

static int row_find(const int *row, int v)
{
    for (int k = 0; k < W && row[k] >= 0; k++)
        if (row[k] == v)
            return k;
    return -1;
}

static int third_vertex(const int *tri, int a, int b)
{
    /* SelectAnotherVerteix (BaseCloth.cpp:281-290) */
    int best = -1;
    for (int k = 0; k < 3; k++)
        if (tri[k] != a && tri[k] != b && (best < 0 || tri[k] < best))
            best = tri[k];
    return best;
}

int orc_tables(int nv, int nt, int ne, const double *pos, const float *uv,
               const int *tris, const int *edges, float density,
               const float bending_k[2], int *stencil, float *area, double *mass,
               int *ell, float *coef, float *diag16, float *edge_k, double *kbend)
{
    /* stencils: BaseCloth.cpp:383-405 */
    for (int e = 0; e < ne; e++)
    {
        const int *ed = edges + 4 * e;
        int *s = stencil + 4 * e;
        if (ed[3] < 0)
        {
            s[0] = s[1] = s[2] = s[3] = -1;
            continue;
        }
        s[0] = ed[0];
        s[1] = ed[1];
        s[2] = third_vertex(tris + 3 * ed[2], ed[0], ed[1]);
        s[3] = third_vertex(tris + 3 * ed[3], ed[0], ed[1]);
    }
    /* areas (MathUtil2.cpp:353-357) and masses (BaseCloth.cpp:418-446) */
    for (int v = 0; v < nv; v++)
        mass[v] = 0.0;
    for (int t = 0; t < nt; t++)
    {
        const double *p0 = pos + 3 * tris[3 * t], *p1 = pos + 3 * tris[3 * t + 1],
                     *p2 = pos + 3 * tris[3 * t + 2];
        double u[3], w[3], c[3];
        for (int k = 0; k < 3; k++)
        {
            u[k] = p1[k] - p0[k];
            w[k] = p2[k] - p0[k];
        }
        c[0] = u[1] * w[2] - u[2] * w[1];
        c[1] = u[2] * w[0] - u[0] * w[2];
        c[2] = u[0] * w[1] - u[1] * w[0];
        double sq = c[0] * c[0] + c[1] * c[1];
        sq = sq + c[2] * c[2];
        area[t] = (float)(0.5 * sqrt(sq));
        for (int k = 0; k < 3; k++)
            mass[tris[3 * t + k]] += (double)area[t] / 3;
    }
    for (int v = 0; v < nv; v++)
        mass[v] = mass[v] * (double)density;
    /* ELL: BaraffClothGpu.cpp:438-500 */
    int *len = (int *)calloc((size_t)nv, sizeof(int));
    for (size_t k = 0; k < (size_t)nv * W; k++)
        ell[k] = -1;
    int bad = 0;
    for (int v = 0; v < nv; v++)
        bad |= row_insert(ell + (size_t)v * W, &len[v], v);
    for (int e = 0; e < ne && !bad; e++)
    {
        const int *s = stencil + 4 * e;
        if (s[0] < 0)
            continue;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                bad |= row_insert(ell + (size_t)s[i] * W, &len[s[i]], s[j]);
    }
    for (int t = 0; t < nt && !bad; t++)
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                bad |= row_insert(ell + (size_t)tris[3 * t + a] * W,
                                  &len[tris[3 * t + a]], tris[3 * t + b]);
    free(len);
    if (bad)
        return -1;
    /* stretch coefficients: BaraffClothGpu.cpp:504-553, BaraffMaterial.cpp:18-32 */
    const double q = M_PI / 4, rc = cos(q), rs = sin(q);
    for (int t = 0; t < nt; t++)
    {
        const float *u0 = uv + 2 * tris[3 * t], *u1 = uv + 2 * tris[3 * t + 1],
                    *u2 = uv + 2 * tris[3 * t + 2];
        const double m00 = (double)(u1[0] - u0[0]), m01 = (double)(u2[0] - u0[0]);
        const double m10 = (double)(u1[1] - u0[1]), m11 = (double)(u2[1] - u0[1]);
        const double id = 1.0 / (m00 * m11 - m10 * m01);
        double inv[2][2];
        inv[0][0] = m11 * id;
        inv[0][1] = -m01 * id;
        inv[1][0] = -m10 * id;
        inv[1][1] = m00 * id;
        float *c = coef + 12 * t;
        for (int pass = 0; pass < 2; pass++)
        {
            double mm[2][2];
            if (pass == 0)
                memcpy(mm, inv, sizeof(mm));
            else /* inv * R45^T, R45 = [[c, -s], [s, c]] */
                for (int i = 0; i < 2; i++)
                {
                    mm[i][0] = inv[i][0] * rc + inv[i][1] * (-rs);
                    mm[i][1] = inv[i][0] * rs + inv[i][1] * rc;
                }
            const float fa = (float)mm[0][0], fb = (float)mm[0][1],
                        fc = (float)mm[1][0], fd = (float)mm[1][1];
            float *o = c + 6 * pass;
            o[0] = -fa - fc;
            o[1] = fa;
            o[2] = fc;
            o[3] = -fb - fd;
            o[4] = fb;
            o[5] = fd;
        }
    }
    /* bending: BaraffClothGpu.cpp:579-680, QBendingMaterial.cpp:20-43 (its
     * Clamp calls discard their results, so nothing is clamped) */
    for (size_t k = 0; k < (size_t)nv * W; k++)
        kbend[k] = 0.0;
    for (int e = 0; e < ne; e++)
    {
        const int *ed = edges + 4 * e;
        float dx = uv[2 * ed[1]] - uv[2 * ed[0]];
        float dy = uv[2 * ed[1] + 1] - uv[2 * ed[0] + 1];
        const float n2 = dx * dx + dy * dy;
        if (n2 > 0.f)
        {
            const float n = sqrtf(n2);
            dx = dx / n;
            dy = dy / n;
        }
        float th = acosf(dx * 1.f + dy * 0.f);
        if (th > M_PI / 2.0f)
            th = (float)(M_PI - th);
        const float ct = cosf(th), st = sinf(th);
        edge_k[e] = bending_k[0] * ct * ct + bending_k[1] * st * st;
        float *dg = diag16 + 16 * e;
        for (int k = 0; k < 16; k++)
            dg[k] = 0.f;
        const int *s = stencil + 4 * e;
        if (s[0] < 0)
            continue;
        const float pre = (float)(3.0 / (area[ed[2]] + area[ed[3]]));
        const double *x0 = pos + 3 * s[0], *x1 = pos + 3 * s[1],
                     *x2 = pos + 3 * s[2], *x3 = pos + 3 * s[3];
        const double c01 = cot_ref(x0, x1, x2), c02 = cot_ref(x0, x1, x3);
        const double c03 = cot_ref(x1, x0, x2), c04 = cot_ref(x1, x0, x3);
        const double cw[4] = {c03 + c04, c01 + c02, -c01 - c03, -c02 - c04};
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
            {
                dg[4 * i + j] = (float)(cw[i] * cw[j] * (double)pre);
                const float val = dg[4 * i + j] * edge_k[e];
                const int slot = row_find(ell + (size_t)s[i] * W, s[j]);
                kbend[(size_t)s[i] * W + slot] += (double)val;
            }
    }
    return 0;
}

/* ------------------------------------------------------------------ forces */
static void stretch_term(double Ku, double Kv, double S, const float *cu,
                         const float *cv, const double *x0, const double *x1,
                         const double *x2, int fix_fv, double *f, double *h)
{
    /* BaraffMaterial.cpp:82-172 */
    double Fu[3], Fv[3];
    for (int k = 0; k < 3; k++)
    {
        Fu[k] = cu[0] * x0[k] + cu[1] * x1[k] + cu[2] * x2[k];
        Fv[k] = cv[0] * x0[k] + cv[1] * x1[k] + cv[2] * x2[k];
    }
    const double nu = sqrt(Fu[0] * Fu[0] + Fu[1] * Fu[1] + Fu[2] * Fu[2]);
    const double nv = sqrt(Fv[0] * Fv[0] + Fv[1] * Fv[1] + Fv[2] * Fv[2]);
    double un[3], vn[3];
    for (int k = 0; k < 3; k++)
    {
        un[k] = nu > 0 ? Fu[k] / nu : Fu[k];
        vn[k] = nv > 0 ? Fv[k] / nv : Fv[k];
    }
    const double Cu = nu - 1, Cv = nv - 1;
    for (int a = 0; a < 3; a++)
        for (int k = 0; k < 3; k++)
            f[3 * a + k] += -S * Ku * Cu * un[k] * cu[a] + -S * Kv * Cv * vn[k] * cv[a];
    /* the weft term reuses |Fu| unless fix_fv (BaraffMaterial.cpp:141-142) */
    const double nvh = fix_fv ? nv : nu;
    double Du[9], Dv[9];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
        {
            Du[3 * r + c] = un[r] * un[c] / nu + (r == c && nu > 1 ? 1 - 1 / nu : 0);
            Dv[3 * r + c] = vn[r] * vn[c] / nvh + (r == c && nvh > 1 ? 1 - 1 / nvh : 0);
        }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            for (int k = 0; k < 9; k++)
                h[9 * (3 * a + b) + k] +=
                    -S * (Ku * cu[a] * cu[b] * Du[k] + Kv * cv[a] * cv[b] * Dv[k]);
}

void orc_triangles(int nt, const int *tris, const float *coef, const float *area,
                   const double *x, const float stretch_k[3], int fix_fv_norm,
                   double *fint, double *hess)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int t = 0; t < nt; t++)
    {
        const double *x0 = x + 3 * tris[3 * t], *x1 = x + 3 * tris[3 * t + 1],
                     *x2 = x + 3 * tris[3 * t + 2];
        double *f = fint + 9 * (size_t)t, *h = hess + 81 * (size_t)t;
        memset(f, 0, 9 * sizeof(double));
        memset(h, 0, 81 * sizeof(double));
        const float *c = coef + 12 * (size_t)t;
        stretch_term(stretch_k[0], stretch_k[1], area[t], c, c + 3, x0, x1, x2,
                     fix_fv_norm, f, h);
        stretch_term(stretch_k[2], stretch_k[2], area[t], c + 6, c + 9, x0, x1, x2,
                     fix_fv_norm, f, h);
    }
}

/* ------------------------------------------------------------------ dihedral */
static double len_f(const double *a, const double *b)
{
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return (double)(float)sqrt((dx * dx + dy * dy) + dz * dz);
}

int orc_dihedral_rest(int nv, int nt, int ne, const double *pos, const int *tris,
                      const int *edges, float bending_k0, double *factor)
{
    (void)nv;
    /* cDihedralMaterial::Init (DihedralBending.cpp:23-91) with the edge
     * stiffness mean(K, K, K) (BaseBendingMaterial.cpp:47, BaraffCloth.cpp:38-43):
     * float edge lengths, float Heron areas over the triangle's edges
     * (v0 v1), (v1 v2), (v2 v0) (BuildTriangleEdgeId, Triangulator.cpp:11-31),
     * float heights 2 A / e, factor -K e / max(1e-7, h0 + h1) in double. */
    const double K = (double)bending_k0;
    const double kedge = ((K + K) + K) / 3.0;
    float *area = (float *)malloc(sizeof(float) * (size_t)(nt > 0 ? nt : 1));
    for (int t = 0; t < nt; t++)
    {
        const int *v = tris + 3 * (size_t)t;
        const double a = len_f(pos + 3 * (size_t)v[0], pos + 3 * (size_t)v[1]);
        const double b = len_f(pos + 3 * (size_t)v[1], pos + 3 * (size_t)v[2]);
        const double c = len_f(pos + 3 * (size_t)v[2], pos + 3 * (size_t)v[0]);
        const double p = (a + b + c) / 2;
        area[t] = (float)sqrt(p * (p - a) * (p - b) * (p - c));
    }
    for (int e = 0; e < ne; e++)
    {
        const int *ed = edges + 4 * (size_t)e;
        factor[e] = 0.0;
        if (ed[3] < 0)
            continue;
        const float L = (float)len_f(pos + 3 * (size_t)ed[0], pos + 3 * (size_t)ed[1]);
        const float h0 = (2.f * area[ed[2]]) / L, h1 = (2.f * area[ed[3]]) / L;
        const float hs = (h0 + h1) > 1e-7f ? (h0 + h1) : 1e-7f;
        factor[e] = -kedge * (double)L / (double)hs;
    }
    free(area);
    return 0;
}

static void cross3(const double *a, const double *b, double *o)
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double *a, const double *b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

void orc_dihedral(int nv, int ne, const int *stencil, const double *factor,
                  const double *x, const int *ell, double *fint, double *K,
                  double *beta_out, double *grad_out)
{
    (void)nv;
    /* cDihedralMaterial::Update + AssignForceAndMatrix (DihedralBending.cpp:
     * 120-270, 382-488) and cBaseBendingMaterial::GetStiffnessMatrix
     * (BaseBendingMaterial.cpp:13-16): per interior edge with stencil
     * (v0 v1 v2 v3), n0 = (v1 - v0) x (v2 - v1), n1 = (v0 - v1) x (v3 - v0),
     * e = v1 - v0, beta = atan2(e^.(n0^ x n1^), n0^.n1^).  dbeta/dn0 and
     * dbeta/dn1 are taken in closed form, -(e x n0) / (|e| |n0|^2) and
     * (e x n1) / (|e| |n1|^2): the values of the reference's
     * -sign(sin beta) (I - n^ n^T) n'^ / (|n| sqrt(1 - (n0^.n1^)^2))
     * (DihedralBending.cpp:160-222), without its loss of precision as
     * beta -> 0.  Vertex gradients by the reference's chain rule (:225-268).
     * force += ((c beta) g) / 2; stiffness block (a, b) += float((c g_a) g_b^T)
     * (the Hessian is kept as float, DihedralBending.cpp:431), summed in
     * double. */
    for (int e = 0; e < ne; e++)
    {
        const int *s = stencil + 4 * (size_t)e;
        if (s[0] < 0)
        {
            if (beta_out)
                beta_out[e] = 0.0;
            if (grad_out)
                memset(grad_out + 12 * (size_t)e, 0, 12 * sizeof(double));
            continue;
        }
        const double *v0 = x + 3 * (size_t)s[0], *v1 = x + 3 * (size_t)s[1],
                     *v2 = x + 3 * (size_t)s[2], *v3 = x + 3 * (size_t)s[3];
        double ev[3], a21[3], a01[3], a30[3], n0[3], n1[3];
        for (int k = 0; k < 3; k++)
        {
            ev[k] = v1[k] - v0[k];
            a21[k] = v2[k] - v1[k];
            a01[k] = v0[k] - v1[k];
            a30[k] = v3[k] - v0[k];
        }
        cross3(ev, a21, n0);
        cross3(a01, a30, n1);
        const double nn0 = dot3(n0, n0), nn1 = dot3(n1, n1), le = sqrt(dot3(ev, ev));
        double n0h[3], n1h[3], eh[3], cx[3];
        for (int k = 0; k < 3; k++)
        {
            n0h[k] = n0[k] / sqrt(nn0);
            n1h[k] = n1[k] / sqrt(nn1);
            eh[k] = ev[k] / le;
        }
        cross3(n0h, n1h, cx);
        const double beta = atan2(dot3(eh, cx), dot3(n0h, n1h));
        double g0[3], g1[3], t0[3], t1[3];
        cross3(ev, n0, t0);
        cross3(ev, n1, t1);
        for (int k = 0; k < 3; k++)
        {
            g0[k] = -t0[k] / (le * nn0);
            g1[k] = t1[k] / (le * nn1);
        }
        double g[12], d12[3], d31[3], d20[3], d03[3], u[3], w[3];
        for (int k = 0; k < 3; k++)
        {
            d12[k] = v1[k] - v2[k];
            d31[k] = v3[k] - v1[k];
            d20[k] = v2[k] - v0[k];
            d03[k] = v0[k] - v3[k];
        }
        cross3(d12, g0, u);
        cross3(d31, g1, w);
        for (int k = 0; k < 3; k++)
            g[k] = u[k] + w[k];
        cross3(d20, g0, u);
        cross3(d03, g1, w);
        for (int k = 0; k < 3; k++)
            g[3 + k] = u[k] + w[k];
        cross3(a01, g0, g + 6);
        cross3(ev, g1, g + 9);
        const double c = factor[e];
        if (beta_out)
            beta_out[e] = beta;
        if (grad_out)
            memcpy(grad_out + 12 * (size_t)e, g, sizeof(g));
        for (int a = 0; a < 4; a++)
        {
            for (int k = 0; k < 3; k++)
                fint[3 * (size_t)s[a] + k] += ((c * beta) * g[3 * a + k]) / 2;
            const int *row = ell + (size_t)s[a] * W;
            for (int b = 0; b < 4; b++)
            {
                const int slot = row_find(row, s[b]);
                double *blk = K + ((size_t)s[a] * W + slot) * 9;
                for (int r = 0; r < 3; r++)
                    for (int q = 0; q < 3; q++)
                        blk[3 * r + q] += (double)(float)((c * g[3 * a + r]) * g[3 * b + q]);
            }
        }
    }
}

/* ------------------------------------------------------------------ system */
void orc_system(int nv, int nt, const int *tris, const int *ell,
                const double *tri_f, const double *tri_h, const double *kbend,
                const double *mass, double gravity, const double *x,
                const double *xpre, const unsigned char *fixed, double dt,
                float ray_a, float ray_b, double *A, double *b, double *fint)
{
    orc_system_ex(nv, nt, tris, ell, tri_f, tri_h, kbend, NULL, NULL, mass, gravity, x, xpre,
                  fixed, dt, ray_a, ray_b, A, b, fint);
}

void orc_system_ex(int nv, int nt, const int *tris, const int *ell,
                   const double *tri_f, const double *tri_h, const double *kbend,
                   const double *bend_K, const double *bend_f, const double *mass,
                   double gravity, const double *x, const double *xpre,
                   const unsigned char *fixed, double dt, float ray_a, float ray_b,
                   double *A, double *b, double *fint)
{
    /* K = stretch - K_b;  A = (1 + dt a) M + (dt b - dt^2) K
     * (BaraffClothGpu.cu:240-281, 445-483); b = dt^2 (g + f) + M (x - x_pre)
     * (:301-344) */
    double *K = (double *)calloc((size_t)nv * W * 9, sizeof(double));
    for (size_t k = 0; k < (size_t)nv * 3; k++)
        fint[k] = 0.0;
    for (int t = 0; t < nt; t++)
        for (int a = 0; a < 3; a++)
        {
            const int va = tris[3 * t + a];
            for (int k = 0; k < 3; k++)
                fint[3 * va + k] += tri_f[9 * (size_t)t + 3 * a + k];
            for (int bb = 0; bb < 3; bb++)
            {
                const int slot = row_find(ell + (size_t)va * W, tris[3 * t + bb]);
                double *blk = K + ((size_t)va * W + slot) * 9;
                const double *hb = tri_h + 81 * (size_t)t + 9 * (3 * a + bb);
                for (int k = 0; k < 9; k++)
                    blk[k] += hb[k];
            }
        }
    for (int v = 0; v < nv; v++)
        for (int s = 0; s < W; s++)
        {
            const int c = ell[(size_t)v * W + s];
            if (c < 0)
                break;
            const double kb = kbend ? kbend[(size_t)v * W + s] : 0.0;
            double *blk = K + ((size_t)v * W + s) * 9;
            for (int k = 0; k < 3; k++)
            {
                blk[4 * k] -= kb;
                fint[3 * v + k] -= kb * x[3 * c + k];
            }
            /* dihedral bending (CPU cloth, BaraffCloth.cpp:205-244): K += its
             * stiffness, f += its force */
            if (bend_K)
                for (int k = 0; k < 9; k++)
                    blk[k] += bend_K[((size_t)v * W + s) * 9 + k];
        }
    if (bend_f)
        for (size_t k = 0; k < (size_t)nv * 3; k++)
            fint[k] += bend_f[k];
    const double cs = dt * (double)ray_b - dt * dt;
    const double cm = 1 + dt * (double)ray_a;
    for (int v = 0; v < nv; v++)
    {
        for (int s = 0; s < W; s++)
        {
            const int c = ell[(size_t)v * W + s];
            double *ab = A + ((size_t)v * W + s) * 9;
            const double *kb = K + ((size_t)v * W + s) * 9;
            for (int k = 0; k < 9; k++)
                ab[k] = c < 0 ? 0.0 : cs * kb[k];
            if (c == v)
                for (int k = 0; k < 3; k++)
                    ab[4 * k] += cm * mass[v];
            else if (c >= 0 && (fixed[v] || fixed[c]))
                for (int k = 0; k < 9; k++)
                    ab[k] = 0.0;
        }
        for (int k = 0; k < 3; k++)
        {
            const double g = (k == 1) ? gravity * mass[v] : 0.0;
            b[3 * v + k] = fixed[v] ? 0.0
                                    : dt * dt * (g + fint[3 * v + k]) +
                                          mass[v] * (x[3 * v + k] - xpre[3 * v + k]);
        }
    }
    free(K);
}

void orc_spmv(int nv, const int *ell, const double *A, const double *x, double *y)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int v = 0; v < nv; v++)
    {
        double acc[3] = {0, 0, 0};
        for (int s = 0; s < W; s++)
        {
            const int c = ell[(size_t)v * W + s];
            if (c < 0)
                break;
            const double *a = A + ((size_t)v * W + s) * 9;
            for (int r = 0; r < 3; r++)
                acc[r] += a[3 * r] * x[3 * c] + a[3 * r + 1] * x[3 * c + 1] +
                          a[3 * r + 2] * x[3 * c + 2];
        }
        for (int r = 0; r < 3; r++)
            y[3 * v + r] = acc[r];
    }
}

/* deterministic parallel dot: fixed chunks, summed in chunk order */
static double pdot(size_t n, const double *a, const double *b, int nth)
{
    enum { CH = 64 };
    double part[CH] = {0};
    const size_t step = (n + CH - 1) / CH;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nth) schedule(static)
#endif
    for (int c = 0; c < CH; c++)
    {
        double s = 0;
        const size_t lo = (size_t)c * step, hi = lo + step < n ? lo + step : n;
        for (size_t i = lo; i < hi; i++)
            s += a[i] * b[i];
        part[c] = s;
    }
    double s = 0;
    for (int c = 0; c < CH; c++)
        s += part[c];
    (void)nth;
    return s;
}

int orc_pcg(int nv, const int *ell, const double *A, const double *b,
            const unsigned char *fixed, double *x, int max_iters, double rel_tol,
            double *res, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#endif
    const int nth = nthreads > 0 ? nthreads : 1;
    const size_t n3 = (size_t)nv * 3;
    double *Mi = (double *)malloc((size_t)nv * 9 * sizeof(double));
    double *r = (double *)malloc(n3 * sizeof(double));
    double *z = (double *)malloc(n3 * sizeof(double));
    double *p = (double *)malloc(n3 * sizeof(double));
    double *q = (double *)malloc(n3 * sizeof(double));
    /* block-Jacobi inverse of the diagonal blocks (PCGSolver.cu:23-47) */
    for (int v = 0; v < nv; v++)
    {
        const int s = row_find(ell + (size_t)v * W, v);
        const double *a = A + ((size_t)v * W + s) * 9;
        double *m = Mi + 9 * (size_t)v;
        m[0] = a[4] * a[8] - a[5] * a[7];
        m[1] = a[2] * a[7] - a[1] * a[8];
        m[2] = a[1] * a[5] - a[2] * a[4];
        m[3] = a[5] * a[6] - a[3] * a[8];
        m[4] = a[0] * a[8] - a[2] * a[6];
        m[5] = a[2] * a[3] - a[0] * a[5];
        m[6] = a[3] * a[7] - a[4] * a[6];
        m[7] = a[1] * a[6] - a[0] * a[7];
        m[8] = a[0] * a[4] - a[1] * a[3];
        const double det = a[0] * m[0] + a[1] * m[3] + a[2] * m[6];
        for (int k = 0; k < 9; k++)
            m[k] /= det;
    }
    for (int v = 0; v < nv; v++)
        if (fixed[v])
            x[3 * v] = x[3 * v + 1] = x[3 * v + 2] = 0.0;
    orc_spmv(nv, ell, A, x, q);
    for (size_t i = 0; i < n3; i++)
        r[i] = fixed[i / 3] ? 0.0 : b[i] - q[i];
    for (int v = 0; v < nv; v++)
        for (int k = 0; k < 3; k++)
        {
            const double *m = Mi + 9 * (size_t)v + 3 * k;
            z[3 * v + k] = m[0] * r[3 * v] + m[1] * r[3 * v + 1] + m[2] * r[3 * v + 2];
        }
    memcpy(p, z, n3 * sizeof(double));
    double rho = pdot(n3, r, z, nth);
    const double bb = pdot(n3, b, b, nth);
    double rr = pdot(n3, r, r, nth);
    int it = 0;
    while (it < max_iters && !(rr <= rel_tol * rel_tol * bb))
    {
        orc_spmv(nv, ell, A, p, q);
        const double pq = pdot(n3, p, q, nth);
        if (pq == 0.0)
            break;
        const double alpha = rho / pq;
        for (size_t i = 0; i < n3; i++)
        {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        for (int v = 0; v < nv; v++)
            for (int k = 0; k < 3; k++)
            {
                const double *m = Mi + 9 * (size_t)v + 3 * k;
                z[3 * v + k] = m[0] * r[3 * v] + m[1] * r[3 * v + 1] + m[2] * r[3 * v + 2];
            }
        const double rho2 = pdot(n3, r, z, nth);
        rr = pdot(n3, r, r, nth);
        const double beta = rho == 0.0 ? 0.0 : rho2 / rho;
        rho = rho2;
        for (size_t i = 0; i < n3; i++)
            p[i] = z[i] + beta * p[i];
        it++;
    }
    if (res)
        *res = sqrt(rr);
    free(Mi);
    free(r);
    free(z);
    free(p);
    free(q);
    return it;
}

/* ------------------------------------------------------------------ collisions */
/* The CPU cloth's collision handling against a static kinematic body
 * (cBVHCollisionDetecter::PerformCD, src/sim/collision/BVHCollisionDetecter.cpp;
 * cBaraffCloth::PrepareCollisionHessian and Repulsion, src/sim/cloth/
 * BaraffCloth.cpp:614-990), with the cloth as object 0 and the body as 1. */

static void nrm3(const double *a, double *o)
{
    const double n = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    for (int k = 0; k < 3; k++)
        o[k] = a[k] / n;
}

static void tri_normal(const double *x, const int *t, double *n)
{
    /* cBaseObject::UpdateTriangleNormal (BaseObject.cpp:119-131) */
    const double *v0 = x + 3 * (size_t)t[0], *v1 = x + 3 * (size_t)t[1],
                 *v2 = x + 3 * (size_t)t[2];
    double a[3], b[3], c[3];
    for (int k = 0; k < 3; k++)
    {
        a[k] = v1[k] - v0[k];
        b[k] = v2[k] - v1[k];
    }
    cross3(a, b, c);
    nrm3(c, n);
}

void orc_body_normals(int nv, int nt, const double *pos, const int *tris, double *tnormal,
                      double *vnormal)
{
    /* cKinematicBody::Init tail: CalcTriangleInitArea, UpdateTriangleNormal,
     * UpdateVertexNormalFromTriangleNormal (BaseObject.cpp:119-160, 292-304):
     * area-weighted sum of triangle normals, normalised. */
    memset(vnormal, 0, sizeof(double) * 3 * (size_t)nv);
    for (int t = 0; t < nt; t++)
    {
        const int *tv = tris + 3 * (size_t)t;
        tri_normal(pos, tv, tnormal + 3 * (size_t)t);
        const double *p0 = pos + 3 * (size_t)tv[0], *p1 = pos + 3 * (size_t)tv[1],
                     *p2 = pos + 3 * (size_t)tv[2];
        /* cMathUtil::CalcTriangleArea (MathUtil2.cpp:344-357): float */
        double e1[3], e2[3], c[3];
        for (int k = 0; k < 3; k++)
        {
            e1[k] = p1[k] - p0[k];
            e2[k] = p2[k] - p0[k];
        }
        cross3(e1, e2, c);
        const double area = (double)(float)(0.5 * sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++)
                vnormal[3 * (size_t)tv[i] + k] += tnormal[3 * (size_t)t + k] * area;
    }
    for (int v = 0; v < nv; v++)
    {
        double *n = vnormal + 3 * (size_t)v;
        const double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (l > 0)
            for (int k = 0; k < 3; k++)
                n[k] /= l;
    }
}

static float clampf01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }

/* ClosestPtPointTriangle (BVHCollisionDetecter.cpp:17-86): Ericson's region
 * test with the dot products rounded to float, as the reference keeps them. */
static void closest_pt_tri(const double *p, const double *a, const double *b, const double *c,
                           double *q, float *bary)
{
    double ab[3], ac[3], ap[3], bp[3], cp[3];
    for (int k = 0; k < 3; k++)
    {
        ab[k] = b[k] - a[k];
        ac[k] = c[k] - a[k];
        ap[k] = p[k] - a[k];
        bp[k] = p[k] - b[k];
        cp[k] = p[k] - c[k];
    }
    bary[0] = bary[1] = bary[2] = 0.f;
    const float d1 = (float)dot3(ab, ap), d2 = (float)dot3(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f)
    {
        bary[0] = 1;
        memcpy(q, a, 3 * sizeof(double));
        return;
    }
    const float d3 = (float)dot3(ab, bp), d4 = (float)dot3(ac, bp);
    if (d3 >= 0.0f && d4 <= d3)
    {
        bary[1] = 1;
        memcpy(q, b, 3 * sizeof(double));
        return;
    }
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f)
    {
        const float v = d1 / (d1 - d3);
        bary[0] = 1 - v;
        bary[1] = v;
        for (int k = 0; k < 3; k++)
            q[k] = a[k] + (double)v * ab[k];
        return;
    }
    const float d5 = (float)dot3(ab, cp), d6 = (float)dot3(ac, cp);
    if (d6 >= 0.0f && d5 <= d6)
    {
        bary[2] = 1;
        memcpy(q, c, 3 * sizeof(double));
        return;
    }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f)
    {
        const float w = d2 / (d2 - d6);
        bary[0] = 1 - w;
        bary[2] = w;
        for (int k = 0; k < 3; k++)
            q[k] = a[k] + (double)w * ac[k];
        return;
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
    {
        const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        bary[1] = 1 - w;
        bary[2] = w;
        for (int k = 0; k < 3; k++)
            q[k] = b[k] + (double)w * (c[k] - b[k]);
        return;
    }
    const float denom = 1.0f / (va + vb + vc);
    const float v = vb * denom, w = vc * denom;
    bary[0] = 1 - v - w;
    bary[1] = v;
    bary[2] = w;
    for (int k = 0; k < 3; k++)
        q[k] = a[k] + ab[k] * (double)v + ac[k] * (double)w;
}

/* EdgeEdgeDist (BVHCollisionDetecter.cpp:100-175): closest points of two
 * segments, Ericson's method with float scalars; s on [p1 q1], t on [p2 q2]. */
static void edge_edge(const double *p1, const double *q1, const double *p2, const double *q2,
                      float *s_out, float *t_out)
{
    double d1[3], d2[3], r[3];
    for (int k = 0; k < 3; k++)
    {
        d1[k] = q1[k] - p1[k];
        d2[k] = q2[k] - p2[k];
        r[k] = p1[k] - p2[k];
    }
    const float a = (float)dot3(d1, d1), e = (float)dot3(d2, d2), f = (float)dot3(d2, r);
    const float EPS = 1e-10f;
    float s = 0, t = 0;
    if (a <= EPS && e <= EPS)
        s = t = 0.0f; /* the reference goes on to the next test */
    if (a <= EPS)
    {
        s = 0.0f;
        t = clampf01(f / e);
    }
    else
    {
        const float c = (float)dot3(d1, r);
        if (e <= EPS)
        {
            t = 0.0f;
            s = clampf01(-c / a);
        }
        else
        {
            const float b = (float)dot3(d1, d2);
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
    *s_out = s;
    *t_out = t;
}

typedef struct
{
    int a, b;
} ipair;

static int cmp_ipair(const void *x, const void *y)
{
    const ipair *p = (const ipair *)x, *q = (const ipair *)y;
    if (p->a != q->a)
        return p->a < q->a ? -1 : 1;
    return p->b < q->b ? -1 : (p->b > q->b ? 1 : 0);
}

static size_t sort_unique(ipair *v, size_t n)
{
    if (n == 0)
        return 0;
    qsort(v, n, sizeof(ipair), cmp_ipair);
    size_t m = 1;
    for (size_t i = 1; i < n; i++)
        if (cmp_ipair(&v[i], &v[m - 1]) != 0)
            v[m++] = v[i];
    return m;
}

/* triangle -> its edges (v0 v1), (v1 v2), (v2 v0) (BuildTriangleEdgeId) */
static void tri_edges(int nt, int ne, const int *tris, const int *edges, int *te)
{
    for (int i = 0; i < 3 * nt; i++)
        te[i] = -1;
    for (int e = 0; e < ne; e++)
        for (int s = 2; s <= 3; s++)
        {
            const int t = edges[4 * (size_t)e + s];
            if (t < 0)
                continue;
            const int *v = tris + 3 * (size_t)t;
            for (int k = 0; k < 3; k++)
            {
                const int a = v[k], b = v[(k + 1) % 3];
                const int lo = a < b ? a : b, hi = a < b ? b : a;
                if (lo == edges[4 * (size_t)e] && hi == edges[4 * (size_t)e + 1])
                    te[3 * (size_t)t + k] = e;
            }
        }
}

static void aabb5(const double *x, const int *t, double *lo, double *hi)
{
    /* leaf AABB of cObjBVH::UpdateAABB: the triangle's box grown by 5 mm */
    for (int k = 0; k < 3; k++)
    {
        double mn = x[3 * (size_t)t[0] + k], mx = mn;
        for (int i = 1; i < 3; i++)
        {
            const double v = x[3 * (size_t)t[i] + k];
            mn = v < mn ? v : mn;
            mx = v > mx ? v : mx;
        }
        lo[k] = mn - 5e-3;
        hi[k] = mx + 5e-3;
    }
}

int orc_contacts(int nv, int nt, int ne, const double *x, const int *tris, const int *edges,
                 int bnv, int bnt, int bne, const double *bpos, const int *btris,
                 const int *bedges, const double *btn, const double *bvn, int max_pt,
                 int *pt_i, double *pt_d, int *n_pt, int max_ee, int *ee_i, double *ee_d,
                 int *n_ee)
{
    (void)nv;
    (void)bnv;
    /* broad phase: triangle pairs whose grown boxes meet (the BVH pair walk
     * reaches exactly these leaves) */
    double *tn = (double *)malloc(sizeof(double) * 3 * (size_t)nt);
    double *clo = (double *)malloc(sizeof(double) * 3 * (size_t)nt),
           *chi = (double *)malloc(sizeof(double) * 3 * (size_t)nt);
    double *blo = (double *)malloc(sizeof(double) * 3 * (size_t)bnt),
           *bhi = (double *)malloc(sizeof(double) * 3 * (size_t)bnt);
    for (int t = 0; t < nt; t++)
    {
        tri_normal(x, tris + 3 * (size_t)t, tn + 3 * (size_t)t);
        aabb5(x, tris + 3 * (size_t)t, clo + 3 * (size_t)t, chi + 3 * (size_t)t);
    }
    for (int t = 0; t < bnt; t++)
        aabb5(bpos, btris + 3 * (size_t)t, blo + 3 * (size_t)t, bhi + 3 * (size_t)t);
    /* body triangles binned on a uniform grid (only to find the box pairs
     * faster; the set of pairs is that of the all-pairs test) */
    double g0[3] = {1e300, 1e300, 1e300}, g1[3] = {-1e300, -1e300, -1e300}, cell = 1e-3;
    for (int t = 0; t < bnt; t++)
        for (int k = 0; k < 3; k++)
        {
            const double l = blo[3 * (size_t)t + k], h = bhi[3 * (size_t)t + k];
            g0[k] = l < g0[k] ? l : g0[k];
            g1[k] = h > g1[k] ? h : g1[k];
            cell = (h - l) > cell ? (h - l) : cell;
        }
    int gd[3];
    for (;;)
    {
        long long tot = 1;
        for (int k = 0; k < 3; k++)
        {
            gd[k] = (int)ceil((g1[k] - g0[k]) / cell);
            gd[k] = gd[k] < 1 ? 1 : gd[k];
            tot *= gd[k];
        }
        if (tot <= (1 << 22))
            break;
        cell *= 1.5;
    }
#define ORC_CELL(v, k)                                                                        \
    (floor(((v) - g0[k]) / cell) < 0.0                                                        \
         ? 0                                                                                  \
         : (floor(((v) - g0[k]) / cell) >= (double)gd[k] ? gd[k] - 1                          \
                                                          : (int)floor(((v) - g0[k]) / cell)))
    const size_t ncell = (size_t)gd[0] * gd[1] * gd[2];
    int *coff = (int *)calloc(ncell + 1, sizeof(int));
    for (int pass = 0; pass < 2; pass++)
    {
        int *ctr = pass ? (int *)calloc(ncell, sizeof(int)) : NULL;
        for (int t = 0; t < bnt; t++)
        {
            int i0[3], i1[3];
            for (int k = 0; k < 3; k++)
            {
                i0[k] = ORC_CELL(blo[3 * (size_t)t + k], k);
                i1[k] = ORC_CELL(bhi[3 * (size_t)t + k], k);
            }
            for (int iz = i0[2]; iz <= i1[2]; iz++)
                for (int iy = i0[1]; iy <= i1[1]; iy++)
                    for (int ix = i0[0]; ix <= i1[0]; ix++)
                    {
                        const size_t c = ((size_t)iz * gd[1] + iy) * gd[0] + ix;
                        if (!pass)
                            coff[c + 1]++;
                        else
                            ctr[c]++;
                    }
        }
        if (!pass)
            for (size_t c = 0; c < ncell; c++)
                coff[c + 1] += coff[c];
        free(ctr);
    }
    int *ctri = (int *)malloc(sizeof(int) * ((size_t)coff[ncell] + 1));
    {
        int *fill = (int *)calloc(ncell, sizeof(int));
        for (int t = 0; t < bnt; t++)
        {
            int i0[3], i1[3];
            for (int k = 0; k < 3; k++)
            {
                i0[k] = ORC_CELL(blo[3 * (size_t)t + k], k);
                i1[k] = ORC_CELL(bhi[3 * (size_t)t + k], k);
            }
            for (int iz = i0[2]; iz <= i1[2]; iz++)
                for (int iy = i0[1]; iy <= i1[1]; iy++)
                    for (int ix = i0[0]; ix <= i1[0]; ix++)
                    {
                        const size_t c = ((size_t)iz * gd[1] + iy) * gd[0] + ix;
                        ctri[coff[c] + fill[c]++] = t;
                    }
        }
        free(fill);
    }
    size_t cap = 1024, np = 0;
    ipair *tp = (ipair *)malloc(sizeof(ipair) * cap);
    for (int T = 0; T < nt; T++)
    {
        const double *al = clo + 3 * (size_t)T, *ah = chi + 3 * (size_t)T;
        int i0[3], i1[3], outside = 0;
        for (int k = 0; k < 3; k++)
        {
            if (ah[k] < g0[k] || al[k] > g1[k])
                outside = 1;
            i0[k] = ORC_CELL(al[k], k);
            i1[k] = ORC_CELL(ah[k], k);
        }
        if (outside)
            continue;
        const size_t np0 = np;
        for (int iz = i0[2]; iz <= i1[2]; iz++)
            for (int iy = i0[1]; iy <= i1[1]; iy++)
                for (int ix = i0[0]; ix <= i1[0]; ix++)
                {
                    const size_t c = ((size_t)iz * gd[1] + iy) * gd[0] + ix;
                    for (int q = coff[c]; q < coff[c + 1]; q++)
                    {
                        const int t = ctri[q];
                        const double *bl = blo + 3 * (size_t)t, *bh = bhi + 3 * (size_t)t;
                        if (al[0] <= bh[0] && ah[0] >= bl[0] && al[1] <= bh[1] && ah[1] >= bl[1] &&
                            al[2] <= bh[2] && ah[2] >= bl[2])
                        {
                            if (np == cap)
                            {
                                cap *= 2;
                                tp = (ipair *)realloc(tp, sizeof(ipair) * cap);
                            }
                            tp[np].a = T;
                            tp[np].b = t;
                            np++;
                        }
                    }
                }
        np = np0 + sort_unique(tp + np0, np - np0);
    }
#undef ORC_CELL
    free(coff);
    free(ctri);
    int *te = (int *)malloc(sizeof(int) * 3 * (size_t)nt);
    int *bte = (int *)malloc(sizeof(int) * 3 * (size_t)bnt);
    tri_edges(nt, ne, tris, edges, te);
    tri_edges(bnt, bne, btris, bedges, bte);
    ipair *p01 = (ipair *)malloc(sizeof(ipair) * (3 * np + 1));
    ipair *p10 = (ipair *)malloc(sizeof(ipair) * (3 * np + 1));
    ipair *pee = (ipair *)malloc(sizeof(ipair) * (9 * np + 1));
    for (size_t i = 0; i < np; i++)
    {
        const int T = tp[i].a, t = tp[i].b;
        for (int k = 0; k < 3; k++)
        {
            p01[3 * i + k].a = tris[3 * (size_t)T + k];
            p01[3 * i + k].b = t;
            p10[3 * i + k].a = btris[3 * (size_t)t + k];
            p10[3 * i + k].b = T;
        }
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
            {
                pee[9 * i + 3 * a + b].a = te[3 * (size_t)T + a];
                pee[9 * i + 3 * a + b].b = bte[3 * (size_t)t + b];
            }
    }
    const size_t n01 = sort_unique(p01, 3 * np), n10 = sort_unique(p10, 3 * np),
                 nee = sort_unique(pee, 9 * np);
    int cpt = 0, cee = 0, overflow = 0;
    /* narrow phase, point-triangle: cloth points against body triangles, then
     * body points against cloth triangles (distance under 3 mm) */
    for (int pass = 0; pass < 2; pass++)
    {
        const ipair *pl = pass == 0 ? p01 : p10;
        const size_t n = pass == 0 ? n01 : n10;
        for (size_t i = 0; i < n; i++)
        {
            const int p = pl[i].a, t = pl[i].b;
            const double *pt = pass == 0 ? x + 3 * (size_t)p : bpos + 3 * (size_t)p;
            const int *tv = pass == 0 ? btris + 3 * (size_t)t : tris + 3 * (size_t)t;
            const double *tx = pass == 0 ? bpos : x;
            double q[3], normal[3], dv[3];
            float bary[3];
            closest_pt_tri(pt, tx + 3 * (size_t)tv[0], tx + 3 * (size_t)tv[1],
                           tx + 3 * (size_t)tv[2], q, bary);
            if (pass == 0)
            {
                memcpy(normal, btn + 3 * (size_t)t, sizeof(normal));
                for (int k = 0; k < 3; k++)
                    dv[k] = pt[k] - q[k];
            }
            else
            {
                memcpy(normal, tn + 3 * (size_t)t, sizeof(normal));
                if (dot3(normal, bvn + 3 * (size_t)p) < 0)
                    for (int k = 0; k < 3; k++)
                        normal[k] *= -1;
                for (int k = 0; k < 3; k++)
                    dv[k] = q[k] - pt[k];
            }
            if (sqrt(dot3(dv, dv)) < 3e-3)
            {
                if (cpt >= max_pt)
                {
                    overflow = 1;
                    continue;
                }
                pt_i[3 * cpt + 0] = pass == 0 ? 1 : 0;
                pt_i[3 * cpt + 1] = p;
                pt_i[3 * cpt + 2] = t;
                for (int k = 0; k < 3; k++)
                    pt_d[7 * cpt + k] = normal[k];
                pt_d[7 * cpt + 3] = (double)(float)dot3(dv, normal);
                for (int k = 0; k < 3; k++)
                    pt_d[7 * cpt + 4 + k] = (double)bary[k];
                cpt++;
            }
        }
    }
    /* narrow phase, edge-edge: cloth edge e0 against body edge e1 */
    for (size_t i = 0; i < nee; i++)
    {
        const int e0 = pee[i].a, e1 = pee[i].b;
        const double *p0 = x + 3 * (size_t)edges[4 * (size_t)e0],
                     *p1 = x + 3 * (size_t)edges[4 * (size_t)e0 + 1];
        const double *p2 = bpos + 3 * (size_t)bedges[4 * (size_t)e1],
                     *p3 = bpos + 3 * (size_t)bedges[4 * (size_t)e1 + 1];
        float s, t;
        edge_edge(p0, p1, p2, p3, &s, &t);
        double c0[3], c1[3], d01[3], d23[3], cr[3], normal[3], on[3], dv[3];
        const float s1 = 1 - s, t1 = 1 - t;
        for (int k = 0; k < 3; k++)
        {
            c0[k] = (double)s1 * p0[k] + (double)s * p1[k];
            c1[k] = (double)t1 * p2[k] + (double)t * p3[k];
            d01[k] = p1[k] - p0[k];
            d23[k] = p3[k] - p2[k];
        }
        cross3(d01, d23, cr);
        nrm3(cr, normal);
        const int bt0 = bedges[4 * (size_t)e1 + 2], bt1 = bedges[4 * (size_t)e1 + 3];
        for (int k = 0; k < 3; k++)
            on[k] = btn[3 * (size_t)bt0 + k] + (bt1 != -1 ? btn[3 * (size_t)bt1 + k] : 0.0);
        {
            double o2[3];
            nrm3(on, o2);
            if (dot3(o2, normal) < 0)
                for (int k = 0; k < 3; k++)
                    normal[k] *= -1;
        }
        for (int k = 0; k < 3; k++)
            dv[k] = c0[k] - c1[k];
        if (sqrt(dot3(dv, dv)) < 3e-3)
        {
            if (cee >= max_ee)
            {
                overflow = 1;
                continue;
            }
            ee_i[3 * cee + 0] = 1;
            ee_i[3 * cee + 1] = e0;
            ee_i[3 * cee + 2] = e1;
            for (int k = 0; k < 3; k++)
                ee_d[6 * cee + k] = normal[k];
            ee_d[6 * cee + 3] = (double)(float)dot3(dv, normal);
            ee_d[6 * cee + 4] = (double)s;
            ee_d[6 * cee + 5] = (double)t;
            cee++;
        }
    }
    *n_pt = cpt;
    *n_ee = cee;
    free(tn);
    free(clo);
    free(chi);
    free(blo);
    free(bhi);
    free(tp);
    free(te);
    free(bte);
    free(p01);
    free(p10);
    free(pee);
    return overflow ? -1 : 0;
}

void orc_contact_hessian(int nv, const int *tris, const int *ell, int n_pt, const int *pt_i,
                         const double *pt_d, double *H)
{
    (void)nv;
    /* PrepareCollisionHessian (BaraffCloth.cpp:928-990): 1e-2 dC/dx dC/dx^T per
     * point-triangle contact, dC/dx = N at a cloth point, -b_i N at the
     * vertices of a cloth triangle; added to the system matrix unscaled */
    for (int c = 0; c < n_pt; c++)
    {
        const double *N = pt_d + 7 * (size_t)c;
        int vid[3];
        double w[3];
        int nvtx;
        if (pt_i[3 * c] == 1)
        {
            vid[0] = pt_i[3 * c + 1];
            w[0] = 1.0;
            nvtx = 1;
        }
        else
        {
            const int *tv = tris + 3 * (size_t)pt_i[3 * c + 2];
            for (int i = 0; i < 3; i++)
            {
                vid[i] = tv[i];
                w[i] = -pt_d[7 * (size_t)c + 4 + i];
            }
            nvtx = 3;
        }
        for (int i = 0; i < nvtx; i++)
            for (int j = 0; j < nvtx; j++)
            {
                const int slot = row_find(ell + (size_t)vid[i] * W, vid[j]);
                double *blk = H + ((size_t)vid[i] * W + slot) * 9;
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++)
                        blk[3 * a + b] += 1e-2 * ((w[i] * N[a]) * (w[j] * N[b]));
            }
    }
}

void orc_repulsion(int nv, const int *tris, const int *edges, const double *mass,
                   const float stretch_k[3], double dt, int n_pt, const int *pt_i,
                   const double *pt_d, int n_ee, const int *ee_i, const double *ee_d,
                   double *dx)
{
    (void)nv;
    /* cBaraffCloth::Repulsion (BaraffCloth.cpp:626-926): Bridson-style
     * impulses along the contact normals, edge-edge contacts first, then
     * point-triangle ones, each reading dx as the earlier ones left it.
     * |Ic| = m |vn| / 2 unless vn > 0.01; |Ir| = min(dt K d, m (0.1 d / dt - vn))
     * unless vn > 0.1 d / dt, d = 3 mm - depth, K = mean stretch stiffness;
     * increments scaled by 0.1. */
    const float kmean = ((stretch_k[0] + stretch_k[1]) + stretch_k[2]) / 3.0f;
    const double K = (double)kmean * 1;
    const double v_thre = 0.01;
    const double scale = (double)0.1f;
    for (int c = 0; c < n_ee; c++)
    {
        /* the edge barycentric coordinates are float, and so is the
         * arithmetic on them alone */
        const double *N = ee_d + 6 * (size_t)c;
        const float a = (float)ee_d[6 * (size_t)c + 4], b = (float)ee_d[6 * (size_t)c + 5];
        const float a1 = 1 - a;
        const int e = ee_i[3 * c + 1];
        const int v0 = edges[4 * (size_t)e], v1 = edges[4 * (size_t)e + 1];
        double vrel[3];
        for (int k = 0; k < 3; k++)
            vrel[k] = ((double)a1 * dx[3 * (size_t)v0 + k] + (double)a * dx[3 * (size_t)v1 + k]) / dt;
        const double m = mass[v0] + mass[v1];
        const double vn = dot3(vrel, N);
        const double Ic = vn > v_thre ? 0 : m * fabs(vn) / 2;
        const double d = 3e-3 - ee_d[6 * (size_t)c + 3];
        double Ir = 0;
        if (!(vn > 0.1f * d / dt))
        {
            const double Ir0 = dt * K * d, Ir1 = m * (0.1f * d / dt - vn);
            Ir = Ir0 < Ir1 ? Ir0 : Ir1;
        }
        const double I = Ic + Ir;
        const float den = 1 + a * a + (1 - a) * (1 - a) + b * b + (1 - b) * (1 - b);
        const double It = 2 * I / (double)den;
        for (int k = 0; k < 3; k++)
        {
            dx[3 * (size_t)v0 + k] += scale * dt * (double)a1 * It / m * N[k];
            dx[3 * (size_t)v1 + k] += scale * dt * (double)a * It / m * N[k];
        }
    }
    for (int c = 0; c < n_pt; c++)
    {
        const double *N = pt_d + 7 * (size_t)c;
        const double *bary = pt_d + 7 * (size_t)c + 4;
        double vrel[3], m;
        const int *tv = tris + 3 * (size_t)pt_i[3 * c + 2];
        if (pt_i[3 * c] == 1)
        {
            const int p = pt_i[3 * c + 1];
            for (int k = 0; k < 3; k++)
                vrel[k] = dx[3 * (size_t)p + k] / dt;
            m = mass[p];
        }
        else
        {
            for (int k = 0; k < 3; k++)
                vrel[k] = (dx[3 * (size_t)tv[0] + k] * bary[0] + dx[3 * (size_t)tv[1] + k] * bary[1] +
                           dx[3 * (size_t)tv[2] + k] * bary[2]) /
                          dt;
            m = mass[tv[0]] + mass[tv[1]] + mass[tv[2]];
        }
        const double vn = dot3(vrel, N);
        const double Ic = vn > v_thre ? 0 : m * fabs(vn) / 2;
        const double d = 3e-3 - pt_d[7 * (size_t)c + 3];
        double Ir = 0;
        if (!(vn > 0.1 * d / dt))
        {
            const double Ir0 = dt * K * d, Ir1 = m * (0.1 * d / dt - vn);
            Ir = Ir0 < Ir1 ? Ir0 : Ir1;
        }
        const double I = Ic + Ir;
        const double It = 2 * I / (1 + dot3(bary, bary));
        if (pt_i[3 * c] == 1)
        {
            const int p = pt_i[3 * c + 1];
            for (int k = 0; k < 3; k++)
                dx[3 * (size_t)p + k] += scale * (dt * It / m * N[k]);
        }
        else
            for (int i = 0; i < 3; i++)
                for (int k = 0; k < 3; k++)
                    dx[3 * (size_t)tv[i] + k] += scale * (dt * bary[i] * It / m * N[k]);
    }
}
