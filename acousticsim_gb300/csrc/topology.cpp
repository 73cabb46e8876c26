// Host-side topology and init-time tables; see topology.h.
#include "topology.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <set>
#include <utility>

namespace cloth {

namespace {

// 0.5 * |(p1 - p0) x (p2 - p0)| in double, rounded to float
// (cMathUtil::CalcTriangleArea3d, src/utils/MathUtil2.cpp:353-357).
float triangle_area(const double *p0, const double *p1, const double *p2)
{
    double a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    double b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double c0 = a[1] * b[2] - a[2] * b[1];
    double c1 = a[2] * b[0] - a[0] * b[2];
    double c2 = a[0] * b[1] - a[1] * b[0];
    double n2 = c0 * c0 + c1 * c1;
    n2 = n2 + c2 * c2;
    return float(0.5 * std::sqrt(n2));
}

// CalcCotangent (src/sim/cloth/QBendingMaterial.cpp:11-19): the dot products
// are rounded to float and the rest is float arithmetic.
double cotangent(const double *A, const double *B, const double *C)
{
    double ab[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
    double ac[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
    float abac = float((ab[0] * ac[0] + ab[1] * ac[1]) + ab[2] * ac[2]);
    float abab = float((ab[0] * ab[0] + ab[1] * ab[1]) + ab[2] * ab[2]);
    float acac = float((ac[0] * ac[0] + ac[1] * ac[1]) + ac[2] * ac[2]);
    float den = abab * acac - abac * abac;
    return double(abac / std::sqrt(den));
}

// CalcCotangentCoeff (QBendingMaterial.cpp:20-43). The reference calls
// cMathUtil::Clamp on the four cotangents and discards the returned values,
// so no clamping takes effect; the same holds here.
void cotangent_coeff(const double *x0, const double *x1, const double *x2,
                     const double *x3, double out[4])
{
    double c01 = cotangent(x0, x1, x2);
    double c02 = cotangent(x0, x1, x3);
    double c03 = cotangent(x1, x0, x2);
    double c04 = cotangent(x1, x0, x3);
    out[0] = c03 + c04;
    out[1] = c01 + c02;
    out[2] = -c01 - c03;
    out[3] = -c02 - c04;
}

// CalcBaraffStretchCoef (src/sim/cloth/BaraffMaterial.cpp:18-32): the inverse
// reference-shape matrix entries are rounded to float first.
void stretch_coef(const double m[2][2], float cu[3], float cv[3])
{
    float a = float(m[0][0]), b = float(m[0][1]);
    float c = float(m[1][0]), d = float(m[1][1]);
    cu[0] = -a - c;
    cu[1] = a;
    cu[2] = c;
    cv[0] = -b - d;
    cv[1] = b;
    cv[2] = d;
}

int other_vertex(const int *tri, int v0, int v1)
{
    // SelectAnotherVerteix (BaseCloth.cpp:281-290): the remaining member of
    // the triangle's vertex set.
    int best = -1;
    for (int k = 0; k < 3; k++)
        if (tri[k] != v0 && tri[k] != v1)
            best = (best < 0) ? tri[k] : std::min(best, tri[k]);
    return best;
}

} // namespace

bool build_grid(const GridDesc &g, Mesh &m, std::string &err)
{
    const int hd = g.subdiv[0], wd = g.subdiv[1];
    if (hd < 1 || wd < 1 || !(g.size[0] > 0) || !(g.size[1] > 0))
    {
        err = "grid: subdivision must be >= 1 and cloth_size > 0";
        return false;
    }
    int rot = int(g.uv_rotation_deg);
    if (rot != 0 && rot != 45 && rot != 90)
    {
        err = "grid: cloth_uv_rotation must be 0, 45 or 90";
        return false;
    }
    const double height = g.size[0], width = g.size[1];
    const double unit_h = height / hd, unit_w = width / wd;
    const int nhl = hd + 1;
    m.nv = (wd + 1) * nhl;
    m.nt = 2 * wd * hd;
    m.ne = (wd + 1) * hd + nhl * wd + hd * wd;
    m.pos.assign(size_t(m.nv) * 3, 0.0);
    m.uv.assign(size_t(m.nv) * 2, 0.f);
    m.tris.clear();
    m.tris.reserve(size_t(m.nt) * 3);
    m.edges.assign(size_t(m.ne) * 4, -2);

    // BuildRectVertices (Triangulator.cpp:395-457), then the init transform
    // (identity rotation, translation init_pos) and the material coordinates
    // (RotateMaterialCoordsAfterReset, :621-658).
    const float ang = float(g.uv_rotation_deg / 180.0 * M_PI);
    const float rc = float(std::cos(double(ang))), rs = float(std::sin(double(ang)));
    for (int i = 0; i < wd + 1; i++)
        for (int j = 0; j < nhl; j++)
        {
            int v = i * nhl + j;
            double p[3] = {i * unit_w - width / 2, j * unit_h - height / 2, 0.0};
            for (int k = 0; k < 3; k++)
                p[k] = p[k] + g.init_pos[k];
            for (int k = 0; k < 3; k++)
                m.pos[size_t(v) * 3 + k] = p[k];
            float px = float(p[0] + (-g.init_pos[0]));
            float py = float(p[1] + (-g.init_pos[1]));
            m.uv[size_t(v) * 2 + 0] = rc * px + (-rs) * py;
            m.uv[size_t(v) * 2 + 1] = rs * px + rc * py;
        }

    // Triangles and edges (Triangulator.cpp:180-390).
    const int epr = 2 * hd + nhl;
    auto set_edge = [&](int id, int a, int b, int t0, int t1) {
        int *e = &m.edges[size_t(id) * 4];
        e[0] = a;
        e[1] = b;
        e[2] = t0;
        e[3] = t1;
    };
    for (int row = 0; row < wd; row++)
        for (int col = 0; col < hd; col++)
        {
            int lu = row * nhl + col, ru = lu + 1, ld = lu + nhl, rd = ld + 1;
            bool even = (row + col) % 2 == 0;
            int top = row * epr + col;
            int left = epr * row + hd + col * 2;
            int skew = left + 1, right = skew + 1, bottom = top + epr;
            if (even)
            {
                int t[6] = {lu, ld, rd, lu, rd, ru};
                m.tris.insert(m.tris.end(), t, t + 6);
            }
            else
            {
                int t[6] = {lu, ld, ru, ld, rd, ru};
                m.tris.insert(m.tris.end(), t, t + 6);
            }
            int T = int(m.tris.size() / 3);
            if (even)
                set_edge(skew, lu, rd, T - 2, T - 1);
            else
                set_edge(skew, ru, ld, T - 2, T - 1);
            {
                int t0 = even ? T - 2 : T - 1;
                int t1 = (row == wd - 1) ? -1 : t0 + hd * 2;
                set_edge(bottom, ld, rd, t0, t1);
            }
            {
                int t0 = T - 1;
                int t1 = (col == hd - 1) ? -1 : t0 + 1;
                set_edge(right, ru, rd, t0, t1);
            }
            if (row == 0)
                set_edge(top, lu, ru, even ? T - 1 : T - 2, -1);
            if (col == 0)
                set_edge(left, lu, ld, T - 2, -1);
        }
    for (int e = 0; e < m.ne; e++)
        if (m.edges[size_t(e) * 4] < 0)
        {
            err = "grid: edge numbering left a hole";
            return false;
        }
    return true;
}

bool derive_edges(Mesh &m, std::string &err)
{
    // cObjUtil::BuildEdge (src/utils/ObjUtil.cpp:140-240): one edge per
    // vertex pair (v0 < v1), numbered in ascending (v0, v1) order; tri0/tri1
    // are the first/second triangle (in triangle order) that uses the pair.
    std::map<std::pair<int, int>, std::pair<int, int>> info;
    for (int t = 0; t < m.nt; t++)
    {
        const int *v = &m.tris[size_t(t) * 3];
        for (int k = 0; k < 3; k++)
        {
            const int a = v[k], b = v[(k + 1) % 3];
            const auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = info.find(key);
            if (it == info.end())
                info.emplace(key, std::make_pair(t, -1));
            else if (it->second.second != -1)
            {
                err = "mesh: edge shared by more than two triangles";
                return false;
            }
            else
                it->second.second = t;
        }
    }
    m.edges.clear();
    m.edges.reserve(info.size() * 4);
    for (const auto &kv : info)
    {
        const int e[4] = {kv.first.first, kv.first.second, kv.second.first, kv.second.second};
        m.edges.insert(m.edges.end(), e, e + 4);
    }
    m.ne = int(info.size());
    return true;
}

void rebuild_bending(const Mesh &m, const Material &mat, Tables &t)
{
    // UpdateBendingMatrix (BaraffClothGpu.cpp:655-680): per-edge stiffness
    // K_u cos^2(theta) + K_v sin^2(theta), theta = uv edge angle folded to
    // [0, pi/2] (InitBendingMatrix, :579-594). All float arithmetic.
    const float Ku = mat.bending_k[0], Kv = mat.bending_k[1];
    t.edge_k.assign(m.ne, 0.f);
    for (int e = 0; e < m.ne; e++)
    {
        const int *ed = &m.edges[size_t(e) * 4];
        float dx = m.uv[size_t(ed[1]) * 2] - m.uv[size_t(ed[0]) * 2];
        float dy = m.uv[size_t(ed[1]) * 2 + 1] - m.uv[size_t(ed[0]) * 2 + 1];
        float nrm = std::sqrt(dx * dx + dy * dy);
        if (nrm > 0.f)
        {
            dx = dx / nrm;
            dy = dy / nrm;
        }
        float dot = dx * 1.f + dy * 0.f;
        float theta = std::acos(dot);
        if (theta > M_PI / 2.0f)
            theta = float(M_PI - theta);
        float ct = std::cos(theta), st = std::sin(theta);
        t.edge_k[e] = Ku * ct * ct + Kv * st * st;
    }
    // UpdateBendingStiffnessMatrixKernel (BaraffClothGpu.cu:387-426): value
    // diag16 * K_e added as value * I3 to block (v_i, v_j).  Summed here in
    // double in edge order and rounded once.
    std::vector<double> acc(t.cols.size(), 0.0);
    for (int e = 0; e < m.ne; e++)
    {
        const int *s = &t.stencil[size_t(e) * 4];
        if (s[0] < 0)
            continue;
        for (int i = 0; i < 4; i++)
        {
            int vi = s[i];
            for (int j = 0; j < 4; j++)
            {
                int vj = s[j];
                float value = t.diag16[size_t(e) * 16 + i * 4 + j] * t.edge_k[e];
                const int *b = &t.cols[t.rowptr[vi]];
                const int *en = &t.cols[t.rowptr[vi + 1]];
                int slot = int(std::lower_bound(b, en, vj) - b);
                acc[size_t(t.rowptr[vi]) + slot] += value;
            }
        }
    }
    t.kbend.resize(acc.size());
    for (size_t k = 0; k < acc.size(); k++)
        t.kbend[k] = mat.bending_model == 1 ? 0.f : float(acc[k]);
}

void rebuild_dihedral_factor(const Mesh &m, const Material &mat, Tables &t)
{
    // The CPU cloth hands the bending material (K, K, K) with K its first
    // bending stiffness (BaraffCloth.cpp:38-43); the edge stiffness is their
    // mean (BaseBendingMaterial.cpp:47).
    const double K = double(mat.bending_k[0]);
    const double kedge = ((K + K) + K) / 3.0;
    // cDihedralMaterial::Init (DihedralBending.cpp:23-91): float rest edge
    // lengths, float Heron areas from them (triangle edges (v0 v1), (v1 v2),
    // (v2 v0), BuildTriangleEdgeId, Triangulator.cpp:11-31), float heights
    // 2 A / e of the two triangles, and -K e / max(1e-7, h0 + h1) in double.
    std::vector<float> len(m.ne);
    std::map<std::pair<int, int>, int> eid;
    for (int e = 0; e < m.ne; e++)
    {
        const int *ed = &m.edges[size_t(e) * 4];
        const double *a = &m.pos[size_t(ed[0]) * 3], *b = &m.pos[size_t(ed[1]) * 3];
        const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
        len[e] = float(std::sqrt(dx * dx + dy * dy + dz * dz));
        eid[std::make_pair(std::min(ed[0], ed[1]), std::max(ed[0], ed[1]))] = e;
    }
    auto edge_len = [&](int a, int b) {
        return double(len[eid.at(std::make_pair(std::min(a, b), std::max(a, b)))]);
    };
    std::vector<float> area(m.nt);
    for (int tt = 0; tt < m.nt; tt++)
    {
        const int *v = &m.tris[size_t(tt) * 3];
        const double a = edge_len(v[0], v[1]), b = edge_len(v[1], v[2]),
                     c = edge_len(v[2], v[0]);
        const double p = (a + b + c) / 2;
        area[tt] = float(std::sqrt(p * (p - a) * (p - b) * (p - c)));
    }
    t.dih_factor.assign(t.n_dih, 0.0);
    for (int q = 0; q < t.n_dih; q++)
    {
        const int e = t.dih_edge[q];
        const int *ed = &m.edges[size_t(e) * 4];
        const float L = len[e];
        const float h0 = (2.f * area[ed[2]]) / L, h1 = (2.f * area[ed[3]]) / L;
        const float hs = std::max(1e-7f, h0 + h1);
        t.dih_factor[q] = -kedge * double(L) / double(hs);
    }
}

bool build_dihedral(const Mesh &m, const Material &mat, Tables &t, std::string &err)
{
    t.dih_edge.clear();
    for (int e = 0; e < m.ne; e++)
        if (t.stencil[size_t(e) * 4] >= 0)
            t.dih_edge.push_back(e);
    t.n_dih = int(t.dih_edge.size());
    if (size_t(t.n_dih) * 16 >= (size_t(1) << 27))
    {
        err = "mesh: too many interior edges for dihedral bending in one cloth";
        return false;
    }
    rebuild_dihedral_factor(m, mat, t);
    // Entry (q, a, b) adds edge q's block (a, b) to row stencil[a], slot of
    // stencil[b]; every pair of one stencil is in the ELL pattern.
    const size_t nnzb = t.cols.size();
    auto slot_of = [&](int row, int col) {
        const int *b = &t.cols[t.rowptr[row]];
        const int *en = &t.cols[t.rowptr[row + 1]];
        return int(std::lower_bound(b, en, col) - b);
    };
    t.dih_count.assign(nnzb, 0);
    std::vector<int> where(size_t(t.n_dih) * 16);
    for (int q = 0; q < t.n_dih; q++)
    {
        const int *s = &t.stencil[size_t(t.dih_edge[q]) * 4];
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++)
            {
                const size_t k = size_t(t.rowptr[s[a]]) + slot_of(s[a], s[b]);
                where[size_t(q) * 16 + a * 4 + b] = int(k);
                t.dih_count[k]++;
            }
    }
    t.dih_start.assign(nnzb, 0);
    int run = 0;
    for (size_t k = 0; k < nnzb; k++)
    {
        if (t.dih_count[k] > 31)
        {
            err = "mesh: more than 31 bending stencils meet in one block";
            return false;
        }
        t.dih_start[k] = run;
        run += t.dih_count[k];
    }
    // filled in edge order, so each block's entries are sorted by q
    t.dih_ent.assign(size_t(run), 0u);
    std::vector<int> fill(nnzb, 0);
    for (int q = 0; q < t.n_dih; q++)
        for (int ab = 0; ab < 16; ab++)
        {
            const int k = where[size_t(q) * 16 + ab];
            t.dih_ent[size_t(t.dih_start[k]) + fill[k]++] =
                (uint32_t(q) << 4) | uint32_t(ab >> 2) << 2 | uint32_t(ab & 3);
        }
    return true;
}

bool build_tables(const Mesh &m, const Material &mat, Tables &t,
                  std::string &err)
{
    t = Tables();
    t.nv = m.nv;
    t.nt = m.nt;
    t.ne = m.ne;
    if (m.nv <= 0 || m.nt <= 0)
    {
        err = "mesh: empty";
        return false;
    }
    for (int k = 0; k < m.nt * 3; k++)
        if (m.tris[k] < 0 || m.tris[k] >= m.nv)
        {
            err = "mesh: triangle vertex id out of range";
            return false;
        }
    for (int tt = 0; tt < m.nt; tt++)
    {
        const int *v = &m.tris[size_t(tt) * 3];
        if (v[0] == v[1] || v[1] == v[2] || v[0] == v[2])
        {
            err = "mesh: degenerate triangle";
            return false;
        }
    }

    // Edge stencils (cBaseCloth::InitGeometry, BaseCloth.cpp:383-405).
    t.stencil.assign(size_t(m.ne) * 4, -1);
    for (int e = 0; e < m.ne; e++)
    {
        const int *ed = &m.edges[size_t(e) * 4];
        if (ed[0] < 0 || ed[0] >= m.nv || ed[1] < 0 || ed[1] >= m.nv ||
            ed[2] < 0 || ed[2] >= m.nt || ed[3] >= m.nt)
        {
            err = "mesh: edge record out of range";
            return false;
        }
        if (ed[3] < 0)
            continue; // boundary
        int *s = &t.stencil[size_t(e) * 4];
        s[0] = ed[0];
        s[1] = ed[1];
        s[2] = other_vertex(&m.tris[size_t(ed[2]) * 3], ed[0], ed[1]);
        s[3] = other_vertex(&m.tris[size_t(ed[3]) * 3], ed[0], ed[1]);
        if (s[2] < 0 || s[3] < 0)
        {
            err = "mesh: edge not contained in its triangles";
            return false;
        }
    }

    // Rest areas (cBaseObject::CalcTriangleInitArea, BaseObject.cpp:292-304)
    // and lumped masses (cBaseCloth::InitMass, BaseCloth.cpp:418-446).
    t.area.resize(m.nt);
    std::vector<double> shared(m.nv, 0.0);
    for (int tt = 0; tt < m.nt; tt++)
    {
        const int *v = &m.tris[size_t(tt) * 3];
        t.area[tt] = triangle_area(&m.pos[size_t(v[0]) * 3],
                                   &m.pos[size_t(v[1]) * 3],
                                   &m.pos[size_t(v[2]) * 3]);
        double a = t.area[tt];
        for (int k = 0; k < 3; k++)
            shared[v[k]] += a / 3;
    }
    t.mass.resize(m.nv);
    for (int v = 0; v < m.nv; v++)
        t.mass[v] = shared[v] * double(mat.density);

    // ELL pattern (cBaraffClothGpu::InitELLMatrix, BaraffClothGpu.cpp:438-500):
    // per vertex, the sorted set of vertices that share an interior-edge
    // stencil with it, plus itself.  Vertex pairs of every triangle are added
    // too; for meshes the reference accepts they are already in the set.
    std::vector<std::vector<int>> rows(m.nv);
    for (int v = 0; v < m.nv; v++)
        rows[v].push_back(v);
    for (int e = 0; e < m.ne; e++)
    {
        const int *s = &t.stencil[size_t(e) * 4];
        if (s[0] < 0)
            continue;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                rows[s[i]].push_back(s[j]);
    }
    for (int tt = 0; tt < m.nt; tt++)
    {
        const int *v = &m.tris[size_t(tt) * 3];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                rows[v[a]].push_back(v[b]);
    }
    t.rowptr.assign(m.nv + 1, 0);
    t.diag_slot.assign(m.nv, -1);
    t.width = 0;
    for (int v = 0; v < m.nv; v++)
    {
        auto &r = rows[v];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        t.width = std::max(t.width, int(r.size()));
        t.rowptr[v + 1] = t.rowptr[v] + int(r.size());
    }
    if (t.width > 32)
    {
        err = "mesh: an ELL row is wider than 32 blocks";
        return false;
    }
    t.cols.resize(t.rowptr[m.nv]);
    for (int v = 0; v < m.nv; v++)
    {
        std::copy(rows[v].begin(), rows[v].end(), t.cols.begin() + t.rowptr[v]);
        for (size_t s = 0; s < rows[v].size(); s++)
            if (rows[v][s] == v)
                t.diag_slot[v] = int(s);
        std::vector<int>().swap(rows[v]);
    }
    auto slot_of = [&](int row, int col) {
        const int *b = &t.cols[t.rowptr[row]];
        const int *en = &t.cols[t.rowptr[row + 1]];
        return int(std::lower_bound(b, en, col) - b);
    };

    // Stretch coefficients (cBaraffClothGpu::InitStretchCoef,
    // BaraffClothGpu.cpp:517-553): Dm^-1 from float uv, inverted in double,
    // then the same for Dm^-1 * R45^T (the bias/shear frame).
    t.coef.resize(size_t(m.nt) * 12);
    const double r45c = std::cos(M_PI / 4), r45s = std::sin(M_PI / 4);
    // RotMat2D(a) = [[c, -s], [s, c]]; R45^T = [[c, s], [-s, c]].
    const double R45T[2][2] = {{r45c, r45s}, {-r45s, r45c}};
    for (int tt = 0; tt < m.nt; tt++)
    {
        const int *v = &m.tris[size_t(tt) * 3];
        const float *u0 = &m.uv[size_t(v[0]) * 2];
        const float *u1 = &m.uv[size_t(v[1]) * 2];
        const float *u2 = &m.uv[size_t(v[2]) * 2];
        double D[2][2] = {{double(u1[0] - u0[0]), double(u2[0] - u0[0])},
                          {double(u1[1] - u0[1]), double(u2[1] - u0[1])}};
        double det = D[0][0] * D[1][1] - D[1][0] * D[0][1];
        double invdet = 1.0 / det;
        double Di[2][2] = {{D[1][1] * invdet, -D[0][1] * invdet},
                           {-D[1][0] * invdet, D[0][0] * invdet}};
        float *c = &t.coef[size_t(tt) * 12];
        stretch_coef(Di, c + 0, c + 3);
        double Dr[2][2];
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                Dr[i][j] = Di[i][0] * R45T[0][j] + Di[i][1] * R45T[1][j];
        stretch_coef(Dr, c + 6, c + 9);
    }

    // Q-bending base table (InitBendingMatrix, BaraffClothGpu.cpp:596-626):
    // cotangent weights from the rest positions, 3 / (A0 + A1) with float areas.
    t.diag16.assign(size_t(m.ne) * 16, 0.f);
    for (int e = 0; e < m.ne; e++)
    {
        const int *s = &t.stencil[size_t(e) * 4];
        if (s[0] < 0)
            continue;
        const int *ed = &m.edges[size_t(e) * 4];
        float prefix = float(3.0 / (t.area[ed[2]] + t.area[ed[3]]));
        double c4[4];
        cotangent_coeff(&m.pos[size_t(s[0]) * 3], &m.pos[size_t(s[1]) * 3],
                        &m.pos[size_t(s[2]) * 3], &m.pos[size_t(s[3]) * 3], c4);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                t.diag16[size_t(e) * 16 + i * 4 + j] =
                    float(c4[i] * c4[j] * double(prefix));
    }
    rebuild_bending(m, mat, t);

    // Triangle -> slot map and the contribution records of the atomic-free
    // assembly: block (a,b) of triangle tt lands in row v_a, slot of v_b
    // (the slot the reference finds with global_to_local_same,
    // BaraffClothGpu.cu:111-126, 179-193).  Records are sorted by
    // (row, slot, triangle) so every block sums its contributions in a fixed
    // order.
    const size_t nnzb = t.cols.size();
    t.tri_slot.resize(size_t(m.nt) * 9);
    t.h_count.assign(nnzb, 0);
    std::vector<int> f_count(m.nv, 0);
    for (int tt = 0; tt < m.nt; tt++)
    {
        const int *v = &m.tris[size_t(tt) * 3];
        for (int a = 0; a < 3; a++)
        {
            f_count[v[a]]++;
            for (int b = 0; b < 3; b++)
            {
                int s = slot_of(v[a], v[b]);
                t.tri_slot[size_t(tt) * 9 + a * 3 + b] = s;
                t.h_count[size_t(t.rowptr[v[a]]) + s]++;
            }
        }
    }
    t.h_start.assign(nnzb, 0);
    long long run = 0;
    for (size_t k = 0; k < nnzb; k++)
    {
        t.h_start[k] = int(run);
        run += t.h_count[k];
        if (t.h_count[k] > 31)
        {
            err = "mesh: more than 31 triangles meet in one block";
            return false;
        }
    }
    if (run >= (1ll << 27))
    {
        err = "mesh: too many triangles for one cloth";
        return false;
    }
    t.f_rowptr.assign(m.nv + 1, 0);
    for (int v = 0; v < m.nv; v++)
        t.f_rowptr[v + 1] = t.f_rowptr[v] + f_count[v];
    std::vector<int> h_fill(nnzb, 0), f_fill(m.nv, 0);
    t.h_dest.resize(size_t(m.nt) * 9);
    t.f_dest.resize(size_t(m.nt) * 3);
    for (int tt = 0; tt < m.nt; tt++)
    {
        const int *v = &m.tris[size_t(tt) * 3];
        for (int a = 0; a < 3; a++)
        {
            t.f_dest[size_t(tt) * 3 + a] = t.f_rowptr[v[a]] + f_fill[v[a]]++;
            for (int b = 0; b < 3; b++)
            {
                size_t k = size_t(t.rowptr[v[a]]) +
                           t.tri_slot[size_t(tt) * 9 + a * 3 + b];
                t.h_dest[size_t(tt) * 9 + a * 3 + b] = t.h_start[k] + h_fill[k]++;
            }
        }
    }
    if (mat.bending_model == 1)
        return build_dihedral(m, mat, t, err);
    if (mat.bending_model != 0)
    {
        err = "material: unknown bending model";
        return false;
    }
    return true;
}

void find_vertices_from_uv(const Mesh &m, const float *uv, int n, int *out)
{
    for (int j = 0; j < n; j++)
    {
        out[j] = -1;
        double best = 0;
        for (int v = 0; v < m.nv; v++)
        {
            float dx = m.uv[size_t(v) * 2] - uv[2 * j];
            float dy = m.uv[size_t(v) * 2 + 1] - uv[2 * j + 1];
            double d = double(std::sqrt(dx * dx + dy * dy));
            if (out[j] < 0 || d < best)
            {
                best = d;
                out[j] = v;
            }
        }
    }
}

} // namespace cloth
