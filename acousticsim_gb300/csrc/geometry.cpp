// The two cloth geometry generators of cTriangulator::BuildGeometry that draw
// from the reference's global random generator (src/geometries/Triangulator.cpp:
// 100-110): "regular_triangle_perturb" (the regular grid with its interior
// vertices jittered, BuildRectVertices :395-457) and "delaunay" (random points
// of a minimum spacing inside a rectangle boundary, Delaunay-triangulated,
// src/geometries/TriangulatorDelaunay.cpp:41-216).
//
// The generator is the reference's cRand (src/utils/Rand.cpp:6-38, 114-121):
// std::default_random_engine seeded with `seed`, doubles from
// std::uniform_real_distribution<double>(0, 1) scaled to [min, max]; the
// reference's main seeds it with 0 (src/main.cpp:153).  The same standard
// library draws the same numbers, so points come out bit for bit.
//
// The triangulation is this file's own Bowyer-Watson insertion (walk to the
// triangle holding the new point, grow the cavity of triangles whose
// circumcircle holds it, connect the cavity's boundary to the point), not the
// reference's third-party delaunator: the Delaunay triangulation of points in
// general position is unique, so the triangles are the same; their order and
// first vertex differ, and with them the edge numbering (edges are numbered
// by first appearance over the triangles, as the reference numbers its own).
#include "topology.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>
#include <random>
#include <unordered_map>

namespace cloth {
namespace {

// The global generator right after cMathUtil::SeedRand(seed) (src/utils/
// MathUtil.cpp:99-103: Seed(seed), then one RandInt() for srand, an integer
// drawn uniformly from [INT_MIN + 1, INT_MAX]), and cRand::RandDouble(min,
// max) (src/utils/Rand.cpp:27-38).
struct RefRand
{
    std::default_random_engine gen;
    std::uniform_real_distribution<double> dist{0.0, 1.0};
    explicit RefRand(unsigned long long seed) : gen(static_cast<unsigned long>(seed))
    {
        std::uniform_int_distribution<int> srand_draw(std::numeric_limits<int>::min() + 1,
                                                      std::numeric_limits<int>::max());
        (void)srand_draw(gen);
    }
    double next(double lo, double hi)
    {
        if (lo == hi)
            return lo;
        const double u = dist(gen);
        return lo + (u * (hi - lo));
    }
};

// ----------------------------------------------------------------- predicates
// Twice the signed area of (a, b, c): > 0 counter-clockwise.  The points are
// floats widened to double, so the differences and products are exact and
// the sign is too.
double orient(const double *a, const double *b, const double *c)
{
    return (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]);
}

// > 0 when d lies inside the circumcircle of the counter-clockwise (a, b, c).
double incircle(const double *a, const double *b, const double *c, const double *d)
{
    const double adx = a[0] - d[0], ady = a[1] - d[1];
    const double bdx = b[0] - d[0], bdy = b[1] - d[1];
    const double cdx = c[0] - d[0], cdy = c[1] - d[1];
    const double al = adx * adx + ady * ady;
    const double bl = bdx * bdx + bdy * bdy;
    const double cl = cdx * cdx + cdy * cdy;
    return al * (bdx * cdy - cdx * bdy) + bl * (cdx * ady - adx * cdy) +
           cl * (adx * bdy - bdx * ady);
}

struct Tri
{
    int v[3];  // counter-clockwise
    int nb[3]; // neighbour across the edge opposite v[k], -1 for none
    bool alive;
};

// Bowyer-Watson over pts (x, y pairs); returns counter-clockwise triangles.
bool triangulate(const std::vector<double> &pts, std::vector<int> &out, std::string &err)
{
    const int n = int(pts.size() / 2);
    if (n < 3)
    {
        err = "delaunay: fewer than three points";
        return false;
    }
    double lo[2] = {pts[0], pts[1]}, hi[2] = {pts[0], pts[1]};
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 2; k++)
        {
            lo[k] = std::min(lo[k], pts[2 * i + k]);
            hi[k] = std::max(hi[k], pts[2 * i + k]);
        }
    const double cx = 0.5 * (lo[0] + hi[0]), cy = 0.5 * (lo[1] + hi[1]);
    const double ext = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), 1e-6);
    // a super triangle far outside every point (its vertices are n, n+1, n+2)
    std::vector<double> P(pts);
    const double S = 64.0 * ext;
    const double sv[6] = {cx - S, cy - S, cx + S, cy - S, cx, cy + S};
    P.insert(P.end(), sv, sv + 6);
    auto at = [&](int v) { return &P[size_t(v) * 2]; };

    std::vector<Tri> T;
    T.reserve(size_t(n) * 2 + 16);
    T.push_back(Tri{{n, n + 1, n + 2}, {-1, -1, -1}, true});
    int last = 0;
    std::vector<int> cavity, stack, mark;
    std::vector<int> first_of, second_of, stamp1, stamp2;
    first_of.assign(size_t(n) + 3, -1);
    second_of.assign(size_t(n) + 3, -1);
    stamp1.assign(size_t(n) + 3, -1);
    stamp2.assign(size_t(n) + 3, -1);
    struct Bnd
    {
        int a, b, out;
    };
    std::vector<Bnd> bnd;
    unsigned walk_rng = 12345u;
    // walk starts (the cavity of a point, every triangle whose circumcircle
    // holds it, does not depend on where the walk starts; a near start keeps
    // the walks short): tri_of[v] is a live triangle at vertex v (a cavity
    // keeps every vertex of the triangles it removes on its boundary, and each
    // boundary vertex gets a new triangle), and a coarse grid over the points'
    // box holds the vertex inserted last in each cell
    std::vector<int> tri_of(size_t(n) + 3, 0);
    const int gside = std::max(1, int(std::sqrt(double(n) / 4.0)));
    const double gw = std::max(hi[0] - lo[0], 1e-300), gh = std::max(hi[1] - lo[1], 1e-300);
    std::vector<int> cell_vertex(size_t(gside) * gside, -1);
    auto cell_xy = [&](const double *q, int &cx, int &cy) {
        cx = std::min(gside - 1, std::max(0, int((q[0] - lo[0]) / gw * gside)));
        cy = std::min(gside - 1, std::max(0, int((q[1] - lo[1]) / gh * gside)));
    };
    for (int p = 0; p < n; p++)
    {
        const double *pp = at(p);
        int gx, gy;
        cell_xy(pp, gx, gy);
        // 1. walk to a triangle holding p (p on an edge counts as inside),
        // from a vertex inserted in p's cell or one next to it
        int t = last;
        for (int r = 0, found = 0; r <= 1 && !found; r++)
            for (int dy = -r; dy <= r && !found; dy++)
                for (int dx = -r; dx <= r && !found; dx++)
                {
                    const int x = gx + dx, y = gy + dy;
                    if (x < 0 || y < 0 || x >= gside || y >= gside)
                        continue;
                    const int v = cell_vertex[size_t(y) * gside + x];
                    if (v >= 0)
                    {
                        t = tri_of[size_t(v)];
                        found = 1;
                    }
                }
        if (!T[size_t(t)].alive)
            t = last;
        for (int steps = 0;; steps++)
        {
            if (steps > 4 * int(T.size()) + 64)
            {
                err = "delaunay: point location did not converge";
                return false;
            }
            const Tri &tr = T[size_t(t)];
            walk_rng = walk_rng * 1664525u + 1013904223u;
            const int k0 = int(walk_rng >> 30) % 3;
            int next = -1;
            for (int j = 0; j < 3; j++)
            {
                const int k = (k0 + j) % 3;
                const int a = tr.v[(k + 1) % 3], b = tr.v[(k + 2) % 3];
                if (orient(at(a), at(b), pp) < 0.0)
                {
                    next = tr.nb[k];
                    break;
                }
            }
            if (next < 0)
                break;
            t = next;
        }
        // 2. the cavity: triangles whose circumcircle holds p, grown from t
        if (mark.size() < T.size())
            mark.resize(T.size(), -1);
        cavity.clear();
        stack.clear();
        stack.push_back(t);
        mark[size_t(t)] = p;
        bnd.clear();
        while (!stack.empty())
        {
            const int c = stack.back();
            stack.pop_back();
            cavity.push_back(c);
            const Tri &tr = T[size_t(c)];
            for (int k = 0; k < 3; k++)
            {
                const int o = tr.nb[k];
                const int a = tr.v[(k + 1) % 3], b = tr.v[(k + 2) % 3];
                if (o >= 0 && mark[size_t(o)] == p)
                    continue; // already in the cavity
                if (o >= 0)
                {
                    const Tri &to = T[size_t(o)];
                    if (incircle(at(to.v[0]), at(to.v[1]), at(to.v[2]), pp) > 0.0)
                    {
                        mark[size_t(o)] = p;
                        stack.push_back(o);
                        continue;
                    }
                }
                bnd.push_back(Bnd{a, b, o});
            }
        }
        // a boundary edge whose neighbour joined the cavity later is interior
        {
            size_t w = 0;
            for (size_t i = 0; i < bnd.size(); i++)
                if (bnd[i].out < 0 || mark[size_t(bnd[i].out)] != p)
                    bnd[w++] = bnd[i];
            bnd.resize(w);
        }
        for (int c : cavity)
            T[size_t(c)].alive = false;
        // 3. connect the boundary to p: (a, b, p) is counter-clockwise
        const int base = int(T.size());
        for (size_t i = 0; i < bnd.size(); i++)
        {
            const Bnd &e = bnd[i];
            if (orient(at(e.a), at(e.b), pp) <= 0.0)
            {
                err = "delaunay: degenerate cavity (collinear or repeated points)";
                return false;
            }
            const int id = base + int(i);
            T.push_back(Tri{{e.a, e.b, p}, {-1, -1, e.out}, true});
            if (e.out >= 0)
            {
                Tri &to = T[size_t(e.out)];
                for (int k = 0; k < 3; k++)
                    if (to.v[(k + 1) % 3] == e.b && to.v[(k + 2) % 3] == e.a)
                        to.nb[k] = id;
            }
            tri_of[size_t(e.a)] = id;
            tri_of[size_t(e.b)] = id;
            stamp1[size_t(e.a)] = p;
            first_of[size_t(e.a)] = id;  // the new triangle with edge p -> a
            stamp2[size_t(e.b)] = p;
            second_of[size_t(e.b)] = id; // the new triangle with edge b -> p
        }
        for (size_t i = 0; i < bnd.size(); i++)
        {
            Tri &tr = T[size_t(base) + i];
            const int a = tr.v[0], b = tr.v[1];
            // across (b -> p): the new triangle starting at b; across (p -> a):
            // the new triangle whose second vertex is a
            if (stamp1[size_t(b)] != p || stamp2[size_t(a)] != p)
            {
                err = "delaunay: cavity boundary is not a closed loop";
                return false;
            }
            tr.nb[0] = first_of[size_t(b)];
            tr.nb[1] = second_of[size_t(a)];
        }
        last = base;
        tri_of[size_t(p)] = base;
        cell_vertex[size_t(gy) * gside + gx] = p;
    }
    out.clear();
    for (const Tri &tr : T)
        if (tr.alive && tr.v[0] < n && tr.v[1] < n && tr.v[2] < n)
            out.insert(out.end(), tr.v, tr.v + 3);
    return true;
}

// Edges numbered by first appearance over the triangles (edges v0v1, v1v2,
// v2v0 of each), as add_edge_into_edge_array does (TriangulatorDelaunay.cpp:9-41).
bool edges_by_appearance(Mesh &m, std::string &err)
{
    std::unordered_map<long long, int> idx;
    m.edges.clear();
    for (int t = 0; t < m.nt; t++)
        for (int k = 0; k < 3; k++)
        {
            int a = m.tris[size_t(t) * 3 + k], b = m.tris[size_t(t) * 3 + (k + 1) % 3];
            if (a > b)
                std::swap(a, b);
            const long long key = (long long)a * (long long)m.nv + b;
            auto it = idx.find(key);
            if (it == idx.end())
            {
                idx.emplace(key, int(m.edges.size() / 4));
                const int e[4] = {a, b, t, -1};
                m.edges.insert(m.edges.end(), e, e + 4);
            }
            else
            {
                int *e = &m.edges[size_t(it->second) * 4];
                if (e[3] != -1)
                {
                    err = "delaunay: edge shared by more than two triangles";
                    return false;
                }
                e[3] = t;
            }
        }
    m.ne = int(m.edges.size() / 4);
    return true;
}

// the init transform (translation; the rotation is identity) and the material
// coordinates (RotateMaterialCoordsAfterReset, Triangulator.cpp:621-658), as
// build_grid applies them
void place(const GridDesc &g, const std::vector<double> &xy, Mesh &m)
{
    const float ang = float(g.uv_rotation_deg / 180.0 * M_PI);
    const float rc = float(std::cos(double(ang))), rs = float(std::sin(double(ang)));
    m.pos.assign(size_t(m.nv) * 3, 0.0);
    m.uv.assign(size_t(m.nv) * 2, 0.f);
    for (int v = 0; v < m.nv; v++)
    {
        double p[3] = {xy[size_t(v) * 2], xy[size_t(v) * 2 + 1], 0.0};
        for (int k = 0; k < 3; k++)
            p[k] = p[k] + g.init_pos[k];
        for (int k = 0; k < 3; k++)
            m.pos[size_t(v) * 3 + k] = p[k];
        const float px = float(p[0] + (-g.init_pos[0]));
        const float py = float(p[1] + (-g.init_pos[1]));
        m.uv[size_t(v) * 2 + 0] = rc * px + (-rs) * py;
        m.uv[size_t(v) * 2 + 1] = rs * px + rc * py;
    }
}

} // namespace

bool perturb_grid(const GridDesc &g, unsigned long long seed, Mesh &m, std::string &err)
{
    // the regular grid first (vertex i * (hd + 1) + j at (i uw, j uh) - centre,
    // then init_pos), then the jitter of BuildRectVertices (Triangulator.cpp:
    // 425-446): vertex (i, j) with i != 0, i != height_div, j != 0 and
    // j != width_div moves by U(-uw/5, uw/5) in x, then U(-uh/5, uh/5) in y,
    // drawn in vertex order; its material coordinates follow the moved position
    if (!build_grid(g, m, err))
        return false;
    const int hd = g.subdiv[0], wd = g.subdiv[1];
    const double height = g.size[0], width = g.size[1];
    const double unit_h = height / hd, unit_w = width / wd;
    const double nh = unit_h / 5, nw = unit_w / 5;
    RefRand rng(seed);
    std::vector<double> xy(size_t(m.nv) * 2);
    for (int i = 0; i < wd + 1; i++)
        for (int j = 0; j < hd + 1; j++)
        {
            const int v = i * (hd + 1) + j;
            double x = i * unit_w - width / 2, y = j * unit_h - height / 2;
            if (i != 0 && i != hd && j != 0 && j != wd)
            {
                x += rng.next(-nw, nw);
                y += rng.next(-nh, nh);
            }
            xy[size_t(v) * 2] = x;
            xy[size_t(v) * 2 + 1] = y;
        }
    place(g, xy, m);
    return true;
}

bool delaunay_cloth(const GridDesc &g, unsigned long long seed, Mesh &m, std::string &err)
{
    // DelaunayTriangulation(cloth_size[1], cloth_size[0], subdivision[0] *
    // subdivision[1]) (Triangulator.cpp:106-110): width along x, in float
    const float width = float(g.size[1]), height = float(g.size[0]);
    const int target = g.subdiv[0] * g.subdiv[1];
    const int rot = int(g.uv_rotation_deg);
    if (rot != 0 && rot != 45 && rot != 90)
    {
        err = "delaunay: cloth_uv_rotation must be 0, 45 or 90";
        return false;
    }
    if (!(width > 0.f) || !(height > 0.f) || target < 4)
    {
        err = "delaunay: cloth_size must be > 0 and subdivision[0] * subdivision[1] >= 4";
        return false;
    }
    // 1. BuildRectangleBoundary (TriangulatorDelaunay.cpp:178-216): points
    // along the rectangle counter-clockwise from the bottom-left corner
    struct P2
    {
        float x, y;
    };
    std::vector<P2> v;
    {
        const float density = std::sqrt(height * width / target);
        const int nx = std::max(static_cast<int>(std::round(width / density)), 2);
        const int ny = std::max(static_cast<int>(std::round(height / density)), 2);
        const float gx = width / (nx - 1), gy = height / (ny - 1);
        const float left = -width / 2, right = width / 2, up = height / 2, down = -height / 2;
        for (int i = 1; i < nx; i++)
            v.push_back({left + i * gx, down});
        for (int i = 1; i < ny; i++)
            v.push_back({right, down + i * gy});
        for (int i = nx - 2; i >= 0; i--)
            v.push_back({left + i * gx, up});
        for (int i = ny - 2; i >= 0; i--)
            v.push_back({left, down + i * gy});
    }
    // 2. random points farther than the threshold from every point so far
    // (TriangulatorDelaunay.cpp:58-80).  A uniform grid of cells of the
    // threshold's size finds every point within it, so each candidate gets the
    // decision the reference's scan over all points gives.
    const float thr = std::sqrt((width * height / target) / M_PI);
    const float cell = std::max(thr, 1e-6f);
    const int gnx = std::max(1, int(std::ceil(width / cell)) + 1);
    const int gny = std::max(1, int(std::ceil(height / cell)) + 1);
    if (double(gnx) * double(gny) > 64.0 * 1024 * 1024)
    {
        err = "delaunay: too many points";
        return false;
    }
    std::vector<std::vector<int>> grid(size_t(gnx) * size_t(gny));
    auto cell_of = [&](float x, float y, int &cx, int &cy) {
        cx = std::min(gnx - 1, std::max(0, int(std::floor((x + width / 2) / cell))));
        cy = std::min(gny - 1, std::max(0, int(std::floor((y + height / 2) / cell))));
    };
    for (int i = 0; i < int(v.size()); i++)
    {
        int cx, cy;
        cell_of(v[size_t(i)].x, v[size_t(i)].y, cx, cy);
        grid[size_t(cy) * gnx + cx].push_back(i);
    }
    RefRand rng(seed);
    long long tries = 0;
    while (int(v.size()) < target)
    {
        if (++tries > 200LL * target + 100000)
        {
            err = "delaunay: could not place the points (rejection sampling stalled)";
            return false;
        }
        P2 q;
        q.x = float(rng.next(-width / 2, width / 2));
        q.y = float(rng.next(-height / 2, height / 2));
        int cx, cy;
        cell_of(q.x, q.y, cx, cy);
        bool far = true;
        for (int dy = -2; dy <= 2 && far; dy++)
            for (int dx = -2; dx <= 2 && far; dx++)
            {
                const int x = cx + dx, y = cy + dy;
                if (x < 0 || y < 0 || x >= gnx || y >= gny)
                    continue;
                for (int id : grid[size_t(y) * gnx + x])
                {
                    const float ex = v[size_t(id)].x - q.x, ey = v[size_t(id)].y - q.y;
                    const float d = std::sqrt(ex * ex + ey * ey);
                    if (!(d > thr))
                    {
                        far = false;
                        break;
                    }
                }
            }
        if (far)
        {
            grid[size_t(cy) * gnx + cx].push_back(int(v.size()));
            v.push_back(q);
        }
    }
    // 3. the first `target` points, triangulated counter-clockwise (the
    // reference turns every triangle to counter-clockwise in x, y)
    m.nv = target;
    std::vector<double> xy(size_t(target) * 2);
    for (int i = 0; i < target; i++)
    {
        xy[size_t(i) * 2] = double(v[size_t(i)].x);
        xy[size_t(i) * 2 + 1] = double(v[size_t(i)].y);
    }
    if (!triangulate(xy, m.tris, err))
        return false;
    m.nt = int(m.tris.size() / 3);
    // A strip far thinner than its subdivision (e.g. 0.01 x 3.0 split 3 x 120)
    // keeps, of its boundary-first point list, only points on one or two
    // boundary lines: collinear (no triangle at all) or joined to the rest by
    // slivers only.  Such a mesh is no cloth: refused, not returned in part.
    {
        std::vector<char> used(size_t(target), 0);
        for (int i : m.tris)
            used[size_t(i)] = 1;
        int unused = 0;
        for (char u : used)
            unused += u ? 0 : 1;
        if (unused > 0)
        {
            err = "delaunay: " + std::to_string(unused) + " of the " + std::to_string(target) +
                  " points are in no triangle (a strip too thin for its subdivision: its "
                  "points are collinear or nearly so); use a wider cloth or fewer subdivisions "
                  "along its length";
            return false;
        }
    }
    place(g, xy, m);
    return edges_by_appearance(m, err);
}

} // namespace cloth
