// OBJ cloth ingest: the reference's cBaseCloth::InitGeometry OBJ branch
// (src/sim/cloth/BaseCloth.cpp:292-356) over cObjUtil::LoadObj
// (src/utils/ObjUtil.cpp:10-139), which reads the file with the vendored
// tinyobjloader 2.x (includes/tinyobjloader/tiny_obj_loader.h).  Restated
// here: the subset of OBJ that loader turns into one triangle shape.
#include "topology.h"

#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace cloth {

namespace {

struct Corner
{
    int v, vt;
};

// "i", "i/j", "i//k", "i/j/k"; 1-based, negative = relative to the end.
bool parse_corner(const std::string &tok, int nv, int nvt, Corner &c)
{
    auto idx = [](const std::string &s, int n, int &out) -> bool {
        if (s.empty())
            return false;
        char *end = nullptr;
        const long i = std::strtol(s.c_str(), &end, 10);
        if (*end != '\0' || i == 0)
            return false;
        out = i > 0 ? int(i - 1) : int(n + i);
        return true;
    };
    const size_t s1 = tok.find('/');
    c.vt = -1;
    if (!idx(tok.substr(0, s1), nv, c.v))
        return false;
    if (s1 != std::string::npos)
    {
        const size_t s2 = tok.find('/', s1 + 1);
        const std::string t = tok.substr(s1 + 1, s2 == std::string::npos ? std::string::npos
                                                                        : s2 - s1 - 1);
        if (!t.empty() && !idx(t, nvt, c.vt))
            return false;
    }
    return true;
}

} // namespace

bool load_obj_cloth(const std::string &path, const double translation[3], bool relocate,
                    Mesh &m, std::string &err)
{
    std::ifstream in(path);
    if (!in)
    {
        err = "obj: cannot open " + path;
        return false;
    }
    // tinyobjloader keeps coordinates as real_t = float
    std::vector<float> v, vt;
    std::vector<Corner> corners; // three per triangle
    std::string line;
    int lineno = 0;
    while (std::getline(in, line))
    {
        lineno++;
        std::istringstream ls(line);
        std::string key;
        if (!(ls >> key) || key[0] == '#')
            continue;
        if (key == "v")
        {
            double x = 0, y = 0, z = 0;
            if (!(ls >> x >> y >> z))
            {
                err = "obj: bad vertex at line " + std::to_string(lineno);
                return false;
            }
            v.push_back(float(x));
            v.push_back(float(y));
            v.push_back(float(z));
        }
        else if (key == "vt")
        {
            double a = 0, b = 0;
            if (!(ls >> a))
            {
                err = "obj: bad texture coordinate at line " + std::to_string(lineno);
                return false;
            }
            ls >> b;
            vt.push_back(float(a));
            vt.push_back(float(b));
        }
        else if (key == "f")
        {
            std::vector<Corner> f;
            std::string tok;
            while (ls >> tok)
            {
                Corner c;
                if (!parse_corner(tok, int(v.size() / 3), int(vt.size() / 2), c) || c.v < 0 ||
                    c.v >= int(v.size() / 3) || c.vt >= int(vt.size() / 2))
                {
                    err = "obj: bad face index at line " + std::to_string(lineno);
                    return false;
                }
                f.push_back(c);
            }
            if (f.size() == 3)
                corners.insert(corners.end(), f.begin(), f.end());
            else if (f.size() == 4)
            {
                // tinyobjloader's quad split: along the shorter diagonal
                // (float arithmetic), [0 1 2] [0 2 3] or [0 1 3] [1 2 3]
                auto P = [&](int k, int a) { return v[3 * size_t(f[k].v) + a]; };
                const float e02x = P(2, 0) - P(0, 0), e02y = P(2, 1) - P(0, 1),
                            e02z = P(2, 2) - P(0, 2);
                const float e13x = P(3, 0) - P(1, 0), e13y = P(3, 1) - P(1, 1),
                            e13z = P(3, 2) - P(1, 2);
                const float s02 = e02x * e02x + e02y * e02y + e02z * e02z;
                const float s13 = e13x * e13x + e13y * e13y + e13z * e13z;
                static const int split02[6] = {0, 1, 2, 0, 2, 3};
                static const int split13[6] = {0, 1, 3, 1, 2, 3};
                const int *q = s02 < s13 ? split02 : split13;
                for (int k = 0; k < 6; k++)
                    corners.push_back(f[q[k]]);
            }
            else
            {
                err = "obj: faces of " + std::to_string(f.size()) +
                      " vertices are not supported (triangles and quads) at line " +
                      std::to_string(lineno);
                return false;
            }
        }
        // vn, o, g, s, usemtl, mtllib: nothing the cloth uses
    }
    const int nobj = int(v.size() / 3);
    if (corners.empty())
    {
        err = "obj: no faces";
        return false;
    }
    // LoadObj: mesh vertex i is OBJ vertex i; every one must be used by a face.
    // The uv of a vertex is that of the last face corner naming it.
    int nv = 0;
    for (const Corner &c : corners)
        nv = std::max(nv, c.v + 1);
    std::vector<char> used(nv, 0);
    std::vector<float> uv(size_t(nv) * 2, 0.f);
    for (const Corner &c : corners)
    {
        used[c.v] = 1;
        if (c.vt >= 0)
        {
            uv[2 * size_t(c.v)] = vt[2 * size_t(c.vt)];
            uv[2 * size_t(c.v) + 1] = vt[2 * size_t(c.vt) + 1];
        }
    }
    (void)nobj;
    for (int i = 0; i < nv; i++)
        if (!used[i])
        {
            err = "obj: vertex " + std::to_string(i + 1) + " is not used by any face";
            return false;
        }
    m = Mesh();
    m.nv = nv;
    m.nt = int(corners.size() / 3);
    m.tris.resize(corners.size());
    for (size_t k = 0; k < corners.size(); k++)
        m.tris[k] = corners[k].v;
    // InitGeometry's OBJ branch (BaseCloth.cpp:321-344): y += 0.2, uv *= 10/3
    // (in float), + cloth_obj_translation, then MoveObjPos when relocating.
    m.pos.resize(size_t(nv) * 3);
    m.uv.resize(size_t(nv) * 2);
    const float uv_scale = float(10 / 3.0);
    for (int i = 0; i < nv; i++)
    {
        double p[3] = {double(v[3 * size_t(i)]), double(v[3 * size_t(i) + 1]),
                       double(v[3 * size_t(i) + 2])};
        p[1] += 0.2;
        for (int k = 0; k < 3; k++)
            m.pos[3 * size_t(i) + k] = p[k] + translation[k];
        m.uv[2 * size_t(i)] = uv[2 * size_t(i)] * uv_scale;
        m.uv[2 * size_t(i) + 1] = uv[2 * size_t(i) + 1] * uv_scale;
    }
    if (relocate)
    {
        // MoveObjPos (BaseCloth.cpp:237-279): highest y (kept as float) to
        // 0.27, then x and z centred on the running mean of the vertices
        // within 1 cm of the top.
        float highest = -1e3f;
        for (int i = 0; i < nv; i++)
            if (m.pos[3 * size_t(i) + 1] > highest)
                highest = float(m.pos[3 * size_t(i) + 1]);
        const double given = 0.27, shift = given - double(highest);
        for (int i = 0; i < nv; i++)
            m.pos[3 * size_t(i) + 1] += shift;
        double o[3] = {0, 0, 0};
        int count = 0;
        for (int i = 0; i < nv; i++)
        {
            const double *p = &m.pos[3 * size_t(i)];
            if ((given - p[1]) < 0.01)
            {
                for (int k = 0; k < 3; k++)
                    o[k] = (o[k] * count + p[k]) / (count + 1);
                count++;
            }
        }
        for (int i = 0; i < nv; i++)
        {
            m.pos[3 * size_t(i)] -= o[0];
            m.pos[3 * size_t(i) + 2] -= o[2];
        }
    }
    return derive_edges(m, err);
}

} // namespace cloth
