// Host-side mesh topology and init-time tables of the implicit cloth step.
// Everything here runs once per cloth (or when the material changes); the
// results are uploaded by cloth_create.  Built with -ffp-contract=off so the
// float/double rounding sequence matches the reference's x86 build on any host.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cloth {

struct Mesh
{
    int nv = 0, nt = 0, ne = 0;
    std::vector<double> pos; // nv*3
    std::vector<float> uv;   // nv*2
    std::vector<int> tris;   // nt*3
    std::vector<int> edges;  // ne*4: v0 v1 tri0 tri1 (tri1 = -1 on the boundary)
};

struct GridDesc
{
    double size[2];  // height, width
    int subdiv[2];   // height_div, width_div
    double init_pos[3];
    float uv_rotation_deg;
};

struct Material
{
    float stretch_k[3];
    float bending_k[2];
    float density;
    float rayleigh_a, rayleigh_b;
    double default_timestep;
    double gravity;
    int fix_fv_norm;
    int bending_model = 0; // 0: quadratic (the GPU cloth's), 1: dihedral (the CPU cloth's)
};

// Everything derived from the mesh on the host.
struct Tables
{
    int nv = 0, nt = 0, ne = 0;
    int width = 0;                  // max ELL row length
    std::vector<int> stencil;       // ne*4 (mEdgeAffectVertexId)
    std::vector<float> area;        // nt   (mTriangleInitArea)
    std::vector<double> mass;       // nv   (cBaseCloth::InitMass)
    std::vector<int> rowptr;        // nv+1 CSR view of the ELL pattern
    std::vector<int> cols;          // nnzb sorted column ids per row
    std::vector<int> diag_slot;     // nv
    std::vector<float> coef;        // nt*12
    std::vector<int> tri_slot;      // nt*9   slot of v_b in row v_a
    std::vector<float> edge_k;      // ne     direction-blended bending stiffness
    std::vector<float> diag16;      // ne*16  QBending base table
    std::vector<float> kbend;       // nnzb   bending scalar per block (+K_b)
    // contribution records of the triangle pass, sorted by (row, slot, tri)
    std::vector<int> h_dest;        // nt*9  record index of block (a,b)
    std::vector<int> h_start;       // nnzb  first record of each block
    std::vector<int> h_count;       // nnzb
    std::vector<int> f_dest;        // nt*3  force record of local vertex a
    std::vector<int> f_rowptr;      // nv+1
    // dihedral bending (bending_model 1): interior edges in edge order
    int n_dih = 0;
    std::vector<int> dih_edge;       // n_dih  edge id
    std::vector<double> dih_factor;  // n_dih  -K e / max(1e-7, h0 + h1), rest state
    // (row, slot) entries: q << 4 | a << 2 | b for stencil vertices a (the
    // row) and b (the column) of interior edge q, sorted by (row, slot, q)
    std::vector<uint32_t> dih_ent;
    std::vector<int> dih_start;      // nnzb  first entry of each block
    std::vector<int> dih_count;      // nnzb
};

// cTriangulator::BuildGeometry_UniformTriangle + BuildRectVertices +
// RotateMaterialCoordsAfterReset (src/geometries/Triangulator.cpp:32-457, 621-658).
bool build_grid(const GridDesc &g, Mesh &m, std::string &err);

// "regular_triangle_perturb" and "delaunay" of cTriangulator::BuildGeometry
// (Triangulator.cpp:100-110) with the reference's generator seeded with
// `seed` right before the build.  geometry.cpp.
bool perturb_grid(const GridDesc &g, unsigned long long seed, Mesh &m, std::string &err);
bool delaunay_cloth(const GridDesc &g, unsigned long long seed, Mesh &m, std::string &err);

// Edge list from triangles when the caller gives none, as cObjUtil::BuildEdge
// numbers it: one edge per vertex pair (v0 < v1) in ascending pair order;
// tri0/tri1 are the first/second triangle that uses the pair.  Fails on edges
// shared by more than two triangles.
bool derive_edges(Mesh &m, std::string &err);

// A cloth mesh from an OBJ file as cBaseCloth::InitGeometry builds it with
// "enable_cloth_from_obj" (BaseCloth.cpp:292-356, cObjUtil::LoadObj): float
// coordinates, y + 0.2, uv * 10/3, + translation, MoveObjPos when relocating;
// triangles and quads (split along the shorter diagonal).  objmesh.cpp.
bool load_obj_cloth(const std::string &path, const double translation[3], bool relocate,
                    Mesh &m, std::string &err);

// cBaseCloth::InitGeometry tail, InitMass, cBaraffClothGpu::InitELLMatrix,
// InitStretchCoef, InitBendingMatrix/UpdateBendingMatrix, and the triangle ->
// slot / contribution maps of the atomic-free assembly.
bool build_tables(const Mesh &m, const Material &mat, Tables &t,
                  std::string &err);

// Only the material-dependent part (edge_k, kbend) for cloth_set_material.
void rebuild_bending(const Mesh &m, const Material &mat, Tables &t);

// cDihedralMaterial::Init (src/sim/cloth/DihedralBending.cpp:23-91) and the
// (row, slot) entry lists of its per-edge Hessians; called by build_tables
// when mat.bending_model is 1.
bool build_dihedral(const Mesh &m, const Material &mat, Tables &t, std::string &err);

// The stiffness-dependent part of it (dih_factor).
void rebuild_dihedral_factor(const Mesh &m, const Material &mat, Tables &t);

// FindVerticesIdFromUV (src/sim/cloth/BaseCloth.cpp:151-189).
void find_vertices_from_uv(const Mesh &m, const float *uv, int n, int *out);

} // namespace cloth
