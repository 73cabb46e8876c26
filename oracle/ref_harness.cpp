// Test infrastructure only: this program links the reference's own CPU cloth
// code (built by oracle/Makefile from the reference sources) and writes golden
// arrays for the parity tests.  Nothing in the product loads or runs it.
//
// Modes
//   topo   <cfg.json> <outdir>                     mesh, index maps, init-time data
//   system <cfg.json> <x.bin> <xpre.bin> <outdir>  per-triangle f/H, bending, A, b, dx
//   step   <cfg.json> <nsteps> [x.bin xpre.bin]    time the stock "fem" UpdatePos
//   collide <cfg.json> <body.json> <x.bin> <dx.bin> <outdir>
//                                                  contacts with one kinematic body,
//                                                  contact Hessian, Repulsion
//   geom   <cfg.json> <seed> <outdir>              cTriangulator::BuildGeometry right
//                                                  after cMathUtil::SeedRand(seed)
//
// Where the reference's GPU host code (src/sim/cloth/BaraffClothGpu.cpp) cannot
// be compiled (it pulls in MSVC-only CUDA headers), the few lines of its init
// routines are restated here on top of the reference helpers it calls
// (CalcBaraffStretchCoef, CalcCotangentCoeff, cRotUtil::RotMat2D), each with
// the file:line it follows.  Blocks are written row-major: (i,j) -> [3*i+j].
#include "geometries/Primitives.h"
#include "geometries/Triangulator.h"
#include "utils/MathUtil.h"
#include "sim/cloth/BaraffCloth.h"
#include "sim/cloth/BaraffMaterial.h"
#include "sim/cloth/DihedralBending.h"
#include "sim/collision/BVHCollisionDetecter.h"
#include "sim/collision/CollisionInfo.h"
#include "sim/kinematic/KinematicBody.h"
#include "sim/cloth/QBendingMaterial.h"
#include "utils/JsonUtil.h"
#include "utils/RotUtil.h"
#include <Eigen/SparseCholesky>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <set>
#include <string>
#include <vector>

// reference helpers (src/sim/cloth/BaraffMaterial.cpp:18, QBendingMaterial.cpp:20)
extern void CalcBaraffStretchCoef(const tMatrix2d &mat, tVector3d &coef_u,
                                  tVector3d &coef_v);
extern tVector CalcCotangentCoeff(const tVector3d &x0, const tVector3d &x1,
                                  const tVector3d &x2, const tVector3d &x3);

static const int kEll = 32; // tCudaVector32i width (BaraffClothGpu.h:19)

// The reference's kinematic body, with its scaled local mesh (the vertices
// the pose transforms) readable for the motion fixture.
struct MotionBody : public cKinematicBody
{
    explicit MotionBody(int id) : cKinematicBody(id) {}
    const tVectorXd &local() const { return mScaledMeshVertices; }
    float time() const { return mCurTime; }
};

// ------------------------------------------------------------------ output
struct Dump
{
    std::string dir;
    std::ofstream manifest;
    explicit Dump(const std::string &d) : dir(d), manifest(d + "/manifest.txt") {}
    template <class T>
    void put(const std::string &name, const char *dtype,
             const std::vector<T> &v, std::vector<long> shape)
    {
        std::ofstream f(dir + "/" + name + ".bin", std::ios::binary);
        f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
        manifest << name << " " << dtype;
        for (long s : shape)
            manifest << " " << s;
        manifest << "\n";
    }
};

static std::vector<double> read_doubles(const std::string &path, size_t n)
{
    std::vector<double> v(n);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char *>(v.data()), n * sizeof(double));
    if (!f)
    {
        std::cerr << "short read " << path << "\n";
        exit(2);
    }
    return v;
}

// ------------------------------------------------------------------ probes
struct MatProbe : public cBaraffMaterial
{
    const tEigenArr<tMatrix3d> &tri_fint() const { return mTriFint; }
    const tEigenArr<tMatrix3d> &tri_hessian() const { return mTriHessian; }
};

struct Probe : public cBaraffCloth
{
    using cBaraffCloth::cBaraffCloth;
    Json::Value conf;

    int nv() const { return GetNumOfVertices(); }
    int ne() const { return GetNumOfEdges(); }
    int nt() const { return GetNumOfTriangles(); }

    // GPU-path vertex mass: cBaraffClothGpu::InitMass -> cBaseCloth::InitMass
    // (BaseCloth.cpp:418-446).  cBaraffCloth overrides InitMass with its own
    // variant, so the base routine is called explicitly here.
    std::vector<double> gpu_mass()
    {
        cBaseCloth::InitMass(conf);
        std::vector<double> m(nv());
        for (int i = 0; i < nv(); i++)
            m[i] = mVertexArray[i]->mMass;
        return m;
    }

    // cBaraffClothGpu::InitELLMatrix (BaraffClothGpu.cpp:438-500)
    std::vector<int> ell()
    {
        std::vector<std::set<int>> aff(nv());
        for (int e = 0; e < ne(); e++)
        {
            if (mEdgeArray[e]->mIsBoundary)
                continue;
            tVector4i c = mEdgeAffectVertexId[e];
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++)
                    aff[c[i]].insert(c[j]);
        }
        for (auto &t : mTriangleArray)
        {
            int v[3] = {t->mId0, t->mId1, t->mId2};
            for (int j = 0; j < 3; j++)
                aff[v[j]].insert(v[j]);
        }
        std::vector<int> out(size_t(nv()) * kEll, -1);
        for (int i = 0; i < nv(); i++)
        {
            int j = 0;
            for (int c : aff[i])
            {
                if (j >= kEll)
                {
                    std::cerr << "row " << i << " wider than 32\n";
                    exit(3);
                }
                out[size_t(i) * kEll + j++] = c;
            }
        }
        return out;
    }

    // cBaraffClothGpu::InitStretchCoef (BaraffClothGpu.cpp:504-553)
    std::vector<float> stretch_coef()
    {
        std::vector<float> out(size_t(nt()) * 12);
        tMatrix2d R45 = cRotUtil::RotMat2D(M_PI / 4);
        for (int i = 0; i < nt(); i++)
        {
            auto tri = mTriangleArray[i];
            auto v0 = mVertexArray[tri->mId0], v1 = mVertexArray[tri->mId1],
                 v2 = mVertexArray[tri->mId2];
            tMatrix2d Dminv;
            Dminv.col(0) = (v1->muv - v0->muv).cast<double>();
            Dminv.col(1) = (v2->muv - v0->muv).cast<double>();
            Dminv = Dminv.inverse().eval();
            tVector3d u, v;
            CalcBaraffStretchCoef(Dminv, u, v);
            for (int k = 0; k < 3; k++)
            {
                out[size_t(i) * 12 + 0 + k] = float(u[k]);
                out[size_t(i) * 12 + 3 + k] = float(v[k]);
            }
            Dminv = Dminv * R45.transpose();
            CalcBaraffStretchCoef(Dminv, u, v);
            for (int k = 0; k < 3; k++)
            {
                out[size_t(i) * 12 + 6 + k] = float(u[k]);
                out[size_t(i) * 12 + 9 + k] = float(v[k]);
            }
        }
        return out;
    }

    // cBaraffClothGpu::InitBendingMatrix / UpdateBendingMatrix
    // (BaraffClothGpu.cpp:573-626, 655-672): per-edge 4x4 scalar table and
    // the direction-blended edge stiffness.
    void bending(float Ku, float Kv, std::vector<float> &diag16,
                 std::vector<float> &edge_k)
    {
        diag16.assign(size_t(ne()) * 16, 0.f);
        edge_k.assign(ne(), 0.f);
        for (int e = 0; e < ne(); e++)
        {
            auto ce = mEdgeArray[e];
            tVector2f dir =
                (mVertexArray[ce->mId1]->muv - mVertexArray[ce->mId0]->muv)
                    .normalized();
            float theta = std::acos(dir.dot(tVector2f(1, 0)));
            if (theta > M_PI / 2.0f)
                theta = M_PI - theta;
            float cos_t = std::cos(theta), sin_t = std::sin(theta);
            edge_k[e] = Ku * cos_t * cos_t + Kv * sin_t * sin_t;
            if (ce->mIsBoundary)
                continue;
            float prefix = 3.0 / (mTriangleInitArea[ce->mTriangleId0] +
                                  mTriangleInitArea[ce->mTriangleId1]);
            tVector4i s = mEdgeAffectVertexId[e];
            tVector coef = CalcCotangentCoeff(
                mVertexArray[s[0]]->mPos.segment(0, 3),
                mVertexArray[s[1]]->mPos.segment(0, 3),
                mVertexArray[s[2]]->mPos.segment(0, 3),
                mVertexArray[s[3]]->mPos.segment(0, 3));
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++)
                    diag16[size_t(e) * 16 + i * 4 + j] =
                        coef[i] * coef[j] * prefix;
        }
    }

    void dump_topo(Dump &d)
    {
        int n = nv(), E = ne(), T = nt();
        std::vector<double> pos(size_t(n) * 3);
        std::vector<float> uv(size_t(n) * 2);
        for (int i = 0; i < n; i++)
        {
            for (int k = 0; k < 3; k++)
                pos[size_t(i) * 3 + k] = mVertexArray[i]->mPos[k];
            uv[size_t(i) * 2 + 0] = mVertexArray[i]->muv[0];
            uv[size_t(i) * 2 + 1] = mVertexArray[i]->muv[1];
        }
        std::vector<int> tris(size_t(T) * 3), edges(size_t(E) * 5),
            stencil(size_t(E) * 4);
        for (int t = 0; t < T; t++)
        {
            tris[size_t(t) * 3 + 0] = mTriangleArray[t]->mId0;
            tris[size_t(t) * 3 + 1] = mTriangleArray[t]->mId1;
            tris[size_t(t) * 3 + 2] = mTriangleArray[t]->mId2;
        }
        for (int e = 0; e < E; e++)
        {
            auto ce = mEdgeArray[e];
            int row[5] = {ce->mId0, ce->mId1, ce->mTriangleId0,
                          ce->mTriangleId1, ce->mIsBoundary ? 1 : 0};
            for (int k = 0; k < 5; k++)
                edges[size_t(e) * 5 + k] = row[k];
            for (int k = 0; k < 4; k++)
                stencil[size_t(e) * 4 + k] = mEdgeAffectVertexId[e][k];
        }
        std::vector<float> area(mTriangleInitArea.begin(),
                                mTriangleInitArea.end());
        std::vector<int> pins(mConstraint_StaticPointIds.begin(),
                              mConstraint_StaticPointIds.end());
        std::vector<double> mass_cpu(n);
        for (int i = 0; i < n; i++)
            mass_cpu[i] = mMassMatrixDiag[3 * i];

        d.put("pos", "f8", pos, {n, 3});
        d.put("uv", "f4", uv, {n, 2});
        d.put("tris", "i4", tris, {T, 3});
        d.put("edges", "i4", edges, {E, 5});
        d.put("stencil", "i4", stencil, {E, 4});
        d.put("tri_area", "f4", area, {T});
        d.put("pins", "i4", pins, {long(pins.size())});
        d.put("mass_cpu", "f8", mass_cpu, {n});
        d.put("mass_gpu", "f8", gpu_mass(), {n});
        d.put("ell", "i4", ell(), {n, kEll});
        d.put("stretch_coef", "f4", stretch_coef(), {T, 12});
        std::vector<float> diag16, edge_k;
        tVector2d kb = cJsonUtil::ReadVectorJson(
                           cJsonUtil::ParseAsValue("cloth_bending_stiffness",
                                                   conf))
                           .segment(0, 2);
        bending(float(kb[0]), float(kb[1]), diag16, edge_k);
        d.put("bend_diag16", "f4", diag16, {E, 16});
        d.put("bend_edge_k", "f4", edge_k, {E});
    }

    // Reference assembled system for one GPU-path step on the given state:
    // stretch/shear from cBaraffMaterial::Update (double), bending from
    // cQBendingMaterial (the GPU's bending model, BaraffClothGpu.cpp:184-207),
    // A and b by the GPU formula (BaraffClothGpu.cu:240-344), pins handled as
    // the GPU solver does (PCGSolver.cu:126-136, 185-222), solved directly.
    void dump_system(Dump &d, std::vector<double> x, std::vector<double> xpre)
    {
        int n = nv(), T = nt();
        // Q-bending is built from the rest state, as InitBendingMatrix is.
        auto qb = std::make_shared<cQBendingMaterial>();
        tVector2d kb = cJsonUtil::ReadVectorJson(
                           cJsonUtil::ParseAsValue("cloth_bending_stiffness",
                                                   conf))
                           .segment(0, 2);
        qb->Init(mVertexArray, mEdgeArray, mTriangleArray,
                 kb[0] * tVector3d::Ones());
        // the CPU cloth's dihedral bending, initialised on the rest state as
        // cBaraffCloth::Init does (BaraffCloth.cpp:36-43: K = (k0, k0, k0) in float)
        auto dih = std::make_shared<cDihedralMaterial>();
        dih->Init(mVertexArray, mEdgeArray, mTriangleArray,
                  (tVector3f::Ones() * float(kb[0])).cast<double>());
        tVector3d ks = cJsonUtil::ReadVectorJson(
                           cJsonUtil::ParseAsValue("cloth_stretch_stiffness",
                                                   conf))
                           .segment(0, 3);
        auto mat = std::make_shared<MatProbe>();
        mat->Init(shared_from_this(), ks);
        std::vector<double> mass = gpu_mass();
        // the bending tables come from the rest state, before SetPos below
        std::vector<float> diag16, edge_k;
        bending(float(kb[0]), float(kb[1]), diag16, edge_k);

        // UpdateConstraintVertexPos (BaraffClothGpu.cpp:411-436)
        for (int vid : mConstraint_StaticPointIds)
            for (int k = 0; k < 3; k++)
            {
                double t = double(float(mClothInitPos[3 * vid + k]));
                x[3 * vid + k] = t;
                xpre[3 * vid + k] = t;
            }
        tVectorXd X = Eigen::Map<tVectorXd>(x.data(), 3 * n);
        tVectorXd XP = Eigen::Map<tVectorXd>(xpre.data(), 3 * n);
        SetPos(X);
        SetPrePos(XP);

        mat->Update();
        std::vector<double> tf(size_t(T) * 9), th(size_t(T) * 81);
        for (int t = 0; t < T; t++)
        {
            const tMatrix3d &F = mat->tri_fint()[t];
            for (int i = 0; i < 3; i++) // vertex i = column i
                for (int k = 0; k < 3; k++)
                    tf[size_t(t) * 9 + i * 3 + k] = F(k, i);
            for (int b = 0; b < 9; b++)
            {
                const tMatrix3d &H = mat->tri_hessian()[size_t(t) * 9 + b];
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++)
                        th[size_t(t) * 81 + b * 9 + r * 3 + c] = H(r, c);
            }
        }
        tVectorXd f_st = mat->CalcTotalForce();
        tSparseMatd K_st = mat->CalcTotalStiffnessMatrix();
        // CPU Q-bending (reference code, isotropic stiffness K_u): the
        // cross-check the reference itself makes (BaraffClothGpu.cpp:184-207).
        tSparseMatd K_qb = qb->GetStiffnessMatrix(); // = -Kb
        // GPU bending: per-edge 4x4 table times the direction-blended edge
        // stiffness, value * I3 per block (UpdateBendingStiffnessMatrixKernel,
        // BaraffClothGpu.cu:387-426), summed in double.
        std::vector<Eigen::Triplet<double>> btrip;
        for (int e = 0; e < ne(); e++)
        {
            if (mEdgeArray[e]->mIsBoundary)
                continue;
            tVector4i s = mEdgeAffectVertexId[e];
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++)
                {
                    float value = diag16[size_t(e) * 16 + i * 4 + j] * edge_k[e];
                    for (int k = 0; k < 3; k++)
                        btrip.emplace_back(3 * s[i] + k, 3 * s[j] + k, double(value));
                }
        }
        tSparseMatd Kb_gpu(3 * n, 3 * n);
        Kb_gpu.setFromTriplets(btrip.begin(), btrip.end());
        tVectorXd f_bd = -(Kb_gpu * X);
        tSparseMatd K = K_st - Kb_gpu;

        double dt = cJsonUtil::ParseAsDouble("default_timestep", conf);
        double ra = cJsonUtil::ParseAsDouble("rayleigh_damping_a", conf);
        double rb = cJsonUtil::ParseAsDouble("rayleigh_damping_b", conf);
        std::vector<int> ellmap = ell();
        // A by the GPU formula from a stiffness matrix (ELL blocks)
        auto build_A = [&](const tSparseMatd &Kt, std::vector<double> &Aout) {
            Aout.assign(size_t(n) * kEll * 9, 0.0);
            for (int i = 0; i < n; i++)
                for (int s = 0; s < kEll; s++)
                {
                    int j = ellmap[size_t(i) * kEll + s];
                    if (j < 0)
                        break;
                    for (int r = 0; r < 3; r++)
                        for (int c = 0; c < 3; c++)
                        {
                            double kv = Kt.coeff(3 * i + r, 3 * j + c);
                            double a = (dt * rb - dt * dt) * kv;
                            if (i == j && r == c)
                                a += (1 + dt * ra) * mass[i];
                            Aout[(size_t(i) * kEll + s) * 9 + r * 3 + c] = a;
                        }
                }
        };
        // b from the stretch force and a bending force
        auto build_b = [&](const tVectorXd &fb, std::vector<double> &bout) {
            bout.assign(size_t(n) * 3, 0.0);
            for (int i = 0; i < n; i++)
                for (int k = 0; k < 3; k++)
                {
                    double g = (k == 1) ? -9.8 * mass[i] : 0.0;
                    bout[3 * i + k] = dt * dt * (g + f_st[3 * i + k] + fb[3 * i + k]) +
                                      mass[i] * (x[3 * i + k] - xpre[3 * i + k]);
                }
        };
        // the pin-projected system (free rows and columns) solved exactly
        std::vector<char> fixed(n, 0);
        for (int vid : mConstraint_StaticPointIds)
            fixed[vid] = 1;
        auto solve = [&](const std::vector<double> &Am, const std::vector<double> &bm) {
            std::vector<int> dof_of(3 * n, -1);
            int nf = 0;
            for (int i = 0; i < n; i++)
                if (!fixed[i])
                    for (int k = 0; k < 3; k++)
                        dof_of[3 * i + k] = nf++;
            std::vector<Eigen::Triplet<double>> trip;
            for (int i = 0; i < n; i++)
            {
                if (fixed[i])
                    continue;
                for (int s = 0; s < kEll; s++)
                {
                    int j = ellmap[size_t(i) * kEll + s];
                    if (j < 0)
                        break;
                    if (fixed[j])
                        continue;
                    for (int r = 0; r < 3; r++)
                        for (int c = 0; c < 3; c++)
                            trip.emplace_back(dof_of[3 * i + r], dof_of[3 * j + c],
                                              Am[(size_t(i) * kEll + s) * 9 + r * 3 + c]);
                }
            }
            Eigen::SparseMatrix<double> Af(nf, nf);
            Af.setFromTriplets(trip.begin(), trip.end());
            tVectorXd bf(nf);
            for (int i = 0; i < 3 * n; i++)
                if (dof_of[i] >= 0)
                    bf[dof_of[i]] = bm[i];
            Eigen::SimplicialLDLT<Eigen::SparseMatrix<double>> ldlt(Af);
            if (ldlt.info() != Eigen::Success)
            {
                std::cerr << "LDLT factorisation failed\n";
                exit(4);
            }
            tVectorXd dxf = ldlt.solve(bf);
            std::vector<double> out(size_t(n) * 3, 0.0);
            for (int i = 0; i < 3 * n; i++)
                if (dof_of[i] >= 0)
                    out[i] = dxf[dof_of[i]];
            return out;
        };

        std::vector<double> A, b;
        build_A(K, A);
        build_b(f_bd, b);
        std::vector<double> dx = solve(A, b);
        std::vector<double> Kst(size_t(n) * kEll * 9, 0.0), Kbd(size_t(n) * kEll, 0.0),
            Kbg(size_t(n) * kEll, 0.0);
        for (int i = 0; i < n; i++)
            for (int s = 0; s < kEll; s++)
            {
                int j = ellmap[size_t(i) * kEll + s];
                if (j < 0)
                    break;
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++)
                        Kst[(size_t(i) * kEll + s) * 9 + r * 3 + c] =
                            K_st.coeff(3 * i + r, 3 * j + c);
                Kbd[size_t(i) * kEll + s] = -K_qb.coeff(3 * i, 3 * j);
                Kbg[size_t(i) * kEll + s] = Kb_gpu.coeff(3 * i, 3 * j);
            }

        // The CPU cloth's bending model (cDihedralMaterial, BaraffCloth.cpp:
        // 36-45, 101, 205-244) on the same state: its force and stiffness
        // replace the quadratic bending in the same GPU-path system.
        dih->Update();
        tVectorXd f_dih = dih->CalcForce(X);
        tSparseMatd K_dih = dih->GetStiffnessMatrix();
        tSparseMatd Kd_tot = K_st + K_dih;
        std::vector<double> Adih, bdih, Kdih(size_t(n) * kEll * 9, 0.0);
        build_A(Kd_tot, Adih);
        build_b(f_dih, bdih);
        std::vector<double> dxdih = solve(Adih, bdih);
        for (int i = 0; i < n; i++)
            for (int s = 0; s < kEll; s++)
            {
                int j = ellmap[size_t(i) * kEll + s];
                if (j < 0)
                    break;
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++)
                        Kdih[(size_t(i) * kEll + s) * 9 + r * 3 + c] =
                            K_dih.coeff(3 * i + r, 3 * j + c);
            }
        std::vector<double> fdih(f_dih.data(), f_dih.data() + 3 * n);
        d.put("dih_f", "f8", fdih, {n, 3});
        d.put("dih_K", "f8", Kdih, {n, kEll, 3, 3});
        d.put("dih_A", "f8", Adih, {n, kEll, 3, 3});
        d.put("dih_b", "f8", bdih, {n, 3});
        d.put("dih_dx", "f8", dxdih, {n, 3});

        std::vector<double> fst(f_st.data(), f_st.data() + 3 * n),
            fbd(f_bd.data(), f_bd.data() + 3 * n), xs(x), xps(xpre);
        d.put("x", "f8", xs, {n, 3});
        d.put("xpre", "f8", xps, {n, 3});
        d.put("tri_fint", "f8", tf, {T, 3, 3});
        d.put("tri_hess", "f8", th, {T, 9, 3, 3});
        d.put("f_stretch", "f8", fst, {n, 3});
        d.put("f_bend", "f8", fbd, {n, 3});
        d.put("K_stretch", "f8", Kst, {n, kEll, 3, 3});
        d.put("Kb_cpu", "f8", Kbd, {n, kEll});
        d.put("Kb_gpu", "f8", Kbg, {n, kEll});
        d.put("A", "f8", A, {n, kEll, 3, 3});
        d.put("b", "f8", b, {n, 3});
        d.put("dx", "f8", dx, {n, 3});
    }

    // The CPU cloth's collision handling against one kinematic body on the
    // state x (cSimScene::PerformCollisionDetection, cBaraffCloth::
    // PrepareCollisionHessian and Repulsion): the body's mesh and normals,
    // the contacts cBVHCollisionDetecter finds, the contact Hessian as ELL
    // blocks, and dx after Repulsion of the given dx.
    void dump_collide(Dump &d, const Json::Value &kb_conf, std::vector<double> x,
                      std::vector<double> dxin)
    {
        int n = nv();
        auto kb = std::make_shared<cKinematicBody>(1);
        kb->Init(kb_conf);
        tVectorXd X = Eigen::Map<tVectorXd>(x.data(), 3 * n);
        SetPos(X);
        // cBaseCloth::Update refreshes the normals after every step
        UpdateTriangleNormal();
        UpdateVertexNormalFromTriangleNormal();
        auto det = std::make_shared<cBVHCollisionDetecter>();
        det->AddObject(shared_from_this(), false);
        det->AddObject(kb, false);
        det->Init();
        det->PerformCD();
        SetPointTriangleCollisionInfo(det->GetObjPointTriangleCollisionInfo(0));
        SetEdgeEdgeCollisionInfo(det->GetObjEdgeEdgeCollisionInfo(0));

        // the body
        const auto &kv = kb->GetVertexArray();
        const auto &kt = kb->GetTriangleArray();
        const auto &ke = kb->GetEdgeArray();
        std::vector<double> kpos, ktn, kvn;
        std::vector<int> ktri, kedge;
        for (auto &v : kv)
            for (int k = 0; k < 3; k++)
            {
                kpos.push_back(v->mPos[k]);
                kvn.push_back(v->mNormal[k]);
            }
        for (auto &t : kt)
        {
            ktri.push_back(t->mId0);
            ktri.push_back(t->mId1);
            ktri.push_back(t->mId2);
            for (int k = 0; k < 3; k++)
                ktn.push_back(t->mNormal[k]);
        }
        for (auto &e : ke)
        {
            kedge.push_back(e->mId0);
            kedge.push_back(e->mId1);
            kedge.push_back(e->mTriangleId0);
            kedge.push_back(e->mIsBoundary ? -1 : e->mTriangleId1);
        }
        long nkv = long(kv.size()), nkt = long(kt.size()), nke = long(ke.size());
        d.put("kb_pos", "f8", kpos, {nkv, 3});
        d.put("kb_vnormal", "f8", kvn, {nkv, 3});
        d.put("kb_tris", "i4", ktri, {nkt, 3});
        d.put("kb_tnormal", "f8", ktn, {nkt, 3});
        d.put("kb_edges", "i4", kedge, {nke, 4});

        // contacts, in the detecter's order
        std::vector<int> pt_i;      // obj0_is_cloth, vertex id, triangle id
        std::vector<double> pt_d;   // normal xyz, depth, bary xyz
        for (auto &c : mPointTriangleCollisionInfo)
        {
            pt_i.push_back(c->obj0_is_cloth_obj1_is_rb ? 1 : 0);
            pt_i.push_back(c->mVertexId0);
            pt_i.push_back(c->mTriangleId1);
            for (int k = 0; k < 3; k++)
                pt_d.push_back(c->mOuterNormal[k]);
            pt_d.push_back(double(c->mDepth));
            for (int k = 0; k < 3; k++)
                pt_d.push_back(c->mBary[k]);
        }
        std::vector<int> ee_i;      // obj0_is_cloth, edge 0, edge 1
        std::vector<double> ee_d;   // normal xyz, depth, bary0, bary1
        for (auto &c : mEdgeEdgeCollisionInfo)
        {
            ee_i.push_back(c->obj0_is_cloth_obj1_is_rb ? 1 : 0);
            ee_i.push_back(c->mEdgeId0);
            ee_i.push_back(c->mEdgeId1);
            for (int k = 0; k < 3; k++)
                ee_d.push_back(c->mOuterNormal[k]);
            ee_d.push_back(double(c->mDepth));
            ee_d.push_back(double(c->mBary0));
            ee_d.push_back(double(c->mBary1));
        }
        long npt = long(mPointTriangleCollisionInfo.size()),
             nee = long(mEdgeEdgeCollisionInfo.size());
        d.put("pt_i", "i4", pt_i, {npt, 3});
        d.put("pt_d", "f8", pt_d, {npt, 7});
        d.put("ee_i", "i4", ee_i, {nee, 3});
        d.put("ee_d", "f8", ee_d, {nee, 6});

        // contact Hessian as ELL blocks
        tSparseMatd H = PrepareCollisionHessian();
        std::vector<int> ellmap = ell();
        std::vector<double> Hb(size_t(n) * kEll * 9, 0.0);
        for (int i = 0; i < n; i++)
            for (int s = 0; s < kEll; s++)
            {
                int j = ellmap[size_t(i) * kEll + s];
                if (j < 0)
                    break;
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++)
                        Hb[(size_t(i) * kEll + s) * 9 + r * 3 + c] =
                            H.coeff(3 * i + r, 3 * j + c);
            }
        d.put("col_H", "f8", Hb, {n, kEll, 3, 3});

        // Repulsion on the given dx
        double dt = cJsonUtil::ParseAsDouble("default_timestep", conf);
        tVectorXd DX = Eigen::Map<tVectorXd>(dxin.data(), 3 * n);
        Repulsion(dt, DX);
        std::vector<double> dxo(DX.data(), DX.data() + 3 * n), xs(x);
        d.put("x", "f8", xs, {n, 3});
        d.put("dx_in", "f8", dxin, {n, 3});
        d.put("dx_out", "f8", dxo, {n, 3});
        std::vector<double> mass_cpu(n);
        for (int i = 0; i < n; i++)
            mass_cpu[i] = mMassMatrixDiag[3 * i];
        d.put("mass_cpu", "f8", mass_cpu, {n});
    }

    // cKinematicBody::Update(dt) `steps` times on a moving body: the local
    // mesh, the vertex positions at Init and after every update, the body
    // clock, and the normals (Init's, which Update leaves alone)
    static void dump_motion(Dump &d, const Json::Value &kb_conf, float dt, int steps)
    {
        auto kb = std::make_shared<MotionBody>(1);
        kb->Init(kb_conf);
        const auto &kv = kb->GetVertexArray();
        const long n = long(kv.size());
        std::vector<double> local(kb->local().data(), kb->local().data() + 3 * n);
        std::vector<double> pos, vn0, vn1;
        std::vector<float> times;
        auto grab = [&](std::vector<double> &out, bool normal) {
            for (auto &v : kv)
                for (int k = 0; k < 3; k++)
                    out.push_back(normal ? v->mNormal[k] : v->mPos[k]);
        };
        grab(pos, false);
        grab(vn0, true);
        times.push_back(kb->time());
        for (int s = 0; s < steps; s++)
        {
            kb->Update(dt);
            grab(pos, false);
            times.push_back(kb->time());
        }
        grab(vn1, true);
        std::vector<int> tris;
        for (auto &t : kb->GetTriangleArray())
        {
            tris.push_back(t->mId0);
            tris.push_back(t->mId1);
            tris.push_back(t->mId2);
        }
        d.put("local", "f8", local, {n, 3});
        d.put("pos", "f8", pos, {long(steps) + 1, n, 3});
        d.put("time", "f4", times, {long(steps) + 1});
        d.put("vnormal_init", "f8", vn0, {n, 3});
        d.put("vnormal_end", "f8", vn1, {n, 3});
        d.put("tris", "i4", tris, {long(tris.size() / 3), 3});
    }

    void step(int nsteps)
    {
        double dt = cJsonUtil::ParseAsDouble("default_timestep", conf);
        auto t0 = std::chrono::steady_clock::now();
        for (int s = 0; s < nsteps; s++)
            UpdatePos(dt);
        auto t1 = std::chrono::steady_clock::now();
        double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        printf("STEP_MS %.3f NV %d NT %d STEPS %d\n", ms / nsteps, nv(), nt(),
               nsteps);
    }
};

int main(int argc, char **argv)
{
    if (argc < 3)
    {
        std::cerr << "usage: ref_harness topo|system|step <cfg.json> ...\n";
        return 1;
    }
    std::string mode = argv[1];
    Json::Value conf;
    if (!cJsonUtil::LoadJson(argv[2], conf))
        return 1;
    if (mode == "geom" && argc >= 5)
    {
        // the geometry generators that draw from the global generator
        // ("regular_triangle_perturb", "delaunay"); main seeds it with 0
        cMathUtil::SeedRand(std::strtoul(argv[3], nullptr, 10));
        std::vector<tVertexPtr> va;
        std::vector<tEdgePtr> ea;
        std::vector<tTrianglePtr> ta;
        cTriangulator::BuildGeometry(conf, va, ea, ta);
        const long n = long(va.size()), T = long(ta.size()), E = long(ea.size());
        std::vector<double> pos(size_t(n) * 3);
        std::vector<float> uv(size_t(n) * 2);
        std::vector<int> tris(size_t(T) * 3), edges(size_t(E) * 5);
        for (long i = 0; i < n; i++)
        {
            for (int k = 0; k < 3; k++)
                pos[size_t(i) * 3 + k] = va[i]->mPos[k];
            uv[size_t(i) * 2 + 0] = va[i]->muv[0];
            uv[size_t(i) * 2 + 1] = va[i]->muv[1];
        }
        for (long t = 0; t < T; t++)
        {
            tris[size_t(t) * 3 + 0] = ta[t]->mId0;
            tris[size_t(t) * 3 + 1] = ta[t]->mId1;
            tris[size_t(t) * 3 + 2] = ta[t]->mId2;
        }
        for (long e = 0; e < E; e++)
        {
            int row[5] = {ea[e]->mId0, ea[e]->mId1, ea[e]->mTriangleId0, ea[e]->mTriangleId1,
                          ea[e]->mIsBoundary ? 1 : 0};
            for (int k = 0; k < 5; k++)
                edges[size_t(e) * 5 + k] = row[k];
        }
        Dump d(argv[4]);
        d.put("pos", "f8", pos, {n, 3});
        d.put("uv", "f4", uv, {n, 2});
        d.put("tris", "i4", tris, {T, 3});
        d.put("edges", "i4", edges, {E, 5});
        return 0;
    }
    auto c = std::make_shared<Probe>(0);
    c->conf = conf;
    c->Init(conf);
    if (mode == "topo" && argc >= 4)
    {
        Dump d(argv[3]);
        c->dump_topo(d);
    }
    else if (mode == "system" && argc >= 6)
    {
        size_t n3 = size_t(c->nv()) * 3;
        Dump d(argv[5]);
        c->dump_system(d, read_doubles(argv[3], n3), read_doubles(argv[4], n3));
    }
    else if (mode == "collide" && argc >= 7)
    {
        Json::Value kb;
        if (!cJsonUtil::LoadJson(argv[3], kb))
            return 1;
        size_t n3 = size_t(c->nv()) * 3;
        Dump d(argv[6]);
        c->dump_collide(d, kb, read_doubles(argv[4], n3), read_doubles(argv[5], n3));
    }
    else if (mode == "motion" && argc >= 7)
    {
        // motion <cloth cfg> <body cfg> <dt> <steps> <outdir>
        Json::Value kb;
        if (!cJsonUtil::LoadJson(argv[3], kb))
            return 1;
        Dump d(argv[6]);
        Probe::dump_motion(d, kb, float(std::atof(argv[4])), std::atoi(argv[5]));
    }
    else if (mode == "step" && argc >= 4)
    {
        if (argc >= 6)
        {
            size_t n3 = size_t(c->nv()) * 3;
            std::vector<double> x = read_doubles(argv[4], n3),
                                xp = read_doubles(argv[5], n3);
            c->SetPos(Eigen::Map<tVectorXd>(x.data(), n3));
            c->SetPrePos(Eigen::Map<tVectorXd>(xp.data(), n3));
        }
        c->step(std::atoi(argv[3]));
    }
    else
    {
        std::cerr << "bad arguments\n";
        return 1;
    }
    return 0;
}
