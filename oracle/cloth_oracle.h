/*
 * cloth_oracle.h - CPU restatement of AcousticSim's implicit cloth step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load this library, as the checker; the product
 * (acousticsim_gb300) never links or calls it.
 *
 * Per-step arithmetic is FP64 (the reference's CPU cloth path computes in
 * double); init-time tables follow the reference's float/double rounding so
 * they can be compared bit for bit with the golden fixtures produced by the
 * reference itself (oracle/ref_harness.cpp).  Blocks are row-major 3x3.
 * ELL rows are CLOTH_ORC_W = 32 wide, -1 padded, sorted (mELLVidToGlobalVid).
 */
#ifndef CLOTH_ORACLE_H
#define CLOTH_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

#define CLOTH_ORC_W 32

/* Regular grid numbering: cTriangulator::BuildGeometry_UniformTriangle
 * (src/geometries/Triangulator.cpp:141-457, 621-658). Sizes with NULL outputs. */
int orc_grid(const double size[2], const int subdiv[2], const double init_pos[3],
             float uv_rotation_deg, int *nv, int *nt, int *ne, double *pos,
             float *uv, int *tris, int *edges /* ne*4 */);

/* Init-time tables (cBaseCloth::InitGeometry/InitMass, cBaraffClothGpu::
 * InitELLMatrix/InitStretchCoef/InitBendingMatrix/UpdateBendingMatrix).
 * Outputs: stencil ne*4, area nt (float), mass nv, ell nv*32, coef nt*12,
 * diag16 ne*16, edge_k ne, kbend nv*32 (bending scalar per ELL block).
 * Returns 0, or -1 when a row is wider than 32. */
int orc_tables(int nv, int nt, int ne, const double *pos, const float *uv,
               const int *tris, const int *edges, float density,
               const float bending_k[2], int *stencil, float *area, double *mass,
               int *ell, float *coef, float *diag16, float *edge_k,
               double *kbend);

/* Per-triangle stretch/shear force and Hessian blocks in FP64
 * (cBaraffMaterial::Update, src/sim/cloth/BaraffMaterial.cpp:173-256).
 * fint nt*9 (force on local vertex a at [3a+k]), hess nt*81 (block (a,b) at
 * [9*(3a+b)]). fix_fv_norm = 0 keeps the reference's |Fu| in the weft term. */
void orc_triangles(int nt, const int *tris, const float *coef, const float *area,
                   const double *x, const float stretch_k[3], int fix_fv_norm,
                   double *fint, double *hess);

/* Assembled system of one GPU-path step (BaraffClothGpu.cu:127-483):
 * A nv*32*9 and b nv*3, with pins (fixed[v] != 0) projected as the GPU solver
 * treats them: off-diagonal blocks of pinned rows and columns zeroed, b = 0 on
 * pinned rows.  Also returns the total internal force fint nv*3. */
void orc_system(int nv, int nt, const int *tris, const int *ell,
                const double *tri_f, const double *tri_h, const double *kbend,
                const double *mass, double gravity, const double *x,
                const double *xpre, const unsigned char *fixed, double dt,
                float ray_a, float ray_b, double *A, double *b, double *fint);

/* The same with a second bending model added: bend_K nv*32*9 (added to K)
 * and bend_f nv*3 (added to the internal force); kbend may be NULL. */
void orc_system_ex(int nv, int nt, const int *tris, const int *ell,
                   const double *tri_f, const double *tri_h, const double *kbend,
                   const double *bend_K, const double *bend_f, const double *mass,
                   double gravity, const double *x, const double *xpre,
                   const unsigned char *fixed, double dt, float ray_a, float ray_b,
                   double *A, double *b, double *fint);

/* Dihedral bending of the CPU cloth (cDihedralMaterial, DihedralBending.cpp).
 * Rest factors per edge (0 on the boundary): -K e / max(1e-7, h0 + h1) from
 * float rest lengths and Heron areas, K = bending_k0. */
int orc_dihedral_rest(int nv, int nt, int ne, const double *pos, const int *tris,
                      const int *edges, float bending_k0, double *factor);
/* Force and stiffness at positions x: fint nv*3 and K nv*32*9 are ADDED TO;
 * beta_out (ne) and grad_out (ne*12, dbeta/dx of v0..v3) may be NULL. */
void orc_dihedral(int nv, int ne, const int *stencil, const double *factor,
                  const double *x, const int *ell, double *fint, double *K,
                  double *beta_out, double *grad_out);

/* Collisions of the CPU cloth with one static kinematic body
 * (cBVHCollisionDetecter, cBaraffCloth::PrepareCollisionHessian / Repulsion).
 * Body normals as the body's Init leaves them: tnormal nt*3, vnormal nv*3. */
void orc_body_normals(int nv, int nt, const double *pos, const int *tris, double *tnormal,
                      double *vnormal);
/* Contacts in the detecter's order.  pt_i: (cloth point?, point id, triangle
 * id) with pt_d: (normal, depth, bary); ee_i: (1, cloth edge, body edge) with
 * ee_d: (normal, depth, bary0, bary1).  Returns -1 when a list overflowed. */
int orc_contacts(int nv, int nt, int ne, const double *x, const int *tris, const int *edges,
                 int bnv, int bnt, int bne, const double *bpos, const int *btris,
                 const int *bedges, const double *btn, const double *bvn, int max_pt,
                 int *pt_i, double *pt_d, int *n_pt, int max_ee, int *ee_i, double *ee_d,
                 int *n_ee);
/* The contact Hessian added into H (nv*32*9). */
void orc_contact_hessian(int nv, const int *tris, const int *ell, int n_pt, const int *pt_i,
                         const double *pt_d, double *H);
/* Repulsion of dx (nv*3, in place). */
void orc_repulsion(int nv, const int *tris, const int *edges, const double *mass,
                   const float stretch_k[3], double dt, int n_pt, const int *pt_i,
                   const double *pt_d, int n_ee, const int *ee_i, const double *ee_d,
                   double *dx);

/* y = A x over ELL blocks. */
void orc_spmv(int nv, const int *ell, const double *A, const double *x, double *y);

/* Block-Jacobi PCG in FP64 (PCGSolver::Solve, PCGSolver.cu:332-481, with the
 * convergence test on ||r|| <= rel_tol ||b||).  x is the start and the result;
 * pinned entries are set to zero.  Returns the iteration count; *res = ||r||. */
int orc_pcg(int nv, const int *ell, const double *A, const double *b,
            const unsigned char *fixed, double *x, int max_iters, double rel_tol,
            double *res, int nthreads);

/* Number of OpenMP threads available (1 without OpenMP). */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
