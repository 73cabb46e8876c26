"""GPU parity of the dihedral bending model (the CPU cloth's cDihedralMaterial,
src/sim/cloth/DihedralBending.cpp) against the reference's own arrays and the
FP64 oracle.

The model gives every block of A a skew part, so these tests also cover the
skew-aware SpMV of every solver.  Tolerances as in test_gpu_parity: assembled
arrays within 1e-5 relative per array, solutions through their true FP64
residual on the reference system."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, project_pins, rel

pytestmark = pytest.mark.gpu

TOL_ASSEMBLY = 1e-5


def _dih(conf):
    return dict(conf, cloth_bending_model="dihedral")


def make(ctx, conf):
    from acousticsim_gb300 import BaraffClothGpu
    return BaraffClothGpu(ctx, conf)


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_dihedral_assembly_matches_reference(ctx, orc, case):
    g, conf = load_golden(case)
    c = make(ctx, _dih(conf))
    c.SetPos(g["x_in"])
    c.SetPrePos(g["xpre_in"])
    c.assemble()
    s = c.export_system()
    dg = c.export_dihedral()
    # per-edge gradients and factors against the oracle at the pin-snapped state
    oc = orc.OracleCloth(c.mesh, _dih(conf), g["topo_pins"])
    oc.x = g["x_in"].reshape(-1).copy()
    oc.snap_pins()
    od = orc.dihedral(oc.tab, oc.dfac, oc.x)
    interior = np.flatnonzero(c.mesh["edges"][:, 3] >= 0)
    assert np.array_equal(dg["edge_ids"], interior)
    GA, Gb = project_pins(g["sys_dih_A"], g["sys_dih_b"], g["topo_ell"], g["topo_pins"])
    errs = {
        "grad": rel(dg["grad"], od["grad"][interior]),
        "factor": rel(dg["factor"], oc.dfac[interior]),
        "force_coef": rel(dg["force_coef"], oc.dfac[interior] * od["beta"][interior] / 2),
        "fint": rel(s["fint"], g["sys_f_stretch"] + g["sys_dih_f"]),
        "A": rel(s["A"], GA),
        "b": rel(s["b"], Gb),
    }
    print(case, errs)
    for k, e in errs.items():
        assert e < TOL_ASSEMBLY, (k, e)
    assert np.all(s["kbend"] == 0)  # the quadratic model is off
    # the skew parts are really there: A is not block-symmetric
    assert np.abs(s["A"] - np.swapaxes(s["A"], 2, 3)).max() > 0
    c.close()


SOLVERS = ["persistent", "persistent_1b", "graph_loop"]


@pytest.fixture(params=SOLVERS)
def solver(request, ctx):
    ctx.set_solver(request.param)
    yield request.param
    ctx.set_solver("persistent")


def _ran(solver):
    # the single-barrier kernel has no skew parts: those sets take the
    # two-barrier persistent kernel, and the stats say so
    return "persistent" if solver == "persistent_1b" else solver


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_dihedral_solve_matches_direct_solve(ctx, orc, case, solver):
    from acousticsim_gb300 import params
    g, conf = load_golden(case)
    c = make(ctx, _dih(conf))
    c.SetPos(g["x_in"])
    c.SetPrePos(g["xpre_in"])
    c.assemble()
    st = c.solve(params(max_iters=20000, rel_tol=1e-6))
    assert st["status"] == "OK", st
    assert st["solver"] == _ran(solver)
    dx = c.get_dx()
    GA, Gb = project_pins(g["sys_dih_A"], g["sys_dih_b"], g["topo_ell"], g["topo_pins"])
    r = Gb.reshape(-1) - orc.spmv(g["topo_ell"], GA, dx)
    true_rel = np.linalg.norm(r) / np.linalg.norm(Gb)
    err = rel(dx, g["sys_dih_dx"].reshape(-1))
    print(case, "iters", st["iters"], "true residual", true_rel, "dx error", err)
    assert true_rel < 5e-6
    assert err < 2e-4  # measured up to 4e-5
    # the FP64 residual kernel applies the skew parts too: it equals the
    # residual of the exported system formed here in FP64, up to the one
    # extra float rounding of the exported entries that hold a skew part
    # (S + W is summed in float by the export, kept apart by the kernel)
    sy = c.export_system()
    A64, b64 = sy["A"].astype(np.float64), sy["b"].astype(np.float64).reshape(-1)
    own = np.linalg.norm(b64 - orc.spmv(sy["ell"], A64, dx)) / np.linalg.norm(b64)
    bound = 1.2e-7 * np.linalg.norm(A64) * np.linalg.norm(dx) / np.linalg.norm(b64)
    skew = 0.5 * (A64 - np.swapaxes(A64, 2, 3))
    skew_part = np.linalg.norm(orc.spmv(sy["ell"], skew, dx)) / np.linalg.norm(b64)
    print("fp64 residual", c.residual_fp64(), "numpy", own, "bound", bound, "skew part",
          skew_part)
    assert abs(c.residual_fp64() - own) <= bound
    c.close()


def test_dihedral_dominated_assembly_vs_oracle(ctx, orc):
    """No stretch stiffness and a stiff dihedral model: A - M, b and the
    internal force are the dihedral terms alone, compared with the oracle
    block by block, skew parts included."""
    dt = 5e-3
    conf = _grid_conf(20, dt, ks=(0.0, 0.0, 0.0), kb=(1.0, 1.0))
    c = make(ctx, conf)
    x, xp = _perturbed(c, 21, dt, sx=1e-2)
    c.SetPos(x)
    c.SetPrePos(xp)
    c.assemble()
    s = c.export_system()
    oc = orc.OracleCloth(c.mesh, conf, c.GetConstraintStaticVertices())
    oc.x, oc.xpre = x.copy(), xp.copy()
    A, b, f, _, _ = oc.system()
    diag = np.zeros_like(A)
    nv = A.shape[0]
    ell = oc.tab["ell"]
    for v in range(nv):
        sd = int(np.flatnonzero(ell[v] == v)[0])
        diag[v, sd] = np.eye(3) * (1 + dt * 0.01) * oc.tab["mass"][v]
    Ag = s["A"].astype(np.float64)
    errs = {"A - M": rel(Ag - diag, A - diag),
            "skew": rel(0.5 * (Ag - np.swapaxes(Ag, 2, 3)), 0.5 * (A - np.swapaxes(A, 2, 3))),
            "b": rel(s["b"], b), "fint": rel(s["fint"], f)}
    print(errs)
    for k, e in errs.items():
        assert e < 1e-5, (k, e)
    c.close()


def _grid_conf(n, dt=2e-3, ks=(1e3, 1e3, 1e2), kb=(1e-3, 1e-3), pins=True):
    conf = {"geometry_type": "regular_triangle", "cloth_size": [1.0, 1.0],
            "subdivision": [n - 1, n - 1], "cloth_init_pos": [0.0, 0.0, 0.0],
            "cloth_uv_rotation": 0, "cloth_stretch_stiffness": list(ks),
            "cloth_bending_stiffness": list(kb), "cloth_density": 0.1,
            "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0, "default_timestep": dt,
            "cloth_bending_model": "dihedral"}
    if pins:
        conf["constraints"] = {"static_point": [[-0.5, 0.5], [0.5, 0.5]]}
    return conf


def _perturbed(c, seed, dt, sx=1e-3, sv=1e-2):
    rng = np.random.default_rng(seed)
    x0 = c.GetInitPos().reshape(-1, 3)
    x = x0 + rng.normal(0, sx, x0.shape)
    v = rng.normal(0, sv, x0.shape)
    return x.reshape(-1), (x - dt * v).reshape(-1)


def test_dihedral_trajectory_vs_oracle(ctx, orc, solver):
    """20 steps of a 48x48 cloth with dihedral bending (stiff enough to matter)
    against the FP64 oracle stepping the same state."""
    from acousticsim_gb300 import params
    n, dt = 48, 2e-3
    conf = _grid_conf(n, dt, kb=(1e-1, 1e-1))
    c = make(ctx, conf)
    x, xp = _perturbed(c, 7, dt)
    c.SetPos(x)
    c.SetPrePos(xp)
    oc = orc.OracleCloth(c.mesh, conf, c.GetConstraintStaticVertices())
    oc.x, oc.xpre = x.copy(), xp.copy()
    for _ in range(20):
        st = c.UpdatePos(0.0, params(max_iters=20000, rel_tol=1e-7))
        assert st["status"] == "OK" and st["solver"] == _ran(solver), st
        oc.step(rel_tol=1e-12)
    disp_err = rel(c.GetPos() - x, oc.x - x)
    print("displacement error after 20 steps", disp_err)
    assert disp_err < 2e-4  # measured 4.9e-5
    c.close()


def test_dihedral_changes_the_motion(ctx):
    """The bending model matters: with a large bending stiffness the dihedral
    and quadratic cloths part ways."""
    from acousticsim_gb300 import params
    p = params(max_iters=20000, rel_tol=1e-7)
    out = []
    for model in ("dihedral", "quadratic"):
        conf = dict(_grid_conf(32, kb=(1.0, 1.0)), cloth_bending_model=model)
        c = make(ctx, conf)
        x, xp = _perturbed(c, 5, 2e-3)
        c.SetPos(x)
        c.SetPrePos(xp)
        for _ in range(5):
            assert c.UpdatePos(0.0, p)["status"] == "OK"
        out.append(c.GetPos() - x)
        c.close()
    assert rel(out[0], out[1]) > 1e-3


@pytest.mark.parametrize("bsolver", ["persistent", "graph_loop"])
def test_mixed_models_batch_equals_alone_bit_exact(ctx, bsolver):
    """Dihedral and quadratic cloths in one launch set: each result is
    bit-identical to stepping that cloth alone."""
    from acousticsim_gb300 import params
    p = params(max_iters=5000, rel_tol=1e-6)
    ctx.set_solver(bsolver)
    specs = [(17, "dihedral"), (40, "quadratic"), (23, "dihedral"), (12, "quadratic")]
    alone, mixed = [], []
    for k, (n, model) in enumerate(specs):
        conf = dict(_grid_conf(n, ks=(10 ** (2 + k % 2),) * 2 + (10 ** (1 + k % 2),),
                               kb=(1e-2, 1e-2)), cloth_bending_model=model)
        a, m = make(ctx, conf), make(ctx, conf)
        x, xp = _perturbed(a, 200 + k, 2e-3)
        for c in (a, m):
            c.SetPos(x)
            c.SetPrePos(xp)
        alone.append(a)
        mixed.append(m)
    ref = []
    for a in alone:
        its = []
        for _ in range(3):
            its.append(a.UpdatePos(0.0, p)["iters"])
        ref.append((a.GetPos(), its))
    its_m = [[] for _ in mixed]
    for _ in range(3):
        stats = ctx.batch_step(mixed, 0.0, p)
        assert all(s["status"] == "OK" and s["solver"] == bsolver for s in stats), stats
        for i, s in enumerate(stats):
            its_m[i].append(s["iters"])
    ctx.set_solver("persistent")
    for (x, its), m, im in zip(ref, mixed, its_m):
        assert its == im
        assert np.array_equal(x, m.GetPos())
    for c in alone + mixed:
        c.close()


def test_dihedral_kernel_variants_bit_identical(ctx):
    """Every skew-aware graph-loop SpMV variant gives the same trajectory."""
    from acousticsim_gb300 import ClothContext, params
    p = params(max_iters=5000, rel_tol=1e-6)
    confs = [_grid_conf(n, kb=(1e-2, 1e-2)) for n in (12, 33, 20)]

    def run(sv):
        ctx.set_solver("graph_loop")
        ctx.set_kernel_variant(sv, (1, 1), autotune=False)
        cl = []
        for k, conf in enumerate(confs):
            c = make(ctx, conf)
            x, xp = _perturbed(c, 400 + k, 2e-3)
            c.SetPos(x)
            c.SetPrePos(xp)
            cl.append(c)
        for _ in range(2):
            st = ctx.batch_step(cl, 0.0, p)
            assert all(s["status"] == "OK" for s in st), st
        out = [c.GetPos() for c in cl]
        for c in cl:
            c.close()
        return out

    ref = run((1, 1, 1))
    for sv in ClothContext.SPMV_VARIANTS[1:]:
        got = run(sv)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), sv
    ctx.set_kernel_variant((1, 3, 1), (1, 1), autotune=True)
    ctx.set_solver("persistent")


def test_dihedral_fp64_solvers(ctx, orc):
    """FP64 PCG and FP32-in-FP64 refinement on a dihedral system reach 1e-8
    and agree with the FP64 oracle's solution."""
    from acousticsim_gb300 import params
    g, conf = load_golden("grid20")
    c = make(ctx, _dih(conf))
    c.SetPos(g["x_in"])
    c.SetPrePos(g["xpre_in"])
    c.assemble()
    st = c.solve_fp64(params(max_iters=20000, rel_tol=1e-10))
    assert st["status"] == "OK", st
    assert c.residual_fp64() < 1e-8
    dx64 = c.get_dx()
    assert rel(dx64, g["sys_dih_dx"].reshape(-1)) < 1e-5
    rs = c.solve_refined(params(max_iters=2000, rel_tol=1e-5), rel_tol=1e-8)
    assert rs["status"] == "OK", rs
    assert c.residual_fp64() < 1e-8
    assert rel(c.get_dx(), g["sys_dih_dx"].reshape(-1)) < 1e-5
    # flexible CG over FP32 PCG steps (the skew block parts in both)
    fs = c.solve_flexible(params(max_iters=20, rel_tol=0.0, warm_start=0), 1e-10, 5000)
    assert fs["status"] == "OK" and fs["rejected"] == 0, fs
    assert c.residual_fp64() < 2e-10
    assert rel(c.get_dx(), g["sys_dih_dx"].reshape(-1)) < 1e-5
    c.close()


def test_dihedral_server_equals_alone(ctx):
    """Served dihedral cloths (skew-aware chunk graph) give the results of
    stepping them alone."""
    from acousticsim_gb300 import ClothServer, params
    p = params(max_iters=5000, rel_tol=1e-6)
    specs = [(14, 2), (25, 3), (18, 1)]
    ctx.set_solver("graph_loop")
    alone = []
    for k, (n, steps) in enumerate(specs):
        c = make(ctx, _grid_conf(n, kb=(1e-2, 1e-2)))
        x, xp = _perturbed(c, 500 + k, 2e-3)
        c.SetPos(x)
        c.SetPrePos(xp)
        its = [c.UpdatePos(0.0, p)["iters"] for _ in range(steps)]
        alone.append((c.GetPos(), its))
        c.close()
    ctx.set_solver("persistent")
    srv = ClothServer(ctx, 1 << 30, 0, 4)
    cl = []
    for k, (n, _) in enumerate(specs):
        c = make(ctx, _grid_conf(n, kb=(1e-2, 1e-2)))
        x, xp = _perturbed(c, 500 + k, 2e-3)
        c.SetPos(x)
        c.SetPrePos(xp)
        cl.append(c)
    idx = [srv.add(c, 0.0, p) for c in cl]
    srv.start()
    order = [i for i, (_, s) in enumerate(specs) for _ in range(s)]
    for tag, i in enumerate(order):
        srv.submit(idx[i], tag)
    srv.drain(60.0)
    res = sorted(srv.poll(cap=len(order) + 4), key=lambda r: r["tag"])
    assert len(res) == len(order)
    per = {i: [] for i in range(len(specs))}
    for r in res:
        assert r["status"] == "OK", r
        per[order[r["tag"]]].append(r["iters"])
    got = [c.GetPos() for c in cl]
    srv.close()
    for c in cl:
        c.close()
    for i, ((x, its), xs) in enumerate(zip(alone, got)):
        assert per[i] == its, (i, per[i], its)
        assert np.array_equal(x, xs), i


def test_dihedral_refusals(ctx):
    """The bending model is fixed at creation; the reference-structured path
    has the GPU cloth's quadratic bending only."""
    from acousticsim_gb300 import ClothError, params
    conf = _grid_conf(12)
    c = make(ctx, conf)
    with pytest.raises(ClothError):
        c.SetMaterial(dict(conf, cloth_bending_model="quadratic"))
    with pytest.raises(ClothError):
        c.UpdatePosPlain(0.0, params(max_iters=100, rel_tol=1e-6))
    # a stiffness change rebuilds the per-edge factors
    c.SetMaterial(dict(conf, cloth_bending_stiffness=[2e-3, 2e-3]))
    c.assemble()
    f2 = c.export_dihedral()["factor"]
    c.SetMaterial(conf)
    c.assemble()
    f1 = c.export_dihedral()["factor"]
    assert np.allclose(f2, 2 * f1, rtol=1e-6)
    c.close()
