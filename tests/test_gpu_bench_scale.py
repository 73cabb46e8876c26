"""Parity at the benchmark's own scale.

The golden fixtures are small (up to 20x20 grids and two OBJ meshes).  Here a
256x256 cloth (65,536 vertices, 130,050 triangles) with the benchmark's
materials, pins and seeded perturbation (x += N(0, 1e-3), v = N(0, 0.01),
dt = 2 ms) is assembled on the GPU and checked array by array against the FP64
oracle (the CPU restatement of cBaraffClothGpu's step, pinned to the
reference's golden arrays): per-triangle forces and Hessian blocks, the total
internal force, A and b, each within 1e-5 relative.  The GPU solve (both PCG
drivers) is then checked by its true FP64 residual on its own system and on
the oracle's FP64 system, and the GPU's FP64-refined solve against the
oracle's solve of the same system to 1e-10."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

N_SIDE = 256
DT = 2e-3
TOL_ASSEMBLY = 1e-5


def _bench_conf(n):
    return {"geometry_type": "regular_triangle", "cloth_size": [1.0, 1.0],
            "subdivision": [n - 1, n - 1], "cloth_init_pos": [0.0, 0.0, 0.0],
            "cloth_uv_rotation": 0, "cloth_stretch_stiffness": [1e3, 1e3, 1e2],
            "cloth_bending_stiffness": [1e-3, 1e-3], "cloth_density": 0.1,
            "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0, "default_timestep": DT,
            "constraints": {"static_point": [[-0.5, 0.5], [0.5, 0.5]]}}


def _bench_state(pos, seed=1234, sx=1e-3):
    rng = np.random.default_rng(seed)
    p = pos.reshape(-1, 3)
    x = p + rng.normal(0.0, sx, p.shape)
    v = rng.normal(0.0, 1e-2, p.shape)
    return x.reshape(-1).copy(), (x - DT * v).reshape(-1).copy()


@pytest.fixture(scope="module")
def bench_case(built):
    from oracle import oracle as orc
    from acousticsim_gb300 import build_grid
    conf = _bench_conf(N_SIDE)
    mesh = build_grid((1.0, 1.0), (N_SIDE - 1, N_SIDE - 1))
    x, xp = _bench_state(mesh["pos"])
    pins = [N_SIDE - 1, N_SIDE * N_SIDE - 1]
    oc = orc.OracleCloth(mesh, conf, pins)
    oc.x, oc.xpre = x.copy(), xp.copy()
    A, b, f, tf, th = oc.system()
    return {"conf": conf, "x": x, "xp": xp, "pins": pins, "oc": oc, "A": A, "b": b, "f": f,
            "tf": tf, "th": th}


def test_bench_scale_assembly_matches_oracle(ctx, bench_case):
    from acousticsim_gb300 import BaraffClothGpu
    bc = bench_case
    c = BaraffClothGpu(ctx, bc["conf"])
    assert sorted(c.GetConstraintStaticVertices()) == sorted(bc["pins"])
    c.SetPos(bc["x"])
    c.SetPrePos(bc["xp"])
    c.assemble()
    s = c.export_system()
    tr = c.export_triangles()
    assert np.array_equal(s["ell"], bc["oc"].tab["ell"])
    errs = {"tri_fint": rel(tr["fint"], bc["tf"]), "tri_hess": rel(tr["hess"], bc["th"]),
            "fint": rel(s["fint"], bc["f"]), "A": rel(s["A"], bc["A"]), "b": rel(s["b"], bc["b"])}
    print(f"{N_SIDE}x{N_SIDE} assembly vs FP64 oracle:", {k: f"{v:.2e}" for k, v in errs.items()})
    for k, e in errs.items():
        assert e < TOL_ASSEMBLY, (k, e)
    c.close()


@pytest.mark.parametrize("solver", ["persistent", "graph_loop"])
def test_bench_scale_solve_meets_tolerance_on_oracle_system(ctx, bench_case, solver):
    """The benchmark's PCG tolerance (1e-6 relative residual) holds for the GPU
    dx on its own system and, up to the FP32 rounding of the assembly, on the
    oracle's FP64 system.  At this size the system's condition number is
    ~1e3, so a 1e-6 residual (or the ~1e-5 FP32 rounding of the forces of a
    nearly flat cloth) allows ~1e-3 in dx itself; dx is compared tightly in
    the next test, where both sides solve the same FP64 system to 1e-10."""
    from acousticsim_gb300 import BaraffClothGpu, params
    from oracle import oracle as orc
    bc = bench_case
    ctx.set_solver(solver)
    c = BaraffClothGpu(ctx, bc["conf"])
    c.SetPos(bc["x"])
    c.SetPrePos(bc["xp"])
    c.assemble()
    s = c.export_system()
    st = c.solve(params(max_iters=20000, rel_tol=1e-6))
    ctx.set_solver("persistent")
    assert st["status"] == "OK" and st["solver"] == solver, st
    dx = c.get_dx()
    A64 = s["A"].astype(np.float64)
    b64 = s["b"].astype(np.float64).reshape(-1)
    own = np.linalg.norm(b64 - orc.spmv(s["ell"], A64, dx)) / np.linalg.norm(b64)
    bo = bc["b"].reshape(-1)
    on_oracle = np.linalg.norm(bo - orc.spmv(bc["oc"].tab["ell"], bc["A"], dx)) / np.linalg.norm(bo)
    if "dx_ref" not in bc:
        bc["dx_ref"], _, _ = orc.pcg(bc["oc"].tab["ell"], bc["A"], bc["b"], bc["oc"].fixed,
                                     rel_tol=1e-10, threads=orc.max_threads())
    err = rel(dx, bc["dx_ref"])
    print(f"{solver}: iters {st['iters']} residual on own system {own:.2e}, on the oracle "
          f"system {on_oracle:.2e}; dx vs oracle (1e-10) {err:.2e}")
    assert own < 5e-6
    assert on_oracle < 2e-5
    assert err < 1e-2  # condition number x tolerance, see the docstring
    c.close()


def test_bench_scale_refined_solve_matches_oracle_tightly(ctx, bench_case):
    """FP32 PCG inside FP64 iterative refinement on the GPU, to 1e-10 FP64
    residual, against the oracle's FP64 PCG on the same exported system to
    1e-10: the two solutions of one FP64 system agree to ~1e-7."""
    from acousticsim_gb300 import BaraffClothGpu, params
    from oracle import oracle as orc
    bc = bench_case
    c = BaraffClothGpu(ctx, bc["conf"])
    c.SetPos(bc["x"])
    c.SetPrePos(bc["xp"])
    c.assemble()
    s = c.export_system()
    st = c.solve_refined(params(max_iters=20000, rel_tol=1e-5), 1e-10, 40)
    assert st["status"] == "OK", st
    dx = c.get_dx()
    A64 = s["A"].astype(np.float64)
    b64 = s["b"].astype(np.float64)
    ref, it, _ = orc.pcg(s["ell"], A64, b64, bc["oc"].fixed, rel_tol=1e-10,
                         threads=orc.max_threads())
    err = rel(dx, ref)
    res = np.linalg.norm(b64.reshape(-1) - orc.spmv(s["ell"], A64, dx)) / np.linalg.norm(b64)
    print(f"refined: {st}; FP64 residual {res:.2e}; oracle iters {it}; dx vs oracle {err:.2e}")
    assert res < 2e-10
    assert err < 1e-5
    c.close()
