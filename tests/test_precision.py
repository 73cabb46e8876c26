"""FP64 residual, mixed-precision iterative refinement and the all-FP64 PCG
on an ill-conditioned system (stretch / bending stiffness 1e7, dt = 10 ms),
checked against a sparse direct solve in FP64 of the same assembled system."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-8


def _conf(n, k_stretch=1e5, k_bend=1e-2, dt=1e-2):
    return {"geometry_type": "regular_triangle", "cloth_size": [1.0, 1.0],
            "subdivision": [n - 1, n - 1], "cloth_init_pos": [0.0, 0.0, 0.0],
            "cloth_uv_rotation": 0,
            "cloth_stretch_stiffness": [k_stretch, k_stretch, k_stretch / 10],
            "cloth_bending_stiffness": [k_bend, k_bend], "cloth_density": 0.1,
            "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0, "default_timestep": dt,
            "constraints": {"static_point": [[-0.5, 0.5], [0.5, 0.5]]}}


def _assembled(ctx, n=48, seed=17):
    from acousticsim_gb300 import BaraffClothGpu
    c = BaraffClothGpu(ctx, _conf(n))
    rng = np.random.default_rng(seed)
    x0 = c.GetInitPos().reshape(-1, 3)
    x = x0 + rng.normal(0, 1e-3, x0.shape)
    xp = x - 1e-2 * rng.normal(0, 1e-2, x0.shape)
    c.SetPos(x.reshape(-1))
    c.SetPrePos(xp.reshape(-1))
    c.assemble(1e-2)
    return c


def _direct(sysd):
    """FP64 sparse LU of the exported (FP32-assembled) system."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    ell, A = sysd["ell"], sysd["A"].astype(np.float64)
    nv, W = ell.shape
    rows, cols, vals = [], [], []
    for s in range(W):
        m = ell[:, s] >= 0
        v = np.nonzero(m)[0]
        cc = ell[m, s]
        for a in range(3):
            for b in range(3):
                rows.append(3 * v + a)
                cols.append(3 * cc + b)
                vals.append(A[m, s, a, b])
    M = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(3 * nv, 3 * nv))
    b = sysd["b"].astype(np.float64).reshape(-1)
    x = spl.splu(M, permc_spec="MMD_AT_PLUS_A").solve(b)
    return M, b, x


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_refinement_reaches_fp64_tolerance(ctx):
    from acousticsim_gb300 import params
    c = _assembled(ctx)
    sysd = c.export_system()
    M, b, x_direct = _direct(sysd)
    st = c.solve_refined(params(max_iters=20000, rel_tol=1e-4, warm_start=0), REL_TOL, 30)
    assert st["status"] == "OK", st
    assert st["rel_residual"] <= REL_TOL and st["outer"] >= 2, st
    assert st["initial_rel_residual"] == pytest.approx(1.0)
    dx = c.get_dx()
    # the FP64 residual of the library matches one formed here
    r_host = np.linalg.norm(b - M @ dx) / np.linalg.norm(b)
    assert r_host <= 2 * REL_TOL
    assert abs(c.residual_fp64() - r_host) <= 1e-2 * r_host + 1e-15
    err = _rel(dx, x_direct)
    print(f"refined: {st}, error vs direct {err:.2e}")
    assert err < 1e-5


def test_fp64_pcg_matches_direct_solve(ctx):
    from acousticsim_gb300 import params
    c = _assembled(ctx)
    M, b, x_direct = _direct(c.export_system())
    st = c.solve_fp64(params(max_iters=50000, rel_tol=REL_TOL))
    assert st["status"] == "OK" and st["solver"] == "fp64", st
    dx = c.get_dx()
    r_host = np.linalg.norm(b - M @ dx) / np.linalg.norm(b)
    assert r_host <= 2 * REL_TOL
    err = _rel(dx, x_direct)
    print(f"fp64 pcg: {st}, true residual {r_host:.2e}, error vs direct {err:.2e}")
    assert err < 1e-5


def test_refined_and_fp64_agree_and_fp32_alone_falls_short(ctx):
    from acousticsim_gb300 import params
    c = _assembled(ctx)
    c.solve_refined(params(max_iters=20000, rel_tol=1e-4, warm_start=0), REL_TOL, 30)
    a = c.get_dx()
    c.solve_fp64(params(max_iters=50000, rel_tol=REL_TOL))
    b = c.get_dx()
    assert _rel(a, b) < 1e-5
    # the FP32 PCG start was replaced: a plain solve needs a new assembly
    from acousticsim_gb300 import ClothError
    with pytest.raises(ClothError):
        c.solve(params())
    # FP32 PCG alone on the same system, run to its own recurrence tolerance:
    # the FP64 residual says how far its answer really is
    c32 = _assembled(ctx)
    st = c32.solve(params(max_iters=50000, rel_tol=REL_TOL))
    r32 = c32.residual_fp64()
    print(f"fp32 alone: {st}, FP64 true residual {r32:.2e}")
    assert r32 > REL_TOL


def test_advance_uses_the_fp64_result(ctx):
    from acousticsim_gb300 import params
    c = _assembled(ctx)
    x0 = c.GetPos()
    c.solve_refined(params(max_iters=20000, rel_tol=1e-4, warm_start=0), REL_TOL, 30)
    dx = c.get_dx()
    c.advance()
    assert np.array_equal(c.GetPos(), x0 + dx)
    assert np.array_equal(c.GetPrePos(), x0)


@pytest.mark.parametrize("k_stretch", [1e5, 1e7])
def test_flexible_cg_matches_direct_solve(ctx, k_stretch):
    """FP64 flexible CG with FP32 PCG inner solves reaches an FP64 residual
    of 1e-10 in fewer FP64 iterations than the FP64 PCG needs for 1e-8, on
    the answer of the direct solve.  (Its error at a given residual is larger
    than the PCG's: the truncated recurrence does not minimise the A-norm
    error, so the tolerance here is two orders tighter.)"""
    from acousticsim_gb300 import BaraffClothGpu, params
    c = BaraffClothGpu(ctx, _conf(48, k_stretch=k_stretch))
    rng = np.random.default_rng(17)
    x0 = c.GetInitPos().reshape(-1, 3)
    c.SetPos((x0 + rng.normal(0, 1e-3, x0.shape)).reshape(-1))
    c.SetPrePos(c.GetPos() - 1e-2 * rng.normal(0, 1e-2, x0.size))
    c.assemble(1e-2)
    M, b, x_direct = _direct(c.export_system())
    tol = 1e-2 * REL_TOL
    st = c.solve_flexible(params(max_iters=30, rel_tol=0.0, warm_start=0), tol, 2000)
    assert st["status"] == "OK" and st["solver"] == "fp64", st
    assert st["rel_residual"] <= tol and st["rejected"] == 0, st
    assert st["inner_iters"] <= 30 * st["outer"]
    dx = c.get_dx()
    r_host = np.linalg.norm(b - M @ dx) / np.linalg.norm(b)
    assert r_host <= 2 * tol
    err = _rel(dx, x_direct)
    st64 = c.solve_fp64(params(max_iters=100000, rel_tol=REL_TOL))
    print(f"flexible: {st}, true residual {r_host:.2e}, error vs direct {err:.2e}; "
          f"fp64 pcg iterations {st64['iters']}")
    assert err < 1e-5
    assert _rel(c.get_dx(), dx) < 1e-4
    assert st["outer"] < st64["iters"]


def test_flexible_cg_refuses_bad_parameters(ctx):
    from acousticsim_gb300 import ClothError, params
    c = _assembled(ctx, n=8)
    with pytest.raises(ClothError):
        c.solve_flexible(params(max_iters=0), REL_TOL, 10)
    with pytest.raises(ClothError):
        c.solve_flexible(params(max_iters=10), 0.0, 10)
