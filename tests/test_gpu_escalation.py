"""Precision escalation of the step (the CPU cloth's dihedral bending).

With the dihedral model on a 512x512 cloth and the benchmark's perturbation
(x += N(0, 1e-3), half the grid spacing), the dihedral stiffness dwarfs the
vertex masses and the first step's system is beyond FP32: the FP32 PCG ends
in NaN or breakdown.  (No smaller case was found that does: grids up to
192 x 192 with densities down to 1e-5 and bending stiffness up to 1 all
converge in FP32.)  The step driver then keeps the pre-step state, re-solves
the assembled system with the all-FP64 PCG and advances in FP64.

Checked: with escalation off the failed step leaves the state alone; with it
on the step succeeds, reports the escalation, and its positions are bit for
bit those of an explicit assemble + FP64 PCG + advance of the same state."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_SIDE = 512
DT = 2e-3


def _conf():
    return {"geometry_type": "regular_triangle", "cloth_size": [1.0, 1.0],
            "subdivision": [N_SIDE - 1, N_SIDE - 1], "cloth_init_pos": [0.0, 0.0, 0.0],
            "cloth_uv_rotation": 0, "cloth_stretch_stiffness": [1e3, 1e3, 1e2],
            "cloth_bending_stiffness": [1e-3, 1e-3], "cloth_density": 0.1,
            "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0, "default_timestep": DT,
            "cloth_bending_model": "dihedral",
            "constraints": {"static_point": [[-0.5, 0.5], [0.5, 0.5]]}}


def _seeded(pos):
    rng = np.random.default_rng(1234)
    p = pos.reshape(-1, 3)
    x = p + rng.normal(0.0, 1e-3, p.shape)
    v = rng.normal(0.0, 1e-2, p.shape)
    return x.reshape(-1).copy(), (x - DT * v).reshape(-1).copy()


def test_failed_fp32_step_is_resolved_in_fp64(built):
    from acousticsim_gb300 import BaraffClothGpu, ClothContext, params
    p = params(max_iters=20000, rel_tol=1e-6)
    ctx = ClothContext(0)
    c = BaraffClothGpu(ctx, _conf())
    x0, xp0 = _seeded(c.GetInitPos())
    pins = c.GetConstraintStaticVertices()
    free = np.ones(c.nv, bool)
    free[pins] = False

    def reset():
        c.Reset()
        c.SetPos(x0)
        c.SetPrePos(xp0)

    # escalation off: the FP32 solve fails and the state stays as it was
    ctx.set_escalation(False)
    reset()
    st = c.UpdatePos(0.0, p)
    print("FP32 only:", st)
    assert st["status"] in ("NAN", "BREAKDOWN"), st
    assert np.array_equal(c.GetPos().reshape(-1, 3)[free], x0.reshape(-1, 3)[free])

    # escalation on (the default): re-solved in FP64 and advanced
    ctx.set_escalation(True)
    reset()
    st = c.UpdatePos(0.0, p)
    print("escalated:", st)
    assert st["status"] == "OK" and st["solver"] == "escalated_fp64", st
    assert st["rel_residual"] <= 1e-6
    assert c.stats()["solver"] == "escalated_fp64"
    x_esc = c.GetPos()

    # the same state by hand: assemble, FP64 PCG from zero, advance
    reset()
    c.assemble()
    st64 = c.solve_fp64(params(max_iters=100000, rel_tol=1e-6, warm_start=0))
    assert st64["status"] == "OK", st64
    assert st64["iters"] == st["iters"]
    c.advance()
    assert np.array_equal(c.GetPos(), x_esc)

    # the next step warm-starts from the FP64 solution and goes on
    reset()
    c.UpdatePos(0.0, p)
    st2 = c.UpdatePos(0.0, p)
    assert st2["status"] == "OK", st2
    c.close()
    ctx.close()


def test_maxiter_step_is_escalated_at_level_2(built):
    """Escalation level 2 also re-solves a step whose FP32 PCG ends at
    max_iters (a capped solve here: 3 iterations on a 32 x 32 cloth); at
    level 1 that step is advanced with the dx it reached, as the reference
    does, and so is a step made without stats at level 2."""
    from acousticsim_gb300 import BaraffClothGpu, ClothContext, ClothError, params
    conf = _conf()
    conf["subdivision"] = [31, 31]
    conf["cloth_bending_model"] = "quadratic"
    p = params(max_iters=3, rel_tol=1e-6)
    ctx = ClothContext(0)
    c = BaraffClothGpu(ctx, conf)
    x0, xp0 = _seeded(c.GetInitPos())

    def reset():
        c.Reset()
        c.SetPos(x0)
        c.SetPrePos(xp0)

    # level 1 (the default): the capped solve is advanced
    reset()
    st = c.UpdatePos(0.0, p)
    assert st["status"] == "MAXITER" and st["solver"] != "escalated_fp64", st
    x_capped = c.GetPos()
    assert not np.array_equal(x_capped, x0)

    # level 2: re-solved in FP64 from the pre-step state and advanced
    ctx.set_escalation(2)
    reset()
    st = c.UpdatePos(0.0, p)
    assert st["status"] == "OK" and st["solver"] == "escalated_fp64", st
    assert st["rel_residual"] <= 1e-6
    x_esc = c.GetPos()
    reset()
    c.assemble()
    st64 = c.solve_fp64(params(max_iters=100000, rel_tol=1e-6, warm_start=0))
    assert st64["status"] == "OK" and st64["iters"] == st["iters"], st64
    c.advance()
    assert np.array_equal(c.GetPos(), x_esc)

    # level 2, no stats: not escalated, the capped dx is applied
    reset()
    c.step_async(0.0, p)
    assert np.array_equal(c.GetPos(), x_capped)

    with pytest.raises(ClothError):
        ctx.set_escalation(3)
    ctx.set_escalation(True)
    c.close()
    ctx.close()
