"""Failure detection of the persistent PCG drivers, without a GPU fault.

The persistent solvers' team barriers are the only device-side waits of the
step.  Each wait is bounded: after the context's spin limit the team sets its
error flag, the kernel returns, and the solve reports CLOTH_ERR_TIMEOUT.  The
test makes the waits run out on purpose with a short limit and the
extra-arrivals hook (every barrier waits for an arrival that no block makes),
checks the status, and then checks that the same context steps normally once
the limit is back to its default."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _conf(n):
    return {"geometry_type": "regular_triangle", "cloth_size": [1.0, 1.0],
            "subdivision": [n - 1, n - 1], "cloth_init_pos": [0.0, 0.0, 0.0],
            "cloth_uv_rotation": 0, "cloth_stretch_stiffness": [1e3, 1e3, 1e2],
            "cloth_bending_stiffness": [1e-3, 1e-3], "cloth_density": 0.1,
            "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0, "default_timestep": 2e-3,
            "constraints": {"static_point": [[-0.5, 0.5], [0.5, 0.5]]}}


# (solver asked for, the name its stats report)
@pytest.mark.parametrize("psolver,ran", [("persistent_2b", "persistent"),
                                         ("persistent_1b", "persistent_1b")])
def test_team_barrier_wait_runs_out_and_context_recovers(built, psolver, ran):
    from acousticsim_gb300 import BaraffClothGpu, ClothContext, params
    p = params(max_iters=5000, rel_tol=1e-6)
    ctx = ClothContext(0)
    ctx.set_solver(psolver)
    cloth = BaraffClothGpu(ctx, _conf(96))  # 9,216 rows: a team of many blocks
    rng = np.random.default_rng(3)
    x0 = cloth.GetInitPos().reshape(-1, 3)
    x = (x0 + rng.normal(0, 1e-3, x0.shape)).reshape(-1)
    xp = x - 2e-3 * rng.normal(0, 1e-2, x.shape)

    # a normal step first: the reference result of this state
    cloth.SetPos(x)
    cloth.SetPrePos(xp)
    st_ok = cloth.UpdatePos(0.0, p)
    assert st_ok["status"] == "OK" and st_ok["solver"] == ran, st_ok
    x_ok = cloth.GetPos()

    # every team barrier waits for one arrival too many, 1,000 polls at most
    ctx.set_spin_limit(1000, 1)
    cloth.Reset()
    cloth.SetPos(x)
    cloth.SetPrePos(xp)
    st = cloth.UpdatePos(0.0, p)
    assert st["status"] == "TIMEOUT", st
    assert st["solver"] == ran
    assert st["iters"] <= 1, st  # gave up at the first barrier

    # default limit again: the same context steps the same state normally
    ctx.set_spin_limit(0, 0)
    cloth.Reset()
    cloth.SetPos(x)
    cloth.SetPrePos(xp)
    st2 = cloth.UpdatePos(0.0, p)
    assert st2["status"] == "OK" and st2["iters"] == st_ok["iters"], (st2, st_ok)
    assert np.array_equal(cloth.GetPos(), x_ok)
    cloth.close()
    ctx.close()
