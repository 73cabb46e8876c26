"""GPU parity of the CPU cloth's collision handling against kinematic bodies
(cBVHCollisionDetecter, cBaraffCloth::PrepareCollisionHessian and Repulsion):
the contacts the device finds against the reference's own lists, the contact
Hessian against the reference's matrix, the ordered repulsion against the
FP64 oracle, and short trajectories against the oracle stepping with the
same contacts."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, rel

pytestmark = pytest.mark.gpu

CASES = ["col_patch", "col_plane"]


def _load(case):
    c = np.load(GOLDEN / f"{case}.npz")
    return c, json.loads(bytes(c["config_json"]).decode())


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


def _cloth(ctx, conf, pins=False):
    from acousticsim_gb300 import BaraffClothGpu
    conf = dict(conf)
    if not pins:
        conf.pop("constraints", None)  # the harness dumps contacts of unsnapped positions
    return BaraffClothGpu(ctx, conf)


def _body(ctx, c):
    from acousticsim_gb300 import ClothBody
    return ClothBody(ctx, c["col_kb_pos"], c["col_kb_tris"])


@pytest.mark.parametrize("case", CASES)
def test_contacts_match_reference(ctx, case):
    c, conf = _load(case)
    cl = _cloth(ctx, conf)
    body = _body(ctx, c)
    cl.SetPos(c["col_x"])
    cl.SetPrePos(c["col_x"])
    cl.set_bodies([body])
    cl.assemble()
    con = cl.get_contacts()
    assert con["overflow"] == 0
    assert np.array_equal(con["pt_i"], c["col_pt_i"])
    assert np.array_equal(con["ee_i"], c["col_ee_i"])
    assert np.abs(con["pt_d"] - c["col_pt_d"]).max() < 1e-15
    assert np.abs(con["ee_d"] - c["col_ee_d"]).max() < 1e-15
    cl.set_bodies([])
    cl.close()
    body.close()


@pytest.mark.parametrize("case", CASES)
def test_contact_hessian_matches_reference(ctx, case):
    c, conf = _load(case)
    cl = _cloth(ctx, conf)
    body = _body(ctx, c)
    cl.SetPos(c["col_x"])
    cl.SetPrePos(c["col_x"])
    cl.set_bodies([body])
    cl.assemble()
    a_with = cl.export_system()["A"].astype(np.float64)
    cl.set_bodies([])
    cl.assemble()
    a_without = cl.export_system()["A"].astype(np.float64)
    H = a_with - a_without
    err = rel(H, c["col_col_H"])
    print(case, "contact Hessian error", err)
    assert err < 1e-5
    cl.close()
    body.close()


@pytest.mark.parametrize("case", CASES)
def test_repulsion_matches_oracle(ctx, orc, case):
    """One step: the device's repulsed dx against the oracle's Repulsion of the
    same PCG dx with the same contacts (FP64 on both sides)."""
    from acousticsim_gb300 import params
    c, conf = _load(case)
    cl = _cloth(ctx, conf)
    body = _body(ctx, c)
    cl.SetPos(c["col_x"])
    cl.SetPrePos(c["col_x"] - conf["default_timestep"] * 0.05)
    cl.set_bodies([body])
    st = cl.UpdatePos(0.0, params(max_iters=20000, rel_tol=1e-6))
    assert st["status"] == "OK", st
    con = cl.get_contacts()
    assert len(con["pt_i"]) + len(con["ee_i"]) > 0
    dx = cl.get_dx()
    dxr = cl.get_repulsed_dx()
    tab = orc.tables(cl.mesh, conf["cloth_density"], conf["cloth_bending_stiffness"])
    ref = orc.repulsion(cl.mesh, tab["mass"], conf["cloth_stretch_stiffness"],
                        conf["default_timestep"], con, dx)
    assert np.abs(ref - dx).max() > 0
    err = rel(dxr - dx, ref - dx)
    print(case, "repulsion rounds", con["repulsion_rounds"], "error", err)
    assert err < 1e-12
    # the step applied it
    assert np.allclose(cl.GetPos() - cl.GetPrePos(), dxr, rtol=0, atol=1e-15)
    cl.set_bodies([])
    cl.close()
    body.close()


def test_collision_trajectory_vs_oracle(ctx, orc):
    """Ten steps of the pinned 20x20 cloth against the curved patch: device
    and FP64 oracle step with contacts, Hessian and repulsion."""
    from acousticsim_gb300 import params
    c, conf = _load("col_patch")
    g = np.load(GOLDEN / "grid20.npz")
    cl = _cloth(ctx, conf, pins=True)
    body = _body(ctx, c)
    x, xp = g["x_in"].reshape(-1), g["xpre_in"].reshape(-1)
    cl.SetPos(x)
    cl.SetPrePos(xp)
    cl.set_bodies([body])
    tn, vn = orc.body_normals(c["col_kb_pos"], c["col_kb_tris"])
    bd = {"pos": c["col_kb_pos"], "tris": c["col_kb_tris"], "edges": c["col_kb_edges"],
          "tnormal": tn, "vnormal": vn}
    oc = orc.OracleCloth(cl.mesh, conf, cl.GetConstraintStaticVertices(), bodies=[bd])
    oc.x, oc.xpre = x.copy(), xp.copy()
    counts = []
    for _ in range(10):
        st = cl.UpdatePos(0.0, params(max_iters=20000, rel_tol=1e-8))
        assert st["status"] == "OK", st
        con = cl.get_contacts()
        oc.step(rel_tol=1e-12)
        oc_n = (len(oc.last_contacts["pt_i"]), len(oc.last_contacts["ee_i"]))
        counts.append(((len(con["pt_i"]), len(con["ee_i"])), oc_n))
    print("contacts per step (device, oracle):", counts)
    assert all(a == b for a, b in counts[:3])
    disp = rel(cl.GetPos() - x, oc.x - x)
    print("displacement error after 10 steps", disp)
    assert disp < 1e-4  # measured 6.5e-6
    cl.set_bodies([])
    cl.close()
    body.close()


def test_collision_refusals(ctx):
    from acousticsim_gb300 import BaraffClothGpu, ClothBody, ClothError, ClothServer, params
    c, conf = _load("col_plane")
    a = _cloth(ctx, conf)
    b = _cloth(ctx, conf)
    body = _body(ctx, c)
    a.set_bodies([body])
    # a cloth with bodies is stepped alone
    with pytest.raises(ClothError):
        ctx.batch_step([a, b], 0.0, params(max_iters=100, rel_tol=1e-6))
    srv = ClothServer(ctx, 1 << 30)
    with pytest.raises(ClothError):
        srv.add(a)
    srv.close()
    # a body in use cannot go
    with pytest.raises(ClothError):
        from acousticsim_gb300 import _native as N
        N.call("cloth_body_destroy", body.handle)
    a.set_bodies([])
    body.close()
    # tiny capacities: the step reports the lost contacts
    a.set_bodies([_body(ctx, c)])
    a.set_contact_capacity(0, 8, 8)
    a.SetPos(c["col_x"])
    a.SetPrePos(c["col_x"])
    st = a.UpdatePos(0.0, params(max_iters=2000, rel_tol=1e-6))
    assert st["status"] == "CONTACTS"
    assert a.get_contacts()["overflow"] == 1
    a.set_bodies([])
    a.close()
    b.close()


def test_moving_body_trajectory_vs_oracle(ctx, orc):
    """The curved patch as a moving body (the reference's time-driven motion:
    translation and XYZ Euler angles interpolated over 40 ms), pressed 3 mm
    towards the pinned 20x20 cloth and turned a little while the cloth steps:
    before each step the body advances by dt (cloth_body_update), and the FP64
    oracle steps against the same body positions (the host pose, pinned to the
    reference's cKinematicBody by tests/test_body_motion.py) with the normals
    of the initial pose, as the reference's moving body keeps them."""
    from acousticsim_gb300 import ClothBody, kinematic_pose, params
    m = np.load(GOLDEN / "body_motion.npz")
    local, tris = m["mo_local"], m["mo_tris"]
    ip, io = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]
    tp, to = [0.004, -0.003, -0.003], [0.02, -0.015, 0.03]
    elapsed = 0.04
    _, conf = _load("col_patch")
    g = np.load(GOLDEN / "grid20.npz")
    dt = np.float32(conf["default_timestep"])
    cl = _cloth(ctx, conf, pins=True)
    body = ClothBody(ctx, local, tris)
    body.set_motion(local, ip, io, tp, to, elapsed)
    p0 = kinematic_pose(local, ip, io, tp, to, elapsed, 0.0)
    assert np.array_equal(body.get_pos(), p0)
    x, xp = g["x_in"].reshape(-1), g["xpre_in"].reshape(-1)
    cl.SetPos(x)
    cl.SetPrePos(xp)
    cl.set_bodies([body])
    tn, vn = orc.body_normals(p0, tris)
    bd = {"pos": p0, "tris": tris, "edges": orc.derive_edges(tris), "tnormal": tn,
          "vnormal": vn}
    oc = orc.OracleCloth(cl.mesh, conf, cl.GetConstraintStaticVertices(), bodies=[bd])
    oc.x, oc.xpre = x.copy(), xp.copy()
    t = np.float32(0.0)
    counts = []
    for _ in range(10):
        body.update(float(dt))
        t = np.float32(t + dt)
        pk = kinematic_pose(local, ip, io, tp, to, elapsed, float(t))
        assert np.array_equal(body.get_pos(), pk)
        bd["pos"] = pk
        st = cl.UpdatePos(0.0, params(max_iters=20000, rel_tol=1e-8))
        assert st["status"] == "OK", st
        con = cl.get_contacts()
        oc.step(rel_tol=1e-12)
        counts.append(((len(con["pt_i"]), len(con["ee_i"])),
                       (len(oc.last_contacts["pt_i"]), len(oc.last_contacts["ee_i"]))))
    print("moving body: contacts per step (device, oracle):", counts)
    assert all(a == b for a, b in counts[:3])
    assert sum(a[0] + a[1] for a, _ in counts) > 0
    disp = rel(cl.GetPos() - x, oc.x - x)
    print("moving body: displacement error after 10 steps", disp)
    assert disp < 1e-4
    cl.set_bodies([])
    cl.close()
    body.close()
