"""Pins the CPU oracle (oracle/cloth_oracle.c) to the reference itself: every
golden fixture was written by the reference's own CPU code (oracle/ref_harness.cpp,
tests/golden/make_golden.py).  Index maps and init-time tables must be bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_mesh, load_golden, project_pins, rel


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


def _mesh(orc, conf):
    if conf.get("enable_cloth_from_obj"):
        # the library's OBJ loader (host code), pinned by the first test below
        return golden_mesh(conf)
    return orc.grid(conf["cloth_size"], conf["subdivision"], conf["cloth_init_pos"],
                    conf["cloth_uv_rotation"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_grid_numbering_bit_exact(orc, case):
    g, conf = load_golden(case)
    m = _mesh(orc, conf)
    assert np.array_equal(m["pos"], g["topo_pos"])
    assert np.array_equal(m["uv"], g["topo_uv"])
    assert np.array_equal(m["tris"], g["topo_tris"])
    assert np.array_equal(m["edges"], g["topo_edges"][:, :4])
    # boundary flag of the reference = no second triangle
    assert np.array_equal(m["edges"][:, 3] < 0, g["topo_edges"][:, 4] == 1)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_tables_bit_exact(orc, case):
    g, conf = load_golden(case)
    m = _mesh(orc, conf)
    t = orc.tables(m, conf["cloth_density"], conf["cloth_bending_stiffness"])
    assert np.array_equal(t["stencil"], g["topo_stencil"])
    assert np.array_equal(t["area"], g["topo_tri_area"])
    assert np.array_equal(t["mass"], g["topo_mass_gpu"])
    assert np.array_equal(t["ell"], g["topo_ell"])
    assert np.array_equal(t["coef"], g["topo_stretch_coef"])
    assert np.array_equal(t["diag16"], g["topo_bend_diag16"])
    assert np.array_equal(t["edge_k"], g["topo_bend_edge_k"])
    assert rel(t["kbend"], g["sys_Kb_gpu"]) < 1e-12


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_triangle_forces_and_hessians(orc, case):
    g, conf = load_golden(case)
    m = _mesh(orc, conf)
    t = orc.tables(m, conf["cloth_density"], conf["cloth_bending_stiffness"])
    oc = orc.OracleCloth(m, conf, g["topo_pins"])
    oc.x = g["x_in"].reshape(-1).copy()
    oc.xpre = g["xpre_in"].reshape(-1).copy()
    A, b, f, tf, th = oc.system()
    assert rel(tf, g["sys_tri_fint"]) < 1e-12
    assert rel(th, g["sys_tri_hess"]) < 1e-12
    assert rel(f, g["sys_f_stretch"] + g["sys_f_bend"]) < 1e-12
    GA, Gb = project_pins(g["sys_A"], g["sys_b"], g["topo_ell"], g["topo_pins"])
    # the reference stores the Rayleigh coefficients as float, the harness
    # used the JSON doubles: agreement to float precision of those constants
    assert rel(A, GA) < 1e-7
    assert rel(b, Gb) < 1e-12


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_pcg_matches_direct_solve(orc, case):
    g, conf = load_golden(case)
    m = _mesh(orc, conf)
    oc = orc.OracleCloth(m, conf, g["topo_pins"])
    oc.x = g["x_in"].reshape(-1).copy()
    oc.xpre = g["xpre_in"].reshape(-1).copy()
    A, b, _, _, _ = oc.system()
    dx, it, res = orc.pcg(oc.tab["ell"], A, b, oc.fixed, rel_tol=1e-13)
    assert res <= 1e-13 * np.linalg.norm(b) * 1.0001
    assert rel(dx, g["sys_dx"].reshape(-1)) < 1e-6


def test_isotropic_bending_equals_cpu_qbending():
    """With K_u = K_v the GPU bending (per-edge table * blended stiffness) must
    equal the reference's CPU Q-bending matrix (BaraffClothGpu.cpp:184-207)."""
    for case in ("grid20", "small_rot90"):
        g, _ = load_golden(case)
        assert rel(g["sys_Kb_gpu"], g["sys_Kb_cpu"]) < 1e-6


def test_oracle_rejects_wide_rows(orc):
    # a fan of 40 triangles around vertex 0: its ELL row has 41 entries
    n = 40
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    pos = np.zeros((n + 1, 3))
    pos[1:, 0] = np.cos(ang)
    pos[1:, 1] = np.sin(ang)
    uv = pos[:, :2].astype(np.float32)
    tris = np.array([[0, 1 + k, 1 + (k + 1) % n] for k in range(n)], np.int32)
    edges = []
    for k in range(n):
        a, b = 1 + k, 1 + (k + 1) % n
        edges.append([0, a, (k - 1) % n, k])
        edges.append([min(a, b), max(a, b), k, -1])
    mesh = {"pos": pos, "uv": uv, "tris": tris, "edges": np.array(edges, np.int32)}
    with pytest.raises(ValueError):
        orc.tables(mesh, 0.1, [1e-3, 1e-3])


# ---------------------------------------------------------------- dihedral bending
# The CPU cloth's bending model (cDihedralMaterial): the golden arrays are the
# reference's own force and stiffness on the fixture states, and the GPU-path
# system and direct solve with that model in place of the quadratic one.

def _dihedral_conf(conf):
    return dict(conf, cloth_bending_model="dihedral")


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_dihedral_force_and_stiffness(orc, case):
    g, conf = load_golden(case)
    m = _mesh(orc, conf)
    t = orc.tables(m, conf["cloth_density"], conf["cloth_bending_stiffness"])
    fac = orc.dihedral_rest(m, conf["cloth_bending_stiffness"][0])
    assert np.all(fac[m["edges"][:, 3] < 0] == 0.0)
    assert np.all(fac[m["edges"][:, 3] >= 0] < 0.0)
    oc = orc.OracleCloth(m, conf, g["topo_pins"])
    oc.x = g["x_in"].reshape(-1).copy()
    oc.snap_pins()
    dh = orc.dihedral(t, fac, oc.x)
    # the closed-form gradient equals the reference's expression away from
    # beta = 0 (the fixtures' angles are 1e-3..1 rad)
    assert rel(dh["f"], g["sys_dih_f"]) < 1e-9
    # the stiffness is float-rounded per edge in both
    assert rel(dh["K"], g["sys_dih_K"]) < 2e-7


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_dihedral_system_and_solve(orc, case):
    g, conf = load_golden(case)
    m = _mesh(orc, conf)
    oc = orc.OracleCloth(m, _dihedral_conf(conf), g["topo_pins"])
    oc.x = g["x_in"].reshape(-1).copy()
    oc.xpre = g["xpre_in"].reshape(-1).copy()
    A, b, _, _, _ = oc.system()
    GA, Gb = project_pins(g["sys_dih_A"], g["sys_dih_b"], g["topo_ell"], g["topo_pins"])
    assert rel(A, GA) < 1e-7
    assert rel(b, Gb) < 1e-9
    dx, it, res = orc.pcg(oc.tab["ell"], A, b, oc.fixed, rel_tol=1e-13)
    assert rel(dx, g["sys_dih_dx"].reshape(-1)) < 1e-6


def test_dihedral_gradient_is_the_derivative_of_beta(orc):
    """dbeta/dx of the oracle against central differences of beta, over
    random stencils, flat and folded ones included."""
    rng = np.random.default_rng(7)
    for trial in range(20):
        P = rng.normal(size=(4, 3))
        if trial < 5:
            P[:, 2] = 0.0  # flat: beta = 0 or pi
        mesh = {"pos": P, "tris": np.array([[0, 1, 2], [1, 0, 3]], np.int32),
                "edges": np.array([[0, 1, 0, 1]], np.int32)}
        tab = {"ell": np.full((4, 32), -1, np.int32), "stencil": np.array([[0, 1, 2, 3]],
                                                                          np.int32)}
        tab["ell"][:, :4] = np.arange(4)
        fac = np.array([-1.0])

        def beta(x):
            return orc.dihedral(tab, fac, x)["beta"][0]

        d = orc.dihedral(tab, fac, P)
        h = 1e-6
        num = np.zeros(12)
        x0 = P.reshape(-1)
        for k in range(12):
            xp, xm = x0.copy(), x0.copy()
            xp[k] += h
            xm[k] -= h
            db = beta(xp) - beta(xm)
            db = (db + np.pi) % (2 * np.pi) - np.pi  # across the +-pi cut
            num[k] = db / (2 * h)
        assert np.allclose(d["grad"].reshape(-1), num, rtol=1e-5, atol=1e-6 * np.abs(num).max())


# ---------------------------------------------------------------- collisions
# The CPU cloth's contacts with a kinematic body, its contact Hessian and its
# Repulsion, as the reference's cBVHCollisionDetecter and cBaraffCloth write
# them on the grid20 state (oracle/ref_harness.cpp "collide").

COLLIDE_CASES = ["col_patch", "col_plane"]


def load_collide(case):
    import json
    from conftest import GOLDEN
    c = np.load(GOLDEN / f"{case}.npz")
    return c, json.loads(bytes(c["config_json"]).decode())


@pytest.mark.parametrize("case", COLLIDE_CASES)
def test_contacts_match_reference(orc, case):
    c, conf = load_collide(case)
    m = _mesh(orc, conf)
    tn, vn = orc.body_normals(c["col_kb_pos"], c["col_kb_tris"])
    assert np.abs(tn - c["col_kb_tnormal"]).max() < 1e-15
    assert np.abs(vn - c["col_kb_vnormal"]).max() < 1e-15
    body = {"pos": c["col_kb_pos"], "tris": c["col_kb_tris"], "edges": c["col_kb_edges"],
            "tnormal": tn, "vnormal": vn}
    con = orc.contacts(m, c["col_x"], body)
    # the same contacts in the same order; normals, depths and barycentric
    # coordinates to the last bits
    assert np.array_equal(con["pt_i"], c["col_pt_i"])
    assert np.array_equal(con["ee_i"], c["col_ee_i"])
    assert np.abs(con["pt_d"] - c["col_pt_d"]).max() < 1e-15
    assert np.abs(con["ee_d"] - c["col_ee_d"]).max() < 1e-15
    assert len(con["pt_i"]) > 50 and len(con["ee_i"]) > 50
    tab = orc.tables(m, conf["cloth_density"], conf["cloth_bending_stiffness"])
    H = orc.contact_hessian(tab, m, con)
    assert rel(H, c["col_col_H"]) < 1e-15
    dxo = orc.repulsion(m, c["col_mass_cpu"], conf["cloth_stretch_stiffness"],
                        conf["default_timestep"], con, c["col_dx_in"])
    d_ref = (c["col_dx_out"] - c["col_dx_in"]).reshape(-1)
    assert np.abs(d_ref).max() > 0
    assert rel(dxo - c["col_dx_in"].reshape(-1), d_ref) < 1e-13
