"""Host-side logic of the product (no GPU): the grid builder and the init-time
tables cloth_create uploads, checked bit for bit against the reference's own
arrays (golden fixtures), plus mesh validation errors."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, rel


@pytest.fixture(scope="module")
def N(built):
    from acousticsim_gb300 import _native
    _native.load()
    return _native


def _grid(conf):
    from conftest import golden_mesh
    return golden_mesh(conf)


def _material(N, conf):
    return N.Material((C.c_float * 3)(*conf["cloth_stretch_stiffness"][:3]),
                      (C.c_float * 2)(*conf["cloth_bending_stiffness"][:2]),
                      conf["cloth_density"], conf["rayleigh_damping_a"],
                      conf["rayleigh_damping_b"], conf["default_timestep"], -9.8, 0)


def host_tables(N, mesh, mat, with_edges=True):
    pos = np.ascontiguousarray(mesh["pos"], np.float64)
    uv = np.ascontiguousarray(mesh["uv"], np.float32)
    tris = np.ascontiguousarray(mesh["tris"], np.int32)
    edges = np.ascontiguousarray(mesh["edges"], np.int32) if with_edges else None
    md = N.MeshDesc(pos.shape[0], tris.shape[0], 0 if edges is None else edges.shape[0],
                    N.ptr(pos, C.c_double), N.ptr(uv, C.c_float), N.ptr(tris, C.c_int),
                    None if edges is None else N.ptr(edges, C.c_int))
    ne, width = C.c_int(), C.c_int()
    N.call("cloth_host_tables", C.byref(md), C.byref(mat), C.byref(ne), C.byref(width),
           None, None, None, None, None, None, None)
    nv, nt = pos.shape[0], tris.shape[0]
    out = {"ell": np.zeros((nv, 32), np.int32), "stencil": np.zeros((ne.value, 4), np.int32),
           "coef": np.zeros((nt, 12), np.float32), "area": np.zeros(nt, np.float32),
           "mass": np.zeros(nv), "kbend": np.zeros((nv, 32), np.float32),
           "tri_slot": np.zeros((nt, 9), np.int32)}
    N.call("cloth_host_tables", C.byref(md), C.byref(mat), None, None,
           N.ptr(out["ell"], C.c_int), N.ptr(out["stencil"], C.c_int),
           N.ptr(out["coef"], C.c_float), N.ptr(out["area"], C.c_float),
           N.ptr(out["mass"], C.c_double), N.ptr(out["kbend"], C.c_float),
           N.ptr(out["tri_slot"], C.c_int))
    out["width"] = width.value
    return out


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_grid_bit_exact(N, case):
    g, conf = load_golden(case)
    m = _grid(conf)
    assert np.array_equal(m["pos"], g["topo_pos"])
    assert np.array_equal(m["uv"], g["topo_uv"])
    assert np.array_equal(m["tris"], g["topo_tris"])
    assert np.array_equal(m["edges"], g["topo_edges"][:, :4])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_tables_bit_exact(N, case):
    g, conf = load_golden(case)
    t = host_tables(N, _grid(conf), _material(N, conf))
    assert np.array_equal(t["ell"], g["topo_ell"])
    assert np.array_equal(t["stencil"], g["topo_stencil"])
    assert np.array_equal(t["coef"], g["topo_stretch_coef"])
    assert np.array_equal(t["area"], g["topo_tri_area"])
    assert np.array_equal(t["mass"], g["topo_mass_gpu"])
    assert t["width"] == (g["topo_ell"] >= 0).sum(1).max()
    # bending scalars: float rounding of a double sum of the reference's table
    assert rel(t["kbend"], g["sys_Kb_gpu"]) < 1e-7


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_triangle_slot_map(N, case):
    """Slot of v_b in the ELL row of v_a, as global_to_local_same finds it
    (BaraffClothGpu.cu:111-126, 179-193), for every triangle pair."""
    g, conf = load_golden(case)
    t = host_tables(N, _grid(conf), _material(N, conf))
    ell, tris = g["topo_ell"], g["topo_tris"]
    for a in range(3):
        for b in range(3):
            s = t["tri_slot"][:, 3 * a + b]
            assert np.array_equal(ell[tris[:, a], s], tris[:, b])


def test_derived_edges_give_same_pattern(N):
    g, conf = load_golden("grid20")
    m = _grid(conf)
    mat = _material(N, conf)
    a = host_tables(N, m, mat, with_edges=True)
    b = host_tables(N, m, mat, with_edges=False)
    assert np.array_equal(a["ell"], b["ell"])
    assert rel(b["kbend"], a["kbend"]) < 1e-6


def test_grid_counts_512(N):
    from acousticsim_gb300 import build_grid
    m = build_grid((1.0, 1.0), (511, 511))
    assert m["pos"].shape[0] == 262144
    assert m["tris"].shape[0] == 522242
    assert m["edges"].shape[0] == 784385


def test_rejects_bad_meshes(N):
    from acousticsim_gb300._native import ClothError
    g, conf = load_golden("small_rot90")
    mat = _material(N, conf)
    m = _grid(conf)
    bad = dict(m)
    bad["tris"] = m["tris"].copy()
    bad["tris"][0, 1] = bad["tris"][0, 0]          # degenerate triangle
    with pytest.raises(ClothError):
        host_tables(N, bad, mat, with_edges=False)
    bad = dict(m)
    bad["tris"] = np.concatenate([m["tris"], m["tris"][:1]])  # edge used by 3 triangles
    with pytest.raises(ClothError):
        host_tables(N, bad, mat, with_edges=False)
    bad = dict(m)
    bad["tris"] = m["tris"].copy()
    bad["tris"][0, 0] = m["pos"].shape[0]         # vertex id out of range
    with pytest.raises(ClothError):
        host_tables(N, bad, mat, with_edges=False)
    # fan of 40 triangles: ELL row of 41 blocks, beyond the 32 the reference holds
    n = 40
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    pos = np.zeros((n + 1, 3))
    pos[1:, 0], pos[1:, 1] = np.cos(ang), np.sin(ang)
    fan = {"pos": pos, "uv": pos[:, :2].astype(np.float32),
           "tris": np.array([[0, 1 + k, 1 + (k + 1) % n] for k in range(n)], np.int32)}
    with pytest.raises(ClothError):
        host_tables(N, fan, mat, with_edges=False)


def test_dihedral_model_tables(N):
    """The dihedral model (the CPU cloth's bending) replaces the quadratic one:
    no quadratic bending scalars, the same ELL pattern; unknown models are refused."""
    import ctypes as C
    g, conf = load_golden("grid20")
    mesh = _grid(conf)
    mat = _material(N, conf)
    q = host_tables(N, mesh, mat)
    mat.bending_model = 1
    d = host_tables(N, mesh, mat)
    assert np.array_equal(d["ell"], q["ell"])
    assert np.any(q["kbend"] != 0) and np.all(d["kbend"] == 0)
    mat.bending_model = 7
    pos = np.ascontiguousarray(mesh["pos"], np.float64)
    uv = np.ascontiguousarray(mesh["uv"], np.float32)
    tris = np.ascontiguousarray(mesh["tris"], np.int32)
    md = N.MeshDesc(pos.shape[0], tris.shape[0], 0, N.ptr(pos, C.c_double),
                    N.ptr(uv, C.c_float), N.ptr(tris, C.c_int), None)
    rc = N.load().cloth_host_tables(C.byref(md), C.byref(mat), None, None, None, None, None,
                                    None, None, None, None)
    assert rc != 0
