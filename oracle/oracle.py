"""ctypes front of oracle/libcloth_oracle.so - the CPU restatement of
AcousticSim's implicit cloth step.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The GPU product never uses it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "libcloth_oracle.so"
W = 32
_lib = None

PD = C.POINTER(C.c_double)
PF = C.POINTER(C.c_float)
PI = C.POINTER(C.c_int)
PU8 = C.POINTER(C.c_ubyte)


def build(force: bool = False) -> Path:
    """Compiles libcloth_oracle.so from oracle/cloth_oracle.c when it is missing
    or older than its sources (gcc, OpenMP, no contraction of multiply-adds)."""
    import os
    import subprocess
    src = [LIB.parent / "cloth_oracle.c", LIB.parent / "cloth_oracle.h"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= p.stat().st_mtime
                                          for p in src):
        return LIB
    tmp = LIB.with_name("libcloth_oracle.build.so")
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
                    "-fopenmp", "-o", str(tmp), str(src[0]), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise ImportError(f"{LIB} missing: run `python -m acousticsim_gb300.build`")
        L = C.CDLL(str(LIB))
        L.orc_grid.argtypes = [PD, PI, PD, C.c_float, PI, PI, PI, PD, PF, PI, PI]
        L.orc_tables.argtypes = [C.c_int, C.c_int, C.c_int, PD, PF, PI, PI, C.c_float, PF,
                                 PI, PF, PD, PI, PF, PF, PF, PD]
        L.orc_triangles.argtypes = [C.c_int, PI, PF, PF, PD, PF, C.c_int, PD, PD]
        L.orc_triangles.restype = None
        L.orc_system.argtypes = [C.c_int, C.c_int, PI, PI, PD, PD, PD, PD, C.c_double, PD, PD,
                                 PU8, C.c_double, C.c_float, C.c_float, PD, PD, PD]
        L.orc_system.restype = None
        L.orc_system_ex.argtypes = [C.c_int, C.c_int, PI, PI, PD, PD, PD, PD, PD, PD,
                                    C.c_double, PD, PD, PU8, C.c_double, C.c_float,
                                    C.c_float, PD, PD, PD]
        L.orc_system_ex.restype = None
        L.orc_dihedral_rest.argtypes = [C.c_int, C.c_int, C.c_int, PD, PI, PI, C.c_float, PD]
        L.orc_dihedral.argtypes = [C.c_int, C.c_int, PI, PD, PD, PI, PD, PD, PD, PD]
        L.orc_dihedral.restype = None
        L.orc_body_normals.argtypes = [C.c_int, C.c_int, PD, PI, PD, PD]
        L.orc_body_normals.restype = None
        L.orc_contacts.argtypes = [C.c_int, C.c_int, C.c_int, PD, PI, PI, C.c_int, C.c_int,
                                   C.c_int, PD, PI, PI, PD, PD, C.c_int, PI, PD, PI, C.c_int,
                                   PI, PD, PI]
        L.orc_contact_hessian.argtypes = [C.c_int, PI, PI, C.c_int, PI, PD, PD]
        L.orc_contact_hessian.restype = None
        L.orc_repulsion.argtypes = [C.c_int, PI, PI, PD, PF, C.c_double, C.c_int, PI, PD,
                                    C.c_int, PI, PD, PD]
        L.orc_repulsion.restype = None
        L.orc_spmv.argtypes = [C.c_int, PI, PD, PD, PD]
        L.orc_spmv.restype = None
        L.orc_pcg.argtypes = [C.c_int, PI, PD, PD, PU8, PD, C.c_int, C.c_double, PD, C.c_int]
        L.orc_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def grid(size=(1.0, 1.0), subdiv=(19, 19), init_pos=(0.0, 0.0, 0.0), uv_rot=0.0) -> dict:
    L = lib()
    s = np.asarray(size, np.float64)
    d = np.asarray(subdiv, np.int32)
    ip = np.asarray(init_pos, np.float64)
    nv, nt, ne = C.c_int(), C.c_int(), C.c_int()
    rc = L.orc_grid(_p(s, C.c_double), _p(d, C.c_int), _p(ip, C.c_double), float(uv_rot),
                    C.byref(nv), C.byref(nt), C.byref(ne), None, None, None, None)
    assert rc == 0
    pos = np.zeros((nv.value, 3))
    uv = np.zeros((nv.value, 2), np.float32)
    tris = np.zeros((nt.value, 3), np.int32)
    edges = np.zeros((ne.value, 4), np.int32)
    L.orc_grid(_p(s, C.c_double), _p(d, C.c_int), _p(ip, C.c_double), float(uv_rot),
               None, None, None, _p(pos, C.c_double), _p(uv, C.c_float), _p(tris, C.c_int),
               _p(edges, C.c_int))
    return {"pos": pos, "uv": uv, "tris": tris, "edges": edges}


def tables(mesh: dict, density: float, bending_k) -> dict:
    L = lib()
    pos = np.ascontiguousarray(mesh["pos"], np.float64)
    uv = np.ascontiguousarray(mesh["uv"], np.float32)
    tris = np.ascontiguousarray(mesh["tris"], np.int32)
    edges = np.ascontiguousarray(mesh["edges"], np.int32)
    nv, nt, ne = pos.shape[0], tris.shape[0], edges.shape[0]
    kb = np.asarray(bending_k, np.float32)
    out = {"stencil": np.zeros((ne, 4), np.int32), "area": np.zeros(nt, np.float32),
           "mass": np.zeros(nv), "ell": np.zeros((nv, W), np.int32),
           "coef": np.zeros((nt, 12), np.float32), "diag16": np.zeros((ne, 16), np.float32),
           "edge_k": np.zeros(ne, np.float32), "kbend": np.zeros((nv, W))}
    rc = L.orc_tables(nv, nt, ne, _p(pos, C.c_double), _p(uv, C.c_float), _p(tris, C.c_int),
                      _p(edges, C.c_int), float(density), _p(kb, C.c_float),
                      _p(out["stencil"], C.c_int), _p(out["area"], C.c_float),
                      _p(out["mass"], C.c_double), _p(out["ell"], C.c_int),
                      _p(out["coef"], C.c_float), _p(out["diag16"], C.c_float),
                      _p(out["edge_k"], C.c_float), _p(out["kbend"], C.c_double))
    if rc != 0:
        raise ValueError("oracle: ELL row wider than 32")
    return out


def triangles(mesh: dict, tab: dict, x: np.ndarray, stretch_k, fix_fv_norm=0):
    L = lib()
    tris = np.ascontiguousarray(mesh["tris"], np.int32)
    nt = tris.shape[0]
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    ks = np.asarray(stretch_k, np.float32)
    f = np.zeros((nt, 3, 3))
    h = np.zeros((nt, 9, 3, 3))
    L.orc_triangles(nt, _p(tris, C.c_int), _p(tab["coef"], C.c_float),
                    _p(tab["area"], C.c_float), _p(x, C.c_double), _p(ks, C.c_float),
                    int(fix_fv_norm), _p(f, C.c_double), _p(h, C.c_double))
    return f, h


def system(mesh: dict, tab: dict, tri_f, tri_h, x, xpre, fixed, dt, ray_a, ray_b,
           gravity=-9.8, bend=None):
    """Assembled system.  bend=None: the GPU cloth's quadratic bending
    (tab["kbend"]); bend=(K, f) from dihedral(): that model instead."""
    L = lib()
    tris = np.ascontiguousarray(mesh["tris"], np.int32)
    nv, nt = tab["ell"].shape[0], tris.shape[0]
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    xpre = np.ascontiguousarray(xpre, np.float64).reshape(-1)
    fixed = np.ascontiguousarray(fixed, np.uint8)
    A = np.zeros((nv, W, 3, 3))
    b = np.zeros((nv, 3))
    f = np.zeros((nv, 3))
    kb, bK, bf = _p(tab["kbend"], C.c_double), None, None
    if bend is not None:
        Kd = np.ascontiguousarray(bend[0], np.float64)
        fd = np.ascontiguousarray(bend[1], np.float64)
        kb, bK, bf = None, _p(Kd, C.c_double), _p(fd, C.c_double)
    L.orc_system_ex(nv, nt, _p(tris, C.c_int), _p(tab["ell"], C.c_int),
                    _p(np.ascontiguousarray(tri_f), C.c_double),
                    _p(np.ascontiguousarray(tri_h), C.c_double), kb, bK, bf,
                    _p(tab["mass"], C.c_double), float(gravity), _p(x, C.c_double),
                    _p(xpre, C.c_double), _p(fixed, C.c_ubyte), float(dt), float(ray_a),
                    float(ray_b), _p(A, C.c_double), _p(b, C.c_double), _p(f, C.c_double))
    return A, b, f


def dihedral_rest(mesh: dict, bending_k0: float) -> np.ndarray:
    """Per-edge rest factor -K e / (h0 + h1) of the dihedral model (0 on the boundary)."""
    pos = np.ascontiguousarray(mesh["pos"], np.float64)
    tris = np.ascontiguousarray(mesh["tris"], np.int32)
    edges = np.ascontiguousarray(mesh["edges"], np.int32)
    fac = np.zeros(edges.shape[0])
    lib().orc_dihedral_rest(pos.shape[0], tris.shape[0], edges.shape[0], _p(pos, C.c_double),
                            _p(tris, C.c_int), _p(edges, C.c_int), float(bending_k0),
                            _p(fac, C.c_double))
    return fac


def dihedral(tab: dict, factor: np.ndarray, x: np.ndarray) -> dict:
    """Dihedral force (nv,3), stiffness (nv,32,3,3), beta (ne) and dbeta/dx (ne,4,3)."""
    nv = tab["ell"].shape[0]
    ne = tab["stencil"].shape[0]
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    f = np.zeros((nv, 3))
    K = np.zeros((nv, W, 3, 3))
    beta = np.zeros(ne)
    grad = np.zeros((ne, 4, 3))
    fac = np.ascontiguousarray(factor, np.float64)
    lib().orc_dihedral(nv, ne, _p(tab["stencil"], C.c_int), _p(fac, C.c_double),
                       _p(x, C.c_double), _p(tab["ell"], C.c_int), _p(f, C.c_double),
                       _p(K, C.c_double), _p(beta, C.c_double), _p(grad, C.c_double))
    return {"f": f, "K": K, "beta": beta, "grad": grad}


def spmv(ell, A, x):
    nv = ell.shape[0]
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    y = np.zeros(nv * 3)
    lib().orc_spmv(nv, _p(ell, C.c_int), _p(np.ascontiguousarray(A), C.c_double),
                   _p(x, C.c_double), _p(y, C.c_double))
    return y


def pcg(ell, A, b, fixed, x0=None, max_iters=100000, rel_tol=1e-12, threads=1):
    nv = ell.shape[0]
    x = np.zeros(nv * 3) if x0 is None else np.array(x0, np.float64).reshape(-1)
    fixed = np.ascontiguousarray(fixed, np.uint8)
    res = C.c_double()
    it = lib().orc_pcg(nv, _p(ell, C.c_int), _p(np.ascontiguousarray(A), C.c_double),
                       _p(np.ascontiguousarray(b, np.float64).reshape(-1), C.c_double),
                       _p(fixed, C.c_ubyte), _p(x, C.c_double), int(max_iters),
                       float(rel_tol), C.byref(res), int(threads))
    return x, it, res.value


def max_threads() -> int:
    return int(lib().orc_max_threads())


class OracleCloth:
    """FP64 CPU step of the GPU path (Q-bending, or the CPU cloth's dihedral
    bending with "cloth_bending_model": "dihedral"; block-Jacobi PCG, pins)."""

    def __init__(self, mesh: dict, conf: dict, pins, bodies=None):
        """bodies: static kinematic bodies (dicts with pos, tris, edges,
        tnormal, vnormal) the cloth collides with, in scene order."""
        self.mesh = mesh
        self.conf = conf
        self.bodies = list(bodies or [])
        self.last_contacts = None
        self.tab = tables(mesh, conf["cloth_density"], conf["cloth_bending_stiffness"][:2])
        self.dihedral = conf.get("cloth_bending_model", "quadratic") == "dihedral"
        self.dfac = (dihedral_rest(mesh, conf["cloth_bending_stiffness"][0])
                     if self.dihedral else None)
        nv = mesh["pos"].shape[0]
        self.fixed = np.zeros(nv, np.uint8)
        self.fixed[np.asarray(pins, np.int64)] = 1
        self.pins = np.asarray(pins, np.int64)
        self.x = mesh["pos"].reshape(-1).astype(np.float64).copy()
        self.xpre = self.x.copy()
        self.dx = np.zeros_like(self.x)

    def snap_pins(self):
        tgt = self.mesh["pos"].astype(np.float32).astype(np.float64).reshape(-1, 3)
        x = self.x.reshape(-1, 3)
        xp = self.xpre.reshape(-1, 3)
        x[self.pins] = tgt[self.pins]
        xp[self.pins] = tgt[self.pins]

    def system(self, dt=None):
        c = self.conf
        dt = c["default_timestep"] if dt is None else dt
        self.snap_pins()
        tf, th = triangles(self.mesh, self.tab, self.x, c["cloth_stretch_stiffness"][:3],
                           c.get("fix_fv_norm", 0))
        bend = None
        if self.dihedral:
            dh = dihedral(self.tab, self.dfac, self.x)
            bend = (dh["K"], dh["f"])
        A, b, f = system(self.mesh, self.tab, tf, th, self.x, self.xpre, self.fixed, dt,
                         c.get("rayleigh_damping_a", 0.0), c.get("rayleigh_damping_b", 0.0),
                         bend=bend)
        return A, b, f, tf, th

    def contacts(self) -> dict:
        """Contacts with every body at the current positions, concatenated in
        the detecter's order (point-triangle lists body by body; edge-edge
        lists body by body)."""
        parts = [contacts(self.mesh, self.x, bd) for bd in self.bodies]
        return {k: np.concatenate([p[k] for p in parts]) for k in ("pt_i", "pt_d", "ee_i", "ee_d")}

    def step(self, dt=None, rel_tol=1e-10, max_iters=100000, threads=1):
        c = self.conf
        dt = c["default_timestep"] if dt is None else dt
        A, b, _, _, _ = self.system(dt)
        con = None
        if self.bodies:
            # PrepareCollisionHessian added to the system matrix, then the pin
            # projection of the GPU solver again
            con = self.contacts()
            A = A + contact_hessian(self.tab, self.mesh, con)
            ell = self.tab["ell"]
            for v in range(ell.shape[0]):
                for s_ in range(ell.shape[1]):
                    col = ell[v, s_]
                    if col < 0:
                        break
                    if col != v and (self.fixed[v] or self.fixed[col]):
                        A[v, s_] = 0
        dx, it, res = pcg(self.tab["ell"], A, b, self.fixed, self.dx, max_iters, rel_tol,
                          threads)
        self.dx = dx
        step_dx = dx
        if con is not None:
            step_dx = repulsion(self.mesh, self.tab["mass"], c["cloth_stretch_stiffness"][:3], dt,
                                con, dx)
        self.last_contacts = con
        self.xpre = self.x.copy()
        self.x = self.x + step_dx
        return it, res


# ---------------------------------------------------------------- collisions
def derive_edges(tris) -> np.ndarray:
    """Edges (v0, v1, tri0, tri1) of a triangle list in cObjUtil::BuildEdge's
    numbering (src/utils/ObjUtil.cpp: ascending vertex pairs, first and second
    triangle, tri1 = -1 on the boundary)."""
    tris = np.asarray(tris, np.int64).reshape(-1, 3)
    seen = {}
    for t, tv in enumerate(tris):
        for k in range(3):
            a, b = int(tv[k]), int(tv[(k + 1) % 3])
            key = (a, b) if a < b else (b, a)
            if key in seen:
                seen[key][1] = t
            else:
                seen[key] = [t, -1]
    return np.array([[k[0], k[1], v[0], v[1]] for k, v in sorted(seen.items())], np.int32)


def body_normals(pos, tris):
    """Triangle and vertex normals of a kinematic body as its Init leaves them."""
    pos = np.ascontiguousarray(pos, np.float64)
    tris = np.ascontiguousarray(tris, np.int32)
    tn = np.zeros((tris.shape[0], 3))
    vn = np.zeros((pos.shape[0], 3))
    lib().orc_body_normals(pos.shape[0], tris.shape[0], _p(pos, C.c_double), _p(tris, C.c_int),
                           _p(tn, C.c_double), _p(vn, C.c_double))
    return tn, vn


def contacts(mesh: dict, x, body: dict, max_pt=1 << 20, max_ee=1 << 20) -> dict:
    """Contacts of the cloth (mesh, positions x) with a static body (pos,
    tris, edges, tnormal, vnormal) in the collision detecter's order."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    tris = np.ascontiguousarray(mesh["tris"], np.int32)
    edges = np.ascontiguousarray(mesh["edges"], np.int32)
    bp = np.ascontiguousarray(body["pos"], np.float64)
    bt = np.ascontiguousarray(body["tris"], np.int32)
    be = np.ascontiguousarray(body["edges"], np.int32)
    tn = np.ascontiguousarray(body["tnormal"], np.float64)
    vn = np.ascontiguousarray(body["vnormal"], np.float64)
    pt_i = np.zeros((max_pt, 3), np.int32)
    pt_d = np.zeros((max_pt, 7))
    ee_i = np.zeros((max_ee, 3), np.int32)
    ee_d = np.zeros((max_ee, 6))
    npt, nee = C.c_int(), C.c_int()
    rc = lib().orc_contacts(x.size // 3, tris.shape[0], edges.shape[0], _p(x, C.c_double),
                            _p(tris, C.c_int), _p(edges, C.c_int), bp.shape[0], bt.shape[0],
                            be.shape[0], _p(bp, C.c_double), _p(bt, C.c_int), _p(be, C.c_int),
                            _p(tn, C.c_double), _p(vn, C.c_double), max_pt, _p(pt_i, C.c_int),
                            _p(pt_d, C.c_double), C.byref(npt), max_ee, _p(ee_i, C.c_int),
                            _p(ee_d, C.c_double), C.byref(nee))
    if rc != 0:
        raise ValueError("oracle: contact list overflow")
    return {"pt_i": pt_i[:npt.value].copy(), "pt_d": pt_d[:npt.value].copy(),
            "ee_i": ee_i[:nee.value].copy(), "ee_d": ee_d[:nee.value].copy()}


def contact_hessian(tab: dict, mesh: dict, con: dict) -> np.ndarray:
    nv = tab["ell"].shape[0]
    H = np.zeros((nv, W, 3, 3))
    lib().orc_contact_hessian(nv, _p(np.ascontiguousarray(mesh["tris"], np.int32), C.c_int),
                              _p(tab["ell"], C.c_int), con["pt_i"].shape[0],
                              _p(np.ascontiguousarray(con["pt_i"]), C.c_int),
                              _p(np.ascontiguousarray(con["pt_d"]), C.c_double),
                              _p(H, C.c_double))
    return H


def repulsion(mesh: dict, mass, stretch_k, dt: float, con: dict, dx) -> np.ndarray:
    out = np.array(dx, np.float64).reshape(-1).copy()
    ks = np.asarray(stretch_k, np.float32)
    lib().orc_repulsion(out.size // 3, _p(np.ascontiguousarray(mesh["tris"], np.int32), C.c_int),
                        _p(np.ascontiguousarray(mesh["edges"], np.int32), C.c_int),
                        _p(np.ascontiguousarray(mass, np.float64), C.c_double),
                        _p(ks, C.c_float), float(dt), con["pt_i"].shape[0],
                        _p(np.ascontiguousarray(con["pt_i"]), C.c_int),
                        _p(np.ascontiguousarray(con["pt_d"]), C.c_double),
                        con["ee_i"].shape[0], _p(np.ascontiguousarray(con["ee_i"]), C.c_int),
                        _p(np.ascontiguousarray(con["ee_d"]), C.c_double), _p(out, C.c_double))
    return out
