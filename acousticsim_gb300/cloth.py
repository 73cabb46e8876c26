"""Host-side mirror of AcousticSim's cloth-simulator API for the GPU cloth.

`BaraffClothGpu` takes the reference's JSON configuration keys and exposes the
methods of cBaraffClothGpu / cBaseCloth (src/sim/cloth/BaraffClothGpu.h:16-27,
src/sim/cloth/BaseCloth.h:19-46) on top of the C ABI in libcloth_gb300.so.
Every call goes to the native library; there is no other implementation.
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable, Sequence

import numpy as np

from . import _native as N


import atexit
import sys
import weakref

# Contexts still open when the interpreter exits are closed here, while the
# native library and this module are intact (finalizers that run during
# interpreter teardown may find neither).
_open_contexts: "weakref.WeakSet[ClothContext]" = weakref.WeakSet()


@atexit.register
def _close_open_contexts() -> None:
    for ctx in list(_open_contexts):
        try:
            ctx.close()
        except Exception:
            pass


class ClothContext:
    """One device and one CUDA stream (cloth_ctx)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        self._cloths = weakref.WeakSet()
        self._servers = weakref.WeakSet()
        self._bodies = weakref.WeakSet()
        N.call("cloth_ctx_create", int(device), C.byref(self._h))
        _open_contexts.add(self)

    @property
    def handle(self):
        return self._h

    def synchronize(self) -> None:
        N.call("cloth_ctx_synchronize", self._h)

    def set_profiling(self, on: bool) -> None:
        N.call("cloth_ctx_set_profiling", self._h, int(bool(on)))

    def reset_profile(self) -> None:
        N.call("cloth_ctx_reset_profile", self._h)

    def profile(self) -> dict:
        ms = (C.c_double * N.NUM_PHASES)()
        n = (C.c_longlong * N.NUM_PHASES)()
        N.call("cloth_ctx_get_profile", self._h, ms, n)
        return {N.PHASE_NAMES[k]: {"ms": ms[k], "launches": n[k]} for k in range(N.NUM_PHASES)}

    def set_solver(self, solver: str) -> None:
        """'persistent' (default: one cooperative launch; falls back to the graph
        loop when the set does not fit), 'persistent_1b' (single-barrier
        iterations where every block's halo is staged), 'persistent_2b' (the
        two-barrier persistent kernel only) or 'graph_loop'."""
        code = {"persistent": N.SOLVER_PERSISTENT, "graph_loop": N.SOLVER_GRAPH_LOOP,
                "persistent_1b": N.SOLVER_PERSISTENT_1B,
                "persistent_2b": N.SOLVER_PERSISTENT_2B}[solver]
        N.call("cloth_ctx_set_solver", self._h, code)

    def set_tail_hand_off(self, max_instances: int = -1) -> None:
        """Graph-loop launch sets hand their last `max_instances` iterating
        cloths to the persistent kernel (same results bit for bit; -1: the SM
        count / 16, 0: never).  For launch sets built after the call."""
        N.call("cloth_ctx_set_tail_hand_off", self._h, int(max_instances))

    def set_spin_limit(self, polls: int = 0, extra_arrivals: int = 0) -> None:
        """Bounded team-barrier waits of the persistent solvers: give up after
        `polls` polls (0: the default) with status TIMEOUT.  `extra_arrivals`
        makes every barrier wait for arrivals no block makes (a test of the
        timeout path); 0 in normal use."""
        N.call("cloth_ctx_set_spin_limit", self._h, int(polls), int(extra_arrivals))

    def set_escalation(self, on: bool | int = True) -> None:
        """Steps whose FP32 PCG ends in NaN or breakdown are re-solved by the
        FP64 PCG and advanced; stats report the solver "escalated_fp64".  On by
        default (level 1); level 2 (on=2) escalates steps whose FP32 PCG ends at
        max_iters too; a step called without stats (step_async) is not
        escalated."""
        N.call("cloth_ctx_set_escalation", self._h, int(on))

    # (rows per thread, slot unroll, tiles per block); slot unroll 0: the
    # bulk-staged SpMV, whose third number is its ring of stages and whose
    # first is 1 when it also stages p over each tile's column range
    SPMV_VARIANTS = [(1, 1, 1), (1, 2, 1), (1, 3, 1), (2, 1, 1), (2, 2, 1), (4, 1, 1),
                     (1, 1, 4), (1, 2, 4), (2, 1, 4), (2, 2, 4), (4, 1, 4), (2, 1, 8),
                     (1, 0, 2), (1, 0, 3), (0, 0, 2), (0, 0, 3), (0, 0, 4)]
    UPDATE_VARIANTS = [(1, 1), (2, 1), (4, 1), (1, 4), (2, 4), (1, 8), (2, 8)]

    def set_kernel_variant(self, spmv=(1, 3, 1), update=(1, 1), autotune: bool = False) -> None:
        """Graph-loop kernels: spmv = (rows per thread, slot unroll, tiles per block),
        update = (rows per thread, tiles per block)."""
        N.call("cloth_ctx_set_kernel_variant", self._h, *map(int, spmv), *map(int, update),
               int(bool(autotune)))

    def kernel_variant(self) -> dict:
        v = [C.c_int() for _ in range(6)]
        N.call("cloth_ctx_get_kernel_variant", self._h, *[C.byref(x) for x in v])
        return {"spmv": tuple(x.value for x in v[:3]), "update": (v[3].value, v[4].value),
                "autotune": bool(v[5].value)}

    def tuning_times(self) -> dict:
        """Per-variant kernel times (ms) of the last autotuning."""
        a = (C.c_float * len(self.SPMV_VARIANTS))()
        b = (C.c_float * len(self.UPDATE_VARIANTS))()
        N.call("cloth_ctx_get_tuning_times", self._h, a, len(a), b, len(b))
        return {"spmv": {"R%dU%dT%d" % v: a[i] for i, v in enumerate(self.SPMV_VARIANTS)},
                "update": {"R%dT%d" % v: b[i] for i, v in enumerate(self.UPDATE_VARIANTS)}}

    def stream_ptr(self) -> int:
        s = C.c_void_p()
        N.call("cloth_ctx_get_stream", self._h, C.byref(s))
        return int(s.value or 0)

    def device_bytes(self) -> int:
        b = C.c_size_t()
        N.call("cloth_ctx_device_bytes", self._h, C.byref(b))
        return int(b.value)

    def batch_step(self, cloths: Sequence["BaraffClothGpu"], dt: float = 0.0,
                   params: N.SolveParams | None = None, stats: bool = True):
        n = len(cloths)
        arr = (C.c_void_p * n)(*[c.handle for c in cloths])
        st = (N.SolveStats * n)() if stats else None
        N.call("cloth_batch_step", self._h, arr, n, float(dt),
               C.byref(params) if params is not None else None, st)
        return [s.as_dict() for s in st] if stats else None

    def close(self) -> None:
        # the context frees every server and cloth it holds; their handles die with it
        for c in list(self._cloths) + list(self._servers) + list(self._bodies):
            c._h = C.c_void_p()
        if self._h:
            N.load().cloth_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        # during interpreter teardown the native library, the CUDA runtime's
        # users (torch) and this module may already be half gone: the atexit
        # handler has closed every context before that point, so do nothing
        try:
            if sys.is_finalizing():
                return
            self.close()
        except Exception:
            pass


def build_grid(cloth_size=(1.0, 1.0), subdivision=(19, 19), init_pos=(0.0, 0.0, 0.0),
               uv_rotation_deg: float = 0.0, geometry_type: str = "regular_triangle",
               seed: int = 0) -> dict:
    """cTriangulator::BuildGeometry for geometry_type "regular_triangle",
    "regular_triangle_perturb" or "delaunay" (the last two draw from the
    reference's generator seeded with `seed`; its main seeds it with 0);
    arrays in numpy."""
    g = N.GridDesc((C.c_double * 2)(*cloth_size), (C.c_int * 2)(*subdivision),
                   (C.c_double * 3)(*init_pos), float(uv_rotation_deg))
    gt = str(geometry_type).encode()
    nv, nt, ne = C.c_int(), C.c_int(), C.c_int()
    N.call("cloth_geometry_build", C.byref(g), gt, int(seed), C.byref(nv), C.byref(nt),
           C.byref(ne), None, None, None, None)
    pos = np.zeros((nv.value, 3), np.float64)
    uv = np.zeros((nv.value, 2), np.float32)
    tris = np.zeros((nt.value, 3), np.int32)
    edges = np.zeros((ne.value, 4), np.int32)
    N.call("cloth_geometry_build", C.byref(g), gt, int(seed), None, None, None,
           N.ptr(pos, C.c_double), N.ptr(uv, C.c_float), N.ptr(tris, C.c_int),
           N.ptr(edges, C.c_int))
    return {"pos": pos, "uv": uv, "tris": tris, "edges": edges}


def load_obj_mesh(path: str, translation=(0.0, 0.0, 0.0), relocate: bool = False) -> dict:
    """cBaseCloth::InitGeometry's OBJ branch ("enable_cloth_from_obj"); arrays in numpy."""
    tr = (C.c_double * 3)(*translation)
    p = str(path).encode()
    nv, nt, ne = C.c_int(), C.c_int(), C.c_int()
    N.call("cloth_mesh_from_obj", p, tr, int(relocate), C.byref(nv), C.byref(nt),
           C.byref(ne), None, None, None, None)
    pos = np.zeros((nv.value, 3), np.float64)
    uv = np.zeros((nv.value, 2), np.float32)
    tris = np.zeros((nt.value, 3), np.int32)
    edges = np.zeros((ne.value, 4), np.int32)
    N.call("cloth_mesh_from_obj", p, tr, int(relocate), None, None, None,
           N.ptr(pos, C.c_double), N.ptr(uv, C.c_float), N.ptr(tris, C.c_int),
           N.ptr(edges, C.c_int))
    return {"pos": pos, "uv": uv, "tris": tris, "edges": edges}


def derive_edges_host(tris) -> np.ndarray:
    """Edges (v0, v1, tri0, tri1) of a triangle list as cObjUtil::BuildEdge
    numbers them (ascending vertex pairs; tri1 = -1 on the boundary)."""
    tris = np.asarray(tris, np.int64).reshape(-1, 3)
    info = {}
    for t, tv in enumerate(tris):
        for k in range(3):
            a, b = int(tv[k]), int(tv[(k + 1) % 3])
            key = (min(a, b), max(a, b))
            if key in info:
                info[key][1] = t
            else:
                info[key] = [t, -1]
    return np.array([[k[0], k[1], v[0], v[1]] for k, v in sorted(info.items())], np.int32)


def _vec(conf: dict, key: str, default=None):
    v = conf.get(key, default)
    if v is None:
        raise KeyError(f"config key '{key}' is missing")
    return list(v)


class BaraffClothGpu:
    """cBaraffClothGpu on the GB300 library.

    conf uses the reference's keys: geometry_type ("regular_triangle",
    "regular_triangle_perturb" or "delaunay"; "rand_seed", default 0, seeds
    the random ones),
    cloth_size, subdivision, cloth_init_pos, cloth_init_orientation (zero),
    cloth_uv_rotation, cloth_stretch_stiffness, cloth_bending_stiffness,
    cloth_density, rayleigh_damping_a/b, default_timestep and
    constraints.static_point.  A mesh dict (pos, uv, tris[, edges]) may be
    passed instead of the grid keys.
    """

    def __init__(self, ctx: ClothContext, conf: dict | None = None, mesh: dict | None = None):
        self.ctx = ctx
        self._h = C.c_void_p()
        if conf is not None:
            self.Init(conf, mesh)

    # ---------------------------------------------------------------- init
    def Init(self, conf: dict, mesh: dict | None = None) -> None:
        """cBaraffClothGpu::Init (BaraffClothGpu.cpp:24-49)."""
        if mesh is None and conf.get("enable_cloth_from_obj", False):
            mesh = load_obj_mesh(conf["cloth_obj_path"],
                                 tuple(_vec(conf, "cloth_obj_translation", [0, 0, 0])[:3]),
                                 bool(conf.get("enable_relocate_obj", False)))
        if mesh is None:
            gt = conf.get("geometry_type", "regular_triangle")
            if gt not in ("regular_triangle", "regular_triangle_perturb", "delaunay"):
                raise ValueError(f"geometry_type '{gt}' is not supported")
            orient = conf.get("cloth_init_orientation", [0, 0, 0, 0])
            if any(float(a) != 0.0 for a in orient):
                raise ValueError("cloth_init_orientation must be zero")
            # "rand_seed": the state of the reference's generator the random
            # geometries draw from (its main seeds it with 0)
            mesh = build_grid(tuple(_vec(conf, "cloth_size")), tuple(int(s) for s in _vec(conf, "subdivision")),
                              tuple(_vec(conf, "cloth_init_pos", [0, 0, 0])[:3]),
                              float(conf.get("cloth_uv_rotation", 0)), gt,
                              int(conf.get("rand_seed", 0)))
        self.mesh = {k: np.ascontiguousarray(v) for k, v in mesh.items()}
        pos = np.ascontiguousarray(self.mesh["pos"], np.float64)
        uv = np.ascontiguousarray(self.mesh["uv"], np.float32)
        tris = np.ascontiguousarray(self.mesh["tris"], np.int32)
        edges = self.mesh.get("edges")
        ne = 0
        eptr = None
        if edges is not None:
            edges = np.ascontiguousarray(edges, np.int32)
            ne = edges.shape[0]
            eptr = N.ptr(edges, C.c_int)
        md = N.MeshDesc(pos.shape[0], tris.shape[0], ne, N.ptr(pos, C.c_double),
                        N.ptr(uv, C.c_float), N.ptr(tris, C.c_int), eptr)
        self.material = self._material(conf)
        N.call("cloth_create", self.ctx.handle, C.byref(md), C.byref(self.material),
               C.byref(self._h))
        self.ctx._cloths.add(self)
        self.nv, self.nt = pos.shape[0], tris.shape[0]
        cons = conf.get("constraints", {})
        if "static_point" in cons:
            uvs = np.ascontiguousarray(np.asarray(cons["static_point"], np.float32).reshape(-1, 2))
            ids = self.FindVerticesIdFromUV(uvs)
            self.AddConstraintStaticVertices(ids)

    @staticmethod
    def _material(conf: dict) -> N.Material:
        ks = _vec(conf, "cloth_stretch_stiffness")[:3]
        kb = _vec(conf, "cloth_bending_stiffness")[:2]
        return N.Material((C.c_float * 3)(*ks), (C.c_float * 2)(*kb),
                          float(conf["cloth_density"]), float(conf.get("rayleigh_damping_a", 0.0)),
                          float(conf.get("rayleigh_damping_b", 0.0)),
                          float(conf["default_timestep"]), float(conf.get("gravity", -9.8)),
                          int(conf.get("fix_fv_norm", 0)),
                          N.BENDING_MODELS[conf.get("cloth_bending_model", "quadratic")])

    @property
    def handle(self):
        return self._h

    def SetMaterial(self, conf: dict) -> None:
        self.material = self._material(conf)
        N.call("cloth_set_material", self._h, C.byref(self.material))

    # ---------------------------------------------------------------- pins
    def FindVerticesIdFromUV(self, uvs: np.ndarray) -> np.ndarray:
        uvs = np.ascontiguousarray(uvs, np.float32).reshape(-1, 2)
        out = np.zeros(uvs.shape[0], np.int32)
        N.call("cloth_find_vertices_from_uv", self._h, N.ptr(uvs, C.c_float), uvs.shape[0],
               N.ptr(out, C.c_int))
        return out

    def AddConstraintStaticVertices(self, vids: Iterable[int]) -> None:
        v = np.ascontiguousarray(np.asarray(list(vids), np.int32))
        N.call("cloth_add_static_vertices", self._h, N.ptr(v, C.c_int), v.size)

    def ClearConstraintStaticVertices(self) -> None:
        N.call("cloth_clear_static_vertices", self._h)

    def GetConstraintStaticVertices(self) -> list[int]:
        n = C.c_int()
        N.call("cloth_get_static_vertices", self._h, None, 0, C.byref(n))
        out = np.zeros(max(1, n.value), np.int32)
        N.call("cloth_get_static_vertices", self._h, N.ptr(out, C.c_int), n.value, C.byref(n))
        return out[: n.value].tolist()

    def ApplyUserPerturbForceOnce(self, vid: int, target) -> None:
        """Drag point for the next step (BaraffClothGpu.cpp:266-281)."""
        t = np.ascontiguousarray(np.asarray(target, np.float32).reshape(3))
        N.call("cloth_set_drag_point", self._h, int(vid), N.ptr(t, C.c_float))

    # ---------------------------------------------------------------- state
    def SetPos(self, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        N.call("cloth_set_pos", self._h, N.ptr(x, C.c_double), x.size // 3)

    def SetPrePos(self, x: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float64).reshape(-1)
        N.call("cloth_set_pre_pos", self._h, N.ptr(x, C.c_double), x.size // 3)

    def GetPos(self) -> np.ndarray:
        x = np.zeros(self.nv * 3, np.float64)
        N.call("cloth_get_pos", self._h, N.ptr(x, C.c_double), self.nv)
        return x

    def GetPrePos(self) -> np.ndarray:
        x = np.zeros(self.nv * 3, np.float64)
        N.call("cloth_get_pre_pos", self._h, N.ptr(x, C.c_double), self.nv)
        return x

    def GetInitPos(self) -> np.ndarray:
        return np.asarray(self.mesh["pos"], np.float64).reshape(-1).copy()

    def matrix_info(self) -> dict:
        nnzb = C.c_longlong()
        w = C.c_int()
        rb = C.c_size_t()
        sb = C.c_size_t()
        N.call("cloth_matrix_info", self._h, C.byref(nnzb), C.byref(w), C.byref(rb),
               C.byref(sb))
        return {"nnzb": nnzb.value, "width": w.value, "resident_bytes": rb.value,
                "solve_bytes": sb.value}

    def GetNumOfVertices(self) -> int:
        return self.nv

    def GetNumOfTriangles(self) -> int:
        return self.nt

    def Reset(self) -> None:
        N.call("cloth_reset", self._h)

    # ---------------------------------------------------------------- step
    def UpdatePos(self, dt: float = 0.0, params: N.SolveParams | None = None) -> dict:
        """One implicit step; like the reference, dt <= 0 means default_timestep."""
        st = N.SolveStats()
        N.call("cloth_step", self._h, float(dt), C.byref(params) if params is not None else None,
               C.byref(st))
        return st.as_dict()

    Update = UpdatePos

    def UpdatePosPlain(self, dt: float = 0.0, params: N.SolveParams | None = None) -> dict:
        """One step through the reference-structured baseline (cloth_step_plain)."""
        st = N.SolveStats()
        N.call("cloth_step_plain", self._h, float(dt),
               C.byref(params) if params is not None else None, C.byref(st))
        return st.as_dict()

    def step_async(self, dt: float = 0.0, params: N.SolveParams | None = None) -> None:
        N.call("cloth_step", self._h, float(dt), C.byref(params) if params is not None else None,
               None)

    def step_host(self, x_in, xpre_in, x_out, dt: float = 0.0,
                  params: N.SolveParams | None = None) -> dict:
        """Step with host buffers (upload x, x_pre; download x), as UpdatePos
        exchanges them; returns the step's stats."""
        st = N.SolveStats()
        N.call("cloth_step_host", self._h, float(dt),
               C.byref(params) if params is not None else None,
               N.ptr(x_in, C.c_double) if x_in is not None else None,
               N.ptr(xpre_in, C.c_double) if xpre_in is not None else None,
               N.ptr(x_out, C.c_double) if x_out is not None else None, C.byref(st))
        return st.as_dict()

    # ---------------------------------------------------------------- seam
    def assemble(self, dt: float = 0.0) -> None:
        N.call("cloth_assemble", self._h, float(dt))

    def solve(self, params: N.SolveParams | None = None) -> dict:
        st = N.SolveStats()
        N.call("cloth_solve", self._h, C.byref(params) if params is not None else None,
               C.byref(st))
        return st.as_dict()

    def solve_refined(self, inner: N.SolveParams, rel_tol: float = 1e-8,
                      max_outer: int = 20) -> dict:
        """FP32 PCG corrections inside an FP64 residual loop (after assemble)."""
        st = N.RefineStats()
        N.call("cloth_solve_refined", self._h, C.byref(inner), float(rel_tol), int(max_outer),
               C.byref(st))
        return st.as_dict()

    def solve_flexible(self, inner: N.SolveParams, rel_tol: float = 1e-8,
                       max_outer: int = 100000) -> dict:
        """FP64 flexible CG with FP32 PCG inner solves (after assemble)."""
        st = N.RefineStats()
        N.call("cloth_solve_flexible", self._h, C.byref(inner), float(rel_tol), int(max_outer),
               C.byref(st))
        return st.as_dict()

    def solve_fp64(self, params: N.SolveParams) -> dict:
        """All-FP64 block-Jacobi PCG from zero (after assemble)."""
        st = N.SolveStats()
        N.call("cloth_solve_fp64", self._h, C.byref(params), C.byref(st))
        return st.as_dict()

    def residual_fp64(self) -> float:
        """||b - A dx|| / ||b|| in FP64 for the current dx."""
        v = C.c_double()
        N.call("cloth_residual_fp64", self._h, C.byref(v))
        return float(v.value)

    def advance(self) -> None:
        N.call("cloth_advance", self._h)

    def stats(self) -> dict:
        st = N.SolveStats()
        N.call("cloth_get_stats", self._h, C.byref(st))
        return st.as_dict()

    def get_dx(self) -> np.ndarray:
        dx = np.zeros(self.nv * 3, np.float64)
        N.call("cloth_get_dx", self._h, N.ptr(dx, C.c_double), self.nv)
        return dx

    def export_system(self) -> dict:
        W = N.ELL_REF_WIDTH
        ell = np.zeros((self.nv, W), np.int32)
        A = np.zeros((self.nv, W, 3, 3), np.float32)
        b = np.zeros((self.nv, 3), np.float32)
        f = np.zeros((self.nv, 3), np.float32)
        kb = np.zeros((self.nv, W), np.float32)
        N.call("cloth_export_system", self._h, N.ptr(ell, C.c_int), N.ptr(A, C.c_float),
               N.ptr(b, C.c_float), N.ptr(f, C.c_float), N.ptr(kb, C.c_float))
        return {"ell": ell, "A": A, "b": b, "fint": f, "kbend": kb}

    def export_triangles(self) -> dict:
        f = np.zeros((self.nt, 3, 3), np.float32)
        h = np.zeros((self.nt, 9, 3, 3), np.float32)
        N.call("cloth_export_triangles", self._h, N.ptr(f, C.c_float), N.ptr(h, C.c_float))
        return {"fint": f, "hess": h}

    def export_dihedral(self) -> dict:
        n = C.c_int()
        N.call("cloth_export_dihedral", self._h, C.byref(n), None, None, None)
        ids = np.zeros(n.value, np.int32)
        g = np.zeros((n.value, 4, 3), np.float32)
        cf = np.zeros((n.value, 2), np.float32)
        N.call("cloth_export_dihedral", self._h, C.byref(n), N.ptr(ids, C.c_int),
               N.ptr(g, C.c_float), N.ptr(cf, C.c_float))
        return {"edge_ids": ids, "grad": g, "factor": cf[:, 0], "force_coef": cf[:, 1]}

    # ---------------------------------------------------------------- collisions
    def set_bodies(self, bodies) -> None:
        """Kinematic bodies this cloth collides with (the CPU cloth's contact
        handling; an empty list turns it off)."""
        bodies = list(bodies)
        arr = (C.c_void_p * max(1, len(bodies)))(*[b.handle for b in bodies])
        N.call("cloth_set_bodies", self._h, arr, len(bodies))
        self._bodies = bodies

    def set_contact_capacity(self, pairs=0, point_triangle=0, edge_edge=0) -> None:
        N.call("cloth_set_contact_capacity", self._h, int(pairs), int(point_triangle),
               int(edge_edge))

    def get_contacts(self) -> dict:
        """Contacts of the last step in the collision detecter's order."""
        st = N.ContactStats()
        N.call("cloth_get_contacts", self._h, C.byref(st), None, None, None, None)
        pt_i = np.zeros((st.n_pt, 3), np.int32)
        pt_d = np.zeros((st.n_pt, 7), np.float64)
        ee_i = np.zeros((st.n_ee, 3), np.int32)
        ee_d = np.zeros((st.n_ee, 6), np.float64)
        N.call("cloth_get_contacts", self._h, C.byref(st), N.ptr(pt_i, C.c_int),
               N.ptr(pt_d, C.c_double), N.ptr(ee_i, C.c_int), N.ptr(ee_d, C.c_double))
        return {"pt_i": pt_i, "pt_d": pt_d, "ee_i": ee_i, "ee_d": ee_d,
                "overflow": st.overflow, "repulsion_rounds": st.repulsion_rounds}

    def get_repulsed_dx(self) -> np.ndarray:
        dx = np.zeros(self.nv * 3, np.float64)
        N.call("cloth_get_repulsed_dx", self._h, N.ptr(dx, C.c_double), self.nv)
        return dx

    def export_tables(self) -> dict:
        ne = C.c_int()
        N.call("cloth_num_vertices", self._h, None, None, C.byref(ne))
        st = np.zeros((ne.value, 4), np.int32)
        coef = np.zeros((self.nt, 12), np.float32)
        area = np.zeros(self.nt, np.float32)
        mass = np.zeros(self.nv, np.float32)
        ts = np.zeros((self.nt, 9), np.int32)
        N.call("cloth_export_tables", self._h, N.ptr(st, C.c_int), N.ptr(coef, C.c_float),
               N.ptr(area, C.c_float), N.ptr(mass, C.c_float), N.ptr(ts, C.c_int))
        return {"stencil": st, "coef": coef, "area": area, "mass": mass, "tri_slot": ts}

    def close(self) -> None:
        # a cloth held by a server stays alive until the server (or the context) goes
        if self._h and N.load().cloth_destroy(self._h) == N.CLOTH_OK:
            self._h = C.c_void_p()

    def __del__(self):
        # during interpreter teardown the native library, the CUDA runtime's
        # users (torch) and this module may already be half gone: the atexit
        # handler has closed every context before that point, so do nothing
        try:
            if sys.is_finalizing():
                return
            self.close()
        except Exception:
            pass


def _vec3(v) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, np.float64).reshape(-1)[:3])


def kinematic_pose(local, init_pos, init_ori, target_pos, target_ori, elapsed_sec: float,
                   time: float) -> np.ndarray:
    """cKinematicBody's pose of a moving body at body time `time` applied to
    its local mesh (host only): world positions, nv x 3."""
    local = np.ascontiguousarray(local, np.float64).reshape(-1, 3)
    out = np.zeros_like(local)
    vs = [_vec3(v) for v in (init_pos, init_ori, target_pos, target_ori)]
    N.call("cloth_kinematic_pose", local.shape[0], N.ptr(local, C.c_double),
           *[N.ptr(v, C.c_double) for v in vs], float(elapsed_sec), float(time),
           N.ptr(out, C.c_double))
    return out


class ClothBody:
    """A kinematic body (cKinematicBody after Init): a world-space triangle
    mesh the cloths of a context can collide with.  Static unless moved with
    set_pos, or given the reference's time-driven motion (set_motion, then
    update(dt) per frame)."""

    def __init__(self, ctx: ClothContext, pos, tris):
        self.ctx = ctx
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        tris = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
        self._h = C.c_void_p()
        N.call("cloth_body_create", ctx.handle, pos.shape[0], tris.shape[0],
               N.ptr(pos, C.c_double), N.ptr(tris, C.c_int), C.byref(self._h))
        self.pos, self.tris = pos, tris
        ctx._bodies.add(self)

    @property
    def handle(self):
        return self._h

    def set_pos(self, pos) -> None:
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1)
        N.call("cloth_body_set_pos", self._h, N.ptr(pos, C.c_double))

    def set_motion(self, local, init_pos, init_ori, target_pos, target_ori,
                   elapsed_sec: float) -> None:
        local = np.ascontiguousarray(local, np.float64).reshape(-1)
        vs = [_vec3(v) for v in (init_pos, init_ori, target_pos, target_ori)]
        N.call("cloth_body_set_motion", self._h, N.ptr(local, C.c_double),
               *[N.ptr(v, C.c_double) for v in vs], float(elapsed_sec))

    def update(self, dt: float) -> None:
        N.call("cloth_body_update", self._h, float(dt))

    def get_pos(self) -> np.ndarray:
        out = np.zeros((self.pos.shape[0], 3), np.float64)
        N.call("cloth_body_get_pos", self._h, N.ptr(out, C.c_double))
        return out

    def close(self) -> None:
        if self._h and N.load().cloth_body_destroy(self._h) == N.CLOTH_OK:
            self._h = C.c_void_p()


class ClothServer:
    """Request server with continuous batching (cloth_server_*).

    Register cloths with `add`, then `start`; `submit(index, tag, t_arrival)`
    queues one step of a cloth, `poll` returns completed requests as dicts
    with the arrival, admission and completion times on the `now()` clock."""

    def __init__(self, ctx: ClothContext, budget_bytes: int, max_inflight: int = 0,
                 chunk_iters: int = 16):
        self._h = C.c_void_p()
        self.ctx = ctx
        self._held = []
        cfg = N.ServerConfig(int(budget_bytes), int(max_inflight), int(chunk_iters))
        N.call("cloth_server_create", ctx.handle, C.byref(cfg), C.byref(self._h))
        ctx._servers.add(self)

    @staticmethod
    def now() -> float:
        return float(N.load().cloth_server_now())

    def add(self, cloth: BaraffClothGpu, dt: float = 0.0,
            params: N.SolveParams | None = None) -> int:
        idx = C.c_int()
        N.call("cloth_server_add", self._h, cloth.handle, float(dt),
               C.byref(params) if params is not None else None, C.byref(idx))
        self._held.append(cloth)
        return idx.value

    def start(self) -> None:
        N.call("cloth_server_start", self._h)

    def submit(self, index: int, tag: int, t_arrival: float = -1.0) -> None:
        N.call("cloth_server_submit", self._h, int(index), int(tag), float(t_arrival))

    def poll(self, cap: int = 4096, wait_s: float = 0.0) -> list[dict]:
        out = (N.ServerResult * cap)()
        n = C.c_int()
        N.call("cloth_server_poll", self._h, out, int(cap), C.byref(n), float(wait_s))
        return [out[k].as_dict() for k in range(n.value)]

    def drain(self, wait_s: float = -1.0) -> None:
        N.call("cloth_server_drain", self._h, float(wait_s))

    def stats(self) -> dict:
        st = N.ServerStats()
        N.call("cloth_server_get_stats", self._h, C.byref(st))
        return st.as_dict()

    def close(self) -> None:
        if self._h:
            N.load().cloth_server_destroy(self._h)
            self._h = C.c_void_p()
        self._held = []

    def __del__(self):
        # during interpreter teardown the native library, the CUDA runtime's
        # users (torch) and this module may already be half gone: the atexit
        # handler has closed every context before that point, so do nothing
        try:
            if sys.is_finalizing():
                return
            self.close()
        except Exception:
            pass
