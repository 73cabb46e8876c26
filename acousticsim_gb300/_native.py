"""ctypes bindings of libcloth_gb300.so (declarations: include/cloth_gb300.h).

The library is loaded from the package directory; when it is missing this
module raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libcloth_gb300.so"

CLOTH_OK = 0
STATUS_NAMES = {
    0: "OK", 1: "INVALID", 2: "CUDA", 3: "OOM", 4: "BUDGET", 5: "MESH", 6: "NAN",
    7: "BREAKDOWN", 8: "MAXITER", 9: "TIMEOUT", 10: "UNSUPPORTED", 11: "STATE",
    12: "CONTACTS",
}
NUM_PHASES = 9
PHASE_NAMES = ["pins", "tri_assemble", "row_assemble", "spmv_dot", "update_dot", "advance",
               "contacts", "repulsion", "reduce"]
ELL_REF_WIDTH = 32
SOLVER_PERSISTENT = 0
SOLVER_GRAPH_LOOP = 1
SOLVER_FP64 = 2
SOLVER_PERSISTENT_1B = 3
SOLVER_PERSISTENT_2B = 4
SOLVER_NAMES = {0: "persistent", 1: "graph_loop", 2: "fp64", 3: "persistent_1b",
                4: "persistent_2b", 5: "escalated_fp64", -1: "plain"}


class GridDesc(C.Structure):
    _fields_ = [("cloth_size", C.c_double * 2), ("subdivision", C.c_int * 2),
                ("init_pos", C.c_double * 3), ("uv_rotation_deg", C.c_float)]


class MeshDesc(C.Structure):
    _fields_ = [("nv", C.c_int), ("nt", C.c_int), ("ne", C.c_int),
                ("pos", C.POINTER(C.c_double)), ("uv", C.POINTER(C.c_float)),
                ("tris", C.POINTER(C.c_int)), ("edges", C.POINTER(C.c_int))]


class Material(C.Structure):
    _fields_ = [("stretch_k", C.c_float * 3), ("bending_k", C.c_float * 2),
                ("density", C.c_float), ("rayleigh_a", C.c_float), ("rayleigh_b", C.c_float),
                ("default_timestep", C.c_double), ("gravity", C.c_double),
                ("fix_fv_norm", C.c_int), ("bending_model", C.c_int)]


BENDING_MODELS = {"quadratic": 0, "dihedral": 1}


class ContactStats(C.Structure):
    _fields_ = [("n_pt", C.c_int), ("n_ee", C.c_int), ("overflow", C.c_int),
                ("repulsion_rounds", C.c_int)]


class SolveParams(C.Structure):
    _fields_ = [("max_iters", C.c_int), ("rel_tol", C.c_double), ("abs_tol", C.c_double),
                ("check_every", C.c_int), ("warm_start", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iters", C.c_int), ("status", C.c_int), ("res_norm", C.c_double),
                ("rhs_norm", C.c_double), ("rel_residual", C.c_double), ("solver", C.c_int)]

    def as_dict(self) -> dict:
        return {"iters": self.iters, "status": STATUS_NAMES.get(self.status, str(self.status)),
                "res_norm": self.res_norm, "rhs_norm": self.rhs_norm,
                "rel_residual": self.rel_residual,
                "solver": SOLVER_NAMES.get(self.solver, str(self.solver))}


class RefineStats(C.Structure):
    _fields_ = [("outer", C.c_int), ("inner_iters", C.c_int), ("status", C.c_int),
                ("solver", C.c_int), ("initial_rel_residual", C.c_double),
                ("rel_residual", C.c_double), ("last_inner_rel_residual", C.c_double),
                ("rejected", C.c_int), ("pad", C.c_int)]

    def as_dict(self) -> dict:
        return {"outer": self.outer, "inner_iters": self.inner_iters,
                "status": STATUS_NAMES.get(self.status, str(self.status)),
                "solver": SOLVER_NAMES.get(self.solver, str(self.solver)),
                "initial_rel_residual": self.initial_rel_residual,
                "rel_residual": self.rel_residual,
                "last_inner_rel_residual": self.last_inner_rel_residual,
                "rejected": self.rejected}


class ServerConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_size_t), ("max_inflight", C.c_int),
                ("chunk_iters", C.c_int)]


class ServerResult(C.Structure):
    _fields_ = [("tag", C.c_longlong), ("cloth", C.c_int), ("status", C.c_int),
                ("iters", C.c_int), ("pad", C.c_int), ("rel_residual", C.c_double),
                ("t_arrival", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double)]

    def as_dict(self) -> dict:
        return {"tag": self.tag, "cloth": self.cloth,
                "status": STATUS_NAMES.get(self.status, str(self.status)), "iters": self.iters,
                "rel_residual": self.rel_residual, "t_arrival": self.t_arrival,
                "t_admit": self.t_admit, "t_done": self.t_done}


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong),
                ("chunks", C.c_longlong), ("admitted_waits", C.c_longlong),
                ("max_inflight_seen", C.c_int), ("registered", C.c_int),
                ("resident_bytes", C.c_size_t), ("pool_bytes", C.c_size_t),
                ("pool_peak_bytes", C.c_size_t), ("own_bytes", C.c_size_t),
                ("max_request_bytes", C.c_size_t)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


P = C.c_void_p
PI = C.POINTER(C.c_int)
PF = C.POINTER(C.c_float)
PD = C.POINTER(C.c_double)

# name -> (restype, argtypes); every symbol of include/cloth_gb300.h
SIGNATURES = {
    "cloth_abi_version": (C.c_int, []),
    "cloth_last_error": (C.c_char_p, []),
    "cloth_status_string": (C.c_char_p, [C.c_int]),
    "cloth_ctx_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "cloth_ctx_destroy": (C.c_int, [P]),
    "cloth_ctx_synchronize": (C.c_int, [P]),
    "cloth_ctx_set_profiling": (C.c_int, [P, C.c_int]),
    "cloth_ctx_get_profile": (C.c_int, [P, PD, C.POINTER(C.c_longlong)]),
    "cloth_ctx_reset_profile": (C.c_int, [P]),
    "cloth_ctx_set_solver": (C.c_int, [P, C.c_int]),
    "cloth_ctx_set_tail_hand_off": (C.c_int, [P, C.c_int]),
    "cloth_ctx_set_spin_limit": (C.c_int, [P, C.c_uint, C.c_uint]),
    "cloth_ctx_set_escalation": (C.c_int, [P, C.c_int]),
    "cloth_ctx_device_bytes": (C.c_int, [P, C.POINTER(C.c_size_t)]),
    "cloth_ctx_set_kernel_variant": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int,
                                               C.c_int, C.c_int]),
    "cloth_ctx_get_kernel_variant": (C.c_int, [P, PI, PI, PI, PI, PI, PI]),
    "cloth_ctx_get_tuning_times": (C.c_int, [P, PF, C.c_int, PF, C.c_int]),
    "cloth_ctx_get_stream": (C.c_int, [P, C.POINTER(P)]),
    "cloth_grid_build": (C.c_int, [C.POINTER(GridDesc), PI, PI, PI, PD, PF, PI, PI]),
    "cloth_geometry_build": (C.c_int, [C.POINTER(GridDesc), C.c_char_p, C.c_ulonglong, PI, PI,
                                       PI, PD, PF, PI, PI]),
    "cloth_mesh_from_obj": (C.c_int, [C.c_char_p, PD, C.c_int, PI, PI, PI, PD, PF, PI, PI]),
    "cloth_host_tables": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(Material), PI, PI, PI, PI, PF,
                                    PF, PD, PF, PI]),
    "cloth_create": (C.c_int, [P, C.POINTER(MeshDesc), C.POINTER(Material), C.POINTER(P)]),
    "cloth_destroy": (C.c_int, [P]),
    "cloth_num_vertices": (C.c_int, [P, PI, PI, PI]),
    "cloth_matrix_info": (C.c_int, [P, C.POINTER(C.c_longlong), PI, C.POINTER(C.c_size_t),
                                    C.POINTER(C.c_size_t)]),
    "cloth_set_material": (C.c_int, [P, C.POINTER(Material)]),
    "cloth_find_vertices_from_uv": (C.c_int, [P, PF, C.c_int, PI]),
    "cloth_add_static_vertices": (C.c_int, [P, PI, C.c_int]),
    "cloth_clear_static_vertices": (C.c_int, [P]),
    "cloth_get_static_vertices": (C.c_int, [P, PI, C.c_int, PI]),
    "cloth_set_drag_point": (C.c_int, [P, C.c_int, PF]),
    "cloth_set_pos": (C.c_int, [P, PD, C.c_int]),
    "cloth_set_pre_pos": (C.c_int, [P, PD, C.c_int]),
    "cloth_get_pos": (C.c_int, [P, PD, C.c_int]),
    "cloth_get_pre_pos": (C.c_int, [P, PD, C.c_int]),
    "cloth_reset": (C.c_int, [P]),
    "cloth_step": (C.c_int, [P, C.c_double, C.POINTER(SolveParams), C.POINTER(SolveStats)]),
    "cloth_step_host": (C.c_int, [P, C.c_double, C.POINTER(SolveParams), PD, PD, PD,
                                  C.POINTER(SolveStats)]),
    "cloth_assemble": (C.c_int, [P, C.c_double]),
    "cloth_solve": (C.c_int, [P, C.POINTER(SolveParams), C.POINTER(SolveStats)]),
    "cloth_advance": (C.c_int, [P]),
    "cloth_get_stats": (C.c_int, [P, C.POINTER(SolveStats)]),
    "cloth_get_dx": (C.c_int, [P, PD, C.c_int]),
    "cloth_export_system": (C.c_int, [P, PI, PF, PF, PF, PF]),
    "cloth_export_triangles": (C.c_int, [P, PF, PF]),
    "cloth_export_dihedral": (C.c_int, [P, PI, PI, PF, PF]),
    "cloth_body_create": (C.c_int, [P, C.c_int, C.c_int, PD, PI, C.POINTER(P)]),
    "cloth_body_destroy": (C.c_int, [P]),
    "cloth_body_set_pos": (C.c_int, [P, PD]),
    "cloth_body_set_motion": (C.c_int, [P, PD, PD, PD, PD, PD, C.c_double]),
    "cloth_body_update": (C.c_int, [P, C.c_float]),
    "cloth_body_get_pos": (C.c_int, [P, PD]),
    "cloth_kinematic_pose": (C.c_int, [C.c_int, PD, PD, PD, PD, PD, C.c_double, C.c_float,
                                       PD]),
    "cloth_set_bodies": (C.c_int, [P, C.POINTER(P), C.c_int]),
    "cloth_set_contact_capacity": (C.c_int, [P, C.c_int, C.c_int, C.c_int]),
    "cloth_get_contacts": (C.c_int, [P, C.POINTER(ContactStats), PI, PD, PI, PD]),
    "cloth_get_repulsed_dx": (C.c_int, [P, PD, C.c_int]),
    "cloth_export_tables": (C.c_int, [P, PI, PF, PF, PF, PI]),
    "cloth_step_plain": (C.c_int, [P, C.c_double, C.POINTER(SolveParams), C.POINTER(SolveStats)]),
    "cloth_batch_step": (C.c_int, [P, C.POINTER(P), C.c_int, C.c_double,
                                   C.POINTER(SolveParams), C.POINTER(SolveStats)]),
    "cloth_pcg_solve_ell32_noalloc": (C.c_int, [C.c_int, P, P, P, P, P, C.c_int,
                                                C.POINTER(SolveParams), C.POINTER(SolveStats),
                                                P]),
    "cloth_residual_fp64": (C.c_int, [P, PD]),
    "cloth_solve_refined": (C.c_int, [P, C.POINTER(SolveParams), C.c_double, C.c_int,
                                      C.POINTER(RefineStats)]),
    "cloth_solve_flexible": (C.c_int, [P, C.POINTER(SolveParams), C.c_double, C.c_int,
                                      C.POINTER(RefineStats)]),
    "cloth_solve_fp64": (C.c_int, [P, C.POINTER(SolveParams), C.POINTER(SolveStats)]),
    "cloth_server_now": (C.c_double, []),
    "cloth_server_create": (C.c_int, [P, C.POINTER(ServerConfig), C.POINTER(P)]),
    "cloth_server_add": (C.c_int, [P, P, C.c_double, C.POINTER(SolveParams), PI]),
    "cloth_server_start": (C.c_int, [P]),
    "cloth_server_submit": (C.c_int, [P, C.c_int, C.c_longlong, C.c_double]),
    "cloth_server_poll": (C.c_int, [P, C.POINTER(ServerResult), C.c_int, PI, C.c_double]),
    "cloth_server_drain": (C.c_int, [P, C.c_double]),
    "cloth_server_get_stats": (C.c_int, [P, C.POINTER(ServerStats)]),
    "cloth_server_destroy": (C.c_int, [P]),
}


class ClothError(RuntimeError):
    def __init__(self, func: str, code: int, msg: str):
        super().__init__(f"{func} -> {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load() -> C.CDLL:
    """Load the native library (once). Raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run `python -m acousticsim_gb300.build`")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(func: str, code: int) -> None:
    if code != CLOTH_OK:
        msg = load().cloth_last_error().decode(errors="replace")
        raise ClothError(func, code, msg)


def call(name: str, *args) -> None:
    check(name, getattr(load(), name)(*args))


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def params(max_iters=1000, rel_tol=1e-6, abs_tol=0.0, check_every=1, warm_start=1) -> SolveParams:
    return SolveParams(int(max_iters), float(rel_tol), float(abs_tol), int(check_every),
                       int(warm_start))


# Solver settings of the reference's PCGSolver::Solve (PCGSolver.cu:346, 444-475):
# at most 100 iterations, absolute ||r|| < 1e-10 tested every 10th iteration.
REFERENCE_PARAMS = dict(max_iters=100, rel_tol=0.0, abs_tol=1e-10, check_every=10, warm_start=1)
