"""Shared fixtures.  `-m gpu` tests need a CUDA GPU; everything else runs on CPU."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"
GOLDEN_CASES = ["grid20", "rect_rot45", "small_rot90", "obj_irregular", "obj_relocated"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def load_golden(name: str):
    g = np.load(GOLDEN / f"{name}.npz")
    conf = json.loads(bytes(g["config_json"]).decode())
    if conf.get("enable_cloth_from_obj"):
        conf["cloth_obj_path"] = str(GOLDEN / conf["cloth_obj_path"])
    return g, conf


def golden_mesh(conf: dict) -> dict:
    """The case's mesh from the library's host code: the OBJ loader for
    "enable_cloth_from_obj" cases, else the regular-grid generator."""
    from acousticsim_gb300 import build_grid, load_obj_mesh
    if conf.get("enable_cloth_from_obj"):
        return load_obj_mesh(conf["cloth_obj_path"], conf.get("cloth_obj_translation", [0, 0, 0]),
                             conf.get("enable_relocate_obj", False))
    return build_grid(tuple(conf["cloth_size"]), tuple(conf["subdivision"]),
                      tuple(conf["cloth_init_pos"]), conf["cloth_uv_rotation"])


def rel(a, ref) -> float:
    """Relative error of a whole array: ||a - ref|| / ||ref||."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(a - ref) / (den if den > 0 else 1.0))


def project_pins(A, b, ell, pins):
    """Pin projection of the GPU solver (PCGSolver.cu:126-136, 185-222):
    off-diagonal blocks of pinned rows and columns zeroed, b = 0 on pinned rows."""
    A = np.array(A, copy=True)
    b = np.array(b, copy=True)
    fixed = np.zeros(ell.shape[0], bool)
    fixed[np.asarray(pins, np.int64)] = True
    for v in range(ell.shape[0]):
        for s in range(ell.shape[1]):
            c = ell[v, s]
            if c < 0:
                break
            if c != v and (fixed[v] or fixed[c]):
                A[v, s] = 0
    b[fixed] = 0
    return A, b


@pytest.fixture(scope="session")
def built():
    from acousticsim_gb300 import build
    build.build_all()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    from acousticsim_gb300 import ClothContext
    c = ClothContext(0)
    yield c
    c.close()
