"""Generates the golden fixtures of tests/golden/*.npz from the reference itself.

    python tests/golden/make_golden.py [--ref <reference source tree>]

Builds the reference's CPU cloth code with oracle/Makefile (outputs only into
oracle/_ref/), runs oracle/_ref/ref_harness on seeded inputs and stores what it
writes.  Needs the reference sources, so it runs where they are mounted; the
fixtures it writes are committed and are all the tests need elsewhere.
"""
from __future__ import annotations

import argparse
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent

BASE = {
    "object_name": "cloth", "object_type": "Cloth", "cloth_type": "fem",
    "geometry_type": "regular_triangle", "damping": 0.0, "max_iters": 100,
    "enable_gravity": True, "enable_cloth_from_obj": False,
    "cloth_init_orientation": [0, 0, 0, 0],
}

# (name, config overrides, seed, position noise, velocity noise)
CASES = [
    # The small CPU configuration: 20x20 grid, 1 m x 1 m, density 0.1,
    # stretch 1e3 / shear 1e2, bending 1e-3, damping 0.01, top corners pinned,
    # dt 5 ms, x += N(0, 1e-3), v = N(0, 0.01).
    ("grid20", {"cloth_size": [1.0, 1.0], "subdivision": [19, 19],
                "cloth_init_pos": [0.0, 0.0, 0.0], "cloth_uv_rotation": 0,
                "cloth_stretch_stiffness": [1e3, 1e3, 1e2],
                "cloth_bending_stiffness": [1e-3, 1e-3], "cloth_density": 0.1,
                "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0,
                "default_timestep": 5e-3,
                "constraints": {"static_point": [[-0.5, 0.5], [0.5, 0.5]]}},
     1, 1e-3, 1e-2),
    # Non-square grid, translated, 45-degree material frame, anisotropic
    # stretch and bending, both Rayleigh terms, three pins.
    ("rect_rot45", {"cloth_size": [0.8, 1.2], "subdivision": [7, 11],
                    "cloth_init_pos": [0.1, 0.5, -0.2], "cloth_uv_rotation": 45,
                    "cloth_stretch_stiffness": [2e3, 5e2, 1.5e2],
                    "cloth_bending_stiffness": [2e-3, 5e-4], "cloth_density": 0.2,
                    "rayleigh_damping_a": 0.02, "rayleigh_damping_b": -0.01,
                    "default_timestep": 4e-3,
                    "constraints": {"static_point": [[-0.5, 0.5], [0.5, 0.5], [0.0, 0.6]]}},
     2, 2e-3, 5e-2),
    # Tiny grid, 90-degree material frame, no pins, large strains.
    ("small_rot90", {"cloth_size": [0.5, 0.4], "subdivision": [4, 3],
                     "cloth_init_pos": [0.0, 0.0, 0.0], "cloth_uv_rotation": 90,
                     "cloth_stretch_stiffness": [1e2, 3e2, 5e1],
                     "cloth_bending_stiffness": [1e-2, 1e-2], "cloth_density": 0.5,
                     "rayleigh_damping_a": 0.0, "rayleigh_damping_b": 0.0,
                     "default_timestep": 1e-2},
     3, 2e-2, 1e-1),
]


# OBJ cloths ("enable_cloth_from_obj"): (name, OBJ file under tests/golden,
# config overrides, seed, position noise, velocity noise).  The OBJ is written
# by irregular_obj() below; the config names it relative to tests/golden.
OBJ_CASES = [
    # 8 x 10 jittered lattice in the XY plane: per cell a quad (split by the
    # loader), two triangles with either diagonal, or a fan around an added
    # centre vertex; vertices numbered in shuffled order; two top pins.
    ("obj_irregular", "irregular.obj",
     {"cloth_obj_size": [0.8, 1.0], "cloth_obj_translation": [0.05, -0.1, 0.02],
      "enable_relocate_obj": False,
      "cloth_stretch_stiffness": [1e3, 8e2, 1e2], "cloth_bending_stiffness": [2e-3, 2e-3],
      "cloth_density": 0.15, "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0,
      "default_timestep": 4e-3,
      "constraints": {"static_point": [[-0.4, 0.5], [0.4, 0.5]]}},
     4, 1e-3, 1e-2),
    # the same file relocated (MoveObjPos: top at y = 0.27, centred in x, z)
    ("obj_relocated", "irregular.obj",
     {"cloth_obj_size": [0.8, 1.0], "cloth_obj_translation": [0.3, 0.1, -0.2],
      "enable_relocate_obj": True,
      "cloth_stretch_stiffness": [1e3, 1e3, 1e2], "cloth_bending_stiffness": [1e-3, 1e-3],
      "cloth_density": 0.1, "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0,
      "default_timestep": 2e-3,
      "constraints": {"static_point": [[-0.4, 0.5], [0.4, 0.5]]}},
     5, 1e-3, 1e-2),
]


def irregular_obj(path: Path, seed: int = 17, nx: int = 8, ny: int = 10) -> None:
    """A seeded irregular cloth mesh (triangles and quads) as an OBJ file."""
    rng = np.random.default_rng(seed)
    w, h = 0.8, 1.0
    pts = []
    for j in range(ny + 1):
        for i in range(nx + 1):
            x = -w / 2 + w * i / nx
            y = -h / 2 + h * j / ny
            if 0 < i < nx and 0 < j < ny:
                x += rng.uniform(-0.2, 0.2) * w / nx
                y += rng.uniform(-0.2, 0.2) * h / ny
            pts.append((x, y))
    idx = lambda i, j: j * (nx + 1) + i
    faces = []
    for j in range(ny):
        for i in range(nx):
            a, b, c, d = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
            kind = rng.integers(0, 4)
            if kind == 0:
                faces.append((a, b, c, d))
            elif kind == 1:
                faces += [(a, b, c), (a, c, d)]
            elif kind == 2:
                faces += [(a, b, d), (b, c, d)]
            else:
                cx = np.mean([pts[k][0] for k in (a, b, c, d)])
                cy = np.mean([pts[k][1] for k in (a, b, c, d)])
                pts.append((cx, cy))
                m = len(pts) - 1
                faces += [(a, b, m), (b, c, m), (c, d, m), (d, a, m)]
    n = len(pts)
    perm = rng.permutation(n)          # OBJ number of lattice point k
    inv = np.argsort(perm)
    vt_perm = rng.permutation(n)       # texture coordinate slot of OBJ vertex q
    with open(path, "w") as f:
        f.write("# seeded irregular cloth (tests/golden/make_golden.py)\n")
        for q in range(n):
            x, y = pts[inv[q]]
            f.write(f"v {x:.6f} {y:.6f} 0.000000\n")
        vt_of = np.empty(n, np.int64)
        for slot in range(n):
            q = int(np.flatnonzero(vt_perm == slot)[0])
            x, y = pts[inv[q]]
            f.write(f"vt {0.3 * x:.6f} {0.3 * y:.6f}\n")
            vt_of[q] = slot
        for fc in faces:
            f.write("f " + " ".join(f"{perm[k] + 1}/{vt_of[perm[k]] + 1}" for k in fc) + "\n")


# Collisions of the CPU cloth with one kinematic body (cBVHCollisionDetecter,
# cBaraffCloth::PrepareCollisionHessian and Repulsion) on the grid20 state:
# (name, cloth case whose config and state are used, kinematic body config).
# "patch.obj" is written by contact_patch() below.
COLLIDE_CASES = [
    # a gently curved patch 1.5 mm in front of the cloth, normals towards it:
    # cloth points near its triangles, its points near cloth triangles, and
    # edge pairs all come within the 3 mm contact distance
    ("col_patch", "grid20",
     {"object_name": "patch", "object_type": "KinematicBody", "type": "custom",
      "mesh_path": "patch.obj", "target_aabb": [0, 0, 0, 0], "scale": [1, 1, 1, 0],
      "translation": [0, 0, 0, 0], "orientation": [0, 0, 0, 0]}),
    # the reference's plane body (2 m square, two triangles) 1.5 mm in front
    ("col_plane", "grid20",
     {"object_name": "plane", "object_type": "KinematicBody", "type": "plane",
      "equation": [0, 0, 1, -0.0015], "plane_scale": 1.0}),
]


# A moving kinematic body (cKinematicBody with "is_static": false): the
# curved patch, posed by translation and XYZ Euler angles interpolated from
# init to target over elasped_time_sec, stepped by Update(dt) past that time
# (name, body config, dt, updates).
MOTION_CASES = [
    ("body_motion",
     {"object_name": "patch", "object_type": "KinematicBody", "type": "custom",
      "mesh_path": "patch.obj", "target_aabb": [0, 0, 0, 0], "scale": [1, 1, 1, 0],
      "translation": [0.02, -0.01, 0.005, 0], "orientation": [0.1, 0.2, -0.05, 0],
      "is_static": False, "target_translation": [-0.03, 0.04, 0.02, 0],
      "target_orientation": [0.25, -0.15, 0.3, 0], "elasped_time_sec": 0.02},
     0.003, 10),
]


# The geometry generators that draw from the reference's global generator,
# right after cMathUtil::SeedRand(seed): (case, config, seed), all written to
# geometry.npz.
GEOM_CASES = [
    ("perturb_13x17", {"geometry_type": "regular_triangle_perturb", "cloth_size": [1.2, 0.9],
                       "subdivision": [13, 17], "cloth_init_pos": [0.1, 0.2, 0.3],
                       "cloth_init_orientation": [0, 0, 0], "cloth_uv_rotation": 45}, 0),
    ("perturb_20x20", {"geometry_type": "regular_triangle_perturb", "cloth_size": [1.0, 1.0],
                       "subdivision": [19, 19], "cloth_init_pos": [0, 0, 0],
                       "cloth_init_orientation": [0, 0, 0], "cloth_uv_rotation": 0}, 7),
    ("delaunay_25x31", {"geometry_type": "delaunay", "cloth_size": [0.7, 1.3],
                        "subdivision": [25, 31], "cloth_init_pos": [0.1, -0.2, 0.05],
                        "cloth_init_orientation": [0, 0, 0], "cloth_uv_rotation": 90}, 3),
    ("delaunay_20x20", {"geometry_type": "delaunay", "cloth_size": [1.0, 1.0],
                        "subdivision": [20, 20], "cloth_init_pos": [0, 0, 0],
                        "cloth_init_orientation": [0, 0, 0], "cloth_uv_rotation": 0}, 0),
]


def contact_patch(path: Path, n: int = 12) -> None:
    """A curved n x n patch over x, y in [-0.35, 0.3] x [-0.25, 0.35] at
    z = 1.5 mm + 0.04 r^2, triangle normals facing -z."""
    xs = np.linspace(-0.35, 0.3, n + 1)
    ys = np.linspace(-0.25, 0.35, n + 1)
    with open(path, "w") as f:
        f.write("# curved contact patch (tests/golden/make_golden.py)\n")
        for y in ys:
            for x in xs:
                z = 0.0015 + 0.04 * ((x + 0.02) ** 2 + (y - 0.05) ** 2)
                f.write(f"v {x:.6f} {y:.6f} {z:.6f}\n")
        idx = lambda i, j: j * (n + 1) + i + 1
        for j in range(n):
            for i in range(n):
                a, b, c, d = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
                # (v1 - v0) x (v2 - v1) along -z
                f.write(f"f {a} {c} {b}\nf {a} {d} {c}\n")


def read_dump(d: Path) -> dict:
    out = {}
    for line in (d / "manifest.txt").read_text().splitlines():
        parts = line.split()
        name, dt, shape = parts[0], parts[1], tuple(int(s) for s in parts[2:])
        out[name] = np.fromfile(d / f"{name}.bin", dtype=np.dtype(dt)).reshape(shape)
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None,
                    help="reference source tree (default: $ACOUSTICSIM_REF, else the "
                         "Makefile's REF)")
    ap.add_argument("--only", nargs="*", default=None, help="case names to regenerate")
    a = ap.parse_args()
    ref_arg = [f"REF={a.ref}"] if a.ref else []
    subprocess.run(["make", "-C", str(ROOT / "oracle"), *ref_arg, "-j8"], check=True,
                   stdout=subprocess.DEVNULL)
    harness = ROOT / "oracle" / "_ref" / "ref_harness"
    cases = [(name, over, seed, sx, sv, None) for name, over, seed, sx, sv in CASES]
    for name, obj, over, seed, sx, sv in OBJ_CASES:
        irregular_obj(OUT / obj)
        o = dict(over, enable_cloth_from_obj=True, cloth_obj_path=obj)
        cases.append((name, o, seed, sx, sv, obj))
    for name, over, seed, sx, sv, obj in cases:
        if a.only and name not in a.only:
            continue
        conf = dict(BASE, **over)
        run_conf = dict(conf)
        if obj is not None:
            run_conf["cloth_obj_path"] = str(OUT / obj)
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            (td / "cfg.json").write_text(json.dumps(run_conf))
            (td / "topo").mkdir()
            subprocess.run([str(harness), "topo", str(td / "cfg.json"), str(td / "topo")],
                           check=True, stdout=subprocess.DEVNULL)
            topo = read_dump(td / "topo")
            rng = np.random.default_rng(seed)
            pos = topo["pos"]
            x = pos + rng.normal(0.0, sx, pos.shape)
            v = rng.normal(0.0, sv, pos.shape)
            xpre = x - conf["default_timestep"] * v
            x.astype(np.float64).tofile(td / "x.bin")
            xpre.astype(np.float64).tofile(td / "xpre.bin")
            (td / "sys").mkdir()
            subprocess.run([str(harness), "system", str(td / "cfg.json"), str(td / "x.bin"),
                            str(td / "xpre.bin"), str(td / "sys")], check=True,
                           stdout=subprocess.DEVNULL)
            sysd = read_dump(td / "sys")
        arrays = {f"topo_{k}": v for k, v in topo.items()}
        arrays.update({f"sys_{k}": v for k, v in sysd.items()})
        arrays["x_in"] = x
        arrays["xpre_in"] = xpre
        arrays["config_json"] = np.frombuffer(json.dumps(conf).encode(), np.uint8)
        np.savez_compressed(OUT / f"{name}.npz", **arrays)
        print(name, "nv", pos.shape[0], "->", OUT / f"{name}.npz")
    for name, cloth_case, kb in COLLIDE_CASES:
        if a.only and name not in a.only:
            continue
        g = np.load(OUT / f"{cloth_case}.npz")
        conf = json.loads(bytes(g["config_json"]).decode())
        run_kb = dict(kb)
        if kb.get("type") == "custom":
            contact_patch(OUT / kb["mesh_path"])
            run_kb["mesh_path"] = str(OUT / kb["mesh_path"])
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            (td / "cfg.json").write_text(json.dumps(conf))
            (td / "kb.json").write_text(json.dumps(run_kb))
            g["x_in"].astype(np.float64).tofile(td / "x.bin")
            g["sys_dx"].astype(np.float64).tofile(td / "dx.bin")
            (td / "col").mkdir()
            subprocess.run([str(harness), "collide", str(td / "cfg.json"), str(td / "kb.json"),
                            str(td / "x.bin"), str(td / "dx.bin"), str(td / "col")],
                           check=True, stdout=subprocess.DEVNULL)
            cold = read_dump(td / "col")
        arrays = {f"col_{k}": v for k, v in cold.items()}
        arrays["config_json"] = np.frombuffer(json.dumps(conf).encode(), np.uint8)
        arrays["body_json"] = np.frombuffer(json.dumps(kb).encode(), np.uint8)
        np.savez_compressed(OUT / f"{name}.npz", **arrays)
        print(name, "contacts pt", cold["pt_i"].shape[0], "ee", cold["ee_i"].shape[0], "->",
              OUT / f"{name}.npz")
    geom = {}
    for name, conf, seed in GEOM_CASES:
        if a.only and name not in a.only and "geometry" not in a.only:
            continue
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            (td / "cfg.json").write_text(json.dumps(conf))
            (td / "g").mkdir()
            subprocess.run([str(harness), "geom", str(td / "cfg.json"), str(seed), str(td / "g")],
                           check=True, stdout=subprocess.DEVNULL)
            gd = read_dump(td / "g")
        for k, v in gd.items():
            geom[f"{name}_{k}"] = v
        geom[f"{name}_config_json"] = np.frombuffer(json.dumps(conf).encode(), np.uint8)
        geom[f"{name}_seed"] = np.array(seed, np.int64)
        print(name, "nv", gd["pos"].shape[0], "nt", gd["tris"].shape[0])
    if geom:
        np.savez_compressed(OUT / "geometry.npz", **geom)
        print("->", OUT / "geometry.npz")
    for name, kb, dt, steps in MOTION_CASES:
        if a.only and name not in a.only:
            continue
        g = np.load(OUT / "grid20.npz")
        conf = json.loads(bytes(g["config_json"]).decode())
        run_kb = dict(kb)
        contact_patch(OUT / kb["mesh_path"])
        run_kb["mesh_path"] = str(OUT / kb["mesh_path"])
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            (td / "cfg.json").write_text(json.dumps(conf))
            (td / "kb.json").write_text(json.dumps(run_kb))
            (td / "mo").mkdir()
            subprocess.run([str(harness), "motion", str(td / "cfg.json"), str(td / "kb.json"),
                            repr(dt), str(steps), str(td / "mo")], check=True,
                           stdout=subprocess.DEVNULL)
            mo = read_dump(td / "mo")
        arrays = {f"mo_{k}": v for k, v in mo.items()}
        arrays["body_json"] = np.frombuffer(json.dumps(kb).encode(), np.uint8)
        arrays["dt"] = np.array(dt, np.float32)
        np.savez_compressed(OUT / f"{name}.npz", **arrays)
        print(name, "vertices", mo["local"].shape[0], "updates", steps, "->",
              OUT / f"{name}.npz")


if __name__ == "__main__":
    sys.exit(main())
