"""Generates the golden fixtures of tests/golden/*.npz from the reference itself.

    python tests/golden/make_golden.py [--ref /root/reference]

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


def read_dump(d: Path) -> dict:
    out = {}
    for line in (d / "manifest.txt").read_text().splitlines():
        parts = line.split()
        name, dt, shape = parts[0], parts[1], tuple(int(s) for s in parts[2:])
        out[name] = np.fromfile(d / f"{name}.bin", dtype=np.dtype(dt)).reshape(shape)
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    a = ap.parse_args()
    subprocess.run(["make", "-C", str(ROOT / "oracle"), f"REF={a.ref}", "-j8"], check=True,
                   stdout=subprocess.DEVNULL)
    harness = ROOT / "oracle" / "_ref" / "ref_harness"
    for name, over, seed, sx, sv in CASES:
        conf = dict(BASE, **over)
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            (td / "cfg.json").write_text(json.dumps(conf))
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


if __name__ == "__main__":
    sys.exit(main())
