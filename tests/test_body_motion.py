"""A moving kinematic body's pose against the reference's own cKinematicBody.

tests/golden/body_motion.npz was written by oracle/ref_harness ("motion"
mode): the reference body built from its JSON ("is_static": false, target
translation and orientation, elasped_time_sec), its scaled local mesh, and its
vertex positions at Init and after each of ten Update(dt) calls (past the
motion's end, where the pose is held), with its normals, which Update leaves
as Init computed them.  The library's host pose (cloth_kinematic_pose, the
same function cloth_body_update uses on a device body) must reproduce every
position bit for bit.  Host only: no GPU."""
from __future__ import annotations

import json

import numpy as np

from conftest import GOLDEN


def test_kinematic_pose_matches_reference_body(built):
    from acousticsim_gb300 import kinematic_pose
    g = np.load(GOLDEN / "body_motion.npz")
    kb = json.loads(bytes(g["body_json"]).decode())
    dt = np.float32(g["dt"])
    local = g["mo_local"]
    t = np.float32(0.0)
    for k in range(g["mo_pos"].shape[0]):
        assert np.float32(g["mo_time"][k]) == t  # the body clock, a float
        w = kinematic_pose(local, kb["translation"], kb["orientation"], kb["target_translation"],
                           kb["target_orientation"], kb["elasped_time_sec"], float(t))
        assert np.array_equal(w, g["mo_pos"][k]), (k, np.abs(w - g["mo_pos"][k]).max())
        t = np.float32(t + dt)
    # held at the target once the body time passes elasped_time_sec
    assert np.array_equal(g["mo_pos"][-1], g["mo_pos"][-2])
    assert np.array_equal(g["mo_vnormal_init"], g["mo_vnormal_end"])
