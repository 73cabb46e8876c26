"""Finite-difference checks of the stretch/shear forces and Hessian blocks
(cBaraffMaterial::CalcFint / CalcHessian, restated by the oracle, which is
pinned to the reference's own arrays by tests/test_oracle_golden.py).  The
reference's own check (cBaraffCloth::CheckForce, BaraffCloth.cpp:399-426)
does not run: its CalcEnergy sums the total energy once per triangle.

The reference's Hessian is the Jacobian of its force at rest and under
isotropic stretch, and a symmetric approximation of it otherwise: the tests
pin both."""
from __future__ import annotations

import numpy as np
import pytest


@pytest.fixture(scope="module")
def orc(built):
    from oracle import oracle
    return oracle


def _blocks(h_t):
    H = np.zeros((9, 9))
    for a in range(3):
        for b in range(3):
            H[3 * a:3 * a + 3, 3 * b:3 * b + 3] = h_t[3 * a + b]
    return H


def _fd_jacobian(orc, mesh, tab, x0, ks, t, eps=1e-6):
    tri = mesh["tris"][t]
    J = np.zeros((9, 9))
    for b in range(3):
        for d in range(3):
            xp, xm = x0.copy(), x0.copy()
            xp[3 * tri[b] + d] += eps
            xm[3 * tri[b] + d] -= eps
            fp, _ = orc.triangles(mesh, tab, xp, ks)
            fm, _ = orc.triangles(mesh, tab, xm, ks)
            J[:, 3 * b + d] = ((fp[t] - fm[t]) / (2 * eps)).reshape(-1)
    return J


@pytest.mark.parametrize("scale", [(1.0, 1.0), (1.05, 1.05), (1.2, 1.2)])
def test_hessian_is_force_jacobian_under_isotropic_stretch(orc, scale):
    """At rest and under isotropic stretch the Hessian blocks are the Jacobian
    of the force (measured: 8e-8 relative, the finite-difference error); under
    anisotropic stretch or compression they are not (5-14 %)."""
    mesh = orc.grid((1.0, 1.0), (3, 3))
    tab = orc.tables(mesh, 0.1, [1e-3, 1e-3, 1e-3])
    x0 = mesh["pos"].copy()
    x0[:, 0] *= scale[0]
    x0[:, 1] *= scale[1]
    x0 = x0.reshape(-1)
    ks = [1e3, 1e3, 1e2]
    _, h = orc.triangles(mesh, tab, x0, ks)
    for t in range(len(mesh["tris"])):
        H = _blocks(h[t])
        J = _fd_jacobian(orc, mesh, tab, x0, ks, t)
        assert np.linalg.norm(J - H) <= 1e-6 * np.linalg.norm(H), t


def test_hessian_is_symmetric_and_approximate_elsewhere(orc):
    mesh = orc.grid((1.0, 1.0), (3, 3))
    tab = orc.tables(mesh, 0.1, [1e-3, 1e-3, 1e-3])
    rng = np.random.default_rng(3)
    x0 = (mesh["pos"] + rng.normal(0.0, 0.01, mesh["pos"].shape)).reshape(-1)
    ks = [1e3, 1e3, 1e2]
    _, h = orc.triangles(mesh, tab, x0, ks)
    worst = 0.0
    for t in range(len(mesh["tris"])):
        H = _blocks(h[t])
        assert np.array_equal(H, H.T), t
        J = _fd_jacobian(orc, mesh, tab, x0, ks, t)
        worst = max(worst, np.linalg.norm(J - H) / np.linalg.norm(H))
    # the dropped terms show under shear and rotation (measured 0.12 here)
    assert 1e-4 < worst < 0.5


def test_bending_matrix_properties(orc):
    """The Q-bending force is -K x with the constant matrix the tables hold
    (cQBendingMaterial): K is symmetric, positive semidefinite and has the
    rigid translations in its null space (the cotangent weights of each edge
    stencil sum to zero)."""
    mesh = orc.grid((1.0, 1.0), (4, 4))
    tab = orc.tables(mesh, 0.1, [1e-3, 2e-3, 1e-3])
    ell, kb = tab["ell"], tab["kbend"]
    n = mesh["pos"].shape[0]
    K = np.zeros((n, n))
    for i in range(n):
        for s in range(ell.shape[1]):
            if ell[i, s] >= 0:
                K[i, ell[i, s]] += kb[i, s]
    scale = np.abs(K).max()
    assert scale > 0
    assert np.allclose(K, K.T, rtol=0, atol=1e-12 * scale)
    assert np.abs(K @ np.ones(n)).max() <= 1e-9 * scale
    assert np.linalg.eigvalsh(K).min() >= -1e-9 * scale
