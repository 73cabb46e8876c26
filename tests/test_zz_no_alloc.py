"""The allocation-free solve (cloth_pcg_solve_ell32_noalloc) against the
library's regular solve (cloth_assemble + cloth_solve) on the same systems.

Callers that cannot allocate device memory at solve time (a frame loop that
must not stall on cudaMalloc or fail for lack of memory mid-frame, or a host
whose device memory belongs to another allocator) hand this entry point an
assembled system in the reference's ELL32 layout; its scratch is a static
device array.  Two calls in a row are checked, each on its own system, so
contents the first call leaves in the shared array cannot leak into the
second.  Collected last on purpose (file name) so a stop-at-first-failure run
has already run every other test."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

# both solves stop at 1e-6 relative residual; their solutions agree to a few
# 1e-6 relative (the solve tests' dx bound)
TOL_DX = 2e-4


def _conf(n):
    return {"geometry_type": "regular_triangle", "cloth_size": [1.0, 1.0],
            "subdivision": [n - 1, n - 1], "cloth_init_pos": [0.0, 0.0, 0.0],
            "cloth_uv_rotation": 0, "cloth_stretch_stiffness": [1e3, 1e3, 1e2],
            "cloth_bending_stiffness": [1e-3, 1e-3], "cloth_density": 0.1,
            "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0, "default_timestep": 2e-3,
            "constraints": {"static_point": [[-0.5, 0.5], [0.5, 0.5]]}}


def _noalloc_solve(sysd, pins, p):
    import torch
    from acousticsim_gb300 import _native as N
    dev = torch.device("cuda", 0)
    # the reference's blocks are column-major: transpose the exported row-major ones
    A = np.ascontiguousarray(np.swapaxes(sysd["A"], 2, 3), np.float32)
    ell = torch.from_numpy(np.ascontiguousarray(sysd["ell"], np.int32)).to(dev)
    A_d = torch.from_numpy(A).to(dev)
    b_d = torch.from_numpy(np.ascontiguousarray(sysd["b"], np.float32)).to(dev)
    x_d = torch.zeros(sysd["b"].shape, dtype=torch.float32, device=dev)
    fixed = torch.tensor(list(pins), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = N.SolveStats()
    N.call("cloth_pcg_solve_ell32_noalloc", int(sysd["b"].shape[0]), ell.data_ptr(),
           A_d.data_ptr(), b_d.data_ptr(), x_d.data_ptr(), fixed.data_ptr(), len(pins),
           C.byref(p), C.byref(st), C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    return x_d.cpu().numpy().astype(np.float64).reshape(-1), st.as_dict()


def test_noalloc_matches_regular_solve_twice(built):
    from acousticsim_gb300 import BaraffClothGpu, ClothContext, params
    from oracle import oracle as orc

    p = params(max_iters=20000, rel_tol=1e-6, warm_start=0)
    ctx = ClothContext(0)
    cloth = BaraffClothGpu(ctx, _conf(64))
    rng = np.random.default_rng(5)
    x0 = cloth.GetInitPos().reshape(-1, 3)
    x = x0 + rng.normal(0, 1e-3, x0.shape)
    xp = x - 2e-3 * rng.normal(0, 1e-2, x0.shape)
    cloth.SetPos(x.reshape(-1))
    cloth.SetPrePos(xp.reshape(-1))
    pins = cloth.GetConstraintStaticVertices()
    for call in range(2):
        # the regular path: assemble, then the library's own solve from zero
        cloth.assemble()
        sysd = cloth.export_system()
        dx_regular = np.zeros(cloth.nv * 3)
        st_ref = cloth.solve(p)
        assert st_ref["status"] == "OK", st_ref
        dx_regular = cloth.get_dx()
        dx_noalloc, st = _noalloc_solve(sysd, pins, p)
        assert st["status"] == "OK", (call, st)
        assert st["rel_residual"] <= 1e-6
        err = rel(dx_noalloc, dx_regular)
        # true residual of both on the FP64 copy of the exported system
        A64 = sysd["A"].astype(np.float64)
        b64 = sysd["b"].astype(np.float64).reshape(-1)
        for dx in (dx_noalloc, dx_regular):
            r = b64 - orc.spmv(sysd["ell"], A64, dx)
            assert np.linalg.norm(r) / np.linalg.norm(b64) < 5e-6
        print(f"call {call}: iters {st['iters']} vs {st_ref['iters']}, dx difference {err:.2e}")
        assert err < TOL_DX, (call, err)
        assert np.all(dx_noalloc.reshape(-1, 3)[pins] == 0.0)
        # next call: a different system (one step later)
        cloth.advance()
    cloth.close()
    ctx.close()


def test_noalloc_rejects_oversized_systems(built):
    import torch
    from acousticsim_gb300 import _native as N
    dev = torch.device("cuda", 0)
    big = 32768 + 1
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    rc = N.load().cloth_pcg_solve_ell32_noalloc(big, buf.data_ptr(), buf.data_ptr(),
                                                buf.data_ptr(), buf.data_ptr(), None, 0,
                                                None, None, None)
    assert rc == 1  # CLOTH_ERR_INVALID, nothing launched
    assert b"exceed" in N.load().cloth_last_error()


def _small_system(n=16):
    from acousticsim_gb300 import BaraffClothGpu, ClothContext
    ctx = ClothContext(0)
    cloth = BaraffClothGpu(ctx, _conf(n))
    cloth.assemble()
    sysd = cloth.export_system()
    pins = cloth.GetConstraintStaticVertices()
    cloth.close()
    ctx.close()
    return sysd, pins


def test_noalloc_rejects_column_ids_outside_the_system(built):
    """A caller-built ELL map with a column id >= nv is reported as
    CLOTH_ERR_INVALID; the id is caught before anything is read through it."""
    import torch
    from acousticsim_gb300 import _native as N, params
    sysd, pins = _small_system()
    nv = sysd["b"].shape[0]
    ell = np.array(sysd["ell"], np.int32, copy=True)
    row = nv // 2
    ell[row, 1] = nv + 5  # a column past the last vertex
    dev = torch.device("cuda", 0)
    A = np.ascontiguousarray(np.swapaxes(sysd["A"], 2, 3), np.float32)
    ell_d = torch.from_numpy(ell).to(dev)
    A_d = torch.from_numpy(A).to(dev)
    b_d = torch.from_numpy(np.ascontiguousarray(sysd["b"], np.float32)).to(dev)
    x_d = torch.zeros(sysd["b"].shape, dtype=torch.float32, device=dev)
    st = N.SolveStats()
    p = params(max_iters=500, rel_tol=1e-6, warm_start=0)
    rc = N.load().cloth_pcg_solve_ell32_noalloc(nv, ell_d.data_ptr(), A_d.data_ptr(),
                                                b_d.data_ptr(), x_d.data_ptr(), None, 0,
                                                C.byref(p), C.byref(st), None)
    torch.cuda.synchronize(dev)
    assert rc == 1, rc  # CLOTH_ERR_INVALID
    assert st.status == 1 and st.iters == 0
    assert b"column" in N.load().cloth_last_error()
    # the same call with the map restored solves normally
    ell_d.copy_(torch.from_numpy(np.ascontiguousarray(sysd["ell"], np.int32)).to(dev))
    x_d.zero_()
    rc = N.load().cloth_pcg_solve_ell32_noalloc(nv, ell_d.data_ptr(), A_d.data_ptr(),
                                                b_d.data_ptr(), x_d.data_ptr(), None, 0,
                                                C.byref(p), C.byref(st), None)
    torch.cuda.synchronize(dev)
    assert rc == 0 and st.status == 0, (rc, st.status)


def test_noalloc_refuses_a_capturing_stream(built):
    """The call reads the solver state on the host, so under stream capture it
    returns CLOTH_ERR_STATE and leaves the capture intact."""
    import torch
    from acousticsim_gb300 import _native as N
    dev = torch.device("cuda", 0)
    sysd, _ = _small_system()
    nv = sysd["b"].shape[0]
    buf = torch.zeros(nv * 32 * 9, dtype=torch.float32, device=dev)
    ell_d = torch.from_numpy(np.ascontiguousarray(sysd["ell"], np.int32)).to(dev)
    side = torch.cuda.Stream(dev)
    y = torch.zeros(4, device=dev)
    g = torch.cuda.CUDAGraph()
    rcs = []
    with torch.cuda.graph(g, stream=side):
        y.add_(1.0)
        rcs.append(N.load().cloth_pcg_solve_ell32_noalloc(
            nv, ell_d.data_ptr(), buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), None, 0,
            None, None, C.c_void_p(side.cuda_stream)))
    g.replay()
    torch.cuda.synchronize(dev)
    assert rcs == [11], rcs  # CLOTH_ERR_STATE
    assert float(y[0]) == 1.0  # the captured work is intact
