"""Request server (cloth_server_*): continuous batching of single-step
requests over resident cloths.

The invariance test is the serving contract: each request's result is the
same alone and in the mix.  Every served cloth has a twin with the same
configuration and initial state that is stepped alone (cloth_step, graph-loop
solver) the same number of times; positions, previous positions and the
per-step PCG iteration counts must agree bit for bit, whatever else shared the
server's chunks, the chunk length and the memory budget."""
from __future__ import annotations

import time

import numpy as np
import pytest

REL_TOL = 1e-6


def _conf(n, k, dt=2e-3):
    return {"geometry_type": "regular_triangle", "cloth_size": [1.0, 1.0],
            "subdivision": [n - 1, n - 1], "cloth_init_pos": [0.0, 0.0, 0.0],
            "cloth_uv_rotation": 0, "cloth_stretch_stiffness": [k, k, k / 10],
            "cloth_bending_stiffness": [1e-3, 1e-3], "cloth_density": 0.1,
            "rayleigh_damping_a": 0.01, "rayleigh_damping_b": 0.0, "default_timestep": dt}


def _state(pos, seed, dt=2e-3):
    rng = np.random.default_rng(seed)
    x = pos.reshape(-1, 3) + rng.normal(0.0, 1e-3, (pos.size // 3, 3))
    v = rng.normal(0.0, 1e-2, x.shape)
    return x.reshape(-1).copy(), (x - dt * v).reshape(-1).copy()


def _cloth(ctx, n, k, seed):
    from acousticsim_gb300 import BaraffClothGpu
    c = BaraffClothGpu(ctx, _conf(n, k))
    c.AddConstraintStaticVertices([i * n + (n - 1) for i in range(n)])  # top edge
    x, xp = _state(c.GetInitPos(), seed)
    c.SetPos(x)
    c.SetPrePos(xp)
    return c


def _workload(count=10, seed=3):
    rng = np.random.default_rng(seed)
    sides = rng.integers(12, 41, count)
    ks = np.exp(rng.uniform(np.log(1e2), np.log(1e3), count))
    steps = rng.integers(1, 5, count)
    return [(int(n), float(k), int(s)) for n, k, s in zip(sides, ks, steps)]


def _twins(ctx, work, p):
    """Each cloth stepped alone; returns positions, previous positions and
    per-step iteration counts."""
    ctx.set_solver("graph_loop")
    out = []
    for i, (n, k, steps) in enumerate(work):
        c = _cloth(ctx, n, k, 100 + i)
        its = []
        for _ in range(steps):
            st = c.UpdatePos(0.0, p)
            assert st["status"] == "OK" and st["solver"] == "graph_loop", st
            its.append(st["iters"])
        out.append((c.GetPos(), c.GetPrePos(), its))
        c.close()
    ctx.set_solver("persistent")
    return out


def _serve(ctx, work, p, budget, max_inflight, chunk_iters, seed=9, gap_s=0.002):
    from acousticsim_gb300 import ClothServer
    srv = ClothServer(ctx, budget, max_inflight, chunk_iters)
    cloths = [_cloth(ctx, n, k, 100 + i) for i, (n, k, _) in enumerate(work)]
    idx = [srv.add(c, 0.0, p) for c in cloths]
    srv.start()
    # interleaved request order, submitted while earlier ones run
    order = [i for i, (_, _, s) in enumerate(work) for _ in range(s)]
    rng = np.random.default_rng(seed)
    rng.shuffle(order)
    for tag, i in enumerate(order):
        srv.submit(idx[i], tag)
        if gap_s > 0:
            time.sleep(float(rng.uniform(0.0, gap_s)))
    srv.drain(120.0)
    res = srv.poll(cap=len(order) + 8)
    stats = srv.stats()
    assert len(res) == len(order) and stats["completed"] == len(order), (len(res), stats)
    # per cloth, results in submission order
    per = {i: [] for i in range(len(work))}
    for r in sorted(res, key=lambda r: r["tag"]):
        assert r["status"] == "OK", r
        assert r["rel_residual"] <= REL_TOL
        assert r["t_arrival"] <= r["t_admit"] <= r["t_done"]
        per[order[r["tag"]]].append(r["iters"])
    out = [(c.GetPos(), c.GetPrePos(), per[i]) for i, c in enumerate(cloths)]
    srv.close()
    for c in cloths:
        c.close()
    return out, stats


def _check_same(served, alone):
    for i, ((x, xp, its), (x0, xp0, its0)) in enumerate(zip(served, alone)):
        assert its == its0, (i, its, its0)
        assert np.array_equal(x, x0), (i, float(np.abs(x - x0).max()))
        assert np.array_equal(xp, xp0), i


@pytest.mark.gpu
def test_served_results_equal_alone(ctx):
    from acousticsim_gb300 import params
    p = params(max_iters=5000, rel_tol=REL_TOL)
    work = _workload()
    alone = _twins(ctx, work, p)
    served, stats = _serve(ctx, work, p, budget=4 << 30, max_inflight=0, chunk_iters=4)
    _check_same(served, alone)
    assert stats["chunks"] > 1
    assert stats["max_inflight_seen"] > 1  # requests really overlapped


@pytest.mark.gpu
def test_chunk_length_does_not_change_results(ctx):
    from acousticsim_gb300 import params
    p = params(max_iters=5000, rel_tol=REL_TOL)
    work = _workload(count=6, seed=4)
    a, _ = _serve(ctx, work, p, budget=4 << 30, max_inflight=0, chunk_iters=1)
    b, _ = _serve(ctx, work, p, budget=4 << 30, max_inflight=0, chunk_iters=64)
    _check_same(a, b)


@pytest.mark.gpu
def test_budget_bounds_admission(ctx):
    """A pool with room for about two requests at a time: admission waits for
    memory, every request still completes, results are unchanged."""
    from acousticsim_gb300 import ClothServer, params
    p = params(max_iters=5000, rel_tol=REL_TOL)
    work = _workload(count=8, seed=5)
    # sizes of the resident state and of one request's work memory
    probe = ClothServer(ctx, 4 << 30)
    cl = [_cloth(ctx, n, k, 100 + i) for i, (n, k, _) in enumerate(work)]
    for c in cl:
        probe.add(c, 0.0, p)
    st = probe.stats()
    probe.close()
    for c in cl:
        c.close()
    budget = st["resident_bytes"] + st["own_bytes"] + int(2.2 * st["max_request_bytes"])
    alone = _twins(ctx, work, p)
    # all requests at once: more work is ready than the pool holds
    served, stats = _serve(ctx, work, p, budget=budget, max_inflight=0, chunk_iters=4,
                           gap_s=0.0)
    _check_same(served, alone)
    assert stats["pool_bytes"] <= budget - st["resident_bytes"] - st["own_bytes"]
    assert stats["pool_peak_bytes"] <= stats["pool_bytes"]
    assert stats["admitted_waits"] > 0


@pytest.mark.gpu
def test_slot_limit(ctx):
    from acousticsim_gb300 import params
    p = params(max_iters=5000, rel_tol=REL_TOL)
    work = _workload(count=6, seed=6)
    alone = _twins(ctx, work, p)
    served, stats = _serve(ctx, work, p, budget=4 << 30, max_inflight=2, chunk_iters=8,
                           gap_s=0.0)
    _check_same(served, alone)
    assert stats["max_inflight_seen"] <= 2


@pytest.mark.gpu
def test_server_errors_and_handback(ctx):
    from acousticsim_gb300 import ClothContext, ClothError, ClothServer, params
    from acousticsim_gb300 import _native as N
    p = params(max_iters=5000, rel_tol=REL_TOL)
    c = _cloth(ctx, 16, 1e3, 1)
    # a budget that cannot hold the cloth
    tiny = ClothServer(ctx, 4096)
    with pytest.raises(ClothError) as e:
        tiny.add(c)
    assert e.value.code == 4  # CLOTH_ERR_BUDGET
    tiny.close()
    srv = ClothServer(ctx, 1 << 30)
    with pytest.raises(ClothError) as e:
        srv.start()  # nothing registered
    assert e.value.code == 11
    i = srv.add(c, 0.0, p)
    # another context's cloth is refused
    other = ClothContext(0)
    c2 = _cloth(other, 16, 1e3, 2)
    with pytest.raises(ClothError) as e:
        srv.add(c2)
    assert e.value.code == 1
    c2.close()
    other.close()
    # the held cloth cannot be stepped or destroyed directly
    with pytest.raises(ClothError) as e:
        c.UpdatePos(0.0, p)
    assert e.value.code == 11
    assert N.load().cloth_destroy(c.handle) == 11
    with pytest.raises(ClothError):
        srv.submit(i, 0)  # not started
    srv.start()
    with pytest.raises(ClothError) as e:
        srv.add(_cloth(ctx, 16, 1e3, 3))  # registration closes at start
    assert e.value.code == 11
    with pytest.raises(ClothError) as e:
        srv.submit(i + 5, 0)
    assert e.value.code == 1
    srv.submit(i, 7)
    srv.drain(60.0)
    (r,) = srv.poll()
    assert r["tag"] == 7 and r["status"] == "OK"
    x_served = c.GetPos()
    srv.close()
    # handed back: the cloth steps on its own again, from the served state
    st = c.UpdatePos(0.0, p)
    assert st["status"] == "OK"
    assert not np.array_equal(c.GetPos(), x_served)
    c.close()


def test_server_null_arguments(built):
    from acousticsim_gb300 import _native as N
    lib = N.load()
    assert lib.cloth_server_create(None, None, None) == 1
    assert lib.cloth_server_submit(None, 0, 0, -1.0) == 1
    assert lib.cloth_server_add(None, None, 0.0, None, None) == 1
    assert lib.cloth_server_start(None) == 1
    assert lib.cloth_server_destroy(None) == 0
    t0 = lib.cloth_server_now()
    assert lib.cloth_server_now() >= t0
