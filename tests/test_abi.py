"""The C ABI without a GPU: the library loads, exports every entry point the
header declares, rejects bad input, and its host-only planner works."""
import ctypes as C

import numpy as np
import pytest

from ecmgenerator_gb300 import _lib


def test_exports_every_declared_symbol(lib):
    names = _lib.declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_default_params_match_reference(lib):
    p = _lib.default_params()
    assert p.max_neighbors == 5  # ORCA(5), Simulator.cpp:55
    assert p.tau_agent == 10.0 and p.tau_obst == 10.0  # ORCA.h:102-103
    assert abs(p.mass - 0.8) < 1e-7 and p.arrival_radius == 20.0 and p.delete_radius == 2.0


def test_create_rejects_bad_params(lib):
    h = C.c_void_p()
    for over in (dict(dt=0.0), dict(max_neighbors=0), dict(max_neighbors=33), dict(neighbor_dist=-1.0),
                 dict(mass=0.0)):
        p = _lib.default_params(**over)
        rc = lib.ecmg_create(C.byref(p), 10, C.byref(h))
        assert rc in (1, 8), (over, rc)  # invalid argument (or no device on a CPU-only host)
    assert lib.ecmg_create(None, 0, C.byref(h)) == 1


def test_null_context_calls_fail_cleanly(lib):
    st = _lib.TickStats()
    assert lib.ecmg_tick(None, 1, C.byref(st)) == 1
    assert lib.ecmg_destroy(None) == 1
    assert lib.ecmg_knn(None, None, 10, 0, 1.0, 0, 0, 1, 1, 1, None, None, None, 0, None) == 1


def test_knn_scratch_size(lib):
    a = lib.ecmg_knn_scratch_bytes(1000, 0.0, 0.0, 100.0, 100.0, 2.0)
    b = lib.ecmg_knn_scratch_bytes(2000, 0.0, 0.0, 100.0, 100.0, 2.0)
    assert 0 < a < b
    assert lib.ecmg_knn_scratch_bytes(10, 0.0, 0.0, 1.0, 1.0, 0.0) == 0


def test_knn_grid_too_large_is_refused_before_any_launch(lib):
    """a box of 65,533 m with 1 m cells is a 65,536 x 65,536 grid: refused
    (scratch size 0, invalid argument) rather than sized with a wrapped int;
    also non-finite boxes.  Host-only: the calls return before any device
    work, so fake non-null device pointers are never touched."""
    fake = 4096
    for box, cell in (((0.0, 0.0, 65533.0, 65533.0), 1.0), ((0.0, 0.0, float("inf"), 1.0), 1.0),
                      ((float("nan"), 0.0, 1.0, 1.0), 1.0), ((0.0, 0.0, 1e30, 1e30), 1e-3)):
        assert lib.ecmg_knn_scratch_bytes(1000, *box, cell) == 0
        assert lib.ecmg_knn(fake, fake, 1000, 4, 1.0, *box, cell, fake, fake, fake, 1 << 30, None) == 1
        assert lib.ecmg_knn_noalloc(fake, fake, 1000, 4, 1.0, *box, cell, fake, fake, None) == 1


def test_planner_host_only(c1_small, port):
    from ecmgenerator_gb300.simulator import Planner

    scene, st, paths = c1_small
    pl = Planner(scene)
    rng = np.random.default_rng(1)
    q = rng.uniform(-3, 103, (3000, 2)).astype(np.float32)
    q[:100, 1] = scene.ecm.v_pos[:100, 1]  # exact vertex heights
    # every quad-corner height (vertices and boundary closest points), with x
    # far outside the quads too: the ray-cast test's hits left of a quad
    ys = np.concatenate([np.asarray(scene.ecm.v_pos).reshape(-1, 2)[:, 1],
                         np.asarray(scene.ecm.he_left).reshape(-1, 2)[:, 1],
                         np.asarray(scene.ecm.he_right).reshape(-1, 2)[:, 1]]).astype(np.float32)
    q2 = np.stack([rng.uniform(-60, 160, 4000), rng.choice(ys, 4000)], 1).astype(np.float32)
    q = np.concatenate([q, q2])
    E = port.ecm(scene.ecm)
    want = np.array([port.point_location(E, float(x), float(y)) for x, y in q])
    got = pl.locate(q)
    assert np.array_equal(got, want)
    assert (want[3000:] >= 0).sum() > 1000
    ok = [p for p in paths if p is not None]
    assert len(ok) == len(paths)
    n_ok = sum(1 for i in range(st.num_agents) if np.allclose(paths[i][0], st.pos[i]) and np.allclose(paths[i][-1], st.goal[i]))
    assert n_ok == st.num_agents
