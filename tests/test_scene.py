"""Synthetic scenes and the host ECM builder."""
import numpy as np

from ecmgenerator_gb300 import agents as ag
from ecmgenerator_gb300 import scene as sc


def test_boxes_respect_gap():
    rng = np.random.default_rng(0)
    b = sc.gen_boxes(rng, 200, 200, 150, 2, 8)
    assert b.shape[0] == 150
    for i in range(len(b)):
        for j in range(i + 1, len(b)):
            dx = abs(b[i, 0] - b[j, 0]) - b[i, 2] - b[j, 2]
            dy = abs(b[i, 1] - b[j, 1]) - b[i, 3] - b[j, 3]
            assert np.hypot(max(dx, 0), max(dy, 0)) >= 2.0


def test_rings_ccw_and_convex():
    s = sc.make_scene(50, 50, np.array([[10, 10, 2, 1], [30, 30, 1, 3]]))
    assert s.obst_convex.all()  # boxes in AddObstacleArea order are CCW, every corner convex
    assert s.obst_next.tolist() == [1, 2, 3, 0, 5, 6, 7, 4]
    assert s.obst_prev.tolist() == [3, 0, 1, 2, 7, 4, 5, 6]


def test_ecm_structure_and_coverage(port):
    cfg = ag.scaled("c1")
    s = ag.build_scene(cfg, seed=2)
    e = s.ecm
    V, E = e.n_vertices, e.n_edges
    assert V > 50 and E > 50
    assert ((e.he_target >= 0) & (e.he_target < V)).all()
    # half-edge 2e+1 is the twin of 2e; vertex half-edges leave the vertex
    for v in range(V):
        h = int(e.v_halfedge[v])
        assert e.he_target[h ^ 1] == v
        start, n = h, 0
        while True:
            assert e.he_target[h ^ 1] == v
            h = int(e.he_next[h])
            n += 1
            if h == start or n > 64:
                break
        assert h == start
    # the cells cover free space
    E_s = port.ecm(e)
    rng = np.random.default_rng(0)
    q = rng.uniform(0, 100, (4000, 2))
    clr = sc.BoxIndex(s).clearance(q[:, 0], q[:, 1])
    q = q[clr > 0.05]
    found = np.array([port.point_location(E_s, float(x), float(y)) for x, y in q])
    assert (found >= 0).mean() > 0.995
    # retraction succeeds almost everywhere
    ok = np.mean([port.retract(E_s, float(x), float(y))[0] for x, y in q[:1500]])
    assert ok > 0.98


def test_workload_is_deterministic():
    cfg = ag.scaled("c1", agents=200)
    a = ag.build_scene(cfg, seed=9)
    b = ag.build_scene(cfg, seed=9)
    assert np.array_equal(a.obst_xy, b.obst_xy) and np.array_equal(a.ecm.v_pos, b.ecm.v_pos)
    sa = ag.spawn_agents(cfg, a, seed=9)
    sb = ag.spawn_agents(cfg, b, seed=9)
    assert np.array_equal(sa.pos, sb.pos) and np.array_equal(sa.goal, sb.goal)
    # no overlap between agents, none inside obstacles
    p, r = sa.pos[:200].astype(np.float64), sa.clear[:200].astype(np.float64)
    d = np.hypot(p[:, None, 0] - p[None, :, 0], p[:, None, 1] - p[None, :, 1])
    np.fill_diagonal(d, 1e9)
    assert (d >= (r[:, None] + r[None, :]) * (1 - 1e-6)).all()
    assert (sc.BoxIndex(a).clearance(p[:, 0], p[:, 1]) >= r - 1e-6).all()
