"""The exact segment-Voronoi ECM builder (scene.build_ecm_exact), on the CPU.

The reference builds its ECM from Boost.Polygon's segment Voronoi diagram
(ECMGenerator/ECMGenerator.cpp:60-256); Boost is not available here, so the
builder is checked against the defining properties of that diagram and
against a scene whose diagram is known in closed form."""
import math

import numpy as np
import pytest

from ecmgenerator_gb300 import scene as sc


def _scene(seed, w, nb, side):
    rng = np.random.default_rng(seed)
    boxes = sc.gen_boxes(rng, w, w, nb, *side)
    return sc.make_scene(w, w, boxes)


def _closed_dist(segs, x):
    a, b = segs[:, 0:2], segs[:, 2:4]
    t = b - a
    u = np.clip(((x - a) * t).sum(1) / (t * t).sum(1), 0.0, 1.0)
    return np.hypot(*(x - (a + u[:, None] * t)).T)


def _canon(e, nd=3):
    keys = [tuple(np.round(v.astype(np.float64), nd)) for v in e.v_pos]
    edges = set()
    for k in range(e.n_edges):
        edges.add(tuple(sorted([keys[int(e.he_target[2 * k + 1])], keys[int(e.he_target[2 * k])]])))
    return set(keys), edges


@pytest.mark.parametrize("seed,w,nb,side", [(3, 100.0, 40, (2.0, 8.0)), (5, 200.0, 120, (1.0, 4.0))])
def test_vertices_are_voronoi_vertices(seed, w, nb, side):
    """every vertex is nearer to no obstacle than to the features its edges
    separate (the empty circle), and those features are equally far"""
    s = _scene(seed, w, nb, side)
    e = sc.build_ecm_exact(s, h=0.2)
    assert e.meta["unresolved_chains"] == 0
    segs = sc._segments(s)
    for i in range(e.n_vertices):
        x = e.v_pos[i].astype(np.float64)
        r = _closed_dist(segs, x).min()
        assert abs(float(e.v_clear[i]) - r) < 2e-5 * max(1.0, r), (i, x, e.v_clear[i], r)
    # both closest points of every half-edge are at the source vertex's
    # clearance: the edge separates two features at equal distance
    src = np.empty(2 * e.n_edges, np.int64)
    src[0::2] = e.he_target[1::2]
    src[1::2] = e.he_target[0::2]
    p = e.v_pos[src].astype(np.float64)
    dl = np.hypot(*(p - e.he_left).T)
    dr = np.hypot(*(p - e.he_right).T)
    assert np.max(np.abs(dl - dr)) < 1e-4
    assert np.max(np.abs(dl - e.v_clear[src])) < 1e-4


def test_result_does_not_depend_on_the_sampling():
    s = _scene(3, 100.0, 40, (2.0, 8.0))
    a = _canon(sc.build_ecm_exact(s, h=0.2))
    b = _canon(sc.build_ecm_exact(s, h=0.1))
    assert a == b


def test_one_cycle_around_every_obstacle():
    """the medial axis of a walkable rectangle with k separated boxes is a
    connected planar graph with one independent cycle around each box"""
    s = _scene(5, 200.0, 120, (1.0, 4.0))
    e = sc.build_ecm_exact(s, h=0.2)
    assert e.n_edges - e.n_vertices + 1 == s.boxes.shape[0]
    # connected
    adj = [[] for _ in range(e.n_vertices)]
    for k in range(e.n_edges):
        a, b = int(e.he_target[2 * k + 1]), int(e.he_target[2 * k])
        adj[a].append(b)
        adj[b].append(a)
    seen, stack = {0}, [0]
    while stack:
        for q in adj[stack.pop()]:
            if q not in seen:
                seen.add(q)
                stack.append(q)
    assert len(seen) == e.n_vertices


def test_square_box_in_a_square_closed_form():
    """a 4 x 4 m box in the middle of a 10 x 10 m area: the border corners,
    one vertex on each diagonal equidistant from two border sides and the
    box corner (t = 3 (2 - sqrt 2)), and two vertices on the normals of the
    box sides through each box corner (half way to the border): 16 vertices,
    4 diagonal + 8 parabolic + 4 straight edges"""
    s = sc.make_scene(10.0, 10.0, np.array([[5.0, 5.0, 2.0, 2.0]]))
    e = sc.build_ecm_exact(s, h=0.1)
    t = 3.0 * (2.0 - math.sqrt(2.0))
    want = {(0.0, 0.0), (10.0, 0.0), (0.0, 10.0), (10.0, 10.0),
            (t, t), (10 - t, t), (t, 10 - t), (10 - t, 10 - t)}
    for c in (3.0, 7.0):
        want |= {(1.5, c), (8.5, c), (c, 1.5), (c, 8.5)}
    got = {tuple(v) for v in np.round(e.v_pos.astype(np.float64), 4)}
    assert got == {tuple(np.round(v, 4)) for v in want}
    assert e.n_edges == 16
    # every vertex's clearance in closed form: 0 at the border corners
    for v, c in zip(e.v_pos.astype(np.float64), e.v_clear):
        r = _closed_dist(sc._segments(s), v).min()
        assert abs(float(c) - r) < 1e-5


def test_integer_sites():
    """construct_voronoi reads the reference's points through an int
    point_traits: with integer coordinates the truncation changes nothing;
    with fractional ones the vertices are those of the truncated geometry"""
    s = sc.make_scene(40.0, 40.0, np.array([[10.0, 12.0, 2.0, 3.0], [27.0, 25.0, 4.0, 2.0]]))
    assert _canon(sc.build_ecm_exact(s, h=0.1)) == _canon(sc.build_ecm_exact(s, h=0.1, int_sites=True))
    s2 = sc.make_scene(40.0, 40.0, np.array([[10.5, 12.25, 2.0, 3.0], [27.0, 25.0, 4.0, 2.0]]))
    e = sc.build_ecm_exact(s2, h=0.1, int_sites=True)
    segs = np.trunc(sc._segments(s2))
    for v in e.v_pos.astype(np.float64):
        d = np.sort(_closed_dist(segs, v))
        # equidistant from at least two segments of the truncated geometry
        assert d[1] - d[0] < 1e-4
