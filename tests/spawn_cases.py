"""Spawn-area scenarios shared by the oracle pinning (CPU, against the
reference build) and the GPU parity tests.

An ``Ops`` adapter applies one list of area operations to the restatement
(oracle/spawn_oracle.Areas), the reference harness (oracle.Ref) or the
library (ecmgenerator_gb300.simulator.Simulator), so the three see the same
areas, IDs and connections."""
from __future__ import annotations

import numpy as np

F32 = np.float32


def free_rect(scene, hw, hh, margin=1.0, seed=0, avoid=()):
    """centre of an axis-aligned rectangle of half size (hw, hh) that keeps
    `margin` from every box, the scene border and the rectangles in `avoid`
    ((x, y, hw, hh) tuples)"""
    rng = np.random.default_rng(seed)
    b = np.asarray(scene.boxes, np.float64).reshape(-1, 4)
    for _ in range(20000):
        x = rng.uniform(hw + margin, scene.width - hw - margin)
        y = rng.uniform(hh + margin, scene.height - hh - margin)
        if b.size and np.any((np.abs(b[:, 0] - x) < b[:, 2] + hw + margin) &
                             (np.abs(b[:, 1] - y) < b[:, 3] + hh + margin)):
            continue
        if any(abs(x - ax) < hw + ahw + margin and abs(y - ay) < hh + ahh + margin for ax, ay, ahw, ahh in avoid):
            continue
        return float(x), float(y)
    raise RuntimeError("no free rectangle")


class Ops:
    """area operations on one of: oracle Areas, oracle.Ref, library Simulator"""

    def __init__(self, target, kind):
        self.t, self.kind = target, kind

    def spawn(self, x, y, hw, hh, cfg=None, ID=-1):
        if self.kind == "lib":
            return self.t.add_spawn_area((x, y), (hw, hh), cfg, ID)
        return self.t.add_spawn_area(x, y, hw, hh, cfg, ID)

    def goal(self, x, y, hw, hh, ID=-1):
        if self.kind == "lib":
            return self.t.add_goal_area((x, y), (hw, hh), ID)
        return self.t.add_goal_area(x, y, hw, hh, ID)

    def connect(self, s, g, rate=0.0):
        if self.kind == "lib":
            return self.t.connect_spawn_goal_areas(s, g, rate)
        return self.t.connect(s, g, rate)

    def disconnect(self, s, g):
        if self.kind == "lib":
            return self.t.deconnect_spawn_goal_areas(s, g)
        return self.t.disconnect(s, g)

    def remove(self, area_type, ID):
        return self.t.remove_area(area_type, ID)


def standard_areas(scene, ops: Ops, clearance=0.5, speed=1.3):
    """two spawn areas, three goal areas, four connections of different
    rates (agents per second), plus an explicit ID and a repeated ID"""
    a0 = free_rect(scene, 4.0, 3.0, seed=1)
    a1 = free_rect(scene, 2.5, 2.5, seed=2, avoid=[a0 + (4.0, 3.0)])
    g0 = free_rect(scene, 3.0, 3.0, seed=3, avoid=[a0 + (4.0, 3.0), a1 + (2.5, 2.5)])
    g1 = free_rect(scene, 2.0, 4.0, seed=4, avoid=[a0 + (4.0, 3.0), a1 + (2.5, 2.5), g0 + (3.0, 3.0)])
    cfg = dict(clearance_min=clearance, preferred_speed_min=speed, clearance_max=clearance * 2,
               preferred_speed_max=speed * 2)
    s0 = ops.spawn(*a0, 4.0, 3.0, cfg)
    s1 = ops.spawn(*a1, 2.5, 2.5, cfg, ID=7)
    same = ops.spawn(*a0, 1.0, 1.0, None, ID=7)  # ID taken: the first area stays
    assert same == 7
    q0 = ops.goal(*g0, 3.0, 3.0)
    q1 = ops.goal(*g1, 2.0, 4.0)
    q2 = ops.goal(*g0, 1.0, 1.0, ID=11)
    ops.connect(s0, q0, 40.0)
    ops.connect(s0, q1, 25.0)
    ops.connect(s1, q2, 90.0)
    ops.connect(s1, q0, 7.5)
    ops.connect(s1, q0, 99.0)  # already connected: ignored
    return dict(spawn=[(s0, a0, (4.0, 3.0)), (s1, a1, (2.5, 2.5))], goal=[q0, q1, q2])


def crowd_in(rect, half, spacing, n_max):
    """agent positions on a square lattice covering a rectangle"""
    (x, y), (hw, hh) = rect, half
    xs = np.arange(x - hw, x + hw + 1e-6, spacing)
    ys = np.arange(y - hh, y + hh + 1e-6, spacing)
    p = np.stack(np.meshgrid(xs, ys), -1).reshape(-1, 2).astype(F32)
    return p[:n_max]
