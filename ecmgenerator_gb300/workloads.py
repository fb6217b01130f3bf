"""Seeded synthetic workloads of the tick (no public dataset exists for them).

    crossing_1m    400x400 m, 200 boxes of side U[1,4] m, 1,000,000 agents in
                   four 250k groups spawned in 60 m bands along the sides,
                   goals in the opposite band (overlap allowed), k = 16
    crossing_100k  the same scene with 100,000 agents
    boxes_100k     1000x1000 m, 4,000 boxes of side U[2,8] m, 100,000 agents
                   spawned without overlap, goals uniform in free space, k = 10
    boxes_1k       100x100 m, 40 boxes, 1,000 agents, k = 10

Radius U[0.2,0.35] m, preferred speed U[1.2,1.5] m/s, ORCA time horizons
2 s, neighbour distance 5 m, dt = 1/60 s.
"""
from __future__ import annotations

import sys
import time

import numpy as np

WORKLOADS = {
    "crossing_1m": dict(cfg="c3", agents=1_000_000, k=16),
    "crossing_100k": dict(cfg="c3", agents=100_000, k=16),
    "boxes_100k": dict(cfg="c2", agents=100_000, k=10),
    "boxes_1k": dict(cfg="c1", agents=1_000, k=10),
}
ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)
DT = 1.0 / 60.0


def make_workload(name, seed, verbose=True):
    """(cfg, scene, agent state with planned paths, paths, k)"""
    from . import agents as ag
    from .simulator import Planner

    w = WORKLOADS[name]
    cfg = ag.scaled(w["cfg"], agents=w["agents"])
    t0 = time.time()
    scene = ag.build_scene(cfg, seed)
    st = ag.spawn_agents(cfg, scene, seed)
    pl = Planner(scene)
    n = st.num_agents
    paths = []
    chunk = 100_000
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        got = pl.find_paths(st.pos[a:b], st.goal[a:b], st.clear[a:b], threads=0, cap=64)
        for i, p in enumerate(got):
            if p is None:
                p = np.stack([st.pos[a + i], st.goal[a + i]])
            paths.append(np.asarray(p, np.float32))
    st.set_paths(paths)
    pl.close()
    if verbose:
        print(f"[workload] {name}: {n} agents, {scene.ecm.n_edges} ECM edges, setup {time.time() - t0:.1f}s",
              file=sys.stderr, flush=True)
    return cfg, scene, st, paths, w["k"]


def make_simulator(name, seed, **kw):
    """a Simulator holding the workload's agents"""
    from .simulator import Simulator

    cfg, scene, st, paths, k = make_workload(name, seed)
    n = st.num_agents
    sim = Simulator(scene, n, DT, max_neighbors=k, **ORCA, **kw)
    sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths)
    return sim, (cfg, scene, st, paths, k)
