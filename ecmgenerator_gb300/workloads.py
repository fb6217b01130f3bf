"""Seeded synthetic workloads of the tick (no public dataset exists for them).

    crossing_1m    400x400 m, 200 boxes of side U[1,4] m, 1,000,000 agents in
                   four 250k groups spawned in 60 m bands along the sides,
                   goals in the opposite band (overlap allowed), k = 16
    crossing_100k  the same scene with 100,000 agents
    crossing_250k  a quarter of the 1M crossing at its density: 200x200 m,
                   50 boxes, 30 m bands, 250,000 agents (profiling case)
    boxes_100k     1000x1000 m, 4,000 boxes of side U[2,8] m, 100,000 agents
                   spawned without overlap, goals uniform in free space, k = 10
    boxes_1k       100x100 m, 40 boxes, 1,000 agents, k = 10
    batch_256      256 independent scenes in one context: side U[50,500] m,
                   side/5 boxes of side U[2,8] m, agents per scene log-uniform
                   in [200, 20,000] scaled to 1.3M in total (overlap allowed
                   where a scene is dense), goals uniform in free space, k = 10

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
    "crossing_250k": dict(cfg="c3", agents=250_000, k=16, over=dict(w=200.0, h=200.0, boxes=50, bands=30.0)),
    "boxes_100k": dict(cfg="c2", agents=100_000, k=10),
    "boxes_1k": dict(cfg="c1", agents=1_000, k=10),
    "batch_256": dict(batch=256, agents=1_300_000, k=10),
}
ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)
DT = 1.0 / 60.0


def make_workload(name, seed, verbose=True, planner="reference", plan=None):
    """(cfg, scene, agent state with planned paths, paths, k); the initial
    paths come from the library's reference planner (ECMPathPlanner::FindPath
    restated) unless planner="fast", or from plan(scene, starts, goals,
    clearances) -> list of paths / None when given; an agent without a path
    walks straight to its goal"""
    from . import agents as ag

    w = WORKLOADS[name]
    cfg = ag.scaled(w["cfg"], agents=w["agents"], **w.get("over", {}))
    t0 = time.time()
    scene = ag.build_scene(cfg, seed)
    st = ag.spawn_agents(cfg, scene, seed)
    if plan is None:
        from .simulator import Planner

        pl = Planner(scene, mode=planner)
        plan = lambda sc, a_, b_, c_: pl.find_paths(a_, b_, c_, threads=0, cap=256)  # noqa: E731
    else:
        pl = None
    n = st.num_agents
    paths = []
    chunk = 100_000
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        got = plan(scene, st.pos[a:b], st.goal[a:b], st.clear[a:b])
        for i, p in enumerate(got):
            if p is None:
                p = np.stack([st.pos[a + i], st.goal[a + i]])
            paths.append(np.asarray(p, np.float32))
    st.set_paths(paths)
    if pl is not None:
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


def add_spawn_areas(sim, scene, rate, n_areas=4, half=2.5, clearance=0.3, speed=1.3, seed=0):
    """Spawn areas for a workload (Simulator::AddSpawnArea / AddGoalArea /
    ConnectSpawnGoalAreas): n_areas squares of half size `half` at
    obstacle-free spots of the scene's middle half, each feeding, at `rate`
    agents per second, a goal area at the free spot nearest to its mirror
    image through the scene centre.  Returns the spawn area IDs."""
    rng = np.random.default_rng(seed)
    b = np.asarray(scene.boxes, np.float64).reshape(-1, 4)
    W, H = scene.width, scene.height

    def free(x, y):
        m = half + 1.0
        return not (b.size and np.any((np.abs(b[:, 0] - x) < b[:, 2] + m) & (np.abs(b[:, 1] - y) < b[:, 3] + m)))

    def spot_near(x, y):
        for r in np.linspace(0.0, min(W, H) / 4, 200):
            for _ in range(8):
                a = rng.uniform(0, 2 * np.pi)
                px, py = x + r * np.cos(a), y + r * np.sin(a)
                if half < px < W - half and half < py < H - half and free(px, py):
                    return float(px), float(py)
        raise RuntimeError("no obstacle-free spot for a spawn area")

    ids = []
    cfg = dict(clearance_min=clearance, preferred_speed_min=speed, clearance_max=clearance, preferred_speed_max=speed)
    for i in range(n_areas):
        a = 2 * np.pi * (i + 0.5) / n_areas
        sx, sy = spot_near(W / 2 + W / 4 * np.cos(a), H / 2 + H / 4 * np.sin(a))
        gx, gy = spot_near(W - sx, H - sy)
        s = sim.add_spawn_area((sx, sy), (half, half), cfg)
        g = sim.add_goal_area((gx, gy), (half, half))
        sim.connect_spawn_goal_areas(s, g, float(rate))
        ids.append(s)
    return ids


def _batch_scene(job):
    """one scene of a batch workload (runs in a worker process)"""
    from . import agents as ag
    from .simulator import Planner

    side, n, seed = job
    dense = n * np.pi * 0.275 ** 2 > 0.3 * side * side
    cfg = dict(w=side, h=side, boxes=int(side // 5), side=(2.0, 8.0), agents=n, k=10, overlap=bool(dense),
               h_ecm=0.25)
    scene = ag.build_scene(cfg, seed)
    st = ag.spawn_agents(cfg, scene, seed)
    pl = Planner(scene)
    got = pl.find_paths(st.pos[:n], st.goal[:n], st.clear[:n], threads=1, cap=256)
    pl.close()
    paths = [np.asarray(p if p is not None else np.stack([st.pos[i], st.goal[i]]), np.float32)
             for i, p in enumerate(got)]
    st.set_paths(paths)
    return cfg, scene, st, paths


def make_batch_workload(name, seed, procs=None, verbose=True):
    """(cfgs, scenes, agent states, paths per scene, k) of a batch workload;
    the scenes are built on worker processes (spawned: safe before and after
    CUDA initialisation)"""
    import multiprocessing as mp
    import os

    w = WORKLOADS[name]
    rng = np.random.default_rng(seed)
    n_sc = w["batch"]
    sides = rng.uniform(50.0, 500.0, n_sc)
    counts = np.exp(rng.uniform(np.log(200.0), np.log(20000.0), n_sc))
    counts = np.maximum(200, np.round(counts * w["agents"] / counts.sum())).astype(int)
    jobs = [(float(sides[i]), int(counts[i]), int(seed * 100003 + i)) for i in range(n_sc)]
    t0 = time.time()
    procs = procs or max(1, min(32, os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(procs) as pool:
        res = pool.map(_batch_scene, jobs, chunksize=1)
    if verbose:
        print(f"[workload] {name}: {n_sc} scenes, {int(counts.sum())} agents, setup {time.time() - t0:.1f}s "
              f"on {procs} processes", file=sys.stderr, flush=True)
    cfgs, scenes, states, paths = zip(*res)
    return list(cfgs), list(scenes), list(states), list(paths), w["k"]
