"""Host-side agent state and the seeded workloads.

``AgentState`` mirrors the Simulator's component arrays
(ECMAgentSimulator/Simulator.h:29-57, Simulator.cpp:21-60): slot-indexed
positions, velocities, attraction points, preferred velocities, clearances
(radii), preferred speeds, active flags and per-agent path polylines (kept as
one CSR: ``path_xy[path_off[i] : path_off[i] + path_len[i]]``).

``workload(name, seed)`` builds the synthetic scenes the benchmarks run:
boxes, ECM, agents, goals and paths, all from one seed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import scene as sc

F32, I32, U8 = np.float32, np.int32, np.uint8


@dataclass
class AgentState:
    n_slots: int
    pos: np.ndarray
    vel: np.ndarray
    attr: np.ndarray
    pref_vel: np.ndarray
    clear: np.ndarray
    pref_speed: np.ndarray
    active: np.ndarray
    path_off: np.ndarray
    path_len: np.ndarray
    path_xy: np.ndarray
    last_idx: int = -1
    num_agents: int = 0
    goal: np.ndarray | None = None

    @classmethod
    def empty(cls, n_slots: int) -> "AgentState":
        z2 = lambda: np.zeros((n_slots, 2), F32)
        return cls(n_slots, z2(), z2(), z2(), z2(), np.zeros(n_slots, F32), np.zeros(n_slots, F32),
                   np.zeros(n_slots, U8), np.zeros(n_slots, I32), np.zeros(n_slots, I32),
                   np.zeros((0, 2), F32), -1, 0, z2())

    def copy(self) -> "AgentState":
        c = AgentState(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in self.__dict__.items()})
        return c

    def set_paths(self, paths: list) -> None:
        """paths[i] is an (n,2) array for slot i (or None to keep the old one)."""
        lens = np.array([len(p) if p is not None else 0 for p in paths], I32)
        off = np.zeros(len(paths), I32)
        off[1:] = np.cumsum(lens)[:-1]
        xy = np.concatenate([np.asarray(p, F32) for p in paths if p is not None and len(p)], 0) \
            if lens.sum() else np.zeros((0, 2), F32)
        self.path_off[: len(paths)] = off
        self.path_len[: len(paths)] = lens
        self.path_xy = np.ascontiguousarray(xy, F32)

    def replace_path(self, slot: int, path: np.ndarray) -> None:
        """Append a new polyline for ``slot`` to the CSR (old storage is left
        in place, as a device-side patch does)."""
        path = np.asarray(path, F32).reshape(-1, 2)
        self.path_off[slot] = self.path_xy.shape[0]
        self.path_len[slot] = path.shape[0]
        self.path_xy = np.ascontiguousarray(np.concatenate([self.path_xy, path], 0), F32)

    def replace_paths(self, slots, paths) -> None:
        """replace_path for many slots with one append (None keeps a slot's path)"""
        keep = [(int(s_), np.asarray(p, F32).reshape(-1, 2)) for s_, p in zip(slots, paths) if p is not None]
        if not keep:
            return
        base = self.path_xy.shape[0]
        lens = np.array([p.shape[0] for _, p in keep], I32)
        offs = base + np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(I32)
        idx = np.array([s_ for s_, _ in keep], np.int64)
        self.path_off[idx] = offs
        self.path_len[idx] = lens
        self.path_xy = np.ascontiguousarray(np.concatenate([self.path_xy] + [p for _, p in keep], 0), F32)

    def goals(self, slots) -> np.ndarray:
        """the last point of each listed slot's path (its goal)"""
        slots = np.asarray(slots, np.int64)
        return self.path_xy[self.path_off[slots] + self.path_len[slots] - 1]

    def path(self, slot: int) -> np.ndarray:
        o, n = int(self.path_off[slot]), int(self.path_len[slot])
        return self.path_xy[o:o + n]


@dataclass
class Workload:
    name: str
    scene: sc.Scene
    state: AgentState
    params: dict
    seed: int
    meta: dict = field(default_factory=dict)


# Workload definitions: scene size, box count and side range, agent count,
# neighbour count k, whether spawns may overlap, ECM sampling step.
CONFIGS = {
    # 100x100 m, 40 boxes [2,8] m, 1k agents, k=10
    "c1": dict(w=100.0, h=100.0, boxes=40, side=(2.0, 8.0), agents=1000, k=10, overlap=False, h_ecm=0.1),
    # 1000x1000 m, 4000 boxes, 100k agents, k=10
    "c2": dict(w=1000.0, h=1000.0, boxes=4000, side=(2.0, 8.0), agents=100000, k=10, overlap=False, h_ecm=0.25),
    # 400x400 m, 200 boxes [1,4] m, 1M agents in four 60 m bands, k=16, overlap allowed
    "c3": dict(w=400.0, h=400.0, boxes=200, side=(1.0, 4.0), agents=1000000, k=16, overlap=True, h_ecm=0.2,
               bands=60.0),
}

ORCA_DEFAULTS = dict(dt=1.0 / 60.0, tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0, max_speed=0.0,
                     mass=0.8, arrival_radius=20.0, delete_radius=2.0)


def scaled(name: str, agents: int | None = None, **over) -> dict:
    cfg = dict(CONFIGS[name])
    if agents is not None:
        cfg["agents"] = agents
    cfg.update(over)
    return cfg


def build_scene(cfg: dict, seed: int) -> sc.Scene:
    rng = np.random.default_rng(seed)
    boxes = sc.gen_boxes(rng, cfg["w"], cfg["h"], cfg["boxes"], *cfg["side"])
    s = sc.make_scene(cfg["w"], cfg["h"], boxes)
    # cfg["ecm"]: "sampled" (default: chains of the sampled diagram split
    # where they bend, so curved bisectors are followed closely) or "exact"
    # (one straight edge per Voronoi edge between exact vertices, the graph
    # the reference builds from Boost's diagram)
    if cfg.get("ecm", "sampled") == "exact":
        s.ecm = sc.build_ecm_exact(s, h=cfg.get("h_ecm", 0.2))
    else:
        s.ecm = sc.build_ecm(s, h=cfg.get("h_ecm", 0.2))
    s.meta = dict(seed=seed, boxes=int(boxes.shape[0]))
    return s


def spawn_agents(cfg: dict, s: sc.Scene, seed: int, n_slots: int | None = None) -> AgentState:
    """Radii U[0.2,0.35], preferred speed U[1.2,1.5], positions uniform in free
    space (no disk overlap unless cfg['overlap']), goals uniform in free space.
    With cfg['bands'] the agents form four groups along the four sides, each
    heading to the opposite band."""
    rng = np.random.default_rng(seed + 7919)
    n = cfg["agents"]
    n_slots = n if n_slots is None else n_slots
    st = AgentState.empty(n_slots)
    rad = rng.uniform(0.2, 0.35, n)
    spd = rng.uniform(1.2, 1.5, n)
    bidx = sc.BoxIndex(s)
    W, H = s.width, s.height
    if "bands" in cfg:
        b = cfg["bands"]
        regions = [(0, 0, b, H), (W - b, 0, W, H), (0, 0, W, b), (0, H - b, W, H)]
        goals_r = [regions[1], regions[0], regions[3], regions[2]]
        grp = np.arange(n) % 4
        pos = np.zeros((n, 2))
        goal = np.zeros((n, 2))
        for g in range(4):
            idx = np.nonzero(grp == g)[0]
            pos[idx] = sc.sample_free(rng, s, idx.size, rad[idx], bidx, region=regions[g],
                                      no_overlap=not cfg["overlap"])
            goal[idx] = sc.sample_free(rng, s, idx.size, 0.5, bidx, region=goals_r[g], no_overlap=False)
    else:
        pos = sc.sample_free(rng, s, n, rad, bidx, no_overlap=not cfg["overlap"])
        goal = sc.sample_free(rng, s, n, 0.5, bidx, no_overlap=False)
    st.pos[:n] = pos.astype(F32)
    st.goal[:n] = goal.astype(F32)
    st.clear[:n] = rad.astype(F32)
    st.pref_speed[:n] = spd.astype(F32)
    st.active[:n] = 1
    st.last_idx = n - 1
    st.num_agents = n
    return st
