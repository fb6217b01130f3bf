"""Python mirror of ``ECM::Simulation::Simulator`` (ECMAgentSimulator/Simulator.h:59-188)
over the C ABI of libecmg.so.

Method names follow the reference (snake_case); the tick runs on the GPU and
nothing here computes simulation results on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import EcmgError, FIELD

F32, I32, U8 = np.float32, np.int32, np.uint8


def _a(x, dt):
    return np.ascontiguousarray(x, dtype=dt)


def _ptr(x):
    return x.ctypes.data if x is not None else None


class Planner:
    """Host-only ECM planner (ecmg_planner_*); needs no GPU."""

    def __init__(self, scene, mode: str = "reference"):
        """mode 'reference' (default: ECMPathPlanner::FindPath restated, the
        reference's paths) or 'fast' (opt-in: A* with landmark bounds and
        greedy shortening, not the reference's paths)"""
        L = self.L = _lib.load()
        self._keep, o, e = _scene_structs(scene)
        h = C.c_void_p()
        rc = L.ecmg_planner_create(C.byref(o), C.byref(e), C.byref(h))
        if rc:
            raise EcmgError(rc, "ecmg_planner_create failed")
        self.h = h
        if mode != "reference":
            rc = L.ecmg_planner_set_mode(self.h, {"fast": 0, "reference": 1}[mode])
            if rc:
                raise EcmgError(rc, "ecmg_planner_set_mode failed")

    def find_paths(self, starts, goals, clearances, threads=0, cap=1024):
        starts, goals, clr = _a(starts, F32).reshape(-1, 2), _a(goals, F32).reshape(-1, 2), _a(clearances, F32)
        n = starts.shape[0]
        out = np.zeros((n, cap, 2), F32)
        cnt = np.zeros(n, I32)
        rc = self.L.ecmg_planner_find_paths(self.h, n, _ptr(starts), _ptr(goals), _ptr(clr), threads, cap, _ptr(out),
                                            _ptr(cnt))
        if rc:
            raise EcmgError(rc, "ecmg_planner_find_paths failed")
        return [out[i, :cnt[i]].copy() if cnt[i] > 0 else None for i in range(n)]

    def locate(self, xy):
        xy = _a(xy, F32).reshape(-1, 2)
        out = np.zeros(xy.shape[0], I32)
        rc = self.L.ecmg_planner_locate(self.h, xy.shape[0], _ptr(xy), _ptr(out))
        if rc:
            raise EcmgError(rc, "ecmg_planner_locate failed")
        return out

    def close(self):
        if getattr(self, "h", None):
            self.L.ecmg_planner_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _scene_structs(scene):
    e = scene.ecm
    keep = [_a(scene.obst_off, I32), _a(scene.obst_xy, F32), _a(e.v_pos, F32), _a(e.v_clear, F32), _a(e.v_idx, I32),
            _a(e.v_halfedge, I32), _a(e.he_target, I32), _a(e.he_next, I32), _a(e.he_left, F32),
            _a(e.he_right, F32)]
    o = _lib.Obstacles(scene.n_obstacles, _ptr(keep[0]), _ptr(keep[1]))
    es = _lib.Ecm(e.n_vertices, _ptr(keep[2]), _ptr(keep[3]), _ptr(keep[4]), _ptr(keep[5]), e.n_edges,
                  _ptr(keep[6]), _ptr(keep[7]), _ptr(keep[8]), _ptr(keep[9]))
    return keep, o, es


class Simulator:
    """Simulator(ecm, planner, environment, maxAgents, simStepTime) on the GPU."""

    def __init__(self, scene, max_agents: int, sim_step_time: float, *, max_neighbors: int = 5,
                 tau_agent: float = 10.0, tau_obst: float = 10.0, neighbor_dist: float = 5.0,
                 max_speed: float = 0.0, use_graph: bool = True, lp3d_fp64: bool = False, grid_cell: float = 0.0,
                 mass: float = 0.8, arrival_radius: float = 20.0, delete_radius: float = 2.0):
        self.L = _lib.load()
        p = _lib.default_params(dt=sim_step_time, max_neighbors=max_neighbors, tau_agent=tau_agent,
                                tau_obst=tau_obst, neighbor_dist=neighbor_dist, max_speed=max_speed,
                                use_graph=int(use_graph), lp3d_fp64=int(lp3d_fp64), grid_cell=grid_cell, mass=mass,
                                arrival_radius=arrival_radius, delete_radius=delete_radius)
        self.params = p
        h = C.c_void_p()
        rc = self.L.ecmg_create(C.byref(p), int(max_agents), C.byref(h))
        if rc:
            raise EcmgError(rc, "ecmg_create failed (is a CUDA device visible?)")
        self.h = h
        self.max_agents = int(max_agents)
        self.k = int(max_neighbors)
        self.scene = scene
        self._keep, o, e = _scene_structs(scene)
        self._ck(self.L.ecmg_set_obstacles(self.h, C.byref(o)))
        self._ck(self.L.ecmg_set_ecm(self.h, C.byref(e)))
        self._plan_cb = None

    # -- plumbing --------------------------------------------------------
    def _ck(self, rc):
        if rc:
            msg = self.L.ecmg_last_error(self.h)
            raise EcmgError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.L.ecmg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- Simulator API ---------------------------------------------------
    def initialize(self):
        """Simulator::Initialize (Simulator.cpp:21-60): storage is allocated by
        the constructor; kept for API parity."""

    def set_planner(self, fn):
        """fn(sx, sy, gx, gy, clearance) -> (n,2) array or None."""
        if fn is None:
            self._plan_cb = None
            self._ck(self.L.ecmg_set_planner(self.h, _lib.PLAN_FN(), None))
            return

        def cb(user, sx, sy, gx, gy, clr, out, cap):
            p = fn(sx, sy, gx, gy, clr)
            if p is None:
                return -1
            p = np.asarray(p, F32).reshape(-1, 2)[:cap]
            for i in range(p.shape[0]):
                out[2 * i] = float(p[i, 0])
                out[2 * i + 1] = float(p[i, 1])
            return int(p.shape[0])

        self._plan_cb = _lib.PLAN_FN(cb)
        self._ck(self.L.ecmg_set_planner(self.h, self._plan_cb, None))

    def spawn_agent(self, start, goal, clearance: float, preferred_speed: float) -> int:
        """Simulator::SpawnAgent; returns the slot or -1 (Simulator.cpp:168-200)."""
        s = C.c_int(-1)
        rc = self.L.ecmg_spawn_agent(self.h, float(start[0]), float(start[1]), float(goal[0]), float(goal[1]),
                                     float(clearance), float(preferred_speed), C.byref(s))
        if rc in (4, 6, 7):
            return -1
        self._ck(rc)
        return s.value

    def add_agents(self, pos, clearance, pref_speed, paths) -> np.ndarray:
        pos = _a(pos, F32).reshape(-1, 2)
        n = pos.shape[0]
        clr, spd = _a(clearance, F32), _a(pref_speed, F32)
        lens = np.array([len(p) for p in paths], I32)
        offs = np.zeros(n, I32)
        if n:
            offs[1:] = np.cumsum(lens)[:-1]
        xy = _a(np.concatenate([np.asarray(p, F32).reshape(-1, 2) for p in paths], 0), F32) if n else \
            np.zeros((0, 2), F32)
        out = np.zeros(n, I32)
        self._ck(self.L.ecmg_add_agents(self.h, n, _ptr(pos), _ptr(clr), _ptr(spd), _ptr(offs), _ptr(lens),
                                        _ptr(xy), _ptr(out)))
        return out

    def destroy_agent(self, idx: int):
        self._ck(self.L.ecmg_destroy_agent(self.h, int(idx)))

    def save_state(self, path: str):
        """checkpoint (ecmg_save_state)"""
        self._ck(self.L.ecmg_save_state(self.h, str(path).encode()))

    def load_state(self, path: str):
        """resume from a checkpoint of a context like this one (ecmg_load_state)"""
        self._ck(self.L.ecmg_load_state(self.h, str(path).encode()))

    # ---- spawn and goal areas (Simulator.h:92-104) ----------------------
    def add_spawn_area(self, position, half_size, config: dict | None = None, ID: int = -1) -> int:
        """Simulator::AddSpawnArea (Simulator.cpp:336-360); config keys as
        SpawnConfiguration (Area.h:82-88), reference defaults 5 / 10 / 5 / 10."""
        cfg = _lib.SpawnConfig(5.0, 10.0, 5.0, 10.0)
        for k, v in (config or {}).items():
            setattr(cfg, k, float(v))
        out = C.c_int()
        self._ck(self.L.ecmg_add_spawn_area(self.h, float(position[0]), float(position[1]), float(half_size[0]),
                                            float(half_size[1]), C.byref(cfg), int(ID), C.byref(out)))
        return out.value

    def add_goal_area(self, position, half_size, ID: int = -1) -> int:
        """Simulator::AddGoalArea (Simulator.cpp:362-381)"""
        out = C.c_int()
        self._ck(self.L.ecmg_add_goal_area(self.h, float(position[0]), float(position[1]), float(half_size[0]),
                                           float(half_size[1]), int(ID), C.byref(out)))
        return out.value

    def remove_area(self, area_type: int, ID: int):
        """Simulator::RemoveArea; area_type 2 = SPAWN, 3 = GOAL (Area.h:11-18)"""
        self._ck(self.L.ecmg_remove_area(self.h, int(area_type), int(ID)))

    def connect_spawn_goal_areas(self, spawn_id: int, goal_id: int, spawn_rate: float = 0.0):
        self._ck(self.L.ecmg_connect_areas(self.h, int(spawn_id), int(goal_id), float(spawn_rate)))

    def deconnect_spawn_goal_areas(self, spawn_id: int, goal_id: int):
        self._ck(self.L.ecmg_disconnect_areas(self.h, int(spawn_id), int(goal_id)))

    def set_area(self, area_type: int, ID: int, position, half_size):
        self._ck(self.L.ecmg_set_area(self.h, int(area_type), int(ID), float(position[0]), float(position[1]),
                                      float(half_size[0]), float(half_size[1])))

    def get_area(self, area_type: int, ID: int) -> dict:
        info = _lib.AreaInfo()
        cap = 256
        g, r, t = np.zeros(cap, I32), np.zeros(cap, F32), np.zeros(cap, F32)
        self._ck(self.L.ecmg_get_area(self.h, int(area_type), int(ID), C.byref(info), _ptr(g), _ptr(r), _ptr(t), cap))
        c = info.config
        return dict(id=info.id, position=(info.x, info.y), half_size=(info.half_w, info.half_h),
                    config=dict(preferred_speed_min=c.preferred_speed_min, preferred_speed_max=c.preferred_speed_max,
                                clearance_min=c.clearance_min, clearance_max=c.clearance_max),
                    connected=g[:min(cap, info.n_connected)].tolist(), spawn_rate=r[:min(cap, info.n_timers)].tolist(),
                    time_since_last_spawn=t[:min(cap, info.n_timers)].tolist())

    def area_ids(self, area_type: int) -> list:
        n = C.c_int()
        self._ck(self.L.ecmg_area_ids(self.h, int(area_type), None, 0, C.byref(n)))
        ids = np.zeros(max(1, n.value), I32)
        self._ck(self.L.ecmg_area_ids(self.h, int(area_type), _ptr(ids), n.value, C.byref(n)))
        return ids[:n.value].tolist()

    def set_spawn_rng(self, fn=None, rand_max: int = 2147483647):
        """fn() -> int in [0, rand_max] replaces the C library's rand();
        None restores it"""
        if fn is None:
            self._rand_cb = None
            self._ck(self.L.ecmg_set_spawn_rng(self.h, _lib.RAND_FN(), None, 0))
            return
        self._rand_cb = _lib.RAND_FN(lambda user: int(fn()))
        self._ck(self.L.ecmg_set_spawn_rng(self.h, self._rand_cb, None, int(rand_max)))

    def push_spawn_random(self, values):
        v = _a(values, I32)
        self._ck(self.L.ecmg_push_spawn_random(self.h, _ptr(v), int(v.size)))

    def spawn_random_pending(self) -> int:
        n = C.c_longlong()
        self._ck(self.L.ecmg_spawn_random_pending(self.h, C.byref(n)))
        return n.value

    def update_spawn_areas(self) -> _lib.TickStats:
        """Simulator::UpdateSpawnAreas alone (Simulator.cpp:494-536)"""
        st = _lib.TickStats()
        self._ck(self.L.ecmg_update_spawn_areas(self.h, C.byref(st)))
        return st

    def get_spawned(self):
        """(slots, start [n,2], goal [n,2]) of the last spawn stage"""
        n = C.c_int()
        self._ck(self.L.ecmg_get_spawned(self.h, None, None, None, 0, C.byref(n)))
        m = n.value
        sl, a, b = np.zeros(max(1, m), I32), np.zeros((max(1, m), 2), F32), np.zeros((max(1, m), 2), F32)
        self._ck(self.L.ecmg_get_spawned(self.h, _ptr(sl), _ptr(a), _ptr(b), m, C.byref(n)))
        return sl[:m], a[:m], b[:m]

    def update(self, dt: float | None = None, ticks: int = 1) -> _lib.TickStats:
        """Simulator::Update; like the reference, dt is ignored and the step
        time given at construction is used (Simulator.cpp:313-323)."""
        st = _lib.TickStats()
        self._ck(self.L.ecmg_tick(self.h, int(ticks), C.byref(st)))
        return st

    def reset(self):
        self._ck(self.L.ecmg_reset(self.h))

    def set_path(self, idx: int, path):
        p = _a(path, F32).reshape(-1, 2)
        self._ck(self.L.ecmg_set_path(self.h, int(idx), _ptr(p), p.shape[0]))

    def get_path(self, idx: int, cap: int = 4096) -> np.ndarray:
        out = np.zeros((cap, 2), F32)
        n = C.c_int()
        self._ck(self.L.ecmg_get_path(self.h, int(idx), _ptr(out), cap, C.byref(n)))
        return out[: min(n.value, cap)].copy()

    def find_path(self, start, goal, clearance, cap=4096):
        out = np.zeros((cap, 2), F32)
        n = C.c_int()
        rc = self.L.ecmg_find_path(self.h, float(start[0]), float(start[1]), float(goal[0]), float(goal[1]),
                                   float(clearance), _ptr(out), cap, C.byref(n))
        return None if rc else out[: min(n.value, cap)].copy()

    # -- getters (Simulator.h:114-126) -------------------------------------
    def _get(self, field, shape, dt):
        out = np.zeros(shape, dt)
        self._ck(self.L.ecmg_get_state(self.h, FIELD[field], _ptr(out)))
        return out

    def set_host_mirror(self, on: bool = True):
        """ecmg_set_host_mirror: every tick ends by writing the host views of
        the positions and velocities (view() of those fields then returns
        without a copy, and the arrays change with every tick)"""
        self._ck(self.L.ecmg_set_host_mirror(self.h, 1 if on else 0))

    def view(self, field: str):
        """Read-only numpy view of the library's host copy of a field
        (ecmg_host_view), as the reference's getters return pointers into the
        Simulator's arrays: refreshed by this call, overwritten by the next
        view of the same field (and by every tick for the positions and
        velocities while set_host_mirror is on)."""
        p = C.c_void_p()
        self._ck(self.L.ecmg_host_view(self.h, FIELD[field], C.byref(p)))
        n = self.max_agents
        if field == "active":
            arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(n,))
        elif field in ("clearance", "speed"):
            arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_float)), shape=(n,))
        else:
            arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_float)), shape=(n, 2))
        arr.flags.writeable = False
        return arr

    def get_num_agents(self) -> int:
        n = C.c_int()
        self._ck(self.L.ecmg_get_counts(self.h, C.byref(n), None, None))
        return n.value

    def get_last_index(self) -> int:
        n = C.c_int()
        self._ck(self.L.ecmg_get_counts(self.h, None, C.byref(n), None))
        return n.value

    def get_position_data(self):
        return self._get("position", (self.max_agents, 2), F32)

    def get_velocity_data(self):
        return self._get("velocity", (self.max_agents, 2), F32)

    def get_preferred_velocity_data(self):
        return self._get("pref_velocity", (self.max_agents, 2), F32)

    def get_attraction_point_data(self):
        return self._get("attraction", (self.max_agents, 2), F32)

    def get_clearance_data(self):
        return self._get("clearance", (self.max_agents,), F32)

    def get_speed_data(self):
        return self._get("speed", (self.max_agents,), F32)

    def get_active_flags(self):
        return self._get("active", (self.max_agents,), U8)

    def set_state(self, field: str, arr):
        dt = U8 if field == "active" else F32
        arr = _a(arr, dt)
        self._ck(self.L.ecmg_set_state(self.h, FIELD[field], _ptr(arr)))

    # -- inspection --------------------------------------------------------
    def set_record(self, on: bool = True):
        self._ck(self.L.ecmg_set_record(self.h, int(on)))

    def get_record(self) -> dict:
        n, k = self.max_agents, self.k
        d = dict(nbr_ids=np.zeros((n, k), I32), nbr_count=np.zeros(n, I32), v_orca=np.zeros((n, 2), F32),
                 lp_fail=np.zeros(n, I32), n_constraints=np.zeros(n, I32), n_obst_constraints=np.zeros(n, I32))
        self._ck(self.L.ecmg_get_record(self.h, _ptr(d["nbr_ids"]), _ptr(d["nbr_count"]), _ptr(d["v_orca"]),
                                        _ptr(d["lp_fail"]), _ptr(d["n_constraints"]), _ptr(d["n_obst_constraints"])))
        return d


    # -- learned active-set proposal ---------------------------------------
    def set_proposal(self, model):
        """model: proposal.ProposalModel or None (plain LP)"""
        self._ck(self.L.ecmg_set_proposal(self.h, model.h if model is not None else None))
        self._proposal = model

    def set_proposal_gate(self, min_accept_rate: float = 0.1, pause_ticks: int = 64):
        self._ck(self.L.ecmg_set_proposal_gate(self.h, float(min_accept_rate), int(pause_ticks)))

    def set_proposal_classes(self, cls_by_slot):
        """proposals per slot from a CUDA uint8 tensor (None: off)"""
        ptr = None
        if cls_by_slot is not None:
            if not cls_by_slot.is_cuda or cls_by_slot.numel() < self.max_agents:
                raise ValueError("expected a CUDA uint8 tensor with one class per slot")
            ptr = cls_by_slot.data_ptr()
        self._ck(self.L.ecmg_set_proposal_classes(self.h, ptr))
        self._proposal_classes = cls_by_slot

    def set_trace(self, on: bool = True):
        self._ck(self.L.ecmg_set_trace(self.h, int(on)))

    def get_trace(self, device: bool = False):
        """(features bf16 [n, 96], labels uint8 [n], slots int32 [n]) of the
        last tick in grid order: CUDA tensors with device=True, else numpy
        (features as the raw bf16 bit patterns, uint16)"""
        n = C.c_int()
        self._ck(self.L.ecmg_get_trace(self.h, None, None, None, 0, C.byref(n)))
        cap = self.max_agents
        if device:
            import torch
            x = torch.empty((cap, 96), dtype=torch.bfloat16, device="cuda")
            y = torch.empty(cap, dtype=torch.uint8, device="cuda")
            sl = torch.empty(cap, dtype=torch.int32, device="cuda")
            self._ck(self.L.ecmg_get_trace(self.h, x.data_ptr(), y.data_ptr(), sl.data_ptr(), cap, C.byref(n)))
            m = n.value
            return x[:m], y[:m], sl[:m]
        x = np.zeros((cap, 96), np.uint16)
        y = np.zeros(cap, U8)
        sl = np.zeros(cap, I32)
        self._ck(self.L.ecmg_get_trace(self.h, _ptr(x), _ptr(y), _ptr(sl), cap, C.byref(n)))
        m = n.value
        return x[:m], y[:m], sl[:m]


class BatchSimulator(Simulator):
    """Many independent scenes advanced by one launch sequence per tick
    (ecmg_create_batch).  Scene s owns global slots
    [slot_base(s), slot_base(s) + max_agents[s]); the getters return all slots."""

    def __init__(self, scenes, max_agents_per_scene, sim_step_time: float, **kw):
        self.L = _lib.load()
        p = _lib.default_params(dt=sim_step_time)
        for key, v in kw.items():
            setattr(p, key, int(v) if key in ("use_graph", "lp3d_fp64", "max_neighbors", "block_size") else v)
        self.params = p
        caps = _a(max_agents_per_scene, I32)
        h = C.c_void_p()
        rc = self.L.ecmg_create_batch(C.byref(p), len(scenes), _ptr(caps), C.byref(h))
        if rc:
            raise EcmgError(rc, "ecmg_create_batch failed (is a CUDA device visible?)")
        self.h = h
        self.max_agents = int(caps.sum())
        self.k = int(p.max_neighbors)
        self.scenes = scenes
        self._keep = []
        for s, sc in enumerate(scenes):
            keep, o, e = _scene_structs(sc)
            self._keep.append(keep)
            self._ck(self.L.ecmg_scene_set_obstacles(self.h, s, C.byref(o)))
            self._ck(self.L.ecmg_scene_set_ecm(self.h, s, C.byref(e)))
        self._plan_cb = None

    def add_agents(self, pos, clearance, pref_speed, paths, scene: int = 0) -> np.ndarray:
        pos = _a(pos, F32).reshape(-1, 2)
        n = pos.shape[0]
        clr, spd = _a(clearance, F32), _a(pref_speed, F32)
        lens = np.array([len(p) for p in paths], I32)
        offs = np.zeros(n, I32)
        if n:
            offs[1:] = np.cumsum(lens)[:-1]
        xy = _a(np.concatenate([np.asarray(p, F32).reshape(-1, 2) for p in paths], 0), F32) if n else \
            np.zeros((0, 2), F32)
        out = np.zeros(n, I32)
        self._ck(self.L.ecmg_scene_add_agents(self.h, int(scene), n, _ptr(pos), _ptr(clr), _ptr(spd), _ptr(offs),
                                              _ptr(lens), _ptr(xy), _ptr(out)))
        return out

    def scene_counts(self, scene: int) -> dict:
        v = [C.c_int() for _ in range(4)]
        self._ck(self.L.ecmg_scene_counts(self.h, int(scene), *[C.byref(x) for x in v]))
        return dict(num_agents=v[0].value, last_index=v[1].value, slot_base=v[2].value, slot_count=v[3].value)


def autotune(sim: Simulator, ticks_per_trial: int = 2) -> dict:
    """ecmg_autotune: pick block size, agents per warp grab and grid cell."""
    r = _lib.TuneResult()
    sim._ck(sim.L.ecmg_autotune(sim.h, int(ticks_per_trial), C.byref(r)))
    return dict(block_size=r.block_size, agents_per_warp_grab=r.agents_per_warp_grab,
                grid_cell_scale=r.grid_cell_scale, best_tick_ms=r.best_tick_ms, trials=r.trials,
                lp_mode={0: "thread", 1: "warp", 2: "fused"}[r.lp_mode], occupancy_divisor=r.occupancy_divisor,
                neighbor_blocks_per_sm=r.neighbor_blocks_per_sm)


def set_launch(sim: Simulator, block_size: int, agents_per_warp_grab: int, grid_cell_scale: float,
               occupancy_divisor: int = 1, neighbor_blocks_per_sm: int = 8):
    sim._ck(sim.L.ecmg_set_launch(sim.h, int(block_size), int(agents_per_warp_grab), float(grid_cell_scale)))
    if occupancy_divisor != 1:
        sim._ck(sim.L.ecmg_set_occupancy(sim.h, int(occupancy_divisor)))
    sim._ck(sim.L.ecmg_set_neighbor_blocks(sim.h, int(neighbor_blocks_per_sm)))


def set_lp_mode(sim: Simulator, mode: str = "warp", agents_per_warp_grab: int = 4):
    """per-agent kernel layout: "thread" (one thread per agent), "warp"
    (one warp per agent) or "fused" (one thread per agent, the neighbour
    search in the same kernel); results are identical"""
    m = {"thread": 0, "warp": 1, "fused": 2}[mode]
    sim._ck(sim.L.ecmg_set_lp_mode(sim.h, m, int(agents_per_warp_grab)))


def set_neighbor_mode(sim: Simulator, mode: str = "kdtree"):
    """'exact' (default): the exact k nearest within neighbor_dist;
    'kdtree': the reference's kd-tree query with its neighbour cache, the
    lists of the unmodified Simulator::Update (ecmg_set_neighbor_mode)"""
    m = {"exact": 0, "kdtree": 1}[mode]
    sim._ck(sim.L.ecmg_set_neighbor_mode(sim.h, m))


def set_replan_overlap(sim: Simulator, mode=1):
    """re-plan searches overlapping the next tick (ecmg_set_replan_overlap;
    same results in every mode): 1 (default) when a search outlasts its
    tick, 2 always, 0 / False never"""
    sim._ck(sim.L.ecmg_set_replan_overlap(sim.h, int(mode)))


def set_planner_mode(sim: Simulator, mode: str = "reference"):
    """built-in planner of re-plans and spawns: 'reference' (default, the
    reference planner's paths) or 'fast' (opt-in), ecmg_set_planner_mode"""
    sim._ck(sim.L.ecmg_set_planner_mode(sim.h, {"fast": 0, "reference": 1}[mode]))
