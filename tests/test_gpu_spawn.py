"""Spawn areas on the GPU against the restatement of UpdateSpawnAreas
(oracle/spawn_oracle.py, itself pinned to the reference's code): every tick,
the restatement runs on the library's agent state at the start of the tick
and the library's spawn stage (inside ecmg_tick) must place the same agents
in the same slots at the same locations with the same goals, keep the same
timers and consume the same random values."""
import numpy as np
import pytest

import spawn_cases as cases
import spawn_oracle as so

pytestmark = pytest.mark.gpu

F32 = np.float32
DT = 1.0 / 60.0
ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def _same(a, b):
    """equal float32 values, NaN where the other has NaN (a NaN's payload
    differs between CPU architectures)"""
    a, b = np.asarray(a, F32), np.asarray(b, F32)
    return a.shape == b.shape and np.array_equal(a, b, equal_nan=True)


class Pair:
    """the library and the restatement, driven side by side"""

    def __init__(self, scene, max_agents, setup, initial=None, seed=3, n_values=400000, k=10, **kw):
        from ecmgenerator_gb300.simulator import Simulator

        self.sim = Simulator(scene, max_agents, DT, max_neighbors=k, **ORCA, **kw)
        self.areas = so.Areas()
        self.info = setup(scene, cases.Ops(self.sim, "lib"))
        assert setup(scene, cases.Ops(self.areas, "oracle")) == self.info
        self.free = list(range(max_agents - 1, -1, -1))
        if initial is not None:
            pos, clr, spd, paths = initial
            slots = self.sim.add_agents(pos, clr, spd, paths)
            for s in slots:
                assert s == self.free.pop()
        rng = np.random.default_rng(seed)
        self.stream = rng.integers(0, 2147483648, n_values, dtype=np.int64)
        self.sim.push_spawn_random(self.stream.astype(np.int32))
        self.head = 0
        self.totals = dict(spawned=0, failed=0, refused=0)

    def plan_ok(self, start, goal, clr):
        return self.sim.find_path((float(start[0]), float(start[1])), (float(goal[0]), float(goal[1])),
                                  float(clr)) is not None

    def tick(self, t):
        sim = self.sim
        pos = sim.get_position_data().copy()
        active = sim.get_active_flags().astype(bool)
        spawns, self.head, counts = so.spawn_stage(self.areas, pos, active, self.free, self.stream, self.head, DT,
                                                   2147483647, plan_ok=self.plan_ok)
        st = sim.update()
        slots, starts, goals = sim.get_spawned()
        assert [s[0] for s in spawns] == slots.tolist(), t
        for j, (slot, start, goal, clr, spd) in enumerate(spawns):
            assert np.array_equal(starts[j], np.array(start, F32)), (t, slot)
            assert np.array_equal(goals[j], np.array(goal, F32)), (t, slot)
            assert sim.get_clearance_data()[slot] == clr and sim.get_speed_data()[slot] == spd
        assert (st.spawned, st.spawn_failed, st.spawn_refused) == (counts["spawned"], counts["failed"],
                                                                   counts["refused"]), t
        for k in self.totals:
            self.totals[k] += counts[k]
        for sid, a in self.areas.spawn.items():
            g = sim.get_area(2, sid)
            assert g["connected"] == a["goals"]
            assert _same(g["spawn_rate"], a["rate"])
            assert _same(g["time_since_last_spawn"], a["since"]), (t, sid)
        assert sorted(self.areas.spawn) == sim.area_ids(2)
        assert len(self.stream) - sim.spawn_random_pending() == self.head, t
        # DestroyAgent of this tick: the free stack takes the slots in slot order
        after = sim.get_active_flags().astype(bool)
        before = active.copy()
        for s in slots:
            before[s] = True
        self.free.extend(np.nonzero(before & ~after)[0].tolist())
        return st

    def close(self):
        self.sim.close()


def _c1(n_agents, seed=7):
    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300.simulator import Planner

    cfg = ag.scaled("c1", agents=n_agents)
    scene = ag.build_scene(cfg, seed=1)
    st = ag.spawn_agents(cfg, scene, seed)
    n = st.num_agents
    paths = Planner(scene).find_paths(st.pos[:n], st.goal[:n], st.clear[:n])
    paths = [p if p is not None else np.stack([st.pos[i], st.goal[i]]) for i, p in enumerate(paths)]
    return scene, (st.pos[:n], st.clear[:n], st.pref_speed[:n], paths)


def test_spawn_stage_matches_oracle_on_moving_crowd(lib):
    scene, init = _c1(1000)
    p = Pair(scene, 1600, lambda s, ops: cases.standard_areas(s, ops), initial=init)
    for t in range(150):
        p.tick(t)
    print(p.totals)
    assert p.totals["spawned"] > 150, p.totals
    assert p.totals["refused"] <= 2, p.totals
    p.close()


def test_spawn_blocked_locations_and_slot_exhaustion(lib):
    """the left half of a spawn area is covered by agents (locations are
    rejected and retried); few slots, so spawns are refused later on"""
    from ecmgenerator_gb300 import agents as ag

    scene = ag.build_scene(ag.scaled("c1"), seed=1)
    probe = cases.standard_areas(scene, cases.Ops(so.Areas(), "oracle"))
    (_, a0, h0) = probe["spawn"][0]
    crowd = cases.crowd_in((a0[0] - h0[0] / 2, a0[1]), (h0[0] / 2, h0[1]), 0.8, 400)
    n = crowd.shape[0]
    init = (crowd, np.full(n, 0.3, F32), np.zeros(n, F32), [np.stack([c, c]) for c in crowd])
    # delete radius 0: the standing crowd (path = its own position) stays
    p = Pair(scene, n + 60, lambda s, ops: cases.standard_areas(s, ops), initial=init, delete_radius=0.0)
    for t in range(90):
        p.tick(t)
    assert p.totals["failed"] > 0 and p.totals["refused"] > 0, p.totals
    p.close()


def test_spawn_area_edits_between_ticks(lib):
    """a zero rate (the timer becomes NaN, nothing spawns),
    DeconnectSpawnGoalAreas leaving rates and timers behind (later goals are
    paired with earlier rates), a removed spawn area, a removed goal area
    (goal (0, 0)) and a moved area"""
    scene, init = _c1(500)
    p = Pair(scene, 1200, lambda s, ops: cases.standard_areas(s, ops), initial=init)
    s0, s1 = p.info["spawn"][0][0], p.info["spawn"][1][0]
    q0, q1, q2 = p.info["goal"]
    for t in range(120):
        for ops in (cases.Ops(p.sim, "lib"), cases.Ops(p.areas, "oracle")):
            if t == 10:
                ops.connect(s1, q1)  # rate 0
            if t == 20:
                ops.disconnect(s0, q0)
            if t == 40:
                ops.remove(2, s1)
            if t == 55:
                ops.connect(s0, q2)
            if t == 80:
                ops.remove(3, q2)
        if t == 90:
            x, y = p.info["spawn"][0][1]
            p.sim.set_area(2, s0, (x + 0.5, y - 0.25), (3.0, 2.0))
            a = p.areas.spawn[s0]
            a["x"], a["y"], a["hw"], a["hh"] = F32(x + 0.5), F32(y - 0.25), F32(3.0), F32(2.0)
        p.tick(t)
        if t == 30:
            assert np.isnan(p.sim.get_area(2, s1)["time_since_last_spawn"][2])
    assert p.totals["spawned"] > 40, p.totals
    p.close()


def test_spawn_many_per_tick_uses_several_windows(lib):
    """hundreds of agents due per tick: the candidate locations of a stage
    exceed one launch's table, so the stage checks several windows"""
    from ecmgenerator_gb300 import agents as ag

    scene = ag.build_scene(ag.scaled("c1"), seed=1)

    def setup(s, ops):
        a = cases.free_rect(s, 4.0, 4.0, seed=11)
        b = cases.free_rect(s, 4.0, 4.0, seed=12, avoid=[a + (4.0, 4.0)])
        g = cases.free_rect(s, 3.0, 3.0, seed=13, avoid=[a + (4.0, 4.0), b + (4.0, 4.0)])
        cfg = dict(clearance_min=0.12, preferred_speed_min=1.0)
        sa, sb = ops.spawn(*a, 4.0, 4.0, cfg), ops.spawn(*b, 4.0, 4.0, cfg)
        q = ops.goal(*g, 3.0, 3.0)
        ops.connect(sa, q, 40000.0)
        ops.connect(sb, q, 25000.0)
        return dict(a=a)

    p = Pair(scene, 6000, setup)
    for t in range(6):
        p.tick(t)
    assert p.totals["spawned"] > 1500 and p.totals["failed"] > 0, p.totals
    p.close()


def test_libc_rand_default_source(lib):
    """without queued values the stage draws from rand(); srand gives the
    reference's sequence"""
    import ctypes

    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300.simulator import Simulator

    libc = ctypes.CDLL(None)
    scene = ag.build_scene(ag.scaled("c1"), seed=1)
    sim = Simulator(scene, 400, DT, **ORCA)
    areas = so.Areas()
    cases.standard_areas(scene, cases.Ops(sim, "lib"))
    cases.standard_areas(scene, cases.Ops(areas, "oracle"))
    libc.srand(21)
    stream = np.array([libc.rand() for _ in range(20000)], np.int64)
    libc.srand(21)
    free = list(range(399, -1, -1))
    head = 0
    for t in range(30):
        pos = sim.get_position_data().copy()
        active = sim.get_active_flags().astype(bool)
        spawns, head, _ = so.spawn_stage(areas, pos, active, free, stream, head, DT, 2147483647)
        sim.update()
        slots, starts, _ = sim.get_spawned()
        assert slots.tolist() == [s[0] for s in spawns]
        assert np.array_equal(starts, np.array([s[1] for s in spawns], F32).reshape(-1, 2))
    # values drawn ahead of use stay queued
    assert head + sim.spawn_random_pending() >= head
    sim.close()


def test_spawn_refused_without_path_frees_its_location(lib):
    """a spawn area half inside a box: locations in the box get no path, so
    those spawns are refused, and the agents after them may use the space a
    refused agent would have blocked (the stage replays its walk after
    planning)"""
    from ecmgenerator_gb300 import agents as ag

    scene = ag.build_scene(ag.scaled("c1"), seed=1)
    bx = scene.boxes[int(np.argmax(scene.boxes[:, 2] * scene.boxes[:, 3]))]

    def setup(s, ops):
        cx, cy, hx, hy = (float(v) for v in bx)
        a = ops.spawn(cx + hx, cy, hx, hy, dict(clearance_min=1.0, preferred_speed_min=1.2))
        g = cases.free_rect(s, 2.0, 2.0, seed=21)
        q = ops.goal(*g, 2.0, 2.0)
        ops.connect(a, q, 300.0)
        return dict(a=a)

    p = Pair(scene, 800, setup)
    for t in range(40):
        p.tick(t)
    assert p.totals["refused"] > 10 and p.totals["spawned"] > 10, p.totals
    p.close()


@pytest.mark.parametrize("mode", ["exact", "kdtree"])
def test_spawn_areas_inside_full_ticks_match_oracle(port, lib, mode):
    """The whole Simulator::Update with spawn areas: the restatement's spawn
    stage feeds the C oracle's tick (exact kNN or the reference's kd-tree with
    its carried cache), the library runs ecmg_tick; positions, velocities and
    neighbour lists stay identical while agents keep appearing."""
    from ecmgenerator_gb300.simulator import Simulator, set_neighbor_mode

    scene, (pos, clr, spd, paths) = _c1(300)
    n = pos.shape[0]
    slots = 700
    sim = Simulator(scene, slots, DT, max_neighbors=10, **ORCA)
    if mode == "kdtree":
        set_neighbor_mode(sim, "kdtree")
    sim.set_record(True)
    sim.add_agents(pos, clr, spd, paths)
    areas = so.Areas()
    cases.standard_areas(scene, cases.Ops(sim, "lib"))
    cases.standard_areas(scene, cases.Ops(areas, "oracle"))
    stream = np.random.default_rng(17).integers(0, 2147483648, 200000, dtype=np.int64)
    sim.push_spawn_random(stream.astype(np.int32))
    # the oracle's state
    from ecmgenerator_gb300 import agents as ag

    st = ag.AgentState.empty(slots)
    st.pos[:n], st.clear[:n], st.pref_speed[:n], st.active[:n] = pos, clr, spd, 1
    st.num_agents, st.last_idx = n, n - 1
    st.set_paths(list(paths) + [None] * (slots - n))
    free = list(range(slots - 1, n - 1, -1))
    O, E = port.obstacles(scene), port.ecm(scene.ecm)
    P = port.params(k=10, libm=0, knn_mode=1 if mode == "kdtree" else 0, **ORCA)
    kd = port.kdtree(10) if mode == "kdtree" else None
    head, spawned = 0, 0
    same = lambda a, b: np.array_equal(a, b, equal_nan=True)  # noqa: E731
    for t in range(90):
        # UpdateMaxAgentIndex, then UpdateSpawnAreas on the oracle's state
        while st.last_idx >= 0 and not st.active[st.last_idx]:
            st.last_idx -= 1
        spawns, head, _ = so.spawn_stage(areas, st.pos, st.active.astype(bool), free, stream, head, DT, 2147483647,
                                         plan_ok=lambda a, b, c: sim.find_path(
                                             (float(a[0]), float(a[1])), (float(b[0]), float(b[1])), float(c)) is not None)
        sim.update()
        lib_slots, _, _ = sim.get_spawned()
        assert lib_slots.tolist() == [sp[0] for sp in spawns], t
        for slot, start, goal, c, v in spawns:
            st.pos[slot] = start
            st.vel[slot] = 0.0
            st.pref_vel[slot] = 0.0
            st.clear[slot], st.pref_speed[slot], st.active[slot] = c, v, 1
            st.num_agents += 1
            st.last_idx = max(st.last_idx, slot)
            st.replace_path(slot, sim.get_path(slot))
        spawned += len(spawns)
        before = st.active.copy()
        res = port.tick(O, E, st, P, kd=kd)
        live = st.active == 1
        rec = sim.get_record()
        assert np.array_equal(rec["nbr_ids"][live], res["nbr_ids"][live]), t
        assert np.array_equal(sim.get_active_flags(), st.active), t
        assert same(sim.get_position_data(), st.pos), t
        assert same(sim.get_velocity_data(), st.vel), t
        free.extend(np.nonzero((before == 1) & (st.active == 0))[0].tolist())
        for s_ in res["replan"]:
            st.replace_path(int(s_), sim.get_path(int(s_)))
        if np.isnan(st.pos[st.active == 1]).any():
            break
    if kd is not None:
        port.lib.og_kdtree_destroy(kd)
    sim.close()
    assert spawned > 50, spawned
