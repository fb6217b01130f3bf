"""Spawn areas: the restatement (oracle/spawn_oracle.py) pinned against the
reference's own UpdateSpawnAreas and area bookkeeping (oracle/_ref, built
from the reference sources), driven by the C library's rand() as the
reference is.  Checked per stage: which slots are filled (LIFO), start
locations, goals (the planned path's last point), clearance and speed, the
spawn timers (bit patterns, NaN included), the free-slot stack and, at the
end, how many random values were consumed."""
import numpy as np
import pytest

import oracle as orc
import spawn_cases as cases
import spawn_oracle as so
from ecmgenerator_gb300 import agents as ag

F32 = np.float32
DT = 1.0 / 60.0


def test_spawn_count_conversion():
    assert so.spawn_count(F32(2.9)) == 2
    assert so.spawn_count(F32(-0.5)) == 0
    assert so.spawn_count(F32(np.nan)) == so.INT_MIN
    assert so.spawn_count(F32(3e9)) == so.INT_MIN
    assert so.spawn_count(F32(-2147483648.0)) == -2147483648


def test_area_point_stays_in_area():
    rng = np.random.default_rng(0)
    for _ in range(2000):
        x, y, hw, hh = rng.uniform(-50, 50), rng.uniform(-50, 50), rng.uniform(0.1, 9), rng.uniform(0.1, 9)
        v1, v2 = rng.integers(0, 2147483648, 2)
        px, py = so.area_point(x, y, hw, hh, v1, v2, 2147483647)
        assert F32(x) - F32(hw) <= px <= F32(x) + F32(hw) + 1e-5
        assert F32(y) - F32(hh) <= py <= F32(y) + F32(hh) + 1e-5


def _live(state):
    """active flags up to m_LastEntityIdx: Simulator::Initialize leaves
    m_ActiveAgents uninitialised (Simulator.cpp:24) and every loop of the
    reference stops at m_LastEntityIdx"""
    a = state["active"].astype(bool)
    a[state["last_idx"] + 1:] = False
    return a


def _bits(a):
    return np.asarray(a, F32).view(np.int32)


def _pin(max_agents, setup, stages, initial=(), between=None, seed=5, n_values=200000):
    scene = ag.build_scene(ag.scaled("c1"), seed=1)
    ref = orc.Ref(scene, max_agents, DT, 5, 2.0, 2.0)
    areas = so.Areas()
    info = setup(scene, cases.Ops(ref, "ref"))
    assert setup(scene, cases.Ops(areas, "oracle")) == info
    free = list(range(max_agents - 1, -1, -1))
    pos = np.zeros((max_agents, 2), F32)
    active = np.zeros(max_agents, bool)
    for p in initial:
        slot = ref.spawn_direct(float(p[0]), float(p[1]), 0.3, 1.2, np.array([p, p], F32))
        assert slot == free.pop()
        pos[slot] = p
        active[slot] = True
    ref.srand(seed)
    stream = np.array([ref.rand() for _ in range(n_values)], np.int64)
    ref.srand(seed)
    rand_max = ref.rand_max()
    head = 0
    totals = dict(spawned=0, failed=0, refused=0)
    for t in range(stages):
        if between:
            between(t, cases.Ops(ref, "ref"), info)
            between(t, cases.Ops(areas, "oracle"), info)
        before = ref.get_state()
        ref.update_spawn_areas()
        after = ref.get_state()
        spawns, head, counts = so.spawn_stage(areas, pos, active, free, stream, head, DT, rand_max)
        for k in totals:
            totals[k] += counts[k]
        new = np.nonzero(_live(after) & ~_live(before))[0]
        assert sorted(s[0] for s in spawns) == new.tolist(), t
        for slot, start, goal, clr, spd in spawns:
            assert np.array_equal(after["pos"][slot], np.array(start, F32)), (t, slot)
            assert after["clear"][slot] == clr and after["pref_speed"][slot] == spd
            path = ref.get_path(slot)
            if len(path):
                assert np.array_equal(path[-1], np.array(goal, F32)), (t, slot, path[-1], goal)
            pos[slot] = start
            active[slot] = True
        for sid, a in areas.spawn.items():
            r = ref.spawn_area_state(sid)
            assert r is not None and r["goals"] == a["goals"]
            assert np.array_equal(_bits(r["rate"]), _bits(a["rate"]))
            assert np.array_equal(_bits(r["since"]), _bits(a["since"])), (t, sid, r["since"], a["since"])
        top, size = ref.free_top()
        assert size == len(free) and top == (free[-1] if free else -1)
    # the next values the reference's generator gives are the first ones the
    # restatement has not consumed
    assert [ref.rand() for _ in range(3)] == stream[head:head + 3].tolist()
    ref.close()
    return totals, head


def _standard(scene, ops):
    return cases.standard_areas(scene, ops)


@pytest.mark.ref
def test_pinned_standard_areas_with_blocked_locations():
    scene = ag.build_scene(ag.scaled("c1"), seed=1)
    probe = cases.standard_areas(scene, cases.Ops(so.Areas(), "oracle"))
    (s0, a0, h0) = probe["spawn"][0]
    # the left half of spawn area 0 is covered by a lattice of agents (holes
    # between lattice points stay valid), so locations are rejected and retried
    crowd = cases.crowd_in((a0[0] - h0[0] / 2, a0[1]), (h0[0] / 2, h0[1]), 0.8, 400)
    totals, head = _pin(600, _standard, 90, initial=crowd)
    assert totals["spawned"] > 100 and totals["failed"] > 0, totals
    assert head > 3 * 2 * totals["spawned"]  # rejected locations consumed values


@pytest.mark.ref
def test_pinned_disconnect_remove_and_zero_rate():
    def between(t, ops, info):
        s0, s1 = info["spawn"][0][0], info["spawn"][1][0]
        q0, q1, q2 = info["goal"]
        if t == 20:
            ops.disconnect(s0, q0)  # goals [q1], rates stay [40, 25]
        if t == 35:
            ops.remove(2, s1)
        if t == 50:
            ops.connect(s0, q2)  # default rate 0, paired with the stale rate 25
        if t == 70:
            ops.disconnect(s0, 99)  # not connected: nothing
            ops.disconnect(5, q1)  # spawn ID not below the area count: ignored
    totals, _ = _pin(600, _standard, 100, between=between)
    assert totals["spawned"] > 50, totals


@pytest.mark.ref
def test_pinned_slot_exhaustion():
    totals, head = _pin(40, _standard, 60)
    assert totals["refused"] > 0, totals


@pytest.mark.ref
def test_pinned_crowded_area_fails():
    def setup(scene, ops):
        a = cases.free_rect(scene, 2.5, 2.5, seed=2)
        g = cases.free_rect(scene, 2.0, 2.0, seed=3, avoid=[a + (2.5, 2.5)])
        s = ops.spawn(*a, 2.5, 2.5, dict(clearance_min=2.0, preferred_speed_min=1.0))
        q = ops.goal(*g, 2.0, 2.0)
        ops.connect(s, q, 60.0)
        return dict(a=a)
    scene = ag.build_scene(ag.scaled("c1"), seed=1)
    a = cases.free_rect(scene, 2.5, 2.5, seed=2)
    crowd = cases.crowd_in(a, (4.0, 4.0), 1.0, 200)
    totals, head = _pin(400, setup, 20, initial=crowd)
    assert totals["spawned"] == 0 and totals["failed"] == 20, totals
    assert head == 20 * 10 * 3
