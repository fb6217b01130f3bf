"""ecmg_set_host_mirror: every tick ends by writing the page-locked host
positions and velocities (the reference's getters point into arrays that
Update itself writes, Simulator.h:114-126).  The views must hold what the
device holds after every tick -- plain ticks, ticks with spawn areas,
carried re-plans with their fix-up launch -- and after every write that is
not a tick (adding and spawning agents, set_state, load_state)."""
import numpy as np
import pytest

import spawn_cases as cases

pytestmark = pytest.mark.gpu

F32 = np.float32
DT = 1.0 / 60.0
ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def _crowd(n, seed):
    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300.simulator import Planner

    cfg = ag.scaled("c1", agents=n)
    scene = ag.build_scene(cfg, seed=seed)
    st = ag.spawn_agents(cfg, scene, seed=seed)
    m = st.num_agents
    paths = Planner(scene).find_paths(st.pos[:m], st.goal[:m], st.clear[:m])
    paths = [p if p is not None else np.stack([st.pos[i], st.goal[i]]) for i, p in enumerate(paths)]
    for i in range(0, m, 5):
        # a path that starts beyond the goal (its disk meets no segment): the
        # agent re-plans at once
        g = st.goal[i].astype(np.float64)
        d = g - st.pos[i]
        far = np.clip(g + 30.0 * d / max(np.hypot(*d), 1e-6), 1.0, scene.width - 1.0)
        paths[i] = np.stack([far, g]).astype(F32)
    return cfg, scene, st, paths


def _check(sim, held, t):
    """the views (fresh, and the arrays held from before) equal the device
    state copied out by ecmg_get_state"""
    pos, vel = sim.get_position_data(), sim.get_velocity_data()
    assert np.array_equal(sim.view("position"), pos), t
    assert np.array_equal(sim.view("velocity"), vel), t
    assert np.array_equal(held[0], pos), t
    assert np.array_equal(held[1], vel), t


def test_mirror_follows_ticks_spawns_and_host_writes(lib):
    from ecmgenerator_gb300.simulator import Simulator, set_replan_overlap

    cfg, scene, st, paths = _crowd(800, 3)
    n = st.num_agents
    sims = []
    for mirror in (True, False):
        sim = Simulator(scene, n + 400, DT, max_neighbors=cfg["k"], **ORCA)
        set_replan_overlap(sim, 2)  # every re-plan carried into a fix-up launch
        sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths)
        cases.standard_areas(scene, cases.Ops(sim, "lib"))
        sim.push_spawn_random(np.random.default_rng(5).integers(0, 2147483648, 200000).astype(np.int32))
        if mirror:
            sim.set_host_mirror(True)
        sims.append(sim)
    a, b = sims
    held = (a.view("position"), a.view("velocity"))
    spawned = fixups = 0
    for t in range(60):
        sa, sb = a.update(), b.update()
        assert (sa.spawned, sa.replans, sa.destroyed) == (sb.spawned, sb.replans, sb.destroyed), t
        spawned += sa.spawned
        fixups += sa.replans_host
        # the arrays held since the start follow the ticks without a new call
        assert np.array_equal(held[0], b.get_position_data()), t
        assert np.array_equal(held[1], b.get_velocity_data()), t
        if t == 20:
            # a host write (one agent added) makes the views stale once
            for sim in sims:
                sim.spawn_agent((float(st.pos[0, 0]), float(st.pos[0, 1])),
                                (float(st.goal[0, 0]), float(st.goal[0, 1])), 0.3, 1.3)
            _check(a, held, t)
        if t == 30:
            pos = b.get_position_data().copy()
            live = b.get_active_flags() == 1
            pos[live] += F32(0.01)
            for sim in sims:
                sim.set_state("position", pos)
            _check(a, held, t)
        _check(a, held, t)
    assert spawned > 0 and fixups > 0, (spawned, fixups)
    # turned off: every view call copies, the ticks leave the arrays alone
    a.set_host_mirror(False)
    before = held[0].copy()
    a.update()
    assert np.array_equal(held[0], before)
    assert np.array_equal(a.view("position"), a.get_position_data())
    a.close()
    b.close()


def test_mirror_after_load_state(lib, tmp_path):
    from ecmgenerator_gb300.simulator import Simulator

    cfg, scene, st, paths = _crowd(300, 4)
    n = st.num_agents
    sim = Simulator(scene, n, DT, max_neighbors=cfg["k"], **ORCA)
    sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths)
    sim.update(ticks=3)
    f = str(tmp_path / "s.bin")
    sim.save_state(f)
    want = sim.get_position_data().copy()
    sim.set_host_mirror(True)
    held = sim.view("position")
    sim.update(ticks=5)
    assert np.array_equal(held, sim.get_position_data())
    sim.load_state(f)
    assert np.array_equal(sim.view("position"), want)
    assert np.array_equal(held, want)
    sim.close()
