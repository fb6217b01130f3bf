"""Re-plans overlapping the next tick (ecmg_set_replan_overlap): the searches
of tick t run on host threads while tick t+1's kernels run; tick t+1 skips
those agents and steps them in a fix-up launch once their paths are in.  The
results must be those of re-plans served inside the tick, bit for bit, and
those of the oracle, whose re-plans come from its own restatement of the
reference planner (the same paths as the library's reference planner)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def _scene(n_agents, seed):
    from ecmgenerator_gb300 import agents as ag

    cfg = ag.scaled("c1", agents=n_agents)
    scene = ag.build_scene(cfg, seed=seed)
    st = ag.spawn_agents(cfg, scene, seed=seed)
    return cfg, scene, st


def _paths(port, scene, st):
    """reference-planner paths; every third agent gets a path that starts
    beyond its goal (its disk meets no segment): it re-plans at once"""
    n = st.num_agents
    E = port.ecm(scene.ecm)
    got = port.find_paths(E, st.pos[:n], st.goal[:n], st.clear[:n], threads=8, cap=4096)
    paths = []
    for i, p in enumerate(got):
        if p is None:
            p = np.stack([st.pos[i], st.goal[i]]).astype(np.float32)
        if i % 3 == 0:
            g = st.goal[i].astype(np.float64)
            d = g - st.pos[i]
            far = g + 30.0 * d / max(np.hypot(*d), 1e-6)
            far = np.clip(far, 1.0, scene.width - 1.0)
            p = np.stack([far, g]).astype(np.float32)
        paths.append(p)
    return paths


def _sim(scene, st, paths, k, overlap):
    from ecmgenerator_gb300.simulator import Simulator, set_replan_overlap

    n = st.num_agents
    sim = Simulator(scene, st.n_slots, 1.0 / 60.0, max_neighbors=k, **ORCA)
    set_replan_overlap(sim, overlap)
    sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths[:n])
    return sim


def test_overlap_matches_in_tick_replans_and_the_oracle(port):
    cfg, scene, st = _scene(600, 4)
    k = cfg["k"]
    paths = _paths(port, scene, st)
    a = _sim(scene, st, paths, k, 2)  # every search carried into the next tick
    b = _sim(scene, st, paths, k, 0)
    c = _sim(scene, st, paths, k, 1)
    st = st.copy()
    st.set_paths(paths)
    O, E = port.obstacles(scene), port.ecm(scene.ecm)
    P = port.params(k=k, libm=0, **ORCA)
    host_replans = 0
    for t in range(30):
        # one tick per call: the overlap carries the searches across calls
        sa, sb, sc = a.update(), b.update(), c.update()
        assert (sa.replans, sa.replans_host, sa.destroyed) == (sb.replans, sb.replans_host, sb.destroyed), t
        assert (sc.replans, sc.replans_host, sc.destroyed) == (sb.replans, sb.replans_host, sb.destroyed), t
        host_replans += sa.replans_host
        res = port.tick(O, E, st, P)
        assert sa.replans == len(res["replan"]), t
        # the oracle's re-plans from the tick-start positions, by its own planner
        if len(res["replan"]):
            slots = [int(s) for s in res["replan"]]
            goals = np.array([st.path(s)[-1] for s in slots], np.float32)
            new = port.find_paths(E, res["replan_pos"], goals, st.clear[slots], threads=8, cap=4096)
            for s, p in zip(slots, new):
                if p is not None:
                    st.replace_path(s, p)
        for name, getter in (("positions", "get_position_data"), ("velocities", "get_velocity_data"),
                             ("attraction points", "get_attraction_point_data")):
            xa, xb, xc = getattr(a, getter)(), getattr(b, getter)(), getattr(c, getter)()
            assert np.array_equal(xa, xb), (t, name)
            assert np.array_equal(xc, xb), (t, name)
        live = st.active == 1
        assert np.array_equal(a.get_active_flags(), st.active), t
        assert np.array_equal(a.get_position_data()[live], st.pos[live]), t
        assert np.array_equal(a.get_velocity_data()[live], st.vel[live]), t
    assert host_replans >= 50  # most of the agents given a path beyond their goal re-plan at once
    # the paths in the end (reading them applies the searches in flight)
    for i in range(st.num_agents):
        pa, pb = a.get_path(i), b.get_path(i)
        assert np.array_equal(pa, pb), i
        assert np.array_equal(c.get_path(i), pb), i
        assert np.array_equal(pa, st.path(i)), i
    a.close()
    b.close()
    c.close()


def test_overlap_across_multi_tick_calls_and_a_drain(port):
    """ticks in one call, and an entry point between ticks that applies the
    searches in flight (destroying an agent), give the in-tick results"""
    cfg, scene, st = _scene(400, 7)
    k = cfg["k"]
    paths = _paths(port, scene, st)
    a = _sim(scene, st, paths, k, 2)
    b = _sim(scene, st, paths, k, 0)
    for sim in (a, b):
        sim.update(ticks=3)
        sim.update()
        sim.destroy_agent(5)
        sim.update(ticks=4)
    assert np.array_equal(a.get_position_data(), b.get_position_data())
    assert np.array_equal(a.get_velocity_data(), b.get_velocity_data())
    assert np.array_equal(a.get_active_flags(), b.get_active_flags())
    for i in range(st.num_agents):
        assert np.array_equal(a.get_path(i), b.get_path(i)), i
    a.close()
    b.close()
