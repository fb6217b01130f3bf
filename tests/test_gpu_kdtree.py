"""Neighbour mode ECMG_NEIGHBORS_KDTREE on the GPU against the oracle's
kd-tree tick (knn_mode 1), which is pinned bit for bit to the unmodified
reference Simulator::Update in tests/test_oracle_vs_reference.py.  Checked
tick after tick: the neighbour lists (stale cache entries included, in cache
order), the LP results, positions, velocities and attraction points.

A stale cache entry can be the querying agent itself; the reference's
collision branch then divides by a zero relative velocity and the agent's
velocity becomes NaN -- on both sides alike.  From the tick after that the
reference is undefined (std::sort on NaN coordinates), so a run stops
comparing there."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def _run(port, scene, st, paths, ticks, k, n_slots=None, autotune_at=None, planner=None, **kw):
    from ecmgenerator_gb300.simulator import Simulator, autotune, set_neighbor_mode, set_planner_mode

    st = st.copy()
    n = st.num_agents
    sim = Simulator(scene, n_slots or st.n_slots, 1.0 / 60.0, max_neighbors=k, **ORCA, **kw)
    set_neighbor_mode(sim, "kdtree")
    if planner:
        set_planner_mode(sim, planner)
    sim.set_record(True)
    sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths[:n])
    O, E = port.obstacles(scene), port.ecm(scene.ecm)
    P = port.params(k=k, libm=0, knn_mode=1, **ORCA)
    kd = port.kdtree(k)
    same = lambda a, b: np.array_equal(a, b, equal_nan=True)  # noqa: E731
    stale = events = done = 0
    for t in range(ticks):
        if autotune_at == t:
            autotune(sim, ticks_per_trial=1)
        stats = sim.update()
        res = port.tick(O, E, st, P, kd=kd)
        live = st.active == 1
        rec = sim.get_record()
        assert np.array_equal(rec["nbr_count"][live], res["nbr_count"][live]), t
        assert np.array_equal(rec["nbr_ids"][live], res["nbr_ids"][live]), t
        assert same(rec["v_orca"][live], res["v_orca"][live]), t
        assert np.array_equal(sim.get_active_flags(), st.active), t
        assert same(sim.get_position_data(), st.pos), t
        assert same(sim.get_velocity_data(), st.vel), t
        assert same(sim.get_attraction_point_data(), st.attr), t
        assert stats.destroyed == len(res["destroyed"]) and stats.replans == len(res["replan"])
        # entries an exact query never gives: the agent itself, duplicates,
        # agents that are no longer active
        for a in np.nonzero(live)[0]:
            ids = res["nbr_ids"][a][:res["nbr_count"][a]]
            stale += int(np.sum(ids == a)) + len(ids) - len(set(ids.tolist())) + int(np.sum(st.active[ids] == 0))
        events += len(res["destroyed"]) + len(res["replan"]) + res["n_lp3d"]
        done = t + 1
        if np.isnan(st.pos[st.active == 1]).any():
            break
        for s in res["replan"]:
            st.replace_path(int(s), sim.get_path(int(s)))
    port.lib.og_kdtree_destroy(kd)
    sim.close()
    return done, events, stale


def test_kdtree_mode_bitexact_c1(port, c1_small):
    scene, st, paths = c1_small
    done, events, quirks = _run(port, scene, st, paths, 240, 10)
    assert done >= 150 and events > 0 and quirks > 0, (done, events, quirks)


@pytest.mark.parametrize("k", [5, 16, 32])
def test_kdtree_mode_bitexact_k(port, c1_small, k):
    scene, st, paths = c1_small
    _run(port, scene, st, paths, 60, k)


def test_kdtree_mode_small_population_keeps_stale_entries(port):
    """few agents, agents reaching their goals: lists carry entries of
    earlier agents (the querying agent itself among them) and of removed
    agents"""
    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300.simulator import Planner

    cfg = ag.scaled("c1", agents=12)
    scene = ag.build_scene(cfg, seed=3)
    st = ag.spawn_agents(cfg, scene, seed=3, n_slots=16)
    n = st.num_agents
    st.goal[:n] = st.pos[:n] + np.array([[3.0, 0.0]], np.float32)  # close goals: agents are removed
    paths = Planner(scene).find_paths(st.pos[:n], st.goal[:n], st.clear[:n])
    paths = [p if p is not None else np.stack([st.pos[i], st.goal[i]]) for i, p in enumerate(paths)]
    st.set_paths(paths)
    done, events, stale = _run(port, scene, st, paths, 150, 4, n_slots=16)
    print("ticks compared", done, "stale entries", stale)
    assert done >= 1 and stale > 0


def test_kdtree_mode_with_the_reference_planner(port, c1_small):
    """re-plans served by the restated reference planner (the reference's
    own paths): with the kd-tree mode, the tick of the unmodified reference"""
    scene, st, paths = c1_small
    done, events, _ = _run(port, scene, st, paths, 120, 10, planner="reference")
    assert done >= 100 and events > 0


def test_kdtree_mode_autotune_keeps_the_cache(port, c1_small):
    scene, st, paths = c1_small
    _run(port, scene, st, paths, 30, 10, autotune_at=10)


def test_kdtree_mode_exclusions(lib, c1_small):
    from ecmgenerator_gb300 import proposal as P
    from ecmgenerator_gb300._lib import EcmgError
    from ecmgenerator_gb300.simulator import Simulator, set_lp_mode, set_neighbor_mode

    scene, st, paths = c1_small
    sim = Simulator(scene, 400, 1.0 / 60.0, max_neighbors=10, **ORCA)
    set_neighbor_mode(sim, "kdtree")
    with pytest.raises(EcmgError):
        set_lp_mode(sim, "warp")
    m = P.ProposalModel(seed=1)
    with pytest.raises(EcmgError):
        sim.set_proposal(m)
    set_neighbor_mode(sim, "exact")
    sim.set_proposal(m)
    with pytest.raises(EcmgError):
        set_neighbor_mode(sim, "kdtree")
    sim.set_proposal(None)
    m.close()
    sim.close()


def test_kdtree_mode_crossing_100k_matches_oracle(port):
    """the 400x400 m crossing with 100,000 agents (dense bands, coordinate
    ties possible) for a few ticks"""
    from ecmgenerator_gb300.workloads import make_workload

    cfg, scene, st, paths, k = make_workload("crossing_100k", 1, verbose=False)
    _run(port, scene, st, paths, 3, k)
