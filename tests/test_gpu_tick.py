"""GPU tick parity against the C oracle (same inputs, same deterministic
transcendentals): neighbour lists, LP results, positions, velocities and
attraction points must be bit-identical, tick after tick."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def _pair(scene, st, paths, k, n_slots=None, lp_mode=None, grab=4, orca=None, **kw):
    from ecmgenerator_gb300.simulator import Simulator, set_lp_mode

    n = st.num_agents
    sim = Simulator(scene, n_slots or st.n_slots, 1.0 / 60.0, max_neighbors=k, **(orca or ORCA), **kw)
    if lp_mode:
        set_lp_mode(sim, lp_mode, grab)
    sim.set_record(True)
    sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths[:n])
    return sim


def _compare(sim, st, res, k):
    rec = sim.get_record()
    live = res["alive"]
    assert np.array_equal(rec["nbr_count"][live], res["nbr_count"][live])
    assert np.array_equal(rec["nbr_ids"][live], res["nbr_ids"][live]), "neighbour lists differ"
    assert np.array_equal(rec["v_orca"][live], res["v_orca"][live]), "LP results differ"
    assert np.array_equal(rec["lp_fail"][live], res["lp_fail"][live])
    assert np.array_equal(rec["n_constraints"][live], res["n_constraints"][live])
    assert np.array_equal(sim.get_active_flags(), st.active)
    assert np.array_equal(sim.get_position_data(), st.pos)
    assert np.array_equal(sim.get_velocity_data(), st.vel)
    assert np.array_equal(sim.get_attraction_point_data(), st.attr)
    assert np.array_equal(sim.get_preferred_velocity_data()[live], st.pref_vel[live])


def _run(port, scene, st, paths, ticks, k, orca=None, **kw):
    st = st.copy()
    sim = _pair(scene, st, paths, k, orca=orca, **kw)
    O, E = port.obstacles(scene), port.ecm(scene.ecm)
    P = port.params(k=k, libm=0, **(orca or ORCA))
    events = 0
    for t in range(ticks):
        stats = sim.update()
        res = port.tick(O, E, st, P)
        res["alive"] = st.active == 1
        _compare(sim, st, res, k)
        assert stats.destroyed == len(res["destroyed"])
        assert stats.replans == len(res["replan"])
        events += len(res["destroyed"]) + len(res["replan"]) + res["n_lp3d"]
        for s in res["replan"]:
            st.replace_path(int(s), sim.get_path(int(s)))
    assert sim.get_num_agents() == st.num_agents
    sim.close()
    return events


def test_tick_bitexact_c1_small(port, c1_small):
    scene, st, paths = c1_small
    _run(port, scene, st, paths, ticks=40, k=10)


def test_tick_bitexact_no_graph(port, c1_small):
    scene, st, paths = c1_small
    _run(port, scene, st, paths, ticks=5, k=10, use_graph=False)


@pytest.mark.parametrize("k", [1, 5, 16, 32])
def test_tick_bitexact_k(port, c1_small, k):
    scene, st, paths = c1_small
    _run(port, scene, st, paths, ticks=4, k=k)


def test_tick_bitexact_warp_layout(port, c1_small):
    """one warp per agent: the same bits as the per-thread kernel and the oracle"""
    scene, st, paths = c1_small
    _run(port, scene, st, paths, ticks=40, k=10, lp_mode="warp", grab=3)


@pytest.mark.parametrize("k", [1, 5, 10, 16, 32])
def test_tick_bitexact_fused_layout(port, c1_small, k):
    """the neighbour search inside the per-agent kernel: the same bits"""
    scene, st, paths = c1_small
    _run(port, scene, st, paths, ticks=40 if k == 10 else 4, k=k, lp_mode="fused")


@pytest.mark.parametrize("k", [1, 16, 32])
def test_tick_bitexact_warp_k(port, c1_small, k):
    scene, st, paths = c1_small
    _run(port, scene, st, paths, ticks=4, k=k, lp_mode="warp", grab=1)


def test_tick_bitexact_warp_dense(port):
    """overlapping crowd (infeasible 2D LPs, RandomizedLP3D for most agents)"""
    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300.simulator import Planner

    cfg = ag.scaled("c3", agents=3000, w=60.0, h=60.0, boxes=8, bands=4.0)
    scene = ag.build_scene(cfg, 3)
    st = ag.spawn_agents(cfg, scene, 3)
    paths = Planner(scene).find_paths(st.pos, st.goal, st.clear)
    paths = [p if p is not None else np.stack([st.pos[i], st.goal[i]]) for i, p in enumerate(paths)]
    st.set_paths(paths)
    for mode in ("thread", "warp", "fused"):
        ev = _run(port, scene, st, paths, ticks=6, k=16, lp_mode=mode)
        assert ev > 1000


@pytest.mark.parametrize("tau", [1.5, 4.0])
def test_tick_bitexact_time_horizon(port, c1_small, tau):
    """agent time horizons off and on a power of two (the latter divides by
    multiplying with the exact reciprocal)"""
    scene, st, paths = c1_small
    _run(port, scene, st, paths, ticks=6, k=10, orca=dict(tau_agent=tau, tau_obst=2.0, neighbor_dist=5.0))


def test_knn_standalone(lib, c1_small):
    """ecmg_knn on device arrays against the oracle's exact kNN."""
    import ctypes as C

    import oracle as orc
    from ecmgenerator_gb300 import _lib

    scene, st, _ = c1_small
    n, k, r = st.n_slots, 10, 5.0
    port = orc.Port()
    s = port.state(st)
    want = np.full((n, k), -1, np.int32)
    for i in range(n):
        ids = np.zeros(k, np.int32)
        d2 = np.zeros(k, np.float32)
        m = port.lib.og_knn_exact(C.byref(s), i, k, C.c_float(r * r), ids.ctypes.data, d2.ctypes.data)
        want[i, :m] = ids[:m]
    import torch  # device memory plumbing only

    dev = torch.device("cuda:0")
    pos = torch.from_numpy(st.pos.copy()).to(dev)
    act = torch.from_numpy(st.active.copy()).to(dev)
    out = torch.full((n, k), -7, dtype=torch.int32, device=dev)
    cnt = torch.zeros(n, dtype=torch.int32, device=dev)
    nbytes = lib.ecmg_knn_scratch_bytes(n, 0.0, 0.0, 100.0, 100.0, 2.0)
    scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    rc = lib.ecmg_knn(pos.data_ptr(), act.data_ptr(), n, k, r, 0.0, 0.0, 100.0, 100.0, 2.0, out.data_ptr(),
                      cnt.data_ptr(), scratch.data_ptr(), nbytes, None)
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.array_equal(got, want)


def test_host_view_matches_getters(c1_small, lib):
    """ecmg_host_view: library-owned host copies, the reference's raw-pointer getters"""
    from ecmgenerator_gb300.simulator import Simulator

    scene, st, paths = c1_small
    sim = Simulator(scene, st.n_slots, 1.0 / 60.0, max_neighbors=10, **ORCA)
    sim.add_agents(st.pos, st.clear, st.pref_speed, paths)
    sim.update(ticks=3)
    v1 = sim.view("position")
    assert np.array_equal(v1, sim.get_position_data())
    p1 = v1.__array_interface__["data"][0]
    sim.update()
    v2 = sim.view("position")
    assert v2.__array_interface__["data"][0] == p1  # same host array, refreshed
    assert np.array_equal(v2, sim.get_position_data())
    for f, g in (("velocity", sim.get_velocity_data), ("pref_velocity", sim.get_preferred_velocity_data),
                 ("attraction", sim.get_attraction_point_data), ("clearance", sim.get_clearance_data),
                 ("speed", sim.get_speed_data), ("active", sim.get_active_flags)):
        assert np.array_equal(sim.view(f), g()), f
    with pytest.raises(ValueError):
        v2[0, 0] = 1.0  # read-only
    sim.close()


def test_failed_search_is_settled_on_the_device(c1_small, lib, port):
    """A re-plan whose search failed from an ECM edge fails again from that
    edge (same goal and clearance): the next failure is settled on the device,
    with the same outcome (the agent keeps its path)."""
    from ecmgenerator_gb300.simulator import Planner, Simulator, set_replan_overlap

    scene, st, paths = c1_small
    pl = Planner(scene)
    O = port.obstacles(scene)
    clr = 3.0
    # an agent too wide for the corridors to its goal, in the open, following
    # a path that is not near it
    pick = None
    for i in range(st.num_agents):
        p, g = st.pos[i].astype(np.float32), st.goal[i].astype(np.float32)
        if np.linalg.norm(p - g) < 30.0:
            continue
        if pl.find_paths(p[None], g[None], np.array([clr], np.float32))[0] is not None:
            continue
        r = 2.0 * 1.3 + clr
        if len(port.find_obstacles(O, float(p[0]), float(p[1]), r * r)) == 0:
            pick = (p, g)
            break
    assert pick is not None
    p0, goal = pick
    far = np.stack([goal + np.float32(0.5), goal]).astype(np.float32)
    # with the searches overlapping the next tick, a failed search is counted
    # in the tick that applies it; the totals are the same
    totals = []
    for overlap in (0, 2):
        sim = Simulator(scene, 4, 1.0 / 60.0, max_neighbors=10, **ORCA)
        set_replan_overlap(sim, overlap)
        slot = int(sim.add_agents(p0[None], [clr], [1.3], [far])[0])
        s1 = sim.update()
        s2 = sim.update(ticks=5)
        if not overlap:
            assert (s1.replans, s1.replans_failed, s1.replans_host) == (1, 1, 1)
            assert s2.replans == 5 and s2.replans_failed == 5 and s2.replans_host < 5
        assert np.array_equal(sim.get_path(slot), far)
        totals.append((s1.replans + s2.replans, s1.replans_failed + s2.replans_failed,
                       s1.replans_host + s2.replans_host))
        if not overlap:
            sim.close()
    assert totals[0] == totals[1]
    # a caller-supplied planner is always asked
    sim.set_planner(lambda *a: None)
    s3 = sim.update(ticks=3)
    assert s3.replans == 3 and s3.replans_host == 3
    sim.close()


def test_agents_outside_the_scene_bitexact(port, c1_small):
    """agents outside the grid rectangle sit in the overflow bucket that every
    query scans; their IRM fails (no ECM cell), their re-plans fail"""
    scene, st, paths = c1_small
    st = st.copy()
    far = np.array([[-40.0, 10.0], [-40.5, 10.2], [150.0, 150.0], [-39.8, 9.9]], np.float32)
    st.pos[:4] = far
    ev = _run(port, scene, st, paths, ticks=6, k=10)
    assert ev > 0


def test_empty_and_single_agent(lib, c1_small):
    from ecmgenerator_gb300.simulator import Simulator

    scene, st, paths = c1_small
    sim = Simulator(scene, 8, 1.0 / 60.0, max_neighbors=10, **ORCA)
    s0 = sim.update(ticks=3)  # nothing to do
    assert s0.agent_steps == 0 and s0.ticks == 3 and sim.get_num_agents() == 0
    slot = int(sim.add_agents(st.pos[:1], st.clear[:1], st.pref_speed[:1], paths[:1])[0])
    s1 = sim.update(ticks=2)
    assert s1.agent_steps == 2 and sim.get_num_agents() == 1
    rec_free = sim.get_position_data()[slot]
    assert np.all(np.isfinite(rec_free))
    sim.destroy_agent(slot)
    s2 = sim.update()
    assert s2.agent_steps == 0 and sim.get_num_agents() == 0
    sim.close()


def test_full_capacity_and_slot_reuse(port, c1_small):
    """every slot in use; destroyed slots are reused last-in first-out"""
    from ecmgenerator_gb300.simulator import Simulator

    scene, st, paths = c1_small
    n = st.num_agents
    sim = Simulator(scene, n, 1.0 / 60.0, max_neighbors=10, **ORCA)
    slots = sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths[:n])
    assert np.array_equal(slots, np.arange(n))
    with pytest.raises(Exception):
        sim.add_agents(st.pos[:1], st.clear[:1], st.pref_speed[:1], paths[:1])
    sim.destroy_agent(7)
    sim.destroy_agent(3)
    again = sim.add_agents(st.pos[:2], st.clear[:2], st.pref_speed[:2], paths[:2])
    assert list(again) == [3, 7]
    st2 = sim.update(ticks=2)
    assert sim.get_num_agents() == n - st2.destroyed
    sim.close()


def test_obstacle_constraint_overflow_is_reported(lib):
    """more than 24 obstacle half-planes for one agent: the tick returns
    ECMG_ERR_BOUND (the agent is computed with the first 24)"""
    from ecmgenerator_gb300 import scene as sc
    from ecmgenerator_gb300._lib import EcmgError
    from ecmgenerator_gb300.simulator import Simulator

    # a ring of 40 small boxes around the agent, all within reach
    ang = np.linspace(0, 2 * np.pi, 40, endpoint=False)
    cx, cy = 50.0 + 3.0 * np.cos(ang), 50.0 + 3.0 * np.sin(ang)
    boxes = np.stack([cx, cy, np.full(40, 0.15), np.full(40, 0.15)], 1)  # centre, half extents
    s = sc.make_scene(100.0, 100.0, boxes)
    s.ecm = sc.build_ecm(s, h=0.2)
    sim = Simulator(s, 4, 1.0 / 60.0, max_neighbors=10, **ORCA)
    sim.add_agents(np.array([[50.0, 50.0]], np.float32), [0.3], [1.4],
                   [np.array([[50.0, 50.0], [90.0, 90.0]], np.float32)])
    with pytest.raises(EcmgError) as e:
        sim.update()
    assert "24" in str(e.value) or "bound" in str(e.value).lower()
    sim.close()
