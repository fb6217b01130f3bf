"""Batches of independent scenes (ecmg_create_batch) and the autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def _scene(seed, n, w=60.0):
    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300.simulator import Planner

    cfg = ag.scaled("c1", agents=n, w=w, h=w, boxes=int(w / 5))
    s = ag.build_scene(cfg, seed)
    st = ag.spawn_agents(cfg, s, seed)
    paths = Planner(s).find_paths(st.pos, st.goal, st.clear)
    paths = [p if p is not None else np.stack([st.pos[i], st.goal[i]]) for i, p in enumerate(paths)]
    st.set_paths(paths)
    return s, st, paths


@pytest.mark.parametrize("mode", ["thread", "fused"])
def test_batch_matches_oracle_per_scene(port, mode):
    from ecmgenerator_gb300.simulator import BatchSimulator, set_lp_mode

    specs = [(21, 120, 40.0), (22, 400, 60.0), (23, 37, 30.0)]
    data = [_scene(*sp) for sp in specs]
    caps = [d[1].n_slots for d in data]
    sim = BatchSimulator([d[0] for d in data], caps, 1.0 / 60.0, max_neighbors=10, **ORCA)
    set_lp_mode(sim, mode, 1)
    sim.set_record(True)
    bases = []
    for i, (s, st, paths) in enumerate(data):
        slots = sim.add_agents(st.pos, st.clear, st.pref_speed, paths, scene=i)
        bases.append(sim.scene_counts(i)["slot_base"])
        assert np.array_equal(slots, bases[-1] + np.arange(st.n_slots))
    states = [d[1].copy() for d in data]
    P = port.params(k=10, libm=0, **ORCA)
    OE = [(port.obstacles(d[0]), port.ecm(d[0].ecm)) for d in data]
    for t in range(12):
        sim.update()
        rec = sim.get_record()
        pos = sim.get_position_data()
        vel = sim.get_velocity_data()
        for i, st in enumerate(states):
            res = port.tick(*OE[i], st, P)
            b, n = bases[i], st.n_slots
            live = st.active == 1
            nb = rec["nbr_ids"][b:b + n].copy()
            nb[nb >= 0] -= b  # global -> scene-local slot ids
            assert np.array_equal(nb[live], res["nbr_ids"][live]), (t, i)
            assert np.array_equal(pos[b:b + n], st.pos), (t, i)
            assert np.array_equal(vel[b:b + n], st.vel), (t, i)
            for s_ in res["replan"]:
                st.replace_path(int(s_), sim.get_path(b + int(s_)))
    sim.close()


def test_autotune_restores_state(port):
    from ecmgenerator_gb300.simulator import Simulator, autotune

    s, st, paths = _scene(31, 600, 60.0)
    sim = Simulator(s, st.n_slots, 1.0 / 60.0, max_neighbors=10, **ORCA)
    sim.add_agents(st.pos, st.clear, st.pref_speed, paths)
    sim.update(ticks=3)
    before = (sim.get_position_data(), sim.get_velocity_data(), sim.get_attraction_point_data(), sim.get_num_agents())
    r = autotune(sim, ticks_per_trial=1)
    assert r["trials"] >= 13 and r["lp_mode"] in ("thread", "warp") and r["occupancy_divisor"] in (1, 2, 3)
    if r["lp_mode"] == "thread":
        assert r["block_size"] in (64, 128, 256) and r["agents_per_warp_grab"] in (32, 64, 128)
    else:
        assert r["agents_per_warp_grab"] in (1, 2, 4, 8)
    after = (sim.get_position_data(), sim.get_velocity_data(), sim.get_attraction_point_data(), sim.get_num_agents())
    for a, b in zip(before, after):
        assert np.array_equal(a, b)
    # the tuned configuration computes the same tick as the oracle
    st2 = st.copy()
    st2.pos[:] = before[0]
    st2.vel[:] = before[1]
    st2.attr[:] = before[2]
    st2.active[:] = sim.get_active_flags()
    st2.num_agents = int(st2.active.sum())
    st2.last_idx = sim.get_last_index()
    for i in range(st2.n_slots):  # paths re-planned during the first ticks
        p = sim.get_path(i)
        if not np.array_equal(p, st2.path(i)):
            st2.replace_path(i, p)
    sim.set_record(True)
    sim.update()
    res = port.tick(port.obstacles(s), port.ecm(s.ecm), st2, port.params(k=10, libm=0, **ORCA))
    live = st2.active == 1
    assert np.array_equal(sim.get_record()["nbr_ids"][live], res["nbr_ids"][live])
    assert np.array_equal(sim.get_position_data(), st2.pos)
    sim.close()


def test_batch_with_learned_proposal_matches_plain(lib):
    """the learned mode over a batch of scenes leaves every scene's
    trajectories as the plain tick's"""
    import os

    from ecmgenerator_gb300 import proposal as P
    from ecmgenerator_gb300.simulator import BatchSimulator

    specs = [(31, 200, 40.0), (32, 350, 60.0)]
    data = [_scene(*sp) for sp in specs]
    caps = [d[1].n_slots for d in data]
    sims = [BatchSimulator([d[0] for d in data], caps, 1.0 / 60.0, max_neighbors=10, **ORCA) for _ in range(2)]
    for sim in sims:
        for i, (s, st, paths) in enumerate(data):
            sim.add_agents(st.pos, st.clear, st.pref_speed, paths, scene=i)
    model = P.ProposalModel(seed=0)
    model.load(os.path.join(os.path.dirname(P.__file__), "data", "proposal.npy"))
    sims[1].set_proposal(model)
    sims[1].set_proposal_gate(0.0, 0)
    acc = 0
    for t in range(20):
        sims[0].update()
        acc += sims[1].update().accepted
        assert np.array_equal(sims[0].get_position_data(), sims[1].get_position_data()), t
        assert np.array_equal(sims[0].get_velocity_data(), sims[1].get_velocity_data()), t
    assert acc > 0
    for sim in sims:
        sim.close()
    model.close()
