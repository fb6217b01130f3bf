"""Parity at the workloads' full sizes: the 1M-agent crossing (four flows of
250k, k = 16) and the 100k-agent 1000 m box scene (k = 10), 600 ticks each.
A whole-tick oracle run takes tens of seconds there, so the GPU runs the 600
ticks and six of them (the first three, ticks 100, 300 and 599) are checked
two ways:

* 2,000 random agents against the oracle's sampled tick (og_tick_sample),
  started from the GPU's own tick-start state and paths: attraction point,
  neighbour list, LP result, velocity and position bit for bit, and the
  destroyed agents;
* every agent's neighbour list through properties that need no oracle: ids of
  agents active at the start of the tick, no self entry, no duplicate,
  EPS < d2 < r^2, ascending by (d2, slot) with d2 recomputed in FP32 from the
  tick-start positions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = 1.0e-4  # KDTree.cpp / ORCA.cpp EPSILON for coincident agents


def _oracle_view(st, sim, sample):
    """the GPU's tick-start state as an oracle state; paths only for the
    sampled slots (the only ones the sampled tick reads)"""
    cur = st.copy()
    cur.pos[:] = sim.get_position_data()
    cur.vel[:] = sim.get_velocity_data()
    cur.attr[:] = sim.get_attraction_point_data()
    cur.active[:] = sim.get_active_flags()
    cur.last_idx = cur.n_slots - 1
    paths = [np.asarray(sim.get_path(int(s)), np.float32).reshape(-1, 2) for s in sample]
    lens = np.array([len(p) for p in paths], np.int32)
    offs = np.concatenate([[1], 1 + np.cumsum(lens)[:-1]]).astype(np.int32)
    cur.path_xy = np.ascontiguousarray(np.concatenate([np.zeros((1, 2), np.float32)] + paths, 0))
    cur.path_off[:] = 0
    cur.path_len[:] = 1
    cur.path_off[sample] = offs
    cur.path_len[sample] = lens
    return cur


def _list_properties(ids, cnt, pos0, act0, live, r2):
    k = ids.shape[1]
    rows = np.nonzero(live)[0]
    L, C = ids[rows], cnt[rows]
    assert (C >= 0).all() and (C <= k).all()
    filled = np.arange(k)[None, :] < C[:, None]
    assert (L[~filled] == -1).all()
    Lf = np.where(filled, L, 0)
    assert (Lf >= 0).all() and (Lf < act0.shape[0]).all()
    assert act0[Lf][filled].all(), "neighbour not active at the start of the tick"
    assert not ((Lf == rows[:, None]) & filled).any(), "self entry"
    q = pos0[Lf]
    p = pos0[rows][:, None, :]
    dx = q[..., 0] - p[..., 0]
    dy = q[..., 1] - p[..., 1]
    d2 = dx * dx + dy * dy  # float32, no fused multiply-add
    assert ((d2 > EPS) & (d2 < r2))[filled].all()
    both = filled[:, 1:]
    asc = (d2[:, :-1] < d2[:, 1:]) | ((d2[:, :-1] == d2[:, 1:]) & (Lf[:, :-1] < Lf[:, 1:]))
    assert asc[both].all(), "list not ascending by (d2, slot) or duplicate entry"
    return int(C.sum())


@pytest.mark.parametrize("name", ["crossing_1m", "boxes_100k"])
def test_full_size_ticks_match_the_oracle(port, name):
    from ecmgenerator_gb300.simulator import Simulator
    from ecmgenerator_gb300.workloads import DT, ORCA, make_workload

    cfg, scene, st, paths, k = make_workload(name, 1, verbose=False)
    n = st.num_agents
    sim = Simulator(scene, n, DT, max_neighbors=k, **ORCA)
    sim.set_record(True)
    sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths)
    O, E = port.obstacles(scene), port.ecm(scene.ecm)
    P = port.params(k=k, libm=0, **ORCA)
    r2 = np.float32(ORCA["neighbor_dist"]) * np.float32(ORCA["neighbor_dist"])
    rng = np.random.default_rng(11)
    checked = entries = 0
    check = {0, 1, 2, 100, 300, 599}
    for t in range(600):
        if t not in check:
            sim.update()
            continue
        act0 = sim.get_active_flags().astype(bool)
        pos0 = sim.get_position_data().copy()
        alive = np.nonzero(act0)[0]
        sample = np.sort(rng.choice(alive, min(2000, len(alive)), replace=False)).astype(np.int32)
        cur = _oracle_view(st, sim, sample)
        want = port.tick_sample(O, E, cur, P, sample, threads=16)
        sim.update()
        rec = sim.get_record()
        act1 = sim.get_active_flags()
        pos1, vel1, attr1 = sim.get_position_data(), sim.get_velocity_data(), sim.get_attraction_point_data()
        gone = want["status"] == 1
        assert (want["status"] != 3).all()
        assert (act1[sample[gone]] == 0).all() and (act1[sample[~gone]] == 1).all(), t
        assert np.array_equal(attr1[sample], want["attr"]), t
        keep = sample[~gone]
        assert np.array_equal(rec["nbr_count"][keep], want["nbr_count"][~gone]), t
        assert np.array_equal(rec["nbr_ids"][keep], want["nbr_ids"][~gone]), t
        assert np.array_equal(rec["v_orca"][keep], want["v_orca"][~gone]), t
        assert np.array_equal(vel1[keep], want["vel"][~gone]), t
        assert np.array_equal(pos1[keep], want["pos"][~gone]), t
        live = (act0 == 1) & (act1 == 1)
        entries += _list_properties(rec["nbr_ids"], rec["nbr_count"], pos0, act0, live, r2)
        checked += len(keep)
    sim.close()
    assert checked > 10000 and entries > 0


def test_full_size_batch_matches_the_oracle(port):
    """the 256-scene batch (1.3M agents, one context, one graph per tick):
    sampled agents of 16 scenes (the largest and the smallest among them)
    against the oracle's sampled tick of their own scene; every agent's
    neighbours from its own scene"""
    from ecmgenerator_gb300.simulator import BatchSimulator
    from ecmgenerator_gb300.workloads import DT, ORCA, make_batch_workload

    cfgs, scenes, states, pathss, k = make_batch_workload("batch_256", 1, verbose=False)
    caps = [st.num_agents for st in states]
    sim = BatchSimulator(scenes, caps, DT, max_neighbors=k, **ORCA)
    sim.set_record(True)
    bases = []
    for i, st in enumerate(states):
        m = st.num_agents
        sim.add_agents(st.pos[:m], st.clear[:m], st.pref_speed[:m], pathss[i], scene=i)
        bases.append(sim.scene_counts(i)["slot_base"])
    bases = np.array(bases)
    assert np.array_equal(bases, np.concatenate([[0], np.cumsum(caps)[:-1]]))
    scene_of = np.repeat(np.arange(len(caps)), caps)
    P = port.params(k=k, libm=0, **ORCA)
    r2 = np.float32(ORCA["neighbor_dist"]) * np.float32(ORCA["neighbor_dist"])
    rng = np.random.default_rng(5)
    order = np.argsort(caps)
    picks = np.unique(np.concatenate([order[:2], order[-2:], rng.choice(len(caps), 12, replace=False)]))
    OE = {int(i): (port.obstacles(scenes[i]), port.ecm(scenes[i].ecm)) for i in picks}
    checked = 0
    check = {0, 1, 2, 100, 300, 599}

    class View:  # one scene's slice of the batch, with scene-local slots
        def __init__(self, b, n):
            self.b, self.n = b, n

        def get_position_data(self):
            return sim.get_position_data()[self.b:self.b + self.n]

        def get_velocity_data(self):
            return sim.get_velocity_data()[self.b:self.b + self.n]

        def get_attraction_point_data(self):
            return sim.get_attraction_point_data()[self.b:self.b + self.n]

        def get_active_flags(self):
            return sim.get_active_flags()[self.b:self.b + self.n]

        def get_path(self, s):
            return sim.get_path(self.b + s)

    for t in range(600):
        if t not in check:
            sim.update()
            continue
        act0 = sim.get_active_flags().astype(bool)
        pos0 = sim.get_position_data().copy()
        want = {}
        for i in picks.tolist():
            b, n = int(bases[i]), caps[i]
            alive = np.nonzero(act0[b:b + n])[0]
            sample = np.sort(rng.choice(alive, min(200, len(alive)), replace=False)).astype(np.int32)
            cur = _oracle_view(states[i], View(b, n), sample)
            want[i] = (sample, port.tick_sample(*OE[i], cur, P, sample, threads=16))
        sim.update()
        rec = sim.get_record()
        act1 = sim.get_active_flags()
        pos1, vel1 = sim.get_position_data(), sim.get_velocity_data()
        for i, (sample, w) in want.items():
            b = int(bases[i])
            gone = w["status"] == 1
            g = b + sample
            assert (act1[g[gone]] == 0).all() and (act1[g[~gone]] == 1).all(), (t, i)
            keep = g[~gone]
            nb = rec["nbr_ids"][keep].copy()
            nb[nb >= 0] -= b  # global -> scene-local slots
            assert np.array_equal(rec["nbr_count"][keep], w["nbr_count"][~gone]), (t, i)
            assert np.array_equal(nb, w["nbr_ids"][~gone]), (t, i)
            assert np.array_equal(rec["v_orca"][keep], w["v_orca"][~gone]), (t, i)
            assert np.array_equal(vel1[keep], w["vel"][~gone]), (t, i)
            assert np.array_equal(pos1[keep], w["pos"][~gone]), (t, i)
            checked += len(keep)
        live = (act0 == 1) & (act1 == 1)
        _list_properties(rec["nbr_ids"], rec["nbr_count"], pos0, act0, live, r2)
        ids, cnt = rec["nbr_ids"][live], rec["nbr_count"][live]
        own = scene_of[np.nonzero(live)[0]]
        filled = np.arange(k)[None, :] < cnt[:, None]
        assert (scene_of[np.where(filled, ids, 0)] == own[:, None])[filled].all(), "neighbour from another scene"
    sim.close()
    assert checked > 5000
