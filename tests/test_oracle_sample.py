"""The oracle's sampled tick (og_tick_sample: one Simulator::Update for listed
agents only, used for parity at the full workload sizes) against its whole
tick (og_tick, pinned to the reference): same attraction points, neighbour
lists, LP results, velocities and positions, bit for bit, tick after tick."""
import numpy as np

ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def test_sampled_tick_equals_whole_tick(port, c1_small):
    scene, st, _ = c1_small
    st = st.copy()
    st.active[7] = 0  # an inactive slot inside the range
    st.num_agents -= 1
    k = 10
    O, E = port.obstacles(scene), port.ecm(scene.ecm)
    P = port.params(k=k, libm=0, **ORCA)
    rng = np.random.default_rng(3)
    seen = np.zeros(4, np.int64)
    for t in range(40):
        sample = rng.choice(st.n_slots, 120, replace=False).astype(np.int32)
        before = st.copy()
        got = port.tick_sample(O, E, before, P, sample, threads=3)
        assert np.array_equal(before.pos, st.pos) and np.array_equal(before.attr, st.attr)  # not modified
        res = port.tick(O, E, st, P)
        destroyed, replan = set(res["destroyed"].tolist()), set(res["replan"].tolist())
        for q, i in enumerate(sample.tolist()):
            s = int(got["status"][q])
            seen[s] += 1
            if s == 3:
                assert not before.active[i] or i > before.last_idx
                continue
            assert (s == 1) == (i in destroyed) and (s == 2) == (i in replan), (t, i, s)
            assert np.array_equal(got["attr"][q], st.attr[i])
            if s == 1:
                continue
            n = res["nbr_count"][i]
            assert got["nbr_count"][q] == n
            assert np.array_equal(got["nbr_ids"][q], res["nbr_ids"][i])
            assert np.array_equal(got["v_orca"][q], res["v_orca"][i])
            assert np.array_equal(got["vel"][q], st.vel[i])
            assert np.array_equal(got["pos"][q], st.pos[i])
    assert seen[0] > 1000 and seen[3] > 0, seen
