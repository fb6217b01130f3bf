"""The GPU tick against fixtures produced by the reference itself
(tests/golden/): from every recorded reference state, one GPU tick must give
the reference's neighbour lists exactly and its LP velocities within 1e-5
relative (FP32); positions, velocities and attraction points follow."""
import numpy as np
import pytest

import goldens

pytestmark = pytest.mark.gpu
TOL_REL = 1e-5


def _rel(got, ref):
    got, ref = got.astype(np.float64), ref.astype(np.float64)
    scale = np.maximum(np.abs(ref).max(-1, keepdims=True), 1e-3)
    return float((np.abs(got - ref) / scale).max(initial=0.0))


@pytest.mark.parametrize("name", ["tick_c1", "tick_dense"])
def test_gpu_per_tick_against_reference(name):
    from ecmgenerator_gb300.simulator import Simulator

    d = goldens.load(name)
    s = goldens.scene_of(d)
    st, paths = goldens.state_of(d)
    n = st.n_slots
    k = int(d["k"])
    sim = Simulator(s, n, 1.0 / 60.0, max_neighbors=k, tau_agent=2.0, tau_obst=2.0, neighbor_dist=float(d["rnb"]))
    sim.set_planner(lambda *a: None)  # re-plans come from the fixture
    sim.set_record(True)
    assert np.array_equal(sim.add_agents(st.pos, st.clear, st.pref_speed, paths), np.arange(n))
    worst = dict(v=0.0, pos=0.0, attr=0.0)
    for t in range(d["nbr"].shape[0]):
        act = sim.get_active_flags()
        for slot in np.nonzero((act == 1) & (d["active"][t] == 0))[0]:
            sim.destroy_agent(int(slot))
        sim.set_state("position", d["pos"][t])
        sim.set_state("velocity", d["vel"][t])
        sim.set_state("attraction", d["attr"][t])
        sim.update()
        rec = sim.get_record()
        live = d["active"][t + 1] == 1
        assert np.array_equal(sim.get_active_flags(), d["active"][t + 1])
        assert np.array_equal(rec["nbr_ids"][live], d["nbr"][t][live].astype(np.int32)), f"tick {t}"
        worst["v"] = max(worst["v"], _rel(rec["v_orca"][live], d["vorca"][t][live]))
        worst["pos"] = max(worst["pos"], float(np.abs(sim.get_position_data() - d["pos"][t + 1]).max()))
        worst["attr"] = max(worst["attr"], float(np.abs(sim.get_attraction_point_data() - d["attr"][t + 1]).max()))
        for slot, p in goldens.path_events(d, t):
            sim.set_path(slot, p)
    sim.close()
    assert worst["v"] <= TOL_REL, worst
    assert worst["pos"] <= 1e-5 and worst["attr"] <= 1e-4, worst
