"""Checkpoint / resume: ticks after ecmg_load_state reproduce the ticks after
ecmg_save_state bit for bit -- agents moving, re-planning, reaching their
goals, spawn areas placing agents from queued random values, and (kd-tree
mode) the neighbour cache carried across the snapshot."""
import numpy as np
import pytest

import spawn_cases as cases

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0
ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)


def _sim(scene, mode):
    from ecmgenerator_gb300.simulator import Simulator, set_neighbor_mode

    sim = Simulator(scene, 700, DT, max_neighbors=10, **ORCA)
    if mode == "kdtree":
        set_neighbor_mode(sim, "kdtree")
    return sim


@pytest.mark.parametrize("mode", ["exact", "kdtree"])
def test_resume_reproduces_the_run(lib, c1_small, tmp_path, mode):
    scene, st, paths = c1_small
    n = st.num_agents
    a = _sim(scene, mode)
    a.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths[:n])
    cases.standard_areas(scene, cases.Ops(a, "lib"))
    a.push_spawn_random(np.random.default_rng(5).integers(0, 2147483648, 100000).astype(np.int32))
    a.update(ticks=30)
    snap = tmp_path / "state.bin"
    a.save_state(str(snap))
    trail_a = []
    for _ in range(40):
        s = a.update()
        trail_a.append((a.get_position_data().copy(), a.get_velocity_data().copy(), a.get_active_flags().copy(),
                        s.spawned, s.destroyed))
    b = _sim(scene, "exact")  # the snapshot brings its neighbour mode
    b.load_state(str(snap))
    assert b.get_num_agents() == trail_a[0][2].sum() - trail_a[0][3] + trail_a[0][4]
    for t in range(40):
        s = b.update()
        pa, va, aa, sp, de = trail_a[t]
        # (kd-tree mode: a stale self-entry can make a velocity NaN, as in the
        # reference; the resumed run must do the same)
        assert np.array_equal(b.get_position_data(), pa, equal_nan=True), t
        assert np.array_equal(b.get_velocity_data(), va, equal_nan=True), t
        assert np.array_equal(b.get_active_flags(), aa), t
        assert (s.spawned, s.destroyed) == (sp, de), t
    assert sum(x[3] for x in trail_a) > 0
    a.close()
    b.close()


def test_snapshot_of_another_context_is_refused(lib, c1_small, tmp_path):
    from ecmgenerator_gb300._lib import EcmgError
    from ecmgenerator_gb300.simulator import Simulator

    scene, st, paths = c1_small
    a = _sim(scene, "exact")
    a.save_state(str(tmp_path / "s.bin"))
    b = Simulator(scene, 500, DT, max_neighbors=10, **ORCA)
    with pytest.raises(EcmgError):
        b.load_state(str(tmp_path / "s.bin"))
    (tmp_path / "bad.bin").write_bytes(b"not a snapshot")
    with pytest.raises(EcmgError):
        a.load_state(str(tmp_path / "bad.bin"))
    a.close()
    b.close()
