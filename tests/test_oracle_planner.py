"""The oracle's own restatement of the reference planner (og_find_path,
oracle/ecmg_oracle.c) against the reference's ECMPathPlanner::FindPath
compiled in oracle/_ref: the same paths, point for point and bit for bit, for
start / goal pairs across three scenes and several clearances.  The oracle
planner is what the benchmark's CPU arm plans with, so that arm never loads
the product library."""
import numpy as np
import pytest

import oracle as orc
from ecmgenerator_gb300 import agents as ag

pytestmark = pytest.mark.ref


@pytest.mark.parametrize("name,seed,agents", [("c1", 1, 400), ("c3", 2, 600), ("c2", 1, 300)])
def test_oracle_planner_matches_reference(port, name, seed, agents):
    cfg = ag.scaled(name, agents=agents)
    scene = ag.build_scene(cfg, seed)
    st = ag.spawn_agents(cfg, scene, seed)
    n = st.num_agents
    rng = np.random.default_rng(seed + 11)
    clr = rng.choice(np.array([0.2, 0.35, 0.6, 1.5], np.float32), n)
    ref = orc.Ref(scene, 4, 1.0 / 60.0, 5, 2.0, 2.0)
    got = port.find_paths(port.ecm(scene.ecm), st.pos[:n], st.goal[:n], clr, threads=4, cap=4096)
    found = long_paths = 0
    for i in range(n):
        want = ref.find_path(st.pos[i], st.goal[i], float(clr[i]))
        if want is None:
            assert got[i] is None, i
            continue
        assert got[i] is not None, i
        assert got[i].shape == want.shape, (i, got[i].shape, want.shape)
        assert np.array_equal(got[i], want), i
        found += 1
        long_paths += len(want) > 3
    ref.close()
    assert found > n // 2 and long_paths > 10, (found, long_paths)
