"""The C oracle next to the reference's own simulator (oracle/_ref, built from
the reference sources in this container): bit-identical trajectories over the
full 600-tick, 1000-agent workload of the 100x100 m scene, and the kd-tree
neighbour query of the reference (quirks included) reproduced exactly."""
import numpy as np
import pytest

import oracle as orc
from ecmgenerator_gb300 import agents as ag

pytestmark = pytest.mark.ref

ORCA = dict(tau_agent=2.0, tau_obst=2.0)


@pytest.fixture(scope="module")
def c1_ref():
    cfg = ag.scaled("c1")
    s = ag.build_scene(cfg, seed=1)
    st = ag.spawn_agents(cfg, s, seed=1)
    ref = orc.Ref(s, st.n_slots, 1.0 / 60.0, cfg["k"], 2.0, 2.0)
    paths = []
    for i in range(st.num_agents):
        p = ref.find_path(st.pos[i], st.goal[i], float(st.clear[i]))
        paths.append(p if p is not None else np.stack([st.pos[i], st.goal[i]]).astype(np.float32))
    st.set_paths(paths)
    for i in range(st.num_agents):
        assert ref.spawn_direct(float(st.pos[i, 0]), float(st.pos[i, 1]), float(st.clear[i]),
                                float(st.pref_speed[i]), paths[i]) == i
    return s, st, ref, cfg


def test_600_ticks_bitexact(port, c1_ref):
    s, st, ref, cfg = c1_ref
    st = st.copy()
    O, E = port.obstacles(s), port.ecm(s.ecm)
    P = port.params(k=cfg["k"], libm=1, **ORCA)
    lp3d = destroyed = replans = 0
    for t in range(600):
        ref.tick_exact(5.0)
        res = port.tick(O, E, st, P, record=False)
        lp3d += res["n_lp3d"]
        destroyed += len(res["destroyed"])
        replans += len(res["replan"])
        for slot, pos in zip(res["replan"], res["replan_pos"]):
            old = st.path(int(slot)).copy()
            p = ref.find_path(pos, old[-1], float(st.clear[slot]))
            if p is None:
                ref.set_path(int(slot), old)  # the reference would keep an empty path (UB)
            else:
                st.replace_path(int(slot), p)
        r = ref.get_state()
        assert np.array_equal(r["pos"], st.pos), t
        assert np.array_equal(r["vel"], st.vel), t
        assert np.array_equal(r["attr"], st.attr), t
        assert np.array_equal(r["active"], st.active), t
        assert r["num_agents"] == st.num_agents
    assert lp3d > 0 and destroyed > 0 and replans > 0  # the run exercised every branch


def test_kdtree_mode_bitexact(port, c1_ref):
    """Reference kd-tree lists (KDTree.cpp:85-202), stale-slot quirks included."""
    import ctypes as C

    s, st, ref, cfg = c1_ref
    k = cfg["k"]
    want, cnt = ref.knn_kdtree()
    st2 = st.copy()
    r = ref.get_state()
    st2.pos[:] = r["pos"]
    st2.active[:] = r["active"]
    st2.num_agents = int(r["active"].sum())
    st2.last_idx = r["last_idx"]
    kd = port.kdtree(k)
    S = port.state(st2)
    port.lib.og_kdtree_build(kd, C.byref(S))
    out = np.zeros(k, np.int32)
    for i in range(st2.last_idx + 1):
        if not st2.active[i]:
            continue
        n = port.lib.og_kdtree_query(kd, C.byref(S), i, out.ctypes.data)
        assert n == cnt[i]
        assert np.array_equal(out, want[i]), i
    port.lib.og_kdtree_destroy(kd)


def test_custom_transcendentals_divergence(port, c1_ref):
    """How far the GPU's transcendentals move a 600-tick trajectory, next to an
    FP64-free estimate of chaos: the spread is reported, not bounded, except
    that neighbour lists on the first tick agree exactly."""
    s, st, ref, cfg = c1_ref
    a, b = st.copy(), st.copy()
    O, E = port.obstacles(s), port.ecm(s.ecm)
    Pa = port.params(k=cfg["k"], libm=1, **ORCA)
    Pb = port.params(k=cfg["k"], libm=0, **ORCA)
    ra = port.tick(O, E, a, Pa)
    rb = port.tick(O, E, b, Pb)
    live = a.active == 1
    assert np.array_equal(ra["nbr_ids"][live], rb["nbr_ids"][live])
    rel = np.abs(ra["v_orca"][live] - rb["v_orca"][live]).max(1) / np.maximum(np.abs(ra["v_orca"][live]).max(1), 1e-3)
    assert rel.max() <= 1e-5


@pytest.mark.ref
@pytest.mark.parametrize("ecm", ["sampled", "exact"])
def test_mode_a_ticks_bitexact_vs_unmodified_update(port, ecm):
    """The oracle's kd-tree mode (knn_mode 1: KDTree::Construct and
    KNearestAgents_R with the neighbour cache carried across agents and ticks)
    against the unmodified Simulator::Update, tick by tick.  Re-plans happen
    inside the reference's Update with its own planner; the oracle takes the
    same paths afterwards (a failed re-plan keeps the old path on both
    sides, where the reference would read path.x[-1]).  On the exact
    segment-Voronoi ECM an agent meets its own cache entry and a NaN
    half-plane, which the LP must pass over as the reference does."""
    cfg = ag.scaled("c1", ecm=ecm)
    s = ag.build_scene(cfg, seed=2)
    st = ag.spawn_agents(cfg, s, seed=2)
    ref = orc.Ref(s, st.n_slots, 1.0 / 60.0, cfg["k"], 2.0, 2.0)
    paths = []
    for i in range(st.num_agents):
        p = ref.find_path(st.pos[i], st.goal[i], float(st.clear[i]))
        paths.append(p if p is not None else np.stack([st.pos[i], st.goal[i]]).astype(np.float32))
    st.set_paths(paths)
    for i in range(st.num_agents):
        assert ref.spawn_direct(float(st.pos[i, 0]), float(st.pos[i, 1]), float(st.clear[i]),
                                float(st.pref_speed[i]), paths[i]) == i
    O, E = port.obstacles(s), port.ecm(s.ecm)
    P = port.params(k=cfg["k"], libm=1, knn_mode=1, **ORCA)
    kd = port.kdtree(cfg["k"])
    replans = lp3d = 0
    for t in range(400):
        old = {}
        res = port.tick(O, E, st, P, kd=kd, record=False)
        ref.update()
        lp3d += res["n_lp3d"]
        for slot in res["replan"]:
            slot = int(slot)
            p = ref.get_path(slot)
            if len(p) == 0:
                ref.set_path(slot, st.path(slot))
            else:
                st.replace_path(slot, p)
            replans += 1
        r = ref.get_state()
        live = r["active"].astype(bool)
        live[r["last_idx"] + 1:] = False
        assert np.array_equal(live, st.active.astype(bool)), t
        assert np.array_equal(r["pos"][live], st.pos[live]), t
        assert np.array_equal(r["vel"][live], st.vel[live]), t
    port.lib.og_kdtree_destroy(kd)
    ref.close()
    assert replans > 0 and lp3d > 0
