"""The C oracle against known answers produced by the reference itself
(tests/golden/, written by tests/golden/make_golden.py from the reference's
own sources).  With the host libm the oracle must reproduce them bit for bit;
with the deterministic transcendentals of the GPU path it must stay within the
per-tick tolerance."""
import numpy as np
import pytest

import goldens

TOL_REL = 1e-5  # per-tick velocity tolerance, relative (FP32)


@pytest.mark.parametrize("name", ["tick_c1", "tick_dense"])
def test_oracle_replays_reference_ticks_bitexact(port, name):
    d = goldens.load(name)
    s = goldens.scene_of(d)
    st, _ = goldens.state_of(d)
    k = int(d["k"])
    O, E = port.obstacles(s), port.ecm(s.ecm)
    P = port.params(k=k, libm=1, neighbor_dist=float(d["rnb"]))
    T = d["nbr"].shape[0]
    for t in range(T):
        res = port.tick(O, E, st, P)
        live = d["active"][t + 1] == 1
        assert np.array_equal(st.active, d["active"][t + 1])
        assert np.array_equal(res["nbr_ids"][live], d["nbr"][t][live].astype(np.int32)), f"tick {t}: neighbours"
        assert np.array_equal(res["v_orca"][live], d["vorca"][t][live]), f"tick {t}: LP result"
        assert np.array_equal(res["lp_fail"][live], d["lp_fail"][t][live].astype(np.int32))
        assert np.array_equal(st.pos, d["pos"][t + 1]), f"tick {t}: positions"
        assert np.array_equal(st.vel, d["vel"][t + 1])
        assert np.array_equal(st.attr, d["attr"][t + 1])
        for slot, p in goldens.path_events(d, t):
            st.replace_path(slot, p)


@pytest.mark.parametrize("name", ["tick_c1", "tick_dense"])
def test_oracle_custom_transcendentals_per_tick(port, name):
    """One tick from each reference state with the GPU's atan/sin/cos: neighbour
    lists identical, LP results within the FP32 tolerance."""
    d = goldens.load(name)
    s = goldens.scene_of(d)
    k = int(d["k"])
    O, E = port.obstacles(s), port.ecm(s.ecm)
    P = port.params(k=k, libm=0, neighbor_dist=float(d["rnb"]))
    st, _ = goldens.state_of(d)
    worst = 0.0
    for t in range(d["nbr"].shape[0]):
        st.pos[:] = d["pos"][t]
        st.vel[:] = d["vel"][t]
        st.attr[:] = d["attr"][t]
        st.active[:] = d["active"][t]
        st.num_agents = int(st.active.sum())
        res = port.tick(O, E, st, P)
        live = d["active"][t + 1] == 1
        assert np.array_equal(res["nbr_ids"][live], d["nbr"][t][live].astype(np.int32))
        ref = d["vorca"][t][live].astype(np.float64)
        got = res["v_orca"][live].astype(np.float64)
        scale = np.maximum(np.abs(ref).max(1, keepdims=True), 1e-3)
        err = np.abs(got - ref) / scale
        worst = max(worst, float(err.max(initial=0)))
        for slot, p in goldens.path_events(d, t):
            st.replace_path(slot, p)
    assert worst <= TOL_REL, worst


def test_oracle_units(port):
    u = goldens.load("units")
    s = goldens.scene_of(u)
    E, O = port.ecm(s.ecm), port.obstacles(s)
    off = 0
    for c in range(u["lp_len"].shape[0]):
        m = int(u["lp_len"][c])
        cons = u["lp_cons"][off:off + m]
        off += m
        f, v = port.lp(cons, tuple(u["lp_opt"][c]), float(u["lp_ms"][c]), int(u["lp_dir"][c]))
        assert f == u["lp_fail"][c]
        assert np.array_equal(np.array(v, np.float32), u["lp_out"][c])
    off = 0
    for c in range(u["l3_len"].shape[0]):
        m = int(u["l3_len"][c])
        cons = u["l3_cons"][off:off + m]
        off += m
        v = port.lp3d(cons, int(u["l3_nobst"][c]), float(u["l3_ms"][c]), int(u["l3_fail"][c]), tuple(u["l3_start"][c]))
        assert np.array_equal(np.array(v, np.float32), u["l3_out"][c])
    cells = np.array([port.point_location(E, float(x), float(y)) for x, y in u["pl_q"]])
    assert np.array_equal(cells, u["pl_cell"])
    for i in range(u["rt_ok"].shape[0]):
        x, y = u["pl_q"][i]
        ok, r, ed = port.retract(E, float(x), float(y))
        assert ok == bool(u["rt_ok"][i])
        if ok:
            assert np.array_equal(np.array(r, np.float32), u["rt_xy"][i]) and ed == u["rt_edge"][i]
    off = 0
    for i in range(u["irm_len"].shape[0]):
        n = int(u["irm_len"][i])
        p = u["irm_path"][off:off + n]
        off += n
        ok, v = port.irm(E, float(u["irm_q"][i, 0]), float(u["irm_q"][i, 1]), p)
        assert ok == bool(u["irm_ok"][i])
        if ok:
            assert np.array_equal(np.array(v, np.float32), u["irm_xy"][i])
    off = 0
    for i in range(u["ob_len"].shape[0]):
        n = int(u["ob_len"][i])
        ids = port.find_obstacles(O, float(u["ob_q"][i, 0]), float(u["ob_q"][i, 1]), float(u["ob_r2"][i]), libm=1)
        assert np.array_equal(ids, u["ob_ids"][off:off + n])
        off += n


def test_oracle_lp_passes_over_nan_constraints(port):
    """RandomizedLP with NaN half-planes (an agent's own entry in the kd-tree
    neighbour cache gives one): the reference passes over a constraint whose
    discriminant is NaN (ORCA.cpp:498-506); the oracle does the same, bit for
    bit, on the reference's own answers"""
    u = goldens.load("lp_nan")
    off = passed_over = 0
    for c in range(u["lp_len"].shape[0]):
        m = int(u["lp_len"][c])
        cons = u["lp_cons"][off:off + m]
        off += m
        f, v = port.lp(cons, tuple(u["lp_opt"][c]), float(u["lp_ms"][c]), int(u["lp_dir"][c]))
        assert f == u["lp_fail"][c], c
        assert np.array_equal(np.array(v, np.float32), u["lp_out"][c], equal_nan=True), c
        passed_over += int(f == m and np.isfinite(u["lp_out"][c]).all())
    assert passed_over > 20  # feasible results although a NaN row was met
