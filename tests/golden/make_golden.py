"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs only where the reference tree exists (it drives oracle/_ref/libecmref.so,
the reference's own C++ sources compiled by oracle/Makefile):

    make -C oracle ref && python tests/golden/make_golden.py

Outputs (numpy .npz, committed):
  tick_c1.npz     400 agents in the 100x100 m / 40-box scene, 12 ticks of the
                  reference Simulator::Update with exact (d2, id) neighbour
                  lists (mode B); per-tick state, neighbour lists, LP results
  tick_dense.npz  400 agents in two opposing 4 m bands of a 20x20 m scene with
                  two boxes (overlapping spawn): LP3D-heavy, 12 ticks
  units.npz       known answers of RandomizedLP / RandomizedLP3D on random
                  half-plane sets, point location, retraction, IRM attraction
                  points and FindNearestObstacles on the c1 scene
  lp_nan.npz      RandomizedLP on half-plane sets with NaN rows

    python tests/golden/make_golden.py [tick_c1 tick_dense units lp_nan]
writes the named fixtures (all of them by default).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ecmgenerator_gb300 import agents as ag  # noqa: E402
from ecmgenerator_gb300 import scene as sc  # noqa: E402
import oracle as orc  # noqa: E402

F32, I32 = np.float32, np.int32
ORCA = dict(dt=1.0 / 60.0, tau_agent=2.0, tau_obst=2.0)
RNB = 5.0


def scene_arrays(s):
    e = s.ecm
    return dict(w=np.float64(s.width), h=np.float64(s.height), boxes=s.boxes, obst_off=s.obst_off, obst_xy=s.obst_xy,
                v_pos=e.v_pos, v_clear=e.v_clear, v_idx=e.v_idx, v_halfedge=e.v_halfedge, he_target=e.he_target,
                he_next=e.he_next, he_left=e.he_left, he_right=e.he_right)


def ref_paths(ref, st, n):
    paths = []
    for i in range(n):
        p = ref.find_path(st.pos[i], st.goal[i], float(st.clear[i]))
        if p is None or len(p) == 0:
            p = np.stack([st.pos[i], st.goal[i]]).astype(F32)
        paths.append(p.astype(F32))
    return paths


def record_ticks(s, st, k, ticks):
    n = st.num_agents
    ref = orc.Ref(s, n, ORCA["dt"], k, ORCA["tau_agent"], ORCA["tau_obst"])
    paths = ref_paths(ref, st, n)
    for i in range(n):
        assert ref.spawn_direct(float(st.pos[i, 0]), float(st.pos[i, 1]), float(st.clear[i]),
                                float(st.pref_speed[i]), paths[i]) == i
    lens = np.array([len(p) for p in paths], I32)
    out = dict(k=np.int32(k), rnb=np.float32(RNB), clear=st.clear[:n].copy(), speed=st.pref_speed[:n].copy(),
               path_len=lens, path_xy=np.concatenate(paths, 0))
    seq = {key: [] for key in ("pos", "vel", "attr", "pref_vel", "active", "nbr", "vorca", "lp_fail", "ncons")}
    path_events = []  # (tick, slot, new path)
    cur_paths = [p.copy() for p in paths]
    s0 = ref.get_state()
    for key in ("pos", "vel", "attr", "active"):
        seq[key].append(s0[key])
    kd, kdc = ref.knn_kdtree()
    out["kd_nbr"], out["kd_cnt"] = kd.astype(I32), kdc.astype(I32)
    for t in range(ticks):
        r = ref.tick_exact(RNB)
        stt = ref.get_state()
        for i in range(n):
            buf = np.zeros((4096, 2), F32)
            m = ref.lib.ref_get_path(ref.h, i, buf.ctypes.data, 4096)
            if m == 0:
                ref.set_path(i, cur_paths[i])  # failed re-plan: keep the previous path
            elif m != len(cur_paths[i]) or not np.array_equal(buf[:m], cur_paths[i]):
                cur_paths[i] = buf[:m].copy()
                path_events.append((t, i, cur_paths[i]))
        for key in ("pos", "vel", "attr", "pref_vel", "active"):
            seq[key].append(stt[key])
        seq["nbr"].append(r["nbr_ids"].astype(np.int16))
        seq["vorca"].append(r["v_orca"])
        seq["lp_fail"].append(r["lp_fail"].astype(np.int16))
        seq["ncons"].append(r["n_constraints"].astype(np.int16))
    for key, v in seq.items():
        out[key] = np.stack(v, 0)
    out["ev_tick"] = np.array([e[0] for e in path_events], I32)
    out["ev_slot"] = np.array([e[1] for e in path_events], I32)
    out["ev_len"] = np.array([len(e[2]) for e in path_events], I32)
    out["ev_xy"] = np.concatenate([e[2] for e in path_events], 0) if path_events else np.zeros((0, 2), F32)
    ref.close()
    return out


def dense_scene(seed):
    rng = np.random.default_rng(seed)
    boxes = np.array([[8.0, 10.0, 0.6, 0.6], [12.5, 9.0, 0.8, 0.5]])
    s = sc.make_scene(20.0, 20.0, boxes)
    s.ecm = sc.build_ecm(s, h=0.05)
    n = 400
    st = ag.AgentState.empty(n)
    bidx = sc.BoxIndex(s)
    rad = rng.uniform(0.2, 0.35, n)
    half = n // 2
    st.pos[:half] = sc.sample_free(rng, s, half, rad[:half], bidx, region=(1, 2, 5, 18), no_overlap=False)
    st.pos[half:] = sc.sample_free(rng, s, n - half, rad[half:], bidx, region=(15, 2, 19, 18), no_overlap=False)
    st.goal[:half] = sc.sample_free(rng, s, half, 0.5, bidx, region=(15, 2, 19, 18), no_overlap=False)
    st.goal[half:] = sc.sample_free(rng, s, n - half, 0.5, bidx, region=(1, 2, 5, 18), no_overlap=False)
    st.clear[:] = rad
    st.pref_speed[:] = rng.uniform(1.2, 1.5, n)
    st.active[:] = 1
    st.last_idx, st.num_agents = n - 1, n
    return s, st


def units(s, st):
    rng = np.random.default_rng(99)
    ref = orc.Ref(s, 8, ORCA["dt"], 10, ORCA["tau_agent"], ORCA["tau_obst"])
    out = {}
    # LP: random half-planes around the origin
    lp_cons, lp_meta, lp_out = [], [], []
    for c in range(300):
        m = int(rng.integers(0, 24))
        pts = rng.normal(0, 0.8, (m, 2))
        ang = rng.uniform(0, 2 * np.pi, m)
        cons = np.concatenate([pts, np.stack([np.cos(ang), np.sin(ang)], 1)], 1).astype(F32)
        opt = rng.normal(0, 1.2, 2).astype(F32)
        ms = np.float32(rng.uniform(0.8, 2.0))
        use_dir = int(c % 5 == 0)
        if use_dir:
            opt = (opt / np.linalg.norm(opt)).astype(F32)
        f, v = ref.lp(cons, opt, ms, use_dir)
        lp_cons.append(cons)
        lp_meta.append((m, opt[0], opt[1], ms, use_dir, f))
        lp_out.append(v)
    out["lp_len"] = np.array([x[0] for x in lp_meta], I32)
    out["lp_opt"] = np.array([(x[1], x[2]) for x in lp_meta], F32)
    out["lp_ms"] = np.array([x[3] for x in lp_meta], F32)
    out["lp_dir"] = np.array([x[4] for x in lp_meta], I32)
    out["lp_fail"] = np.array([x[5] for x in lp_meta], I32)
    out["lp_cons"] = np.concatenate(lp_cons, 0) if lp_cons else np.zeros((0, 4), F32)
    out["lp_out"] = np.array(lp_out, F32)
    # LP3D: infeasible sets (inputs: start velocity = the failed LP's output)
    l3_cons, l3_meta, l3_out = [], [], []
    while len(l3_meta) < 150:
        m = int(rng.integers(3, 20))
        nob = int(rng.integers(0, min(4, m)))
        pts = rng.normal(0, 1.0, (m, 2))
        ang = rng.uniform(0, 2 * np.pi, m)
        cons = np.concatenate([pts, np.stack([np.cos(ang), np.sin(ang)], 1)], 1).astype(F32)
        opt = rng.normal(0, 1.0, 2).astype(F32)
        ms = np.float32(rng.uniform(0.8, 2.0))
        f, v = ref.lp(cons, opt, ms, 0)
        if f >= m:
            continue
        v3 = ref.lp3d(cons, nob, ms, f, v)
        l3_cons.append(cons)
        l3_meta.append((m, nob, ms, f, v[0], v[1]))
        l3_out.append(v3)
    out["l3_len"] = np.array([x[0] for x in l3_meta], I32)
    out["l3_nobst"] = np.array([x[1] for x in l3_meta], I32)
    out["l3_ms"] = np.array([x[2] for x in l3_meta], F32)
    out["l3_fail"] = np.array([x[3] for x in l3_meta], I32)
    out["l3_start"] = np.array([(x[4], x[5]) for x in l3_meta], F32)
    out["l3_cons"] = np.concatenate(l3_cons, 0)
    out["l3_out"] = np.array(l3_out, F32)
    # point location / retraction / IRM on the c1 scene
    q = rng.uniform(-2, s.width + 2, (2000, 2)).astype(F32)
    q[:100, 1] = s.ecm.v_pos[rng.integers(0, s.ecm.n_vertices, 100), 1]  # exact vertex heights
    out["pl_q"] = q
    out["pl_cell"] = np.array([ref.point_location(float(x), float(y)) for x, y in q], I32)
    rt = [ref.retract(float(x), float(y)) for x, y in q[:1000]]
    out["rt_ok"] = np.array([r[0] for r in rt], I32)
    out["rt_xy"] = np.array([r[1] for r in rt], F32)
    out["rt_edge"] = np.array([r[2] for r in rt], I32)
    irm_path, irm_len, irm_ok, irm_xy, irm_q = [], [], [], [], []
    for i in range(400):
        j = int(rng.integers(0, st.num_agents))
        p = ref.find_path(st.pos[j], st.goal[j], float(st.clear[j]))
        if p is None:
            continue
        x = st.pos[j] + rng.normal(0, 1.0, 2).astype(F32)
        ok, v = ref.irm(float(x[0]), float(x[1]), p)
        irm_q.append(x)
        irm_path.append(p)
        irm_len.append(len(p))
        irm_ok.append(int(ok))
        irm_xy.append(v)
    out["irm_q"] = np.array(irm_q, F32)
    out["irm_len"] = np.array(irm_len, I32)
    out["irm_path"] = np.concatenate(irm_path, 0).astype(F32)
    out["irm_ok"] = np.array(irm_ok, I32)
    out["irm_xy"] = np.array(irm_xy, F32)
    # obstacle candidates (FindNearestObstacles) for the first 8 agents
    ob_q, ob_r2, ob_len, ob_ids = [], [], [], []
    for i in range(300):
        x = rng.uniform(0, s.width, 2).astype(F32)
        r2 = np.float32(rng.uniform(1.0, 40.0))
        ref.set_state(pos=np.tile(x, (8, 1)))
        ids = ref.find_obstacles(0, float(r2))
        ob_q.append(x)
        ob_r2.append(r2)
        ob_len.append(len(ids))
        ob_ids.append(ids)
    out["ob_q"] = np.array(ob_q, F32)
    out["ob_r2"] = np.array(ob_r2, F32)
    out["ob_len"] = np.array(ob_len, I32)
    out["ob_ids"] = np.concatenate(ob_ids, 0).astype(I32) if ob_ids else np.zeros(0, I32)
    ref.close()
    return out


def lp_nan():
    """RandomizedLP (ORCA.cpp:428-587) on constraint sets with NaN rows -- the
    half-plane of an agent with itself (0 / 0), which the kd-tree neighbour
    cache can hand to GenerateConstraints: a NaN discriminant takes neither
    branch at ORCA.cpp:498-506, so the constraint is passed over"""
    rng = np.random.default_rng(7)
    s = sc.make_scene(20.0, 20.0, np.array([[10.0, 10.0, 1.0, 1.0]]))
    s.ecm = sc.build_ecm_exact(s, h=0.1)
    ref = orc.Ref(s, 8, ORCA["dt"], 10, ORCA["tau_agent"], ORCA["tau_obst"])  # its LP entry points only
    cons_l, meta, outs = [], [], []
    for c in range(200):
        m = int(rng.integers(2, 20))
        pts = rng.normal(0, 0.8, (m, 2))
        ang = rng.uniform(0, 2 * np.pi, m)
        cons = np.concatenate([pts, np.stack([np.cos(ang), np.sin(ang)], 1)], 1).astype(F32)
        nan_rows = rng.choice(m, int(rng.integers(1, 3)), replace=False)
        cons[nan_rows] = np.nan
        opt = rng.normal(0, 1.2, 2).astype(F32)
        ms = np.float32(rng.uniform(0.8, 2.0))
        use_dir = int(c % 4 == 0)
        if use_dir:
            opt = (opt / np.linalg.norm(opt)).astype(F32)
        f, v = ref.lp(cons, opt, ms, use_dir)
        cons_l.append(cons)
        meta.append((m, opt[0], opt[1], ms, use_dir, f))
        outs.append(v)
    ref.close()
    return dict(lp_len=np.array([x[0] for x in meta], I32), lp_opt=np.array([(x[1], x[2]) for x in meta], F32),
                lp_ms=np.array([x[3] for x in meta], F32), lp_dir=np.array([x[4] for x in meta], I32),
                lp_fail=np.array([x[5] for x in meta], I32), lp_cons=np.concatenate(cons_l, 0),
                lp_out=np.array(outs, F32))


def main(names):
    if not orc.ref_available():
        orc.build(ref=True)
    cfg = ag.scaled("c1", agents=400)
    written = []
    if {"tick_c1", "units"} & names:
        s = ag.build_scene(cfg, seed=3)
        st = ag.spawn_agents(cfg, s, seed=3)
    if "tick_c1" in names:
        d = scene_arrays(s)
        d.update(record_ticks(s, st, 10, 12))
        np.savez_compressed(os.path.join(HERE, "tick_c1.npz"), **d)
        written.append("tick_c1.npz")
    if "tick_dense" in names:
        sd, std_ = dense_scene(4)
        d = scene_arrays(sd)
        d.update(record_ticks(sd, std_, 16, 12))
        np.savez_compressed(os.path.join(HERE, "tick_dense.npz"), **d)
        written.append("tick_dense.npz")
    if "units" in names:
        d = scene_arrays(s)
        d.update(units(s, st))
        np.savez_compressed(os.path.join(HERE, "units.npz"), **d)
        written.append("units.npz")
    if "lp_nan" in names:
        np.savez_compressed(os.path.join(HERE, "lp_nan.npz"), **lp_nan())
        written.append("lp_nan.npz")
    for f in written:
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main(set(sys.argv[1:]) or {"tick_c1", "tick_dense", "units", "lp_nan"})
