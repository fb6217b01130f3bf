"""FP32 against an FP64 host run of the same ORCA, on the CPU-runnable
configuration (100x100 m, 40 boxes, 1,000 agents, k = 10, 600 ticks).

Three runs of the oracle, each serving its own re-plans with the library's
host planner:
  A  FP32 with the deterministic atan/sin/cos -- what the GPU computes (the GPU
     tick equals it bit for bit, tests/test_gpu_*.py);
  B  FP32 with the host libm -- the reference (bit for bit, pinned in
     tests/test_oracle_vs_reference.py);
  C  FP64 with the host libm (liboracle64.so).
Reported: the relative velocity difference of one tick taken from the same
state (A's, at ticks 0, 100, 300, 599), and the position difference after 600
ticks of each run (agents alive in both).  A and B against C give the size of
FP32 rounding itself; A against B is the GPU against the reference."""
import numpy as np

ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)
PROBES = (0, 100, 300, 599)


def _replace(st, s, path):
    path = np.asarray(path, st.path_xy.dtype).reshape(-1, 2)
    st.path_off[s] = st.path_xy.shape[0]
    st.path_len[s] = path.shape[0]
    st.path_xy = np.ascontiguousarray(np.concatenate([st.path_xy, path], 0), st.path_xy.dtype)


def _tick(port, OE, P, st, planner):
    res = port.tick(*OE, st, P, record=False)
    r = res["replan"]
    if len(r):
        got = planner.find_paths(res["replan_pos"].astype(np.float32), st.goal[r], st.clear[r].astype(np.float32),
                                 cap=256)
        for s, p in zip(r.tolist(), got):
            if p is not None:  # no path: the agent keeps its previous one
                _replace(st, s, p)
    return res


def _rel(a, b, live):
    d = np.linalg.norm(a[live].astype(np.float64) - b[live].astype(np.float64), axis=1)
    return d / np.maximum(np.linalg.norm(b[live].astype(np.float64), axis=1), 1e-2)


def _stats(x, bound):
    return dict(median=float(np.median(x)), p99=float(np.percentile(x, 99)), max=float(x.max()),
                within=float(np.mean(x <= bound)), beyond=int(np.sum(x > bound)), n=int(x.size))


def test_fp32_against_fp64_host_run(port):
    import oracle as orc
    from ecmgenerator_gb300.simulator import Planner
    from ecmgenerator_gb300.workloads import make_workload

    p64 = orc.Port64()
    cfg, scene, st, paths, k = make_workload("boxes_1k", 1, verbose=False)
    planner = Planner(scene)
    OE32 = (port.obstacles(scene), port.ecm(scene.ecm))
    OE64 = (p64.obstacles(scene), p64.ecm(scene.ecm))
    PA = port.params(k=k, libm=0, **ORCA)
    PB = port.params(k=k, libm=1, **ORCA)
    PC = p64.params(k=k, **ORCA)
    A, B, C = st.copy(), st.copy(), p64.as_f64(st)
    one = {"A-C": [], "B-C": [], "A-B": []}
    for t in range(600):
        if t in PROBES:  # one tick of each arithmetic from A's state
            a, b, c = A.copy(), A.copy(), p64.as_f64(A)
            port.tick(*OE32, a, PA, record=False)
            port.tick(*OE32, b, PB, record=False)
            p64.tick(*OE64, c, PC, record=False)
            live = (a.active == 1) & (c.active == 1)
            one["A-C"].append(_rel(a.vel, c.vel, live))
            one["B-C"].append(_rel(b.vel, c.vel, live))
            one["A-B"].append(_rel(a.vel, b.vel, live))
        _tick(port, OE32, PA, A, planner)
        _tick(port, OE32, PB, B, planner)
        _tick(p64, OE64, PC, C, planner)
    planner.close()
    report = {}
    for key, v in one.items():
        report["velocity, one tick, " + key] = _stats(np.concatenate(v), 1e-5)
    for key, (x, y) in {"A-C": (A, C), "B-C": (B, C), "A-B": (A, B)}.items():
        live = (x.active == 1) & (y.active == 1)
        d = np.linalg.norm(x.pos[live].astype(np.float64) - y.pos[live].astype(np.float64), axis=1)
        report["position after 600 ticks, " + key] = _stats(d, 1e-3)
    for key, v in report.items():
        print(f"{key}: median {v['median']:.3g}  p99 {v['p99']:.3g}  max {v['max']:.3g}  "
              f"beyond the bound {v['beyond']} of {v['n']}")
    # FP32 rounding of one tick is ~1e-7 relative for most agents; the GPU's
    # transcendentals move it by less than the 1e-5 bound
    assert report["velocity, one tick, A-C"]["median"] < 1e-5
    assert report["velocity, one tick, A-B"]["median"] < 1e-5
    assert report["velocity, one tick, A-B"]["max"] < 1e-5
    # after 600 ticks the crowd is chaotic: one rounding difference grows.
    # The two FP32 runs (own transcendentals vs the host libm) must stay far
    # closer to each other than either is to FP64: with the reference
    # planner's paths 13 of 955 agents differ by more than 1 mm between them,
    # against 89 between FP32 and FP64
    ab, ac = report["position after 600 ticks, A-B"], report["position after 600 ticks, A-C"]
    assert ab["median"] < 1e-5 and ab["within"] >= 0.98
    assert ab["beyond"] * 4 <= ac["beyond"]
