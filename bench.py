"""Benchmark of the GPU crowd tick (one JSON line on stdout).

Workload (default): the dense crossing-flow scene -- 400x400 m, 200 boxes of
side U[1,4] m, 1,000,000 agents in four groups of 250k spawned in 60 m bands
along the sides with goals in the opposite band, radius U[0.2,0.35] m,
preferred speed U[1.2,1.5] m/s, ORCA with 16 neighbours within 5 m, time
horizons 2 s, dt = 1/60 s, FP32.  Seeded synthetic data (no dataset exists).

A step is one Simulator::Update of every agent.  `value` is agent-steps/s
from CUDA events on the library's stream around each tick (inputs resident in
HBM; L2 is flushed before every timed tick).  `e2e` is the same metric through
the public API (Simulator.update + reading positions and velocities back into
host memory), wall-clock.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]
Under torchrun (N > 1) every rank runs an independent replica on its GPU
("replicas only": a single scene has no exchange the reference performs).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOADS = {
    "crossing_1m": dict(cfg="c3", agents=1_000_000, k=16),
    "crossing_100k": dict(cfg="c3", agents=100_000, k=16),
    "boxes_100k": dict(cfg="c2", agents=100_000, k=10),
    "boxes_1k": dict(cfg="c1", agents=1_000, k=10),
}
ORCA = dict(tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0)
DT = 1.0 / 60.0
ALG_BYTES_PER_AGENT = 64  # algorithmic state traffic of the per-agent kernel


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(name, seed):
    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300.simulator import Planner

    w = WORKLOADS[name]
    cfg = ag.scaled(w["cfg"], agents=w["agents"])
    t0 = time.time()
    scene = ag.build_scene(cfg, seed)
    st = ag.spawn_agents(cfg, scene, seed)
    pl = Planner(scene)
    n = st.num_agents
    paths = []
    chunk = 100_000
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        got = pl.find_paths(st.pos[a:b], st.goal[a:b], st.clear[a:b], threads=0, cap=64)
        for i, p in enumerate(got):
            if p is None:
                p = np.stack([st.pos[a + i], st.goal[a + i]])
            paths.append(np.asarray(p, np.float32))
    st.set_paths(paths)
    log(f"[bench] workload {name}: {n} agents, {scene.ecm.n_edges} ECM edges, setup {time.time() - t0:.1f}s")
    return cfg, scene, st, paths, w["k"]


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def reduce_over_ranks(ms, steps, world, device):
    """Whole-job numbers of independent replicas: the slowest rank's time and
    the sum of the agent-steps every rank processed."""
    if world <= 1:
        return ms, float(steps)
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms, float(steps)], dtype=torch.float64, device=device)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(t[1])


def cpu_baseline(scene, st, k, threads, budget_s=12.0):
    """The C oracle (reference algorithm: kd-tree kNN, linear point location,
    ORCA, LP/LP3D) on a random sample of the same workload's agents; the
    kd-tree build over all agents is timed once and amortised per tick."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as orc

    orc.build()
    port = orc.Port()
    O, E = port.obstacles(scene), port.ecm(scene.ecm)
    P = port.params(k=k, libm=1, knn_mode=1, **ORCA)
    rng = np.random.default_rng(0)
    n = st.num_agents
    m = 256
    tb, ta = port.time_sample(O, E, st, P, rng.choice(n, m, replace=False), threads)
    per = ta / m
    m2 = int(max(m, min(n, (budget_s - tb) / max(per, 1e-9) * 0.9)))
    sample = rng.choice(n, m2, replace=False)
    tb, ta = port.time_sample(O, E, st, P, sample, threads)
    tick_s = tb + ta * (n / m2)
    return {"value": n / tick_s, "unit": "agent-steps/s", "cores": threads, "kind": "port",
            "sample": f"one tick of {n} agents extrapolated from {m2} sampled agents (kd-tree build {tb:.2f}s over all "
                      f"agents + {ta:.2f}s for the sample), C oracle with host libm, {threads} thread(s)",
            "ms_per_tick": tick_s * 1e3}


def run_ours(args):
    import ctypes as C

    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from ecmgenerator_gb300.simulator import Simulator

    cfg, scene, st, paths, k = make_workload(args.workload, args.seed)
    n = st.num_agents
    sim = Simulator(scene, n, DT, max_neighbors=k, **ORCA)
    sim.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths)
    stream = torch.cuda.ExternalStream(sim.L.ecmg_stream(sim.h))
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        sim.update()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    steps = 0
    agent_ms = 0.0
    tot = dict(lp3d=0, replans=0, replans_failed=0, destroyed=0, device_ms=0.0)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()  # L2 flush (512 MB > 129 MB L2) before every timed tick
                ev[i][0].record(stream)
            s = sim.update()
            with torch.cuda.stream(stream):
                ev[i][1].record(stream)
            steps += s.agent_steps
            agent_ms += s.agent_kernel_ms
            tot["lp3d"] += s.lp3d
            tot["replans"] += s.replans
            tot["replans_failed"] += s.replans_failed
            tot["destroyed"] += s.destroyed
            tot["device_ms"] += s.device_ms
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    ms_all, steps_all = reduce_over_ranks(ms, steps, world, "cuda")
    value = steps_all / (ms_all / 1e3)
    # e2e through the public API: update + positions/velocities back to host
    e2e_steps = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s = sim.update()
        _ = sim.get_position_data()
        _ = sim.get_velocity_data()
        e2e_steps += s.agent_steps
    t1 = time.perf_counter()
    e2e = {"value": e2e_steps * max(world, 1) / (t1 - t0), "unit": "agent-steps/s", "h2d_bytes_per_step": 64,
           "d2h_bytes_per_step": 16 * n + 64}
    kern_ms = agent_ms / max(args.steps, 1)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs") or 6800.0
    achieved = ALG_BYTES_PER_AGENT * (steps / max(args.steps, 1)) / (kern_ms / 1e3) / 1e9 if kern_ms > 0 else 0.0
    traffic = None
    tf = os.path.join(HERE, "profiles", "k_agents_traffic.json")
    if os.path.exists(tf):
        try:
            t = json.load(open(tf)).get(args.workload)
            if t:
                traffic = t["dram_bytes_per_agent"] * (steps / max(args.steps, 1))
        except (OSError, ValueError, KeyError):
            traffic = None
    out = {
        "metric": "agent-steps/s (plain GPU ORCA tick)", "value": value, "unit": "agent-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_all / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded scene, agents and paths)",
        "config": {"workload": args.workload, "agents": n, "max_neighbors": k, "neighbor_dist_m": 5.0,
                   "time_horizon_s": 2.0, "dt_s": DT, "scene": cfg["cfg"] if "cfg" in cfg else args.workload,
                   "l2": "flushed before every timed tick (512 MB write)", "parallelism": f"replicas x{world}",
                   "seed": args.seed},
        "e2e": e2e,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "kernel": "k_agents", "kernel_ms": kern_ms,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s"},
        "gpu_launches": 6 * args.steps,
        "clocks": clk.summary(),
        "tick_ms_device": ms / args.steps,
        "tick_stats": {"lp3d_per_tick": tot["lp3d"] / args.steps, "replans_per_tick": tot["replans"] / args.steps,
                       "replans_failed_per_tick": tot["replans_failed"] / args.steps,
                       "destroyed_per_tick": tot["destroyed"] / args.steps,
                       "graph_ms_per_tick": tot["device_ms"] / args.steps},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(scene, st, k, threads=1, budget_s=args.cpu_budget)
    sim.close()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    cfg, scene, st, paths, k = make_workload(args.workload, args.seed)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(scene, st, k, threads=threads, budget_s=2.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(scene, st, k, threads=threads, budget_s=min(args.cpu_budget / 2, 120.0 / args.steps)))
    t1 = time.perf_counter()
    v = float(np.median([x["value"] for x in vals]))
    ms = 1e3 * st.num_agents / v
    out = {"impl": "reference", "metric": "agent-steps/s (plain GPU ORCA tick)", "value": v, "unit": "agent-steps/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene, agents and paths)",
           "config": {"workload": args.workload, "agents": st.num_agents, "max_neighbors": k, "seed": args.seed},
           "cpu_baseline": {"value": v, "unit": "agent-steps/s", "cores": threads, "kind": "port",
                            "sample": vals[0]["sample"]},
           "e2e": {"value": v, "unit": "agent-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "wall_s": t1 - t0}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="crossing_1m", choices=sorted(WORKLOADS))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        from ecmgenerator_gb300 import build

        build.build()
        run_ours(args)


if __name__ == "__main__":
    main()
