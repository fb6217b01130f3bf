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
import gc
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from ecmgenerator_gb300.workloads import DT, ORCA, WORKLOADS  # noqa: E402


def KD_BYTES_PER_AGENT(k, levels=20):
    """algorithmic bytes per agent of the kd-tree neighbour pipeline: member
    list and slot-order compaction 31, four key gathers 80, four 4-pass radix
    sorts of (key, value) 320, segment init 12, per level side / flags /
    scan / partition 95 (level 0 partitions two lists, +61), query 12 + 4k,
    composition 2 + 8k, emission 14 + 17k"""
    return 532 + 95 * levels + 29 * k


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(name, seed, planner="reference"):
    from ecmgenerator_gb300.workloads import make_workload as mk

    return mk(name, seed, planner=planner)


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
            # the first query of a fresh nvidia-smi holds the driver for ~10 ms:
            # let it happen before the timed region starts
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0:
                time.sleep(0.02)
            time.sleep(0.3)
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
            time.sleep(0.3)  # the sampler's exit, like its start, briefly holds the driver

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


def load_or_train_model(plain, learned, args):
    """The proposal network: committed weights when present, else trained
    here on traces of 8 plain ticks (both simulators advance by 8 ticks, so
    they stay in the same state)."""
    from ecmgenerator_gb300 import proposal as P

    m = P.ProposalModel(seed=0)
    path = args.proposal or os.path.join(HERE, "ecmgenerator_gb300", "data", "proposal.npy")
    if os.path.exists(path):
        m.load(path)
        return m, {"weights": os.path.relpath(path, HERE)}
    t0 = time.time()
    x, y = P.collect_traces(plain, ticks=8)
    learned.update(ticks=8)
    loss, acc = m.train(x, y, steps=1500, batch=65536, lr=1e-3, seed=3)
    info = {"weights": "trained in this run on traces of its own warm-up ticks", "rows": int(x.shape[0]),
            "steps": 1500, "batch": 65536, "train_s": time.time() - t0, "loss": float(loss[-50:].mean()),
            "acc": float(acc[-50:].mean()), "classes": P.class_histogram(y)}
    log(f"[bench] trained proposal: {info}")
    del x, y
    return m, info


def apply_launch(plain, learned, args):
    """launch configuration of the per-agent kernel: autotuned on the plain
    simulator's current state (restored afterwards), or fixed by --lp-mode"""
    from ecmgenerator_gb300.simulator import autotune, set_launch, set_lp_mode

    if args.lp_mode == "tune":
        r = autotune(plain, ticks_per_trial=2)
        log(f"[bench] autotune: {r}")
        grab = r["agents_per_warp_grab"]
        for s_ in (plain, learned):
            if r["lp_mode"] == "warp":
                set_launch(s_, 128, 32, r["grid_cell_scale"], 1, r["neighbor_blocks_per_sm"])
                set_lp_mode(s_, "warp", grab)
            else:
                set_launch(s_, r["block_size"], grab, r["grid_cell_scale"], r["occupancy_divisor"],
                           r["neighbor_blocks_per_sm"])
                set_lp_mode(s_, r["lp_mode"], 1)
        return r
    grab = 4 if args.lp_mode == "warp" else 32
    for s_ in (plain, learned):
        if args.grid_scale > 0:
            set_launch(s_, 128, 32, args.grid_scale)
        set_lp_mode(s_, args.lp_mode, grab if args.lp_mode == "warp" else 1)
    return {"lp_mode": args.lp_mode, "agents_per_warp_grab": grab, "grid_cell_scale": args.grid_scale or None}


class TickTimer:
    """CUDA events on the library's stream around each tick, L2 flushed
    (512 MB write, > 129 MB L2) before every timed tick."""

    def __init__(self, sim, flush):
        import torch

        self.sim = sim
        self.stream = torch.cuda.ExternalStream(sim.L.ecmg_stream(sim.h))
        self.flush = flush
        self.ev = []
        self.per_tick = []  # (graph ms, host ms) of each timed tick
        self.steps = 0
        self.agent_ms = 0.0
        self.tot = dict(lp3d=0, replans=0, replans_failed=0, replans_host=0, destroyed=0, device_ms=0.0, host_ms=0.0,
                        proposed=0, accepted=0, gated=0, attract_ms=0.0, neighbors_ms=0.0, proposal_ms=0.0,
                        orca_ms=0.0, spawned=0, spawn_failed=0, spawn_refused=0, spawn_ms=0.0, spawn_check_ms=0.0,
                        spawn_candidates=0, graph_builds=0, spawn_kernels=0)

    def tick(self):
        import torch

        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(self.stream):
            self.flush.zero_()
            e0.record(self.stream)
        s = self.sim.update()
        with torch.cuda.stream(self.stream):
            e1.record(self.stream)
        self.ev.append((e0, e1))
        self.per_tick.append((round(s.device_ms, 3), round(s.host_ms, 3)))
        self.steps += s.agent_steps
        self.agent_ms += s.agent_kernel_ms
        for k in self.tot:
            self.tot[k] += getattr(s, k)
        return s

    def ms(self):
        return sum(a.elapsed_time(b) for a, b in self.ev)


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from ecmgenerator_gb300.simulator import Simulator
    from ecmgenerator_gb300.workloads import add_spawn_areas

    batch = WORKLOADS[args.workload].get("batch")
    if batch:
        if args.spawn_rate > 0 or args.neighbors != "exact":
            raise SystemExit("batch workloads run the exact neighbour mode without spawn areas")
        from ecmgenerator_gb300.simulator import BatchSimulator
        from ecmgenerator_gb300.workloads import make_batch_workload

        cfgs, scenes, states, pathss, k = make_batch_workload(args.workload, args.seed)
        n = sum(x.num_agents for x in states)
        big = int(np.argmax([x.num_agents for x in states]))
        # the CPU baseline samples the largest scene
        cfg, scene, st, paths = cfgs[big], scenes[big], states[big], pathss[big]
        scene_desc = (f"{len(scenes)} independent scenes, side U[50,500] m, side/5 boxes of side U[2,8] m, "
                      f"{min(x.num_agents for x in states)}-{max(x.num_agents for x in states)} agents per scene")
        sims = []
        for _ in range(2):
            s_ = BatchSimulator(scenes, [x.num_agents for x in states], DT, max_neighbors=k, **ORCA)
            for i, x in enumerate(states):
                m = x.num_agents
                s_.add_agents(x.pos[:m], x.clear[:m], x.pref_speed[:m], pathss[i], scene=i)
            sims.append(s_)
        spawn_slots = 0
    else:
        cfg, scene, st, paths, k = make_workload(args.workload, args.seed, args.planner)
        n = st.num_agents
        scene_desc = f'{cfg["w"]:.0f}x{cfg["h"]:.0f} m, {cfg["boxes"]} boxes'
        sims = []
        spawn_slots = 0
    # two simulators in the same state: the plain tick and the tick with the
    # learned proposal (their trajectories are identical)
    if args.spawn_rate > 0:
        # room for the spawned agents; every simulator draws the same
        # recorded random stream (the C library's rand() is shared)
        spawn_slots = min(200_000, int(args.spawn_rate * DT * 4 * 2000) + 1024)
        stream = np.random.default_rng(args.seed + 99).integers(
            0, 2147483647, 33 * (int(args.spawn_rate * DT) + 1) * 4 * 4000, dtype=np.int32)
    for _ in range(0 if batch else 2):
        s_ = Simulator(scene, n + spawn_slots, DT, max_neighbors=k, lp3d_fp64=args.lp3d_fp64, **ORCA)
        s_.add_agents(st.pos[:n], st.clear[:n], st.pref_speed[:n], paths)
        if args.spawn_rate > 0:
            add_spawn_areas(s_, scene, args.spawn_rate)
            s_.push_spawn_random(stream)
        sims.append(s_)
    plain, learned = sims
    if args.planner != "reference":
        from ecmgenerator_gb300.simulator import set_planner_mode

        for s_ in sims:
            set_planner_mode(s_, args.planner)
    if args.neighbors == "kdtree":
        # the reference's kd-tree query (no learned proposal in this mode)
        from ecmgenerator_gb300.simulator import set_neighbor_mode

        for s_ in sims:
            set_neighbor_mode(s_, "kdtree")
        args.plain_only = True
        if args.lp_mode == "warp":
            args.lp_mode = "thread"
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    plain.update()
    learned.update()
    launch = apply_launch(plain, learned, args)
    for _ in range(args.warmup):
        plain.update()
        learned.update()
    model, model_info = load_or_train_model(plain, learned, args) if not args.plain_only else (None, None)
    if model is not None:
        learned.set_proposal(model)
        if args.no_gate:
            learned.set_proposal_gate(0.0, 0)
        learned.update()  # capture of the learned graph
        plain.update()
    torch.cuda.synchronize()
    # the workload holds ~1M small path arrays: a cyclic-GC pass over them
    # stalls the host for ~10 ms, so collect now and keep the collector off
    # while timing
    gc.collect()
    gc.freeze()
    gc.disable()
    tp, tl = TickTimer(plain, flush), TickTimer(learned, flush)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        # alternating blocks of plain and learned ticks (each simulator ends
        # K ticks later, in the same state as the other)
        nblk = 4 if args.steps >= 4 else 1
        bounds = [args.steps * b // nblk for b in range(nblk + 1)]
        for b in range(nblk):
            for i in range(bounds[b], bounds[b + 1]):
                tp.tick()
            if model is not None:
                for i in range(bounds[b], bounds[b + 1]):
                    tl.tick()
        torch.cuda.synchronize()
    blocks = {"plain_ms": [round(sum(a.elapsed_time(c) for a, c in tp.ev[bounds[b]:bounds[b + 1]]), 3)
                           for b in range(nblk)],
              "plain_tick_ms": [round(a.elapsed_time(c), 3) for a, c in tp.ev],
              "plain_graph_host_ms": tp.per_tick}
    if model is not None:
        blocks["learned_ms"] = [round(sum(a.elapsed_time(c) for a, c in tl.ev[bounds[b]:bounds[b + 1]]), 3)
                                for b in range(nblk)]
    same = bool(np.array_equal(plain.get_position_data(), learned.get_position_data()))
    main_t = tl if model is not None else tp
    ms = main_t.ms()
    ms_all, steps_all = reduce_over_ranks(ms, main_t.steps, world, "cuda")
    value = steps_all / (ms_all / 1e3)
    p_ms_all, p_steps_all = reduce_over_ranks(tp.ms(), tp.steps, world, "cuda")
    plain_value = p_steps_all / (p_ms_all / 1e3)
    no_gate = None
    if model is not None and not args.no_gate:
        # the learned tick with the model forced on every tick (no gate),
        # K ticks after the timed blocks: what the model itself costs here;
        # the gate is restored afterwards (the e2e run below uses it)
        learned.set_proposal_gate(0.0, 0)
        for _ in range(2):
            learned.update()
        tn = TickTimer(learned, flush)
        torch.cuda.synchronize()
        for _ in range(args.steps):
            tn.tick()
        torch.cuda.synchronize()
        learned.set_proposal_gate(0.1, 64)
        n_ms, n_steps = reduce_over_ranks(tn.ms(), tn.steps, world, "cuda")
        K_ = max(args.steps, 1)
        no_gate = {"value": n_steps / (n_ms / 1e3), "ms_per_step": n_ms / K_,
                   "vs_plain": (n_steps / (n_ms / 1e3)) / plain_value,
                   "proposed_per_tick": tn.tot["proposed"] / K_, "accepted_per_tick": tn.tot["accepted"] / K_,
                   "features_and_inference_ms_per_tick": tn.tot["proposal_ms"] / K_,
                   "per_agent_kernel_ms_per_tick": tn.tot["orca_ms"] / K_,
                   "note": "the learned tick with the gate open on every tick (model on), timed after the "
                           "gated blocks; 2D LPs with a proposal are those the model did not class as other"}
    # e2e through the public API: update + positions/velocities back to host
    e2e = {}
    for name, sim in (("learned", learned), ("plain", plain)):
        if name == "learned" and model is None:
            continue
        e2e_steps = 0
        # every tick ends by writing the getters' host arrays
        sim.set_host_mirror(True)
        for _ in range(args.warmup):
            sim.update()
            _ = sim.view("position")
            _ = sim.view("velocity")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s = sim.update()
            _ = sim.view("position")  # ecmg_host_view: the reference's getters (raw host pointers)
            _ = sim.view("velocity")
            e2e_steps += s.agent_steps
        t1 = time.perf_counter()
        e2e[name] = e2e_steps * max(world, 1) / (t1 - t0)
    gc.enable()
    e2e_main = {"value": e2e["learned" if model is not None else "plain"], "unit": "agent-steps/s",
                "h2d_bytes_per_step": 64, "d2h_bytes_per_step": 16 * n + 64,
                "plain": e2e["plain"], "note": "wall clock of Simulator.update() + the position and velocity getters "
                "(ecmg_host_view) per tick; each tick ends with a device copy of the positions and velocities "
                "into the page-locked host arrays the getters return (ecmg_set_host_mirror); h2d = counters, d2h = positions and velocities + "
                "counters"}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs") or 6800.0
    per_tick = main_t.steps / max(args.steps, 1)
    # the dominant kernel of the tick by measured device time, with its
    # algorithmic bytes per agent: k_neighbors reads its snapshot position and
    # writes k neighbour indices (candidate positions are cache reuse);
    # k_agents reads the snapshot (pos, vel, radius), speed, preferred
    # velocity, active flag, slot, neighbour count and k indices, and writes
    # pos and vel
    kern = {"k_neighbors": (main_t.tot["neighbors_ms"], 8 + 4 * k), "k_agents": (main_t.tot["orca_ms"], 57 + 4 * k)}
    fused = launch.get("lp_mode") == "fused" and args.neighbors != "kdtree"
    if fused:
        # the search inside the per-agent kernel: the agent's state in and
        # out (snapshot pos, vel, radius, speed, preferred velocity, active
        # flag, slot in; pos, vel out); the lists it writes and reads back
        # are intermediate
        kern = {"k_agents_knn": (main_t.tot["orca_ms"], 53)}
    if args.neighbors == "kdtree":
        # the kd-tree pipeline (build, query, cache composition) in place of
        # k_neighbors; its algorithmic bytes per agent are derived in DESIGN
        kern = {"kd-tree pipeline": (main_t.tot["neighbors_ms"], KD_BYTES_PER_AGENT(k, (n + spawn_slots).bit_length())),
                "k_agents": (main_t.tot["orca_ms"], 57 + 4 * k)}
    kernel_ms = {"k_attract": main_t.tot["attract_ms"] / args.steps}
    if not fused:
        kernel_ms["k_neighbors"] = main_t.tot["neighbors_ms"] / args.steps
    kernel_ms["features+k_mlp_infer"] = main_t.tot["proposal_ms"] / args.steps
    kernel_ms["k_agents_knn" if fused else "k_agents"] = main_t.tot["orca_ms"] / args.steps
    kname = max(kern, key=lambda q: kern[q][0])
    kern_ms = kern[kname][0] / max(args.steps, 1)
    alg_bytes = kern[kname][1]
    achieved = alg_bytes * per_tick / (kern_ms / 1e3) / 1e9 if kern_ms > 0 else 0.0
    traffic = None
    limiter = None
    tf = os.path.join(HERE, "profiles", "kernel_traffic.json")
    if os.path.exists(tf):
        try:
            rec = json.load(open(tf)).get(kname, {})
            t = rec.get(args.workload)
            if t:
                traffic = t * per_tick
            # the pipe that bounds the kernel in its ncu capture (neither kernel
            # streams memory, so the HBM fraction alone does not name the bound)
            limiter = rec.get("limiter")
        except (OSError, ValueError, AttributeError):
            traffic = None
    T = main_t.tot
    launches = plain.L.ecmg_kernels_per_tick(plain.h) * args.steps + tp.tot["spawn_kernels"]
    if model is not None:
        launches += learned.L.ecmg_kernels_per_tick(learned.h) * (args.steps - T["gated"]) + \
            plain.L.ecmg_kernels_per_tick(plain.h) * T["gated"] + tl.tot["spawn_kernels"]
    out = {
        "metric": "agent-steps/s at 1M agents: learned-proposal vs plain GPU ORCA; ms/tick",
        "value": value, "unit": "agent-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_all / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded scene, agents and paths)",
        "config": workload_config(args, n, k, scene_desc, world),
        "mode": "learned proposal" if model is not None else "plain",
        "lp3d_projection": "fp64" if args.lp3d_fp64 else "fp32 (the reference's)",
        "neighbors": "exact (d2, index)" if args.neighbors == "exact" else "kd-tree (the reference's query)",
        # what the parity tests establish for this arithmetic (not measured by this run)
        "parity": {
            "vs_oracle": "bit-identical neighbour lists, LP results, positions and velocities every tick "
                         "(tests/test_gpu_tick.py); at full size (this 1M crossing, the 100k box scene, the 1.3M "
                         "batch) 600 ticks with 2,000 agents checked bit for bit at ticks 0, 1, 2, 100, 300, 599 "
                         "(tests/test_gpu_fullsize.py)",
            "oracle_vs_reference": "the C oracle equals the reference's own sources compiled here, bit for bit, "
                                   "600 ticks x 1,000 agents (tests/test_oracle_vs_reference.py)",
            "vs_reference_libm": "per tick every velocity within 1e-5 relative of the reference's libm run (max "
                                 "7.9e-8); after 600 ticks 942 of 955 agents within 1e-3 m of its positions (max "
                                 "3.2 cm), where FP32 itself puts 89-92 agents beyond 1e-3 m of an FP64 run "
                                 "(tests/test_oracle_fp64.py)",
        },
        "launch": launch,
        "plain": {"value": plain_value, "ms_per_step": p_ms_all / args.steps,
                  "lp3d_per_tick": tp.tot["lp3d"] / args.steps,
                  "graph_ms_per_tick": tp.tot["device_ms"] / args.steps,
                  "host_ms_per_tick": tp.tot["host_ms"] / args.steps,
                  "replans_host_per_tick": tp.tot["replans_host"] / args.steps},
        "learned_vs_plain": value / plain_value if model is not None else None,
        "timed_blocks": blocks,
        "proposal": None if model is None else {
            **model_info, "proposed_per_tick": T["proposed"] / args.steps,
            "accepted_per_tick": T["accepted"] / args.steps,
            "acceptance_rate": T["accepted"] / max(1, main_t.steps), "gated_ticks": T["gated"],
            "trajectories_identical": same, "no_gate": no_gate},
        "e2e": e2e_main,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "kernel": kname, "kernel_ms": kern_ms, "alg_bytes_per_agent": alg_bytes,
                     "compute_frac": (limiter or {}).get("compute_frac"),
                     "compute_pipe": (limiter or {}).get("compute_pipe"),
                     "limiter": limiter,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s",
                     "kernel_ms_per_tick": kernel_ms},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "tick_stats": {"lp3d_per_tick": T["lp3d"] / args.steps, "replans_per_tick": T["replans"] / args.steps,
                       "replans_failed_per_tick": T["replans_failed"] / args.steps,
                       "replans_host_per_tick": T["replans_host"] / args.steps,
                       "destroyed_per_tick": T["destroyed"] / args.steps,
                       "graph_ms_per_tick": T["device_ms"] / args.steps,
                       "host_ms_per_tick": T["host_ms"] / args.steps,
                       "graph_builds": T["graph_builds"]},
    }
    if args.spawn_rate > 0:
        K = max(args.steps, 1)
        out["spawn"] = {"areas": 4, "rate_per_area": args.spawn_rate, "spawned_per_tick": T["spawned"] / K,
                        "no_location_per_tick": T["spawn_failed"] / K, "refused_per_tick": T["spawn_refused"] / K,
                        "candidates_per_tick": T["spawn_candidates"] / K, "stage_ms_per_tick": T["spawn_ms"] / K,
                        "check_ms_per_tick": T["spawn_check_ms"] / K,
                        "note": "UpdateSpawnAreas at the start of every timed tick (inside the timed region): "
                                "candidate locations tested on the device against all agents, spawned agents "
                                "planned on the host; stage_ms includes the planning, check_ms the device test "
                                "with its copies and wait"}
        out["spawn_rate_per_area"] = args.spawn_rate
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(scene, st, k, threads=1, budget_s=args.cpu_budget)
    for s_ in sims:
        s_.close()
    if model is not None:
        model.close()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def workload_config(args, n, k, scene_desc, world):
    """the `config` object of both arms: the workload only"""
    return {"workload": args.workload, "agents": n, "max_neighbors": k, "neighbor_dist_m": 5.0,
            "time_horizon_s": 2.0, "dt_s": DT, "scene": scene_desc,
            "l2": "inputs larger than L2 (agent state ~0.2 GB at 1M agents); the GPU arm also flushes L2 "
                  "(512 MB write) before every timed tick",
            "parallelism": f"replicas x{world}", "seed": args.seed, "planner": args.planner}


def run_reference(args):
    """The reference's CPU tick on the host cores: the C port of
    Simulator::Update (pinned bit for bit to the reference's own sources on
    x86-64) in the reference's kd-tree neighbour mode with the host libm,
    whole ticks on every host thread (og_tick_mt), re-plans served inside the
    timed tick by the port of ECMPathPlanner::FindPath.  Scene, agents and
    initial paths are built without the product library (the oracle's planner
    plans them), so nothing of the GPU library is loaded in this process."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    if WORKLOADS[args.workload].get("batch"):
        raise SystemExit("the reference arm runs single-scene workloads")
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as orc
    from ecmgenerator_gb300.workloads import make_workload as mk

    orc.build()
    port = orc.Port()
    threads = os.cpu_count() or 1
    t0 = time.time()
    holder = {}

    def plan(scene, a_, b_, c_):
        if "E" not in holder:
            holder["E"] = port.ecm(scene.ecm)
        return port.find_paths(holder["E"], a_, b_, c_, threads=threads, cap=256)

    cfg, scene, st, paths, k = mk(args.workload, args.seed, planner="reference", plan=plan)
    del paths
    setup_s = time.time() - t0
    n = st.num_agents
    O, E = port.obstacles(scene), holder["E"]
    P = port.params(k=k, libm=1, knn_mode=1, **ORCA)
    kd = port.kdtree(k)
    stats = dict(replans=0, replans_ok=0, destroyed=0, lp3d=0)

    def tick():
        agents = st.num_agents
        destroyed, replan, rpos, nlp3d = port.tick_mt(O, E, st, P, kd, threads)
        if replan.size:
            # Simulator::UpdatePath from the tick-start position to the path's goal
            got = port.find_paths(E, rpos, st.goals(replan), st.clear[replan], threads=threads, cap=256)
            st.replace_paths(replan, got)
            stats["replans_ok"] += sum(g_ is not None for g_ in got)
        stats["replans"] += int(replan.size)
        stats["destroyed"] += int(destroyed.size)
        stats["lp3d"] += int(nlp3d)
        return agents

    for _ in range(args.warmup):
        tick()
    for key in stats:
        stats[key] = 0
    times, steps = [], 0
    for _ in range(args.steps):
        t1 = time.perf_counter()
        steps += tick()
        times.append(time.perf_counter() - t1)
    total = sum(times)
    v = steps / total
    one = cpu_baseline(scene, st, k, threads=1, budget_s=args.cpu_budget)
    out = {"impl": "reference", "metric": "agent-steps/s at 1M agents: learned-proposal vs plain GPU ORCA; ms/tick",
           "value": v, "unit": "agent-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded scene, agents and paths)",
           "config": workload_config(args, n, k, f'{cfg["w"]:.0f}x{cfg["h"]:.0f} m, {cfg["boxes"]} boxes', world),
           "neighbors": "kd-tree (the reference's KDTree query, neighbour cache per thread)",
           "cpu_baseline": {"value": v, "unit": "agent-steps/s", "cores": threads,
                            "kind": "port (C restatement of the reference, pinned bit for bit to the reference's "
                                    "own sources on x86-64)",
                            "sample": f"{args.steps} whole ticks of all {n} agents after {args.warmup} warm-up "
                                      f"ticks, state advanced tick by tick, re-plans inside the timed ticks, "
                                      f"{threads} host threads"},
           "one_thread": one,
           "e2e": {"value": v, "unit": "agent-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "tick_ms": [round(1e3 * x, 1) for x in times],
           "tick_stats": {k_: v_ / max(args.steps, 1) for k_, v_ in stats.items()},
           "setup_s": setup_s}
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
    ap.add_argument("--plain-only", action="store_true", help="time the plain tick only")
    ap.add_argument("--neighbors", default="exact", choices=["exact", "kdtree"],
                    help="exact kNN (default) or the reference's kd-tree query with its neighbour cache")
    ap.add_argument("--spawn-rate", type=float, default=0.0,
                    help="agents/s per spawn area, 4 spawn areas (UpdateSpawnAreas every tick); 0: none")
    ap.add_argument("--planner", default="reference", choices=["reference", "fast"],
                    help="host planner of the initial paths and re-plans: the reference's FindPath restated "
                         "(default) or the opt-in fast A* (not the reference's paths)")
    ap.add_argument("--proposal", default=None, help="proposal weights (.npy)")
    ap.add_argument("--no-gate", action="store_true", help="keep the proposal model on every tick")
    ap.add_argument("--lp-mode", default="tune", choices=["tune", "thread", "warp", "fused"],
                    help="per-agent kernel layout (default: autotuned)")
    ap.add_argument("--lp3d-fp64", action="store_true",
                    help="build the 3D-LP bisector intersections in FP64 (ecmg_params.lp3d_fp64)")
    ap.add_argument("--grid-scale", type=float, default=0.0,
                    help="with a fixed --lp-mode: agent-grid cell scale (cell = scale * sqrt(k / density))")
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
