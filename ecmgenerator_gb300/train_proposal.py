"""Train the learned active-set proposal on traces of the plain tick.

    python -m ecmgenerator_gb300.train_proposal --out proposal.npy \
        [--workloads boxes_100k:100,crossing_1m:40] [--rows 50000000] \
        [--steps 20000] [--batch 65536] [--lr 1e-3]

Each workload runs its plain tick (seeds distinct from the benchmark's) in
trace mode; the rows (features, class of the LP result) stay on the GPU and
the network is trained there by the library's own forward/backward kernels.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def collect(workloads, rows, seed, warm=5, every=1):
    import torch

    from . import proposal as P
    from .workloads import make_simulator

    xs, ys = [], []
    per = rows // max(1, len(workloads))
    for i, (name, ticks) in enumerate(workloads):
        sim, _ = make_simulator(name, seed + 101 * i)
        sim.update(ticks=warm)
        x, y = P.collect_traces(sim, ticks=ticks, every=every, max_rows=per)
        sim.close()
        print(f"[train] {name}: {x.shape[0]} rows, classes {json.dumps(P.class_histogram(y))}",
              file=sys.stderr, flush=True)
        xs.append(x)
        ys.append(y)
    x, y = torch.cat(xs), torch.cat(ys)
    return x, y


def train(x, y, steps, batch, lr, seed=0, model=None):
    from . import proposal as P

    m = model or P.ProposalModel(seed=seed)
    t0 = time.time()
    loss, acc = m.train(x, y, steps=steps, batch=batch, lr=lr, seed=seed + 7)
    dt = time.time() - t0
    print(f"[train] {steps} steps of {batch} in {dt:.1f}s; loss {loss[:10].mean():.3f} -> {loss[-100:].mean():.3f}, "
          f"accuracy {acc[-100:].mean():.3f}", file=sys.stderr, flush=True)
    return m, dict(seconds=dt, loss_first=float(loss[:10].mean()), loss_last=float(loss[-100:].mean()),
                   acc_last=float(acc[-100:].mean()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--workloads", default="boxes_100k:100,crossing_1m:40")
    ap.add_argument("--rows", type=float, default=50e6)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1000)
    a = ap.parse_args()
    from . import build

    build.build()
    wl = [(w.split(":")[0], int(w.split(":")[1])) for w in a.workloads.split(",")]
    x, y = collect(wl, int(a.rows), a.seed)
    m, info = train(x, y, a.steps, a.batch, a.lr, seed=a.seed)
    np.save(a.out, m.get_params())
    info.update(rows=int(x.shape[0]), workloads=a.workloads, steps=a.steps, batch=a.batch, lr=a.lr)
    print(json.dumps(info), flush=True)


if __name__ == "__main__":
    main()
