"""Trains the learned Newton warm start on trajectories of the plain solver.

    python endobeams.jl_gb300/train_warm_start.py [--sims 64] [--steps 60] [--out PATH]

Runs a population of braided stents (seed 7: a different draw from the
benchmark's seed-2 population) with the HHT predictor on the GPU, capturing
one sample per node and committed step (eb_ws_capture), then fits the per-node
network with the library's own forward/backward kernels (eb_mlp_train) and
writes the model (network, feature and output normalisation) as .npz with a
.json summary beside it.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sims", type=int, default=64)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--stride", type=int, default=1)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=os.path.join(HERE, "models", "warm_start_stents.npz"))
    a = ap.parse_args()

    import __graft_entry__ as g
    eb = g.load_package()
    from endobeams_gb300 import scenes, warm_start as W

    vs = scenes.stent_variants(a.sims, seed=a.seed)
    built = [scenes.stent_variant(v) for v in vs]
    confs = [b[0] for b in built]
    inters = [b[2] for b in built]
    p = built[0][1]
    p.tolerance_residual = 1e-7
    p.tolerance_displacement = 1e-8
    p.krylov_restart = 32
    p.precision = "mixed"
    eng = eb.GpuSimulations(confs, p, inters)
    nodes = sum(len(c.nodes) for c in confs)
    eng.capture(capacity=(nodes // a.stride + 1) * a.steps, stride=a.stride)
    dt = np.full(eng.n, p.initial_timestep)
    t0 = time.time()
    sim_steps = 0
    newton = 0
    for _ in range(a.steps):
        k, _ = eng.step(dt)
        failed = k > p.max_iterations
        if failed.any():
            dt[failed] /= 2
            eng.rollback(failed.astype(np.int32))
        eng.commit((~failed).astype(np.int32))
        sim_steps += int((~failed).sum())
        newton += int(np.sum(k[~failed] - 1))
    F, T = eng.samples()
    eng.close()
    t_cap = time.time() - t0
    t0 = time.time()
    model = W.train_model(F, T, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed)
    t_train = time.time() - t0
    model.info.update({"population": f"{a.sims} stents, stent_variants(seed={a.seed})", "sim_steps": sim_steps,
                       "plain_newton_iters_per_step": newton / max(sim_steps, 1), "capture_s": t_cap,
                       "train_s": t_train, "device": eb.device_info()[1]})
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    model.save(a.out)
    with open(os.path.splitext(a.out)[0] + ".json", "w") as fh:
        json.dump(model.info, fh, indent=1)
    print(json.dumps({k: v for k, v in model.info.items() if k != "train_loss"}))


if __name__ == "__main__":
    main()
