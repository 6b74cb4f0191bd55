#!/usr/bin/env python3
"""Benchmark of the batched GB300 hot path: whole-job HHT steps/s.

One "step" is one HHT step (predictor + Newton corrector with GMRES solves)
of every simulation of the workload, through the library's C ABI.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workloads (synthetic, seeded; no dataset):
  nets256 — configuration 2: 256 square nets, sides U{20..40} (seed 0), 1 mm
            spacing, xy jitter U(±0.5 mm), r = 0.1 mm, E = 100 GPa, gravity,
            dropped on a sphere R = 15 mm given as a 128³ SDF at 0.3 mm; μ = 0.2,
            Δt = 5e-5 s.

Under torchrun (N > 1) every rank runs its own full copy of the workload on
its GPU (weak scaling; simulations are independent, no collective in the
data path); the timed region is bracketed by barriers and the slowest rank's
time is reported.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# FP64 floating-point operations the device beam kernel executes per element
# evaluation: 202 DADD + 368 DMUL + 714 DFMA counted by ncu's SASS counters on
# k_beam (profiles/beam_kernel_nets16.md).
F_ELEM_FP64 = 1998.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="nets256")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--cpu-sample", type=int, default=2, help="simulations in the CPU-baseline sample")
    ap.add_argument("--cpu-steps", type=int, default=10, help="steps per simulation in the CPU-baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


# ------------------------------------------------------------------ workload

def build_workload(name: str, precision: str = "fp64", rank: int = 0):
    import __graft_entry__ as g
    g.load_package()
    from endobeams_gb300 import scenes
    if name in ("nets256", "nets16"):
        count = 256 if name == "nets256" else 16
        sides = scenes.net_sides(256, seed=0)[:count]
        sdf = scenes.sphere_sdf()
        confs, inters = [], []
        params = None
        for i, side in enumerate(sides):
            c, p, it = scenes.net_on_sphere(int(side), seed=1 + i, sdf=sdf)
            confs.append(c)
            inters.append(it)
            params = p
        params.tolerance_residual = 1e-5
        params.tolerance_displacement = 1e-8
        params.precision = precision
        desc = {"workload": f"{name}: {count} nets (sides U{{20..40}}) on a 128^3 sphere SDF, dt=5e-5",
                "sims": count, "nodes": int(sum(len(c.nodes) for c in confs)),
                "elements": int(sum(len(c.beams) for c in confs)),
                "tolerance_residual": 1e-5, "tolerance_displacement": 1e-8, "precision": precision}
        return confs, params, inters, desc
    raise SystemExit(f"unknown workload {name}")


# ------------------------------------------------------------------ clocks

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ GPU arm

class Driver:
    """The batched time loop of run_simulation! at fixed Δt (the workload's Δt is its maximum)."""

    def __init__(self, eng, params):
        self.eng = eng
        self.p = params
        self.S = eng.n
        self.t = np.zeros(self.S)
        self.dt = np.full(self.S, params.initial_timestep)
        self.ok_steps = 0
        self.newton = 0
        self.krylov = 0
        self.batch_iters = 0

    def step(self, e2e=False, ubuf=None):
        eng = self.eng
        if e2e:
            eng.set_loads_all(eng.loads_all(self.t + self.dt))
        k, _ = eng.step(self.dt)
        st = eng.stats()
        self.newton += sum(s["newton_iterations"] for s in st)
        self.batch_iters += max(s["newton_iterations"] for s in st)
        self.krylov += sum(s["krylov_iterations"] for s in st)
        failed = k > self.p.max_iterations
        ok = ~failed
        if failed.any():
            self.dt[failed] /= 2
            eng.rollback(failed.astype(np.int32))
        eng.commit(ok.astype(np.int32))
        self.t[ok] += self.dt[ok]
        self.ok_steps += int(ok.sum())
        if e2e:
            eng.displacements(ubuf)
        return k


def gpu_arm(args, rank, world):
    import __graft_entry__ as g
    eb = g.load_package()
    from endobeams_gb300 import _lib
    confs, params, inters, desc = build_workload(args.workload, args.precision, rank)
    params.timing = True
    n_gpu, gname = eb.device_info()
    if n_gpu < 1:
        raise SystemExit("no CUDA device")
    eng = eb.GpuSimulations(confs, params, inters)
    drv = Driver(eng, params)
    for _ in range(args.warmup):
        drv.step()
    eng.phase_times(reset=True)
    drv.ok_steps = drv.newton = drv.krylov = 0
    barrier(world)
    clocks = ClockSampler()
    clocks.start()
    eng.timer_start()
    for _ in range(args.steps):
        drv.step()
    ms = eng.timer_stop()
    clk = clocks.stop()
    ms = allreduce_max(ms, world)
    phase_ms, launches = eng.phase_times(reset=True)
    sim_steps = drv.ok_steps
    newton_per_step = drv.newton / max(sim_steps, 1)
    krylov_per_newton = drv.krylov / max(drv.newton, 1)
    value = world * sim_steps / (ms / 1e3)
    # ---- end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        total_nodes = desc["nodes"]
        ubuf = np.zeros((total_nodes, 3))
        n_loaded = sum(len(c.loads.concentrated_force.loaded_dofs) for c in confs if c.loads is not None)
        drv.ok_steps = drv.newton = drv.batch_iters = 0
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            drv.step(e2e=True, ubuf=ubuf)
        wall = allreduce_max(time.perf_counter() - t0, world)
        S = drv.S
        bi = drv.batch_iters / max(args.steps, 1)  # batched Newton iterations per step
        # loads, per-sim step constants (cK, cC, cM, dt), active masks (step + each iteration), commit mask
        h2d = 8 * n_loaded + 32 * S + 4 * S + 4 * S * bi + 4 * S
        # displacements, per-iteration Newton norms, per-step solver statistics
        d2h = 24 * total_nodes + 32 * S * bi + 20 * S
        e2e = {"value": world * drv.ok_steps / wall, "unit": "HHT steps/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
    # ---- roofline of the dominant kernel
    peak_fp64 = eb.fp64_peak_tflops()
    dom = max(phase_ms, key=lambda k: phase_ms[k])
    roof = None
    beam_launches = launches["beam"]
    if beam_launches:
        avg_beam_ms = phase_ms["beam"] / beam_launches
        flops = (F_ELEM_FP64 or float("nan")) * desc["elements"]
        achieved = flops / (avg_beam_ms * 1e-3) / 1e12
        roof = {"kernel": "k_beam (corotational element, FP64)", "bound": "fp64", "achieved": achieved,
                "peak": peak_fp64, "peak_source": "measured (eb_fp64_peak FMA probe on this GPU)",
                "unit": "TFLOP/s", "frac": achieved / peak_fp64, "traffic": None,
                "avg_launch_ms": avg_beam_ms, "share_of_step": phase_ms["beam"] / sum(phase_ms.values())}
    out = {
        "metric": "HHT steps/s (whole job), batched plain Newton",
        "value": value, "unit": "HHT steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64+f32-krylov", "data": "synthetic",
        "config": dict(desc, l2="state and staging arrays exceed L2 (129 MB) each step", device=gname),
        "newton_iters_per_step": newton_per_step, "krylov_iters_per_newton": krylov_per_newton,
        "phase_ms": {k: round(v, 3) for k, v in phase_ms.items()}, "dominant_phase": dom,
        "gpu_launches": int(sum(launches.values())),
        "roofline": roof, "e2e": e2e, "clocks": clk,
    }
    eng.close()
    return out, confs, params, inters, desc


# ------------------------------------------------------------------ CPU arms (oracle restatement)

def cpu_rate(workload, precision, sample, steps, cores):
    """Oracle HHT steps/s on `sample` simulations x `steps` steps with `cores` spawned processes.

    Model construction (pattern, SDF prefilter) happens before each worker's clock starts."""
    idx = list(range(sample))
    chunks = [idx[i::cores] for i in range(cores) if idx[i::cores]]
    if len(chunks) == 1:
        res = [_timed_chunk((workload, precision, chunks[0], steps))]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(len(chunks)) as pool:
            res = pool.map(_timed_chunk, [(workload, precision, c, steps) for c in chunks])
    done = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    return done / wall, wall


def _timed_chunk(payload):
    workload, precision, idx, steps = payload
    import __graft_entry__ as g
    O = g.load_oracle()
    import bridge
    confs, params, inters, _ = build_workload(workload, precision)
    models = [O.OracleModel(bridge.scene_from_conf(confs[i], inters[i]), bridge.params_from(params)) for i in idx]
    t0 = time.perf_counter()
    done = 0
    for m in models:
        done += O.run_simulation(m, max_steps=steps)["steps"]
    return done, time.perf_counter() - t0


# ------------------------------------------------------------------ distributed helpers

def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("LOCAL_RANK", "0"))
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    args = parse()
    rank, world = dist_init()
    if args.impl == "reference":
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        sample = max(args.cpu_sample, cores)
        rate, wall = cpu_rate(args.workload, args.precision, sample, args.cpu_steps, cores)
        _, _, _, desc = build_workload(args.workload, args.precision)
        line = {"metric": "HHT steps/s (whole job), batched plain Newton", "impl": "reference", "value": rate,
                "unit": "HHT steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": desc,
                "cpu_baseline": {"value": rate, "unit": "HHT steps/s", "cores": cores, "kind": "port",
                                 "sample": f"{sample} of {desc['sims']} sims x {args.cpu_steps} steps, "
                                           f"C++ oracle + SciPy SuperLU, {cores} processes, {wall:.1f} s"},
                "e2e": {"value": rate, "unit": "HHT steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    out, confs, params, inters, desc = gpu_arm(args, rank, world)
    if rank == 0:
        if not args.no_cpu:
            rate, wall = cpu_rate(args.workload, args.precision, args.cpu_sample, args.cpu_steps, 1)
            out["cpu_baseline"] = {"value": rate, "unit": "HHT steps/s", "cores": 1, "kind": "port",
                                   "sample": f"{args.cpu_sample} of {desc['sims']} sims x {args.cpu_steps} steps, "
                                             f"C++ oracle + SciPy SuperLU, 1 core, {wall:.1f} s"}
        print(json.dumps(out))


if __name__ == "__main__":
    main()
