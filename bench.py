#!/usr/bin/env python3
"""Benchmark of the batched GB300 hot path: whole-job HHT steps/s and Newton iterations/step.

One "step" is one HHT step (predictor + Newton corrector with GMRES solves)
of every simulation of the workload, through the library's C ABI.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workloads (synthetic, seeded; no dataset):
  stents1024 (default) — 1024 braided stents drawn with seed 2: wires in
            {16,24,32,48}, radius U[3,5] mm, pitch U[35,55] deg, elements per
            wire U{100..400}, length ~20 mm, crossings merged, r = 0.05 mm,
            E = 50 GPa, each released stress free into its own cylinder SDF
            (radius U[0.85,0.95] of the stent's, 0.1 mm grid sized to the stent);
            mu = 0.1, dt = 1e-5 s, FP32 GMRES inside FP64 refinement.  The
            population runs as resident groups sized to the device memory,
            each group as concurrent lanes (--lanes, default 4: one engine,
            host thread and CUDA stream each, so one lane's kernels fill the
            SMs another lane's Newton tail leaves idle); the learned warm start (committed model) gives the initial guess
            of each predictor solve.  The line also carries the same groups
            and step window with the plain HHT predictor, and the plain
            single-stent path (48 wires, R = 4 mm, 45 deg, 200 elements per
            wire, cylinder 3.5 mm) on the same GPU.
  stent   — the single 48-wire stent above.
  nets256 — 256 square nets, sides U{20..40} (seed 0), 1 mm spacing, xy jitter
            U(±0.5 mm), r = 0.1 mm, E = 100 GPa, gravity, dropped on a sphere
            R = 15 mm given as a 128³ SDF at 0.3 mm; mu = 0.2, dt = 5e-5 s.

Under torchrun (N > 1) every rank binds the GPU of its local rank and
simulates its own shard of a population N times as large (weak scaling;
simulations are independent, no collective in the data path); the timed
region is bracketed by barriers and the slowest rank's time is reported.
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
# evaluation: 1,702 DADD + 3,085 DMUL + 5,987 DFMA (FMA = 2) counted by ncu's
# SASS counters on a launch in which every element of a 48-wire stent is
# evaluated.
F_ELEM_FP64 = 1702.0 + 3085.0 + 2 * 5987.0
# The algorithmic count of the same evaluation, from the oracle's restatement compiled over an
# operation-counting double (oracle/flop_count.cpp, tests/test_flop_count.py): adds, multiplies,
# divides and square roots of one undamped element (the stents' damping is zero).
F_ELEM_ALGORITHMIC = 12153.0 + 14362.0 + 164.0 + 8.0

# Bytes one contact-element evaluation must read: both node records (X0, u, u_dot, w_dot: 12
# doubles; R, dR: 18) = 480 B, the element's R_e0, l0, radius (88 B), its index words (13 B)
# and the 27-coefficient quadratic B-spline stencil at each of the 3 Gauss points (648 B).
# Elements in contact also write their 2.4 KB of tangents; those writes are not counted.
B_CONTACT_ELEM = 480.0 + 88.0 + 13.0 + 648.0

# DRAM bytes k_gmres moves per algorithmic byte (band, inverses, tangent): 158.2 GB read + written
# against 151.9 GB algorithmic over the 24 k_gmres launches of 2 steps of 16 stents (ncu
# dram__bytes_read.sum + dram__bytes_write.sum); the full workload's launches are too large to
# capture, so the line scales its algorithmic bytes per launch by this ratio.
KRYLOV_TRAFFIC_RATIO = 158.2 / 151.9

METRIC = "HHT steps/s & Newton iters/step, batched+learned vs plain"
MODEL = os.path.join(ROOT, "endobeams.jl_gb300", "models", "warm_start_stents.npz")
# Newton tolerances of the stents.  The configurations ask for 1e-8.  The normalised residual of
# the reference's algorithm has an FP64 floor that grows as the elements get shorter (rounding
# of the element forces against the small contact and inertial loads; measured with the oracle:
# 2e-9 at 0.15 mm elements, 1e-8 at 0.094 mm, 2.4e-8 at 0.071 mm); a stent whose floor is above
# its tolerance never converges.  Stents with elements of at least 0.12 mm (floor <= 5e-9) run
# at 1e-8, shorter-element stents at 1e-7; the displacement tolerance is 1e-8 for all.
STENT_TOL_RES = 1e-8
STENT_TOL_RES_SHORT = 1e-7
STENT_ELEM_1E8 = 0.12e-3
STENT_TOL_DISP = 1e-8
# Inexact Newton: each Newton solve runs GMRES (FP32 inner, FP64 refinement) to 1e-4 of its
# right-hand side instead of 1e-10.  Every step still converges to the same residual and
# displacement tolerances (64 stents: 4.03 Newton iterations per step instead of 3.89, states
# within 1e-14 m of the 1e-10 runs; 2.4x the HHT steps/s).
NEWTON_FORCING = 1e-4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="stents1024")
    ap.add_argument("--precision", default=None, choices=[None, "fp64", "mixed"])
    ap.add_argument("--warm-start", default=None, choices=[None, "off", "learned", "learned_x0"])
    ap.add_argument("--count", type=int, default=None, help="population size override (stents)")
    ap.add_argument("--band-lu", default="tensor", choices=["fp32", "tensor"],
                    help="band LU engine of the stents' preconditioner")
    ap.add_argument("--refactor", default="cost", choices=["threshold", "cost", "always"],
                    help="stents: when a band LU is refactorised")
    ap.add_argument("--refactor-cost", type=float, default=0.12,
                    help="--refactor cost: GMRES iterations one LU is worth per DOF of half bandwidth "
                         "(256 stents with four lanes, 15 steps: 0.05 112.7, 0.08 115.5, 0.12 124.1, "
                         "0.16 125.8, 0.24 115.4 HHT steps/s)")
    ap.add_argument("--mem-frac", type=float, default=0.75, help="device memory fraction per resident group")
    ap.add_argument("--lanes", type=int, default=4,
                    help="concurrent lanes per resident group (one engine, host thread and stream each)")
    ap.add_argument("--cpu-sample", type=int, default=2, help="simulations in the CPU-baseline sample of the GPU arm")
    ap.add_argument("--cpu-steps", type=int, default=3, help="steps per simulation in that CPU-baseline sample")
    ap.add_argument("--ref-sample", type=int, default=48,
                    help="--impl reference: simulations spread over the population, each warmed up and timed "
                         "over the same step window as the GPU arm")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-batch and single-stent legs")
    ap.add_argument("--output-every", type=int, default=0,
                    help="add a VTK-output leg: write every K steps (0: off)")
    ap.add_argument("--output-sims", type=int, default=16, help="simulations of the VTK-output leg")
    ap.add_argument("--output-dir", default=None, help="directory of the VTK-output leg (default: a temporary one)")
    return ap.parse_args()


# ------------------------------------------------------------------ workloads

def _pkg():
    import __graft_entry__ as g
    return g.load_package()


def stent_tol_res(conf):
    """Residual tolerance of one stent: 1e-8 unless its mean element is shorter than 0.12 mm."""
    X, c = conf.nodes.X0, conf.beams.conn
    le = float(np.linalg.norm(X[c[:, 1]] - X[c[:, 0]], axis=1).mean())
    return STENT_TOL_RES if le >= STENT_ELEM_1E8 else STENT_TOL_RES_SHORT


SOLVER = dict(band_lu="tensor", refactor="cost", refactor_cost=0.12)  # set from the command line


def stent_params(p, precision="mixed", warm="off"):
    p.tolerance_residual = STENT_TOL_RES
    p.tolerance_displacement = STENT_TOL_DISP
    p.krylov_restart = 32
    # a stent's band LU costs ~0.1-1.5 s on one SM: it is reused, and refactorised by the cost rule
    # when the GMRES iterations lost to its ageing reach its cost (64 stents, 20 steps: 15.2 HHT
    # steps/s refactorising only past 200 iterations, 26-29 by the cost rule); 200 stays a cap
    p.refactor_its = 0 if SOLVER["refactor"] == "always" else 200
    p.refactor_policy = "cost" if SOLVER["refactor"] == "cost" else "threshold"
    p.refactor_cost = SOLVER["refactor_cost"]
    p.band_lu = SOLVER["band_lu"]
    p.linear_tol = NEWTON_FORCING
    p.precision = precision
    p.warm_start = warm
    return p


def shard(sizes, per_rank, rank, world):
    """Indices of this rank's simulations: the population of per_rank x world simulations split
    into equal-count shards by a greedy balance on size (largest first to the least-loaded rank
    with room), returned in population order.  One rank gets the whole population."""
    if world == 1:
        return list(range(len(sizes)))
    load = [0] * world
    cnt = [0] * world
    mine = []
    for i in sorted(range(len(sizes)), key=lambda i: (-sizes[i], i)):
        r = min((q for q in range(world) if cnt[q] < per_rank), key=lambda q: (load[q], q))
        load[r] += sizes[i]
        cnt[r] += 1
        if r == rank:
            mine.append(i)
    return sorted(mine)


class Workload:
    """A named workload: simulations built lazily in resident groups; under torchrun each
    rank builds its own shard of a population world times as large (weak scaling)."""

    def __init__(self, name, precision=None, warm=None, count=None, rank=0, world=1):
        _pkg()
        from endobeams_gb300 import scenes
        self.scenes = scenes
        self.name = name
        self.kind = "stents" if name.startswith("stent") else "nets"
        if self.kind == "nets":
            if name not in ("nets256", "nets16"):
                raise SystemExit(f"unknown workload {name}")
            self.count = 256 if name == "nets256" else 16
            sides = scenes.net_sides(max(256, self.count * world), seed=0)[:self.count * world]
            self.sides = [sides[i] for i in shard(list(sides), self.count, rank, world)]
            self.precision = precision or "fp64"
            self.warm = "off"
            self.sdf = None
        else:
            import re
            m = re.fullmatch(r"stent(\d+)x(\d+)", name)
            if name == "stent":
                self.variants = [None]
            elif m:  # one stent with the given wires x elements per wire (profiling size)
                self.variants = [("custom", int(m.group(1)), int(m.group(2)))]
            elif name.startswith("stents"):
                n = count or int(name[len("stents"):] or 1024)
                allv = scenes.stent_variants(max(1024, n * world), seed=2)[:n * world]
                self.variants = [allv[i] for i in shard([v["wires"] * v["elems_per_wire"] for v in allv], n, rank,
                                                        world)]
            else:
                raise SystemExit(f"unknown workload {name}")
            self.count = len(self.variants)
            self.precision = precision or "mixed"
            self.warm = warm or ("learned_x0" if (name.startswith("stents") and os.path.exists(MODEL)) else "off")
        self.tol_res = {}  # per simulation index: its residual tolerance (stents)

    def stats(self, i):
        """(nodes, elements, RCM half bandwidth in nodes, SDF points, Krylov restart) of simulation i (cached)."""
        if not hasattr(self, "_stats"):
            self._stats = {}
        if i not in self._stats:
            from endobeams_gb300 import _lib
            c, p, it = self.build(i)
            _, w = _lib.rcm_order(len(c.nodes), c.beams.conn)
            m = getattr(it, "master", None) if it is not None else None
            pts = (m.dims[0] + 2) * (m.dims[1] + 2) * (m.dims[2] + 2) if m is not None and hasattr(m, "dims") else 0
            self._stats[i] = (len(c.nodes), len(c.beams), w, pts, p.krylov_restart)
        return self._stats[i]

    def build(self, i):
        s = self.scenes
        if self.kind == "nets":
            if self.sdf is None:
                self.sdf = s.sphere_sdf()
            c, p, it = s.net_on_sphere(int(self.sides[i]), seed=1 + i, sdf=self.sdf)
            p.tolerance_residual = 1e-5
            p.tolerance_displacement = 1e-8
            p.linear_tol = NEWTON_FORCING
            p.precision = self.precision
            return c, p, it
        v = self.variants[i]
        if v is None:
            c, p, it = s.braided_stent()
        elif isinstance(v, tuple):
            c, p, it = s.braided_stent(wires=v[1], elems_per_wire=v[2], grid=None)
        else:
            c, p, it = s.stent_variant(v)
        self.tol_res[i] = stent_tol_res(c)
        return c, stent_params(p, self.precision, self.warm), it

    @property
    def n_tol8(self):
        return sum(1 for t in self.tol_res.values() if t == STENT_TOL_RES)

    def describe(self, nodes, elements, groups):
        if self.kind == "nets":
            w = f"{self.name}: {self.count} nets (sides U{{20..40}}) on a 128^3 sphere SDF, dt=5e-5"
            tol = (1e-5, 1e-8)
        elif self.name == "stent":
            w = "stent: one braided stent (48 wires, R 4 mm, 45 deg, 200 elements/wire) in a 3.5 mm cylinder SDF, dt=1e-5"
            tol = (STENT_TOL_RES, STENT_TOL_DISP)
        else:
            w = (f"{self.name}: {self.count} braided stents (seed 2; wires {{16,24,32,48}}, R U[3,5] mm, pitch "
                 f"U[35,55] deg, U{{100..400}} elements/wire, own cylinder SDF at 0.1 mm), dt=1e-5")
            tol = (f"1e-8 (elements >= 0.12 mm: {self.n_tol8} sims), 1e-7 (shorter: {self.count - self.n_tol8})",
                   STENT_TOL_DISP)
        return {"workload": w, "sims": self.count, "nodes": int(nodes), "elements": int(elements),
                "resident_groups": groups, "tolerance_residual": tol[0], "tolerance_displacement": tol[1],
                "linear_tol": NEWTON_FORCING, "band_lu": SOLVER["band_lu"], "refactor": SOLVER["refactor"],
                "precision": self.precision, "warm_start": self.warm}


def est_bytes(stats):
    """Device bytes eb_create will hold for one simulation (layout of eb_internal.cuh):
    element staging, six FP64 BSR matrices plus the FP32 tangent, node state, DOF vectors,
    Krylov basis, FP32 band and its diagonal-block inverses, SDF coefficients."""
    n, ne, w, pts, m = stats
    b = 6 * w + 5
    blocks = n + 2 * ne
    band = 4 * (6 * n) * (2 * b + 1) if b <= 891 else 0
    per_dof = 14 * 8 + 1 + 16 + (2 * m + 1) * 8 + 8 + 4 + 256  # ... Krylov basis V and its preconditioned Z
    return 6300 * ne + 2200 * blocks + 1100 * n + per_dof * 6 * n + band + 8 * pts


def plan_groups(wl, budget):
    """Greedy resident groups in population order under a device-byte budget.

    Population order mixes costly and cheap stents in every group, so the costliest
    ones (one CTA each, largest first) overlap with the cheap ones.  Filling the groups
    in decreasing cost instead put the 552 costliest stents in one group, where they
    queue in 3.6 waves on the 152 SMs: 97.7 instead of 192.6 HHT steps/s."""
    groups, cur, acc = [], [], 0
    for i in range(wl.count):
        bts = est_bytes(wl.stats(i))
        if cur and acc + bts > budget:
            groups.append(cur)
            cur, acc = [], 0
        cur.append(i)
        acc += bts
    if cur:
        groups.append(cur)
    return groups


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
    """The batched time loop of run_simulation! (per-simulation Δt halving and rollback)."""

    def __init__(self, eng, params, elems=None):
        self.eng = eng
        self.p = params
        self.elems = np.asarray(elems if elems is not None else np.zeros(eng.n), np.int64)
        self.S = eng.n
        self.t = np.zeros(self.S)
        self.dt = np.full(self.S, params.initial_timestep)
        self.reset()

    def reset(self):
        self.ok_steps = 0
        self.newton = 0
        self.krylov = 0
        self.pred_krylov = 0
        self.batch_iters = 0
        self.ws_used = 0
        self.ws_steps = 0
        self.elem_evals = 0

    def step(self, e2e=False, ubuf=None):
        eng = self.eng
        if e2e:
            eng.set_loads_all(eng.loads_all(self.t + self.dt))
        k, _ = eng.step(self.dt)
        st = eng.stats()
        self.newton += sum(s["newton_iterations"] for s in st)
        self.batch_iters += max(s["newton_iterations"] for s in st)
        self.krylov += sum(s["krylov_iterations"] for s in st)
        self.pred_krylov += sum(s["predictor_krylov_iterations"] for s in st)
        # element evaluations of the corrector iterations (one k_beam pass per iteration of each sim)
        self.elem_evals += int(sum(int(e) * s["newton_iterations"] for e, s in zip(self.elems, st)))
        self.ws_used += sum(s["warm_start_used"] for s in st)
        self.ws_steps += len(st)
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


def _lib_phases():
    from endobeams_gb300 import _lib
    return list(_lib.PHASES)


def _in_lanes(fn, items):
    """fn(item) for every item, each on its own host thread (the library releases the
    interpreter during its calls, so the lanes' steps overlap on the GPU)."""
    import threading
    from endobeams_gb300 import _lib
    device = _lib.current_device()
    errors = []

    def run(it):
        try:
            _lib.set_device(device)
            fn(it)
        except BaseException as e:
            errors.append(e)

    threads = [threading.Thread(target=run, args=(it,)) for it in items]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    if errors:
        raise errors[0]


def run_group(eb, wl, idx, args, world, e2e=True, warm=None):
    """Creates one resident group, warms up W steps, times K steps; returns a dict of totals.

    The group runs as `--lanes` concurrent lanes (api.lane_split: round-robin in decreasing
    size), one engine each, stepped by its own host thread on its own stream.  Every timed
    step goes through the public API with host buffers: the step's loads are uploaded from
    host memory (eb_set_loads_all) and all displacements are read back
    (eb_get_displacements).  The same K steps give both figures: the device span between
    CUDA events (the earliest lane's start to the latest lane's stop: `ms`, the whole-job
    HHT steps/s) and the host wall clock around them (`e2e`)."""
    built = [wl.build(i) for i in idx]
    params = built[0][1]
    if warm is not None:
        params.warm_start = warm
    params.timing = True
    parts = eb.api.lane_split([len(b[0].beams) for b in built], args.lanes)
    lanes = []
    for part in parts:
        confs = [built[j][0] for j in part]
        inters = [built[j][2] for j in part]
        eng = eb.GpuSimulations(confs, params, inters)
        if wl.kind == "stents":
            eng.set_tolerances(residual=[wl.tol_res[idx[j]] for j in part])
        if params.warm_start in ("learned", "learned_x0"):
            from endobeams_gb300 import warm_start as W
            eng.set_warm_start(W.WarmStartModel.load(MODEL))
        nodes = sum(len(c.nodes) for c in confs)
        lanes.append({"eng": eng, "drv": Driver(eng, params, [len(c.beams) for c in confs]),
                      "ubuf": np.zeros((nodes, 3)), "nodes": nodes, "elements": sum(len(c.beams) for c in confs),
                      "loaded": sum(len(c.loads.concentrated_force.loaded_dofs) for c in confs if c.loads is not None)})
    use_e2e = e2e and not args.no_e2e

    def steps(n):
        def go(ln):
            for _ in range(n):
                ln["drv"].step(e2e=use_e2e, ubuf=ln["ubuf"])
        _in_lanes(go, lanes)

    steps(args.warmup)
    launch_shapes = [ln["eng"].autotune() for ln in lanes][0]
    for ln in lanes:
        ln["eng"].phase_times(reset=True)
        ln["drv"].reset()
    barrier(world)
    for ln in lanes:
        ln["eng"].timer_start()
    t0 = time.perf_counter()
    steps(args.steps)
    wall = time.perf_counter() - t0
    for ln in lanes:
        ln["eng"].timer_stop()
    span = max(a["eng"].timer_between(b["eng"]) for a in lanes for b in lanes)
    ms = allreduce_max(span, world)
    wall = allreduce_max(wall, world)
    # per phase: the time during which any lane ran it (union of the lanes' intervals on one
    # time axis); the summed lane times below exceed the span when the lanes overlap
    ref = lanes[0]["eng"]
    phase_union = {k: eb.api.union_ms([ln["eng"].phase_intervals(k, ref) for ln in lanes]) for k in _lib_phases()}
    phase_ms, launches = None, None
    for ln in lanes:  # each lane's phase intervals on its own stream (the lanes overlap)
        pm, la = ln["eng"].phase_times(reset=True)
        phase_ms = dict(pm) if phase_ms is None else {k: phase_ms[k] + pm[k] for k in pm}
        launches = dict(la) if launches is None else {k: launches[k] + la[k] for k in la}
    D = [ln["drv"] for ln in lanes]
    tot = lambda f: sum(getattr(d, f) for d in D)
    mem = sum(ln["eng"].memory()[0] for ln in lanes)
    band_sims = sum(ln["eng"].memory()[1] for ln in lanes)
    out = {"sim_steps": tot("ok_steps"), "ms": ms, "newton": tot("newton"), "krylov": tot("krylov"),
           "pred_krylov": tot("pred_krylov"), "ws_used": tot("ws_used"), "ws_steps": tot("ws_steps"),
           "phase_ms": phase_ms, "launches": launches, "elem_evals": tot("elem_evals"),
           "nodes": sum(ln["nodes"] for ln in lanes), "elements": sum(ln["elements"] for ln in lanes),
           "sims": len(idx), "device_bytes": mem, "band_sims": band_sims, "e2e": None,
           "launch_shapes": launch_shapes, "lanes": len(lanes), "phase_union_ms": phase_union}
    if use_e2e:
        h2d = d2h = 0
        for ln in lanes:
            S = ln["drv"].S
            bi = ln["drv"].batch_iters / max(args.steps, 1)
            # loads, per-sim step constants (cK, cC, cM, dt), active masks (step + each iteration), commit mask
            h2d += 8 * ln["loaded"] + 32 * S + 4 * S + 4 * S * bi + 4 * S
            # displacements, per-iteration Newton norms, per-step solver statistics
            d2h += 24 * ln["nodes"] + 40 * S * bi + 20 * S
        out["e2e"] = {"sim_steps": out["sim_steps"], "wall_s": wall, "h2d": h2d, "d2h": d2h, "device_ms": ms,
                      "newton": out["newton"], "krylov": out["krylov"]}
    for ln in lanes:
        ln["eng"].close()
    return out


def output_leg(eb, wl, args):
    """Steps/s of the first `--output-sims` simulations with VTK output every `--output-every`
    steps (asynchronous writer, files on disk) against the same steps without output."""
    import shutil
    import tempfile
    idx = list(range(min(args.output_sims, wl.count)))
    built = [wl.build(i) for i in idx]
    confs, inters, params = [b[0] for b in built], [b[2] for b in built], built[0][1]
    params.warm_start = "off"
    res = {}
    root = args.output_dir or tempfile.mkdtemp(prefix="eb_vtk_")
    n_steps = max(args.steps, args.output_every)
    for with_out in (False, True):
        eng = eb.GpuSimulations(confs, params, inters)
        drv = Driver(eng, params, [len(c.beams) for c in confs])
        for _ in range(args.warmup):
            drv.step()
        drv.reset()
        if with_out:
            dirs = eb.api.output_dirs(root, len(idx))
            eng.vtk_open(dirs)
        writes, t_call = 0, 0.0
        t0 = time.perf_counter()
        for k in range(n_steps):
            drv.step()
            if with_out and (k + 1) % args.output_every == 0:
                c0 = time.perf_counter()
                eng.vtk_write(writes, k + 1, drv.t)
                t_call += time.perf_counter() - c0
                writes += 1
        if with_out:
            eng.vtk_flush()
        wall = time.perf_counter() - t0
        if with_out:
            eng.vtk_close()
        eng.close()
        res["with" if with_out else "without"] = {"steps_per_s": drv.ok_steps / wall, "wall_s": wall}
        if with_out:
            nbytes = sum(os.path.getsize(os.path.join(dp, f)) for dp, _, fs in os.walk(root) for f in fs)
            res["with"].update(writes=writes, files_bytes=nbytes, mean_vtk_write_call_ms=1e3 * t_call / max(writes, 1))
    if args.output_dir is None:
        shutil.rmtree(root, ignore_errors=True)
    res["every"] = args.output_every
    res["sims"] = len(idx)
    res["steps"] = n_steps
    res["overhead_frac"] = 1 - res["with"]["steps_per_s"] / res["without"]["steps_per_s"]
    return res


def gmres_bytes_per_iter(wl, idx):
    """Algorithmic bytes one GMRES iteration reads per simulation (FP32 band L and U, the
    32x32 diagonal-block inverses, the FP32 tangent and its block index), summed over idx."""
    tot = 0
    for i in idx:
        n, ne, w, _, _ = wl.stats(i)
        b = 6 * w + 5
        N = 6 * n
        tot += 4 * N * (2 * b + 1) + 2 * 4 * 32 * N + (n + 2 * ne) * (36 * 4 + 4)
    return tot


def gpu_arm(args, rank, world):
    eb = _pkg()
    from endobeams_gb300 import _lib
    wl = Workload(args.workload, args.precision, args.warm_start, args.count, rank=rank, world=world)
    n_gpu, gname = eb.device_info()
    if n_gpu < 1:
        raise SystemExit("no CUDA device")
    free, total = _lib.device_memory()
    groups = plan_groups(wl, int(args.mem_frac * free)) if wl.kind == "stents" else [list(range(wl.count))]
    clocks = ClockSampler()
    clocks.start()
    tot = None
    for g_idx in groups:
        r = run_group(eb, wl, g_idx, args, world)
        if tot is None:
            tot = r
            tot["e2e"] = dict(r["e2e"]) if r["e2e"] else None
            tot["phase_ms"] = dict(r["phase_ms"])
            tot["phase_union_ms"] = dict(r["phase_union_ms"])
            tot["launches"] = dict(r["launches"])
            tot["device_bytes_max"] = r["device_bytes"]
        else:
            for k in ("sim_steps", "ms", "newton", "krylov", "pred_krylov", "ws_used", "ws_steps", "nodes", "elements",
                      "sims", "band_sims", "elem_evals"):
                tot[k] += r[k]
            tot["device_bytes_max"] = max(tot["device_bytes_max"], r["device_bytes"])
            for k in tot["phase_ms"]:
                tot["phase_ms"][k] += r["phase_ms"][k]
                tot["phase_union_ms"][k] += r["phase_union_ms"][k]
                tot["launches"][k] += r["launches"][k]
            if tot["e2e"] and r["e2e"]:
                for k in ("sim_steps", "wall_s", "h2d", "d2h", "device_ms", "newton", "krylov"):
                    tot["e2e"][k] += r["e2e"][k]
    clk = clocks.stop()
    value = world * tot["sim_steps"] / (tot["ms"] / 1e3)
    steps = args.steps
    e2e = None
    if tot["e2e"]:
        e = tot["e2e"]
        e2e = {"value": world * e["sim_steps"] / e["wall_s"], "unit": "HHT steps/s",
               "h2d_bytes_per_step": int(e["h2d"] / max(steps, 1)), "d2h_bytes_per_step": int(e["d2h"] / max(steps, 1)),
               "wall_s": e["wall_s"], "device_s": e["device_ms"] / 1e3,
               "note": "the timed steps themselves: loads uploaded from host memory and all displacements "
                       "read back every step, host wall clock"}
    phase_ms, launches = tot["phase_ms"], tot["launches"]
    dom = max(phase_ms, key=lambda k: phase_ms[k])
    # The phase times are each lane's intervals on its own stream; the lanes overlap, so the
    # rooflines take each phase's union over the lanes (the time during which any lane ran it):
    # the work of all lanes over that time is the rate the GPU sustained on the phase.
    dev_ms = {k: max(v, 1e-9) for k, v in tot["phase_union_ms"].items()}
    # ---- rooflines: the element kernel (FP64 pipe) and the Krylov kernel (HBM)
    peak_fp64 = eb.fp64_peak_tflops()
    rooflines = {}
    if launches["beam"] and tot["elem_evals"]:
        # FP64 flops of every element evaluation of the timed corrector iterations over the phase's device time
        avg_beam_ms = phase_ms["beam"] / launches["beam"]
        ach = F_ELEM_FP64 * tot["elem_evals"] / (dev_ms["beam"] * 1e-3) / 1e12
        ach_alg = F_ELEM_ALGORITHMIC * tot["elem_evals"] / (dev_ms["beam"] * 1e-3) / 1e12
        rooflines["beam"] = {"kernel": "k_beam (corotational element, FP64)", "bound": "fp64", "achieved": ach,
                             "algorithmic_flops_per_element": F_ELEM_ALGORITHMIC,
                             "achieved_algorithmic": ach_alg,
                             "executed_flops_per_element": F_ELEM_FP64,
                             "peak": peak_fp64, "peak_source": "measured (eb_fp64_peak FMA probe on this GPU)",
                             "unit": "TFLOP/s", "frac": ach / peak_fp64, "traffic": None,
                             "avg_launch_ms": avg_beam_ms, "share_of_step": phase_ms["beam"] / sum(phase_ms.values())}
    peaks = _measured_peaks()
    if launches["contact"] and tot["elem_evals"] and wl.kind == "stents":
        # every stent element is a contact element: one contact evaluation per element evaluation
        ach = B_CONTACT_ELEM * tot["elem_evals"] / (dev_ms["contact"] * 1e-3) / 1e9
        hbm = peaks.get("hbm_gbs")
        rooflines["contact"] = {"kernel": "k_contact (beam-to-SDF contact element, FP64)", "bound": "hbm",
                                "achieved": ach, "peak": hbm,
                                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if hbm else None, "unit": "GB/s",
                                "frac": (ach / hbm) if hbm else None, "traffic": None,
                                "algorithmic_bytes_per_element": B_CONTACT_ELEM,
                                "note": "reads only; in-contact elements also write 2.4 KB each. The kernel is bound "
                                        "by the FP64 pipe (75% active under ncu on 16 stents), not by HBM",
                                "share_of_step": phase_ms["contact"] / sum(phase_ms.values())}
    if launches["krylov"] and wl.kind == "stents":
        per_iter = gmres_bytes_per_iter(wl, range(wl.count))
        iters_per_sim = tot["krylov"] / max(tot["sims"], 1)  # summed over the timed steps
        bytes_total = per_iter * iters_per_sim
        ach = bytes_total / (dev_ms["krylov"] * 1e-3) / 1e9
        hbm = peaks.get("hbm_gbs")
        per_launch = bytes_total / max(launches["krylov"], 1)
        rooflines["krylov"] = {"kernel": "k_gmres (per-simulation restarted GMRES, band-LU preconditioned)",
                               "bound": "hbm", "achieved": ach, "peak": hbm,
                               "peak_source": "MEASURED_PEAKS.json hbm_gbs" if hbm else None, "unit": "GB/s",
                               "frac": (ach / hbm) if hbm else None,
                               "traffic": KRYLOV_TRAFFIC_RATIO * per_launch,
                               "traffic_note": "bytes per launch: the algorithmic bytes per launch x the DRAM/"
                                               "algorithmic ratio ncu measured on 16 stents (1.04)",
                               "algorithmic_bytes_per_launch": per_launch,
                               "avg_launch_ms": phase_ms["krylov"] / max(launches["krylov"], 1),
                               "time_basis": "union over the lanes of their Krylov intervals (lanes overlap: "
                                             "each lane's launches run beside the others'); avg_launch_ms is one "
                                             "lane's launch on its own stream",
                               "phase_union_ms": dev_ms["krylov"],
                               "algorithmic_bytes_per_iteration": per_iter / max(wl.count, 1),
                               "share_of_step": phase_ms["krylov"] / sum(phase_ms.values())}
    roof = rooflines.get("krylov") if dom in ("krylov", "precond") and "krylov" in rooflines else rooflines.get("beam")
    out = {
        "metric": METRIC if wl.kind == "stents" else "HHT steps/s (whole job), batched plain Newton",
        "value": value, "unit": "HHT steps/s", "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": tot["ms"] / max(steps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if wl.precision == "fp64" else "f64+f32-krylov", "data": "synthetic",
        "config": dict(wl.describe(tot["nodes"], tot["elements"], len(groups)),
                       l2="state, band and staging arrays exceed L2 (129 MB) each step", device=gname,
                       device_bytes_per_group_max=int(tot["device_bytes_max"]), band_preconditioned_sims=tot["band_sims"],
                       launch_shapes_first_group=tot["launch_shapes"], lanes_per_group=tot["lanes"]),
        "newton_iters_per_step": tot["newton"] / max(tot["sim_steps"], 1),
        "krylov_iters_per_newton": tot["krylov"] / max(tot["newton"], 1),
        "predictor_krylov_iters_per_step": tot["pred_krylov"] / max(tot["sim_steps"], 1),
        "phase_ms": {k: round(v, 3) for k, v in phase_ms.items()},
        "phase_ms_basis": "summed over the lanes' own streams (the lanes overlap, so the sum exceeds the span)",
        "phase_union_ms": {k: round(v, 3) for k, v in tot["phase_union_ms"].items()},
        "dominant_phase": dom,
        "gpu_launches": int(sum(launches.values())),
        "roofline": roof, "rooflines": rooflines, "e2e": e2e, "clocks": clk,
    }
    if wl.warm in ("learned", "learned_x0"):
        out["warm_start"] = {"model": os.path.relpath(MODEL, ROOT), "mode": wl.warm,
                             "learned_start_accepted_frac": tot["ws_used"] / max(tot["ws_steps"], 1)}
    # ---- comparison legs: the same groups with the plain predictor, and the plain single stent
    if wl.kind == "stents" and wl.count > 1 and not args.no_compare:
        if wl.warm in ("learned", "learned_x0"):
            pl = {"sim_steps": 0, "ms": 0.0, "newton": 0, "krylov": 0, "pred_krylov": 0}
            for g_idx in groups:
                r = run_group(eb, wl, g_idx, args, world, e2e=False, warm="off")
                for k in pl:
                    pl[k] += r[k]
            pv = world * pl["sim_steps"] / (pl["ms"] / 1e3)
            out["batched_plain"] = {"value": pv, "sims": wl.count,
                                    "newton_iters_per_step": pl["newton"] / max(pl["sim_steps"], 1),
                                    "krylov_iters_per_newton": pl["krylov"] / max(pl["newton"], 1),
                                    "predictor_krylov_iters_per_step": pl["pred_krylov"] / max(pl["sim_steps"], 1),
                                    "note": "the same resident groups and step window, HHT predictor without the "
                                            "network"}
            out["learned_vs_plain"] = value / pv
        single = Workload("stent", wl.precision, "off")
        r = run_group(eb, single, [0], args, world, e2e=False)
        sv = world * r["sim_steps"] / (r["ms"] / 1e3)
        out["plain_single_sim"] = {"value": sv, "unit": "HHT steps/s",
                                   "newton_iters_per_step": r["newton"] / max(r["sim_steps"], 1),
                                   "workload": single.describe(r["nodes"], r["elements"], 1)["workload"]}
        out["speedup_vs_plain_single_sim"] = value / sv
    if args.output_every > 0:
        out["vtk_output"] = output_leg(eb, wl, args)
    return out, wl


def _measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
    except Exception:
        return {}
    out = {}
    for k, v in d.items():
        if isinstance(v, (int, float)):
            out[k] = float(v)
    return out


# ------------------------------------------------------------------ CPU arms (oracle restatement)

def cpu_rate(workload, precision, idx, steps, cores, warmup=0):
    """Oracle HHT steps/s on the simulations `idx` of the workload with `cores` spawned processes:
    each simulation takes `warmup` untimed steps, then `steps` timed ones (the GPU arm's step
    window).  Model construction (pattern, SDF prefilter) and the warm-up happen outside the
    clock; the rate is all timed steps over the busiest process's timed seconds."""
    idx = list(idx)
    chunks = [idx[i::cores] for i in range(cores) if idx[i::cores]]
    if len(chunks) == 1:
        res = [_timed_chunk((workload, precision, chunks[0], steps, warmup))]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(len(chunks)) as pool:
            res = pool.map(_timed_chunk, [(workload, precision, c, steps, warmup) for c in chunks])
    done = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    return done / wall, wall


def spread(count, sample):
    """`sample` simulation indices spread evenly over a population of `count`."""
    sample = min(sample, count)
    return sorted(set(int(round(x)) for x in np.linspace(0, count - 1, sample)))


def _timed_chunk(payload):
    workload, precision, idx, steps, warmup = payload
    import __graft_entry__ as g
    O = g.load_oracle()
    import bridge
    wl = Workload(workload, precision, "off")
    models = []
    for i in idx:
        c, p, it = wl.build(i % wl.count)
        if wl.kind == "stents":
            p.tolerance_residual = wl.tol_res[i % wl.count]
        models.append(O.OracleModel(bridge.scene_from_conf(c, it), bridge.params_from(p)))
    done, busy = 0, 0.0
    for m in models:
        state = O.run_simulation(m, max_steps=warmup) if warmup else None
        t0 = time.perf_counter()
        r = O.run_simulation(m, max_steps=steps, resume=state)
        busy += time.perf_counter() - t0
        done += r["steps"] - (state["steps"] if state else 0)
    return done, busy


# ------------------------------------------------------------------ distributed helpers

DEVICE = None  # CUDA ordinal this process uses (None: no GPU visible)


def device_for_rank(local_rank, n_visible):
    """The GPU a rank binds: its local rank among the devices it sees.  A launcher that gives each
    rank one device (CUDA_VISIBLE_DEVICES per rank) leaves one visible device: ordinal 0."""
    if n_visible < 1:
        return None
    return local_rank % n_visible


def dist_init(bind=True):
    """Reads RANK / WORLD_SIZE / LOCAL_RANK, binds this rank's GPU through the library
    (eb_set_device) whatever CUDA_VISIBLE_DEVICES holds (bind=False: the CPU-only reference
    arm touches no GPU), and joins the gloo group for the timing barrier and max (N > 1)."""
    global DEVICE
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    if bind:
        eb = _pkg()
        from endobeams_gb300 import _lib
        n_visible, _ = eb.device_info()
        DEVICE = device_for_rank(local, n_visible)
        if DEVICE is not None:
            _lib.check(_lib.load().eb_set_device(DEVICE), "eb_set_device")
    if world > 1:
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
    SOLVER.update(band_lu=args.band_lu, refactor=args.refactor, refactor_cost=args.refactor_cost)
    rank, world = dist_init(bind=args.impl != "reference")
    if args.impl == "reference":
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        wl = Workload(args.workload, args.precision, "off", args.count)
        idx = spread(wl.count, args.ref_sample)
        rate, wall = cpu_rate(args.workload, wl.precision, idx, args.steps, cores, warmup=args.warmup)
        sample = (f"{len(idx)} of {wl.count} sims spread over the population, {args.warmup} untimed + "
                  f"{args.steps} timed steps each (the GPU arm's window), C++ oracle + SciPy SuperLU, "
                  f"{cores} processes, {wall:.1f} s timed")
        line = {"metric": METRIC if wl.kind == "stents" else "HHT steps/s (whole job), batched plain Newton",
                "impl": "reference", "value": rate, "unit": "HHT steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": wl.describe(0, 0, 0)["workload"], "sims": wl.count, "sample": len(idx)},
                "cpu_baseline": {"value": rate, "unit": "HHT steps/s", "cores": cores, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": rate, "unit": "HHT steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    out, wl = gpu_arm(args, rank, world)
    if rank == 0:
        if not args.no_cpu:
            rate, wall = cpu_rate(args.workload, wl.precision, range(args.cpu_sample), args.cpu_steps, 1)
            out["cpu_baseline"] = {"value": rate, "unit": "HHT steps/s", "cores": 1, "kind": "port",
                                   "sample": f"{args.cpu_sample} of {wl.count} sims x {args.cpu_steps} steps, "
                                             f"C++ oracle + SciPy SuperLU, 1 core, {wall:.1f} s"}
        print(json.dumps(out))


if __name__ == "__main__":
    main()
