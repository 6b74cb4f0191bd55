"""Host-side logic that needs no GPU: API semantics, scene generators, and the
batched time loop's Δt policy against the oracle's restatement of
run_simulation.jl:38-112 on scripted Newton outcomes."""
import numpy as np
import pytest

import oracle as O


def test_boundary_conditions_semantics(eb):
    bc = eb.BoundaryConditions(eb.Encastre(range(2, 7)), eb.ImposedDisplacement(1, lambda t: 2 * t), 126)
    assert list(bc.fixed_dofs) == [0, 1, 2, 3, 4, 5]          # sorted union, 0-based
    assert list(bc.displaced_indices) == [0]
    assert len(bc.free_dofs) == 120
    bc2 = eb.BoundaryConditions(12)
    assert len(bc2.fixed_dofs) == 0 and len(bc2.free_dofs) == 12


def test_beams_use_one_based_connectivity(eb):
    X = np.zeros((3, 3))
    X[:, 0] = [0, 1, 2]
    nodes = eb.NodesBeams(X)
    beams = eb.Beams(nodes, [(1, 2), (2, 3)], 1.0, 0.3, 1.0, 0.1, 0.0)
    assert beams.conn.tolist() == [[0, 1], [1, 2]]
    assert np.allclose(nodes.R, np.eye(3).flatten("F"))


def test_scene_sizes(scenes):
    conf, _, _ = scenes.cantilever()
    assert len(conf.nodes) == 21 and len(conf.beams) == 20
    conf, _, inter = scenes.ring_drop()
    assert len(conf.nodes) == 64 and len(conf.beams) == 64 and inter.master.dims == (64, 64, 64)
    for side in (20, 40):
        conf, _, _ = scenes.net_on_sphere(side, sdf=scenes.sphere_sdf(n=8, h=1e-3))
        assert len(conf.beams) == 2 * side * (side - 1)
    conf, _, inter = scenes.braided_stent()
    assert len(conf.beams) == 9600 and len(conf.nodes) == 8664  # 9648 nodes before merging 984 crossings
    assert inter.master.dims == (96, 96, 256)
    sides = scenes.net_sides(256, seed=0)
    assert sides.min() >= 20 and sides.max() <= 40


def test_stent_crossings_coincide(scenes):
    conf, _, _ = scenes.braided_stent(wires=16, elems_per_wire=40)
    X = conf.nodes.X0
    # every node is used, and merged crossing nodes have four incident elements
    deg = np.bincount(conf.beams.conn.ravel(), minlength=len(X))
    assert deg.min() >= 1 and set(np.unique(deg)) <= {1, 2, 3, 4}
    assert (deg == 4).sum() > 0


class _ScriptedEngine:
    """Stands in for GpuSimulations: returns scripted k per step and records the calls."""

    def __init__(self, scripts):
        self.scripts = [list(s) for s in scripts]
        self.n = len(scripts)
        self.calls = []

    def set_time(self, s, t):
        self.calls.append(("t", s, round(t, 12)))

    def step(self, dt, active):
        k = np.array([self.scripts[s].pop(0) if active[s] else 0 for s in range(self.n)], np.int32)
        self.calls.append(("dt", tuple(np.round(dt, 15)), tuple(active)))
        return k, np.zeros(self.n, np.int32)

    def stats(self):
        return [dict(newton_iterations=1, krylov_iterations=1)] * self.n

    def commit(self, mask):
        self.calls.append(("commit", tuple(mask)))

    def rollback(self, mask):
        self.calls.append(("rollback", tuple(mask)))

    def sync_nodes(self):
        pass

    def autotune(self):
        return {}

    def vtk_open(self, dirs, points_per_beam=10):
        self.calls.append(("vtk_open", tuple(dirs)))

    def vtk_write(self, counter, step, t, mask=None):
        m = np.ones(self.n, bool) if mask is None else np.asarray(mask, bool)
        c, st, tt = (np.broadcast_to(x, (self.n,)) for x in (counter, step, t))
        self.calls.append(("vtk", tuple((s, int(c[s]), int(st[s]), round(float(tt[s]), 12))
                                        for s in range(self.n) if m[s])))

    def vtk_close(self):
        self.calls.append(("vtk_close",))


class _ScriptedModel:
    """Stands in for the oracle's OracleModel in oracle.run_simulation."""

    def __init__(self, script, params):
        self.script = list(script)
        self.log = []
        self.p = params

    def step(self, t1, dt):
        self.log.append((round(t1, 12), dt))
        return self.script.pop(0)

    def update_converged(self):
        self.log.append("commit")

    def update_not_converged(self):
        self.log.append("rollback")


@pytest.mark.parametrize("script", [
    [3] * 12,                                   # steady: Δt grows ×1.5 after 4 successes (capped)
    [3, 3, 21, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3],   # a failure halves Δt and rolls back
    [9, 9, 9, 9, 9, 3, 3, 3, 3, 3, 3, 3],       # k > 8 blocks growth
])
def test_time_loop_policy_matches_reference(eb, script):
    p = eb.SimulationParams(alpha=-0.05, beta=0.28, gamma=0.55, initial_timestep=0.01, min_timestep=1e-4,
                            max_timestep=0.02, simulation_end_time=0.1, max_iterations=20)
    eng = _ScriptedEngine([script + [3] * 50, script + [3] * 50])
    res = eb.run_simulations([None, None], p, engine=eng)
    op = O.Params(alpha=-0.05, beta=0.28, gamma=0.55, initial_timestep=0.01, min_timestep=1e-4, max_timestep=0.02,
                  simulation_end_time=0.1, max_iterations=20)
    om = _ScriptedModel(script + [3] * 50, op)
    ores = O.run_simulation(om)
    # same number of committed steps, same k sequence and same final time for every simulation
    for s in range(2):
        assert res.steps[s] == ores["steps"]
        assert res.ks[s] == ores["ks"]
        assert abs(res.t[s] - ores["t"]) < 1e-12
    # same Δt sequence
    dts = [c[1][0] for c in eng.calls if c[0] == "dt"]
    assert np.allclose(dts, [d for (_, d) in [x for x in om.log if isinstance(x, tuple)]])


def _reference_writes(script, p):
    """The output schedule of run_simulation! (run_simulation.jl:30-32, 86-90), restated:
    (write_counter, step, tⁿ) of every write_VTK call."""
    import math
    t, dt, succ, step, write_t = 0.0, p.initial_timestep, 0, 1, 0.0
    ks = list(script)
    out = [(0, 1, 0.0)]
    counter = 1
    while p.simulation_end_time - t > 1.0e-10:
        t1 = t + dt
        k = ks.pop(0)
        if k > p.max_iterations:
            dt /= 2
            succ = 0
            continue
        succ += 1
        if succ >= p.accelerate_after_success_it and k <= 8:
            dt = min(dt * 1.5, p.max_timestep)
            succ = 0
        due = write_t + p.output_timestep
        if t1 > due or math.isclose(t1, due, rel_tol=math.sqrt(np.finfo(float).eps), abs_tol=0.0):
            out.append((counter, step, round(t, 12)))
            counter += 1
            write_t = t1
        t = t1
        step += 1
    return out


@pytest.mark.parametrize("every", [0.005, 0.02, 0.031])
def test_vtk_output_schedule_matches_reference(eb, every, tmp_path):
    """run_simulations with output_dir: the writes (counter, step, start time of the step)
    per simulation are the reference's, including after rejected steps and Δt changes."""
    script = [3, 3, 21, 3, 3, 3, 3, 3, 21, 21, 3, 3, 3, 3, 3, 3]
    p = eb.SimulationParams(alpha=-0.05, beta=0.28, gamma=0.55, initial_timestep=0.01, min_timestep=1e-4,
                            max_timestep=0.02, simulation_end_time=0.1, max_iterations=20,
                            output_dir=str(tmp_path), output_timestep=every)
    eng = _ScriptedEngine([script + [3] * 50, [3] * 80])
    eb.run_simulations([None, None], p, engine=eng)
    assert eng.calls[0] == ("vtk_open", (str(tmp_path / "sim_00000"), str(tmp_path / "sim_00001")))
    assert eng.calls[-1] == ("vtk_close",)
    got = {0: [], 1: []}
    for c in eng.calls:
        if c[0] == "vtk":
            for sim, counter, step, t in c[1]:
                got[sim].append((counter, step, t))
    assert got[0] == _reference_writes(script + [3] * 50, p)
    assert got[1] == _reference_writes([3] * 80, p)


def test_plane_axis_and_output_dirs(eb, tmp_path):
    assert eb.PlaneSurface(0.0, "x").axis_index == 0 and eb.PlaneSurface(1.0, "Z").axis_index == 2
    assert eb.PlaneSurface(0.0, 1).axis_index == 1
    with pytest.raises(ValueError):
        eb.PlaneSurface(0.0, "w").axis_index
    from endobeams_gb300 import api
    assert api.output_dirs(str(tmp_path), 1) == [str(tmp_path)]
    assert api.output_dirs(str(tmp_path), 3)[2] == str(tmp_path / "sim_00002")


def test_triangulated_surface_grid_covers_the_mesh(eb):
    V = np.array([[0, 0, 0], [2, 0, 0], [0, 1, 0], [0, 0, 0.5]], float)
    T = np.array([[1, 2, 3], [1, 2, 4], [1, 3, 4], [2, 3, 4]])
    ts = eb.TriangulatedSurface(V, T, spacing=0.1, margin=2)
    o, h, dims = ts.grid()
    assert h == 0.1 and np.allclose(o, [-0.2, -0.2, -0.2])
    hi = o + (dims - 1) * h
    assert np.all(hi >= V.max(0) + 2 * h - 1e-12)
    ts2 = eb.TriangulatedSurface(V, T)  # default spacing: 1/64 of the largest extent
    assert ts2.grid()[1] == pytest.approx(2.0 / 64)


def test_one_simulation_aborts_alone(eb):
    """A simulation whose Δt falls below min_timestep leaves the batch on its own (the reference
    aborts its one simulation, run_simulation.jl:61-66): it is rolled back at every failure and
    never committed again, while the other simulation takes exactly the steps it takes alone."""
    p = eb.SimulationParams(alpha=-0.05, beta=0.28, gamma=0.55, initial_timestep=0.01, min_timestep=1e-3,
                            max_timestep=0.02, simulation_end_time=0.1, max_iterations=20)
    good = [3] * 80
    bad = [3, 3] + [21] * 80                     # converges twice, then never again
    alone = _ScriptedEngine([list(good)])
    ra = eb.run_simulations([None], p, engine=alone)
    eng = _ScriptedEngine([list(bad), list(good)])
    res = eb.run_simulations([None, None], p, engine=eng)
    assert res.aborted == [True, False]
    assert res.steps[0] == 2 and res.ks[0] == [3, 3]
    assert res.steps[1] == ra.steps[0] and res.ks[1] == ra.ks[0] and res.t[1] == ra.t[0]
    # Δt of the aborting simulation: 0.01 halved until below 1e-3 (four failures), then inactive
    dts0 = [c[1][0] for c in eng.calls if c[0] == "dt" and c[2][0]]
    assert dts0 == [0.01, 0.01, 0.01, 0.005, 0.0025, 0.00125]
    rb = [c[1][0] for c in eng.calls if c[0] == "rollback"]
    assert sum(rb) == 4
    commits0 = [c[1][0] for c in eng.calls if c[0] == "commit"]
    assert sum(commits0) == 2


def test_single_simulation_abort_raises(eb):
    """run_simulation (one configuration) raises like the reference's error("Simulation aborted.")."""
    from endobeams_gb300 import api
    p = eb.SimulationParams(alpha=-0.05, beta=0.28, gamma=0.55, initial_timestep=0.01, min_timestep=1e-3,
                            max_timestep=0.02, simulation_end_time=0.1, max_iterations=20)
    res = api.run_simulations([None], p, engine=_ScriptedEngine([[21] * 20]))
    assert res.aborted == [True] and res.steps == [0]


def test_lane_split_deals_by_size(eb):
    """Lanes get the simulations round-robin in decreasing size (ties by index): every
    simulation once, lane sizes within one of each other, and no more lanes than sims."""
    sizes = [5, 40, 12, 40, 7, 3, 25]
    parts = eb.api.lane_split(sizes, 3)
    assert parts == [[1, 2, 5], [3, 4], [6, 0]]
    assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
    assert eb.api.lane_split(sizes, 1) == [[1, 3, 6, 2, 4, 0, 5]]
    assert len(eb.api.lane_split([1, 2], 8)) == 2


def test_union_of_phase_intervals(eb):
    u = eb.api.union_ms
    assert u([]) == 0.0
    assert u([np.array([[0.0, 2.0], [1.0, 3.0]]), np.array([[5.0, 6.0]])]) == 4.0
    assert u([np.array([[0.0, 10.0]]), np.array([[1.0, 2.0], [3.0, 4.0]])]) == 10.0
    assert u([np.array([[4.0, 5.0], [0.0, 1.0]])]) == 2.0


class _ScriptedConf:
    """A configuration stand-in for the lane tests: its element count and its k script."""

    def __init__(self, n_elements, script):
        self.beams = [None] * n_elements
        self.script = list(script)


def test_lanes_run_each_simulation_like_one_batch(eb, monkeypatch, tmp_path):
    """run_simulations(lanes=3) on scripted engines: each lane gets its own engine and
    thread, and every simulation takes the steps, k sequence and final time it takes in one
    batch, with its output in its own sim_<index> directory."""
    import threading
    engines = []

    def make(confs, params, inters):
        e = _ScriptedEngine([c.script for c in confs])
        e.thread = threading.current_thread().name
        engines.append(e)
        return e

    monkeypatch.setattr(eb.api, "GpuSimulations", make)
    monkeypatch.setattr(eb.api._lib, "current_device", lambda: 0)
    monkeypatch.setattr(eb.api._lib, "set_device", lambda d: None)
    scripts = [[3] * 40, [3, 21, 3] + [3] * 40, [9] * 5 + [3] * 40, [21, 21] + [3] * 40, [4] * 40]
    sizes = [100, 400, 250, 50, 300]
    p = eb.SimulationParams(alpha=-0.05, beta=0.28, gamma=0.55, initial_timestep=0.01, min_timestep=1e-4,
                            max_timestep=0.02, simulation_end_time=0.1, max_iterations=20)
    one = eb.run_simulations([_ScriptedConf(n, s) for n, s in zip(sizes, scripts)], p)
    p.output_dir = str(tmp_path)
    engines.clear()
    three = eb.run_simulations([_ScriptedConf(n, s) for n, s in zip(sizes, scripts)], p, lanes=3)
    assert len(engines) == 3 and len({e.thread for e in engines}) == 3
    assert three.steps == one.steps and three.ks == one.ks and three.aborted == one.aborted
    assert np.allclose(three.t, one.t, rtol=0, atol=1e-12)
    # the lanes hold the simulations lane_split deals them and open those simulations' directories
    parts = eb.api.lane_split(sizes, 3)
    assert sorted(e.n for e in engines) == sorted(len(q) for q in parts)
    for e in engines:
        dirs = next(c[1] for c in e.calls if c[0] == "vtk_open")
        lane = [int(d[-5:]) for d in dirs]
        assert lane in parts
    opened = sorted(d for e in engines for c in e.calls if c[0] == "vtk_open" for d in c[1])
    assert opened == sorted(str(tmp_path / f"sim_{s:05d}") for s in range(5))
