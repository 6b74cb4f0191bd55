"""GPU against the oracle on the benchmark configurations and on the reference's own
contact scenes, each with the solver settings the benchmark uses for it.

* configuration 0 (cantilever) over its whole run, 2,000 steps;
* configuration 1 (ring drop onto the plane SDF) over 300 steps (first contact at ~200);
* configuration 2: four nets of the 256-net population (sides U{20..40}, seed 0) on the
  128³ sphere SDF, batched, 50 steps;
* configuration 3: the 48-wire, 200-elements-per-wire braided stent in its cylinder
  SDF, mixed precision, 5 steps at residual tolerance 1e-8;
* the net of test/test_beams2rigid_contact_1_analytical.jl (from its input files,
  frozen in tests/golden/reference_net.npz) on the analytic sphere, 80 steps, through
  first contact;
* the beam of test/test_beams2rigid_contact_2_analytical.jl, node 1 driven by the
  imposed triangular wave against the analytic sphere, its whole run (t = 2.5 s).

The oracle solves every Newton system exactly (sparse LU); the GPU runs GMRES to the
benchmark's relative tolerance.  The bar is the one of the configurations: the same
committed steps, the final positions within 1e-6 of the structure's size.  The
residual tolerance of configurations 0-2 is 1e-5, above their FP64 floor
(tests/test_tolerance_floor.py); the displacement tolerance is 1e-8 everywhere.
"""
import os

import numpy as np
import pytest

import bridge

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
NEWTON_FORCING = 1e-4  # the benchmark's inexact-Newton linear tolerance


def _oracle(O, conf, p, inter, max_steps=None):
    m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
    r = O.run_simulation(m, max_steps=max_steps)
    return m, r


def _k_mismatch(a, b):
    n = min(len(a), len(b))
    return sum(1 for x, y in zip(a[:n], b[:n]) if x != y) + abs(len(a) - len(b))


def test_cantilever_whole_run(eb, O, scenes):
    conf, p, inter = scenes.cantilever()          # 2,000 steps of 1 ms
    p.tolerance_residual = 1e-5
    ref, rr = _oracle(O, conf, p, inter)
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"] == 2000
    assert _k_mismatch(res.ks[0], rr["ks"]) <= 20  # Newton counts agree on >= 99% of the steps
    err = np.abs(conf.nodes.un - ref.un).max()
    assert err <= 1e-6 * 0.1, err
    assert np.abs(conf.nodes.un[-1, 2]) > 0.05    # the tip has moved 7 cm: the run is not trivial


def test_ring_drop_through_first_contact(eb, O, scenes):
    """300 steps: the ring falls, touches the floor near step 200 and bounces back up."""
    conf, p, inter = scenes.ring_drop(steps=300)
    p.tolerance_residual = 1e-5
    m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
    zmin = []
    rr = O.run_simulation(m, on_step=lambda *a: zmin.append((conf.nodes.X0[:, 2] + m.un[:, 2]).min()))
    assert min(zmin) < 2e-4 * 1.25               # the lowest node entered the contact band
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"] == 300
    assert _k_mismatch(res.ks[0], rr["ks"]) <= 3
    err = np.abs(conf.nodes.un - m.un).max()
    assert err <= 1e-6 * 0.02, err


def test_net_population_sample(eb, O, scenes):
    """Four nets of the 256-net workload (the benchmark's sides, seeds and sphere grid) in one
    batch, each against its own oracle run."""
    sides = scenes.net_sides(256, seed=0)[:4]
    sdf = scenes.sphere_sdf()
    built = [scenes.net_on_sphere(int(sd), seed=1 + i, sdf=sdf, steps=50) for i, sd in enumerate(sides)]
    confs, inters, p = [b[0] for b in built], [b[2] for b in built], built[0][1]
    p.tolerance_residual = 1e-5
    p.tolerance_displacement = 1e-8
    p.linear_tol = NEWTON_FORCING
    res = eb.run_simulations(confs, p, inters)
    for i, sd in enumerate(sides):
        c, _, it = scenes.net_on_sphere(int(sd), seed=1 + i, sdf=sdf, steps=50)
        ref, rr = _oracle(O, c, p, it)
        assert res.steps[i] == rr["steps"] == 50
        err = np.abs(confs[i].nodes.un - ref.un).max()
        assert err <= 1e-6 * 1e-3 * sd, (i, err)
    assert all(np.abs(c.nodes.un[:, 2]).max() > 1e-5 for c in confs)  # every net is falling


def test_braided_stent_configuration(eb, O, scenes):
    """Configuration 3's stent (48 wires x 200 elements, 8,664 nodes) released in its
    3.5 mm cylinder: FP32 GMRES + FP64 refinement at the benchmark's settings, 5 steps,
    residual tolerance 1e-8 (this stent's FP64 floor is ~2e-9)."""
    conf, p, inter = scenes.braided_stent(steps=5)
    p.tolerance_residual = 1e-8
    p.tolerance_displacement = 1e-8
    p.krylov_restart = 32
    p.refactor_its = 200
    p.linear_tol = NEWTON_FORCING
    ref, rr = _oracle(O, conf, p, inter)
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"] == 5
    err = np.abs(conf.nodes.un - ref.un).max()
    assert err <= 1e-6 * 0.02, err
    assert np.abs(conf.nodes.un).max() > 1e-7    # the wall has started to compress the stent


def test_reference_net_on_sphere(eb, O, scenes):
    d = np.load(os.path.join(HERE, "golden", "reference_net.npz"))
    conf, p, inter = scenes.reference_net_on_sphere(d["positions"], d["connectivity"])
    ref, rr = _oracle(O, conf, p, inter, max_steps=80)
    conf, p, inter = scenes.reference_net_on_sphere(d["positions"], d["connectivity"])
    res = eb.run_simulation(conf, p, inter, max_steps=80)
    assert res.steps[0] == rr["steps"] == 80
    assert res.ks[0] == rr["ks"]
    assert abs(res.t[0] - rr["t"]) < 1e-12
    err = np.abs(conf.nodes.un - ref.un).max()
    assert err <= 1e-6 * 0.225, err
    # the net has passed the contact threshold of the sphere (radius 55 mm + wire radius)
    r = np.linalg.norm(conf.nodes.X0 + conf.nodes.un, axis=1).min()
    assert r < 0.055 + 2e-4


def test_reference_imposed_wave_on_sphere(eb, O, scenes):
    """The imposed displacement (k_bc_lift with a non-zero imposed increment every step)
    drives the beam into the sphere over the reference's whole run."""
    conf, p, inter = scenes.reference_imposed_wave()
    ref, rr = _oracle(O, conf, p, inter)
    conf, p, inter = scenes.reference_imposed_wave()
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"]
    assert res.ks[0] == rr["ks"]
    err = np.abs(conf.nodes.un - ref.un).max()
    assert err <= 1e-6 * 0.1, err
    assert abs(conf.nodes.un[0, 0] - scenes.wave_displacement(res.t[0])) < 1e-12  # the imposed DOF
    assert conf.nodes.un[-1, 1] > 0.01           # the sphere has pushed the tip sideways
