"""Trilinear voxel-SDF option on the GPU (the reference interpolates quadratically):
the contact element against the oracle's trilinear restatement, and the ring drop of
configuration 1 through first contact against the oracle.  On the floor z = 0 (a
linear field, which both interpolants reproduce exactly inside the grid) the trilinear
run also matches the reference's quadratic B-spline run within the Newton tolerance."""
import numpy as np
import pytest

import bridge
from states import contact_states, rel_err

pytestmark = pytest.mark.gpu


def test_contact_trilinear_sdf_parity(eb, O):
    center, Rs, rb = np.array([0.1, -0.2, 0.3]), 1.0, 0.01
    h = 0.02
    xs = np.arange(-1.2, 1.45, h)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    field = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - Rs
    surf, coef = O.surface_arrays(dict(kind="sdf", field=field, x0=tuple(center + xs[0]), h=(h, h, h),
                                       interp="trilinear"))
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    inp = contact_states(512, center, Rs, rb, seed=9)
    ref = O.compute_contact_batch(inp, props, surf, coef)
    out, flags = eb.contact_eval(inp, props, surf, values=field)
    touched = np.linalg.norm(ref[:, 13:157], axis=1) > 0
    assert touched.sum() > 400
    assert np.array_equal(flags.astype(bool), touched)
    # the energy of a Gauss point barely in contact is a difference of close numbers (g = φ − r
    # near zero), so its per-element relative error carries the rounding of φ divided by g
    for name, a, b, tol in [("E", 0, 1, 1e-6), ("Tc", 1, 13, 1e-10), ("K", 13, 157, 1e-10), ("C", 157, 301, 1e-10)]:
        err = rel_err(out[touched, a:b], ref[touched, a:b])
        assert err.max() <= tol, f"{name}: {err.max():.3e}"
    e_all = np.linalg.norm(out[touched, 0] - ref[touched, 0]) / np.linalg.norm(ref[touched, 0])
    assert e_all <= 1e-10


def _ring(eb, scenes, interp):
    conf, p, inter = scenes.ring_drop(steps=220)
    p.tolerance_residual = 1e-5
    m = inter.master
    sdf = eb.DiscreteSignedDistanceField.from_grid(m.values, m.origin, m.spacing, interpolation=interp)
    return conf, p, eb.RigidInteraction(sdf, inter.slave, inter.properties)


def test_ring_drop_on_trilinear_sdf(eb, O, scenes):
    conf, p, inter = _ring(eb, scenes, "trilinear")
    ref = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
    assert bridge.scene_from_conf(conf, inter).surface["interp"] == "trilinear"
    rr = O.run_simulation(ref)
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"] == 220
    # Newton counts agree except where a step's residual lands on the tolerance (rounding)
    assert sum(1 for a, b in zip(res.ks[0], rr["ks"]) if a != b) <= 3
    assert np.abs(conf.nodes.un - ref.un).max() <= 1e-6 * 0.02
    assert (conf.nodes.X0[:, 2] + conf.nodes.un[:, 2]).min() < 2.5e-4  # on the floor
    quad, pq, iq = _ring(eb, scenes, "quadratic")
    eb.run_simulation(quad, pq, iq)
    # the two interpolants agree on the linear floor field, so the runs differ only where a
    # step's Newton iterations end at a different iterate within the tolerance (measured 1.1e-9
    # of the ring size)
    assert np.abs(quad.nodes.un - conf.nodes.un).max() <= 1e-6 * 0.02
