"""The analytic plane surface (PlaneSurface, def_interactions.jl:24-27) in the
oracle.  The reference declares the type without a gap function; the one used
here (gap = x[axis] - position - r, normal e_axis, zero curvature) is pinned to
the reference's own discrete-SDF path: the quadratic B-spline interpolant of
the linear field x[axis] - position reproduces it exactly away from the grid
boundary, so contact forces and tangents on the plane and on that SDF agree to
rounding, element by element and over a whole run."""
import numpy as np
import pytest

import bridge
from states import plane_states, rel_err


def _linear_sdf(O, axis, position, h=0.02, lo=-0.5, n=51):
    xs = lo + h * np.arange(n)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    field = (X, Y, Z)[axis] - position
    surf = np.zeros(14)
    surf[0] = 1
    surf[5:8] = (n, n, n)
    surf[8:11] = lo
    surf[11:14] = h
    return surf, O.sdf_prefilter(field)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_plane_contact_matches_linear_sdf(O, axis):
    rb, position = 0.01, 0.013
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    plane = np.zeros(14)
    plane[0], plane[1], plane[2] = 2, axis, position
    inp = plane_states(256, axis, position, rb, seed=11 + axis)
    ref_plane = O.compute_contact_batch(inp, props, plane, None)
    sdf, coef = _linear_sdf(O, axis, position)
    ref_sdf = O.compute_contact_batch(inp, props, sdf, coef)
    touched = np.linalg.norm(ref_plane[:, 13:157], axis=1) > 0
    assert touched.sum() > 150
    assert np.array_equal(touched, np.linalg.norm(ref_sdf[:, 13:157], axis=1) > 0)
    for name, a, b in [("Tc", 1, 13), ("K", 13, 157), ("C", 157, 301)]:
        err = rel_err(ref_plane[touched, a:b], ref_sdf[touched, a:b])
        assert err.max() <= 1e-8, f"axis {axis} {name}: {err.max():.3e}"


def test_plane_gap_known_values(O):
    """Gap sign and magnitude: a horizontal element at height z over z = 0 with
    radius r is in contact exactly when z - r <= r/4; the force points up."""
    rb = 0.01
    props = np.array([1e4, 0.0, 1e-3, 0.0])
    plane = np.zeros(14)
    plane[0], plane[1], plane[2] = 2, 2, 0.0
    inp = plane_states(4, 2, 0.0, rb, seed=3, spread=0.0)
    for p, z, touch in [(inp[0], 1.20 * rb, True), (inp[1], 1.26 * rb, False), (inp[2], 0.9 * rb, True)]:
        l0 = p[72]
        p[0:3], p[3:6] = (-l0 / 2, 0.0, z), (l0 / 2, 0.0, z)
        p[6:12] = 0.0
        eye = np.eye(3).flatten("F")
        for off in (12, 21, 30, 39):
            p[off:off + 9] = eye
        p[48:60] = 0.0
        p[73:82] = O.get_Re0(p[None, 0:3], p[None, 3:6])[0]
        out = O.compute_contact_batch(p[None], props, plane, None)[0]
        Tc = out[1:13]
        assert (np.abs(Tc).max() > 0) == touch
        if touch:
            # the contact residual pushes both nodes along +z, nothing in x or y
            assert Tc[2] < 0 and Tc[8] < 0 or Tc[2] > 0 and Tc[8] > 0
            assert np.abs(Tc[[0, 1, 6, 7]]).max() <= 1e-12 * np.abs(Tc[[2, 8]]).max()


def test_ring_drop_plane_matches_sdf_plane(O, scenes):
    """Ring touching the ground from the first step: 30 oracle steps on the
    analytic plane and on the 64³ SDF of the same plane give the same trajectory."""
    out = []
    for surface in ("plane", "sdf"):
        conf, p, inter = scenes.ring_drop(steps=30, surface=surface, height=2.2e-4)
        p.tolerance_residual = 1e-5
        m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
        r = O.run_simulation(m)
        out.append((m.un.copy(), r["ks"]))
    assert out[0][1] == out[1][1]
    assert np.abs(out[0][0] - out[1][0]).max() <= 1e-9 * 0.02
