"""Device element kernels vs the oracle's compute_beams / compute_contact_beams.

Tolerance: normwise relative error per output block ≤ 1e-12 (the element
parity bar), except the contact energy (a diagnostic whose regularised
penalty Π(g) sums terms of opposite sign, held to 1e-9) and the
discrete-SDF contact outputs, where the gap
g = φ(x) − r is a difference of nearly equal numbers (φ ~ r near contact):
interpolating φ in a different summation order moves g by ~eps·|φ|/|g|
relative, so those blocks are held to 1e-10.
"""
import numpy as np
import pytest

from states import beam_states, contact_states, plane_states, rel_err

pytestmark = pytest.mark.gpu

BLOCKS = [("strain", 0, 1), ("kinetic", 1, 2), ("Tint", 2, 14), ("Tk", 14, 26), ("K", 26, 170), ("M", 170, 314),
          ("C", 314, 458)]


@pytest.mark.parametrize("small", [False, True])
def test_beam_element_parity(eb, O, small):
    inp = beam_states(512, seed=3 + small, small=small)
    ref = O.compute_beams_batch(inp)
    out = eb.element_eval(inp)
    for name, a, b in BLOCKS:
        if name == "strain" and small:
            continue  # O(θ²) energy of a 1e-7 rad state is rounding noise in both
        err = rel_err(out[:, a:b], ref[:, a:b])
        assert err.max() <= 1e-12, f"{name}: max rel err {err.max():.3e}"


def test_beam_element_zero_state(eb, O):
    """Undeformed element at rest: all forces vanish, tangents match."""
    inp = beam_states(8, seed=5, angle=0.0)
    inp[:, 6:12] = 0.0
    inp[:, 48:72] = 0.0
    eye = np.eye(3).flatten("F")
    for off in (12, 21, 30, 39):
        inp[:, off:off + 9] = eye
    ref = O.compute_beams_batch(inp)
    out = eb.element_eval(inp)
    assert np.abs(out[:, 2:26]).max() < 1e-9 * np.abs(ref[:, 26:170]).max()
    for name, a, b in [("K", 26, 170), ("M", 170, 314)]:
        assert rel_err(out[:, a:b], ref[:, a:b]).max() <= 1e-12


def _sphere_setup():
    center = np.array([0.1, -0.2, 0.3])
    Rs, rb = 1.0, 0.01
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    surf = np.zeros(14)
    surf[1:4], surf[4] = center, Rs
    return center, Rs, rb, props, surf


def test_contact_sphere_parity(eb, O):
    center, Rs, rb, props, surf = _sphere_setup()
    inp = contact_states(512, center, Rs, rb)
    ref = O.compute_contact_batch(inp, props, surf, None)
    out, flags = eb.contact_eval(inp, props, surf)
    touched = np.linalg.norm(ref[:, 13:157], axis=1) > 0
    assert touched.sum() > 400
    assert np.array_equal(flags.astype(bool), touched)
    for name, a, b, tol in [("E", 0, 1, 1e-9), ("Tc", 1, 13, 1e-12), ("K", 13, 157, 1e-12), ("C", 157, 301, 1e-12)]:
        err = rel_err(out[touched, a:b], ref[touched, a:b])
        assert err.max() <= tol, f"{name}: {err.max():.3e}"


def test_contact_sdf_parity(eb, O):
    center, Rs, rb, props, _ = _sphere_setup()
    h = 0.02
    xs = np.arange(-1.2, 1.45, h)
    n = len(xs)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    field = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - Rs
    surf = np.zeros(14)
    surf[0] = 1
    surf[5:8] = (n, n, n)
    surf[8:11] = center + xs[0]
    surf[11:14] = h
    coef = O.sdf_prefilter(field)
    inp = contact_states(512, center, Rs, rb, seed=7)
    ref = O.compute_contact_batch(inp, props, surf, coef)
    out, flags = eb.contact_eval(inp, props, surf, values=field)
    touched = np.linalg.norm(ref[:, 13:157], axis=1) > 0
    assert touched.sum() > 400
    assert np.array_equal(flags.astype(bool), touched)
    for name, a, b in [("E", 0, 1), ("Tc", 1, 13), ("K", 13, 157), ("C", 157, 301)]:
        err = rel_err(out[touched, a:b], ref[touched, a:b])
        assert err.max() <= 1e-10, f"{name}: {err.max():.3e}"


@pytest.mark.parametrize("axis", [0, 2])
def test_contact_plane_parity(eb, O, axis):
    """Analytic PlaneSurface (x[axis] = 0.013) against the oracle's plane."""
    rb, position = 0.01, 0.013
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    surf = np.zeros(14)
    surf[0], surf[1], surf[2] = 2, axis, position
    inp = plane_states(512, axis, position, rb, seed=21 + axis)
    ref = O.compute_contact_batch(inp, props, surf, None)
    out, flags = eb.contact_eval(inp, props, surf)
    touched = np.linalg.norm(ref[:, 13:157], axis=1) > 0
    assert touched.sum() > 300
    assert np.array_equal(flags.astype(bool), touched)
    for name, a, b, tol in [("E", 0, 1, 1e-9), ("Tc", 1, 13, 1e-12), ("K", 13, 157, 1e-12), ("C", 157, 301, 1e-12)]:
        err = rel_err(out[touched, a:b], ref[touched, a:b])
        assert err.max() <= tol, f"{name}: {err.max():.3e}"
