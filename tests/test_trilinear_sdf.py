"""Trilinear voxel-SDF option (not in the reference, which interpolates its SDF with a
quadratic B-spline): the oracle's restatement and the device formulas compiled for the host.

The trilinear interpolant reproduces any polynomial a + bx + cy + dz + exy + fxz + gyz + hxyz
sampled on the grid exactly, inside every cell: value, gradient and the mixed second
derivatives (the pure ones are zero).  The device contact element on a trilinear SDF is then
held to the oracle's at the discrete-SDF bar of the GPU tests."""
import ctypes

import numpy as np
import pytest

from states import contact_states, rel_err
from test_host_kernels import GAUSS, P, host  # noqa: F401  (fixture)

C0 = np.array([0.3, -0.7, 1.1, 0.4, 0.9, -0.5, 0.25, 0.6])  # a b c d e f g h


def _poly(x, y, z, c=C0):
    return c[0] + c[1] * x + c[2] * y + c[3] * z + c[4] * x * y + c[5] * x * z + c[6] * y * z + c[7] * x * y * z


def _grid(n=(7, 6, 5), h=(0.3, 0.25, 0.2), o=(-0.9, -0.6, -0.4), fn=_poly):
    xs, ys, zs = (o[a] + h[a] * np.arange(n[a]) for a in range(3))
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    surf = np.zeros(14)
    surf[0] = 3
    surf[5:8], surf[8:11], surf[11:14] = n, o, h
    return fn(X, Y, Z), surf


def test_oracle_trilinear_reproduces_multilinear_polynomials(O):
    field, surf = _grid()
    _, coef = O.surface_arrays(dict(kind="sdf", field=field, x0=tuple(surf[8:11]), h=tuple(surf[11:14]),
                                    interp="trilinear"))
    assert O.surface_arrays(dict(kind="sdf", field=field, x0=(0, 0, 0), h=(1, 1, 1), interp="trilinear"))[0][0] == 3
    rng = np.random.default_rng(5)
    lo, hi = surf[8:11], surf[8:11] + (surf[5:8] - 1) * surf[11:14]
    pts = rng.uniform(lo, hi, (200, 3))
    out = O.sdf_eval_batch(surf, coef, pts, 0.01)
    x, y, z = pts.T
    c = C0
    assert np.allclose(out[:, 0], _poly(x, y, z), rtol=0, atol=1e-13)
    grad = np.stack([c[1] + c[4] * y + c[5] * z + c[7] * y * z, c[2] + c[4] * x + c[6] * z + c[7] * x * z,
                     c[3] + c[5] * x + c[6] * y + c[7] * x * y], 1)
    assert np.allclose(out[:, 1:4], grad, rtol=0, atol=1e-12)
    H = out[:, 4:13].reshape(-1, 3, 3)
    assert np.allclose(H[:, [0, 1, 2], [0, 1, 2]], 0.0, atol=0)
    assert np.allclose(H[:, 0, 1], c[4] + c[7] * z, atol=1e-12) and np.allclose(H[:, 1, 0], H[:, 0, 1])
    assert np.allclose(H[:, 0, 2], c[5] + c[7] * y, atol=1e-12)
    assert np.allclose(H[:, 1, 2], c[6] + c[7] * x, atol=1e-12)


def test_oracle_trilinear_is_continuous_across_cells(O):
    field, surf = _grid(fn=lambda x, y, z: np.sin(3 * x) * np.cos(2 * y) + z * z)
    _, coef = O.surface_arrays(dict(kind="sdf", field=field, x0=tuple(surf[8:11]), h=tuple(surf[11:14]),
                                    interp="trilinear"))
    # on either side of the face x = x0 + 3 hx, and at the grid points themselves
    xf = surf[8] + 3 * surf[11]
    pts = np.array([[xf - 1e-12, 0.05, 0.1], [xf + 1e-12, 0.05, 0.1]])
    v = O.sdf_eval_batch(surf, coef, pts, 0.01)[:, 0]
    assert abs(v[0] - v[1]) < 1e-10
    gp = np.array([[surf[8] + 2 * surf[11], surf[9] + 3 * surf[12], surf[10] + 1 * surf[13]]])
    assert abs(O.sdf_eval_batch(surf, coef, gp, 0.01)[0, 0] - field[1, 3, 2]) < 1e-14


@pytest.mark.parametrize("interp", ["quadratic", "trilinear"])
def test_device_formulas_on_voxel_sdf_match_oracle(O, host, interp):  # noqa: F811
    center, Rs, rb = np.array([0.1, -0.2, 0.3]), 1.0, 0.01
    h = 0.02
    xs = np.arange(-1.2, 1.45, h)
    n = len(xs)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    field = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - Rs
    surf, coef = O.surface_arrays(dict(kind="sdf", field=field, x0=tuple(center + xs[0]), h=(h, h, h),
                                       interp=interp))
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    inp = contact_states(384, center, Rs, rb, seed=41)
    ref = O.compute_contact_batch(inp, props, surf, coef)
    out = np.zeros((len(inp), 301))
    host.host_contact_eval_grid(ctypes.c_int64(len(inp)), inp.ctypes.data_as(P), GAUSS.ctypes.data_as(P),
                                props.ctypes.data_as(P), surf.ctypes.data_as(P), coef.ctypes.data_as(P),
                                out.ctypes.data_as(P))
    touched = np.linalg.norm(ref[:, 13:157], axis=1) > 0
    assert touched.sum() > 250
    assert np.array_equal(np.linalg.norm(out[:, 13:157], axis=1) > 0, touched)
    for name, a, b in [("E", 0, 1), ("Tc", 1, 13), ("K", 13, 157), ("C", 157, 301)]:
        err = rel_err(out[touched, a:b], ref[touched, a:b]).max()
        assert err <= 1e-10, f"{name}: {err:.3e}"
