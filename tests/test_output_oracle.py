"""The oracle's restatement of recompute_at_gausspts_beams!
(src/IO/visualization_beams.jl:122-162).  The reference has no test of its
output; these are the interpolation's own properties: the end points of every
element are its nodes, an unbent element interpolates along its chord, the
bending shape follows the end rotations (cubic Hermite: the chord-normal
offset at mid-span is l0/8 of the rotation difference), and strain/stress
are 1 - l/l0 and E (1 - l/l0)."""
import numpy as np
from scipy.spatial.transform import Rotation as Rot

import bridge


def _model(O, scenes):
    conf, p, inter = scenes.cantilever(steps=3)
    return O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))


def test_end_points_are_the_nodes(O, scenes):
    m = _model(O, scenes)
    rng = np.random.default_rng(0)
    m.u = m.u + rng.normal(size=m.u.shape) * 1e-3
    m.R = np.stack([Rot.from_rotvec(v).as_matrix().flatten("F") for v in rng.normal(size=(m.n, 3)) * 0.1])
    P = 7
    o = O.OracleModel.beam_output(m, P)
    x = m.X0 + m.u
    pts = o["points"].reshape(m.ne, P, 3)
    assert np.abs(pts[:, 0] - x[m.conn[:, 0]]).max() <= 1e-15
    assert np.abs(pts[:, -1] - x[m.conn[:, 1]]).max() <= 1e-15
    d = o["displacement"].reshape(m.ne, P, 3)
    assert np.abs(d[:, 0] - m.u[m.conn[:, 0]]).max() == 0
    assert np.abs(d[:, -1] - m.u[m.conn[:, 1]]).max() <= 1e-18


def test_unbent_element_follows_its_chord(O, scenes):
    m = _model(O, scenes)
    m.u = m.u + np.array([1e-3, -2e-3, 5e-4])  # rigid translation, identity rotations
    P = 10
    o = O.OracleModel.beam_output(m, P)
    x = m.X0 + m.u
    z = np.linspace(-1, 1, P)
    a, b = x[m.conn[:, 0]], x[m.conn[:, 1]]
    expect = a[:, None, :] + ((z + 1) / 2)[None, :, None] * (b - a)[:, None, :]
    assert np.abs(o["points"].reshape(m.ne, P, 3) - expect).max() <= 1e-15
    assert np.abs(o["strain"]).max() <= 1e-15
    assert np.abs(o["velocity"]).max() == 0


def test_bending_shape_and_axial_fields(O, scenes):
    """Both end sections rotated by ±θ about the local z axis (a constant-curvature
    bend): the mid point moves off the chord by l0 θ / 4 (N3(l0/2) = l0/8, N4 = -l0/8)."""
    m = _model(O, scenes)
    th = 1e-3
    e = 4
    a, b = m.conn[e]
    Re0 = m.Re0[e].reshape(3, 3, order="F")
    ez = Re0[:, 2]
    m.R[a] = Rot.from_rotvec(ez * th).as_matrix().flatten("F")
    m.R[b] = Rot.from_rotvec(-ez * th).as_matrix().flatten("F")
    P = 3
    o = O.OracleModel.beam_output(m, P)
    mid = o["points"][P * e + 1]
    chord_mid = 0.5 * (m.X0[a] + m.X0[b])
    off = mid - chord_mid
    l0 = m.l0[e]
    assert abs(np.dot(off, Re0[:, 1]) - l0 * th / 4) <= 1e-6 * l0 * th
    # stretched element: strain 1 - l/l0, stress E (1 - l/l0)
    m2 = _model(O, scenes)
    m2.u[m2.conn[e, 1]] += 1e-4 * (m2.X0[b] - m2.X0[a]) / l0
    o2 = O.OracleModel.beam_output(m2, P)
    ln = np.linalg.norm((m2.X0[b] + m2.u[b]) - (m2.X0[a] + m2.u[a]))
    assert np.allclose(o2["strain"][P * e:P * e + P], 1 - ln / l0, rtol=0, atol=1e-15)
    assert np.allclose(o2["stress"][P * e:P * e + P], m2.E[e] * (1 - ln / l0), rtol=1e-15, atol=0)
