"""Mesh-to-SDF on the device (eb_sdf_from_mesh) against the oracle's restatement
and exact answers, and a triangulated master surface (TriangulatedSurface →
device SDF) in a full run against the oracle."""
import time

import numpy as np
import pytest

import bridge
import mesh_oracle as M

pytestmark = pytest.mark.gpu


def _gpu(eb, V, T, origin, h, dims):
    sdf = eb.DiscreteSignedDistanceField.from_mesh(V, np.asarray(T) + 1, origin, h, dims)
    return sdf.values.ravel()  # [k, j, i] -> x fastest


def test_cube_exact_on_device(eb):
    V, T = M.cube_mesh()
    args = ((-1.0, -1.0, -1.0), 0.25, (13, 13, 13))
    got = _gpu(eb, V, T, *args)
    assert np.abs(got - M.sdf_from_mesh(V, T, *args)).max() <= 1e-14


@pytest.mark.parametrize("level", [2, 3])
def test_icosphere_matches_oracle(eb, level):
    V, T = M.icosphere(level, 1.0, center=(0.1, -0.2, 0.05))
    args = ((-1.5, -1.4, -1.6), 0.13, (24, 23, 25))
    got = _gpu(eb, V, T, *args)
    ref = M.sdf_from_mesh(V, T, *args)
    assert np.abs(got - ref).max() <= 1e-13


def test_rejects_bad_triangles(eb):
    V, T = M.cube_mesh()
    with pytest.raises(eb.EbError, match="out of range"):
        _gpu(eb, V, T + 100, (0, 0, 0), 0.5, (3, 3, 3))


def test_ring_on_triangulated_floor_matches_oracle(eb, O, scenes):
    """Ring resting on the top face of a box given as a triangle mesh (the ring is
    outside the box: inside=False).  The device builds the SDF at create; the oracle
    builds its own on the same grid; positions agree within 1e-6 of the ring size."""
    conf, p, inter = scenes.ring_drop(steps=40, height=2.2e-4)
    V, T = M.cube_mesh()
    V = V * np.array([0.04, 0.04, 0.01]) - np.array([0.02, 0.02, 0.01])  # top face z = 0
    inter.master = eb.TriangulatedSurface(V, T + 1, spacing=5e-4, inside=False)
    p.tolerance_residual = 1e-5
    m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
    rr = O.run_simulation(m)
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"]
    assert np.abs(conf.nodes.un - m.un).max() <= 1e-6 * 0.02


def test_mesh_sdf_throughput(eb):
    """Throughput on a 5,120-triangle sphere and a 64^3 grid (printed)."""
    V, T = M.icosphere(4, 1.0)
    args = ((-1.3, -1.3, -1.3), 2.6 / 63, (64, 64, 64))
    _gpu(eb, V, T, (-1, -1, -1), 1.0, (2, 2, 2))
    t0 = time.perf_counter()
    vals = _gpu(eb, V, T, *args)
    dt = time.perf_counter() - t0
    pairs = len(T) * 64 ** 3
    P = M.grid_points(*args)
    assert np.abs(vals - (1.0 - np.linalg.norm(P, axis=1))).max() <= 2e-3
    print(f"mesh SDF: {len(T)} triangles x {64 ** 3} points in {dt * 1e3:.1f} ms = {pairs / dt / 1e9:.2f} G pairs/s")
