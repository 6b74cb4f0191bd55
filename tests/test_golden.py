"""The oracle against its recorded golden fixtures (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import bridge

GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_beam_elements(O, gold):
    out = O.compute_beams_batch(gold["beam_in"])
    for a, b in [(0, 2), (2, 14), (14, 26), (26, 170), (170, 314), (314, 458)]:
        assert _rel(out[:, a:b], gold["beam_out"][:, a:b]) <= 1e-13


def test_contact_elements(O, gold):
    out = O.compute_contact_batch(gold["contact_in"], gold["contact_props"], gold["contact_surf"], None)
    assert _rel(out, gold["contact_out"]) <= 1e-13


def test_sdf_prefilter_and_eval(O, gold):
    coef = O.sdf_prefilter(gold["sdf_field"])
    assert _rel(coef, gold["sdf_coef"]) <= 1e-14
    ev = O.sdf_eval_batch(gold["sdf_surf"], coef, gold["sdf_pts"], 0.05)
    assert _rel(ev, gold["sdf_eval"]) <= 1e-13


def test_sdf_interpolates_grid_values(O, gold):
    """The prefiltered quadratic B-spline reproduces the grid values at the grid points."""
    s = gold["sdf_surf"]
    field = gold["sdf_field"]
    coef = O.sdf_prefilter(field)
    nz, ny, nx = field.shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    pts = np.stack([s[8] + i.ravel() * s[11], s[9] + j.ravel() * s[12], s[10] + k.ravel() * s[13]], 1)
    ev = O.sdf_eval_batch(s, coef, pts, 0.0)
    assert np.abs(ev[:, 0] - field.ravel()).max() <= 1e-12 * np.abs(field).max()


@pytest.mark.parametrize("name,steps", [("cantilever", 20), ("ring", 10)])
def test_trajectories(O, scenes, gold, name, steps):
    fn = {"cantilever": scenes.cantilever, "ring": scenes.ring_drop}[name]
    conf, p, inter = fn(steps=steps)
    p.tolerance_residual = 1e-5
    m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
    traj = []
    O.run_simulation(m, on_step=lambda *a: traj.append(m.un.copy()))
    ref = gold[f"traj_{name}"]
    assert len(traj) == len(ref)
    assert np.abs(np.asarray(traj) - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-6)
