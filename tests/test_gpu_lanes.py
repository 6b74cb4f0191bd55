"""Concurrent lanes (run_simulations(lanes=L)): the simulations are dealt onto L engines,
each advanced by its own host thread on its own stream.  A simulation's arithmetic does
not depend on which simulations share its batch (under the threshold refactorisation
rule, which decides per simulation), so every simulation ends bit for bit where the
single batch ends, with the same Newton iterations per step."""
import numpy as np
import pytest
from vtk_read import read_pvd, read_vtp

pytestmark = pytest.mark.gpu


def _nets(scenes, steps):
    sdf = scenes.sphere_sdf(n=48, h=0.8e-3)
    built = [scenes.net_on_sphere(side, seed=1 + i, sdf=sdf, steps=steps) for i, side in enumerate((12, 20, 9, 16, 14))]
    p = built[0][1]
    p.tolerance_residual = 1e-5
    p.refactor_policy = "threshold"
    return [b[0] for b in built], p, [b[2] for b in built]


def test_lanes_match_single_batch(eb, scenes):
    confs1, p1, inters1 = _nets(scenes, 12)
    r1 = eb.run_simulations(confs1, p1, inters1)
    confs3, p3, inters3 = _nets(scenes, 12)
    r3 = eb.run_simulations(confs3, p3, inters3, lanes=3)
    assert r1.steps == r3.steps == [12] * 5
    assert r1.ks == r3.ks
    assert r1.krylov_iterations == r3.krylov_iterations
    for a, b in zip(confs1, confs3):
        assert np.array_equal(a.nodes.un, b.nodes.un)
        assert np.array_equal(a.nodes.Rn, b.nodes.Rn)


def test_lanes_write_each_simulations_output(eb, scenes, tmp_path):
    """Each simulation's files land in its own sim_<index> directory whichever lane ran it:
    one write per converged step plus the initial state, and the last node file holds
    that simulation's final state."""
    confs, p, inters = _nets(scenes, 4)
    p.output_dir = str(tmp_path)
    p.output_timestep = p.initial_timestep / 2
    res = eb.run_simulations(confs, p, inters, lanes=2)
    for s, c in enumerate(confs):
        d = tmp_path / f"sim_{s:05d}"
        coll = read_pvd(str(d / "simulation.pvd"))
        assert len(coll) == 2 * (res.steps[s] + 1)
        N, _ = read_vtp(str(d / f"beams_nodes_{res.steps[s]}.vtp"))
        assert np.array_equal(N["Displacement"], c.nodes.un)
        assert np.array_equal(N["connectivity"].reshape(-1, 2), c.beams.conn)
