"""An SDF read from a legacy-VTK file (read_vtk_sdf, src/IO/read_input_files.jl:154-195) drives
the GPU contact exactly as the same grid given in memory: a ring dropped on the plane SDF of
configuration 1, written to a file with full precision and read back, takes the same steps to
the same bits."""
import numpy as np
import pytest

from test_sdf_file import write_vtk_sdf

pytestmark = pytest.mark.gpu


def test_ring_on_sdf_file_matches_in_memory_grid(eb, scenes, tmp_path):
    conf, p, inter = scenes.ring_drop(steps=210)
    p.tolerance_residual = 1e-5
    m = inter.master
    path = str(tmp_path / "plane.vtk")
    write_vtk_sdf(path, m.values, m.origin, m.spacing)
    conf2, p2, inter2 = scenes.ring_drop(steps=210)
    p2.tolerance_residual = 1e-5
    inter2 = eb.RigidInteraction(eb.DiscreteSignedDistanceField(path, True), inter2.slave, inter2.properties)
    r1 = eb.run_simulation(conf, p, inter)
    r2 = eb.run_simulation(conf2, p2, inter2)
    assert r1.steps == r2.steps and r1.ks == r2.ks
    assert np.array_equal(conf.nodes.un, conf2.nodes.un)
    assert (conf.nodes.X0[:, 2] + conf.nodes.un[:, 2]).min() < 2.5e-4  # the ring is on the floor (contact from step ~195)
