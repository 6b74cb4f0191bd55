"""The oracle's mesh-to-SDF restatement (oracle/mesh_oracle.py), pinned by exact
answers: for the 12-triangle unit cube the signed distance is known in closed
form (faces, edges, corners), independently of how the faces are triangulated
or oriented; an icosphere approaches the analytic sphere distance as it is
refined.  The legacy-VTK triangle-mesh reader mirrors read_vtk_triangle_mesh
(src/IO/read_input_files.jl:81-152)."""
import numpy as np
import pytest

import mesh_oracle as M


def _cube_exact(P):
    """Signed distance to the unit cube, positive inside."""
    q = np.abs(P - 0.5) - 0.5
    outside = np.linalg.norm(np.maximum(q, 0.0), axis=1)
    inside = np.minimum(np.max(q, axis=1), 0.0)
    return -(outside + inside)


def test_cube_exact_distances():
    V, T = M.cube_mesh()
    origin, h, dims = (-1.0, -1.0, -1.0), 0.25, (13, 13, 13)
    got = M.sdf_from_mesh(V, T, origin, h, dims)
    P = M.grid_points(origin, h, dims)
    ref = _cube_exact(P)
    on_surface = np.abs(ref) < 1e-12
    assert np.abs(got - ref)[~on_surface].max() <= 1e-14
    assert np.abs(got[on_surface]).max() <= 1e-14
    c = np.argmin(np.linalg.norm(P - 0.5, axis=1))
    assert got[c] == pytest.approx(0.5, abs=0.125)  # grid point nearest the centre, inside
    far = np.argmax(np.linalg.norm(P - 0.5, axis=1))
    assert got[far] == pytest.approx(-np.sqrt(3) * 1.0, abs=1e-12)  # corner (-1,-1,-1) to (0,0,0)


def test_orientation_does_not_matter():
    V, T = M.cube_mesh()
    args = ((-0.5, -0.5, -0.5), 0.2, (11, 11, 11))
    a = M.sdf_from_mesh(V, T, *args)
    b = M.sdf_from_mesh(V, T[:, ::-1], *args)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("level,tol", [(1, 0.1), (3, 0.01)])
def test_icosphere_approaches_the_sphere(level, tol):
    R = 1.0
    V, T = M.icosphere(level, R)
    args = ((-1.6, -1.6, -1.6), 0.4, (9, 9, 9))
    got = M.sdf_from_mesh(V, T, *args)
    P = M.grid_points(*args)
    ref = R - np.linalg.norm(P, axis=1)
    assert np.abs(got - ref).max() <= tol * R
    assert np.all(np.sign(got[np.abs(ref) > tol]) == np.sign(ref[np.abs(ref) > tol]))


def test_vtk_triangle_mesh_round_trip(eb, tmp_path):
    V, T = M.icosphere(1, 2.5, center=(1.0, -2.0, 0.5))
    path = tmp_path / "mesh.vtk"
    M.write_vtk_triangle_mesh(path, V, T)
    pts, tris = eb.read_vtk_triangle_mesh(str(path))
    assert np.array_equal(np.array(pts), V)
    assert np.array_equal(np.array(tris), T + 1)  # 1-based like the reference
