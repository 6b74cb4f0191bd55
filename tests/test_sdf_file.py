"""read_vtk_sdf (src/IO/read_input_files.jl:154-195) and DiscreteSignedDistanceField(filename,
inside) (def_interactions.jl:67-82): a legacy-VTK structured-points SDF written here in the
layout the reference reads (four header lines, DIMENSIONS, SPACING, ORIGIN, POINT_DATA, two
more lines, then the values x fastest over as many lines as they take) comes back as the same
grid, bit for bit; inside=false flips its sign as the reference does."""
import numpy as np
import pytest


def write_vtk_sdf(path, values_kji, origin, spacing, per_line=7):
    nz, ny, nx = values_kji.shape
    flat = values_kji.ravel()  # x fastest
    with open(path, "w") as fh:
        fh.write("# vtk DataFile Version 3.0\nsigned distance field\nASCII\nDATASET STRUCTURED_POINTS\n")
        fh.write(f"DIMENSIONS {nx} {ny} {nz}\n")
        fh.write("SPACING {!r} {!r} {!r}\n".format(*map(float, spacing)))
        fh.write("ORIGIN {!r} {!r} {!r}\n".format(*map(float, origin)))
        fh.write(f"POINT_DATA {flat.size}\nSCALARS sdf double 1\nLOOKUP_TABLE default\n")
        for i in range(0, flat.size, per_line):
            fh.write(" ".join(repr(float(v)) for v in flat[i:i + per_line]) + "\n")


def sphere_grid(n=(11, 9, 13), h=0.1, R=0.3, seed=3):
    rng = np.random.default_rng(seed)
    o = (-0.5, -0.4, -0.6)
    xs, ys, zs = (o[a] + h * np.arange(n[a]) for a in range(3))
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    vals = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - R + 1e-3 * rng.standard_normal(X.shape)
    return vals, o, (h, h, h)


def test_read_vtk_sdf_round_trip(eb, tmp_path):
    from endobeams_gb300 import api
    vals, o, h = sphere_grid()
    path = str(tmp_path / "sdf.vtk")
    write_vtk_sdf(path, vals, o, h)
    dims, spacing, origin, flat = api.read_vtk_sdf(path)
    assert dims == [11, 9, 13] and tuple(spacing) == h and tuple(origin) == o
    assert np.array_equal(flat, vals.ravel())
    inside = eb.DiscreteSignedDistanceField(path, True)
    outside = eb.DiscreteSignedDistanceField(path, False)
    ref = eb.DiscreteSignedDistanceField.from_grid(vals, o, h)
    assert np.array_equal(inside.values, ref.values) and inside.dims == ref.dims
    assert inside.origin == ref.origin and inside.spacing == ref.spacing and inside.dom == ref.dom
    assert outside.inside is False and np.array_equal(outside.values, ref.values)


def test_outside_flag_negates_in_the_oracle_scene(eb, tmp_path):
    """The sign flip of inside=false reaches the contact field (oracle bridge side)."""
    import bridge
    vals, o, h = sphere_grid()
    path = str(tmp_path / "sdf.vtk")
    write_vtk_sdf(path, vals, o, h)
    conf, p, inter = _ring_with(eb, eb.DiscreteSignedDistanceField(path, False))
    sc = bridge.scene_from_conf(conf, inter)
    assert np.array_equal(sc.surface["field"], -vals)
    conf, p, inter = _ring_with(eb, eb.DiscreteSignedDistanceField(path, True))
    assert np.array_equal(bridge.scene_from_conf(conf, inter).surface["field"], vals)


def _ring_with(eb, sdf):
    from endobeams_gb300 import scenes
    conf, p, inter = scenes.ring_drop(steps=5)
    return conf, p, eb.RigidInteraction(sdf, inter.slave, inter.properties)
