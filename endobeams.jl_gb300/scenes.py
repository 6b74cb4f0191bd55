"""Synthetic scenes with the shapes, sizes and parameters of the benchmark
configurations (seeded, SI units).  No dataset or external mesh is needed.

Each builder returns ``(conf, params, inter)`` built with the public API:

* ``frame_test_beams``  — the right-angle frame of the reference's own
  known-answer test (test/test_beams.jl:13-104).
* ``cantilever``        — straight beam, clamped, ramped tip load (configuration 0).
* ``ring_drop``         — ring falling under gravity onto a plane SDF (configuration 1).
* ``net_on_sphere``     — one jittered square net dropped on a sphere SDF (configuration 2, one sim).
* ``braided_stent``     — braided stent with merged crossings released in a cylinder SDF
  (configurations 3 and 4).
* ``reference_net_on_sphere`` — the net of the reference's contact test
  (test/test_beams2rigid_contact_1_analytical.jl:14-107) on its analytic sphere.
* ``reference_imposed_wave``  — the reference's beam driven by an imposed triangular wave
  against an analytic sphere (test/test_beams2rigid_contact_2_analytical.jl:13-128).

Gravity is not implemented in the reference (def_bcs_and_loads.jl:80); it is
applied here as constant nodal `ConcentratedForce`s: f_z = -g ρA Σ l/2 over
the node's elements.
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np

from .api import (BeamElementSurface, Beams, BeamsConfiguration, BoundaryConditions, ConcentratedForce,
                  DiscreteSignedDistanceField, Encastre, ImposedDisplacement, InteractionProperties, Loads,
                  NodesBeams, PlaneSurface, RigidInteraction, SimulationParams, SphereSurface)

G_ACC = 9.81


def hht(alpha: float):
    return dict(alpha=alpha, beta=0.25 * (1 - alpha) ** 2, gamma=0.5 * (1 - 2 * alpha))


def _lumped_gravity(X, conn, rho, radius, g=G_ACC):
    """Nodal f_z (N) of the lumped self-weight; returns (1-based dofs, values)."""
    l = np.linalg.norm(X[conn[:, 1]] - X[conn[:, 0]], axis=1)
    w = rho * np.pi * radius ** 2 * l / 2 * g
    fz = np.zeros(X.shape[0])
    np.add.at(fz, conn[:, 0], w)
    np.add.at(fz, conn[:, 1], w)
    dofs = 6 * np.arange(X.shape[0]) + 3  # 1-based u_z
    return dofs, -fz


def _const_force(dofs, vals):
    table = {int(d): float(v) for d, v in zip(dofs, vals)}
    return ConcentratedForce(lambda t, i: table[i], list(table.keys()))


def grid_sdf(fn, origin, spacing, dims, inside=True) -> DiscreteSignedDistanceField:
    """Samples φ(x, y, z) on a regular grid (x fastest) into a DiscreteSignedDistanceField."""
    nx, ny, nz = dims
    xs = origin[0] + spacing * np.arange(nx)
    ys = origin[1] + spacing * np.arange(ny)
    zs = origin[2] + spacing * np.arange(nz)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return DiscreteSignedDistanceField.from_grid(fn(X, Y, Z), origin, spacing, inside=inside)


# ------------------------------------------------------------------ reference test frame

def frame_test_beams(T: float = 0.15):
    """test/test_beams.jl: 9-node right-angle frame, tip load 100 t on DOF 27, clamped node 1."""
    X = np.array([[0, 0, 0], [0, 2.5, 0], [0, 5, 0], [0, 7.5, 0], [0, 10, 0], [-2.5, 10, 0], [-5, 10, 0],
                  [-7.5, 10, 0], [-10, 10, 0]], float)
    conn = np.array([[i, i + 1] for i in range(1, 9)])
    nodes = NodesBeams(X, plane="xy")
    beams = Beams(nodes, conn, 1e6, 0.3, 1.0, 0.3, 0.0)
    loads = Loads(ConcentratedForce(lambda t, i: 100 * t, [27]))
    conf = BeamsConfiguration(nodes, beams, loads, BoundaryConditions(Encastre(range(1, 7)), 6 * len(nodes)))
    params = SimulationParams(**hht(-0.2), initial_timestep=1e-4, min_timestep=1e-4, max_timestep=1e-4,
                              output_timestep=1e-2, simulation_end_time=T, tolerance_residual=1e-3,
                              tolerance_displacement=1e-3, max_iterations=20)
    return conf, params, None


# ------------------------------------------------------------------ configuration 0

def cantilever(n_elem: int = 20, steps: int = 2000, tol: float = 1e-8):
    """L = 100 mm along x, r = 0.5 mm, steel, clamped node 1, tip u_z force 5 min(t, 1) N; Δt = 1e-3."""
    L = 0.1
    X = np.zeros((n_elem + 1, 3))
    X[:, 0] = np.linspace(0.0, L, n_elem + 1)
    conn = np.array([[i + 1, i + 2] for i in range(n_elem)])
    nodes = NodesBeams(X)
    beams = Beams(nodes, conn, 2e11, 0.33, 7850.0, 5e-4, 0.0)
    tip_dof = 6 * n_elem + 3  # 1-based u_z of the last node
    loads = Loads(ConcentratedForce(lambda t, i: 5.0 * min(t, 1.0), [tip_dof]))
    conf = BeamsConfiguration(nodes, beams, loads, BoundaryConditions(Encastre(range(1, 7)), 6 * len(nodes)))
    dt = 1e-3
    params = SimulationParams(**hht(-0.05), initial_timestep=dt, min_timestep=dt, max_timestep=dt,
                              simulation_end_time=steps * dt, tolerance_residual=tol, tolerance_displacement=tol,
                              max_iterations=20)
    return conf, params, None


# ------------------------------------------------------------------ configuration 1

def ring_drop(n_elem: int = 64, steps: int = 5000, tol: float = 1e-8, eta_n: float = 0.0, surface: str = "sdf",
              height: float = 0.002):
    """Ring R = 10 mm in the xz plane, lowest point `height` above z = 0, gravity; the ground is the
    plane z = 0 as an SDF 64³ at 0.5 mm (surface="sdf") or as an analytic PlaneSurface ("plane")."""
    Rr, r = 0.01, 2e-4
    ang = 2 * np.pi * np.arange(n_elem) / n_elem
    zc = height + Rr
    X = np.stack([Rr * np.cos(ang), np.zeros(n_elem), zc + Rr * np.sin(ang)], axis=1)
    conn0 = np.array([[i, (i + 1) % n_elem] for i in range(n_elem)])
    rho, E = 6500.0, 5e10
    nodes = NodesBeams(X)
    beams = Beams(nodes, conn0 + 1, E, 0.33, rho, r, 0.0)
    dofs, vals = _lumped_gravity(X, conn0, rho, r)
    conf = BeamsConfiguration(nodes, beams, Loads(_const_force(dofs, vals)), None)
    h, n = 0.5e-3, 64
    if surface == "plane":
        master = PlaneSurface(0.0, "z")
    else:
        master = grid_sdf(lambda x, y, z: z, (-h * (n - 1) / 2, -h * (n - 1) / 2, -0.004), h, (n, n, n))
    inter = RigidInteraction(master, BeamElementSurface(conn0 + 1), InteractionProperties(1e4, 0.3, 1e-3, eta_n))
    dt = 1e-4
    params = SimulationParams(**hht(-0.05), initial_timestep=dt, min_timestep=dt / 64, max_timestep=dt,
                              simulation_end_time=steps * dt, tolerance_residual=tol, tolerance_displacement=tol,
                              max_iterations=20)
    return conf, params, inter


# ------------------------------------------------------------------ configuration 2 (one net)

def net_on_sphere(side: int, seed: int = 1, sdf: Optional[DiscreteSignedDistanceField] = None, steps: int = 4000,
                  tol: float = 1e-8, rho: float = 7850.0, drop: float = 0.5e-3):
    """side x side nodes at 1 mm spacing, xy jitter U(±0.5 mm), r = 0.1 mm, E = 100 GPa, gravity,
    sphere R = 15 mm (SDF 128³ at 0.3 mm), μ = 0.2, Δt = 5e-5."""
    rng = np.random.default_rng(seed)
    s, r, Rs = 1e-3, 1e-4, 0.015
    ii, jj = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    X = np.zeros((side * side, 3))
    X[:, 0] = (ii.ravel() - (side - 1) / 2) * s + rng.uniform(-0.5e-3, 0.5e-3, side * side)
    X[:, 1] = (jj.ravel() - (side - 1) / 2) * s + rng.uniform(-0.5e-3, 0.5e-3, side * side)
    X[:, 2] = Rs + r + drop
    idx = np.arange(side * side).reshape(side, side)
    conn0 = np.concatenate([np.stack([idx[:-1, :].ravel(), idx[1:, :].ravel()], 1),
                            np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1)])
    nodes = NodesBeams(X)
    beams = Beams(nodes, conn0 + 1, 1e11, 0.33, rho, r, 0.0)
    dofs, vals = _lumped_gravity(X, conn0, rho, r)
    conf = BeamsConfiguration(nodes, beams, Loads(_const_force(dofs, vals)), None)
    if sdf is None:
        sdf = sphere_sdf()
    inter = RigidInteraction(sdf, BeamElementSurface(conn0 + 1), InteractionProperties(1e4, 0.2, 1e-3, 0.0))
    dt = 5e-5
    params = SimulationParams(**hht(-0.05), initial_timestep=dt, min_timestep=dt / 64, max_timestep=dt,
                              simulation_end_time=steps * dt, tolerance_residual=tol, tolerance_displacement=tol,
                              max_iterations=20)
    return conf, params, inter


def sphere_sdf(R: float = 0.015, n: int = 128, h: float = 0.3e-3):
    o = -h * (n - 1) / 2
    return grid_sdf(lambda x, y, z: np.sqrt(x * x + y * y + z * z) - R, (o, o, o), h, (n, n, n))


def net_sides(count: int = 256, seed: int = 0):
    return np.random.default_rng(seed).integers(20, 41, size=count)


# ------------------------------------------------------------------ configurations 3 and 4

def braided_stent(wires: int = 48, R: float = 4e-3, pitch_deg: float = 45.0, elems_per_wire: int = 200,
                  crossing_every: Optional[int] = 5, length: Optional[float] = None, r: float = 5e-5, E: float = 5e10, rho: float = 6500.0,
                  crimp_radius: Optional[float] = None, cyl_radius: float = 3.5e-3, h: float = 1e-4,
                  grid: Optional[tuple] = (96, 96, 256), dt: float = 1e-5, steps: int = 10000, tol: float = 1e-8,
                  precision: str = "mixed", mu: float = 0.1):
    """Braided stent: wires/2 right- and wires/2 left-handed helices on radius R.

    Node spacing along z is chosen so that every ``crossing_every``-th node of
    a wire lies on a crossing with a wire of the other hand; those nodes are
    merged (shared).  The stent length follows: L = elems·(πR/tanφ)/(n·q)
    (n = wires/2, q = crossing_every), 20.9 mm for the default 48 wires at 45°.
    With ``length`` given, q is the integer that brings L closest to it.
    ``grid=None`` sizes the SDF grid (spacing h) to the stent: ±(max(R, cyl) +
    0.5 mm) across and ±(L/2 + 1 mm) along the axis.

    Start (the reference has no crimping procedure): the stent is released at
    t = 0, at rest and stress free at its nominal radius R, inside a cylinder
    SDF φ = cyl_radius − ρ (positive in the lumen) of smaller radius, so the
    vessel wall compresses the oversized stent through the penalty contact.

    ``crimp_radius`` (optional) instead maps u⁰ to that radius with the axial
    stretch that keeps helix arc length and R = I (the rotation factor of
    that pure-stretch map).  With merged crossings this start is far from
    equilibrium: every element next to a crossing carries an end-rotation
    mismatch equal to the pitch change (about 30° for 4 → 1.5 mm), and the
    resulting nodal accelerations (~1e9 m/s²) make the release diverge
    within a few steps at Δt = 1e-5."""
    n = wires // 2
    tanp = math.tan(math.radians(pitch_deg))
    if length is not None:
        crossing_every = max(1, int(round(elems_per_wire * math.pi * R / (tanp * n * length))))
    q = crossing_every
    dz = math.pi * R / (tanp * n * q)  # crossings every πR/(n tanφ) in z
    L = elems_per_wire * dz
    zs = dz * np.arange(elems_per_wire + 1)
    # node ids: + wires own all their nodes; - wires reuse the + node at crossings
    plus_ids = np.arange(n * (elems_per_wire + 1)).reshape(n, elems_per_wire + 1)
    pos = []
    for i in range(n):
        th = 2 * np.pi * i / n + zs * tanp / R
        pos.append(np.stack([R * np.cos(th), R * np.sin(th), zs], 1))
    X = list(np.concatenate(pos))
    next_id = len(X)
    minus_ids = np.zeros((n, elems_per_wire + 1), np.int64)
    for j in range(n):
        for k in range(elems_per_wire + 1):
            if k % q == 0:
                i = (j - k // q) % n  # + wire crossing wire j at node k
                minus_ids[j, k] = plus_ids[i, k]
            else:
                th = 2 * np.pi * j / n - zs[k] * tanp / R
                X.append(np.array([R * np.cos(th), R * np.sin(th), zs[k]]))
                minus_ids[j, k] = next_id
                next_id += 1
    X = np.asarray(X)
    X[:, 2] -= L / 2
    conn0 = np.concatenate([np.stack([w[:-1], w[1:]], 1) for w in list(plus_ids) + list(minus_ids)])
    if crimp_radius is None:
        nodes = NodesBeams(X)
    else:
        sc = crimp_radius / R
        stretch = math.sqrt(1 + tanp ** 2 * (1 - sc ** 2))
        Xc = np.stack([X[:, 0] * sc, X[:, 1] * sc, X[:, 2] * stretch], 1)
        nodes = NodesBeams(X, u0=Xc - X)
    beams = Beams(nodes, conn0 + 1, E, 0.33, rho, r, 0.0)
    conf = BeamsConfiguration(nodes, beams, None, None)
    if grid is None:
        a = max(R, cyl_radius) + 0.5e-3
        grid = (2 * int(math.ceil(a / h)) + 1,) * 2 + (2 * int(math.ceil((L / 2 + 1e-3) / h)) + 1,)
    nx, ny, nz = grid
    o = (-h * (nx - 1) / 2, -h * (ny - 1) / 2, -h * (nz - 1) / 2)
    sdf = grid_sdf(lambda x, y, z: cyl_radius - np.sqrt(x * x + y * y), o, h, grid)
    inter = RigidInteraction(sdf, BeamElementSurface(conn0 + 1), InteractionProperties(1e4, mu, 1e-3, 0.0))
    params = SimulationParams(**hht(-0.05), initial_timestep=dt, min_timestep=dt / 1024, max_timestep=dt,
                              simulation_end_time=steps * dt, tolerance_residual=tol, tolerance_displacement=tol,
                              max_iterations=20, precision=precision)
    return conf, params, inter


def stent_variants(count: int = 1024, seed: int = 2):
    """Stent-population draws: wires ∈ {16,24,32,48}, R ∈ U[3,5] mm, pitch ∈ U[35,55]°,
    elements per wire ∈ U{100..400}, cylinder radius ∈ U[0.85,0.95]·R."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        out.append(dict(wires=int(rng.choice([16, 24, 32, 48])), R=float(rng.uniform(3e-3, 5e-3)),
                        pitch_deg=float(rng.uniform(35, 55)), elems_per_wire=int(rng.integers(100, 401)),
                        cyl_frac=float(rng.uniform(0.85, 0.95))))
    return out


def stent_variant(v: dict, steps: int = 10000, tol: float = 1e-8, precision: str = "mixed", length: float = 0.02):
    """One stent of the population (a draw of ``stent_variants``): L ≈ 20 mm, its own
    cylinder SDF of radius cyl_frac·R on a grid at 0.1 mm sized to the stent."""
    return braided_stent(wires=v["wires"], R=v["R"], pitch_deg=v["pitch_deg"], elems_per_wire=v["elems_per_wire"],
                         crossing_every=None, length=length, cyl_radius=v["cyl_frac"] * v["R"], grid=None,
                         steps=steps, tol=tol, precision=precision)


# ------------------------------------------------------------------ the reference's own contact scenes

def reference_net_on_sphere(positions, connectivity, steps: Optional[int] = None, end_time: float = 100.0):
    """test/test_beams2rigid_contact_1_analytical.jl:14-107: a net (node positions and 1-based
    connectivity as the test reads them from test/input/pos_net.txt and conn_net.txt) moving at
    u̇_y = -1 mm/s onto a sphere R = 55 mm at the origin; E = 10 Pa, ν = 0, ρ = 1500, r = 0.2 mm,
    damping 1e-3; kₙ = 1e-6, μ = 0.01, εᵗ = 0.5, ηₙ = 1e-3; α = -0.2, Δt from 0.01 (min 1e-6,
    max 0.1), tolerances 1e-3.  ``steps`` limits the run (the reference runs to t = 100 s)."""
    X = np.asarray(positions, float)
    conn = np.asarray(connectivity, np.int64)
    ud0 = np.zeros_like(X)
    ud0[:, 1] = -0.001
    nodes = NodesBeams(X, None, ud0, None, None, None, None, plane="xy")
    beams = Beams(nodes, conn, 10.0, 0.0, 1500.0, 2e-4, 1e-3)
    conf = BeamsConfiguration(nodes, beams, None, None)
    inter = RigidInteraction(SphereSurface([0.0, 0.0, 0.0], 0.055), BeamElementSurface(conn),
                             InteractionProperties(1e-6, 0.01, 0.5, 1e-3, 1e-6, 1e-3, 0.0))
    params = SimulationParams(**hht(-0.2), initial_timestep=0.01, min_timestep=1e-6, max_timestep=0.1,
                              output_timestep=1.0, simulation_end_time=end_time, tolerance_residual=1e-3,
                              tolerance_displacement=1e-3, max_iterations=20)
    return conf, params, inter


def wave_displacement(t: float, max_displacement: float = 0.1, time_threshold: float = 2.5) -> float:
    """The imposed x-displacement of test_beams2rigid_contact_2_analytical.jl:64-73: a triangular
    wave of amplitude 10 cm and quarter period 2.5 s (zero after 4 quarters)."""
    v = max_displacement / time_threshold
    T = time_threshold
    return ((t <= T) * v * t + (T < t <= 2 * T) * (-v * t + 2 * max_displacement)
            + (2 * T < t <= 3 * T) * v * (t - 2 * T) + (3 * T < t <= 4 * T) * (-v * t + 4 * max_displacement))


def reference_imposed_wave(end_time: float = 2.5):
    """test/test_beams2rigid_contact_2_analytical.jl:13-128: a 10 cm beam along z (20
    elements), node 1's DOFs 2:6 clamped and DOF 1 (u_x) driven by ``wave_displacement``,
    pushed against a sphere R = 4 cm centred at (5, 0.5, 8) cm; E = 50 MPa, ν = 0.33,
    ρ = 7850, r = 0.3 mm; kₙ = 10, μ = 0, εᵗ = 100, ηₙ = 1e-3; α = -0.05, Δt = 0.01
    (min 1e-6), tolerances 1e-5, at most 5 Newton iterations."""
    L, n = 0.1, 20
    X = np.zeros((n + 1, 3))
    X[:, 2] = np.linspace(0.0, L, n + 1)
    nodes = NodesBeams(X, plane="xy")
    conn = np.array([[i + 1, i + 2] for i in range(n)])
    beams = Beams(nodes, conn, 5e7, 0.33, 7850.0, 3e-4, 0.0)
    bcs = BoundaryConditions(Encastre(range(2, 7)), ImposedDisplacement(1, wave_displacement), 6 * (n + 1))
    conf = BeamsConfiguration(nodes, beams, None, bcs)
    inter = RigidInteraction(SphereSurface([0.05, 0.005, 0.08], 0.04), BeamElementSurface(conn),
                             InteractionProperties(10.0, 0.0, 100.0, 1e-3, 10.0, 1e-3, 0.0))
    params = SimulationParams(**hht(-0.05), initial_timestep=1e-2, min_timestep=1e-6, max_timestep=1e-2,
                              output_timestep=1e-2, simulation_end_time=end_time, tolerance_residual=1e-5,
                              tolerance_displacement=1e-5, max_iterations=5)
    return conf, params, inter
