"""Host API mirroring EndoBeams.jl's public interface (src/EndoBeams.jl:37-43).

The constructors keep the reference's names, argument order and 1-based
indexing for connectivity and degrees of freedom, so a script written for
the Julia package reads the same here:

    nodes = NodesBeams(X, u0, ud0, udd0, w0, wd0, wdd0)
    beams = Beams(nodes, connectivity, E, nu, rho, radius, damping)
    conf  = BeamsConfiguration(nodes, beams, Loads(ConcentratedForce(f, [27])),
                               BoundaryConditions(Encastre(range(1, 7)), 6 * n))
    params = SimulationParams(alpha=a, beta=b, gamma=g, ...)
    run_simulation(conf, params)          # run_simulation! (src/run_simulation.jl:1)

Every step runs on the GPU through libendobeams_gb300 (there is no CPU
path); ``run_simulations`` runs many independent configurations in one
batched handle.  With ``SimulationParams.output_dir`` set, VTK files are
written as the reference's write_VTK does (src/IO/visualization_beams.jl),
by the library's asynchronous writer.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check, f64, i32, i64, ptr

# ------------------------------------------------------------------ configuration objects


def _dofs(x) -> np.ndarray:
    """1-based Int / UnitRange / Vector of DOFs -> sorted 0-based int64 array (order kept)."""
    if isinstance(x, (int, np.integer)):
        return np.array([int(x) - 1], np.int64)
    return np.asarray(list(x), dtype=np.int64) - 1


class NodesBeams:
    """NodesBeams(X, u⁰, u̇⁰, ü⁰, w⁰, ẇ⁰, ẅ⁰, plane=nothing, R=nothing) (def_node_beam.jl:55-90)."""

    def __init__(self, X, u0=None, ud0=None, udd0=None, w0=None, wd0=None, wdd0=None, plane=None, R=None):
        self.X0 = f64(X).reshape(-1, 3)
        n = self.X0.shape[0]
        z = lambda a: f64(a).reshape(n, 3) if a is not None else np.zeros((n, 3))
        self.u, self.ud, self.udd = z(u0), z(ud0), z(udd0)
        self.w, self.wd, self.wdd = z(w0), z(wd0), z(wdd0)
        if R is None:
            self.R = np.tile(np.eye(3).flatten(order="F"), (n, 1))
        else:
            R = f64(R)
            self.R = R.reshape(n, 9) if R.ndim != 3 else np.stack([r.flatten(order="F") for r in R])
        self.dR = np.tile(np.eye(3).flatten(order="F"), (n, 1))
        self.plane = plane
        # state at the last converged step (uⁿ, u̇ⁿ, ... of NodeBeam)
        self.un, self.udn, self.uddn = self.u.copy(), self.ud.copy(), self.udd.copy()
        self.wn, self.wdn, self.wddn = self.w.copy(), self.wd.copy(), self.wdd.copy()
        self.Rn, self.dRn = self.R.copy(), self.dR.copy()

    def __len__(self):
        return self.X0.shape[0]


class Beams:
    """Beams(nodes, connectivity, E, ν, ρ, radius, damping, Rₑ⁰=nothing) (def_beam.jl:102-142).

    ``connectivity`` is 1-based like the reference (rows of node pairs)."""

    def __init__(self, nodes: NodesBeams, connectivity, E, nu, rho, radius, damping, Re0=None):
        conn = np.asarray([tuple(c) for c in connectivity] if not isinstance(connectivity, np.ndarray) else connectivity)
        self.conn = i64(conn).reshape(-1, 2) - 1
        ne = self.conn.shape[0]
        bc = lambda x: np.broadcast_to(np.asarray(x, float), (ne,)).copy()
        self.E, self.nu, self.rho, self.radius, self.damping = bc(E), bc(nu), bc(rho), bc(radius), bc(damping)
        self.Re0 = None if Re0 is None else f64(Re0).reshape(ne, 9)

    def __len__(self):
        return self.conn.shape[0]


@dataclass
class ConcentratedForce:
    """ConcentratedForce(force_function(t, dof), loaded_dofs) (def_bcs_and_loads.jl:66-77); dofs 1-based."""
    force_function: Callable[[float, int], float]
    loaded_dofs: Sequence[int]


@dataclass
class Loads:
    concentrated_force: Optional[ConcentratedForce] = None


@dataclass
class Encastre:
    blocked_dofs: Sequence[int]


@dataclass
class ImposedDisplacement:
    displaced_dofs: Sequence[int]
    imposed_displacements_function: Callable[[float], float]


class BoundaryConditions:
    """BoundaryConditions constructors of def_bcs_and_loads.jl:21-64 (dofs 1-based)."""

    def __init__(self, *args):
        ndofs = int(args[-1])
        bcs = args[:-1]
        enc = next((b for b in bcs if isinstance(b, Encastre)), None)
        imp = next((b for b in bcs if isinstance(b, ImposedDisplacement)), None)
        fixed = []
        if enc is not None:
            fixed += list(_dofs(enc.blocked_dofs))
        disp = list(_dofs(imp.displaced_dofs)) if imp is not None else []
        if enc is not None and imp is not None:
            fixed = sorted(disp + fixed)
        elif imp is not None:
            fixed = disp
        self.fixed_dofs = np.asarray(fixed, np.int64)
        mask = np.ones(ndofs, bool)
        mask[self.fixed_dofs] = False
        self.free_dofs = np.nonzero(mask)[0]
        self.displaced_indices = np.asarray([i for i, d in enumerate(self.fixed_dofs) if d in set(disp)], np.int64)
        self.imposed_displacements = np.zeros(len(self.fixed_dofs))
        self.imposed_displacements_function = imp.imposed_displacements_function if imp is not None else None


class BeamsConfiguration:
    """BeamsConfiguration(nodes, beams, loads, bcs) (def_configurations.jl:15-26)."""

    def __init__(self, nodes: NodesBeams, beams: Beams, loads: Optional[Loads] = None,
                 bcs: Optional[BoundaryConditions] = None):
        self.nodes, self.beams, self.loads = nodes, beams, loads
        self.ndofs = 6 * len(nodes)
        self.bcs = bcs if bcs is not None else BoundaryConditions(self.ndofs)


@dataclass
class InteractionProperties:
    """InteractionProperties(kₙ, μ, εᵗ, ηₙ, kₜ, ηₜ, u̇ₛ) (def_interactions.jl:6-14); kₜ, ηₜ, u̇ₛ are unused."""
    kn: float
    mu: float
    eps_t: float
    eta_n: float
    kt: float = 0.0
    eta_t: float = 0.0
    u_s: float = 0.0


@dataclass
class SphereSurface:
    center: Sequence[float]
    radius: float


@dataclass
class PlaneSurface:
    """PlaneSurface(position, axis) (def_interactions.jl:24-27): the plane x[axis] = position.

    The reference declares it without a gap function.  Here the body lies on
    the positive side: gap = x[axis] - position - r, normal e_axis, zero
    curvature (the sphere's convention, utils_compute_interactions_beams.jl:2-36)."""
    position: float
    axis: str  # 'x', 'y' or 'z'

    @property
    def axis_index(self) -> int:
        a = self.axis
        if isinstance(a, str) and a.lower() in ("x", "y", "z"):
            return "xyz".index(a.lower())
        if isinstance(a, (int, np.integer)) and 0 <= int(a) <= 2:
            return int(a)
        raise ValueError(f"PlaneSurface.axis must be 'x', 'y' or 'z', got {a!r}")


class DiscreteSignedDistanceField:
    """DiscreteSignedDistanceField(filename, inside) (def_interactions.jl:67-82).

    The grid is kept as given (x fastest); the quadratic B-spline prefilter
    runs in the library.  ``from_grid`` builds one from an array.

    ``interpolation="trilinear"`` (not in the reference) interpolates the
    samples trilinearly instead (8 taps, no prefilter; the gradient jumps
    across cell faces and the Hessian keeps only its mixed terms)."""

    def __init__(self, filename: Optional[str] = None, inside: bool = True, flag_load_from_file_iterative=False,
                 *, values=None, origin=None, spacing=None, interpolation: str = "quadratic"):
        if interpolation not in ("quadratic", "trilinear"):
            raise ValueError("interpolation must be 'quadratic' or 'trilinear'")
        self.interpolation = interpolation
        if filename is not None:
            dims, spacing, origin, values = read_vtk_sdf(filename)
            values = np.asarray(values, float).reshape(dims[2], dims[1], dims[0])
        self.values = f64(values)  # [k, j, i]
        nz, ny, nx = self.values.shape
        self.dims = (nx, ny, nz)
        self.origin = tuple(float(x) for x in origin)
        self.spacing = tuple(float(x) for x in np.broadcast_to(np.asarray(spacing, float), (3,)))
        self.inside = bool(inside)
        ends = [self.origin[a] + (self.dims[a] - 1) * self.spacing[a] for a in range(3)]
        self.dom = (self.origin[0], ends[0], self.origin[1], ends[1], self.origin[2], ends[2])

    @classmethod
    def from_grid(cls, values, origin, spacing, inside=True, interpolation="quadratic"):
        return cls(None, inside, values=values, origin=origin, spacing=spacing, interpolation=interpolation)

    @classmethod
    def from_mesh(cls, positions, triangles, origin, spacing, dims, inside=True):
        """Signed distance of a closed triangle mesh sampled on the grid, computed on the
        device (eb_sdf_from_mesh): positive inside the mesh, as the reference's SDF files are
        for bodies inside the surface.  ``triangles`` are 1-based like read_vtk_triangle_mesh's."""
        V = f64(positions).reshape(-1, 3)
        T = i64(triangles).reshape(-1, 3) - 1
        d = i64([int(x) for x in dims])
        o = f64(origin)
        h = f64(np.broadcast_to(np.asarray(spacing, float), (3,)))
        out = np.zeros(int(d[0] * d[1] * d[2]))
        check(_lib.load().eb_sdf_from_mesh(len(V), ptr(V), len(T), ptr(T, C.c_int64), ptr(d, C.c_int64), ptr(o),
                                           ptr(h), ptr(out)), "eb_sdf_from_mesh")
        return cls.from_grid(out.reshape(int(d[2]), int(d[1]), int(d[0])), o, h, inside=inside)


def read_vtk_triangle_mesh(file_path: str):
    """read_vtk_triangle_mesh (read_input_files.jl:81-152): the POINTS (one per line) and
    the 3-node cells of a legacy-VTK file; returns (positions list, 1-based triangles list)."""
    nodes, tris = [], []
    in_points = in_cells = False
    n_points = n_cells = 0
    with open(file_path) as fh:
        for line in fh:
            line = line.rstrip("\n")
            if not line or line.startswith("#"):
                continue
            if "POINTS" in line:
                in_points, n_points = True, int(line.split()[1])
                continue
            if in_points:
                if len(nodes) < n_points:
                    nodes.append([float(x) for x in line.split()])
                if len(nodes) == n_points:
                    in_points = False
                continue
            if "CELLS" in line:
                in_cells, n_cells = True, int(line.split()[1])
                continue
            if in_cells:
                cell = [int(x) for x in line.split()]
                if cell[0] == 3:
                    tris.append([c + 1 for c in cell[1:]])
                if len(tris) == n_cells:
                    break
    return [np.array(p, float) for p in nodes], [np.array(t, np.int64) for t in tris]


@dataclass
class TriangulatedSurface:
    """TriangulatedSurface(positions, triangles) (def_interactions.jl:46-49), 1-based triangles.

    The reference declares it without contact functions.  Here it becomes a master
    surface through its signed distance field, computed on the device at create on a
    grid of `spacing` (default: 1/64 of the mesh's largest extent) padded by `margin`
    cells; `inside` as for DiscreteSignedDistanceField."""
    positions: Sequence
    triangles: Sequence
    spacing: Optional[float] = None
    margin: int = 4
    inside: bool = True

    def grid(self):
        """(origin, spacing, dims) of the SDF grid."""
        V = f64(np.asarray(self.positions, float)).reshape(-1, 3)
        lo, hi = V.min(0), V.max(0)
        h = float(self.spacing) if self.spacing else float((hi - lo).max()) / 64
        dims = np.ceil((hi - lo) / h).astype(int) + 2 * self.margin + 1
        return lo - self.margin * h, h, dims

    def to_sdf(self) -> "DiscreteSignedDistanceField":
        o, h, dims = self.grid()
        return DiscreteSignedDistanceField.from_mesh(self.positions, self.triangles, o, h, dims, inside=self.inside)


def read_vtk_sdf(filename: str):
    """Legacy-VTK structured-points reader with the layout of read_vtk_sdf (read_input_files.jl:154-195)."""
    with open(filename) as fh:
        for _ in range(4):
            fh.readline()
        dims = [int(x) for x in fh.readline().split()[1:4]]
        spacing = [float(x) for x in fh.readline().split()[1:4]]
        origin = [float(x) for x in fh.readline().split()[1:4]]
        n = int(fh.readline().split()[1])
        fh.readline()
        fh.readline()
        vals = []
        while len(vals) < n:
            vals += [float(x) for x in fh.readline().split()]
    return dims, spacing, origin, np.asarray(vals[:n])


class BeamElementSurface:
    """BeamElementSurface(contact_beams) (def_interactions.jl:52-65); 1-based element ids or a connectivity matrix."""

    def __init__(self, x):
        a = np.asarray(x)
        if a.ndim == 2:
            self.contact_beams = np.arange(a.shape[0], dtype=np.int64)
        else:
            self.contact_beams = np.asarray(list(x), np.int64) - 1


@dataclass
class RigidInteraction:
    master: object
    slave: BeamElementSurface
    properties: InteractionProperties


@dataclass
class SimulationParams:
    """SimulationParams (def_params.jl:1-35) plus the linear-solver knobs of this implementation."""
    alpha: float
    beta: float
    gamma: float
    verbose: bool = False
    record_timings: bool = False
    output_dir: str = ""
    initial_timestep: float = 1e-2
    min_timestep: float = 1e-10
    max_timestep: float = 1e-2
    output_timestep: float = 1e-4
    simulation_end_time: float = 1e-2
    accelerate_after_success_it: int = 4
    stop_on_energy_threshold: bool = False
    energy_threshold: float = 0.0
    tcompt_max: float = 1800.0
    stop_long_simulation: bool = False
    tolerance_residual: float = 1e-5
    tolerance_displacement: float = 1e-5
    max_iterations: int = 20
    nG_beams: int = 3
    wG_beams: tuple = (5 / 9, 8 / 9, 5 / 9)
    zG_beams: tuple = (-math.sqrt(3 / 5), 0.0, math.sqrt(3 / 5))
    # linear solver (replaces PARDISO)
    precision: str = "fp64"          # "fp64" | "mixed"
    krylov_restart: int = 64
    krylov_max_iter: int = 4000
    linear_tol: float = 1e-10
    inner_tol: float = 1e-4
    max_refinements: int = 60
    threads_per_sim: int = 0
    timing: bool = False             # per-phase CUDA-event timing inside each step
    preconditioner: str = "band"     # "band" (FP32 band LU, RCM order) | "block_jacobi"
    refactor_its: int = 16           # reuse the band LU until a solve needs more GMRES iterations (0: always refactor)
    refactor_policy: str = "threshold"  # "threshold" (refactor_its only) | "cost" (excess iterations vs LU cost)
    refactor_cost: float = 0.2       # "cost": GMRES iterations one band LU is worth per DOF of half bandwidth
    band_lu: str = "fp32"            # "fp32" (CUDA cores) | "tensor" (trailing updates on the tensor cores)
    stage_band: int = 1              # 1: stream band blocks into shared memory with bulk async copies; 0: off;
                                     # 2: test of the bounded wait (the first block's wait runs out)
    warm_start: str = "off"          # "off": HHT predictor; "learned": per-node MLP start (set_warm_start);
                                     # "learned_x0": HHT predictor with the MLP increment as its GMRES initial guess
    use_graph: bool = True           # replay each Newton iteration from a CUDA graph
    autotune: bool = True            # run_simulations: pick kernel block sizes after the first step
    forcing: str = "fixed"           # "fixed": every solve to linear_tol; "ew": inexact Newton
                                     # (Eisenstat-Walker forcing terms between linear_tol and forcing_max)
    forcing_max: float = 1e-2

    def to_c(self) -> _lib.EbParams:
        p = _lib.default_params()
        p.alpha, p.beta, p.gamma = self.alpha, self.beta, self.gamma
        p.tolerance_residual, p.tolerance_displacement = self.tolerance_residual, self.tolerance_displacement
        p.max_iterations = int(self.max_iterations)
        for i in range(3):
            p.gauss_w[i] = self.wG_beams[i]
            p.gauss_z[i] = self.zG_beams[i]
        p.precision = _lib.EB_PREC_MIXED if self.precision == "mixed" else _lib.EB_PREC_FP64
        p.krylov_restart = int(self.krylov_restart)
        p.krylov_max_iter = int(self.krylov_max_iter)
        p.linear_tol = float(self.linear_tol)
        p.inner_tol = float(self.inner_tol)
        p.max_refinements = int(self.max_refinements)
        p.threads_per_sim = int(self.threads_per_sim)
        p.timing = 1 if self.timing else 0
        p.preconditioner = 1 if self.preconditioner == "block_jacobi" else 0
        p.refactor_its = int(self.refactor_its)
        p.refactor_policy = {"threshold": 0, "cost": 1}[self.refactor_policy]
        p.refactor_cost = float(self.refactor_cost)
        p.band_lu = {"fp32": 0, "tensor": 1}[self.band_lu]
        p.stage_band = int(self.stage_band)
        modes = {"off": 0, "learned": 1, "learned_x0": 2}
        if self.warm_start not in modes:
            raise ValueError("warm_start must be 'off', 'learned' or 'learned_x0'")
        p.warm_start = modes[self.warm_start]
        p.use_graph = int(bool(self.use_graph))
        if self.forcing not in ("fixed", "ew"):
            raise ValueError("forcing must be 'fixed' or 'ew'")
        p.forcing = 1 if self.forcing == "ew" else 0
        p.forcing_max = float(self.forcing_max)
        return p


# ------------------------------------------------------------------ the batched engine

class GpuSimulations:
    """One device handle holding many independent configurations.

    Methods map one-to-one onto the C ABI: ``step`` is solve_step_dynamics!,
    ``commit``/``rollback`` are update_converged!/update_not_converged!."""

    def __init__(self, confs: Sequence[BeamsConfiguration], params: SimulationParams,
                 inters: Optional[Sequence[Optional[RigidInteraction]]] = None):
        self.L = _lib.load()
        self.confs = list(confs)
        self.params = params
        self.inters = list(inters) if inters is not None else [None] * len(self.confs)
        self._keep = []
        descs = (_lib.EbSimDesc * len(self.confs))()
        for s, (conf, inter) in enumerate(zip(self.confs, self.inters)):
            self._fill(descs[s], conf, inter)
        self.cparams = params.to_c()
        h = C.c_void_p()
        check(self.L.eb_create(C.byref(self.cparams), len(self.confs), descs, C.byref(h)), "eb_create")
        self._keep = []  # host arrays are borrowed only for the duration of eb_create
        self.h = h
        self.n = len(self.confs)
        self._stats = (_lib.EbSimStats * self.n)()

    def _k(self, a):
        self._keep.append(a)
        return a

    def _fill(self, d: _lib.EbSimDesc, conf: BeamsConfiguration, inter: Optional[RigidInteraction]):
        nd, bm = conf.nodes, conf.beams
        d.n_nodes, d.n_elem = len(nd), len(bm)
        for name in ("X0", "u", "ud", "udd", "w", "wd", "wdd"):
            setattr(d, name, ptr(self._k(f64(getattr(nd, name)))))
        d.R = ptr(self._k(f64(nd.R)))
        d.conn = ptr(self._k(i64(bm.conn)), C.c_int64)
        for name in ("E", "nu", "rho", "radius", "damping"):
            setattr(d, name, ptr(self._k(f64(getattr(bm, name)))))
        d.Re0 = ptr(self._k(f64(bm.Re0))) if bm.Re0 is not None else None
        fixed = i64(conf.bcs.fixed_dofs)
        d.n_fixed = len(fixed)
        d.fixed_dofs = ptr(self._k(fixed), C.c_int64) if len(fixed) else None
        cf = conf.loads.concentrated_force if conf.loads is not None else None
        if cf is not None and len(cf.loaded_dofs):
            ld = _dofs(cf.loaded_dofs)
            d.n_loaded = len(ld)
            d.loaded_dofs = ptr(self._k(i64(ld)), C.c_int64)
            d.fext0 = ptr(self._k(f64([cf.force_function(0.0, int(i) + 1) for i in ld])))
        if inter is not None:
            m, pr = inter.master, inter.properties
            d.kn, d.mu, d.eps_t, d.eta_n = pr.kn, pr.mu, pr.eps_t, pr.eta_n
            ce = i64(inter.slave.contact_beams)
            d.n_contact_elems = len(ce)
            d.contact_elems = ptr(self._k(ce), C.c_int64)
            if isinstance(m, SphereSurface):
                d.surface = _lib.EB_SURFACE_SPHERE
                for i in range(3):
                    d.sphere_center[i] = float(m.center[i])
                d.sphere_radius = float(m.radius)
            elif isinstance(m, PlaneSurface):
                d.surface = _lib.EB_SURFACE_PLANE
                d.plane_axis = m.axis_index
                d.plane_position = float(m.position)
            elif isinstance(m, (DiscreteSignedDistanceField, TriangulatedSurface)):
                if isinstance(m, TriangulatedSurface):
                    m = m.to_sdf()
                d.surface = _lib.EB_SURFACE_SDF
                for i in range(3):
                    d.sdf_dims[i] = m.dims[i]
                    d.sdf_origin[i] = m.origin[i]
                    d.sdf_spacing[i] = m.spacing[i]
                d.sdf_values = ptr(self._k(f64(m.values)))
                d.sdf_inside = 1 if m.inside else 0
                d.sdf_interp = 1 if getattr(m, "interpolation", "quadratic") == "trilinear" else 0
            else:
                raise NotImplementedError(f"surface {type(m).__name__} has no gap function")

    # ---- per-step inputs (update_loads!, update_boundary_conditions!)
    def set_time(self, s: int, t: float):
        conf = self.confs[s]
        cf = conf.loads.concentrated_force if conf.loads is not None else None
        if cf is not None and len(cf.loaded_dofs):
            vals = f64([cf.force_function(t, int(i) + 1) for i in _dofs(cf.loaded_dofs)])
            check(self.L.eb_set_loads(self.h, s, ptr(vals)), "eb_set_loads")
        bcs = conf.bcs
        if bcs.imposed_displacements_function is not None and len(bcs.displaced_indices):
            bcs.imposed_displacements[bcs.displaced_indices] = bcs.imposed_displacements_function(t)
            check(self.L.eb_set_imposed(self.h, s, ptr(f64(bcs.imposed_displacements))), "eb_set_imposed")

    def step(self, dt, active=None):
        dt = f64(np.broadcast_to(np.asarray(dt, float), (self.n,)))
        act = None if active is None else i32(active)
        k = np.zeros(self.n, np.int32)
        st = np.zeros(self.n, np.int32)
        check(self.L.eb_step(self.h, ptr(dt), ptr(act, C.c_int32) if act is not None else None,
                             ptr(k, C.c_int32), ptr(st, C.c_int32)), "eb_step")
        return k, st

    def commit(self, mask=None):
        m = None if mask is None else i32(mask)
        check(self.L.eb_commit(self.h, ptr(m, C.c_int32) if m is not None else None), "eb_commit")

    def rollback(self, mask=None):
        m = None if mask is None else i32(mask)
        check(self.L.eb_rollback(self.h, ptr(m, C.c_int32) if m is not None else None), "eb_rollback")

    def state(self, s: int, at_n: bool = False) -> dict:
        n = len(self.confs[s].nodes)
        out = {k: np.zeros((n, 3)) for k in ("u", "ud", "udd", "w", "wd", "wdd")}
        out["R"] = np.zeros((n, 9))
        out["dR"] = np.zeros((n, 9))
        f = self.L.eb_get_state_n if at_n else self.L.eb_get_state
        check(f(self.h, s, *(ptr(out[k]) for k in ("u", "ud", "udd", "w", "wd", "wdd", "R", "dR"))), "eb_get_state")
        return out

    def set_state(self, s: int, **fields):
        """Assigns node fields of simulation s between steps (u, ud, udd, w, wd, wdd: n x 3;
        R, dR: n x 9 column-major), to both its committed and working state (eb_set_state)."""
        names = ("u", "ud", "udd", "w", "wd", "wdd", "R", "dR")
        bad = set(fields) - set(names)
        if bad:
            raise ValueError(f"unknown node fields {sorted(bad)}")
        n = len(self.confs[s].nodes)
        arrs = {k: f64(np.asarray(v, float).reshape(n, 9 if k in ("R", "dR") else 3)) for k, v in fields.items()}
        check(self.L.eb_set_state(self.h, s, *(ptr(arrs[k]) if k in arrs else None for k in names)), "eb_set_state")

    def set_max_iterations(self, max_iterations=None):
        """Per-simulation Newton iteration caps (None: params.max_iterations for all)."""
        if max_iterations is None:
            check(self.L.eb_set_max_iterations(self.h, None), "eb_set_max_iterations")
            self.max_iterations = np.full(self.n, int(self.params.max_iterations))
            return
        m = i32(np.broadcast_to(np.asarray(max_iterations), (self.n,)))
        check(self.L.eb_set_max_iterations(self.h, m.ctypes.data_as(C.c_void_p)), "eb_set_max_iterations")
        self.max_iterations = m.astype(int)

    def set_tolerances(self, residual=None, displacement=None):
        """Per-simulation Newton tolerances (None: the params value for all simulations)."""
        r = None if residual is None else f64(np.broadcast_to(np.asarray(residual, float), (self.n,)))
        d = None if displacement is None else f64(np.broadcast_to(np.asarray(displacement, float), (self.n,)))
        check(self.L.eb_set_tolerances(self.h, ptr(r) if r is not None else None, ptr(d) if d is not None else None),
              "eb_set_tolerances")

    def forces(self, s: int) -> dict:
        N = 6 * len(self.confs[s].nodes)
        out = {k: np.zeros(N) for k in ("Tint", "Tk", "Tc")}
        check(self.L.eb_get_forces(self.h, s, ptr(out["Tint"]), ptr(out["Tk"]), ptr(out["Tc"])), "eb_get_forces")
        return out

    def loads_all(self, t_next) -> np.ndarray:
        """Loaded-dof values of every simulation at its t^{n+1} (concatenated in simulation order)."""
        vals = []
        for s, conf in enumerate(self.confs):
            cf = conf.loads.concentrated_force if conf.loads is not None else None
            if cf is not None and len(cf.loaded_dofs):
                t = float(np.broadcast_to(t_next, (self.n,))[s])
                vals += [cf.force_function(t, int(i) + 1) for i in _dofs(cf.loaded_dofs)]
        return f64(vals)

    def set_loads_all(self, values: np.ndarray):
        if len(values):
            check(self.L.eb_set_loads_all(self.h, ptr(f64(values))), "eb_set_loads_all")

    def displacements(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        total = sum(len(c.nodes) for c in self.confs)
        out = np.zeros((total, 3)) if out is None else out
        check(self.L.eb_get_displacements(self.h, ptr(out)), "eb_get_displacements")
        return out

    def timer_start(self):
        check(self.L.eb_timer_start(self.h), "eb_timer_start")

    def timer_stop(self) -> float:
        ms = C.c_double(0.0)
        check(self.L.eb_timer_stop(self.h, C.byref(ms)), "eb_timer_stop")
        return ms.value

    def timer_between(self, last: "GpuSimulations") -> float:
        """Device ms from this engine's timer_start to ``last``'s timer_stop (engines stepped
        concurrently on their own streams)."""
        ms = C.c_double(0.0)
        check(self.L.eb_timer_between(self.h, last.h, C.byref(ms)), "eb_timer_between")
        return ms.value

    def phase_times(self, reset: bool = False):
        ms = np.zeros(8)
        n = np.zeros(8, np.int64)
        check(self.L.eb_get_phase_times(self.h, ptr(ms), ptr(n, C.c_int64), 1 if reset else 0), "eb_get_phase_times")
        return dict(zip(_lib.PHASES, ms)), dict(zip(_lib.PHASES, n))

    def phase_intervals(self, phase: str, ref: Optional["GpuSimulations"] = None) -> np.ndarray:
        """(n, 2) start/end ms of every `phase` interval since this engine's timer_start, on the
        time axis of ``ref``'s timer_start (default: this engine's)."""
        k = _lib.PHASES.index(phase)
        ref = ref or self
        cnt = C.c_int64(0)
        check(self.L.eb_get_phase_intervals(self.h, ref.h, k, None, None, 0, C.byref(cnt)), "eb_get_phase_intervals")
        a, b = np.zeros(cnt.value), np.zeros(cnt.value)
        check(self.L.eb_get_phase_intervals(self.h, ref.h, k, ptr(a), ptr(b), cnt.value, C.byref(cnt)),
              "eb_get_phase_intervals")
        return np.stack([a, b], axis=1)

    def autotune(self) -> dict:
        """Picks the fastest block sizes of the element, contact and assembly kernels on the current
        state (eb_autotune); results do not depend on the choice.  Call between steps."""
        ch = np.zeros(4, np.int32)
        check(self.L.eb_autotune(self.h, ptr(ch, C.c_int32)), "eb_autotune")
        return dict(zip(("beam", "contact", "assembly_matrix", "assembly_vector"), (int(x) for x in ch)))

    def set_launch_shapes(self, beam: int, contact: int, assembly_matrix: int, assembly_vector: int):
        sh = np.array([beam, contact, assembly_matrix, assembly_vector], np.int32)
        check(self.L.eb_set_launch_shapes(self.h, ptr(sh, C.c_int32)), "eb_set_launch_shapes")

    # ---- output (src/IO/visualization_beams.jl)
    def beam_output(self, s: int, points_per_beam: int = 10) -> dict:
        """recompute_at_gausspts_beams! of simulation s's current state (visualization_beams.jl:122-162):
        points, displacement, velocity (NP x 3), strain, stress (NP), NP = n_elem * points_per_beam."""
        ne = len(self.confs[s].beams)
        NP = ne * int(points_per_beam)
        out = np.zeros(11 * NP)
        check(self.L.eb_beam_output(self.h, int(s), int(points_per_beam), ptr(out)), "eb_beam_output")
        return dict(points=out[:3 * NP].reshape(NP, 3), displacement=out[3 * NP:6 * NP].reshape(NP, 3),
                    velocity=out[6 * NP:9 * NP].reshape(NP, 3), strain=out[9 * NP:10 * NP], stress=out[10 * NP:])

    def vtk_open(self, dirs, points_per_beam: int = 10):
        """Starts asynchronous VTK output: one directory per simulation (None or "" = none)."""
        arr = (C.c_char_p * self.n)(*[(d or "").encode() for d in dirs])
        check(self.L.eb_vtk_open(self.h, arr, int(points_per_beam)), "eb_vtk_open")

    def vtk_write(self, counter, step, t, mask=None):
        """Queues beams_<counter>.vtp and beams_nodes_<counter>.vtp of the simulations in mask
        (write_VTK_beams, visualization_beams.jl:74-120); returns before the files are written."""
        c, st, tt = (np.ascontiguousarray(np.broadcast_to(x, (self.n,)), dtype=dt)
                     for x, dt in ((counter, np.int32), (step, np.int32), (t, np.float64)))
        m = None if mask is None else i32(mask)
        check(self.L.eb_vtk_write(self.h, ptr(m, C.c_int32) if m is not None else None, ptr(c, C.c_int32),
                                  ptr(st, C.c_int32), ptr(tt)), "eb_vtk_write")

    def vtk_flush(self):
        check(self.L.eb_vtk_flush(self.h), "eb_vtk_flush")

    def vtk_close(self):
        """Waits for the queued files and writes each directory's simulation.pvd."""
        check(self.L.eb_vtk_close(self.h), "eb_vtk_close")

    # ---- learned warm start
    def set_warm_start(self, model):
        """Installs a warm_start.WarmStartModel (None removes it)."""
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
        if model is None:
            check(self.L.eb_ws_set_model(self.h, None, None, None, None), "eb_ws_set_model")
            return
        P, a, b, o = f32(model.params), f32(model.in_shift), f32(model.in_scale), f32(model.out_scale)
        check(self.L.eb_ws_set_model(self.h, ptr(P, C.c_float), ptr(a, C.c_float), ptr(b, C.c_float),
                                     ptr(o, C.c_float)), "eb_ws_set_model")

    def capture(self, capacity: int, stride: int = 1):
        """Starts (capacity > 0) or stops (0) capturing training samples at each commit."""
        check(self.L.eb_ws_capture(self.h, int(capacity), int(stride)), "eb_ws_capture")

    def samples(self):
        """(raw features n x 39, raw targets n x 6) captured so far; rows of uncommitted simulations are dropped."""
        w = C.c_int64(0)
        check(self.L.eb_ws_samples(self.h, 0, 0, None, None, C.byref(w)), "eb_ws_samples")
        n = int(w.value)
        F = np.zeros((n, 39), np.float32)
        T = np.zeros((n, 6), np.float32)
        if n:
            check(self.L.eb_ws_samples(self.h, 0, n, ptr(F, C.c_float), ptr(T, C.c_float), C.byref(w)),
                  "eb_ws_samples")
        ok = np.isfinite(T).all(1) & np.isfinite(F).all(1)
        return F[ok], T[ok]

    def memory(self):
        """(device bytes held by this batch, simulations preconditioned by the band LU)."""
        b, n = C.c_int64(0), C.c_int32(0)
        check(self.L.eb_get_memory(self.h, C.byref(b), C.byref(n)), "eb_get_memory")
        return int(b.value), int(n.value)

    def stats(self):
        check(self.L.eb_get_stats(self.h, self._stats), "eb_get_stats")
        return [{f: getattr(x, f) for f, _ in _lib.EbSimStats._fields_} for x in self._stats]

    def sync_nodes(self):
        """Copies the device state back into the NodesBeams objects (uⁿ… and u…)."""
        for s, conf in enumerate(self.confs):
            nd = conf.nodes
            a = self.state(s, at_n=False)
            b = self.state(s, at_n=True)
            nd.u, nd.ud, nd.udd, nd.w, nd.wd, nd.wdd, nd.R, nd.dR = (a[k] for k in ("u", "ud", "udd", "w", "wd", "wdd", "R", "dR"))
            nd.un, nd.udn, nd.uddn, nd.wn, nd.wdn, nd.wddn, nd.Rn, nd.dRn = (b[k] for k in ("u", "ud", "udd", "w", "wd", "wdd", "R", "dR"))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.eb_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class RunResult:
    steps: List[int]
    ks: List[List[int]]
    t: List[float]
    wall_s: float
    newton_iterations: List[int] = field(default_factory=list)
    krylov_iterations: List[int] = field(default_factory=list)
    # per simulation: True when its Δt fell below min_timestep and it stopped at its last
    # converged state (the reference aborts that simulation, run_simulation.jl:61-66)
    aborted: List[bool] = field(default_factory=list)


def output_dirs(output_dir: str, n: int) -> List[str]:
    """Output directory of each simulation: output_dir itself for one simulation, else
    output_dir/sim_<index> (five digits)."""
    if n == 1:
        return [output_dir]
    return [os.path.join(output_dir, f"sim_{s:05d}") for s in range(n)]


def union_ms(intervals: Sequence[np.ndarray]) -> float:
    """Length of the union of (start, end) intervals (ms), e.g. one phase over concurrent lanes."""
    iv = np.concatenate([np.asarray(x, float).reshape(-1, 2) for x in intervals]) if len(intervals) else np.zeros((0, 2))
    if not len(iv):
        return 0.0
    iv = iv[np.argsort(iv[:, 0])]
    total, s0, e0 = 0.0, iv[0, 0], iv[0, 1]
    for s1, e1 in iv[1:]:
        if s1 > e0:
            total += e0 - s0
            s0, e0 = s1, e1
        else:
            e0 = max(e0, e1)
    return float(total + e0 - s0)


def lane_split(sizes: Sequence[int], lanes: int) -> List[List[int]]:
    """Simulation indices of each lane: dealt round-robin in decreasing size, so that every
    lane holds a similar mix of costly and cheap simulations."""
    order = sorted(range(len(sizes)), key=lambda s: (-int(sizes[s]), s))
    lanes = max(1, min(int(lanes), len(order)))
    return [order[l::lanes] for l in range(lanes)]


def _run_lanes(confs, params, inters, max_steps, on_step, points_per_beam, dirs, lanes) -> RunResult:
    """run_simulations over concurrent lanes: one engine per lane, each stepped by its own
    host thread on its own stream (the library releases the interpreter during its calls)."""
    import threading
    S = len(confs)
    inters = list(inters) if inters is not None else [None] * S
    parts = lane_split([len(c.beams) for c in confs], lanes)
    if params.output_dir and dirs is None:
        dirs = output_dirs(params.output_dir, S)
    device = _lib.current_device()
    results: List[Optional[RunResult]] = [None] * len(parts)
    errors: List[BaseException] = []

    def lane(l, idx):
        try:
            _lib.set_device(device)
            results[l] = run_simulations([confs[i] for i in idx], params, [inters[i] for i in idx], max_steps,
                                         on_step=on_step, points_per_beam=points_per_beam,
                                         dirs=[dirs[i] for i in idx] if dirs is not None else None)
        except BaseException as e:  # re-raised on the calling thread
            errors.append(e)

    t0 = time.perf_counter()
    threads = [threading.Thread(target=lane, args=(l, idx)) for l, idx in enumerate(parts)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    if errors:
        raise errors[0]
    merged = RunResult(steps=[0] * S, ks=[[] for _ in range(S)], t=[0.0] * S, wall_s=time.perf_counter() - t0,
                       newton_iterations=[0] * S, krylov_iterations=[0] * S, aborted=[False] * S)
    for idx, r in zip(parts, results):
        for j, i in enumerate(idx):
            merged.steps[i], merged.ks[i], merged.t[i] = r.steps[j], r.ks[j], r.t[j]
            merged.newton_iterations[i], merged.krylov_iterations[i] = r.newton_iterations[j], r.krylov_iterations[j]
            merged.aborted[i] = r.aborted[j]
    return merged


def run_simulations(confs, params: SimulationParams, inters=None, max_steps: Optional[int] = None,
                    engine: Optional[GpuSimulations] = None, on_step=None, points_per_beam: int = 10,
                    lanes: int = 1, dirs: Optional[List[str]] = None) -> RunResult:
    """The time loop of run_simulation! (run_simulation.jl:38-112) for many
    configurations at once: each keeps its own t, Δt and success counter, and
    all simulations still running advance together in one batched step.

    ``lanes`` > 1 (without ``engine``) deals the simulations onto that many
    engines, each advanced by its own host thread on its own CUDA stream: a
    lane's Newton iterations do not wait for the slowest simulation of another
    lane, and one lane's kernels run on the SMs that another lane's tail leaves
    idle.  Each simulation takes the same steps as in a single batch, except
    where the cost refactorisation rule's piggybacking (a batch-level choice of
    when to refresh band factors) differs between the groupings; ``on_step``
    is then called from the lane threads with each lane's engine and indices.
    ``dirs`` overrides the per-simulation output directories.

    With params.output_dir set, VTK files are written as the reference does
    (run_simulation.jl:30-32, 86-90: the initial state, then after a converged
    step once output_timestep has passed, labelled with the step's start time),
    by the library's asynchronous writer (one directory per simulation).

    A simulation whose halved Δt falls below min_timestep is aborted on its
    own (the reference raises "Simulation aborted." for its one simulation,
    run_simulation.jl:61-66): it is rolled back to its last converged state and
    leaves the batch, the others run on unchanged, and ``RunResult.aborted``
    marks it.  A step whose norms are not finite (EB_SIM_NAN) counts as not
    converged, so it is rolled back and retried with half the Δt like any
    other failed step."""
    if lanes > 1 and engine is None and len(confs) > 1:
        return _run_lanes(confs, params, inters, max_steps, on_step, points_per_beam, dirs, lanes)
    eng = engine or GpuSimulations(confs, params, inters)
    p = params
    S = eng.n
    t = np.zeros(S)
    dt = np.full(S, float(p.initial_timestep))
    succ = np.zeros(S, int)
    step = np.ones(S, int)
    ks = [[] for _ in range(S)]
    newton = np.zeros(S, int)
    krylov = np.zeros(S, int)
    aborted = np.zeros(S, bool)
    tuned = False
    out = bool(p.output_dir)
    if out:
        eng.vtk_open(dirs if dirs is not None else output_dirs(p.output_dir, S), points_per_beam)
        counter = np.zeros(S, np.int32)
        write_t = np.zeros(S)
        eng.vtk_write(counter, step, t)
        counter += 1
    t0 = time.perf_counter()
    while True:
        running = (p.simulation_end_time - t > 1.0e-10) & ~aborted
        if max_steps is not None:
            running &= step <= max_steps
        if not running.any():
            break
        dt_used = dt.copy()
        for s in np.nonzero(running)[0]:
            eng.set_time(int(s), float(t[s] + dt_used[s]))  # update_loads! / update_boundary_conditions!
        k, _ = eng.step(dt_used, running.astype(np.int32))
        st = eng.stats()
        for s in np.nonzero(running)[0]:
            newton[s] += st[s]["newton_iterations"]
            krylov[s] += st[s]["krylov_iterations"]
        maxit = getattr(eng, "max_iterations", None)
        maxit = np.full(S, p.max_iterations) if maxit is None else np.asarray(maxit)
        failed = running & (k > maxit)                  # run_simulation.jl:55-71
        ok = running & ~failed
        if failed.any():
            dt[failed] = dt[failed] / 2
            aborted |= failed & (dt < p.min_timestep)     # :61-66, per simulation
            eng.rollback(failed.astype(np.int32))        # update_not_converged!, :69
            succ[failed] = 0
        succ[ok] += 1
        grow = ok & (succ >= p.accelerate_after_success_it) & (k <= 8)  # :79-84
        dt[grow] = np.minimum(dt[grow] * 1.5, p.max_timestep)
        succ[grow] = 0
        if out:
            t1 = t + dt_used
            due = write_t + p.output_timestep
            tol = math.sqrt(np.finfo(float).eps) * np.maximum(np.abs(t1), np.abs(due))
            w = ok & ((t1 > due) | (np.abs(t1 - due) <= tol))           # run_simulation.jl:86-90
            if w.any():
                eng.vtk_write(counter, step, t, mask=w.astype(np.int32))
                counter[w] += 1
                write_t[w] = t1[w]
        if ok.any():
            eng.commit(ok.astype(np.int32))              # update_converged!, :100
        for s in np.nonzero(ok)[0]:
            ks[s].append(int(k[s]))
        t[ok] = t[ok] + dt_used[ok]
        step[ok] += 1
        if on_step is not None:
            on_step(eng, ok, k)
        if p.autotune and not tuned and ok.any():
            eng.autotune()  # between steps: results do not depend on the block sizes it picks
            tuned = True
    if out:
        eng.vtk_close()
    wall = time.perf_counter() - t0
    eng.sync_nodes()
    return RunResult(steps=list(step - 1), ks=ks, t=list(t), wall_s=wall, newton_iterations=list(newton),
                     krylov_iterations=list(krylov), aborted=[bool(a) for a in aborted])


def run_simulation(conf: BeamsConfiguration, params: SimulationParams, inter: Optional[RigidInteraction] = None,
                   max_steps: Optional[int] = None) -> RunResult:
    """run_simulation!(conf, params, inter) (src/run_simulation.jl:1-119) on the GPU.

    Like the reference, raises when Δt falls below min_timestep (run_simulation.jl:61-66); the
    configuration's nodes then hold the last converged state."""
    res = run_simulations([conf], params, [inter], max_steps=max_steps)
    if res.aborted[0]:
        raise RuntimeError("Simulation aborted: Δt < min_timestep")
    return res
