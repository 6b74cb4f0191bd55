"""ORACLE — test infrastructure only.

CPU FP64 restatement of EndoBeams.jl's time step (HHT-α predictor + Newton
corrector), used by ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline arm of ``bench.py`` to check the device results.  The product
library never imports this module.

The element, contact and nodal-rotation arithmetic runs in the C++ library
``oracle/_build/liboracle_eb.so`` (a literal restatement, see the .cpp
headers); this file restates the step algebra of the reference:

* sparsity pattern and 144-entry scatter maps — src/sparse_matrices.jl:6-104
* material constants and Rₑ⁰ — src/beams/def_beam.jl:74-149
* predictor / corrector / step — src/predictor.jl, src/corrector.jl,
  src/solve_step_dynamics.jl, src/utils_solver.jl, src/utils_bcs_and_loads.jl
* time loop and Δt policy — src/run_simulation.jl:38-112

The linear solve of src/linearsolvers.jl (MKL PARDISO, closed binary, not
present) is replaced by SciPy's SuperLU, an exact sparse LU like PARDISO.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_eb.so")

EPS64 = np.finfo(np.float64).eps
GAUSS = np.array([5 / 9, 8 / 9, 5 / 9, -math.sqrt(3 / 5), 0.0, math.sqrt(3 / 5)])  # def_params.jl:31-33

# packed element record layout (must match oracle/eb_oracle.hpp)
EI = dict(X1=0, X2=3, U1=6, U2=9, R1=12, R2=21, DR1=30, DR2=39, UD1=48, UD2=51, WD1=54, WD2=57,
          UDD1=60, UDD2=63, WDD1=66, WDD2=69, L0=72, RE0=73, KU=82, KT=83, KTT=86, JR=89, AR=92, DAMP=93,
          RADIUS=94, SIZE=96)
EO = dict(ES=0, EK=1, TINT=2, TK=14, K=26, M=170, C=314, SIZE=458)
CO = dict(E=0, TC=1, K=13, C=157, SIZE=301)

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle library (make, in-tree; rebuilt when a source is newer) and return its path."""
    subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int64
        D = ctypes.c_double
        L.orc_compute_beams_batch.argtypes = [I, P, P, P]
        L.orc_compute_contact_batch.argtypes = [I, P, P, P, P, P, P]
        L.orc_sdf_prefilter.argtypes = [I, I, I, P, P]
        L.orc_sdf_eval_batch.argtypes = [P, P, I, P, D, P]
        L.orc_assemble.argtypes = [I, I] + [P] * 8 + [P] * 8 + [P, P, I, P, P, P, P, P, P, P, I, P, P, D, P, P]
        L.orc_local_predictor.argtypes = [I] + [P] * 14 + [D, D, D]
        L.orc_beam_output.argtypes = [I] + [P] * 8 + [ctypes.c_int32, P]
        L.orc_local_corrector.argtypes = [I] + [P] * 14 + [D, D, D]
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


# ----------------------------------------------------------------- per-element entry points

def compute_beams_batch(inp: np.ndarray, gauss: np.ndarray = GAUSS) -> np.ndarray:
    inp = _c(inp).reshape(-1, EI["SIZE"])
    out = np.zeros((inp.shape[0], EO["SIZE"]))
    lib().orc_compute_beams_batch(inp.shape[0], _p(inp), _p(_c(gauss)), _p(out))
    return out


def compute_contact_batch(inp: np.ndarray, props, surf: np.ndarray, coef: Optional[np.ndarray],
                          gauss: np.ndarray = GAUSS) -> np.ndarray:
    inp = _c(inp).reshape(-1, EI["SIZE"])
    out = np.zeros((inp.shape[0], CO["SIZE"]))
    coef = None if coef is None else _c(coef)
    lib().orc_compute_contact_batch(inp.shape[0], _p(inp), _p(_c(gauss)), _p(_c(props)), _p(_c(surf)),
                                    _p(coef), _p(out))
    return out


def sdf_prefilter(field: np.ndarray) -> np.ndarray:
    """Quadratic B-spline coefficients of a grid given as field[k, j, i] (x fastest)."""
    field = _c(field)
    nz, ny, nx = field.shape
    coef = np.zeros((nz + 2, ny + 2, nx + 2))
    lib().orc_sdf_prefilter(nx, ny, nz, _p(field), _p(coef))
    return coef


def sdf_eval_batch(surf: np.ndarray, coef: np.ndarray, pts: np.ndarray, radius: float) -> np.ndarray:
    pts = _c(pts).reshape(-1, 3)
    out = np.zeros((pts.shape[0], 14))
    lib().orc_sdf_eval_batch(_p(_c(surf)), _p(_c(coef)), pts.shape[0], _p(pts), float(radius), _p(out))
    return out


# ----------------------------------------------------------------- model setup

def beam_constants(E, nu, rho, radius, l0):
    """BeamMaterialProperties + K̄ⁱⁿᵗ_beam (def_beam.jl:74-85, 135-149).

    Returns Kbar (n,7) = [K̄ū, K̄Θ(3), K̄ΘΘ(3)], Jr (n,3), Ar (n,)."""
    E, nu, rho, radius, l0 = (np.broadcast_to(np.asarray(x, float), np.shape(l0)) for x in (E, nu, rho, radius, l0))
    G = E / (2 * (1 + nu))
    A = np.pi * radius ** 2
    I22 = np.pi * radius ** 4 / 4
    I33 = I22
    Io = I22 + I33
    Jr = np.stack([rho * Io, rho * I22, rho * I33], axis=1)
    Ar = rho * A
    Kbar = np.stack([A * E / l0, G * Io / l0, 4 * E * I33 / l0, 4 * E * I22 / l0,
                     -G * Io / l0, 2 * E * I33 / l0, 2 * E * I22 / l0], axis=1)
    return Kbar, Jr, Ar


def get_Re0(X1: np.ndarray, X2: np.ndarray) -> np.ndarray:
    """get_Rₑ⁰ (def_beam.jl:93-116); returns (n,9) column-major."""
    out = np.zeros((X1.shape[0], 9))
    for e in range(X1.shape[0]):
        d = X2[e] - X1[e]
        l0 = np.linalg.norm(d)
        E10 = d / l0
        v = np.cross(np.array([1.0, 0.0, 0.0]), E10)
        s = np.linalg.norm(v)
        c = E10[0]
        if c < -(1 - 2 * EPS64):
            R = np.diag([-1.0, 1.0, -1.0])
        elif c > (1 - 2 * EPS64):
            R = np.eye(3)
        else:
            Sv = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
            R = np.eye(3) + Sv + ((1 - c) / s ** 2) * Sv @ Sv
        out[e] = R.flatten(order="F")
    return out


def sparsity(n_nodes: int, conn: np.ndarray, fixed_dofs: np.ndarray):
    """sparsity_beams (sparse_matrices.jl:6-77): CSC pattern, per-element
    144-entry scatter maps (column-major local index) and sparsity_free."""
    ndofs = 6 * n_nodes
    ne = conn.shape[0]
    dofs = np.concatenate([6 * conn[:, :1] + np.arange(6), 6 * conn[:, 1:2] + np.arange(6)], axis=1)  # (ne,12)
    rows = np.repeat(dofs[:, None, :], 12, axis=1)  # [e, jj, ii] -> dofs[ii]
    cols = np.repeat(dofs[:, :, None], 12, axis=2)  # [e, jj, ii] -> dofs[jj]
    keys = (cols.astype(np.int64) * ndofs + rows).reshape(ne, 144)
    uniq, inv = np.unique(keys.ravel(), return_inverse=True)
    spmap = inv.reshape(ne, 144).astype(np.int64)
    indices = (uniq % ndofs).astype(np.int64)
    colsu = uniq // ndofs
    indptr = np.zeros(ndofs + 1, dtype=np.int64)
    np.add.at(indptr, colsu + 1, 1)
    indptr = np.cumsum(indptr)
    fixed = np.zeros(ndofs, bool)
    fixed[np.asarray(fixed_dofs, dtype=np.int64)] = True
    free_nz = ~(fixed[indices] | fixed[colsu])
    sparsity_free = np.nonzero(free_nz)[0].astype(np.int64)
    return indptr, indices, spmap, sparsity_free


@dataclass
class Params:
    """SimulationParams (def_params.jl:1-35), fields used by the hot path."""
    alpha: float
    beta: float
    gamma: float
    initial_timestep: float = 1e-2
    min_timestep: float = 1e-10
    max_timestep: float = 1e-2
    simulation_end_time: float = 1e-2
    accelerate_after_success_it: int = 4
    tolerance_residual: float = 1e-5
    tolerance_displacement: float = 1e-5
    max_iterations: int = 20


@dataclass
class Scene:
    """Plain-array description of a beam configuration (0-based indices)."""
    X0: np.ndarray
    conn: np.ndarray
    E: np.ndarray
    nu: np.ndarray
    rho: np.ndarray
    radius: np.ndarray
    damping: np.ndarray
    u0: Optional[np.ndarray] = None
    ud0: Optional[np.ndarray] = None
    udd0: Optional[np.ndarray] = None
    w0: Optional[np.ndarray] = None
    wd0: Optional[np.ndarray] = None
    wdd0: Optional[np.ndarray] = None
    R0: Optional[np.ndarray] = None
    Re0: Optional[np.ndarray] = None
    fixed_dofs: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    displaced_idx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    imposed_fn: Optional[Callable[[float], float]] = None
    loaded_dofs: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    force_fn: Optional[Callable[[float, int], float]] = None  # (t, 1-based dof)
    contact_props: Optional[tuple] = None  # (kn, mu, eps_t, eta_n)
    surface: Optional[dict] = None  # {"kind": "sphere", center, radius} | {"kind": "sdf", field, x0, h, interp}
    #                                | {"kind": "plane", axis (0..2), position}
    contact_elems: Optional[np.ndarray] = None


def surface_arrays(surface: Optional[dict]):
    """Packs a surface into the [kind, cx, cy, cz, R, nx, ny, nz, x0(3), h(3)] record + coefficients
    (a plane as [2, axis, position, 0 ...])."""
    s = np.zeros(14)
    coef = None
    if surface is None:
        return s, coef
    if surface["kind"] == "sphere":
        s[0] = 0
        s[1:4] = surface["center"]
        s[4] = surface["radius"]
    elif surface["kind"] == "plane":
        s[0] = 2
        s[1] = surface["axis"]
        s[2] = surface["position"]
    else:
        field = np.asarray(surface["field"], float)
        nz, ny, nx = field.shape
        s[0] = 3 if surface.get("interp") == "trilinear" else 1
        s[5:8] = (nx, ny, nz)
        s[8:11] = surface["x0"]
        s[11:14] = surface["h"]
        if s[0] == 3:  # the samples themselves, in the padded layout (sample (i,j,k) at (i+1,j+1,k+1))
            coef = np.zeros((nz + 2, ny + 2, nx + 2))
            coef[1:-1, 1:-1, 1:-1] = field
            coef = coef.ravel()
        else:
            coef = sdf_prefilter(field)
    return s, coef


class OracleModel:
    """One simulation: configuration + SimulationState (def_structures.jl:96-103)."""

    def __init__(self, sc: Scene, params: Params):
        self.p = params
        n = sc.X0.shape[0]
        self.n = n
        self.N = 6 * n
        z3 = np.zeros((n, 3))
        self.X0 = _c(sc.X0)
        self.conn = _c(sc.conn, np.int64)
        ne = self.conn.shape[0]
        self.ne = ne
        self.l0 = np.linalg.norm(self.X0[self.conn[:, 1]] - self.X0[self.conn[:, 0]], axis=1)
        bc = lambda x: np.broadcast_to(np.asarray(x, float), (ne,)).copy()
        self.radius = bc(sc.radius)
        self.damping = bc(sc.damping)
        self.E = _c(bc(sc.E))
        self.Kbar, self.Jr, self.Ar = beam_constants(bc(sc.E), bc(sc.nu), bc(sc.rho), self.radius, self.l0)
        self.Kbar, self.Jr, self.Ar = _c(self.Kbar), _c(self.Jr), _c(self.Ar)
        self.Re0 = _c(sc.Re0) if sc.Re0 is not None else get_Re0(self.X0[self.conn[:, 0]], self.X0[self.conn[:, 1]])
        # node state at n+1 and at n (def_node_beam.jl:6-48)
        g = lambda a: _c(a) if a is not None else z3.copy()
        self.u, self.ud, self.udd = g(sc.u0), g(sc.ud0), g(sc.udd0)
        self.w, self.wd, self.wdd = g(sc.w0), g(sc.wd0), g(sc.wdd0)
        eye = np.tile(np.eye(3).flatten(order="F"), (n, 1))
        self.R = _c(sc.R0) if sc.R0 is not None else eye.copy()
        self.dR = eye.copy()
        self.commit_nodes()
        # BCs (def_bcs_and_loads.jl)
        self.fixed = np.asarray(sc.fixed_dofs, np.int64)
        fmask = np.zeros(self.N, bool)
        fmask[self.fixed] = True
        self.free = np.nonzero(~fmask)[0]
        self.displaced_idx = np.asarray(sc.displaced_idx, np.int64)
        self.imposed = np.zeros(len(self.fixed))
        self.imposed_fn = sc.imposed_fn
        self.loaded = np.asarray(sc.loaded_dofs, np.int64)
        self.force_fn = sc.force_fn
        # contact
        self.contact = sc.contact_props is not None
        if self.contact:
            self.props = _c(sc.contact_props)
            self.surf, self.coef = surface_arrays(sc.surface)
            self.celems = _c(sc.contact_elems if sc.contact_elems is not None else np.arange(ne), np.int64)
        # sparse structures (sparse_matrices.jl:80-104)
        self.indptr, self.indices, self.spmap, self.sp_free = sparsity(n, self.conn, self.fixed)
        self.nnz = len(self.indices)
        import scipy.sparse as sp
        A = sp.csc_matrix((np.arange(1, self.nnz + 1, dtype=np.float64), self.indices, self.indptr),
                          shape=(self.N, self.N))
        Af = A[self.free][:, self.free]
        Af.sort_indices()
        assert np.array_equal(Af.data.astype(np.int64) - 1, self.sp_free)
        self.free_indptr, self.free_indices = Af.indptr.copy(), Af.indices.copy()
        # Forces (def_structures.jl:10-30) and Matrices
        self.f_n = {k: np.zeros(self.N) for k in ("fext", "Tint", "Tk", "Tc")}
        if len(self.loaded) and self.force_fn is not None:
            for i in self.loaded:
                self.f_n["fext"][i] = self.force_fn(0.0, int(i) + 1)
        self.f_1 = {k: v.copy() for k, v in self.f_n.items()}
        self.m_n = {k: np.zeros(self.nnz) for k in ("K", "C", "M")}
        self.m_1 = {k: np.zeros(self.nnz) for k in ("K", "C", "M")}
        self.D, self.Dd, self.Ddd = np.zeros(self.N), np.zeros(self.N), np.zeros(self.N)
        self.dD, self.r = np.zeros(self.N), np.zeros(self.N)
        self.energies = np.zeros(3)
        self.Ktan = np.zeros(self.nnz)
        # initialize_state_simulation! (inizialization.jl:37-44): beams only, then matricesⁿ ← matricesⁿ⁺¹
        self.assemble(with_contact=False)
        for k in ("K", "C", "M"):
            self.m_n[k][:] = self.m_1[k]
        self.last_lin_err = 0.0

    # ---- output (visualization_beams.jl:122-175)
    def beam_output(self, pts: int = 10) -> dict:
        """recompute_at_gausspts_beams! of the current state: per element `pts` points;
        returns points, displacement, velocity (NP x 3), strain, stress (NP)."""
        NP = self.ne * pts
        out = np.zeros(11 * NP)
        lib().orc_beam_output(self.ne, _p(self.X0), _p(self.u), _p(self.ud), _p(self.R), _p(self.conn),
                              _p(self.l0), _p(self.Re0), _p(self.E), int(pts), _p(out))
        return dict(points=out[:3 * NP].reshape(NP, 3), displacement=out[3 * NP:6 * NP].reshape(NP, 3),
                    velocity=out[6 * NP:9 * NP].reshape(NP, 3), strain=out[9 * NP:10 * NP],
                    stress=out[10 * NP:])

    def node_output(self) -> dict:
        """recompute_at_nodes_beams! (visualization_beams.jl:165-175): positions and displacements;
        the reference never updates the nodes' contact fields, so they stay zero."""
        return dict(points=self.X0 + self.u, displacement=self.u.copy())

    # ---- node state commits (utils_solver.jl:252-305)
    def commit_nodes(self):
        self.un, self.udn, self.uddn = self.u.copy(), self.ud.copy(), self.udd.copy()
        self.wn, self.wdn, self.wddn = self.w.copy(), self.wd.copy(), self.wdd.copy()
        self.Rn, self.dRn = self.R.copy(), self.dR.copy()

    def update_converged(self):
        self.commit_nodes()
        for k in ("Tint", "Tk", "Tc", "fext"):
            self.f_n[k][:] = self.f_1[k]
        for k in ("K", "C", "M"):
            self.m_n[k][:] = self.m_1[k]

    def update_not_converged(self):
        self.u, self.ud, self.udd = self.un.copy(), self.udn.copy(), self.uddn.copy()
        self.w, self.wd, self.wdd = self.wn.copy(), self.wdn.copy(), self.wddn.copy()
        self.R, self.dR = self.Rn.copy(), self.dRn.copy()
        for k in ("Tint", "Tk", "Tc", "fext"):
            self.f_1[k][:] = self.f_n[k]
        for k in ("K", "C", "M"):
            self.m_1[k][:] = self.m_n[k]

    # ---- assembly (assemble_beams.jl, compute&assemble…:447-501)
    def assemble(self, with_contact=True):
        L = lib()
        nc = len(self.celems) if (with_contact and self.contact) else 0
        L.orc_assemble(self.n, self.ne, _p(self.X0), _p(self.u), _p(self.ud), _p(self.udd), _p(self.wd),
                       _p(self.wdd), _p(self.R), _p(self.dR), _p(self.conn), _p(self.l0), _p(self.Re0),
                       _p(self.Kbar), _p(self.Jr), _p(self.Ar), _p(self.damping), _p(self.radius), _p(_c(GAUSS)),
                       _p(self.spmap), self.nnz, _p(self.m_1["K"]), _p(self.m_1["C"]), _p(self.m_1["M"]),
                       _p(self.f_1["Tint"]), _p(self.f_1["Tk"]), _p(self.f_1["Tc"]), _p(self.energies), nc,
                       _p(self.celems) if nc else None, _p(self.props) if nc else None, self.p.alpha,
                       _p(self.surf) if nc else None, _p(self.coef) if (nc and self.coef is not None) else None)

    # ---- loads and BCs (utils_bcs_and_loads.jl)
    def update_loads(self, t):
        if len(self.loaded) and self.force_fn is not None:
            for i in self.loaded:
                self.f_1["fext"][i] = self.force_fn(t, int(i) + 1)

    def update_bcs(self, t):
        for i in self.displaced_idx:
            self.imposed[i] = self.imposed_fn(t)

    def apply_bcs(self):  # utils_bcs_and_loads.jl:5-29
        for idx, dof in enumerate(self.fixed):
            d = self.imposed[idx] - self.D[dof]
            self.dD[dof] = d
            lo, hi = self.indptr[dof], self.indptr[dof + 1]
            self.r[self.indices[lo:hi]] -= d * self.Ktan[lo:hi]

    def solve_free(self):  # utils_solver.jl:94-120
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        r_free = self.r[self.free]
        A = sp.csc_matrix((self.Ktan[self.sp_free], self.free_indices, self.free_indptr),
                          shape=(len(self.free), len(self.free)))
        x = spla.splu(A).solve(r_free)
        self.dD[self.free] = x
        return r_free, x

    # ---- predictor (predictor.jl:1-27)
    def predictor(self, dt):
        a, b, g = self.p.alpha, self.p.beta, self.p.gamma
        self.dD[:] = 0
        D = self.D.reshape(self.n, 6)
        Dd = self.Dd.reshape(self.n, 6)
        Ddd = self.Ddd.reshape(self.n, 6)
        D[:, :3] = self.u; Dd[:, :3] = self.ud; Ddd[:, :3] = self.udd
        D[:, 3:] = 0.0; Dd[:, 3:] = self.wd; Ddd[:, 3:] = self.wdd
        self.Ktan[:] = ((1 + a) * self.m_n["K"] + (g / (b * dt)) * self.m_n["C"]) + (1 / (b * dt * dt)) * self.m_n["M"]
        self.r[:] = (((1 + a) * self.f_1["fext"] - self.f_n["Tint"]) - self.f_n["Tk"]) - a * self.f_n["fext"]
        temp = (g / b) * self.Dd - ((dt / 2 * (2 * b - g)) / b) * self.Ddd
        self.r += self._spmv(self.m_n["C"], temp)
        temp = dt * self.Dd + (dt * dt / 2) * self.Ddd
        self.r += (1 / (b * dt * dt)) * self._spmv(self.m_n["M"], temp)
        self.apply_bcs()
        self.solve_free()
        # compute_global_predictor! (utils_solver.jl:157-172)
        Ddn = self.Dd.copy()
        self.D += self.dD
        self.Dd += ((g / (b * dt)) * self.dD - (g / b) * Ddn) + ((dt * (2 * b - g)) / (2 * b)) * self.Ddd
        self.Ddd += (1 / (b * dt * dt)) * ((self.dD - dt * Ddn) - (dt * dt / 2) * self.Ddd)
        lib().orc_local_predictor(self.n, _p(self.D), _p(self.Dd), _p(self.Ddd), _p(self.u), _p(self.ud),
                                  _p(self.udd), _p(self.w), _p(self.wd), _p(self.wdd), _p(self.R), _p(self.dR),
                                  _p(self.Rn), _p(self.wdn), _p(self.wddn), g, b, dt)

    def _spmv(self, nz, x):
        import scipy.sparse as sp
        A = sp.csc_matrix((nz, self.indices, self.indptr), shape=(self.N, self.N))
        return A @ x

    # ---- corrector (corrector.jl:1-59); returns k (= iterations + 1)
    def corrector(self, dt, trace=None):
        a, b, g = self.p.alpha, self.p.beta, self.p.gamma
        self.dD[:] = 0
        D = self.D.reshape(self.n, 6)
        Dd = self.Dd.reshape(self.n, 6)
        Ddd = self.Ddd.reshape(self.n, 6)
        D[:, :3] = self.u; Dd[:, :3] = self.ud; Ddd[:, :3] = self.udd
        D[:, 3:] = self.w; Dd[:, 3:] = self.wd; Ddd[:, 3:] = self.wdd
        k = 1
        res_norm = math.inf
        dD_norm = math.inf
        while (res_norm > self.p.tolerance_residual or dD_norm > self.p.tolerance_displacement) and \
                k <= self.p.max_iterations:
            self.assemble(with_contact=True)
            self.Ktan[:] = ((1 + a) * self.m_1["K"] + (g / (b * dt)) * self.m_1["C"]) + (1 / (b * dt * dt)) * self.m_1["M"]
            f1, fn = self.f_1, self.f_n
            self.r[:] = ((1 + a) * ((f1["fext"] + f1["Tc"]) - f1["Tint"]) -
                         a * ((fn["fext"] + fn["Tc"]) - fn["Tint"])) - f1["Tk"]
            self.apply_bcs()
            r_free, x = self.solve_free()
            self.D += self.dD
            self.Dd += (g / (b * dt)) * self.dD
            self.Ddd += (1 / (b * dt * dt)) * self.dD
            lib().orc_local_corrector(self.n, _p(self.D), _p(self.Dd), _p(self.Ddd), _p(self.dD), _p(self.u),
                                      _p(self.ud), _p(self.udd), _p(self.wd), _p(self.wdd), _p(self.R),
                                      _p(self.dR), _p(self.Rn), _p(self.wdn), _p(self.wddn), g, b, dt)
            # compute_norms_corrector (utils_solver.jl:126-151)
            dD_norm = float(np.linalg.norm(x))
            res_norm = float(np.linalg.norm(r_free))
            s = (f1["fext"] + f1["Tc"]) + f1["Tk"]
            f_norm = float(np.linalg.norm(s[self.free]))
            e_norm = float(np.linalg.norm(s[self.fixed])) if len(self.fixed) else 0.0
            if f_norm + e_norm > 1e-12:
                res_norm = res_norm / (f_norm + e_norm)
            if trace is not None:
                trace.append((k, res_norm, dD_norm))
            k += 1
        return k

    # ---- solve_step_dynamics! (solve_step_dynamics.jl:1-14)
    def step(self, t1, dt, trace=None):
        self.update_loads(t1)
        self.update_bcs(t1)
        self.predictor(dt)
        return self.corrector(dt, trace)

    def node_state(self):
        return dict(u=self.u.copy(), ud=self.ud.copy(), udd=self.udd.copy(), w=self.w.copy(), wd=self.wd.copy(),
                    wdd=self.wdd.copy(), R=self.R.copy(), dR=self.dR.copy())


def run_simulation(model: OracleModel, max_steps: Optional[int] = None, on_step=None, resume: Optional[dict] = None):
    """run_simulation! time loop (run_simulation.jl:38-112), without file output.

    Returns a dict with the step count, the per-step k values and the final time.
    ``resume`` (a dict returned by an earlier call on the same model, or None) continues that
    loop where it stopped — its t, Δt, success counter and step number — for ``max_steps``
    more committed steps."""
    p = model.p
    t = resume["t"] if resume else 0.0
    dt = resume["dt"] if resume else p.initial_timestep
    succ = resume["succ"] if resume else 0
    step0 = resume["steps"] if resume else 0
    step = step0 + 1
    ks = []
    while p.simulation_end_time - t > 1.0e-10:
        if max_steps is not None and step > step0 + max_steps:
            break
        t1 = t + dt
        n_it = model.step(t1, dt)
        if n_it > p.max_iterations:
            dt = dt / 2
            if dt < p.min_timestep:
                raise RuntimeError("Simulation aborted: dt < min_timestep")
            model.update_not_converged()
            succ = 0
            continue
        succ += 1
        if succ >= p.accelerate_after_success_it and n_it <= 8:
            dt = min(dt * 1.5, p.max_timestep)
            succ = 0
        model.update_converged()
        ks.append(n_it)
        if on_step is not None:
            on_step(step, t1, dt, n_it)
        t = t1
        step += 1
    return dict(steps=step - 1, ks=ks, t=t, dt=dt, succ=succ)
