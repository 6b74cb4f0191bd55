"""endobeams_gb300 — GB300-native (sm_103a) hot path of EndoBeams.jl.

Importable as ``endobeams_gb300`` (see ``load_package`` in __graft_entry__.py,
which registers this directory under that name).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import EbError, check, device_info, f64, i32, ptr
from .api import (BeamElementSurface, Beams, BeamsConfiguration, BoundaryConditions, ConcentratedForce,
                  DiscreteSignedDistanceField, Encastre, GpuSimulations, ImposedDisplacement, InteractionProperties,
                  Loads, NodesBeams, PlaneSurface, RigidInteraction, RunResult, SimulationParams, SphereSurface,
                  read_vtk_sdf, read_vtk_triangle_mesh, run_simulation, run_simulations,
                  TriangulatedSurface)

GAUSS = np.array([5 / 9, 8 / 9, 5 / 9, -np.sqrt(3 / 5), 0.0, np.sqrt(3 / 5)])


def element_eval(inp: np.ndarray, gauss: np.ndarray = GAUSS) -> np.ndarray:
    """compute_beams on the device for packed element records (n x 96 -> n x 458)."""
    inp = f64(inp).reshape(-1, 96)
    out = np.zeros((inp.shape[0], 458))
    check(_lib.load().eb_element_eval(inp.shape[0], ptr(inp), ptr(f64(gauss)), ptr(out)), "eb_element_eval")
    return out


def contact_eval(inp: np.ndarray, props, surf, values=None, gauss: np.ndarray = GAUSS):
    """compute_contact_beams on the device (n x 96 -> n x 301, plus per-element touch flags)."""
    inp = f64(inp).reshape(-1, 96)
    out = np.zeros((inp.shape[0], 301))
    flags = np.zeros(inp.shape[0], np.int32)
    vals = None if values is None else f64(values)
    check(_lib.load().eb_contact_eval(inp.shape[0], ptr(inp), ptr(f64(gauss)), ptr(f64(props)), ptr(f64(surf)),
                                      ptr(vals), ptr(out), ptr(flags, C.c_int32)), "eb_contact_eval")
    return out, flags


def fp64_peak_tflops() -> float:
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    v = C.c_double(0.0)
    check(_lib.load().eb_fp64_peak(C.byref(v)), "eb_fp64_peak")
    return v.value


__all__ = [
    "NodesBeams", "Beams", "BeamsConfiguration", "ConcentratedForce", "Loads", "Encastre", "ImposedDisplacement",
    "BoundaryConditions", "InteractionProperties", "SphereSurface", "PlaneSurface", "DiscreteSignedDistanceField",
    "BeamElementSurface", "RigidInteraction", "SimulationParams", "run_simulation", "run_simulations",
    "GpuSimulations", "RunResult", "element_eval", "contact_eval", "device_info", "read_vtk_sdf", "EbError",
    "read_vtk_triangle_mesh", "TriangulatedSurface",
]
