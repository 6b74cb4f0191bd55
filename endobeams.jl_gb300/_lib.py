"""ctypes binding of libendobeams_gb300.so (the C ABI of include/endobeams_gb300.h).

This is the same binding a Julia host would write with ``ccall``: plain
structs, pointers and sizes.  Loading the library needs no GPU; every compute
entry point needs one and fails loudly without it (there is no CPU path).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libendobeams_gb300.so")

EB_OK = 0
EB_PREC_FP64 = 0
EB_PREC_MIXED = 1
EB_SURFACE_NONE, EB_SURFACE_SPHERE, EB_SURFACE_SDF, EB_SURFACE_PLANE = 0, 1, 2, 3
SIM_STATUS = {0: "OK", 1: "NOT_CONVERGED", 2: "NAN", 3: "KRYLOV_STAGNATED"}

P_d = C.POINTER(C.c_double)
P_i64 = C.POINTER(C.c_int64)
P_i32 = C.POINTER(C.c_int32)
P_f = C.POINTER(C.c_float)


class EbParams(C.Structure):
    _fields_ = [
        ("alpha", C.c_double), ("beta", C.c_double), ("gamma", C.c_double),
        ("tolerance_residual", C.c_double), ("tolerance_displacement", C.c_double),
        ("max_iterations", C.c_int32),
        ("gauss_w", C.c_double * 3), ("gauss_z", C.c_double * 3),
        ("precision", C.c_int32), ("krylov_restart", C.c_int32), ("krylov_max_iter", C.c_int32),
        ("linear_tol", C.c_double), ("inner_tol", C.c_double),
        ("max_refinements", C.c_int32), ("threads_per_sim", C.c_int32), ("timing", C.c_int32),
        ("preconditioner", C.c_int32), ("refactor_its", C.c_int32), ("stage_band", C.c_int32),
        ("warm_start", C.c_int32), ("use_graph", C.c_int32),
        ("forcing", C.c_int32), ("forcing_max", C.c_double),
        ("refactor_policy", C.c_int32), ("band_lu", C.c_int32), ("refactor_cost", C.c_double),
    ]


class EbSimDesc(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int64), ("n_elem", C.c_int64),
        ("X0", P_d), ("u", P_d), ("ud", P_d), ("udd", P_d), ("w", P_d), ("wd", P_d), ("wdd", P_d),
        ("R", P_d), ("conn", P_i64),
        ("E", P_d), ("nu", P_d), ("rho", P_d), ("radius", P_d), ("damping", P_d), ("Re0", P_d),
        ("n_fixed", C.c_int64), ("fixed_dofs", P_i64),
        ("n_loaded", C.c_int64), ("loaded_dofs", P_i64), ("fext0", P_d),
        ("surface", C.c_int32),
        ("kn", C.c_double), ("mu", C.c_double), ("eps_t", C.c_double), ("eta_n", C.c_double),
        ("n_contact_elems", C.c_int64), ("contact_elems", P_i64),
        ("sphere_center", C.c_double * 3), ("sphere_radius", C.c_double),
        ("sdf_dims", C.c_int64 * 3), ("sdf_origin", C.c_double * 3), ("sdf_spacing", C.c_double * 3),
        ("sdf_values", P_d), ("sdf_inside", C.c_int32), ("sdf_interp", C.c_int32),
        ("plane_axis", C.c_int32), ("plane_position", C.c_double),
    ]


class EbSimStats(C.Structure):
    _fields_ = [
        ("newton_iterations", C.c_int32), ("krylov_iterations", C.c_int32), ("refinements", C.c_int32),
        ("status", C.c_int32), ("last_res_norm", C.c_double), ("last_dD_norm", C.c_double),
        ("max_linear_rel_residual", C.c_double), ("warm_start_used", C.c_int32),
        ("predictor_krylov_iterations", C.c_int32),
        ("predictor_rhs_norm", C.c_double), ("start_res_norm", C.c_double),
    ]


# every symbol include/endobeams_gb300.h declares, with its ctypes signature
SIGNATURES = {
    "eb_last_error": (C.c_char_p, []),
    "eb_default_params": (C.c_int, [C.POINTER(EbParams)]),
    "eb_create": (C.c_int, [C.POINTER(EbParams), C.c_int32, C.POINTER(EbSimDesc), C.POINTER(C.c_void_p)]),
    "eb_destroy": (C.c_int, [C.c_void_p]),
    "eb_set_loads": (C.c_int, [C.c_void_p, C.c_int32, P_d]),
    "eb_set_imposed": (C.c_int, [C.c_void_p, C.c_int32, P_d]),
    "eb_step": (C.c_int, [C.c_void_p, P_d, P_i32, P_i32, P_i32]),
    "eb_commit": (C.c_int, [C.c_void_p, P_i32]),
    "eb_rollback": (C.c_int, [C.c_void_p, P_i32]),
    "eb_get_state": (C.c_int, [C.c_void_p, C.c_int32] + [P_d] * 8),
    "eb_get_state_n": (C.c_int, [C.c_void_p, C.c_int32] + [P_d] * 8),
    "eb_set_state": (C.c_int, [C.c_void_p, C.c_int32] + [P_d] * 8),
    "eb_set_max_iterations": (C.c_int, [C.c_void_p, C.c_void_p]),
    "eb_set_tolerances": (C.c_int, [C.c_void_p, P_d, P_d]),
    "eb_get_stats": (C.c_int, [C.c_void_p, C.POINTER(EbSimStats)]),
    "eb_get_memory": (C.c_int, [C.c_void_p, P_i64, P_i32]),
    "eb_get_forces": (C.c_int, [C.c_void_p, C.c_int32, P_d, P_d, P_d]),
    "eb_element_eval": (C.c_int, [C.c_int64, P_d, P_d, P_d]),
    "eb_contact_eval": (C.c_int, [C.c_int64, P_d, P_d, P_d, P_d, P_d, P_d, P_i32]),
    "eb_device_info": (C.c_int, [P_i32, C.c_char_p, C.c_int32]),
    "eb_rcm_order": (C.c_int, [C.c_int64, P_i64, P_i32, P_i32, P_i32]),
    "eb_device_memory": (C.c_int, [P_i64, P_i64]),
    "eb_mlp_forward": (C.c_int, [P_f, P_f, C.c_int64, P_f]),
    "eb_mlp_loss_grad": (C.c_int, [P_f, P_f, P_f, C.c_int64, P_d, P_f]),
    "eb_mlp_train": (C.c_int, [P_f, P_f, P_f, C.c_int64, C.c_int32, C.c_int32, C.c_float, C.c_uint64, P_d]),
    "eb_ws_set_model": (C.c_int, [C.c_void_p, P_f, P_f, P_f, P_f]),
    "eb_ws_capture": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32]),
    "eb_ws_samples": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, P_f, P_f, P_i64]),
    "eb_set_device": (C.c_int, [C.c_int32]),
    "eb_get_device": (C.c_int, [P_i32]),
    "eb_timer_start": (C.c_int, [C.c_void_p]),
    "eb_timer_stop": (C.c_int, [C.c_void_p, P_d]),
    "eb_timer_between": (C.c_int, [C.c_void_p, C.c_void_p, P_d]),
    "eb_get_phase_intervals": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, P_d, P_d, C.c_int64, P_i64]),
    "eb_get_phase_times": (C.c_int, [C.c_void_p, P_d, P_i64, C.c_int32]),
    "eb_set_loads_all": (C.c_int, [C.c_void_p, P_d]),
    "eb_get_displacements": (C.c_int, [C.c_void_p, P_d]),
    "eb_fp64_peak": (C.c_int, [P_d]),
    "eb_umma_selftest": (C.c_int, [P_f, P_f, C.c_int32, C.c_int32, P_f]),
    "eb_beam_output": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, P_d]),
    "eb_autotune": (C.c_int, [C.c_void_p, P_i32]),
    "eb_sdf_from_mesh": (C.c_int, [C.c_int64, P_d, C.c_int64, P_i64, P_i64, P_d, P_d, P_d]),
    "eb_set_launch_shapes": (C.c_int, [C.c_void_p, P_i32]),
    "eb_vtk_open": (C.c_int, [C.c_void_p, C.POINTER(C.c_char_p), C.c_int32]),
    "eb_vtk_write": (C.c_int, [C.c_void_p, P_i32, P_i32, P_i32, P_d]),
    "eb_vtk_flush": (C.c_int, [C.c_void_p]),
    "eb_vtk_close": (C.c_int, [C.c_void_p]),
    "eb_contact_eval_noalloc": (C.c_int, [C.c_int64, C.c_void_p, P_d, P_d, P_d, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]),
}
EB_NOALLOC_SDF_MAX_COEFS = 287496
PHASES = ("predictor", "beam", "contact", "assembly", "residual", "precond", "krylov", "update")

_lib = None


class EbError(RuntimeError):
    pass


def load(path: str = LIB_PATH):
    """Loads the library (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build_lib
        build_lib.build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc: int, what: str = ""):
    if rc != EB_OK:
        msg = load().eb_last_error().decode(errors="replace")
        raise EbError(f"{what} failed ({rc}): {msg}")


def ptr(a, ctype=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def i64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int64)


def i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def device_info():
    L = load()
    n = C.c_int32(0)
    name = C.create_string_buffer(256)
    rc = L.eb_device_info(C.byref(n), name, 256)
    return (n.value, name.value.decode()) if rc == EB_OK else (0, "")


def current_device() -> int:
    """The calling thread's current CUDA device."""
    d = C.c_int32(0)
    check(load().eb_get_device(C.byref(d)), "eb_get_device")
    return int(d.value)


def set_device(device: int) -> None:
    """Makes ``device`` current for the calling thread (handles it creates or steps)."""
    check(load().eb_set_device(int(device)), "eb_set_device")


def device_memory():
    """(free, total) bytes of the current device."""
    f, t = C.c_int64(0), C.c_int64(0)
    check(load().eb_device_memory(C.byref(f), C.byref(t)), "eb_device_memory")
    return int(f.value), int(t.value)


def rcm_order(n: int, edges: np.ndarray):
    """(positions, half bandwidth) of the band preconditioner's reverse Cuthill-McKee order
    of an n-node graph given as an (m, 2) array of 0-based edges."""
    e = np.asarray(edges, np.int64).reshape(-1, 2)
    src = np.concatenate([e[:, 0], e[:, 1]])
    dst = np.concatenate([e[:, 1], e[:, 0]]).astype(np.int32)
    order = np.argsort(src, kind="stable")
    adjncy = np.ascontiguousarray(dst[order])
    xadj = np.zeros(n + 1, np.int64)
    np.add.at(xadj, src + 1, 1)
    xadj = np.cumsum(xadj)
    pos = np.zeros(n, np.int32)
    bw = C.c_int32(0)
    check(load().eb_rcm_order(n, ptr(xadj, C.c_int64), ptr(adjncy, C.c_int32), ptr(pos, C.c_int32), C.byref(bw)),
          "eb_rcm_order")
    return pos, int(bw.value)


def default_params() -> EbParams:
    p = EbParams()
    check(load().eb_default_params(C.byref(p)), "eb_default_params")
    return p
