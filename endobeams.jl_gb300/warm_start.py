"""Learned Newton warm start: the per-node MLP, its training and its use in a batch.

The reference starts each Newton loop from the HHT predictor
(src/predictor.jl:1-27): a linear solve with the previous step's tangent.
Here a per-node network predicts the whole step increment instead:

    ΔD_i = Δt·Ḋ_i + ½Δt²·D̈_i + Δt²·out_scale ⊙ mlp((f_i − in_shift) / in_scale)

for the 3 translations and the 3 rotation components of node i (the kinematic
part uses the node's committed velocity and acceleration, the same vectors the
HHT predictor starts from).  The raw features f_i (EB_WS_NRAW of them) are the
node's displacement, velocity, acceleration, angular velocity and acceleration,
the signed distance and its gradient at the node, and, for its first two beam
neighbours j, u_j − u_i, u̇_j − u̇_i, φ_j and ∇φ_j.

Plain Newton stays the arbiter: every step still iterates to the same
tolerances, and a simulation whose learned start has a larger first residual
than the HHT predictor's right-hand side falls back to the predictor for that
step.  Training data come from the plain solver itself (eb_ws_capture).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from ._lib import check, ptr

NIN, NOUT, NPARAMS = 48, 6, 23558
NRAW = 39


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def mlp_forward(params, X) -> np.ndarray:
    L = _lib.load()
    X = _f32(X).reshape(-1, NIN)
    Y = np.zeros((X.shape[0], NOUT), np.float32)
    check(L.eb_mlp_forward(ptr(_f32(params), C.c_float), ptr(X, C.c_float), X.shape[0], ptr(Y, C.c_float)),
          "eb_mlp_forward")
    return Y


def mlp_loss_grad(params, X, T):
    L = _lib.load()
    X = _f32(X).reshape(-1, NIN)
    T = _f32(T).reshape(-1, NOUT)
    g = np.zeros(NPARAMS, np.float32)
    loss = C.c_double(0.0)
    check(L.eb_mlp_loss_grad(ptr(_f32(params), C.c_float), ptr(X, C.c_float), ptr(T, C.c_float), X.shape[0],
                             C.byref(loss), ptr(g, C.c_float)), "eb_mlp_loss_grad")
    return loss.value, g


def mlp_train(params, X, T, epochs: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0):
    """Adam on the device with the library's own forward/backward kernels.
    Returns (trained params, loss per epoch)."""
    L = _lib.load()
    p = _f32(params).copy()
    X = _f32(X).reshape(-1, NIN)
    T = _f32(T).reshape(-1, NOUT)
    losses = np.zeros(max(epochs, 1))
    check(L.eb_mlp_train(ptr(p, C.c_float), ptr(X, C.c_float), ptr(T, C.c_float), X.shape[0], int(epochs), int(batch),
                         float(lr), int(seed), ptr(losses)), "eb_mlp_train")
    return p, losses[:epochs]


@dataclass
class WarmStartModel:
    """Network parameters plus the feature and output normalisation."""
    params: np.ndarray                  # NPARAMS float32
    in_shift: np.ndarray                # NIN
    in_scale: np.ndarray                # NIN
    out_scale: np.ndarray               # NOUT
    info: Optional[dict] = None

    def save(self, path: str):
        np.savez(path, params=self.params, in_shift=self.in_shift, in_scale=self.in_scale, out_scale=self.out_scale,
                 info=np.asarray(repr(self.info or {})))

    @classmethod
    def load(cls, path: str) -> "WarmStartModel":
        z = np.load(path, allow_pickle=False)
        return cls(_f32(z["params"]), _f32(z["in_shift"]), _f32(z["in_scale"]), _f32(z["out_scale"]),
                   {"source": str(z["info"])} if "info" in z else None)


def normalisation(F: np.ndarray, Tr: np.ndarray):
    """Per-feature shift/scale of raw features F (n x NRAW) and per-output scale of raw targets Tr."""
    F = np.asarray(F, np.float64)
    Tr = np.asarray(Tr, np.float64)
    shift = np.zeros(NIN, np.float32)
    scale = np.ones(NIN, np.float32)
    mu = F.mean(0)
    sd = F.std(0)
    sd = np.where(sd > 0, sd, 1.0)
    shift[:NRAW] = mu
    scale[:NRAW] = sd
    out = Tr.std(0)
    out = np.where(out > 0, out, 1.0).astype(np.float32)
    return shift, scale, out


def normalise(F, Tr, shift, scale, out_scale):
    X = np.zeros((F.shape[0], NIN), np.float32)
    X[:, :NRAW] = (np.asarray(F, np.float64) - shift[:NRAW]) / scale[:NRAW]
    T = (np.asarray(Tr, np.float64) / out_scale).astype(np.float32)
    return X, T


def init_params(seed: int = 0, out_gain: float = 0.1) -> np.ndarray:
    """He-style initial parameters (output layer scaled by out_gain)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float32)
    o1, o2 = NIN * 128 + 128, NIN * 128 + 128 + 128 * 128 + 128
    p[:NIN * 128] = rng.standard_normal(NIN * 128) * np.sqrt(2.0 / NIN)
    p[o1:o1 + 128 * 128] = rng.standard_normal(128 * 128) * np.sqrt(2.0 / 128)
    p[o2:o2 + 128 * 6] = rng.standard_normal(128 * 6) * np.sqrt(1.0 / 128) * out_gain
    return p


def train_model(F, Tr, epochs: int = 30, batch: int = 8192, lr: float = 1e-3, seed: int = 0,
                hold_out: float = 0.1) -> WarmStartModel:
    """Fits the network to captured samples (raw features F, raw targets Tr) on the GPU."""
    F = np.asarray(F, np.float32)
    Tr = np.asarray(Tr, np.float32)
    shift, scale, oscale = normalisation(F, Tr)
    X, T = normalise(F, Tr, shift, scale, oscale)
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(X))
    nv = int(len(X) * hold_out)
    va, tr = idx[:nv], idx[nv:]
    p, losses = mlp_train(init_params(seed), X[tr], T[tr], epochs, batch, lr, seed)
    val = float(np.mean((mlp_forward(p, X[va]) - T[va]) ** 2)) if nv else float("nan")
    info = {"samples": int(len(X)), "epochs": int(epochs), "batch": int(batch), "lr": float(lr),
            "train_loss": [float(x) for x in losses], "val_loss": val}
    return WarmStartModel(p, shift, scale, oscale, info)
