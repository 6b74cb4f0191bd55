"""Tensor cores (tcgen05): the single-tile self-test of the operand layout, MMA and
tensor-memory epilogue, and the band LU whose trailing updates run on them.

The tile test holds eb_umma_selftest against numpy: with the operands rounded to
BF16 the product must be the FP32-accumulated product of the rounded values; with
the BF16-pair split (three products) it must approach the FP32 product to ~1e-5.
The LU test runs the same stent with the FP32 and the tensor-core factorisation:
both are only GMRES preconditioners, so the Newton steps and the positions must
agree with each other and with the oracle, and the tensor-core factors (FP32-level
products) may cost at most a few more GMRES iterations."""
import ctypes as C

import numpy as np
import pytest

import bridge

pytestmark = pytest.mark.gpu


def _bf16(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16  # round to nearest even
    return r.astype(np.uint32).view(np.float32)


def _tile(eb, A, B, split):
    from endobeams_gb300 import _lib
    L = _lib.load()
    N = B.shape[0]
    D = np.zeros((128, N), np.float32)
    rc = L.eb_umma_selftest(_lib.ptr(np.ascontiguousarray(A, np.float32), C.c_float),
                            _lib.ptr(np.ascontiguousarray(B, np.float32), C.c_float), N, split,
                            _lib.ptr(D, C.c_float))
    _lib.check(rc, "eb_umma_selftest")
    return D


@pytest.mark.parametrize("N", [64, 128, 256])
def test_umma_tile_bf16(eb, N):
    rng = np.random.default_rng(N)
    A = rng.standard_normal((128, 32)).astype(np.float32)
    B = rng.standard_normal((N, 32)).astype(np.float32)
    D = _tile(eb, A, B, 0)
    ref = _bf16(A).astype(np.float64) @ _bf16(B).astype(np.float64).T
    assert np.abs(D - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("N", [128, 256])
@pytest.mark.parametrize("split,bound", [(1, 4e-5), (2, 2e-6)])
def test_umma_tile_split_bf16(eb, N, split, bound):
    """BF16 pairs (three products) reach ~1e-5 of |A||B|; three-part splits (six products, the
    band LU's arithmetic) reach FP32's level: within the bound 32 u = 1.9e-6 of an FP32 sum of
    32 products (measured ~5e-7)."""
    rng = np.random.default_rng(7 + N)
    A = (rng.standard_normal((128, 32)) * np.exp(rng.uniform(-4, 4, (128, 1)))).astype(np.float32)
    B = (rng.standard_normal((N, 32)) * np.exp(rng.uniform(-4, 4, (N, 1)))).astype(np.float32)
    D = _tile(eb, A, B, split)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    assert (np.abs(D - ref) / scale).max() <= bound


def test_tensor_core_band_lu_stent(eb, O, scenes):
    """A 16-wire stent (100 elements per wire, b ~ 200) for 6 steps: tensor-core and FP32
    factorisations reach the same steps; positions within 1e-6 of the stent size of the
    oracle's exact-LU run and within 1e-9 of each other."""
    out = {}
    for lu in ("fp32", "tensor"):
        conf, p, inter = scenes.braided_stent(wires=16, elems_per_wire=100, grid=None, steps=6)
        p.tolerance_residual = 1e-8
        p.krylov_restart = 32
        p.refactor_its = 0  # refactorise every solve: every solve uses fresh tensor-core factors
        p.band_lu = lu
        res = eb.run_simulation(conf, p, inter)
        out[lu] = (conf.nodes.un.copy(), res.krylov_iterations[0], res.ks[0])
    conf, p, inter = scenes.braided_stent(wires=16, elems_per_wire=100, grid=None, steps=6)
    p.tolerance_residual = 1e-8
    m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
    rr = O.run_simulation(m)
    assert out["fp32"][2] == out["tensor"][2] == rr["ks"]
    L = 0.02
    assert np.abs(out["tensor"][0] - m.un).max() <= 1e-6 * L
    assert np.abs(out["tensor"][0] - out["fp32"][0]).max() <= 1e-9 * L
    assert out["tensor"][1] <= 1.15 * out["fp32"][1] + 2
