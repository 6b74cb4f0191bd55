"""The device element and contact formulas (eb_beam.cuh, eb_contact.cuh)
compiled for the host with g++ and held to the oracle on the CPU, at the
device parity bar: every output block within 1e-12 normwise relative
(contact energy 1e-9, as on the GPU).  The GPU suite checks the compiled
kernels themselves; this catches an algebra change without a GPU."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from states import beam_states, contact_states, plane_states, rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
GAUSS = np.array([5 / 9, 8 / 9, 5 / 9, -np.sqrt(3 / 5), 0.0, np.sqrt(3 / 5)])
P = ctypes.c_void_p


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    so = str(tmp_path_factory.mktemp("hostk") / "kernels_host.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-x", "c++",
                    os.path.join(HERE, "host", "kernels_host.cpp"), "-o", so], check=True)
    return ctypes.CDLL(so)


def _elements(host, inp):
    out = np.zeros((len(inp), 458))
    host.host_element_eval(ctypes.c_int64(len(inp)), inp.ctypes.data_as(P), GAUSS.ctypes.data_as(P),
                           out.ctypes.data_as(P))
    return out


def _contacts(host, inp, props, surf):
    out = np.zeros((len(inp), 301))
    host.host_contact_eval(ctypes.c_int64(len(inp)), inp.ctypes.data_as(P), GAUSS.ctypes.data_as(P),
                           props.ctypes.data_as(P), surf.ctypes.data_as(P), out.ctypes.data_as(P))
    return out


@pytest.mark.parametrize("small", [False, True])
def test_element_formulas_match_oracle(O, host, small):
    inp = beam_states(256, seed=30 + small, small=small)
    ref = O.compute_beams_batch(inp)
    out = _elements(host, inp)
    for name, a, b in [("Tint", 2, 14), ("Tk", 14, 26), ("K", 26, 170), ("M", 170, 314), ("C", 314, 458)]:
        err = rel_err(out[:, a:b], ref[:, a:b]).max()
        assert err <= 1e-12, f"{name}: {err:.3e}"


@pytest.mark.parametrize("surface", ["sphere", "plane"])
def test_contact_formulas_match_oracle(O, host, surface):
    rb = 0.01
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    surf = np.zeros(14)
    if surface == "sphere":
        center = np.array([0.1, -0.2, 0.3])
        surf[1:4], surf[4] = center, 1.0
        inp = contact_states(512, center, 1.0, rb, seed=33)
    else:
        surf[0], surf[1], surf[2] = 2, 1, 0.013
        inp = plane_states(512, 1, 0.013, rb, seed=34)
    ref = O.compute_contact_batch(inp, props, surf, None)
    out = _contacts(host, inp, props, surf)
    touched = np.linalg.norm(ref[:, 13:157], axis=1) > 0
    assert touched.sum() > 300
    assert np.array_equal(np.linalg.norm(out[:, 13:157], axis=1) > 0, touched)
    for name, a, b, tol in [("E", 0, 1, 1e-9), ("Tc", 1, 13, 1e-12), ("K", 13, 157, 1e-12), ("C", 157, 301, 1e-12)]:
        err = rel_err(out[touched, a:b], ref[touched, a:b]).max()
        assert err <= tol, f"{name}: {err:.3e}"
