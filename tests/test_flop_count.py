"""Algorithmic FP64 operation counts of one element evaluation, from the oracle's
restatements compiled over an operation-counting double (oracle/flop_count.cpp).

These are the per-unit figures behind the element rooflines, counted on the
restatement of the reference rather than on any GPU code: one beam element
evaluation (compute_beams.jl:1-538, exact, dynamic, three Gauss points) and one
contact element evaluation against a quadratic B-spline SDF
(compute&assemble_interactions_beams.jl:1-445), per Gauss point in and out of
contact.  The counting build must compute exactly what the oracle library
computes (same operations, same order, no contraction), which pins it to the
oracle."""
import os
import subprocess

import numpy as np
import pytest

from states import beam_states, contact_states

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ODIR = os.path.join(ROOT, "oracle")


@pytest.fixture(scope="module")
def counter(tmp_path_factory):
    d = tmp_path_factory.mktemp("flop")
    exe = str(d / "flop_count")
    src = [os.path.join(ODIR, f) for f in ("flop_count.cpp", "flop_count_beams.cpp", "flop_count_contact.cpp")]
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-o", exe] + src,
                   check=True, cwd=ODIR)
    return exe, d


def _run(counter, O, mode, inp, extra=()):
    exe, d = counter
    paths = {k: str(d / f"{mode}_{k}.bin") for k in ("in", "gauss", "out", "surf", "coef", "props")}
    np.ascontiguousarray(inp, float).tofile(paths["in"])
    np.asarray(O.GAUSS, float).tofile(paths["gauss"])
    args = [exe, mode, paths["in"], str(len(inp)), paths["gauss"], paths["out"]]
    if mode == "contact":
        surf, coef, props = extra
        np.asarray(surf, float).tofile(paths["surf"])
        np.asarray(coef if coef is not None else np.zeros(1), float).tofile(paths["coef"])
        np.asarray(props, float).tofile(paths["props"])
        args += [paths["surf"], paths["coef"], paths["props"]]
    r = subprocess.run(args, check=True, capture_output=True, text=True)
    counts = np.array([[int(x) for x in line.split()] for line in r.stdout.strip().splitlines()])
    out = np.fromfile(paths["out"]).reshape(len(inp), -1)
    return counts, out


@pytest.mark.parametrize("damping,counts", [(0.0, (12153, 14362, 164, 8, 22)),    # the stents (damping 0)
                                             (0.01, (12531, 14800, 164, 8, 22))])
def test_beam_element_operation_count(counter, O, damping, counts):
    inp = beam_states(16, seed=7, damping=(damping,))
    got, out = _run(counter, O, "beam", inp)
    assert np.array_equal(out, O.compute_beams_batch(inp))   # the counting build is the oracle
    # every generic state takes the same branches: (adds, muls, divs, sqrts, sin/cos/acos calls)
    for c in got:
        assert tuple(int(x) for x in c) == counts, c


def test_contact_element_operation_count(counter, O):
    center, Rs, rb = np.array([0.1, -0.2, 0.3]), 1.0, 0.01
    h = 0.02
    xs = np.arange(-1.2, 1.45, h)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    field = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - Rs
    surf, coef = O.surface_arrays(dict(kind="sdf", field=field, x0=tuple(center + xs[0]), h=(h, h, h)))
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    inp = contact_states(64, center, Rs, rb, seed=9)
    counts, out = _run(counter, O, "contact", inp, (surf, coef, props))
    assert np.array_equal(out, O.compute_contact_batch(inp, props, surf, coef))
    flops = counts[:, :4].sum(axis=1)
    touched = np.linalg.norm(out[:, 13:157], axis=1) > 0
    # an element with no Gauss point in contact: its frame and three SDF value lookups
    assert (flops[~touched] == CONTACT_FREE).all() and (~touched).sum() >= 1
    # each Gauss point in contact adds CONTACT_PER_POINT, plus CONTACT_BRANCH when its gap is
    # in the penalty's other regime (regularize_gap_penalty, interactions_beams_regularization.jl)
    extra = flops - CONTACT_FREE
    n_in = extra // CONTACT_PER_POINT
    k = (extra - n_in * CONTACT_PER_POINT) // CONTACT_BRANCH
    assert np.array_equal(n_in * CONTACT_PER_POINT + k * CONTACT_BRANCH, extra)
    assert ((0 <= k) & (k <= n_in) & (n_in <= 3)).all()
    assert (n_in[touched] >= 1).all() and (n_in == 3).sum() > 32


CONTACT_FREE = 6843
CONTACT_PER_POINT = 9413
CONTACT_BRANCH = 29
