"""Device element kernels against the recorded oracle fixtures (tests/golden/)."""
import os

import numpy as np
import pytest

from states import rel_err

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz")


def test_beam_kernel_matches_fixture(eb):
    g = np.load(GOLD)
    out = eb.element_eval(g["beam_in"])
    for a, b in [(2, 14), (14, 26), (26, 170), (170, 314), (314, 458)]:
        assert rel_err(out[:, a:b], g["beam_out"][:, a:b]).max() <= 1e-12


def test_contact_kernel_matches_fixture(eb):
    g = np.load(GOLD)
    out, flags = eb.contact_eval(g["contact_in"], g["contact_props"], g["contact_surf"])
    ref = g["contact_out"]
    touched = np.linalg.norm(ref[:, 13:157], axis=1) > 0
    assert np.array_equal(flags.astype(bool), touched)
    for a, b in [(1, 13), (13, 157), (157, 301)]:
        assert rel_err(out[touched, a:b], ref[touched, a:b]).max() <= 1e-12
