"""The oracle against the reference's only known-answer test,
test/test_beams.jl:113-119 (right-angle frame, tip u_z, atol 1e-2)."""
import os

import numpy as np
import pytest

import bridge


def _frame(O, scenes, T):
    conf, p, inter = scenes.frame_test_beams(T=T)
    m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
    res = O.run_simulation(m)
    return m, res


def test_frame_T015(O, scenes):
    m, res = _frame(O, scenes, 0.15)
    assert res["steps"] == 1500
    assert abs(m.un[-1, 2] - (-0.0100)) <= 1e-2          # test_beams.jl:114
    assert abs(m.un[-1, 2] - (-0.010034697661826674)) <= 1e-10


def test_frame_T15(O, scenes):
    m, res = _frame(O, scenes, 1.5)
    assert abs(m.un[-1, 2] - 5.8332) <= 1e-2             # test_beams.jl:116
    assert abs(m.un[-1, 2] - 5.832078775117576) <= 1e-6


@pytest.mark.skipif(os.environ.get("EB_SLOW") != "1", reason="150 000 steps; set EB_SLOW=1")
def test_frame_T15_long(O, scenes):
    m, res = _frame(O, scenes, 15.0)
    assert abs(m.un[-1, 2] - 10.3849) <= 1e-2            # test_beams.jl:118
