"""Generates the golden fixtures of tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

The fixtures freeze the oracle's outputs (element and contact evaluations,
SDF prefilter/evaluation, short trajectories) so that later changes to the
oracle, and the same oracle built on another host (x86-64 here, aarch64 on
the GPU machine), are checked against one recorded set.  The oracle itself
is pinned to the reference's known answers (test/test_beams.jl:113-119) by
tests/test_oracle_known_answers.py.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

import __graft_entry__ as g  # noqa: E402

O = g.load_oracle()
import bridge  # noqa: E402
from states import beam_states, contact_states  # noqa: E402


def main():
    g.load_package()
    from endobeams_gb300 import scenes
    out = {}
    b1 = beam_states(16, seed=101)
    b2 = beam_states(8, seed=102, small=True)
    out["beam_in"] = np.concatenate([b1, b2])
    out["beam_out"] = O.compute_beams_batch(out["beam_in"])
    center, Rs, rb = np.array([0.1, -0.2, 0.3]), 1.0, 0.01
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    surf = np.zeros(14)
    surf[1:4], surf[4] = center, Rs
    out["contact_in"] = contact_states(16, center, Rs, rb, seed=103)
    out["contact_props"] = props
    out["contact_surf"] = surf
    out["contact_out"] = O.compute_contact_batch(out["contact_in"], props, surf, None)
    rng = np.random.default_rng(104)
    field = rng.normal(size=(5, 6, 7))
    coef = O.sdf_prefilter(field)
    ssurf = np.zeros(14)
    ssurf[0] = 1
    ssurf[5:8] = (7, 6, 5)
    ssurf[8:11] = (0.1, -0.2, 0.3)
    ssurf[11:14] = (0.5, 0.4, 0.3)
    pts = np.stack([rng.uniform(0.1, 0.1 + 6 * 0.5, 32), rng.uniform(-0.2, -0.2 + 5 * 0.4, 32),
                    rng.uniform(0.3, 0.3 + 4 * 0.3, 32)], 1)
    out["sdf_field"], out["sdf_coef"], out["sdf_surf"], out["sdf_pts"] = field, coef, ssurf, pts
    out["sdf_eval"] = O.sdf_eval_batch(ssurf, coef, pts, 0.05)
    for name, fn, steps in (("cantilever", scenes.cantilever, 20), ("ring", scenes.ring_drop, 10)):
        conf, p, inter = fn(steps=steps)
        p.tolerance_residual = 1e-5
        m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
        traj = []
        O.run_simulation(m, on_step=lambda *a, _m=m, _t=traj: _t.append(_m.un.copy()))
        out[f"traj_{name}"] = np.asarray(traj)
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "oracle_golden.npz"))


if __name__ == "__main__":
    main()
