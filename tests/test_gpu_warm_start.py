"""Learned Newton warm start on the GPU: sample capture from the plain solver,
training with the library's own kernels, the per-simulation fallback to the
HHT predictor, and what the trained network gains over the method without it.

Plain Newton stays the arbiter: with or without the learned start every step
iterates to the same tolerances, so trajectories agree within the Newton
tolerance (checked at 1e-6 of the structure size)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(eb, mk, steps, mode, model=None, capture=0):
    conf, p, inter = mk()
    p.tolerance_residual = 1e-5
    p.warm_start = mode
    eng = eb.GpuSimulations([conf], p, [inter])
    if model is not None:
        eng.set_warm_start(model)
    if capture:
        eng.capture(capture, 1)
    dt = np.full(1, p.initial_timestep)
    ks, used, solves = [], [], 0
    for _ in range(steps):
        k, status = eng.step(dt)
        st = eng.stats()[0]
        assert k[0] <= p.max_iterations and status[0] == 0
        ks.append(int(k[0]))
        used.append(st["warm_start_used"])
        # corrector solves + the predictor's solve when the HHT predictor ran
        solves += int(k[0]) - 1 + (0 if (mode == "learned" and st["warm_start_used"]) else 1)
        eng.commit(np.ones(1, np.int32))
    out = {"ks": np.array(ks), "used": np.array(used), "solves": solves, "u": eng.state(0)["u"]}
    if capture:
        out["samples"] = eng.samples()
    eng.close()
    return out


def test_model_far_off_falls_back_every_step_bitwise(eb, scenes):
    """A network whose increments are far off is rejected at every step; the
    fallback (restore, HHT predictor, redo the first assembly) reproduces the
    plain trajectory bit for bit."""
    from endobeams_gb300 import warm_start as W
    mk = lambda: scenes.ring_drop(steps=5000)
    plain = _run(eb, mk, 15, "off")
    bad = W.WarmStartModel(W.init_params(0, out_gain=10.0), np.zeros(48, np.float32), np.ones(48, np.float32),
                           np.full(6, 1e9, np.float32))
    learned = _run(eb, mk, 15, "learned", bad)
    assert learned["used"].sum() == 0
    assert np.array_equal(plain["ks"], learned["ks"])
    assert np.array_equal(plain["u"], learned["u"])


def test_capture_train_and_measured_gain(eb, scenes):
    """Ring drop: capture 200 plain steps, train on the device, rerun with the
    learned start.  Every step converges, positions agree with the plain run
    within 1e-6 of the ring size, and the gain is reported (Newton iterations
    and linear solves per step, fraction of accepted learned starts)."""
    from endobeams_gb300 import warm_start as W
    mk = lambda: scenes.ring_drop(steps=5000)
    n = 200
    plain = _run(eb, mk, n, "off", capture=1_000_000)
    F, T = plain["samples"]
    assert len(F) == 64 * n and np.isfinite(F).all() and np.isfinite(T).all()
    model = W.train_model(F, T, epochs=150, batch=1024, lr=1e-3, seed=0)
    tl = model.info["train_loss"]
    assert tl[-1] < 0.2 * tl[0]
    learned = _run(eb, mk, n, "learned", model)
    du = float(np.abs(plain["u"] - learned["u"]).max())
    assert du <= 1e-6 * 0.02, du
    # the same network as the initial guess of the predictor's solve: same Newton iterates,
    # fewer GMRES iterations in the predictor solves
    mk5 = lambda: _tol5(scenes.ring_drop(steps=5000))
    p0 = _run_x0(eb, mk5, n, "off")
    x0 = _run_x0(eb, mk5, n, "learned_x0", model)
    # the predictor's solve ends at the same linear tolerance from another start: the Newton
    # iterates agree to that tolerance (a step whose residual lands on the Newton tolerance may
    # take one iteration more or less)
    assert int(np.sum(p0["ks"] != x0["ks"])) <= 3
    assert float(np.abs(p0["u"] - x0["u"]).max()) <= 1e-6 * 0.02
    gain = {"scene": "ring drop, 200 steps", "val_loss": model.info["val_loss"],
            "newton_per_step_plain": float(np.mean(plain["ks"] - 1)),
            "newton_per_step_learned": float(np.mean(learned["ks"] - 1)),
            "solves_per_step_plain": plain["solves"] / n, "solves_per_step_learned": learned["solves"] / n,
            "accepted_fraction": float(learned["used"].mean()), "max_du_m": du,
            "predictor_gmres_plain": int(p0["pred"].sum()), "predictor_gmres_learned_x0": int(x0["pred"].sum()),
            "gmres_plain": int(p0["krylov"]), "gmres_learned_x0": int(x0["krylov"])}
    print("warm-start gain:", json.dumps(gain))
    assert x0["pred"].sum() < p0["pred"].sum()


def test_committed_stent_model_runs_and_matches_plain(eb, scenes):
    """The committed stent model (trained on plain-solver trajectories of a
    seed-7 stent population) on an unseen small stent: every step converges and
    the trajectory matches the plain one within the Newton tolerance."""
    import os
    from endobeams_gb300 import warm_start as W
    path = os.path.join(os.path.dirname(eb.__file__), "models", "warm_start_stents.npz")
    model = W.WarmStartModel.load(path)

    def mk():
        c, p, it = scenes.braided_stent(wires=16, elems_per_wire=60, grid=None)
        p.krylov_restart = 32
        return c, p, it

    plain = _run(eb, mk, 6, "off")
    learned = _run(eb, mk, 6, "learned", model)
    assert float(np.abs(plain["u"] - learned["u"]).max()) <= 1e-6 * 8e-3


def _tol5(built):
    c, p, it = built
    p.tolerance_residual = 1e-5
    return c, p, it


def _run_x0(eb, mk, steps, mode, model=None):
    """Steps with per-step statistics: Newton iterations and the predictor solve's GMRES iterations."""
    conf, p, inter = mk()
    p.warm_start = mode
    eng = eb.GpuSimulations([conf], p, [inter])
    if model is not None:
        eng.set_warm_start(model)
    dt = np.full(1, p.initial_timestep)
    ks, pred, total = [], [], 0
    for _ in range(steps):
        k, status = eng.step(dt)
        st = eng.stats()[0]
        assert k[0] <= p.max_iterations and status[0] == 0
        ks.append(int(k[0]))
        pred.append(st["predictor_krylov_iterations"])
        total += st["krylov_iterations"]
        eng.commit(np.ones(1, np.int32))
    out = {"ks": np.array(ks), "pred": np.array(pred), "krylov": total, "u": eng.state(0)["u"]}
    eng.close()
    return out


def test_learned_initial_guess_on_held_out_stents(eb, scenes):
    """The committed stent model (trained on a seed-7 population) as the initial guess of the HHT
    predictor's GMRES solve, on stents it has not seen: the Newton iterates are the plain ones to
    the linear tolerance (same Newton counts, positions within 1e-6 of the stent size) and the
    guess, scaled by the α that minimises its residual, costs no GMRES iterations.  On these
    stiff structures it gains none either: the network's error in the axial modes, amplified by
    their stiffness, leaves α near zero (even the exact converged increment would only cut the
    predictor's initial residual to 0.13-0.3 of its right-hand side, measured with the oracle)."""
    import os
    from endobeams_gb300 import warm_start as W
    path = os.path.join(os.path.dirname(eb.__file__), "models", "warm_start_stents.npz")
    model = W.WarmStartModel.load(path)
    gains = []
    for wires, epw, R in ((16, 80, 3.5e-3), (24, 60, 4.5e-3)):
        def mk():
            c, p, it = scenes.braided_stent(wires=wires, elems_per_wire=epw, R=R, cyl_radius=0.9 * R, grid=None)
            p.krylov_restart = 32
            p.tolerance_residual = 1e-8
            p.linear_tol = 1e-4
            p.precision = "mixed"
            return c, p, it
        plain = _run_x0(eb, mk, 12, "off")
        x0 = _run_x0(eb, mk, 12, "learned_x0", model)
        assert int(np.sum(plain["ks"] != x0["ks"])) <= 1
        assert float(np.abs(plain["u"] - x0["u"]).max()) <= 1e-6 * 0.02
        gains.append((int(plain["pred"][1:].sum()), int(x0["pred"][1:].sum()), plain["krylov"], x0["krylov"]))
    print("learned initial guess (predictor GMRES its plain -> x0, all GMRES its plain -> x0):", gains)
    assert sum(g[1] for g in gains) <= sum(g[0] for g in gains)
