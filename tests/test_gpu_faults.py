"""Per-simulation failure isolation in a batch, with the faults made on the host.

SURVEY's fault cases for the batched runtime: NaN written into one
simulation's node state between steps, and one simulation whose Newton
iteration cap (max_iterations = 1) it cannot meet.  The faulty simulation is
rolled back at every attempt (EB_SIM_NAN / EB_SIM_NOT_CONVERGED), its Δt is
halved until it falls below min_timestep and it is aborted on its own
(run_simulation.jl:55-71); the other simulations of the batch end bit for
bit where an undisturbed batch ends.  No GPU fault is involved: the NaN is an
ordinary value the kernels carry, and every loop on the device is bounded.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EB_SIM_NOT_CONVERGED, EB_SIM_NAN = 1, 2


def _rings(scenes, steps=12):
    built = [scenes.ring_drop(steps=steps, height=h) for h in (2e-3, 1e-3, 4e-4)]
    p = built[0][1]
    p.tolerance_residual = 1e-5
    return [b[0] for b in built], p, [b[2] for b in built]


def _undisturbed(eb, scenes):
    confs, p, inters = _rings(scenes)
    res = eb.run_simulations(confs, p, inters)
    assert res.aborted == [False] * 3 and res.steps == [12] * 3
    return [c.nodes.un.copy() for c in confs], [c.nodes.Rn.copy() for c in confs]


def test_nan_in_one_simulation_is_isolated(eb, scenes):
    ref_u, ref_R = _undisturbed(eb, scenes)
    confs, p, inters = _rings(scenes)
    eng = eb.GpuSimulations(confs, p, inters)
    calls, status = [0], []

    def on_step(e, ok, k):
        calls[0] += 1
        if k[1] > 0:  # simulation 1 took part in this step (inactive simulations report k = 0)
            status.append(e.stats()[1]["status"])
        if calls[0] == 4:  # after four converged steps, a NaN in node 5's u_z of simulation 1
            u = e.state(1)["u"]
            u[5, 2] = np.nan
            e.set_state(1, u=u)

    res = eb.run_simulations(confs, p, inters, engine=eng, on_step=on_step)
    assert res.aborted == [False, True, False]
    assert res.steps[1] == 4                      # nothing after the NaN was committed
    assert status[:4] == [0, 0, 0, 0]
    # Δt halved from 1e-4 below min_timestep = 1e-4/64: seven rejected attempts, all NaN
    assert status[4:] == [EB_SIM_NAN] * 7
    for i in (0, 2):
        assert res.steps[i] == 12
        assert np.array_equal(confs[i].nodes.un, ref_u[i])
        assert np.array_equal(confs[i].nodes.Rn, ref_R[i])


def test_iteration_cap_in_one_simulation_is_isolated(eb, scenes):
    ref_u, ref_R = _undisturbed(eb, scenes)
    confs, p, inters = _rings(scenes)
    eng = eb.GpuSimulations(confs, p, inters)
    eng.set_max_iterations([20, 1, 20])         # simulation 1 cannot converge in one iteration
    status = []
    res = eb.run_simulations(confs, p, inters, engine=eng,
                             on_step=lambda e, ok, k: k[1] > 0 and status.append((e.stats()[1]["status"], int(k[1]))))
    assert res.aborted == [False, True, False]
    assert res.steps[1] == 0
    assert status == [(EB_SIM_NOT_CONVERGED, 2)] * 7   # k = iterations + 1 > cap, seven halvings
    for i in (0, 2):
        assert res.steps[i] == 12
        assert np.array_equal(confs[i].nodes.un, ref_u[i])
        assert np.array_equal(confs[i].nodes.Rn, ref_R[i])
    # the rolled-back simulation still holds its initial (committed) state
    assert np.all(confs[1].nodes.un == 0.0)
