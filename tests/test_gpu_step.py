"""Full HHT steps on the GPU (predictor + Newton corrector + GMRES) vs the oracle
(same algorithm with an exact sparse LU).  Position parity bar: 1e-6 of the
structure size."""
import numpy as np
import pytest

import bridge

pytestmark = pytest.mark.gpu


def _oracle_run(O, conf, params, inter, max_steps=None):
    m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(params))
    r = O.run_simulation(m, max_steps=max_steps)
    return m, r


def test_cantilever_steps(eb, O, scenes):
    conf, p, inter = scenes.cantilever(steps=40)
    p.tolerance_residual = 1e-5
    ref, rr = _oracle_run(O, conf, p, inter)
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"] == 40
    assert res.ks[0] == rr["ks"]
    err = np.abs(conf.nodes.un - ref.un).max()
    assert err <= 1e-6 * 0.1, err
    assert np.abs(conf.nodes.Rn - ref.Rn).max() <= 1e-6


def test_frame_known_answer_gpu(eb, scenes):
    """test/test_beams.jl:113-114 on the GPU: tip u_z at T = 0.15 ≈ -0.0100 (atol 1e-2)."""
    conf, p, inter = scenes.frame_test_beams(T=0.15)
    eb.run_simulation(conf, p, inter)
    assert abs(conf.nodes.un[-1, 2] - (-0.0100)) <= 1e-2
    assert abs(conf.nodes.un[-1, 2] - (-0.010034697661826674)) <= 1e-8  # oracle value


def test_ring_drop_steps(eb, O, scenes):
    conf, p, inter = scenes.ring_drop(steps=60)
    p.tolerance_residual = 1e-5
    ref, rr = _oracle_run(O, conf, p, inter)
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"]
    err = np.abs(conf.nodes.un - ref.un).max()
    assert err <= 1e-6 * 0.02, err


def test_ring_on_analytic_plane_steps(eb, O, scenes):
    """Ring resting on an analytic PlaneSurface from the first step (contact in
    every step): step counts equal, positions within 1e-6 of the ring size."""
    conf, p, inter = scenes.ring_drop(steps=60, surface="plane", height=2.2e-4)
    p.tolerance_residual = 1e-5
    ref, rr = _oracle_run(O, conf, p, inter)
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"]
    assert list(res.ks[0]) == list(rr["ks"])
    err = np.abs(conf.nodes.un - ref.un).max()
    assert err <= 1e-6 * 0.02, err


def test_batch_matches_single(eb, scenes):
    """A simulation's result does not depend on the other simulations in its batch (bitwise)."""
    p = scenes.cantilever(steps=5)[1]
    p.tolerance_residual = 1e-5
    single = scenes.cantilever(steps=5)[0]
    eb.run_simulation(single, p)
    batch = [scenes.cantilever(steps=5)[0] for _ in range(3)] + [scenes.ring_drop(steps=5)[0]]
    inters = [None, None, None, scenes.ring_drop(steps=5)[2]]
    eb.run_simulations(batch, p, inters)
    for c in batch[:3]:
        assert np.array_equal(c.nodes.un, single.nodes.un)


def test_rerun_bitwise(eb, scenes):
    outs = []
    for _ in range(2):
        conf, p, inter = scenes.ring_drop(steps=10)
        p.tolerance_residual = 1e-5
        eb.run_simulation(conf, p, inter)
        outs.append(conf.nodes.un.copy())
    assert np.array_equal(outs[0], outs[1])


def test_preconditioners_agree(eb, scenes):
    """FP32 band-LU and 6x6 block-Jacobi preconditioning converge to the same steps."""
    out = {}
    for pc in ("band", "block_jacobi"):
        conf, p, inter = scenes.ring_drop(steps=30)
        p.tolerance_residual = 1e-5
        p.preconditioner = pc
        res = eb.run_simulation(conf, p, inter)
        out[pc] = (conf.nodes.un.copy(), res.krylov_iterations[0], res.newton_iterations[0])
    assert np.abs(out["band"][0] - out["block_jacobi"][0]).max() <= 1e-9 * 0.02
    assert out["band"][1] < out["block_jacobi"][1]


def test_mixed_precision_solver(eb, O, scenes):
    """FP32 Krylov + FP64 refinement reaches the same steps as the oracle's exact solve."""
    conf, p, inter = scenes.cantilever(steps=20)
    p.tolerance_residual = 1e-5
    p.precision = "mixed"
    ref, rr = _oracle_run(O, conf, p, inter)
    res = eb.run_simulation(conf, p, inter)
    assert res.steps[0] == rr["steps"]
    assert np.abs(conf.nodes.un - ref.un).max() <= 1e-6 * 0.1


def test_staged_band_solve_bitwise(eb, scenes):
    """Band blocks streamed into shared memory by bulk async copies give the same
    arithmetic as reading them from global memory: identical steps, bit for bit,
    on a net whose band spans many 32-column blocks."""
    out = {}
    for staged in (True, False):
        conf, p, inter = scenes.net_on_sphere(24, steps=8, sdf=scenes.sphere_sdf(n=48, h=0.8e-3))
        p.tolerance_residual = 1e-5
        p.stage_band = staged
        res = eb.run_simulation(conf, p, inter)
        assert res.steps[0] == 8
        out[staged] = (conf.nodes.un.copy(), res.krylov_iterations[0])
    assert np.array_equal(out[True][0], out[False][0])
    assert out[True][1] == out[False][1]


def test_bulk_copy_wait_timeout_is_reported(eb, scenes):
    """The shared-memory staging waits on mbarriers with an iteration limit.  With
    stage_band = 2 the first block's wait expects bytes that no copy delivers: the
    wait runs out, the step reports EB_SIM_WAIT_TIMEOUT as "not converged", the
    context stays usable, and the next steps (staging switched off) converge."""
    from endobeams_gb300 import _lib
    conf, p, inter = scenes.net_on_sphere(24, steps=8, sdf=scenes.sphere_sdf(n=48, h=0.8e-3))
    p.tolerance_residual = 1e-5
    p.stage_band = 2
    eng = eb.GpuSimulations([conf], p, [inter])
    dt = np.full(1, p.initial_timestep)
    k, status = eng.step(dt)
    assert status[0] == 4 and k[0] > p.max_iterations
    eng.rollback(np.ones(1, np.int32))
    for _ in range(3):
        k, status = eng.step(dt)
        assert status[0] == 0 and k[0] <= p.max_iterations
        eng.commit(np.ones(1, np.int32))
    eng.close()


def test_stent_steps_match_oracle(eb, O, scenes):
    """A small braided stent released into its cylinder (SDF contact, mixed
    precision, tolerance 1e-8): the same Newton iteration counts as the oracle's
    exact-LU path and positions within 1e-6 of the stent size (measured ~1e-17 m)."""
    conf, p, inter = scenes.braided_stent(wires=16, elems_per_wire=60, grid=None, precision="mixed")
    p.tolerance_residual = 1e-8
    p.tolerance_displacement = 1e-8
    p.krylov_restart = 32
    ref, rr = _oracle_run(O, conf, p, inter, max_steps=6)
    res = eb.run_simulation(conf, p, inter, max_steps=6)
    assert res.ks[0] == rr["ks"]
    assert np.abs(conf.nodes.un - ref.un).max() <= 1e-6 * 8e-3


@pytest.mark.parametrize("forcing", ["fixed", "ew"])
def test_stent_inexact_newton_matches_oracle(eb, O, scenes, forcing):
    """Inexact Newton — GMRES to 1e-4 relative per Newton solve, or Eisenstat-Walker
    forcing terms in [1e-10, 1e-2] — against the oracle's exact-LU Newton: every step
    still converges to the same tolerances, so positions agree within 1e-6 of the stent
    size; Newton iteration counts may differ by one."""
    conf, p, inter = scenes.braided_stent(wires=16, elems_per_wire=60, grid=None, precision="mixed")
    p.tolerance_residual = 1e-7
    p.tolerance_displacement = 1e-8
    p.krylov_restart = 32
    ref, rr = _oracle_run(O, conf, p, inter, max_steps=6)
    if forcing == "fixed":
        p.linear_tol = 1e-4
    else:
        p.forcing, p.linear_tol, p.forcing_max = "ew", 1e-10, 1e-2
    res = eb.run_simulation(conf, p, inter, max_steps=6)
    assert res.steps[0] == rr["steps"] == 6
    assert all(abs(a - b) <= 1 for a, b in zip(res.ks[0], rr["ks"]))
    assert np.abs(conf.nodes.un - ref.un).max() <= 1e-6 * 8e-3


def test_stent_population_batch_matches_single(eb, scenes):
    """Stents of different sizes, each with its own SDF, batched in one handle give
    bit-identical results to running each alone (per-simulation CTAs, fixed-order
    reductions, no cross-simulation state)."""
    vs = [dict(wires=16, R=3.2e-3, pitch_deg=40.0, elems_per_wire=60, cyl_frac=0.9),
          dict(wires=24, R=4.1e-3, pitch_deg=50.0, elems_per_wire=40, cyl_frac=0.88)]
    mk = lambda v: scenes.stent_variant(v, tol=1e-7)
    singles = []
    for v in vs:
        c, p, it = mk(v)
        p.krylov_restart = 32
        eb.run_simulation(c, p, it, max_steps=3)
        singles.append(c.nodes.un.copy())
    built = [mk(v) for v in vs]
    p = built[0][1]
    p.krylov_restart = 32
    eb.run_simulations([b[0] for b in built], p, [b[2] for b in built], max_steps=3)
    for b, u in zip(built, singles):
        assert np.array_equal(b[0].nodes.un, u)


def test_graph_replay_matches_direct_launches(eb, scenes):
    """Newton iterations replayed from a CUDA graph give the same bits as the
    same launches issued one by one."""
    for refactor_its in (16, 0):  # 0: the band is refactorised inside every captured iteration
        out = {}
        for graph in (True, False):
            conf, p, inter = scenes.ring_drop(steps=20)
            p.tolerance_residual = 1e-5
            p.refactor_its = refactor_its
            p.use_graph = graph
            res = eb.run_simulation(conf, p, inter)
            out[graph] = (conf.nodes.un.copy(), res.ks[0])
        assert np.array_equal(out[True][0], out[False][0]) and out[True][1] == out[False][1]


def test_two_occupancy_classes_graph_matches_direct_and_single(eb, scenes):
    """A 48-wire stent (wide band: one CTA per SM) and a 16-wire stent (two per SM) in
    one handle: the GMRES launch splits into two classes on two streams.  Replayed from
    graphs (forked and joined inside the capture) or launched directly, and each stent
    alone, the trajectories are bit for bit the same."""
    def mk(wires):
        c, p, it = scenes.stent_variant(dict(wires=wires, R=4e-3, pitch_deg=45.0, elems_per_wire=80,
                                             cyl_frac=0.9), tol=1e-7)
        p.krylov_restart = 32
        p.tolerance_displacement = 1e-8
        p.linear_tol = 1e-4
        return c, p, it

    def run(wires_list, graph):
        built = [mk(w) for w in wires_list]
        p = built[0][1]
        p.use_graph = graph
        confs = [b[0] for b in built]
        res = eb.run_simulations(confs, p, [b[2] for b in built], max_steps=3)
        return [c.nodes.un.copy() for c in confs], res.ks

    both_graph = run([48, 16], True)
    both_direct = run([48, 16], False)
    alone = [run([48], True), run([16], True)]
    for s in range(2):
        assert np.array_equal(both_graph[0][s], both_direct[0][s]) and both_graph[1][s] == both_direct[1][s]
        assert np.array_equal(both_graph[0][s], alone[s][0][0]) and both_graph[1][s] == alone[s][1][0]


def test_launch_shapes_change_no_result(eb, scenes):
    """Every block size the autotuner may pick gives the same trajectory bit for bit
    (ring on the SDF plane, contact from the first step), and eb_autotune refuses to
    run between eb_step and eb_commit."""
    def run(shapes, tune=False):
        conf, p, inter = scenes.ring_drop(steps=12, height=2.2e-4)
        p.tolerance_residual = 1e-5
        p.autotune = tune
        eng = eb.GpuSimulations([conf], p, [inter])
        if shapes is not None:
            eng.set_launch_shapes(*shapes)
        res = eb.run_simulations([conf], p, [inter], engine=eng)
        u = eng.state(0)["u"]
        chosen = eng.autotune() if tune else None
        eng.close()
        return u, res.ks[0], chosen

    base, ks, _ = run(None)
    for shapes in [(64, 64, 128, 128), (256, 256, 512, 512), (128, 256, 256, 128)]:
        u, k, _ = run(shapes)
        assert k == ks and np.array_equal(u, base), shapes
    u, k, chosen = run(None, tune=True)
    assert k == ks and np.array_equal(u, base)
    assert chosen["beam"] in (64, 128, 256) and chosen["contact"] in (64, 128, 256)
    assert chosen["assembly_matrix"] in (128, 256, 512) and chosen["assembly_vector"] in (128, 256, 512)
    conf, p, inter = scenes.ring_drop(steps=12, height=2.2e-4)
    eng = eb.GpuSimulations([conf], p, [inter])
    eng.step(np.full(1, p.initial_timestep))
    with pytest.raises(eb.EbError, match="between steps"):
        eng.autotune()
    eng.commit()
    eng.autotune()
    eng.close()
