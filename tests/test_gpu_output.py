"""Output pipeline on the GPU: the reinterpolation kernel against the oracle's
recompute_at_gausspts_beams!, and the asynchronous VTK writer's files (read
back) against the kernel and the reference's output schedule
(run_simulation.jl:30-32, 86-90)."""
import os

import numpy as np
import pytest

import bridge
from vtk_read import read_pvd, read_vtp

pytestmark = pytest.mark.gpu


def _gpu_state_into_oracle(O, eng, conf, inter, p):
    m = O.OracleModel(bridge.scene_from_conf(conf, inter), bridge.params_from(p))
    st = eng.state(0)
    m.u, m.ud, m.R = st["u"].copy(), st["ud"].copy(), st["R"].copy()
    return m


@pytest.mark.parametrize("pts", [2, 10])
def test_beam_output_matches_oracle(eb, O, scenes, pts):
    """Ring on the analytic plane after 20 steps (bent, moving, in contact): positions,
    displacements and velocities within 1e-12 (normwise relative) of the oracle on the
    same state; strain = 1 - l/l0 is a difference of O(1) numbers (the ring's strain is
    ~1e-8), so it is held to 1e-14 absolute and the stress to 1e-14 E."""
    conf, p, inter = scenes.ring_drop(steps=20, surface="plane", height=2.2e-4)
    p.tolerance_residual = 1e-5
    eng = eb.GpuSimulations([conf], p, [inter])
    eb.run_simulations([conf], p, [inter], engine=eng)
    m = _gpu_state_into_oracle(O, eng, conf, inter, p)
    ref = O.OracleModel.beam_output(m, pts)
    out = eng.beam_output(0, pts)
    eng.close()
    for k in ("points", "displacement", "velocity"):
        err = np.linalg.norm(out[k] - ref[k]) / np.linalg.norm(ref[k])
        assert err <= 1e-12, f"{k}: {err:.3e}"
    assert np.abs(out["strain"] - ref["strain"]).max() <= 1e-14
    assert np.abs(out["stress"] - ref["stress"]).max() <= 1e-14 * m.E.max()


def test_vtk_files_follow_the_reference_schedule(eb, scenes, tmp_path):
    """Cantilever, 12 steps, output every step: files beams_0..12 and beams_nodes_0..12,
    simulation.pvd listing both per write; the last file holds exactly the final
    state's reinterpolation, labelled with the last step's start time and step number."""
    conf, p, inter = scenes.cantilever(steps=12)
    p.tolerance_residual = 1e-5
    p.output_dir = str(tmp_path / "out")
    p.output_timestep = p.initial_timestep / 2
    eng = eb.GpuSimulations([conf], p, [inter])
    res = eb.run_simulations([conf], p, [inter], engine=eng)
    n_steps = res.steps[0]
    last = eng.beam_output(0, 10)
    u = eng.state(0)["u"]
    eng.close()
    d = p.output_dir
    files = sorted(os.listdir(d))
    assert f"beams_{n_steps}.vtp" in files and f"beams_nodes_{n_steps}.vtp" in files
    assert f"beams_{n_steps + 1}.vtp" not in files
    coll = read_pvd(os.path.join(d, "simulation.pvd"))
    assert len(coll) == 2 * (n_steps + 1)
    assert coll[0] == (0.0, 0, "beams_0.vtp") and coll[1] == (0.0, 1, "beams_nodes_0.vtp")
    A, piece = read_vtp(os.path.join(d, f"beams_{n_steps}.vtp"))
    ne = len(conf.beams)
    assert piece["NumberOfPoints"] == 10 * ne and piece["NumberOfLines"] == ne
    assert np.array_equal(A["Points"], last["points"])
    assert np.array_equal(A["Displacement"], last["displacement"])
    assert np.array_equal(A["Velocity"], last["velocity"])
    assert np.array_equal(A["Strain"], last["strain"]) and np.array_equal(A["Stress"], last["stress"])
    assert np.array_equal(A["connectivity"], np.arange(10 * ne)) and np.array_equal(A["offsets"], 10 * np.arange(1, ne + 1))
    assert int(A["step"][0]) == n_steps
    assert A["time"][0] == coll[-1][0] and abs(A["time"][0] - (res.t[0] - p.initial_timestep)) <= 1e-12
    N, npiece = read_vtp(os.path.join(d, f"beams_nodes_{n_steps}.vtp"))
    X0 = np.asarray(conf.nodes.X0)
    assert np.array_equal(N["Displacement"], u) and np.array_equal(N["Points"], X0 + u)
    assert np.array_equal(N["connectivity"].reshape(-1, 2), conf.beams.conn)
    assert not N["In Contact"].any() and not N["Contact Force"].any() and not N["Contact Distance"].any()
    # initial file: the undeformed configuration
    I, _ = read_vtp(os.path.join(d, "beams_0.vtp"))
    assert int(I["step"][0]) == 1 and I["time"][0] == 0.0 and not I["Displacement"].any()


def test_vtk_batch_directories_and_output_interval(eb, scenes, tmp_path):
    """Two cantilevers in one handle write into sim_00000 / sim_00001; with
    output_timestep = 3 Δt a write happens every third step."""
    confs, inters = [], []
    for _ in range(2):
        c, p, it = scenes.cantilever(steps=9)
        p.tolerance_residual = 1e-5
        confs.append(c)
        inters.append(it)
    p.output_dir = str(tmp_path / "batch")
    p.output_timestep = 3 * p.initial_timestep
    eng = eb.GpuSimulations(confs, p, inters)
    res = eb.run_simulations(confs, p, inters, engine=eng)
    eng.close()
    for s in range(2):
        d = os.path.join(p.output_dir, f"sim_{s:05d}")
        coll = read_pvd(os.path.join(d, "simulation.pvd"))
        times = sorted({t for t, _, _ in coll})
        assert len(times) == 1 + res.steps[s] // 3, (times, res.steps[s])


def test_vtk_open_rejects_unwritable_directory(eb, scenes, tmp_path):
    conf, p, inter = scenes.cantilever(steps=2)
    blocker = tmp_path / "file"
    blocker.write_text("x")
    eng = eb.GpuSimulations([conf], p, [inter])
    with pytest.raises(eb.EbError, match="cannot create output directory"):
        eng.vtk_open([str(blocker / "sub")])
    eng.close()
