"""Host-side pieces of bench.py: workload naming, the device-memory estimator and
the resident-group planner (no GPU needed)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_workload_names_and_population():
    import bench
    wl = bench.Workload("stents1024")
    assert wl.count == 1024 and wl.kind == "stents" and wl.precision == "mixed"
    c, p, it = wl.build(0)
    assert p.tolerance_residual == bench.STENT_TOL_RES and p.krylov_restart == 32
    one = bench.Workload("stent24x60")
    c, p, it = one.build(0)
    assert len(c.beams) == 24 * 60 and one.warm == "off"
    nets = bench.Workload("nets16")
    assert nets.count == 16 and nets.warm == "off"


def test_memory_estimate_and_groups():
    import bench
    wl = bench.Workload("stents1024", count=12)
    sizes = [bench.est_bytes(wl.stats(i)) for i in range(12)]
    # a stent holds 0.1-0.8 GB (the 64-stent batch measured 17.3 GB; estimator 17.7 GB)
    assert all(0.05e9 < s < 1.5e9 for s in sizes), sizes
    groups = bench.plan_groups(wl, int(1.01 * max(sizes) * 3))
    assert sum(len(g) for g in groups) == 12 and [i for g in groups for i in g] == list(range(12))
    assert all(sum(sizes[i] for i in g) <= 1.01 * max(sizes) * 3 or len(g) == 1 for g in groups)
    assert len(bench.plan_groups(wl, 10 ** 15)) == 1


def test_reference_arm_line():
    """`bench.py --impl reference` prints one JSON line with the GPU arm's metric, unit and
    workload description, the step window it was given, a cpu_baseline describing the run and
    an e2e block without host-device copies (the arm runs the oracle on the host cores)."""
    import json
    import subprocess
    import bench
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--ref-sample", "1"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "HHT steps/s"
    assert line["steps"] == 1 and line["warmup"] == 0 and line["higher_is_better"] is True
    assert line["value"] > 0 and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "HHT steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["workload"] == bench.Workload("stents1024").describe(0, 0, 0)["workload"]
    assert line["config"]["sims"] == 1024 and line["config"]["sample"] == 1
