"""The multi-GPU helpers of bench.py (weak scaling: every rank simulates its own
shard of a population world times as large, balanced on element counts; the
only collectives are a barrier and a max over ranks) exercised with two gloo
ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.dist_init()
    dev = bench.DEVICE
    bench.barrier(w)
    mx = bench.allreduce_max(float(10 * (r + 1)), w)
    wl = bench.Workload("stents64", rank=r, world=w)
    shard = [tuple(sorted(v.items())) for v in wl.variants]
    q.put((r, w, mx, shard, dev))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in range(2)), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[:3] for o in out] == [(0, 2, 20.0), (1, 2, 20.0)]
    assert [o[4] for o in out] == [None, None]  # no GPU visible here: nothing is bound
    # shards: 64 stents each, disjoint, together the first 128 of the population, balanced
    sys.path.insert(0, ROOT)
    import __graft_entry__
    __graft_entry__.load_package()
    from endobeams_gb300 import scenes
    pop = [tuple(sorted(v.items())) for v in scenes.stent_variants(128, seed=2)]
    a, b = out[0][3], out[1][3]
    assert len(a) == len(b) == 64 and not set(a) & set(b) and sorted(a + b) == sorted(pop)
    elems = lambda sh: sum(dict(v)["wires"] * dict(v)["elems_per_wire"] for v in sh)
    assert abs(elems(a) - elems(b)) <= 0.02 * max(elems(a), elems(b))


def test_device_binding_per_local_rank():
    """Each rank binds its local rank's GPU among those it sees; with one device per rank
    (CUDA_VISIBLE_DEVICES set per rank by the launcher) every rank binds ordinal 0."""
    sys.path.insert(0, ROOT)
    import bench
    assert [bench.device_for_rank(r, 8) for r in range(8)] == list(range(8))
    assert [bench.device_for_rank(r, 1) for r in range(4)] == [0, 0, 0, 0]
    assert [bench.device_for_rank(r, 2) for r in range(4)] == [0, 1, 0, 1]
    assert bench.device_for_rank(3, 0) is None
