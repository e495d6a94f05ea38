"""The multi-GPU path of bench.py on CPU: world_size-2 gloo ranks, each tracing its own
Halton range (replicas, no collective on the data path), the max-over-ranks timer and the
host-side frame sum. The oracle stands in for each rank's GPU, so this runs here."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, outdir):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    import bench
    from hussar_gb300 import PathTracer, scenes
    from oracle import pyoracle

    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = scenes.dihedral_workload(poses=91, samples_per_pose=1)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    S = 1 << 13
    off, n = bench.replica_range(rank, S)
    ora = pyoracle.Scene(w.mesh)
    frame, tw = ora.simulate(w.rf, w.frame, w.tx[45], w.rx[45], t, n, offset=off, precision=64, threads=1)
    total = bench.sum_frames(dist, frame)
    slowest = bench.max_over_ranks(dist, float(rank + 1))
    if rank == 0:
        np.save(os.path.join(outdir, "sum.npy"), total)
        np.save(os.path.join(outdir, "max.npy"), np.array([slowest]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_equal_one_run(tmp_path, oracle_lib):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    total = np.load(tmp_path / "sum.npy")
    assert float(np.load(tmp_path / "max.npy")[0]) == float(world)
    from hussar_gb300 import PathTracer, scenes
    w = scenes.dihedral_workload(poses=91, samples_per_pose=1)
    t = PathTracer()
    t.doGuiding = False
    t.maxDepth = w.max_depth
    ref, tw = oracle_lib.Scene(w.mesh).simulate(w.rf, w.frame, w.tx[45], w.rx[45], t, world * (1 << 13),
                                                precision=64, threads=1)
    assert np.linalg.norm(ref) > 0
    assert np.linalg.norm(total - ref) / np.linalg.norm(ref) < 1e-12
