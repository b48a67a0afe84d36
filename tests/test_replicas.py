"""The N-GPU layout of the path (replicas, no data-path collective) on CPU:
two gloo ranks each trace their own share of a ray batch with the C oracle
(standing in for their GPU) and reduce the counters as bench.py does; the
union of the shares equals one process tracing everything, and the reduced
counters are the max time and the summed work."""
import os
import socket

import numpy as np
import pytest

from conftest import load_golden


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, outdir):
    import importlib
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "oracle"), os.path.join(root, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    replicas = importlib.import_module("magrathea-pathfinder_gb300.replicas")
    import oracle
    g = load_golden("amr")
    O = oracle.Oracle(g["records"], {k: g["cosmo_" + k] for k in ("t", "a", "dadt")}, float(g["cosmo_length"]),
                      nthreads=1)
    launch = g["launch"]
    sl = replicas.shard(launch.shape[0], rank, world)
    steps, _, _ = O.propagate(launch[sl], order=2, nsteps=int(g["nsteps"]), stop="redshift",
                              stop_ref=float(g["zs"][-1]), jacobian=False)
    # a rank-dependent "elapsed time" so that the max is checkable
    t_max, work = replicas.reduce_counters(dist, 10.0 + rank, float(steps.sum()))
    np.save(os.path.join(outdir, "steps_%d.npy" % rank), steps)
    np.save(os.path.join(outdir, "red_%d.npy" % rank), np.array([t_max, work]))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_shards_cover_the_batch_and_counters_reduce(tmp_path, oracle_mod):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    g = load_golden("amr")
    O = oracle_mod.Oracle(g["records"], {k: g["cosmo_" + k] for k in ("t", "a", "dadt")}, float(g["cosmo_length"]))
    ref, _, _ = O.propagate(g["launch"], order=2, nsteps=int(g["nsteps"]), stop="redshift",
                            stop_ref=float(g["zs"][-1]), jacobian=False)
    got = np.concatenate([np.load(tmp_path / ("steps_%d.npy" % r)) for r in range(world)])
    np.testing.assert_array_equal(got, ref)
    for r in range(world):
        t_max, work = np.load(tmp_path / ("red_%d.npy" % r))
        assert t_max == 10.0 + (world - 1)
        assert work == float(ref.sum())
    del torch


def test_batch_ids_interleave_ranks():
    import importlib
    replicas = importlib.import_module("magrathea-pathfinder_gb300.replicas")
    nb, world = 7, 3
    seen = [replicas.batch_ids(k, r, world, nb) for k in range(2) for r in range(world)]
    assert seen == [0, 1, 2, 3, 4, 5]
    sl = [replicas.shard(10, r, 3) for r in range(3)]
    assert [(s.start, s.stop) for s in sl] == [(0, 4), (4, 7), (7, 10)]
