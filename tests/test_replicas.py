"""The N > 1 path of bench.py: independent replicas, one process per GPU, seeds apart per rank, no
collective on the data path; the job's time is the slowest rank's and its throughput counts every
rank's ICs.  Run here as world_size-2 gloo ranks on the CPU, with the oracle's IC in place of the
GPU step (what the replica path does between its barriers)."""
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as td

    import bench
    import oracle
    from mitos_gb300.perturb import load_table

    td.init_process_group("gloo", rank=rank, world_size=ws)
    ws_, rank_, _ = bench.dist_setup()
    table = load_table()
    steps = 2
    seeds = [bench.replica_seed(42, rank_) + i for i in range(steps)]
    pks = [oracle.ic_pipeline(oracle.ic_params(16, 16, 64.0, s, table, pk_bins=8))["pk_p"] for s in seeds]
    seconds = 1.0 + rank_  # rank 1 is the slow one
    slowest = bench.max_over_ranks(seconds, td)
    value = bench.job_throughput(ws_, steps, slowest)
    td.barrier()
    td.destroy_process_group()
    q.put((rank_, ws_, seeds, [p.tolist() for p in pks], slowest, value))


def test_replicas_two_ranks_gloo(table):
    import oracle
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (r0, w0, s0, pk0, t0, v0), (r1, w1, s1, pk1, t1, v1) = out
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert set(s0).isdisjoint(s1)
    # the job's time is the slowest rank's on every rank; throughput counts both ranks' ICs
    assert t0 == t1 == 2.0
    assert v0 == v1 == 2 * 2 / 2.0
    # each replica is the single-process IC of its seed: nothing crosses ranks on the data path
    for seeds, pks in ((s0, pk0), (s1, pk1)):
        for s, pk in zip(seeds, pks):
            ref = oracle.ic_pipeline(oracle.ic_params(16, 16, 64.0, s, table, pk_bins=8))["pk_p"]
            assert np.array_equal(np.array(pk), ref, equal_nan=True)
    assert not np.array_equal(np.array(pk0[0]), np.array(pk1[0]), equal_nan=True)


def test_single_process_helpers():
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.replica_seed(42, 0) == 42 and bench.replica_seed(42, 3) == 3042
    assert bench.job_throughput(4, 10, 2.0) == 20.0
