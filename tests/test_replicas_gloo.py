"""The replica (multi-GPU) path of bench.py on two CPU ranks over gloo.

One sequence cannot be sharded (a frame needs the previous frame's model), so
`bench.py --gpus N` runs N independent replicas: rank r renders the sequence
of seed r, and the ranks exchange only a barrier and the maximum of their
timed regions (whole-job frames/s = N x K / max time).  This test runs those
host-side parts with world size 2: process-group set-up from the torchrun
environment, the barrier, the max over ranks, distinct per-rank sequences,
and the reference arm's rank-0-only rule.
"""
import multiprocessing as mp
import os
import socket
import sys
from types import SimpleNamespace

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    ws, r, local = bench.dist_init(SimpleNamespace(impl="ours"))
    backend = dist.get_backend()
    bench.barrier_sync(ws)
    m = bench.max_over_ranks(ws, 10.0 + 5.0 * rank)
    seeds = bench.load_synth().seeds(rank)
    ref = bench.run_reference(SimpleNamespace(warmup=1, steps=1), ws, r, local) if rank == 1 else "skipped"
    bench.barrier_sync(ws)
    dist.destroy_process_group()
    q.put((r, ws, backend, m, tuple(seeds), ref))


def test_two_replicas_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in (0, 1)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ws0, b0, m0, s0, _), (r1, ws1, b1, m1, s1, ref1) = out
    assert (r0, r1) == (0, 1) and ws0 == ws1 == 2 and b0 == b1 == "gloo"
    assert m0 == m1 == 15.0            # the slowest rank's time, on every rank
    assert s0 != s1                    # independent sequences (weak scaling)
    assert ref1 is None                # the reference arm runs on rank 0 only
