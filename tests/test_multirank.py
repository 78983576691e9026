"""The multi-GPU form of the path is replicas only: each rank generates its
own randomisations (its own seed), the only collectives are the timing
barrier and the max over ranks, and rank 0 alone prints.  These tests run
that logic as two gloo ranks on the CPU (bench.py's own helpers), and the
reference arm's rank handling (rank 0 works and prints, the others exit)."""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist

    import bench
    w, r, _local = bench.dist_setup(backend="gloo")
    res = {"world": w, "rank": r}
    bench.barrier(w)
    # the step time each rank reports is the slowest rank's
    res["max"] = bench.max_over_ranks(0.25 * (r + 1), w)
    # each rank has its own randomisations: inputs seeded by rank
    g, shifts = bench.workload_inputs(bench.SEED + 1000 * r)
    res["g_sum"] = int(g.astype(np.uint64).sum() % (1 << 61))
    # the reference arm: rank 0 runs (on a small sample) and prints one line, other ranks print nothing
    bench.CPU_SAMPLE_LOG2N = 6
    bench.REF_LOG2N = 6

    class A:
        steps, warmup, gpus = 1, 3, w

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(A)
    res["printed"] = buf.getvalue()
    dist.destroy_process_group()
    out.put(res)


def test_two_gloo_ranks_replica_logic():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    by_rank = {r["rank"]: r for r in results}
    assert set(by_rank) == {0, 1} and all(r["world"] == 2 for r in results)
    assert all(r["max"] == pytest.approx(0.5) for r in results)
    assert by_rank[0]["g_sum"] != by_rank[1]["g_sum"]
    assert by_rank[1]["printed"] == ""
    line = json.loads(by_rank[0]["printed"])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
