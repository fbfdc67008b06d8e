"""Multi-process host logic of bench.py on CPU (world size 2, gloo).

The level-set path does not shard across GPUs (replicas only: every rank
runs its own copy of the workload, with no data-path collective).  What the
N > 1 launch relies on is host logic: the process-group setup from the
torchrun environment, the barrier around the timed region, the maximum of
the ranks' times, and the reference arm printing from rank 0 only.  Each
rank here is a spawned CPU process on 127.0.0.1 with every GPU hidden (so
the process group is gloo even on a machine with one GPU, where two NCCL
ranks would have to share it), and the ranks are killed if they do not
finish in time.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cpu_only():
    # before anything initialises CUDA in this (spawned) process
    os.environ["CUDA_VISIBLE_DEVICES"] = ""


def _run_ranks(target, args_of, n):
    """start n spawned ranks, collect one queue item each, always reap them"""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=target, args=args_of(r, q), daemon=True) for r in range(n)]
    for p in procs:
        p.start()
    try:
        res = [q.get(timeout=120) for _ in procs]
        for p in procs:
            p.join(timeout=60)
            assert p.exitcode == 0
        return res
    finally:
        for p in procs:
            if p.is_alive():
                p.kill()
                p.join(timeout=10)


def _rank_main(rank, world, port, out):
    _cpu_only()
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, REPO)
    import bench
    r, w = bench.dist_setup(world)
    bench.dist_barrier(w)
    t = bench.dist_max(0.5 + rank, w)          # rank times 0.5 and 1.5: the job takes 1.5
    # whole-job throughput of replicas: every rank's units over the slowest rank's time
    value = w * 1000 / t
    bench.dist_barrier(w)
    out.put((r, w, t, value))
    torch.distributed.destroy_process_group()


def test_two_replicas_barrier_and_max_time():
    port = _free_port()
    res = sorted(_run_ranks(_rank_main, lambda r, q: (r, 2, port, q), 2))
    assert [r for r, *_ in res] == [0, 1]
    for _, w, t, value in res:
        assert w == 2 and t == 1.5 and abs(value - 2000 / 1.5) < 1e-9


def _ref_rank(rank, world, out):
    _cpu_only()
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world)})
    sys.path.insert(0, REPO)
    import contextlib
    import io

    import bench

    class A:
        workload = "adjcheck"      # the reference arm's shortest answer (no adjoint in the reference)
        steps, warmup, grid, segment = 1, 0, None, None
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(A())
    out.put((rank, buf.getvalue()))


def test_reference_arm_prints_from_rank_zero_only():
    res = dict(_run_ranks(_ref_rank, lambda r, q: (r, 2, q), 2))
    assert '"impl": "reference"' in res[0] and res[1] == ""
