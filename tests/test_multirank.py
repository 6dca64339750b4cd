"""The N > 1 path of bench.py on CPU: two gloo ranks, as torchrun starts them.

The wires are independent, so every rank steps its own replica of the wire batch
(weak scaling) and the ranks exchange nothing but the final timings: the job's time is
the slowest rank's, and the whole-job rate counts every rank's wire-steps.
"""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    try:
        r, w, local = bench.env()
        d = bench.dist_init(w, backend="gloo")
        ms = bench.max_over_ranks(d, times[r])
        rate = bench.job_rate(w, 32, 10, ms)
        d.barrier()
        d.destroy_process_group()
        q.put((r, w, local, ms, rate, None))
    except Exception as e:   # reported to the parent
        q.put((rank, world, rank, None, None, repr(e)))


def _run(world, times):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, world, port, times, q)) for r in range(world)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out)


def test_two_ranks_take_the_slowest_time():
    out = _run(2, [3.0, 5.5])
    for r, (rank, world, local, ms, rate, err) in enumerate(out):
        assert err is None, err
        assert (rank, world, local) == (r, 2, r)
        assert ms == 5.5   # every rank gets the job's time
        # 2 ranks x 32 wires x 10 steps in 5.5 ms
        assert abs(rate - 2 * 32 * 10 / 5.5e-3) < 1e-6 * rate


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.dist_init(1) is None
    assert bench.max_over_ranks(None, 7.25) == 7.25
    assert bench.job_rate(1, 8, 4, 2.0) == 8 * 4 / 2e-3
