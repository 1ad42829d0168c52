"""The multi-GPU path is replicas only: ranks run independent samplers on
disjoint chain ids and meet only in the bench's bookkeeping (sum of
leapfrogs, max of device and wall time).  Exercised here with world_size-2
gloo process groups on the CPU, including a rank that fails before the
reduction (its peer must get an error, not hang)."""
import multiprocessing as mp
import socket

import pytest

from cmdstan_gb300.replicas import chain_id_base, reduce_job


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, fail_rank, q):
    import datetime
    import torch.distributed as dist
    try:
        dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world,
                                timeout=datetime.timedelta(seconds=20))
        if rank == fail_rank:
            q.put((rank, "failed-before-reduce"))
            raise SystemExit(3)
        out = reduce_job(100.0 * (rank + 1), 10.0 + rank, 20.0 - rank, dist, device=None)
        q.put((rank, out))
        dist.destroy_process_group()
    except SystemExit:
        raise
    except Exception as e:  # the surviving rank reports the collective's error
        q.put((rank, "error: %s" % type(e).__name__))


def _run(world, fail_rank=-1, timeout=60):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, world, port, fail_rank, q)) for r in range(world)]
    for p in ps:
        p.start()
    res = {}
    for _ in range(world):
        r, v = q.get(timeout=timeout)
        res[r] = v
    for p in ps:
        p.join(timeout=timeout)
        if p.is_alive():
            p.kill()
    return res, [p.exitcode for p in ps]


def test_chain_ids_are_disjoint_blocks():
    assert chain_id_base(0, 1024) == 1
    assert chain_id_base(1, 1024) == 1025
    ids = [set(range(chain_id_base(r, 256), chain_id_base(r, 256) + 256)) for r in range(8)]
    assert all(not (a & b) for i, a in enumerate(ids) for b in ids[i + 1:])
    with pytest.raises(ValueError):
        chain_id_base(-1, 4)


def test_single_process_is_identity():
    assert reduce_job(5, 2.5, 3.0) == (5.0, 2.5, 3.0)


def test_two_ranks_sum_leapfrogs_and_take_slowest_times():
    res, codes = _run(2)
    assert codes == [0, 0]
    for r in (0, 1):
        assert res[r] == (300.0, 11.0, 20.0)


def test_failed_rank_surfaces_as_error_on_its_peer():
    res, codes = _run(2, fail_rank=1)
    assert res[1] == "failed-before-reduce"
    assert codes[1] == 3
    assert isinstance(res[0], str) and res[0].startswith("error"), res[0]
