"""Multi-replica path on CPU: two gloo ranks, disjoint history ranges, merged tallies.

Each rank runs its share of the histories through the oracle (standing in
for its GPU); the all_reduce merge must equal one run over all histories.
"""

import os
import socket

import numpy as np
import pytest

from opengate_gb300 import replicas as Rp


def test_history_ranges_partition():
    for n, w in ((10, 3), (1000, 7), (5, 8), (0, 2)):
        ranges = [Rp.history_range(r, w, n, first=100) for r in range(w)]
        assert ranges[0][0] == 100 and ranges[-1][1] == 100 + n
        for (a, b), (c, d) in zip(ranges, ranges[1:]):
            assert b == c and a <= b
    with pytest.raises(ValueError):
        Rp.history_range(2, 2, 10)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, n, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    from opengate_gb300 import workloads as W
    from oracle import oracle as O

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc = W.water_pencil(n=16)
    b, e = Rp.history_range(rank, world, n)
    edep, edep2, cnt = O.run_dose(sc, e - b, 99, first=b, batch=e - b)
    (m_edep, m_edep2), total = Rp.merge_tallies([edep, edep2], cnt["histories"])
    if rank == 0:
        q.put((m_edep, m_edep2, total))
    dist.destroy_process_group()


def test_two_rank_gloo_merge_equals_single_run():
    import multiprocessing as mp

    from opengate_gb300 import workloads as W
    from oracle import oracle as O

    O.lib(32)  # build before forking workers
    n = 6000
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    m_edep, m_edep2, total = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sc = W.water_pencil(n=16)
    # one run whose batches are exactly the two ranks' ranges
    e0, q0, c0 = O.run_dose(sc, n // 2, 99, first=0, batch=n // 2)
    e1, q1, c1 = O.run_dose(sc, n // 2, 99, first=n // 2, batch=n // 2)
    assert total == n == c0["histories"] + c1["histories"]
    np.testing.assert_array_equal(m_edep, e0 + e1)
    np.testing.assert_array_equal(m_edep2, q0 + q1)


def test_device_merge_without_process_group_is_identity():
    """merge_tallies_device leaves the images alone and returns the rank's count when
    no process group is up (a single replica)."""

    class NoImages:
        def image_device(self, which):
            raise AssertionError("no device image may be touched")

    assert Rp.merge_tallies_device(NoImages(), (0, 1), 1234) == 1234


def _gloo_device_merge(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        Rp.merge_tallies_device(object(), (0,), 10)
        q.put((rank, "no error"))
    except RuntimeError as e:
        q.put((rank, str(e)))
    dist.destroy_process_group()


def test_device_merge_refuses_gloo():
    """The device merge runs NCCL collectives on device buffers; under gloo it refuses
    (the host merge, merge_tallies, is the one for CPU process groups)."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gloo_device_merge, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all("nccl" in m for m in got.values()), got
