"""Walker-range sharding over ranks ("replicas only": no data-path
collective), run as two gloo processes on the CPU.

Each rank walks its own walker range (walker_offset) of the same acquisition
with the oracle; summing the ranks' FP64 sums (one all_reduce, only for the
check) must give the single-process walk, because a walker's Philox stream is
keyed by its global id.  The bench's max-over-ranks timing helper is checked in
the same processes."""
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _case():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases as K
    lat, cyl = K.hex_cylinders(kappa=2e-5)
    return lat, cyl, K.seq_mix(), K


def _rank(rank, world, port, n, steps, q):
    try:
        sys.path.insert(0, ROOT)
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                          WORLD_SIZE=str(world))
        import torch
        import torch.distributed as dist
        dist.init_process_group("gloo", rank=rank, world_size=world)
        from oracle import oracle as O
        import bench
        lat, cyl, seqs, K = _case()
        per = n // world
        # flags 3: T2 relaxation + permeable membranes
        p = K.params(per, steps, flags=3, offset=rank * per)
        sums, _, caps = O.walk(lat, cyl, seqs, p, O.KERN64)
        t = torch.from_numpy(np.ascontiguousarray(sums))
        dist.all_reduce(t)
        bench.barrier(world)
        tmax = bench.max_over_ranks(float(rank + 1) * 0.5, world)
        if rank == 0:
            q.put(("ok", t.numpy().copy(), tmax, int(caps)))
        dist.destroy_process_group()
    except Exception as e:  # reported to the parent, which fails the test
        q.put(("error", repr(e), None, None))


def test_two_rank_walker_shards_sum_to_the_whole(orc):
    import multiprocessing as mp
    O = orc
    n, steps = 512, 120
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, n, steps, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        status, sums, tmax, caps = q.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert status == "ok", sums
    lat, cyl, seqs, K = _case()
    p = K.params(n, steps, flags=3)
    whole, _, _ = O.walk(lat, cyl, seqs, p, O.KERN64)
    np.testing.assert_allclose(sums, whole, rtol=1e-12, atol=1e-12 * n)
    assert tmax == 1.0  # max over ranks of (0.5, 1.0)
    assert caps == 0
    for p in procs:
        assert p.exitcode == 0
