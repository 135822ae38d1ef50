"""Multi-rank replica exchange, emulated on CPU with gloo (world size 2 and 3).

Every rank must take the same decisions as a single process holding all
replicas, and those must be the decisions of k_pt_swap (the counter-based
draws (s, swap_index, 0xFFFFFFFF) of the run's seed), checked against the
oracle's independent Philox.  A rank that leaves between steps is noticed by
the others at their next collective (a short process-group timeout).
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle as O
from espins_gb300 import distributed as D

TEMS = list(np.geomspace(5.0, 40.0, 12))
SEED = 0x0123456789ABCDEF


def _energies(step, R):
    rng = np.random.default_rng(1000 + step)
    return -3000.0 + 400.0 * np.sort(rng.normal(size=R))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, steps, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ex = D.ReplicaExchange(TEMS, rank, world, SEED)
    hist = []
    for st in range(steps):
        e_rep = _energies(st, len(TEMS))  # energy of each replica at this step
        mine = [e_rep[r] for r in ex.my_replicas]
        sw = ex.exchange(mine, start=(st % 2) + 1, dist=dist)
        hist.append(sw)
    out[rank] = (hist, ex.repl_at.copy(), ex.num_swaps.copy(), ex.my_temperatures())
    dist.barrier()
    dist.destroy_process_group()


def _single(steps):
    ex = D.ReplicaExchange(TEMS, 0, 1, SEED)
    hist = []
    for st in range(steps):
        hist.append(ex.exchange(list(_energies(st, len(TEMS))), start=(st % 2) + 1))
    return hist, ex.repl_at.copy(), ex.num_swaps.copy()


@pytest.mark.parametrize("world", [2, 3])
def test_ranks_agree_with_one_process(world):
    steps = 40
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, steps, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    ref_hist, ref_map, ref_swaps = _single(steps)
    for r in range(world):
        hist, repl_at, swaps, temps = out[r]
        assert hist == ref_hist
        assert np.array_equal(repl_at, ref_map)
        assert np.array_equal(swaps, ref_swaps)
        lo, hi = D.block_split(len(TEMS), world)[r]
        inv = np.argsort(ref_map)
        assert temps == [int(inv[k]) for k in range(lo, hi)]
    # some pairs swapped, some did not
    flat = [s for h in ref_hist for s in h]
    assert 0 < len(flat) < steps * (len(TEMS) // 2)


def test_philox_matches_oracle():
    for ctr, key in [((0, 0, 0, 0), (0, 0)), ((5, 17, 0, 0xFFFFFFFF), (0x89ABCDEF, 0x01234567)),
                     ((2**32 - 1,) * 4, (2**32 - 1,) * 2)]:
        assert list(D.philox4x32_10(ctr, key)) == [int(x) for x in O.philox4x32_10(ctr, key)]


def _leaver(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=3))
    ex = D.ReplicaExchange(TEMS, rank, world, SEED)
    ex.exchange([0.0] * len(ex.my_replicas), 1, dist=dist)
    if rank == 1:
        out[rank] = "left"
        os._exit(0)  # leaves between steps, nothing in flight
    try:
        ex.exchange([0.0] * len(ex.my_replicas), 2, dist=dist)
        out[rank] = "no error"
    except Exception as exc:  # noqa: BLE001
        out[rank] = "error: " + type(exc).__name__


def test_a_rank_that_leaves_is_detected_at_the_next_exchange():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_leaver, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert out[1] == "left"
    assert out[0].startswith("error")
