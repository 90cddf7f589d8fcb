"""Host-side logic that needs no GPU."""
import os
import socket

import numpy as np
import pytest

from lokigpu import synth


def _reference_sequential_removal(N, m, rng):
    """The reference's placement of excess secondaries
    (Code/LoKI-MC/Sources/BoltzmannMC.C:1379-1407): while secondaries remain,
    draw r uniformly over N + remaining; r < N replaces slot r with the last
    secondary, otherwise secondary r - N is dropped. Returns the set of
    survivors (original i -> i, secondary j -> N + j)."""
    slots = list(range(N))
    pending = [N + j for j in range(m)]
    while pending:
        r = min(int(rng.random() * (N + len(pending))), N + len(pending) - 1)
        if r < N:
            slots[r] = pending.pop()
        else:
            k = r - N
            pending[k], pending[-1] = pending[-1], pending[k]
            pending.pop()
    return set(slots)


def test_sequential_removal_is_a_uniform_subset():
    """The GPU's population control removes a uniformly random m-subset of the
    N + m pool in parallel; the reference's sequential procedure has the same
    law: every member survives with probability N / (N + m), pairs with
    probability N (N-1) / ((N+m)(N+m-1))."""
    rng = np.random.default_rng(5)
    N, m, trials = 6, 3, 60000
    single = np.zeros(N + m)
    pair = 0
    for _ in range(trials):
        s = _reference_sequential_removal(N, m, rng)
        for i in s:
            single[i] += 1
        pair += (0 in s) and (N in s)
    p1 = N / (N + m)
    p2 = N * (N - 1) / ((N + m) * (N + m - 1))
    sd1 = np.sqrt(p1 * (1 - p1) / trials)
    assert np.all(np.abs(single / trials - p1) < 5 * sd1), single / trials
    assert abs(pair / trials - p2) < 5 * np.sqrt(p2 * (1 - p2) / trials)


def test_synthetic_gases_are_seeded_and_shaped():
    a, b = synth.flatten([synth.n2_like_gas()]), synth.flatten([synth.n2_like_gas()])
    assert a.n == 40 and np.array_equal(a.rel_dens, b.rel_dens)
    assert all(np.array_equal(x, y) for x, y in zip(a.raw_v, b.raw_v))
    o2 = synth.flatten([synth.o2_like_gas()])
    assert o2.n == 25 and (o2.ptype == 2).sum() == 1  # one attachment
    att = int(np.flatnonzero(o2.ptype == 2)[0])
    assert o2.eloss[att] == 4.4 and abs(max(o2.raw_v[att]) - 1.4e-22) < 1e-30
    mix = synth.flatten([synth.n2_like_gas(fraction=0.8), synth.o2_like_gas(fraction=0.2)])
    assert mix.n == 65 and list(mix.gas_first) == [0, 40] and list(mix.gas_last) == [39, 64]
    for seed in range(5):
        g = synth.random_gas(seed, "R", 1.0)
        n = synth.flatten([g]).n
        assert 10 <= n <= 45, n


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import sys

    import torch
    import torch.distributed as dist

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    out = bench.aggregate_ranks(10.0 + rank, 100.0 * (rank + 1), 1000.0 * (rank + 1), torch.device("cpu"))
    q.put((rank, out))
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks_gloo():
    """bench.py under torchrun: replicas only, job time = slowest rank,
    collisions summed over ranks."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert res[0] == res[1] == (11.0, 300.0, 3000.0)
