"""The packet hand-out protocol of the persistent warp-packet searches
(take_packet in csrc/queries.cu: a pool per SM refilled in chunks from one
batch-wide counter), modelled step by step on the CPU: under random
interleavings of the warps' atomic operations every packet of the batch is
taken exactly once and every warp stops, with pools and with the counter alone.
The GPU tests run the kernels themselves."""
import random

import pytest

K, DONE, SPINS = 32, (1 << 40) - 1, 1 << 16  # kPoolChunk, kPoolDone, kPoolSpins


def _run(total_packets, n_sm, warps_per_sm, seed, pools=True):
    rng = random.Random(seed)
    mem = {"work": 0, **{s: 0 for s in range(n_sm)}}
    taken = []

    def take(sm):  # one yield per atomic operation
        if not pools:
            p = mem["work"]
            mem["work"] += 1
            yield
            return p if p < total_packets else None
        for _ in range(SPINS):
            old = mem[sm]
            mem[sm] = old + 1
            yield
            first, t = old >> 24, old & 0xFFFFFF
            if first == DONE:
                return None
            if first != 0 and t < K:
                return first - 1 + t
            if (first == 0 and t == 0) or (first != 0 and t == K):
                nxt = mem["work"]
                mem["work"] += K
                yield
                mem[sm] = ((nxt + 1) << 24) if nxt < total_packets else (DONE << 24)
                yield
        p = mem["work"]
        mem["work"] += 1
        yield
        return p if p < total_packets else None

    def warp(sm):
        empty = 0
        while True:
            g = take(sm)
            try:
                while True:
                    next(g)
                    yield
            except StopIteration as e:
                p = e.value
            if p is None:
                return
            if p >= total_packets:
                empty += 1
                assert empty <= SPINS
                continue
            empty = 0
            taken.append(p)
            yield

    ws = [warp(s) for s in range(n_sm) for _ in range(warps_per_sm)]
    live = list(range(len(ws)))
    steps = 0
    while live:
        i = rng.choice(live)
        try:
            next(ws[i])
        except StopIteration:
            live.remove(i)
        steps += 1
        assert steps < 5_000_000
    assert sorted(taken) == list(range(total_packets))


@pytest.mark.parametrize("pools", [True, False])
@pytest.mark.parametrize("total", [0, 1, 31, 32, 33, 100, 2049])
def test_every_packet_taken_once(pools, total):
    for seed in range(3):
        _run(total, 3, 4, seed, pools)
