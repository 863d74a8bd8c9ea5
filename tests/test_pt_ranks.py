"""Parallel tempering with the systems split across ranks (oxdna_gb300.pt), on CPU with gloo.

* partition: every system on exactly one rank, each rank's load within the mean plus the largest
  system, for the size distribution of the 256-system workload;
* a ladder of 24 systems split over two ranks (torch.distributed, gloo, 127.0.0.1) takes, round
  after round, the same swap decisions as one engine holding every system, fed the same
  energies and the same draw stream: the same final temperatures on every rank, and the same
  temperature changes and momentum rescalings applied to every system.  The engines are
  stand-ins that serve given energies and record what is applied to them (no GPU).
"""
import os
import socket

import numpy as np
import pytest

from oxdna_gb300 import pt


class FakeEngine:
    def __init__(self, U):
        self.U = np.asarray(U, np.float64)
        self.calls = []

    def energies(self):
        return self.U.copy(), None, None

    def set_temperature(self, T, k):
        self.calls.append(("T", k, float(T)))

    def scale_momenta(self, f, k):
        self.calls.append(("scale", k, float(f)))


def _ladder(n=24, seed=3, rounds=12):
    rng = np.random.default_rng(seed)
    temps = 0.0933 * (0.12 / 0.0933) ** (np.arange(n) / (n - 1))
    rng.shuffle(temps)
    sizes = np.round(np.exp(rng.uniform(np.log(16), np.log(4000), n))).astype(np.int64)
    # energies near -1.5 per nucleotide, spread so that some swaps pass and some fail
    U_rounds = [-1.5 * sizes + rng.normal(scale=0.02 * np.sqrt(sizes), size=n) * 30 for _ in range(rounds)]
    return temps, sizes, U_rounds


def _single_engine(temps, U_rounds, seed):
    rng = np.random.default_rng(seed)
    calls, parity = [], 0
    for U in U_rounds:
        eng = FakeEngine(U)
        draws = rng.uniform(size=pt.pairs_in_round(len(temps), parity))
        old = temps
        temps, swaps = pt.swap_round(old, U, parity, draws)
        pt.apply_swaps(eng, old, swaps)
        calls.append(sorted(eng.calls))
        parity ^= 1
    return temps, calls


def _worker(rank, world, port, temps, sizes, U_rounds, seed, queue):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = pt.partition(sizes, world)[rank]
        lad = pt.RankLadder(mine, temps, seed)
        calls = []
        for U in U_rounds:
            eng = FakeEngine(U[mine])
            lad.exchange(eng)
            calls.append([(c[0], int(mine[c[1]]), c[2]) for c in eng.calls])
        queue.put((rank, lad.temps.tolist(), calls, lad.tried, lad.accepted))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_balances_the_batched_workload():
    rng = np.random.default_rng(1)
    sizes = np.round(np.exp(rng.uniform(np.log(16), np.log(4000), 256))).astype(np.int64)
    for n in (1, 2, 4, 8):
        parts = pt.partition(sizes, n)
        assert sorted(np.concatenate(parts).tolist()) == list(range(256))
        loads = np.array([sizes[p].sum() for p in parts])
        assert loads.max() <= sizes.sum() / n + sizes.max()
        if n > 1:
            assert loads.max() / loads.mean() < 1.02


def test_ladder_split_over_two_ranks_matches_one_engine():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    seed = 11
    temps, sizes, U_rounds = _ladder()
    want_temps, want_calls = _single_engine(temps, U_rounds, seed)
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, temps, sizes, U_rounds, seed, queue)) for r in range(2)]
    for p in procs:
        p.start()
    got = [queue.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    accepted = sum(len([c for c in round_ if c[0] == "T"]) for round_ in want_calls) // 2
    assert 0 < accepted < sum(pt.pairs_in_round(len(temps), k % 2) for k in range(len(U_rounds)))
    for rank, t, calls, tried, acc in got:
        assert np.array_equal(np.array(t), want_temps), rank
        assert acc == accepted
    for k in range(len(U_rounds)):
        merged = sorted(got[0][2][k] + got[1][2][k])
        assert merged == want_calls[k], k
