"""Parallel tempering over a batch of independent systems: on one engine, or with the systems
split across ranks (one engine per GPU).

The reference has no counterpart inside one process: its replica exchange runs one oxDNA
process per replica (MPI / oxpy scripts) and many small systems share a GPU through MPS.  Here a
ladder of systems lives in batched engines; a swap exchanges the temperatures of two systems
(their parameter tables and thermostats) and rescales their momenta, never coordinates, so the
only data a multi-rank ladder exchanges is one FP64 energy per system per round.

* swap_round: the Metropolis decisions of one round of neighbour swaps, a pure function of the
  temperatures, the potential energies, the round's parity and its uniform draws (one per tried
  pair, drawn whether or not the pair needs it, so every rank consumes the same stream);
* partition: the size-balanced split of the systems over ranks (largest first, each to the rank
  with the least nucleotides so far);
* RankLadder: one rank's share of a ladder split across ranks; every rank keeps the whole
  temperature ladder, the ranks sum their systems' energies into one global array (an
  all-reduce of n_systems doubles), all take the same decisions, and each applies those that
  touch its own systems.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def swap_round(temps: Sequence[float], U: Sequence[float], parity: int, draws: Sequence[float]):
    """One round of swaps between neighbouring rungs of a temperature ladder.  temps[k] and
    U[k] are the temperature and potential energy of system k; rungs (r, r + 1) with r of the
    given parity are tried in increasing r, pair m with the uniform draws[m], under
    min(1, exp((1/T_r - 1/T_r+1) (U_r - U_r+1))).  Returns the new temperatures and the list of
    accepted pairs (i, j) of system indices (i at the lower rung)."""
    temps = np.array(temps, np.float64, copy=True)
    U = np.asarray(U, np.float64)
    order = np.argsort(temps, kind="stable")  # order[r] = system at rung r
    swaps = []
    for m, r in enumerate(range(parity, len(order) - 1, 2)):
        i, j = int(order[r]), int(order[r + 1])
        d = (1.0 / temps[i] - 1.0 / temps[j]) * (U[i] - U[j])
        if d >= 0 or draws[m] < np.exp(d):
            temps[i], temps[j] = temps[j], temps[i]
            swaps.append((i, j))
    return temps, swaps


def pairs_in_round(n_systems: int, parity: int) -> int:
    """how many rung pairs a round of the given parity tries"""
    return len(range(parity, n_systems - 1, 2))


def apply_swaps(engine, old_temps, swaps, local_of=None):
    """Applies accepted swaps to an engine (MDSystem): each system of a pair takes the other's
    temperature and rescales its momenta by sqrt(T_new / T_old).  local_of maps a system index to
    the engine's own index (None: the engine holds every system; systems it lacks are skipped)."""
    for i, j in swaps:
        for a, b in ((i, j), (j, i)):
            k = a if local_of is None else local_of.get(a)
            if k is None:
                continue
            engine.set_temperature(float(old_temps[b]), k)
            engine.scale_momenta(float(np.sqrt(old_temps[b] / old_temps[a])), k)


def partition(sizes: Sequence[int], n_parts: int) -> List[np.ndarray]:
    """Size-balanced split of systems over n_parts ranks: systems by decreasing size (ties by
    index), each to the rank holding the fewest nucleotides so far (ties: the lowest rank);
    each rank's systems are returned in increasing index.  The largest load is at most the mean
    plus the largest system."""
    sizes = np.asarray(sizes, np.int64)
    if n_parts < 1:
        raise ValueError("n_parts must be at least 1")
    load = np.zeros(n_parts, np.int64)
    parts: List[list] = [[] for _ in range(n_parts)]
    for k in sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k)):
        r = int(np.argmin(load))
        parts[r].append(k)
        load[r] += sizes[k]
    return [np.array(sorted(p), np.int64) for p in parts]


class RankLadder:
    """This rank's share of a temperature ladder split across ranks (torch.distributed, any
    backend: the energies travel as one float64 tensor on `device`).

    systems: the global indices of this rank's systems, in the order of its engine; temps: the
    whole ladder's current temperatures (every rank holds the same array); seed: the shared seed
    of the swap draws."""

    def __init__(self, systems: Sequence[int], temps: Sequence[float], seed: int, group=None, device="cpu"):
        self.systems = np.asarray(systems, np.int64)
        self.local_of = {int(g): k for k, g in enumerate(self.systems)}
        self.temps = np.array(temps, np.float64, copy=True)
        self.rng = np.random.default_rng(seed)
        self.group = group
        self.device = device
        self.parity = 0
        self.tried = 0
        self.accepted = 0

    def gather_energies(self, U_local) -> np.ndarray:
        import torch
        import torch.distributed as dist
        buf = torch.zeros(len(self.temps), dtype=torch.float64, device=self.device)
        if len(self.systems):
            buf[torch.as_tensor(self.systems, device=self.device)] = torch.as_tensor(
                np.atleast_1d(np.asarray(U_local, np.float64)), device=self.device)
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=self.group)
        return buf.cpu().numpy()

    def exchange(self, engine, U_local=None) -> List[Tuple[int, int]]:
        """One round: this rank's energies (from the engine unless given), the global decision,
        the local changes; returns the accepted pairs (global indices)."""
        if U_local is None:
            U_local, _, _ = engine.energies()
        U = self.gather_energies(U_local)
        draws = self.rng.uniform(size=pairs_in_round(len(self.temps), self.parity))
        old = self.temps
        self.temps, swaps = swap_round(old, U, self.parity, draws)
        apply_swaps(engine, old, swaps, self.local_of)
        self.tried += len(draws)
        self.accepted += len(swaps)
        self.parity ^= 1
        return swaps
