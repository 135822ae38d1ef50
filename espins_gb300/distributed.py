"""Replica exchange across ranks without moving spins.

The reference's parallel tempering gathers every configuration on the root
rank, swaps, and scatters them back every pt_steps_swap sweeps
(src/pt.F90:873-907, pt_swap :1235-1288): 3 N R doubles each way.  Here each
rank keeps its replicas for the whole run; an exchange step is

1. an allgather of the running energy of every temperature slot (R FP64
   values) and of the slot -> replica assignment,
2. the same decisions on every rank: for pairs (s, s+1), s = start-1,
   start+1, ..., x = (1/T_s - 1/T_{s+1}) (E_s - E_{s+1}); swap if x > 0 or
   u < exp(x), u drawn from the Philox4x32-10 stream keyed by the run's seed
   with counter (s, swap_index, 0xFFFFFFFF) -- the draws of k_pt_swap,
3. a local relabelling: every rank learns which temperature each of its own
   replicas now has.

This is the host side of a multi-GPU build; on one GPU the same decisions are
taken by k_pt_swap.  It runs over any torch.distributed backend (gloo on CPU
in the tests).
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr: Sequence[int], key: Sequence[int]) -> Tuple[int, int, int, int]:
    """Philox4x32-10 (Salmon et al., SC'11), the generator of the GPU kernels."""
    c0, c1, c2, c3 = (int(v) & MASK for v in ctr)
    k0, k1 = (int(v) & MASK for v in key)
    for r in range(10):
        if r:
            k0 = (k0 + W0) & MASK
            k1 = (k1 + W1) & MASK
        p0 = M0 * c0
        p1 = M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & MASK, p1 & MASK, ((p0 >> 32) ^ c3 ^ k1) & MASK, p0 & MASK
    return c0, c1, c2, c3


def u53(a: int, b: int) -> float:
    return ((a >> 5) * 67108864.0 + (b >> 6)) * (1.0 / 9007199254740992.0)


def swap_decisions(start: int, inv_t: np.ndarray, e_slot: np.ndarray, swap_index: int, seed: int,
                   group: int = 0) -> List[int]:
    """Slots s (0-based) whose pair (s, s+1) exchanges, as k_pt_swap decides.
    With group > 0 the slots form independent groups of `group` temperatures
    and pairs stay inside a group."""
    R = len(inv_t)
    G = group if group > 0 else R
    key = (seed & MASK, (seed >> 32) & MASK)
    out = []
    pairs = [g * G + s for g in range(R // G) for s in range(start - 1, G - 1, 2)]
    for s in pairs:
        x = (inv_t[s] - inv_t[s + 1]) * (e_slot[s] - e_slot[s + 1])
        swap = x > 0.0
        if not swap:
            v = philox4x32_10((s, swap_index & MASK, (swap_index >> 32) & MASK, 0xFFFFFFFF), key)
            swap = u53(v[0], v[1]) < math.exp(x)
        if swap:
            out.append(s)
    return out


def block_split(R: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous blocks of replicas per rank, as comms_array_split (comms.F90:153-176)."""
    base, rem = divmod(R, world)
    out, start = [], 0
    for r in range(world):
        n = base + (1 if r < rem else 0)
        out.append((start, start + n))
        start += n
    return out


class ReplicaExchange:
    """Label bookkeeping of one rank: global replica ids it owns, slot maps."""

    def __init__(self, tems: Sequence[float], rank: int, world: int, seed: int):
        self.R = len(tems)
        self.inv_t = 1.0 / np.asarray(tems, dtype=np.float64)
        self.rank, self.world, self.seed = rank, world, seed
        lo, hi = block_split(self.R, world)[rank]
        self.my_replicas = list(range(lo, hi))
        self.repl_at = np.arange(self.R)   # slot -> replica
        self.temp_of = np.arange(self.R)   # replica -> slot
        self.num_swaps = np.zeros((self.R, 2), dtype=np.int64)
        self.swap_index = 0

    def exchange(self, my_energies: Sequence[float], start: int, dist=None) -> List[int]:
        """One exchange step.  my_energies: running energy of each owned replica.
        Returns the slots whose pairs swapped (identical on every rank)."""
        e_rep = np.zeros(self.R)
        mine = np.zeros(self.R)
        for r, e in zip(self.my_replicas, my_energies):
            mine[r] = e
        if dist is not None and self.world > 1:
            import torch
            t = torch.from_numpy(mine)
            dist.all_reduce(t)   # each replica is owned by exactly one rank: a sum is an allgather
            e_rep = t.numpy().copy()
        else:
            e_rep = mine
        e_slot = e_rep[self.repl_at]
        swapped = swap_decisions(start, self.inv_t, e_slot, self.swap_index, self.seed)
        for s in range(start - 1, self.R - 1, 2):
            self.num_swaps[s, 0] += 1
            self.num_swaps[s + 1, 0] += 1
        for s in swapped:
            ra, rb = self.repl_at[s], self.repl_at[s + 1]
            self.repl_at[s], self.repl_at[s + 1] = rb, ra
            self.temp_of[rb], self.temp_of[ra] = s, s + 1
            self.num_swaps[s, 1] += 1
            self.num_swaps[s + 1, 1] += 1
        self.swap_index += 1
        return swapped

    def my_temperatures(self) -> List[int]:
        """Temperature slot of each owned replica (what its GPU must use next)."""
        return [int(self.temp_of[r]) for r in self.my_replicas]
