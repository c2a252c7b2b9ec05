"""Charge-sector (symmetry) constructors for block-sparse tensors.

Torque itself has no charges: its caller maps symmetry sectors to coordinate
boxes (src/tensor/block_sparse.h:109-145).  These helpers do that mapping:
every leg is split into contiguous coordinate ranges, one per charge sector,
laid out in the order the charges are given; a block exists for every tuple of
sectors whose signed charges satisfy the conservation rule.  Blocks are
enumerated in column-major order of the sector indices (leg 0 fastest), the
reference's index convention (src/util/space.h:11-24).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np


@dataclass
class Leg:
    """One tensor leg: sector charges, sector sizes and direction (+1 incoming,
    -1 outgoing)."""
    charges: Sequence[int]
    sizes: Sequence[int]
    direction: int = 1

    def __post_init__(self):
        self.charges = [int(q) for q in self.charges]
        self.sizes = [int(s) for s in self.sizes]
        if len(self.charges) != len(self.sizes) or any(s <= 0 for s in self.sizes):
            raise ValueError("sector charges and positive sizes must pair up")

    @property
    def dim(self) -> int:
        return int(sum(self.sizes))

    @property
    def offsets(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum(self.sizes)[:-1]]).astype(np.int64)

    def flipped(self) -> "Leg":
        return Leg(self.charges, self.sizes, -self.direction)


@dataclass
class BlockList:
    """Boxes of a block-sparse tensor: begin/end are n_blocks x rank (row = block)."""
    dimension: np.ndarray
    begin: np.ndarray
    end: np.ndarray
    sectors: np.ndarray  # n_blocks x rank sector indices

    @property
    def n_blocks(self) -> int:
        return int(self.begin.shape[0])

    @property
    def block_dims(self) -> np.ndarray:
        return self.end - self.begin + 1

    @property
    def n_elem(self) -> int:
        return int(np.prod(self.block_dims, axis=1).sum()) if self.n_blocks else 0

    def points(self):
        """(begin, end) as rank x n_blocks matrices (the arma::umat layout)."""
        return self.begin.T.copy(), self.end.T.copy()


def charge_blocks(legs: List[Leg], total: int = 0, modulus: Optional[int] = None) -> BlockList:
    """All sector tuples with sum(direction * charge) == total (mod `modulus`
    for Z_n symmetries), in column-major order of the sector indices."""
    if modulus or not legs:
        shape = [len(l.charges) for l in legs]
        grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
        sidx = np.stack([g.ravel(order="F") for g in grids], axis=1).astype(np.int64)
        sidx = sidx.reshape(-1, len(legs))
        q = np.zeros(sidx.shape[0], np.int64)
        for l, leg in enumerate(legs):
            q += leg.direction * np.asarray(leg.charges, np.int64)[sidx[:, l]]
        keep = ((q - total) % modulus == 0) if modulus else (q == total)
        sidx = sidx[keep]
    else:
        sidx = _u1_tuples(legs, total)
    begin = np.zeros_like(sidx)
    end = np.zeros_like(sidx)
    for l, leg in enumerate(legs):
        off = leg.offsets
        sz = np.asarray(leg.sizes, np.int64)
        begin[:, l] = off[sidx[:, l]]
        end[:, l] = off[sidx[:, l]] + sz[sidx[:, l]] - 1
    dim = np.asarray([leg.dim for leg in legs], np.int64)
    return BlockList(dim, begin, end, sidx)


def _u1_tuples(legs: List[Leg], total: int) -> np.ndarray:
    """Sector tuples of U(1) legs with sum(direction * charge) == total, built
    leg by leg and pruned by the charge range the remaining legs can still
    add; returned in column-major order (leg 0 fastest)."""
    qs = [leg.direction * np.asarray(leg.charges, np.int64) for leg in legs]
    lo = np.zeros(len(legs) + 1, np.int64)
    hi = np.zeros(len(legs) + 1, np.int64)
    for l in range(len(legs) - 1, -1, -1):
        lo[l] = lo[l + 1] + qs[l].min()
        hi[l] = hi[l + 1] + qs[l].max()
    part = np.zeros((1, 0), np.int64)
    charge = np.zeros(1, np.int64)
    for l in range(len(legs)):
        n = len(qs[l])
        rep = np.repeat(np.arange(part.shape[0]), n)
        idx = np.tile(np.arange(n, dtype=np.int64), part.shape[0])
        c = charge[rep] + qs[l][idx]
        need = total - c
        ok = (need >= lo[l + 1]) & (need <= hi[l + 1])
        part = np.concatenate([part[rep[ok]], idx[ok, None]], axis=1)
        charge = c[ok]
    if part.shape[0] == 0:
        return part
    order = np.lexsort(part.T)  # last key primary: leg 0 varies fastest
    return part[order]


def gaussian_sizes(charges: Sequence[int], peak: float, width2: float) -> List[int]:
    """s_q = max(1, round(peak * exp(-q^2 / width2))), rounding half up."""
    return [max(1, int(np.floor(peak * np.exp(-(q * q) / width2) + 0.5))) for q in charges]


def fuse_sector_order(a: Leg, b: Leg, modulus: Optional[int] = None):
    """Charge-ordered fusion of two adjacent legs: the fused leg's sectors are
    the (sector_a, sector_b) pairs sorted by fused charge (stable in column-major
    order of the pair), each pair a contiguous range of size s_a * s_b.
    Returns (fused Leg, offset of each pair [n_a, n_b])."""
    pairs = [(ia, ib) for ib in range(len(b.charges)) for ia in range(len(a.charges))]

    def qf(p):
        q = a.direction * a.charges[p[0]] + b.direction * b.charges[p[1]]
        return q % modulus if modulus else q
    order = sorted(range(len(pairs)), key=lambda t: qf(pairs[t]))
    off = np.zeros((len(a.charges), len(b.charges)), np.int64)
    charges, sizes = [], []
    run = 0
    for t in order:
        ia, ib = pairs[t]
        off[ia, ib] = run
        sz = a.sizes[ia] * b.sizes[ib]
        run += sz
        charges.append(qf(pairs[t]))
        sizes.append(sz)
    return Leg(charges, sizes, 1), off
