"""Norm <psi|psi> of a square open-boundary PEPS with Z2 symmetry, contracted
exactly (no truncation) column by column on the GPU.

Site (r, c) is a rank-5 tensor T[l, u, r, d, p]: virtual legs of dimension D
with two Z2 sectors of D/2 each, a physical leg of dimension d with sectors
1 + 1, and dimension-1 boundary legs (one even sector) on the lattice edge.  A
block exists for every sector tuple of even total charge.  Entries are float64
N(0,1) / sqrt(block size) from numpy's PCG64 generator seeded with `seed`,
drawn site by site in row-major order, block by block.

The double layer E = sum_p T[l,u,r,d,p] T[l',u',r',d',p] is one block-sparse
contraction; its legs are reordered to (l l' u u' r r' d d') and each pair is
fused into one bond of dimension D^2 (charge-ordered fusion), after which the
dimension-1 boundary bonds are fused into a neighbouring leg.  The network is
then contracted in the order: column 0 top to bottom, then every further
column top to bottom, each step one block-sparse contraction over all bonds
the two tensors share; the last step closes the network to a scalar.  The
reference project benchmarks a PEPS contraction of this kind
(test/gpu/peps_test.cu); it has no leg fusion, which this driver needs.
"""
from __future__ import annotations

import time
from dataclasses import dataclass
from typing import Dict, List

import numpy as np

from .sectors import BlockList, Leg, charge_blocks, fuse_sector_order


@dataclass
class Site:
    r: int
    c: int
    legs: List[Leg]        # l, u, r, d, p
    blocks: BlockList
    data: np.ndarray


def bond_leg(D: int, direction: int) -> Leg:
    return Leg([0, 1], [D // 2, D - D // 2], direction)


def boundary_leg(direction: int) -> Leg:
    return Leg([0], [1], direction)


def sites(L: int = 4, D: int = 6, d: int = 2, seed: int = 1) -> List[Site]:
    rng = np.random.default_rng(seed)
    out = []
    for r in range(L):
        for c in range(L):
            legs = [boundary_leg(+1) if c == 0 else bond_leg(D, +1),
                    boundary_leg(+1) if r == 0 else bond_leg(D, +1),
                    boundary_leg(-1) if c == L - 1 else bond_leg(D, -1),
                    boundary_leg(-1) if r == L - 1 else bond_leg(D, -1),
                    Leg([0, 1], [d // 2, d - d // 2], -1)]
            bl = charge_blocks(legs, 0, modulus=2)
            sizes = np.prod(bl.block_dims, axis=1)
            data = np.concatenate([rng.standard_normal(int(n)) / np.sqrt(n) for n in sizes])
            out.append(Site(r, c, legs, bl, data))
    return out


def _labels(r: int, c: int):
    """Bond labels of site (r, c): horizontal bond h(r, c) joins (r, c-1) and
    (r, c); vertical bond v(r, c) joins (r-1, c) and (r, c)."""
    return [("h", r, c), ("v", r, c), ("h", r, c + 1), ("v", r + 1, c)]


def double_layer(tq, s: Site, L: int, precision="native", slices=0, stream=None):
    """(tensor, bond labels) of the double-layer tensor of site s, boundary
    bonds removed; precision is that of the physical-leg contraction."""
    b, e = s.blocks.points()
    T = tq.BlockSparseTensor(s.blocks.dimension, s.data, b, e, stream=stream)
    E = T.contract(T, [[4, 4]], precision=precision, layout="reduced", slices=slices,
                   stream=stream)
    E = E.hard_transpose([0, 4, 1, 5, 2, 6, 3, 7], stream=stream)
    legs = []
    for k in range(4):
        E, fused = E.fuse_sectors(k, s.legs[k], s.legs[k], modulus=2, stream=stream)
        legs.append(fused)
    # boundary bonds (dimension 1, one sector) fused away into a neighbour leg;
    # the neighbour keeps its place, so the bond order stays l, u, r, d
    k = 0
    while k < len(legs):
        if legs[k].dim == 1 and len(legs) > 1:
            if k + 1 < len(legs):
                nb = legs[k + 1]
                E = E.fuse_legs(k, [0, 1], np.concatenate([[0], np.cumsum(nb.sizes)]),
                                nb.offsets.reshape(1, -1), stream=stream)
            else:
                pa = legs[k - 1]
                E = E.fuse_legs(k - 1, np.concatenate([[0], np.cumsum(pa.sizes)]), [0, 1],
                                pa.offsets.reshape(-1, 1), stream=stream)
            del legs[k]
            continue
        k += 1
    return E, _squeeze_labels(s.r, s.c, L)


def _squeeze_labels(r, c, L):
    lab = _labels(r, c)
    keep = []
    for (kind, rr, cc) in lab:
        if kind == "h" and (cc == 0 or cc == L):
            continue
        if kind == "v" and (rr == 0 or rr == L):
            continue
        keep.append((kind, rr, cc))
    return keep


def network(tq, L=4, D=6, d=2, seed=1, precision="native", slices=0, stream=None):
    """Double-layer tensors and their bond labels, by (r, c)."""
    out = {}
    for s in sites(L, D, d, seed):
        out[(s.r, s.c)] = double_layer(tq, s, L, precision, slices, stream)
    return out


def contract_norm(tq, net: Dict, L=4, precision="native", slices=0, stream=None):
    """<psi|psi> of the network: column by column, top to bottom.  Returns
    (norm, useful flops, wall seconds)."""
    order = [(r, c) for c in range(L) for r in range(L)]
    X, xl = net[order[0]]
    flops = 0.0
    t0 = time.perf_counter()
    for rc in order[1:]:
        E, el = net[rc]
        shared = [l for l in xl if l in el]
        pairs = [[xl.index(l), el.index(l)] for l in shared]
        P = tq.ContractionPlan(X, E, pairs, precision=precision, layout="reduced",
                               slices=slices, stream=stream)
        P.execute(stream)
        P.check(stream)
        flops += P.flops
        X = P.result
        xl = [l for l in xl if l not in shared] + [l for l in el if l not in shared]
    assert not xl, xl
    norm = float(X.to_number())
    return norm, flops, time.perf_counter() - t0
