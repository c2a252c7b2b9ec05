"""Synthetic block-sparse workloads with the shapes the benchmarks are quoted on.

All inputs are synthetic and seeded: entries are float64 N(0,1) drawn with
numpy's PCG64 generator (``np.random.default_rng(seed).standard_normal``, the
same stream on x86_64 and aarch64), filled in block-list order, A then B.

u1_rank4(...) is the U(1) pair A[a,b,c,d] x B[c,d,e,f] contracted over (c,d):
legs a,b of A incoming and c,d outgoing; legs c,d of B incoming and e,f
outgoing; a block exists iff incoming minus outgoing charges sum to zero.
  - small:  sectors q in -2..2 of sizes {3,5,8,5,3}, dim 24 per leg, seed 0
            (85 blocks per tensor, 325 matched pairs);
  - uneven: sectors q in -16..16 of sizes max(1, round(48 exp(-q^2/32))),
            488 per leg, seed 2 (23,969 blocks per tensor, 593,505 pairs,
            block GEMMs from 1x1x1 up to 2304x2304x2304).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .sectors import BlockList, Leg, charge_blocks, gaussian_sizes


@dataclass
class Contraction:
    name: str
    A: BlockList
    B: BlockList
    a_data: np.ndarray
    b_data: np.ndarray
    pairs: np.ndarray  # n x 2 contracting indices

    def flops(self) -> float:
        """Useful flops: sum over matched block pairs of 2*m*n*k."""
        return useful_flops(self.A, self.B, self.pairs)


def useful_flops(A: BlockList, B: BlockList, pairs) -> float:
    """Sum over matched pairs of 2*m*n*k, for sector-aligned boxes (pairs match
    iff their contracted boxes are equal), grouped by contracted box."""
    return pair_stats(A, B, pairs)[0]


def pair_stats(A: BlockList, B: BlockList, pairs):
    """(useful flops, matched pairs) of a sector-aligned contraction."""
    pairs = np.asarray(pairs).reshape(-1, 2)
    al, bl = pairs[:, 0], pairs[:, 1]
    fa = [l for l in range(A.begin.shape[1]) if l not in set(al.tolist())]
    fb = [l for l in range(B.begin.shape[1]) if l not in set(bl.tolist())]
    da, db = A.block_dims, B.block_dims
    m = np.prod(da[:, fa], axis=1).astype(float) if fa else np.ones(A.n_blocks)
    n = np.prod(db[:, fb], axis=1).astype(float) if fb else np.ones(B.n_blocks)
    k = np.prod(da[:, al], axis=1).astype(float) if len(al) else np.ones(A.n_blocks)
    ka = np.concatenate([A.begin[:, al], A.end[:, al]], 1)
    kb = np.concatenate([B.begin[:, bl], B.end[:, bl]], 1)
    keys, inv = np.unique(np.concatenate([ka, kb], 0), axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    ia, ib = inv[:A.n_blocks], inv[A.n_blocks:]
    mk = np.bincount(ia, weights=m * k, minlength=len(keys))
    ca = np.bincount(ia, minlength=len(keys)).astype(float)
    nb = np.bincount(ib, weights=n, minlength=len(keys))
    cb = np.bincount(ib, minlength=len(keys)).astype(float)
    return float(2.0 * np.sum(mk * nb)), int(np.sum(ca * cb))


def u1_rank4(charges, sizes, seed: int, name: str) -> Contraction:
    def leg(d):
        return Leg(charges, sizes, d)
    A = charge_blocks([leg(+1), leg(+1), leg(-1), leg(-1)])
    B = charge_blocks([leg(+1), leg(+1), leg(-1), leg(-1)])
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(A.n_elem)
    b = rng.standard_normal(B.n_elem)
    return Contraction(name, A, B, a, b, np.array([[2, 0], [3, 1]], np.int64))


def small_u1() -> Contraction:
    """Dim-24 legs, 5 sectors, seed 0: the CPU-runnable case."""
    return u1_rank4([-2, -1, 0, 1, 2], [3, 5, 8, 5, 3], 0, "u1-rank4-dim24-q5")


def uneven_u1(peak: float = 48.0, qmax: int = 16, seed: int = 2, data: bool = True) -> Contraction:
    """Gaussian-profiled sectors q=-qmax..qmax, s_q = max(1, round(peak e^{-q^2/32}))."""
    q = list(range(-qmax, qmax + 1))
    s = gaussian_sizes(q, peak, 32.0)
    if data:
        return u1_rank4(q, s, seed, "u1-rank4-gauss%d-q%d" % (int(peak), 2 * qmax + 1))

    def leg(d):
        return Leg(q, s, d)
    A = charge_blocks([leg(+1), leg(+1), leg(-1), leg(-1)])
    B = charge_blocks([leg(+1), leg(+1), leg(-1), leg(-1)])
    return Contraction("u1-rank4-gauss%d-q%d" % (int(peak), 2 * qmax + 1), A, B,
                       np.zeros(0), np.zeros(0), np.array([[2, 0], [3, 1]], np.int64))


# ---------------------------------------------------------------- PEPS sweep
def scaled_sectors(dim: int):
    """U(1) sectors of a leg of dimension `dim`, Gaussian-profiled like the
    uneven case and scaled to the dimension: charges -Q..Q with Q = max(1,
    dim // 12), weights exp(-q^2 / (2 sigma^2)) with sigma = max(1, Q / 2),
    sizes by largest remainder so they sum to dim, each at least 1."""
    Q = max(1, dim // 12)
    q = np.arange(-Q, Q + 1)
    w = np.exp(-q.astype(float) ** 2 / (2.0 * max(1.0, Q / 2.0) ** 2))
    raw = w / w.sum() * dim
    s = np.maximum(1, np.floor(raw)).astype(int)
    while s.sum() < dim:
        s[np.argmax(raw - s)] += 1
    while s.sum() > dim:
        k = np.argmax(np.where(s > 1, s - raw, -np.inf))
        s[k] -= 1
    return q.tolist(), s.tolist()


@dataclass
class SiteUpdate:
    """One PEPS-sweep site update: E1[chi,l,u,chi'] x T[l,u,r,d,p] over (l,u)
    gives X[chi,chi',r,d,p]; X x E2[chi',r,d,chi''] over (chi',r,d) gives
    Y[chi,p,chi'']."""
    D: int
    chi: int
    T: BlockList
    E1: BlockList
    E2: BlockList
    t_data: np.ndarray
    e1_data: np.ndarray
    e2_data: np.ndarray
    pairs1 = np.array([[1, 0], [2, 1]], np.int64)
    pairs2 = np.array([[1, 0], [2, 1], [3, 2]], np.int64)


def peps_sweep(n: int = 256, seed: int = 3, data: bool = True):
    """n independent site updates: D ~ U{4..10}, chi ~ U{16..64} (drawn first,
    all instances), then the entries N(0,1), instance by instance, T, E1, E2,
    from numpy's PCG64 with `seed`.  Directions: T (l,u in; r,d,p out), E1 (chi
    in, l,u out, chi' in), E2 (chi' out, r,d in, chi'' out); physical leg p has
    charges {0, 1} of size 1 each."""
    rng = np.random.default_rng(seed)
    Ds = rng.integers(4, 11, size=n)
    chis = rng.integers(16, 65, size=n)
    out = []
    for D, chi in zip(Ds.tolist(), chis.tolist()):
        qd, sd = scaled_sectors(D)
        qc, sc = scaled_sectors(chi)
        p = ([0, 1], [1, 1])
        T = charge_blocks([Leg(qd, sd, +1), Leg(qd, sd, +1), Leg(qd, sd, -1), Leg(qd, sd, -1),
                           Leg(*p, -1)])
        E1 = charge_blocks([Leg(qc, sc, +1), Leg(qd, sd, -1), Leg(qd, sd, -1), Leg(qc, sc, +1)])
        E2 = charge_blocks([Leg(qc, sc, -1), Leg(qd, sd, +1), Leg(qd, sd, +1), Leg(qc, sc, -1)])
        if data:
            t = rng.standard_normal(T.n_elem)
            e1 = rng.standard_normal(E1.n_elem)
            e2 = rng.standard_normal(E2.n_elem)
        else:
            t = e1 = e2 = np.zeros(0)
        out.append(SiteUpdate(D, chi, T, E1, E2, t, e1, e2))
    return out


# ---------------------------------------------------------------- random contractions
@dataclass
class RandomContraction:
    """One random U(1) block-sparse contraction: A's legs a_legs[k] contract
    with B's legs b_legs[k] (pairs = [[a_legs[k], b_legs[k]]])."""
    index: int
    A: BlockList
    B: BlockList
    pairs: np.ndarray
    a_legs: list
    b_legs: list
    legs_A: list = None  # sectors.Leg per leg of A
    legs_B: list = None

    def spec(self) -> dict:
        """JSON-ready description (rebuild with from_spec)."""
        leg = lambda l: [l.charges, l.sizes, l.direction]
        return {"index": self.index, "A": [leg(l) for l in self.legs_A],
                "B": [leg(l) for l in self.legs_B], "pairs": self.pairs.tolist()}


def from_spec(d: dict) -> RandomContraction:
    la = [Leg(*x) for x in d["A"]]
    lb = [Leg(*x) for x in d["B"]]
    pairs = np.asarray(d["pairs"], np.int64).reshape(-1, 2)
    return RandomContraction(int(d["index"]), charge_blocks(la), charge_blocks(lb), pairs,
                             pairs[:, 0].tolist(), pairs[:, 1].tolist(), la, lb)


def _profile_sizes(dim: int, n: int, gaussian: bool):
    """n sector sizes summing to dim (each >= 1): Gaussian weights
    exp(-q^2 / (2 (n/4)^2)) over q = -(n//2).., or uniform; largest remainder."""
    q = np.arange(n) - n // 2
    w = np.exp(-q.astype(float) ** 2 / (2.0 * max(1.0, n / 4.0) ** 2)) if gaussian else np.ones(n)
    raw = w / w.sum() * dim
    s = np.maximum(1, np.floor(raw)).astype(int)
    while s.sum() < dim:
        s[np.argmax(raw - s)] += 1
    while s.sum() > dim:
        k = np.argmax(np.where(s > 1, s - raw, -np.inf))
        s[k] -= 1
    return q.tolist(), s.tolist()


def _n_charge_tuples(legs) -> int:
    """Blocks charge_blocks(legs) would produce, by convolving charge counts."""
    dist = {0: 1}
    for leg in legs:
        nd = {}
        for q0, c0 in dist.items():
            for q in leg.charges:
                k = q0 + leg.direction * q
                nd[k] = nd.get(k, 0) + c0
        dist = nd
    return dist.get(0, 0)


def random_contractions(n: int = 2000, seed: int = 4, max_elem: int = 1 << 22,
                        max_blocks: int = 50000, max_flops: float = 2e10,
                        max_pairs: int = 1 << 18):
    """n random U(1) contractions, seeded: ranks 3-6, leg dims log-uniform in
    16..1024, 2-41 sectors per leg (consecutive charges around 0) with a
    Gaussian or uniform size profile, 1-3 contracted legs (A outgoing, B
    incoming), free-leg directions random.  Caps, so that one GPU runs every
    candidate schedule of all n in minutes: each tensor at most max_elem
    elements and max_blocks blocks, the contraction at most max_flops useful
    flops and max_pairs matched block pairs (legs are halved, largest first,
    and sector counts lowered until the caps hold).  Entries are not drawn
    here: the caller fills N(0,1) data."""
    rng = np.random.default_rng(seed)
    out = []
    i = 0
    while len(out) < n:
        ra, rb = int(rng.integers(3, 7)), int(rng.integers(3, 7))
        nc = int(rng.integers(1, min(3, ra - 1, rb - 1) + 1))
        nlegs = ra + rb - nc
        dims = np.exp(rng.uniform(np.log(16), np.log(1024), nlegs)).astype(int)
        nsec = rng.integers(2, 42, nlegs)
        gauss = rng.random(nlegs) < 0.5
        dirs = rng.choice([-1, 1], nlegs)
        # legs 0..nc-1 are the contracted ones; A = [free A..., contracted], B = [contracted, free B...]
        perm_a = rng.permutation(ra)
        perm_b = rng.permutation(rb)
        A = B = pairs = None
        for _ in range(64):
            nsec = np.minimum(nsec, dims)

            def leg(j, d):
                q, s = _profile_sizes(int(dims[j]), int(nsec[j]), bool(gauss[j]))
                return Leg(q, s, d)
            con = [leg(j, -1) for j in range(nc)]
            fa = [leg(nc + j, int(dirs[nc + j])) for j in range(ra - nc)]
            fb = [leg(ra + j, int(dirs[ra + j])) for j in range(rb - nc)]
            a_list = fa + con
            b_list = [c.flipped() for c in con] + fb
            a_order = [a_list[p] for p in perm_a]
            b_order = [b_list[p] for p in perm_b]
            nba, nbb = _n_charge_tuples(a_order), _n_charge_tuples(b_order)
            fill = lambda legs, nb: nb * np.prod([l.dim / len(l.sizes) for l in legs])
            ea, eb = fill(a_order, nba), fill(b_order, nbb)
            A = B = None
            if nba <= max_blocks and nbb <= max_blocks and ea <= 2 * max_elem and eb <= 2 * max_elem:
                A = charge_blocks(a_order)
                B = charge_blocks(b_order)
                a_pos = {p: k for k, p in enumerate(perm_a)}
                b_pos = {p: k for k, p in enumerate(perm_b)}
                a_legs = [a_pos[ra - nc + c] for c in range(nc)]
                b_legs = [b_pos[c] for c in range(nc)]
                pairs = np.array([[a, b] for a, b in zip(a_legs, b_legs)], np.int64)
                if A.n_elem <= max_elem and B.n_elem <= max_elem and A.n_blocks and B.n_blocks:
                    fl, npairs = pair_stats(A, B, pairs)
                    if fl <= max_flops and npairs <= max_pairs:
                        break
            # shrink: too many blocks or pairs -> fewer sectors on the most split
            # leg; too large -> halve the largest leg
            many = nba > max_blocks or nbb > max_blocks or (
                A is not None and B is not None and pair_stats(A, B, pairs)[1] > max_pairs)
            j = int(np.argmax(dims))
            if many or dims[j] <= 16:
                k = int(np.argmax(nsec))
                nsec[k] = max(2, nsec[k] // 2)
            else:
                dims[j] = max(16, dims[j] // 2)
        else:
            i += 1
            continue
        if pair_stats(A, B, pairs)[0] > 0:
            out.append(RandomContraction(i, A, B, pairs, a_legs, b_legs, a_order, b_order))
        i += 1
    return out
