"""Dense FP64 restatement of the PEPS norm <psi|psi>.

TEST INFRASTRUCTURE ONLY: the oracle the block-sparse PEPS-norm path is
checked against; only ``tests/`` and ``bench.py`` import it.  The reference's
PEPS benchmark (test/gpu/peps_test.cu) contracts dense site tensors; here every
site tensor is zero-filled to a dense array, the double layer is
E[l l', u u', r r', d d'] = sum_p T[l,u,r,d,p] T[l',u',r',d',p] with the natural
(x + D x') bond order (the value of a closed network does not depend on the
basis order of its internal bonds, so it need not match the charge-ordered
fusion of the GPU path), dimension-1 boundary bonds are dropped, and the
network is contracted with numpy tensordot in the order and over the bond
labels the caller gives.
"""
from __future__ import annotations

import numpy as np

from . import oracle as orc


def dense_site(dimension, begin, end, data):
    return orc.densify(orc.HostBS(np.asarray(dimension), begin, end, np.asarray(data)))


def double_layer(T):
    l, u, r, d, _ = T.shape
    E = np.einsum("lurdp,LURDp->lLuUrRdD", T, T, optimize=True)
    E = E.reshape(l * l, u * u, r * r, d * d)
    return E.reshape([n for n in E.shape if n != 1]) if E.ndim else E


def norm(tensors, labels, order):
    """tensors[(r, c)] dense double layers, labels[(r, c)] their bond labels;
    contraction in `order`, each step over every shared bond."""
    X, xl = tensors[order[0]], list(labels[order[0]])
    for rc in order[1:]:
        E, el = tensors[rc], list(labels[rc])
        shared = [b for b in xl if b in el]
        X = np.tensordot(X, E, axes=([xl.index(b) for b in shared], [el.index(b) for b in shared]))
        xl = [b for b in xl if b not in shared] + [b for b in el if b not in shared]
    assert not xl
    return float(X)
