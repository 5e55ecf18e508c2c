"""The radix tree the build makes bottom-up (one climber per leaf; a node
over keys [l, r] is the left child of the node split between r and r + 1 or
the right child of the node split between l - 1 and l, whichever boundary's
keys share the longer prefix, equal keys ordered by index; the first child
to arrive hands the second its reference and far end) is the oracle's
top-down Karras tree, node for node.  Restated here in Python over the
oracle's sorted keys for small soups, duplicate-heavy and all-equal keys,
with the leaves visited in random orders; the GPU build is checked against
the oracle stage by stage in tests/test_gpu_build.py."""
from __future__ import annotations

import random

import numpy as np
import pytest

from helpers import radix_tree_canonical

LEAF = 0x80000000


def _delta(ka: int, kb: int, b: int) -> int:
    if ka == kb:
        return 64 + 32 - (b ^ (b + 1)).bit_length()
    return 64 - (ka ^ kb).bit_length()


def bottom_up_tree(keys, order):
    """The climb, one leaf after another in `order` (any order of arrival
    gives the same tree)."""
    n = len(keys)
    keys = [int(k) for k in keys]
    bin_nodes = np.zeros((n - 1, 4), np.uint32)
    word = [None] * (n - 1)
    root = None
    for j in order:
        me, l, r = LEAF | j, j, j
        for _ in range(256):
            if l == 0:
                left = True
            elif r == n - 1:
                left = False
            else:
                left = _delta(keys[r], keys[r + 1], r) > _delta(keys[l - 1], keys[l], l - 1)
            p = r if left else l - 1
            got, word[p] = word[p], (me, l if left else r)
            if got is None:
                break
            sib, far = got
            nl, nr = (l, far) if left else (far, r)
            bin_nodes[p] = (me if left else sib, sib if left else me, nl, nr)
            me, l, r = p, nl, nr
            if (l, r) == (0, n - 1):
                root = p
                break
    return bin_nodes, root


def _soup(n, rng, distinct=None):
    if distinct is None:
        v = rng.uniform(0, 1, (n * 3, 3)).astype(np.float32)
    else:
        base = rng.uniform(0, 1, (distinct * 3, 3)).astype(np.float32).reshape(distinct, 3, 3)
        v = base[rng.integers(0, distinct, n)].reshape(-1, 3)
    return [(v, None, None)]


@pytest.mark.parametrize("n,distinct,seed", [(2, None, 1), (3, None, 2), (17, None, 3), (1000, None, 4),
                                             (3000, None, 5), (2000, 20, 6), (500, 1, 7), (64, 3, 8)])
def test_bottom_up_order_builds_the_karras_tree(orc, n, distinct, seed):
    rng = np.random.default_rng(seed)
    _, rc, (ks, _, bn) = orc.build_blas(_soup(n, rng, distinct), 0, debug=True)
    assert rc == 0
    want = radix_tree_canonical(bn)
    for trial in range(3):
        order = list(range(n))
        random.Random(seed * 10 + trial).shuffle(order)
        got, root = bottom_up_tree(ks, order)
        np.testing.assert_array_equal(radix_tree_canonical(got), want)
        assert tuple(got[root][2:]) == (0, n - 1)
        # internal node i splits between keys i and i + 1
        left = got[:, 0].astype(np.int64)
        leaf = (left & LEAF) != 0
        assert np.array_equal(np.where(leaf, left & 0x7FFFFFFF, got[np.where(leaf, 0, left), 3]), np.arange(n - 1))
