"""The oracle's query-strided Merkle tree (StridedMerkleTree.commit,
zorch/commit/strided_merkle.py:100-152) against the reference's structural
checks (zorch/commit/testing/strided_merkle_test.py:61-116), no GPU."""

from __future__ import annotations

import numpy as np

import oracle.oracle as o


def _m(h, w=3):
    return o.to_mont(o.KOALABEAR, np.arange(h * w).reshape(h, w))


def test_rows_per_query_1_is_the_plain_tree():
    p2 = o.Poseidon2.koalabear16_golden()
    a, b = o.strided_merkle_commit(p2, _m(8), 1), o.merkle_commit_rows(p2, _m(8))
    assert len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b))


def test_layer_shapes_and_coset_roundtrip():
    p2 = o.Poseidon2.koalabear16_golden()
    m = _m(16)
    layers = o.strided_merkle_commit(p2, m, 4)
    assert [l.shape for l in layers] == [(4, 8), (2, 8), (1, 8)]
    root = layers[-1][0]
    for idx in range(4):
        nodes = [p2.hash(r) for r in m[idx::4]]
        while len(nodes) > 1:
            nodes = [p2.compress(nodes[2 * x], nodes[2 * x + 1]) for x in range(len(nodes) // 2)]
        node, i = nodes[0], idx
        for lv in layers[:-1]:
            node = p2.compress(node, lv[i ^ 1]) if i % 2 == 0 else p2.compress(lv[i ^ 1], node)
            i //= 2
        assert np.array_equal(node, root)


def test_rows_per_query_equal_height_is_one_node():
    p2 = o.Poseidon2.koalabear16_golden()
    layers = o.strided_merkle_commit(p2, _m(8), 8)
    assert [l.shape for l in layers] == [(1, 8)]
