"""Query-strided Merkle tree on the GPU == the oracle's restatement of the
reference's strided levels, plus the reference's structural checks
(zorch/commit/testing/strided_merkle_test.py:61-190): rows_per_query = 1 is
the plain tree; every query's opened coset and stored path rebuild the root;
rows_per_query = height collapses to one node; a tampered row is rejected."""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from zorch_gb300 import _lib  # noqa: E402
from zorch_gb300.field import to_device, to_host  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")


@pytest.fixture(scope="module")
def perms(orc):
    from zorch_gb300.commit import Poseidon2, koalabear16_params

    return {0: (Poseidon2.builtin(0), orc.Poseidon2.babybear16()),
            1: (koalabear16_params(orc.load_koalabear_fixture()),
                orc.Poseidon2.koalabear16_golden())}


def _matrix(orc, field, h, w, seed):
    x = np.random.default_rng(seed).integers(0, orc.MODULUS[field], (h, w), dtype=np.uint64)
    return orc.to_mont(field, x.astype(np.uint32))


@pytest.mark.parametrize("field", [0, 1])
@pytest.mark.parametrize("h,w,rpq", [(16, 3, 4), (8, 3, 1), (1 << 12, 8, 16), (1 << 10, 20, 2),
                                     (64, 1, 64), (1 << 16, 4, 8)])
def test_strided_commit_matches_oracle(orc, perms, field, h, w, rpq):
    from zorch_gb300.commit import StridedMerkleTree

    gpu, cpu = perms[field]
    m = _matrix(orc, field, h, w, h + w + rpq)
    tree = StridedMerkleTree(gpu, rpq)
    root, layers = tree.commit(to_device(m).reshape(h, w))
    want = orc.strided_merkle_commit(cpu, m, rpq)
    assert len(layers) == len(want)
    for got, exp in zip(layers, want):
        assert np.array_equal(to_host(got), exp)


def test_rows_per_query_1_is_the_plain_tree(orc, perms):
    from zorch_gb300.commit import MerkleTree, StridedMerkleTree

    gpu, _ = perms[1]
    m = to_device(_matrix(orc, 1, 256, 5, 3)).reshape(256, 5)
    _, a = StridedMerkleTree(gpu, 1).commit(m)
    _, b = MerkleTree(gpu).commit(m)
    assert np.array_equal(to_host(a.flat), to_host(b.flat))


@pytest.mark.parametrize("rpq", [1, 4, 16])
def test_open_reconstruct_roundtrip_and_tamper(orc, perms, rpq):
    from zorch_gb300.commit import Opening, StridedMerkleTree

    gpu, _ = perms[0]
    h, w = 256, 3
    m = to_device(_matrix(orc, 0, h, w, 9)).reshape(h, w)
    tree = StridedMerkleTree(gpu, rpq)
    root, layers = tree.commit(m)
    s = tree.query_stride(h)
    idx = torch.arange(s, dtype=torch.int32, device="cuda")
    op = tree.open(m, layers, idx)
    assert op.row.shape == (s, rpq, w)
    for i in range(0, s, max(1, s // 8)):
        assert torch.equal(op.row[i], tree.opened_rows(m, i))
        assert tree.verify(root, i, Opening(op.row[i], op.path[:, i]))
    bad = op.row[1].clone()
    bad[0, 0] ^= 1
    assert not tree.verify(root, 1, Opening(bad, op.path[:, 1]))
    with pytest.raises(IndexError):
        tree.open(m, layers, torch.tensor([s], dtype=torch.int32, device="cuda"))


def test_rows_per_query_equal_height_is_one_node(orc, perms):
    from zorch_gb300.commit import StridedMerkleTree

    gpu, _ = perms[0]
    m = to_device(_matrix(orc, 0, 8, 3, 4)).reshape(8, 3)
    root, layers = StridedMerkleTree(gpu, 8).commit(m)
    assert len(layers) == 1 and layers.num_leaves == 1
    assert torch.equal(layers[0][0], root)
