"""Error behaviour of the reference-facing API, following the reference's own
negative tests: zorch/coding/testing/reed_solomon_test.py:154-161 (k-ary fold
forms), :263-271 (message length, power-of-two shapes), :302-312 (fold factor,
short k-ary layer), :355-357 (eval_domain size), :596-600 (length-one fold);
zorch/commit/testing/merkle_test.py:255-290 (matrix shape, leaf count) and
:333 (open index). The shape checks run before any device work, so the
first group needs no GPU."""

from __future__ import annotations

import pytest

torch = pytest.importorskip("torch")


def test_reed_solomon_rejects_non_power_of_two_shapes():
    from zorch_gb300.coding import BitReversedReedSolomon, ReedSolomon
    from zorch_gb300.field import BABYBEAR

    with pytest.raises(ValueError):
        ReedSolomon(3, 2, BABYBEAR)
    with pytest.raises(ValueError):
        ReedSolomon(4, 3, BABYBEAR)
    with pytest.raises(ValueError):
        BitReversedReedSolomon(6, 2, BABYBEAR)


def test_fold_factor_must_be_power_of_two_and_built():
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.field import BABYBEAR

    with pytest.raises(ValueError):
        ReedSolomon(16, 4, BABYBEAR, fold_factor=3)
    with pytest.raises(ValueError):
        ReedSolomon(16, 4, BABYBEAR, fold_factor=1)
    with pytest.raises(NotImplementedError):
        ReedSolomon(64, 4, BABYBEAR, fold_factor=32)


def test_wrong_message_length_raises_before_device_work():
    from zorch_gb300.coding import BitReversedReedSolomon, ReedSolomon
    from zorch_gb300.field import BABYBEAR

    msg = torch.zeros(5, dtype=torch.int32)
    with pytest.raises(ValueError):
        ReedSolomon(4, 2, BABYBEAR).encode(msg)
    with pytest.raises(ValueError):
        BitReversedReedSolomon(4, 2, BABYBEAR).encode(msg)
    with pytest.raises(ValueError):
        ReedSolomon(4, 2, BABYBEAR).encode(torch.zeros((4, 3), dtype=torch.int32), ef4=True)


def test_short_layers_are_rejected_by_the_folds():
    from zorch_gb300.coding import BitReversedReedSolomon, ReedSolomon
    from zorch_gb300.field import BABYBEAR

    beta = torch.zeros(1, dtype=torch.int32)
    with pytest.raises(ValueError):
        ReedSolomon(4, 2, BABYBEAR).fold(torch.zeros(1, dtype=torch.int32), beta)
    with pytest.raises(ValueError):
        BitReversedReedSolomon(4, 2, BABYBEAR).fold(torch.zeros(1, dtype=torch.int32), beta)
    with pytest.raises(ValueError):
        ReedSolomon(16, 4, BABYBEAR, fold_factor=4).fold_group(
            torch.zeros(2, dtype=torch.int32), beta)


def test_eval_domain_rejects_non_power_of_two():
    from zorch_gb300.coding import eval_domain
    from zorch_gb300.field import BABYBEAR

    with pytest.raises(ValueError):
        eval_domain(BABYBEAR, 6, device="cpu")


def test_host_input_must_be_page_locked():
    from zorch_gb300.field import BABYBEAR, to_mont_from_host

    with pytest.raises(ValueError):
        to_mont_from_host(BABYBEAR, torch.zeros(8, dtype=torch.int32))


@pytest.mark.gpu
def test_merkle_and_strided_shape_errors():
    from zorch_gb300 import _lib
    from zorch_gb300.commit import MerkleTree, Poseidon2, StridedMerkleTree

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")
    perm = Poseidon2.builtin()
    tree = MerkleTree(perm)
    with pytest.raises(ValueError):
        tree.commit(torch.zeros(8, dtype=torch.int32, device="cuda"))        # not 2-D
    with pytest.raises(ValueError):
        tree.commit(torch.zeros((6, 2), dtype=torch.int32, device="cuda"))   # 6 leaves
    m = torch.zeros((8, 2), dtype=torch.int32, device="cuda")
    _, layers = tree.commit(m)
    with pytest.raises(IndexError):
        tree.open(m, layers, 8)
    with pytest.raises(ValueError):
        StridedMerkleTree(perm, 3)
    with pytest.raises(ValueError):
        StridedMerkleTree(perm, 16).commit(m)                                # rpq > leaves


@pytest.mark.gpu
def test_open_paths_reject_malformed_requests():
    from zorch_gb300 import _lib
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2
    from zorch_gb300.field import BABYBEAR
    from zorch_gb300.pcs import BasefoldProver
    from zorch_gb300.transcript import DuplexTranscript

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")
    perm = Poseidon2.builtin()
    prover = BasefoldProver(ReedSolomon(16, 2, BABYBEAR, coset_shift=31),
                            MerkleTree(perm, column_major=True), num_queries=2)
    t = DuplexTranscript.new(perm)
    z = torch.zeros((4, 4), dtype=torch.int32, device="cuda")
    with pytest.raises(ValueError):
        prover.open_batch([], z, t)                                          # no matrices
    _, data = prover.commit_columns(torch.zeros((2, 16), dtype=torch.int32, device="cuda"))
    with pytest.raises(ValueError):
        prover.open_batch([data], z[:3], t)                                  # 3 != log2(16)
    with pytest.raises(ValueError):
        t.grind(32)
    with pytest.raises(ValueError):
        t.check_witness(torch.zeros(2, dtype=torch.int32, device="cuda"), pow_bits=1)
