"""The transcript hop run inside a tree's root launch (zc_merkle_commit_hop,
zc_fri_fold_commit_hop; PreFoldPairCommitRound(fuse_hop=True)) changes
nothing: fold rounds with and without it give the same roots, challenges,
folded layers, digest layers and final transcript state, for trees that fit
one subtree launch, trees with a fused top, and trees wider than the
level-wise threshold; built-in and run-time permutations; base and EF4
challenges; natural and bit-reversed codes."""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from zorch_gb300 import _lib  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")


CASES = [  # field, log message length, log blowup, rounds, challenge limbs, bit-reversed
    (0, 6, 1, 6, 4, False),
    (0, 12, 1, 10, 1, False),
    (0, 16, 1, 12, 4, False),
    (1, 10, 2, 9, 4, False),
    (1, 11, 1, 8, 1, True),
    (0, 13, 1, 11, 4, True),
]


@pytest.mark.parametrize("case", CASES)
def test_fused_hop_rounds_equal_separate_hops(orc, case):
    from zorch_gb300.coding import BitReversedReedSolomon, ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2, koalabear16_params
    from zorch_gb300.field import field_of, to_device
    from zorch_gb300.pcs import FoldState, PreFoldPairCommitRound, fold_rounds
    from zorch_gb300.transcript import DuplexTranscript

    field, log_k, log_b, rounds, limbs, br = case
    f = field_of(field)
    perm = (koalabear16_params(orc.load_koalabear_fixture()) if field == 1
            else Poseidon2.builtin(f))
    k = 1 << log_k
    code = (BitReversedReedSolomon(k, 1 << log_b, f, coset_shift=None) if br else
            ReedSolomon(k, 1 << log_b, f, coset_shift=f.generator))
    coeffs = orc.to_mont(field, np.random.default_rng(log_k).integers(
        0, f.p, size=k, dtype=np.uint64).astype(np.uint32))
    cw = code.encode(to_device(coeffs))
    seed = to_device(orc.to_mont(field, np.arange(5, dtype=np.uint32)))
    out = []
    for fuse in (False, True):
        rnd = PreFoldPairCommitRound(code, MerkleTree(perm), limbs, last_round=rounds - 1,
                                     fuse_hop=fuse)
        t = DuplexTranscript.new(perm).observe(seed)
        state, t, roots = fold_rounds(rnd, FoldState(cw), t, rounds)
        out.append((state, t, roots))
    (s0, t0, r0), (s1, t1, r1) = out
    for a, b in zip(r0, r1):
        assert torch.equal(a, b)
    for a, b in zip(s0.betas, s1.betas):
        assert torch.equal(a, b)
    for a, b in zip(s0.layers, s1.layers):
        assert torch.equal(a.codeword, b.codeword)
        assert torch.equal(a.digest_layers.flat, b.digest_layers.flat)
    assert torch.equal(s0.codeword, s1.codeword)
    assert torch.equal(t0.state, t1.state)
