"""FriProver.prove on the GPU (zorch/pcs/fri/prover.py:101-187): v = f(z)
(zc_eval_poly), the DEEP quotient layer (zc_deep_quotient), the fold rounds,
the query openings and f's opening -- proof bytes equal to the oracle's,
including config 3 at full size (2^22 coefficients, blowup 2, 15 EF4-challenge
rounds to 2^8, 100 queries); the host FriVerifier accepts the GPU's proofs and
rejects tampered ones, for natural and bit-reversed codes."""

from __future__ import annotations

import dataclasses

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


def _perms(orc, field):
    from zorch_gb300.commit import Poseidon2, koalabear16_params
    from zorch_gb300.field import field_of

    if field == 1:
        return orc.Poseidon2.koalabear16_golden(), koalabear16_params(orc.load_koalabear_fixture())
    return orc.Poseidon2.babybear16(), Poseidon2.builtin(field_of(field))


def _prove(orc, field, log_k, log_b, rounds, queries, limbs, zs, shift, bit_reversed=False,
           seed=1):
    from zorch_gb300.coding import BitReversedReedSolomon, ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.field import field_of, to_device
    from zorch_gb300.pcs import FriParams, FriProver
    from zorch_gb300.stage import OpeningClaim, OpeningWitness
    from zorch_gb300.transcript import DuplexTranscript

    f = field_of(field)
    p2, perm = _perms(orc, field)
    k = 1 << log_k
    polys = [orc.to_mont(field, np.random.default_rng(seed + i).integers(
        0, f.p, size=k, dtype=np.uint64).astype(np.uint32)) for i in range(len(zs))]
    code = (BitReversedReedSolomon(k, 1 << log_b, f, coset_shift=shift) if bit_reversed else
            ReedSolomon(k, 1 << log_b, f, coset_shift=shift))
    params = FriParams(code, MerkleTree(perm), rounds, queries, limbs)
    prover = FriProver(params)
    roots, data = prover.commit([to_device(c) for c in polys])
    res = prover.prove(OpeningClaim(roots, list(zs)), OpeningWitness(data),
                       DuplexTranscript.new(perm))
    return f, p2, perm, params, polys, roots, res


CASES = [  # field, log_k, log_blowup, rounds, queries, challenge limbs, z, coset shift
    (1, 2, 1, 2, 3, 1, 2, None),
    (1, 2, 1, 2, 3, 1, 2, 3),
    (0, 10, 1, 10, 8, 1, 5, 31),
    (0, 10, 1, 10, 8, 4, (5, 7, 11, 13), 31),
    (0, 12, 2, 12, 16, 4, 2, 31),
    (1, 8, 1, 8, 5, 4, (3, 1, 4, 1), None),
    (0, 14, 1, 14, 32, 4, (123, 4, 5, 6), 31),
]
# rounds = log2(message_len) in every case: the quotient (degree < k - 1)
# then folds to a constant final layer, which is what the verifier checks
# (ReedSolomon.check_final, zorch/coding/reed_solomon.py:309-313).


def _oracle_bytes(orc, f, p2, polys, zs, log_b, rounds, queries, limbs, shift):
    t = orc.Transcript(p2)
    out, vals = b"", []
    sh = f.mont(shift) if shift is not None else 0
    for coeffs, z in zip(polys, zs):
        cw = orc.rs_encode(f.id, coeffs, log_b, sh)
        n = cw.size
        layers = orc.merkle_commit(p2, cw, n // 2, 2, 1, n // 2)
        zw = np.asarray([f.mont(x) for x in (z if isinstance(z, tuple) else (z,))], np.uint32)
        pf = orc.fri_open(p2, f.id, coeffs, cw, layers, zw, rounds, queries, limbs, t, sh)
        out += pf.to_bytes()
        vals.append(pf.value)
    return out, vals


@pytest.mark.parametrize("case", CASES)
def test_fri_prove_bytes_match_oracle_and_verify(orc, case):
    from zorch_gb300.field import to_host
    from zorch_gb300.pcs import FriVerifier
    from zorch_gb300.stage import OpeningClaim

    field, log_k, log_b, rounds, queries, limbs, z, shift = case
    zs = [z, (z if isinstance(z, int) else z[::-1])]
    f, p2, perm, params, polys, roots, res = _prove(orc, field, log_k, log_b, rounds, queries,
                                                    limbs, zs, shift)
    proofs = res.reduction_proof.proof
    got = b"".join(p.to_bytes() for p in proofs)
    want, vals = _oracle_bytes(orc, f, p2, polys, zs, log_b, rounds, queries, limbs, shift)
    assert got == want
    assert np.array_equal(to_host(res.reduction_proof.values).reshape(-1),
                          np.concatenate(vals))
    vr = FriVerifier(params).verify(OpeningClaim(roots, zs), res.reduction_proof, None)
    assert vr.ok


@pytest.mark.parametrize("rounds", [15, 22])
def test_fri_prove_config3_full_size(orc, rounds):
    """Config 3's polynomial: 2^22 BabyBear coefficients, blowup 2, shift 31,
    EF4 challenges, 100 queries, opened at an EF4 point. With 15 rounds (the
    config's fold down to 2^8) the proof bytes equal the oracle's; with 22
    rounds (down to a constant, the reference verifier's final check) they do
    too and the verifier accepts."""
    from zorch_gb300.pcs import FriVerifier
    from zorch_gb300.stage import OpeningClaim

    z = (987654321, 12345, 678, 9)
    f, p2, perm, params, polys, roots, res = _prove(orc, 0, 22, 1, rounds, 100, 4, [z], 31)
    got = res.reduction_proof.proof[0].to_bytes()
    want, _ = _oracle_bytes(orc, f, p2, polys, [z], 1, rounds, 100, 4, 31)
    assert got == want
    if rounds == 22:
        assert FriVerifier(params).verify(OpeningClaim(roots, [z]), res.reduction_proof,
                                          None).ok


@pytest.mark.parametrize("case", [(1, 2, 1, 2, 3, 1, 2, None),
                                  (0, 10, 1, 10, 12, 4, (7, 1, 2, 3), 31)])
def test_fri_bit_reversed_round_trip(case):
    """The bit-reversed code (FriBitReversedRoundTripTest,
    zorch/pcs/fri/testing/fri_test.py:121-150): honest openings verify, a
    wrong value is rejected."""
    from zorch_gb300.pcs import FriVerifier
    from zorch_gb300.stage import OpeningClaim, OpeningProof

    field, log_k, log_b, rounds, queries, limbs, z, shift = case
    from oracle import oracle as orc

    f, p2, perm, params, polys, roots, res = _prove(orc, field, log_k, log_b, rounds, queries,
                                                    limbs, [z], shift, bit_reversed=True)
    ver = FriVerifier(params)
    claim = OpeningClaim(roots, [z])
    assert ver.verify(claim, res.reduction_proof, None).ok
    bad = res.reduction_proof.values.clone()
    bad.view(-1)[0] += 1
    assert not ver.verify(claim, OpeningProof(bad, res.reduction_proof.proof), None).ok


def test_fri_prove_tamper_and_errors(orc):
    from zorch_gb300.pcs import FriVerifier
    from zorch_gb300.stage import OpeningClaim, OpeningProof, OpeningWitness
    from zorch_gb300.transcript import DuplexTranscript

    f, p2, perm, params, polys, roots, res = _prove(orc, 0, 10, 1, 10, 8, 4, [5], 31)
    ver = FriVerifier(params)
    claim = OpeningClaim(roots, [5])
    pf = res.reduction_proof.proof[0]
    fin = pf.final_layer.clone()
    fin.view(-1)[0] += 1
    bad = OpeningProof(res.reduction_proof.values, [dataclasses.replace(pf, final_layer=fin)])
    assert not ver.verify(claim, bad, None).ok
    from zorch_gb300.pcs import FriProver

    prover = FriProver(params)
    _, data = prover.commit([torch.zeros(1 << 10, dtype=torch.int32, device="cuda")])
    with pytest.raises(ValueError):  # one polynomial, two points
        prover.prove(OpeningClaim(roots, [5, 6]), OpeningWitness(data),
                     DuplexTranscript.new(perm))
    short = dataclasses.replace(pf, fri_roots=pf.fri_roots[:0], query_openings=[])
    with pytest.raises(ValueError):
        ver.verify(claim, OpeningProof(res.reduction_proof.values, [short]), None)
