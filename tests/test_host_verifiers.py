"""The product's host-side verifiers on a machine without a GPU: Poseidon2
handles fall back to host-only constants, and BasefoldVerifier
(zorch/pcs/basefold/verifier.py:429-540) and stacked_basefold_verify
(zorch/pcs/jagged/verifier.py:165-356) accept the proofs the oracle's
restated provers produce and reject tampered ones; the host duplex transcript
squeezes what the oracle's does. The provers here are the oracle's, so this
cross-checks the product verifiers against an independent prover."""

from __future__ import annotations

import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")



def _verdict(verifier, *args) -> bool:
    """The boolean of BasefoldVerifier.verify_batch's (ok, transcript)."""
    ok, _ = verifier.verify_batch(*args)
    return ok

def _t(a) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.uint32)).view(np.int32))


def rand_mont(orc, field, shape, seed):
    x = np.random.default_rng(seed).integers(0, orc.MODULUS[field], size=shape, dtype=np.uint64)
    return orc.to_mont(field, x.astype(np.uint32))


def test_host_transcript_matches_the_oracle(orc):
    from zorch_gb300.commit import koalabear16_params
    from zorch_gb300.transcript import HostDuplexTranscript

    perm = koalabear16_params(orc.load_koalabear_fixture())
    ht = HostDuplexTranscript(perm)
    ot = orc.Transcript(orc.Poseidon2.koalabear16_golden())
    for i, (m, n) in enumerate([(3, 1), (8, 4), (13, 0), (0, 9), (21, 2)]):
        vals = rand_mont(orc, 1, (m,), 10 + i)
        ht, got = ht.observe_and_sample(vals, n)
        ot.observe(vals)
        assert np.array_equal(got, ot.sample(n))


def _basefold_case(orc, widths=(3, 2), v=8, queries=6):
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2
    from zorch_gb300.field import BABYBEAR
    from zorch_gb300.pcs import BasefoldProof, BasefoldVerifier
    from zorch_gb300.commit import Opening

    cperm = orc.Poseidon2.babybear16()
    mats = []
    for i, w in enumerate(widths):
        cols = rand_mont(orc, 0, (w, 1 << v), 40 + i)
        cw = orc.rs_encode(0, cols, 1, BABYBEAR.mont(31))
        mats.append({"cols": cols, "codeword": cw, "layers": orc.merkle_commit_columns(cperm, cw)})
    z = rand_mont(orc, 0, (v, 4), 50)
    want = orc.basefold_open(cperm, 0, mats, z, 1, BABYBEAR.mont(31), queries,
                             orc.Transcript(cperm))
    proof = BasefoldProof(
        _t(want["uni_msgs"]), _t(want["fri_roots"]), _t(want["final_poly"]),
        [Opening(_t(r), _t(p)) for r, p in want["component_openings"]],
        [Opening(_t(r), _t(p)) for r, p in want["query_openings"]],
        _t(want["positions"].astype(np.uint32)))
    verifier = BasefoldVerifier(ReedSolomon(1 << v, 2, BABYBEAR, coset_shift=31),
                                MerkleTree(Poseidon2.builtin(BABYBEAR), column_major=True),
                                num_queries=queries)
    roots = [_t(m["layers"][-1][0]) for m in mats]
    values = [_t(x) for x in want["values"]]
    return verifier, roots, _t(z), values, proof


def test_basefold_verifier_accepts_the_oracle_proof_on_cpu(orc):
    verifier, roots, z, values, proof = _basefold_case(orc)
    assert _verdict(verifier, roots, [z], values, proof)


def test_basefold_stage_form_on_cpu(orc):
    """The reference's stage seam (zorch/pcs/basefold/verifier.py:99-113):
    verify(OpeningClaim(commitment, [z]), OpeningProof(values, proof),
    transcript) on a single committed matrix -> VerifyResult(TrivialClaim(),
    transcript, ok); a wrong value is a False verdict; two points raise."""
    from zorch_gb300.stage import OpeningClaim, OpeningProof, TrivialClaim

    verifier, roots, z, values, proof = _basefold_case(orc, widths=(5,))
    vr = verifier.verify(OpeningClaim(roots[0], [z]), OpeningProof(values[0], proof))
    assert vr.ok and vr.reduced_claim == TrivialClaim()
    bad = values[0].clone()
    bad.view(-1)[0] ^= 1
    assert not verifier.verify(OpeningClaim(roots[0], [z]), OpeningProof(bad, proof)).ok
    with pytest.raises(ValueError):
        verifier.verify(OpeningClaim(roots[0], [z, z]), OpeningProof(values[0], proof))


def test_basefold_verifier_rejects_tampering_on_cpu(orc):
    verifier, roots, z, values, proof = _basefold_case(orc)

    def flip(t, i):
        t = t.clone()
        t.view(-1)[i] ^= 1
        return t

    assert not _verdict(verifier, roots, [z], values,
                               dataclasses.replace(proof, uni_msgs=flip(proof.uni_msgs, 2)))
    assert not _verdict(verifier, roots, [z], values,
                               dataclasses.replace(proof, final_poly=flip(proof.final_poly, 0)))
    assert not _verdict(verifier, roots, [z], [flip(values[0], 1), *values[1:]], proof)
    q = proof.query_openings[1]
    bad = dataclasses.replace(q, row=flip(q.row, 3))
    assert not _verdict(verifier, roots, [z], values, dataclasses.replace(
        proof, query_openings=[proof.query_openings[0], bad, *proof.query_openings[2:]]))
    assert not _verdict(verifier, [flip(roots[0], 5), *roots[1:]], [z], values, proof)


def test_stacked_verifier_accepts_the_oracle_proof_on_cpu(orc):
    """The SP1 stacked open as the oracle restates it (SP1's KoalaBear
    Poseidon2), verified by the product's host verifier; a consistent
    statement: dense_eval is the MLE of the batch evaluations."""
    from zorch_gb300.coding import BitReversedReedSolomon
    from zorch_gb300.commit import Poseidon2, SingleMatrixCommitmentScheme
    from zorch_gb300.field import KOALABEAR
    from zorch_gb300.jagged import StackedOpenProof, _ef_eval_mle_msb, stacked_basefold_verify
    from zorch_gb300.transcript import HostDuplexTranscript

    d = orc.load_sp1_fixture()
    gperm = Poseidon2.from_params(KOALABEAR, d["alpha"], d["external_initial"],
                                  d["external_terminal"], d["internal_rc"], d["internal_diag"],
                                  d["internal_j_scale"])
    cperm = orc.sp1_koalabear16()
    v, widths, queries, f = 6, (3, 2), 5, KOALABEAR
    S, n = 1 << v, 1 << (v + 1)
    blocks = [rand_mont(orc, 1, (w, S), 60 + i) for i, w in enumerate(widths)]
    z = rand_mont(orc, 1, (v + 3, 4), 70)
    probe = orc.sp1_stacked_open(cperm, 1, blocks, z, np.zeros(4, np.uint32), v, 1, queries,
                                 orc.Transcript(cperm))
    flat = [f.ef_from_mont(r) for e in probe["batch_evals"] for r in e.reshape(-1, 4)]
    lead = [f.ef_from_mont(r) for r in z[:3]]
    de = np.array(f.ef_to_mont(_ef_eval_mle_msb(f, flat + [(0, 0, 0, 0)] * (8 - len(flat)),
                                                lead)), np.uint32)
    want = orc.sp1_stacked_open(cperm, 1, blocks, z, de, v, 1, queries, orc.Transcript(cperm),
                                pow_bits=4)
    comps, comp_ops = [], []
    for b in blocks:
        cw = orc.rs_encode_bitrev(1, b, 1)
        layers = orc.merkle_commit_columns(cperm, cw)
        comps.append(_t(orc.smcs_bind_root(cperm, layers[-1][0], n.bit_length() - 1,
                                           b.shape[0])))
        rows, paths = orc.merkle_open(cw, n, b.shape[0], 1, n, layers, want["positions"])
        comp_ops.append((_t(rows), _t(paths)))
    proof = StackedOpenProof(
        comps, _t(want["raw_roots"]), _t(want["bound_roots"]),
        _t(want["uni_msgs"]).reshape(v, 2, 4), _t(want["final_poly"]), _t(want["pow_witness"]),
        [_t(e) for e in want["batch_evals"]], comp_ops,
        [(_t(r), _t(p)) for r, p in want["query_openings"]],
        _t(want["positions"].astype(np.uint32)))
    smcs = SingleMatrixCommitmentScheme(gperm)
    code = BitReversedReedSolomon(S, 2, f)
    _, ok = stacked_basefold_verify(smcs, code, list(widths), _t(z), de, v, proof,
                                    HostDuplexTranscript(gperm), num_queries=queries, pow_bits=4)
    assert ok
    bad = dataclasses.replace(proof, final_poly=_t(want["final_poly"] ^ np.uint32(1)))
    _, ok = stacked_basefold_verify(smcs, code, list(widths), _t(z), de, v, bad,
                                    HostDuplexTranscript(gperm), num_queries=queries, pow_bits=4)
    assert not ok


def test_device_entries_refuse_host_only_handles():
    """Without a CUDA device a handle is host-only; a device entry given one
    returns an error status instead of launching."""
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present: handles carry device constants")
    from zorch_gb300 import _lib
    from zorch_gb300.commit import Poseidon2
    from zorch_gb300.field import BABYBEAR

    p = Poseidon2.builtin(BABYBEAR)
    buf = np.zeros(16, np.uint32)
    st = _lib.lib().zc_poseidon2_permute(p.handle, buf.ctypes.data, 1, None)
    assert st != 0
    assert b"no device copy" in _lib.lib().zc_last_error()
