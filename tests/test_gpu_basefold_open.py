"""Basefold batch open on the GPU (BasefoldProver.open_batch) == the oracle's
restatement, bit for bit: per-matrix evaluations, sumcheck messages, fold
roots, the final codeword, query positions and every opening; the host
verifier (BasefoldVerifier) accepts the proof and rejects tampered ones
(zorch/pcs/basefold/testing/basefold_test.py:171-243 are the reference's
round-trip and tamper cases)."""

from __future__ import annotations

import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from zorch_gb300 import _lib  # noqa: E402
from zorch_gb300.field import BABYBEAR, KOALABEAR, to_device, to_host  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")


def rand_mont(orc, field, shape, seed):
    x = np.random.default_rng(seed).integers(0, orc.MODULUS[field], size=shape, dtype=np.uint64)
    return orc.to_mont(field, x.astype(np.uint32))


def dev(x):
    return to_device(np.asarray(x, np.uint32))


def _perms(orc, field):
    from zorch_gb300.commit import Poseidon2, koalabear16_params

    if field == 0:
        return Poseidon2.builtin(BABYBEAR), orc.Poseidon2.babybear16()
    return koalabear16_params(orc.load_koalabear_fixture()), orc.Poseidon2.koalabear16_golden()


CASES = [  # field, widths, v, log_blowup, shift, queries
    (0, (1,), 6, 1, 31, 4),
    (0, (3, 2), 10, 2, 31, 8),
    (1, (4,), 8, 1, None, 5),
    (0, (16, 5, 1), 12, 1, 31, 16),
    (1, (2,), 1, 1, 3, 3),
]


def _open(orc, field, widths, v, log_blowup, shift, queries):
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.field import field_of
    from zorch_gb300.pcs import BasefoldProver, BasefoldVerifier
    from zorch_gb300.transcript import DuplexTranscript

    f = field_of(field)
    gperm, cperm = _perms(orc, field)
    code = ReedSolomon(1 << v, 1 << log_blowup, f, coset_shift=shift)
    tree = MerkleTree(gperm, column_major=True)
    prover = BasefoldProver(code, tree, num_queries=queries)
    verifier = BasefoldVerifier(code, tree, num_queries=queries)
    mats, datas, roots = [], [], []
    for i, w in enumerate(widths):
        cols = rand_mont(orc, field, (w, 1 << v), 100 + 7 * i + v)
        root, data = prover.commit_columns(dev(cols).reshape(w, 1 << v))
        roots.append(root)
        datas.append(data)
        cw = to_host(data.codeword)
        mats.append({"cols": cols, "codeword": cw, "layers": orc.merkle_commit_columns(cperm, cw)})
    z = rand_mont(orc, field, (v, 4), 900 + v)
    values, proof, _ = prover.open_batch(datas, dev(z).reshape(v, 4),
                                         DuplexTranscript.new(gperm))
    sh = f.mont(shift) if shift else 0
    want = orc.basefold_open(cperm, field, mats, z, log_blowup, sh, queries, orc.Transcript(cperm))
    return verifier, roots, dev(z).reshape(v, 4), values, proof, want


def _verdict(verifier, *args) -> bool:
    """The boolean of BasefoldVerifier.verify_batch's (ok, transcript)."""
    ok, _ = verifier.verify_batch(*args)
    return ok


@pytest.mark.parametrize("case", CASES)
def test_basefold_open_matches_oracle(orc, case):
    verifier, roots, z, values, proof, want = _open(orc, *case)
    for got, w in zip(values, want["values"]):
        assert np.array_equal(to_host(got), w)
    assert np.array_equal(to_host(proof.uni_msgs), want["uni_msgs"])
    assert np.array_equal(to_host(proof.fri_roots), want["fri_roots"])
    assert np.array_equal(to_host(proof.final_poly), want["final_poly"])
    assert np.array_equal(to_host(proof.positions).view(np.int32), want["positions"])
    for op, (rows, paths) in zip(proof.component_openings, want["component_openings"]):
        assert np.array_equal(to_host(op.row), rows) and np.array_equal(to_host(op.path), paths)
    for op, (rows, paths) in zip(proof.query_openings, want["query_openings"]):
        assert np.array_equal(to_host(op.row), rows) and np.array_equal(to_host(op.path), paths)
    assert _verdict(verifier, roots, [z], values, proof)


def test_basefold_verifier_rejects_tampering(orc):
    verifier, roots, z, values, proof, _ = _open(orc, *CASES[1])
    assert _verdict(verifier, roots, [z], values, proof)
    bad_msgs = proof.uni_msgs.clone()
    bad_msgs[0, 0] ^= 1
    assert not _verdict(verifier, roots, [z], values, dataclasses.replace(proof, uni_msgs=bad_msgs))
    comp = proof.component_openings[0]
    bad_row = comp.row.clone()
    bad_row[0, 0] ^= 1
    bad_comp = dataclasses.replace(comp, row=bad_row)
    assert not _verdict(verifier, roots, [z], values, dataclasses.replace(
        proof, component_openings=[bad_comp, *proof.component_openings[1:]]))
    bad_vals = [values[0].clone(), *values[1:]]
    bad_vals[0][0, 1] ^= 1
    assert not _verdict(verifier, roots, [z], bad_vals, proof)
    bad_final = proof.final_poly.clone()
    bad_final[0, 0] ^= 1
    assert not _verdict(verifier, roots, [z], values, dataclasses.replace(proof, final_poly=bad_final))
    q = proof.query_openings[2]
    bad_q = dataclasses.replace(q, row=q.row.clone())
    bad_q.row[1, 3] ^= 1
    assert not _verdict(verifier, roots, [z], values, dataclasses.replace(
        proof, query_openings=[*proof.query_openings[:2], bad_q, *proof.query_openings[3:]]))


def test_eval_mle_and_eq_match_oracle(orc):
    from zorch_gb300.field import BABYBEAR as F

    L = _lib.lib()
    for w, m in ((3, 5), (2, 13), (1, 0), (4, 16)):
        cols = rand_mont(orc, 0, (w, 1 << m), 31 + m)
        z = rand_mont(orc, 0, (max(m, 1), 4), 32 + m)[:m]
        out = torch.empty((w, 4), dtype=torch.int32, device="cuda")
        nb = L.zc_eval_mle_workspace_bytes(w, m)
        ws = torch.empty((nb + 15) // 4, dtype=torch.int32, device="cuda")
        zd = dev(z if m else np.zeros((1, 4), np.uint32))
        _lib.check(L.zc_eval_mle(F.id, dev(cols).data_ptr(), w, m, zd.data_ptr(), out.data_ptr(),
                                 ws.data_ptr(), nb, 0), "eval_mle")
        assert np.array_equal(to_host(out), orc.eval_mle_base(0, cols, z)), (w, m)
    for m in (0, 3, 12, 13, 17):
        z = rand_mont(orc, 1, (max(m, 1), 4), 50 + m)[:m]
        out = torch.empty(((1 << m), 4), dtype=torch.int32, device="cuda")
        nb = L.zc_eq_expand_workspace_bytes(m)
        ws = torch.empty(max((nb + 15) // 4, 4), dtype=torch.int32, device="cuda")
        zd = dev(z if m else np.zeros((1, 4), np.uint32))
        _lib.check(L.zc_eq_expand(KOALABEAR.id, zd.data_ptr(), m, out.data_ptr(), ws.data_ptr(),
                                  nb, 0), "eq_expand")
        assert np.array_equal(to_host(out), orc.eq_expand(1, z)), m


def test_ef4_inverse_matches_oracle(orc):
    L = _lib.lib()
    for field in (0, 1):
        a = rand_mont(orc, field, (37, 4), 80 + field)
        a[5] = 0  # zero maps to zero
        a[6, 1:] = 0  # a base-field element
        out = torch.empty((37, 4), dtype=torch.int32, device="cuda")
        _lib.check(L.zc_ef4_inv(field, dev(a).data_ptr(), out.data_ptr(), 37, 0), "ef4_inv")
        got = to_host(out)
        for i in range(37):
            assert np.array_equal(got[i], orc.ef4_inv(field, a[i])), (field, i)


def test_graphed_open_replays_the_eager_open(orc):
    """GraphedBasefoldOpen: one capture, replays at new points and transcripts
    give the eager open's values and proof bytes."""
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2
    from zorch_gb300.pcs import BasefoldProver, GraphedBasefoldOpen
    from zorch_gb300.transcript import DuplexTranscript

    v, perm = 11, Poseidon2.builtin(BABYBEAR)
    code = ReedSolomon(1 << v, 2, BABYBEAR, coset_shift=31)
    prover = BasefoldProver(code, MerkleTree(perm, column_major=True), num_queries=9)
    datas = []
    for i, w in enumerate((5, 3)):
        _, d = prover.commit_columns(dev(rand_mont(orc, 0, (w, 1 << v), 300 + i)).reshape(w, -1))
        datas.append(d)
    graphed = GraphedBasefoldOpen(prover, datas)
    for k in range(3):
        z = dev(rand_mont(orc, 0, (v, 4), 400 + k)).reshape(v, 4)
        t = DuplexTranscript.new(perm).observe(dev(rand_mont(orc, 0, (k + 1,), 500 + k)))
        values, proof, t_out = prover.open_batch(datas, z, t)
        g_values, g_proof, g_t = graphed.replay(z, t)
        for a, b in zip(values, g_values):
            assert torch.equal(a, b)
        assert torch.equal(proof.uni_msgs, g_proof.uni_msgs)
        assert torch.equal(proof.fri_roots, g_proof.fri_roots)
        assert torch.equal(proof.final_poly, g_proof.final_poly)
        assert torch.equal(proof.positions, g_proof.positions)
        for a, b in zip(proof.component_openings + proof.query_openings,
                        g_proof.component_openings + g_proof.query_openings):
            assert torch.equal(a.row, b.row) and torch.equal(a.path, b.path)
        assert torch.equal(t_out.state, g_t.state)


def test_basefold_prove_stage_form(orc):
    """BasefoldProver.prove / BasefoldVerifier.verify, the reference's stage
    seam (zorch/pcs/basefold/prover.py:195-209, verifier.py:99-113): the
    single-matrix open equals open_batch on that matrix, and verifies."""
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.field import BABYBEAR
    from zorch_gb300.pcs import BasefoldProver, BasefoldVerifier
    from zorch_gb300.stage import OpeningClaim, OpeningWitness, TrivialClaim
    from zorch_gb300.transcript import DuplexTranscript

    gperm, _ = _perms(orc, 0)
    v, w, q = 10, 6, 12
    code = ReedSolomon(1 << v, 2, BABYBEAR, coset_shift=31)
    tree = MerkleTree(gperm, column_major=True)
    prover = BasefoldProver(code, tree, num_queries=q)
    root, data = prover.commit_columns(dev(rand_mont(orc, 0, (w, 1 << v), 5)).reshape(w, 1 << v))
    z = dev(rand_mont(orc, 0, (v, 4), 6)).reshape(v, 4)
    res = prover.prove(OpeningClaim(root, [z]), OpeningWitness(data), DuplexTranscript.new(gperm))
    assert res.reduced_claim == TrivialClaim()
    vals, proof, _ = prover.open_batch([data], [z], DuplexTranscript.new(gperm))
    assert torch.equal(res.reduction_proof.values, vals[0])
    assert res.reduction_proof.proof.to_bytes() == proof.to_bytes()
    vr = BasefoldVerifier(code, tree, num_queries=q).verify(OpeningClaim(root, [z]),
                                                            res.reduction_proof)
    assert vr.ok
