"""The FRI open (FriProver.prove / _open_one, zorch/pcs/fri/prover.py:101-187)
on the CPU: the oracle's restated prover against the product's host verifier
(FriVerifier, zorch/pcs/fri/verifier.py:31-140), the cases of the reference's
own round-trip tests (zorch/pcs/fri/testing/fri_test.py) -- honest openings
verify, a wrong value or a tampered final layer is rejected, batch and
layer-count mismatches raise -- plus the DEEP quotient's defining identity."""

from __future__ import annotations

import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _t(a) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.uint32)).view(np.int32))


def _case(orc, field, log_k, log_b, rounds, queries, limbs, z, shift=None, seed=1):
    """(params, verifier inputs) for one committed polynomial opened at z by
    the oracle's prover."""
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2, koalabear16_params
    from zorch_gb300.commit import Opening
    from zorch_gb300.field import field_of
    from zorch_gb300.pcs import FriParams, FriProof

    f = field_of(field)
    if field == 1:
        p2 = orc.Poseidon2.koalabear16_golden()
        perm = koalabear16_params(orc.load_koalabear_fixture())
    else:
        p2 = orc.Poseidon2.babybear16()
        perm = Poseidon2.builtin(f)
    k = 1 << log_k
    coeffs = orc.to_mont(field, np.random.default_rng(seed).integers(
        0, f.p, size=k, dtype=np.uint64).astype(np.uint32))
    sh = f.mont(shift) if shift is not None else 0
    cw = orc.rs_encode(field, coeffs, log_b, sh)
    n = cw.size
    f_layers = orc.merkle_commit(p2, cw, n // 2, 2, 1, n // 2)
    zw = np.asarray([f.mont(x) for x in (z if isinstance(z, tuple) else (z,))], np.uint32)
    t = orc.Transcript(p2)
    want = orc.fri_open(p2, field, coeffs, cw, f_layers, zw, rounds, queries, limbs, t, sh)
    ph = want.phase
    proof = FriProof(_t(want.value).reshape(()) if zw.size == 1 else _t(want.value),
                     _t(ph.roots), _t(ph.final_layer.reshape(-1) if ph.final_layer.shape[1] == 1
                                      else ph.final_layer),
                     Opening(_t(want.f_rows), _t(want.f_paths)),
                     [Opening(_t(r), _t(p)) for r, p in zip(ph.rows, ph.paths)])
    code = ReedSolomon(k, 1 << log_b, f, coset_shift=shift)
    params = FriParams(code, MerkleTree(perm), rounds, queries, limbs)
    root = f_layers[-1][0]
    return params, root, zw, want, proof, cw, coeffs


CASES = [  # field, log_k, log_blowup, rounds, queries, challenge limbs, z, coset shift
    (1, 2, 1, 2, 3, 1, 2, None),          # the reference's test shape (message 4, blowup 2)
    (1, 2, 1, 2, 3, 1, 2, 3),             # its coset variant (shift 3)
    (0, 10, 1, 10, 8, 1, 5, 31),
    (0, 10, 1, 10, 8, 4, (5, 7, 11, 13), 31),
    (0, 9, 2, 9, 16, 4, 2, 31),
    (1, 8, 1, 8, 5, 4, (3, 1, 4, 1), None),
]


@pytest.mark.parametrize("case", CASES)
def test_oracle_fri_open_verifies(orc, case):
    from zorch_gb300.pcs import FriVerifier

    field, log_k, log_b, rounds, queries, limbs, z, shift = case
    params, root, zw, want, proof, _, _ = _case(orc, field, log_k, log_b, rounds, queries, limbs,
                                                z, shift)
    ok, _ = FriVerifier(params)._verify_opening(_t(root).reshape(1, 8), [_t(zw)],
                                                _t(want.value).reshape(1, -1), [proof], None)
    assert ok


@pytest.mark.parametrize("case", CASES[:1] + CASES[3:4])
def test_tampered_fri_open_rejected(orc, case):
    from zorch_gb300.pcs import FriVerifier

    field, log_k, log_b, rounds, queries, limbs, z, shift = case
    params, root, zw, want, proof, _, _ = _case(orc, field, log_k, log_b, rounds, queries, limbs,
                                                z, shift)
    ver = FriVerifier(params)
    r = _t(root).reshape(1, 8)
    v = _t(want.value).reshape(1, -1)
    bad_v = v.clone()
    bad_v[0, 0] += 1
    assert not ver._verify_opening(r, [_t(zw)], bad_v, [proof], None)[0]
    fin = proof.final_layer.clone()
    fin.view(-1)[0] += 1
    assert not ver._verify_opening(r, [_t(zw)], v, [dataclasses.replace(proof, final_layer=fin)],
                                   None)[0]
    bad_root = r.clone()
    bad_root[0, 3] ^= 1
    assert not ver._verify_opening(bad_root, [_t(zw)], v, [proof], None)[0]
    row = proof.query_openings[0].row.clone()
    row[0, 0] ^= 1
    ops = [dataclasses.replace(proof.query_openings[0], row=row)] + proof.query_openings[1:]
    assert not ver._verify_opening(r, [_t(zw)], v,
                                   [dataclasses.replace(proof, query_openings=ops)], None)[0]


def test_batch_and_layer_count_mismatches_raise(orc):
    from zorch_gb300.pcs import FriVerifier

    params, root, zw, want, proof, _, _ = _case(orc, *CASES[0][:7], CASES[0][7])
    ver = FriVerifier(params)
    r = _t(root).reshape(1, 8)
    with pytest.raises(ValueError):
        ver._verify_opening(r, [_t(zw), _t(zw)], _t(np.zeros(2, np.uint32)), [], None)
    short = dataclasses.replace(proof, fri_roots=proof.fri_roots[:0], query_openings=[])
    with pytest.raises(ValueError):
        ver._verify_opening(r, [_t(zw)], _t(want.value).reshape(1, -1), [short], None)


@pytest.mark.parametrize("limbs", [1, 4])
def test_deep_quotient_identity(orc, limbs):
    """q(x) (x - z) + v == f(x) on the domain points, and v = f(z) by Horner
    restated on canonical values."""
    from zorch_gb300.field import BABYBEAR as F

    k, log_b = 64, 1
    coeffs = orc.to_mont(0, np.random.default_rng(3).integers(0, F.p, size=k,
                                                              dtype=np.uint64).astype(np.uint32))
    cw = orc.rs_encode(0, coeffs, log_b, F.mont(31))
    z = np.asarray([F.mont(x) for x in ((9,) if limbs == 1 else (9, 2, 6, 5))], np.uint32)
    v = orc.eval_poly_at(0, coeffs, z)
    # Horner restated in Python on canonical values
    zc = [F.canon(int(x)) for x in z] + [0] * (4 - limbs)
    acc = (0, 0, 0, 0)
    for c in reversed([F.canon(int(x)) for x in coeffs]):
        acc = F.ef_add(F.ef_mul(acc, zc), (c, 0, 0, 0))
    assert tuple(F.canon(int(x)) for x in v) + (0,) * (4 - limbs) == acc
    q = orc.deep_quotient(0, cw, z, v, F.mont(31)).reshape(cw.size, -1)
    dom = orc.eval_domain(0, cw.size.bit_length() - 1, F.mont(31))
    for j in range(0, cw.size, 7):
        x = F.canon(int(dom[j]))
        qj = tuple(F.canon(int(w)) for w in q[j]) + (0,) * (4 - limbs)
        lhs = F.ef_add(F.ef_mul(qj, F.ef_sub((x, 0, 0, 0), tuple(zc))), acc)
        assert lhs == (F.canon(int(cw[j])), 0, 0, 0)
