"""The CPU oracle pinned before anything is checked against it.

- Poseidon2 / sponge / compression / Merkle: the reference's Plonky3
  KoalaBear-16 golden root (zorch/commit/testing/merkle_test.py:51-63), plus the
  structural round trips of merkle_test.py:75-330.
- RS encode: Horner on the recovered domain (reed_solomon_test.py:48-60), coset
  encode, linearity, and the fold/encode commute (reed_solomon_test.py:72-99).
- Transcript: the duplex's stream property (absorbing a concatenation equals
  absorbing the parts, zorch/challenge.py:84-89) and squeeze order.
- The built-in BabyBear Poseidon2 instance: the oracle's independent Grain-LFSR
  derivation equals the constants compiled into the CUDA library.
"""

from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rand(field_p: int, shape, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).integers(0, field_p, size=shape, dtype=np.uint64).astype(np.uint32)


def test_koalabear_golden_root(orc):
    d = orc.load_koalabear_fixture()
    p2 = orc.Poseidon2.koalabear16_golden()
    m = orc.to_mont(orc.KOALABEAR, np.arange(32, dtype=np.uint32).reshape(4, 8))
    layers = orc.merkle_commit_rows(p2, m)
    assert [l.shape for l in layers] == [(4, 8), (2, 8), (1, 8)]
    root = orc.from_mont(orc.KOALABEAR, layers[-1][0])
    assert root.tolist() == d["merkle_4x8_root"]


def test_koalabear_leaf_is_row_sponge_and_node_is_compress(orc):
    p2 = orc.Poseidon2.koalabear16_golden()
    m = orc.to_mont(orc.KOALABEAR, np.arange(32, dtype=np.uint32).reshape(4, 8))
    layers = orc.merkle_commit_rows(p2, m)
    for i in range(4):
        assert np.array_equal(layers[0][i], p2.hash(m[i]))
    assert np.array_equal(layers[1][0], p2.compress(layers[0][0], layers[0][1]))


def _reconstruct(p2, leaf_digest, idx, path):
    node = leaf_digest
    for sib in path:
        node = p2.compress(node, sib) if idx % 2 == 0 else p2.compress(sib, node)
        idx //= 2
    return node


@pytest.mark.parametrize("field", [0, 1])
def test_merkle_open_reconstructs_root(orc, field):
    p2 = orc.Poseidon2.babybear16() if field == 0 else orc.Poseidon2.koalabear16_golden()
    m = _rand(orc.MODULUS[field], (64, 5), 3)
    m = orc.to_mont(field, m)
    layers = orc.merkle_commit_rows(p2, m)
    idx = np.arange(64, dtype=np.int32)
    rows, paths = orc.merkle_open(m, 64, 1, 5, 0, layers, idx)
    for k in range(64):
        assert np.array_equal(rows[k], m[k])
        got = _reconstruct(p2, p2.hash(rows[k]), k, paths[:, k])
        assert np.array_equal(got, layers[-1][0])
    tampered = paths.copy()
    tampered[2, 5, 0] ^= 1
    assert not np.array_equal(_reconstruct(p2, p2.hash(rows[5]), 5, tampered[:, 5]), layers[-1][0])
    with pytest.raises(IndexError):
        orc.merkle_open(m, 64, 1, 5, 0, layers, np.array([64], np.int32))


def test_column_major_equals_row_major_of_transpose(orc):
    p2 = orc.Poseidon2.babybear16()
    cols = orc.to_mont(0, _rand(orc.P_BABYBEAR, (13, 32), 5))
    a = orc.merkle_commit_columns(p2, cols)
    b = orc.merkle_commit_rows(p2, np.ascontiguousarray(cols.T))
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_sponge_partial_block_and_empty(orc):
    p2 = orc.Poseidon2.babybear16()
    x = orc.to_mont(0, _rand(orc.P_BABYBEAR, 11, 9))
    s = np.zeros(16, np.uint32)
    s[:8] = x[:8]
    s = p2.permute(s)
    s[:3] = x[8:]
    s = p2.permute(s)
    assert np.array_equal(p2.hash(x), s[:8])
    assert np.array_equal(p2.hash(np.zeros(0, np.uint32)), np.zeros(8, np.uint32))


def test_babybear_instance_matches_cuda_header(orc):
    hdr = (ROOT / "zorch_gb300" / "csrc" / "poseidon2_babybear16.h").read_text()

    def arr(name):
        body = re.search(name + r"[^=]*=\s*\{(.*?)\};", hdr, re.S).group(1)
        return np.array([int(v) for v in re.findall(r"(\d+)u", body)], np.uint32)

    ei, et, ir, dg = orc.Poseidon2.babybear16().export_canonical()
    assert np.array_equal(arr("ZC_BB16_EXT_INIT").reshape(4, 16), ei)
    assert np.array_equal(arr("ZC_BB16_EXT_TERM").reshape(4, 16), et)
    assert np.array_equal(arr("ZC_BB16_INT_RC"), ir)
    assert np.array_equal(arr("ZC_BB16_DIAG"), dg)


@pytest.mark.parametrize("field", [0, 1])
@pytest.mark.parametrize("log_k,log_b", [(0, 1), (3, 1), (5, 2), (6, 3)])
def test_rs_encode_matches_horner(orc, field, log_k, log_b):
    p = orc.MODULUS[field]
    m = orc.to_mont(field, _rand(p, 1 << log_k, log_k))
    shift = int(orc.to_mont(field, np.array([31 if field == 0 else 3]))[0])
    for sh in (0, shift):
        got = orc.rs_encode(field, m, log_b, sh, 0)
        want = orc.rs_encode_horner(field, m, log_b, sh, 0)
        assert np.array_equal(got, want)


def test_rs_encode_linear_and_batched(orc):
    f = 0
    a = orc.to_mont(f, _rand(orc.P_BABYBEAR, (3, 64), 1))
    enc = orc.rs_encode(f, a, 2, int(orc.to_mont(f, [31])[0]))
    for i in range(3):
        assert np.array_equal(enc[i], orc.rs_encode(f, a[i], 2, int(orc.to_mont(f, [31])[0])))
    s = (a[0].astype(np.uint64) + a[1]) % orc.P_BABYBEAR
    es = (enc[0].astype(np.uint64) + enc[1]) % orc.P_BABYBEAR
    assert np.array_equal(orc.rs_encode(f, s.astype(np.uint32), 2, int(orc.to_mont(f, [31])[0])),
                          es.astype(np.uint32))


def _ef4_from_base(field, x):
    out = np.zeros((x.size, 4), np.uint32)
    out[:, 0] = x
    return out


@pytest.mark.parametrize("ef_beta", [False, True])
def test_fold_commutes_with_encode(orc, ef_beta):
    """fold(encode_h(m), beta) == encode_{h^2}(m_even + beta*m_odd)."""
    f, p = 0, orc.P_BABYBEAR
    k, log_b = 32, 2
    m = orc.to_mont(f, _rand(p, k, 11))
    h = int(orc.to_mont(f, [31])[0])
    cw = orc.rs_encode(f, m, log_b, h)
    beta = orc.to_mont(f, _rand(p, 4 if ef_beta else 1, 12))
    folded = orc.fri_fold(f, cw, False, beta, ef_beta, h)
    h2 = orc.LIB.orc_mul(f, h, h)
    even, odd = m[0::2], m[1::2]
    if ef_beta:
        want = np.zeros((k // 2 << log_b, 4), np.uint32)
        for e in range(4):
            be = np.array([orc.LIB.orc_mul(f, int(beta[e]), int(x)) for x in odd], np.uint32)
            coeff = be if e else ((even.astype(np.uint64) + be) % p).astype(np.uint32)
            want[:, e] = orc.rs_encode(f, coeff, log_b, h2)
    else:
        be = np.array([orc.LIB.orc_mul(f, int(beta[0]), int(x)) for x in odd], np.uint32)
        want = orc.rs_encode(f, ((even.astype(np.uint64) + be) % p).astype(np.uint32), log_b, h2)
    assert np.array_equal(folded, want)


def test_transcript_stream_property_and_order(orc):
    p2 = orc.Poseidon2.babybear16()
    vals = orc.to_mont(0, _rand(orc.P_BABYBEAR, 21, 4))
    t1 = orc.Transcript(p2).observe(vals)
    t2 = orc.Transcript(p2).observe(vals[:5]).observe(vals[5:13]).observe(vals[13:])
    assert all(np.array_equal(a, b) for a, b in zip(t1.st.wire(), t2.st.wire()))
    a, b = t1.sample(11), t2.sample(11)
    assert np.array_equal(a, b)
    # squeeze order: a fresh permute pops output_buffer[7] first
    t = orc.Transcript(p2).observe(vals[:8])
    st = np.zeros(16, np.uint32)
    st[:8] = vals[:8]
    st = p2.permute(st)
    assert t.sample(3).tolist() == [st[7], st[6], st[5]]


def _verify_commit_phase(orc, p2, field, proof, n0, R, Q, beta_limbs, shift):
    """Independent replay: Merkle paths rebuild each root, each opened pair
    folds to the next layer's opened value (zorch/pcs/fold.py:392-468)."""
    limbs = orc.layer_limbs(R, beta_limbs)
    t = orc.Transcript(p2)
    betas = []
    for r in range(R):
        t.observe(proof.roots[r])
        betas.append(t.sample(beta_limbs))
    t.observe(proof.final_layer)
    pos = (t.sample(Q) % np.uint32(n0)).astype(np.int32)
    assert np.array_equal(pos, proof.positions)
    a = pos.copy()
    sh = shift
    for r in range(R):
        n = n0 >> r
        L = n // 2
        a = a % L
        for q in range(Q):
            row = proof.rows[r][q]
            got = _reconstruct(p2, p2.hash(row), int(a[q]), proof.paths[r][:, q])
            assert np.array_equal(got, proof.roots[r])
        # fold the opened pairs at their positions with a one-pair "codeword"
        lo = proof.rows[r][:, : limbs[r]]
        hi = proof.rows[r][:, limbs[r]:]
        for q in range(Q):
            x = orc.eval_domain(field, n.bit_length() - 1, sh)[a[q]]
            # a length-2 codeword on domain {x, -x}: fold with shift x, generator any
            pair = np.concatenate([lo[q], hi[q]])
            g = orc.fri_fold(field, pair.reshape(2, -1).squeeze(), limbs[r] == 4, betas[r],
                             beta_limbs == 4, int(x))
            g = g.reshape(-1)
            if r + 1 < R:
                nL = (n // 2) // 2
                nxt = proof.rows[r + 1][q]
                la = limbs[r + 1]
                want = nxt[:la] if a[q] < nL else nxt[la:]
            else:
                want = proof.final_layer[a[q]].reshape(-1)
            assert np.array_equal(g, want)
        sh = orc.LIB.orc_mul(field, sh, sh)
    # the final layer of an honest low-degree codeword is constant
    assert (proof.final_layer == proof.final_layer[0]).all()


@pytest.mark.parametrize("beta_limbs", [1, 4])
def test_fri_commit_phase_verifies(orc, beta_limbs):
    f = 0
    p2 = orc.Poseidon2.babybear16()
    k, log_b, R, Q = 64, 1, 6, 9
    h = int(orc.to_mont(f, [31])[0])
    cw = orc.rs_encode(f, orc.to_mont(f, _rand(orc.P_BABYBEAR, k, 21)), log_b, h)
    proof = orc.fri_commit_phase(p2, f, cw, R, Q, beta_limbs, orc.Transcript(p2), h)
    _verify_commit_phase(orc, p2, f, proof, k << log_b, R, Q, beta_limbs, h)
    assert len(proof.to_bytes()) == 4 * (R * 8 + proof.final_layer.size +
                                        sum(r.size for r in proof.rows) + sum(p.size for p in proof.paths))
