"""The oracle's k-ary fold (ReedSolomon.fold_group,
zorch/coding/reed_solomon.py:357-381) against the reference's own relations
(zorch/coding/testing/reed_solomon_test.py:344-392), no GPU: at k = 2 it is
the binary butterfly; it commutes with encoding -- folding the codeword of p
by beta gives the codeword of sum_m beta^m p[m::k] on the x^k domain (shift
h^k) -- for every k and with or without a coset."""

from __future__ import annotations

import numpy as np
import pytest

import oracle.oracle as o


def rand_mont(field, shape, seed):
    x = np.random.default_rng(seed).integers(0, o.MODULUS[field], size=shape, dtype=np.uint64)
    return o.to_mont(field, x.astype(np.uint32))


@pytest.mark.parametrize("ef_in,ef_beta", [(False, False), (True, True), (False, True)])
def test_k2_equals_binary_butterfly(ef_in, ef_beta):
    F = o.KOALABEAR
    cw = rand_mont(F, (128, 4) if ef_in else (128,), 1)
    beta = rand_mont(F, 4 if ef_beta else 1, 2)
    sh = int(o.to_mont(F, [3])[0])
    assert np.array_equal(o.fri_fold_k(F, cw, ef_in, beta, ef_beta, 1, sh),
                          o.fri_fold(F, cw, ef_in, beta, ef_beta, sh))


@pytest.mark.parametrize("log_k", [1, 2, 3, 4])
@pytest.mark.parametrize("shift", [None, 31])
def test_fold_group_encode_commute(log_k, shift):
    F = o.BABYBEAR
    k, L = 1 << log_k, 64
    p_ = rand_mont(F, L, 10 + log_k)
    sh = int(o.to_mont(F, [shift])[0]) if shift else 0
    cw = o.rs_encode(F, p_, 1, sh)  # blowup 2
    beta = rand_mont(F, 1, 20 + log_k)
    folded = o.fri_fold_k(F, cw, False, beta, False, log_k, sh)
    pf = np.zeros(L // k, np.uint32)
    bp = int(o.to_mont(F, [1])[0])
    for m in range(k):
        for i in range(L // k):
            pf[i] = (int(pf[i]) + o.LIB.orc_mul(F, bp, int(p_[m + k * i]))) % o.P_BABYBEAR
        bp = o.LIB.orc_mul(F, bp, int(beta[0]))
    shk = sh
    for _ in range(log_k):
        shk = o.LIB.orc_mul(F, shk, shk) if shk else 0
    assert np.array_equal(folded, o.rs_encode(F, pf, 1, shk))
