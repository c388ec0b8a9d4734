"""CPU emulation of the quarter- and half-warp Poseidon2 permutations
(p2_permute_quarter, p2_permute_half / half_permute_bb16 in
zorch_gb300/csrc/poseidon2.cuh). Quarter: lane q of a quarter
holds the M4 block q (state words 4q .. 4q+3); the external layer is the block
matrix on each lane's own words plus the sums over the four blocks (the two
xor-shuffle levels); in the partial rounds every lane keeps word 0, runs its
S-box redundantly and forms the sum of words 1..15 from its local words and
the same two shuffle levels. Half: lane l holds word l; the external layer is
y_l = s_b + x_l + 2 x_(l+1 in its block) (the block sum s_b by two xor
shuffles) plus the sum over the lane class l mod 4 (xor 4, xor 8); the partial
round sums lanes 1..15 while lane 0 runs its S-box. Restated with exact
integers, lane by lane, and compared with the oracle's permutation for the
built-in BabyBear-16 instance and the reference's KoalaBear-16 golden
instance."""

from __future__ import annotations

import numpy as np
import pytest


def _m4(x, p):
    t01, t23 = (x[0] + x[1]) % p, (x[2] + x[3]) % p
    t0123 = (t01 + t23) % p
    t01123, t01233 = (t0123 + x[1]) % p, (t0123 + x[3]) % p
    return [(t01123 + t01) % p, (t01123 + 2 * x[2]) % p, (t01233 + t23) % p,
            (t01233 + 2 * x[0]) % p]


def _ext(lanes, p):
    lanes = [_m4(x, p) for x in lanes]
    # s[k] on every lane after the xor-1 and xor-2 shuffle levels
    s = [sum(lanes[q][k] for q in range(4)) % p for k in range(4)]
    return [[(lanes[q][k] + s[k]) % p for k in range(4)] for q in range(4)]


def quarter_permute(state, ei, et, ir, dg, alpha, j, p):
    lanes = [[int(state[4 * q + k]) for k in range(4)] for q in range(4)]
    lanes = _ext(lanes, p)
    for r in range(len(ei)):
        lanes = [[pow((lanes[q][k] + int(ei[r][4 * q + k])) % p, alpha, p) for k in range(4)]
                 for q in range(4)]
        lanes = _ext(lanes, p)
    w0 = [lanes[0][0]] * 4  # word 0 on every lane (one shuffle from lane 0)
    for r in range(len(ir)):
        s0 = [pow((w0[q] + int(ir[r])) % p, alpha, p) for q in range(4)]
        # words 1..15 of the round input: lane 0 leaves out its word 0
        part = [sum(lanes[q][k] for k in range(4) if (q, k) != (0, 0)) % p for q in range(4)]
        part = [sum(part) % p] * 4  # the xor-1 and xor-2 shuffle levels
        new = []
        for q in range(4):
            total = (part[q] + s0[q]) * j % p
            new.append([(total + int(dg[4 * q + k]) * lanes[q][k]) % p for k in range(4)])
            w0[q] = (total + int(dg[0]) * s0[q]) % p
        assert len(set(w0)) == 1  # every lane derives the same word 0
        new[0][0] = w0[0]
        lanes = new
    for r in range(len(et)):
        lanes = [[pow((lanes[q][k] + int(et[r][4 * q + k])) % p, alpha, p) for k in range(4)]
                 for q in range(4)]
        lanes = _ext(lanes, p)
    return [lanes[q][k] for q in range(4) for k in range(4)]


def _half_ext(x, p):
    y = []
    for l in range(16):
        b = l & ~3
        s_b = sum(x[b:b + 4]) % p
        y.append((s_b + x[l] + 2 * x[b | ((l + 1) & 3)]) % p)
    c = [sum(y[(l & 3) + 4 * i] for i in range(4)) % p for l in range(16)]
    return [(y[l] + c[l]) % p for l in range(16)]


def half_permute(state, ei, et, ir, dg, alpha, j, p):
    x = _half_ext([int(v) for v in state], p)
    for r in range(len(ei)):
        x = _half_ext([pow((x[l] + int(ei[r][l])) % p, alpha, p) for l in range(16)], p)
    for r in range(len(ir)):
        s0 = pow((x[0] + int(ir[r])) % p, alpha, p)  # lane 0's S-box
        rest = sum(x[1:]) % p                        # lanes 1..15 (four xor levels)
        total = (rest + s0) * j % p                  # s0 broadcast from lane 0
        x = [(total + int(dg[l]) * (s0 if l == 0 else x[l])) % p for l in range(16)]
    for r in range(len(et)):
        x = _half_ext([pow((x[l] + int(et[r][l])) % p, alpha, p) for l in range(16)], p)
    return x


@pytest.mark.parametrize("which", ["babybear16", "koalabear16"])
def test_warp_layouts_equal_the_oracle_permutation(orc, which):
    if which == "babybear16":
        p2, p, j = orc.Poseidon2.babybear16(), orc.P_BABYBEAR, 1
        field = 0
    else:
        d = orc.load_koalabear_fixture()
        p2, p, j = orc.Poseidon2.koalabear16_golden(), orc.P_KOALABEAR, int(d["internal_j_scale"])
        field = 1
    ei, et, ir, dg = p2.export_canonical()
    rng = np.random.default_rng(7)
    for _ in range(4):
        x = rng.integers(0, p, size=16, dtype=np.uint64).astype(np.uint32)
        want = orc.from_mont(field, p2.permute(orc.to_mont(field, x)))
        assert quarter_permute(x, ei, et, ir, dg, p2.alpha, j, p) == [int(v) for v in want]
        assert half_permute(x, ei, et, ir, dg, p2.alpha, j, p) == [int(v) for v in want]
