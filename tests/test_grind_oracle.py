"""The oracle's proof-of-work grind (zorch/transcript.py:417-481,
zorch/grind.py:66-93) against a brute force over the oracle transcript, with
the reference's grind cases (zorch/testing/transcript_test.py:266-355):
the grind result passes check_witness, every smaller witness fails it, the
prover and verifier reach the same state, and pow_bits outside [0, 32) is
refused."""

from __future__ import annotations

import numpy as np
import pytest


def _seeded(orc, p2, pending: int):
    t = orc.Transcript(p2)
    t.observe(orc.to_mont(p2.field, np.arange(1, 9 + pending, dtype=np.uint32)))
    return t


def _passes(orc, t, w: int, bits: int) -> bool:
    c = t.copy()
    return c.check_witness(int(orc.to_mont(c.p2.field, [w])[0]), bits)


@pytest.mark.parametrize("field", [0, 1])
@pytest.mark.parametrize("pending", [0, 3, 7])
@pytest.mark.parametrize("bits", [0, 1, 5, 9])
def test_grind_is_lowest_passing_witness(orc, field, pending, bits):
    p2 = orc.Poseidon2.babybear16() if field == 0 else orc.Poseidon2.koalabear16_golden()
    t = _seeded(orc, p2, pending)
    w = t.grind(bits)
    assert _passes(orc, t, w, bits)
    assert not any(_passes(orc, t, v, bits) for v in range(w))


def test_grind_prover_and_verifier_agree(orc):
    p2 = orc.Poseidon2.koalabear16_golden()
    t = _seeded(orc, p2, 2)
    w = t.grind(8)
    prover, verifier = t.copy(), t.copy()
    wm = int(orc.to_mont(1, [w])[0])
    assert prover.check_witness(wm, 8) and verifier.check_witness(wm, 8)
    assert np.array_equal(prover.sample(3), verifier.sample(3))


def test_grind_zero_bits_is_zero_witness(orc):
    t = orc.Transcript(orc.Poseidon2.babybear16())
    assert t.grind(0) == 0


@pytest.mark.parametrize("bits", [-1, 32])
def test_grind_rejects_out_of_range_bits(orc, bits):
    t = orc.Transcript(orc.Poseidon2.babybear16())
    with pytest.raises(ValueError):
        t.grind(bits)
