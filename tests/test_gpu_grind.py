"""Proof-of-work grind on the GPU (zc_duplex_grind behind
DuplexTranscript.grind, zorch/transcript.py:439-481) == the oracle's
literal search, for both fields, every pending-input depth and several
difficulties; the advanced transcript equals the oracle's after
check_witness, and the host verifier (HostDuplexTranscript.check_witness)
accepts the witness and rejects others (zorch/testing/transcript_test.py:
266-355 are the reference's cases)."""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from zorch_gb300 import _lib  # noqa: E402
from zorch_gb300.field import to_device, to_host  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")


def _perms(orc, field):
    from zorch_gb300.commit import Poseidon2, koalabear16_params
    from zorch_gb300.field import BABYBEAR

    if field == 0:
        return Poseidon2.builtin(BABYBEAR), orc.Poseidon2.babybear16()
    return koalabear16_params(orc.load_koalabear_fixture()), orc.Poseidon2.koalabear16_golden()


def _seeded(orc, field, pending):
    from zorch_gb300.transcript import DuplexTranscript

    gperm, cperm = _perms(orc, field)
    vals = orc.to_mont(field, np.arange(1, 9 + pending, dtype=np.uint32))
    t = DuplexTranscript.new(gperm).observe(to_device(vals))
    ot = orc.Transcript(cperm)
    ot.observe(vals)
    return gperm, t, ot


@pytest.mark.parametrize("field", [0, 1])
@pytest.mark.parametrize("pending", list(range(8)))
@pytest.mark.parametrize("bits", [0, 1, 6, 12])
def test_grind_matches_oracle(orc, field, pending, bits):
    _, t, ot = _seeded(orc, field, pending)
    t2, witness = t.grind(bits)
    want = ot.grind(bits)
    assert int(to_host(witness.reshape(1))[0]) == int(orc.to_mont(field, [want])[0])
    assert ot.check_witness(int(orc.to_mont(field, [want])[0]), bits)
    assert np.array_equal(to_host(t2.state), np.frombuffer(bytes(ot.st), np.uint32))


@pytest.mark.parametrize("field", [0, 1])
def test_grind_high_difficulty(orc, field):
    """A witness deep in the search (about 2^18 candidates): every witness below
    it must fail, which only a search that ordered its sweeps correctly gives."""
    from zorch_gb300.transcript import HostDuplexTranscript

    gperm, t, _ = _seeded(orc, field, 4)
    t2, witness = t.grind(18)
    ok = t.check_witness(witness, pow_bits=18)[1]
    assert bool(ok.item())
    ht = HostDuplexTranscript(gperm, to_host(t.state).copy())
    w = int(to_host(witness.reshape(1))[0])
    assert ht.check_witness([w], pow_bits=18)[1]
    canon = gperm.field.canon(w)
    # the oracle's literal search agrees (a few seconds of CPU at 2^18)
    _, _, ot = _seeded(orc, field, 4)
    assert ot.grind(18) == canon


def test_host_check_witness_rejects_other_witnesses(orc):
    from zorch_gb300.transcript import HostDuplexTranscript

    gperm, t, ot = _seeded(orc, 1, 5)
    _, witness = t.grind(10)
    ht = HostDuplexTranscript(gperm, to_host(t.state).copy())
    w = gperm.field.canon(int(to_host(witness.reshape(1))[0]))
    for v in (w, w + 1, w + 2, 0):
        c = ot.copy()
        want = c.check_witness(gperm.field.mont(v), 10)
        assert ht.check_witness([gperm.field.mont(v)], pow_bits=10)[1] == want
        if v <= w:
            assert want == (v == w)
    with pytest.raises(ValueError):
        ht.check_witness([0], pow_bits=32)
    with pytest.raises(ValueError):
        t.grind(-1)
