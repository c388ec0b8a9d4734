"""Fiat-Shamir duplex transcript (drop-in for DuplexTranscript,
zorch/transcript.py:239-481) with its state resident on the GPU.

Overwrite-mode duplex sponge, width 16, rate 8: `observe` absorbs full rate
blocks and keeps the tail pending; `sample` permutes when input is pending or
the output buffer is drained and pops `output_buffer[out_pos - 1]` (the last
rate lane first). Each step is one single-thread kernel (zc_duplex_step) on
the current stream, so a whole fold loop runs without a host round trip and
can be captured in a CUDA graph. The state is the 34-word FFI wire layout
(in_buf, out_buf, sponge, in_pos, out_pos; zorch/transcript.py:1015-1021).

The API is functional like the reference: every call returns a new
transcript and leaves the receiver unchanged (the 136-byte state is copied).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .commit import Poseidon2
from .field import full_u32, ptr, stream_handle


class DuplexTranscript:
    rate = 8
    width = 16

    def __init__(self, perm: Poseidon2, state: torch.Tensor) -> None:
        self.permutation = perm
        self.state = state

    @classmethod
    def new(cls, perm: Poseidon2 | None = None, rate: int = 8, device="cuda") -> "DuplexTranscript":
        if rate != 8:
            raise NotImplementedError("only rate 8 (width 16) is built")
        perm = perm if perm is not None else Poseidon2.builtin()
        return cls(perm, full_u32(_lib.DUPLEX_WORDS, 0, device))

    @property
    def field(self):
        return self.permutation.field

    # -- in-place steps (used by the provers; the public API copies first) --
    def _step(self, values: torch.Tensor | None, n: int, out: torch.Tensor | None = None,
              positions: torch.Tensor | None = None, block_len: int = 0) -> None:
        v = values.contiguous() if values is not None else None
        m = v.numel() if v is not None else 0
        _lib.check(_lib.lib().zc_duplex_step(
            self.permutation.handle, ptr(self.state), ptr(v) if m else None, m, n,
            ptr(out), ptr(positions), block_len, stream_handle()), "duplex_step")

    def observe_(self, values: torch.Tensor) -> "DuplexTranscript":
        self._step(values, 0)
        return self

    def sample_(self, n: int = 1) -> torch.Tensor:
        out = torch.empty(n, dtype=torch.int32, device=self.state.device)
        self._step(None, n, out)
        return out

    def observe_and_sample_(self, values: torch.Tensor, n: int = 1) -> torch.Tensor:
        out = torch.empty(n, dtype=torch.int32, device=self.state.device)
        self._step(values, n, out)
        return out

    def sample_positions_(self, block_len: int, count: int,
                          values: torch.Tensor | None = None) -> torch.Tensor:
        pos = torch.empty(count, dtype=torch.int32, device=self.state.device)
        self._step(values, count, None, pos, block_len)
        return pos

    # -- functional API mirroring the reference --
    def _copy(self) -> "DuplexTranscript":
        return DuplexTranscript(self.permutation, self.state.clone())

    def observe(self, values: torch.Tensor) -> "DuplexTranscript":
        return self._copy().observe_(values)

    def sample(self, n: int = 1) -> tuple["DuplexTranscript", torch.Tensor]:
        t = self._copy()
        return t, t.sample_(n)

    def observe_and_sample(self, values: torch.Tensor, n: int = 1):
        t = self._copy()
        return t, t.observe_and_sample_(values, n)

    # -- proof of work (zorch/transcript.py:417-481) --
    def check_witness(self, witness: torch.Tensor, *, pow_bits: int):
        """Observe `witness` (one field element), squeeze one challenge and
        report whether its low `pow_bits` canonical bits are zero; returns the
        advanced transcript and a device bool (check_witness,
        zorch/transcript.py:417-437)."""
        _validate_pow_bits(pow_bits)
        if witness.numel() != 1 or witness.dtype != torch.int32:
            raise ValueError("witness must be one field element (int32 Montgomery word)")
        t, ch = self.observe_and_sample(witness.reshape(1), 1)
        canon = torch.empty_like(ch)
        _lib.check(_lib.lib().zc_from_mont(self.field.id, ptr(ch), ptr(canon), 1,
                                           stream_handle()), "from_mont")
        return t, (canon & ((1 << pow_bits) - 1)) == 0

    def grind(self, pow_bits: int) -> tuple["DuplexTranscript", torch.Tensor]:
        """The lowest proof-of-work witness, searched on the device
        (zc_duplex_grind), and the transcript advanced past it by
        check_witness (DuplexTranscript.grind, zorch/transcript.py:461-481).
        No host round trip: the witness stays a device word."""
        _validate_pow_bits(pow_bits)
        witness = torch.empty(1, dtype=torch.int32, device=self.state.device)
        _lib.check(_lib.lib().zc_duplex_grind(self.permutation.handle, ptr(self.state), pow_bits,
                                              ptr(witness), stream_handle()), "duplex_grind")
        t, _ = self.check_witness(witness, pow_bits=pow_bits)
        return t, witness.reshape(())

    def wire(self) -> tuple[torch.Tensor, ...]:
        s = self.state
        return s[0:8], s[8:16], s[16:32], s[32:33], s[33:34]


def _validate_pow_bits(pow_bits: int) -> None:
    if not 0 <= pow_bits < 32:
        raise ValueError(f"pow_bits must be in [0, 32), got {pow_bits}")


def sample_challenge(t: DuplexTranscript, limbs: int = 1):
    """`limbs` consecutive squeezes as one challenge (EF4: the coefficients
    c0..c3), zorch/transcript.py:122-137."""
    if limbs < 1:
        raise ValueError(f"limbs must be >= 1, got {limbs}")
    return t.sample(limbs)


def sample_positions(t: DuplexTranscript, block_len: int, count: int):
    """Query positions = (Montgomery bits of each squeeze) mod block_len
    (zorch/pcs/fold.py:173-182)."""
    t2 = t._copy()
    return t2, t2.sample_positions_(block_len, count)


class HostDuplexTranscript:
    """The host-FS form: the same duplex on the CPU through the C ABI's host
    hop (the reference's FFI hop contract, zorch/transcript.py:1005-1112)."""

    def __init__(self, perm: Poseidon2, state: np.ndarray | None = None) -> None:
        self.permutation = perm
        self.state = np.zeros(_lib.DUPLEX_WORDS, np.uint32) if state is None else state

    def hop(self, values, n: int) -> tuple["HostDuplexTranscript", np.ndarray]:
        v = np.ascontiguousarray(np.asarray(values if values is not None else [], np.uint32)).reshape(-1)
        s = self.state
        o = np.zeros(_lib.DUPLEX_WORDS, np.uint32)
        ch = np.zeros(max(n, 1), np.uint32)
        a = s.ctypes.data
        b = o.ctypes.data
        _lib.check(_lib.lib().zc_duplex_hop_host(
            self.permutation.handle, a, a + 32, a + 64, a + 128, a + 132,
            v.ctypes.data if v.size else None, v.size, n,
            b, b + 32, b + 64, b + 128, b + 132, ch.ctypes.data), "duplex_hop_host")
        return HostDuplexTranscript(self.permutation, o), ch[:n]

    def observe(self, values) -> "HostDuplexTranscript":
        return self.hop(values, 0)[0]

    def sample(self, n: int = 1):
        return self.hop(None, n)

    def observe_and_sample(self, values, n: int = 1):
        return self.hop(values, n)

    def check_witness(self, witness, *, pow_bits: int):
        """The verifier's proof-of-work check on the host: observe the
        witness (Montgomery word), squeeze once, test the low `pow_bits`
        canonical bits (zorch/transcript.py:417-437)."""
        _validate_pow_bits(pow_bits)
        w = np.asarray(witness, np.uint32).reshape(-1)
        if w.size != 1:
            raise ValueError("witness must be one field element")
        t, ch = self.hop(w, 1)
        canon = self.permutation.field.canon(int(ch[0]))
        return t, (canon & ((1 << pow_bits) - 1)) == 0
