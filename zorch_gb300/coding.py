"""Reed-Solomon codes over BabyBear / KoalaBear on the GPU (drop-in for
zorch/coding/reed_solomon.py:71-540).

`ReedSolomon.encode` is the coset low-degree extension (zc_rs_encode), `fold`
the natural-order conjugate-pair FRI fold (zc_fri_fold);
`BitReversedReedSolomon` is the same code with codewords in bit-reversed order
(zc_rs_encode_bitrev, zc_fri_fold_bitrev). Tensors are torch.int32 CUDA
tensors of Montgomery words; the coset shift and generator are canonical ints
(e.g. coset_shift=31, generator=31 for BabyBear).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .field import BABYBEAR, Field, field_of, ptr, stream_handle


def _is_pow2(x: int) -> bool:
    return x > 0 and (x & (x - 1)) == 0


def _log2(x: int) -> int:
    return x.bit_length() - 1


def rs_encode(field: Field, message: torch.Tensor, log_blowup: int, shift_mont: int = 0,
              generator: int = 0, out: torch.Tensor | None = None, *,
              bit_reversed: bool = False) -> torch.Tensor:
    """zc_rs_encode (zc_rs_encode_bitrev) over the last axis of `message` (any
    leading batch shape)."""
    k = message.shape[-1]
    if not _is_pow2(k):
        raise ValueError(f"message_len must be a power of two, got {k}")
    batch = message.numel() // k
    n = k << log_blowup
    if out is None:
        out = torch.empty(*message.shape[:-1], n, dtype=torch.int32, device=message.device)
    L = _lib.lib()
    ws_bytes = L.zc_rs_encode_workspace_bytes(batch, _log2(k), log_blowup)
    ws = torch.empty(max(ws_bytes // 4, 1), dtype=torch.int32, device=message.device)
    fn = L.zc_rs_encode_bitrev if bit_reversed else L.zc_rs_encode
    _lib.check(fn(field.id, ptr(message.contiguous()), batch, _log2(k), log_blowup, shift_mont,
                  generator, ptr(out), ptr(ws), ws_bytes, stream_handle()), "rs_encode")
    return out


def ntt(field, x: torch.Tensor, generator: int = 0) -> torch.Tensor:
    """Forward NTT over the last axis, natural order in and out (lax.ntt NTT)."""
    return rs_encode(field_of(field), x, 0, 0, generator)


def intt(field, x: torch.Tensor, generator: int = 0) -> torch.Tensor:
    """Inverse NTT over the last axis (lax.ntt INTT): (1/k) * NTT(x)[-i mod k]."""
    f = field_of(field)
    k = x.shape[-1]
    y = ntt(f, x, generator)
    rev = torch.remainder(-torch.arange(k, device=x.device), k)
    y = y.index_select(-1, rev).contiguous()
    out = torch.empty_like(y)
    _lib.check(_lib.lib().zc_scale(f.id, ptr(y), ptr(out), y.numel(), f.inv_mont(f.mont(k)),
                                   stream_handle()), "scale")
    return out


def eval_domain(field, n: int, *, shift: int | None = None, generator: int | None = None,
                device="cuda") -> torch.Tensor:
    """[shift * w^j] in NTT order (zorch/coding/reed_solomon.py:49-68), read off
    the encoder applied to e_1 exactly as the reference does."""
    f = field_of(field)
    if not _is_pow2(n):
        raise ValueError(f"eval_domain size must be a power of two, got {n}")
    sh = f.mont(shift) if shift is not None else 0
    if n == 1:
        return torch.full((1,), sh or f.one_mont, dtype=torch.int32, device=device)
    e1 = torch.zeros(n, dtype=torch.int32, device=device)
    e1[1] = f.one_mont
    return rs_encode(f, e1, 0, sh, generator or 0)


class ReedSolomon:
    """Reed-Solomon code; implements the reference's FoldableCode seam
    (zorch/coding/foldable_code.py:27-70) for the binary natural-order fold."""

    bit_reversed = False

    def __init__(self, message_len: int, blowup: int, field=BABYBEAR, *,
                 coset_shift: int | None = None, fold_factor: int = 2,
                 generator: int | None = None) -> None:
        if not _is_pow2(message_len):
            raise ValueError(f"message_len must be a power of two, got {message_len}")
        if not _is_pow2(blowup):
            raise ValueError(f"blowup must be a power of two, got {blowup}")
        if not _is_pow2(fold_factor) or fold_factor < 2:
            raise ValueError(f"fold_factor must be a power of two >= 2, got {fold_factor}")
        if fold_factor > 16:
            raise NotImplementedError("k-ary folds are built for fold_factor <= 16")
        self.field = field_of(field)
        if generator not in (None, 0, self.field.generator):
            raise NotImplementedError("only the field's canonical generator is built")
        self.message_len = message_len
        self.blowup = blowup
        self.block_len = message_len * blowup
        self.coset_shift = coset_shift
        self.generator = generator
        self.fold_factor = fold_factor
        self._shift_mont = self.field.mont(coset_shift) if coset_shift is not None else 0

    def _key(self):
        return (self.message_len, self.block_len, self.field.id, self.coset_shift,
                self.fold_factor, self.generator)

    def __eq__(self, other) -> bool:
        return isinstance(other, ReedSolomon) and self._key() == other._key()

    def __hash__(self) -> int:
        return hash(self._key())

    @property
    def log_blowup(self) -> int:
        return _log2(self.blowup)

    def encode(self, message: torch.Tensor, out: torch.Tensor | None = None, *,
               ef4: bool = False) -> torch.Tensor:
        """Coset LDE of the last axis. `ef4=True`: the message is EF4 with the 4
        coefficients on a trailing axis ([..., k, 4]); the base-field roots make
        the transform act limb by limb, as lax.ntt decomposes extension fields."""
        if ef4:
            if message.shape[-1] != 4:
                raise ValueError("an EF4 message needs a trailing axis of 4 limbs")
            limbs = message.movedim(-1, -2).contiguous()  # [..., 4, k]
            cw = self.encode(limbs)
            return cw.movedim(-2, -1).contiguous()
        if message.shape[-1] != self.message_len:
            raise ValueError(f"message last axis must be {self.message_len}, "
                             f"got {message.shape[-1]}")
        return rs_encode(self.field, message, self.log_blowup, self._shift_mont,
                         self.generator or 0, out)

    def extend(self, evals: torch.Tensor) -> torch.Tensor:
        """LDE of the base-subgroup evaluations to the block-length (coset)
        codeword: encode(INTT(evals)) (zorch/coding/reed_solomon.py:190-208)."""
        if evals.shape[-1] != self.message_len:
            raise ValueError(f"evals last axis must be {self.message_len}, "
                             f"got {evals.shape[-1]}")
        return self.encode(intt(self.field, evals, self.generator or 0))

    def domain(self) -> torch.Tensor:
        return eval_domain(self.field, self.block_len, shift=self.coset_shift,
                           generator=self.generator)

    def level_shift_mont(self, level: int) -> int:
        """coset_shift^(2^level) in Montgomery form (zorch/coding/reed_solomon.py:331-339)."""
        if self.coset_shift is None:
            return 0
        return self.field.mont(pow(self.coset_shift, 1 << level, self.field.p))

    def level_of(self, n: int) -> int:
        return _log2(self.block_len // n)

    def fold(self, codeword: torch.Tensor, beta: torch.Tensor,
             out: torch.Tensor | None = None) -> torch.Tensor:
        """Natural-order (x, -x) fold; base layers are [n], EF4 layers [n, 4];
        beta is a device tensor of 1 (base) or 4 (EF4) words."""
        n = codeword.shape[0]
        if n < 2:
            raise ValueError(f"fri_fold requires a codeword of length >= 2, got {n}")
        ef_in = codeword.dim() == 2
        ef_beta = beta.numel() == 4
        lo = 4 if (ef_in or ef_beta) else 1
        if out is None:
            shape = (n // 2, 4) if lo == 4 else (n // 2,)
            out = torch.empty(shape, dtype=torch.int32, device=codeword.device)
        level = self.level_of(n)
        _lib.check(_lib.lib().zc_fri_fold(self.field.id, ptr(codeword), n, int(ef_in),
                                          ptr(beta.contiguous()), int(ef_beta),
                                          self.level_shift_mont(level), self.generator or 0,
                                          ptr(out), stream_handle()), "fri_fold")
        return out

    def pair_leaves(self, codeword: torch.Tensor) -> torch.Tensor:
        """Leaf p = (cw[p], cw[p + n/2]) in base limbs (materialised copy)."""
        half = codeword.shape[0] // 2
        return torch.stack([codeword[:half], codeword[half:]], dim=1).reshape(half, -1)

    def pair_indices(self, positions: torch.Tensor, level: int):
        return positions, positions + (self.block_len >> (level + 1))

    def layer_positions(self, positions: torch.Tensor, num_rounds: int) -> list[torch.Tensor]:
        """a_i = q_i mod (n / 2^{i+1}) (zorch/coding/reed_solomon.py:320-329)."""
        out, q = [], positions
        for i in range(num_rounds):
            q = torch.remainder(q, self.block_len >> (i + 1))
            out.append(q)
        return out

    def check_final(self, final: torch.Tensor, claim: torch.Tensor) -> bool:
        return bool((final == claim).all())

    # -- KFoldableCode: the k-ary fold (zorch/coding/reed_solomon.py:340-426) --
    @property
    def log_fold_factor(self) -> int:
        return _log2(self.fold_factor)

    def group_level_shift_mont(self, level: int) -> int:
        """coset_shift^(k^level) (:418-426)."""
        return self.level_shift_mont(self.log_fold_factor * level)

    def group_level_of(self, n: int) -> int:
        return _log2(self.block_len // n) // self.log_fold_factor

    def fold_group(self, codeword: torch.Tensor, beta: torch.Tensor,
                   out: torch.Tensor | None = None) -> torch.Tensor:
        """k-ary fold of a natural-order layer (:357-381): n -> n/k."""
        k = self.fold_factor
        n = codeword.shape[0]
        if n < k:
            raise ValueError(f"fold_group requires a codeword length >= fold_factor {k}, got {n}")
        ef_in = codeword.dim() == 2
        ef_beta = beta.numel() == 4
        if out is None:
            shape = (n // k, 4) if (ef_in or ef_beta) else (n // k,)
            out = torch.empty(shape, dtype=torch.int32, device=codeword.device)
        level = self.group_level_of(n)
        _lib.check(_lib.lib().zc_fri_fold_k(
            self.field.id, ptr(codeword.contiguous()), n, int(ef_in), ptr(beta.contiguous()),
            int(ef_beta), self.log_fold_factor, self.group_level_shift_mont(level),
            self.generator or 0, ptr(out), stream_handle()), "fri_fold_k")
        return out

    def group_leaves(self, codeword: torch.Tensor) -> torch.Tensor:
        """Leaf p = (cw[p], cw[p + n/k], ..., cw[p + (k-1)n/k]) in base limbs
        (materialised; the commit round addresses it in place)."""
        k = self.fold_factor
        n = codeword.shape[0]
        return codeword.reshape(k, n // k, -1).transpose(0, 1).reshape(n // k, -1)

    def group_indices(self, positions: torch.Tensor, level: int) -> tuple:
        sub = self.block_len >> (self.log_fold_factor * (level + 1))
        return tuple(positions + m * sub for m in range(self.fold_factor))

    def group_layer_positions(self, positions: torch.Tensor, num_rounds: int) -> list:
        """a_i = q_i mod (n / k^{i+1}) (:395-406)."""
        out, q = [], positions
        for i in range(num_rounds):
            q = torch.remainder(q, self.block_len >> (self.log_fold_factor * (i + 1)))
            out.append(q)
        return out

    def fold_group_values(self, group, beta, positions, level: int) -> list:
        """Host-side k-ary fold of opened groups (the verifier's path, :383-393):
        `group` [Q, k] (or [Q, k, 4]) Montgomery words, `beta` 1 or 4 words,
        `positions` [Q]; returns canonical EF4 tuples."""
        f = self.field
        g = np.asarray(group).reshape(len(positions), self.fold_factor, -1)
        b = [int(x) for x in np.asarray(beta).reshape(-1)]
        bt = f.ef_from_mont((b + [0, 0, 0])[:4])
        n = self.block_len >> (self.log_fold_factor * level)
        w = f.root_of_unity(_log2(n), self.generator or None)
        sh = f.canon(self.group_level_shift_mont(level)) if self.coset_shift is not None else 1
        out = []
        for qi, p in enumerate(int(x) for x in np.asarray(positions).reshape(-1)):
            xs = [sh * pow(w, p + m * (n // self.fold_factor), f.p) % f.p
                  for m in range(self.fold_factor)]
            acc = (0, 0, 0, 0)
            for m in range(self.fold_factor):
                num, den = (1, 0, 0, 0), 1
                for j in range(self.fold_factor):
                    if j != m:
                        num = f.ef_mul(num, f.ef_sub(bt, (xs[j], 0, 0, 0)))
                        den = den * (xs[m] - xs[j]) % f.p
                lm = f.ef_scale(num, pow(den, f.p - 2, f.p))
                words = [int(x) for x in g[qi, m]]
                val = f.ef_from_mont(words + [0] * (4 - len(words)))
                acc = f.ef_add(acc, f.ef_mul(val, lm))
            out.append(acc)
        return out


def bit_reverse_indices(positions: torch.Tensor, n: int) -> torch.Tensor:
    """Each index reversed over log2(n) bits (zorch/coding/reed_solomon.py:429-437)."""
    bits = _log2(n)
    rev = torch.zeros_like(positions)
    for b in range(bits):
        rev |= ((positions >> b) & 1) << (bits - 1 - b)
    return rev


class BitReversedReedSolomon:
    """Reed-Solomon with codewords in bit-reversed evaluation order
    (zorch/coding/reed_solomon.py:440-540): the pair (f(x), f(-x)) of a fold
    sits at (2p, 2p+1), and folding a bit-reversed layer yields the next
    layer, again bit-reversed. The fold math is ReedSolomon's."""

    bit_reversed = True

    def __init__(self, message_len: int, blowup: int, field=BABYBEAR, *,
                 coset_shift: int | None = None) -> None:
        self._natural = ReedSolomon(message_len, blowup, field, coset_shift=coset_shift)
        self.message_len = message_len
        self.blowup = blowup
        self.block_len = self._natural.block_len
        self.field = self._natural.field
        self.coset_shift = coset_shift
        self.generator = None
        self._shift_mont = self._natural._shift_mont

    def __eq__(self, other) -> bool:
        return isinstance(other, BitReversedReedSolomon) and self._natural == other._natural

    def __hash__(self) -> int:
        return hash((BitReversedReedSolomon, self._natural))

    @property
    def log_blowup(self) -> int:
        return self._natural.log_blowup

    def encode(self, message: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """Coset LDE of the last axis in bit-reversed order (:476-478)."""
        if message.shape[-1] != self.message_len:
            raise ValueError(f"message last axis must be {self.message_len}, "
                             f"got {message.shape[-1]}")
        return rs_encode(self.field, message, self.log_blowup, self._natural._shift_mont, 0, out,
                         bit_reversed=True)

    def domain(self) -> torch.Tensor:
        """The points `encode` evaluates on, in codeword (bit-reversed) order."""
        d = self._natural.domain()
        return d.index_select(0, bit_reverse_indices(
            torch.arange(d.shape[0], device=d.device), d.shape[0]))

    def fold(self, codeword: torch.Tensor, beta: torch.Tensor,
             out: torch.Tensor | None = None) -> torch.Tensor:
        """Adjacent-pair fold (:484-492); base layers [n], EF4 layers [n, 4]."""
        n = codeword.shape[0]
        if n < 2:
            raise ValueError(f"fold requires a codeword of length >= 2, got {n}")
        ef_in = codeword.dim() == 2
        ef_beta = beta.numel() == 4
        if out is None:
            shape = (n // 2, 4) if (ef_in or ef_beta) else (n // 2,)
            out = torch.empty(shape, dtype=torch.int32, device=codeword.device)
        level = self._natural.level_of(n)
        _lib.check(_lib.lib().zc_fri_fold_bitrev(
            self.field.id, ptr(codeword.contiguous()), n, int(ef_in), ptr(beta.contiguous()),
            int(ef_beta), self._natural.level_shift_mont(level), 0, ptr(out), stream_handle()),
            "fri_fold_bitrev")
        return out

    def level_shift_mont(self, level: int) -> int:
        return self._natural.level_shift_mont(level)

    def level_of(self, n: int) -> int:
        return self._natural.level_of(n)

    def pair_indices(self, positions: torch.Tensor, level: int):
        """The pair landing at `positions` is adjacent (:508-510)."""
        return positions * 2, positions * 2 + 1

    def pair_leaves(self, codeword: torch.Tensor) -> torch.Tensor:
        """Leaf p = (codeword[2p], codeword[2p+1]) in base limbs: a view (:512-515)."""
        return codeword.reshape(codeword.shape[0] // 2, -1)

    def layer_positions(self, positions: torch.Tensor, num_rounds: int) -> list[torch.Tensor]:
        """Each fold halves the index, a_i = q >> (i+1) (:517-524)."""
        out, q = [], positions
        for _ in range(num_rounds):
            q = q >> 1
            out.append(q)
        return out

    def check_final(self, final: torch.Tensor, claim: torch.Tensor) -> bool:
        return self._natural.check_final(final, claim)
