"""Field descriptors and canonical <-> Montgomery conversion.

Device data is Montgomery u32 (x * 2^32 mod p) held in torch.int32 tensors as
raw bit patterns -- the storage of zk_dtypes' `babybear_mont` /
`koalabear_mont` and the reference's Fiat-Shamir wire form
(zorch/transcript.py:986-999).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _lib


@dataclass(frozen=True)
class Field:
    id: int
    name: str
    p: int
    generator: int
    two_adicity: int
    ef4_w: int  # EF4 = F[x]/(x^4 - w)

    @property
    def one_mont(self) -> int:
        return (1 << 32) % self.p

    def mont(self, x: int) -> int:
        return ((x % self.p) << 32) % self.p

    def canon(self, x: int) -> int:
        return x * pow(1 << 32, self.p - 2, self.p) % self.p

    def mul_mont(self, a: int, b: int) -> int:
        return a * b * pow(1 << 32, self.p - 2, self.p) % self.p

    def pow_mont(self, a: int, e: int) -> int:
        return self.mont(pow(self.canon(a), e, self.p))

    def inv_mont(self, a: int) -> int:
        return self.mont(pow(self.canon(a), self.p - 2, self.p))

    def root_of_unity(self, log_n: int, generator: int | None = None) -> int:
        g = generator or self.generator
        return pow(g, (self.p - 1) >> log_n, self.p)


    # -- EF4 = F[x]/(x^4 - w) on the host, canonical coefficient tuples (c0..c3);
    # verifier-side scalar arithmetic (a few operations per round or query).
    def ef_mul(self, a, b) -> tuple:
        p, w = self.p, self.ef4_w
        t = [0] * 7
        for i in range(4):
            for j in range(4):
                t[i + j] += a[i] * b[j]
        return tuple((t[i] + (w * t[i + 4] if i < 3 else 0)) % p for i in range(4))

    def ef_add(self, a, b) -> tuple:
        return tuple((x + y) % self.p for x, y in zip(a, b))

    def ef_sub(self, a, b) -> tuple:
        return tuple((x - y) % self.p for x, y in zip(a, b))

    def ef_scale(self, a, s: int) -> tuple:
        return tuple(x * s % self.p for x in a)

    def ef_inv(self, a) -> tuple:
        """a^(p^4 - 2)."""
        e = self.p ** 4 - 2
        r, b = (1, 0, 0, 0), tuple(a)
        while e:
            if e & 1:
                r = self.ef_mul(r, b)
            b = self.ef_mul(b, b)
            e >>= 1
        return r

    def ef_from_mont(self, words) -> tuple:
        return tuple(self.canon(int(x)) for x in words)

    def ef_to_mont(self, a) -> list:
        return [self.mont(x) for x in a]


BABYBEAR = Field(_lib.BABYBEAR, "babybear", 2013265921, 31, 27, 11)
KOALABEAR = Field(_lib.KOALABEAR, "koalabear", 2130706433, 3, 24, 3)
FIELDS = {BABYBEAR.id: BABYBEAR, KOALABEAR.id: KOALABEAR}


def field_of(f: "Field | int | str") -> Field:
    if isinstance(f, Field):
        return f
    if isinstance(f, str):
        return {"babybear": BABYBEAR, "koalabear": KOALABEAR}[f.lower()]
    return FIELDS[int(f)]


# ---------------------------------------------------------------- host ----
def to_mont_np(field, x) -> np.ndarray:
    f = field_of(field)
    x = np.asarray(x, dtype=np.uint64) % np.uint64(f.p)
    return ((x << np.uint64(32)) % np.uint64(f.p)).astype(np.uint32)


def from_mont_np(field, x) -> np.ndarray:
    f = field_of(field)
    rinv = np.uint64(pow(1 << 32, f.p - 2, f.p))
    x = np.asarray(x, dtype=np.uint64)
    # x < p < 2^31 and rinv < 2^31, so the product fits in 62 bits
    return ((x * rinv) % np.uint64(f.p)).astype(np.uint32)


# -------------------------------------------------------------- device ----
def stream_handle(stream: torch.cuda.Stream | None = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def ptr(t: torch.Tensor | None) -> int | None:
    """Device pointer of a contiguous 32-bit CUDA tensor (None passes through)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if t.element_size() != 4:
        raise ValueError(f"expected a 32-bit tensor, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return t.data_ptr()


def to_device(x: np.ndarray, device="cuda") -> torch.Tensor:
    """Host u32 array -> int32 device tensor of the same bits."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.uint32)).view(np.int32)
    return torch.from_numpy(a).to(device)


def to_host(t: torch.Tensor) -> np.ndarray:
    """int32 device tensor -> u32 host array of the same bits."""
    return t.detach().contiguous().cpu().numpy().view(np.uint32)


def full_u32(shape, value: int = 0, device="cuda") -> torch.Tensor:
    """An int32 device tensor with every word set to `value` (a u32 bit
    pattern) on the current stream by zc_fill_u32: a memset for zero, else
    the library's fill kernel -- no framework kernel and no host copy."""
    t = torch.empty(shape, dtype=torch.int32, device=device)
    _lib.check(_lib.lib().zc_fill_u32(ptr(t), t.numel(), int(value) & 0xFFFFFFFF,
                                      stream_handle()), "fill_u32")
    return t


def copy_rows(dst: torch.Tensor, src: torch.Tensor) -> torch.Tensor:
    """dst[i] = src[i] for 2D device tensors whose rows are contiguous (inner
    stride 1) but may sit at any row pitch -- e.g. every tree's root row out
    of a stack of digest layers -- as one 2D copy-engine transfer on the
    current stream (zc_copy_rows), not a framework gather kernel."""
    if src.dim() != 2 or dst.shape != src.shape or dst.dtype != src.dtype:
        raise ValueError(f"copy_rows: 2D tensors of one shape and dtype, got "
                         f"{tuple(dst.shape)} {dst.dtype} and {tuple(src.shape)} {src.dtype}")
    rows, cols = src.shape
    if rows == 0 or cols == 0:
        return dst
    if (cols > 1 and (src.stride(1) != 1 or dst.stride(1) != 1)) or not (src.is_cuda and dst.is_cuda):
        raise ValueError("copy_rows: rows must be contiguous device memory")
    es = src.element_size()
    row = cols * es  # a single row's pitch is free (its stride may be anything)
    dp = dst.stride(0) * es if rows > 1 else row
    sp = src.stride(0) * es if rows > 1 else row
    _lib.check(_lib.lib().zc_copy_rows(dst.data_ptr(), dp, src.data_ptr(), sp, row, rows,
                                       stream_handle()), "copy_rows")
    return dst


def parts_to_pinned(parts: list[torch.Tensor]) -> torch.Tensor:
    """Concatenate device tensors into one page-locked host buffer with one
    asynchronous device->host copy per part on the current stream (copy
    engine only, no gather kernel). The result is valid once the stream has
    reached the copies (synchronise or record an event)."""
    flat = [p.reshape(-1) for p in parts]
    total = sum(p.numel() for p in flat)
    host = torch.empty(total, dtype=torch.int32, pin_memory=True)
    off = 0
    for p in flat:
        if p.numel():
            host[off: off + p.numel()].copy_(p, non_blocking=True)
        off += p.numel()
    return host


def parts_to_bytes(parts: list[torch.Tensor]) -> bytes:
    """Mont-u32 little-endian bytes of the parts in order (one device->host
    copy per part, then one stream synchronisation)."""
    host = parts_to_pinned(parts)
    torch.cuda.current_stream().synchronize()
    return host.numpy().view(np.uint32).astype("<u4").tobytes()


def to_mont(field, t: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """Canonical -> Montgomery on the device (zc_to_mont)."""
    f = field_of(field)
    out = torch.empty_like(t) if out is None else out
    _lib.check(_lib.lib().zc_to_mont(f.id, ptr(t), ptr(out), t.numel(), stream_handle()),
               "to_mont")
    return out


def to_mont_from_host(field, host: torch.Tensor, out: torch.Tensor | None = None,
                      device="cuda", max_ctas: int = 0) -> torch.Tensor:
    """Canonical page-locked host words -> Montgomery device words in one
    kernel that reads the host buffer directly over the host link
    (zc_to_mont_from_host): no staging copy through the copy engine, and a
    bounded number of CTAs (max_ctas, 0 = the library default) so the
    kernels of other streams keep most SMs. `host` must be pinned
    (ValueError otherwise)."""
    f = field_of(field)
    if host.device.type != "cpu" or not host.is_pinned():
        raise ValueError("to_mont_from_host needs a page-locked (pinned) host tensor")
    src = host.contiguous()
    if out is None:
        out = torch.empty(src.shape, dtype=torch.int32, device=device)
    _lib.check(_lib.lib().zc_to_mont_from_host(f.id, src.data_ptr(), ptr(out), src.numel(),
                                               max_ctas, stream_handle()), "to_mont_from_host")
    return out


def from_mont(field, t: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    f = field_of(field)
    out = torch.empty_like(t) if out is None else out
    _lib.check(_lib.lib().zc_from_mont(f.id, ptr(t), ptr(out), t.numel(), stream_handle()),
               "from_mont")
    return out


def random_canonical(field, shape, seed: int) -> np.ndarray:
    """Seeded uniform draw in [0, p) (PCG64 via numpy.random.default_rng)."""
    f = field_of(field)
    return np.random.default_rng(seed).integers(0, f.p, size=shape, dtype=np.uint64).astype(np.uint32)
