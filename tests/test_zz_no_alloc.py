"""zc_rs_encode_noalloc: the LDE entry point that allocates nothing.

It exists for callers that cannot allocate device memory when they call in:
an XLA/FRX custom-call handler, whose framework owns the GPU's memory and
preallocates most of it, or a serving loop that must not stall on the
allocator. Its four-step intermediate lives in a fixed 64 MiB static device
array; this file checks, through the C ABI, that its output equals the
workspace entry point's (zc_rs_encode) exactly, on two calls in a row, and
that a column too large for the fixed array is refused. Collected last on
purpose: the other GPU tests have run when it runs.
"""

from __future__ import annotations

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from zorch_gb300 import _lib  # noqa: E402
from zorch_gb300.field import BABYBEAR, KOALABEAR, ptr, stream_handle  # noqa: E402

# (field, batch, log_k, log_blowup): every case is past the single-pass size
# (k > 4096 or k * blowup > 2^14), so each runs the four-step passes through
# the scratch; the third needs several chunks (2^22-word columns, 4 per
# 2^24-word chunk).
CASES = [(BABYBEAR, 3, 16, 2), (KOALABEAR, 2, 13, 3), (BABYBEAR, 6, 20, 2), (KOALABEAR, 5, 14, 1)]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _data(field, batch, log_k, seed):
    x = torch.empty((batch, 1 << log_k), dtype=torch.int32, device="cuda")
    _lib.check(_lib.lib().zc_fill_uniform(field.id, ptr(x), x.numel(), seed, stream_handle()),
               "fill")
    from zorch_gb300.field import to_mont

    return to_mont(field, x)


def _noalloc(field, x, log_b, shift_mont):
    batch, k = x.shape
    out = torch.empty((batch, k << log_b), dtype=torch.int32, device="cuda")
    _lib.check(_lib.lib().zc_rs_encode_noalloc(field.id, ptr(x), batch, k.bit_length() - 1,
                                               log_b, shift_mont, 0, ptr(out), stream_handle()),
               "rs_encode_noalloc")
    return out


@pytest.mark.parametrize("call", [1, 2])
def test_noalloc_equals_workspace_entry_point(call):
    from zorch_gb300.coding import rs_encode

    for i, (field, batch, log_k, log_b) in enumerate(CASES):
        x = _data(field, batch, log_k, 31 * call + i)
        shift = field.mont(field.generator)
        got = _noalloc(field, x, log_b, shift)
        want = rs_encode(field, x, log_b, shift, 0)  # zc_rs_encode with a caller workspace
        torch.cuda.synchronize()
        assert torch.equal(got, want), (call, field.name, batch, log_k, log_b)


def test_noalloc_refuses_a_column_larger_than_its_scratch():
    x = torch.zeros((1, 1 << 23), dtype=torch.int32, device="cuda")
    out = torch.empty((1, 1 << 25), dtype=torch.int32, device="cuda")
    status = _lib.lib().zc_rs_encode_noalloc(BABYBEAR.id, ptr(x), 1, 23, 2, 0, 0, ptr(out),
                                             stream_handle())
    assert status == _lib.ZC_BAD_SHAPE
    assert "scratch" in _lib.lib().zc_last_error().decode()
