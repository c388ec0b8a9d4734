"""The configurations at their full sizes.

Where the oracle finishes in seconds the comparison is byte for byte (the
config-3 commit phase at 2^22 coefficients, blowup 2, 15 rounds, 100
queries). Where it would not (the 2^20 x 64 trace at blowup 4, the 48-matrix
uneven batch), size-independent properties are checked instead: every opened
row equals the codeword there, every authentication path rebuilds the root
through the oracle's hash, codeword entries equal a Horner evaluation of the
message on the coset domain, internal nodes equal the compression of their
children, and the batched path equals the per-matrix path exactly.
"""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from zorch_gb300 import _lib  # noqa: E402
from zorch_gb300.field import BABYBEAR, to_device, to_host, to_mont  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")


def _canonical(shape, seed):
    return np.random.default_rng(seed).integers(0, BABYBEAR.p, size=shape,
                                                dtype=np.uint64).astype(np.uint32)


def test_config2_trace_commit_properties(orc):
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2
    from zorch_gb300.pcs import BasefoldProver

    log_h, w, log_b, Q = 20, 64, 2, 128
    x = _canonical((w, 1 << log_h), 2)
    code = ReedSolomon(1 << log_h, 1 << log_b, BABYBEAR, coset_shift=31, generator=31)
    prover = BasefoldProver(code, MerkleTree(Poseidon2.builtin(), column_major=True))
    xm = to_mont(BABYBEAR, to_device(x).reshape(w, -1))
    root, data = prover.commit_columns(xm)
    n = 1 << (log_h + log_b)
    rng = np.random.default_rng(3)
    idx = rng.integers(0, n, size=Q).astype(np.int32)
    op = prover.open_rows(data, torch.from_numpy(idx).cuda())
    p2 = orc.Poseidon2.babybear16()
    root_h = to_host(root)
    rows, paths = to_host(op.row), to_host(op.path)
    cw_cols = {}
    for q in range(Q):
        assert np.array_equal(orc.reconstruct_root(p2, rows[q], int(idx[q]), paths[:, q]), root_h)
    # opened rows are the codeword's rows
    cw = data.codeword
    gathered = to_host(cw[:, torch.from_numpy(idx).long().cuda()].T.contiguous())
    assert np.array_equal(gathered, rows)
    # codeword entries = Horner of the message on shift * w^j
    xm_h = orc.to_mont(0, x)
    sh = BABYBEAR.mont(31)
    for c in rng.integers(0, w, size=3):
        for j in rng.integers(0, n, size=4):
            pt = orc.domain_point(0, log_h + log_b, sh, int(j))
            cw_cols.setdefault(int(c), None)
            assert int(to_host(cw[int(c), int(j)].reshape(1))[0]) == orc.eval_poly(0, xm_h[c], pt)
    # internal nodes compress their children
    for level in (1, 5, 12, 22):
        lay, below = to_host(data.digest_layers[level]), data.digest_layers[level - 1]
        for i in rng.integers(0, lay.shape[0], size=3):
            kids = to_host(below[2 * int(i): 2 * int(i) + 2])
            assert np.array_equal(lay[i], p2.compress(kids[0], kids[1]))


def test_config3_fri_commit_phase_full_size_bytes(orc):
    """2^22 coefficients, blowup 2, EF4 challenges, fold to 2^8 (15 rounds),
    100 queries: proof bytes identical to the oracle's."""
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2
    from zorch_gb300.pcs import FriParams, FriProver
    from zorch_gb300.transcript import DuplexTranscript

    log_k, log_b, R, Q = 22, 1, 15, 100
    x = _canonical(1 << log_k, 4)
    perm = Poseidon2.builtin()
    code = ReedSolomon(1 << log_k, 2, BABYBEAR, coset_shift=31, generator=31)
    cw = code.encode(to_mont(BABYBEAR, to_device(x)))
    proof, _, _ = FriProver(FriParams(code, MerkleTree(perm), R, Q, 4)).commit_phase(
        cw, DuplexTranscript.new(perm))
    got = proof.to_bytes()
    p2 = orc.Poseidon2.babybear16()
    cw_o = orc.rs_encode(0, orc.to_mont(0, x), log_b, BABYBEAR.mont(31))
    assert np.array_equal(to_host(cw), cw_o)
    want = orc.fri_commit_phase(p2, 0, cw_o, R, Q, 4, orc.Transcript(p2), BABYBEAR.mont(31))
    assert proof.final_layer.shape[0] == 1 << 8
    assert got == want.to_bytes()


def test_config4_uneven_batch_equals_per_matrix(orc):
    """48 matrices, log2 heights 12..22, widths 1..128, blowup 2/4/8, one
    batched launch set vs 48 per-matrix commits; paths verify via the oracle."""
    from zorch_gb300.batch import BatchCommitter, MatrixJob
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.field import ptr, stream_handle

    rng = np.random.default_rng(44)
    shapes = [(int(rng.integers(1, 129)), int(rng.integers(12, 23)), int(rng.choice([1, 2, 3])))
              for _ in range(48)]
    mats = []
    for i, (w, lh, lb) in enumerate(shapes):
        xx = torch.empty((w, 1 << lh), dtype=torch.int32, device="cuda")
        _lib.check(_lib.lib().zc_fill_uniform(0, ptr(xx), xx.numel(), 4400 + i, stream_handle()),
                   "fill")
        mats.append((to_mont(BABYBEAR, xx), lb))
    bc = BatchCommitter()
    batched = bc.commit([MatrixJob(x, lb) for x, lb in mats])
    tree = MerkleTree(bc.perm, column_major=True)
    from zorch_gb300.coding import rs_encode

    p2 = orc.Poseidon2.babybear16()
    for (x, lb), b in zip(mats, batched):
        cw = rs_encode(BABYBEAR, x, lb, BABYBEAR.mont(31), 0)
        assert torch.equal(cw, b.codeword)
        root, _ = tree.commit(cw)
        assert torch.equal(root, b.root)
        idx = torch.from_numpy(rng.integers(0, cw.shape[1], size=2).astype(np.int32)).cuda()
        op = tree.open_layout(_lib.Leaves(ptr(cw), cw.shape[1], cw.shape[0], 1, cw.shape[1]),
                              b.layers, idx, cw.shape[0])
        rows, paths = to_host(op.row), to_host(op.path)
        for q in range(2):
            assert np.array_equal(
                orc.reconstruct_root(p2, rows[q], int(idx[q]), paths[:, q]), to_host(b.root))
    del batched
    torch.cuda.empty_cache()
