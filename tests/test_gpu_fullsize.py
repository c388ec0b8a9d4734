"""The configurations at their full sizes, byte for byte against the oracle
(its C restatement runs with OpenMP on every host core):

- config 2: the 2^20 x 64 trace at blowup 4 -- the root and all 128 opened
  rows and authentication paths;
- config 3: the FRI commit phase at 2^22 coefficients, blowup 2, 15 rounds,
  100 queries -- the proof bytes;
- config 4: the bench's own 48 seeded uneven matrices -- all 48 roots of the
  batched commit;
- config 5: the bench's own 24-request served stream -- every request of at
  most 2^20 rows (commitment and fold-and-open proof, per-polynomial and
  row-leaf modes); the taller requests equal the plain path's bytes, and
  one column of the tallest request equals the oracle's pair-leaf root.

Size-independent properties are checked beside the bytes: opened rows equal
the codeword, paths rebuild the root through the oracle's hash, codeword
entries equal a Horner evaluation of the message on the coset domain.
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


def test_config2_trace_commit_bytes(orc):
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
    root_h, rows, paths = to_host(root), to_host(op.row), to_host(op.path)
    # the oracle: LDE, row-leaf tree, openings
    p2 = orc.Poseidon2.babybear16()
    xm_h = orc.to_mont(0, x)
    cw_o = orc.rs_encode(0, xm_h, log_b, BABYBEAR.mont(31))
    layers = orc.merkle_commit_columns(p2, cw_o)
    rows_o, paths_o = orc.merkle_open(cw_o, n, w, 1, n, layers, idx)
    assert np.array_equal(root_h, layers[-1][0])
    assert np.array_equal(rows, rows_o.reshape(rows.shape))
    assert np.array_equal(paths, paths_o.reshape(paths.shape))
    # properties beside the bytes: paths rebuild the root, entries are Horner
    for q in range(0, Q, 16):
        assert np.array_equal(orc.reconstruct_root(p2, rows[q], int(idx[q]), paths[:, q]), root_h)
    sh = BABYBEAR.mont(31)
    for c in rng.integers(0, w, size=3):
        for j in rng.integers(0, n, size=4):
            pt = orc.domain_point(0, log_h + log_b, sh, int(j))
            assert int(cw_o[int(c), int(j)]) == orc.eval_poly(0, xm_h[c], pt)


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


def test_config4_uneven_batch_bytes(orc):
    """The bench's 48 uneven matrices (seed 5: widths 1..128, log2 heights
    12..22, blowup 2/4/8, zc_fill_uniform data seeded 900 + i), one batched
    commit: every codeword's root equals the oracle's, and a per-matrix
    commit gives the same digest layers."""
    from zorch_gb300.batch import BatchCommitter, MatrixJob
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.field import ptr, stream_handle

    rng = np.random.default_rng(5)
    shapes = [(int(rng.integers(1, 129)), int(rng.integers(12, 23)), int(rng.choice([1, 2, 3])))
              for _ in range(48)]
    canon = []
    for i, (w, lh, lb) in enumerate(shapes):
        xx = torch.empty((w, 1 << lh), dtype=torch.int32, device="cuda")
        _lib.check(_lib.lib().zc_fill_uniform(0, ptr(xx), xx.numel(), 900 + i, stream_handle()),
                   "fill")
        canon.append(xx)
    # every job on the work-list kernels (direct_min_words=0), then the default
    # routing (the largest jobs on the single-matrix kernels): same roots
    bc = BatchCommitter(direct_min_words=0)
    jobs = [MatrixJob(to_mont(BABYBEAR, x), lb) for x, (_, _, lb) in zip(canon, shapes)]
    batched = bc.commit(jobs)
    roots = [to_host(b.root) for b in batched]
    routed = BatchCommitter().commit(jobs)
    assert all(np.array_equal(to_host(r.root), root) for r, root in zip(routed, roots))
    del routed, jobs
    tree = MerkleTree(bc.perm, column_major=True)
    for b in batched[:6]:  # per-matrix commit == batched, layer for layer
        _, layers = tree.commit(b.codeword)
        assert torch.equal(layers.flat, b.layers.flat)
    hosts = [to_host(x) for x in canon]
    del batched, canon
    torch.cuda.empty_cache()
    p2 = orc.Poseidon2.babybear16()
    for (w, lh, lb), x, root in zip(shapes, hosts, roots):
        cw = orc.rs_encode(0, orc.to_mont(0, x), lb, BABYBEAR.mont(31))
        assert np.array_equal(orc.merkle_commit_columns(p2, cw)[-1][0], root), (w, lh, lb)
        del cw


def test_config5_served_stream_bytes(orc):
    """The bench's 24-request stream (seed 5, heights 2^14..2^24, widths
    1..256, blowup 2|4, 30% fold-and-open) served in both modes: each request
    of at most 2^20 rows is byte-identical to the oracle's replay; every
    taller one equals the plain path's bytes, and the tallest request's first
    column root equals the oracle's pair-leaf root."""
    import serve_oracle
    from zorch_gb300.serve import Server, fill_request, make_stream, run_plain

    reqs = make_stream(24, 5, rate_hz=0.0, log_h=(14, 24))
    for r in reqs:
        fill_request(r)
    torch.cuda.synchronize()
    p2 = orc.Poseidon2.babybear16()
    for mode in ("fri", "matrix"):
        served = Server(max_batch=8, streams=4, mode=mode).run(reqs)
        small = [r for r in reqs if r.log_h <= 20]
        tall = [r for r in reqs if r.log_h > 20]
        assert len(small) >= 12
        for r in small:
            want = serve_oracle.request_words(orc, p2, r, orc.to_mont(0, to_host(r.resident)),
                                              mode)
            assert np.array_equal(np.frombuffer(served[r.rid].proof, np.uint32), want), r
        plain = run_plain(tall, mode=mode)
        for r, pl in zip(tall, plain):
            assert served[r.rid].proof == pl.proof, r
        if mode == "fri":
            top = max(tall, key=lambda q: (q.log_h, q.log_blowup))
            col = orc.to_mont(0, to_host(top.resident[0]))
            cw = orc.rs_encode(0, col, top.log_blowup, BABYBEAR.mont(31))
            L = cw.size // 2
            root = orc.merkle_commit(p2, cw, L, 2, 1, L)[-1][0]
            assert np.array_equal(np.frombuffer(served[top.rid].proof, np.uint32)[:8], root)
        del served
        torch.cuda.empty_cache()
