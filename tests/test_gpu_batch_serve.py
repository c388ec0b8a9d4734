"""Batched and served paths: identical bytes to the per-matrix path and to the
oracle, whatever the batch composition (integer work: exact equality)."""

from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import serve_oracle  # noqa: E402
from zorch_gb300 import _lib  # noqa: E402
from zorch_gb300.field import BABYBEAR, to_host  # noqa: E402

SHAPES = [  # (width, log_h, log_blowup)
    (1, 12, 1), (3, 10, 2), (64, 13, 2), (5, 15, 1), (17, 9, 3), (2, 16, 2), (128, 12, 3),
    (1, 17, 1), (9, 14, 2), (4, 4, 1), (1, 0, 1),
]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")


def _mats(seed=0):
    from zorch_gb300.field import ptr, stream_handle

    out = []
    for i, (w, lh, lb) in enumerate(SHAPES):
        x = torch.empty((w, 1 << lh), dtype=torch.int32, device="cuda")
        _lib.check(_lib.lib().zc_fill_uniform(0, ptr(x), x.numel(), 1000 * seed + i,
                                              stream_handle()), "fill")
        from zorch_gb300.field import to_mont

        out.append((to_mont(BABYBEAR, x), lb))
    return out


@pytest.mark.parametrize("tile", [0, 13, 15])
def test_batched_encode_equals_per_matrix(tile):
    from zorch_gb300.batch import BatchCommitter, MatrixJob
    from zorch_gb300.coding import rs_encode

    mats = _mats(1)
    bc = BatchCommitter(tile_override=tile)
    outs = bc.encode([MatrixJob(x, lb) for x, lb in mats])
    for (x, lb), o in zip(mats, outs):
        want = rs_encode(BABYBEAR, x, lb, BABYBEAR.mont(31), 0)
        assert torch.equal(o, want)


def test_batched_encode_small_workspace_waves():
    """A workspace that fits only one intermediate at a time forces waves and
    the chunked single-job path; the bytes do not change."""
    from zorch_gb300.batch import BatchCommitter, MatrixJob
    from zorch_gb300.coding import rs_encode

    mats = _mats(2)
    bc = BatchCommitter()
    ws = torch.empty((1 << 17) // 4 + 64, dtype=torch.int32, device="cuda")
    outs = bc.encode([MatrixJob(x, lb) for x, lb in mats], workspace=ws)
    for (x, lb), o in zip(mats, outs):
        assert torch.equal(o, rs_encode(BABYBEAR, x, lb, BABYBEAR.mont(31), 0))


def test_batched_merkle_equals_per_matrix_and_oracle(orc):
    from zorch_gb300.batch import BatchCommitter, MatrixJob
    from zorch_gb300.commit import MerkleTree

    mats = _mats(3)
    bc = BatchCommitter()
    committed = bc.commit([MatrixJob(x, lb) for x, lb in mats])
    tree = MerkleTree(bc.perm, column_major=True)
    p2 = orc.Poseidon2.babybear16()
    for c in committed:
        root, layers = tree.commit(c.codeword)
        assert torch.equal(c.layers.flat, layers.flat)
        if c.codeword.numel() <= (1 << 16):
            want = orc.merkle_commit_columns(p2, to_host(c.codeword))
            assert np.array_equal(to_host(c.root), want[-1][0])


def test_graphed_batch_replay():
    from zorch_gb300.batch import BatchCommitter, GraphedBatch, MatrixJob

    mats = _mats(4)
    bc = BatchCommitter()
    g = GraphedBatch(bc, [(x.shape[0], x.shape[1], lb) for x, lb in mats])
    for seed in (5, 6):
        mats = _mats(seed)
        got = g.replay([x for x, _ in mats])
        want = bc.commit([MatrixJob(x, lb) for x, lb in mats])
        for a, b in zip(got, want):
            assert torch.equal(a.codeword, b.codeword)
            assert torch.equal(a.layers.flat, b.layers.flat)


def test_autotuner_choice_keeps_bytes(tmp_path):
    from zorch_gb300.batch import Autotuner, BatchCommitter, MatrixJob

    tuner = Autotuner(tmp_path / "tune.json")
    tl = tuner.tune(14, 8, 2)
    assert tl in (13, 14, 15)
    tuner.save()
    again = Autotuner(tmp_path / "tune.json")
    assert again.tile_log(16, 8) == tl
    c = again.choice(16, 8)
    assert c["radix"] in (3, 4) and c["top"] in (6, 7, 8)
    mats = _mats(7)
    a = BatchCommitter(tuner=tuner).commit([MatrixJob(x, lb) for x, lb in mats])
    b = BatchCommitter().commit([MatrixJob(x, lb) for x, lb in mats])
    for x, y in zip(a, b):
        assert torch.equal(x.layers.flat, y.layers.flat)


def test_large_jobs_on_single_matrix_kernels_keep_bytes():
    """Jobs of at least direct_min_words codeword words run on the single-matrix
    kernels inside a batch (eager and graphed): the codewords and digest
    layers equal those of the work-list kernels, natural and bit-reversed."""
    from zorch_gb300.batch import BatchCommitter, GraphedBatch, MatrixJob

    def fill(w, log_h, seed):
        from zorch_gb300.field import ptr, stream_handle, to_mont

        x = torch.empty((w, 1 << log_h), dtype=torch.int32, device="cuda")
        _lib.check(_lib.lib().zc_fill_uniform(0, ptr(x), x.numel(), seed, stream_handle()), "fill")
        return to_mont(BABYBEAR, x)

    # (width, log2 height, log2 blowup): the first and third reach 2^22 codeword words
    shapes = [(8, 20, 1), (3, 12, 2), (2, 19, 3), (1, 16, 1)]
    mats = [(fill(w, lh, 40 + i), lb) for i, (w, lh, lb) in enumerate(shapes)]
    for br in (False, True):
        jobs = [MatrixJob(x, lb, bit_reversed=br) for x, lb in mats]
        want = BatchCommitter(direct_min_words=0).commit(jobs)
        got = BatchCommitter(direct_min_words=1 << 22).commit(jobs)
        for a, b in zip(got, want):
            assert torch.equal(a.codeword, b.codeword)
            assert torch.equal(a.layers.flat, b.layers.flat)
    g = GraphedBatch(BatchCommitter(direct_min_words=1 << 22), [(x.shape[0], x.shape[1], lb)
                                                                for x, lb in mats])
    want = BatchCommitter(direct_min_words=0).commit([MatrixJob(x, lb) for x, lb in mats])
    for a, b in zip(g.replay([x for x, _ in mats]), want):
        assert torch.equal(a.codeword, b.codeword)
        assert torch.equal(a.layers.flat, b.layers.flat)


@pytest.mark.parametrize("tile,radix,top", [(13, 2, 1), (15, 3, 4), (14, 4, 8), (0, 2, 6)])
def test_tuning_choices_keep_bytes(tile, radix, top):
    """Every tile, radix and tree-top depth the tuner may pick gives the same
    codewords and digest layers as the defaults."""
    from zorch_gb300.batch import BatchCommitter, MatrixJob

    mats = _mats(11)
    forced = BatchCommitter(tile_override=tile, radix_override=radix, top_override=top).commit(
        [MatrixJob(x, lb) for x, lb in mats])
    plain = BatchCommitter().commit([MatrixJob(x, lb) for x, lb in mats])
    for x, y in zip(forced, plain):
        assert torch.equal(x.codeword, y.codeword)
        assert torch.equal(x.layers.flat, y.layers.flat)


def _small_stream(seed, n=10):
    from zorch_gb300.serve import fill_request, make_stream

    reqs = make_stream(n, seed, rate_hz=0.0, log_h=(9, 13), log_w=(0.0, 4.0), fold_frac=0.5)
    for r in reqs:
        fill_request(r)
    torch.cuda.synchronize()
    return reqs


@pytest.mark.parametrize("mode", ["fri", "matrix"])
def test_served_results_same_alone_and_in_the_mix(mode):
    from zorch_gb300.serve import Server

    reqs = _small_stream(11)
    mixed = Server(max_batch=6, streams=2, mode=mode).run(reqs)
    assert [r.rid for r in mixed] == [r.rid for r in reqs]
    for r, m in zip(reqs, mixed):
        alone = Server(max_batch=1, streams=1, mode=mode).run([r])[0]
        assert alone.proof == m.proof
        head = 32 * (r.width if mode == "fri" else 1)
        assert len(m.proof) > head if r.fold else len(m.proof) == head


@pytest.mark.parametrize("mode", ["fri", "matrix"])
def test_served_bytes_equal_plain_path(mode):
    """Like for like: every request of a mixed stream gets the same bytes from
    the continuous-batching server as from the plain one-call-per-polynomial
    ("fri", FriProver.commit per column) or one-call-per-matrix ("matrix",
    BasefoldProver.commit) drop-in path."""
    from zorch_gb300.serve import Server, run_plain

    reqs = _small_stream(17, 12)
    served = Server(max_batch=5, streams=3, mode=mode).run(reqs)
    plain = run_plain(reqs, mode=mode)
    assert [r.rid for r in served] == [r.rid for r in plain]
    for a, b in zip(served, plain):
        assert a.proof == b.proof


def test_batched_pair_trees_equal_per_polynomial_commit(orc):
    """BatchCommitter.commit_polys (every column's pair-leaf tree, tree families
    in one batched commit) == FriProver.commit_one per column == the oracle."""
    from zorch_gb300.batch import BatchCommitter, MatrixJob
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.pcs import FriParams, FriProver

    mats = _mats(21)
    bc = BatchCommitter()
    committed = bc.commit_polys([MatrixJob(x, lb) for x, lb in mats])
    p2 = orc.Poseidon2.babybear16()
    for (x, lb), c in zip(mats, committed):
        h = x.shape[1]
        code = ReedSolomon(h, 1 << lb, BABYBEAR, coset_shift=31, generator=31)
        prover = FriProver(FriParams(code, MerkleTree(bc.perm), 0, 0))
        for col in range(0, x.shape[0], max(1, x.shape[0] // 5)):
            cp = prover.commit_one(x[col])
            assert torch.equal(cp.codeword, c.codeword[col])
            assert torch.equal(cp.digest_layers.flat, c.flat[col])
            assert torch.equal(cp.root, c.roots[col])
            if c.codeword.shape[1] <= (1 << 14):
                cw = to_host(c.codeword[col])
                L = cw.size // 2
                want = orc.merkle_commit(p2, cw, L, 2, 1, L)
                assert np.array_equal(to_host(c.roots[col]), want[-1][0])


def test_served_host_fed_equals_resident():
    """Inputs fed from page-locked host memory (read by the conversion kernel
    over the host link) give the same proofs as inputs already on the device;
    likewise for the plain path."""
    from zorch_gb300.serve import Server, run_plain

    reqs = _small_stream(13)
    for r in reqs:
        r.host = r.resident.cpu().pin_memory()
    for mode in ("fri", "matrix"):
        server = Server(max_batch=4, streams=3, mode=mode)
        resident = server.run(reqs)
        fed = server.run(reqs, host_fed=True)
        assert [a.proof for a in resident] == [b.proof for b in fed]
        plain_fed = run_plain(reqs, host_fed=True, perm=server.perm, mode=mode)
        plain = run_plain(reqs, perm=server.perm, mode=mode)
        assert [a.proof for a in plain] == [b.proof for b in plain_fed]
        assert [a.proof for a in plain] == [b.proof for b in resident]


@pytest.mark.parametrize("mode", ["fri", "matrix"])
def test_served_proofs_match_oracle(orc, mode):
    """Commitment and fold-and-open proof bytes of served requests equal the
    oracle's, replayed from the same seeded data."""
    from zorch_gb300.serve import Server

    reqs = _small_stream(12, 8)
    reqs = [r for r in reqs if r.fold][:2] + [r for r in reqs if not r.fold][:2]
    res = Server(mode=mode).run(reqs)
    p2 = orc.Poseidon2.babybear16()
    for r, got in zip(sorted(reqs, key=lambda q: q.rid), res):
        x = orc.to_mont(0, to_host(r.resident))
        want = serve_oracle.request_words(orc, p2, r, x, mode)
        assert np.array_equal(np.frombuffer(got.proof, dtype=np.uint32), want)


def test_partial_lagrange_batching_matches_oracle(orc):
    from zorch_gb300.serve import batch_columns
    from zorch_gb300.transcript import DuplexTranscript

    for w in (1, 2, 5, 8, 33):
        x = np.random.default_rng(w).integers(0, BABYBEAR.p, size=(w, 64),
                                                dtype=np.uint64).astype(np.uint32)
        xm = orc.to_mont(0, x)
        from zorch_gb300.commit import Poseidon2
        from zorch_gb300.field import to_device

        t = DuplexTranscript.new(Poseidon2.builtin())
        got = to_host(batch_columns(to_device(xm).reshape(w, 64), t))
        to = orc.Transcript(orc.Poseidon2.babybear16())
        nbv = (w - 1).bit_length()
        want = orc.rlc_columns(0, xm, to.sample(4 * nbv) if nbv else [])
        assert np.array_equal(got.reshape(want.shape), want)
        if w == 1:
            assert np.array_equal(want[:, 0], xm[0]) and not want[:, 1:].any()


def test_plain_path_per_polynomial_roots(orc):
    from zorch_gb300.serve import run_plain

    reqs = [r for r in _small_stream(13, 6)][:3]
    res = run_plain(reqs, mode="fri")
    p2 = orc.Poseidon2.babybear16()
    for r, got in zip(reqs, res):
        x = orc.to_mont(0, to_host(r.resident))
        words = np.frombuffer(got.proof, dtype=np.uint32)
        for c in range(r.width):
            cw = orc.rs_encode(0, x[c], r.log_blowup, BABYBEAR.mont(31))
            L = cw.size // 2
            root = orc.merkle_commit(p2, cw, L, 2, 1, L)[-1][0]
            assert np.array_equal(words[8 * c: 8 * c + 8], root)


def test_chunked_pair_trees_keep_roots():
    """Trees committed in column chunks through a reused buffer (the unopened
    wide requests of the server) give the same roots as the whole family."""
    from zorch_gb300.batch import BatchCommitter, MatrixJob

    mats = _mats(22)
    bc = BatchCommitter()
    jobs = [MatrixJob(x, lb) for x, lb in mats]
    whole = bc.commit_polys(jobs)
    for cap in (1, 32 * 3 * (1 << 15)):
        chunked = bc.commit_polys(jobs, keep_layers=[False] * len(jobs), layer_cap=cap)
        for a, b in zip(whole, chunked):
            assert torch.equal(a.roots, b.roots)
            assert torch.equal(a.codeword, b.codeword)
