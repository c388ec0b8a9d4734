"""The bit-reversed code, the SP1 single-matrix commitment and the stacked
fold rounds on the GPU, against the reference's SP1 KoalaBear pipeline dump
(tests/golden/sp1_fibonacci) and against the oracle.

The prep-round test runs the whole product path -- BitReversedReedSolomon
encode of the 2^21-word preprocessed column (KoalaBear, blowup 4), the
column-major SMCS commit with SP1's Poseidon2, the openings at the dumped
query positions -- and compares every opened row and sibling digest with the
dump (zorch/pcs/jagged/testing/open_test.py:279-287). The fold test folds the
dumped opened pairs of a fold layer on the GPU and compares with the next
layer's dumped values. Integer work: the tolerance is zero.
"""

from __future__ import annotations

import dataclasses
import lzma

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from zorch_gb300 import _lib  # noqa: E402
from zorch_gb300.field import BABYBEAR, KOALABEAR, to_device, to_host  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.check(_lib.lib().zc_init(0), "init")


def rand_mont(orc, field, shape, seed):
    p = orc.MODULUS[field]
    x = np.random.default_rng(seed).integers(0, p, size=shape, dtype=np.uint64).astype(np.uint32)
    return orc.to_mont(field, x)


def dev(x):
    return to_device(np.asarray(x, np.uint32))


@pytest.fixture(scope="module")
def sp1(orc):
    from zorch_gb300.commit import Poseidon2

    d = orc.load_sp1_fixture()
    gpu = Poseidon2.from_params(KOALABEAR, d["alpha"], d["external_initial"],
                                d["external_terminal"], d["internal_rc"], d["internal_diag"],
                                d["internal_j_scale"])
    return gpu, orc.sp1_koalabear16()


@pytest.fixture(scope="module")
def golden(orc):
    g = orc.GOLDEN / "sp1_fibonacci"
    prep = np.frombuffer(lzma.decompress((g / "prep_dense.u32.xz").read_bytes()), "<u4")
    return {"prep": prep.astype(np.uint32), "round": np.load(g / "prep_round.npz"),
            "chain": np.load(g / "fold_chain.npz")}


def test_prep_round_commit_and_openings_match_sp1_dump(orc, sp1, golden):
    from zorch_gb300.coding import BitReversedReedSolomon
    from zorch_gb300.commit import SingleMatrixCommitmentScheme, VerifyCode
    from zorch_gb300.jagged import sample_query_positions  # noqa: F401  (API surface)

    perm, cpu = sp1
    z = golden["round"]
    S = 1 << int(z["log_stacking_height"])
    code = BitReversedReedSolomon(S, 1 << int(z["log_blowup"]), KOALABEAR)
    smcs = SingleMatrixCommitmentScheme(perm)
    block = dev(golden["prep"]).reshape(1, S)  # stacked column-major: one column
    cw = code.encode(block)  # [1, S * blowup], bit-reversed
    commitment, layers = smcs.commit(cw, column_major=True)
    n = cw.shape[1]
    pos = dev(orc.sp1_query_positions(z["query_indices"], n)).to(torch.int32)
    rows, proofs = smcs.open_batch(pos, cw.reshape(n, 1), layers)
    assert np.array_equal(to_host(rows), z["rows"])
    assert np.array_equal(to_host(proofs), z["paths"])
    # the separator-bound commitment: device bind == host bind == verifier
    raw = to_host(layers.root)
    assert np.array_equal(to_host(commitment), orc.smcs_bind_root(cpu, raw, n.bit_length() - 1, 1))
    for q in range(0, 52, 13):
        assert smcs.verify_batch(commitment, (n, 1), int(pos[q]), rows[q], proofs[:, q]) == \
            VerifyCode.OK
    bad = rows[0].clone()
    bad[0] ^= 1
    assert smcs.verify_batch(commitment, (n, 1), int(pos[0]), bad, proofs[:, 0]) == \
        VerifyCode.ROOT_MISMATCH
    assert smcs.verify_batch(commitment, (n, 1), n, rows[0], proofs[:, 0]) == \
        VerifyCode.INDEX_OUT_OF_BOUNDS
    assert smcs.verify_batch(commitment, (n, 1), int(pos[0]), rows[0], proofs[:-1, 0]) == \
        VerifyCode.WRONG_HEIGHT


def test_batch_eval_matches_sp1_dump(orc, golden):
    """zc_eval_mle of the prep column at the stacking point == the dumped
    batch evaluation (zorch/pcs/jagged/open.py:202-204)."""
    z = golden["round"]
    m = int(z["log_stacking_height"])
    L = _lib.lib()
    out = torch.empty((1, 4), dtype=torch.int32, device="cuda")
    nb = L.zc_eval_mle_workspace_bytes(1, m)
    ws = torch.empty((nb + 15) // 4, dtype=torch.int32, device="cuda")
    zd = dev(z["z_final"][-m:])
    _lib.check(L.zc_eval_mle(KOALABEAR.id, dev(golden["prep"]).data_ptr(), 1, m, zd.data_ptr(),
                             out.data_ptr(), ws.data_ptr(), nb, 0), "eval_mle")
    assert np.array_equal(to_host(out), z["batch_evals"])


@pytest.mark.parametrize("i", [0, 1, 10, 19, 20])
def test_bitrev_fold_matches_sp1_dump(orc, golden, i):
    from zorch_gb300.coding import BitReversedReedSolomon

    ch = golden["chain"]
    n0 = 1 << 23
    code = BitReversedReedSolomon(1 << 21, 4, KOALABEAR)
    qpos = orc.sp1_query_positions(ch["query_indices"], n0)
    n = n0 >> i
    rows = ch[f"rows_f{i}"]
    layer = np.zeros((n, 4), np.uint32)
    for q in range(rows.shape[0]):
        p = int(qpos[q]) >> (i + 1)
        layer[2 * p: 2 * p + 2] = rows[q].reshape(2, 4)
    g = to_host(code.fold(dev(layer), dev(ch["fri_betas"][i])))
    last = i + 1 == ch["fri_betas"].shape[0]
    for q in range(rows.shape[0]):
        p = int(qpos[q]) >> (i + 1)
        want = ch["final_poly"] if last else ch[f"rows_f{i + 1}"][q].reshape(2, 4)[p & 1]
        assert np.array_equal(g[p], want), (i, q)


@pytest.mark.parametrize("field", [0, 1])
@pytest.mark.parametrize("log_k,log_b,batch", [(0, 1, 2), (3, 2, 3), (10, 2, 2), (12, 2, 2),
                                               (13, 1, 2), (14, 2, 1), (16, 3, 1), (21, 2, 1),
                                               (17, 2, 40)])  # the wide LDE variant
def test_bitrev_encode_matches_oracle(orc, field, log_k, log_b, batch):
    from zorch_gb300.coding import rs_encode
    from zorch_gb300.field import field_of

    f = field_of(field)
    m = rand_mont(orc, field, (batch, 1 << log_k), 7 * log_k + log_b)
    for shift in (None, f.generator):
        sh = f.mont(shift) if shift else 0
        got = to_host(rs_encode(f, dev(m).reshape(batch, -1), log_b, sh, bit_reversed=True))
        want = orc.rs_encode_bitrev(field, m, log_b, sh)
        assert np.array_equal(got, want), (log_k, log_b, shift)


def test_batched_lde_mixes_natural_and_bit_reversed(orc):
    from zorch_gb300.batch import BatchCommitter, MatrixJob

    bc = BatchCommitter(BABYBEAR)
    shapes = [(3, 1 << 10, 2, False), (2, 1 << 14, 1, True), (1, 1 << 16, 2, True),
              (4, 1 << 9, 3, True), (1, 1 << 15, 1, False)]
    jobs, want = [], []
    for s, (w, h, lb, br) in enumerate(shapes):
        m = rand_mont(orc, 0, (w, h), 50 + s)
        jobs.append(MatrixJob(dev(m).reshape(w, h), lb, 31, bit_reversed=br))
        enc = orc.rs_encode_bitrev if br else orc.rs_encode
        want.append(enc(0, m, lb, int(orc.to_mont(0, [31])[0])))
    outs = bc.encode(jobs)
    for o_, w_ in zip(outs, want):
        assert np.array_equal(to_host(o_), w_)


def test_smcs_bind_root_matches_oracle(orc, sp1, perms_bb):
    from zorch_gb300.commit import SingleMatrixCommitmentScheme

    for (gpu, cpu), f in ((sp1, 1), (perms_bb, 0)):
        smcs = SingleMatrixCommitmentScheme(gpu)
        for s, (lh, w) in enumerate([(0, 1), (5, 8), (23, 1), (21, 255)]):
            raw = rand_mont(orc, f, 8, 900 + s)
            got = to_host(smcs.bind_root(dev(raw), lh, w))
            assert np.array_equal(got, orc.smcs_bind_root(cpu, raw, lh, w))
            assert np.array_equal(smcs.bind_root_host(raw, lh, w), got)


@pytest.fixture(scope="module")
def perms_bb(orc):
    from zorch_gb300.commit import Poseidon2

    return Poseidon2.builtin(BABYBEAR), orc.Poseidon2.babybear16()


@pytest.mark.parametrize("field,log_n,rounds", [(1, 12, 6), (0, 10, 9), (1, 3, 2)])
def test_stacked_fold_commit_matches_oracle(orc, sp1, perms_bb, field, log_n, rounds):
    from zorch_gb300.coding import BitReversedReedSolomon
    from zorch_gb300.commit import SingleMatrixCommitmentScheme
    from zorch_gb300.jagged import StackedFoldCommit

    gpu, cpu = sp1 if field == 1 else perms_bb
    shift = None if field == 1 else 31
    n = 1 << log_n
    code = BitReversedReedSolomon(n // 4, 4, field, coset_shift=shift)
    cw = rand_mont(orc, field, (n, 4), 40 + log_n)
    betas = rand_mont(orc, field, (rounds, 4), 41 + log_n)
    sf = StackedFoldCommit(SingleMatrixCommitmentScheme(gpu), code)
    layers, final = sf.run_replay(dev(cw).reshape(n, 4), dev(betas).reshape(rounds, 4))
    sh = code.level_shift_mont(0)
    raw, bound, olayers, ofinal = orc.sp1_stacked_fold_chain(cpu, field, cw, betas, sh)
    assert np.array_equal(to_host(final), ofinal)
    for r, layer in enumerate(layers):
        assert np.array_equal(to_host(layer.raw_root), raw[r]), r
        assert np.array_equal(to_host(layer.bound_root), bound[r]), r
        want_flat = np.concatenate([lv.reshape(-1) for lv in olayers[r][1]])
        assert np.array_equal(to_host(layer.digest_layers.flat).reshape(-1), want_flat), r
    pos = np.random.default_rng(5).integers(0, n, 16).astype(np.int32)
    opened = sf.open_layers(layers, torch.tensor(pos, device="cuda"))
    for r, (rows, proofs) in enumerate(opened):
        leaves, dl = olayers[r]
        idx = pos >> (r + 1)
        wr, wp = orc.merkle_open(leaves, leaves.shape[0], 1, 8, 0, dl, idx)
        assert np.array_equal(to_host(rows), wr) and np.array_equal(to_host(proofs), wp), r


def test_sp1_query_positions_use_canonical_bits(orc, sp1):
    from zorch_gb300.jagged import sample_query_positions
    from zorch_gb300.transcript import DuplexTranscript

    gpu, cpu = sp1
    t = DuplexTranscript.new(gpu)
    vals = rand_mont(orc, 1, 13, 3)
    t = t.observe(dev(vals))
    _, pos = sample_query_positions(t, 1 << 20, 52)
    ot = orc.Transcript(cpu)
    ot.observe(vals)
    raw = ot.sample(52)
    assert np.array_equal(to_host(pos).astype(np.uint32),
                          orc.from_mont(1, raw) & np.uint32((1 << 20) - 1))


@pytest.mark.parametrize("widths,v,log_blowup,queries,pow_bits",
                         [((3, 2), 6, 2, 5, 0), ((1,), 10, 2, 16, 0), ((7, 1, 4), 9, 1, 8, 0),
                          ((2, 3), 7, 1, 6, 10)])
def test_stacked_open_matches_oracle(orc, sp1, widths, v, log_blowup, queries, pow_bits):
    """The whole stacked open (zorch/pcs/jagged/open.py:362-460) on the GPU ==
    the oracle's restatement, field for field, and the folded codeword is the
    constant encoding of the reduced claim."""
    from zorch_gb300.coding import BitReversedReedSolomon
    from zorch_gb300.commit import SingleMatrixCommitmentScheme
    from zorch_gb300.jagged import stacked_basefold_open, stacked_commit
    from zorch_gb300.transcript import DuplexTranscript

    gperm, cperm = sp1
    S = 1 << v
    code = BitReversedReedSolomon(S, 1 << log_blowup, KOALABEAR)
    smcs = SingleMatrixCommitmentScheme(gperm)
    blocks = [rand_mont(orc, 1, (w, S), 60 + 3 * i + v) for i, w in enumerate(widths)]
    rounds = [stacked_commit(smcs, code, dev(b).reshape(b.shape)) for b in blocks]
    z = rand_mont(orc, 1, (v + 2, 4), 70 + v)
    de = rand_mont(orc, 1, 4, 71 + v)
    proof, _ = stacked_basefold_open(smcs, code, rounds, dev(z).reshape(v + 2, 4), dev(de), v,
                                     num_queries=queries, pow_bits=pow_bits,
                                     transcript=DuplexTranscript.new(gperm))
    want = orc.sp1_stacked_open(cperm, 1, blocks, z, de, v, log_blowup, queries,
                                orc.Transcript(cperm), pow_bits)
    assert np.array_equal(to_host(proof.pow_witness), want["pow_witness"])
    for got, w in zip(proof.batch_evals, want["batch_evals"]):
        assert np.array_equal(to_host(got), w)
    assert np.array_equal(to_host(proof.univariate_messages).reshape(v, 8), want["uni_msgs"])
    assert np.array_equal(to_host(proof.fri_raw_roots), want["raw_roots"])
    assert np.array_equal(to_host(proof.fri_commitments), want["bound_roots"])
    assert np.array_equal(to_host(proof.final_poly), want["final_poly"])
    assert np.array_equal(to_host(proof.positions), want["positions"].astype(np.uint32))
    for (rows, paths), (wr, wp) in zip(proof.query_openings, want["query_openings"]):
        assert np.array_equal(to_host(rows), wr) and np.array_equal(to_host(paths), wp)
    n = S << log_blowup
    for rd, b, (rows, paths), com in zip(rounds, blocks, proof.component_openings,
                                         proof.component_commitments):
        cw = orc.rs_encode_bitrev(1, b, log_blowup)
        layers = orc.merkle_commit_columns(cperm, cw)
        wr, wp = orc.merkle_open(cw, n, b.shape[0], 1, n, layers, want["positions"])
        assert np.array_equal(to_host(rows), wr) and np.array_equal(to_host(paths), wp)
        assert np.array_equal(to_host(com),
                              orc.smcs_bind_root(cperm, layers[-1][0], n.bit_length() - 1,
                                                 b.shape[0]))
    assert all(np.array_equal(x, want["final_claim"]) for x in want["final_codeword"])


def _stacked_case(orc, sp1, pow_bits, widths=(3, 2), v=7, queries=6):
    """A stacked open over rounds of `widths` columns with a consistent
    statement: dense_eval is the MLE of the batch evaluations at the leading
    coordinates of z_final (SP1's stacking identity)."""
    from zorch_gb300.coding import BitReversedReedSolomon
    from zorch_gb300.commit import SingleMatrixCommitmentScheme
    from zorch_gb300.jagged import _ef_eval_mle_msb, stacked_basefold_open, stacked_commit
    from zorch_gb300.transcript import DuplexTranscript

    gperm, _ = sp1
    f = KOALABEAR
    S = 1 << v
    code = BitReversedReedSolomon(S, 2, f)
    smcs = SingleMatrixCommitmentScheme(gperm)
    blocks = [rand_mont(orc, 1, (w, S), 90 + i) for i, w in enumerate(widths)]
    rounds = [stacked_commit(smcs, code, dev(b).reshape(b.shape)) for b in blocks]
    z = rand_mont(orc, 1, (v + 3, 4), 95)
    zd = dev(z).reshape(v + 3, 4)
    probe, _ = stacked_basefold_open(smcs, code, rounds, zd, dev(np.zeros(4, np.uint32)), v,
                                     num_queries=queries, pow_bits=0,
                                     transcript=DuplexTranscript.new(gperm))
    flat = [f.ef_from_mont(r) for e in probe.batch_evals for r in to_host(e).reshape(-1, 4)]
    lead = [f.ef_from_mont(r) for r in z[:3]]
    de = np.array(f.ef_to_mont(_ef_eval_mle_msb(f, flat + [(0, 0, 0, 0)] * (8 - len(flat)),
                                                lead)), np.uint32)
    proof, _ = stacked_basefold_open(smcs, code, rounds, zd, dev(de), v, num_queries=queries,
                                     pow_bits=pow_bits, transcript=DuplexTranscript.new(gperm))
    return smcs, code, list(widths), zd, de, v, proof


@pytest.mark.parametrize("pow_bits", [0, 7])
def test_stacked_open_verifies(orc, sp1, pow_bits):
    """Open -> verify completeness (zorch/pcs/jagged/testing/open_test.py's
    real-transcript round trip) through the host verifier."""
    from zorch_gb300.jagged import stacked_basefold_verify
    from zorch_gb300.transcript import HostDuplexTranscript

    smcs, code, widths, zd, de, v, proof = _stacked_case(orc, sp1, pow_bits)
    _, ok = stacked_basefold_verify(smcs, code, widths, zd, de, v, proof,
                                    HostDuplexTranscript(sp1[0]), num_queries=6,
                                    pow_bits=pow_bits)
    assert ok


def test_stacked_verify_rejects_tampering(orc, sp1):
    from zorch_gb300.jagged import stacked_basefold_verify
    from zorch_gb300.transcript import HostDuplexTranscript

    smcs, code, widths, zd, de, v, proof = _stacked_case(orc, sp1, 5)

    def check(p, de_=de, pow_bits=5):
        return stacked_basefold_verify(smcs, code, widths, zd, de_, v, p,
                                       HostDuplexTranscript(sp1[0]), num_queries=6,
                                       pow_bits=pow_bits)[1]

    assert check(proof)

    def flip(t, idx):
        t = t.clone()
        t.view(-1)[idx] ^= 1
        return t

    bad_de = de.copy()
    bad_de[1] ^= 1
    assert not check(proof, de_=bad_de)
    assert not check(dataclasses.replace(proof, univariate_messages=flip(
        proof.univariate_messages, 3)))
    assert not check(dataclasses.replace(proof, final_poly=flip(proof.final_poly, 0)))
    assert not check(dataclasses.replace(proof, fri_raw_roots=flip(proof.fri_raw_roots, 9)))
    assert not check(dataclasses.replace(proof, pow_witness=flip(proof.pow_witness, 0)))
    assert not check(dataclasses.replace(proof, batch_evals=[flip(proof.batch_evals[0], 2),
                                                             *proof.batch_evals[1:]]))
    rows, paths = proof.component_openings[1]
    assert not check(dataclasses.replace(proof, component_openings=[
        proof.component_openings[0], (flip(rows, 4), paths)]))
    rows, paths = proof.query_openings[2]
    assert not check(dataclasses.replace(proof, query_openings=[
        *proof.query_openings[:2], (flip(rows, 5), paths), *proof.query_openings[3:]]))
    with pytest.raises(ValueError):
        check(dataclasses.replace(proof, batch_evals=proof.batch_evals[:1]))


def test_graphed_stacked_open_replays_the_eager_open(orc, sp1):
    """GraphedStackedOpen: one capture, replays at new statements and
    transcripts give the eager open's proof, field for field."""
    from zorch_gb300.jagged import GraphedStackedOpen, stacked_basefold_open
    from zorch_gb300.transcript import DuplexTranscript

    smcs, code, widths, zd, de, v, _ = _stacked_case(orc, sp1, 3)
    rounds = _rounds_of(orc, sp1, code, smcs)
    g = GraphedStackedOpen(smcs, code, rounds, zd.shape[0], v, num_queries=6, pow_bits=3)
    for k in range(3):
        z = dev(rand_mont(orc, 1, tuple(zd.shape), 700 + k)).reshape(zd.shape)
        d = dev(rand_mont(orc, 1, 4, 710 + k))
        t = DuplexTranscript.new(sp1[0]).observe(dev(rand_mont(orc, 1, (k + 2,), 720 + k)))
        want, wt = stacked_basefold_open(smcs, code, rounds, z, d, v, num_queries=6, pow_bits=3,
                                         transcript=t)
        got, gt = g.replay(z, d, t)
        for name in ("fri_raw_roots", "fri_commitments", "univariate_messages", "final_poly",
                     "pow_witness", "positions"):
            assert torch.equal(getattr(got, name), getattr(want, name)), name
        for a, b in zip(got.batch_evals, want.batch_evals):
            assert torch.equal(a, b)
        for (ra, pa), (rb, pb) in zip(got.query_openings + got.component_openings,
                                      want.query_openings + want.component_openings):
            assert torch.equal(ra, rb) and torch.equal(pa, pb)
        assert torch.equal(gt.state, wt.state)


def _rounds_of(orc, sp1, code, smcs, widths=(3, 2), v=7):
    from zorch_gb300.jagged import stacked_commit

    S = 1 << v
    blocks = [rand_mont(orc, 1, (w, S), 90 + i) for i, w in enumerate(widths)]
    return [stacked_commit(smcs, code, dev(b).reshape(b.shape)) for b in blocks]
