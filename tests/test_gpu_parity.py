"""CUDA path == CPU oracle, bit for bit, through the C ABI (libzc.so).

Seeded inputs at sizes the oracle finishes in seconds; every codeword, digest
layer, root, authentication path, Fiat-Shamir word and proof byte is compared
exactly (integer work: the tolerance is zero).
"""

from __future__ import annotations

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
def perms(orc):
    from zorch_gb300.commit import Poseidon2, koalabear16_params

    return {
        "bb": (Poseidon2.builtin(BABYBEAR), orc.Poseidon2.babybear16(), 0),
        "kb": (koalabear16_params(orc.load_koalabear_fixture()),
               orc.Poseidon2.koalabear16_golden(), 1),
    }


def test_mont_conversion(orc):
    from zorch_gb300.field import from_mont, to_mont

    for f in (0, 1):
        x = np.random.default_rng(f).integers(0, 2**32, size=1000, dtype=np.uint64).astype(np.uint32)
        m = to_host(to_mont(f, dev(x)))
        assert np.array_equal(m, orc.to_mont(f, x % orc.MODULUS[f]))
        assert np.array_equal(to_host(from_mont(f, dev(m))), x % orc.MODULUS[f])


@pytest.mark.parametrize("which", ["bb", "kb"])
def test_permutation(orc, perms, which):
    gpu, cpu, f = perms[which]
    st = rand_mont(orc, f, (300, 16), 5)
    got = to_host(gpu.permute(dev(st)))
    want = np.stack([cpu.permute(s) for s in st])
    assert np.array_equal(got, want)


def test_koalabear_golden_root_on_gpu(orc, perms):
    from zorch_gb300.commit import MerkleTree

    gpu, _, _ = perms["kb"]
    d = orc.load_koalabear_fixture()
    m = orc.to_mont(1, np.arange(32, dtype=np.uint32).reshape(4, 8))
    root, layers = MerkleTree(gpu).commit(dev(m).reshape(4, 8))
    assert [tuple(l.shape) for l in layers] == [(4, 8), (2, 8), (1, 8)]
    assert orc.from_mont(1, to_host(root)).tolist() == d["merkle_4x8_root"]


@pytest.mark.parametrize("which", ["bb", "kb"])
@pytest.mark.parametrize("L,w", [(1, 8), (2, 1), (4, 0), (8, 9), (256, 2), (512, 8),
                                 (1024, 64), (4096, 17), (1 << 15, 3)])
def test_merkle_row_major(orc, perms, which, L, w):
    from zorch_gb300.commit import MerkleTree

    gpu, cpu, f = perms[which]
    m = rand_mont(orc, f, (L, w), L + w)
    _, layers = MerkleTree(gpu).commit(dev(m).reshape(L, w))
    want = orc.merkle_commit_rows(cpu, m) if w else orc.merkle_commit(cpu, m, L, 1, 0, 0)
    for lg, lw in zip(layers, want):
        assert np.array_equal(to_host(lg), lw)


@pytest.mark.parametrize("L,w", [(16, 5), (2048, 64), (1 << 14, 1)])
def test_merkle_column_major_and_open(orc, perms, L, w):
    from zorch_gb300.commit import MerkleTree

    gpu, cpu, f = perms["bb"]
    cols = rand_mont(orc, f, (w, L), 7 * L + w)
    tree = MerkleTree(gpu, column_major=True)
    root, layers = tree.commit(dev(cols).reshape(w, L))
    want = orc.merkle_commit_columns(cpu, cols)
    assert np.array_equal(to_host(root), want[-1][0])
    idx = np.random.default_rng(L).integers(0, L, size=37).astype(np.int32)
    op = tree.open_rows(dev(np.ascontiguousarray(cols.T)).reshape(L, w), layers,
                        torch.from_numpy(idx).cuda())
    rows, paths = orc.merkle_open(cols, L, w, 1, L, want, idx)
    assert np.array_equal(to_host(op.row), rows)
    assert np.array_equal(to_host(op.path), paths)
    with pytest.raises(IndexError):
        tree.open_rows(dev(np.ascontiguousarray(cols.T)).reshape(L, w), layers,
                       torch.tensor([L], device="cuda"))


@pytest.mark.parametrize("field", [0, 1])
@pytest.mark.parametrize("log_k,log_b,batch", [(0, 1, 2), (1, 1, 1), (3, 2, 3), (6, 3, 2),
                                               (10, 2, 2), (12, 1, 1), (12, 2, 2), (12, 3, 1),
                                               (13, 1, 2), (14, 2, 1), (16, 1, 1), (17, 3, 1),
                                               (20, 1, 1),
                                               # the wide (radix-2^5, 2^15-word tile) variant:
                                               # >= two tiles per SM
                                               (18, 1, 40), (15, 3, 80)])
def test_rs_encode(orc, field, log_k, log_b, batch):
    from zorch_gb300.coding import rs_encode
    from zorch_gb300.field import field_of

    f = field_of(field)
    m = rand_mont(orc, field, (batch, 1 << log_k), 100 * log_k + log_b)
    for shift in (None, f.generator):
        sh = f.mont(shift) if shift else 0
        got = to_host(rs_encode(f, dev(m).reshape(batch, -1), log_b, sh))
        want = orc.rs_encode(field, m, log_b, sh)
        assert np.array_equal(got, want), (log_k, log_b, shift)


def test_rs_encode_matches_horner_small(orc):
    from zorch_gb300.coding import ReedSolomon

    code = ReedSolomon(32, 4, BABYBEAR, coset_shift=31, generator=31)
    m = rand_mont(orc, 0, 32, 3)
    got = to_host(code.encode(dev(m)))
    assert np.array_equal(got, orc.rs_encode_horner(0, m, 2, BABYBEAR.mont(31)))


def test_eval_domain(orc):
    from zorch_gb300.coding import eval_domain

    got = to_host(eval_domain(BABYBEAR, 64, shift=31))
    assert np.array_equal(got, orc.eval_domain(0, 6, BABYBEAR.mont(31)))


@pytest.mark.parametrize("ef_in,ef_beta", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("log_n,level", [(1, 0), (5, 0), (12, 3)])
def test_fold(orc, ef_in, ef_beta, log_n, level):
    from zorch_gb300.coding import ReedSolomon

    n = 1 << log_n
    code = ReedSolomon(n << level >> 1, 2, BABYBEAR, coset_shift=31, generator=31)
    cw = rand_mont(orc, 0, (n, 4) if ef_in else (n,), log_n * 10 + ef_in)
    beta = rand_mont(orc, 0, 4 if ef_beta else 1, 9)
    got = to_host(code.fold(dev(cw).reshape(cw.shape), dev(beta)))
    want = orc.fri_fold(0, cw, bool(ef_in), beta, bool(ef_beta), code.level_shift_mont(level))
    assert np.array_equal(got.reshape(want.shape), want)


@pytest.mark.parametrize("ef_in,ef_beta", [(0, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("log_n", [2, 3, 9, 12])
def test_fused_fold_commit(orc, perms, ef_in, ef_beta, log_n):
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.pcs import PreFoldPairCommitRound

    gpu, cpu, _ = perms["bb"]
    n = 1 << log_n
    code = ReedSolomon(n // 2, 2, BABYBEAR, coset_shift=31)
    cw = rand_mont(orc, 0, (n, 4) if ef_in else (n,), log_n + 3 * ef_in)
    beta = rand_mont(orc, 0, 4 if ef_beta else 1, 19)
    rnd = PreFoldPairCommitRound(code, MerkleTree(gpu))
    out, layer = rnd.fold_commit(dev(cw).reshape(cw.shape), dev(beta), 0)
    want = orc.fri_fold(0, cw, bool(ef_in), beta, bool(ef_beta), BABYBEAR.mont(31))
    assert np.array_equal(to_host(out).reshape(want.shape), want)
    limbs = 4 if (ef_in or ef_beta) else 1
    L = n // 4
    wl = orc.merkle_commit(cpu, want, L, 2, limbs, L * limbs)
    for lg, lw in zip(layer.digest_layers, wl):
        assert np.array_equal(to_host(lg), lw)


def _script(orc, seed):
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(25):
        if rng.random() < 0.5:
            ops.append(("o", rand_mont(orc, 0, int(rng.integers(0, 20)), int(rng.integers(1 << 30)))))
        else:
            ops.append(("s", int(rng.integers(1, 12))))
    return ops


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_transcript_device_matches_oracle(orc, perms, seed):
    from zorch_gb300.transcript import DuplexTranscript, HostDuplexTranscript

    gpu, cpu, _ = perms["bb"]
    t = DuplexTranscript.new(gpu)
    th = HostDuplexTranscript(gpu)
    to = orc.Transcript(cpu)
    for op, arg in _script(orc, seed):
        if op == "o":
            t = t.observe(dev(arg)) if arg.size else t
            th = th.observe(arg)
            to.observe(arg)
        else:
            t, got = t.sample(arg)
            th, goth = th.sample(arg)
            want = to.sample(arg)
            assert np.array_equal(to_host(got), want)
            assert np.array_equal(goth, want)
        wire = np.concatenate(to.st.wire())
        assert np.array_equal(to_host(t.state), wire)
        assert np.array_equal(th.state, wire)


def test_duplex_hop_ffi_contract(orc, perms):
    """zc_duplex_hop: six operands in, five advanced + n words out (device)."""
    from zorch_gb300.field import ptr, stream_handle

    gpu, cpu, _ = perms["bb"]
    to = orc.Transcript(cpu)
    to.observe(rand_mont(orc, 0, 5, 1))
    state = dev(np.concatenate(to.st.wire()))
    vals = rand_mont(orc, 0, 13, 2)
    v = dev(vals)
    out = torch.zeros_like(state)
    ch = torch.zeros(6, dtype=torch.int32, device="cuda")
    s0 = state.data_ptr()
    o0 = out.data_ptr()
    _lib.check(_lib.lib().zc_duplex_hop(gpu.handle, s0, s0 + 32, s0 + 64, s0 + 128, s0 + 132,
                                        ptr(v), 13, 6, o0, o0 + 32, o0 + 64, o0 + 128, o0 + 132,
                                        ptr(ch), stream_handle()), "hop")
    to.observe(vals)
    want = to.sample(6)
    assert np.array_equal(to_host(ch), want)
    assert np.array_equal(to_host(out), np.concatenate(to.st.wire()))


@pytest.mark.parametrize("beta_limbs", [1, 4])
@pytest.mark.parametrize("log_k,log_b,R,Q", [(6, 1, 5, 9), (11, 1, 9, 100), (13, 2, 11, 64)])
def test_fri_commit_phase_proof_bytes(orc, perms, beta_limbs, log_k, log_b, R, Q):
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.pcs import FriParams, FriProver
    from zorch_gb300.transcript import DuplexTranscript

    gpu, cpu, _ = perms["bb"]
    code = ReedSolomon(1 << log_k, 1 << log_b, BABYBEAR, coset_shift=31, generator=31)
    coeffs = rand_mont(orc, 0, 1 << log_k, log_k)
    cw = code.encode(dev(coeffs))
    prover = FriProver(FriParams(code, MerkleTree(gpu), R, Q, beta_limbs))
    proof, t, _ = prover.commit_phase(cw, DuplexTranscript.new(gpu))
    cw_o = orc.rs_encode(0, coeffs, log_b, BABYBEAR.mont(31))
    assert np.array_equal(to_host(cw), cw_o)
    to = orc.Transcript(cpu)
    want = orc.fri_commit_phase(cpu, 0, cw_o, R, Q, beta_limbs, to, BABYBEAR.mont(31))
    assert np.array_equal(to_host(proof.roots), want.roots)
    assert np.array_equal(to_host(proof.final_layer).reshape(want.final_layer.shape),
                          want.final_layer)
    assert np.array_equal(to_host(proof.positions).astype(np.int32), want.positions)
    assert proof.to_bytes() == want.to_bytes()
    assert np.array_equal(to_host(t.state), np.concatenate(to.st.wire()))


def test_basefold_matrix_commit(orc, perms):
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.pcs import BasefoldProver

    gpu, cpu, _ = perms["bb"]
    K, log_s, log_b = 6, 13, 2
    code = ReedSolomon(1 << log_s, 1 << log_b, BABYBEAR, coset_shift=31, generator=31)
    cols = rand_mont(orc, 0, (K, 1 << log_s), 77)
    prover = BasefoldProver(code, MerkleTree(gpu, column_major=True))
    root, data = prover.commit_columns(dev(cols).reshape(K, -1))
    cw = orc.rs_encode(0, cols, log_b, BABYBEAR.mont(31))
    assert np.array_equal(to_host(data.codeword), cw)
    layers = orc.merkle_commit_columns(cpu, cw)
    assert np.array_equal(to_host(root), layers[-1][0])
    idx = np.random.default_rng(5).integers(0, cw.shape[1], size=128).astype(np.int32)
    op = prover.open_rows(data, torch.from_numpy(idx).cuda())
    rows, paths = orc.merkle_open(cw, cw.shape[1], K, 1, cw.shape[1], layers, idx)
    assert np.array_equal(to_host(op.row), rows)
    assert np.array_equal(to_host(op.path), paths)


def test_config1_plain_commit(orc, perms):
    """One 2^16 polynomial, blowup 2, shift 31, single-element leaves: the
    codeword and the root, bit-exact."""
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.field import to_mont

    gpu, cpu, _ = perms["bb"]
    coeffs_c = np.random.default_rng(1).integers(0, BABYBEAR.p, size=1 << 16,
                                                  dtype=np.uint64).astype(np.uint32)
    code = ReedSolomon(1 << 16, 2, BABYBEAR, coset_shift=31, generator=31)
    cw = code.encode(to_mont(0, dev(coeffs_c)))
    root, _ = MerkleTree(gpu).commit(cw.reshape(-1, 1))
    cw_o = orc.rs_encode(0, orc.to_mont(0, coeffs_c), 1, BABYBEAR.mont(31))
    assert np.array_equal(to_host(cw), cw_o)
    assert np.array_equal(to_host(root), orc.merkle_commit_rows(cpu, cw_o.reshape(-1, 1))[-1][0])


def test_merkle_verify_roundtrip_and_tamper(orc, perms):
    """open -> verify (zorch/commit/merkle.py:327-331), a tampered sibling or
    row fails, an out-of-range index is rejected."""
    from zorch_gb300.commit import MerkleTree, Opening

    for which in ("bb", "kb"):
        gpu, _, f = perms[which]
        m = dev(rand_mont(orc, f, (64, 9), 17)).reshape(64, 9)
        tree = MerkleTree(gpu)
        root, layers = tree.commit(m)
        for i in (0, 1, 37, 63):
            op = tree.open(m, layers, i)
            assert tree.verify(root, i, op)
        op = tree.open(m, layers, 5)
        bad_path = op.path.clone()
        bad_path[3, 0] ^= 1
        assert not tree.verify(root, 5, Opening(op.row, bad_path))
        bad_row = op.row.clone()
        bad_row[0] ^= 1
        assert not tree.verify(root, 5, Opening(bad_row, op.path))
        assert not tree.verify(root, 64, op)


def _dft_inverse(orc, f, evals):
    """O(k^2) inverse DFT with the oracle's field ops (independent of any NTT)."""
    k = len(evals)
    w = orc.root_of_unity(f, k.bit_length() - 1)
    p = orc.MODULUS[f]
    winv = orc.to_mont(f, [pow(int(orc.from_mont(f, [w])[0]), p - 2, p)])[0]
    kinv = orc.to_mont(f, [pow(k, p - 2, p)])[0]
    out = []
    for i in range(k):
        acc = 0
        x = int(orc.to_mont(f, [1])[0])
        step = int(orc.to_mont(f, [1])[0])
        for _ in range(i):
            step = orc.LIB.orc_mul(f, step, int(winv))
        for j in range(k):
            acc = (acc + orc.LIB.orc_mul(f, int(evals[j]), x)) % p
            x = orc.LIB.orc_mul(f, x, step)
        out.append(orc.LIB.orc_mul(f, acc, int(kinv)))
    return np.array(out, np.uint32)


@pytest.mark.parametrize("k,blowup,shift", [(4, 2, None), (8, 4, 7), (16, 2, 3), (64, 2, 31)])
def test_extend_matches_coset_polynomial_evaluation(orc, k, blowup, shift):
    """reed_solomon_test.py:179-199: extend(evals) == Horner(INTT(evals)) on the
    (coset) domain, with INTT by an independent O(k^2) inverse DFT."""
    from zorch_gb300.coding import ReedSolomon

    evals = rand_mont(orc, 0, k, k + blowup)
    rs = ReedSolomon(k, blowup, BABYBEAR, coset_shift=shift)
    got = to_host(rs.extend(dev(evals)))
    coeffs = _dft_inverse(orc, 0, evals)
    sh = BABYBEAR.mont(shift) if shift else 0
    assert np.array_equal(got, orc.rs_encode_horner(0, coeffs, blowup.bit_length() - 1, sh))
    if shift is None:  # the LDE agrees with the evaluations on the base subgroup
        assert np.array_equal(got[::blowup], evals)


def test_codeword_is_low_degree_and_ef4_encode(orc):
    """reed_solomon_test.py:211-217 (INTT of a codeword has zero top
    coefficients) and :247-253 (EF4 messages encode limb by limb)."""
    from zorch_gb300.coding import ReedSolomon, intt

    k, blowup = 8, 2
    rs = ReedSolomon(k, blowup, BABYBEAR)
    coeffs = rand_mont(orc, 0, k, 2)
    rec = to_host(intt(BABYBEAR, rs.encode(dev(coeffs))))
    assert np.array_equal(rec[:k], coeffs) and not rec[k:].any()
    rsc = ReedSolomon(k, blowup, BABYBEAR, coset_shift=3)
    msg = rand_mont(orc, 0, (3, k, 4), 25)
    cw = to_host(rsc.encode(dev(msg).reshape(3, k, 4), ef4=True))
    for r in range(3):
        for e in range(4):
            want = orc.rs_encode(0, msg[r, :, e], 1, BABYBEAR.mont(3))
            assert np.array_equal(cw[r, :, e], want)


def test_graphed_fri_commit_phase_equals_eager(orc, perms):
    """The CUDA-graph replay of encode + commit phase gives the eager bytes
    for two different inputs in a row."""
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree
    from zorch_gb300.pcs import FriParams, FriProver, GraphedFriCommitPhase
    from zorch_gb300.transcript import DuplexTranscript

    gpu, _, _ = perms["bb"]
    code = ReedSolomon(1 << 12, 2, BABYBEAR, coset_shift=31, generator=31)
    prover = FriProver(FriParams(code, MerkleTree(gpu), 9, 40, 4))
    g = GraphedFriCommitPhase(prover)
    for seed in (1, 2):
        coeffs = dev(rand_mont(orc, 0, 1 << 12, 700 + seed))
        got = g.replay(coeffs).to_bytes()
        eager, _, _ = prover.commit_phase(code.encode(coeffs), DuplexTranscript.new(gpu))
        assert got == eager.to_bytes()


def test_to_mont_reads_pinned_host_memory(orc):
    """zc_host_device_ptr + zc_to_mont convert a page-locked host buffer in one
    kernel reading over the host link, equal to the device conversion; a
    pageable buffer is refused."""
    from zorch_gb300.field import to_mont, to_mont_from_host

    x = np.random.default_rng(4).integers(0, orc.P_BABYBEAR, size=(3, 1001), dtype=np.uint64)
    host = torch.from_numpy(x.astype(np.uint32).view(np.int32))
    got = to_mont_from_host(BABYBEAR, host.pin_memory())
    assert torch.equal(got, to_mont(BABYBEAR, host.cuda()))
    with pytest.raises(ValueError):
        to_mont_from_host(BABYBEAR, host)


def test_copy_rows_gathers_strided_rows():
    """copy_rows (zc_copy_rows, one 2D copy-engine transfer) gathers every
    tree's root row out of a stack of digest layers, as the batched commits
    use it, and refuses rows that are not contiguous."""
    from zorch_gb300.field import copy_rows

    layers = torch.arange(5 * 7 * 8, dtype=torch.int32, device="cuda").reshape(5, 7, 8)
    out = torch.full((5, 8), -1, dtype=torch.int32, device="cuda")
    copy_rows(out, layers[:, -1, :])
    assert torch.equal(out, layers[:, -1, :])
    one = torch.empty((1, 8), dtype=torch.int32, device="cuda")
    copy_rows(one, layers[2:3, 3, :])
    assert torch.equal(one, layers[2:3, 3, :])
    with pytest.raises(ValueError):
        copy_rows(torch.empty((8, 5), dtype=torch.int32, device="cuda"), layers[:, -1, :].t())
