"""k-ary FRI fold on the GPU (coset-INTT form) == the oracle's Lagrange form,
and the k-group commit rounds (PreFoldKGroupCommitRound,
zorch/pcs/fold.py:118-139) with their query phase, checked like the
reference's KGroupFoldRoundTripTest (zorch/pcs/testing/fold_test.py:40-140)."""

from __future__ import annotations

import dataclasses

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
    x = np.random.default_rng(seed).integers(0, orc.MODULUS[field], size=shape, dtype=np.uint64)
    return orc.to_mont(field, x.astype(np.uint32))


def dev(x):
    return to_device(np.asarray(x, np.uint32))


@pytest.mark.parametrize("field", [0, 1])
@pytest.mark.parametrize("log_k", [1, 2, 3, 4])
@pytest.mark.parametrize("ef_in,ef_beta", [(False, False), (False, True), (True, True),
                                           (True, False)])
def test_fold_group_matches_oracle(orc, field, log_k, ef_in, ef_beta):
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.field import field_of

    f = field_of(field)
    shift = f.generator
    code = ReedSolomon(1 << 10, 2, f, coset_shift=shift, fold_factor=1 << log_k)
    n = code.block_len
    for level in (0, 1):
        m = n >> (log_k * level)
        cw = rand_mont(orc, field, (m, 4) if ef_in else (m,), 7 * log_k + level)
        beta = rand_mont(orc, field, 4 if ef_beta else 1, 3 + level)
        got = to_host(code.fold_group(dev(cw).reshape(cw.shape), dev(beta)))
        want = orc.fri_fold_k(field, cw, ef_in, beta, ef_beta, log_k,
                              code.group_level_shift_mont(level))
        assert np.array_equal(got.reshape(want.shape), want), level
        if log_k == 1:  # k = 2 is the binary butterfly
            assert np.array_equal(got, to_host(code.fold(dev(cw).reshape(cw.shape), dev(beta))))


def test_fold_group_values_matches_whole_layer_fold(orc):
    from zorch_gb300.coding import ReedSolomon

    code = ReedSolomon(16, 4, KOALABEAR, coset_shift=3, fold_factor=4)  # block_len 64
    cw = dev(rand_mont(orc, 1, (64, 4), 38)).reshape(64, 4)
    beta = dev(rand_mont(orc, 1, 4, 39))
    layer1 = code.fold_group(cw, beta)
    folded = to_host(code.fold_group(layer1, beta))
    positions = torch.tensor([0, 1, 3], dtype=torch.int32, device="cuda")
    idx = torch.stack(code.group_indices(positions, 1), dim=-1).long()
    got = code.fold_group_values(to_host(layer1[idx]), to_host(beta), to_host(positions), 1)
    f = KOALABEAR
    for qi, p in enumerate([0, 1, 3]):
        assert got[qi] == f.ef_from_mont([int(x) for x in folded[p]])


def _kgroup_rounds(orc, k, num_rounds, num_queries, tamper=None):
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, koalabear16_params
    from zorch_gb300.pcs import (FoldState, PreFoldKGroupCommitRound, fold_rounds,
                                 open_group_layer, verify_group_fold_chain)
    from zorch_gb300.transcript import DuplexTranscript, HostDuplexTranscript, sample_positions

    perm = koalabear16_params(orc.load_koalabear_fixture())
    tree = MerkleTree(perm)
    code = ReedSolomon(16, 2, KOALABEAR, fold_factor=k)
    f = code.encode(dev(rand_mont(orc, 1, 16, 1)))
    t = DuplexTranscript.new(perm)
    state, t, roots = fold_rounds(PreFoldKGroupCommitRound(code, tree), FoldState(f), t,
                                  num_rounds)
    final = state.codeword
    t, positions = sample_positions(t.observe(final), code.block_len, num_queries)
    a = code.group_layer_positions(positions, num_rounds)
    openings = [open_group_layer(tree, layer, a[i], k) for i, layer in enumerate(state.layers)]
    # oracle: the same rounds on the CPU
    cp = orc.Poseidon2.koalabear16_golden()
    ot = orc.Transcript(cp)
    cw = to_host(f)
    oroots, obetas = [], []
    for _ in range(num_rounds):
        n = cw.shape[0]
        dl = orc.merkle_commit(cp, cw, n // k, k, 1, n // k)
        ot.observe(dl[-1][0])
        beta = ot.sample(1)
        oroots.append(dl[-1][0])
        obetas.append(beta)
        cw = orc.fri_fold_k(1, cw, False, beta, False, k.bit_length() - 1, 0)
    assert np.array_equal(to_host(torch.stack(roots)), np.stack(oroots))
    assert np.array_equal(to_host(final), cw)
    # verifier: replay the transcript on the host, check paths and the chain
    if tamper == "final":
        final = final.clone()
        final[1] ^= 1
    if tamper == "group":
        op = openings[0]
        openings = [dataclasses.replace(op, row=op.row.clone()), *openings[1:]]
        openings[0].row[0, 0] ^= 1
    ht = HostDuplexTranscript(perm)
    betas = []
    for r in roots:
        ht, b = ht.observe_and_sample(to_host(r), 1)
        betas.append(b)
    ht, raw = ht.observe_and_sample(to_host(final), num_queries)
    pos = [int(x) % code.block_len for x in raw]
    ok = pos == [int(x) for x in to_host(positions).view(np.int32)]
    if 16 >> ((k.bit_length() - 1) * num_rounds) <= 1:  # folded to a constant
        ok &= bool((final == final[0]).all())
    from zorch_gb300.commit import Opening

    for i, op in enumerate(openings):
        ai = [int(x) for x in to_host(a[i]).view(np.int32)]
        for qi, p in enumerate(ai):
            ok &= tree.verify(roots[i], p, Opening(op.row[qi], op.path[:, qi]))
    ok &= verify_group_fold_chain(code, openings, betas, a, final)
    return ok


@pytest.mark.parametrize("k,rounds", [(4, 2), (2, 4), (8, 1), (16, 1)])
def test_kgroup_round_trip(orc, k, rounds):
    assert _kgroup_rounds(orc, k, rounds, 3)


@pytest.mark.parametrize("tamper", ["final", "group"])
def test_kgroup_tamper_rejected(orc, tamper):
    assert not _kgroup_rounds(orc, 4, 2, 3, tamper)
