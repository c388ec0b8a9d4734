"""The oracle against the reference's SP1 KoalaBear pipeline dump
(zorch/pcs/jagged/testing/testdata/gpu_fibonacci, byte-matched by
zorch/pcs/jagged/testing/open_test.py:242-303), no GPU.

- prep round: BitReversedReedSolomon.encode of the preprocessed dense column
  (KoalaBear, no coset, canonical root 3^((p-1)/n), blowup 4), its column-major
  SMCS Merkle tree with SP1's Poseidon2, and the component openings at the 52
  query positions -- rows and all 23 sibling levels;
- fold chain: every kept fold layer's query opening rebuilds a root that the
  SP1 separator binds to the dumped fri_commitments[i]; folding each opened
  pair with fri_betas[i] at the bit-reversed domain point gives the next
  layer's opened value, and the last fold gives the final poly.
"""

from __future__ import annotations

import lzma

import numpy as np
import pytest

import oracle.oracle as o

G = o.GOLDEN / "sp1_fibonacci"
KB = o.KOALABEAR


@pytest.fixture(scope="module")
def p2():
    return o.sp1_koalabear16()


@pytest.fixture(scope="module")
def prep():
    return np.frombuffer(lzma.decompress((G / "prep_dense.u32.xz").read_bytes()),
                         "<u4").astype(np.uint32)


@pytest.fixture(scope="module")
def chain():
    return np.load(G / "fold_chain.npz")


def test_sp1_params_fold_r_inverse(p2):
    d = o.load_sp1_fixture()
    assert d["internal_j_scale"] * 2**32 % o.P_KOALABEAR == 1
    assert len(d["internal_diag"]) == 16 and d["alpha"] == 3


def test_prep_round_component_openings(p2, prep):
    z = np.load(G / "prep_round.npz")
    log_blowup = int(z["log_blowup"])
    assert prep.size == 1 << int(z["log_stacking_height"])
    cw = o.rs_encode_bitrev(KB, prep.reshape(1, -1), log_blowup)  # [1, 2^23]
    n = cw.shape[1]
    layers = o.merkle_commit_columns(p2, cw)
    pos = o.sp1_query_positions(z["query_indices"], n)
    rows, paths = o.merkle_open(cw, n, 1, 1, n, layers, pos)
    assert np.array_equal(rows, z["rows"])
    assert paths.shape == z["paths"].shape
    assert np.array_equal(paths, z["paths"])


def test_batch_eval_of_the_prep_column(prep):
    """eval_mle of the prep column at the stacking point z_final[-21:]
    (zorch/pcs/jagged/open.py:202-204) == the dumped batch evaluation: pins the
    eq-table orientation (z[0] the most significant index bit)."""
    z = np.load(G / "prep_round.npz")
    got = o.eval_mle_base(KB, prep.reshape(1, -1), z["z_final"][-int(z["log_stacking_height"]):])
    assert np.array_equal(got, z["batch_evals"])


def test_fold_layer_openings_bind_to_fri_commitments(p2, chain):
    coms = chain["fri_commitments"]
    n0 = 1 << 23
    qpos = o.sp1_query_positions(chain["query_indices"], n0)
    for i in (int(v) for v in chain["path_layers"]):
        rows, paths = chain[f"rows_f{i}"], chain[f"paths_f{i}"]
        depth = paths.shape[0]
        assert depth == 22 - i  # leaves = n_i / 2 = 2^(22 - i)
        for q in range(rows.shape[0]):
            root = o.reconstruct_root(p2, rows[q], int(qpos[q]) >> (i + 1), paths[:, q])
            assert np.array_equal(o.smcs_bind_root(p2, root, depth, 8), coms[i]), (i, q)


def test_fold_chain_consistency(chain):
    betas = chain["fri_betas"]
    n0 = 1 << 23
    qpos = o.sp1_query_positions(chain["query_indices"], n0)
    rounds = betas.shape[0]
    for i in range(rounds):
        n = n0 >> i
        rows = chain[f"rows_f{i}"]
        for q in range(rows.shape[0]):
            p = int(qpos[q]) >> (i + 1)  # pair index: the leaf (2p, 2p+1) of layer i
            x = o.domain_point(KB, n.bit_length() - 1, 0,
                               o.bit_reverse(p, (n // 2).bit_length() - 1))
            # a 2-element natural layer with shift x folds exactly at x
            g = o.fri_fold(KB, rows[q].reshape(2, 4), True, betas[i], True, x).reshape(-1)
            want = (chain[f"rows_f{i + 1}"][q].reshape(2, 4)[p & 1] if i + 1 < rounds
                    else chain["final_poly"])
            assert np.array_equal(g, want), (i, q)


@pytest.mark.parametrize("field", [o.BABYBEAR, o.KOALABEAR])
def test_bitrev_encode_is_bit_reversed_natural(field):
    rng = np.random.default_rng(7)
    k, lb = 1 << 9, 2
    c = o.to_mont(field, rng.integers(0, o.MODULUS[field], (3, k), dtype=np.uint64))
    shift = int(o.to_mont(field, [31])[0]) if field == o.BABYBEAR else 0
    nat = o.rs_encode(field, c, lb, shift)
    br = o.rs_encode_bitrev(field, c, lb, shift)
    bits = (k << lb).bit_length() - 1
    perm = np.array([o.bit_reverse(j, bits) for j in range(k << lb)])
    assert np.array_equal(br, nat[:, perm])


@pytest.mark.parametrize("ef_in,ef_beta", [(False, False), (False, True), (True, True)])
def test_bitrev_fold_commutes_with_bit_reversal(ef_in, ef_beta):
    """fold_bitrev(brev(f)) == brev(fold(f)) (zorch/coding/reed_solomon.py:443-447)."""
    rng = np.random.default_rng(11)
    field, n = o.BABYBEAR, 1 << 10
    shift = int(o.to_mont(field, [31])[0])
    shape = (n, 4) if ef_in else (n,)
    f = o.to_mont(field, rng.integers(0, o.P_BABYBEAR, shape, dtype=np.uint64))
    beta = o.to_mont(field, rng.integers(0, o.P_BABYBEAR, 4 if ef_beta else 1, dtype=np.uint64))
    bits = n.bit_length() - 1
    perm = np.array([o.bit_reverse(j, bits) for j in range(n)])
    half_perm = np.array([o.bit_reverse(j, bits - 1) for j in range(n // 2)])
    nat = o.fri_fold(field, f, ef_in, beta, ef_beta, shift)
    br = o.fri_fold_bitrev(field, f[perm], ef_in, beta, ef_beta, shift)
    assert np.array_equal(br, nat[half_perm])
