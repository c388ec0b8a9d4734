"""Test helper: the oracle's bytes for one request of a served stream."""

from __future__ import annotations

import numpy as np

from zorch_gb300.field import BABYBEAR


def request_words(orc, p2, r, x_mont, mode):
    """The oracle's bytes for one request of the stream (as u32 words):
    commitment, then for fold requests the fold-and-open proof."""
    from zorch_gb300.serve import FOLD_FINAL_LOG, FOLD_QUERIES

    cw = orc.rs_encode(0, x_mont, r.log_blowup, BABYBEAR.mont(31))
    w, n = cw.shape
    if mode == "fri":
        L = n // 2
        col_layers = [orc.merkle_commit(p2, cw[c], L, 2, 1, L) for c in range(w)]
        commitment = np.concatenate([ly[-1][0] for ly in col_layers])
    else:
        layers = orc.merkle_commit_columns(p2, cw)
        commitment = layers[-1][0]
    parts = [commitment]
    if r.fold:
        t = orc.Transcript(p2)
        t.observe(commitment)
        nbv = (w - 1).bit_length()
        rlc = orc.rlc_columns(0, cw, t.sample(4 * nbv) if nbv else [])
        rounds = r.log_h + r.log_blowup - FOLD_FINAL_LOG
        t.observe([BABYBEAR.mont(rounds)])
        proof = orc.fri_commit_phase(p2, 0, rlc, rounds, FOLD_QUERIES, 4, t, BABYBEAR.mont(31))
        parts += [proof.roots.reshape(-1), proof.final_layer.reshape(-1),
                  proof.positions.astype(np.uint32)]
        if mode == "fri":
            a = (proof.positions.astype(np.int64) % L).astype(np.int32)
            for c in range(w):
                rows, paths = orc.merkle_open(cw[c], L, 2, 1, L, col_layers[c], a)
                parts += [rows.reshape(-1), paths.reshape(-1)]
        else:
            rows, paths = orc.merkle_open(cw, n, w, 1, n, layers, proof.positions)
            parts += [rows.reshape(-1), paths.reshape(-1)]
        for rr, pp in zip(proof.rows, proof.paths):
            parts += [rr.reshape(-1), pp.reshape(-1)]
    return np.concatenate(parts)
