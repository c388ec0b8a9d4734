"""PCS layer on the GPU kernels: the pre-fold pair-leaf commit round, the fold
driver, query openings, and the FRI / Basefold commit entry points
(drop-in for zorch/pcs/fold.py, zorch/prove.py, zorch/pcs/fri/prover.py,
zorch/pcs/basefold/prover.py:190-193, 437-455, zorch/pcs/matrix_commit.py).

Layer layout: a base-field layer is a [n] tensor, an EF4 layer a [n, 4]
tensor (coefficients c0..c3, the to_base_field bitcast of
zorch/pcs/fold.py:42-52). A layer's pair leaves (zorch/coding/reed_solomon.py:
303-307) are addressed in place -- leaf p = (cw[p], cw[p + n/2]) -- never copied.
"""

from __future__ import annotations

from dataclasses import dataclass, field as dc_field
from typing import Sequence

import numpy as np
import torch

from . import _lib
from .coding import ReedSolomon
from .commit import DigestLayers, MerkleTree, Opening, leaves_layout
from .field import ptr, stream_handle, to_host
from .transcript import DuplexTranscript


def limbs_of(layer: torch.Tensor) -> int:
    return 4 if layer.dim() == 2 else 1


def to_base_field(leaves: torch.Tensor) -> torch.Tensor:
    """EF4 leaves [..., 4] reinterpreted as base limbs folded into the last axis."""
    if leaves.dim() >= 2 and leaves.shape[-1] == 4 and leaves.dim() > 2:
        return leaves.reshape(*leaves.shape[:-2], -1)
    return leaves


def pair_layout(layer: torch.Tensor) -> _lib.Leaves:
    n = layer.shape[0]
    limbs = limbs_of(layer)
    return leaves_layout(layer, n // 2, 2, limbs, (n // 2) * limbs)


@dataclass
class CommittedLayer:
    """A committed pre-fold layer kept for the query phase (zorch/pcs/fold.py:68-78)."""

    codeword: torch.Tensor
    digest_layers: DigestLayers

    @property
    def limbs(self) -> int:
        return limbs_of(self.codeword)

    @property
    def root(self) -> torch.Tensor:
        return self.digest_layers.root


@dataclass
class FoldState:
    """Carry of the commit-and-fold recurrence (zorch/pcs/fold.py:81-87). `pending`
    holds the next layer when its tree was already built by the fused
    fold-and-commit kernel."""

    codeword: torch.Tensor
    layers: tuple = ()
    pending: CommittedLayer | None = None


@dataclass
class PreFoldPairCommitRound:
    """commit pair leaves -> observe(root) -> sample beta -> fold
    (zorch/pcs/fold.py:90-115). `challenge_limbs` = 1 draws a base-field beta
    (the reference's native wire), 4 an EF4 beta as sample_challenge(t, EF4, 4)
    (zorch/transcript.py:122-137). With `fused`, the fold of round r runs in
    the same kernel as the pair-leaf hashing of round r+1's layer."""

    code: ReedSolomon
    tree: MerkleTree
    challenge_limbs: int = 1
    fused: bool = True
    last_round: int | None = None  # index of the final round (no commit after it)

    def commit_layer(self, cw: torch.Tensor) -> CommittedLayer:
        n = cw.shape[0]
        _, layers = self.tree.commit_layout(pair_layout(cw), cw.device)
        return CommittedLayer(cw, layers)

    def __call__(self, state: FoldState, t: DuplexTranscript):
        cw = state.codeword
        layer = state.pending if state.pending is not None else self.commit_layer(cw)
        t = t._copy()
        beta = t.observe_and_sample_(layer.root, self.challenge_limbs)
        n = cw.shape[0]
        level = len(state.layers)
        is_last = self.last_round is not None and level >= self.last_round
        if self.fused and not is_last and n >= 4:
            out, pending = self.fold_commit(cw, beta, level)
        else:
            out, pending = self.code.fold(cw, beta), None
        return FoldState(out, state.layers + (layer,), pending), t, layer.root

    def fold_commit(self, cw: torch.Tensor, beta: torch.Tensor, level: int):
        n = cw.shape[0]
        ef_in = cw.dim() == 2
        ef_beta = beta.numel() == 4
        lo = 4 if (ef_in or ef_beta) else 1
        out = torch.empty((n // 2, 4) if lo == 4 else (n // 2,), dtype=torch.int32,
                          device=cw.device)
        L = n // 4
        flat = torch.empty((2 * L - 1, 8), dtype=torch.int32, device=cw.device)
        _lib.check(_lib.lib().zc_fri_fold_commit(
            self.tree.perm.handle, ptr(cw), n, int(ef_in), ptr(beta), int(ef_beta),
            self.code.level_shift_mont(level), self.code.generator or 0, ptr(out), ptr(flat),
            stream_handle()), "fri_fold_commit")
        return out, CommittedLayer(out, DigestLayers(flat, L))


def fold_rounds(rnd, state, transcript, rounds: int):
    """Run `rnd` exactly `rounds` times (zorch/prove.py:26-37)."""
    msgs = []
    for _ in range(rounds):
        state, transcript, msg = rnd(state, transcript)
        msgs.append(msg)
    return state, transcript, msgs


def open_layer(tree: MerkleTree, layer: CommittedLayer, indices: torch.Tensor) -> Opening:
    """open_rows over a layer's pair leaves (zorch/pcs/fold.py:142-149); the
    indices are reduced mod the layer's leaf count, so no range check."""
    return tree.open_layout(pair_layout(layer.codeword), layer.digest_layers, indices,
                            2 * layer.limbs, check=False)


@dataclass
class CommitPhaseProof:
    """Commit-phase proof: per-round roots, the cleartext final layer, the
    query positions and each layer's opened pair leaf with its path."""

    roots: torch.Tensor               # [R, 8]
    betas: list[torch.Tensor]         # R x (1 or 4,)
    final_layer: torch.Tensor         # [n_R] or [n_R, 4]
    positions: torch.Tensor           # [Q]
    openings: list[Opening] = dc_field(default_factory=list)

    def to_bytes(self) -> bytes:
        """Mont-u32 little-endian in pytree flatten order: roots, final layer,
        then each layer's rows and path levels."""
        parts = [self.roots.reshape(-1), self.final_layer.reshape(-1)]
        for op in self.openings:
            parts += [op.row.reshape(-1), op.path.reshape(-1)]
        return to_host(torch.cat(parts)).astype("<u4").tobytes()


@dataclass(frozen=True)
class FriParams:
    """Public FRI configuration (zorch/pcs/fri/config.py:39-46)."""

    code: ReedSolomon
    tree: MerkleTree
    num_rounds: int
    num_queries: int
    challenge_limbs: int = 1


@dataclass
class FriCommittedPoly:
    """zorch/pcs/fri/prover.py:55-72: coeffs, codeword and its pair-leaf tree."""

    coeffs: torch.Tensor
    codeword: torch.Tensor
    digest_layers: DigestLayers

    @property
    def root(self) -> torch.Tensor:
        return self.digest_layers.root


@dataclass
class FriProverData:
    polys: tuple


class FriProver:
    """FRI prover over the GPU kernels (zorch/pcs/fri/prover.py:81-133)."""

    def __init__(self, params: FriParams) -> None:
        self.params = params

    def commit_one(self, coeffs: torch.Tensor, out: torch.Tensor | None = None) -> FriCommittedPoly:
        """_commit_one (zorch/pcs/fri/prover.py:141-148): encode, then the
        pair-leaf Merkle commit of the codeword."""
        code, tree = self.params.code, self.params.tree
        cw = code.encode(coeffs, out)
        _, layers = tree.commit_layout(pair_layout(cw), cw.device)
        return FriCommittedPoly(coeffs, cw, layers)

    def commit(self, polys: Sequence[torch.Tensor]):
        """One call per polynomial, roots stacked (zorch/pcs/fri/prover.py:92-99)."""
        committed = [self.commit_one(p) for p in polys]
        return torch.stack([c.root for c in committed]), FriProverData(tuple(committed))

    def commit_phase(self, codeword: torch.Tensor, transcript: DuplexTranscript,
                     first_layer: CommittedLayer | None = None):
        """Fold rounds down to block_len >> num_rounds, observe the final layer,
        sample the query positions and open every layer (the commit/query phase
        of _open_one, zorch/pcs/fri/prover.py:151-187, on `codeword` itself)."""
        p = self.params
        rnd = PreFoldPairCommitRound(p.code, p.tree, p.challenge_limbs,
                                     last_round=p.num_rounds - 1)
        state = FoldState(codeword, (), first_layer)
        t = transcript._copy()
        betas = []
        roots = []
        for _ in range(p.num_rounds):
            state, t, root = rnd(state, t)
            roots.append(root)
        final = state.codeword
        n0 = codeword.shape[0]
        positions = t.sample_positions_(n0, p.num_queries, values=final)
        openings = []
        q = positions
        for i, layer in enumerate(state.layers):
            q = torch.remainder(q, n0 >> (i + 1))
            openings.append(open_layer(p.tree, layer, q))
        roots_t = torch.stack(roots) if roots else torch.empty((0, 8), dtype=torch.int32,
                                                               device=codeword.device)
        return CommitPhaseProof(roots_t, betas, final, positions, openings), t, state


@dataclass
class BasefoldProverData:
    digest_layers: DigestLayers
    codeword: torch.Tensor  # [K, block_len]: column-major; codeword.T rows are the leaves
    widths: tuple


class BasefoldProver:
    """Basefold matrix commit (zorch/pcs/basefold/prover.py:190-193, 437-455):
    one batched LDE over the [K, S] columns, leaves = codeword rows."""

    def __init__(self, code: ReedSolomon, tree: MerkleTree, num_queries: int = 4) -> None:
        self.code = code
        self.tree = tree
        self.num_queries = num_queries

    def commit_columns(self, columns: torch.Tensor):
        """columns [K, S] (the reference's mle.T) -> (root, prover data)."""
        cw = self.code.encode(columns)
        K, n = cw.shape
        _, layers = self.tree.commit_layout(leaves_layout(cw, n, K, 1, n), cw.device)
        return layers.root, BasefoldProverData(layers, cw, (K,))

    def commit(self, polys: Sequence[torch.Tensor]):
        return self.commit_columns(torch.stack(list(polys), dim=0))

    def open_rows(self, data: BasefoldProverData, indices: torch.Tensor) -> Opening:
        K, n = data.codeword.shape
        return self.tree.open_layout(leaves_layout(data.codeword, n, K, 1, n),
                                     data.digest_layers, indices, K)


class GraphedFriCommitPhase:
    """The encode + FRI commit phase of one polynomial shape captured once into
    a CUDA graph: every round's fused fold-and-commit, the device transcript
    steps and the query openings replay with one launch. The transcript starts
    from the empty state; `replay(coeffs)` copies new Montgomery coefficients
    into the static input and returns the (static) proof tensors, overwritten
    by each replay."""

    def __init__(self, prover: FriProver, device="cuda") -> None:
        self.prover = prover
        code = prover.params.code
        self.coeffs = torch.zeros(code.message_len, dtype=torch.int32, device=device)
        self._run()  # kernel attributes, allocator warm-up
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.proof = self._run()

    def _run(self) -> CommitPhaseProof:
        code = self.prover.params.code
        cw = code.encode(self.coeffs)
        t = DuplexTranscript.new(self.prover.params.tree.perm, device=self.coeffs.device)
        proof, _, _ = self.prover.commit_phase(cw, t)
        return proof

    def replay(self, coeffs: torch.Tensor | None = None) -> CommitPhaseProof:
        if coeffs is not None:
            self.coeffs.copy_(coeffs, non_blocking=True)
        self.graph.replay()
        return self.proof
