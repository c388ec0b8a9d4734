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
from .field import full_u32, parts_to_bytes, ptr, stream_handle, to_host
from .stage import (OpeningClaim, OpeningProof, OpeningWitness, ProveResult, TrivialClaim,
                    VerifyResult)
from .transcript import DuplexTranscript


def stack_rows(rows: Sequence[torch.Tensor], shape=None, device=None) -> torch.Tensor:
    """torch.stack of equally shaped device tensors by one device-to-device
    copy per row into a preallocated tensor (copy engine, no gather kernel)."""
    if not rows:
        return torch.empty((0, *(shape or ())), dtype=torch.int32, device=device)
    out = torch.empty((len(rows), *rows[0].shape), dtype=rows[0].dtype, device=rows[0].device)
    for i, r in enumerate(rows):
        out[i].copy_(r, non_blocking=True)
    return out


def limbs_of(layer: torch.Tensor) -> int:
    return 4 if layer.dim() == 2 else 1


def to_base_field(leaves: torch.Tensor) -> torch.Tensor:
    """EF4 leaves [..., 4] reinterpreted as base limbs folded into the last axis."""
    if leaves.dim() >= 2 and leaves.shape[-1] == 4 and leaves.dim() > 2:
        return leaves.reshape(*leaves.shape[:-2], -1)
    return leaves


def pair_layout(layer: torch.Tensor, bit_reversed: bool = False) -> _lib.Leaves:
    """A layer's pair leaves in place: (cw[p], cw[p + n/2]) in natural order,
    the adjacent (cw[2p], cw[2p+1]) in bit-reversed order
    (zorch/coding/reed_solomon.py:303-307, 512-515)."""
    n = layer.shape[0]
    limbs = limbs_of(layer)
    if bit_reversed:
        return leaves_layout(layer, n // 2, 1, 2 * limbs, 0)
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
    betas: tuple = ()  # the challenge sampled in each round so far
    # the pending layer's challenge when the previous round's launch already
    # ran this round's transcript hop (fuse_hop); the transcript is past it
    pending_beta: torch.Tensor | None = None


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
    # Run each round's observe(root) + sample(beta) inside the launch that
    # computes the root (zc_merkle_commit_hop / zc_fri_fold_commit_hop): one
    # launch fewer per round. The transcript a round returns is then already
    # past the next round's hop, so this is only for rounds that follow each
    # other directly on one transcript (FriProver.commit_phase).
    fuse_hop: bool = False

    def commit_layer(self, cw: torch.Tensor) -> CommittedLayer:
        _, layers = self.tree.commit_layout(pair_layout(cw, self.code.bit_reversed), cw.device)
        return CommittedLayer(cw, layers)

    def commit_layer_hop(self, cw: torch.Tensor, t: DuplexTranscript):
        """commit_layer, then observe(root) + sample(beta) in the root's launch."""
        L = cw.shape[0] // 2
        flat = torch.empty((2 * L - 1, 8), dtype=torch.int32, device=cw.device)
        beta = torch.empty(self.challenge_limbs, dtype=torch.int32, device=cw.device)
        _lib.check(_lib.lib().zc_merkle_commit_hop(
            self.tree.perm.handle, pair_layout(cw, self.code.bit_reversed), ptr(flat),
            ptr(t.state), self.challenge_limbs, ptr(beta), stream_handle()), "merkle_commit_hop")
        return CommittedLayer(cw, DigestLayers(flat, L)), beta

    def __call__(self, state: FoldState, t: DuplexTranscript):
        cw = state.codeword
        t = t._copy()
        if state.pending is not None and state.pending_beta is not None:
            layer, beta = state.pending, state.pending_beta
        elif state.pending is None and self.fuse_hop:
            layer, beta = self.commit_layer_hop(cw, t)
        else:
            layer = state.pending if state.pending is not None else self.commit_layer(cw)
            beta = t.observe_and_sample_(layer.root, self.challenge_limbs)
        n = cw.shape[0]
        level = len(state.layers)
        is_last = self.last_round is not None and level >= self.last_round
        next_beta = None
        if self.fused and not is_last and n >= 4:
            if self.fuse_hop:
                out, pending, next_beta = self.fold_commit(cw, beta, level, t)
            else:
                out, pending = self.fold_commit(cw, beta, level)
        else:
            out, pending = self.code.fold(cw, beta), None
        return FoldState(out, state.layers + (layer,), pending, state.betas + (beta,),
                         next_beta), t, layer.root

    def fold_commit(self, cw: torch.Tensor, beta: torch.Tensor, level: int,
                    hop: DuplexTranscript | None = None):
        """The fold of this round fused with the commit of the next layer;
        with `hop`, also that layer's observe(root) + sample(beta) on `hop`
        (in place), returning the sampled beta as a third value."""
        n = cw.shape[0]
        ef_in = cw.dim() == 2
        ef_beta = beta.numel() == 4
        lo = 4 if (ef_in or ef_beta) else 1
        out = torch.empty((n // 2, 4) if lo == 4 else (n // 2,), dtype=torch.int32,
                          device=cw.device)
        L = n // 4
        flat = torch.empty((2 * L - 1, 8), dtype=torch.int32, device=cw.device)
        if hop is not None:
            nxt = torch.empty(self.challenge_limbs, dtype=torch.int32, device=cw.device)
            _lib.check(_lib.lib().zc_fri_fold_commit_hop(
                self.tree.perm.handle, ptr(cw), n, int(ef_in), ptr(beta), int(ef_beta),
                self.code.level_shift_mont(level), self.code.generator or 0,
                int(self.code.bit_reversed), ptr(out), ptr(flat), ptr(hop.state),
                self.challenge_limbs, ptr(nxt), stream_handle()), "fri_fold_commit_hop")
            return out, CommittedLayer(out, DigestLayers(flat, L)), nxt
        fn = (_lib.lib().zc_fri_fold_commit_bitrev if self.code.bit_reversed
              else _lib.lib().zc_fri_fold_commit)
        _lib.check(fn(
            self.tree.perm.handle, ptr(cw), n, int(ef_in), ptr(beta), int(ef_beta),
            self.code.level_shift_mont(level), self.code.generator or 0, ptr(out), ptr(flat),
            stream_handle()), "fri_fold_commit")
        return out, CommittedLayer(out, DigestLayers(flat, L))


def group_layout(layer: torch.Tensor, k: int) -> _lib.Leaves:
    """k-group leaves of a natural-order layer in place: leaf p =
    (cw[p], cw[p + n/k], ..., cw[p + (k-1)n/k]) in base limbs."""
    n = layer.shape[0]
    limbs = limbs_of(layer)
    return leaves_layout(layer, n // k, k, limbs, (n // k) * limbs)


@dataclass
class PreFoldKGroupCommitRound:
    """commit the k-group leaves -> observe(root) -> sample beta -> k-ary fold
    (zorch/pcs/fold.py:118-139): one leaf is one k-th-root coset, so one path
    opens all k legs the fold consumes."""

    code: ReedSolomon
    tree: MerkleTree

    def __call__(self, state: FoldState, t: DuplexTranscript):
        cw = state.codeword
        k = self.code.fold_factor
        _, layers = self.tree.commit_layout(group_layout(cw, k), cw.device)
        layer = CommittedLayer(cw, layers)
        t = t._copy()
        beta = t.observe_and_sample_(layer.root, 1)
        out = self.code.fold_group(cw, beta)
        return FoldState(out, state.layers + (layer,)), t, layer.root


def open_group_layer(tree: MerkleTree, layer: CommittedLayer, indices: torch.Tensor,
                     k: int) -> Opening:
    """open_rows over a layer's k-group leaves."""
    return tree.open_layout(group_layout(layer.codeword, k), layer.digest_layers, indices,
                            k * layer.limbs, check=False)


def verify_group_fold_chain(code: ReedSolomon, query_openings, betas, leaf_indices,
                            final_poly) -> bool:
    """Each opened k-group folds to the next layer's opened leg, the last to the
    final poly (zorch/pcs/fold.py:471-505), on the host."""
    f = code.field
    k = code.fold_factor
    final = to_host(final_poly) if torch.is_tensor(final_poly) else np.asarray(final_poly)
    final = final.reshape(final.shape[0], -1)
    ok = True
    nr = len(query_openings)
    host = lambda x: to_host(x) if torch.is_tensor(x) else np.asarray(x, np.uint32)  # noqa: E731
    for i in range(nr):
        rows = host(query_openings[i].row)
        pos = [int(x) for x in host(leaf_indices[i]).view(np.int32)]
        folded = code.fold_group_values(rows, host(betas[i]), pos, i)
        if i + 1 < nr:
            nxt_pos = torch.as_tensor(host(leaf_indices[i + 1]).view(np.int32))
            members = [host(m).view(np.int32) for m in code.group_indices(nxt_pos, i + 1)]
            nxt = host(query_openings[i + 1].row).reshape(len(pos), k, -1)
            for qi, p in enumerate(pos):
                legs = [m for m in range(k) if int(members[m][qi]) == p]
                if len(legs) != 1:
                    return False
                words = [int(x) for x in nxt[qi, legs[0]]]
                ok &= folded[qi] == f.ef_from_mont(words + [0] * (4 - len(words)))
        else:
            for qi, p in enumerate(pos):
                words = [int(x) for x in final[p]]
                ok &= folded[qi] == f.ef_from_mont(words + [0] * (4 - len(words)))
    return bool(ok)


def fold_rounds(rnd, state, transcript, rounds: int):
    """Run `rnd` exactly `rounds` times (zorch/prove.py:26-37)."""
    msgs = []
    for _ in range(rounds):
        state, transcript, msg = rnd(state, transcript)
        msgs.append(msg)
    return state, transcript, msgs


def open_layer(tree: MerkleTree, layer: CommittedLayer, positions: torch.Tensor,
               level: int = 0, bit_reversed: bool = False) -> Opening:
    """open_rows over layer `level`'s pair leaves (zorch/pcs/fold.py:142-149)
    at its layer positions -- positions mod the layer's leaf count in natural
    order, positions >> (level + 1) in bit-reversed order
    (code.layer_positions, zorch/coding/reed_solomon.py:320-329, 521-528) --
    reduced by the opening kernel: no range check, no reduction launch."""
    return tree.open_layout_reduced(pair_layout(layer.codeword, bit_reversed),
                                    layer.digest_layers, positions, 2 * layer.limbs,
                                    level + 1 if bit_reversed else 0)


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
        return parts_to_bytes(parts)


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
        _, layers = tree.commit_layout(pair_layout(cw, code.bit_reversed), cw.device)
        return FriCommittedPoly(coeffs, cw, layers)

    def commit(self, polys: Sequence[torch.Tensor]):
        """One call per polynomial, roots stacked (zorch/pcs/fri/prover.py:92-99)."""
        committed = [self.commit_one(p) for p in polys]
        return stack_rows([c.root for c in committed]), FriProverData(tuple(committed))

    def commit_phase(self, codeword: torch.Tensor, transcript: DuplexTranscript,
                     first_layer: CommittedLayer | None = None):
        """Fold rounds down to block_len >> num_rounds, observe the final layer,
        sample the query positions and open every layer (the commit/query phase
        of _open_one, zorch/pcs/fri/prover.py:151-187, on `codeword` itself)."""
        p = self.params
        # fuse_hop stays off: on the 2^22, 15-round commit phase replayed from
        # a CUDA graph the separate hop launch measured 0.05 ms faster per
        # proof (6.26 vs 6.31 ms) than the hop inside the root launch
        rnd = PreFoldPairCommitRound(p.code, p.tree, p.challenge_limbs,
                                     last_round=p.num_rounds - 1)
        state = FoldState(codeword, (), first_layer)
        t = transcript._copy()
        roots = []
        for _ in range(p.num_rounds):
            state, t, root = rnd(state, t)
            roots.append(root)
        final = state.codeword
        n0 = codeword.shape[0]
        positions = t.sample_positions_(n0, p.num_queries, values=final)
        br = p.code.bit_reversed
        openings = [open_layer(p.tree, layer, positions, i, br)
                    for i, layer in enumerate(state.layers)]
        roots_t = stack_rows(roots, (8,), codeword.device)
        return CommitPhaseProof(roots_t, list(state.betas), final, positions, openings), t, state


    # -- the open: ProverStage.prove (zorch/pcs/fri/prover.py:101-187) --------
    def prove(self, claim: OpeningClaim, witness: OpeningWitness,
              transcript: DuplexTranscript) -> ProveResult:
        """Open the committed polynomials at the claim's points. Terminal: the
        claim reduces to TrivialClaim(); the reduction proof is
        OpeningProof(values, [FriProof per polynomial])."""
        values, proofs, t = self._open(witness.prover_data, claim.points, transcript)
        return ProveResult(TrivialClaim(), OpeningProof(values, proofs), t)

    def _open(self, prover_data: FriProverData, points: Sequence, transcript: DuplexTranscript):
        """One _open_one per polynomial, threading one transcript through them
        in order (zorch/pcs/fri/prover.py:114-133). Returns (values [k] base /
        [k, 4] EF4, proofs, transcript)."""
        if len(prover_data.polys) != len(points):
            raise ValueError(f"batch mismatch: {len(prover_data.polys)} polys vs "
                             f"{len(points)} points")
        t = transcript._copy()
        values, proofs = [], []
        for committed, z in zip(prover_data.polys, points):
            proof, t = self._open_one(committed, fri_point(self.params.code.field, z), t)
            values.append(proof.value)
            proofs.append(proof)
        if not values:
            return torch.empty(0, dtype=torch.int32), proofs, t
        return stack_rows(values), proofs, t

    def _open_one(self, committed: FriCommittedPoly, z: torch.Tensor, t: DuplexTranscript):
        """_open_one (zorch/pcs/fri/prover.py:151-187) on the device with no
        host synchronisation: v = f(z) (zc_eval_poly), the layer-0 DEEP
        quotient (cw - v) / (domain - z) (zc_deep_quotient), observe f's root,
        the pre-fold pair commit rounds, the final layer and the query
        positions (commit_phase), and f's pair leaf at each layer-0 position."""
        code, tree = self.params.code, self.params.tree
        f = code.field
        dev = committed.codeword.device
        zl = z.numel()
        L = _lib.lib()
        st = stream_handle()
        coeffs = committed.coeffs.contiguous()
        k = coeffs.numel()
        v = torch.empty(zl, dtype=torch.int32, device=dev)
        nb = L.zc_eval_poly_workspace_bytes(k)
        ws = torch.empty((nb + 15) // 4, dtype=torch.int32, device=dev)
        _lib.check(L.zc_eval_poly(f.id, ptr(coeffs), k, ptr(z), zl, ptr(v), ptr(ws), nb, st),
                   "eval_poly")
        n = committed.codeword.shape[0]
        q = torch.empty((n,) if zl == 1 else (n, 4), dtype=torch.int32, device=dev)
        _lib.check(L.zc_deep_quotient(f.id, ptr(committed.codeword), n, ptr(z), zl, ptr(v),
                                      code._shift_mont, code.generator or 0,
                                      int(code.bit_reversed), ptr(q), st), "deep_quotient")
        t = t._copy()
        t.observe_(committed.root)
        phase, t, _ = self.commit_phase(q, t)
        br = code.bit_reversed
        f_open = tree.open_layout_reduced(pair_layout(committed.codeword, br),
                                          committed.digest_layers, phase.positions, 2,
                                          1 if br else 0)
        proof = FriProof(v.reshape(()) if zl == 1 else v, phase.roots, phase.final_layer,
                         f_open, phase.openings, phase.positions)
        return proof, t


def point_words(field, z) -> np.ndarray:
    """An opening point as host Montgomery words (see fri_point)."""
    if torch.is_tensor(z) or isinstance(z, np.ndarray):
        w = _host(z).reshape(-1)
    else:
        w = np.asarray([field.mont(int(x)) for x in (z if isinstance(z, (tuple, list)) else [z])],
                       np.uint32)
    if w.size not in (1, 4):
        raise ValueError(f"an opening point has 1 (base) or 4 (EF4) limbs, got {w.size}")
    return w


def fri_point(field, z) -> torch.Tensor:
    """An opening point as device Montgomery words: a tensor (1 word: base, 4:
    EF4) passes through; a Python int is a canonical base element; a 4-tuple
    of ints a canonical EF4 element."""
    if torch.is_tensor(z):
        if z.numel() not in (1, 4):
            raise ValueError(f"an opening point has 1 (base) or 4 (EF4) limbs, got {z.numel()}")
        return z.reshape(-1).to(torch.int32).contiguous()
    words = [field.mont(int(x)) for x in (z if isinstance(z, (tuple, list)) else [z])]
    if len(words) not in (1, 4):
        raise ValueError(f"an opening point has 1 (base) or 4 (EF4) limbs, got {len(words)}")
    return torch.tensor(np.asarray(words, np.uint32).view(np.int32), device="cuda")


@dataclass
class FriProof:
    """zorch/pcs/fri/config.py:56-69: value = f(z); fri_roots = the quotient's
    pre-fold layer roots [R, 8]; final_layer; f_opening = f's pair leaf at each
    query's layer-0 position (rebuilds the quotient at layer 0);
    query_openings = each fold layer's pair leaf. `positions` (the sampled
    query positions) is derived by both sides and is not on the wire."""

    value: torch.Tensor
    fri_roots: torch.Tensor
    final_layer: torch.Tensor
    f_opening: Opening
    query_openings: list[Opening]
    positions: torch.Tensor | None = None

    def parts(self) -> list[torch.Tensor]:
        """The wire tensors in pytree flatten order: value, fri_roots,
        final_layer, f_opening (row, path), query_openings (row, path each)."""
        out = [self.value.reshape(-1), self.fri_roots, self.final_layer, self.f_opening.row,
               self.f_opening.path]
        for op in self.query_openings:
            out += [op.row, op.path]
        return out

    def to_bytes(self) -> bytes:
        """Mont-u32 little endian in pytree flatten order."""
        return parts_to_bytes(self.parts())


def _host(x) -> np.ndarray:
    return to_host(x) if torch.is_tensor(x) else np.asarray(x, np.uint32)


class FriVerifier:
    """FRI verifier on the host (zorch/pcs/fri/verifier.py:31-140): replays the
    transcript, checks the final layer is constant, every opened leaf against
    its root, the layer-0 quotient pair rebuilt from f's opened leaf, and the
    fold chain down to the final layer. A bad proof is a False verdict;
    structural mismatches raise ValueError, as the reference does."""

    def __init__(self, params: FriParams) -> None:
        self.params = params

    def verify(self, claim: OpeningClaim, reduction_proof: OpeningProof, transcript):
        ok, t = self._verify_opening(claim.commitment, claim.points, reduction_proof.values,
                                     reduction_proof.proof, transcript)
        return VerifyResult(TrivialClaim(), t, ok)

    def _verify_opening(self, commitment, points, values, proof, transcript):
        from .transcript import HostDuplexTranscript

        roots = _host(commitment).reshape(-1, 8)
        vals = _host(values)
        k = roots.shape[0]
        nvals = vals.shape[0] if vals.ndim else 1
        if not (len(points) == nvals == len(proof) == k):
            raise ValueError(f"batch mismatch: commitment={k}, points={len(points)}, "
                             f"values={nvals}, proof={len(proof)}")
        rounds = self.params.num_rounds
        for pf in proof:
            if pf.fri_roots.shape[0] != rounds or len(pf.query_openings) != rounds:
                raise ValueError(f"malformed proof: expected {rounds} fold layers, got "
                                 f"{pf.fri_roots.shape[0]} roots / {len(pf.query_openings)} "
                                 "openings")
        t = host_transcript(self.params.tree.perm, transcript)
        oks = []
        vals = vals.reshape(k, -1)
        for f_root, z, v, pf in zip(roots, points, vals, proof):
            t, ok = self._verify_one(f_root, z, v, pf, t)
            oks.append(ok)
        return all(oks), t

    def _verify_one(self, f_root, z, v, pf: FriProof, t):
        p = self.params
        code, tree = p.code, p.tree
        f = code.field
        n = code.block_len
        zw = point_words(f, z)
        zl = zw.size
        vw = np.asarray(v, np.uint32).reshape(-1)
        if vw.size != zl:
            return t, False
        pad = lambda w: tuple(f.ef_from_mont(list(w) + [0] * (4 - len(w))))  # noqa: E731
        zc, vc = pad(zw), pad(vw)
        t = t.observe(f_root)
        betas = []
        for r in _host(pf.fri_roots).reshape(-1, 8):
            t, b = t.observe_and_sample(r, p.challenge_limbs)
            betas.append(pad(b))
        final = _host(pf.final_layer)
        t = t.observe(final.reshape(-1))
        fin = final.reshape(final.shape[0], -1)
        ok = bool((fin == fin[0]).all())
        t, raw = t.sample(p.num_queries)
        positions = [int(x) % n for x in raw]
        br = code.bit_reversed

        def leaf_index(q: int, level: int) -> int:
            return q >> (level + 1) if br else q % (n >> (level + 1))

        # Merkle: f's pair leaf at a_0, every fold layer's pair leaf at a_i
        f_rows = _host(pf.f_opening.row)
        for qi, q in enumerate(positions):
            ok &= tree.verify(torch.as_tensor(np.asarray(f_root, np.uint32).view(np.int32)),
                              leaf_index(q, 0),
                              Opening(pf.f_opening.row[qi], pf.f_opening.path[:, qi]))
            for i, op in enumerate(pf.query_openings):
                ok &= tree.verify(torch.as_tensor(_host(pf.fri_roots)[i].view(np.int32)),
                                  leaf_index(q, i), Opening(op.row[qi], op.path[:, qi]))
        if not ok:
            return t, False
        shift = code.coset_shift
        gen = code.generator or None

        def point(level: int, j: int) -> int:
            """Layer `level`'s domain point at natural index j."""
            nl = n >> level
            sh = pow(shift, 1 << level, f.p) if shift is not None else 1
            return sh * pow(f.root_of_unity(nl.bit_length() - 1, gen), j, f.p) % f.p

        def pair_points(level: int, a: int) -> tuple:
            """(lo, hi) codeword indices of the pair at leaf a and the lo
            point's natural index (hi's point is its negation)."""
            nl = n >> level
            if br:
                bits = nl.bit_length() - 1
                j = int(format(2 * a, f"0{bits}b")[::-1], 2) if bits else 0
                return 2 * a, 2 * a + 1, j
            return a, a + nl // 2, a

        layer0 = [_host(op.row) for op in pf.query_openings]
        inv2 = pow(2, f.p - 2, f.p)
        for qi, q in enumerate(positions):
            a0 = leaf_index(q, 0)
            _, _, j0 = pair_points(0, a0)
            x_lo = point(0, j0)
            x_hi = (f.p - x_lo) % f.p
            f_lo, f_hi = f.canon(int(f_rows[qi, 0])), f.canon(int(f_rows[qi, 1]))
            # the quotient pair rebuilt from f's opened leaf == the committed layer-0 leaf
            for fx, x, slot in ((f_lo, x_lo, 0), (f_hi, x_hi, 1)):
                num = f.ef_sub((fx, 0, 0, 0), vc)
                den = f.ef_sub((x, 0, 0, 0), zc)
                g = (0, 0, 0, 0) if den == (0, 0, 0, 0) else f.ef_mul(num, f.ef_inv(den))
                lw = layer0[0][qi].reshape(2, -1)[slot] if p.num_rounds else None
                if lw is not None:
                    ok &= g == pad(lw)
            # fold chain
            for i in range(p.num_rounds):
                a = leaf_index(q, i)
                leaf = layer0[i][qi].reshape(2, -1)
                lo, hi = pad(leaf[0]), pad(leaf[1])
                _, _, j = pair_points(i, a)
                x = point(i, j)
                inv2x = pow(2 * x % f.p, f.p - 2, f.p)
                folded = f.ef_add(f.ef_scale(f.ef_add(lo, hi), inv2),
                                  f.ef_mul(f.ef_scale(f.ef_sub(lo, hi), inv2x), betas[i]))
                if i + 1 < p.num_rounds:
                    a_next = leaf_index(q, i + 1)
                    lo_n, _, _ = pair_points(i + 1, a_next)
                    nxt = layer0[i + 1][qi].reshape(2, -1)
                    expected = pad(nxt[0] if a == lo_n else nxt[1])
                else:
                    expected = pad(fin[a])
                ok &= folded == expected
        return t, bool(ok)


def host_transcript(perm, transcript=None):
    """The verifier's host transcript: fresh (None), a HostDuplexTranscript
    as is, or a device DuplexTranscript's state read back."""
    from .transcript import HostDuplexTranscript

    if transcript is None:
        return HostDuplexTranscript(perm)
    if isinstance(transcript, HostDuplexTranscript):
        return transcript
    return HostDuplexTranscript(perm, to_host(transcript.state).copy())


@dataclass
class BasefoldProverData:
    """zorch/pcs/basefold/prover.py:65-83: digest layers, the codeword (column
    major [K, block_len]; codeword.T rows are the leaves) and the message
    columns [K, S] (the reference's mle.T, kept for the open)."""

    digest_layers: DigestLayers
    codeword: torch.Tensor
    widths: tuple
    columns: torch.Tensor | None = None


@dataclass
class BasefoldProof:
    """zorch/pcs/basefold/config.py BasefoldProof: per round the sumcheck
    message (s(0), s(1)) and the pre-fold pair-leaf root, the cleartext final
    codeword, every matrix opened at the query positions and every fold layer's
    pair leaf at its halved position."""

    uni_msgs: torch.Tensor            # [v, 8]: s(0) c0..c3, s(1) c0..c3
    fri_roots: torch.Tensor           # [v, 8]
    final_poly: torch.Tensor          # [blowup, 4]
    component_openings: list[Opening]
    query_openings: list[Opening]
    positions: torch.Tensor           # [Q]

    def to_bytes(self) -> bytes:
        """Mont-u32 little endian in pytree flatten order: messages, roots,
        final poly, component then query openings (row, path)."""
        parts = [self.uni_msgs.reshape(-1), self.fri_roots.reshape(-1),
                 self.final_poly.reshape(-1)]
        for op in list(self.component_openings) + list(self.query_openings):
            parts += [op.row.reshape(-1), op.path.reshape(-1)]
        return parts_to_bytes(parts)


def _ceil_log2(x: int) -> int:
    return (x - 1).bit_length() if x > 1 else 0


class BasefoldProver:
    """Basefold PCS prover (zorch/pcs/basefold/prover.py:160-247, 419-547):
    the matrix commit (one batched LDE over the [K, S] columns, leaves =
    codeword rows) and the native batch open (staggered batching of the
    matrices, interleaved sumcheck + pre-fold pair commits, queries)."""

    def __init__(self, code: ReedSolomon, tree: MerkleTree, num_queries: int = 4) -> None:
        self.code = code
        self.tree = tree
        self.num_queries = num_queries

    def commit_columns(self, columns: torch.Tensor):
        """columns [K, S] (the reference's mle.T) -> (root, prover data)."""
        cw = self.code.encode(columns)
        K, n = cw.shape
        _, layers = self.tree.commit_layout(leaves_layout(cw, n, K, 1, n), cw.device)
        return layers.root, BasefoldProverData(layers, cw, (K,), columns.contiguous())

    def prove(self, claim: OpeningClaim, witness: OpeningWitness,
              transcript: DuplexTranscript) -> ProveResult:
        """Open a single committed matrix, the degenerate one-matrix batch
        (zorch/pcs/basefold/prover.py:195-209): the claim's points are one
        shared EF4 point; the reduction proof is OpeningProof(values [w, 4],
        proof) and the claim reduces to TrivialClaim()."""
        values, proof, t = self.open_batch([witness.prover_data], claim.points, transcript)
        return ProveResult(TrivialClaim(), OpeningProof(values[0], proof), t)

    def open_batch(self, rounds: Sequence[BasefoldProverData], points,
                   transcript: DuplexTranscript):
        """Batch-open the committed matrices at the shared EF4 point
        (zorch/pcs/basefold/prover.py:211-244; _open_batch_body, :503-547, and
        _fold_and_query, :419-480). `points` is the one-point sequence of the
        reference ([z], z of shape [v, 4], Montgomery words on the device) or
        z itself. Returns (values: per matrix [w, 4], proof, transcript). The
        whole open runs on the device with no host synchronisation, so it can
        be captured in a CUDA graph (GraphedBasefoldOpen)."""
        if torch.is_tensor(points):
            z = points
        else:
            if len(points) != 1:
                raise ValueError(f"BaseFold opens the matrices at one shared point, got "
                                 f"{len(points)}")
            z = points[0]
        if not rounds:
            raise ValueError("BaseFold opens at least one committed matrix, got none")
        if z.dim() != 2 or z.shape[1] != 4 or z.shape[0] < 1:
            raise ValueError("the opening point is EF4 [num_vars >= 1, 4]")
        code, tree, f = self.code, self.tree, self.code.field
        v = z.shape[0]
        S = 1 << v
        if code.message_len != S:
            raise ValueError(f"point dimension {v} doesn't match MLE height {code.message_len}")
        for pd in rounds:
            if pd.columns is None or pd.columns.shape[1] != S:
                raise ValueError("prover data without its [K, S] message columns")
        dev = z.device
        L = _lib.lib()
        st = stream_handle()
        zc = z.contiguous()
        t = transcript._copy()
        for pd in rounds:
            t.observe_(pd.digest_layers.root)
        values = []
        for pd in rounds:
            w = pd.columns.shape[0]
            out = torch.empty((w, 4), dtype=torch.int32, device=dev)
            nb = L.zc_eval_mle_workspace_bytes(w, v)
            ws = torch.empty((nb + 15) // 4, dtype=torch.int32, device=dev)
            _lib.check(L.zc_eval_mle(f.id, ptr(pd.columns), w, v, ptr(zc), ptr(out), ptr(ws), nb,
                                     st), "eval_mle")
            t.observe_(out.reshape(-1))
            values.append(out)
        total = sum(int(pd.columns.shape[0]) for pd in rounds)
        nbv = _ceil_log2(total)
        chal = torch.zeros((max(nbv, 1), 4), dtype=torch.int32, device=dev)
        if nbv:
            chal[:nbv, 0] = t.sample_(nbv)
        n = code.block_len
        mle = torch.empty((S, 4), dtype=torch.int32, device=dev)
        cw = torch.empty((n, 4), dtype=torch.int32, device=dev)
        claim = torch.empty(4, dtype=torch.int32, device=dev)
        off = 0
        for pd, vals in zip(rounds, values):
            w = pd.columns.shape[0]
            acc = int(off > 0)
            _lib.check(L.zc_rlc_columns_ex(f.id, ptr(pd.columns), S, w, ptr(chal), nbv, off, acc,
                                           ptr(mle), st), "rlc mle")
            _lib.check(L.zc_rlc_columns_ex(f.id, ptr(pd.codeword), n, w, ptr(chal), nbv, off, acc,
                                           ptr(cw), st), "rlc codeword")
            _lib.check(L.zc_rlc_values(f.id, ptr(vals), w, ptr(chal), nbv, off, acc, ptr(claim),
                                       st), "rlc values")
            off += w
        nv = torch.zeros(4, dtype=torch.int32, device=dev)
        nv[:1].fill_(f.mont(v))  # a fill kernel: no host copy, capturable
        t.observe_(nv)
        zinv = torch.empty_like(zc)  # 1/z per coordinate, on the device
        _lib.check(L.zc_ef4_inv(f.id, ptr(zc), ptr(zinv), v, st), "ef4_inv")
        eq = torch.empty((max(S // 2, 1), 4), dtype=torch.int32, device=dev)
        nb = L.zc_eq_expand_workspace_bytes(v - 1)
        ews = torch.empty(max((nb + 15) // 4, 4), dtype=torch.int32, device=dev)
        _lib.check(L.zc_eq_expand(f.id, ptr(zc), v - 1, ptr(eq), ptr(ews), nb, st), "eq_expand")
        scb = L.zc_sumcheck_workspace_bytes()
        scws = torch.empty(scb // 4, dtype=torch.int32, device=dev)
        msgs = torch.empty((v, 8), dtype=torch.int32, device=dev)
        rnd = PreFoldPairCommitRound(code, tree, 1)
        layers: list[CommittedLayer] = []
        pending = None
        for i in range(v):
            M = S >> (i + 1)
            _lib.check(L.zc_sumcheck_message(f.id, ptr(mle), M, ptr(eq), ptr(claim),
                                             ptr(zinv[v - 1 - i]), ptr(msgs[i]), ptr(scws), scb,
                                             st), "sumcheck_message")
            t.observe_(msgs[i])
            layer = pending if pending is not None else rnd.commit_layer(cw)
            beta = t.observe_and_sample_(layer.root, 1)
            if i < v - 1 and cw.shape[0] >= 4:
                cw_next, pending = rnd.fold_commit(cw, beta, i)
            else:
                cw_next, pending = code.fold(cw, beta), None
            mle_next = torch.empty((M, 4), dtype=torch.int32, device=dev)
            eq_next = torch.empty((M // 2, 4), dtype=torch.int32, device=dev) if M >= 2 else None
            _lib.check(L.zc_sumcheck_fold(f.id, ptr(mle), M, ptr(beta), 1, ptr(msgs[i]),
                                          ptr(mle_next), ptr(eq) if eq_next is not None else None,
                                          ptr(eq_next) if eq_next is not None else None,
                                          ptr(claim), st), "sumcheck_fold")
            layers.append(layer)
            mle, eq, cw = mle_next, eq_next, cw_next
        final = cw
        positions = t.sample_positions_(n, self.num_queries, values=final)
        comp = [self.open_rows(pd, positions, check=False) for pd in rounds]
        queries = [open_layer(tree, layer, positions) for layer in layers]
        proof = BasefoldProof(msgs, torch.stack([ly.root for ly in layers]), final, comp,
                              queries, positions)
        return values, proof, t

    def commit(self, polys: Sequence[torch.Tensor]):
        return self.commit_columns(torch.stack(list(polys), dim=0))

    def open_rows(self, data: BasefoldProverData, indices: torch.Tensor,
                  check: bool = True) -> Opening:
        K, n = data.codeword.shape
        return self.tree.open_layout(leaves_layout(data.codeword, n, K, 1, n),
                                     data.digest_layers, indices, K, check=check)


class BasefoldVerifier:
    """The native Basefold batch verifier on the host
    (zorch/pcs/basefold/verifier.py:429-540): replays the transcript, checks
    every sumcheck round against the running claim, the final codeword
    against the reduced claim, every Merkle opening against its root, the
    batched component rows against fold layer 0, and the fold chain down to
    the final codeword. Returns a boolean verdict, never raises on a bad proof."""

    def __init__(self, code: ReedSolomon, tree: MerkleTree, num_queries: int = 4) -> None:
        self.code = code
        self.tree = tree
        self.num_queries = num_queries

    def verify(self, claim: OpeningClaim, reduction_proof: OpeningProof, transcript=None):
        """A single-matrix open, the degenerate one-matrix batch
        (zorch/pcs/basefold/verifier.py:99-113): VerifyResult(TrivialClaim(),
        transcript, ok)."""
        ok, t = self.verify_batch([claim.commitment], claim.points, [reduction_proof.values],
                                  reduction_proof.proof, transcript)
        return VerifyResult(TrivialClaim(), t, ok)

    def verify_batch(self, commitments, points, values, proof: BasefoldProof, transcript=None):
        """(ok, transcript) for a batch open at one shared point
        (zorch/pcs/basefold/verifier.py:115-151). `points` is [z] (or z);
        `transcript` the verifier's starting transcript (None: fresh)."""
        if torch.is_tensor(points) or isinstance(points, np.ndarray):
            z = points
        else:
            if len(points) != 1:
                raise ValueError(f"BaseFold opens the matrices at one shared point, got "
                                 f"{len(points)}")
            z = points[0]
        if not (len(commitments) == len(values) == len(proof.component_openings)):
            raise ValueError(f"batch mismatch: {len(commitments)} commitments, {len(values)} "
                             f"value vectors, {len(proof.component_openings)} component openings")
        f, code, tree = self.code.field, self.code, self.tree
        host = lambda x: to_host(x) if torch.is_tensor(x) else np.asarray(x, np.uint32)  # noqa: E731
        ef = lambda words: f.ef_from_mont(words)  # noqa: E731
        zc = [ef(r) for r in host(z).reshape(-1, 4)]
        v = len(zc)
        n = code.block_len
        msgs = host(proof.uni_msgs).reshape(-1, 8)
        roots = host(proof.fri_roots).reshape(-1, 8)
        t = host_transcript(tree.perm, transcript)
        if msgs.shape[0] != v or roots.shape[0] != v or code.message_len != 1 << v:
            return False, t
        for c in commitments:
            t = t.observe(host(c).reshape(-1))
        vals = [host(x).reshape(-1, 4) for x in values]
        for x in vals:
            t = t.observe(x.reshape(-1))
        total = sum(x.shape[0] for x in vals)
        nbv = _ceil_log2(total)
        chal = []
        if nbv:
            t, s = t.sample(nbv)
            chal = [f.canon(int(x)) for x in s]

        def weight(idx: int) -> tuple:
            w = (1, 0, 0, 0)
            for j, r in enumerate(chal):
                bit = (idx >> (nbv - 1 - j)) & 1
                w = f.ef_scale(w, r) if bit else f.ef_scale(w, (1 - r) % f.p)
            return w

        wts = [weight(c) for c in range(total)]
        claim = (0, 0, 0, 0)
        for c, x in enumerate(np.concatenate(vals)):
            claim = f.ef_add(claim, f.ef_mul(wts[c], ef(x)))
        t = t.observe(np.array([f.mont(v), 0, 0, 0], np.uint32))
        ok = True
        betas = []
        for i in range(v):
            s0, s1 = ef(msgs[i, :4]), ef(msgs[i, 4:])
            zl = zc[v - 1 - i]
            one_minus = f.ef_sub((1, 0, 0, 0), zl)
            ok &= claim == f.ef_add(f.ef_mul(one_minus, s0), f.ef_mul(zl, s1))
            t = t.observe(msgs[i])
            t, b = t.observe_and_sample(roots[i], 1)
            beta = f.canon(int(b[0]))
            betas.append(beta)
            claim = f.ef_add(s0, f.ef_scale(s1, beta))
        final = host(proof.final_poly).reshape(-1, 4)
        ok &= final.shape[0] == n >> v and all(ef(x) == claim for x in final)
        t = t.observe(final.reshape(-1))
        t, raw = t.sample(self.num_queries)
        positions = [int(x) % n for x in raw]
        if [int(x) for x in host(proof.positions).view(np.int32)] != positions:
            return False, t
        # Merkle openings
        for pos_i, q in enumerate(positions):
            for r, (c, op) in enumerate(zip(commitments, proof.component_openings)):
                row = Opening(op.row[pos_i], op.path[:, pos_i])
                ok &= tree.verify(c if torch.is_tensor(c) else torch.tensor(c), q, row)
            a = q
            for i, op in enumerate(proof.query_openings):
                a = a % (n >> (i + 1))
                ok &= tree.verify(torch.as_tensor(roots[i].view(np.int32)), a,
                                  Opening(op.row[pos_i], op.path[:, pos_i]))
        if not ok:
            return False, t
        # batched component rows == fold layer 0's leg at the position
        shift = code.coset_shift
        for pos_i, q in enumerate(positions):
            comp = (0, 0, 0, 0)
            off = 0
            for op in proof.component_openings:
                row = host(op.row)[pos_i]
                for c, x in enumerate(row):
                    comp = f.ef_add(comp, f.ef_scale(wts[off + c], f.canon(int(x))))
                off += len(row)
            leaf0 = host(proof.query_openings[0].row)[pos_i].reshape(2, 4)
            a0 = q % (n >> 1)
            ok &= comp == ef(leaf0[0] if q == a0 else leaf0[1])
            # fold chain
            a = q
            for i in range(v):
                ni = n >> i
                a = q % (ni >> 1)
                leaf = host(proof.query_openings[i].row)[pos_i].reshape(2, 4)
                lo, hi = ef(leaf[0]), ef(leaf[1])
                sh = pow(shift, 1 << i, f.p) if shift is not None else 1
                x = sh * pow(f.root_of_unity((ni).bit_length() - 1, code.generator or None), a,
                             f.p) % f.p
                inv2x = pow(2 * x % f.p, f.p - 2, f.p)
                inv2 = pow(2, f.p - 2, f.p)
                folded = f.ef_add(f.ef_scale(f.ef_add(lo, hi), inv2),
                                  f.ef_scale(f.ef_sub(lo, hi), betas[i] * inv2x % f.p))
                if i + 1 < v:
                    a_next = q % (ni >> 2)
                    nxt = host(proof.query_openings[i + 1].row)[pos_i].reshape(2, 4)
                    expected = ef(nxt[0] if a == a_next else nxt[1])
                else:
                    expected = ef(final[a])
                ok &= folded == expected
        return bool(ok), t


class GraphedBasefoldOpen:
    """BasefoldProver.open_batch over fixed committed matrices captured once
    into a CUDA graph: the evaluations, the batching, every sumcheck round with
    its fused fold-and-commit and transcript steps, the query positions and all
    openings replay with one launch. `replay(z, transcript)` copies the point
    and the transcript state into static inputs and returns (values, proof,
    transcript) -- static tensors that the next replay overwrites. The
    matrices' device buffers are baked into the graph: reuse it for as many
    openings of those commitments as needed."""

    def __init__(self, prover: BasefoldProver, rounds: Sequence[BasefoldProverData],
                 device="cuda") -> None:
        self.prover = prover
        self.rounds = list(rounds)
        v = prover.code.message_len.bit_length() - 1
        self.z = torch.zeros((v, 4), dtype=torch.int32, device=device)
        self.state = torch.zeros(_lib.DUPLEX_WORDS, dtype=torch.int32, device=device)
        self._run()  # kernel attributes, allocator warm-up
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.out = self._run()

    def _run(self):
        t = DuplexTranscript(self.prover.tree.perm, self.state)
        return self.prover.open_batch(self.rounds, self.z, t)

    def replay(self, z: torch.Tensor, transcript: DuplexTranscript):
        if z.shape != self.z.shape:
            raise ValueError(f"point shape {tuple(z.shape)} != captured {tuple(self.z.shape)}")
        self.z.copy_(z, non_blocking=True)
        self.state.copy_(transcript.state, non_blocking=True)
        self.graph.replay()
        return self.out


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
        self.coeffs = full_u32(code.message_len, 0, device)
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
