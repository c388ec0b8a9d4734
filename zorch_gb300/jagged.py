"""The commit-and-fold half of SP1's stacked BaseFold open on the GPU
(drop-in for the fold loop and query openings of zorch/pcs/jagged/open.py:237-330).

Each round's layer is a bit-reversed EF4 codeword [n, 4]; it is committed as
its [n/2, 8] base-limb rows (the adjacent conjugate pair of a fold is one row)
through the SP1 single-matrix commitment, whose separator-bound root the
transcript observes, and folded by BitReversedReedSolomon.fold. Round r+1's
commit runs in the same kernel as round r's fold (zc_fri_fold_commit_bitrev),
and every root is bound on the device, so the loop never synchronises with
the host. The interleaved sumcheck message of the reference loop (:266-276) is
not on this path: the caller supplies each round's beta (the reference's
byte-match replays them the same way, zorch/pcs/jagged/testing/open_test.py:90-128).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Sequence

import torch

from . import _lib
from .coding import BitReversedReedSolomon
from .commit import DigestLayers, SingleMatrixCommitmentScheme, leaves_layout
from .field import from_mont, ptr, stream_handle
from .transcript import DuplexTranscript


@dataclass
class StackedFoldLayer:
    """One committed fold layer: the codeword [n, 4], its digest layers over
    the [n/2, 8] pair rows, and the raw and separator-bound roots."""

    codeword: torch.Tensor
    digest_layers: DigestLayers
    raw_root: torch.Tensor
    bound_root: torch.Tensor

    @property
    def leaves(self) -> torch.Tensor:
        """The committed [n/2, 8] rows, a view of the codeword."""
        return self.codeword.reshape(self.codeword.shape[0] // 2, 8)


def sample_query_positions(t: DuplexTranscript, block_len: int, num_queries: int):
    """SP1's sample_bits rule (zorch/pcs/jagged/open.py:116-125): one squeeze
    per query, the CANONICAL value masked to log2(block_len) low bits."""
    if block_len <= 0 or block_len & (block_len - 1):
        raise ValueError(f"block_len must be a power of two, got {block_len}")
    t2, raw = t.sample(num_queries)
    canon = from_mont(t.field, raw)
    return t2, canon & (block_len - 1)


class StackedFoldCommit:
    """Commit -> bind -> fold rounds over a bit-reversed EF4 codeword."""

    def __init__(self, smcs: SingleMatrixCommitmentScheme, code: BitReversedReedSolomon) -> None:
        self.smcs = smcs
        self.code = code

    def commit_layer(self, cw: torch.Tensor) -> StackedFoldLayer:
        """smcs.commit(bitcast(cw).reshape(n/2, 8)) (zorch/pcs/jagged/open.py:278-282)."""
        n = cw.shape[0]
        if cw.dim() != 2 or cw.shape[1] != 4 or n < 2:
            raise ValueError("a stacked fold layer is an EF4 codeword [n >= 2, 4]")
        rows = cw.contiguous()
        bound, layers = self.smcs.commit_layout(leaves_layout(rows, n // 2, 1, 8, 0), 8)
        return StackedFoldLayer(rows, layers, layers.root, bound)

    def fold_commit(self, cw: torch.Tensor, beta: torch.Tensor,
                    level: int) -> tuple[torch.Tensor, StackedFoldLayer | None]:
        """Fold layer `cw` by `beta`; when the folded layer has >= 2 elements its
        commit runs fused with the fold (n >= 4)."""
        n = cw.shape[0]
        out = torch.empty((n // 2, 4), dtype=torch.int32, device=cw.device)
        if n < 4:
            return self.code.fold(cw, beta, out), None
        L = n // 4
        flat = torch.empty((2 * L - 1, 8), dtype=torch.int32, device=cw.device)
        _lib.check(_lib.lib().zc_fri_fold_commit_bitrev(
            self.smcs.perm.handle, ptr(cw), n, 1, ptr(beta.contiguous()), int(beta.numel() == 4),
            self.code.level_shift_mont(level), 0, ptr(out), ptr(flat), stream_handle()),
            "fri_fold_commit_bitrev")
        layers = DigestLayers(flat, L)
        bound = self.smcs.bind_root(layers.root, (L).bit_length() - 1, 8)
        return out, StackedFoldLayer(out, layers, layers.root, bound)

    def run(self, codeword: torch.Tensor, num_rounds: int,
            next_beta: Callable[[int, StackedFoldLayer], torch.Tensor]
            ) -> tuple[list[StackedFoldLayer], torch.Tensor]:
        """`num_rounds` commit-and-fold rounds; `next_beta(r, layer)` returns round
        r's EF4 beta (4 device words) after the layer is committed -- e.g. an
        observe of the bound root and a 4-squeeze challenge, or a replay.
        Returns the committed layers and the final folded codeword."""
        if num_rounds < 0 or (1 << num_rounds) > codeword.shape[0]:
            raise ValueError("more fold rounds than the codeword has halvings")
        cw = codeword
        layers: list[StackedFoldLayer] = []
        pending = None
        for r in range(num_rounds):
            layer = pending if pending is not None else self.commit_layer(cw)
            layers.append(layer)
            beta = next_beta(r, layer)
            cw, pending = self.fold_commit(cw, beta, self.code.level_of(cw.shape[0]))
        return layers, cw

    def run_replay(self, codeword: torch.Tensor, betas: Sequence[torch.Tensor] | torch.Tensor):
        """run() with the betas given up front ([R, 4] device words)."""
        return self.run(codeword, len(betas), lambda r, _layer: betas[r])

    def open_layers(self, layers: Sequence[StackedFoldLayer], positions: torch.Tensor):
        """Each layer's pair row opened at the halved positions a_i = q >> (i+1)
        (BitReversedReedSolomon.layer_positions; zorch/pcs/jagged/open.py:313-317):
        a list of (rows [Q, 8], proofs [depth_i, Q, 8])."""
        idx = self.code.layer_positions(positions.to(torch.int32), len(layers))
        return [self.smcs.open_batch(i, layer.leaves, layer.digest_layers)
                for i, layer in zip(idx, layers)]
