"""The claim-reduction seam the PCS provers sit behind (drop-in for
zorch/stage.py:31-103 and zorch/pcs/stage.py:28-81).

A stage's prover returns `ProveResult(reduced_claim, reduction_proof,
transcript)` and its verifier `VerifyResult(reduced_claim, transcript, ok)`.
An opening is terminal: it reduces its claim to `TrivialClaim()`. The PCS
seam is a committer (`commit(polys) -> (commitment, prover_data)`) plus that
terminal stage, whose claim names the commitment and the points
(`OpeningClaim`), whose witness is the prover data (`OpeningWitness`) and
whose reduction proof is `OpeningProof(values, proof)`.

The roles are structural protocols, as in the reference: a class conforms by
shape; subclassing one makes a missing role method fail at construction.
"""

from __future__ import annotations

from abc import abstractmethod
from dataclasses import dataclass
from typing import Any, Generic, Protocol, Sequence, TypeVar

Claim = TypeVar("Claim")
ReducedClaim = TypeVar("ReducedClaim")
ReductionProof = TypeVar("ReductionProof")
TranscriptT = TypeVar("TranscriptT")
Commitment = TypeVar("Commitment")
ProverData = TypeVar("ProverData")
Proof = TypeVar("Proof")

Claim_contra = TypeVar("Claim_contra", contravariant=True)
Witness_contra = TypeVar("Witness_contra", contravariant=True)
ReductionProof_contra = TypeVar("ReductionProof_contra", contravariant=True)
C_co = TypeVar("C_co", covariant=True)
D_co = TypeVar("D_co", covariant=True)


@dataclass(frozen=True)
class TrivialClaim:
    """The claim that holds by construction (zorch/stage.py:31-38)."""


@dataclass(frozen=True)
class ProveResult(Generic[ReducedClaim, ReductionProof, TranscriptT]):
    """A reduced claim, its reduction proof and the advanced transcript."""

    reduced_claim: ReducedClaim
    reduction_proof: ReductionProof
    transcript: TranscriptT


@dataclass(frozen=True)
class VerifyResult(Generic[ReducedClaim, TranscriptT]):
    """The verifier-derived reduced claim, the advanced transcript and the
    verdict (a boolean; a bad proof is a False verdict, not an exception)."""

    reduced_claim: ReducedClaim
    transcript: TranscriptT
    ok: Any


class ProverStage(Protocol[Claim_contra, Witness_contra, ReducedClaim, ReductionProof,
                           TranscriptT]):
    """The prover role of one claim reduction (zorch/stage.py:66-81)."""

    @abstractmethod
    def prove(self, claim: Claim_contra, witness: Witness_contra,
              transcript: TranscriptT) -> ProveResult[ReducedClaim, ReductionProof,
                                                      TranscriptT]: ...


class VerifierStage(Protocol[Claim_contra, ReducedClaim, ReductionProof_contra, TranscriptT]):
    """The verifier role of the same reduction (zorch/stage.py:84-103)."""

    @abstractmethod
    def verify(self, claim: Claim_contra, reduction_proof: ReductionProof_contra,
               transcript: TranscriptT) -> VerifyResult[ReducedClaim, TranscriptT]: ...


class Committer(Protocol[C_co, D_co]):
    """Binds to a batch of polynomials (zorch/pcs/stage.py:28-35)."""

    def commit(self, polys: Sequence[Any]) -> tuple[C_co, D_co]: ...


@dataclass(frozen=True)
class OpeningClaim(Generic[Commitment]):
    """The committed polynomials evaluate at `points` (zorch/pcs/stage.py:38-48);
    the values are the prover's to compute."""

    commitment: Commitment
    points: Sequence[Any]


@dataclass(frozen=True)
class OpeningWitness(Generic[ProverData]):
    """The prover data `commit` retained (zorch/pcs/stage.py:51-55)."""

    prover_data: ProverData


@dataclass(frozen=True)
class OpeningProof(Generic[Proof]):
    """The claimed evaluations and the scheme's opening proof
    (zorch/pcs/stage.py:76-81)."""

    values: Any
    proof: Proof
