"""Continuous-batching commit server and the plain per-polynomial path beside it.

Requests (a BabyBear matrix of 2^log_h rows x width columns, a blowup, and
for some a fold-and-open) arrive over time. `Server.run` admits arrived
requests by their HBM footprint against a budget, batches every admitted
request into one batched LDE + batched Merkle commit (zorch_gb300.batch) on
one of several CUDA streams, so batches formed while others are still on the
GPU overlap on the device; fold requests then run their fold-and-commit
rounds and query openings on the same stream. A request's codeword and
digest layers stay resident until its openings are taken. Latency =
completion time - arrival time.

`run_plain` serves the same stream one request at a time through the
drop-in API with one call per polynomial (FriProver.commit, zorch/pcs/fri/
prover.py:92-99: encode one column, commit its pair-leaf tree) and a host
synchronisation per call, as the reference's eager loop does.

A request's result bytes do not depend on what it was batched with; the
tests check each one alone and in the mix.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field as dc_field

import numpy as np
import torch

from . import _lib
from .batch import BatchCommitter, MatrixJob
from .coding import ReedSolomon
from .commit import MerkleTree, Poseidon2, leaves_layout
from .field import BABYBEAR, ptr, stream_handle, to_mont, to_mont_from_host
from .pcs import FriParams, FriProver
from .transcript import DuplexTranscript


@dataclass
class Request:
    rid: int
    arrival: float  # seconds after stream start
    log_h: int
    width: int
    log_blowup: int
    fold: bool
    seed: int
    host: torch.Tensor | None = None      # pinned canonical [w, h] (host-fed runs)
    resident: torch.Tensor | None = None  # device canonical [w, h] (HBM-resident runs)

    @property
    def elements(self) -> int:
        return self.width << self.log_h

    @property
    def log_n(self) -> int:
        return self.log_h + self.log_blowup

    def footprint(self) -> int:
        """HBM bytes held while the request is in flight."""
        n = 1 << self.log_n
        b = 4 * self.elements          # input (converted to Montgomery in place)
        b += 4 * self.width * n         # LDE
        b += min(4 * self.width * n, 1 << 30)  # four-step intermediate share
        b += 64 * n                     # digest layers (2n - 1 digests of 32 B)
        if self.fold:
            b += 16 * n + 48 * n        # RLC codeword + fold layers and their trees
        return b


@dataclass
class Result:
    rid: int
    root: np.ndarray
    proof: bytes = b""
    arrival: float = 0.0
    done: float = 0.0

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def make_stream(n: int, seed: int, rate_hz: float, *, log_h=(14, 24), log_w=(0.0, 8.0),
                log_blowups=(1, 2), fold_frac: float = 0.3) -> list[Request]:
    """Config-5 style stream: Poisson arrivals at rate_hz; log2 height uniform
    over the integers in log_h; width = max(1, round(2^u)), u ~ U(log_w);
    blowup 2 or 4; fold_frac of the requests fold and open."""
    rng = np.random.default_rng(seed)
    hs = rng.integers(log_h[0], log_h[1] + 1, size=n)
    ws = np.maximum(1, np.rint(2.0 ** rng.uniform(log_w[0], log_w[1], size=n))).astype(int)
    bs = rng.choice(np.asarray(log_blowups), size=n)
    folds = rng.random(n) < fold_frac
    arrivals = np.cumsum(rng.exponential(1.0 / rate_hz, size=n)) if rate_hz > 0 else np.zeros(n)
    return [Request(i, float(arrivals[i]), int(hs[i]), int(ws[i]), int(bs[i]), bool(folds[i]),
                    int(seed * 1000003 + i)) for i in range(n)]


def fill_request(req: Request, device="cuda", pinned: bool = False) -> None:
    """Seeded synthetic canonical data for the request (device fill; copied to
    pinned host memory when `pinned`)."""
    x = torch.empty((req.width, 1 << req.log_h), dtype=torch.int32, device=device)
    _lib.check(_lib.lib().zc_fill_uniform(BABYBEAR.id, ptr(x), x.numel(), req.seed,
                                          stream_handle()), "fill_uniform")
    if pinned:
        req.host = x.cpu().pin_memory()
    else:
        req.resident = x


FOLD_FINAL_LOG = 8
FOLD_QUERIES = 64


def batch_columns(cw: torch.Tensor, t: DuplexTranscript) -> torch.Tensor:
    """Draw ceil(log2 w) EF4 challenges (sample_challenge, 4 squeezes each) and
    combine the columns with their partial-Lagrange weights (zc_rlc_columns):
    the single-round case of sample_rlc_coeffs_bits + batch_staggered
    (zorch/pcs/jagged/open.py:88-105, zorch/pcs/basefold/batching.py:66-80)."""
    w, n = cw.shape
    nbv = (w - 1).bit_length()
    chal = t.sample_(4 * nbv) if nbv else None
    out = torch.empty((n, 4), dtype=torch.int32, device=cw.device)
    _lib.check(_lib.lib().zc_rlc_columns(BABYBEAR.id, ptr(cw), n, w, ptr(chal), ptr(out),
                                         stream_handle()), "rlc_columns")
    return out


def fold_and_open(req: Request, cw: torch.Tensor, root: torch.Tensor, perm: Poseidon2,
                  tree: MerkleTree, layers=None) -> tuple:
    """Open a committed matrix the Basefold way without the sumcheck: observe
    the root, batch the columns into one EF4 codeword, observe the fold-round
    count (the domain separation of zorch/pcs/jagged/open.py:262-263), fold
    with EF4 challenges down to 2^8 committing every layer, observe the final
    layer, sample 64 positions, and open the matrix rows and every fold layer
    there."""
    n = cw.shape[1]
    t = DuplexTranscript.new(perm, device=cw.device)
    t.observe_(root)
    rlc = batch_columns(cw, t)
    rounds = max(req.log_n - FOLD_FINAL_LOG, 0)
    # a fill kernel, not a host->device copy: the copy would block this thread
    # until the batch's stream drained
    t.observe_(torch.full((1,), BABYBEAR.mont(rounds), dtype=torch.int32, device=cw.device))
    code = ReedSolomon(1 << req.log_h, 1 << req.log_blowup, BABYBEAR, coset_shift=31,
                       generator=31)
    prover = FriProver(FriParams(code, tree, rounds, FOLD_QUERIES, 4))
    proof, t, _ = prover.commit_phase(rlc, t)
    layers = layers if layers is not None else _ResidentLayers.get(req.rid)
    # positions are drawn below n on the device: no range read-back (a sync)
    rows = tree.open_layout(leaves_layout(cw, n, cw.shape[0], 1, n), layers, proof.positions,
                            cw.shape[0], check=False)
    return proof, rows


class _ResidentLayers:
    """Digest layers of committed matrices kept on the device until opened."""

    _table: dict = {}

    @classmethod
    def put(cls, rid: int, layers) -> None:
        cls._table[rid] = layers

    @classmethod
    def get(cls, rid: int):
        return cls._table[rid]

    @classmethod
    def drop(cls, rid: int) -> None:
        cls._table.pop(rid, None)


def _proof_bytes(root: torch.Tensor, proof, rows) -> torch.Tensor:
    parts = [root.reshape(-1)]
    if proof is not None:
        parts += [proof.roots.reshape(-1), proof.final_layer.reshape(-1),
                  proof.positions.reshape(-1), rows.row.reshape(-1), rows.path.reshape(-1)]
        for op in proof.openings:
            parts += [op.row.reshape(-1), op.path.reshape(-1)]
    return torch.cat(parts)


@dataclass
class _Batch:
    reqs: list
    event: torch.cuda.Event
    outs: list
    keep: list = dc_field(default_factory=list)


def admit(pending: deque, now: float, in_use: int, budget: float, max_batch: int):
    """Admission rule, FIFO by arrival: take arrived requests while their HBM
    footprint fits the budget, up to max_batch; a request larger than the
    whole budget is rejected. Returns (admitted, rejected, in_use)."""
    ready, rejected = [], []
    while pending and pending[0].arrival <= now and len(ready) < max_batch:
        fp = pending[0].footprint()
        if fp > budget:
            rejected.append(pending.popleft())
            continue
        if in_use + fp > budget:
            break
        in_use += fp
        ready.append(pending.popleft())
    return ready, rejected, in_use


class Server:
    """Continuous batching under an HBM admission budget."""

    def __init__(self, budget_bytes: float = 150e9, max_batch: int = 32, streams: int = 3,
                 perm: Poseidon2 | None = None, tuner=None) -> None:
        self.budget = budget_bytes
        self.max_batch = max_batch
        self.perm = perm if perm is not None else Poseidon2.builtin(BABYBEAR)
        self.committer = BatchCommitter(self.perm, BABYBEAR, tuner=tuner)
        self.tree = MerkleTree(self.perm)
        self.streams = [torch.cuda.Stream() for _ in range(streams)]
        self.batches_launched = 0

    def _launch(self, reqs: list[Request], host_fed: bool, stream: torch.cuda.Stream) -> _Batch:
        with torch.cuda.stream(stream):
            jobs, keep = [], []
            for r in reqs:
                if host_fed:  # read the pinned input over the host link
                    x = to_mont_from_host(BABYBEAR, r.host)
                else:
                    x = to_mont(BABYBEAR, r.resident)
                jobs.append(MatrixJob(x, r.log_blowup, 31))
                keep.append(x)
            committed = self.committer.commit(jobs)
            outs = []
            for r, c in zip(reqs, committed):
                _ResidentLayers.put(r.rid, c.layers)
                proof = rows = None
                if r.fold:
                    proof, rows = fold_and_open(r, c.codeword, c.root, self.perm, self.tree)
                flat = _proof_bytes(c.root, proof, rows)
                host = torch.empty(flat.shape, dtype=flat.dtype, pin_memory=True)
                host.copy_(flat, non_blocking=True)
                outs.append(host)
                keep += [c, flat]
            ev = torch.cuda.Event()
            ev.record(stream)
        self.batches_launched += 1
        return _Batch(reqs, ev, outs, keep)

    def run(self, requests: list[Request], host_fed: bool = False) -> list[Result]:
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        inflight: deque[_Batch] = deque()
        results: list[Result] = []
        in_use = 0
        si = 0
        t0 = time.perf_counter()
        while pending or inflight:
            now = time.perf_counter() - t0
            # retire finished batches (in launch order per stream is not required)
            still = deque()
            for b in inflight:
                if b.event.query():
                    done = time.perf_counter() - t0
                    for r, host in zip(b.reqs, b.outs):
                        words = host.numpy().view(np.uint32)
                        results.append(Result(r.rid, words[:8].copy(), words.tobytes(),
                                              r.arrival, done))
                        in_use -= r.footprint()
                        _ResidentLayers.drop(r.rid)
                else:
                    still.append(b)
            inflight = still
            # admit arrived requests that fit the budget
            ready, rejected, in_use = admit(pending, now, in_use, self.budget, self.max_batch)
            for r in rejected:
                results.append(Result(r.rid, np.zeros(8, np.uint32), b"", r.arrival, now))
            if ready:
                inflight.append(self._launch(ready, host_fed, self.streams[si % len(self.streams)]))
                si += 1
                continue
            if inflight:
                # blocked by the budget / batch size, or waiting for the next arrival:
                # poll completions at a short interval
                wait = 5e-5
                if pending and pending[0].arrival > now:
                    wait = min(wait, pending[0].arrival - now)
                time.sleep(max(wait, 0.0))
            elif pending:
                time.sleep(max(0.0, min(pending[0].arrival - now, 0.01)))
        return sorted(results, key=lambda r: r.rid)


def run_plain(requests: list[Request], host_fed: bool = False,
              perm: Poseidon2 | None = None) -> list[Result]:
    """One request at a time, one call per polynomial (FriProver.commit), a
    host synchronisation per call; fold requests run the same fold-and-open as
    the server on their batched columns."""
    perm = perm if perm is not None else Poseidon2.builtin(BABYBEAR)
    tree = MerkleTree(perm)
    results = []
    t0 = time.perf_counter()
    for r in sorted(requests, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        if host_fed:
            x = to_mont_from_host(BABYBEAR, r.host)
        else:
            x = to_mont(BABYBEAR, r.resident)
        code = ReedSolomon(1 << r.log_h, 1 << r.log_blowup, BABYBEAR, coset_shift=31,
                           generator=31)
        prover = FriProver(FriParams(code, tree, 0, 0))
        n = 1 << r.log_n
        cw = torch.empty((r.width, n), dtype=torch.int32, device=x.device)
        roots = []
        for c in range(r.width):
            cp = prover.commit_one(x[c], out=cw[c])
            roots.append(cp.root)
            torch.cuda.synchronize()
        stacked = torch.stack(roots)
        parts = [stacked.reshape(-1)]
        if r.fold:
            t = DuplexTranscript.new(perm, device=x.device)
            t.observe_(stacked)
            rlc = batch_columns(cw, t)
            rounds = max(r.log_n - FOLD_FINAL_LOG, 0)
            t.observe_(torch.tensor([BABYBEAR.mont(rounds)], dtype=torch.int32, device=x.device))
            fri = FriProver(FriParams(code, tree, rounds, FOLD_QUERIES, 4))
            proof, t, _ = fri.commit_phase(rlc, t)
            parts += [proof.roots.reshape(-1), proof.final_layer.reshape(-1),
                      proof.positions.reshape(-1)]
            for op in proof.openings:
                parts += [op.row.reshape(-1), op.path.reshape(-1)]
        words = torch.cat(parts).cpu().numpy().view(np.uint32)
        results.append(Result(r.rid, words[:8].copy(), words.tobytes(), r.arrival,
                              time.perf_counter() - t0))
    return results
