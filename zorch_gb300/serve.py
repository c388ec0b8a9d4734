"""Continuous-batching commit server and the plain per-call path beside it.

Requests (a BabyBear matrix of 2^log_h rows x width columns, a blowup, and
for some a fold-and-open) arrive over time. `Server.run` admits arrived
requests by their HBM footprint against a budget and commits every admitted
request in one batched commit (zorch_gb300.batch) on one of several CUDA
streams, so batches formed while others are still on the GPU overlap on the
device; fold requests then run their fold-and-commit rounds and query
openings on the same stream. A request's codeword and digest layers stay
resident until its openings are taken. Latency = completion - arrival.

Two commitment modes, each with its plain counterpart producing the same
bytes:

- "fri": every column is its own polynomial with its own pair-leaf tree, the
  commitment is the stacked roots -- FriProver.commit
  (zorch/pcs/fri/prover.py:92-99, 141-148). The server commits all columns of
  all admitted requests in one batched LDE and one batched tree commit (a
  tree family per request); `run_plain` makes one call per polynomial
  (FriProver.commit_one).
- "matrix": one row-leaf tree per request, the commitment is its root --
  BasefoldProver.commit (zorch/pcs/basefold/prover.py:437-455). The server
  batches the requests' matrices; `run_plain` makes one commit call per
  request.

A request's result bytes do not depend on what it was batched with or on
which path made them: the tests compare every request served, alone and in
the mix, with the plain path's bytes and with the oracle.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field as dc_field
from typing import Callable

import numpy as np
import torch

from . import _lib
from .batch import BatchCommitter, MatrixJob
from .coding import ReedSolomon
from .commit import DigestLayers, MerkleTree, Opening, Poseidon2, leaves_layout
from .field import (BABYBEAR, full_u32, parts_to_pinned, ptr, stream_handle, to_mont,
                    to_mont_from_host)
from .pcs import BasefoldProver, FriParams, FriProver, pair_layout
from .transcript import DuplexTranscript

MODES = ("fri", "matrix")
# Digest layers of a "fri" request whose trees are not opened are committed in
# column chunks of at most this many bytes (only the roots are kept).
FRI_LAYER_CAP = 16 << 30


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

    def footprint(self, mode: str = "fri") -> int:
        """HBM bytes held while the request is in flight."""
        n = 1 << self.log_n
        b = 4 * self.elements          # input in Montgomery form
        b += 4 * self.width * n         # LDE
        b += min(4 * self.width * n, 1 << 30)  # four-step intermediate share
        if mode == "fri":
            # one pair-leaf tree (n - 1 digests) per column; only opened
            # requests keep every column's tree, the others one chunk's worth
            layers = 32 * self.width * n
            b += layers if self.fold else min(layers, FRI_LAYER_CAP)
        else:
            b += 64 * n                 # one row-leaf tree (2n - 1 digests)
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


def request_work(r: Request, mode: str = "fri") -> int:
    """Poseidon2 permutations of a request's commit and fold-and-open -- the
    hashing that is most of its device time: the cost model of the server's
    admission order and of the calibrated arrival rate."""
    n = 1 << r.log_n
    perms = r.width * (n - 1) if mode == "fri" else n * ((r.width + 7) // 8) + n - 1
    if r.fold:
        perms += n  # the fold layers' pair-leaf trees: n/2 + n/4 + ... leaves and nodes
    return perms


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


def fold_parts(req: Request, cw: torch.Tensor, commitment: torch.Tensor, perm: Poseidon2,
               tree: MerkleTree, open_commitment: Callable[[torch.Tensor], list[Opening]]
               ) -> list[torch.Tensor]:
    """Fold-and-open of a committed request, the Basefold way without the
    sumcheck: observe the commitment (the matrix root, or the stacked column
    roots), batch the columns into one EF4 codeword, observe the fold-round
    count (the domain separation of zorch/pcs/jagged/open.py:262-263), fold
    with EF4 challenges down to 2^8 committing every layer, observe the final
    layer, sample 64 positions, and open the commitment and every fold layer
    there. Returns the proof's parts in wire order: fold roots, final layer,
    positions, the commitment's openings (row, path), the fold layers'
    openings (row, path)."""
    t = DuplexTranscript.new(perm, device=cw.device)
    t.observe_(commitment.reshape(-1))
    rlc = batch_columns(cw, t)
    rounds = max(req.log_n - FOLD_FINAL_LOG, 0)
    # a device fill, not a host->device copy: a pageable copy would block the
    # calling thread until the stream drained
    t.observe_(full_u32(1, BABYBEAR.mont(rounds), cw.device))
    code = ReedSolomon(1 << req.log_h, 1 << req.log_blowup, BABYBEAR, coset_shift=31,
                       generator=31)
    prover = FriProver(FriParams(code, tree, rounds, FOLD_QUERIES, 4))
    proof, _, _ = prover.commit_phase(rlc, t)
    parts = [proof.roots, proof.final_layer, proof.positions]
    for op in open_commitment(proof.positions):
        parts += [op.row, op.path]
    for op in proof.openings:
        parts += [op.row, op.path]
    return parts


def open_matrix(tree: MerkleTree, cw: torch.Tensor, layers: DigestLayers):
    """Opening of a row-leaf matrix commitment at the query positions."""
    w, n = cw.shape
    return lambda pos: [tree.open_layout(leaves_layout(cw, n, w, 1, n), layers, pos, w,
                                         check=False)]


def open_columns(tree: MerkleTree, cw: torch.Tensor, layers: Callable[[int], DigestLayers]):
    """Openings of every column's pair-leaf tree at the query positions mod
    n/2 (each column's layer-0 position, zorch/coding/reed_solomon.py:320-329)."""
    return lambda pos: [tree.open_layout_reduced(pair_layout(cw[c]), layers(c), pos, 2)
                        for c in range(cw.shape[0])]


class _Resident:
    """Committed requests kept on the device until their openings are taken."""

    _table: dict = {}

    @classmethod
    def put(cls, rid: int, obj) -> None:
        cls._table[rid] = obj

    @classmethod
    def drop(cls, rid: int) -> None:
        cls._table.pop(rid, None)


@dataclass
class _Batch:
    reqs: list
    events: list   # one per request: its proof bytes are in `outs` once it fires
    outs: list
    keep: list = dc_field(default_factory=list)
    done: list = dc_field(default_factory=list)


def admit(pending: deque, now: float, in_use: int, budget: float, max_batch: int,
          mode: str = "fri"):
    """Admission rule, FIFO by arrival: take arrived requests while their HBM
    footprint fits the budget, up to max_batch; a request larger than the
    whole budget is rejected. Returns (admitted, rejected, in_use)."""
    ready, rejected = [], []
    while pending and pending[0].arrival <= now and len(ready) < max_batch:
        fp = pending[0].footprint(mode)
        if fp > budget:
            rejected.append(pending.popleft())
            continue
        if in_use + fp > budget:
            break
        in_use += fp
        ready.append(pending.popleft())
    return ready, rejected, in_use


def admit_sjf(pending: deque, now: float, in_use: int, budget: float, max_batch: int,
              mode: str = "fri", max_wait: float = 2.0, class_ratio: float = 8.0):
    """Admission rule, shortest work first within one size class: among the
    arrived requests, those that have waited longer than max_wait go first
    (oldest first), then the rest by ascending work (request_work). The batch
    takes requests in that order whose work is within class_ratio of the
    first one's (so a small request never waits on a large one's batch),
    while their footprints fit the budget, up to max_batch. If the first
    request does not fit, nothing is admitted (a large request that has
    waited is not overtaken forever). A request larger than the whole budget
    is rejected. Returns (admitted, rejected, in_use)."""
    arrived = [r for r in pending if r.arrival <= now]
    rejected = [r for r in arrived if r.footprint(mode) > budget]
    cand = [r for r in arrived if r.footprint(mode) <= budget]
    old = [r for r in cand if now - r.arrival > max_wait]
    young = sorted((r for r in cand if now - r.arrival <= max_wait),
                   key=lambda r: (request_work(r, mode), r.arrival))
    order = old + young
    ready = []
    if order:
        w0 = request_work(order[0], mode)
        for r in order:
            if len(ready) >= max_batch:
                break
            w = request_work(r, mode)
            if ready and not (w0 / class_ratio <= w <= w0 * class_ratio):
                continue
            fp = r.footprint(mode)
            if in_use + fp > budget:
                if not ready:
                    break
                continue
            in_use += fp
            ready.append(r)
    gone = {id(r) for r in ready + rejected}
    keep = [r for r in pending if id(r) not in gone]
    pending.clear()
    pending.extend(keep)
    return ready, rejected, in_use


def _input(r: Request, host_fed: bool) -> torch.Tensor:
    if host_fed:  # the conversion kernel reads the pinned input over the host link
        return to_mont_from_host(BABYBEAR, r.host)
    return to_mont(BABYBEAR, r.resident)


class Server:
    """Continuous batching under an HBM admission budget.

    policy "sjf" (default): admit_sjf -- shortest work first within a size
    class, with an aging bound; batches whose work is at most priority_work
    permutations run on high-priority streams (streams - 1 of them, round
    robin), larger ones in order on one low-priority stream. The batched
    kernels retire their CTAs per work item, so the GPU's block scheduler
    starts a small batch's blocks while a large batch is still running.
    policy "fifo": admit (arrival order), every batch on the streams in turn.
    A request's result is taken as soon as its own bytes are copied back."""

    def __init__(self, budget_bytes: float = 150e9, max_batch: int = 32, streams: int = 3,
                 perm: Poseidon2 | None = None, tuner=None, mode: str = "fri",
                 policy: str = "sjf", priority_work: int = 1 << 25,
                 max_wait: float = 2.0) -> None:
        if mode not in MODES:
            raise ValueError(f"mode must be one of {MODES}, got {mode!r}")
        if policy not in ("sjf", "fifo"):
            raise ValueError(f"policy must be 'sjf' or 'fifo', got {policy!r}")
        self.mode = mode
        self.policy = policy
        self.budget = budget_bytes
        self.max_batch = max_batch
        self.priority_work = priority_work
        self.max_wait = max_wait
        self.perm = perm if perm is not None else Poseidon2.builtin(BABYBEAR)
        self.committer = BatchCommitter(self.perm, BABYBEAR, tuner=tuner)
        self.tree = MerkleTree(self.perm)
        if policy == "sjf":
            # a lower number is a higher priority; out-of-range values are clamped
            self.fast = [torch.cuda.Stream(priority=-10) for _ in range(max(streams - 1, 1))]
            self.slow = [torch.cuda.Stream(priority=0)]
        else:
            self.fast = []
            self.slow = [torch.cuda.Stream() for _ in range(streams)]
        self.batches_launched = 0
        self._rr = 0

    def _stream_for(self, reqs: list[Request]) -> torch.cuda.Stream:
        work = sum(request_work(r, self.mode) for r in reqs)
        pool = self.fast if self.fast and work <= self.priority_work else self.slow
        self._rr += 1
        return pool[self._rr % len(pool)]

    def _launch(self, reqs: list[Request], host_fed: bool, stream: torch.cuda.Stream) -> _Batch:
        with torch.cuda.stream(stream):
            xs = [_input(r, host_fed) for r in reqs]
            jobs = [MatrixJob(x, r.log_blowup, 31) for x, r in zip(xs, reqs)]
            keep = list(xs)
            outs, events = [], []
            if self.mode == "fri":
                committed = self.committer.commit_polys(jobs, [r.fold for r in reqs],
                                                        FRI_LAYER_CAP)
            else:
                committed = self.committer.commit(jobs)
            for r, c in zip(reqs, committed):
                _Resident.put(r.rid, c)
                if self.mode == "fri":
                    commitment = c.roots
                    opener = open_columns(self.tree, c.codeword, c.layers)
                else:
                    commitment = c.root
                    opener = open_matrix(self.tree, c.codeword, c.layers)
                parts = [commitment]
                if r.fold:
                    parts += fold_parts(r, c.codeword, commitment, self.perm, self.tree, opener)
                outs.append(parts_to_pinned(parts))
                ev = torch.cuda.Event()
                ev.record(stream)
                events.append(ev)
                keep += [c, parts]
        self.batches_launched += 1
        return _Batch(reqs, events, outs, keep, [False] * len(reqs))

    def run(self, requests: list[Request], host_fed: bool = False) -> list[Result]:
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        inflight: deque[_Batch] = deque()
        results: list[Result] = []
        in_use = 0
        t0 = time.perf_counter()
        while pending or inflight:
            now = time.perf_counter() - t0
            # retire each request as soon as its own bytes are back
            still = deque()
            for b in inflight:
                for i, (r, host, ev) in enumerate(zip(b.reqs, b.outs, b.events)):
                    if not b.done[i] and ev.query():
                        b.done[i] = True
                        words = host.numpy().view(np.uint32)
                        results.append(Result(r.rid, words[:8].copy(), words.tobytes(),
                                              r.arrival, time.perf_counter() - t0))
                        in_use -= r.footprint(self.mode)
                        _Resident.drop(r.rid)
                if not all(b.done):
                    still.append(b)
            inflight = still
            # admit arrived requests that fit the budget
            if self.policy == "sjf":
                ready, rejected, in_use = admit_sjf(pending, now, in_use, self.budget,
                                                    self.max_batch, self.mode, self.max_wait)
            else:
                ready, rejected, in_use = admit(pending, now, in_use, self.budget,
                                                self.max_batch, self.mode)
            for r in rejected:
                results.append(Result(r.rid, np.zeros(8, np.uint32), b"", r.arrival, now))
            if ready:
                inflight.append(self._launch(ready, host_fed, self._stream_for(ready)))
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


def plain_request(r: Request, x: torch.Tensor, perm: Poseidon2, tree: MerkleTree,
                  mode: str = "fri") -> list[torch.Tensor]:
    """One request through the drop-in API, one commit call per polynomial
    ("fri": FriProver.commit_one per column, roots stacked) or per matrix
    ("matrix": BasefoldProver.commit); returns the proof parts."""
    code = ReedSolomon(1 << r.log_h, 1 << r.log_blowup, BABYBEAR, coset_shift=31, generator=31)
    if mode == "fri":
        prover = FriProver(FriParams(code, tree, 0, 0))
        cw = torch.empty((r.width, 1 << r.log_n), dtype=torch.int32, device=x.device)
        commitment = torch.empty((r.width, 8), dtype=torch.int32, device=x.device)
        kept = []  # digest layers are kept only when the request opens them
        for c in range(r.width):
            cp = prover.commit_one(x[c], out=cw[c])
            commitment[c].copy_(cp.root)
            if r.fold:
                kept.append(cp.digest_layers)
        opener = open_columns(tree, cw, lambda c: kept[c])
    else:
        root, data = BasefoldProver(code, tree).commit_columns(x)
        cw, commitment = data.codeword, root
        opener = open_matrix(tree, cw, data.digest_layers)
    parts = [commitment]
    if r.fold:
        parts += fold_parts(r, cw, commitment, perm, tree, opener)
    return parts


def run_plain(requests: list[Request], host_fed: bool = False,
              perm: Poseidon2 | None = None, mode: str = "fri",
              budget_bytes: float = 150e9) -> list[Result]:
    """One request at a time, as arrivals allow, through the drop-in API
    (plain_request); a request's result is read back (a host
    synchronisation) before the next one starts. A request whose footprint
    exceeds the budget is rejected (empty result), as the server does."""
    if mode not in MODES:
        raise ValueError(f"mode must be one of {MODES}, got {mode!r}")
    perm = perm if perm is not None else Poseidon2.builtin(BABYBEAR)
    tree = MerkleTree(perm)
    results = []
    t0 = time.perf_counter()
    for r in sorted(requests, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        if r.footprint(mode) > budget_bytes:
            results.append(Result(r.rid, np.zeros(8, np.uint32), b"", r.arrival,
                                  time.perf_counter() - t0))
            continue
        parts = plain_request(r, _input(r, host_fed), perm, tree, mode)
        host = parts_to_pinned(parts)
        torch.cuda.current_stream().synchronize()
        words = host.numpy().view(np.uint32)
        results.append(Result(r.rid, words[:8].copy(), words.tobytes(), r.arrival,
                              time.perf_counter() - t0))
    return results
