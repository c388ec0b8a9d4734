#!/usr/bin/env python
"""Benchmark of the polynomial-commitment hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl zorch|reference]
                    [--workload trace|served]

Prints ONE JSON line (rank 0). Workloads (seeded synthetic BabyBear data,
uniform in [0, p), canonical form converted to Montgomery inside each step):

- trace:  a 2^20 x 64 matrix, every column coset-LDE'd at blowup 4 (shift 31,
          generator 31) to 2^22 x 64, row leaves hashed (Poseidon2-16 sponge,
          64 elements per leaf), binary compression to one root, then 128
          seeded query openings (row + authentication path).
- served: the continuous-batching commit stream (see zorch_gb300/serve.py).

value = input field elements committed per second with inputs resident in
HBM; e2e = the same through the public API from pinned host buffers with the
host<->device copies inside the timed region. --impl reference times the
reference algorithm's CPU restatement (the oracle; the reference itself is
Python over FRX wheels absent from this image) on the host cores.
Multi-GPU: replicas only (each rank runs the same workload; no collective).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

P = 2013265921
METRIC = "field elements committed/s (batched/served vs plain GPU path)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["zorch", "reference"], default="zorch")
    ap.add_argument("--workload", choices=["trace", "served", "fri", "uneven", "paths"],
                    default="served")
    ap.add_argument("--log-rows", type=int, default=20)
    ap.add_argument("--cols", type=int, default=64)
    ap.add_argument("--log-blowup", type=int, default=2)
    ap.add_argument("--queries", type=int, default=128)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--requests", type=int, default=24)
    ap.add_argument("--rate", type=float, default=400.0, help="served stream arrivals per second")
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--min-log-h", type=int, default=14)
    ap.add_argument("--max-log-h", type=int, default=24)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--max-batch", type=int, default=8)
    ap.add_argument("--streams", type=int, default=4)
    ap.add_argument("--cal-requests", type=int, default=200,
                    help="requests of the calibrated-rate served stream")
    return ap.parse_args()


def make_stream_for(args):
    from zorch_gb300.serve import make_stream

    return make_stream(args.requests, args.seed, rate_hz=args.rate,
                       log_h=(args.min_log_h, args.max_log_h))


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, device=None) -> float:
    """The slowest rank's time (replicas: every rank times the same work)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------- clocks -----
class Clocks:
    """nvidia-smi sampling during the timed region (reads only)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int) -> None:
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0) for r in rows)}


# ------------------------------------------------------- CPU baseline -----
def cpu_trace_sample(log_rows, cols, log_blowup, queries, threads=0, reps=1):
    """The oracle (C restatement, OpenMP) on a bounded slice of the trace
    workload: encode + row-leaf Merkle commit + openings."""
    from oracle import oracle as orc

    if threads:
        orc.set_threads(threads)
    rng = np.random.default_rng(7)
    x = rng.integers(0, P, size=(cols, 1 << log_rows), dtype=np.uint64).astype(np.uint32)
    p2 = orc.Poseidon2.babybear16()
    shift = orc.to_mont(0, np.array([31], np.uint32))[0]
    idx = rng.integers(0, 1 << (log_rows + log_blowup), size=queries).astype(np.int32)
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        xm = orc.to_mont(0, x)
        cw = orc.rs_encode(0, xm, log_blowup, int(shift))
        layers = orc.merkle_commit_columns(p2, cw)
        orc.merkle_open(cw, cw.shape[1], cols, 1, cw.shape[1], layers, idx)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return (cols << log_rows) / best, best, orc.threads()


# Height cap of the CPU samples of the served stream (per-polynomial pair-leaf
# commitments): the cpu_baseline leg passes the 24-request stream once at
# 2^16 rows; each step of the reference arm at 2^14 rows (a few seconds on 16
# Arm cores), so that a 20-step run ends within a few minutes.
CPU_CAP_LOG_H = 16
REF_CAP_LOG_H = 14


def cpu_served_sample(args, cap_log_h=CPU_CAP_LOG_H, mode="fri"):
    """The oracle on a bounded sample of the served stream: every request of
    the seeded stream with its height capped at 2^cap_log_h rows -- LDE, the
    commitment ("fri": every column's pair-leaf tree, "matrix": one row-leaf
    tree), and for fold requests the partial-Lagrange batching, EF4 fold
    rounds to 2^8 and 64 query openings of the commitment and every layer."""
    from oracle import oracle as orc
    from zorch_gb300.serve import FOLD_FINAL_LOG, FOLD_QUERIES, make_stream

    reqs = make_stream(args.requests, args.seed, rate_hz=args.rate,
                       log_h=(args.min_log_h, args.max_log_h))
    p2 = orc.Poseidon2.babybear16()
    shift = int(orc.to_mont(0, np.array([31], np.uint32))[0])
    rng = np.random.default_rng(11)
    elements = 0
    t0 = time.perf_counter()
    for r in reqs:
        lh = min(r.log_h, cap_log_h)
        x = rng.integers(0, P, size=(r.width, 1 << lh), dtype=np.uint64).astype(np.uint32)
        cw = orc.rs_encode(0, orc.to_mont(0, x), r.log_blowup, shift)
        w, n = cw.shape
        if mode == "fri":
            L = n // 2
            col_layers = [orc.merkle_commit(p2, cw[c], L, 2, 1, L) for c in range(w)]
            commitment = np.concatenate([ly[-1][0] for ly in col_layers])
        else:
            layers = orc.merkle_commit_columns(p2, cw)
            commitment = layers[-1][0]
        elements += r.width << lh
        if r.fold:
            t = orc.Transcript(p2)
            t.observe(commitment)
            nbv = (r.width - 1).bit_length()
            rlc = orc.rlc_columns(0, cw, t.sample(4 * nbv) if nbv else [])
            rounds = max(lh + r.log_blowup - FOLD_FINAL_LOG, 0)
            t.observe(orc.to_mont(0, np.array([rounds], np.uint32)))
            if rounds:
                proof = orc.fri_commit_phase(p2, 0, rlc, rounds, FOLD_QUERIES, 4, t, shift)
                if mode == "fri":
                    a = (proof.positions.astype(np.int64) % L).astype(np.int32)
                    for c in range(w):
                        orc.merkle_open(cw[c], L, 2, 1, L, col_layers[c], a)
                else:
                    orc.merkle_open(cw, n, w, 1, n, layers, proof.positions)
    dt = time.perf_counter() - t0
    return elements / dt, dt, orc.threads(), elements


# ---------------------------------------------------------- workloads -----
def trace_workload(args, device):
    import torch

    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2
    from zorch_gb300.field import BABYBEAR, to_mont, to_mont_from_host
    from zorch_gb300.pcs import BasefoldProver

    rows, cols = 1 << args.log_rows, args.cols
    perm = Poseidon2.builtin(BABYBEAR)
    code = ReedSolomon(rows, 1 << args.log_blowup, BABYBEAR, coset_shift=31, generator=31)
    prover = BasefoldProver(code, MerkleTree(perm, column_major=True), args.queries)
    rng = np.random.default_rng(20240601)
    host = rng.integers(0, P, size=(cols, rows), dtype=np.uint64).astype(np.uint32).view(np.int32)
    pinned = torch.from_numpy(host).pin_memory()
    canon = pinned.to(device)
    xm = torch.empty_like(canon)
    n = rows << args.log_blowup
    idx = torch.from_numpy(rng.integers(0, n, size=args.queries).astype(np.int32)).to(device)
    stream = torch.cuda.current_stream()
    ev = {}

    def step(e2e=False, timing=None):
        if timing is not None:
            timing[0].record(stream)
        if e2e:  # the conversion kernel reads the pinned input over the host link
            to_mont_from_host(BABYBEAR, pinned, xm)
        else:
            to_mont(BABYBEAR, canon, xm)
        cw = code.encode(xm)
        if timing is not None:
            timing[1].record(stream)
        K, nn = cw.shape
        from zorch_gb300.commit import leaves_layout

        root, layers = prover.tree.commit_layout(leaves_layout(cw, nn, K, 1, nn), device)
        if timing is not None:
            timing[2].record(stream)
        # The device-resident steps leave the index-range flag unread (a host
        # sync per step); the end-to-end steps, on the same indices, read it.
        op = prover.tree.open_layout(leaves_layout(cw, nn, K, 1, nn), layers, idx, K,
                                     check=e2e)
        if e2e:
            out = torch.cat([root.reshape(-1), op.row.reshape(-1), op.path.reshape(-1)])
            host_out = out.cpu()
            return host_out.numel() * 4
        return 0

    bufs = [xm, torch.empty_like(canon)]
    side = torch.cuda.Stream()

    def e2e_pipelined(nsteps):
        """nsteps end-to-end commits through the public API, as a stream of
        traces is served: the host read of trace k+1 (on a side stream, into
        the other input buffer) overlaps trace k's LDE and hashing, and every
        trace's root, rows and paths are copied back to page-locked host
        memory; all of it inside the caller's timed region."""
        from zorch_gb300.commit import leaves_layout

        main = torch.cuda.current_stream()
        ready = [torch.cuda.Event(), torch.cuda.Event()]
        free = [torch.cuda.Event(), torch.cuda.Event()]
        with torch.cuda.stream(side):
            to_mont_from_host(BABYBEAR, pinned, bufs[0])
            ready[0].record(side)
        outs = []
        for k in range(nsteps):
            b = k & 1
            main.wait_event(ready[b])
            if k + 1 < nsteps:
                with torch.cuda.stream(side):
                    if k >= 1:
                        side.wait_event(free[b ^ 1])  # trace k-1 has encoded it
                    to_mont_from_host(BABYBEAR, pinned, bufs[b ^ 1])
                    ready[b ^ 1].record(side)
            cw = code.encode(bufs[b])
            free[b].record(main)
            K, nn = cw.shape
            root, layers = prover.tree.commit_layout(leaves_layout(cw, nn, K, 1, nn), device)
            op = prover.tree.open_layout(leaves_layout(cw, nn, K, 1, nn), layers, idx, K,
                                         check=False)
            out = torch.cat([root.reshape(-1), op.row.reshape(-1), op.path.reshape(-1)])
            host_out = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
            host_out.copy_(out, non_blocking=True)
            outs.append(host_out)
        torch.cuda.synchronize()
        return sum(o.numel() * 4 for o in outs)

    info = {
        "e2e_pipelined": e2e_pipelined,
        "elements": cols * rows,
        "h2d_bytes": cols * rows * 4,
        "d2h_bytes": 4 * (8 + args.queries * cols + (args.log_rows + args.log_blowup) * args.queries * 8),
        "config": {"workload": f"trace commit {rows}x{cols}, blowup {1 << args.log_blowup}, "
                               f"row leaves, {args.queries} query openings",
                   "rows": rows, "cols": cols, "blowup": 1 << args.log_blowup,
                   "queries": args.queries, "field": "babybear", "hash": "poseidon2-16 (built-in)",
                   "l2": "inputs larger than L2 (256 MiB in, 1 GiB LDE)"},
        "leaves": n, "perms_leaf": n * ((cols + 7) // 8), "perms_node": n - 1,
        "ntt_bytes": 4 * cols * rows + 4 * cols * n,
    }
    return step, info


def served_workload(args, device, rank):
    """Config-5 stream: Poisson arrivals, log2 heights 14..24, widths
    log-uniform 1..256, blowup 2 or 4, 30% fold-and-open. The same seeded
    stream is served by the continuous-batching server and by the plain
    drop-in path, in each commitment mode ("fri": one pair-leaf tree per
    column, FriProver.commit; "matrix": one row-leaf tree per request,
    BasefoldProver.commit) -- the two arms of a mode return identical bytes."""
    import torch

    from zorch_gb300.batch import Autotuner, _bucket
    from zorch_gb300.serve import Server, fill_request, make_stream, run_plain

    reqs = make_stream(args.requests, args.seed, rate_hz=args.rate, log_h=(args.min_log_h,
                                                                            args.max_log_h))
    for r in reqs:
        fill_request(r, device)
    torch.cuda.synchronize()
    # autotune every (log_n, log2 width) bucket of the stream not yet cached:
    # LDE tile and radix, tree-top depth (untimed set-up, kept in the cache)
    tuner = Autotuner()
    for r in reqs:
        if _bucket(r.log_n, r.width) not in tuner.table:
            cols = r.resident[:min(r.width, 8)]
            tuner.tune(r.log_h, cols.shape[0], r.log_blowup, reps=2, columns=cols,
                       bucket_width=r.width)
    tuner.save()
    servers = {m: Server(budget_bytes=args.budget_gb * 1e9, max_batch=args.max_batch,
                         streams=args.streams, tuner=tuner, mode=m) for m in ("fri", "matrix")}

    def served(mode, host_fed=False, stream=None):
        t0 = time.perf_counter()
        res = servers[mode].run(stream if stream is not None else reqs, host_fed=host_fed)
        torch.cuda.synchronize()
        return res, time.perf_counter() - t0

    def plain(mode, stream=None):
        t0 = time.perf_counter()
        res = run_plain(stream if stream is not None else reqs, perm=servers[mode].perm,
                        mode=mode, budget_bytes=args.budget_gb * 1e9)
        torch.cuda.synchronize()
        return res, time.perf_counter() - t0

    return reqs, served, plain, servers


def served_hash_roofline(reqs, server, mode):
    """LDE and hash device time of the served stream's commits, one request at
    a time on the current stream with CUDA events around each phase (the
    server overlaps requests on several streams, so per-kernel times are
    taken on this serial replay of the same commits). Every buffer is
    allocated before the first event, so the timed regions hold kernels only.
    Returns (lde_ms, hash_ms, permutations, lde_bytes)."""
    import torch

    from zorch_gb300.batch import MatrixJob
    from zorch_gb300.field import BABYBEAR, to_mont
    from zorch_gb300.serve import FRI_LAYER_CAP

    bc = server.committer
    stream = torch.cuda.current_stream()
    lde_ms = hash_ms = 0.0
    perms = lde_bytes = 0
    for r in reqs:
        x = to_mont(BABYBEAR, r.resident)
        w, n = r.width, 1 << r.log_n
        job = MatrixJob(x, r.log_blowup, 31)
        cw = torch.empty((w, n), dtype=torch.int32, device=x.device)
        ws = torch.empty((bc.encode_workspace_bytes([job], [cw]) + 3) // 4 + 64,
                         dtype=torch.int32, device=x.device)
        ws = ws[(-ws.data_ptr() % 256) // 4:]  # 256-byte aligned view
        if mode == "fri":
            per = w if 32 * w * n <= FRI_LAYER_CAP else max(1, FRI_LAYER_CAP // (32 * n))
            buf = torch.empty((min(per, w), n - 1, 8), dtype=torch.int32, device=x.device)
        else:
            per, buf = w, torch.empty((2 * n - 1, 8), dtype=torch.int32, device=x.device)
        ctr = torch.empty(64, dtype=torch.int32, device=x.device)
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(stream)
        bc.encode([job], [cw], ws)
        e[1].record(stream)
        if mode == "fri":
            for c0 in range(0, w, per):
                cnt = min(per, w - c0)
                bc.pair_trees([cw[c0:c0 + cnt]], flats=[buf[:cnt]], counters=ctr)
            perms += w * (n - 1)
        else:
            bc.merkle([cw], flats=[buf], counters=ctr)
            perms += n * ((w + 7) // 8) + n - 1
        e[2].record(stream)
        torch.cuda.synchronize()
        lde_ms += e[0].elapsed_time(e[1])
        hash_ms += e[1].elapsed_time(e[2])
        lde_bytes += 4 * r.elements + 4 * w * n
        del cw, x, buf, ws
    return lde_ms, hash_ms, perms, lde_bytes


def calibrated_stream(args, n, seed, rate, device):
    """A long stream of the config-5 distribution at a set arrival rate whose
    requests read their inputs from one shared seeded buffer (views of its
    first w*h words): the data of a request does not change its cost, and the
    stream's inputs then take one buffer instead of one per request. With
    device None only the shapes are drawn."""
    import torch

    from zorch_gb300 import _lib
    from zorch_gb300.field import ptr, stream_handle
    from zorch_gb300.serve import make_stream

    reqs = make_stream(n, seed, rate_hz=rate, log_h=(args.min_log_h, args.max_log_h))
    if device is None:
        return reqs
    big = max(r.elements for r in reqs)
    buf = torch.empty(big, dtype=torch.int32, device=device)
    _lib.check(_lib.lib().zc_fill_uniform(0, ptr(buf), big, seed, stream_handle()), "fill")
    for r in reqs:
        r.resident = buf[: r.elements].view(r.width, 1 << r.log_h)
    torch.cuda.synchronize()
    return reqs


def fri_workload(args, device):
    """Config 3: one 2^22-coefficient polynomial, blowup 2, FRI commit phase with
    EF4 challenges down to 2^8 (15 rounds) and 100 query openings."""
    import torch

    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2
    from zorch_gb300.field import BABYBEAR, ptr, stream_handle, to_mont, to_mont_from_host
    from zorch_gb300.pcs import FriParams, FriProver
    from zorch_gb300.transcript import DuplexTranscript
    from zorch_gb300 import _lib

    log_k = 22
    perm = Poseidon2.builtin(BABYBEAR)
    code = ReedSolomon(1 << log_k, 2, BABYBEAR, coset_shift=31, generator=31)
    prover = FriProver(FriParams(code, MerkleTree(perm), 15, 100, 4))
    x = torch.empty(1 << log_k, dtype=torch.int32, device=device)
    _lib.check(_lib.lib().zc_fill_uniform(0, ptr(x), x.numel(), 3, stream_handle()), "fill")

    pinned = x.cpu().pin_memory()

    from zorch_gb300.pcs import GraphedFriCommitPhase

    graphed = GraphedFriCommitPhase(prover, device)
    xm = torch.empty_like(x)

    def run(e2e=False):
        """Canonical coefficients -> Montgomery -> graph replay (encode + 15
        fold-and-commit rounds + transcript + openings)."""
        if e2e:
            to_mont_from_host(BABYBEAR, pinned, xm)
        else:
            to_mont(BABYBEAR, x, xm)
        return graphed.replay(xm)

    def run_eager():
        cw = code.encode(to_mont(BABYBEAR, x))
        proof, _, _ = prover.commit_phase(cw, DuplexTranscript.new(perm, device=device))
        return proof

    run.eager = run_eager
    return run, 1 << log_k


def uneven_workload(args, device):
    """Config 4: 48 matrices, log2 heights 12..22, widths 1..128, blowup
    2/4/8 (one seeded draw each): one batched commit vs 48 plain calls."""
    import torch

    from zorch_gb300.batch import Autotuner, BatchCommitter, GraphedBatch, _bucket
    from zorch_gb300.coding import ReedSolomon
    from zorch_gb300.commit import MerkleTree, Poseidon2
    from zorch_gb300.field import BABYBEAR, ptr, stream_handle, to_mont, to_mont_from_host
    from zorch_gb300.pcs import BasefoldProver
    from zorch_gb300 import _lib

    rng = np.random.default_rng(args.seed)
    shapes = [(int(rng.integers(1, 129)), int(rng.integers(12, 23)), int(rng.choice([1, 2, 3])))
              for _ in range(48)]
    mats = []
    for i, (w, lh, lb) in enumerate(shapes):
        xx = torch.empty((w, 1 << lh), dtype=torch.int32, device=device)
        _lib.check(_lib.lib().zc_fill_uniform(0, ptr(xx), xx.numel(), 900 + i, stream_handle()),
                   "fill")
        mats.append((xx, lb))
    perm = Poseidon2.builtin(BABYBEAR)
    tuner = Autotuner()  # tune the batch's buckets not yet cached (untimed set-up)
    for (x, lb), (w, lh, _) in zip(mats, shapes):
        if _bucket(lh + lb, w) not in tuner.table:
            tuner.tune(lh, min(w, 8), lb, reps=2, perm=perm, columns=x[:min(w, 8)],
                       bucket_width=w)
    tuner.save()
    bc = BatchCommitter(perm, BABYBEAR, tuner=tuner)
    # the whole batch (persistent LDE and tree launches) captured in one graph
    graphed = GraphedBatch(bc, [(w, 1 << lh, lb) for w, lh, lb in shapes], device)
    tree = MerkleTree(perm, column_major=True)
    elements = sum(w << lh for w, lh, _ in shapes)

    def batched():
        for dst, (x, _) in zip(graphed.inputs, mats):
            to_mont(BABYBEAR, x, out=dst)
        return graphed.replay()

    def plain():
        roots = []
        for x, lb in mats:
            code = ReedSolomon(x.shape[1], 1 << lb, BABYBEAR, coset_shift=31, generator=31)
            root, _ = BasefoldProver(code, tree).commit_columns(to_mont(BABYBEAR, x))
            roots.append(root)
            torch.cuda.synchronize()
        return roots

    pinned = [x.cpu().pin_memory() for x, _ in mats]

    def batched_host():
        """End to end: canonical inputs read from page-locked host memory by the
        conversion kernel, one batched commit, the 48 roots read back."""
        for dst, h in zip(graphed.inputs, pinned):
            to_mont_from_host(BABYBEAR, h, out=dst)
        res = graphed.replay()
        return torch.stack([r.root for r in res]).cpu()

    return batched, plain, batched_host, elements, shapes


def paths_workload(args, device):
    """Latency of the PCS paths around the commit (Basefold open, the SP1
    stacked open, the k-ary fold rounds, the query-strided Merkle commit, the
    proof-of-work grind and one transcript hop) through the public API on the
    GPU, each beside the oracle on the same inputs on the host cores (the
    CPU-baseline leg), with the two outputs compared. GPU times are wall time
    per call with a device synchronize on both sides, mean over --steps calls
    after warm-up; the oracle runs once per path."""
    import torch

    from zorch_gb300.coding import BitReversedReedSolomon, ReedSolomon
    from zorch_gb300.commit import (MerkleTree, Poseidon2, SingleMatrixCommitmentScheme,
                                    StridedMerkleTree)
    from zorch_gb300.field import BABYBEAR, KOALABEAR, to_device, to_host
    from zorch_gb300.jagged import stacked_basefold_open, stacked_commit
    from zorch_gb300.pcs import BasefoldProver, FoldState, PreFoldKGroupCommitRound, fold_rounds
    from zorch_gb300.transcript import DuplexTranscript

    cpu = not args.no_cpu_baseline
    orc = None
    if cpu:
        from oracle import oracle as orc
    rng = np.random.default_rng(args.seed)

    def mont(field, shape):
        """Seeded uniform field elements, Montgomery words (x 2^32 mod p)."""
        pm = np.uint64(BABYBEAR.p if field == 0 else KOALABEAR.p)
        x = rng.integers(0, int(pm), size=shape, dtype=np.uint64)
        return ((x << np.uint64(32)) % pm).astype(np.uint32)

    def gpu_time(fn):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            out = fn()
        torch.cuda.synchronize()
        return 1e3 * (time.perf_counter() - t0) / args.steps, out

    def cpu_time(fn):
        t0 = time.perf_counter()
        out = fn()
        return 1e3 * (time.perf_counter() - t0), out

    rows = {}
    bb = Poseidon2.builtin(BABYBEAR)
    sp1d = json.loads(open(os.path.join(ROOT, "tests", "golden", "sp1_fibonacci",
                                        "sp1_koalabear16.json")).read())
    sp1 = Poseidon2.from_params(KOALABEAR, sp1d["alpha"], sp1d["external_initial"],
                                sp1d["external_terminal"], sp1d["internal_rc"],
                                sp1d["internal_diag"], sp1d["internal_j_scale"])
    kb = json.loads(open(os.path.join(ROOT, "tests", "golden", "koalabear16.json")).read())
    kbp = Poseidon2.from_params(KOALABEAR, kb["alpha"], kb["external_initial"],
                                kb["external_terminal"], kb["internal_rc"], kb["internal_diag"],
                                kb.get("internal_j_scale", 1))

    # f1: Basefold batch open, 2^20 x 8 BabyBear columns, blowup 2, 64 queries
    v, w, q = 20, 8, 64
    code = ReedSolomon(1 << v, 2, BABYBEAR, coset_shift=31)
    prover = BasefoldProver(code, MerkleTree(bb, column_major=True), num_queries=q)
    cols_h = mont(0, (w, 1 << v))
    z_h = mont(0, (v, 4))
    _, data = prover.commit_columns(to_device(cols_h).reshape(w, 1 << v))
    zd = to_device(z_h).reshape(v, 4)
    g_ms, (_, proof, _) = gpu_time(lambda: prover.open_batch([data], zd, DuplexTranscript.new(bb)))
    row = {"config": f"2^{v} x {w} BabyBear columns, blowup 2, {q} queries", "gpu_ms": g_ms}
    if cpu:
        cw = to_host(data.codeword)
        p2 = orc.Poseidon2.babybear16()
        mats = [{"cols": cols_h, "codeword": cw, "layers": orc.merkle_commit_columns(p2, cw)}]
        c_ms, want = cpu_time(lambda: orc.basefold_open(p2, 0, mats, z_h, 1, BABYBEAR.mont(31), q,
                                                         orc.Transcript(p2)))
        row.update(cpu_ms=c_ms, equal=bool(
            np.array_equal(to_host(proof.fri_roots), want["fri_roots"])
            and np.array_equal(to_host(proof.final_poly), want["final_poly"])))
    rows["basefold_open"] = row
    # the same open replayed from one CUDA graph (GraphedBasefoldOpen)
    from zorch_gb300.pcs import GraphedBasefoldOpen

    gbo = GraphedBasefoldOpen(prover, [data])
    t_empty = DuplexTranscript.new(bb)
    g_ms, (_, gproof, _) = gpu_time(lambda: gbo.replay(zd, t_empty))
    grow = {"config": row["config"] + ", one graph replay", "gpu_ms": g_ms,
            "equal_to_eager": bool(torch.equal(gproof.fri_roots, proof.fri_roots)
                                   and torch.equal(gproof.final_poly, proof.final_poly)
                                   and torch.equal(gproof.uni_msgs, proof.uni_msgs))}
    if cpu:
        grow["cpu_ms"] = row["cpu_ms"]
    rows["basefold_open_graphed"] = grow

    # f2: SP1 stacked BaseFold open, two committed rounds (8 + 4 columns) of 2^20, blowup 2
    v, q = 20, 64
    scode = BitReversedReedSolomon(1 << v, 2, KOALABEAR)
    smcs = SingleMatrixCommitmentScheme(sp1)
    blocks = [mont(1, (8, 1 << v)), mont(1, (4, 1 << v))]
    srounds = [stacked_commit(smcs, scode, to_device(b).reshape(b.shape)) for b in blocks]
    zf, de = mont(1, (v + 2, 4)), mont(1, (4,))
    zfd, ded = to_device(zf).reshape(v + 2, 4), to_device(de)
    g_ms, (sproof, _) = gpu_time(lambda: stacked_basefold_open(
        smcs, scode, srounds, zfd, ded, v, num_queries=q, pow_bits=0,
        transcript=DuplexTranscript.new(sp1)))
    row = {"config": f"KoalaBear, rounds of 8 + 4 columns x 2^{v}, blowup 2, {q} queries",
           "gpu_ms": g_ms}
    if cpu:
        p2 = orc.sp1_koalabear16()
        c_ms, want = cpu_time(lambda: orc.sp1_stacked_open(p2, 1, blocks, zf, de, v, 1, q,
                                                            orc.Transcript(p2)))
        row.update(cpu_ms=c_ms, equal=bool(
            np.array_equal(to_host(sproof.fri_commitments), want["bound_roots"])
            and np.array_equal(to_host(sproof.final_poly), want["final_poly"])))
    rows["sp1_stacked_open"] = row
    from zorch_gb300.jagged import GraphedStackedOpen

    gso = GraphedStackedOpen(smcs, scode, srounds, v + 2, v, num_queries=q, pow_bits=0)
    t_sp1 = DuplexTranscript.new(sp1)
    g_ms, (gsp, _) = gpu_time(lambda: gso.replay(zfd, ded, t_sp1))
    grow = {"config": row["config"] + ", one graph replay", "gpu_ms": g_ms,
            "equal_to_eager": bool(torch.equal(gsp.fri_commitments, sproof.fri_commitments)
                                   and torch.equal(gsp.final_poly, sproof.final_poly))}
    if cpu:
        grow["cpu_ms"] = row["cpu_ms"]
    rows["sp1_stacked_open_graphed"] = grow

    # f4: k-ary fold-and-commit rounds (k = 4, two rounds) over a 2^22 KoalaBear codeword
    k, nr = 4, 2
    kcode = ReedSolomon(1 << 21, 2, KOALABEAR, fold_factor=k)
    ktree = MerkleTree(kbp)
    msg = to_device(mont(1, (1 << 21,)))
    kcw = kcode.encode(msg)

    def kary():
        st, _, roots = fold_rounds(PreFoldKGroupCommitRound(kcode, ktree), FoldState(kcw),
                                   DuplexTranscript.new(kbp), nr)
        return st.codeword, roots
    g_ms, (kfinal, kroots) = gpu_time(kary)
    row = {"config": f"k = {k}, {nr} rounds from a 2^22 KoalaBear codeword", "gpu_ms": g_ms}
    if cpu:
        cp = orc.Poseidon2.koalabear16_golden()
        cw0 = to_host(kcw)

        def kary_cpu():
            ot, cw, rts = orc.Transcript(cp), cw0, []
            for _ in range(nr):
                n = cw.shape[0]
                dl = orc.merkle_commit(cp, cw, n // k, k, 1, n // k)
                ot.observe(dl[-1][0])
                rts.append(dl[-1][0])
                cw = orc.fri_fold_k(1, cw, False, ot.sample(1), False, 2, 0)
            return cw, rts
        c_ms, (wcw, wroots) = cpu_time(kary_cpu)
        row.update(cpu_ms=c_ms, equal=bool(
            np.array_equal(to_host(torch.stack(kroots)), np.stack(wroots))
            and np.array_equal(to_host(kfinal), wcw)))
    rows["kary_fold_commit"] = row

    # f4: query-strided Merkle commit (WHIR), 2^20 x 8 BabyBear rows, 16 rows per query
    h, sw, rpq = 1 << 20, 8, 16
    mat = mont(0, (h, sw))
    md = to_device(mat).reshape(h, sw)
    stree = StridedMerkleTree(bb, rpq)
    g_ms, (sroot, _) = gpu_time(lambda: stree.commit(md))
    row = {"config": f"2^20 x {sw} BabyBear rows, {rpq} rows per query", "gpu_ms": g_ms}
    if cpu:
        c_ms, want = cpu_time(lambda: orc.strided_merkle_commit(orc.Poseidon2.babybear16(), mat,
                                                                 rpq))
        row.update(cpu_ms=c_ms, equal=bool(np.array_equal(to_host(sroot).reshape(-1),
                                                          want[-1].reshape(-1))))
    rows["strided_merkle_commit"] = row

    # f3: proof-of-work grind (pow_bits 18) and one transcript hop (observe 8, squeeze 1)
    seed_vals = mont(0, (5,))
    t0 = DuplexTranscript.new(bb).observe(to_device(seed_vals))
    g_ms, (_, wit) = gpu_time(lambda: t0.grind(18))
    row = {"config": "pow_bits 18, BabyBear duplex transcript", "gpu_ms": g_ms}
    if cpu:
        ot = orc.Transcript(orc.Poseidon2.babybear16())
        ot.observe(seed_vals)
        c_ms, wcanon = cpu_time(lambda: ot.grind(18))
        row.update(cpu_ms=c_ms, equal=int(to_host(wit.reshape(1))[0]) == BABYBEAR.mont(wcanon))
    rows["grind"] = row
    vals8 = to_device(mont(0, (8,)))
    tt = DuplexTranscript.new(bb)
    hop_ms, _ = gpu_time(lambda: tt.observe_and_sample_(vals8, 1))
    rows["transcript_hop"] = {"config": "observe 8 + squeeze 1 on the device (one launch)",
                              "gpu_ms": hop_ms}
    for r in rows.values():
        if "cpu_ms" in r:
            r["speedup"] = r["cpu_ms"] / r["gpu_ms"]
    return rows, (orc.threads() if cpu else None)


def pct(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if len(xs) else None


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return reference_arm(args, rank, world)

    import torch

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=device)
    from zorch_gb300 import _lib

    _lib.check(_lib.lib().zc_init(local), "init")
    if args.workload == "paths":
        rows, threads = paths_workload(args, device)
        if rank == 0:
            print(json.dumps({
                "metric": "PCS path latency (Basefold open, SP1 stacked open, k-ary fold, "
                          "strided Merkle commit, grind, transcript hop)",
                "value": rows["basefold_open"]["gpu_ms"], "unit": "ms per Basefold open",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                "dtype": "u32 (BabyBear / KoalaBear, Montgomery)", "data": "synthetic, seeded",
                "workload": "paths", "rows": rows,
                "cpu_baseline": None if threads is None else {
                    "kind": "port", "cores": threads,
                    "sample": "the oracle once per path on the same inputs"}}), flush=True)
        return
    step, info = trace_workload(args, device)
    stream = torch.cuda.current_stream()

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    # ---- device-resident timed region
    marks = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    clocks = Clocks(local).start()
    launches0 = _lib.lib().zc_launch_count()
    barrier()
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        step(timing=marks[k])
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    launches = _lib.lib().zc_launch_count() - launches0
    ms = t_start.elapsed_time(t_end)
    ms_max = max_over_ranks(ms, device)
    ntt_ms = sum(m[0].elapsed_time(m[1]) for m in marks) / args.steps
    hash_ms = sum(m[1].elapsed_time(m[2]) for m in marks) / args.steps

    # ---- end-to-end through the public API from pinned host memory
    for _ in range(2):
        step(e2e=True)  # also reads the index-range flag of the openings
    torch.cuda.synchronize()
    pipelined = info.get("e2e_pipelined") if args.workload == "trace" else None
    if pipelined:
        pipelined(2)
    barrier()
    e0 = time.perf_counter()
    if pipelined:
        pipelined(args.steps)
    else:
        for _ in range(args.steps):
            step(e2e=True)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - e0, device)

    elems_total = info["elements"] * args.steps * world
    value = elems_total / (ms_max / 1e3)
    e2e_value = elems_total / e2e_s
    served_info = None
    if args.workload == "fri":
        run, elements = fri_workload(args, device)
        for _ in range(max(args.warmup, 3)):
            run()
        torch.cuda.synchronize()
        clocks = Clocks(local).start()
        l0 = _lib.lib().zc_launch_count()
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        for _ in range(args.steps):
            proof = run()
        s1.record(stream)
        torch.cuda.synchronize()
        clk = clocks.stop()
        launches = _lib.lib().zc_launch_count() - l0
        ms_max = max_over_ranks(s0.elapsed_time(s1), device)
        value = elements * args.steps * world / (ms_max / 1e3)
        e0 = time.perf_counter()
        for _ in range(args.steps):
            b = run(e2e=True).to_bytes()
        e2e_value = elements * args.steps / max_over_ranks(time.perf_counter() - e0, device)
        info["h2d_bytes"] = 4 * elements
        info["d2h_bytes"] = len(b)
        for _ in range(3):
            run.eager()
        torch.cuda.synchronize()
        q0 = time.perf_counter()
        for k in range(args.steps):
            if k == 0:  # marks one eager proof for a profiler's range filter
                torch.cuda.nvtx.range_push("fri_eager")
            run.eager()
            if k == 0:
                torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        served_info = {"eager_ms_per_proof": 1e3 * (time.perf_counter() - q0) / args.steps,
                       "graphed_ms_per_proof": ms_max / args.steps,
                       "bytes_equal_graph_vs_eager": run.eager().to_bytes() == run().to_bytes()}
        info["config"] = {"workload": "FRI commit phase: 2^22 coefficients, blowup 2, shift 31, "
                                      "15 arity-2 rounds to 2^8 with EF4 challenges, 100 queries",
                          "field": "babybear", "hash": "poseidon2-16 (built-in)",
                          "l2": "inputs larger than L2 (32 MiB codeword x 2 + layers)"}
    if args.workload == "uneven":
        batched, plain, batched_host, elements, shapes = uneven_workload(args, device)
        for _ in range(2):
            batched()
        plain()
        torch.cuda.synchronize()
        clocks = Clocks(local).start()
        l0 = _lib.lib().zc_launch_count()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            batched()
        torch.cuda.synchronize()
        b_s = max_over_ranks(time.perf_counter() - t0, device)
        clk = clocks.stop()
        launches = _lib.lib().zc_launch_count() - l0
        t0 = time.perf_counter()
        plain()
        p_s = max_over_ranks(time.perf_counter() - t0, device)
        ms_max = b_s * 1e3
        value = elements * args.steps * world / b_s
        batched_host()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            batched_host()
        e2e_value = elements * args.steps * world / max_over_ranks(time.perf_counter() - t0,
                                                                   device)
        info["h2d_bytes"] = 4 * elements
        info["d2h_bytes"] = 48 * 32
        served_info = {"plain_per_matrix": {"value": elements / p_s, "unit": "elem/s",
                                             "path": "48 BasefoldProver.commit calls, sync each"},
                       "batched_over_plain": (elements * args.steps / b_s) / (elements / p_s),
                       "elements_per_step": elements}
        info["config"] = {"workload": "uneven batch: 48 matrices, log2 h 12..22, w 1..128, "
                                      "blowup 2|4|8, one batched commit replayed from a CUDA "
                                      "graph, autotuned tile/radix/tree top per bucket",
                          "field": "babybear",
                          "l2": "inputs larger than L2"}
    served_roof = None
    if args.workload == "served":
        reqs, served, plain, servers = served_workload(args, device, rank)
        modes = {}
        for mode in ("fri", "matrix"):
            for _ in range(max(args.warmup, 3)):
                served(mode)
            l0 = _lib.lib().zc_launch_count()
            if mode == "fri":
                clocks = Clocks(local).start()
            barrier()
            times, lat = [], []
            torch.cuda.nvtx.range_push(f"served_{mode}")  # for a profiler's range filter
            for _ in range(args.steps):
                res, dt = served(mode)
                times.append(dt)
                lat += [r.latency for r in res]
            torch.cuda.nvtx.range_pop()
            barrier()
            m = {"launches": _lib.lib().zc_launch_count() - l0, "s": max_over_ranks(sum(times),
                                                                                    device)}
            if mode == "fri":
                clk = clocks.stop()
            plain(mode)  # warm
            p_res, p_dt = plain(mode)
            done = [r for r in res if r.proof]
            elements = sum(q.elements for q, r in zip(reqs, res) if r.proof)
            m.update({
                "res": res, "elements": elements, "lat": lat,
                "plain_dt": p_dt, "plain_res": p_res,
                "bytes_equal": len(done) > 0 and all(a.proof == b.proof
                                                    for a, b in zip(res, p_res)),
                "rejected": len(res) - len(done)})
            modes[mode] = m
        # end to end: inputs from pinned host memory read by the conversion
        # kernel, proofs back in pinned buffers, all inside the timed region
        for r in reqs:
            r.host = r.resident.cpu().pin_memory()
        torch.cuda.synchronize()
        for mode in ("fri", "matrix"):
            served(mode, host_fed=True)
            h_runs = max(1, min(args.steps, 3))
            h0 = time.perf_counter()
            for _ in range(h_runs):
                h_res, _ = served(mode, host_fed=True)
            torch.cuda.synchronize()
            modes[mode]["h_dt"] = max_over_ranks(time.perf_counter() - h0, device) / h_runs
            modes[mode]["bytes_equal_host_fed"] = all(
                a.proof == b.proof for a, b in zip(modes[mode]["res"], h_res))
        for r in reqs:
            r.host = None
        # hash / LDE rooflines on the served stream's own commits (serial replay)
        lde_ms, hash_ms_sv, perms_sv, lde_bytes_sv = served_hash_roofline(reqs, servers["fri"],
                                                                          "fri")
        served_roof = {"lde_ms": lde_ms, "hash_ms": hash_ms_sv, "perms": perms_sv,
                       "lde_bytes": lde_bytes_sv}
        blocks = {}
        for mode, m in modes.items():
            el = m["elements"]
            blocks[mode] = {
                "value": el * args.steps * world / m["s"], "unit": "elem/s",
                "requests_per_s": len(reqs) * args.steps / (m["s"] / world),
                "latency_ms": {"p50": 1e3 * pct(m["lat"], 50), "p99": 1e3 * pct(m["lat"], 99)},
                "e2e": el * world / m["h_dt"],
                "plain": {"value": el / m["plain_dt"], "unit": "elem/s",
                          "requests_per_s": len(reqs) / m["plain_dt"],
                          "latency_ms": {
                              "p50": 1e3 * pct([r.latency for r in m["plain_res"]], 50),
                              "p99": 1e3 * pct([r.latency for r in m["plain_res"]], 99)},
                          "path": ("one FriProver.commit_one call per polynomial (column); "
                                   "result read back per request" if mode == "fri" else
                                   "one BasefoldProver.commit call per request; result read "
                                   "back per request")},
                "served_over_plain": (el * args.steps / m["s"]) / (el / m["plain_dt"]),
                "bytes_identical_served_vs_plain": m["bytes_equal"],
                "bytes_identical_host_fed": m["bytes_equal_host_fed"],
                "rejected_over_budget": m["rejected"],
                "commitment": ("per-polynomial pair-leaf roots (FriProver.commit)"
                               if mode == "fri" else
                               "one row-leaf root per request (BasefoldProver.commit)"),
            }
        # calibrated served rate: arrivals at 0.8 x the plain path's measured
        # request rate, a long stream, both arms on the same stream
        del reqs
        torch.cuda.empty_cache()
        from zorch_gb300.serve import request_work

        cal = {}
        for mode in ("fri", "matrix"):
            # the plain path's capacity in permutations/s on the 24-request
            # stream, over the mean permutations of a request of the longer
            # stream (hashing is most of a request's device time)
            shapes = make_stream_for(args)
            rate = sum(request_work(q, mode) for q in shapes) / modes[mode]["plain_dt"]
            probe = calibrated_stream(args, args.cal_requests, args.seed + 1, 1.0, None)
            mean = sum(request_work(q, mode) for q in probe) / len(probe)
            lam = 0.8 * rate / mean
            stream_c = calibrated_stream(args, args.cal_requests, args.seed + 1, lam, device)
            served(mode, stream=stream_c[:8])  # warm the shapes' kernels
            c_res, c_dt = served(mode, stream=stream_c)
            p_res, p_dt = plain(mode, stream=stream_c)
            ok = [r for r in c_res if r.proof]
            cal[mode] = {
                "rate_per_s": lam, "requests": len(stream_c),
                "rate_rule": "0.8 x the plain path's permutations/s on the 24-request stream / "
                             "the mean permutations per request of this stream",
                "rejected_over_budget": len(c_res) - len(ok),
                "served": {"requests_per_s": len(ok) / c_dt,
                           "latency_ms": {"p50": 1e3 * pct([r.latency for r in ok], 50),
                                          "p99": 1e3 * pct([r.latency for r in ok], 99)}},
                "plain": {"requests_per_s": len(ok) / p_dt,
                          "latency_ms": {
                              "p50": 1e3 * pct([r.latency for r in p_res if r.proof], 50),
                              "p99": 1e3 * pct([r.latency for r in p_res if r.proof], 99)}},
                "bytes_identical_served_vs_plain": all(a.proof == b.proof
                                                       for a, b in zip(c_res, p_res)),
            }
            blocks[mode]["calibrated"] = cal[mode]
            del stream_c
            torch.cuda.empty_cache()
        head = modes["fri"]
        value = blocks["fri"]["value"]
        e2e_value = blocks["fri"]["e2e"]
        launches = head["launches"]
        served_info = {
            "headline_mode": "fri", "requests": args.requests,
            "elements_per_step": head["elements"],
            "requests_per_s": blocks["fri"]["requests_per_s"],
            "fold_requests": sum(q.fold for q in make_stream_for(args)),
            "latency_ms": blocks["fri"]["latency_ms"],
            "served_over_plain": blocks["fri"]["served_over_plain"],
            "fri": blocks["fri"], "matrix": blocks["matrix"],
        }
        info["h2d_bytes"] = 4 * head["elements"]
        info["d2h_bytes"] = sum(len(r.proof) for r in head["res"])
        ms_max = head["s"] * 1e3
        info["config"] = {"workload": f"served commit stream: {args.requests} requests, Poisson "
                                      f"{args.rate:g}/s, log2 h {args.min_log_h}..{args.max_log_h}, "
                                      "w log-uniform 1..256, blowup 2|4, 30% fold to 2^8 + 64 "
                                      "queries; headline: per-polynomial commitments "
                                      "(FriProver.commit bytes)", "budget_gb": args.budget_gb,
                          "max_batch": args.max_batch, "streams": args.streams,
                          "policy": "shortest work first within a size class, 2 s aging bound; "
                                    f"{args.streams - 1} high-priority streams for batches of "
                                    "<= 2^25 permutations, 1 low-priority stream for larger",
                          "field": "babybear", "hash": "poseidon2-16 (built-in)",
                          "l2": "inputs larger than L2"}

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    # Hash kernel (dominant): integer instructions executed per Poseidon2
    # permutation of the built-in BabyBear-16 instance, from the ncu capture
    # summarised in profiles/ (thread-level SASS instructions).
    inst_per_perm = float(os.environ.get("ZC_INST_PER_PERM", "6070"))
    # DRAM bytes per hashed LDE word of the k_leaf launch (134.27 MB read +
    # 8.60 MB written for 2^19 leaves x 64 words, profiles/), scaled to this
    # workload's leaf launch by its word count.
    traffic_per_word = (134.273792e6 + 8.598272e6) / float(1 << 25)
    perms = info["perms_leaf"] + info["perms_node"]
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    int_peak = sms * 128 * sm_mhz * 1e6 / 1e9  # Ginst/s: SMs x 128 lanes x clock
    peak_src = (f"{sms} SMs (cudaDevAttrMultiProcessorCount) x 128 lanes x sm_max_mhz "
                "(MEASURED_PEAKS.json): the thread-instruction issue peak")
    binding = ("FMA-heavy pipe (the Montgomery products' wide and high multiplies): 81 % of "
               "its peak cycles in the ncu capture of the leaf launch "
               "(profiles/k_leaf_poseidon2_trace_2p17x64_blowup4.md)")

    def hash_roof(perms_, ms_, kernel, traffic):
        ach = perms_ * inst_per_perm / (ms_ / 1e3) / 1e9
        return {"bound": "int32", "kernel": kernel, "achieved": ach, "peak": int_peak,
                "unit": "Ginst/s", "frac": ach / int_peak, "traffic": traffic,
                "peak_source": peak_src, "binding_unit": binding, "ms": ms_, "perms": perms_,
                "perm_rate": perms_ / (ms_ / 1e3), "inst_per_perm": inst_per_perm}

    # Thread instructions per output word of the radix-2^5 LDE passes (ncu,
    # 2^17 x 64 blowup-4 capture; 175 for the radix-2^4 build) against the
    # butterflies' own: log2(k)/2 = 8.5 radix-2 butterflies per output word at
    # ~11 field instructions each.
    lde_wide = {"binding_unit": "integer issue at 512 threads per SM (128 registers per "
                                "thread; issue active 49-55 % in the ncu capture), not HBM",
                "inst_per_output_word": 136.7, "butterfly_floor_per_output_word": 93.5,
                "issue_frac": 93.5 / 136.7,
                "issue_source": "profiles/k_lde_wide_trace_2p17x64_blowup4.md"}

    def ntt_roof(bytes_, ms_, kernel, issue):
        ach = bytes_ / (ms_ / 1e3) / 1e9
        return {"bound": "hbm", "kernel": kernel, "achieved": ach, "peak": hbm_peak,
                "unit": "GB/s", "frac": ach / hbm_peak, "ms": ms_,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)", **issue}

    trace_roof = hash_roof(perms, hash_ms, "Poseidon2 Merkle hashing of the 2^20 x 64 trace "
                           "commit (k_leaf leaves + levels + fused top)",
                           traffic_per_word * info["leaves"] * args.cols)
    trace_roof["traffic_note"] = "bytes per launch, scaled from the 2^19 x 64 ncu capture"
    trace_ntt = ntt_roof(info["ntt_bytes"], ntt_ms, "coset LDE of the 2^20 x 64 trace "
                                                    "(k_lde_pass1 + pass2, radix-2^5 variant)",
                         lde_wide)
    if served_roof is not None:
        roofline = hash_roof(served_roof["perms"], served_roof["hash_ms"],
                             "Poseidon2 pair-leaf Merkle hashing of the served stream "
                             "(k_tree_batch leaves + levels, k_tree_top), CUDA events around "
                             "each request's tree commit on a serial replay", None)
        roofline["traffic_note"] = ("not captured on the served stream; the leaf kernel reads "
                                    "each codeword word once (trace capture: 1.00x the "
                                    "algorithmic bytes)")
        roofline_ntt = ntt_roof(served_roof["lde_bytes"], served_roof["lde_ms"],
                                "coset LDE of the served stream (the largest requests on the "
                                "radix-2^5 single-matrix passes, which carry most of its "
                                "outputs; the rest on the batched radix-2^4 phases)",
                                lde_wide)
    else:
        roofline, roofline_ntt = trace_roof, trace_ntt
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "elem/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": ms_max / args.steps,
        "workload": args.workload,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 (BabyBear, Montgomery)",
        "data": "synthetic: seeded uniform [0, p) canonical BabyBear elements",
        "config": info["config"] | {"parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "elem/s", "h2d_bytes_per_step": info["h2d_bytes"],
                "d2h_bytes_per_step": info["d2h_bytes"]},
        "roofline": roofline,
        "roofline_ntt": roofline_ntt,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if served_roof is not None:
        out["roofline_trace"] = trace_roof
        out["roofline_ntt_trace"] = trace_ntt
    if served_info is not None:
        out[{"served": "served", "fri": "fri", "uneven": "batched"}[args.workload]] = served_info
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # bounded samples repeated until about 10 s of CPU work
        runs, secs, e = 0, 0.0, 0
        while runs < 8 and (secs < 10.0 or runs == 0):
            if args.workload == "served":
                _, s_, thr, e_ = cpu_served_sample(args, cap_log_h=CPU_CAP_LOG_H)
            else:
                _, s_, thr = cpu_trace_sample(16, args.cols, args.log_blowup, args.queries)
                e_ = args.cols << 16
            runs, secs, e = runs + 1, secs + s_, e + e_
        v = e / secs
        if args.workload == "served":
            sample = (f"oracle C restatement on the served stream with heights capped at "
                      f"2^{CPU_CAP_LOG_H}, {runs} run(s): {e} elements in {secs:.1f} s")
        else:
            sample = (f"oracle C restatement, 2^16 x {args.cols} slice of the trace workload, "
                      f"{runs} run(s) in {secs:.1f} s")
        out["cpu_baseline"] = {"value": v, "unit": "elem/s", "cores": thr, "kind": "port",
                               "sample": sample}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def reference_arm(args, rank, world):
    """The reference algorithm's CPU path (oracle restatement, all host
    threads) on bounded samples of the same workload; rank 0 only."""
    if rank != 0:
        return
    log_rows = 16
    served = args.workload == "served"
    for _ in range(max(args.warmup, 1)):
        if served:
            cpu_served_sample(args, cap_log_h=10)
        else:
            cpu_trace_sample(12, args.cols, args.log_blowup, args.queries)
    vals, secs, elems = [], 0.0, 0
    for _ in range(args.steps):
        if served:
            v, s, thr, e = cpu_served_sample(args, cap_log_h=REF_CAP_LOG_H)
        else:
            v, s, thr = cpu_trace_sample(log_rows, args.cols, args.log_blowup, args.queries)
            e = args.cols << log_rows
        vals.append(v)
        secs += s
        elems += e
    value = elems / secs
    out = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "elem/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs / len(vals) * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32 (BabyBear, Montgomery)",
        "data": "synthetic: seeded uniform [0, p) canonical BabyBear elements",
        "config": {"workload": (f"served stream sample: the {args.requests}-request stream with "
                                f"heights capped at 2^{REF_CAP_LOG_H}, per-polynomial "
                                "pair-leaf commitments" if served else
                                f"trace commit 2^{log_rows}x{args.cols} slice, blowup "
                                f"{1 << args.log_blowup}, row leaves, {args.queries} openings")},
        "cpu_baseline": {"value": value, "unit": "elem/s", "cores": thr, "kind": "port",
                         "sample": ("each step: every request of the served stream, height capped "
                                    f"at 2^{REF_CAP_LOG_H}, incl. fold-and-open" if served else
                                    f"2^{log_rows} x {args.cols} per step") +
                                   "; the reference is Python over FRX/hash-frx wheels absent "
                                   "here, so its C restatement (oracle/) runs instead"},
        "e2e": {"value": value, "unit": "elem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
