"""Host-side logic that needs no GPU: admission under the HBM budget, the
config-5 request stream, and the replicas' max-over-ranks timing on two gloo
ranks."""

from __future__ import annotations

import os
from collections import deque

import pytest


def test_stream_is_seeded_and_shaped():
    from zorch_gb300.serve import make_stream

    a = make_stream(200, 5, rate_hz=10.0)
    b = make_stream(200, 5, rate_hz=10.0)
    assert [(r.log_h, r.width, r.log_blowup, r.fold, r.arrival) for r in a] == \
        [(r.log_h, r.width, r.log_blowup, r.fold, r.arrival) for r in b]
    assert all(14 <= r.log_h <= 24 and 1 <= r.width <= 256 and r.log_blowup in (1, 2) for r in a)
    arr = [r.arrival for r in a]
    assert arr == sorted(arr) and arr[0] > 0
    assert 0.15 < sum(r.fold for r in a) / len(a) < 0.45


def test_admission_fifo_budget_and_rejection():
    from zorch_gb300.serve import Request, admit

    def req(i, arrival, log_h, width):
        return Request(i, arrival, log_h, width, 1, False, i)

    small = req(0, 0.0, 10, 1).footprint()
    q = deque([req(0, 0.0, 10, 1), req(1, 0.1, 10, 1), req(2, 0.2, 30, 256),
               req(3, 0.3, 10, 1), req(4, 5.0, 10, 1)])
    # budget for two small requests: FIFO up to the budget; a request larger than
    # the whole budget can never fit, so it is rejected rather than blocking the queue
    ready, rej, used = admit(q, 1.0, 0, 2 * small, 8)
    assert [r.rid for r in ready] == [0, 1] and used == 2 * small
    assert [r.rid for r in rej] == [2] and q[0].rid == 3
    # memory freed: the next arrived request is admitted
    ready, rej, used = admit(q, 1.0, 0, 2 * small, 8)
    assert not rej and [r.rid for r in ready] == [3]
    # not yet arrived
    ready, rej, used = admit(q, 1.0, 0, 1e18, 8)
    assert not ready and [r.rid for r in q] == [4]
    # max_batch caps one admission
    q = deque([req(i, 0.0, 10, 1) for i in range(10)])
    ready, _, _ = admit(q, 0.0, 0, 1e18, 3)
    assert len(ready) == 3 and len(q) == 7


def test_admission_shortest_work_first_with_aging():
    from zorch_gb300.serve import Request, admit_sjf, request_work

    def req(i, arrival, log_h, width, fold=False):
        return Request(i, arrival, log_h, width, 1, fold, i)

    big, mid, tiny = req(0, 0.0, 20, 64), req(1, 0.1, 16, 8), req(2, 0.2, 12, 1)
    assert request_work(tiny) < request_work(mid) < request_work(big)
    # the least work first; one size class per batch (big is not batched with tiny)
    q = deque([big, mid, tiny, req(3, 9.0, 10, 1)])
    ready, rej, used = admit_sjf(q, 1.0, 0, 1e18, 8)
    assert [r.rid for r in ready] == [2] and not rej
    assert [r.rid for r in q] == [0, 1, 3]
    ready, _, _ = admit_sjf(q, 1.0, 0, 1e18, 8)
    assert [r.rid for r in ready] == [1]
    # a request that has waited longer than max_wait goes first
    q = deque([big, req(4, 2.5, 12, 1)])
    ready, _, _ = admit_sjf(q, 3.0, 0, 1e18, 8, max_wait=2.0)
    assert [r.rid for r in ready] == [0]
    # the head does not fit the budget: nothing is admitted, nothing overtakes it
    q = deque([big, req(5, 0.0, 12, 1)])
    ready, _, used = admit_sjf(q, 3.0, 0, big.footprint() + 1, 8, max_wait=2.0, )
    assert [r.rid for r in ready] == [0]
    ready, _, _ = admit_sjf(q, 3.0, used, big.footprint() + 1, 8, max_wait=0.0)
    assert not ready
    # larger than the whole budget: rejected
    q = deque([req(6, 0.0, 30, 256), req(7, 0.0, 10, 1)])
    ready, rej, _ = admit_sjf(q, 1.0, 0, 1e12, 8)
    assert [r.rid for r in rej] == [6] and [r.rid for r in ready] == [7] and not q


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    out[rank] = bench.max_over_ranks(1.0 + rank, device="cpu")
    dist.destroy_process_group()


def test_max_over_ranks_gloo_two_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    import random

    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = random.randint(20000, 40000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert dict(out) == {0: 2.0, 1: 2.0}


def test_autotuner_cache_reads_old_and_new_entries(tmp_path):
    """The tuning cache maps a (log_n, log2 width) bucket to its choices; a
    bare integer (a tile choice alone) still reads, unknown buckets give the
    library defaults (0), and a save/load round trip keeps every field."""
    import json

    from zorch_gb300.batch import Autotuner, _bucket

    path = tmp_path / "tune.json"
    path.write_text(json.dumps({"20:3": 13, "22:6": {"tile": 15, "radix": 3, "top": 7}}))
    t = Autotuner(path)
    assert t.choice(20, 8) == {"tile": 13, "radix": 0, "top": 0}
    assert t.choice(22, 64) == {"tile": 15, "radix": 3, "top": 7}
    assert t.choice(22, 100) == {"tile": 15, "radix": 3, "top": 7}   # same log2-width bucket
    assert t.choice(18, 1) == {"tile": 0, "radix": 0, "top": 0}
    assert t.tile_log(22, 64) == 15
    t.table[_bucket(16, 2)] = {"tile": 14, "radix": 4, "top": 6}
    t.save()
    again = Autotuner(path)
    assert again.choice(16, 3) == {"tile": 14, "radix": 4, "top": 6}
    path.write_text("not json")
    assert Autotuner(path).choice(16, 3) == {"tile": 0, "radix": 0, "top": 0}


def test_batch_committer_choice_prefers_overrides():
    from zorch_gb300.batch import Autotuner, BatchCommitter

    class Fixed(Autotuner):
        def __init__(self):
            self.table = {}

        def choice(self, log_n, width):
            return {"tile": 13, "radix": 3, "top": 6}

    bc = BatchCommitter.__new__(BatchCommitter)
    bc.tuner, bc.tile_override, bc.radix_override, bc.top_override = Fixed(), 0, 4, 0
    assert bc._choice(20, 8) == {"tile": 13, "radix": 4, "top": 6}
    bc.tuner = None
    assert bc._choice(20, 8) == {"tile": 0, "radix": 4, "top": 0}


def test_batch_committer_routes_large_jobs_to_single_matrix_kernels():
    """Jobs whose codeword reaches direct_min_words words take the single-matrix
    kernels, in job order; the rest stay on the work lists; 0 turns it off."""
    import torch

    from zorch_gb300.batch import BatchCommitter, MatrixJob

    bc = BatchCommitter.__new__(BatchCommitter)
    bc.direct_min_words = 1 << 22
    jobs = [MatrixJob(torch.empty((w, 1 << lh), dtype=torch.int32), lb)
            for w, lh, lb in [(8, 20, 1), (3, 12, 2), (2, 19, 3), (1, 16, 1), (64, 15, 1)]]
    assert bc._split(jobs) == ([0, 2, 4], [1, 3])
    bc.direct_min_words = 0
    assert bc._split(jobs) == ([], [0, 1, 2, 3, 4])


def test_xla_ffi_shim_is_header_gated(tmp_path, monkeypatch):
    """libzc_xla.so is built only where xla/ffi/api/ffi.h is found; the
    committed handlers name the four custom-call targets."""
    from zorch_gb300 import build as zb

    monkeypatch.setenv("XLA_FFI_INCLUDE_DIR", str(tmp_path))
    if zb.xla_ffi_include_dir() is None:
        assert zb.build_xla() is None
    src = zb.XLA_SRC.read_text()
    for name in ("zc_rs_encode_ffi", "zc_merkle_commit_ffi", "zc_fri_fold_commit_ffi",
                 "zc_duplex_hop_ffi"):
        assert f"XLA_FFI_DEFINE_HANDLER_SYMBOL({name}," in src
