"""The tree driver's shape (ZC_LEVELWISE_MIN_LOG: the widest level that runs
as a fused subtree instead of one thread per node; ZC_SUBTREE_T: first-level
nodes per fused-subtree CTA) is a tuning choice that changes no byte: under
several shapes, each in its own process (the shape is read once per process),
the digest layers of plain Merkle commits and the bytes of a FRI commit-phase
proof equal those of the default shape in this process, which the other GPU
tests pin to the oracle."""

from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

# Trees of 2^3 .. 2^17 leaves (every split between level-wise launches, the
# fused subtree and its top), then a 12-round FRI commit phase from 2^16
# coefficients. Prints one hex digest over all outputs.
SCRIPT = r"""
import hashlib, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from zorch_gb300 import _lib
from zorch_gb300.coding import ReedSolomon
from zorch_gb300.commit import MerkleTree, Poseidon2
from zorch_gb300.field import BABYBEAR, to_device, to_host, to_mont
from zorch_gb300.pcs import FriParams, FriProver
from zorch_gb300.transcript import DuplexTranscript
torch.cuda.set_device(0)
_lib.check(_lib.lib().zc_init(0), "init")
h = hashlib.sha256()
perm = Poseidon2.builtin(BABYBEAR)
rng = np.random.default_rng(11)
for log_l in (3, 7, 9, 12, 14, 15, 17):
    x = rng.integers(0, BABYBEAR.p, size=(1 << log_l, 4), dtype=np.uint64).astype(np.uint32)
    _, layers = MerkleTree(perm).commit(to_mont(BABYBEAR, to_device(x)))
    h.update(to_host(layers.flat).tobytes())
code = ReedSolomon(1 << 16, 2, BABYBEAR, coset_shift=31, generator=31)
c = rng.integers(0, BABYBEAR.p, size=1 << 16, dtype=np.uint64).astype(np.uint32)
cw = code.encode(to_mont(BABYBEAR, to_device(c)))
proof, _, _ = FriProver(FriParams(code, MerkleTree(perm), 12, 20, 4)).commit_phase(
    cw, DuplexTranscript.new(perm))
h.update(proof.to_bytes())
torch.cuda.synchronize()
print(h.hexdigest())
"""


def _digest(env_shape: dict[str, str] | None) -> str:
    env = dict(os.environ)
    env.pop("ZC_LEVELWISE_MIN_LOG", None)
    env.pop("ZC_SUBTREE_T", None)
    if env_shape:
        env.update(env_shape)
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT)], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.strip().splitlines()[-1]


@pytest.fixture(scope="module")
def default_digest():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _digest(None)


@pytest.mark.parametrize("levelwise_log,subtree_t", [(8, 2), (10, 32), (13, 256), (16, 64),
                                                     (20, 128)])
def test_tree_shape_changes_no_byte(default_digest, levelwise_log, subtree_t):
    got = _digest({"ZC_LEVELWISE_MIN_LOG": str(levelwise_log), "ZC_SUBTREE_T": str(subtree_t)})
    assert got == default_digest, (levelwise_log, subtree_t)


def test_default_digest_is_deterministic(default_digest):
    assert hashlib.sha256(default_digest.encode()).hexdigest()  # a digest was produced
    assert _digest(None) == default_digest
