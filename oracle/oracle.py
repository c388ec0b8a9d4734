"""CPU ORACLE -- test infrastructure only.

numpy/ctypes front end over the C restatement in zc_oracle.c. Only the tests,
`__graft_entry__.smoke()` and the bench's CPU-baseline leg import this module;
the product (`zorch_gb300`) never does. Field values are Montgomery u32 (the
storage of zk_dtypes' *_mont dtypes), canonical values are converted with
`to_mont` / `from_mont`.

Parity: Poseidon2/sponge/compression/Merkle are pinned to the reference's
Plonky3 KoalaBear-16 golden (tests/golden/koalabear16.json); the bit-reversed
KoalaBear encode, the column-major commit and openings, the bit-reversed fold,
and the SP1 single-matrix commitment are pinned to the reference's SP1
pipeline dump (tests/golden/sp1_fibonacci). The BabyBear Poseidon2 instance is
project-defined, so BabyBear roots, challenges and proof bytes are "parity
unpinned vs reference" (oracle == CUDA only).
"""

from __future__ import annotations

import ctypes as C
import json
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import build as _build

BABYBEAR, KOALABEAR = 0, 1
P_BABYBEAR = 2013265921
P_KOALABEAR = 2130706433
MODULUS = {BABYBEAR: P_BABYBEAR, KOALABEAR: P_KOALABEAR}

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _load() -> C.CDLL:
    lib = C.CDLL(str(_build.build()))
    vp, i64, i32, u32 = C.c_void_p, C.c_int64, C.c_int, C.c_uint32
    sig = {
        "orc_set_threads": (None, [i32]),
        "orc_get_threads": (i32, []),
        "orc_modulus": (u32, [i32]),
        "orc_to_mont": (u32, [i32, u32]),
        "orc_from_mont": (u32, [i32, u32]),
        "orc_mul": (u32, [i32, u32, u32]),
        "orc_to_mont_vec": (None, [i32, _u32p, _u32p, i64]),
        "orc_from_mont_vec": (None, [i32, _u32p, _u32p, i64]),
        "orc_ef4_mul": (None, [i32, _u32p, _u32p, _u32p]),
        "orc_root_of_unity": (u32, [i32, i32, u32]),
        "orc_p2_size": (i32, []),
        "orc_p2_babybear16": (None, [vp]),
        "orc_p2_from_canonical": (None, [vp, i32, i32, i32, i32, _u32p, _u32p, _u32p, _u32p, u32]),
        "orc_p2_export_canonical": (None, [vp, _u32p, _u32p, _u32p, _u32p]),
        "orc_p2_permute": (None, [vp, _u32p]),
        "orc_sponge_hash": (None, [vp, _u32p, i64, _u32p]),
        "orc_compress": (None, [vp, _u32p, _u32p, _u32p]),
        "orc_merkle_commit": (i32, [vp, _u32p, i64, i32, i32, i64, _u32p]),
        "orc_merkle_open": (i32, [_u32p, i64, i32, i32, i64, _u32p, _i32p, i32, _u32p, _u32p]),
        "orc_rs_encode": (i32, [i32, _u32p, i64, i32, i32, u32, u32, _u32p]),
        "orc_rs_encode_horner": (i32, [i32, _u32p, i32, i32, u32, u32, _u32p]),
        "orc_eval_domain": (None, [i32, i32, u32, u32, _u32p]),
        "orc_eval_poly": (u32, [i32, _u32p, i64, u32]),
        "orc_domain_point": (u32, [i32, i32, u32, u32, i64]),
        "orc_fri_fold": (i32, [i32, _u32p, i64, i32, _u32p, i32, u32, u32, _u32p]),
        "orc_rs_encode_bitrev": (i32, [i32, _u32p, i64, i32, i32, u32, u32, _u32p]),
        "orc_fri_fold_bitrev": (i32, [i32, _u32p, i64, i32, _u32p, i32, u32, u32, _u32p]),
        "orc_smcs_bind_root": (None, [vp, _u32p, u32, u32, _u32p]),
        "orc_fri_fold_k": (i32, [i32, _u32p, i64, i32, _u32p, i32, i32, u32, u32, _u32p]),
        "orc_strided_merkle_commit": (i32, [vp, _u32p, i64, i32, i32, i64, i32, _u32p]),
        "orc_ef4_inv": (None, [i32, _u32p, _u32p]),
        "orc_eq_expand": (None, [i32, _u32p, i32, _u32p]),
        "orc_eval_mle_base": (None, [i32, _u32p, i32, i32, _u32p, _u32p]),
        "orc_eval_mle_ef4": (None, [i32, _u32p, i32, _u32p, _u32p]),
        "orc_mle_fold": (None, [i32, _u32p, i64, _u32p, _u32p]),
        "orc_rlc_columns_ex": (None, [i32, _u32p, i64, i32, _u32p, i32, i32, i32, _u32p]),
        "orc_duplex_init": (None, [vp]),
        "orc_duplex_observe": (None, [vp, vp, _u32p, i64]),
        "orc_duplex_sample": (None, [vp, vp, i32, _u32p]),
        "orc_duplex_grind": (u32, [vp, vp, i32]),
        "orc_rlc_columns": (None, [i32, _u32p, i64, i32, _u32p, _u32p]),
        "orc_fri_commit_phase": (i32, [vp, i32, _u32p, i32, i32, u32, u32, i32, i32, i32, vp,
                                       _u32p, _u32p, _u32p, _i32p, _u32p, _u32p]),
        "orc_eval_poly_ef4": (None, [i32, _u32p, i64, _u32p, _u32p]),
        "orc_deep_quotient": (i32, [i32, _u32p, i64, _u32p, i32, _u32p, u32, u32, i32, _u32p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


LIB = _load()


def set_threads(n: int) -> None:
    LIB.orc_set_threads(int(n))


def threads() -> int:
    return int(LIB.orc_get_threads())


def u32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def to_mont(field: int, x) -> np.ndarray:
    x = u32(x)
    out = np.empty_like(x)
    LIB.orc_to_mont_vec(field, x.reshape(-1), out.reshape(-1), x.size)
    return out


def from_mont(field: int, x) -> np.ndarray:
    x = u32(x)
    out = np.empty_like(x)
    LIB.orc_from_mont_vec(field, x.reshape(-1), out.reshape(-1), x.size)
    return out


def root_of_unity(field: int, log_n: int, generator: int = 0) -> int:
    return int(LIB.orc_root_of_unity(field, log_n, generator))


class Poseidon2:
    """A width-16 Poseidon2 parameterisation (constants stored Montgomery)."""

    def __init__(self) -> None:
        self._buf = C.create_string_buffer(int(LIB.orc_p2_size()))
        self.ptr = C.cast(self._buf, C.c_void_p)
        self.field = BABYBEAR

    @classmethod
    def babybear16(cls) -> "Poseidon2":
        p = cls()
        LIB.orc_p2_babybear16(p.ptr)
        p.field = BABYBEAR
        p.alpha, p.rounds_f_half, p.rounds_p = 7, 4, 13
        return p

    @classmethod
    def from_canonical(cls, field, alpha, ext_init, ext_term, int_rc, diag, j_scale=1):
        p = cls()
        ext_init, ext_term = u32(ext_init).reshape(-1), u32(ext_term).reshape(-1)
        int_rc, diag = u32(int_rc), u32(diag)
        LIB.orc_p2_from_canonical(p.ptr, field, alpha, ext_init.size // 16, int_rc.size,
                                  ext_init, ext_term, int_rc, diag, j_scale)
        p.field, p.alpha = field, alpha
        p.rounds_f_half, p.rounds_p = ext_init.size // 16, int_rc.size
        return p

    @classmethod
    def koalabear16_golden(cls) -> "Poseidon2":
        d = load_koalabear_fixture()
        return cls.from_canonical(KOALABEAR, d["alpha"], d["external_initial"],
                                  d["external_terminal"], d["internal_rc"],
                                  d["internal_diag"], d["internal_j_scale"])

    def export_canonical(self):
        ei = np.zeros(self.rounds_f_half * 16, np.uint32)
        et = np.zeros(self.rounds_f_half * 16, np.uint32)
        ir = np.zeros(self.rounds_p, np.uint32)
        dg = np.zeros(16, np.uint32)
        LIB.orc_p2_export_canonical(self.ptr, ei, et, ir, dg)
        return ei.reshape(-1, 16), et.reshape(-1, 16), ir, dg

    def permute(self, state) -> np.ndarray:
        s = u32(state).copy()
        LIB.orc_p2_permute(self.ptr, s)
        return s

    def hash(self, row) -> np.ndarray:
        row = u32(row).reshape(-1)
        out = np.zeros(8, np.uint32)
        LIB.orc_sponge_hash(self.ptr, row, row.size, out)
        return out

    def compress(self, left, right) -> np.ndarray:
        out = np.zeros(8, np.uint32)
        LIB.orc_compress(self.ptr, u32(left), u32(right), out)
        return out


GOLDEN = Path(__file__).resolve().parent.parent / "tests" / "golden"


def load_koalabear_fixture() -> dict:
    return json.loads((GOLDEN / "koalabear16.json").read_text())


def load_sp1_fixture() -> dict:
    """SP1's KoalaBear-16 instance (zorch/commit/testing/sp1_koalabear16.py)."""
    return json.loads((GOLDEN / "sp1_fibonacci" / "sp1_koalabear16.json").read_text())


def sp1_koalabear16() -> "Poseidon2":
    d = load_sp1_fixture()
    return Poseidon2.from_canonical(KOALABEAR, d["alpha"], d["external_initial"],
                                    d["external_terminal"], d["internal_rc"],
                                    d["internal_diag"], d["internal_j_scale"])


def smcs_bind_root(p2: Poseidon2, raw_root, log_height: int, width: int) -> np.ndarray:
    """SingleMatrixCommitmentScheme.bind_root (zorch/commit/smcs.py:118-140)."""
    out = np.zeros(8, np.uint32)
    LIB.orc_smcs_bind_root(p2.ptr, u32(raw_root).reshape(-1), log_height, width, out)
    return out


# ------------------------------------------------------------------ Merkle --
def merkle_commit(p2: Poseidon2, base: np.ndarray, num_leaves: int, groups: int, g: int,
                  gstride: int) -> list[np.ndarray]:
    """Generalised leaf layout: leaf p = concat_q base[q*gstride + p*g : +g]."""
    base = u32(base).reshape(-1)
    layers = np.zeros((2 * num_leaves - 1) * 8, np.uint32)
    rc = LIB.orc_merkle_commit(p2.ptr, base, num_leaves, groups, g, gstride, layers)
    if rc:
        raise ValueError(f"merkle_commit failed ({rc})")
    out, off, n = [], 0, num_leaves
    while True:
        out.append(layers[8 * off: 8 * (off + n)].reshape(n, 8))
        if n == 1:
            break
        off += n
        n //= 2
    return out


def strided_merkle_commit(p2: Poseidon2, matrix: np.ndarray, rows_per_query: int):
    """StridedMerkleTree.commit of a row-major [height, w] matrix
    (zorch/commit/strided_merkle.py:100-152): stored layers from the query
    layer (height / rows_per_query nodes) to the root."""
    m = u32(matrix)
    h, w = m.shape
    s = h // rows_per_query
    flat = np.zeros((2 * s - 1) * 8, np.uint32)
    rc = LIB.orc_strided_merkle_commit(p2.ptr, m.reshape(-1), h, 1, w, 0, rows_per_query, flat)
    if rc:
        raise ValueError("strided commit needs power-of-two height and rows_per_query <= height")
    out, off, n = [], 0, s
    while True:
        out.append(flat[8 * off: 8 * (off + n)].reshape(n, 8))
        if n == 1:
            break
        off += n
        n //= 2
    return out


def merkle_commit_rows(p2: Poseidon2, matrix: np.ndarray) -> list[np.ndarray]:
    """Row-major leaves `(L, w)` (MerkleTree.commit)."""
    m = u32(matrix)
    return merkle_commit(p2, m, m.shape[0], 1, m.shape[1], 0)


def merkle_commit_columns(p2: Poseidon2, cols: np.ndarray) -> list[np.ndarray]:
    """Column-major leaves `(w, L)`: leaf r = cols[:, r] (codeword.T rows)."""
    m = u32(cols)
    return merkle_commit(p2, m, m.shape[1], m.shape[0], 1, m.shape[1])


def merkle_open(base, num_leaves, groups, g, gstride, layers: list[np.ndarray], idx):
    flat = np.concatenate([l.reshape(-1) for l in layers])
    idx = np.ascontiguousarray(np.asarray(idx, np.int32))
    depth = len(layers) - 1
    rows = np.zeros((idx.size, groups * g), np.uint32)
    paths = np.zeros((max(depth, 0), idx.size, 8), np.uint32)
    rc = LIB.orc_merkle_open(u32(base).reshape(-1), num_leaves, groups, g, gstride, flat, idx,
                             idx.size, rows, paths)
    if rc:
        raise IndexError("merkle_open index out of range")
    return rows, paths


# ---------------------------------------------------------------------- RS --
def rs_encode(field: int, coeffs: np.ndarray, log_blowup: int, shift_mont: int = 0,
              generator: int = 0) -> np.ndarray:
    c = u32(coeffs)
    batch_shape = c.shape[:-1]
    k = c.shape[-1]
    log_k = k.bit_length() - 1
    batch = int(np.prod(batch_shape)) if batch_shape else 1
    out = np.zeros((batch, k << log_blowup), np.uint32)
    rc = LIB.orc_rs_encode(field, c.reshape(-1), batch, log_k, log_blowup, shift_mont,
                           generator, out.reshape(-1))
    if rc:
        raise ValueError(f"rs_encode failed ({rc})")
    return out.reshape(*batch_shape, k << log_blowup)


def rs_encode_bitrev(field: int, coeffs: np.ndarray, log_blowup: int, shift_mont: int = 0,
                     generator: int = 0) -> np.ndarray:
    """BitReversedReedSolomon.encode (zorch/coding/reed_solomon.py:476-478)."""
    c = u32(coeffs)
    batch_shape = c.shape[:-1]
    k = c.shape[-1]
    batch = int(np.prod(batch_shape)) if batch_shape else 1
    out = np.zeros((batch, k << log_blowup), np.uint32)
    rc = LIB.orc_rs_encode_bitrev(field, c.reshape(-1), batch, k.bit_length() - 1, log_blowup,
                                  shift_mont, generator, out.reshape(-1))
    if rc:
        raise ValueError(f"rs_encode_bitrev failed ({rc})")
    return out.reshape(*batch_shape, k << log_blowup)


def rs_encode_horner(field, coeffs, log_blowup, shift_mont=0, generator=0) -> np.ndarray:
    c = u32(coeffs)
    k = c.size
    out = np.zeros(k << log_blowup, np.uint32)
    LIB.orc_rs_encode_horner(field, c, k.bit_length() - 1, log_blowup, shift_mont, generator, out)
    return out


def eval_poly(field: int, coeffs, x: int) -> int:
    c = u32(coeffs).reshape(-1)
    return int(LIB.orc_eval_poly(field, c, c.size, x))


def domain_point(field: int, log_n: int, shift_mont: int, j: int, generator: int = 0) -> int:
    return int(LIB.orc_domain_point(field, log_n, shift_mont, generator, j))


def reconstruct_root(p2: "Poseidon2", row, index: int, path) -> np.ndarray:
    """Rebuild a root from an opened row and its sibling path (leaf first),
    MerkleTree.reconstruct_root (zorch/commit/merkle.py:264-285)."""
    node = p2.hash(row)
    for sib in path:
        node = p2.compress(node, sib) if index % 2 == 0 else p2.compress(sib, node)
        index //= 2
    return node


def eval_domain(field: int, log_n: int, shift_mont: int = 0, generator: int = 0) -> np.ndarray:
    out = np.zeros(1 << log_n, np.uint32)
    LIB.orc_eval_domain(field, log_n, shift_mont, generator, out)
    return out


def fri_fold(field, cw, ef_in: bool, beta, ef_beta: bool, shift_mont=0, generator=0):
    cw = u32(cw)
    n = cw.shape[0]
    lo = 4 if (ef_in or ef_beta) else 1
    out = np.zeros((n // 2, lo) if lo == 4 else (n // 2,), np.uint32)
    b = np.zeros(4, np.uint32)
    b[: (4 if ef_beta else 1)] = u32(beta).reshape(-1)[: (4 if ef_beta else 1)]
    rc = LIB.orc_fri_fold(field, cw.reshape(-1), n, int(ef_in), b, int(ef_beta), shift_mont,
                          generator, out.reshape(-1))
    if rc:
        raise ValueError("fri_fold needs a power-of-two length >= 2")
    return out


def fri_fold_bitrev(field, cw, ef_in: bool, beta, ef_beta: bool, shift_mont=0, generator=0):
    """BitReversedReedSolomon.fold (zorch/coding/reed_solomon.py:484-492)."""
    cw = u32(cw)
    n = cw.shape[0]
    lo = 4 if (ef_in or ef_beta) else 1
    out = np.zeros((n // 2, lo) if lo == 4 else (n // 2,), np.uint32)
    b = np.zeros(4, np.uint32)
    b[: (4 if ef_beta else 1)] = u32(beta).reshape(-1)[: (4 if ef_beta else 1)]
    rc = LIB.orc_fri_fold_bitrev(field, cw.reshape(-1), n, int(ef_in), b, int(ef_beta),
                                 shift_mont, generator, out.reshape(-1))
    if rc:
        raise ValueError("fri_fold_bitrev needs a power-of-two length >= 2")
    return out


def fri_fold_k(field, cw, ef_in: bool, beta, ef_beta: bool, log_k: int, shift_mont=0,
               generator=0):
    """ReedSolomon.fold_group (zorch/coding/reed_solomon.py:357-381)."""
    cw = u32(cw)
    n = cw.shape[0]
    lo = 4 if (ef_in or ef_beta) else 1
    out = np.zeros((n >> log_k, lo) if lo == 4 else (n >> log_k,), np.uint32)
    b = np.zeros(4, np.uint32)
    b[: (4 if ef_beta else 1)] = u32(beta).reshape(-1)[: (4 if ef_beta else 1)]
    rc = LIB.orc_fri_fold_k(field, cw.reshape(-1), n, int(ef_in), b, int(ef_beta), log_k,
                            shift_mont, generator, out.reshape(-1))
    if rc:
        raise ValueError("fri_fold_k needs a power-of-two length >= k")
    return out


def bit_reverse(j: int, bits: int) -> int:
    return int(format(int(j), f"0{bits}b")[::-1], 2) if bits else 0


def sp1_query_positions(raw, block_len: int) -> np.ndarray:
    """SP1's sample_bits rule (zorch/pcs/jagged/open.py:116-125): the CANONICAL
    value of each squeeze masked to log2(block_len) low bits."""
    return (u32(raw) & np.uint32(block_len - 1)).astype(np.int32)


def sp1_stacked_fold_chain(p2: Poseidon2, field: int, codeword, betas, shift_mont: int = 0):
    """The commit/fold half of the stacked BaseFold open's fold loop
    (zorch/pcs/jagged/open.py:262-296) with the betas given (as the reference's
    byte-match replays them): per round, the EF4 bit-reversed layer viewed as
    [n/2, 8] base rows is committed through the SP1 SMCS (raw root, bound root)
    and folded with the round's beta. Returns (raw_roots, bound_roots, layers,
    final_codeword); layers[i] = (rows [n_i/2, 8], digest layers)."""
    cw = u32(codeword).reshape(-1, 4)
    raw, bound, layers = [], [], []
    for beta in u32(betas).reshape(-1, 4):
        n = cw.shape[0]
        leaves = cw.reshape(n // 2, 8)
        dl = merkle_commit_rows(p2, leaves)
        raw.append(dl[-1][0])
        bound.append(smcs_bind_root(p2, dl[-1][0], (n // 2).bit_length() - 1, 8))
        layers.append((leaves, dl))
        cw = fri_fold_bitrev(field, cw, True, beta, True, shift_mont)
        shift_mont = LIB.orc_mul(field, shift_mont, shift_mont) if shift_mont else 0
    return np.stack(raw), np.stack(bound), layers, cw


# -------------------------------------------------------------- transcript --
class Duplex(C.Structure):
    _fields_ = [("in_buf", C.c_uint32 * 8), ("out_buf", C.c_uint32 * 8),
                ("sponge", C.c_uint32 * 16), ("in_pos", C.c_int32), ("out_pos", C.c_int32)]

    def wire(self) -> tuple[np.ndarray, ...]:
        return (np.array(self.in_buf, np.uint32), np.array(self.out_buf, np.uint32),
                np.array(self.sponge, np.uint32), np.array([self.in_pos], np.int32).view(np.uint32),
                np.array([self.out_pos], np.int32).view(np.uint32))


class Transcript:
    def __init__(self, p2: Poseidon2) -> None:
        self.p2 = p2
        self.st = Duplex()
        LIB.orc_duplex_init(C.byref(self.st))

    def observe(self, values) -> "Transcript":
        v = u32(values).reshape(-1)
        LIB.orc_duplex_observe(self.p2.ptr, C.byref(self.st), v, v.size)
        return self

    def sample(self, n: int = 1) -> np.ndarray:
        out = np.zeros(max(n, 1), np.uint32)
        LIB.orc_duplex_sample(self.p2.ptr, C.byref(self.st), n, out)
        return out[:n]

    def copy(self) -> "Transcript":
        t = Transcript(self.p2)
        t.st = Duplex.from_buffer_copy(self.st)
        return t

    def grind(self, pow_bits: int) -> int:
        """Lowest canonical proof-of-work witness (zorch/transcript.py:439-481);
        the transcript is not advanced (observe the witness and sample once,
        as check_witness does)."""
        if not 0 <= pow_bits < 32:
            raise ValueError(f"pow_bits must be in [0, 32), got {pow_bits}")
        return int(LIB.orc_duplex_grind(self.p2.ptr, C.byref(self.st), pow_bits))

    def check_witness(self, witness_mont: int, pow_bits: int) -> bool:
        """Observe the witness (Montgomery word), sample once, test the low
        `pow_bits` canonical bits (zorch/transcript.py:417-437)."""
        self.observe([witness_mont])
        s = int(self.sample(1)[0])
        return (from_mont(self.p2.field, [s])[0] & ((1 << pow_bits) - 1)) == 0


# ------------------------------------------------------- FRI commit phase --
@dataclass
class CommitPhaseProof:
    roots: np.ndarray          # (R, 8)
    betas: np.ndarray          # (R, 4) (limb 0 only for base challenges)
    final_layer: np.ndarray    # (n_R, limbs)
    positions: np.ndarray      # (Q,)
    rows: list[np.ndarray]     # per layer (Q, 2*limbs_i)
    paths: list[np.ndarray]    # per layer (depth_i, Q, 8)

    def to_bytes(self) -> bytes:
        parts = [self.roots, self.final_layer]
        for r, p in zip(self.rows, self.paths):
            parts += [r, p]
        return b"".join(np.ascontiguousarray(x, dtype="<u4").tobytes() for x in parts)


def rlc_columns(field: int, cw, challenges) -> np.ndarray:
    """Partial-Lagrange batching; `challenges` = ceil(log2 w) EF4 values (4 words each)."""
    cw = u32(cw)
    w, n = cw.shape
    out = np.zeros((n, 4), np.uint32)
    ch = u32(challenges).reshape(-1)
    LIB.orc_rlc_columns(field, cw.reshape(-1), n, w, ch if ch.size else np.zeros(4, np.uint32),
                        out.reshape(-1))
    return out


def layer_limbs(num_rounds: int, beta_limbs: int, ef_in: bool = False) -> list[int]:
    limbs = [4 if ef_in else 1]
    for _ in range(num_rounds):
        limbs.append(4 if (limbs[-1] == 4 or beta_limbs == 4) else 1)
    return limbs


def fri_commit_phase(p2: Poseidon2, field: int, codeword, num_rounds: int, num_queries: int,
                     beta_limbs: int, transcript: Transcript, shift_mont=0, generator=0):
    cw = u32(codeword)
    ef_in = cw.ndim == 2
    n0 = cw.shape[0]
    cw = cw.reshape(-1)
    log_n = n0.bit_length() - 1
    limbs = layer_limbs(num_rounds, beta_limbs, ef_in)
    roots = np.zeros((num_rounds, 8), np.uint32)
    betas = np.zeros((num_rounds, 4), np.uint32)
    nf = n0 >> num_rounds
    final = np.zeros((nf, limbs[-1]), np.uint32)
    pos = np.zeros(num_queries, np.int32)
    row_sizes = [num_queries * 2 * limbs[r] for r in range(num_rounds)]
    depths = [log_n - 1 - r for r in range(num_rounds)]
    path_sizes = [d * num_queries * 8 for d in depths]
    rows = np.zeros(max(sum(row_sizes), 1), np.uint32)
    paths = np.zeros(max(sum(path_sizes), 1), np.uint32)
    rc = LIB.orc_fri_commit_phase(p2.ptr, field, cw, log_n, int(ef_in), shift_mont, generator,
                                  num_rounds,
                                  num_queries, beta_limbs, C.byref(transcript.st), roots.reshape(-1),
                                  betas.reshape(-1), final.reshape(-1), pos, rows, paths)
    if rc:
        raise ValueError(f"fri_commit_phase failed ({rc})")
    rl, pl, ro, po = [], [], 0, 0
    for r in range(num_rounds):
        rl.append(rows[ro: ro + row_sizes[r]].reshape(num_queries, 2 * limbs[r]))
        pl.append(paths[po: po + path_sizes[r]].reshape(depths[r], num_queries, 8))
        ro += row_sizes[r]
        po += path_sizes[r]
    return CommitPhaseProof(roots, betas, final, pos, rl, pl)


# ---------------------------------------------------------------- FRI open --
def eval_poly_at(field: int, coeffs, z) -> np.ndarray:
    """f(z) (_eval_poly, zorch/pcs/fri/prover.py:42-49) for a base point
    (1 word) or an EF4 point (4 words); Montgomery words in and out."""
    c = u32(coeffs).reshape(-1)
    z = u32(z).reshape(-1)
    if z.size == 1:
        return np.array([LIB.orc_eval_poly(field, c, c.size, int(z[0]))], np.uint32)
    out = np.zeros(4, np.uint32)
    LIB.orc_eval_poly_ef4(field, c, c.size, z, out)
    return out


def deep_quotient(field: int, cw, z, v, shift_mont: int = 0, generator: int = 0,
                  bit_reversed: bool = False) -> np.ndarray:
    """(cw - v) / (domain - z) (zorch/pcs/fri/prover.py:164): [n] for a base
    point, [n, 4] for an EF4 point."""
    cw = u32(cw).reshape(-1)
    z = u32(z).reshape(-1)
    v = u32(v).reshape(-1)
    limbs = z.size
    out = np.zeros(cw.size * limbs, np.uint32)
    rc = LIB.orc_deep_quotient(field, cw, cw.size, z, limbs, v, shift_mont, generator,
                               int(bit_reversed), out)
    if rc:
        raise ValueError(f"deep_quotient failed ({rc})")
    return out if limbs == 1 else out.reshape(-1, 4)


@dataclass
class FriOpenProof:
    """FriProof (zorch/pcs/fri/config.py:56-69) in pytree flatten order:
    value, fri_roots, final_layer, f_opening (row, path), query openings."""

    value: np.ndarray
    phase: CommitPhaseProof
    f_rows: np.ndarray
    f_paths: np.ndarray

    def to_bytes(self) -> bytes:
        parts = [self.value, self.phase.roots, self.phase.final_layer, self.f_rows, self.f_paths]
        for r, p in zip(self.phase.rows, self.phase.paths):
            parts += [r, p]
        return b"".join(np.ascontiguousarray(x, dtype="<u4").tobytes() for x in parts)


def fri_open(p2: Poseidon2, field: int, coeffs, codeword, f_layers, z, num_rounds: int,
             num_queries: int, beta_limbs: int, transcript: Transcript, shift_mont: int = 0,
             generator: int = 0) -> FriOpenProof:
    """_open_one (zorch/pcs/fri/prover.py:151-187) on a natural-order
    codeword with its committed pair-leaf layers: v = f(z); the DEEP quotient
    layer; observe f's root; the fold rounds, final layer and positions
    (fri_commit_phase); f's pair leaf opened at each position mod n/2.
    `transcript` is advanced in place."""
    cw = u32(codeword).reshape(-1)
    n = cw.size
    v = eval_poly_at(field, coeffs, z)
    q = deep_quotient(field, cw, z, v, shift_mont, generator)
    transcript.observe(f_layers[-1][0])
    phase = fri_commit_phase(p2, field, q, num_rounds, num_queries, beta_limbs, transcript,
                             shift_mont, generator)
    a0 = (phase.positions.astype(np.int64) % (n // 2)).astype(np.int32)
    rows, paths = merkle_open(cw, n // 2, 2, 1, n // 2, f_layers, a0)
    return FriOpenProof(v, phase, rows, paths)


# ------------------------------------------------------------ basefold open --
def ef4_mul(field: int, a, b) -> np.ndarray:
    out = np.zeros(4, np.uint32)
    LIB.orc_ef4_mul(field, u32(a).reshape(-1), u32(b).reshape(-1), out)
    return out


def ef4_inv(field: int, a) -> np.ndarray:
    out = np.zeros(4, np.uint32)
    LIB.orc_ef4_inv(field, u32(a).reshape(-1), out)
    return out


def ef4_add(field: int, a, b) -> np.ndarray:
    p = MODULUS[field]
    return ((u32(a).astype(np.uint64) + u32(b).astype(np.uint64)) % p).astype(np.uint32)


def ef4_sub(field: int, a, b) -> np.ndarray:
    p = MODULUS[field]
    return ((u32(a).astype(np.uint64) + p - u32(b).astype(np.uint64)) % p).astype(np.uint32)


def eq_expand(field: int, z) -> np.ndarray:
    z = u32(z).reshape(-1, 4)
    out = np.zeros((1 << z.shape[0], 4), np.uint32)
    LIB.orc_eq_expand(field, z.reshape(-1), z.shape[0], out.reshape(-1))
    return out


def eval_mle_base(field: int, cols, z) -> np.ndarray:
    """eval_mle of base columns [w, 2^m] at the EF4 point z [m, 4] -> [w, 4]."""
    cols = u32(cols)
    z = u32(z).reshape(-1, 4)
    out = np.zeros((cols.shape[0], 4), np.uint32)
    LIB.orc_eval_mle_base(field, cols.reshape(-1), cols.shape[0], z.shape[0], z.reshape(-1),
                          out.reshape(-1))
    return out


def eval_mle_ef4(field: int, mle, z) -> np.ndarray:
    mle = u32(mle).reshape(-1, 4)
    z = u32(z).reshape(-1, 4)
    out = np.zeros(4, np.uint32)
    LIB.orc_eval_mle_ef4(field, mle.reshape(-1), z.shape[0],
                         z.reshape(-1) if z.size else np.zeros(4, np.uint32), out)
    return out


def mle_fold(field: int, mle, beta) -> np.ndarray:
    mle = u32(mle).reshape(-1, 4)
    b = np.zeros(4, np.uint32)
    bb = u32(beta).reshape(-1)
    b[: bb.size] = bb
    out = np.zeros((mle.shape[0] // 2, 4), np.uint32)
    LIB.orc_mle_fold(field, mle.reshape(-1), mle.shape[0], b, out.reshape(-1))
    return out


def basefold_open(p2: Poseidon2, field: int, mats, z, log_blowup: int, shift_mont: int,
                  num_queries: int, t: "Transcript") -> dict:
    """BasefoldProver.open_batch over committed base-field matrices at the EF4
    point z, the native wire (zorch/pcs/basefold/prover.py:215-247, 503-547,
    419-480; kernel zorch/pcs/basefold/kernel.py:52-78; choreography
    zorch/pcs/fold.py:277-299, 385-389):
    observe each root -> observe each matrix's eval_mle values -> sample
    ceil(log2 total width) batch challenges (base, as EF4) -> staggered
    partial-Lagrange batching of MLEs, codewords and values -> observe the
    round count (EF4) -> per round: message (s(0), s(1)) observed, pre-fold
    pair leaves committed and the root observed, beta = one base squeeze, fold
    codeword / MLE / claim -> observe the final codeword -> query positions
    (Montgomery bits mod n) -> open every matrix and every fold layer.
    mats: dicts with cols [w, S], codeword [w, n] (column-major, base) and
    layers (digest layers of the row leaves)."""
    z = u32(z).reshape(-1, 4)
    v = z.shape[0]
    S = 1 << v
    n = S << log_blowup
    one = np.zeros(4, np.uint32)
    one[0] = to_mont(field, [1])[0]
    for m in mats:
        t.observe(m["layers"][-1][0])
    values = []
    for m in mats:
        vals = eval_mle_base(field, m["cols"], z)
        t.observe(vals.reshape(-1))
        values.append(vals)
    total = sum(int(m["cols"].shape[0]) for m in mats)
    nbv = (total - 1).bit_length() if total > 1 else 0
    chal = np.zeros((max(nbv, 1), 4), np.uint32)
    if nbv:
        chal[:nbv, 0] = t.sample(nbv)
    mle = np.zeros((S, 4), np.uint32)
    cw = np.zeros((n, 4), np.uint32)
    off = 0
    for m in mats:
        w = int(m["cols"].shape[0])
        LIB.orc_rlc_columns_ex(field, u32(m["cols"]).reshape(-1), S, w, chal.reshape(-1), nbv, off,
                               int(off > 0), mle.reshape(-1))
        LIB.orc_rlc_columns_ex(field, u32(m["codeword"]).reshape(-1), n, w, chal.reshape(-1), nbv,
                               off, int(off > 0), cw.reshape(-1))
        off += w
    wt = eq_expand(field, chal[:nbv])
    claim = np.zeros(4, np.uint32)
    for c, val in enumerate(np.concatenate(values)):
        claim = ef4_add(field, claim, ef4_mul(field, wt[c], val))
    vm = np.zeros(4, np.uint32)
    vm[0] = to_mont(field, [v])[0]
    t.observe(vm)
    msgs, roots, betas, layers = [], [], [], []
    sh = shift_mont
    for i in range(v):
        zs = z[: v - i]
        s0 = eval_mle_ef4(field, mle[0::2], zs[:-1])
        s1 = ef4_add(field, ef4_mul(field, ef4_sub(field, claim, s0), ef4_inv(field, zs[-1])), s0)
        msg = np.concatenate([s0, s1])
        t.observe(msg)
        N = cw.shape[0]
        dl = merkle_commit(p2, cw, N // 2, 2, 4, (N // 2) * 4)
        t.observe(dl[-1][0])
        beta = t.sample(1)[0]
        layers.append((cw, dl))
        msgs.append(msg)
        roots.append(dl[-1][0])
        betas.append(beta)
        cw = fri_fold(field, cw, True, [beta], False, sh)
        mle = mle_fold(field, mle, [beta])
        claim = ef4_add(field, s0, ef4_mul(field, np.array([beta, 0, 0, 0], np.uint32), s1))
        sh = int(LIB.orc_mul(field, sh, sh)) if sh else 0
    final = cw
    t.observe(final.reshape(-1))
    positions = (t.sample(num_queries) % np.uint32(n)).astype(np.int32)
    comp = []
    for m in mats:
        w = int(m["cols"].shape[0])
        comp.append(merkle_open(m["codeword"], n, w, 1, n, m["layers"], positions))
    queries = []
    for i, (lcw, dl) in enumerate(layers):
        N = lcw.shape[0]
        a = (positions % (N // 2)).astype(np.int32)
        queries.append(merkle_open(lcw, N // 2, 2, 4, (N // 2) * 4, dl, a))
    return {"values": values, "uni_msgs": np.stack(msgs) if msgs else np.zeros((0, 8), np.uint32),
            "fri_roots": np.stack(roots) if roots else np.zeros((0, 8), np.uint32),
            "betas": np.array(betas, np.uint32), "final_poly": final, "positions": positions,
            "component_openings": comp, "query_openings": queries, "final_claim": claim}


def sp1_stacked_open(p2: Poseidon2, field: int, blocks, z_final, dense_eval, log_s: int,
                     log_blowup: int, num_queries: int, t: "Transcript",
                     pow_bits: int = 0) -> dict:
    """stacked_basefold_open (zorch/pcs/jagged/open.py:362-460; prologue
    :185-229, fold zone :237-330, queries :333-359): batch
    evaluations at the stacking point, dense_eval and evaluations observed,
    ceil(log2 total width) EF4 challenges (4 squeezes each) -> partial-Lagrange
    weights, the batched MLE re-encoded bit-reversed, the round count observed
    (base), per round message (s(0), s(1)) -> SMCS commit of the [n/2, 8] rows
    -> observe message, bound root -> EF4 beta -> folds; final poly =
    codeword[0] observed; grind(pow_bits) = the lowest passing witness
    observed, squeeze once (:304-307); SP1 positions; openings. blocks: per round [K, S] Montgomery columns."""
    v = log_s
    S = 1 << v
    n = S << log_blowup
    zs = u32(z_final).reshape(-1, 4)[-v:]
    blocks = [u32(b) for b in blocks]
    evals = [eval_mle_base(field, b, zs) for b in blocks]
    t.observe(u32(dense_eval).reshape(-1))
    for e in evals:
        t.observe(e.reshape(-1))
    total = sum(b.shape[0] for b in blocks)
    nbv = (total - 1).bit_length() if total > 1 else 0
    chal = np.zeros((max(nbv, 1), 4), np.uint32)
    if nbv:
        chal[:nbv] = t.sample(4 * nbv).reshape(nbv, 4)
    mle = np.zeros((S, 4), np.uint32)
    off = 0
    for b in blocks:
        LIB.orc_rlc_columns_ex(field, b.reshape(-1), S, b.shape[0], chal.reshape(-1), nbv, off,
                               int(off > 0), mle.reshape(-1))
        off += b.shape[0]
    wt = eq_expand(field, chal[:nbv])
    claim = np.zeros(4, np.uint32)
    for c, val in enumerate(np.concatenate(evals)):
        claim = ef4_add(field, claim, ef4_mul(field, wt[c], val))
    cw = rs_encode_bitrev(field, mle.T.copy(), log_blowup).T.copy()  # [n, 4], limb by limb
    t.observe(to_mont(field, [v]))
    msgs, raw, bound, betas, layers = [], [], [], [], []
    for i in range(v):
        rest = zs[: v - i - 1]
        s0 = eval_mle_ef4(field, mle[0::2], rest)
        s1 = ef4_add(field, ef4_mul(field, ef4_sub(field, claim, s0), ef4_inv(field, zs[v - 1 - i])),
                     s0)
        N = cw.shape[0]
        leaves = cw.reshape(N // 2, 8)
        dl = merkle_commit_rows(p2, leaves)
        b_root = smcs_bind_root(p2, dl[-1][0], (N // 2).bit_length() - 1, 8)
        msg = np.concatenate([s0, s1])
        t.observe(msg)
        t.observe(b_root)
        beta = t.sample(4)
        msgs.append(msg)
        raw.append(dl[-1][0])
        bound.append(b_root)
        betas.append(beta)
        layers.append((leaves, dl))
        cw = fri_fold_bitrev(field, cw, True, beta, True)
        mle = mle_fold(field, mle, beta)
        claim = ef4_add(field, s0, ef4_mul(field, beta, s1))
    final = cw[0].copy()
    t.observe(final)
    witness = to_mont(field, [t.grind(pow_bits)])
    t.observe(witness)
    t.sample(1)
    raw_q = t.sample(num_queries)
    positions = sp1_query_positions(from_mont(field, raw_q), n)
    queries = []
    for i, (leaves, dl) in enumerate(layers):
        a = (positions >> (i + 1)).astype(np.int32)
        queries.append(merkle_open(leaves, leaves.shape[0], 1, 8, 0, dl, a))
    return {"batch_evals": evals, "uni_msgs": np.stack(msgs), "raw_roots": np.stack(raw),
            "bound_roots": np.stack(bound), "betas": np.stack(betas), "final_poly": final,
            "final_codeword": cw, "final_claim": claim, "positions": positions,
            "pow_witness": witness, "query_openings": queries}
