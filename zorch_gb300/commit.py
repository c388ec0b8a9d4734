"""Poseidon2 sponge/compression Merkle trees on the GPU (drop-in for
zorch/commit/merkle.py:46-331, arity 2).

`Poseidon2` wraps a width-16 parameterisation (hash-frx Poseidon2Params): the
built-in BabyBear-16 instance or any instance given by canonical constants.
`MerkleTree.commit` hashes every leaf with PaddingFreeSponge<16,8,8> and folds
pairs with TruncatedPermutation<2,8,16>, keeping every digest layer in one flat
device buffer (leaf digests first, root last).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .field import BABYBEAR, KOALABEAR, field_of, ptr, stream_handle


class Poseidon2:
    """A width-16 Poseidon2 permutation living on the device."""

    def __init__(self, handle: int, field, owned: bool) -> None:
        self._h = handle
        self.field = field_of(field)
        self._owned = owned

    @classmethod
    def builtin(cls, field=BABYBEAR) -> "Poseidon2":
        h = C.c_void_p()
        _lib.check(_lib.lib().zc_poseidon2_builtin(field_of(field).id, C.byref(h)),
                   "poseidon2_builtin")
        return cls(h.value, field, False)

    @classmethod
    def from_params(cls, field, alpha: int, ext_init, ext_term, int_rc, diag,
                    j_scale: int = 1) -> "Poseidon2":
        """Canonical constants: ext_init/ext_term (R_F/2, 16), int_rc (R_P,), diag (16,)."""
        f = field_of(field)
        ei = np.ascontiguousarray(np.asarray(ext_init, np.uint32).reshape(-1))
        et = np.ascontiguousarray(np.asarray(ext_term, np.uint32).reshape(-1))
        ir = np.ascontiguousarray(np.asarray(int_rc, np.uint32))
        dg = np.ascontiguousarray(np.asarray(diag, np.uint32))
        if ei.size % 16 or ei.size != et.size or dg.size != 16:
            raise ValueError("Poseidon2 width-16 constants have the wrong shape")
        h = C.c_void_p()
        _lib.check(_lib.lib().zc_poseidon2_create(
            f.id, alpha, ei.size // 16, ir.size, ei.ctypes.data, et.ctypes.data,
            ir.ctypes.data if ir.size else None, dg.ctypes.data, j_scale, C.byref(h)),
            "poseidon2_create")
        return cls(h.value, f, True)

    @property
    def handle(self) -> int:
        return self._h

    def permute(self, states: torch.Tensor) -> torch.Tensor:
        """Permute [count, 16] states (a copy is returned)."""
        s = states.contiguous().clone()
        _lib.check(_lib.lib().zc_poseidon2_permute(self._h, ptr(s), s.numel() // 16,
                                                   stream_handle()), "poseidon2_permute")
        return s

    def permute_host(self, states: np.ndarray) -> np.ndarray:
        """Permute [count, 16] host states on the CPU (a copy is returned)."""
        s = np.ascontiguousarray(np.asarray(states, np.uint32)).copy()
        _lib.check(_lib.lib().zc_poseidon2_permute_host(self._h, s.ctypes.data, s.size // 16),
                   "poseidon2_permute_host")
        return s

    def hash_host(self, row) -> np.ndarray:
        """PaddingFreeSponge<16, 8, 8> on the CPU."""
        row = np.asarray(row, np.uint32).reshape(-1)
        st = np.zeros(16, np.uint32)
        for i in range(0, row.size, 8):
            blk = row[i: i + 8]
            st[: blk.size] = blk
            st = self.permute_host(st)
        return st[:8].copy()

    def compress_host(self, left, right) -> np.ndarray:
        st = np.concatenate([np.asarray(left, np.uint32), np.asarray(right, np.uint32)])
        return self.permute_host(st)[:8].copy()

    def __del__(self) -> None:
        if getattr(self, "_owned", False) and self._h:
            try:
                _lib.lib().zc_poseidon2_destroy(self._h)
            except Exception:
                pass
            self._h = 0


def level_offset(num_leaves: int, level: int) -> int:
    return 2 * num_leaves - ((2 * num_leaves) >> level)


class DigestLayers:
    """All digest layers of one tree in a flat [(2L-1), 8] device buffer."""

    def __init__(self, flat: torch.Tensor, num_leaves: int) -> None:
        self.flat = flat
        self.num_leaves = num_leaves

    @property
    def depth(self) -> int:
        return self.num_leaves.bit_length() - 1

    def __len__(self) -> int:
        return self.depth + 1

    def __getitem__(self, level: int) -> torch.Tensor:
        if level < 0:
            level += len(self)
        off = level_offset(self.num_leaves, level)
        return self.flat[off: off + (self.num_leaves >> level)]

    def __iter__(self):
        return (self[i] for i in range(len(self)))

    @property
    def root(self) -> torch.Tensor:
        return self.flat[-1]


@dataclass(frozen=True)
class Opening:
    """Batched openings: rows [Q, w] and path [depth, Q, 8] (leaf first)."""

    row: torch.Tensor
    path: torch.Tensor


def leaves_layout(base: torch.Tensor, num_leaves: int, groups: int, group_len: int,
                  group_stride: int) -> _lib.Leaves:
    return _lib.Leaves(ptr(base), num_leaves, groups, group_len, group_stride)


class MerkleTree:
    """Arity-2 Merkle commitment over a single matrix (zorch/commit/merkle.py:59-331).

    `column_major=False` reads a leaf as a row of `[num_leaves, leaf_width]`;
    True as a column of `[leaf_width, num_leaves]` (zorch/commit/merkle.py:72-80)."""

    arity = 2
    digest_elems = 8

    def __init__(self, perm: Poseidon2 | None = None, *, column_major: bool = False) -> None:
        self.perm = perm if perm is not None else Poseidon2.builtin(BABYBEAR)
        self.column_major = column_major

    def __eq__(self, other) -> bool:
        return (isinstance(other, MerkleTree) and self.perm.handle == other.perm.handle
                and self.column_major == other.column_major)

    def __hash__(self) -> int:
        return hash((self.perm.handle, self.column_major))

    def _layout(self, matrix: torch.Tensor) -> _lib.Leaves:
        if matrix.dim() != 2:
            raise ValueError(f"matrix must be 2-D, got ndim={matrix.dim()}")
        m = matrix.contiguous()
        if self.column_major:
            w, L = m.shape
            return leaves_layout(m, L, w, 1, L)
        L, w = m.shape
        return leaves_layout(m, L, 1, w, 0)

    def commit_layout(self, lv: _lib.Leaves, device="cuda",
                      out: torch.Tensor | None = None) -> tuple[torch.Tensor, DigestLayers]:
        L = lv.num_leaves
        if L == 0:
            raise ValueError("matrix must contain at least one leaf")
        if L & (L - 1):
            raise ValueError(f"leaf count ({L}) must be a power of two")
        flat = out if out is not None else torch.empty((2 * L - 1, 8), dtype=torch.int32,
                                                       device=device)
        _lib.check(_lib.lib().zc_merkle_commit(self.perm.handle, lv, ptr(flat), stream_handle()),
                   "merkle_commit")
        layers = DigestLayers(flat, L)
        return layers.root, layers

    def commit(self, matrix: torch.Tensor) -> tuple[torch.Tensor, DigestLayers]:
        """(raw_root (8,), digest_layers) (zorch/commit/merkle.py:118-134)."""
        return self.commit_layout(self._layout(matrix), matrix.device)

    def open_layout(self, lv: _lib.Leaves, layers: DigestLayers, indices: torch.Tensor,
                    width: int, check: bool = True) -> Opening:
        """Batched openings. `check` reads the device out-of-range flag back
        (a host synchronisation); callers whose indices are in range by
        construction, or that are being captured into a CUDA graph, pass False."""
        idx = indices.to(torch.int32).contiguous()
        q = idx.numel()
        rows = torch.empty((q, width), dtype=torch.int32, device=idx.device)
        paths = torch.empty((layers.depth, q, 8), dtype=torch.int32, device=idx.device)
        check = check and not torch.cuda.is_current_stream_capturing()
        # the flag is only zeroed (a fill launch) when it is read back
        flag = torch.zeros(1, dtype=torch.int32, device=idx.device) if check else None
        _lib.check(_lib.lib().zc_merkle_open(lv, ptr(layers.flat), ptr(idx), q, ptr(rows),
                                             ptr(paths), ptr(flag), stream_handle()),
                   "merkle_open")
        if check and int(flag.item()):
            raise IndexError(f"leaf index out of range [0, {lv.num_leaves})")
        return Opening(rows, paths)

    def open_layout_reduced(self, lv: _lib.Leaves, layers: DigestLayers,
                            indices: torch.Tensor, width: int, shift: int = 0) -> Opening:
        """Openings at leaf (indices[i] >> shift) mod num_leaves, reduced by the
        kernel: a fold layer's opening at the layer position of the query
        positions -- q mod (n >> (i+1)) in natural order (shift 0), q >> (i+1)
        in bit-reversed order (zorch/coding/reed_solomon.py:320-329, 521-528).
        No host synchronisation."""
        idx = indices.to(torch.int32).contiguous()
        q = idx.numel()
        rows = torch.empty((q, width), dtype=torch.int32, device=idx.device)
        paths = torch.empty((layers.depth, q, 8), dtype=torch.int32, device=idx.device)
        _lib.check(_lib.lib().zc_merkle_open_reduced(lv, ptr(layers.flat), ptr(idx), q, shift,
                                                     ptr(rows), ptr(paths), stream_handle()),
                   "merkle_open_reduced")
        return Opening(rows, paths)

    def open_rows(self, matrix: torch.Tensor, layers: DigestLayers,
                  indices: torch.Tensor, check: bool = True) -> Opening:
        """Open `matrix` (always leaf-major [L, w] like the reference) at every
        index (zorch/pcs/fold.py:142-149); `check` as in open_layout."""
        m = matrix.contiguous()
        lv = leaves_layout(m, m.shape[0], 1, m.shape[1], 0)
        return self.open_layout(lv, layers, indices, m.shape[1], check=check)

    def reconstruct_root(self, index: int, opening: Opening) -> np.ndarray:
        """Rebuild the raw root from an opening's row and leaf-first path
        (zorch/commit/merkle.py:264-285), on the host."""
        node = self.perm.hash_host(opening.row.detach().cpu().numpy().view(np.uint32))
        path = opening.path.detach().cpu().numpy().view(np.uint32)
        idx = int(index)
        for sib in path.reshape(-1, 8):
            node = self.perm.compress_host(node, sib) if idx % 2 == 0 else \
                self.perm.compress_host(sib, node)
            idx //= 2
        return node

    def verify(self, root: torch.Tensor, index: int, opening: Opening) -> bool:
        """zorch/commit/merkle.py:327-331: out-of-range indices are rejected,
        else the rebuilt root must equal the committed one."""
        depth = opening.path.reshape(-1, 8).shape[0]
        if not 0 <= int(index) < (1 << depth):
            return False
        want = root.detach().cpu().numpy().view(np.uint32).reshape(-1)
        return bool(np.array_equal(self.reconstruct_root(index, opening), want))

    def open(self, matrix: torch.Tensor, layers: DigestLayers, index: int) -> Opening:
        if not 0 <= int(index) < matrix.shape[0]:
            raise IndexError(f"leaf index {index} out of range [0, {matrix.shape[0]})")
        op = self.open_rows(matrix, layers, torch.tensor([int(index)], device=matrix.device))
        return Opening(op.row[0], op.path[:, 0])


def koalabear16_params(fixture: dict) -> Poseidon2:
    """A Poseidon2 from a KoalaBear-16 parameter dict (canonical constants)."""
    return Poseidon2.from_params(KOALABEAR, fixture["alpha"], fixture["external_initial"],
                                 fixture["external_terminal"], fixture["internal_rc"],
                                 fixture["internal_diag"], fixture.get("internal_j_scale", 1))


class VerifyCode:
    """SMCS verifier return codes (zorch/commit/smcs.py:31-44)."""

    OK = 0
    WRONG_HEIGHT = 2
    INDEX_OUT_OF_BOUNDS = 3
    ROOT_MISMATCH = 4


class SingleMatrixCommitmentScheme:
    """SP1's single-matrix commitment over the Merkle tree (zorch/commit/smcs.py:47-228):
    a Merkle root over the rows (or, `column_major=True`, the columns) of one
    power-of-two-height base-field matrix, bound to the matrix shape by SP1's
    domain separator commit = compress([root, sponge([log_height, width])])."""

    def __init__(self, perm: Poseidon2) -> None:
        self.perm = perm
        self._tree = MerkleTree(perm)
        self._tree_column_major = MerkleTree(perm, column_major=True)
        self.digest_elems = 8

    def commit(self, matrix: torch.Tensor, *,
               column_major: bool = False) -> tuple[torch.Tensor, DigestLayers]:
        """(commitment (8,), digest layers) (zorch/commit/smcs.py:69-106); a
        column-major [width, height] matrix commits as its transpose would."""
        tree = self._tree_column_major if column_major else self._tree
        raw_root, layers = tree.commit(matrix)
        height, width = matrix.shape[::-1] if column_major else matrix.shape
        return self.bind_root(raw_root, height.bit_length() - 1, width), layers

    def commit_layout(self, lv: _lib.Leaves, width: int,
                      out: torch.Tensor | None = None) -> tuple[torch.Tensor, DigestLayers]:
        """commit over an explicit leaf layout (zc_leaves)."""
        raw_root, layers = self._tree.commit_layout(lv, out=out)
        return self.bind_root(raw_root, lv.num_leaves.bit_length() - 1, width), layers

    def bind_root(self, raw_root: torch.Tensor, log_height: int, width: int,
                  out: torch.Tensor | None = None) -> torch.Tensor:
        """compress([raw_root, sponge([log_height, width])]) on the device
        (zorch/commit/smcs.py:118-140)."""
        if out is None:
            out = torch.empty(8, dtype=torch.int32, device=raw_root.device)
        _lib.check(_lib.lib().zc_smcs_bind_root(self.perm.handle, ptr(raw_root.contiguous()),
                                                log_height, width, ptr(out), stream_handle()),
                   "smcs_bind_root")
        return out

    def bind_root_host(self, raw_root, log_height: int, width: int) -> np.ndarray:
        """bind_root on the host (for verifiers)."""
        f = self.perm.field
        params = self.perm.hash_host(np.array([f.mont(log_height), f.mont(width)], np.uint32))
        return self.perm.compress_host(np.asarray(raw_root, np.uint32).reshape(-1), params)

    def open_batch(self, indices: torch.Tensor, matrix: torch.Tensor,
                   layers: DigestLayers, check: bool = True) -> tuple[torch.Tensor, torch.Tensor]:
        """(rows [Q, width], proofs [log_height, Q, 8]) (zorch/commit/smcs.py:158-183):
        `matrix` is the committed row-major [height, width] matrix. `check`
        reads the device's out-of-range flag back (a host synchronisation);
        callers whose indices are in range by construction pass False."""
        op = self._tree.open_rows(matrix, layers, indices, check=check)
        return op.row, op.path

    def verify_batch(self, commitment, dims: tuple[int, int], index: int, row, proof) -> int:
        """One opened row against a commitment, on the host
        (zorch/commit/smcs.py:185-228): a VerifyCode."""
        height, width = dims
        log_height = height.bit_length() - 1
        proof = np.asarray(proof.detach().cpu() if torch.is_tensor(proof) else proof)
        proof = proof.view(np.uint32).reshape(-1, 8)
        if proof.shape[0] != log_height:
            return VerifyCode.WRONG_HEIGHT
        if not 0 <= int(index) < height:
            return VerifyCode.INDEX_OUT_OF_BOUNDS
        row = torch.as_tensor(np.asarray(
            row.detach().cpu() if torch.is_tensor(row) else row).view(np.int32))
        raw = self._tree.reconstruct_root(int(index), Opening(row, torch.as_tensor(
            proof.view(np.int32))))
        bound = self.bind_root_host(raw, log_height, width)
        want = np.asarray(commitment.detach().cpu() if torch.is_tensor(commitment)
                          else commitment).view(np.uint32).reshape(-1)
        return VerifyCode.OK if np.array_equal(bound, want) else VerifyCode.ROOT_MISMATCH


class StridedMerkleTree:
    """Query-strided binary Merkle commitment (zorch/commit/strided_merkle.py:43-230):
    one query opens the `rows_per_query` rows {i, i+s, i+2s, ...} (s = height /
    rows_per_query) under a single path; the strided levels below the s-node
    query layer are not stored (the verifier re-hashes the opened coset)."""

    def __init__(self, perm: Poseidon2, rows_per_query: int) -> None:
        if rows_per_query < 1 or rows_per_query & (rows_per_query - 1):
            raise ValueError(f"rows_per_query ({rows_per_query}) must be a power of two")
        self.perm = perm
        self.rows_per_query = rows_per_query
        self.digest_elems = 8
        self._top = MerkleTree(perm)

    def __eq__(self, other) -> bool:
        return (isinstance(other, StridedMerkleTree) and self.perm.handle == other.perm.handle
                and self.rows_per_query == other.rows_per_query)

    def __hash__(self) -> int:
        return hash((self.perm.handle, self.rows_per_query))

    def query_stride(self, height: int) -> int:
        return height // self.rows_per_query

    def commit(self, matrix: torch.Tensor) -> tuple[torch.Tensor, DigestLayers]:
        """(raw_root (8,), digest layers from the query layer to the root)."""
        if matrix.dim() != 2:
            raise ValueError(f"matrix must be 2-D, got ndim={matrix.dim()}")
        h, w = matrix.shape
        if h & (h - 1) or h == 0:
            raise ValueError(f"matrix height ({h}) must be a power of two")
        if self.rows_per_query > h:
            raise ValueError(f"rows_per_query ({self.rows_per_query}) > leaves ({h})")
        m = matrix.contiguous()
        s = self.query_stride(h)
        flat = torch.empty((2 * s - 1, 8), dtype=torch.int32, device=m.device)
        _lib.check(_lib.lib().zc_strided_merkle_commit(
            self.perm.handle, leaves_layout(m, h, 1, w, 0), self.rows_per_query, ptr(flat),
            stream_handle()), "strided_merkle_commit")
        layers = DigestLayers(flat, s)
        return layers.root, layers

    def opened_rows(self, matrix: torch.Tensor, index: int) -> torch.Tensor:
        s = self.query_stride(matrix.shape[0])
        if not 0 <= index < s:
            raise ValueError(f"index {index} out of range [0, {s})")
        return matrix[index::s]

    def open(self, matrix: torch.Tensor, layers: DigestLayers,
             indices: torch.Tensor) -> Opening:
        """Batched openings: rows [Q, rows_per_query, w] (the strided cosets)
        and the stored sibling path [log2 s, Q, 8] from the query layer up."""
        h, w = matrix.shape
        s = self.query_stride(h)
        idx = indices.to(torch.int32).contiguous()
        if idx.numel() and (int(idx.min()) < 0 or int(idx.max()) >= s):
            raise IndexError(f"query index out of range [0, {s})")
        members = idx.long()[:, None] + s * torch.arange(self.rows_per_query,
                                                         device=idx.device)[None, :]
        rows = matrix[members.reshape(-1)].reshape(idx.numel(), self.rows_per_query, w)
        empty = _lib.Leaves(None, s, 0, 0, 0)
        q = idx.numel()
        paths = torch.empty((layers.depth, q, 8), dtype=torch.int32, device=idx.device)
        dummy = torch.empty(1, dtype=torch.int32, device=idx.device)
        _lib.check(_lib.lib().zc_merkle_open(empty, ptr(layers.flat), ptr(idx), q, ptr(dummy),
                                             ptr(paths), None, stream_handle()), "merkle_open")
        return Opening(rows, paths)

    def reconstruct_root(self, index: int, opening: Opening) -> np.ndarray:
        """Re-hash the opened coset, fold it adjacent-pairwise to its query-layer
        node, then climb the stored path by the index parity, on the host
        (zorch/commit/strided_merkle.py:198-230)."""
        rows = opening.row.detach().cpu().numpy().view(np.uint32)
        layer = [self.perm.hash_host(r) for r in rows.reshape(self.rows_per_query, -1)]
        while len(layer) > 1:
            layer = [self.perm.compress_host(layer[2 * x], layer[2 * x + 1])
                     for x in range(len(layer) // 2)]
        node, idx = layer[0], int(index)
        for sib in opening.path.detach().cpu().numpy().view(np.uint32).reshape(-1, 8):
            node = self.perm.compress_host(node, sib) if idx % 2 == 0 else \
                self.perm.compress_host(sib, node)
            idx //= 2
        return node

    def verify(self, root: torch.Tensor, index: int, opening: Opening) -> bool:
        depth = opening.path.reshape(-1, 8).shape[0]
        if not 0 <= int(index) < (1 << depth):
            return False
        want = root.detach().cpu().numpy().view(np.uint32).reshape(-1)
        return bool(np.array_equal(self.reconstruct_root(index, opening), want))
