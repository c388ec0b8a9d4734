"""Generate the golden fixtures from the reference.

The reference cannot be imported here (its FRX / hash-frx / zk_dtypes wheels are
absent), so this script reads its test sources as TEXT with `ast` and writes the
literal constants into `koalabear16.json`:

- the Plonky3 (commit 4318eba) KoalaBear width-16 Poseidon2 parameterisation,
  zorch/testkit/koalabear16.py:25 (`_WIDTH, _ER, _IR, _ALPHA`), :46 (initial
  external round constants), :121 (terminal), :196 (internal), :219 (internal
  diagonal);
- the Plonky3 Merkle root golden over arange(32) as a 4x8 matrix with
  PaddingFreeSponge<16,8,8> leaves and TruncatedPermutation<2,8,16> nodes,
  zorch/commit/testing/merkle_test.py:51-63.

All values are canonical (not Montgomery) u32. Run once in a container that has
the reference checked out; the JSON is committed so tests need no reference.

`sp1_fibonacci/` holds the SP1 KoalaBear slice of the reference's jagged-PCS
pipeline dump (zorch/pcs/jagged/testing/testdata/gpu_fibonacci, byte-matched
by zorch/pcs/jagged/testing/open_test.py:242-303):

- `sp1_koalabear16.json`: SP1's KoalaBear width-16 Poseidon2 instance
  (zorch/commit/testing/sp1_koalabear16.py:25-248); the R^-1 factor the
  reference folds into the internal diagonal (:244-247) is applied here, so
  `internal_diag` / `internal_j_scale` are the engine's canonical inputs;
- `prep_dense.u32.xz`: the preprocessed round's dense buffer (2^21 Montgomery
  words, testdata/zerocheck_dense/prep_dense.npy, sliced to the round's raw
  area as open_test.py:147-150 does), lzma-compressed raw little-endian;
- `prep_round.npz`: that round's component openings at the 52 query positions
  (outputs/component_openings_r0.npz: rows and the 23 sibling levels), the
  query draws (outputs/challenges.npz `query_indices`), the opening point
  z_final (outputs/outer_sumcheck_point.npy) and the round's column
  evaluation at its last 21 coordinates (outputs/batch_evals_r0.npz, the
  eval_mle of open.py:202-204);
- `fold_chain.npz`: the FRI fold betas and separator-bound fold-layer roots
  (challenges.npz `fri_betas`, fri_commitments.npy), the final poly, and the
  query openings (rows, sibling paths) of a subset of the fold layers
  (query_openings_f{i}.npz). The main round's dense buffer is not in the
  reference checkout, so the fold chain is checked per query, not re-run.

    python tests/golden/make_golden.py /path/to/zorch-checkout
"""

from __future__ import annotations

import ast
import json
import lzma
import sys
from pathlib import Path

import numpy as np

KOALABEAR_P = 2**31 - 2**24 + 1
# Fold layers whose query openings are kept (rows are kept for every layer).
SP1_PATH_LAYERS = (0, 1, 2, 10, 19, 20)


def _literal_assignments(path: Path) -> dict[str, object]:
    tree = ast.parse(path.read_text())
    out: dict[str, object] = {}
    for node in tree.body:
        if isinstance(node, ast.Assign):
            for target in node.targets:
                if isinstance(target, ast.Name):
                    try:
                        out[target.id] = ast.literal_eval(node.value)
                    except ValueError:
                        pass
                elif isinstance(target, ast.Tuple) and isinstance(node.value, ast.Tuple):
                    for t, v in zip(target.elts, node.value.elts):
                        if isinstance(t, ast.Name):
                            try:
                                out[t.id] = ast.literal_eval(v)
                            except ValueError:
                                pass
    return out


def _golden_root(path: Path) -> list[int]:
    """The list literal inside `_PLONKY3_MERKLE_ROOT_4X8 = fnp.array([...], dtype=F)`."""
    tree = ast.parse(path.read_text())
    for node in tree.body:
        if (
            isinstance(node, ast.Assign)
            and isinstance(node.targets[0], ast.Name)
            and node.targets[0].id == "_PLONKY3_MERKLE_ROOT_4X8"
        ):
            call = node.value
            assert isinstance(call, ast.Call)
            return list(ast.literal_eval(call.args[0]))
    raise KeyError("_PLONKY3_MERKLE_ROOT_4X8 not found")


def main(ref_root: str) -> None:
    ref = Path(ref_root)
    kb = _literal_assignments(ref / "zorch/testkit/koalabear16.py")
    root = _golden_root(ref / "zorch/commit/testing/merkle_test.py")
    fixture = {
        "source": {
            "params": "zorch/testkit/koalabear16.py:25-236 (Plonky3 4318eba)",
            "root": "zorch/commit/testing/merkle_test.py:51-63",
        },
        "field": "koalabear",
        "modulus": 2**31 - 2**24 + 1,
        "width": kb["_WIDTH"],
        "alpha": kb["_ALPHA"],
        "external_rounds": kb["_ER"],
        "internal_rounds": kb["_IR"],
        "external_initial": kb["_EXTERNAL_INITIAL"],
        "external_terminal": kb["_EXTERNAL_TERMINAL"],
        "internal_rc": kb["_INTERNAL_RC"],
        "internal_diag": kb["_INTERNAL_DIAG"],
        "internal_j_scale": 1,
        "merkle_4x8_input": list(range(32)),
        "merkle_4x8_root": root,
    }
    out = Path(__file__).with_name("koalabear16.json")
    out.write_text(json.dumps(fixture, indent=1) + "\n")
    print(f"wrote {out}")


def sp1(ref_root: str) -> None:
    ref = Path(ref_root)
    out = Path(__file__).with_name("sp1_fibonacci")
    out.mkdir(exist_ok=True)
    kb = _literal_assignments(ref / "zorch/commit/testing/sp1_koalabear16.py")
    rinv = kb["_MONTY_INVERSE"]
    assert rinv * 2**32 % KOALABEAR_P == 1
    params = {
        "source": "zorch/commit/testing/sp1_koalabear16.py:25-248 (SP1 cc4eb1f38)",
        "field": "koalabear",
        "width": kb["_WIDTH"],
        "alpha": kb["_ALPHA"],
        "external_rounds": kb["_ER"],
        "internal_rounds": kb["_IR"],
        "external_initial": kb["_EXTERNAL_INITIAL"],
        "external_terminal": kb["_EXTERNAL_TERMINAL"],
        "internal_rc": kb["_INTERNAL_RC"],
        "internal_diag": [d * rinv % KOALABEAR_P for d in kb["_INTERNAL_DIAG"]],
        "internal_j_scale": rinv,
    }
    (out / "sp1_koalabear16.json").write_text(json.dumps(params, indent=1) + "\n")

    data = ref / "zorch/pcs/jagged/testing/testdata"
    meta = json.loads((data / "gpu_fibonacci/meta.json").read_text())
    r0 = meta["rounds"][0]
    area = sum(int(r) * int(c) for r, c in zip(r0["row_counts"], r0["column_counts"]))
    prep = np.load(data / "zerocheck_dense/prep_dense.npy")[:area].astype("<u4")
    (out / "prep_dense.u32.xz").write_bytes(lzma.compress(prep.tobytes(), preset=9))

    outs = data / "gpu_fibonacci/outputs"
    ch = np.load(outs / "challenges.npz")
    co = np.load(outs / "component_openings_r0.npz")
    depth = len([k for k in co.files if k.startswith("proof_l")])
    np.savez_compressed(
        out / "prep_round.npz",
        log_stacking_height=np.int64(r0["log_stacking_height"]),
        log_blowup=np.int64(meta["basefold"]["log_blowup"]),
        query_indices=ch["query_indices"].astype(np.uint32),
        rows=co["rows"].astype(np.uint32),
        paths=np.stack([co[f"proof_l{l}"] for l in range(depth)]).astype(np.uint32),
        z_final=np.load(outs / "outer_sumcheck_point.npy").astype(np.uint32),
        batch_evals=np.load(outs / "batch_evals_r0.npz")["mle0"].astype(np.uint32),
    )

    betas = ch["fri_betas"].astype(np.uint32)
    layers = {}
    for i in range(betas.shape[0]):
        q = np.load(outs / f"query_openings_f{i}.npz")
        layers[f"rows_f{i}"] = q["rows"].astype(np.uint32)
        if i in SP1_PATH_LAYERS:
            d = len([k for k in q.files if k.startswith("proof_l")])
            layers[f"paths_f{i}"] = np.stack([q[f"proof_l{l}"] for l in range(d)]).astype(np.uint32)
    np.savez_compressed(
        out / "fold_chain.npz",
        fri_betas=betas,
        fri_commitments=np.load(outs / "fri_commitments.npy").astype(np.uint32),
        final_poly=np.load(outs / "final_poly.npy").astype(np.uint32).reshape(-1),
        query_indices=ch["query_indices"].astype(np.uint32),
        path_layers=np.asarray(SP1_PATH_LAYERS, np.int64),
        **layers,
    )
    print(f"wrote {out}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
    sp1(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
