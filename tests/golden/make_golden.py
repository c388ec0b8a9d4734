"""Generate the KoalaBear-16 Poseidon2 / Merkle golden fixture from the reference.

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

    python tests/golden/make_golden.py /path/to/zorch-checkout
"""

from __future__ import annotations

import ast
import json
import sys
from pathlib import Path


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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
