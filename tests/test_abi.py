"""The C ABI library loads and exports every symbol include/zc.h declares
(no compute calls: runs without a GPU)."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols() -> list[str]:
    text = (ROOT / "include" / "zc.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(zc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["zc_rs_encode", "zc_merkle_commit", "zc_merkle_open", "zc_fri_fold",
              "zc_fri_fold_commit", "zc_duplex_hop", "zc_duplex_step", "zc_init"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    from zorch_gb300 import _lib

    lib = ctypes.CDLL(str(_lib.lib()._name))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_status_strings_and_host_hop_without_gpu():
    """Host-only entry points run without a device."""
    from zorch_gb300 import _lib

    L = _lib.lib()
    assert L.zc_status_str(_lib.ZC_NOT_POW2).decode() == "size is not a power of two"
    assert L.zc_version() >= 1


def test_workspace_sizes():
    from zorch_gb300 import _lib

    L = _lib.lib()
    assert L.zc_rs_encode_workspace_bytes(3, 10, 2) == 0  # single pass
    assert L.zc_rs_encode_workspace_bytes(2, 16, 1) == 2 * 4 * (1 << 17)
    assert L.zc_rs_encode_workspace_bytes(64, 20, 2) == 1 << 30  # capped chunk


def test_host_permutation_matches_oracle(orc):
    """The host form of the permutation (no GPU needed) equals the oracle's,
    for the built-in BabyBear instance and the golden KoalaBear instance."""
    import numpy as np

    from zorch_gb300.commit import Poseidon2, koalabear16_params

    try:
        bb = Poseidon2.builtin()
    except Exception:  # creating a handle needs a CUDA context
        import pytest

        pytest.skip("no CUDA device for the handle's device copy")
    kb = koalabear16_params(orc.load_koalabear_fixture())
    for gpu, cpu, f in ((bb, orc.Poseidon2.babybear16(), 0),
                        (kb, orc.Poseidon2.koalabear16_golden(), 1)):
        st = orc.to_mont(f, np.arange(16 * 5, dtype=np.uint32).reshape(5, 16))
        assert np.array_equal(gpu.permute_host(st), np.stack([cpu.permute(s) for s in st]))


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the ABI structs (zorch_gb300/_lib.py) have the
    header's size and field offsets, as a C compiler lays them out."""
    import shutil
    import subprocess

    from zorch_gb300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest

        pytest.skip("no C compiler")
    structs = {"zc_leaves": _lib.Leaves, "zc_lde_job": _lib.LdeJob,
               "zc_merkle_job": _lib.MerkleJob}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "zc.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    # the header declares stream arguments as void*, so no CUDA header is needed
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
