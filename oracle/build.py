"""Build the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

Plain gcc on the oracle's own C sources; no cmake. The reference is pure Python
over closed FRX/hash-frx/zk_dtypes wheels, so there is no reference source to
compile into oracle/_ref -- the oracle restatement is the only CPU path.
"""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    src = [HERE / "zc_oracle.c"]
    deps = src + [HERE / "zc_oracle.h"]
    if OUT.exists() and not force and all(OUT.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-Wall", "-Wextra",
           "-Wno-unused-parameter", *map(str, src), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
