"""Build the CUDA library libzc.so in-tree for sm_103a (GB300).

Seven translation units compiled in parallel with nvcc, then linked into
zorch_gb300/_build/libzc.so. No cmake, no torch extension machinery: the
library exposes a plain C ABI (include/zc.h) that Python reaches via ctypes.
"""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libzc.so"
SOURCES = ["zc_core.cu", "zc_ntt.cu", "zc_merkle.cu", "zc_fold.cu", "zc_fold_bitrev.cu",
           "zc_sumcheck.cu", "zc_deep.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def toolchain_available() -> bool:
    import shutil

    return Path(_nvcc()).exists() or shutil.which("nvcc") is not None


def _deps() -> list[Path]:
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [
        ROOT / "include" / "zc.h", Path(__file__)]


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile libzc.so; `extra` (or the ZC_NVCC_FLAGS environment variable)
    adds nvcc flags (e.g. -DNAME=VALUE, -maxrregcount=N). A change of flags
    forces a rebuild."""
    extra = list(extra or []) + os.environ.get("ZC_NVCC_FLAGS", "").split()
    stamp = OUT_DIR / "flags.txt"
    flags_id = " ".join(extra)
    same_flags = stamp.exists() and stamp.read_text() == flags_id
    if LIB.exists() and not force and same_flags:
        newest = max(d.stat().st_mtime for d in _deps())
        if LIB.stat().st_mtime >= newest:
            return LIB
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    flags = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
             "-I", str(ROOT / "include"), *ARCH, *(extra or [])]
    if verbose:
        flags += ["-Xptxas", "-v"]

    def compile_one(src: str) -> Path:
        obj = OUT_DIR / (Path(src).stem + ".o")
        cmd = [_nvcc(), *flags, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(flags_id)
    return LIB


# ------------------------------------------------------------ XLA FFI ----
XLA_SRC = CSRC / "zc_xla.cc"
XLA_LIB = OUT_DIR / "libzc_xla.so"


def xla_ffi_include_dir() -> Path | None:
    """The directory holding xla/ffi/api/ffi.h: XLA_FFI_INCLUDE_DIR, else an
    installed jaxlib's (or jax's) include directory; None when absent."""
    cands = []
    if os.environ.get("XLA_FFI_INCLUDE_DIR"):
        cands.append(Path(os.environ["XLA_FFI_INCLUDE_DIR"]))
    for mod in ("jaxlib", "jax"):
        try:
            m = __import__(mod)
        except Exception:  # noqa: BLE001 - absent or broken install: not a build error
            continue
        cands.append(Path(m.__file__).resolve().parent / "include")
    for c in cands:
        if (c / "xla" / "ffi" / "api" / "ffi.h").exists():
            return c
    return None


def build_xla(force: bool = False) -> Path | None:
    """libzc_xla.so, the XLA FFI handlers of zc_xla.cc over libzc.so, built
    only where the XLA FFI headers are found; None (and nothing built)
    otherwise."""
    inc = xla_ffi_include_dir()
    if inc is None:
        return None
    lib = build()
    if XLA_LIB.exists() and not force and XLA_LIB.stat().st_mtime >= max(
            XLA_SRC.stat().st_mtime, lib.stat().st_mtime):
        return XLA_LIB
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(inc),
           "-I", str(ROOT / "include"), "-I", str(cuda / "include"), str(XLA_SRC),
           "-o", str(XLA_LIB), "-L", str(OUT_DIR), "-lzc", f"-Wl,-rpath,{OUT_DIR}",
           "-L", str(cuda / "lib64"), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"zc_xla.cc failed to build:\n{r.stderr}")
    return XLA_LIB


if __name__ == "__main__":
    print(build(force=True, verbose="-v" in sys.argv))
