"""zorch-gb300: GB300-native (sm_103a) polynomial-commitment hot path of
fractalyze/zorch -- Reed-Solomon coset LDE, Poseidon2 Merkle commitment and
FRI/Basefold fold-and-commit rounds -- behind the reference's PCS / Round /
Transcript API, on hand-written CUDA kernels reached through a C ABI
(include/zc.h, libzc.so)."""

from .field import BABYBEAR, KOALABEAR, Field, field_of  # noqa: F401

__all__ = ["BABYBEAR", "KOALABEAR", "Field", "field_of"]


def load_library():
    """Load libzc.so (raises if it is missing and cannot be built)."""
    from . import _lib

    return _lib.lib()
