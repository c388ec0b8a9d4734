"""Derive the built-in BabyBear width-16 Poseidon2 instance and write its header.

The reference ships no BabyBear Poseidon2 parameterisation (its only instances
are KoalaBear-16, zorch/testkit/koalabear16.py and
zorch/commit/testing/sp1_koalabear16.py), so this project defines one from the
published procedure and records every choice here:

- field p = 2^31 - 2^27 + 1, width t = 16, S-box x^7 (the smallest alpha with
  gcd(alpha, p-1) = 1), R_F = 8 full rounds (4 initial + 4 terminal) and
  R_P = 13 partial rounds;
- external layer: the Poseidon2 "M4 block circulant" layer, M4 = circ(2,3,1,1)
  rows [[2,3,1,1],[1,2,3,1],[1,1,2,3],[3,1,1,2]], then each lane adds the sum of
  the lanes congruent to it mod 4 (the same layer the KoalaBear instance uses);
- internal layer: state[i] <- sum(state) + diag[i] * state[i] with the small
  "shift friendly" diagonal below, accepted only if the Poseidon2 condition
  holds: for i = 1..2t the minimal polynomial of M_I^i has degree t and is
  irreducible (Poseidon2 paper, eprint 2023/323, internal matrix section);
- round constants: the Grain LFSR of the Poseidon paper (eprint 2019/458,
  appendix "round constants"), initialised with field = 1 (prime field),
  s-box = 0, n = 31, t = 16, R_F = 8, R_P = 13, the remaining 30 bits set,
  160 warm-up clocks, the self-shrinking output rule, and rejection sampling of
  31-bit big-endian words >= p. (R_F + R_P) * t elements are drawn in round
  order; a partial round uses the first element of its row.

Run from the repo root; it rewrites poseidon2_babybear16.h beside this file.
"""

from __future__ import annotations

from fractions import Fraction
from pathlib import Path

P = 2**31 - 2**27 + 1
T = 16
ALPHA = 7
R_F = 8
R_P = 13
N_BITS = 31


def grain_bits(field: int, sbox: int, n: int, t: int, r_f: int, r_p: int):
    """The Poseidon Grain LFSR bit stream (80-bit state, self-shrinking)."""
    init = []
    init += [int(b) for b in format(field, "02b")]
    init += [int(b) for b in format(sbox, "04b")]
    init += [int(b) for b in format(n, "012b")]
    init += [int(b) for b in format(t, "012b")]
    init += [int(b) for b in format(r_f, "010b")]
    init += [int(b) for b in format(r_p, "010b")]
    init += [1] * 30
    assert len(init) == 80
    state = init

    def clock() -> int:
        nb = state[62] ^ state[51] ^ state[38] ^ state[23] ^ state[13] ^ state[0]
        state.pop(0)
        state.append(nb)
        return nb

    for _ in range(160):
        clock()
    while True:
        b = clock()
        while b == 0:
            clock()
            b = clock()
        yield clock()


def round_constants() -> list[list[int]]:
    gen = grain_bits(1, 0, N_BITS, T, R_F, R_P)
    rows = []
    for _ in range(R_F + R_P):
        row = []
        for _ in range(T):
            while True:
                v = 0
                for _ in range(N_BITS):
                    v = (v << 1) | next(gen)
                if v < P:
                    break
            row.append(v)
        rows.append(row)
    return rows


def _inv(a: int) -> int:
    return pow(a % P, P - 2, P)


def _frac(f: Fraction) -> int:
    return f.numerator % P * _inv(f.denominator) % P


# Small diagonal entries whose products reduce to shifts/adds (-2, 1, 2, 1/2,
# 3, 4, -1/2, -3, -4, 1/2^8, 1/4, 1/8, 1/2^27, -1/2^8, -1/16, -1/2^27).
DIAG_FRACTIONS = [
    Fraction(-2), Fraction(1), Fraction(2), Fraction(1, 2), Fraction(3), Fraction(4),
    Fraction(-1, 2), Fraction(-3), Fraction(-4), Fraction(1, 2**8), Fraction(1, 4),
    Fraction(1, 8), Fraction(1, 2**27), Fraction(-1, 2**8), Fraction(-1, 16),
    Fraction(-1, 2**27),
]


def internal_matrix(diag: list[int]) -> list[list[int]]:
    return [[(1 + (diag[i] if i == j else 0)) % P for j in range(T)] for i in range(T)]


def _matmul(a, b):
    n = len(a)
    return [[sum(a[i][k] * b[k][j] for k in range(n)) % P for j in range(n)] for i in range(n)]


def _charpoly(m: list[list[int]]) -> list[int]:
    """Characteristic polynomial mod P (monic, ascending coefficients) by
    reduction to upper Hessenberg form and the Hessenberg recurrence."""
    n = len(m)
    a = [row[:] for row in m]
    for k in range(n - 2):
        piv = next((i for i in range(k + 1, n) if a[i][k] % P), None)
        if piv is None:
            continue
        if piv != k + 1:
            a[k + 1], a[piv] = a[piv], a[k + 1]
            for r in range(n):
                a[r][k + 1], a[r][piv] = a[r][piv], a[r][k + 1]
        inv = _inv(a[k + 1][k])
        for i in range(k + 2, n):
            f = a[i][k] * inv % P
            if f:
                for c in range(n):
                    a[i][c] = (a[i][c] - f * a[k + 1][c]) % P
                for r in range(n):
                    a[r][k + 1] = (a[r][k + 1] + f * a[r][i]) % P
    # p_0 = 1; p_k(x) = (x - a_kk) p_{k-1} - sum_{i<k} a_ik * prod(sub) * p_{i-1}
    polys = [[1]]
    for k in range(n):
        nxt = [0] + polys[k][:]  # x * p_{k}
        for i, c in enumerate(polys[k]):
            nxt[i] = (nxt[i] - a[k][k] * c) % P
        prod = 1
        for i in range(k - 1, -1, -1):
            prod = prod * a[i + 1][i] % P
            coef = prod * a[i][k] % P
            for j, c in enumerate(polys[i]):
                nxt[j] = (nxt[j] - coef * c) % P
        polys.append(nxt)
    return polys[n]


def check_internal_diag(diag: list[int]) -> bool:
    from sympy import GF, Poly, symbols

    x = symbols("x")
    m = internal_matrix(diag)
    cur = m
    for _ in range(2 * T):
        cp = _charpoly(cur)
        poly = Poly(list(reversed(cp)), x, domain=GF(P))
        if poly.degree() != T or not poly.is_irreducible:
            return False
        cur = _matmul(m, cur)
    return True


def main() -> None:
    diag = [_frac(f) for f in DIAG_FRACTIONS]
    if not check_internal_diag(diag):
        raise SystemExit("internal diagonal fails the Poseidon2 minimal-polynomial check")
    rc = round_constants()
    half = R_F // 2
    ext_init = rc[:half]
    internal = [row[0] for row in rc[half : half + R_P]]
    ext_term = rc[half + R_P :]

    def mont(vals):
        return [(v << 32) % P for v in vals]

    def arr(vals):
        return ", ".join(f"{v}u" for v in vals)

    lines = [
        "// Generated by gen_poseidon2_babybear16.py -- do not edit.",
        "// Built-in BabyBear width-16 Poseidon2 instance: x^7, 4+4 full rounds,",
        "// 13 partial rounds, Grain-LFSR round constants, checked internal diagonal.",
        "// All values canonical (not Montgomery).",
        "#pragma once",
        "#include <stdint.h>",
        f"#define ZC_BB16_ALPHA {ALPHA}",
        f"#define ZC_BB16_ROUNDS_F_HALF {half}",
        f"#define ZC_BB16_ROUNDS_P {R_P}",
        "static const uint32_t ZC_BB16_EXT_INIT[4][16] = {",
        *[f"  {{{arr(r)}}}," for r in ext_init],
        "};",
        "static const uint32_t ZC_BB16_EXT_TERM[4][16] = {",
        *[f"  {{{arr(r)}}}," for r in ext_term],
        "};",
        f"static const uint32_t ZC_BB16_INT_RC[{R_P}] = {{{arr(internal)}}};",
        f"static const uint32_t ZC_BB16_DIAG[16] = {{{arr(diag)}}};",
        "// Montgomery forms (x * 2^32 mod p), what the kernels load.",
        "#define ZC_BB16_EXT_INIT_MONT_INIT {" + arr(mont(v for r in ext_init for v in r)) + "}",
        "#define ZC_BB16_EXT_TERM_MONT_INIT {" + arr(mont(v for r in ext_term for v in r)) + "}",
        "#define ZC_BB16_INT_RC_MONT_INIT {" + arr(mont(internal)) + "}",
        "#define ZC_BB16_DIAG_MONT_INIT {" + arr(mont(diag)) + "}",
        "",
    ]
    out = Path(__file__).with_name("poseidon2_babybear16.h")
    out.write_text("\n".join(lines))
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
