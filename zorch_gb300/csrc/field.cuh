// 31-bit Montgomery prime fields (BabyBear, KoalaBear) and their degree-4
// extensions, on the integer pipes. Storage is the Montgomery form x * 2^32 mod p
// -- the same u32 bit pattern zk_dtypes' *_mont dtypes hold and the reference's
// Fiat-Shamir wire carries (zorch/transcript.py:986-999). Every value a kernel
// stores is fully reduced to [0, p), so equal field elements are equal words.
#pragma once
#include <stdint.h>

#ifndef ZC_HD
#define ZC_HD __host__ __device__ __forceinline__
#endif

namespace zc {

constexpr uint32_t inv_mod_2_32(uint32_t p) {
  uint32_t x = 1;
  for (int i = 0; i < 5; i++) x *= 2u - p * x;
  return x;
}
constexpr uint32_t mont_of(uint32_t p, uint64_t x) {
  return (uint32_t)(((x % p) << 32) % p);
}

template <uint32_t P_, uint32_t GEN_, uint32_t W_, int TWO_ADICITY_, int ID_>
struct Mont31 {
  static constexpr uint32_t P = P_;
  static constexpr uint32_t MU = inv_mod_2_32(P_);  // p^-1 mod 2^32
  static constexpr uint32_t ONE = (uint32_t)((((uint64_t)1) << 32) % P_);
  static constexpr uint32_t R2 = (uint32_t)(((uint64_t)ONE * ONE) % P_);
  static constexpr uint32_t GEN = GEN_;  // multiplicative generator, canonical
  static constexpr uint32_t W = mont_of(P_, W_);  // EF4 non-residue (x^4 = W), Montgomery
  static constexpr uint32_t TWO = mont_of(P_, 2);
  static constexpr uint32_t INV2 = mont_of(P_, (P_ + 1) / 2);
  static constexpr int TWO_ADICITY = TWO_ADICITY_;
  static constexpr int ID = ID_;
};

// BabyBear p = 2^31 - 2^27 + 1, generator 31, EF4 = F[x]/(x^4 - 11).
using BabyBear = Mont31<2013265921u, 31u, 11u, 27, 0>;
// KoalaBear p = 2^31 - 2^24 + 1, generator 3, EF4 = F[x]/(x^4 - 3).
using KoalaBear = Mont31<2130706433u, 3u, 3u, 24, 1>;

// Montgomery product: (a*b - m*p) / 2^32 with m = (a*b) * p^-1 mod 2^32; the low
// words cancel exactly, so only the high halves are subtracted.
template <class F>
ZC_HD uint32_t mmul(uint32_t a, uint32_t b) {
  uint64_t t = (uint64_t)a * b;
  uint32_t lo = (uint32_t)t, hi = (uint32_t)(t >> 32);
  uint32_t m = lo * F::MU;
#ifdef __CUDA_ARCH__
  uint32_t mp = __umulhi(m, F::P);
#else
  uint32_t mp = (uint32_t)(((uint64_t)m * F::P) >> 32);
#endif
  uint32_t r = hi - mp;
  return hi < mp ? r + F::P : r;
}

// Signed Montgomery product on (-p, p], values as int32: |a b - m p| <=
// p^2 + 2^31 p < 2^32 p, so the result lies in (-p, p) and a chain of products
// needs no correction step between them (snorm brings the last one back to
// [0, p)). The low words of a b and m p are equal, so the high words differ by
// exactly (a b - m p) / 2^32.
template <class F>
ZC_HD int32_t smul(int32_t a, int32_t b) {
  const int64_t c = (int64_t)a * b;
  const uint32_t m = (uint32_t)c * F::MU;
#ifdef __CUDA_ARCH__
  const int32_t mp = __mulhi((int32_t)m, (int32_t)F::P);
#else
  const int32_t mp = (int32_t)(((int64_t)(int32_t)m * (int64_t)F::P) >> 32);
#endif
  return (int32_t)(c >> 32) - mp;
}

// (-p, p) -> [0, p): the unsigned minimum of r and r + p.
template <class F>
ZC_HD uint32_t snorm(int32_t r) {
  const uint32_t u = (uint32_t)r, v = u + F::P;
  return u < v ? u : v;
}

template <class F>
ZC_HD uint32_t madd(uint32_t a, uint32_t b) {
  uint32_t r = a + b;
  uint32_t s = r - F::P;
  return s < r ? s : r;  // unsigned min: picks r-p when r >= p
}

template <class F>
ZC_HD uint32_t msub(uint32_t a, uint32_t b) {
  uint32_t r = a - b;
  return a < b ? r + F::P : r;
}

template <class F>
ZC_HD uint32_t mneg(uint32_t a) {
  return a ? F::P - a : 0u;
}

template <class F>
ZC_HD uint32_t mpow(uint32_t a, uint64_t e) {
  uint32_t r = F::ONE;
  while (e) {
    if (e & 1) r = mmul<F>(r, a);
    a = mmul<F>(a, a);
    e >>= 1;
  }
  return r;
}

template <class F>
ZC_HD uint32_t minv(uint32_t a) {
  return mpow<F>(a, (uint64_t)F::P - 2);
}

template <class F>
ZC_HD uint32_t to_mont(uint32_t x) {
  return mmul<F>(x % F::P, F::R2);
}
template <class F>
ZC_HD uint32_t from_mont(uint32_t x) {
  return mmul<F>(x, 1u);
}

// Root of unity of order 2^log_n: generator^((p-1)/2^log_n), generator canonical.
template <class F>
ZC_HD uint32_t root_of_unity(int log_n, uint32_t generator) {
  uint32_t g = to_mont<F>(generator ? generator : F::GEN);
  return mpow<F>(g, (uint64_t)(F::P - 1) >> log_n);
}

// ------------------------------------------------------------------ EF4 --
struct ef4 {
  uint32_t c[4];
};

template <class F>
ZC_HD ef4 ef_add(const ef4& a, const ef4& b) {
  return {{madd<F>(a.c[0], b.c[0]), madd<F>(a.c[1], b.c[1]), madd<F>(a.c[2], b.c[2]),
           madd<F>(a.c[3], b.c[3])}};
}
template <class F>
ZC_HD ef4 ef_sub(const ef4& a, const ef4& b) {
  return {{msub<F>(a.c[0], b.c[0]), msub<F>(a.c[1], b.c[1]), msub<F>(a.c[2], b.c[2]),
           msub<F>(a.c[3], b.c[3])}};
}
template <class F>
ZC_HD ef4 ef_scale(const ef4& a, uint32_t s) {
  return {{mmul<F>(a.c[0], s), mmul<F>(a.c[1], s), mmul<F>(a.c[2], s), mmul<F>(a.c[3], s)}};
}
// (a0 + a1 x + a2 x^2 + a3 x^3)(b0 + ...) mod x^4 - W
template <class F>
ZC_HD ef4 ef_mul(const ef4& a, const ef4& b) {
  uint32_t t4 = madd<F>(madd<F>(mmul<F>(a.c[1], b.c[3]), mmul<F>(a.c[2], b.c[2])),
                        mmul<F>(a.c[3], b.c[1]));
  uint32_t t5 = madd<F>(mmul<F>(a.c[2], b.c[3]), mmul<F>(a.c[3], b.c[2]));
  uint32_t t6 = mmul<F>(a.c[3], b.c[3]);
  ef4 r;
  r.c[0] = madd<F>(mmul<F>(a.c[0], b.c[0]), mmul<F>(F::W, t4));
  r.c[1] = madd<F>(madd<F>(mmul<F>(a.c[0], b.c[1]), mmul<F>(a.c[1], b.c[0])),
                   mmul<F>(F::W, t5));
  r.c[2] = madd<F>(madd<F>(madd<F>(mmul<F>(a.c[0], b.c[2]), mmul<F>(a.c[1], b.c[1])),
                           mmul<F>(a.c[2], b.c[0])),
                   mmul<F>(F::W, t6));
  r.c[3] = madd<F>(madd<F>(mmul<F>(a.c[0], b.c[3]), mmul<F>(a.c[1], b.c[2])),
                   madd<F>(mmul<F>(a.c[2], b.c[1]), mmul<F>(a.c[3], b.c[0])));
  return r;
}

// EF4 inverse through the norm. With y = x^2, a = e(y) + x o(y) for
// e = a0 + a2 y, o = a1 + a3 y, and a(x) a(-x) = e^2 - y o^2 = c0 + c1 y in
// F[y]/(y^2 - W); (c0 + c1 y)(c0 - c1 y) = c0^2 - W c1^2 = n lies in F. So
// a^-1 = a(-x) (c0 - c1 x^2) / n, one base-field inversion; zero maps to zero.
template <class F>
ZC_HD ef4 ef_inv(const ef4& a) {
  const uint32_t a0 = a.c[0], a1 = a.c[1], a2 = a.c[2], a3 = a.c[3];
  const uint32_t a13 = mmul<F>(a1, a3), a02 = mmul<F>(a0, a2);
  const uint32_t c0 = msub<F>(madd<F>(mmul<F>(a0, a0), mmul<F>(F::W, mmul<F>(a2, a2))),
                              mmul<F>(F::W, madd<F>(a13, a13)));
  const uint32_t c1 = msub<F>(madd<F>(a02, a02),
                              madd<F>(mmul<F>(a1, a1), mmul<F>(F::W, mmul<F>(a3, a3))));
  const uint32_t n = msub<F>(mmul<F>(c0, c0), mmul<F>(F::W, mmul<F>(c1, c1)));
  const ef4 conj{{a0, mneg<F>(a1), a2, mneg<F>(a3)}};
  const ef4 d{{c0, 0u, mneg<F>(c1), 0u}};
  return ef_scale<F>(ef_mul<F>(conj, d), minv<F>(n));
}

}  // namespace zc
