// Width-16 Poseidon2 permutation, sponge and 2-to-1 compression on one thread's
// registers. Semantics follow hash-frx / Plonky3 as pinned by the reference's
// KoalaBear-16 golden root (zorch/commit/testing/merkle_test.py:51-63):
// initial external layer, R_F/2 full rounds, R_P partial rounds, R_F/2 full
// rounds; external layer = M4 = circ(2,3,1,1) per 4-lane block plus the
// lane-class sums; internal layer s_i <- j*sum(s) + diag_i * s_i.
//
// Two constant providers:
//  - Bb16Builtin: the built-in BabyBear-16 instance (x^7, 4+4+13), constants in
//    __constant__ memory, compile-time shape;
//  - RtParams:    any width-16 instance passed at run time (the reference's
//    Poseidon2Params), staged into shared memory by the kernel.
#pragma once
#include "field.cuh"
#include "poseidon2_babybear16.h"

namespace zc {

// Run-time Poseidon2 parameters (all Montgomery). Mirrors hash-frx's
// Poseidon2Params fields as used at zorch/testkit/koalabear16.py:253-263.
struct P2Params {
  uint32_t field_id;
  uint32_t alpha;
  uint32_t rounds_f_half;
  uint32_t rounds_p;
  uint32_t ext_init[8][16];
  uint32_t ext_term[8][16];
  uint32_t int_rc[64];
  uint32_t diag[16];
  uint32_t j_scale;
  uint32_t j_is_one;
};

static __constant__ uint32_t c_bb16_ext_init[64] = ZC_BB16_EXT_INIT_MONT_INIT;
static __constant__ uint32_t c_bb16_ext_term[64] = ZC_BB16_EXT_TERM_MONT_INIT;
static __constant__ uint32_t c_bb16_int_rc[ZC_BB16_ROUNDS_P] = ZC_BB16_INT_RC_MONT_INIT;
static __constant__ uint32_t c_bb16_diag[16] = ZC_BB16_DIAG_MONT_INIT;

// Round-constant addition and S-box x -> (x + c)^alpha for x, c in [0, p):
// x + c - p lies in [-p, p) and is one three-operand add, and the power chain
// runs on signed Montgomery products (smul) with a single normalisation at
// the end. Exponents other than 3, 5, 7 take the generic square-and-multiply.
template <class F, int ALPHA>
ZC_HD uint32_t ark_sbox_a(uint32_t x, uint32_t c, uint32_t alpha) {
  const int32_t a = (int32_t)(x + c - F::P);
  if (ALPHA == 3) return snorm<F>(smul<F>(smul<F>(a, a), a));
  if (ALPHA == 5) {
    const int32_t a2 = smul<F>(a, a);
    return snorm<F>(smul<F>(smul<F>(a2, a2), a));
  }
  if (ALPHA == 7) {
    const int32_t a2 = smul<F>(a, a);
    return snorm<F>(smul<F>(smul<F>(a2, a), smul<F>(a2, a2)));
  }
  return mpow<F>(madd<F>(x, c), alpha);
}

// Multiplications by the built-in BabyBear diagonal entries without a
// Montgomery product (the representation is linear, so a constant c acts on
// Mont(x) as on x). p = 15 * 2^27 + 1, so for k <= 27 and q = (-x) mod 2^k,
// x + q*p is divisible by 2^k and x * 2^-k = ((x + q) >> k) + q * 15 * 2^(27-k).
struct Bb {
  static constexpr uint32_t P = BabyBear::P;
  __device__ __forceinline__ static uint32_t dbl(uint32_t x) { return madd<BabyBear>(x, x); }
  __device__ __forceinline__ static uint32_t half(uint32_t x) {
    return (x & 1u) ? (x >> 1) + ((P + 1) >> 1) : (x >> 1);
  }
  template <int K>
  __device__ __forceinline__ static uint32_t div2exp(uint32_t x) {
    static_assert(K >= 1 && K <= 27, "k out of range");
    const uint32_t q = (0u - x) & ((1u << K) - 1u);
    const uint32_t r = ((x + q) >> K) + q * (15u << (27 - K));
    const uint32_t t = r - P;
    return t < r ? t : r;
  }
};

struct Bb16Builtin {
  using F = BabyBear;
  // Internal layer s_i <- sum + d_i s_i for the built-in diagonal
  // [-2, 1, 2, 1/2, 3, 4, -1/2, -3, -4, 2^-8, 1/4, 1/8, 2^-27, -2^-8, -1/16, -2^-27]
  // on the integer ALU pipe instead of 16 Montgomery products.
  __device__ __forceinline__ void internal_layer(uint32_t* s) const {
    using B = Bb;
    uint32_t part = madd<F>(madd<F>(madd<F>(s[1], s[2]), madd<F>(s[3], s[4])),
                            madd<F>(madd<F>(s[5], s[6]), madd<F>(s[7], s[8])));
    part = madd<F>(part, madd<F>(madd<F>(madd<F>(s[9], s[10]), madd<F>(s[11], s[12])),
                                 madd<F>(madd<F>(s[13], s[14]), s[15])));
    const uint32_t sum = madd<F>(part, s[0]);
    s[0] = msub<F>(part, s[0]);  // sum - 2 s0
    s[1] = madd<F>(sum, s[1]);
    s[2] = madd<F>(sum, B::dbl(s[2]));
    s[3] = madd<F>(sum, B::half(s[3]));
    s[4] = madd<F>(sum, madd<F>(B::dbl(s[4]), s[4]));
    s[5] = madd<F>(sum, B::dbl(B::dbl(s[5])));
    s[6] = msub<F>(sum, B::half(s[6]));
    s[7] = msub<F>(sum, madd<F>(B::dbl(s[7]), s[7]));
    s[8] = msub<F>(sum, B::dbl(B::dbl(s[8])));
    s[9] = madd<F>(sum, B::div2exp<8>(s[9]));
    s[10] = madd<F>(sum, B::div2exp<2>(s[10]));
    s[11] = madd<F>(sum, B::div2exp<3>(s[11]));
    s[12] = madd<F>(sum, B::div2exp<27>(s[12]));
    s[13] = msub<F>(sum, B::div2exp<8>(s[13]));
    s[14] = msub<F>(sum, B::div2exp<4>(s[14]));
    s[15] = msub<F>(sum, B::div2exp<27>(s[15]));
  }
  static constexpr int RF_HALF = ZC_BB16_ROUNDS_F_HALF;
  __device__ __forceinline__ int rf_half() const { return RF_HALF; }
  __device__ __forceinline__ int rp() const { return ZC_BB16_ROUNDS_P; }
  __device__ __forceinline__ uint32_t ei(int r, int i) const { return c_bb16_ext_init[r * 16 + i]; }
  __device__ __forceinline__ uint32_t et(int r, int i) const { return c_bb16_ext_term[r * 16 + i]; }
  __device__ __forceinline__ uint32_t ir(int r) const { return c_bb16_int_rc[r]; }
  __device__ __forceinline__ uint32_t dg(int i) const { return c_bb16_diag[i]; }
  __device__ __forceinline__ uint32_t ark_sbox(uint32_t x, uint32_t c) const {
    return ark_sbox_a<F, 7>(x, c, 7);
  }
  __device__ __forceinline__ uint32_t jsum(uint32_t s) const { return s; }
};

template <class F_>
struct RtParams {
  using F = F_;
  const P2Params* p;  // shared memory on the device, plain memory on the host
  ZC_HD int rf_half() const { return (int)p->rounds_f_half; }
  ZC_HD int rp() const { return (int)p->rounds_p; }
  ZC_HD uint32_t ei(int r, int i) const { return p->ext_init[r][i]; }
  ZC_HD uint32_t et(int r, int i) const { return p->ext_term[r][i]; }
  ZC_HD uint32_t ir(int r) const { return p->int_rc[r]; }
  ZC_HD uint32_t dg(int i) const { return p->diag[i]; }
  ZC_HD uint32_t ark_sbox(uint32_t x, uint32_t c) const {
    switch (p->alpha) {
      case 3: return ark_sbox_a<F, 3>(x, c, 3);
      case 5: return ark_sbox_a<F, 5>(x, c, 5);
      case 7: return ark_sbox_a<F, 7>(x, c, 7);
      default: return ark_sbox_a<F, 0>(x, c, p->alpha);
    }
  }
  ZC_HD uint32_t jsum(uint32_t s) const { return p->j_is_one ? s : mmul<F>(s, p->j_scale); }
  // Generic internal layer s_i <- j*sum(s) + diag_i * s_i.
  ZC_HD void internal_layer(uint32_t* s) const {
    uint32_t a0 = madd<F>(madd<F>(s[0], s[1]), madd<F>(s[2], s[3]));
    uint32_t a1 = madd<F>(madd<F>(s[4], s[5]), madd<F>(s[6], s[7]));
    uint32_t a2 = madd<F>(madd<F>(s[8], s[9]), madd<F>(s[10], s[11]));
    uint32_t a3 = madd<F>(madd<F>(s[12], s[13]), madd<F>(s[14], s[15]));
    uint32_t sum = jsum(madd<F>(madd<F>(a0, a1), madd<F>(a2, a3)));
#pragma unroll
    for (int i = 0; i < 16; i++) s[i] = madd<F>(sum, mmul<F>(dg(i), s[i]));
  }
};

// External (M4 block-circulant) linear layer.
template <class F>
ZC_HD void p2_ext_linear(uint32_t* s) {
#pragma unroll
  for (int c = 0; c < 16; c += 4) {
    uint32_t x0 = s[c], x1 = s[c + 1], x2 = s[c + 2], x3 = s[c + 3];
    uint32_t t01 = madd<F>(x0, x1), t23 = madd<F>(x2, x3);
    uint32_t t0123 = madd<F>(t01, t23);
    uint32_t t01123 = madd<F>(t0123, x1), t01233 = madd<F>(t0123, x3);
    s[c + 3] = madd<F>(t01233, madd<F>(x0, x0));
    s[c + 1] = madd<F>(t01123, madd<F>(x2, x2));
    s[c + 0] = madd<F>(t01123, t01);
    s[c + 2] = madd<F>(t01233, t23);
  }
  uint32_t sums[4];
#pragma unroll
  for (int k = 0; k < 4; k++)
    sums[k] = madd<F>(madd<F>(s[k], s[4 + k]), madd<F>(s[8 + k], s[12 + k]));
#pragma unroll
  for (int i = 0; i < 16; i++) s[i] = madd<F>(s[i], sums[i & 3]);
}

#pragma nv_exec_check_disable
template <class K>
ZC_HD void p2_permute(uint32_t* s, const K& k) {
  using F = typename K::F;
  p2_ext_linear<F>(s);
#pragma unroll 1
  for (int r = 0; r < k.rf_half(); r++) {
#pragma unroll
    for (int i = 0; i < 16; i++) s[i] = k.ark_sbox(s[i], k.ei(r, i));
    p2_ext_linear<F>(s);
  }
#pragma unroll 1
  for (int r = 0; r < k.rp(); r++) {
    s[0] = k.ark_sbox(s[0], k.ir(r));
    k.internal_layer(s);
  }
#pragma unroll 1
  for (int r = 0; r < k.rf_half(); r++) {
#pragma unroll
    for (int i = 0; i < 16; i++) s[i] = k.ark_sbox(s[i], k.et(r, i));
    p2_ext_linear<F>(s);
  }
}

// TruncatedPermutation<2, 8, 16>: permute(l || r)[0:8].
#pragma nv_exec_check_disable
template <class K>
ZC_HD void p2_compress(const uint32_t* l, const uint32_t* r, uint32_t* out,
                                            const K& k) {
  uint32_t s[16];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    s[i] = l[i];
    s[8 + i] = r[i];
  }
  p2_permute(s, k);
#pragma unroll
  for (int i = 0; i < 8; i++) out[i] = s[i];
}

// ------------------------------------------------------------- halves ---
// The same permutation on a half-warp (lanes 16h .. 16h+15): lane l of the
// half holds state word l. One thread's permutation is a dependency chain of
// ~7000 instructions (~9.4 us at 2.07 GHz, measured); on a half-warp each lane
// runs one S-box per round and the linear layers are butterflies of shuffles,
// which brings a permutation to ~3 us. The latency-bound parts of a commit --
// the narrow top levels of a tree and the transcript -- use halves.
//  - external layer: y_j = s_b + x_j + 2 x_{j+1} is M4 = circ(2,3,1,1) on the
//    4-word block b (s_b = block sum, j + 1 mod 4), then y += the sum of y over
//    the lane class (xor 4, xor 8);
//  - partial round: the sum of lanes 1..15 is reduced while lane 0 runs its
//    S-box, and lane 0's new word is broadcast and added afterwards.
// Constants come from a P2Params in shared memory. Every lane of the warp must
// make the call (full-warp shuffles), active half or not.
constexpr unsigned kFullMask = 0xffffffffu;

template <class F>
__device__ __forceinline__ uint32_t half_sum16(uint32_t v) {
  v = madd<F>(v, __shfl_xor_sync(kFullMask, v, 1));
  v = madd<F>(v, __shfl_xor_sync(kFullMask, v, 2));
  v = madd<F>(v, __shfl_xor_sync(kFullMask, v, 4));
  return madd<F>(v, __shfl_xor_sync(kFullMask, v, 8));
}

template <class F>
__device__ __forceinline__ uint32_t half_ext_linear(uint32_t x) {
  const int lane = threadIdx.x & 31;
  const uint32_t nxt = __shfl_sync(kFullMask, x, (lane & ~3) | ((lane + 1) & 3));
  uint32_t s = madd<F>(x, __shfl_xor_sync(kFullMask, x, 1));
  s = madd<F>(s, __shfl_xor_sync(kFullMask, s, 2));
  const uint32_t y = madd<F>(madd<F>(s, x), madd<F>(nxt, nxt));
  uint32_t c = madd<F>(y, __shfl_xor_sync(kFullMask, y, 4));
  c = madd<F>(c, __shfl_xor_sync(kFullMask, c, 8));
  return madd<F>(y, c);
}

// The rounds are rolled loops (constants read from shared memory one round
// ahead): a permutation runs only a few times per launch here, so its code
// is fetched cold, and a short loop body costs far fewer instruction-cache
// misses than unrolled rounds.
template <class F, int ALPHA>
__device__ __forceinline__ uint32_t half_permute_a(uint32_t x, const P2Params* p) {
  const int l = threadIdx.x & 15;
  const int rfh = (int)p->rounds_f_half, rp = (int)p->rounds_p;
  const uint32_t alpha = p->alpha, dg = p->diag[l], js = p->j_scale;
  const bool jone = p->j_is_one != 0;
  x = half_ext_linear<F>(x);
  uint32_t c = rfh > 0 ? p->ext_init[0][l] : p->int_rc[0];
#pragma unroll 1
  for (int r = 0; r < rfh; r++) {
    const uint32_t c_next = r + 1 < rfh ? p->ext_init[r + 1][l] : p->int_rc[0];
    x = half_ext_linear<F>(ark_sbox_a<F, ALPHA>(x, c, alpha));
    c = c_next;
  }
#pragma unroll 1
  for (int r = 0; r < rp; r++) {
    const uint32_t c_next = r + 1 < rp ? p->int_rc[r + 1] : p->ext_term[0][l];
    const uint32_t s0 = ark_sbox_a<F, ALPHA>(x, c, alpha);  // lane 0's is used
    const uint32_t rest = half_sum16<F>(l == 0 ? 0u : x);   // lanes 1..15
    const uint32_t dx = mmul<F>(dg, l == 0 ? s0 : x);
    uint32_t sum = madd<F>(rest, __shfl_sync(kFullMask, s0, threadIdx.x & 16));
    if (!jone) sum = mmul<F>(sum, js);
    x = madd<F>(sum, dx);
    c = c_next;
  }
  if (rp == 0) c = p->ext_term[0][l];
#pragma unroll 1
  for (int r = 0; r < rfh; r++) {
    const uint32_t c_next = p->ext_term[r + 1 < rfh ? r + 1 : r][l];
    x = half_ext_linear<F>(ark_sbox_a<F, ALPHA>(x, c, alpha));
    c = c_next;
  }
  return x;
}

// Lane l (of the caller's half-warp) passes state word l and gets word l of
// the permuted state back. `p` points to shared memory.
template <class F>
__device__ __forceinline__ uint32_t p2_permute_half(uint32_t x, const P2Params* p) {
  switch (p->alpha) {
    case 3: return half_permute_a<F, 3>(x, p);
    case 5: return half_permute_a<F, 5>(x, p);
    case 7: return half_permute_a<F, 7>(x, p);
    default: return half_permute_a<F, 0>(x, p);
  }
}

// ----------------------------------------------------------- quarters ---
// The same permutation on a quarter-warp (lanes 4g .. 4g+3): lane q of the
// quarter holds the M4 block q (state words 4q .. 4q+3) in registers. The
// block matrix M4 is then local arithmetic, and only the sums over the four
// blocks need shuffles (xor 1, xor 2). In the partial rounds every lane keeps
// word 0 itself and runs its S-box redundantly, so the round needs no
// broadcast: the sum over words 1..15 (local, then two shuffle levels) runs
// while the S-box does, and every lane derives the new word 0 from the sum.
// Per permutation this is about 2.3x fewer thread instructions than the
// half-warp form, at no longer a dependency chain; it is the form used where
// many latency-bound permutations run side by side (tree tops, transcript).
// Every lane of the warp must make the call (full-warp shuffles).
template <class F>
__device__ __forceinline__ void m4_block(uint32_t (&x)[4]) {
  const uint32_t t01 = madd<F>(x[0], x[1]), t23 = madd<F>(x[2], x[3]);
  const uint32_t t0123 = madd<F>(t01, t23);
  const uint32_t t01123 = madd<F>(t0123, x[1]), t01233 = madd<F>(t0123, x[3]);
  const uint32_t y3 = madd<F>(t01233, madd<F>(x[0], x[0]));
  const uint32_t y1 = madd<F>(t01123, madd<F>(x[2], x[2]));
  x[0] = madd<F>(t01123, t01);
  x[2] = madd<F>(t01233, t23);
  x[1] = y1;
  x[3] = y3;
}

template <class F>
__device__ __forceinline__ void quarter_ext_linear(uint32_t (&x)[4]) {
  m4_block<F>(x);
  uint32_t s[4];
#pragma unroll
  for (int k = 0; k < 4; k++) s[k] = madd<F>(x[k], __shfl_xor_sync(kFullMask, x[k], 1));
#pragma unroll
  for (int k = 0; k < 4; k++) s[k] = madd<F>(s[k], __shfl_xor_sync(kFullMask, s[k], 2));
#pragma unroll
  for (int k = 0; k < 4; k++) x[k] = madd<F>(x[k], s[k]);
}

template <class F, int ALPHA>
__device__ __forceinline__ void quarter_permute_a(uint32_t (&x)[4], const P2Params* p) {
  const int q = threadIdx.x & 3;
  const int rfh = (int)p->rounds_f_half, rp = (int)p->rounds_p;
  const uint32_t alpha = p->alpha, js = p->j_scale, d0 = p->diag[0];
  const bool jone = p->j_is_one != 0;
  uint32_t dg[4];
#pragma unroll
  for (int k = 0; k < 4; k++) dg[k] = p->diag[4 * q + k];
  quarter_ext_linear<F>(x);
#pragma unroll 1
  for (int r = 0; r < rfh; r++) {
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = ark_sbox_a<F, ALPHA>(x[k], p->ext_init[r][4 * q + k], alpha);
    quarter_ext_linear<F>(x);
  }
  // word 0 on every lane of the quarter
  uint32_t w0 = __shfl_sync(kFullMask, x[0], threadIdx.x & ~3);
#pragma unroll 1
  for (int r = 0; r < rp; r++) {
    const uint32_t s0 = ark_sbox_a<F, ALPHA>(w0, p->int_rc[r], alpha);
    // words 1..15 of this round's input (lane 0's x[0] is word 0: left out)
    uint32_t part = madd<F>(madd<F>(q ? x[0] : 0u, x[1]), madd<F>(x[2], x[3]));
    part = madd<F>(part, __shfl_xor_sync(kFullMask, part, 1));
    part = madd<F>(part, __shfl_xor_sync(kFullMask, part, 2));
    uint32_t dx[4];
#pragma unroll
    for (int k = 0; k < 4; k++) dx[k] = mmul<F>(dg[k], x[k]);
    uint32_t sum = madd<F>(part, s0);
    if (!jone) sum = mmul<F>(sum, js);
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = madd<F>(sum, dx[k]);
    w0 = madd<F>(sum, mmul<F>(d0, s0));
    if (q == 0) x[0] = w0;
  }
#pragma unroll 1
  for (int r = 0; r < rfh; r++) {
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = ark_sbox_a<F, ALPHA>(x[k], p->ext_term[r][4 * q + k], alpha);
    quarter_ext_linear<F>(x);
  }
}

// Lane q (of the caller's quarter-warp) passes state words 4q .. 4q+3 and gets
// them back permuted. `p` points to shared memory.
template <class F>
__device__ __forceinline__ void p2_permute_quarter(uint32_t (&x)[4], const P2Params* p) {
  switch (p->alpha) {
    case 3: quarter_permute_a<F, 3>(x, p); break;
    case 5: quarter_permute_a<F, 5>(x, p); break;
    case 7: quarter_permute_a<F, 7>(x, p); break;
    default: quarter_permute_a<F, 0>(x, p); break;
  }
}

// The built-in BabyBear-16 instance on a half-warp, for permutations that run
// alone (the transcript's one-warp chains): the same rounds as half_permute_a,
// unrolled, with this lane's external-round constants and diagonal entry
// passed in registers (ei, et, dg: loaded once per kernel) and the
// partial-round constants read as constant-bank operands, so no round loads
// a constant or runs loop control.
static_assert(ZC_BB16_ROUNDS_F_HALF == 4, "built-in instance: 4 + 4 full rounds");
__device__ __forceinline__ uint32_t half_permute_bb16(uint32_t x, const uint32_t (&ei)[4],
                                                      const uint32_t (&et)[4], uint32_t dg) {
  using F = BabyBear;
  const int l = threadIdx.x & 15;
  x = half_ext_linear<F>(x);
#pragma unroll
  for (int r = 0; r < 4; r++) x = half_ext_linear<F>(ark_sbox_a<F, 7>(x, ei[r], 7));
#pragma unroll
  for (int r = 0; r < ZC_BB16_ROUNDS_P; r++) {
    const uint32_t s0 = ark_sbox_a<F, 7>(x, c_bb16_int_rc[r], 7);  // lane 0's is used
    const uint32_t rest = half_sum16<F>(l == 0 ? 0u : x);           // lanes 1..15
    const uint32_t dx = mmul<F>(dg, l == 0 ? s0 : x);
    x = madd<F>(madd<F>(rest, __shfl_sync(kFullMask, s0, threadIdx.x & 16)), dx);
  }
#pragma unroll
  for (int r = 0; r < 4; r++) x = half_ext_linear<F>(ark_sbox_a<F, 7>(x, et[r], 7));
  return x;
}

// Stage run-time params into shared memory (whole block participates).
__device__ __forceinline__ void stage_params(P2Params* dst, const P2Params* src) {
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(P2Params) / 4); i += blockDim.x) d[i] = s[i];
  __syncthreads();
}

}  // namespace zc
