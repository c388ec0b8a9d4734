// The DEEP side of the FRI open (FriProver._open_one, zorch/pcs/fri/prover.py:
// 151-187): the claimed value v = f(z) from the coefficients, and the layer-0
// quotient g = (f - v) / (x - z) over the evaluation domain, z either a base
// element or an EF4 element (then v and g are EF4).
//
// eval: a two-level Horner. Thread t of T (coalesced, interleaved) evaluates
// P_t = sum_j c[t + jT] u^j with u = z^T; a block combines its threads'
// P_t z^(t - t0) by a shared-memory tree (level s multiplies the upper half by
// z^(2^s)); a second one-block launch combines the block partials the same way
// with z^256.
//
// quotient: each thread takes 8 consecutive domain points, forms the
// denominators x_j - z and inverts them together (Montgomery's batch trick:
// prefix products, one inversion, back substitution -- 3 products per element
// plus one inversion per 8), so an EF4 quotient costs about three EF4 products
// per element. A zero denominator (z on the domain) gives a zero quotient, the
// 0^-1 = 0 convention of a Fermat inverse.
#include "internal.cuh"

namespace zc {

// Element of L limbs (1: base, 4: EF4) carried in an ef4.
template <class F, int L>
__device__ __forceinline__ ef4 e_mul(const ef4& a, const ef4& b) {
  if constexpr (L == 1) return ef4{{mmul<F>(a.c[0], b.c[0]), 0u, 0u, 0u}};
  else return ef_mul<F>(a, b);
}
template <class F, int L>
__device__ __forceinline__ ef4 e_add(const ef4& a, const ef4& b) {
  if constexpr (L == 1) return ef4{{madd<F>(a.c[0], b.c[0]), 0u, 0u, 0u}};
  else return ef_add<F>(a, b);
}
template <class F, int L>
__device__ __forceinline__ ef4 e_inv(const ef4& a) {
  if constexpr (L == 1) return ef4{{minv<F>(a.c[0]), 0u, 0u, 0u}};
  else return ef_inv<F>(a);
}
template <int L>
__device__ __forceinline__ ef4 e_load(const uint32_t* p) {
  ef4 r{{p[0], 0u, 0u, 0u}};
  if constexpr (L == 4) {
    r.c[1] = p[1];
    r.c[2] = p[2];
    r.c[3] = p[3];
  }
  return r;
}
template <int L>
__device__ __forceinline__ void e_store(uint32_t* p, const ef4& a) {
  if constexpr (L == 1) p[0] = a.c[0];
  else *reinterpret_cast<uint4*>(p) = make_uint4(a.c[0], a.c[1], a.c[2], a.c[3]);
}
template <int L>
__device__ __forceinline__ bool e_zero(const ef4& a) {
  if constexpr (L == 1) return a.c[0] == 0u;
  else return (a.c[0] | a.c[1] | a.c[2] | a.c[3]) == 0u;
}

constexpr int kEvalT = 256;
constexpr int kEvalMaxBlocks = 128;

// sm[0] = sum_i sm[i] zz^i over the kEvalT slots (zz = z^stride of the slots).
template <class F, int L>
__device__ __forceinline__ void combine_slots(ef4* sm, ef4 zz, int count) {
  const int t = threadIdx.x;
  for (int s = 1; s < count; s <<= 1) {
    __syncthreads();
    if ((t & (2 * s - 1)) == 0 && t + s < count) sm[t] = e_add<F, L>(sm[t], e_mul<F, L>(sm[t + s], zz));
    zz = e_mul<F, L>(zz, zz);
  }
  __syncthreads();
}

template <class F, int L>
__global__ void __launch_bounds__(kEvalT) k_eval_partial(const uint32_t* c, int64_t k,
                                                         const uint32_t* z, int log_threads,
                                                         uint32_t* part) {
  __shared__ ef4 sm[kEvalT];
  const ef4 zz = e_load<L>(z);
  ef4 u = zz;  // z^T, T = 2^log_threads
  for (int i = 0; i < log_threads; i++) u = e_mul<F, L>(u, u);
  const int64_t T = (int64_t)1 << log_threads;
  const int64_t t = (int64_t)blockIdx.x * kEvalT + threadIdx.x;
  ef4 acc{{0u, 0u, 0u, 0u}};
  if (t < k) {
    int64_t j = (k - 1 - t) / T;  // last j with t + jT < k
    for (; j >= 0; j--) {
      acc = e_mul<F, L>(acc, u);
      acc.c[0] = madd<F>(acc.c[0], __ldg(c + t + j * T));
    }
  }
  sm[threadIdx.x] = acc;
  combine_slots<F, L>(sm, zz, kEvalT);
  if (threadIdx.x == 0) e_store<4>(part + 4 * blockIdx.x, sm[0]);
}

template <class F, int L>
__global__ void __launch_bounds__(kEvalMaxBlocks) k_eval_final(const uint32_t* part, int blocks,
                                                               const uint32_t* z, uint32_t* out) {
  __shared__ ef4 sm[kEvalMaxBlocks];
  ef4 zz = e_load<L>(z);  // z^kEvalT between consecutive block partials
  for (int i = 0; (1 << i) < kEvalT; i++) zz = e_mul<F, L>(zz, zz);
  sm[threadIdx.x] = threadIdx.x < blocks ? e_load<4>(part + 4 * threadIdx.x)
                                         : ef4{{0u, 0u, 0u, 0u}};
  combine_slots<F, L>(sm, zz, blockDim.x);
  if (threadIdx.x == 0) e_store<L>(out, sm[0]);
}

constexpr int kDeepM = 8;

// g[j] = (cw[j] - v) / (x_j - z), x_j = shift * w^j (natural) or
// shift * w^brev(j) (bit-reversed codeword), for the 8 points of one thread.
template <class F, int L, bool BR>
__global__ void __launch_bounds__(256) k_deep_quotient(const uint32_t* cw, int64_t n, int log_n,
                                                       const uint32_t* z, const uint32_t* v,
                                                       uint32_t shift, uint32_t w,
                                                       uint32_t* out) {
  const int64_t j0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kDeepM;
  if (j0 >= n) return;
  const ef4 zz = e_load<L>(z), vv = e_load<L>(v);
  ef4 d[kDeepM], pre[kDeepM];
  uint32_t f[kDeepM];
  bool zero[kDeepM];
  uint32_t x = BR ? 0u : mmul<F>(shift, mpow<F>(w, (uint64_t)j0));
#pragma unroll
  for (int i = 0; i < kDeepM; i++) {
    const int64_t j = j0 + i;
    const bool on = j < n;
    if (BR && on) {
      const uint64_t e = log_n ? (__brevll((unsigned long long)j) >> (64 - log_n)) : 0;
      x = mmul<F>(shift, mpow<F>(w, e));
    }
    ef4 di{{msub<F>(x, zz.c[0]), mneg<F>(zz.c[1]), mneg<F>(zz.c[2]), mneg<F>(zz.c[3])}};
    if (L == 1) di.c[1] = di.c[2] = di.c[3] = 0u;
    zero[i] = !on || e_zero<L>(di);
    d[i] = zero[i] ? ef4{{F::ONE, 0u, 0u, 0u}} : di;
    f[i] = on ? __ldg(cw + j) : 0u;
    pre[i] = i ? e_mul<F, L>(pre[i - 1], d[i]) : d[i];
    if (!BR) x = mmul<F>(x, w);
  }
  ef4 inv = e_inv<F, L>(pre[kDeepM - 1]);
#pragma unroll
  for (int i = kDeepM - 1; i >= 0; i--) {
    const ef4 di_inv = i ? e_mul<F, L>(inv, pre[i - 1]) : inv;
    if (i) inv = e_mul<F, L>(inv, d[i]);
    const int64_t j = j0 + i;
    if (j < n) {
      ef4 num{{msub<F>(f[i], vv.c[0]), mneg<F>(vv.c[1]), mneg<F>(vv.c[2]), mneg<F>(vv.c[3])}};
      ef4 q = e_mul<F, L>(num, di_inv);
      if (zero[i]) q = ef4{{0u, 0u, 0u, 0u}};
      e_store<L>(out + j * L, q);
    }
  }
}

}  // namespace zc

using namespace zc;

extern "C" {

size_t zc_eval_poly_workspace_bytes(int64_t k) {
  (void)k;
  return 16 * kEvalMaxBlocks;
}

zc_status zc_eval_poly(zc_field field, const uint32_t* coeffs, int64_t k, const uint32_t* z,
                       int32_t z_limbs, uint32_t* out, void* workspace, size_t workspace_bytes,
                       void* stream) {
  if (k < 1 || !coeffs || !z || !out || (z_limbs != 1 && z_limbs != 4)) return ZC_BAD_ARG;
  if (!workspace || workspace_bytes < zc_eval_poly_workspace_bytes(k) ||
      (uintptr_t)workspace % 16 || (z_limbs == 4 && ((uintptr_t)out % 16 || (uintptr_t)z % 4)))
    return ZC_BAD_ARG;
  ZC_TRY(ensure_init());
  cudaStream_t st = (cudaStream_t)stream;
  int64_t blocks = (k + kEvalT - 1) / kEvalT;
  if (blocks > kEvalMaxBlocks) blocks = kEvalMaxBlocks;
  int lb = 0;
  while ((1ll << (lb + 1)) <= blocks) lb++;
  blocks = 1ll << lb;  // T = blocks * kEvalT, a power of two
  const int log_threads = lb + 8;
  uint32_t* part = (uint32_t*)workspace;
  return with_field(field, [&](auto f) -> zc_status {
    using F = decltype(f);
    if (z_limbs == 1) {
      k_eval_partial<F, 1><<<(unsigned)blocks, kEvalT, 0, st>>>(coeffs, k, z, log_threads, part);
      ZC_TRY(launch_check());
      k_eval_final<F, 1><<<1, kEvalMaxBlocks, 0, st>>>(part, (int)blocks, z, out);
    } else {
      k_eval_partial<F, 4><<<(unsigned)blocks, kEvalT, 0, st>>>(coeffs, k, z, log_threads, part);
      ZC_TRY(launch_check());
      k_eval_final<F, 4><<<1, kEvalMaxBlocks, 0, st>>>(part, (int)blocks, z, out);
    }
    return launch_check();
  });
}

zc_status zc_deep_quotient(zc_field field, const uint32_t* cw, int64_t n, const uint32_t* z,
                           int32_t z_limbs, const uint32_t* v, uint32_t shift_mont,
                           uint32_t generator, int32_t bit_reversed, uint32_t* out,
                           void* stream) {
  if (!cw || !z || !v || !out || (z_limbs != 1 && z_limbs != 4)) return ZC_BAD_ARG;
  if (!is_pow2(n)) return ZC_NOT_POW2;
  if (z_limbs == 4 && (uintptr_t)out % 16) return ZC_BAD_ARG;
  ZC_TRY(ensure_init());
  cudaStream_t st = (cudaStream_t)stream;
  const int log_n = ilog2(n);
  const int64_t threads = (n + kDeepM - 1) / kDeepM;
  const unsigned grid = (unsigned)((threads + 255) / 256);
  return with_field(field, [&](auto f) -> zc_status {
    using F = decltype(f);
    if (generator && generator != F::GEN) return ZC_UNSUPPORTED;
    if (log_n > F::TWO_ADICITY) return ZC_BAD_SHAPE;
    const uint32_t w = root_of_unity<F>(log_n, 0);
    const uint32_t sh = shift_mont ? shift_mont : F::ONE;
    if (z_limbs == 1) {
      if (bit_reversed)
        k_deep_quotient<F, 1, true><<<grid, 256, 0, st>>>(cw, n, log_n, z, v, sh, w, out);
      else
        k_deep_quotient<F, 1, false><<<grid, 256, 0, st>>>(cw, n, log_n, z, v, sh, w, out);
    } else {
      if (bit_reversed)
        k_deep_quotient<F, 4, true><<<grid, 256, 0, st>>>(cw, n, log_n, z, v, sh, w, out);
      else
        k_deep_quotient<F, 4, false><<<grid, 256, 0, st>>>(cw, n, log_n, z, v, sh, w, out);
    }
    return launch_check();
  });
}

}  // extern "C"
