// The FRI fold kernels and their launchers, shared by the natural-order unit
// (zc_fold.cu) and the bit-reversed unit (zc_fold_bitrev.cu), which compile
// in parallel.
#pragma once
#include "tree.cuh"

namespace zc {

template <class F, int LI, int LB, bool BR>
__global__ void k_fold(const uint32_t* f, int64_t n, const uint32_t* beta, uint32_t inv2s,
                       uint32_t winv, uint32_t* g) {
  using M = FoldMath<F, LI, LB>;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t half = n >> 1;
  if (j >= half) return;
  uint32_t bt[4];
#pragma unroll
  for (int e = 0; e < LB; e++) bt[e] = __ldg(beta + e);
  uint32_t out[4];
  if (BR)  // pair (f[2j], f[2j+1]) at x_j = shift w^brev(j)
    M::fold(f + 2 * j * LI, 1, 0,
            mmul<F>(inv2s, mpow<F>(winv, (uint64_t)brev64(j, ilog2_dev(half)))), bt, out);
  else
    M::fold(f, half, j, mmul<F>(inv2s, mpow<F>(winv, (uint64_t)j)), bt, out);
#pragma unroll
  for (int e = 0; e < M::LO; e++) g[j * M::LO + e] = out[e];
}

// k-ary fold (ReedSolomon.fold_group, zorch/coding/reed_solomon.py:357-381) by
// the coset form of fri_fold_k (:551-586): group p < n/K is
// (f[p], f[p + n/K], ..., f[p + (K-1) n/K]) on the points x0 w_K^m, x0 =
// shift w_n^p, so its interpolant is Q(Y) = P(x0 Y) = sum_j c_j Y^j with
// c = (1/K) sum_m g_m w_K^(-jm), and out[p] = Q(beta / x0) (Horner). The
// interpolant is unique, so this equals the Lagrange form of the reference.
template <class F, int LI, int LB, int K>
__global__ void k_fold_k(const uint32_t* f, int64_t n, const uint32_t* beta, uint32_t shinv,
                         uint32_t winv, uint32_t wkinv, uint32_t kinv, uint32_t* g) {
  constexpr int LO = (LI == 4 || LB == 4) ? 4 : 1;
  const int64_t sub = n / K;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= sub) return;
  ef4 v[K];
#pragma unroll
  for (int m = 0; m < K; m++) {
    v[m] = ef4{{0, 0, 0, 0}};
#pragma unroll
    for (int e = 0; e < LI; e++) v[m].c[e] = __ldg(f + (p + m * sub) * LI + e);
  }
  uint32_t wk[K];  // w_K^(-j)
  wk[0] = F::ONE;
#pragma unroll
  for (int j = 1; j < K; j++) wk[j] = mmul<F>(wk[j - 1], wkinv);
  const uint32_t x0inv = mmul<F>(shinv, mpow<F>(winv, (uint64_t)p));
  ef4 u{{0, 0, 0, 0}};
#pragma unroll
  for (int e = 0; e < LB; e++) u.c[e] = mmul<F>(__ldg(beta + e), x0inv);
  ef4 acc{{0, 0, 0, 0}};
#pragma unroll
  for (int j = K - 1; j >= 0; j--) {
    ef4 c{{0, 0, 0, 0}};
#pragma unroll
    for (int m = 0; m < K; m++) c = ef_add<F>(c, ef_scale<F>(v[m], wk[(j * m) & (K - 1)]));
    c = ef_scale<F>(c, kinv);
    acc = ef_add<F>(LB == 4 ? ef_mul<F>(acc, u) : ef_scale<F>(acc, u.c[0]), c);
  }
#pragma unroll
  for (int e = 0; e < LO; e++) g[p * LO + e] = acc.c[e];
}

template <class F, int LI, int LB>
zc_status fold_k_launch(const uint32_t* cw, int64_t n, const uint32_t* beta, int log_k,
                        uint32_t shift_mont, uint32_t* out, cudaStream_t st) {
  const int log_n = ilog2(n);
  const uint32_t winv = minv<F>(root_of_unity<F>(log_n, 0));
  const uint32_t wkinv = mpow<F>(winv, (uint64_t)(n >> log_k));
  const uint32_t shinv = minv<F>(shift_mont ? shift_mont : F::ONE);
  const uint32_t kinv = minv<F>(to_mont<F>(1u << log_k));
  const int64_t sub = n >> log_k;
  const unsigned grid = (unsigned)((sub + 127) / 128);
  switch (log_k) {
    case 1: k_fold_k<F, LI, LB, 2><<<grid, 128, 0, st>>>(cw, n, beta, shinv, winv, wkinv, kinv, out); break;
    case 2: k_fold_k<F, LI, LB, 4><<<grid, 128, 0, st>>>(cw, n, beta, shinv, winv, wkinv, kinv, out); break;
    case 3: k_fold_k<F, LI, LB, 8><<<grid, 128, 0, st>>>(cw, n, beta, shinv, winv, wkinv, kinv, out); break;
    default: k_fold_k<F, LI, LB, 16><<<grid, 128, 0, st>>>(cw, n, beta, shinv, winv, wkinv, kinv, out); break;
  }
  return launch_check();
}

template <class F>
struct FoldScalars {
  uint32_t inv2s, winv, w4inv;
};

template <class F>
zc_status fold_scalars(int64_t n, uint32_t shift_mont, uint32_t generator, FoldScalars<F>* o) {
  if (generator != 0 && generator != F::GEN) {
    set_error("only the field's canonical generator is built");
    return ZC_UNSUPPORTED;
  }
  const int log_n = ilog2(n);
  const uint32_t w = root_of_unity<F>(log_n, generator);
  o->winv = minv<F>(w);
  const uint32_t sh = shift_mont ? shift_mont : F::ONE;
  o->inv2s = mmul<F>(F::INV2, minv<F>(sh));
  o->w4inv = n >= 4 ? mpow<F>(o->winv, (uint64_t)(n >> 2)) : F::ONE;
  return ZC_OK;
}

template <class F, int LI, int LB, bool BR>
zc_status fold_launch(const uint32_t* cw, int64_t n, const uint32_t* beta, uint32_t shift_mont,
                      uint32_t generator, uint32_t* out, cudaStream_t st) {
  FoldScalars<F> fs;
  ZC_TRY(fold_scalars<F>(n, shift_mont, generator, &fs));
  const int64_t half = n >> 1;
  const int B = 256;
  k_fold<F, LI, LB, BR><<<(unsigned)((half + B - 1) / B), B, 0, st>>>(cw, n, beta, fs.inv2s,
                                                                      fs.winv, out);
  return launch_check();
}

template <class K, int LI, int LB, bool BR>
zc_status fold_commit_launch(const uint32_t* cw, int64_t n, const uint32_t* beta,
                             uint32_t shift_mont, uint32_t generator, uint32_t* out,
                             uint32_t* layers, const P2Params* rt, cudaStream_t st,
                             RootHop hop) {
  using F = typename K::F;
  FoldScalars<F> fs;
  ZC_TRY(fold_scalars<F>(n, shift_mont, generator, &fs));
  FoldLeaf<F, LI, LB, BR> leaf{cw, out, beta, n, fs.inv2s, fs.winv, fs.w4inv};
  return commit_tree<K>(leaf, layers, n >> 2, rt, st, hop);
}

template <bool BR>
zc_status fri_fold_any(zc_field field, const uint32_t* cw, int64_t n, int ef_in,
                       const uint32_t* beta, int ef_beta, uint32_t shift_mont, uint32_t generator,
                       uint32_t* out, cudaStream_t st) {
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    if (ef_in && ef_beta)
      return fold_launch<F, 4, 4, BR>(cw, n, beta, shift_mont, generator, out, st);
    if (ef_in) return fold_launch<F, 4, 1, BR>(cw, n, beta, shift_mont, generator, out, st);
    if (ef_beta) return fold_launch<F, 1, 4, BR>(cw, n, beta, shift_mont, generator, out, st);
    return fold_launch<F, 1, 1, BR>(cw, n, beta, shift_mont, generator, out, st);
  });
}

template <bool BR>
zc_status fold_commit_any(const zc_poseidon2* p, const uint32_t* cw, int64_t n, int ef_in,
                          const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                          uint32_t generator, uint32_t* out, uint32_t* layers, cudaStream_t st,
                          RootHop hop = RootHop{nullptr, nullptr, 0}) {
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    if (ef_in && ef_beta)
      return fold_commit_launch<K, 4, 4, BR>(cw, n, beta, shift_mont, generator, out, layers, rt,
                                             st, hop);
    if (ef_in)
      return fold_commit_launch<K, 4, 1, BR>(cw, n, beta, shift_mont, generator, out, layers, rt,
                                             st, hop);
    if (ef_beta)
      return fold_commit_launch<K, 1, 4, BR>(cw, n, beta, shift_mont, generator, out, layers, rt,
                                             st, hop);
    return fold_commit_launch<K, 1, 1, BR>(cw, n, beta, shift_mont, generator, out, layers, rt,
                                           st, hop);
  });
}

// The bit-reversed fused fold-and-commit (zc_fold_bitrev.cu).
zc_status fold_commit_bitrev(const zc_poseidon2* p, const uint32_t* cw, int64_t n, int ef_in,
                             const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                             uint32_t generator, uint32_t* out, uint32_t* layers, cudaStream_t st,
                             RootHop hop);

}  // namespace zc
