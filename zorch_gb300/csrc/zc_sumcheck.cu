// The Basefold open's multilinear side on the GPU: eq tables, MLE
// evaluation of committed columns, staggered batching, and the interleaved
// sumcheck rounds (zorch/pcs/basefold/prover.py:419-547,
// zorch/pcs/basefold/kernel.py:52-78, zorch/poly/multilinear.py:92-109,
// zorch/poly/eq.py:55-130). EF4 values are 4 Montgomery limbs (c0..c3).
//
// Field sums are exact, so every reduction here is a deterministic tree of
// per-block partial sums whatever the order.
#include <algorithm>

#include "internal.cuh"

namespace zc {

__device__ __forceinline__ ef4 ld4(const uint32_t* p) {
  const uint4 v = *reinterpret_cast<const uint4*>(p);
  return ef4{{v.x, v.y, v.z, v.w}};
}
__device__ __forceinline__ void st4(uint32_t* p, const ef4& a) {
  *reinterpret_cast<uint4*>(p) = make_uint4(a.c[0], a.c[1], a.c[2], a.c[3]);
}
template <class F>
__device__ __forceinline__ ef4 ef_base(const ef4& a, uint32_t b) {  // EF4 * base
  return ef_scale<F>(a, b);
}

// Block-wide EF4 sum (blockDim a multiple of 32, <= 1024); the result is
// valid in thread 0.
template <class F>
__device__ ef4 block_sum(ef4 v) {
  __shared__ uint32_t red[4][32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int e = 0; e < 4; e++) v.c[e] = madd<F>(v.c[e], __shfl_xor_sync(0xffffffffu, v.c[e], o));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();  // red reused across calls
  if (lane == 0)
#pragma unroll
    for (int e = 0; e < 4; e++) red[e][warp] = v.c[e];
  __syncthreads();
  ef4 r{{0, 0, 0, 0}};
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int e = 0; e < 4; e++) r.c[e] = lane < nw ? red[e][lane] : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int e = 0; e < 4; e++) r.c[e] = madd<F>(r.c[e], __shfl_xor_sync(0xffffffffu, r.c[e], o));
  }
  return r;
}

// expand_eq_to_hypercube(z, 1) for m <= kEqSmall variables on one block:
// out[2i] = s - s z_j, out[2i+1] = s z_j per step (z[0] ends on the top bit).
constexpr int kEqSmall = 12;
template <class F>
__global__ void __launch_bounds__(1024) k_eq_small(const uint32_t* z, int m, uint32_t* out) {
  if (threadIdx.x == 0) st4(out, ef4{{F::ONE, 0, 0, 0}});
  __syncthreads();
  for (int j = 0; j < m; j++) {
    const ef4 zj = ld4(z + 4 * j);
    const int half = 1 << j;
    // read all of level j before anyone writes level j+1 (in place)
    ef4 lo[4], hi[4];
    int cnt = 0;
    for (int i = threadIdx.x; i < half && cnt < 4; i += blockDim.x, cnt++) {
      const ef4 s = ld4(out + 4 * i);
      hi[cnt] = ef_mul<F>(s, zj);
      lo[cnt] = ef_sub<F>(s, hi[cnt]);
    }
    __syncthreads();
    cnt = 0;
    for (int i = threadIdx.x; i < half && cnt < 4; i += blockDim.x, cnt++) {
      st4(out + 4 * (2 * i), lo[cnt]);
      st4(out + 4 * (2 * i + 1), hi[cnt]);
    }
    __syncthreads();
  }
}

// out[i] = hi[i >> m2] * lo[i & (2^m2 - 1)]: the table of z = (z_hi, z_lo) as
// the outer product of the halves' tables (exact, so equal to the doubling).
template <class F>
__global__ void k_eq_outer(const uint32_t* hi, const uint32_t* lo, int m2, int64_t total,
                           uint32_t* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    st4(out + 4 * i, ef_mul<F>(ld4(hi + 4 * (i >> m2)), ld4(lo + 4 * (i & ((1ll << m2) - 1)))));
}

inline int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b > 0 ? b : 1);
}

// Workspace of zc_eq_expand: the two half tables for m > kEqSmall.
inline size_t eq_ws_bytes(int m) {
  if (m <= kEqSmall) return 0;
  const int m1 = m / 2, m2 = m - m1;
  return (size_t)16 * (((size_t)1 << m1) + ((size_t)1 << m2));
}

template <class F>
zc_status eq_expand(const uint32_t* z, int m, uint32_t* out, uint32_t* ws, cudaStream_t st) {
  if (m <= kEqSmall) {
    k_eq_small<F><<<1, 1024, 0, st>>>(z, m, out);
    return launch_check();
  }
  const int m1 = m / 2, m2 = m - m1;
  uint32_t* th = ws;
  uint32_t* tl = ws + ((size_t)4 << m1);
  k_eq_small<F><<<1, 1024, 0, st>>>(z, m1, th);
  ZC_TRY(launch_check());
  k_eq_small<F><<<1, 1024, 0, st>>>(z + 4 * m1, m2, tl);
  ZC_TRY(launch_check());
  const int64_t total = (int64_t)1 << m;
  k_eq_outer<F><<<grid_for(total, 256), 256, 0, st>>>(th, tl, m2, total, out);
  return launch_check();
}

// eval_mle of base columns with eq = hi (x) lo: partial[c][h] =
// sum_l lo[l] cols[c][h 2^m2 + l], one block per (h, c).
template <class F>
__global__ void __launch_bounds__(256) k_eval_inner(const uint32_t* cols, int64_t S, int m2,
                                                    const uint32_t* lo, uint32_t* partial,
                                                    int64_t H) {
  const int64_t h = blockIdx.x, c = blockIdx.y;
  const int64_t L = (int64_t)1 << m2;
  const uint32_t* col = cols + c * S + h * L;
  ef4 acc{{0, 0, 0, 0}};
  for (int64_t l = threadIdx.x; l < L; l += blockDim.x)
    acc = ef_add<F>(acc, ef_base<F>(ld4(lo + 4 * l), __ldg(col + l)));
  acc = block_sum<F>(acc);
  if (threadIdx.x == 0) st4(partial + 4 * (c * H + h), acc);
}

// out[c] = sum_h hi[h] partial[c][h], one block per column.
template <class F>
__global__ void __launch_bounds__(256) k_eval_outer(const uint32_t* partial, const uint32_t* hi,
                                                    int64_t H, uint32_t* out) {
  const int64_t c = blockIdx.x;
  ef4 acc{{0, 0, 0, 0}};
  for (int64_t h = threadIdx.x; h < H; h += blockDim.x)
    acc = ef_add<F>(acc, ef_mul<F>(ld4(hi + 4 * h), ld4(partial + 4 * (c * H + h))));
  acc = block_sum<F>(acc);
  if (threadIdx.x == 0) st4(out + 4 * c, acc);
}

// eval_mle workspace: half tables + partial sums.
inline void eval_split(int m, int* m1, int* m2) {
  *m2 = m < kEqSmall ? m : kEqSmall;
  *m1 = m - *m2;
}
inline size_t eval_ws_bytes(int w, int m) {
  int m1, m2;
  eval_split(m, &m1, &m2);
  const size_t H = (size_t)1 << m1;
  return (size_t)16 * (H + ((size_t)1 << m2) + (size_t)w * H) + eq_ws_bytes(m1);
}

template <class F>
zc_status eval_mle(const uint32_t* cols, int w, int m, const uint32_t* z, uint32_t* out,
                   uint32_t* ws, cudaStream_t st) {
  int m1, m2;
  eval_split(m, &m1, &m2);
  const int64_t H = (int64_t)1 << m1, S = (int64_t)1 << m;
  uint32_t* hi = ws;
  uint32_t* lo = hi + 4 * H;
  uint32_t* partial = lo + ((size_t)4 << m2);
  uint32_t* eqws = partial + 4 * (size_t)w * H;
  ZC_TRY(eq_expand<F>(z, m1, hi, eqws, st));           // z[0 .. m1): high index bits
  ZC_TRY(eq_expand<F>(z + 4 * m1, m2, lo, eqws, st));  // z[m1 .. m): low index bits
  k_eval_inner<F><<<dim3((unsigned)H, (unsigned)w), 256, 0, st>>>(cols, S, m2, lo, partial, H);
  ZC_TRY(launch_check());
  k_eval_outer<F><<<(unsigned)w, 256, 0, st>>>(partial, hi, H, out);
  return launch_check();
}

// ---------------------------------------------------------------- rounds --
// s0 partials: sum_j eq[j] mle[2j] over M pairs (mle has 2M EF4 entries).
template <class F>
__global__ void __launch_bounds__(256) k_sc_reduce(const uint32_t* mle, const uint32_t* eq,
                                                   int64_t M, uint32_t* partial) {
  ef4 acc{{0, 0, 0, 0}};
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < M;
       j += (int64_t)gridDim.x * blockDim.x)
    acc = ef_add<F>(acc, ef_mul<F>(ld4(eq + 4 * j), ld4(mle + 8 * j)));
  acc = block_sum<F>(acc);
  if (threadIdx.x == 0) st4(partial + 4 * blockIdx.x, acc);
}

// msg = (s0, s1): s0 = sum of partials, s1 = (claim - s0) / z_last + s0
// (zorch/pcs/basefold/kernel.py:52-66).
template <class F>
__global__ void __launch_bounds__(256) k_sc_message(const uint32_t* partial, int np,
                                                    const uint32_t* claim, const uint32_t* zinv,
                                                    uint32_t* msg) {
  ef4 acc{{0, 0, 0, 0}};
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc = ef_add<F>(acc, ld4(partial + 4 * i));
  acc = block_sum<F>(acc);
  if (threadIdx.x == 0) {
    const ef4 s1 = ef_add<F>(ef_mul<F>(ef_sub<F>(ld4(claim), acc), ld4(zinv)), acc);
    st4(msg, acc);
    st4(msg + 4, s1);
  }
}

// The round's fold (zorch/pcs/basefold/kernel.py:68-74, mle_fold
// zorch/poly/multilinear.py:101-109, contract_hypercube_step zorch/poly/eq.py:65-77):
// mle_out[j] = mle[2j] + beta mle[2j+1] (j < M), eq_out[k] = eq[2k] + eq[2k+1]
// (k < M/2, when eq_out), claim = s0 + beta s1 (block 0).
template <class F>
__global__ void k_sc_fold(const uint32_t* mle, int64_t M, const uint32_t* beta, int beta_limbs,
                          const uint32_t* msg, uint32_t* mle_out, const uint32_t* eq,
                          uint32_t* eq_out, uint32_t* claim) {
  ef4 b{{__ldg(beta), 0, 0, 0}};
  if (beta_limbs == 4) b = ld4(beta);
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < M;
       j += (int64_t)gridDim.x * blockDim.x) {
    const ef4 e0 = ld4(mle + 8 * j), e1 = ld4(mle + 8 * j + 4);
    st4(mle_out + 4 * j, ef_add<F>(e0, beta_limbs == 4 ? ef_mul<F>(b, e1) : ef_base<F>(e1, b.c[0])));
    if (eq_out && j < M / 2)
      st4(eq_out + 4 * j, ef_add<F>(ld4(eq + 8 * j), ld4(eq + 8 * j + 4)));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const ef4 s0 = ld4(msg), s1 = ld4(msg + 4);
    st4(claim, ef_add<F>(s0, beta_limbs == 4 ? ef_mul<F>(b, s1) : ef_base<F>(s1, b.c[0])));
  }
}

// Staggered batching with an offset into the weight table and accumulation
// (batch_staggered, zorch/pcs/basefold/batching.py:66-80).
template <class F>
__global__ void k_rlc_ex(const uint32_t* cw, int64_t n, int w, const uint32_t* chal, int nbv,
                         int offset, int accumulate, uint32_t* out) {
  extern __shared__ uint32_t wt[];  // 2^nbv x 4
  if (threadIdx.x == 0) {
    wt[0] = F::ONE;
    wt[1] = wt[2] = wt[3] = 0;
    for (int j = 0; j < nbv; j++) {
      const ef4 r{{chal[4 * j], chal[4 * j + 1], chal[4 * j + 2], chal[4 * j + 3]}};
      for (int i = (1 << j) - 1; i >= 0; i--) {
        const ef4 s{{wt[4 * i], wt[4 * i + 1], wt[4 * i + 2], wt[4 * i + 3]}};
        const ef4 hi = ef_mul<F>(s, r);
        const ef4 lo = ef_sub<F>(s, hi);
        for (int e = 0; e < 4; e++) {
          wt[4 * (2 * i) + e] = lo.c[e];
          wt[4 * (2 * i + 1) + e] = hi.c[e];
        }
      }
    }
  }
  __syncthreads();
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    ef4 r{{0, 0, 0, 0}};
    if (accumulate) r = ld4(out + 4 * j);
    for (int c = 0; c < w; c++) {
      const uint32_t x = __ldg(cw + (int64_t)c * n + j);
      const uint32_t* wc = wt + 4 * (offset + c);
#pragma unroll
      for (int e = 0; e < 4; e++) r.c[e] = madd<F>(r.c[e], mmul<F>(wc[e], x));
    }
    st4(out + 4 * j, r);
  }
}

// out = sum_c weights[offset + c] values[c] (EF4 x EF4), accumulated; one
// thread (the claim of the batch, a handful of columns).
template <class F>
__global__ void k_rlc_values(const uint32_t* values, int w, const uint32_t* chal, int nbv,
                             int offset, int accumulate, uint32_t* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  ef4 acc{{0, 0, 0, 0}};
  if (accumulate) acc = ld4(out);
  for (int c = 0; c < w; c++) {
    // weight offset+c = prod_j (bit j of (offset+c) from the top ? r_j : 1 - r_j)
    ef4 wgt{{F::ONE, 0, 0, 0}};
    const int idx = offset + c;
    for (int j = 0; j < nbv; j++) {
      const ef4 r = ld4(chal + 4 * j);
      const bool bit = (idx >> (nbv - 1 - j)) & 1;
      wgt = bit ? ef_mul<F>(wgt, r) : ef_sub<F>(wgt, ef_mul<F>(wgt, r));
    }
    acc = ef_add<F>(acc, ef_mul<F>(wgt, ld4(values + 4 * c)));
  }
  st4(out, acc);
}

constexpr int kReduceBlocks = 256;

template <class F>
__global__ void k_ef4_inv(const uint32_t* in, uint32_t* out, int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    st4(out + 4 * i, ef_inv<F>(ld4(in + 4 * i)));
}

}  // namespace zc

using namespace zc;

extern "C" {

size_t zc_eq_expand_workspace_bytes(int32_t m) { return m < 0 ? 0 : eq_ws_bytes(m); }

zc_status zc_eq_expand(zc_field field, const uint32_t* z, int32_t m, uint32_t* out, void* ws,
                       size_t ws_bytes, void* stream) {
  if (m < 0 || !out || (m > 0 && !z)) return ZC_BAD_ARG;
  if (m > 2 * kEqSmall) return ZC_BAD_SHAPE;
  if ((uintptr_t)out % 16 || (uintptr_t)ws % 16) return ZC_BAD_ARG;
  if (ws_bytes < eq_ws_bytes(m) || (eq_ws_bytes(m) && !ws)) return ZC_OOM;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    return eq_expand<F>(z, m, out, (uint32_t*)ws, (cudaStream_t)stream);
  });
}

size_t zc_eval_mle_workspace_bytes(int32_t w, int32_t m) {
  return (w <= 0 || m < 0) ? 0 : eval_ws_bytes(w, m);
}

zc_status zc_eval_mle(zc_field field, const uint32_t* cols, int32_t w, int32_t m,
                      const uint32_t* z, uint32_t* out, void* ws, size_t ws_bytes, void* stream) {
  if (w <= 0 || m < 0 || m > 30 || !cols || !out || (m > 0 && !z)) return ZC_BAD_ARG;
  if ((uintptr_t)out % 16 || (uintptr_t)ws % 16) return ZC_BAD_ARG;
  if (!ws || ws_bytes < eval_ws_bytes(w, m)) return ZC_OOM;
  int m1, m2;
  eval_split(m, &m1, &m2);
  if (((int64_t)1 << m1) > 65535 || w > 65535) return ZC_BAD_SHAPE;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    return eval_mle<F>(cols, w, m, z, out, (uint32_t*)ws, (cudaStream_t)stream);
  });
}

zc_status zc_rlc_columns_ex(zc_field field, const uint32_t* cw, int64_t n, int32_t w,
                            const uint32_t* challenges, int32_t nbv, int32_t offset,
                            int32_t accumulate, uint32_t* out, void* stream) {
  if (!cw || !out || n < 0 || w < 1 || nbv < 0 || nbv > 12 || offset < 0 ||
      offset + w > (1 << nbv) || (nbv > 0 && !challenges))
    return ZC_BAD_ARG;
  if ((uintptr_t)out % 16) return ZC_BAD_ARG;
  if (n == 0) return ZC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    k_rlc_ex<F><<<grid_for(n, 256), 256, ((size_t)16) << nbv, st>>>(cw, n, w, challenges, nbv,
                                                                    offset, accumulate, out);
    return launch_check();
  });
}

zc_status zc_rlc_values(zc_field field, const uint32_t* values, int32_t w,
                        const uint32_t* challenges, int32_t nbv, int32_t offset,
                        int32_t accumulate, uint32_t* out, void* stream) {
  if (!values || !out || w < 1 || nbv < 0 || nbv > 30 || offset < 0 ||
      (nbv < 30 && offset + w > (1 << nbv)) || (nbv > 0 && !challenges))
    return ZC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    k_rlc_values<F><<<1, 32, 0, st>>>(values, w, challenges, nbv, offset, accumulate, out);
    return launch_check();
  });
}

zc_status zc_ef4_inv(zc_field field, const uint32_t* in, uint32_t* out, int64_t count,
                     void* stream) {
  if (count < 0 || (count > 0 && (!in || !out))) return ZC_BAD_ARG;
  if ((uintptr_t)in % 16 || (uintptr_t)out % 16) {
    set_error("EF4 operands must be 16-byte aligned");
    return ZC_BAD_ARG;
  }
  if (count == 0) return ZC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    const int64_t blocks = std::min<int64_t>((count + 127) / 128, 152 * 4);
    k_ef4_inv<F><<<(unsigned)blocks, 128, 0, st>>>(in, out, count);
    return launch_check();
  });
}

size_t zc_sumcheck_workspace_bytes(void) { return (size_t)16 * kReduceBlocks; }

zc_status zc_sumcheck_message(zc_field field, const uint32_t* mle, int64_t M, const uint32_t* eq,
                              const uint32_t* claim, const uint32_t* zinv, uint32_t* msg,
                              void* ws, size_t ws_bytes, void* stream) {
  if (!mle || !eq || !claim || !zinv || !msg || M < 1) return ZC_BAD_ARG;
  if (!ws || ws_bytes < (size_t)16 * kReduceBlocks || (uintptr_t)ws % 16) return ZC_OOM;
  if ((uintptr_t)mle % 16 || (uintptr_t)eq % 16 || (uintptr_t)claim % 16 ||
      (uintptr_t)zinv % 16 || (uintptr_t)msg % 16)
    return ZC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) -> zc_status {
    using F = decltype(f);
    const int blocks = (int)((M + 255) / 256 < kReduceBlocks ? (M + 255) / 256 : kReduceBlocks);
    k_sc_reduce<F><<<blocks, 256, 0, st>>>(mle, eq, M, (uint32_t*)ws);
    ZC_TRY(launch_check());
    k_sc_message<F><<<1, 256, 0, st>>>((const uint32_t*)ws, blocks, claim, zinv, msg);
    return launch_check();
  });
}

zc_status zc_sumcheck_fold(zc_field field, const uint32_t* mle, int64_t M, const uint32_t* beta,
                           int32_t beta_limbs, const uint32_t* msg, uint32_t* mle_out,
                           const uint32_t* eq, uint32_t* eq_out, uint32_t* claim, void* stream) {
  if (!mle || !beta || !msg || !mle_out || !claim || M < 1 || (beta_limbs != 1 && beta_limbs != 4))
    return ZC_BAD_ARG;
  if (eq_out && (!eq || M < 2)) return ZC_BAD_ARG;
  if ((uintptr_t)mle % 16 || (uintptr_t)mle_out % 16 || (uintptr_t)claim % 16 ||
      (uintptr_t)msg % 16 || (eq && (uintptr_t)eq % 16) || (eq_out && (uintptr_t)eq_out % 16))
    return ZC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    k_sc_fold<F><<<grid_for(M, 256), 256, 0, st>>>(mle, M, beta, beta_limbs, msg, mle_out, eq,
                                                   eq_out, claim);
    return launch_check();
  });
}

}  // extern "C"
