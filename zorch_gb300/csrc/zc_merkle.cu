// Merkle commit, openings, and the FRI fold -- plain, and fused with the
// hashing of the next layer.
//
// Large trees: one thread per leaf (k_leaf, no barriers, full occupancy) writes
// the leaf digests; each level with more than 2^15 nodes is one launch of one
// thread per parent. The small top of a tree, and whole small trees, run as
// fused CTA subtrees (k_subtree): T = blockDim.x threads hash T leaves (or
// compress T child pairs), keep the digests in shared memory and compress up to
// the subtree root, writing every level (the tree keeps all layers for
// openings, zorch/commit/merkle.py:187-202) without reading a level back.
#include <string.h>

#include <type_traits>

#include "internal.cuh"

namespace zc {

constexpr int kMaxT = 256;

// Leaf p = concat over q < G of base[q*gs + p*g .. +g] (zc_leaves).
struct LayoutLeaf {
  const uint32_t* base;
  int G, g;
  int64_t gs;
  template <class K>
  __device__ __forceinline__ void digest(int64_t p, uint32_t* d, const K& k) const {
    // PaddingFreeSponge<16, 8, 8> (overwrite mode, no padding)
    uint32_t s[16];
#pragma unroll
    for (int j = 0; j < 16; j++) s[j] = 0;
    const int w = G * g;
    const uint32_t* src = base + p * (int64_t)g;
    int q = 0, r = 0;
    for (int e = 0; e < w; e += 8) {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        if (e + j < w) {
          s[j] = __ldg(src + (int64_t)q * gs + r);
          if (++r == g) {
            r = 0;
            q++;
          }
        }
      }
      p2_permute(s, k);
    }
#pragma unroll
    for (int j = 0; j < 8; j++) d[j] = s[j];
  }
};

// Node p of level l0 from children 2p, 2p+1 of the stored level l0-1.
struct NodeLeaf {
  const uint32_t* in;
  template <class K>
  __device__ __forceinline__ void digest(int64_t p, uint32_t* d, const K& k) const {
    uint32_t a[8], b[8];
    load_digest(in + 16 * p, a);
    load_digest(in + 16 * p + 8, b);
    p2_compress(a, b, d, k);
  }
};

// Query-layer node y of a query-strided tree (StridedMerkleTree,
// zorch/commit/strided_merkle.py:100-152): the binary tree, adjacent pairs in
// coset order, over the sponge-hashed rows y, y + s, ..., y + (rpq-1) s -- what
// the reference's strided levels compute for residue y. One thread folds the
// coset with a binary-counter stack (row r merges while bit b of r is set).
constexpr int kMaxStridedLog = 8;
struct StridedLeaf {
  LayoutLeaf rows;
  int64_t s;
  int log_rpq;
  template <class K>
  __device__ __forceinline__ void digest(int64_t p, uint32_t* d, const K& k) const {
    uint32_t stack[kMaxStridedLog][8];
    const int rpq = 1 << log_rpq;
    uint32_t cur[8];
    for (int r = 0; r < rpq; r++) {
      rows.digest(p + (int64_t)r * s, cur, k);
      int b = 0;
      for (; (r >> b) & 1; b++) {
        uint32_t out[8];
        p2_compress(stack[b], cur, out, k);
#pragma unroll
        for (int i = 0; i < 8; i++) cur[i] = out[i];
      }
      if (b < kMaxStridedLog)
#pragma unroll
        for (int i = 0; i < 8; i++) stack[b][i] = cur[i];
    }
#pragma unroll
    for (int i = 0; i < 8; i++) d[i] = cur[i];
  }
};

// fri_fold_values on one element j of a natural-order layer of n elements:
// g = (f[j] + f[j+n/2])/2 + beta * (f[j] - f[j+n/2]) * xinv, xinv = 1/(2 x_j)
// (zorch/coding/reed_solomon.py:543-548).
template <class F, int LI, int LB>
struct FoldMath {
  static constexpr int LO = (LI == 4 || LB == 4) ? 4 : 1;
  __device__ __forceinline__ static void fold(const uint32_t* f, int64_t half, int64_t j,
                                              uint32_t xinv, const uint32_t* beta,
                                              uint32_t* out) {
    uint32_t a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0};
#pragma unroll
    for (int e = 0; e < LI; e++) {
      a[e] = __ldg(f + j * LI + e);
      b[e] = __ldg(f + (j + half) * LI + e);
    }
    uint32_t sum[4], d[4];
#pragma unroll
    for (int e = 0; e < LI; e++) {
      sum[e] = mmul<F>(madd<F>(a[e], b[e]), F::INV2);
      d[e] = mmul<F>(msub<F>(a[e], b[e]), xinv);
    }
    if (LO == 1) {
      out[0] = madd<F>(sum[0], mmul<F>(beta[0], d[0]));
    } else if (LB == 1) {  // EF4 layer, base challenge
#pragma unroll
      for (int e = 0; e < 4; e++) out[e] = madd<F>(sum[e], mmul<F>(beta[0], d[e]));
    } else if (LI == 1) {  // base layer, EF4 challenge: beta * d is a scalar multiple
#pragma unroll
      for (int e = 0; e < 4; e++) {
        uint32_t t = mmul<F>(beta[e], d[0]);
        out[e] = e == 0 ? madd<F>(sum[0], t) : t;
      }
    } else {
      ef4 B{{beta[0], beta[1], beta[2], beta[3]}}, D{{d[0], d[1], d[2], d[3]}};
      ef4 r = ef_mul<F>(B, D);
#pragma unroll
      for (int e = 0; e < 4; e++) out[e] = madd<F>(sum[e], r.c[e]);
    }
  }
};

__device__ __forceinline__ int64_t brev64(int64_t i, int bits) {
  return bits ? (int64_t)(__brevll((unsigned long long)i) >> (64 - bits)) : 0;
}

// Leaf p of the next layer's pair tree, computed from the current layer f (n
// elements) and written to g on the way. Natural order (BR = false): the leaf
// is (g[p], g[p + n/4]), g[j] folded from (f[j], f[j + n/2]) at x_j = shift w^j.
// Bit-reversed order (BR = true, BitReversedReedSolomon.fold,
// zorch/coding/reed_solomon.py:484-492, 532-540): the leaf is (g[2p], g[2p+1]),
// g[i] folded from (f[2i], f[2i+1]) at x_i = shift w^brev(i) (i read over
// log2(n/2) bits); brev(2p+1) = brev(2p) + n/4, so x_{2p+1} = x_{2p} w^(n/4).
template <class F, int LI, int LB, bool BR = false>
struct FoldLeaf {
  using M = FoldMath<F, LI, LB>;
  static constexpr int LO = M::LO;
  const uint32_t* f;
  uint32_t* g;
  const uint32_t* beta;
  int64_t n;
  uint32_t inv2s;  // 1 / (2 shift)
  uint32_t winv;   // w_n^-1
  uint32_t w4inv;  // w_n^(-n/4)
  template <class K>
  __device__ __forceinline__ void digest(int64_t p, uint32_t* d, const K& k) const {
    const int64_t quarter = n >> 2, half = n >> 1;
    uint32_t bt[4];
#pragma unroll
    for (int e = 0; e < LB; e++) bt[e] = __ldg(beta + e);
    uint32_t o0[4], o1[4];
    int64_t i0, i1;
    if (BR) {
      const uint32_t x0 = mmul<F>(inv2s, mpow<F>(winv, (uint64_t)brev64(2 * p, ilog2_dev(half))));
      M::fold(f + 4 * p * LI, 1, 0, x0, bt, o0);
      M::fold(f + (4 * p + 2) * LI, 1, 0, mmul<F>(x0, w4inv), bt, o1);
      i0 = 2 * p;
      i1 = 2 * p + 1;
    } else {
      const uint32_t x0 = mmul<F>(inv2s, mpow<F>(winv, (uint64_t)p));
      M::fold(f, half, p, x0, bt, o0);
      M::fold(f, half, p + quarter, mmul<F>(x0, w4inv), bt, o1);
      i0 = p;
      i1 = p + quarter;
    }
    uint32_t s[16];
#pragma unroll
    for (int j = 0; j < 16; j++) s[j] = 0;
#pragma unroll
    for (int e = 0; e < LO; e++) {
      g[i0 * LO + e] = o0[e];
      g[i1 * LO + e] = o1[e];
      s[e] = o0[e];
      s[LO + e] = o1[e];
    }
    p2_permute(s, k);  // 2*LO <= 8 elements: one absorb block
#pragma unroll
    for (int j = 0; j < 8; j++) d[j] = s[j];
  }
};

// Nodes per tree-top CTA of the batched commit (k_tree_top) at its first
// level; its threads: 8 per node, so each level above is one round of
// half-warp permutations.
constexpr int kSubT = 128;
// Nodes per fused-subtree CTA (k_subtree) at its first level, and its
// threads: 8 per node up to 1024 (64 half-warps), at least a warp. With 256
// first-level nodes a launch fuses 9 levels.
#ifndef ZC_SUBTREE_T
#define ZC_SUBTREE_T 256
#endif
constexpr int kSubMaxT = ZC_SUBTREE_T;
static_assert(kSubMaxT >= 2 && kSubMaxT <= 256 && (kSubMaxT & (kSubMaxT - 1)) == 0,
              "subtree width must be a power of two in [2, 256]");
inline int subtree_threads(int T) {
  const int t = 8 * T > 32 ? 8 * T : 32;
  return t < 1024 ? t : 1024;
}

// Half-warp permutation of the caller's field (lane l passes state word l).
template <class F>
__device__ __forceinline__ uint32_t half_perm(uint32_t x, const P2Params* hp) {
  return p2_permute_half<F>(x, hp);
}

// One level of a subtree: parent i (< width) = compress(children 2i, 2i+1)
// read from the [word][node] slots `src` (row stride `stride`), written to the
// `dst` slots and to the tree's level at `lay`. Half-warp h takes nodes
// h, h + H, ... (H halves); a warp with no node in a round skips it (a
// warp-uniform branch: the shuffles need every lane of a running warp).
template <class F>
__device__ __forceinline__ void subtree_level(const uint32_t* src, uint32_t* dst, int stride,
                                              uint32_t* lay, int width, const P2Params* hp) {
  const int t = threadIdx.x, l = t & 15, H = blockDim.x >> 4;
  const int child_off = l >> 3, word = l & 7;
  for (int r = 0; r < width; r += H) {
    if (r + 2 * (t >> 5) >= width) continue;
    const int node = r + (t >> 4);
    const bool on = node < width;
    uint32_t x = on ? src[word * stride + 2 * node + child_off] : 0u;
    x = half_perm<F>(x, hp);
    if (on && l < 8) {
      lay[8 * node + l] = x;
      dst[l * stride + node] = x;
    }
  }
}

// One subtree of T first-level nodes per CTA (blockDim = subtree_threads(T)):
// the first level is T leaf digests (one thread each; for NodeLeaf, half-warps
// compressing stored children), then every level up to the subtree root is
// compressed by half-warps out of ping-pong shared-memory slots, each level
// written to `layers`.
template <class K, class Leaf>
__global__ void __launch_bounds__(1024) k_subtree(Leaf leaf, uint32_t* layers, int64_t L,
                                                       int l0, int T, const P2Params* rt) {
  using F = typename K::F;
  __shared__ P2Params s_rt;
  __shared__ uint32_t sm[2][8 * kSubMaxT];  // [word][node] digest slots
  K k = KIn<K>::make(rt, &s_rt);
  const P2Params* hp = KIn<K>::half(rt, &s_rt);
  const int t = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * T;
  uint32_t* lay0 = layers + 8 * (level_offset(L, l0) + base);
  if constexpr (std::is_same<Leaf, NodeLeaf>::value) {
    const int l = t & 15, H = blockDim.x >> 4;
    for (int r = 0; r < T; r += H) {
      if (r + 2 * (t >> 5) >= T) continue;
      const int node = r + (t >> 4);
      const bool on = node < T;
      uint32_t x = on ? leaf.in[16 * (base + node) + l] : 0u;
      x = half_perm<F>(x, hp);
      if (on && l < 8) {
        lay0[8 * node + l] = x;
        sm[0][l * kSubMaxT + node] = x;
      }
    }
  } else {
    if (t < T) {
      uint32_t d[8];
      leaf.digest(base + t, d, k);
      store_digest(lay0 + 8 * t, d);
#pragma unroll
      for (int i = 0; i < 8; i++) sm[0][i * kSubMaxT + t] = d[i];
    }
  }
  int cur = 0, lvl = l0, width = T;
  while (width > 1) {
    __syncthreads();
    width >>= 1;
    lvl++;
    subtree_level<F>(sm[cur], sm[cur ^ 1], kSubMaxT,
                     layers + 8 * (level_offset(L, lvl) + (int64_t)blockIdx.x * width), width, hp);
    cur ^= 1;
  }
}

// Resident 256-thread CTAs per SM k_leaf is compiled for: five for the
// built-in instance (its level and leaf forms then use 40-46 registers, where
// the unbounded build gave the level form 32; the 2^22 x 64 trace hash went
// 9.18 -> 9.00 ms); no bound for run-time parameter sets, whose constants come
// from shared memory and which would spill under it. The batched tree kernel
// keeps the compiler's choice: bounding it measured slower.
template <class K>
struct HashOcc {
  static constexpr int v = 1;
};
template <>
struct HashOcc<Bb16Builtin> {
  static constexpr int v = 5;
};

// One thread per leaf (or per parent for NodeLeaf): no shared memory, no
// barriers, so every warp stays busy for the whole launch.
template <class K, class Leaf>
__global__ void __launch_bounds__(kMaxT, HashOcc<K>::v) k_leaf(Leaf leaf, uint32_t* out, int64_t count,
                                                const P2Params* rt) {
  __shared__ P2Params s_rt;
  K k = KIn<K>::make(rt, &s_rt);
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= count) return;
  uint32_t d[8];
  leaf.digest(p, d, k);
  store_digest(out + 8 * p, d);
}

// Levels with more than this many nodes run one thread per node (k_leaf with
// NodeLeaf, throughput-bound: a level this wide fills the GPU); the narrower
// top of the tree is latency-bound and runs as fused CTA subtrees of
// half-warp permutations (k_subtree with NodeLeaf), log2(T)+1 levels per
// launch. A level of 2^16 nodes as single-thread permutations occupies a
// fifth of the GPU's threads and takes one permutation's latency (~9 us); as
// 256 subtree CTAs it takes nine half-warp rounds for nine levels.
#ifndef ZC_LEVELWISE_MIN_LOG
#define ZC_LEVELWISE_MIN_LOG 16
#endif
constexpr int64_t kLevelWiseMin = (int64_t)1 << ZC_LEVELWISE_MIN_LOG;

// Launches the levels above `l_done` (all levels <= l_done already stored).
template <class K>
zc_status finish_tree(uint32_t* layers, int64_t L, int l_done, const P2Params* rt,
                      cudaStream_t st) {
  const int depth = ilog2(L);
  int l = l_done;
  while (l < depth) {
    const int64_t parents = (L >> l) >> 1;
    NodeLeaf nl{layers + 8 * level_offset(L, l)};
    if (parents > kLevelWiseMin) {
      k_leaf<K, NodeLeaf><<<(unsigned)((parents + kMaxT - 1) / kMaxT), kMaxT, 0, st>>>(
          nl, layers + 8 * level_offset(L, l + 1), parents, rt);
      ZC_TRY(launch_check());
      l += 1;
      continue;
    }
    const int T = parents < kSubMaxT ? (int)parents : kSubMaxT;
    k_subtree<K, NodeLeaf><<<(unsigned)(parents / T), subtree_threads(T), 0, st>>>(
        nl, layers, L, l + 1, T, rt);
    ZC_TRY(launch_check());
    l += 1 + ilog2(T);
  }
  return ZC_OK;
}

template <class K, class Leaf>
zc_status commit_tree(const Leaf& leaf, uint32_t* layers, int64_t L, const P2Params* rt,
                      cudaStream_t st) {
  if (L > kLevelWiseMin) {
    k_leaf<K, Leaf><<<(unsigned)((L + kMaxT - 1) / kMaxT), kMaxT, 0, st>>>(leaf, layers, L, rt);
    ZC_TRY(launch_check());
    return finish_tree<K>(layers, L, 0, rt, st);
  }
  const int T0 = L < kSubMaxT ? (int)L : kSubMaxT;
  k_subtree<K, Leaf><<<(unsigned)(L / T0), subtree_threads(T0), 0, st>>>(leaf, layers, L, 0, T0,
                                                                         rt);
  ZC_TRY(launch_check());
  return finish_tree<K>(layers, L, ilog2(T0), rt, st);
}

// Rows and sibling paths of q leaves. reduce != 0: leaf = (idx >> shift) mod
// num_leaves (a power of two) -- the layer positions of
// zorch/coding/reed_solomon.py:320-329 (natural order, shift 0: a_i = q mod
// (n >> (i+1))) and :521-528 (bit-reversed order, shift i+1: a_i = q >> (i+1))
// computed here rather than by the caller.
__global__ void k_open(zc_leaves lv, const uint32_t* layers, const int32_t* idx, int q, int depth,
                       uint32_t* rows, uint32_t* paths, uint32_t* oob, int reduce, int shift) {
  const int qi = blockIdx.x;
  int64_t i = idx[qi];
  if (reduce)
    i = (int64_t)(((uint64_t)(uint32_t)idx[qi] >> shift) & (uint64_t)(lv.num_leaves - 1));
  if (i < 0 || i >= lv.num_leaves) {
    if (threadIdx.x == 0 && oob) atomicOr(oob, 1u);
    i = i < 0 ? 0 : lv.num_leaves - 1;
  }
  const int w = lv.groups * lv.group_len;
  for (int e = threadIdx.x; e < w; e += blockDim.x) {
    const int gq = e / lv.group_len, r = e - gq * lv.group_len;
    rows[(int64_t)qi * w + e] = lv.base[gq * lv.group_stride + i * lv.group_len + r];
  }
  const int64_t L = lv.num_leaves;
  for (int x = threadIdx.x; x < depth * 8; x += blockDim.x) {
    const int l = x >> 3, word = x & 7;
    const int64_t node = (i >> l) ^ 1;
    paths[((int64_t)l * q + qi) * 8 + word] = layers[8 * (level_offset(L, l) + node) + word];
  }
}

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
                             uint32_t* layers, const P2Params* rt, cudaStream_t st) {
  using F = typename K::F;
  FoldScalars<F> fs;
  ZC_TRY(fold_scalars<F>(n, shift_mont, generator, &fs));
  FoldLeaf<F, LI, LB, BR> leaf{cw, out, beta, n, fs.inv2s, fs.winv, fs.w4inv};
  return commit_tree<K>(leaf, layers, n >> 2, rt, st);
}

// compress([raw_root, sponge([log_height, width])]) on one warp (both halves
// compute the same permutations).
template <class K>
__global__ void __launch_bounds__(32) k_bind_root(const P2Params* rt, const uint32_t* raw_root,
                                                  uint32_t log_height, uint32_t width,
                                                  uint32_t* out) {
  using F = typename K::F;
  __shared__ P2Params s_rt;
  KIn<K>::make(rt, &s_rt);
  const P2Params* hp = KIn<K>::half(rt, &s_rt);
  const int lane = threadIdx.x & 31, l = lane & 15;
  // sponge: state = [log_height, width, 0 ...] (one absorb block), permute
  uint32_t x = l == 0 ? to_mont<F>(log_height) : (l == 1 ? to_mont<F>(width) : 0u);
  x = half_perm<F>(x, hp);
  // compress: state = raw_root || params (params = words 0..7 of the sponge)
  const uint32_t par = __shfl_sync(kFullMask, x, (lane & 16) | (l & 7));
  uint32_t y = l < 8 ? raw_root[l] : par;
  y = half_perm<F>(y, hp);
  __syncwarp();  // raw_root may alias out: every lane has read it
  if (lane < 8) out[lane] = y;
}

// ------------------------------------------------------------ batched ----
// Many trees (leaf layouts of different widths and heights) per launch: a leaf
// launch over (tree, 256-leaf chunk) items, one launch per level over
// (tree, 256-parent chunk) items for every tree that still has a wide level,
// and one top launch with one CTA per tree compressing its last <= 256 nodes
// to the root in shared memory. The tree table is a __grid_constant__ kernel
// parameter; CTAs claim items from an atomic counter (dynamic balance across
// cheap 1-element and expensive 128-element leaves).
constexpr int kMaxTreeJobs = 48;
constexpr int kTopLog = 8;

// One job is `count` trees of the same shape: tree t reads its leaves at
// base + t * bstride and writes its layers at layers + t * lstride (the columns
// of one request, each committed as its own polynomial).
struct TreeJobDev {
  const uint32_t* base;
  uint32_t* layers;
  int64_t L;
  int64_t gs;
  int64_t bstride, lstride;
  int64_t chunks;  // 256-node chunks per tree at the level being produced
  int32_t G, g;
  int32_t depth, top;
  int32_t count;
};

struct TreeBatch {
  int32_t njobs;
  int32_t level;  // level phase: the level being produced
  int64_t total;
  int64_t prefix[kMaxTreeJobs + 1];       // work items before job j
  int64_t tree_prefix[kMaxTreeJobs + 1];  // trees before job j (top launch)
  TreeJobDev job[kMaxTreeJobs];
};

__device__ __forceinline__ int find_tree(const int64_t* prefix, int njobs, int64_t it) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= it) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// LEVEL = 0: leaf chunks; LEVEL = 1: parent chunks of B.level.
template <class K, int LEVEL>
__global__ void __launch_bounds__(kMaxT) k_tree_batch(const __grid_constant__ TreeBatch B,
                                                      unsigned long long* counter,
                                                      const P2Params* rt) {
  __shared__ P2Params s_rt;
  __shared__ long long s_item;
  K k = KIn<K>::make(rt, &s_rt);
  for (;;) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    const int64_t it = s_item;
    __syncthreads();
    if (it >= B.total) break;
    const int j = find_tree(B.prefix, B.njobs, it);
    const TreeJobDev& J = B.job[j];
    const int64_t local = it - B.prefix[j];
    const int64_t tree = local / J.chunks;
    const int64_t p = (local - tree * J.chunks) * kMaxT + threadIdx.x;
    uint32_t* lay = J.layers + tree * J.lstride;
    uint32_t d[8];
    if (LEVEL == 0) {
      if (p < J.L) {
        LayoutLeaf leaf{J.base + tree * J.bstride, J.G, J.g, J.gs};
        leaf.digest(p, d, k);
        store_digest(lay + 8 * p, d);
      }
    } else {
      const int l = B.level;
      if (p < (J.L >> l)) {
        NodeLeaf nl{lay + 8 * level_offset(J.L, l - 1)};
        nl.digest(p, d, k);
        store_digest(lay + 8 * (level_offset(J.L, l) + p), d);
      }
    }
  }
}

// One CTA per tree: level `top` (<= 256 nodes, already stored) to the root,
// each level compressed by half-warps (64 halves: the first level of up to 128
// parents takes up to two rounds, every later level one).
template <class K>
__global__ void __launch_bounds__(8 * kSubT) k_tree_top(const __grid_constant__ TreeBatch B,
                                                       const P2Params* rt) {
  using F = typename K::F;
  constexpr int S = 2 * kSubT;  // slot stride: up to 256 nodes
  __shared__ P2Params s_rt;
  __shared__ uint32_t sm[2][8 * S];
  KIn<K>::make(rt, &s_rt);
  const P2Params* hp = KIn<K>::half(rt, &s_rt);
  const int j = find_tree(B.tree_prefix, B.njobs, (int64_t)blockIdx.x);
  const TreeJobDev& J = B.job[j];
  uint32_t* lay = J.layers + ((int64_t)blockIdx.x - B.tree_prefix[j]) * J.lstride;
  int lvl = J.top;
  int width = (int)(J.L >> lvl);
  const uint32_t* src = lay + 8 * level_offset(J.L, lvl);
  for (int i = threadIdx.x; i < width * 8; i += blockDim.x) sm[0][(i & 7) * S + (i >> 3)] = src[i];
  int cur = 0;
  while (width > 1) {
    __syncthreads();
    width >>= 1;
    lvl++;
    subtree_level<F>(sm[cur], sm[cur ^ 1], S, lay + 8 * level_offset(J.L, lvl), width, hp);
    cur ^= 1;
  }
}

template <class K>
zc_status tree_batch_wave(const zc_merkle_job* jobs, int n, unsigned long long* ctr,
                          const P2Params* rt, cudaStream_t st) {
  TreeBatch B;
  memset(&B, 0, sizeof(B));
  B.njobs = n;
  int max_top = 0;
  int64_t trees = 0;
  for (int i = 0; i < n; i++) {
    TreeJobDev& d = B.job[i];
    d.base = jobs[i].leaves.base;
    d.layers = jobs[i].layers;
    d.L = jobs[i].leaves.num_leaves;
    d.gs = jobs[i].leaves.group_stride;
    d.G = jobs[i].leaves.groups;
    d.g = jobs[i].leaves.group_len;
    d.count = jobs[i].count > 1 ? jobs[i].count : 1;
    d.bstride = jobs[i].leaf_stride;
    d.lstride = jobs[i].layer_stride;
    d.depth = ilog2(d.L);
    const int tl = jobs[i].top_log ? jobs[i].top_log : kTopLog;
    d.top = d.depth > tl ? d.depth - tl : 0;
    max_top = d.top > max_top ? d.top : max_top;
    B.tree_prefix[i] = trees;
    trees += d.count;
  }
  B.tree_prefix[n] = trees;
  ZC_CUDA(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long) * (max_top + 1), st));
  for (int l = 0; l <= max_top; l++) {
    int64_t tot = 0;
    for (int i = 0; i < n; i++) {
      TreeJobDev& d = B.job[i];
      B.prefix[i] = tot;
      d.chunks = ((d.L >> l) + kMaxT - 1) / kMaxT;
      if (l == 0 || l <= d.top) tot += d.chunks * d.count;
    }
    B.prefix[n] = tot;
    B.total = tot;
    B.level = l;
    if (tot == 0) continue;
    // one CTA per work item (each claims items from the counter until none
    // is left): CTAs retire as their items finish, so the block scheduler can
    // start blocks of a higher-priority stream between them -- a batch of
    // small served requests then does not wait for a large one to drain
    const int64_t grid = tot < 0x7fffffff ? tot : 0x7fffffff;
    if (l == 0)
      k_tree_batch<K, 0><<<(unsigned)grid, kMaxT, 0, st>>>(B, ctr + l, rt);
    else
      k_tree_batch<K, 1><<<(unsigned)grid, kMaxT, 0, st>>>(B, ctr + l, rt);
    ZC_TRY(launch_check());
  }
  if (trees > 0x7fffffff) return ZC_BAD_SHAPE;
  k_tree_top<K><<<(unsigned)trees, 8 * kSubT, 0, st>>>(B, rt);
  return launch_check();
}

// Staggered partial-Lagrange batching of one committed matrix's columns into
// one EF4 codeword (sample_rlc_coeffs_bits + batch_staggered,
// zorch/pcs/jagged/open.py:88-105, zorch/pcs/basefold/batching.py:66-80):
// weights = eq(., r) over nbv = ceil(log2 w) EF4 challenges, table built by
// the MSB-first interleaving step (zorch/poly/eq.py:55-62: high = s*r,
// low = s - high), column c weighted by entry c; out[j] = sum_c wt_c cw[c][j].
template <class F>
__global__ void k_rlc(const uint32_t* cw, int64_t n, int w, const uint32_t* chal, int nbv,
                      uint32_t* out) {
  extern __shared__ uint32_t wt[];  // 2^nbv x 4 (EF4)
  if (threadIdx.x == 0) {
    wt[0] = F::ONE;
    wt[1] = wt[2] = wt[3] = 0;
    for (int j = 0; j < nbv; j++) {
      const ef4 r{{chal[4 * j], chal[4 * j + 1], chal[4 * j + 2], chal[4 * j + 3]}};
      for (int i = (1 << j) - 1; i >= 0; i--) {  // in place, from the top
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
    uint32_t r[4] = {0, 0, 0, 0};
    for (int c = 0; c < w; c++) {
      const uint32_t x = __ldg(cw + (int64_t)c * n + j);
#pragma unroll
      for (int e = 0; e < 4; e++) r[e] = madd<F>(r[e], mmul<F>(wt[4 * c + e], x));
    }
    reinterpret_cast<uint4*>(out)[j] = make_uint4(r[0], r[1], r[2], r[3]);
  }
}

// Seeded synthetic field data: SplitMix64(seed, index) reduced mod p.
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void k_fill_u32(uint32_t* out, int64_t n, uint32_t value) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = value;
}

__global__ void k_fill_uniform(uint32_t* out, int64_t n, uint64_t seed, uint32_t p) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (uint32_t)(splitmix64(seed * 0x100000001B3ull + (uint64_t)i) % p);
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
                          uint32_t generator, uint32_t* out, uint32_t* layers, cudaStream_t st) {
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    if (ef_in && ef_beta)
      return fold_commit_launch<K, 4, 4, BR>(cw, n, beta, shift_mont, generator, out, layers, rt, st);
    if (ef_in)
      return fold_commit_launch<K, 4, 1, BR>(cw, n, beta, shift_mont, generator, out, layers, rt, st);
    if (ef_beta)
      return fold_commit_launch<K, 1, 4, BR>(cw, n, beta, shift_mont, generator, out, layers, rt, st);
    return fold_commit_launch<K, 1, 1, BR>(cw, n, beta, shift_mont, generator, out, layers, rt, st);
  });
}

}  // namespace zc

using namespace zc;

extern "C" {

zc_status zc_merkle_commit(const zc_poseidon2* p, zc_leaves lv, uint32_t* layers, void* stream) {
  if (!layers || (!lv.base && lv.groups * lv.group_len > 0) || lv.groups < 0 ||
      lv.group_len < 0)
    return ZC_BAD_ARG;
  if (!is_pow2(lv.num_leaves)) {
    set_error("leaf count must be a power of two");
    return ZC_NOT_POW2;
  }
  if ((uintptr_t)layers % 16) return ZC_BAD_ARG;
  if ((int64_t)lv.groups * lv.group_len > (1 << 20)) return ZC_BAD_SHAPE;
  cudaStream_t st = (cudaStream_t)stream;
  LayoutLeaf leaf{lv.base, lv.groups, lv.group_len, lv.group_stride};
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    return commit_tree<K>(leaf, layers, lv.num_leaves, rt, st);
  });
}

zc_status zc_strided_merkle_commit(const zc_poseidon2* p, zc_leaves lv, int32_t rows_per_query,
                                   uint32_t* layers, void* stream) {
  if (!layers || (!lv.base && lv.groups * lv.group_len > 0) || lv.groups < 0 ||
      lv.group_len < 0)
    return ZC_BAD_ARG;
  if (!is_pow2(lv.num_leaves) || !is_pow2(rows_per_query)) {
    set_error("height and rows_per_query must be powers of two");
    return ZC_NOT_POW2;
  }
  if (rows_per_query > lv.num_leaves || ilog2(rows_per_query) >= kMaxStridedLog) {
    set_error("rows_per_query exceeds the height or 2^7");
    return ZC_BAD_SHAPE;
  }
  if ((uintptr_t)layers % 16) return ZC_BAD_ARG;
  if ((int64_t)lv.groups * lv.group_len > (1 << 20)) return ZC_BAD_SHAPE;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t s = lv.num_leaves / rows_per_query;
  StridedLeaf leaf{LayoutLeaf{lv.base, lv.groups, lv.group_len, lv.group_stride}, s,
                   ilog2(rows_per_query)};
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    return commit_tree<K>(leaf, layers, s, rt, st);
  });
}

zc_status zc_merkle_open(zc_leaves lv, const uint32_t* layers, const int32_t* idx, int32_t q,
                         uint32_t* rows, uint32_t* paths, uint32_t* oob_flag, void* stream) {
  if (q < 0 || !layers || !idx || (q > 0 && (!rows || !paths))) return ZC_BAD_ARG;
  if (!is_pow2(lv.num_leaves)) return ZC_NOT_POW2;
  if (q == 0) return ZC_OK;
  const int depth = ilog2(lv.num_leaves);
  k_open<<<q, 128, 0, (cudaStream_t)stream>>>(lv, layers, idx, q, depth, rows, paths, oob_flag,
                                              0, 0);
  return launch_check();
}

zc_status zc_merkle_open_reduced(zc_leaves lv, const uint32_t* layers, const int32_t* idx,
                                 int32_t q, int32_t shift, uint32_t* rows, uint32_t* paths,
                                 void* stream) {
  if (q < 0 || !layers || !idx || (q > 0 && (!rows || !paths))) return ZC_BAD_ARG;
  if (shift < 0 || shift > 31) return ZC_BAD_ARG;
  if (!is_pow2(lv.num_leaves) || lv.num_leaves > (1ll << 32)) return ZC_NOT_POW2;
  if (q == 0) return ZC_OK;
  const int depth = ilog2(lv.num_leaves);
  k_open<<<q, 128, 0, (cudaStream_t)stream>>>(lv, layers, idx, q, depth, rows, paths, nullptr,
                                              1, shift);
  return launch_check();
}

zc_status zc_fri_fold(zc_field field, const uint32_t* cw, int64_t n, int ef_in,
                      const uint32_t* beta, int ef_beta, uint32_t shift_mont, uint32_t generator,
                      uint32_t* out, void* stream) {
  if (!cw || !beta || !out) return ZC_BAD_ARG;
  if (!is_pow2(n) || n < 2) {
    set_error("fri_fold requires a power-of-two codeword of length >= 2");
    return ZC_NOT_POW2;
  }
  return fri_fold_any<false>(field, cw, n, ef_in, beta, ef_beta, shift_mont, generator, out,
                             (cudaStream_t)stream);
}

zc_status zc_fri_fold_k(zc_field field, const uint32_t* cw, int64_t n, int ef_in,
                        const uint32_t* beta, int ef_beta, int log_k, uint32_t shift_mont,
                        uint32_t generator, uint32_t* out, void* stream) {
  if (!cw || !beta || !out || log_k < 1 || log_k > 4) return ZC_BAD_ARG;
  if (!is_pow2(n) || n < ((int64_t)1 << log_k)) {
    set_error("fold_group requires a power-of-two codeword of length >= fold_factor");
    return ZC_NOT_POW2;
  }
  if (generator != 0 && generator != (field == ZC_FIELD_BABYBEAR ? BabyBear::GEN : KoalaBear::GEN)) {
    set_error("only the field's canonical generator is built");
    return ZC_UNSUPPORTED;
  }
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    if (ilog2(n) > F::TWO_ADICITY) return ZC_BAD_SHAPE;
    if (ef_in && ef_beta) return fold_k_launch<F, 4, 4>(cw, n, beta, log_k, shift_mont, out, st);
    if (ef_in) return fold_k_launch<F, 4, 1>(cw, n, beta, log_k, shift_mont, out, st);
    if (ef_beta) return fold_k_launch<F, 1, 4>(cw, n, beta, log_k, shift_mont, out, st);
    return fold_k_launch<F, 1, 1>(cw, n, beta, log_k, shift_mont, out, st);
  });
}

zc_status zc_fri_fold_bitrev(zc_field field, const uint32_t* cw, int64_t n, int ef_in,
                             const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                             uint32_t generator, uint32_t* out, void* stream) {
  if (!cw || !beta || !out) return ZC_BAD_ARG;
  if (!is_pow2(n) || n < 2) {
    set_error("fri_fold requires a power-of-two codeword of length >= 2");
    return ZC_NOT_POW2;
  }
  return fri_fold_any<true>(field, cw, n, ef_in, beta, ef_beta, shift_mont, generator, out,
                            (cudaStream_t)stream);
}

zc_status zc_fri_fold_commit(const zc_poseidon2* p, const uint32_t* cw, int64_t n, int ef_in,
                             const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                             uint32_t generator, uint32_t* out, uint32_t* next_layers,
                             void* stream) {
  if (!cw || !beta || !out || !next_layers) return ZC_BAD_ARG;
  if (!is_pow2(n) || n < 4) {
    set_error("fri_fold_commit requires a power-of-two codeword of length >= 4");
    return ZC_NOT_POW2;
  }
  if ((uintptr_t)next_layers % 16) return ZC_BAD_ARG;
  return fold_commit_any<false>(p, cw, n, ef_in, beta, ef_beta, shift_mont, generator, out,
                                next_layers, (cudaStream_t)stream);
}

zc_status zc_fri_fold_commit_bitrev(const zc_poseidon2* p, const uint32_t* cw, int64_t n,
                                    int ef_in, const uint32_t* beta, int ef_beta,
                                    uint32_t shift_mont, uint32_t generator, uint32_t* out,
                                    uint32_t* next_layers, void* stream) {
  if (!cw || !beta || !out || !next_layers) return ZC_BAD_ARG;
  if (!is_pow2(n) || n < 4) {
    set_error("fri_fold_commit requires a power-of-two codeword of length >= 4");
    return ZC_NOT_POW2;
  }
  if ((uintptr_t)next_layers % 16) return ZC_BAD_ARG;
  return fold_commit_any<true>(p, cw, n, ef_in, beta, ef_beta, shift_mont, generator, out,
                               next_layers, (cudaStream_t)stream);
}

zc_status zc_smcs_bind_root(const zc_poseidon2* p, const uint32_t* raw_root, uint32_t log_height,
                            uint32_t width, uint32_t* out, void* stream) {
  if (!raw_root || !out || ((uintptr_t)out % 16)) return ZC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    k_bind_root<K><<<1, 32, 0, st>>>(rt, raw_root, log_height, width, out);
    return launch_check();
  });
}

zc_status zc_merkle_commit_batch(const zc_poseidon2* p, const zc_merkle_job* jobs,
                                 int32_t njobs, void* workspace, size_t workspace_bytes,
                                 void* stream) {
  if (njobs < 0 || (njobs > 0 && !jobs) || !workspace || workspace_bytes < 256) return ZC_BAD_ARG;
  if ((uintptr_t)workspace % 256) return ZC_BAD_ARG;
  for (int i = 0; i < njobs; i++) {
    const zc_merkle_job& j = jobs[i];
    if (!j.layers || (uintptr_t)j.layers % 16) return ZC_BAD_ARG;
    if (!is_pow2(j.leaves.num_leaves)) return ZC_NOT_POW2;
    if (j.leaves.groups < 0 || j.leaves.group_len < 0 ||
        (!j.leaves.base && j.leaves.groups * j.leaves.group_len > 0))
      return ZC_BAD_ARG;
    if (j.top_log < 0 || j.top_log > kTopLog) {
      set_error("top_log must be 0 (default) or 1..8");
      return ZC_BAD_ARG;
    }
    if (j.count < 0) return ZC_BAD_ARG;
    if (j.count > 1 && (j.layer_stride < 8 * (2 * j.leaves.num_leaves - 1) ||
                        j.layer_stride % 4 || j.leaf_stride < 0)) {
      set_error("a tree family needs layer_stride >= (2L-1)*8 words (a multiple of 4) "
                "and leaf_stride >= 0");
      return ZC_BAD_ARG;
    }
    if (ilog2(j.leaves.num_leaves) - (j.top_log ? j.top_log : kTopLog) + 1 > 30)
      return ZC_BAD_SHAPE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* ctr = (unsigned long long*)workspace;
  return with_perm(p, [&](auto k, const P2Params* rt) -> zc_status {
    using K = decltype(k);
    for (int i = 0; i < njobs; i += kMaxTreeJobs) {
      const int n = njobs - i < kMaxTreeJobs ? njobs - i : kMaxTreeJobs;
      ZC_TRY(tree_batch_wave<K>(jobs + i, n, ctr, rt, st));
    }
    return ZC_OK;
  });
}

zc_status zc_rlc_columns(zc_field field, const uint32_t* cw, int64_t n, int32_t w,
                         const uint32_t* challenges, uint32_t* out, void* stream) {
  if (!cw || !out || n < 0 || w < 1 || w > 4096) return ZC_BAD_ARG;
  const int nbv = ilog2(w);
  if (nbv > 0 && !challenges) return ZC_BAD_ARG;
  if ((uintptr_t)out % 16) return ZC_BAD_ARG;
  if (n == 0) return ZC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_rlc<F><<<(unsigned)blocks, 256, ((size_t)16) << nbv, st>>>(cw, n, w, challenges, nbv, out);
    return launch_check();
  });
}

zc_status zc_fill_u32(uint32_t* out, int64_t n, uint32_t value, void* stream) {
  if ((!out && n > 0) || n < 0) return ZC_BAD_ARG;
  if (n == 0) return ZC_OK;
  if (value == 0) {
    ZC_CUDA(cudaMemsetAsync(out, 0, (size_t)n * 4, (cudaStream_t)stream));
    return ZC_OK;
  }
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_fill_u32<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(out, n, value);
  return launch_check();
}

zc_status zc_fill_uniform(zc_field field, uint32_t* out, int64_t n, uint64_t seed, void* stream) {
  if (!out || n < 0) return ZC_BAD_ARG;
  if (n == 0) return ZC_OK;
  const uint32_t p = field == ZC_FIELD_BABYBEAR ? BabyBear::P : KoalaBear::P;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_fill_uniform<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(out, n, seed, p);
  return launch_check();
}

}  // extern "C"
