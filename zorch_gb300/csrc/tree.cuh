// The Merkle tree machinery shared by the commit and the fused fold-and-commit
// translation units: leaf layouts, the per-level and fused-subtree kernels,
// the tree driver, and the transcript hop run by a tree's root launch.
//
// Large trees: one thread per leaf (k_leaf, no barriers, full occupancy) writes
// the leaf digests; each level wider than kLevelWiseMin nodes is one launch of
// one thread per parent. The small top of a tree, and whole small trees, run
// as fused CTA subtrees (k_subtree): the first level by one thread per leaf
// (or a half-warp per parent), every level above by half-warps out of shared
// memory, writing every level (the tree keeps all layers for openings,
// zorch/commit/merkle.py:187-202) without reading a level back.
#pragma once
#include <string.h>

#include <type_traits>

#include "duplex.cuh"
#include "internal.cuh"

namespace zc {

constexpr int kMaxT = 256;

// A transcript hop run by the CTA that computes a tree's root, in the same
// launch: observe the 8 root words, squeeze n words -- the observe(root) +
// sample(beta) a pre-fold round makes right after committing its layer
// (zorch/pcs/fold.py:106-113). state: the 34-word packed duplex state, read
// and advanced in place; nullptr: no hop.
struct RootHop {
  uint32_t* state;
  uint32_t* chal;
  int n;
};

// One full warp (all 32 lanes: half-warp permutations shuffle across it).
// Not inlined: compiled once per field, not into every subtree variant.
template <class F>
__device__ __noinline__ void root_hop(const RootHop hop, const uint32_t* root, const P2Params* hp) {
  const HalfPerm<F> perm{hp};
  Duplex t;
  memcpy(&t, hop.state, sizeof(Duplex));
  duplex_observe(t, root, 8, perm);
  for (int i = 0; i < hop.n; i++) {
    uint32_t w;
    duplex_sample(t, 1, &w, perm);
    if (threadIdx.x == 0) hop.chal[i] = w;
  }
  __syncwarp();
  if (threadIdx.x == 0) memcpy(hop.state, &t, sizeof(Duplex));
}

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
// threads: 8 per node up to 1024 (64 half-warps), at least a warp. 128
// measured fastest on the GB300 (config 3's FRI commit phase: 6.21 ms graphed
// at 128 against 6.37-6.72 ms at 256 with the level-wise threshold at
// 2^14..2^16; the trace hash within 1 %).
#ifndef ZC_SUBTREE_T
#define ZC_SUBTREE_T 128
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
                                                       int l0, int T, const P2Params* rt,
                                                       RootHop hop) {
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
  if (hop.state) {  // passed only to a one-CTA launch that ends at the root
    __syncthreads();
    if (threadIdx.x < 32) {
      uint32_t root[8];
#pragma unroll
      for (int i = 0; i < 8; i++) root[i] = sm[cur][i * kSubMaxT];
      root_hop<F>(hop, root, hp);
    }
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
// launch. 2^13 measured fastest (see ZC_SUBTREE_T).
#ifndef ZC_LEVELWISE_MIN_LOG
#define ZC_LEVELWISE_MIN_LOG 13
#endif
constexpr int64_t kLevelWiseMin = (int64_t)1 << ZC_LEVELWISE_MIN_LOG;

// Launches the levels above `l_done` (all levels <= l_done already stored).
template <class K>
zc_status finish_tree(uint32_t* layers, int64_t L, int l_done, const P2Params* rt,
                      cudaStream_t st, RootHop hop = RootHop{nullptr, nullptr, 0}) {
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
    const bool top = parents == T;  // this launch's single CTA makes the root
    k_subtree<K, NodeLeaf><<<(unsigned)(parents / T), subtree_threads(T), 0, st>>>(
        nl, layers, L, l + 1, T, rt, top ? hop : RootHop{nullptr, nullptr, 0});
    ZC_TRY(launch_check());
    l += 1 + ilog2(T);
  }
  return ZC_OK;
}

template <class K, class Leaf>
zc_status commit_tree(const Leaf& leaf, uint32_t* layers, int64_t L, const P2Params* rt,
                      cudaStream_t st, RootHop hop = RootHop{nullptr, nullptr, 0}) {
  if (L > kLevelWiseMin) {
    k_leaf<K, Leaf><<<(unsigned)((L + kMaxT - 1) / kMaxT), kMaxT, 0, st>>>(leaf, layers, L, rt);
    ZC_TRY(launch_check());
    return finish_tree<K>(layers, L, 0, rt, st, hop);
  }
  const int T0 = L < kSubMaxT ? (int)L : kSubMaxT;
  const bool top = L == T0;
  k_subtree<K, Leaf><<<(unsigned)(L / T0), subtree_threads(T0), 0, st>>>(
      leaf, layers, L, 0, T0, rt, top ? hop : RootHop{nullptr, nullptr, 0});
  ZC_TRY(launch_check());
  return finish_tree<K>(layers, L, ilog2(T0), rt, st, hop);
}

constexpr int kMaxHopChallenges = 64;

inline zc_status check_hop(const uint32_t* state, int32_t n_chal, const uint32_t* chal) {
  if (!state || n_chal < 0 || n_chal > kMaxHopChallenges || (n_chal > 0 && !chal)) {
    set_error("a root hop needs the 34-word state and 0..64 challenge words");
    return ZC_BAD_ARG;
  }
  return ZC_OK;
}

}  // namespace zc
