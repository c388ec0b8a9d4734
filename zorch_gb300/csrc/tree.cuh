// The Merkle tree machinery shared by the commit and the fused fold-and-commit
// translation units: leaf layouts, the per-level and fused-subtree kernels,
// the tree driver, and the transcript hop run by a tree's root launch.
//
// Large trees: one thread per leaf (k_leaf, no barriers, full occupancy) writes
// the leaf digests; each level wider than tree_shape().levelwise_min nodes is
// one launch of one thread per parent. The small top of a tree, and whole
// small trees, run as fused CTA subtrees (k_subtree): the first level by one
// thread per leaf (or a quarter-warp per parent), every level above by
// quarter- or half-warps out of shared memory, writing every level (the tree
// keeps all layers for openings, zorch/commit/merkle.py:187-202) without
// reading a level back.
#pragma once
#include <stdlib.h>
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
// level; its threads: 4 per node, so every level above is one round
// (subtree_level: quarter-warps while a level has more than 32 parents,
// half-warps above).
constexpr int kSubT = 128;
// Largest number of nodes per fused-subtree CTA (k_subtree) at its first
// level; its threads: 4 per node (a quarter-warp permutation per parent), at
// least a warp.
constexpr int kSubCap = 256;

// The tree driver's shape: levels with more than `levelwise_min` nodes run one
// thread per node; the top runs as fused subtrees of `subtree_t` first-level
// nodes per CTA. Defaults 2^14 and 128 (the 2^22 FRI commit phase, graphed:
// 6.01 ms against 6.08 at 2^13, 6.12 at 2^15, 6.18 with 256-node subtrees).
// The environment variables ZC_LEVELWISE_MIN_LOG (8..20) and ZC_SUBTREE_T (a
// power of two in 2..256) override them for tuning (read once; no byte of any
// result depends on them).
struct TreeShape {
  int64_t levelwise_min;
  int subtree_t;
};
inline const TreeShape& tree_shape() {
  static const TreeShape shape = [] {
    TreeShape t{(int64_t)1 << 14, 128};
    if (const char* e = getenv("ZC_LEVELWISE_MIN_LOG")) {
      const int v = atoi(e);
      if (v >= 8 && v <= 20) t.levelwise_min = (int64_t)1 << v;
    }
    if (const char* e = getenv("ZC_SUBTREE_T")) {
      const int v = atoi(e);
      if (v >= 2 && v <= kSubCap && (v & (v - 1)) == 0) t.subtree_t = v;
    }
    return t;
  }();
  return shape;
}

inline int subtree_threads(int T) {
  const int t = 4 * T > 32 ? 4 * T : 32;
  return t < 1024 ? t : 1024;
}

// Half-warp permutation of the caller's field (lane l passes state word l).
template <class F>
__device__ __forceinline__ uint32_t half_perm(uint32_t x, const P2Params* hp) {
  return p2_permute_half<F>(x, hp);
}
// The same for the provider K: the built-in instance runs unrolled
// (half_permute_bb16), its lane constants read from the staged copy.
template <class K>
__device__ __forceinline__ uint32_t half_perm_k(uint32_t x, const P2Params* hp) {
  if constexpr (std::is_same<K, Bb16Builtin>::value) {
    const int l = threadIdx.x & 15;
    uint32_t ei[4], et[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      ei[r] = hp->ext_init[r][l];
      et[r] = hp->ext_term[r][l];
    }
    return half_permute_bb16(x, ei, et, hp->diag[l]);
  } else {
    return p2_permute_half<typename K::F>(x, hp);
  }
}

// One level of a subtree: parent i (< width) = compress(children 2i, 2i+1)
// read from the digest slots `src` ([node][8 words], 16-byte aligned),
// written to the `dst` slots and to the tree's level at `lay`. A level with
// more parents than the CTA has half-warps runs on quarter-warps (one round of
// up to blockDim/4 parents; a quarter's permutation costs ~2.3x fewer thread
// instructions, which is what counts when every warp is busy); a narrower
// level runs on half-warps, whose permutation has the shorter dependency
// chain (each lane issues a quarter of the instructions), which is what
// counts when the level is a latency chain. Parents are taken round-robin by
// quarter (half) g = g, g + Q, ...; a warp with no parent in a round skips it
// (a warp-uniform branch: the shuffles need every lane of a running warp).
template <class K>
__device__ __forceinline__ void subtree_level(const uint32_t* src, uint32_t* dst, uint32_t* lay,
                                              int width, const P2Params* hp) {
  using F = typename K::F;
  const int t = threadIdx.x;
  if (width > (int)(blockDim.x >> 4)) {  // quarter-warps: lane q holds words 4q .. 4q+3
    const int q = t & 3, Q = blockDim.x >> 2;
    for (int r = 0; r < width; r += Q) {
      if (r + 8 * (t >> 5) >= width) continue;
      const int node = r + (t >> 2);
      const bool on = node < width;
      uint4 v = on ? reinterpret_cast<const uint4*>(src)[4 * node + q] : make_uint4(0, 0, 0, 0);
      uint32_t x[4] = {v.x, v.y, v.z, v.w};
      p2_permute_quarter<F>(x, hp);
      if (on && q < 2) {
        const uint4 o = make_uint4(x[0], x[1], x[2], x[3]);
        reinterpret_cast<uint4*>(lay)[2 * node + q] = o;
        reinterpret_cast<uint4*>(dst)[2 * node + q] = o;
      }
    }
    return;
  }
  // half-warps (one round: width <= blockDim/16): lane l holds word l
  const int l = t & 15, node = t >> 4;
  if (2 * (t >> 5) >= width) return;
  const bool on = node < width;
  uint32_t x = on ? src[16 * node + l] : 0u;
  x = half_perm_k<K>(x, hp);
  if (on && l < 8) {
    lay[8 * node + l] = x;
    dst[8 * node + l] = x;
  }
}

// One subtree of T first-level nodes per CTA (blockDim = subtree_threads(T)):
// the first level is T leaf digests (one thread each; for NodeLeaf, quarter-
// or half-warps compressing stored children), then every level up to the
// subtree root is compressed out of ping-pong shared-memory slots
// (subtree_level), each level written to `layers`.
template <class K, class Leaf>
__global__ void __launch_bounds__(1024) k_subtree(Leaf leaf, uint32_t* layers, int64_t L,
                                                       int l0, int T, const P2Params* rt,
                                                       RootHop hop) {
  using F = typename K::F;
  __shared__ P2Params s_rt;
  __shared__ __align__(16) uint32_t sm[2][8 * kSubCap];  // [node][word] digest slots
  K k = KIn<K>::make(rt, &s_rt);
  const P2Params* hp = KIn<K>::half(rt, &s_rt);
  const int t = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * T;
  uint32_t* lay0 = layers + 8 * (level_offset(L, l0) + base);
  if constexpr (std::is_same<Leaf, NodeLeaf>::value) {
    subtree_level<K>(leaf.in + 16 * base, sm[0], lay0, T, hp);
  } else {
    if (t < T) {
      uint32_t d[8];
      leaf.digest(base + t, d, k);
      store_digest(lay0 + 8 * t, d);
      store_digest(sm[0] + 8 * t, d);
    }
  }
  int cur = 0, lvl = l0, width = T;
  while (width > 1) {
    __syncthreads();
    width >>= 1;
    lvl++;
    subtree_level<K>(sm[cur], sm[cur ^ 1],
                     layers + 8 * (level_offset(L, lvl) + (int64_t)blockIdx.x * width), width, hp);
    cur ^= 1;
  }
  if (hop.state) {  // passed only to a one-CTA launch that ends at the root
    __syncthreads();
    if (threadIdx.x < 32) {
      uint32_t root[8];
#pragma unroll
      for (int i = 0; i < 8; i++) root[i] = sm[cur][i];
      root_hop<F>(hop, root, hp);
    }
  }
}

// Resident 256-thread CTAs per SM k_leaf is compiled for: five for the
// built-in instance (its level and leaf forms then use 40-46 registers, where
// the unbounded build gave the level form 32; the 2^22 x 64 trace hash went
// 9.18 -> 9.00 ms); no bound for run-time parameter sets, whose constants come
// from shared memory and which would spill under it. The batched tree kernel
// keeps the compiler's choice: bounding it to five or six resident CTAs
// measured slower on the served stream (1.136 / 1.153 against 1.163 G elem/s).
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

// Levels with more than tree_shape().levelwise_min nodes run one thread per
// node (k_leaf with NodeLeaf, throughput-bound: a level this wide fills the
// GPU); the narrower top of the tree is latency-bound and runs as fused CTA
// subtrees (k_subtree with NodeLeaf), log2(T)+1 levels per launch.
// Launches the levels above `l_done` (all levels <= l_done already stored).
template <class K>
zc_status finish_tree(uint32_t* layers, int64_t L, int l_done, const P2Params* rt,
                      cudaStream_t st, RootHop hop = RootHop{nullptr, nullptr, 0}) {
  const int depth = ilog2(L);
  const int sub_t = tree_shape().subtree_t;
  int l = l_done;
  while (l < depth) {
    const int64_t parents = (L >> l) >> 1;
    NodeLeaf nl{layers + 8 * level_offset(L, l)};
    if (parents > tree_shape().levelwise_min) {
      k_leaf<K, NodeLeaf><<<(unsigned)((parents + kMaxT - 1) / kMaxT), kMaxT, 0, st>>>(
          nl, layers + 8 * level_offset(L, l + 1), parents, rt);
      ZC_TRY(launch_check());
      l += 1;
      continue;
    }
    const int T = parents < sub_t ? (int)parents : sub_t;
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
  if (L > tree_shape().levelwise_min) {
    k_leaf<K, Leaf><<<(unsigned)((L + kMaxT - 1) / kMaxT), kMaxT, 0, st>>>(leaf, layers, L, rt);
    ZC_TRY(launch_check());
    return finish_tree<K>(layers, L, 0, rt, st, hop);
  }
  const int sub_t = tree_shape().subtree_t;
  const int T0 = L < sub_t ? (int)L : sub_t;
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
