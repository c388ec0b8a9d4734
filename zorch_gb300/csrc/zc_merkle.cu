// Merkle commits (single, strided, batched over many trees), openings, the
// SP1 root binding, the partial-Lagrange column batching and device fills.
// The tree kernels themselves are in tree.cuh.
#include <string.h>

#include <type_traits>

#include "tree.cuh"

namespace zc {

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
  for (int done = 0; kItemsPerCta == 0 || done < kItemsPerCta; done++) {
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
// each level compressed in one round (subtree_level: quarter-warps for the
// levels wider than 32 parents, half-warps above).
template <class K>
__global__ void __launch_bounds__(4 * kSubT) k_tree_top(const __grid_constant__ TreeBatch B,
                                                       const P2Params* rt) {
  constexpr int S = 2 * kSubT;  // up to 256 nodes
  __shared__ P2Params s_rt;
  __shared__ __align__(16) uint32_t sm[2][8 * S];  // [node][word] digest slots
  KIn<K>::make(rt, &s_rt);
  const P2Params* hp = KIn<K>::half(rt, &s_rt);
  const int j = find_tree(B.tree_prefix, B.njobs, (int64_t)blockIdx.x);
  const TreeJobDev& J = B.job[j];
  uint32_t* lay = J.layers + ((int64_t)blockIdx.x - B.tree_prefix[j]) * J.lstride;
  int lvl = J.top;
  int width = (int)(J.L >> lvl);
  const uint4* src = reinterpret_cast<const uint4*>(lay + 8 * level_offset(J.L, lvl));
  for (int i = threadIdx.x; i < width * 2; i += blockDim.x) reinterpret_cast<uint4*>(sm[0])[i] = src[i];
  int cur = 0;
  while (width > 1) {
    __syncthreads();
    width >>= 1;
    lvl++;
    subtree_level<K>(sm[cur], sm[cur ^ 1], lay + 8 * level_offset(J.L, lvl), width, hp);
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
  int dev = 0, sms = 0, occ = 0;
  ZC_CUDA(cudaGetDevice(&dev));
  ZC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  ZC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_tree_batch<K, 0>, kMaxT, 0));
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
    const int64_t grid = batch_grid(tot, occ, sms);
    if (l == 0)
      k_tree_batch<K, 0><<<(unsigned)grid, kMaxT, 0, st>>>(B, ctr + l, rt);
    else
      k_tree_batch<K, 1><<<(unsigned)grid, kMaxT, 0, st>>>(B, ctr + l, rt);
    ZC_TRY(launch_check());
  }
  if (trees > 0x7fffffff) return ZC_BAD_SHAPE;
  k_tree_top<K><<<(unsigned)trees, 4 * kSubT, 0, st>>>(B, rt);
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

zc_status zc_merkle_commit_hop(const zc_poseidon2* p, zc_leaves lv, uint32_t* layers,
                               uint32_t* state, int32_t n_chal, uint32_t* chal, void* stream) {
  if (!layers || (!lv.base && lv.groups * lv.group_len > 0) || lv.groups < 0 ||
      lv.group_len < 0)
    return ZC_BAD_ARG;
  if (!is_pow2(lv.num_leaves)) {
    set_error("leaf count must be a power of two");
    return ZC_NOT_POW2;
  }
  if ((uintptr_t)layers % 16) return ZC_BAD_ARG;
  if ((int64_t)lv.groups * lv.group_len > (1 << 20)) return ZC_BAD_SHAPE;
  ZC_TRY(check_hop(state, n_chal, chal));
  cudaStream_t st = (cudaStream_t)stream;
  LayoutLeaf leaf{lv.base, lv.groups, lv.group_len, lv.group_stride};
  const RootHop hop{state, chal, n_chal};
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    return commit_tree<K>(leaf, layers, lv.num_leaves, rt, st, hop);
  });
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

zc_status zc_copy_rows(void* dst, int64_t dst_pitch, const void* src, int64_t src_pitch,
                       int64_t row_bytes, int64_t rows, void* stream) {
  if (rows < 0 || row_bytes < 0 || dst_pitch < row_bytes || src_pitch < row_bytes) {
    set_error("copy_rows: pitches must be >= the row size, sizes >= 0");
    return ZC_BAD_ARG;
  }
  if (rows == 0 || row_bytes == 0) return ZC_OK;
  if (!dst || !src) return ZC_BAD_ARG;
  ZC_CUDA(cudaMemcpy2DAsync(dst, (size_t)dst_pitch, src, (size_t)src_pitch, (size_t)row_bytes,
                            (size_t)rows, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return ZC_OK;
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
