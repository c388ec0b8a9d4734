// Shared host/device helpers: status codes, launch checks, level offsets.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/zc.h"

namespace zc {

#define ZC_TRY(expr)                       \
  do {                                     \
    zc_status _s = (expr);                 \
    if (_s != ZC_OK) return _s;            \
  } while (0)

#define ZC_CUDA(expr)                                  \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) return zc::cuda_fail(_e);   \
  } while (0)

zc_status cuda_fail(cudaError_t e);
zc_status launch_check();

inline bool is_pow2(int64_t x) { return x > 0 && (x & (x - 1)) == 0; }
inline int ilog2(int64_t x) {
  int l = 0;
  while (((int64_t)1 << l) < x) l++;
  return l;
}

// Work items a CTA of the batched (work-list) kernels takes before it retires
// (0: CTAs stay resident until the list is empty). Retiring CTAs let the block
// scheduler start blocks of a higher-priority stream in between, so a small
// served batch does not wait for a large one to drain.
#ifndef ZC_ITEMS_PER_CTA
#define ZC_ITEMS_PER_CTA 8
#endif
constexpr int kItemsPerCta = ZC_ITEMS_PER_CTA;

// Grid of a work-list launch over `total` items: every item is claimed (grid *
// items per CTA >= total), never more CTAs than items; resident CTAs only
// (occ per SM) when CTAs do not retire. A list shorter than kItemsPerCta
// resident waves gets one CTA per item up to a full wave, so that a small
// batch still spreads over every SM.
inline int64_t batch_grid(int64_t total, int occ, int sms) {
  const int64_t wave = (int64_t)(occ > 0 ? occ : 1) * sms;
  int64_t grid = kItemsPerCta > 0 ? (total + kItemsPerCta - 1) / kItemsPerCta : wave;
  if (kItemsPerCta > 0 && grid < wave) grid = total < wave ? total : wave;
  if (grid > total) grid = total;
  return grid < 0x7fffffff ? grid : 0x7fffffff;
}

// log2 of a power of two, on the device.
__device__ __forceinline__ int ilog2_dev(int64_t x) { return 63 - __clzll((long long)x); }

// Digest-layer layout of an arity-2 tree over L leaves: level l (leaf digests
// = level 0, root = level log2 L) starts at node offset 2L - (2L >> l).
__host__ __device__ __forceinline__ int64_t level_offset(int64_t L, int l) {
  return 2 * L - ((2 * L) >> l);
}

__device__ __forceinline__ void store_digest(uint32_t* dst, const uint32_t* d) {
  uint4* p = reinterpret_cast<uint4*>(dst);
  p[0] = make_uint4(d[0], d[1], d[2], d[3]);
  p[1] = make_uint4(d[4], d[5], d[6], d[7]);
}
__device__ __forceinline__ void load_digest(const uint32_t* src, uint32_t* d) {
  const uint4* p = reinterpret_cast<const uint4*>(src);
  uint4 a = p[0], b = p[1];
  d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w;
  d[4] = b.x; d[5] = b.y; d[6] = b.z; d[7] = b.w;
}

}  // namespace zc
