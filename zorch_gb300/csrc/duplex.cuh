// The Fiat-Shamir duplex state machine (DuplexTranscript,
// zorch/transcript.py:239-481) shared by the transcript kernels and the
// tree-top kernels that run a round's transcript hop in the same launch.
#pragma once
#include "internal.cuh"

namespace zc {

// ------------------------------------------------------------ duplex ------
// The DuplexTranscript state machine (zorch/transcript.py:239-481) on one
// thread. Packed state: in_buf[8] out_buf[8] sponge[16] in_pos out_pos.
struct Duplex {
  uint32_t in_buf[8];
  uint32_t out_buf[8];
  uint32_t sponge[16];
  int32_t in_pos;
  int32_t out_pos;
};

// _observe_body (zorch/transcript.py:637-748): the stream in_buf[0:in_pos] ++
// values is absorbed a full rate block at a time (overwrite sponge[0:8],
// permute); the tail stays pending; a fresh output iff no tail remains.
// `perm(s)` permutes the 16-word sponge in place: one thread on the host, a
// half-warp on the device (HalfPerm).
#pragma nv_exec_check_disable
template <class Perm>
ZC_HD void duplex_observe(Duplex& t, const uint32_t* v, int64_t m, const Perm& perm) {
  if (m <= 0) return;
  int pos = t.in_pos & 7;  // a corrupt caller state cannot index past the buffer
  for (int64_t i = 0; i < m; i++) {
    t.in_buf[pos++] = v[i];
    if (pos == 8) {
      for (int j = 0; j < 8; j++) t.sponge[j] = t.in_buf[j];
      perm(t.sponge);
      pos = 0;
    }
  }
  for (int j = pos; j < 8; j++) t.in_buf[j] = 0;
  t.in_pos = pos;
  if (pos == 0) {
    for (int j = 0; j < 8; j++) t.out_buf[j] = t.sponge[j];
    t.out_pos = 8;
  } else {
    for (int j = 0; j < 8; j++) t.out_buf[j] = 0;
    t.out_pos = 0;
  }
}

// _sample_one (zorch/transcript.py:370-387) n times; _duplexing (:299-313)
// merges the pending prefix over sponge[0:in_pos] (:154-163) and permutes.
#pragma nv_exec_check_disable
template <class Perm>
ZC_HD void duplex_sample(Duplex& t, int n, uint32_t* out, const Perm& perm) {
  t.in_pos &= 7;
  if (t.out_pos < 0 || t.out_pos > 8) t.out_pos = 0;
  for (int i = 0; i < n; i++) {
    if (t.in_pos > 0 || t.out_pos == 0) {
      for (int j = 0; j < t.in_pos; j++) t.sponge[j] = t.in_buf[j];
      perm(t.sponge);
      for (int j = 0; j < 8; j++) {
        t.in_buf[j] = 0;
        t.out_buf[j] = t.sponge[j];
      }
      t.in_pos = 0;
      t.out_pos = 8;
    }
    t.out_pos -= 1;
    out[i] = t.out_buf[t.out_pos];
  }
}

template <class K>
struct HostPerm {
  const K& k;
  void operator()(uint32_t* s) const { p2_permute(s, k); }
};

// Every lane of the (single) warp holds the same Duplex state and runs the same
// control flow; a permutation runs on each half-warp (both compute the same
// result) and is gathered back into every lane's copy.
template <class HP>
__device__ __forceinline__ void half_apply(uint32_t* s, const HP& perm) {
  const int lane = threadIdx.x & 31;
  uint32_t x = 0;
#pragma unroll
  for (int j = 0; j < 16; j++) x = (lane & 15) == j ? s[j] : x;
  x = perm.half(x);
#pragma unroll
  for (int j = 0; j < 16; j++) s[j] = __shfl_sync(kFullMask, x, (lane & 16) | j);
}

template <class F>
struct HalfPerm {
  const P2Params* p;  // shared memory
  __device__ uint32_t half(uint32_t x) const { return p2_permute_half<F>(x, p); }
  __device__ void operator()(uint32_t* s) const { half_apply(s, *this); }
};

// The built-in BabyBear-16 instance (half_permute_bb16): the constants of this
// lane's word are loaded into registers once, when the transcript kernel
// starts.
struct HalfPermBb16 {
  uint32_t ei[4], et[4], dg;
  __device__ HalfPermBb16() {
    const int l = threadIdx.x & 15;
#pragma unroll
    for (int r = 0; r < 4; r++) {
      ei[r] = c_bb16_ext_init[r * 16 + l];
      et[r] = c_bb16_ext_term[r * 16 + l];
    }
    dg = c_bb16_diag[l];
  }
  __device__ uint32_t half(uint32_t x) const { return half_permute_bb16(x, ei, et, dg); }
  __device__ void operator()(uint32_t* s) const { half_apply(s, *this); }
};

// duplex_observe on the device (same result): full rate blocks are absorbed
// with the sponge kept one word per lane (lane l of each half holds word l),
// each block's eight values loaded straight into lanes 0..7 -- the next
// block's loads issued before the current permutation -- so a long observe
// (a final fold layer, a sponge chain of hundreds of blocks) costs one
// half-warp permutation per block and no per-word state shuffling. The
// pending prefix and the tail take the generic path.
template <class HP>
__device__ void half_observe(Duplex& t, const uint32_t* v, int64_t m, const HP& perm) {
  if (m <= 0) return;
  int pos = t.in_pos & 7;
  int64_t i = 0;
  for (; pos != 0 && i < m; i++) {  // complete a pending block first
    t.in_buf[pos++] = v[i];
    if (pos == 8) {
      for (int j = 0; j < 8; j++) t.sponge[j] = t.in_buf[j];
      perm(t.sponge);
      pos = 0;
    }
  }
  if (m - i >= 8) {
    const int lane = threadIdx.x & 31, l = lane & 15;
    uint32_t x = 0;
#pragma unroll
    for (int j = 0; j < 16; j++) x = l == j ? t.sponge[j] : x;
    uint32_t nxt = l < 8 ? v[i + l] : 0u;
    for (; m - i >= 8; i += 8) {
      const uint32_t cur = nxt;
      if (m - i >= 16 && l < 8) nxt = v[i + 8 + l];  // issued before the permutation
      if (l < 8) x = cur;
      x = perm.half(x);
    }
#pragma unroll
    for (int j = 0; j < 16; j++) t.sponge[j] = __shfl_sync(kFullMask, x, (lane & 16) | j);
  }
  for (; i < m; i++) {  // the tail stays pending (m - i < 8)
    t.in_buf[pos++] = v[i];
  }
  for (int j = pos; j < 8; j++) t.in_buf[j] = 0;
  t.in_pos = pos;
  if (pos == 0) {
    for (int j = 0; j < 8; j++) t.out_buf[j] = t.sponge[j];
    t.out_pos = 8;
  } else {
    for (int j = 0; j < 8; j++) t.out_buf[j] = 0;
    t.out_pos = 0;
  }
}
template <class F>
__device__ void duplex_observe(Duplex& t, const uint32_t* v, int64_t m, const HalfPerm<F>& perm) {
  half_observe(t, v, m, perm);
}
__device__ inline void duplex_observe(Duplex& t, const uint32_t* v, int64_t m,
                                      const HalfPermBb16& perm) {
  half_observe(t, v, m, perm);
}

}  // namespace zc
