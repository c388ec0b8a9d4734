// Reed-Solomon coset low-degree extension (ReedSolomon.encode,
// zorch/coding/reed_solomon.py:177-188): out[j] = sum_i m_i (h w_n^j)^i,
// natural order in and out, n = k * b.
//
// Decomposition: with j = b*t + s (s < b, t < k),
//   out[b*t + s] = NTT_k(m_i * g_s^i)[t],   g_s = h * w_n^s,
// i.e. b coset NTTs of size k over the unpadded message (the zero padding of
// the reference is never materialised). Each size-k NTT runs in shared memory:
//  - k <= 4096 and b*k <= 16384: one pass, one CTA per column holding all b
//    cosets, so the b*k outputs are written as one contiguous block;
//  - otherwise the four-step (Bailey) split k = k1 * k2: pass 1 runs k2-point
//    NTTs down strided columns (a tile of consecutive i1 per CTA, one coset
//    per CTA), multiplies by w_k^(i1*t2) and writes a [b][k2][k1] intermediate
//    to the caller's workspace; pass 2 runs the k1-point NTTs along its rows
//    for all b cosets of a t2 tile and writes contiguous b*TT runs of out.
// In shared memory the transform is a radix-2 decimation-in-frequency NTT
// (natural order in, bit-reversed order out), processed in balanced register
// passes of up to 4 stages.
//
// Bit-reversed codewords (BitReversedReedSolomon.encode,
// zorch/coding/reed_solomon.py:476-478) cost nothing extra: with n = b*k and
// j = b*t + s, brev_n(j) = brev_b(s)*k + brev_k(t), and with t = t2 + k2*t1 in
// the four-step split brev_k(t) = brev_k2(t2)*k1 + brev_k1(t1) -- the second
// term is exactly the position in the DIF output row. So each transformed row
// lands as one contiguous run of the bit-reversed codeword.
#include <string.h>

#include <mutex>

#include "internal.cuh"

namespace zc {

// w^i tables for the primitive 2^TA-th root w = gen^((p-1)/2^TA) (TA = the
// field's two-adicity): lo[i] = w^i (i < 2^14), hi[i] = w^(i*2^14). Static
// device memory -- no allocation; filled once per device by zc_init.
constexpr int kRootLoBits = 14;
__device__ uint32_t g_roots_bb[(1 << kRootLoBits) + (1 << (BabyBear::TWO_ADICITY - kRootLoBits))];
__device__ uint32_t g_roots_kb[(1 << kRootLoBits) + (1 << (KoalaBear::TWO_ADICITY - kRootLoBits))];

template <class F>
__device__ __forceinline__ uint32_t* roots_tab();
template <>
__device__ __forceinline__ uint32_t* roots_tab<BabyBear>() { return g_roots_bb; }
template <>
__device__ __forceinline__ uint32_t* roots_tab<KoalaBear>() { return g_roots_kb; }

template <class F>
__global__ void k_init_roots() {
  constexpr int lo = 1 << kRootLoBits, hi = 1 << (F::TWO_ADICITY - kRootLoBits);
  const uint32_t w = root_of_unity<F>(F::TWO_ADICITY, 0);
  uint32_t* t = roots_tab<F>();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < lo + hi; i += gridDim.x * blockDim.x) {
    const uint64_t e = i < lo ? (uint64_t)i : (uint64_t)(i - lo) << kRootLoBits;
    t[i] = mpow<F>(w, e);
  }
}

zc_status init_root_tables() {
  k_init_roots<BabyBear><<<64, 256>>>();
  ZC_TRY(launch_check());
  k_init_roots<KoalaBear><<<64, 256>>>();
  ZC_TRY(launch_check());
  return ZC_OK;
}

// w_{2^log_n}^e for e < 2^log_n.
template <class F>
__device__ __forceinline__ uint32_t omega_pow(int log_n, uint32_t e) {
  const uint32_t E = e << (F::TWO_ADICITY - log_n);
  const uint32_t* t = roots_tab<F>();
  return mmul<F>(t[E & ((1u << kRootLoBits) - 1)], t[(1u << kRootLoBits) + (E >> kRootLoBits)]);
}

__device__ __forceinline__ int pad(int i) { return i + (i >> 5); }
__device__ __forceinline__ int brev(int i, int bits) {
  return bits ? (int)(__brev((unsigned)i) >> (32 - bits)) : 0;
}
// brev(j, R) for a j known at compile time once a member loop is unrolled.
template <int R>
__host__ __device__ constexpr int brev_r(int j) {
  int r = 0;
  for (int b = 0; b < R; b++) r |= ((j >> b) & 1) << (R - 1 - b);
  return r;
}
__host__ __device__ __forceinline__ int padded(int m) { return m + (m >> 5); }
// Row stride of a tile of rows of m words: padded, then odd, so that threads
// of a warp reading the same position of consecutive rows hit distinct banks.
__host__ __device__ __forceinline__ int row_stride(int m) { return padded(m) | 1; }

// tab[i] = base^i for i < count (count a power of two), by doubling.
template <class F>
__device__ void pow_table(uint32_t* tab, int count, uint32_t base) {
  if (threadIdx.x == 0) {
    tab[0] = F::ONE;
    if (count > 1) tab[1] = base;
  }
  __syncthreads();
  for (int len = 2; len < count; len <<= 1) {
    const uint32_t step = mmul<F>(tab[len >> 1], tab[len >> 1]);
    for (int i = threadIdx.x; i < len; i += blockDim.x) tab[len + i] = mmul<F>(tab[i], step);
    __syncthreads();
  }
}

// tab[i] = w_{2^log_m}^i for i < count <= 2^log_m, read straight off the
// root tables (independent entries: no multiply chain, no barrier).
template <class F>
__device__ void root_table(uint32_t* tab, int count, int log_m) {
  for (int i = threadIdx.x; i < count; i += blockDim.x) tab[i] = omega_pow<F>(log_m, (uint32_t)i);
}

// One radix-2^R pass of a decimation-in-frequency NTT over `rows` rows of
// m = 2^logm words (row stride rs): the stages of half-size 2^h0 down to
// 2^(h0-R+1). A group is the 2^R elements base + j*S, S = 2^(h0-R+1); the
// butterfly (u, v) -> (u + v, (u - v) * w_{2H}^pos) with pos the offset in the
// 2H-block. Consecutive threads take consecutive rows (row-major tiles) so a
// warp's shared-memory accesses fall on distinct banks.
// The R stages of one radix-2^R group held in registers: members j at
// positions base + j S (S = 2^lS, off = base mod S); stage r's twiddle is
// tw[pos << (sh0 + r)] with pos = off + (j mod 2^hb) S.
template <class F, int R>
__device__ __forceinline__ void dif_group(uint32_t (&v)[1 << R], const uint32_t* tw, int off,
                                          int lS, int sh0) {
  constexpr int G = 1 << R;
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int hb = R - 1 - r;  // local bit of this stage
    // pos = off + jm S with jm = j mod 2^hb: index = (off << sh) + jm (S << sh)
    const int sh = sh0 + r;
    const int tb = off << sh, ts = 1 << (lS + sh);
#pragma unroll
    for (int j = 0; j < G; j++) {
      if (!(j & (1 << hb))) {
        const int j2 = j | (1 << hb);
        const uint32_t w = tw[tb + (j & ((1 << hb) - 1)) * ts];
        const uint32_t u = v[j], t = v[j2];
        v[j] = madd<F>(u, t);
        // u - t in (-p, p) feeds the signed product directly
        v[j2] = snorm<F>(smul<F>((int32_t)(u - t), (int32_t)w));
      }
    }
  }
}

template <class F, int R>
__device__ __forceinline__ void dif_pass(uint32_t* a, int log_rows, int logm, int rs,
                                         const uint32_t* tw, int h0) {
  constexpr int G = 1 << R;
  const int lS = h0 - R + 1;
  const int glog = logm - R;
  const int total = 1 << (log_rows + glog);
  const int rmask = (1 << log_rows) - 1;
  // Stage r of this pass reads the twiddle tw[pos << (sh0 + r)].
  const int sh0 = logm - 1 - h0;
  for (int gi = threadIdx.x; gi < total; gi += blockDim.x) {
    const int row = gi & rmask, g = gi >> log_rows;
    const int off = g & ((1 << lS) - 1), blk = g >> lS;
    const int base = (blk << (h0 + 1)) | off;
    // Member j sits at pad(base + j S) = pad(base) + pad(j S): base's low five
    // bits plus j S never carry past a 32-word boundary that j S does not
    // itself cross (off < S, and the group spans 2^(h0+1) aligned words), so
    // the member offsets are the same for every group of the pass.
    uint32_t* ar = a + row * rs + pad(base);
    uint32_t v[G];
#pragma unroll
    for (int j = 0; j < G; j++) v[j] = ar[pad(j << lS)];
    dif_group<F, R>(v, tw, off, lS, sh0);
#pragma unroll
    for (int j = 0; j < G; j++) ar[pad(j << lS)] = v[j];
  }
}

// DIF NTT of each row, natural order in, bit-reversed order out (position p
// holds output index brev(p)); stages split into balanced passes of <= 4.
// Largest radix-2^R register pass by default (radix-2^5 passes spill under
// the 64-register cap the two-CTA occupancy needs).
constexpr int kMaxRadixLog = 4;
// The wide four-step variant (k_lde_pass1/2 with MR = 5): radix-2^5 register
// passes -- two passes for a 2^10 row instead of three, so one shared-memory
// round trip and one barrier fewer per four-step pass -- need 128 registers,
// hence 512 threads per SM: two 256-thread CTAs on 2^14-word tiles (one CTA's
// loads overlap the other's arithmetic), or one 512-thread CTA on 2^15-word
// tiles. Used for large transforms (lde_launch).
constexpr int kWideRadixLog = 5;
#ifndef ZC_LDE_WIDE_THREADS
#define ZC_LDE_WIDE_THREADS 256
#endif
static_assert(ZC_LDE_WIDE_THREADS == 256 || ZC_LDE_WIDE_THREADS == 512,
              "wide LDE CTAs of 256 or 512 threads");
constexpr int kWideThreads = ZC_LDE_WIDE_THREADS;
constexpr int kWideTileLog = kWideThreads == 256 ? 14 : 15;

// max_r (2..4) bounds the passes' radix: ceil(logm / max_r) balanced passes.
template <class F>
__device__ void smem_ntt_dif(uint32_t* a, int log_rows, int logm, int rs, const uint32_t* tw,
                             int max_r = kMaxRadixLog) {
  const int passes = (logm + max_r - 1) / max_r;
  int h0 = logm - 1;
  for (int q = 0; q < passes; q++) {
    const int remaining = h0 + 1;
    const int R = (remaining + (passes - q) - 1) / (passes - q);
    switch (R) {
      case 4: dif_pass<F, 4>(a, log_rows, logm, rs, tw, h0); break;
      case 3: dif_pass<F, 3>(a, log_rows, logm, rs, tw, h0); break;
      case 2: dif_pass<F, 2>(a, log_rows, logm, rs, tw, h0); break;
      default: dif_pass<F, 1>(a, log_rows, logm, rs, tw, h0); break;
    }
    __syncthreads();
    h0 -= R;
  }
}

constexpr int kThreads = 512;
[[maybe_unused]] constexpr int kLogThreads = 9;
// Threads and resident CTAs per SM of the four-step passes with largest radix
// 2^MR: the wide build's 128 registers allow 512 threads per SM.
template <int MR>
constexpr int lde_threads() {
  return MR > 4 ? kWideThreads : kThreads;
}
template <int MR>
constexpr int lde_min_blocks() {
  return MR > 4 ? 65536 / (128 * kWideThreads) : 2;
}

// Asynchronous 4-byte global -> shared copies (cp.async): a tile's loads are
// all in flight at once, overlapping the twiddle-table set-up, instead of one
// register-staged load per loop iteration waiting on memory.
__device__ __forceinline__ void cp_async4(uint32_t* smem_dst, const uint32_t* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// One column, all b cosets (single pass). `sm` is the block's dynamic smem.
// Layout: work[b][rs] | tw[k/2] | hp[k] | wl[128] | wh[128].
template <class F>
__device__ void lde_small_body(const uint32_t* x, uint32_t* out, int log_k, int log_b,
                               uint32_t h, int64_t c, uint32_t* sm, int brev_out,
                               int max_r = kMaxRadixLog) {
  const int k = 1 << log_k, b = 1 << log_b, log_n = log_k + log_b;
  const int rs = row_stride(k);
  uint32_t* work = sm;
  uint32_t* tw = work + b * rs;
  uint32_t* hp = tw + (k > 1 ? k / 2 : 1);
  uint32_t* wl = hp + k;    // w_n^e, e < 128
  uint32_t* wh = wl + 128;  // w_n^(128 e), e < 128
  const uint32_t* xc = x + (c << log_k);
  for (int idx = threadIdx.x; idx < (b << log_k); idx += blockDim.x)
    cp_async4(work + (idx >> log_k) * rs + pad(idx & (k - 1)), xc + (idx & (k - 1)));
  root_table<F>(tw, k > 1 ? k / 2 : 1, log_k);
  const uint32_t nmask = (1u << log_n) - 1;  // w_n^e depends on e mod n
  for (int e = threadIdx.x; e < 128; e += blockDim.x) {
    wl[e] = omega_pow<F>(log_n, (uint32_t)e & nmask);
    wh[e] = omega_pow<F>(log_n, ((uint32_t)e << 7) & nmask);
  }
  pow_table<F>(hp, k, h);
  cp_async_wait_all();
  for (int idx = threadIdx.x; idx < (b << log_k); idx += blockDim.x) {
    const int s = idx >> log_k, i = idx & (k - 1);
    uint32_t* slot = work + s * rs + pad(i);
    int32_t v = smul<F>((int32_t)*slot, (int32_t)hp[i]);
    if (s) {
      const int e = s * i;  // < n <= 2^14
      v = smul<F>(v, smul<F>((int32_t)wl[e & 127], (int32_t)wh[e >> 7]));
    }
    *slot = snorm<F>(v);
  }
  __syncthreads();
  smem_ntt_dif<F>(work, log_b, log_k, rs, tw, max_r);
  uint32_t* oc = out + (c << log_n);
  if (brev_out) {  // out[brev_b(s) k + p] = row s, position p
    for (int idx = threadIdx.x; idx < (b << log_k); idx += blockDim.x) {
      const int s = brev(idx >> log_k, log_b), p = idx & (k - 1);
      oc[idx] = work[s * rs + pad(p)];
    }
    return;
  }
  for (int idx = threadIdx.x; idx < (b << log_k); idx += blockDim.x) {
    const int t = idx >> log_b, s = idx & (b - 1);
    oc[idx] = work[s * rs + pad(brev(t, log_k))];
  }
}

template <class F>
__global__ void __launch_bounds__(kThreads, 2) k_lde_small(const uint32_t* x, uint32_t* out,
                                                        int log_k, int log_b, uint32_t h,
                                                        int brev_out) {
  extern __shared__ uint32_t sm[];
  lde_small_body<F>(x, out, log_k, log_b, h, blockIdx.x, sm, brev_out);
}

// Pass 1 item (coset s, i1 tile, column c): the k2-point DIF NTTs down the
// strided columns i1 of the message scaled by g_s^(i1 + k1 i2); writes the
// untwiddled intermediate z[c][s][t2][i1] (t2 = bit-reversed position).
// Layout: work[TI][rs] | tw[k2/2] | gi[TI].
template <class F>
__device__ void lde_pass1_body(const uint32_t* x, uint32_t* z, int log_k1, int log_k2, int log_b,
                               int log_ti, uint32_t h, int s, int tile, int64_t c,
                               uint32_t* sm, int max_r = kMaxRadixLog) {
  const int k1 = 1 << log_k1, k2 = 1 << log_k2, TI = 1 << log_ti;
  const int log_k = log_k1 + log_k2, log_n = log_k + log_b;
  const int rs = row_stride(k2);
  uint32_t* work = sm;
  uint32_t* tw = work + TI * rs;
  uint32_t* gi = tw + (k2 > 1 ? k2 / 2 : 1);
  const int i1_0 = tile * TI;
  // Thread t always owns column d = t mod TI (TI <= kThreads, both powers of
  // two) and walks i2 = t / TI, + kThreads / TI, ...: the column offsets are
  // loop-invariant and the row offsets step by constants.
  const int d = threadIdx.x & (TI - 1), i2_0 = threadIdx.x >> log_ti;
  const int di = kThreads >> log_ti;
  uint32_t* wd = work + d * rs;
  {
    const uint32_t* src = x + (c << log_k) + i1_0 + d + ((int64_t)i2_0 << log_k1);
    const int64_t sstep = (int64_t)di << log_k1;
    for (int i2 = i2_0; i2 < k2; i2 += di, src += sstep) cp_async4(wd + pad(i2), src);
  }
  const uint32_t gs = mmul<F>(h, s ? omega_pow<F>(log_n, (uint32_t)s) : F::ONE);
  const uint32_t G = mpow<F>(gs, (uint64_t)k1);
  root_table<F>(tw, k2 > 1 ? k2 / 2 : 1, log_k2);
  for (int i = threadIdx.x; i < TI; i += blockDim.x) gi[i] = mpow<F>(gs, (uint64_t)(i1_0 + i));
  // word (d, i2) is scaled by gs^(i1_0 + d + k1 i2) = gi[d] G^i2: a running
  // product per thread, G^i2_0 then times G^di per step (no table, no barriers)
  const uint32_t g_first = mpow<F>(G, (uint64_t)i2_0), g_step = mpow<F>(G, (uint64_t)di);
  __syncthreads();
  cp_async_wait_all();
  {  // each thread scales the words it loaded itself (no barrier needed)
    int32_t fac = smul<F>((int32_t)gi[d], (int32_t)g_first);
    for (int i2 = i2_0; i2 < k2; i2 += di) {
      uint32_t* slot = wd + pad(i2);
      *slot = snorm<F>(smul<F>((int32_t)*slot, fac));
      fac = smul<F>(fac, (int32_t)g_step);
    }
  }
  __syncthreads();
  smem_ntt_dif<F>(work, log_ti, log_k2, rs, tw, max_r);
  uint32_t* zd = z + ((c << log_b) + s) * ((int64_t)1 << log_k) + i1_0 + d;
  for (int p = i2_0; p < k2; p += di) zd[(uint32_t)brev(p, log_k2) << log_k1] = wd[pad(p)];
}

// ---------------------------------------------------------- fused passes --
// The four-step passes with the first radix pass fed straight from global
// memory and the last radix pass writing straight to global memory: each
// thread loads its group's 2^R members into registers (coalesced across the
// warp, all loads in flight at once), applies the coset / four-step scale
// there, runs the R stages and writes shared memory; the middle passes are
// dif_pass; the last pass reads shared memory, runs its stages and stores the
// outputs at their final positions. Compared with staging the tile through
// per-word cp.async copies, a separate scale loop and a separate output loop,
// this removes one shared-memory round trip and two barrier-separated loops
// per pass (the words, products and results are the same).
#ifndef ZC_LDE_FUSED
#define ZC_LDE_FUSED 1
#endif

// Balanced radix of pass q of `passes` over the stages left (h0 + 1).
__host__ __device__ __forceinline__ int pass_radix(int h0, int passes, int q) {
  return (h0 + 1 + (passes - q) - 1) / (passes - q);
}
__host__ __device__ __forceinline__ int pass_count(int logm, int max_r) {
  return (logm + max_r - 1) / max_r;
}
// log2 of the first pass's member stride S (= its number of groups per row).
__host__ __device__ __forceinline__ int first_stride_log(int logm, int max_r) {
  return logm - pass_radix(logm - 1, pass_count(logm, max_r), 0);
}

// Pass 1, one radix pass: rows d < TI (the i1 columns of the tile), row length
// k2 (the i2 index). first: the members come from x, scaled by
// gs^(i1 + k1 i2) = gi[d] * G^off * (G^S)^j; last: the outputs go to z at the
// bit-reversed position brev(p) << log_k1.
template <class F, int R>
__device__ __forceinline__ void p1_pass(uint32_t* work, int rs, int log_ti, int log_k1,
                                        int log_k2, int h0, bool first, bool last,
                                        const uint32_t* xs, const uint32_t* gi, const uint32_t* Gt,
                                        uint32_t GS, const uint32_t* tw, uint32_t* zd) {
  constexpr int G = 1 << R;
  const int lS = h0 - R + 1;
  const int total = 1 << (log_ti + log_k2 - R);
  const int rmask = (1 << log_ti) - 1;
  const int sh0 = log_k2 - 1 - h0;
  for (int it = threadIdx.x; it < total; it += blockDim.x) {
    const int d = it & rmask, g = it >> log_ti;
    const int off = g & ((1 << lS) - 1), blk = g >> lS;
    const int base = (blk << (h0 + 1)) | off;  // first pass: blk == 0, base == off
    uint32_t* ar = work + d * rs + pad(base);
    uint32_t v[G];
    if (first) {
      const uint32_t* src = xs + d + ((int64_t)off << log_k1);
#pragma unroll
      for (int j = 0; j < G; j++) v[j] = __ldg(src + ((int64_t)j << (lS + log_k1)));
      int32_t f = smul<F>((int32_t)gi[d], (int32_t)Gt[off]);
#pragma unroll
      for (int j = 0; j < G; j++) {
        v[j] = snorm<F>(smul<F>((int32_t)v[j], f));
        if (j + 1 < G) f = smul<F>(f, (int32_t)GS);
      }
    } else {
#pragma unroll
      for (int j = 0; j < G; j++) v[j] = ar[pad(j << lS)];
    }
    dif_group<F, R>(v, tw, off, lS, sh0);
    if (last) {  // lS == 0: members are the positions base + j, base = blk 2^R, so
                 // brev(base + j) = brev(base) + brev_R(j) 2^(log_k2 - R)
      uint32_t* zp = zd + d + ((uint32_t)brev(base, log_k2) << log_k1);
      const int so = log_k1 + log_k2 - R;
#pragma unroll
      for (int j = 0; j < G; j++) zp[(uint32_t)brev_r<R>(j) << so] = v[j];
    } else {
#pragma unroll
      for (int j = 0; j < G; j++) ar[pad(j << lS)] = v[j];
    }
  }
}

// Pass-1 item with fused load and store. Layout: work[TI][rs] | tw[k2/2] |
// gi[TI] | Gt[S] (S = the first pass's member stride). MR: the largest radix
// compiled in (max_r <= MR).
template <class F, int MR = kMaxRadixLog>
__device__ void lde_pass1_fused(const uint32_t* x, uint32_t* z, int log_k1, int log_k2, int log_b,
                                int log_ti, uint32_t h, int s, int tile, int64_t c, uint32_t* sm,
                                int max_r) {
  const int k1 = 1 << log_k1, k2 = 1 << log_k2, TI = 1 << log_ti;
  const int log_k = log_k1 + log_k2, log_n = log_k + log_b;
  const int rs = row_stride(k2);
  const int lS0 = first_stride_log(log_k2, max_r);
  uint32_t* work = sm;
  uint32_t* tw = work + TI * rs;
  uint32_t* gi = tw + (k2 > 1 ? k2 / 2 : 1);
  uint32_t* Gt = gi + TI;
  const int i1_0 = tile * TI;
  const uint32_t gs = mmul<F>(h, s ? omega_pow<F>(log_n, (uint32_t)s) : F::ONE);
  const uint32_t G = mpow<F>(gs, (uint64_t)k1);
  root_table<F>(tw, k2 > 1 ? k2 / 2 : 1, log_k2);
  for (int i = threadIdx.x; i < TI; i += blockDim.x) gi[i] = mpow<F>(gs, (uint64_t)(i1_0 + i));
  for (int i = threadIdx.x; i < (1 << lS0); i += blockDim.x) Gt[i] = mpow<F>(G, (uint64_t)i);
  const uint32_t GS = mpow<F>(G, (uint64_t)1 << lS0);
  __syncthreads();
  const uint32_t* xs = x + (c << log_k) + i1_0;
  uint32_t* zd = z + ((c << log_b) + s) * ((int64_t)1 << log_k) + i1_0;
  const int passes = pass_count(log_k2, max_r);
  int h0 = log_k2 - 1;
  for (int q = 0; q < passes; q++) {
    const int R = pass_radix(h0, passes, q);
    const bool first = q == 0, last = q == passes - 1;
    switch (R) {
      case 5: if constexpr (MR >= 5) p1_pass<F, 5>(work, rs, log_ti, log_k1, log_k2, h0, first, last, xs, gi, Gt, GS, tw, zd); break;
      case 4: p1_pass<F, 4>(work, rs, log_ti, log_k1, log_k2, h0, first, last, xs, gi, Gt, GS, tw, zd); break;
      case 3: p1_pass<F, 3>(work, rs, log_ti, log_k1, log_k2, h0, first, last, xs, gi, Gt, GS, tw, zd); break;
      case 2: p1_pass<F, 2>(work, rs, log_ti, log_k1, log_k2, h0, first, last, xs, gi, Gt, GS, tw, zd); break;
      default: p1_pass<F, 1>(work, rs, log_ti, log_k1, log_k2, h0, first, last, xs, gi, Gt, GS, tw, zd); break;
    }
    if (!last) __syncthreads();
    h0 -= R;
  }
}

// Pass 2, first radix pass from z: a thread takes one group position `off` of
// row dt for every coset s in turn (consecutive threads on consecutive off:
// coalesced loads), the scale w_k^(t i1) = w_k^(t off) (w_k^(t S))^j computed
// once for the b rows. Shared rows are ordered r = dt * b + s.
template <class F, int R>
__device__ __forceinline__ void p2_first(uint32_t* work, int rs, int log_b, int log_tt, int log_k1,
                                         int log_k, int t2_0, const uint32_t* zc_,
                                         const uint32_t* tw, bool last, uint32_t* oc,
                                         int log_k2, int brev_out) {
  constexpr int G = 1 << R;
  const int h0 = log_k1 - 1, lS = h0 - R + 1;
  const int total = 1 << (log_tt + lS);
  const int b = 1 << log_b;
  const uint32_t kmask = (1u << log_k) - 1;
  for (int it = threadIdx.x; it < total; it += blockDim.x) {
    const int off = it & ((1 << lS) - 1), dt = it >> lS;
    const uint32_t t = (uint32_t)(t2_0 + dt);
    int32_t f[G];
    f[0] = (int32_t)omega_pow<F>(log_k, (t * (uint32_t)off) & kmask);
    const int32_t step = (int32_t)omega_pow<F>(log_k, (t << lS) & kmask);
#pragma unroll
    for (int j = 1; j < G; j++) f[j] = smul<F>(f[j - 1], step);
    for (int s = 0; s < b; s++) {
      const uint32_t* src = zc_ + ((int64_t)s << log_k) + ((int64_t)t << log_k1) + off;
      uint32_t v[G];
#pragma unroll
      for (int j = 0; j < G; j++) v[j] = __ldg(src + (j << lS));
#pragma unroll
      for (int j = 0; j < G; j++) v[j] = snorm<F>(smul<F>((int32_t)v[j], f[j]));
      dif_group<F, R>(v, tw, off, lS, 0);
      if (last) {  // a single pass (k1 <= 16): off == 0, positions j
#pragma unroll
        for (int j = 0; j < G; j++) {
          if (brev_out)
            oc[((int64_t)brev(s, log_b) << log_k) + ((int64_t)brev((int)t, log_k2) << log_k1) + j] = v[j];
          else
            oc[((int64_t)t << log_b) + s + ((int64_t)brev_r<R>(j) << (log_k2 + log_b))] = v[j];  // R == log_k1
        }
      } else {
        uint32_t* ar = work + ((dt << log_b) + s) * rs + pad(off);
#pragma unroll
        for (int j = 0; j < G; j++) ar[pad(j << lS)] = v[j];
      }
    }
  }
}

// Pass 2, last radix pass to `out`: consecutive threads on consecutive rows
// r = dt * b + s, so natural-order stores out[b (t2 + k2 t1) + s] are
// coalesced and the shared-memory reads fall on distinct banks.
template <class F, int R>
__device__ __forceinline__ void p2_last(uint32_t* work, int rs, int log_b, int log_tt, int log_k1,
                                        int log_k2, int log_k, int t2_0, int h0,
                                        const uint32_t* tw, uint32_t* oc, int brev_out) {
  constexpr int G = 1 << R;
  const int log_rows = log_b + log_tt;
  const int total = 1 << (log_rows + log_k1 - R);
  const int rmask = (1 << log_rows) - 1;
  const int sh0 = log_k1 - 1 - h0;  // h0 == R - 1: lS == 0
  for (int it = threadIdx.x; it < total; it += blockDim.x) {
    const int r = it & rmask, g = it >> log_rows;
    const int s = r & ((1 << log_b) - 1), dt = r >> log_b;
    const int base = g << R;
    uint32_t* ar = work + r * rs + pad(base);
    uint32_t v[G];
#pragma unroll
    for (int j = 0; j < G; j++) v[j] = ar[pad(j)];
    dif_group<F, R>(v, tw, 0, 0, sh0);
    const int t = t2_0 + dt;
    if (brev_out) {
      uint32_t* orow = oc + ((int64_t)brev(s, log_b) << log_k) +
                       ((int64_t)brev(t, log_k2) << log_k1) + base;
#pragma unroll
      for (int j = 0; j < G; j++) orow[j] = v[j];
    } else {
      // base = g 2^R: brev(base + j) = brev(base) + brev_R(j) 2^(log_k1 - R)
      const int sh = log_k2 + log_b;
      uint32_t* ob = oc + ((int64_t)t << log_b) + s + ((int64_t)brev(base, log_k1) << sh);
      const int so = log_k1 - R + sh;
#pragma unroll
      for (int j = 0; j < G; j++) ob[(uint32_t)brev_r<R>(j) << so] = v[j];  // < n <= 2^30
    }
  }
}

// Pass-2 item with fused load and store. Layout: work[b*TT][rs] | tw[k1/2].
template <class F, int MR = kMaxRadixLog>
__device__ void lde_pass2_fused(const uint32_t* z, uint32_t* out, int log_k1, int log_k2,
                                int log_b, int log_tt, int tile, int64_t c, uint32_t* sm,
                                int brev_out, int max_r) {
  const int k1 = 1 << log_k1;
  const int log_k = log_k1 + log_k2, log_n = log_k + log_b;
  const int log_rows = log_b + log_tt;
  const int rs = row_stride(k1);
  uint32_t* work = sm;
  uint32_t* tw = work + (rs << log_rows);
  const int t2_0 = tile << log_tt;
  const uint32_t* zc_ = z + (c << log_n);
  uint32_t* oc = out + (c << log_n);
  root_table<F>(tw, k1 > 1 ? k1 / 2 : 1, log_k1);
  __syncthreads();
  const int passes = pass_count(log_k1, max_r);
  int h0 = log_k1 - 1;
  for (int q = 0; q < passes; q++) {
    int R = pass_radix(h0, passes, q);
    // the first pass maps a warp onto 2^(log_k1 - R) consecutive offsets of a
    // row: keep that at >= 32 (conflict-free shared-memory writes) by taking
    // the smaller radix first (a 2^9 row: 4 + 5, not 5 + 4)
    if (q == 0 && passes > 1 && log_k1 - R < 5) R = log_k1 / passes;
    const bool first = q == 0, last = q == passes - 1;
    if (first) {
      switch (R) {
        case 5: if constexpr (MR >= 5) p2_first<F, 5>(work, rs, log_b, log_tt, log_k1, log_k, t2_0, zc_, tw, last, oc, log_k2, brev_out); break;
        case 4: p2_first<F, 4>(work, rs, log_b, log_tt, log_k1, log_k, t2_0, zc_, tw, last, oc, log_k2, brev_out); break;
        case 3: p2_first<F, 3>(work, rs, log_b, log_tt, log_k1, log_k, t2_0, zc_, tw, last, oc, log_k2, brev_out); break;
        case 2: p2_first<F, 2>(work, rs, log_b, log_tt, log_k1, log_k, t2_0, zc_, tw, last, oc, log_k2, brev_out); break;
        default: p2_first<F, 1>(work, rs, log_b, log_tt, log_k1, log_k, t2_0, zc_, tw, last, oc, log_k2, brev_out); break;
      }
    } else if (last) {
      switch (R) {
        case 5: if constexpr (MR >= 5) p2_last<F, 5>(work, rs, log_b, log_tt, log_k1, log_k2, log_k, t2_0, h0, tw, oc, brev_out); break;
        case 4: p2_last<F, 4>(work, rs, log_b, log_tt, log_k1, log_k2, log_k, t2_0, h0, tw, oc, brev_out); break;
        case 3: p2_last<F, 3>(work, rs, log_b, log_tt, log_k1, log_k2, log_k, t2_0, h0, tw, oc, brev_out); break;
        case 2: p2_last<F, 2>(work, rs, log_b, log_tt, log_k1, log_k2, log_k, t2_0, h0, tw, oc, brev_out); break;
        default: p2_last<F, 1>(work, rs, log_b, log_tt, log_k1, log_k2, log_k, t2_0, h0, tw, oc, brev_out); break;
      }
    } else {
      switch (R) {
        case 5: if constexpr (MR >= 5) dif_pass<F, 5>(work, log_rows, log_k1, rs, tw, h0); break;
        case 4: dif_pass<F, 4>(work, log_rows, log_k1, rs, tw, h0); break;
        case 3: dif_pass<F, 3>(work, log_rows, log_k1, rs, tw, h0); break;
        case 2: dif_pass<F, 2>(work, log_rows, log_k1, rs, tw, h0); break;
        default: dif_pass<F, 1>(work, log_rows, log_k1, rs, tw, h0); break;
      }
    }
    if (!last) __syncthreads();
    h0 -= R;
  }
}

template <class F, int MR = kMaxRadixLog>
__global__ void __launch_bounds__(lde_threads<MR>(), lde_min_blocks<MR>()) k_lde_pass1(const uint32_t* x, uint32_t* z, int log_k1,
                                                        int log_k2, int log_b, int log_ti,
                                                        uint32_t h) {
  extern __shared__ uint32_t sm[];
#if ZC_LDE_FUSED
  lde_pass1_fused<F, MR>(x, z, log_k1, log_k2, log_b, log_ti, h, blockIdx.x, blockIdx.y,
                         blockIdx.z, sm, MR);
#else
  lde_pass1_body<F>(x, z, log_k1, log_k2, log_b, log_ti, h, blockIdx.x, blockIdx.y, blockIdx.z,
                    sm);
#endif
}

// Pass 2 item (t2 tile, column c): rows (s, t2) for all b cosets and TT
// values of t2; each row is multiplied by w_k^(t2 i1), transformed by a
// k1-point DIF NTT, and written to out[b (t2 + k2 t1) + s] (t1 = bit-reversed
// position) in contiguous runs of b*TT words -- or, for a bit-reversed
// codeword, row (s, t2) to the k1 contiguous words at brev_b(s) k + brev_k2(t2) k1.
// Layout: work[b*TT][rs] | tw[k1/2].
template <class F>
__device__ void lde_pass2_body(const uint32_t* z, uint32_t* out, int log_k1, int log_k2,
                               int log_b, int log_tt, int tile, int64_t c, uint32_t* sm,
                               int brev_out, int max_r = kMaxRadixLog) {
  const int k1 = 1 << log_k1, TT = 1 << log_tt;
  const int log_k = log_k1 + log_k2, log_n = log_k + log_b;
  const int log_rows = log_b + log_tt;
  const int rs = row_stride(k1);
  uint32_t* work = sm;
  uint32_t* tw = work + (rs << log_rows);
  const int t2_0 = tile * TT;
  const uint32_t* zc_ = z + (c << log_n);
  // Thread t owns positions i1 = t mod tpr, + tpr, ... (tpr = min(k1,
  // kThreads) threads per row, consecutive threads on consecutive words) of
  // rows dt = t / tpr, + dt_step, ... of every coset s; it loads and scales
  // exactly these words, so the scale needs no barrier after the loads.
  const int lt = log_k1 < kLogThreads ? log_k1 : kLogThreads;
  const int tpr = 1 << lt;
  const int i1_0 = threadIdx.x & (tpr - 1);
  const int dt_0 = threadIdx.x >> lt, dt_step = kThreads >> lt;
  const int b = 1 << log_b;
  for (int i1 = i1_0; i1 < k1; i1 += tpr)
    for (int s = 0; s < b; s++) {
      uint32_t* wp = work + (s << log_tt) * rs + pad(i1);
      const uint32_t* zp = zc_ + ((int64_t)s << log_k) + ((int64_t)t2_0 << log_k1) + i1;
      for (int dt = dt_0; dt < TT; dt += dt_step)
        cp_async4(wp + dt * rs, zp + ((uint32_t)dt << log_k1));
    }
  root_table<F>(tw, k1 > 1 ? k1 / 2 : 1, log_k1);
  // word (s, dt, i1) is scaled by w_k^((t2_0 + dt) i1), the same for every
  // coset s: a running product over this thread's rows, stepping by
  // w_k^(dt_step i1)
  const uint32_t kmask = (1u << log_k) - 1;
  __syncthreads();
  cp_async_wait_all();
  for (int i1 = i1_0; i1 < k1; i1 += tpr) {
    int32_t fac = (int32_t)omega_pow<F>(log_k, ((uint32_t)(t2_0 + dt_0) * (uint32_t)i1) & kmask);
    const int32_t step = (int32_t)omega_pow<F>(log_k, ((uint32_t)dt_step * (uint32_t)i1) & kmask);
    for (int dt = dt_0; dt < TT; dt += dt_step) {
      uint32_t* wp = work + dt * rs + pad(i1);
      for (int s = 0; s < b; s++) {
        uint32_t* slot = wp + (s << log_tt) * rs;
        *slot = snorm<F>(smul<F>((int32_t)*slot, fac));
      }
      fac = smul<F>(fac, step);
    }
  }
  __syncthreads();
  smem_ntt_dif<F>(work, log_rows, log_k1, rs, tw, max_r);
  uint32_t* oc = out + (c << log_n);
  const int rows = 1 << log_rows;
  if (brev_out) {  // row (s, t2) -> the k1 contiguous words at brev_b(s) k + brev_k2(t2) k1
    for (int s = 0; s < b; s++)
      for (int dt = dt_0; dt < TT; dt += dt_step) {
        const uint32_t* wr = work + ((s << log_tt) + dt) * rs;
        uint32_t* orow = oc + ((int64_t)brev(s, log_b) << log_k) +
                         ((int64_t)brev(t2_0 + dt, log_k2) << log_k1);
        for (int p = i1_0; p < k1; p += tpr) orow[p] = wr[pad(p)];
      }
    return;
  }
  {  // out[b (t2 + k2 t1) + s]: thread t owns row (s, dt) = t mod rows and walks
     // the positions p = t / rows, + kThreads / rows, ... (rows <= kThreads)
    const int ri = threadIdx.x & (rows - 1);
    const int s = ri & ((1 << log_b) - 1), dt = ri >> log_b;
    const uint32_t* wr = work + ((s << log_tt) + dt) * rs;
    uint32_t* ob = oc + ((int64_t)(t2_0 + dt) << log_b) + s;
    const int sh = log_k2 + log_b;
    for (int p = threadIdx.x >> log_rows; p < k1; p += kThreads >> log_rows)
      ob[(uint32_t)brev(p, log_k1) << sh] = wr[pad(p)];  // offset < n <= 2^30
  }
}

template <class F, int MR = kMaxRadixLog>
__global__ void __launch_bounds__(lde_threads<MR>(), lde_min_blocks<MR>()) k_lde_pass2(const uint32_t* z, uint32_t* out,
                                                        int log_k1, int log_k2, int log_b,
                                                        int log_tt, int brev_out) {
  extern __shared__ uint32_t sm[];
#if ZC_LDE_FUSED
  lde_pass2_fused<F, MR>(z, out, log_k1, log_k2, log_b, log_tt, blockIdx.x, blockIdx.y, sm,
                         brev_out, MR);
#else
  lde_pass2_body<F>(z, out, log_k1, log_k2, log_b, log_tt, blockIdx.x, blockIdx.y, sm, brev_out);
#endif
}

struct LdePlan {
  bool small;
  int log_k1, log_k2, log_ti, log_tt;
  size_t smem_small, smem1, smem2;
};

constexpr int kSmallMaxLogK = 12;
constexpr int kSmallMaxLogN = 14;
constexpr int kTileLog = 14;  // elements per shared-memory tile (2^14 = 64 KB)

inline LdePlan plan_lde(int log_k, int log_b, int tile_log = 0, int max_r = kMaxRadixLog) {
  LdePlan p{};
  const int k = 1 << log_k, b = 1 << log_b;
  const int tl = tile_log > 0 ? tile_log : kTileLog;
  p.small = log_k <= kSmallMaxLogK && log_k + log_b <= kSmallMaxLogN;
  p.smem_small = 4 * ((size_t)b * row_stride(k) + (k > 1 ? k / 2 : 1) + k + 256);
  p.log_k2 = log_k / 2;
  p.log_k1 = log_k - p.log_k2;
  int ti = tl - p.log_k2;
  if (p.log_k2 >= 12 && ti < 3) ti = 3;
  if (ti > p.log_k1) ti = p.log_k1;
  if (ti < 0) ti = 0;
  p.log_ti = ti;
  int tt = tl - p.log_k1 - log_b;
  if (tt > p.log_k2) tt = p.log_k2;
  if (tt < 0) tt = 0;
  p.log_tt = tt;
  const int k1 = 1 << p.log_k1, k2 = 1 << p.log_k2;
  p.smem1 = 4 * ((size_t)(1 << p.log_ti) * row_stride(k2) + (k2 > 1 ? k2 / 2 : 1) +
                 (1 << p.log_ti));
#if ZC_LDE_FUSED
  p.smem1 += (size_t)4 << first_stride_log(p.log_k2, max_r);  // the G^off table
#endif
  p.smem2 = 4 * ((size_t)(b << p.log_tt) * row_stride(k1) + (k1 > 1 ? k1 / 2 : 1));
  return p;
}

// Whether a four-step LDE of `batch` columns of 2^log_n outputs takes the
// wide variant: at least two of its tiles per SM (2^20 x 64 at blowup 4 with
// one 512-thread CTA per SM: 2.10 ms against 2.23 ms for the radix-2^4 form
// on the GB300).
inline bool lde_wide(int64_t batch, int log_n) {
#if ZC_LDE_FUSED
  static const int sms = [] {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      n = 152;
    return n;
  }();
  const int64_t tiles = log_n >= kWideTileLog ? batch << (log_n - kWideTileLog) : 0;
  return tiles >= 2 * (int64_t)sms;
#else
  (void)batch;
  (void)log_n;
  return false;
#endif
}

template <class F, int MR>
zc_status lde_four_step(const uint32_t* x, int64_t batch, int log_k, int log_b, uint32_t h,
                        uint32_t* out, void* ws, size_t ws_bytes, cudaStream_t st, int brev_out,
                        const LdePlan& p);

template <class F>
zc_status lde_launch(const uint32_t* x, int64_t batch, int log_k, int log_b, uint32_t h,
                     uint32_t* out, void* ws, size_t ws_bytes, cudaStream_t st,
                     int brev_out = 0) {
  if (!plan_lde(log_k, log_b).small && lde_wide(batch, log_k + log_b)) {
    const LdePlan pw = plan_lde(log_k, log_b, kWideTileLog, kWideRadixLog);
    if (pw.smem1 <= 227 * 1024 && pw.smem2 <= 227 * 1024)
      return lde_four_step<F, kWideRadixLog>(x, batch, log_k, log_b, h, out, ws, ws_bytes, st,
                                             brev_out, pw);
  }
  const LdePlan p = plan_lde(log_k, log_b);
  const int log_n = log_k + log_b;
  const size_t smem_cap = 227 * 1024;
  if ((p.small && p.smem_small > smem_cap) ||
      (!p.small && (p.smem1 > smem_cap || p.smem2 > smem_cap))) {
    set_error("LDE tile does not fit in shared memory (blowup too large for this size)");
    return ZC_UNSUPPORTED;
  }
  if (p.small) {
    ZC_CUDA(cudaFuncSetAttribute(k_lde_small<F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)p.smem_small));
    for (int64_t c0 = 0; c0 < batch; c0 += 0x7fffffff) {
      const int64_t cols = batch - c0 < 0x7fffffff ? batch - c0 : 0x7fffffff;
      k_lde_small<F><<<(unsigned)cols, kThreads, p.smem_small, st>>>(
          x + (c0 << log_k), out + (c0 << log_n), log_k, log_b, h, brev_out);
      ZC_TRY(launch_check());
    }
    return ZC_OK;
  }
  return lde_four_step<F, kMaxRadixLog>(x, batch, log_k, log_b, h, out, ws, ws_bytes, st,
                                        brev_out, p);
}

// The two four-step passes over column chunks that fit the workspace.
template <class F, int MR>
zc_status lde_four_step(const uint32_t* x, int64_t batch, int log_k, int log_b, uint32_t h,
                        uint32_t* out, void* ws, size_t ws_bytes, cudaStream_t st, int brev_out,
                        const LdePlan& p) {
  const int log_n = log_k + log_b;
  const size_t col_bytes = (size_t)4 << log_n;
  if (!ws || ws_bytes < col_bytes) {
    set_error("rs_encode workspace smaller than one column's LDE (4 * 2^(log_k+log_b) bytes)");
    return ZC_OOM;
  }
  if ((uintptr_t)ws % 16) return ZC_BAD_ARG;
  int64_t chunk = (int64_t)(ws_bytes / col_bytes);
  if (chunk > 65535) chunk = 65535;
  if (chunk > batch) chunk = batch;
  ZC_CUDA(cudaFuncSetAttribute(k_lde_pass1<F, MR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)p.smem1));
  ZC_CUDA(cudaFuncSetAttribute(k_lde_pass2<F, MR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)p.smem2));
  uint32_t* z = (uint32_t*)ws;
  for (int64_t c0 = 0; c0 < batch; c0 += chunk) {
    const int64_t cols = batch - c0 < chunk ? batch - c0 : chunk;
    dim3 g1(1u << log_b, 1u << (p.log_k1 - p.log_ti), (unsigned)cols);
    k_lde_pass1<F, MR><<<g1, lde_threads<MR>(), p.smem1, st>>>(x + (c0 << log_k), z, p.log_k1,
                                                               p.log_k2, log_b, p.log_ti, h);
    ZC_TRY(launch_check());
    dim3 g2(1u << (p.log_k2 - p.log_tt), (unsigned)cols);
    k_lde_pass2<F, MR><<<g2, lde_threads<MR>(), p.smem2, st>>>(z, out + (c0 << log_n), p.log_k1,
                                                               p.log_k2, log_b, p.log_tt,
                                                               brev_out);
    ZC_TRY(launch_check());
  }
  return ZC_OK;
}

// ------------------------------------------------------------ batched ----
// Many LDE jobs (matrices of different heights, widths and blowups) in two
// launches: phase A runs every single-pass column and every pass-1 tile of
// every job, phase B every pass-2 tile. The job table is a __grid_constant__
// kernel parameter; CTAs claim (job, tile) items from an atomic counter in the
// workspace, so large and small jobs share the machine.
constexpr int kMaxLdeJobs = 48;

struct LdeJobDev {
  const uint32_t* x;
  uint32_t* out;
  uint32_t* z;
  int64_t batch;
  uint32_t h;
  int8_t log_k, log_b, log_k1, log_k2, log_ti, log_tt, small, brev_out, max_r;
};

struct LdeBatch {
  int32_t njobs;
  int32_t phase;
  int64_t total;
  int64_t prefix[kMaxLdeJobs + 1];
  LdeJobDev job[kMaxLdeJobs];
};

__device__ __forceinline__ int find_job(const int64_t* prefix, int njobs, int64_t it) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= it) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <class F>
__global__ void __launch_bounds__(kThreads, 2) k_lde_batch(const __grid_constant__ LdeBatch B,
                                                        unsigned long long* counter) {
  extern __shared__ uint32_t sm[];
  __shared__ long long s_item;
  for (int done = 0; kItemsPerCta == 0 || done < kItemsPerCta; done++) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(counter, 1ull);
    __syncthreads();
    const int64_t it = s_item;
    if (it >= B.total) break;
    const int j = find_job(B.prefix, B.njobs, it);
    const LdeJobDev& J = B.job[j];
    const int64_t local = it - B.prefix[j];
    if (B.phase == 0 && J.small) {
      lde_small_body<F>(J.x, J.out, J.log_k, J.log_b, J.h, local, sm, J.brev_out, J.max_r);
    } else if (B.phase == 0) {
      const int b = 1 << J.log_b;
      const int64_t per_col = (int64_t)b << (J.log_k1 - J.log_ti);
      const int64_t c = local / per_col;
      const int r = (int)(local - c * per_col);
#if ZC_LDE_FUSED
      lde_pass1_fused<F>(J.x, J.z, J.log_k1, J.log_k2, J.log_b, J.log_ti, J.h, r & (b - 1),
                         r >> J.log_b, c, sm, J.max_r);
#else
      lde_pass1_body<F>(J.x, J.z, J.log_k1, J.log_k2, J.log_b, J.log_ti, J.h, r & (b - 1),
                        r >> J.log_b, c, sm, J.max_r);
#endif
    } else {
      const int64_t tiles = (int64_t)1 << (J.log_k2 - J.log_tt);
      const int64_t c = local / tiles;
#if ZC_LDE_FUSED
      lde_pass2_fused<F>(J.z, J.out, J.log_k1, J.log_k2, J.log_b, J.log_tt,
                         (int)(local - c * tiles), c, sm, J.brev_out, J.max_r);
#else
      lde_pass2_body<F>(J.z, J.out, J.log_k1, J.log_k2, J.log_b, J.log_tt,
                        (int)(local - c * tiles), c, sm, J.brev_out, J.max_r);
#endif
    }
    __syncthreads();  // the item's shared memory is free again
  }
}

inline size_t job_z_bytes(const zc_lde_job& j) {
  const LdePlan p = plan_lde(j.log_k, j.log_blowup, j.tile_log);
  return p.small ? 0 : (((size_t)j.batch * 4) << (j.log_k + j.log_blowup));
}

constexpr size_t kCounterBytes = 256;

template <class F>
zc_status lde_batch_wave(const zc_lde_job* jobs, int n, uint32_t* zbase, unsigned long long* ctr,
                         cudaStream_t st) {
  LdeBatch B;  // launch parameters (copied into the launch)
  memset(&B, 0, sizeof(B));
  B.njobs = n;
  size_t smem_a = 0, smem_b = 0;
  uint32_t* z = zbase;
  int64_t totA = 0, totB = 0;
  int64_t prefB[kMaxLdeJobs + 1];
  for (int i = 0; i < n; i++) {
    const zc_lde_job& j = jobs[i];
    const LdePlan p = plan_lde(j.log_k, j.log_blowup, j.tile_log,
                               j.radix_log ? j.radix_log : kMaxRadixLog);
    LdeJobDev& d = B.job[i];
    d.x = j.coeffs;
    d.out = j.out;
    d.batch = j.batch;
    d.h = j.shift_mont ? j.shift_mont : F::ONE;
    d.log_k = (int8_t)j.log_k;
    d.log_b = (int8_t)j.log_blowup;
    d.log_k1 = (int8_t)p.log_k1;
    d.log_k2 = (int8_t)p.log_k2;
    d.log_ti = (int8_t)p.log_ti;
    d.log_tt = (int8_t)p.log_tt;
    d.small = p.small ? 1 : 0;
    d.brev_out = j.bit_reversed ? 1 : 0;
    d.max_r = (int8_t)(j.radix_log ? j.radix_log : kMaxRadixLog);
    d.z = p.small ? nullptr : z;
    if (!p.small) z += ((size_t)j.batch) << (j.log_k + j.log_blowup);
    B.prefix[i] = totA;
    prefB[i] = totB;
    if (p.small) {
      totA += j.batch;
      smem_a = smem_a > p.smem_small ? smem_a : p.smem_small;
    } else {
      totA += (j.batch << j.log_blowup) << (p.log_k1 - p.log_ti);
      totB += j.batch << (p.log_k2 - p.log_tt);
      smem_a = smem_a > p.smem1 ? smem_a : p.smem1;
      smem_b = smem_b > p.smem2 ? smem_b : p.smem2;
    }
  }
  B.prefix[n] = totA;
  prefB[n] = totB;
  ZC_CUDA(cudaMemsetAsync(ctr, 0, 2 * sizeof(unsigned long long), st));
  for (int phase = 0; phase < 2; phase++) {
    const int64_t total = phase ? totB : totA;
    const size_t smem = phase ? smem_b : smem_a;
    if (total == 0) continue;
    B.phase = phase;
    B.total = total;
    if (phase) memcpy(B.prefix, prefB, sizeof(prefB));
    ZC_CUDA(cudaFuncSetAttribute(k_lde_batch<F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    int dev = 0, sms = 0, occ = 0;
    ZC_CUDA(cudaGetDevice(&dev));
    ZC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ZC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_lde_batch<F>, kThreads, smem));
    const int64_t grid = batch_grid(total, occ, sms);
    k_lde_batch<F><<<(unsigned)grid, kThreads, smem, st>>>(B, ctr + phase);
    ZC_TRY(launch_check());
  }
  return ZC_OK;
}

template <class F>
zc_status lde_batch_launch(const zc_lde_job* jobs, int njobs, void* ws, size_t ws_bytes,
                           cudaStream_t st) {
  if ((uintptr_t)ws % 256) return ZC_BAD_ARG;
  unsigned long long* ctr = (unsigned long long*)ws;
  uint32_t* zbase = (uint32_t*)((char*)ws + kCounterBytes);
  const size_t zcap = ws_bytes > kCounterBytes ? ws_bytes - kCounterBytes : 0;
  int i = 0;
  while (i < njobs) {
    // a job whose intermediate alone exceeds the workspace runs chunked, alone
    const size_t zi = job_z_bytes(jobs[i]);
    if (zi > zcap) {
      const zc_lde_job& j = jobs[i];
      ZC_TRY(lde_launch<F>(j.coeffs, j.batch, j.log_k, j.log_blowup,
                           j.shift_mont ? j.shift_mont : F::ONE, j.out, zbase, zcap, st,
                           j.bit_reversed ? 1 : 0));
      i++;
      continue;
    }
    int n = 0;
    size_t used = 0;
    while (i + n < njobs && n < kMaxLdeJobs) {
      const size_t zb = job_z_bytes(jobs[i + n]);
      if (zb > zcap) break;
      if (used + zb > zcap) break;
      used += zb;
      n++;
    }
    ZC_TRY(lde_batch_wave<F>(jobs + i, n, zbase, ctr, st));
    i += n;
  }
  return ZC_OK;
}

// ----------------------------------------------------- allocation-free --
// Scratch for zc_rs_encode_noalloc: the four-step intermediate of one chunk of
// columns lives in this fixed device array instead of a caller workspace. It is
// reserved when the library's device code is loaded on a GPU and held until the
// process exits, on every GPU that loads the library.
constexpr size_t kNoAllocScratchWords = (size_t)1 << 24;  // 64 MiB
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];

static std::mutex g_noalloc_mu;
static uint32_t* g_noalloc_ptr[64];

// The device address of the scratch array on the current device. In host code
// the symbol names a host-side stand-in, never a device address, so the
// address is fetched with cudaGetSymbolAddress once per device, with that
// device current, and cached.
static zc_status noalloc_scratch(uint32_t** out) {
  int dev = 0;
  ZC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return ZC_BAD_ARG;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e);
    g_noalloc_ptr[dev] = (uint32_t*)p;
  }
  *out = g_noalloc_ptr[dev];
  return ZC_OK;
}

}  // namespace zc

using namespace zc;

extern "C" {

size_t zc_rs_encode_workspace_bytes(int64_t batch, int log_k, int log_blowup) {
  if (batch <= 0 || log_k < 0 || log_blowup < 0) return 0;
  const LdePlan p = plan_lde(log_k, log_blowup);
  if (p.small) return 0;
  const size_t col = (size_t)4 << (log_k + log_blowup);
  size_t cols = (size_t)batch;
  const size_t cap = (size_t)1 << 30;  // 1 GiB of intermediate per chunk by default
  if (cols * col > cap) cols = cap / col ? cap / col : 1;
  return cols * col;
}

static zc_status rs_encode(zc_field field, const uint32_t* coeffs, int64_t batch, int log_k,
                           int log_blowup, uint32_t shift_mont, uint32_t generator, uint32_t* out,
                           void* workspace, size_t workspace_bytes, void* stream, int brev_out) {
  if (!coeffs || !out || batch < 0 || log_k < 0 || log_blowup < 0) return ZC_BAD_ARG;
  if (batch == 0) return ZC_OK;
  return with_field(field, [&](auto f) -> zc_status {
    using F = decltype(f);
    if (log_k + log_blowup > F::TWO_ADICITY || log_k > 24) {
      set_error("LDE size exceeds the supported two-adic range");
      return ZC_BAD_SHAPE;
    }
    if (generator != 0 && generator != F::GEN) {
      set_error("only the field's canonical generator is built");
      return ZC_UNSUPPORTED;
    }
    ZC_TRY(ensure_init());
    const uint32_t h = shift_mont ? shift_mont : F::ONE;
    return lde_launch<F>(coeffs, batch, log_k, log_blowup, h, out, workspace, workspace_bytes,
                         (cudaStream_t)stream, brev_out);
  });
}

zc_status zc_rs_encode(zc_field field, const uint32_t* coeffs, int64_t batch, int log_k,
                       int log_blowup, uint32_t shift_mont, uint32_t generator, uint32_t* out,
                       void* workspace, size_t workspace_bytes, void* stream) {
  return rs_encode(field, coeffs, batch, log_k, log_blowup, shift_mont, generator, out,
                   workspace, workspace_bytes, stream, 0);
}

zc_status zc_rs_encode_bitrev(zc_field field, const uint32_t* coeffs, int64_t batch, int log_k,
                              int log_blowup, uint32_t shift_mont, uint32_t generator,
                              uint32_t* out, void* workspace, size_t workspace_bytes,
                              void* stream) {
  return rs_encode(field, coeffs, batch, log_k, log_blowup, shift_mont, generator, out,
                   workspace, workspace_bytes, stream, 1);
}

zc_status zc_rs_encode_noalloc(zc_field field, const uint32_t* coeffs, int64_t batch, int log_k,
                               int log_blowup, uint32_t shift_mont, uint32_t generator,
                               uint32_t* out, void* stream) {
  if (!coeffs || !out || batch < 0 || log_k < 0 || log_blowup < 0) return ZC_BAD_ARG;
  if (batch == 0) return ZC_OK;
  return with_field(field, [&](auto f) -> zc_status {
    using F = decltype(f);
    if (log_k + log_blowup > F::TWO_ADICITY || log_k > 24) {
      set_error("LDE size exceeds the supported two-adic range");
      return ZC_BAD_SHAPE;
    }
    if (generator != 0 && generator != F::GEN) {
      set_error("only the field's canonical generator is built");
      return ZC_UNSUPPORTED;
    }
    const LdePlan p = plan_lde(log_k, log_blowup);
    if (!p.small && (((size_t)1) << (log_k + log_blowup)) > kNoAllocScratchWords) {
      set_error("zc_rs_encode_noalloc: one column's LDE (2^(log_k+log_blowup) words) exceeds "
                "the 2^24-word (64 MiB) fixed scratch; use zc_rs_encode with a workspace");
      return ZC_BAD_SHAPE;
    }
    ZC_TRY(ensure_init());
    uint32_t* scratch = nullptr;
    ZC_TRY(noalloc_scratch(&scratch));
    const uint32_t h = shift_mont ? shift_mont : F::ONE;
    return lde_launch<F>(coeffs, batch, log_k, log_blowup, h, out, scratch,
                         kNoAllocScratchWords * 4, (cudaStream_t)stream);
  });
}

size_t zc_rs_encode_batch_workspace_bytes(const zc_lde_job* jobs, int32_t njobs) {
  if (!jobs || njobs <= 0) return kCounterBytes;
  size_t z = 0;
  for (int i = 0; i < njobs; i++) z += job_z_bytes(jobs[i]);
  const size_t cap = (size_t)8 << 30;  // waves bound the intermediate at 8 GiB by default
  size_t biggest = 0;
  for (int i = 0; i < njobs; i++) {
    const size_t zi = job_z_bytes(jobs[i]);
    biggest = zi > biggest ? zi : biggest;
  }
  if (z > cap) z = biggest > cap ? biggest : cap;
  return kCounterBytes + z;
}

zc_status zc_rs_encode_batch(zc_field field, const zc_lde_job* jobs, int32_t njobs,
                             uint32_t generator, void* workspace, size_t workspace_bytes,
                             void* stream) {
  if (njobs < 0 || (njobs > 0 && !jobs) || !workspace) return ZC_BAD_ARG;
  if (njobs == 0) return ZC_OK;
  return with_field(field, [&](auto f) -> zc_status {
    using F = decltype(f);
    if (generator != 0 && generator != F::GEN) {
      set_error("only the field's canonical generator is built");
      return ZC_UNSUPPORTED;
    }
    for (int i = 0; i < njobs; i++) {
      const zc_lde_job& j = jobs[i];
      if (!j.coeffs || !j.out || j.batch < 0 || j.log_k < 0 || j.log_blowup < 0) return ZC_BAD_ARG;
      if (j.radix_log != 0 && (j.radix_log < 2 || j.radix_log > kMaxRadixLog)) {
        set_error("radix_log must be 0 (default) or 2..4");
        return ZC_BAD_ARG;
      }
      if (j.log_k + j.log_blowup > F::TWO_ADICITY || j.log_k > 24) return ZC_BAD_SHAPE;
      const LdePlan p = plan_lde(j.log_k, j.log_blowup, j.tile_log,
                                 j.radix_log ? j.radix_log : kMaxRadixLog);
      const size_t cap = 227 * 1024;
      if ((p.small && p.smem_small > cap) || (!p.small && (p.smem1 > cap || p.smem2 > cap)))
        return ZC_UNSUPPORTED;
    }
    ZC_TRY(ensure_init());
    return lde_batch_launch<F>(jobs, njobs, workspace, workspace_bytes, (cudaStream_t)stream);
  });
}

}  // extern "C"
