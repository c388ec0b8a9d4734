// Status/error plumbing, per-device init, Poseidon2 handles, the batched
// permutation and the Fiat-Shamir duplex (device and host forms).
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>

#include <type_traits>

#include "duplex.cuh"
#include "internal.cuh"

namespace zc {

static thread_local char g_err[512] = "";

void set_error(const char* msg) {
  strncpy(g_err, msg, sizeof(g_err) - 1);
  g_err[sizeof(g_err) - 1] = 0;
}

zc_status cuda_fail(cudaError_t e) {
  snprintf(g_err, sizeof(g_err), "CUDA error %d: %s", (int)e, cudaGetErrorString(e));
  return ZC_CUDA_ERR;
}

static std::atomic<unsigned long long> g_launches{0};

zc_status launch_check() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ZC_OK : cuda_fail(e);
}

zc_status init_root_tables();  // zc_ntt.cu

static std::mutex g_init_mu;
static bool g_init_done[64];

zc_status ensure_init() {
  int dev = 0;
  ZC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return ZC_BAD_ARG;
  std::lock_guard<std::mutex> lock(g_init_mu);
  if (g_init_done[dev]) return ZC_OK;
  ZC_TRY(init_root_tables());
  ZC_CUDA(cudaDeviceSynchronize());  // tables visible to every stream afterwards
  g_init_done[dev] = true;
  return ZC_OK;
}

// Calls fn(perm) with the transcript's half-warp permutation: the unrolled
// built-in form for the built-in instance, the run-time form (constants
// staged to shared memory) otherwise.
template <class K, class Fn>
__device__ __forceinline__ void with_half_perm(const P2Params* rt, P2Params* s_rt, Fn&& fn) {
  if constexpr (std::is_same<K, Bb16Builtin>::value) {
    const HalfPermBb16 perm;
    fn(perm);
  } else {
    KIn<K>::make(rt, s_rt);
    const HalfPerm<typename K::F> perm{KIn<K>::half(rt, s_rt)};
    fn(perm);
  }
}

// One warp; lane 0 writes the results.
template <class K>
__global__ void __launch_bounds__(32) k_duplex_step(const P2Params* rt, uint32_t* state,
                                                    const uint32_t* values, int64_t m, int n,
                                                    uint32_t* out, int32_t* positions,
                                                    int64_t block_len) {
  __shared__ P2Params s_rt;
  with_half_perm<K>(rt, &s_rt, [&](const auto& perm) {
    Duplex t;
    memcpy(&t, state, sizeof(Duplex));
    duplex_observe(t, values, m, perm);
    for (int i = 0; i < n; i++) {
      uint32_t w;
      duplex_sample(t, 1, &w, perm);
      if (threadIdx.x == 0) {
        if (out) out[i] = w;
        if (positions) positions[i] = (int32_t)(w % (uint32_t)block_len);
      }
    }
    __syncwarp();
    if (threadIdx.x == 0) memcpy(state, &t, sizeof(Duplex));
  });
}

template <class K>
__global__ void __launch_bounds__(32) k_duplex_hop(
    const P2Params* rt, const uint32_t* in_buf, const uint32_t* out_buf, const uint32_t* sponge,
    const uint32_t* in_pos, const uint32_t* out_pos, const uint32_t* values, int64_t m, int n,
    uint32_t* in_buf_o, uint32_t* out_buf_o, uint32_t* sponge_o, uint32_t* in_pos_o,
    uint32_t* out_pos_o, uint32_t* chal) {
  __shared__ P2Params s_rt;
  with_half_perm<K>(rt, &s_rt, [&](const auto& perm) {
    Duplex t;
    for (int j = 0; j < 8; j++) {
      t.in_buf[j] = in_buf[j];
      t.out_buf[j] = out_buf[j];
    }
    for (int j = 0; j < 16; j++) t.sponge[j] = sponge[j];
    t.in_pos = (int32_t)in_pos[0];
    t.out_pos = (int32_t)out_pos[0];
    duplex_observe(t, values, m, perm);
    for (int i = 0; i < n; i++) {
      uint32_t w;
      duplex_sample(t, 1, &w, perm);
      if (threadIdx.x == 0) chal[i] = w;
    }
    // inputs may alias outputs: every lane has read them by now
    __syncwarp();
    if (threadIdx.x != 0) return;
    for (int j = 0; j < 8; j++) {
      in_buf_o[j] = t.in_buf[j];
      out_buf_o[j] = t.out_buf[j];
    }
    for (int j = 0; j < 16; j++) sponge_o[j] = t.sponge[j];
    in_pos_o[0] = (uint32_t)t.in_pos;
    out_pos_o[0] = (uint32_t)t.out_pos;
  });
}

template <class F>
__global__ void k_convert(const uint32_t* in, uint32_t* out, int64_t n, int to) {
  // 16-byte accesses when both sides are aligned (more bytes in flight per
  // thread, which a read of page-locked host memory over the host link needs)
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t head = 0;
  if (((uintptr_t)in % 16) == 0 && ((uintptr_t)out % 16) == 0) {
    const int64_t n4 = n >> 2;
    const uint4* in4 = reinterpret_cast<const uint4*>(in);
    uint4* out4 = reinterpret_cast<uint4*>(out);
    for (int64_t i = tid; i < n4; i += stride) {
      const uint4 v = in4[i];
      out4[i] = to ? make_uint4(to_mont<F>(v.x), to_mont<F>(v.y), to_mont<F>(v.z), to_mont<F>(v.w))
                   : make_uint4(from_mont<F>(v.x), from_mont<F>(v.y), from_mont<F>(v.z),
                                from_mont<F>(v.w));
    }
    head = n4 << 2;
  }
  for (int64_t i = head + tid; i < n; i += stride)
    out[i] = to ? to_mont<F>(in[i]) : from_mont<F>(in[i]);
}

template <class F>
__global__ void k_scale(const uint32_t* in, uint32_t* out, int64_t n, uint32_t s) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = mmul<F>(in[i], s);
}

template <class K>
__global__ void k_permute(const P2Params* rt, uint32_t* states, int64_t count) {
  __shared__ P2Params s_rt;
  K k = KIn<K>::make(rt, &s_rt);
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint32_t s[16];
  for (int j = 0; j < 16; j++) s[j] = states[i * 16 + j];
  p2_permute(s, k);
  for (int j = 0; j < 16; j++) states[i * 16 + j] = s[j];
}

// ------------------------------------------------------------- grind ------
// Proof-of-work search (DuplexTranscript._grind_search, zorch/transcript.py:
// 439-459, over grind_search, zorch/grind.py:66-93): the lowest witness w in
// [0, p) whose challenge -- observe w as a field element, sample once -- has
// `mask` clear in its canonical value. Observing one word and sampling once
// is always exactly one permutation: of the sponge with the pending prefix
// in_buf[0:in_pos] and then w written over its front, and the challenge is
// lane 7 of the result (a completed block is absorbed and lane 7 popped; a
// partial one is duplexed and lane 7 popped). One thread per candidate on a
// persistent grid: thread i tries i, i + S, i + 2S, ... and stops once its
// candidate exceeds the best hit so far, so every witness below the final
// minimum is tried and the result is the same for every grid size.
constexpr int kGrindT = 256;

template <class K>
__global__ void __launch_bounds__(kGrindT) k_grind(const P2Params* rt, const uint32_t* state,
                                                  uint32_t mask, uint32_t* best) {
  using F = typename K::F;
  __shared__ P2Params s_rt;
  K k = KIn<K>::make(rt, &s_rt);
  const Duplex* t = reinterpret_cast<const Duplex*>(state);
  const int in_pos = t->in_pos & 7;
  uint32_t base[16];
#pragma unroll
  for (int j = 0; j < 16; j++) base[j] = (j < 8 && j < in_pos) ? t->in_buf[j] : t->sponge[j];
  const uint32_t stride = gridDim.x * blockDim.x;
  const volatile uint32_t* vbest = best;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < F::P; c += stride) {
    if (c > *vbest) break;
    const uint32_t w = to_mont<F>(c);
    uint32_t s[16];
#pragma unroll
    for (int j = 0; j < 16; j++) s[j] = j == in_pos ? w : base[j];
    p2_permute(s, k);
    if ((from_mont<F>(s[7]) & mask) == 0) atomicMin(best, c);
  }
}

// The witness as a field element (Montgomery), 0 when no candidate passed.
template <class F>
__global__ void k_grind_finish(uint32_t* best) {
  const uint32_t c = best[0];
  best[0] = c == 0xffffffffu ? 0u : to_mont<F>(c);
}

}  // namespace zc

using namespace zc;

extern "C" {

const char* zc_status_str(zc_status s) {
  switch (s) {
    case ZC_OK: return "ok";
    case ZC_BAD_SHAPE: return "bad shape";
    case ZC_NOT_POW2: return "size is not a power of two";
    case ZC_OOB_INDEX: return "index out of range";
    case ZC_OOM: return "workspace too small or out of memory";
    case ZC_TIMEOUT: return "device wait timed out";
    case ZC_CUDA_ERR: return "CUDA error";
    case ZC_BAD_ARG: return "bad argument";
    case ZC_UNSUPPORTED: return "unsupported configuration";
  }
  return "unknown status";
}

const char* zc_last_error(void) { return g_err; }
unsigned long long zc_launch_count(void) { return g_launches.load(); }
int zc_version(void) { return 1; }

zc_status zc_init(int device) {
  if (device >= 0) ZC_CUDA(cudaSetDevice(device));
  ZC_TRY(ensure_init());
  ZC_CUDA(cudaDeviceSynchronize());
  return ZC_OK;
}

// Whether this process can use a CUDA device at all (checked once).
static bool have_device() {
  static const bool have = [] {
    int n = 0;
    const bool ok = cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
    cudaGetLastError();  // clear the error a failed query recorded
    return ok;
  }();
  return have;
}

// Device copy of the constants; without any CUDA device the handle stays
// host-only (dev == nullptr): the host permutation, sponge, compression and
// duplex hop work, every device entry refuses it (with_perm).
static zc_status upload_params(zc_poseidon2* h) {
  h->dev = nullptr;
  if (!have_device()) return ZC_OK;
  ZC_CUDA(cudaMalloc((void**)&h->dev, sizeof(P2Params)));
  ZC_CUDA(cudaMemcpy(h->dev, &h->host, sizeof(P2Params), cudaMemcpyHostToDevice));
  return ZC_OK;
}

zc_status zc_poseidon2_builtin(zc_field field, const zc_poseidon2** out) {
  if (!out) return ZC_BAD_ARG;
  if (field != ZC_FIELD_BABYBEAR) {
    set_error("no built-in Poseidon2 instance for this field; create one with zc_poseidon2_create");
    return ZC_UNSUPPORTED;
  }
  static std::mutex mu;
  static zc_poseidon2* inst[64] = {};
  int dev = 0;  // slot 0 serves the host-only instance of a machine without a GPU
  if (have_device()) ZC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return ZC_BAD_ARG;
  std::lock_guard<std::mutex> lock(mu);
  if (!inst[dev]) {
    zc_poseidon2* h = new zc_poseidon2();
    memset(&h->host, 0, sizeof(h->host));
    h->field = ZC_FIELD_BABYBEAR;
    h->builtin = 1;
    const uint32_t ei[64] = ZC_BB16_EXT_INIT_MONT_INIT, et[64] = ZC_BB16_EXT_TERM_MONT_INIT;
    const uint32_t ir[ZC_BB16_ROUNDS_P] = ZC_BB16_INT_RC_MONT_INIT, dg[16] = ZC_BB16_DIAG_MONT_INIT;
    h->host.field_id = 0;
    h->host.alpha = ZC_BB16_ALPHA;
    h->host.rounds_f_half = ZC_BB16_ROUNDS_F_HALF;
    h->host.rounds_p = ZC_BB16_ROUNDS_P;
    memcpy(h->host.ext_init, ei, sizeof(ei));
    memcpy(h->host.ext_term, et, sizeof(et));
    memcpy(h->host.int_rc, ir, sizeof(ir));
    memcpy(h->host.diag, dg, sizeof(dg));
    h->host.j_scale = BabyBear::ONE;
    h->host.j_is_one = 1;
    zc_status s = upload_params(h);
    if (s != ZC_OK) {
      delete h;
      return s;
    }
    inst[dev] = h;
  }
  *out = inst[dev];
  return ZC_OK;
}

zc_status zc_poseidon2_create(zc_field field, int alpha, int rounds_f_half, int rounds_p,
                              const uint32_t* ext_init, const uint32_t* ext_term,
                              const uint32_t* int_rc, const uint32_t* diag, uint32_t j_scale,
                              zc_poseidon2** out) {
  if (!out || !ext_init || !ext_term || !int_rc || !diag) return ZC_BAD_ARG;
  if (field != ZC_FIELD_BABYBEAR && field != ZC_FIELD_KOALABEAR) return ZC_BAD_ARG;
  if (rounds_f_half < 0 || rounds_f_half > 8 || rounds_p < 0 || rounds_p > 64 || alpha < 2) {
    set_error("Poseidon2 shape out of range (rounds_f_half <= 8, rounds_p <= 64)");
    return ZC_UNSUPPORTED;
  }
  zc_poseidon2* h = new zc_poseidon2();
  memset(&h->host, 0, sizeof(h->host));
  h->field = field;
  h->builtin = 0;
  auto conv = [&](uint32_t x) {
    return field == ZC_FIELD_BABYBEAR ? to_mont<BabyBear>(x) : to_mont<KoalaBear>(x);
  };
  h->host.field_id = (uint32_t)field;
  h->host.alpha = (uint32_t)alpha;
  h->host.rounds_f_half = (uint32_t)rounds_f_half;
  h->host.rounds_p = (uint32_t)rounds_p;
  for (int r = 0; r < rounds_f_half; r++)
    for (int i = 0; i < 16; i++) {
      h->host.ext_init[r][i] = conv(ext_init[r * 16 + i]);
      h->host.ext_term[r][i] = conv(ext_term[r * 16 + i]);
    }
  for (int r = 0; r < rounds_p; r++) h->host.int_rc[r] = conv(int_rc[r]);
  for (int i = 0; i < 16; i++) h->host.diag[i] = conv(diag[i]);
  h->host.j_scale = conv(j_scale);
  h->host.j_is_one = (j_scale == 1);
  zc_status s = upload_params(h);
  if (s != ZC_OK) {
    delete h;
    return s;
  }
  *out = h;
  return ZC_OK;
}

zc_status zc_poseidon2_destroy(zc_poseidon2* p) {
  if (!p || p->builtin) return ZC_BAD_ARG;
  if (p->dev) cudaFree(p->dev);
  delete p;
  return ZC_OK;
}

zc_status zc_poseidon2_permute(const zc_poseidon2* p, uint32_t* states, int64_t count,
                               void* stream) {
  if (!states || count < 0) return ZC_BAD_ARG;
  if (count == 0) return ZC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    int64_t blocks = (count + 127) / 128;
    k_permute<K><<<(unsigned)blocks, 128, 0, st>>>(rt, states, count);
    return launch_check();
  });
}

// CTAs of 1024 threads for a conversion that reads page-locked host memory.
constexpr int64_t kHostReadCtas = 64;

static zc_status convert(zc_field field, const uint32_t* in, uint32_t* out, int64_t n, int to,
                         void* stream) {
  if (!in || !out || n < 0) return ZC_BAD_ARG;
  if (n == 0) return ZC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_convert<F><<<(unsigned)blocks, 256, 0, st>>>(in, out, n, to);
    return launch_check();
  });
}

zc_status zc_to_mont_from_host(zc_field field, const void* host, uint32_t* out, int64_t n,
                               int32_t max_ctas, void* stream) {
  if (!host || !out || n < 0) return ZC_BAD_ARG;
  if (n == 0) return ZC_OK;
  void* src = nullptr;
  ZC_TRY(zc_host_device_ptr(host, &src));
  cudaStream_t st = (cudaStream_t)stream;
  // a bounded number of CTAs: the host link, not the SM count, limits this
  // kernel, and the SMs it leaves free keep running the other streams' work
  const int64_t cap = max_ctas > 0 ? max_ctas : kHostReadCtas;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    int64_t blocks = (n + 1023) / 1024;
    if (blocks > cap) blocks = cap;
    k_convert<F><<<(unsigned)blocks, 1024, 0, st>>>(static_cast<const uint32_t*>(src), out, n, 1);
    return launch_check();
  });
}

zc_status zc_host_device_ptr(const void* host, void** dev) {
  if (!host || !dev) return ZC_BAD_ARG;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess || a.type != cudaMemoryTypeHost) {
    cudaGetLastError();  // clear the error the failed query recorded
    set_error("not page-locked host memory");
    return ZC_BAD_ARG;
  }
  void* d = nullptr;
  const cudaError_t e = cudaHostGetDevicePointer(&d, const_cast<void*>(host), 0);
  if (e != cudaSuccess) return cuda_fail(e);
  *dev = d;
  return ZC_OK;
}

zc_status zc_to_mont(zc_field field, const uint32_t* in, uint32_t* out, int64_t n, void* stream) {
  return convert(field, in, out, n, 1, stream);
}

zc_status zc_from_mont(zc_field field, const uint32_t* in, uint32_t* out, int64_t n,
                       void* stream) {
  return convert(field, in, out, n, 0, stream);
}

zc_status zc_poseidon2_permute_host(const zc_poseidon2* p, uint32_t* states, int64_t count) {
  if (!p || (!states && count > 0) || count < 0) return ZC_BAD_ARG;
  for (int64_t i = 0; i < count; i++) {
    if (p->field == ZC_FIELD_BABYBEAR)
      p2_permute(states + 16 * i, RtParams<BabyBear>{&p->host});
    else
      p2_permute(states + 16 * i, RtParams<KoalaBear>{&p->host});
  }
  return ZC_OK;
}

zc_status zc_scale(zc_field field, const uint32_t* in, uint32_t* out, int64_t n, uint32_t s_mont,
                   void* stream) {
  if (!in || !out || n < 0) return ZC_BAD_ARG;
  if (n == 0) return ZC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  return with_field(field, [&](auto f) {
    using F = decltype(f);
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_scale<F><<<(unsigned)blocks, 256, 0, st>>>(in, out, n, s_mont);
    return launch_check();
  });
}

zc_status zc_duplex_step(const zc_poseidon2* p, uint32_t* state, const uint32_t* values,
                         int64_t m, int32_t n, uint32_t* out, int32_t* positions,
                         int64_t block_len, void* stream) {
  if (!state || m < 0 || n < 0 || (m > 0 && !values)) return ZC_BAD_ARG;
  if (positions && (block_len <= 0 || block_len > 0xffffffffLL)) return ZC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    k_duplex_step<K><<<1, 32, 0, st>>>(rt, state, values, m, n, out, positions, block_len);
    return launch_check();
  });
}

zc_status zc_duplex_grind(const zc_poseidon2* p, const uint32_t* state, int32_t pow_bits,
                          uint32_t* witness, void* stream) {
  if (!p || !state || !witness) return ZC_BAD_ARG;
  if (pow_bits < 0 || pow_bits >= 32) {
    set_error("pow_bits must be in [0, 32)");
    return ZC_BAD_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (pow_bits == 0) {  // the canonical zero witness always passes
    ZC_CUDA(cudaMemsetAsync(witness, 0, 4, st));
    return ZC_OK;
  }
  ZC_CUDA(cudaMemsetAsync(witness, 0xff, 4, st));
  // about two expected hits' worth of candidates per sweep, at most one full
  // wave of resident threads (grind_window_for, zorch/grind.py:33-47)
  const int64_t want = std::min<int64_t>(int64_t(1) << (pow_bits + 1), 152 * 2048);
  const unsigned blocks = (unsigned)std::max<int64_t>(4, (want + kGrindT - 1) / kGrindT);
  const uint32_t mask = (uint32_t)((1ull << pow_bits) - 1);
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    k_grind<K><<<blocks, kGrindT, 0, st>>>(rt, state, mask, witness);
    ZC_TRY(launch_check());
    k_grind_finish<typename K::F><<<1, 1, 0, st>>>(witness);
    return launch_check();
  });
}

zc_status zc_duplex_hop(const zc_poseidon2* p, const uint32_t* in_buf, const uint32_t* out_buf,
                        const uint32_t* sponge, const uint32_t* in_pos, const uint32_t* out_pos,
                        const uint32_t* values, int64_t m, int32_t n, uint32_t* in_buf_o,
                        uint32_t* out_buf_o, uint32_t* sponge_o, uint32_t* in_pos_o,
                        uint32_t* out_pos_o, uint32_t* challenges, void* stream) {
  if (!in_buf || !out_buf || !sponge || !in_pos || !out_pos || !in_buf_o || !out_buf_o ||
      !sponge_o || !in_pos_o || !out_pos_o || m < 0 || n < 0 || (m > 0 && !values) ||
      (n > 0 && !challenges))
    return ZC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  return with_perm(p, [&](auto k, const P2Params* rt) {
    using K = decltype(k);
    k_duplex_hop<K><<<1, 32, 0, st>>>(rt, in_buf, out_buf, sponge, in_pos, out_pos, values, m,
                                      n, in_buf_o, out_buf_o, sponge_o, in_pos_o, out_pos_o,
                                      challenges);
    return launch_check();
  });
}

zc_status zc_duplex_hop_host(const zc_poseidon2* p, const uint32_t* in_buf,
                             const uint32_t* out_buf, const uint32_t* sponge,
                             const uint32_t* in_pos, const uint32_t* out_pos,
                             const uint32_t* values, int64_t m, int32_t n, uint32_t* in_buf_o,
                             uint32_t* out_buf_o, uint32_t* sponge_o, uint32_t* in_pos_o,
                             uint32_t* out_pos_o, uint32_t* challenges) {
  if (!p || !in_buf || !out_buf || !sponge || !in_pos || !out_pos || !in_buf_o || !out_buf_o ||
      !sponge_o || !in_pos_o || !out_pos_o || m < 0 || n < 0 || (m > 0 && !values) ||
      (n > 0 && !challenges))
    return ZC_BAD_ARG;
  Duplex t;
  memcpy(t.in_buf, in_buf, 32);
  memcpy(t.out_buf, out_buf, 32);
  memcpy(t.sponge, sponge, 64);
  t.in_pos = (int32_t)in_pos[0];
  t.out_pos = (int32_t)out_pos[0];
  if (t.in_pos < 0 || t.in_pos >= 8 || t.out_pos < 0 || t.out_pos > 8) return ZC_BAD_ARG;
  if (p->field == ZC_FIELD_BABYBEAR) {
    const RtParams<BabyBear> k{&p->host};
    const HostPerm<RtParams<BabyBear>> perm{k};
    duplex_observe(t, values, m, perm);
    duplex_sample(t, n, challenges, perm);
  } else {
    const RtParams<KoalaBear> k{&p->host};
    const HostPerm<RtParams<KoalaBear>> perm{k};
    duplex_observe(t, values, m, perm);
    duplex_sample(t, n, challenges, perm);
  }
  memcpy(in_buf_o, t.in_buf, 32);
  memcpy(out_buf_o, t.out_buf, 32);
  memcpy(sponge_o, t.sponge, 64);
  in_pos_o[0] = (uint32_t)t.in_pos;
  out_pos_o[0] = (uint32_t)t.out_pos;
  return ZC_OK;
}

}  // extern "C"
