// Library-internal declarations shared by the translation units.
#pragma once
#include "common.cuh"
#include "poseidon2.cuh"

struct zc_poseidon2 {
  zc::P2Params host;     // Montgomery constants, host copy (host-side duplex hop)
  zc::P2Params* dev;     // device copy (run-time-parameter kernels)
  zc_field field;
  int builtin;           // 1: kernels use the compile-time BabyBear-16 instance
};

namespace zc {

// Builds the per-thread constant provider inside a kernel. Run-time params are
// staged into shared memory by the whole block (every thread must call make).
template <class K>
struct KIn;
template <>
struct KIn<Bb16Builtin> {
  __device__ static Bb16Builtin make(const P2Params*, P2Params*) { return {}; }
  // The half-warp permutation reads P2Params from shared memory: stage them.
  __device__ static const P2Params* half(const P2Params* g, P2Params* s) {
    stage_params(s, g);
    return s;
  }
};
template <class F>
struct KIn<RtParams<F>> {
  __device__ static RtParams<F> make(const P2Params* g, P2Params* s) {
    stage_params(s, g);
    return RtParams<F>{s};
  }
  // Already staged by make (same shared copy).
  __device__ static const P2Params* half(const P2Params*, P2Params* s) { return s; }
};

// Calls fn(K{}, device_params) with the provider matching the handle.
void set_error(const char* msg);

template <class Fn>
zc_status with_perm(const zc_poseidon2* p, Fn&& fn) {
  if (!p) return ZC_BAD_ARG;
  if (!p->dev) {
    set_error("Poseidon2 handle has no device copy (created without a CUDA device)");
    return ZC_BAD_ARG;
  }
  if (p->builtin) return fn(Bb16Builtin{}, p->dev);
  if (p->field == ZC_FIELD_BABYBEAR) return fn(RtParams<BabyBear>{}, p->dev);
  return fn(RtParams<KoalaBear>{}, p->dev);
}

template <class Fn>
zc_status with_field(zc_field f, Fn&& fn) {
  if (f == ZC_FIELD_BABYBEAR) return fn(BabyBear{});
  if (f == ZC_FIELD_KOALABEAR) return fn(KoalaBear{});
  return ZC_BAD_ARG;
}

zc_status ensure_init();

}  // namespace zc
