// The FRI folds in natural order -- binary and k-ary -- and the fold of round
// r fused with the pair-leaf commit of round r+1 (and, optionally, round r+1's
// transcript hop in the root's launch).
#include "fold.cuh"

using namespace zc;

extern "C" {

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

zc_status zc_fri_fold_commit_hop(const zc_poseidon2* p, const uint32_t* cw, int64_t n, int ef_in,
                                 const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                                 uint32_t generator, int32_t bit_reversed, uint32_t* out,
                                 uint32_t* next_layers, uint32_t* state, int32_t n_chal,
                                 uint32_t* chal, void* stream) {
  if (!cw || !beta || !out || !next_layers) return ZC_BAD_ARG;
  if (!is_pow2(n) || n < 4) {
    set_error("fri_fold_commit requires a power-of-two codeword of length >= 4");
    return ZC_NOT_POW2;
  }
  if ((uintptr_t)next_layers % 16) return ZC_BAD_ARG;
  ZC_TRY(check_hop(state, n_chal, chal));
  const RootHop hop{state, chal, n_chal};
  cudaStream_t st = (cudaStream_t)stream;
  return bit_reversed ? fold_commit_bitrev(p, cw, n, ef_in, beta, ef_beta, shift_mont,
                                           generator, out, next_layers, st, hop)
                      : fold_commit_any<false>(p, cw, n, ef_in, beta, ef_beta, shift_mont,
                                               generator, out, next_layers, st, hop);
}

}  // extern "C"
