// The FRI fold of bit-reversed layers (BitReversedReedSolomon.fold,
// zorch/coding/reed_solomon.py:484-492, 532-540) and its fused
// fold-and-commit, in a unit of their own so they compile in parallel with
// the natural-order forms.
#include "fold.cuh"

namespace zc {

zc_status fold_commit_bitrev(const zc_poseidon2* p, const uint32_t* cw, int64_t n, int ef_in,
                             const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                             uint32_t generator, uint32_t* out, uint32_t* layers, cudaStream_t st,
                             RootHop hop) {
  return fold_commit_any<true>(p, cw, n, ef_in, beta, ef_beta, shift_mont, generator, out, layers,
                               st, hop);
}

}  // namespace zc

using namespace zc;

extern "C" {

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

}  // extern "C"
