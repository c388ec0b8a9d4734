/*
 * CPU ORACLE -- test infrastructure only. A plain-C restatement of the
 * reference commit path (fractalyze/zorch) used to check the CUDA kernels bit for
 * bit. Nothing in the product links or calls this library; only the tests, the
 * smoke check and the bench's CPU-baseline leg do.
 *
 * Parity status: the Poseidon2 / sponge / compression / Merkle semantics are
 * pinned to the reference's Plonky3 KoalaBear-16 golden root
 * (zorch/commit/testing/merkle_test.py:51-63). The BabyBear Poseidon2 instance
 * is project-defined (the reference ships none), so BabyBear roots, paths,
 * challenges and proof bytes are "parity unpinned vs reference" -- pinned only
 * between this oracle and the CUDA path. NTT / fold semantics are pinned
 * relationally (Horner on the recovered domain, fold/encode commute), as the
 * reference's own tests do (zorch/coding/testing/reed_solomon_test.py:48-99).
 *
 * Representation: every field value crossing this API is a Montgomery u32
 * (x * 2^32 mod p), the storage form of zk_dtypes' *_mont dtypes and the wire
 * form of the reference's FS FFI contract (zorch/transcript.py:986-999).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BABYBEAR = 0, ORC_KOALABEAR = 1 };

typedef struct {
  int field;
  int alpha;
  int rounds_f_half;
  int rounds_p;
  uint32_t ext_init[8][16]; /* Montgomery */
  uint32_t ext_term[8][16];
  uint32_t int_rc[64];
  uint32_t diag[16];
  uint32_t j_scale;
} orc_p2;

typedef struct {
  uint32_t in_buf[8];
  uint32_t out_buf[8];
  uint32_t sponge[16];
  int32_t in_pos;
  int32_t out_pos;
} orc_duplex;

/* threads used by the OpenMP loops (<= 0: library default) */
void orc_set_threads(int n);
int orc_get_threads(void);

/* field helpers */
uint32_t orc_modulus(int field);
uint32_t orc_to_mont(int field, uint32_t x);
uint32_t orc_from_mont(int field, uint32_t x);
void orc_to_mont_vec(int field, const uint32_t* in, uint32_t* out, int64_t n);
void orc_from_mont_vec(int field, const uint32_t* in, uint32_t* out, int64_t n);
uint32_t orc_mul(int field, uint32_t a, uint32_t b);
void orc_ef4_mul(int field, const uint32_t* a, const uint32_t* b, uint32_t* out);
uint32_t orc_root_of_unity(int field, int log_n, uint32_t generator_canon);

/* Poseidon2 width 16 */
int orc_p2_size(void);
void orc_p2_babybear16(orc_p2* out);
void orc_p2_from_canonical(orc_p2* out, int field, int alpha, int rounds_f_half,
                           int rounds_p, const uint32_t* ext_init,
                           const uint32_t* ext_term, const uint32_t* int_rc,
                           const uint32_t* diag, uint32_t j_scale);
void orc_p2_export_canonical(const orc_p2* p, uint32_t* ext_init, uint32_t* ext_term,
                             uint32_t* int_rc, uint32_t* diag);
void orc_p2_permute(const orc_p2* p, uint32_t* state);

/* sponge / compression (Plonky3 PaddingFreeSponge<16,8,8>, TruncatedPermutation<2,8,16>) */
void orc_sponge_hash(const orc_p2* p, const uint32_t* in, int64_t m, uint32_t* out8);
void orc_compress(const orc_p2* p, const uint32_t* l8, const uint32_t* r8, uint32_t* out8);

/* Merkle (arity 2). Leaf p = concat over q < groups of base[q*gstride + p*g .. +g].
 * layers: (2L-1)*8 words, leaf digests first, root last. */
int orc_merkle_commit(const orc_p2* p, const uint32_t* base, int64_t num_leaves,
                      int groups, int g, int64_t gstride, uint32_t* layers);
int orc_merkle_open(const uint32_t* base, int64_t num_leaves, int groups, int g,
                    int64_t gstride, const uint32_t* layers, const int32_t* idx,
                    int q, uint32_t* rows, uint32_t* paths);

/* Query-strided Merkle tree (rows_per_query rows per query-layer node). */
int orc_strided_merkle_commit(const orc_p2* p, const uint32_t* base, int64_t height, int groups,
                              int g, int64_t gstride, int rpq, uint32_t* layers);

/* Reed-Solomon coset LDE, natural order in and out. */
int orc_rs_encode(int field, const uint32_t* coeffs, int64_t batch, int log_k,
                  int log_blowup, uint32_t shift_mont, uint32_t generator,
                  uint32_t* out);
int orc_rs_encode_horner(int field, const uint32_t* coeffs, int log_k,
                         int log_blowup, uint32_t shift_mont, uint32_t generator,
                         uint32_t* out);
/* BitReversedReedSolomon.encode: orc_rs_encode, each row bit-reversed. */
int orc_rs_encode_bitrev(int field, const uint32_t* coeffs, int64_t batch, int log_k,
                         int log_blowup, uint32_t shift_mont, uint32_t generator,
                         uint32_t* out);
uint32_t orc_eval_poly(int field, const uint32_t* coeffs, int64_t k, uint32_t x);
uint32_t orc_domain_point(int field, int log_n, uint32_t shift_mont, uint32_t generator,
                          int64_t j);
void orc_eval_domain(int field, int log_n, uint32_t shift_mont, uint32_t generator,
                     uint32_t* out);

/* FRI fold (natural order): out has n/2 elements of (ef_in|ef_beta ? 4 : 1) limbs. */
int orc_fri_fold(int field, const uint32_t* cw, int64_t n, int ef_in,
                 const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                 uint32_t generator, uint32_t* out);

/* FRI fold of a bit-reversed layer (pairs adjacent); output bit-reversed. */
int orc_fri_fold_bitrev(int field, const uint32_t* cw, int64_t n, int ef_in,
                        const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                        uint32_t generator, uint32_t* out);

/* k-ary Lagrange fold of a natural-order layer (k = 2^log_k <= 64). */
int orc_fri_fold_k(int field, const uint32_t* cw, int64_t n, int ef_in, const uint32_t* beta,
                   int ef_beta, int log_k, uint32_t shift_mont, uint32_t generator,
                   uint32_t* out);

/* SP1 single-matrix commitment domain separator. */
void orc_smcs_bind_root(const orc_p2* p, const uint32_t* raw_root, uint32_t log_height,
                        uint32_t width, uint32_t* out8);

/* Basefold sumcheck pieces (EF4 values are 4 Montgomery limbs c0..c3). */
void orc_ef4_inv(int field, const uint32_t* a, uint32_t* out);
void orc_eq_expand(int field, const uint32_t* z, int m, uint32_t* out);
void orc_eval_mle_base(int field, const uint32_t* cols, int w, int m, const uint32_t* z,
                       uint32_t* out);
void orc_eval_mle_ef4(int field, const uint32_t* mle, int m, const uint32_t* z, uint32_t* out);
void orc_mle_fold(int field, const uint32_t* mle, int64_t M, const uint32_t* beta, uint32_t* out);
void orc_rlc_columns_ex(int field, const uint32_t* cw, int64_t n, int w, const uint32_t* chal,
                        int nbv, int offset, int accumulate, uint32_t* out);

/* FRI open: f(z) for an EF4 point, and the DEEP quotient (cw - v)/(x - z). */
void orc_eval_poly_ef4(int field, const uint32_t* coeffs, int64_t k, const uint32_t* z,
                       uint32_t* out);
int orc_deep_quotient(int field, const uint32_t* cw, int64_t n, const uint32_t* z, int z_limbs,
                      const uint32_t* v, uint32_t shift_mont, uint32_t generator, int bitrev,
                      uint32_t* out);

/* Duplex transcript (overwrite mode, rate 8, width 16) */
void orc_duplex_init(orc_duplex* t);
void orc_duplex_observe(const orc_p2* p, orc_duplex* t, const uint32_t* v, int64_t m);
void orc_duplex_sample(const orc_p2* p, orc_duplex* t, int n, uint32_t* out);
/* lowest canonical proof-of-work witness (0 when none) */
uint32_t orc_duplex_grind(const orc_p2* p, const orc_duplex* t, int pow_bits);

/* FRI / Basefold commit phase (pre-fold pair commit rounds, then queries). */
void orc_rlc_columns(int field, const uint32_t* cw, int64_t n, int w, const uint32_t* alpha,
                     uint32_t* out);
int orc_fri_commit_phase(const orc_p2* p, int field, const uint32_t* codeword,
                         int log_n, int ef_in, uint32_t shift_mont, uint32_t generator,
                         int num_rounds, int num_queries, int beta_limbs,
                         orc_duplex* t, uint32_t* roots, uint32_t* betas,
                         uint32_t* final_layer, int32_t* positions,
                         uint32_t* rows, uint32_t* paths);

#ifdef __cplusplus
}
#endif
