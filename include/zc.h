/*
 * zorch-gb300 C ABI: the drop-in boundary under zorch's commit path.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*), launches asynchronously on that stream and returns a
 * status. Field values are Montgomery u32 (x * 2^32 mod p) -- the storage of
 * zk_dtypes' *_mont dtypes and the wire form of the reference's Fiat-Shamir FFI
 * contract (zorch/transcript.py:986-999, 1015-1021). Buffers are owned by the
 * caller; kernels write outputs only and never alias inputs. No entry point
 * allocates device memory except zc_poseidon2_create (its parameter block) and
 * zc_init (once per device); scratch is a caller-provided workspace.
 *
 * Each declaration names the reference interface it replaces (paths within
 * fractalyze/zorch).
 */
#ifndef ZORCH_GB300_ZC_H_
#define ZORCH_GB300_ZC_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  ZC_OK = 0,
  ZC_BAD_SHAPE = 1,   /* ValueError in the reference (zorch/coding/reed_solomon.py:178-182) */
  ZC_NOT_POW2 = 2,    /* ValueError (zorch/coding/reed_solomon.py:92-99, zorch/commit/merkle.py:148-149) */
  ZC_OOB_INDEX = 3,   /* IndexError (zorch/commit/merkle.py:220-221) */
  ZC_OOM = 4,         /* workspace too small / allocation failed */
  ZC_TIMEOUT = 5,     /* a bounded device wait gave up */
  ZC_CUDA_ERR = 6,    /* CUDA runtime error; zc_last_error() has the text */
  ZC_BAD_ARG = 7,     /* null pointer, misaligned buffer, bad enum */
  ZC_UNSUPPORTED = 8  /* NotImplementedError (e.g. an arity or generator not built) */
} zc_status;

typedef enum { ZC_FIELD_BABYBEAR = 0, ZC_FIELD_KOALABEAR = 1 } zc_field;

/* Leaf layout of a Merkle commit: leaf p (0 <= p < num_leaves) is the
 * concatenation over q < groups of base[q*group_stride + p*group_len ...
 * + group_len). Row-major [L, w] leaves: groups=1, group_len=w. Column-major
 * [w, L] (zorch/commit/merkle.py:72-80 column_major=True, and the codeword.T
 * rows of zorch/pcs/basefold/prover.py:445-447): groups=w, group_len=1,
 * group_stride=L. FRI pair leaves of an n-element codeword with `limbs` words
 * per element (zorch/coding/reed_solomon.py:303-307 + zorch/pcs/fold.py:42-52):
 * groups=2, group_len=limbs, group_stride=(n/2)*limbs. */
typedef struct {
  const uint32_t* base;
  int64_t num_leaves;
  int32_t groups;
  int32_t group_len;
  int64_t group_stride;
} zc_leaves;

/* Opaque width-16 Poseidon2 parameterisation living in device memory
 * (hash-frx Poseidon2Params, used at zorch/testkit/koalabear16.py:239-263). */
typedef struct zc_poseidon2 zc_poseidon2;

/* Duplex transcript state, the five FFI operands in order
 * (zorch/transcript.py:1015-1021, 1041-1053): in_buf(8), out_buf(8),
 * sponge(16), in_pos(1), out_pos(1) -- 34 u32 words. */
#define ZC_DUPLEX_WORDS 34

const char* zc_status_str(zc_status s);
const char* zc_last_error(void);
int zc_version(void);
/* Kernels this library has launched in the process so far (all devices). */
unsigned long long zc_launch_count(void);

/* Build per-device constant tables. Called implicitly on first use; call it
 * explicitly before any CUDA-graph capture. */
zc_status zc_init(int device);

/* Canonical <-> Montgomery conversion of n field words (inputs in canonical
 * form are reduced mod p first). zk_dtypes performs this at array
 * construction (fnp.array(..., dtype=koalabear_mont),
 * zorch/commit/testing/merkle_test.py:51-63); in-place (in == out) is allowed. */
zc_status zc_to_mont(zc_field field, const uint32_t* in, uint32_t* out, int64_t n, void* stream);
zc_status zc_from_mont(zc_field field, const uint32_t* in, uint32_t* out, int64_t n,
                       void* stream);

/* out[i] = in[i] * s (Montgomery scalar): the 1/n of an inverse NTT
 * (lax.ntt INTT, used by ReedSolomon.extend, zorch/coding/reed_solomon.py:190-208). */
zc_status zc_scale(zc_field field, const uint32_t* in, uint32_t* out, int64_t n, uint32_t s_mont,
                   void* stream);

/* The device address of a page-locked host buffer (cudaHostGetDevicePointer),
 * so a kernel -- e.g. zc_to_mont -- reads host inputs directly over the host
 * link instead of a staging copy: no counterpart in the reference (its
 * inputs arrive as device arrays). ZC_BAD_ARG if `host` is not page-locked. */
zc_status zc_host_device_ptr(const void* host, void** dev);
/* Canonical -> Montgomery of n words read straight from page-locked host
 * memory `host` (the conversion kernel's loads cross the host link; no
 * staging copy), into device `out`, on at most max_ctas CTAs of 1024 threads
 * (<= 0: the library default, 64) so that the SMs it leaves free keep
 * running other streams. ZC_BAD_ARG if `host` is not page-locked. */
zc_status zc_to_mont_from_host(zc_field field, const void* host, uint32_t* out, int64_t n,
                               int32_t max_ctas, void* stream);

/* ---- Poseidon2 parameters -------------------------------------------- */
/* The built-in BabyBear width-16 instance (x^7, 4+4 full, 13 partial rounds).
 * The reference ships no BabyBear instance; see gen_poseidon2_babybear16.py. */
zc_status zc_poseidon2_builtin(zc_field field, const zc_poseidon2** out);
/* Any width-16 instance from canonical host arrays: ext_init/ext_term are
 * rounds_f_half x 16, int_rc is rounds_p, diag is 16; j_scale is the
 * internal_j_scale (1 = identity). Replaces Poseidon2(Poseidon2Params(...)). */
zc_status zc_poseidon2_create(zc_field field, int alpha, int rounds_f_half, int rounds_p,
                              const uint32_t* ext_init, const uint32_t* ext_term,
                              const uint32_t* int_rc, const uint32_t* diag,
                              uint32_t j_scale, zc_poseidon2** out);
zc_status zc_poseidon2_destroy(zc_poseidon2* p);
/* Permute `count` independent 16-word states in place (hash-frx Permutation.permute). */
zc_status zc_poseidon2_permute(const zc_poseidon2* p, uint32_t* states, int64_t count,
                               void* stream);

/* The same permutation on the calling CPU thread over host memory (for
 * verifiers: MerkleTree.reconstruct_root / verify, zorch/commit/merkle.py:264-331). */
zc_status zc_poseidon2_permute_host(const zc_poseidon2* p, uint32_t* states, int64_t count);

/* ---- Reed-Solomon coset LDE ------------------------------------------ */
/* Replaces ReedSolomon.encode (zorch/coding/reed_solomon.py:177-188):
 * out[b, j] = sum_i coeffs[b, i] * (shift * w^j)^i for j < 2^(log_k+log_blowup),
 * natural order in and out, w = generator^((p-1)/n). shift_mont = 0 means no
 * coset (coset_shift=None). generator 0 = the field's canonical generator
 * (31 for BabyBear, 3 for KoalaBear); other generators are ZC_UNSUPPORTED.
 * coeffs: [batch, 2^log_k]; out: [batch, 2^(log_k+log_blowup)]. */
size_t zc_rs_encode_workspace_bytes(int64_t batch, int log_k, int log_blowup);
zc_status zc_rs_encode(zc_field field, const uint32_t* coeffs, int64_t batch, int log_k,
                       int log_blowup, uint32_t shift_mont, uint32_t generator,
                       uint32_t* out, void* workspace, size_t workspace_bytes,
                       void* stream);

/* Replaces BitReversedReedSolomon.encode (zorch/coding/reed_solomon.py:476-478):
 * the codeword of zc_rs_encode with each row in bit-reversed order,
 * out[b, brev(j)] = sum_i coeffs[b, i] * (shift * w^j)^i, so the fold pairs
 * (2p, 2p+1) are adjacent. Arguments, workspace and errors as zc_rs_encode. */
zc_status zc_rs_encode_bitrev(zc_field field, const uint32_t* coeffs, int64_t batch, int log_k,
                              int log_blowup, uint32_t shift_mont, uint32_t generator,
                              uint32_t* out, void* workspace, size_t workspace_bytes,
                              void* stream);

/* The LDE of zc_rs_encode without any device allocation and without a
 * caller workspace: no counterpart in the reference. For callers that cannot
 * allocate device memory at call time -- a handler inside an XLA/FRX custom
 * call (the framework owns the device memory and by default preallocates most
 * of it, so a cudaMalloc there can fail or fragment its pool), or a serving
 * loop that must not stall on the allocator. The
 * four-step intermediate lives in a fixed 64 MiB (2^24-word) static device
 * array that every GPU loading this library holds until the process exits;
 * columns are processed in chunks that fit it, and a size whose single column
 * needs more (2^(log_k+log_blowup) > 2^24 words) is rejected with
 * ZC_BAD_SHAPE. The array is shared by every call and keeps the last call's
 * contents (nothing in it needs to start at zero); calls that overlap on the
 * GPU (different streams, or different host threads) race on it -- serialise
 * them. The first call on a device performs set-up (root tables, the device
 * address of the array) and synchronises that device: make it before any
 * stream capture, and early, before another runtime preallocates the memory.
 * A cudaDeviceReset discards that set-up with every other per-device table of
 * this library: do not use the library on a device after resetting it.
 * Arguments and results as zc_rs_encode. */
zc_status zc_rs_encode_noalloc(zc_field field, const uint32_t* coeffs, int64_t batch, int log_k,
                               int log_blowup, uint32_t shift_mont, uint32_t generator,
                               uint32_t* out, void* stream);

/* Batched LDE: many jobs (matrices of different heights, widths, blowups) in
 * two launches over a (job, tile) work list -- the batched form of
 * the one-call-per-matrix encode of zorch/pcs/basefold/prover.py:437-447.
 * tile_log selects the shared-memory tile (2^tile_log words; 0 = default),
 * the knob the autotuner sets per (log_n, width) bucket. The workspace holds
 * the four-step intermediates (jobs are split into waves that fit) and must be
 * 256-byte aligned. */
typedef struct {
  const uint32_t* coeffs; /* [batch, 2^log_k] */
  uint32_t* out;          /* [batch, 2^(log_k+log_blowup)] */
  int64_t batch;
  int32_t log_k;
  int32_t log_blowup;
  uint32_t shift_mont;    /* 0: no coset */
  int32_t tile_log;       /* 0: default */
  int32_t bit_reversed;   /* 1: bit-reversed codeword (zc_rs_encode_bitrev) */
  int32_t radix_log;      /* largest radix-2^r shared-memory pass, 2..4; 0: default 4 */
} zc_lde_job;
size_t zc_rs_encode_batch_workspace_bytes(const zc_lde_job* jobs, int32_t njobs);
zc_status zc_rs_encode_batch(zc_field field, const zc_lde_job* jobs, int32_t njobs,
                             uint32_t generator, void* workspace, size_t workspace_bytes,
                             void* stream);

/* ---- Merkle trees (arity 2) ------------------------------------------- */
/* Replaces MerkleTree.commit = hash_leaves + fold_digests
 * (zorch/commit/merkle.py:118-202) over PaddingFreeSponge<16,8,8> leaves and
 * TruncatedPermutation<2,8,16> nodes. layers: (2L-1)*8 words, level l (leaf
 * digests l=0 ... root l=log2 L) at node offset 2L - (2L >> l). L must be a
 * power of two. */
zc_status zc_merkle_commit(const zc_poseidon2* p, zc_leaves leaves, uint32_t* layers,
                           void* stream);
/* Replaces StridedMerkleTree.commit (zorch/commit/strided_merkle.py:100-152):
 * the leaves are the num_leaves rows of `leaves`; query-layer node y
 * (s = num_leaves / rows_per_query of them) is the binary tree over rows
 * y, y + s, ..., y + (rows_per_query - 1) s; layers: (2s-1)*8 words, the
 * query layer first (the strided levels below it are not stored), root last.
 * rows_per_query a power of two <= 128. Opening paths come from zc_merkle_open
 * over s leaves with an empty row layout. */
zc_status zc_strided_merkle_commit(const zc_poseidon2* p, zc_leaves leaves, int32_t rows_per_query,
                                   uint32_t* layers, void* stream);
/* Replaces open_rows / MerkleTree.open (zorch/pcs/fold.py:142-149,
 * zorch/commit/merkle.py:204-235): rows [q, w], paths [depth][q][8] leaf first.
 * Out-of-range indices are clamped on the device and reported as ZC_OOB_INDEX
 * through *oob_flag (device word, may be NULL) -- the host checks before use. */
zc_status zc_merkle_open(zc_leaves leaves, const uint32_t* layers, const int32_t* idx,
                         int32_t q, uint32_t* rows, uint32_t* paths, uint32_t* oob_flag,
                         void* stream);
/* zc_merkle_open at leaf (idx[i] >> shift) mod num_leaves: a fold layer's
 * opening at the layer position of the sampled query positions
 * (code.layer_positions: natural order a_i = q mod (n >> (i+1)), shift 0,
 * zorch/coding/reed_solomon.py:320-329; bit-reversed order a_i = q >> (i+1),
 * shift i+1, :521-528; opened by _open_one, zorch/pcs/fri/prover.py:176-181),
 * with the reduction done by the kernel. Every index is in range by
 * construction, so there is no flag. shift in [0, 31]. */
zc_status zc_merkle_open_reduced(zc_leaves leaves, const uint32_t* layers, const int32_t* idx,
                                 int32_t q, int32_t shift, uint32_t* rows, uint32_t* paths,
                                 void* stream);

/* Batched commit of many trees (the per-matrix MerkleTree.commit calls of a
 * batch, zorch/commit/merkle.py:118-202, and the per-polynomial _commit_one
 * calls of FriProver.commit, zorch/pcs/fri/prover.py:92-99, 141-148) in
 * 1 + (max depth - 8) + 1 launches. A job with count > 1 is a family of
 * `count` trees of one shape: tree t hashes the leaves of `leaves` with its
 * base moved by t*leaf_stride words and writes its layers at
 * layers + t*layer_stride (e.g. each column of a [w, n] codeword as its own
 * pair-leaf tree). workspace: >= 256 bytes, 256-byte aligned (per-launch work
 * counters). */
typedef struct {
  zc_leaves leaves;
  uint32_t* layers;     /* (2L-1)*8 words per tree */
  int32_t top_log;      /* the levels of <= 2^top_log nodes run fused in one CTA per
                           tree (half-warp permutations), 1..8; 0: default 8 */
  int32_t count;        /* trees in the family; 0 or 1: one tree */
  int64_t leaf_stride;  /* words between successive trees' leaf bases */
  int64_t layer_stride; /* words between successive trees' layers, >= (2L-1)*8,
                           a multiple of 4 */
} zc_merkle_job;
zc_status zc_merkle_commit_batch(const zc_poseidon2* p, const zc_merkle_job* jobs,
                                 int32_t njobs, void* workspace, size_t workspace_bytes,
                                 void* stream);

/* ---- FRI fold ---------------------------------------------------------- */
/* Replaces ReedSolomon.fold -> fri_fold -> fri_fold_values
 * (zorch/coding/reed_solomon.py:273-278, 543-548, 589-604) on a natural-order
 * layer of n elements (ef_in: 4 limbs each, else 1), beta on the device
 * (ef_beta: 4 limbs, else 1), shift_mont the layer's coset shift
 * coset_shift^(2^level) (:331-339). out: n/2 elements, 4 limbs if either
 * input is EF4. */
zc_status zc_fri_fold(zc_field field, const uint32_t* cw, int64_t n, int ef_in,
                      const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                      uint32_t generator, uint32_t* out, void* stream);
/* The fold fused with the next round's pair-leaf commit
 * (PreFoldPairCommitRound, zorch/pcs/fold.py:90-115): writes the folded layer
 * `out` and the complete digest layers of its pair-leaf tree
 * (n/4 leaves) into next_layers. n >= 4. */
zc_status zc_fri_fold_commit(const zc_poseidon2* p, const uint32_t* cw, int64_t n, int ef_in,
                             const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                             uint32_t generator, uint32_t* out, uint32_t* next_layers,
                             void* stream);

/* zc_fri_fold_commit (bit_reversed = 0) or zc_fri_fold_commit_bitrev (1)
 * followed, in the launch that computes the new tree's root, by the next
 * round's transcript hop (PreFoldPairCommitRound, zorch/pcs/fold.py:106-113):
 * observe the 8 root words into the packed 34-word duplex state `state`
 * (read and advanced in place) and squeeze n_chal (0..64) words into `chal`
 * -- the same state and words as zc_duplex_step(state, root, 8, n_chal), one
 * launch fewer per fold round. */
zc_status zc_fri_fold_commit_hop(const zc_poseidon2* p, const uint32_t* cw, int64_t n, int ef_in,
                                 const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                                 uint32_t generator, int32_t bit_reversed, uint32_t* out,
                                 uint32_t* next_layers, uint32_t* state, int32_t n_chal,
                                 uint32_t* chal, void* stream);
/* zc_merkle_commit followed, in the root's launch, by the same transcript hop
 * (a first pre-fold round's commit, observe(root), sample). */
zc_status zc_merkle_commit_hop(const zc_poseidon2* p, zc_leaves leaves, uint32_t* layers,
                               uint32_t* state, int32_t n_chal, uint32_t* chal, void* stream);

/* Replaces ReedSolomon.fold_group (zorch/coding/reed_solomon.py:357-381;
 * fri_fold_k :551-586): the k-ary fold, k = 2^log_k (log_k 1..4), of a
 * natural-order layer of n elements. Group p < n/k is
 * (cw[p], cw[p + n/k], ..., cw[p + (k-1) n/k]) on the points
 * shift_mont * w_n^(p + m n/k); out[p] is its degree-(k-1) interpolant at
 * beta. Limb conventions as zc_fri_fold. */
zc_status zc_fri_fold_k(zc_field field, const uint32_t* cw, int64_t n, int ef_in,
                        const uint32_t* beta, int ef_beta, int log_k, uint32_t shift_mont,
                        uint32_t generator, uint32_t* out, void* stream);
/* Replaces BitReversedReedSolomon.fold (zorch/coding/reed_solomon.py:484-492,
 * 532-540) on a bit-reversed layer: out[p] folds the adjacent pair
 * (cw[2p], cw[2p+1]) at x_p = shift_mont * w_n^brev(p) (p read over
 * log2(n/2) bits); the output is the next layer, again bit-reversed.
 * Arguments as zc_fri_fold. */
zc_status zc_fri_fold_bitrev(zc_field field, const uint32_t* cw, int64_t n, int ef_in,
                             const uint32_t* beta, int ef_beta, uint32_t shift_mont,
                             uint32_t generator, uint32_t* out, void* stream);
/* zc_fri_fold_bitrev fused with the commit of the folded layer as the SP1
 * stacked open commits it (zorch/pcs/jagged/open.py:270-282): leaf p of
 * next_layers is out[2p] || out[2p+1] in base limbs (n/4 leaves). n >= 4. */
zc_status zc_fri_fold_commit_bitrev(const zc_poseidon2* p, const uint32_t* cw, int64_t n,
                                    int ef_in, const uint32_t* beta, int ef_beta,
                                    uint32_t shift_mont, uint32_t generator, uint32_t* out,
                                    uint32_t* next_layers, void* stream);
/* Replaces SingleMatrixCommitmentScheme.bind_root (zorch/commit/smcs.py:118-140):
 * out = compress([raw_root, sponge([log_height, width])]), the two shape
 * words as field elements; raw_root and out are 8 device words (out 16-byte
 * aligned). */
zc_status zc_smcs_bind_root(const zc_poseidon2* p, const uint32_t* raw_root, uint32_t log_height,
                            uint32_t width, uint32_t* out, void* stream);

/* ---- FRI open: the DEEP quotient --------------------------------------- */
/* Replaces _eval_poly (zorch/pcs/fri/prover.py:42-49): out = sum_i
 * coeffs[i] z^i for k >= 1 base coefficients, z a base element (z_limbs = 1)
 * or an EF4 element (z_limbs = 4, out 16-byte aligned); out has z_limbs words.
 * workspace: zc_eval_poly_workspace_bytes(k) bytes, 16-byte aligned. */
size_t zc_eval_poly_workspace_bytes(int64_t k);
zc_status zc_eval_poly(zc_field field, const uint32_t* coeffs, int64_t k, const uint32_t* z,
                       int32_t z_limbs, uint32_t* out, void* workspace, size_t workspace_bytes,
                       void* stream);
/* The layer-0 DEEP quotient of _open_one (zorch/pcs/fri/prover.py:160-164):
 * out[j] = (cw[j] - v) / (x_j - z) over the n-point evaluation domain, x_j =
 * shift * w_n^j (bit_reversed = 0) or shift * w_n^brev(j) (the
 * BitReversedReedSolomon codeword order); z and v (device words) have z_limbs
 * (1 or 4) limbs, and so does each output element (EF4 output 16-byte
 * aligned). A zero denominator (z on the domain) gives a zero quotient.
 * shift_mont 0: no coset. generator as zc_rs_encode. */
zc_status zc_deep_quotient(zc_field field, const uint32_t* cw, int64_t n, const uint32_t* z,
                           int32_t z_limbs, const uint32_t* v, uint32_t shift_mont,
                           uint32_t generator, int32_t bit_reversed, uint32_t* out,
                           void* stream);

/* ---- Basefold open: the multilinear side ------------------------------ */
/* EF4 values are 4 Montgomery words (c0..c3), 16-byte aligned on the device.
 * Replaces expand_eq_to_hypercube(z, 1) (zorch/poly/eq.py:92-130): out[i] =
 * eq(i, z) for i < 2^m, z[0] on the most significant index bit; m <= 24.
 * workspace: zc_eq_expand_workspace_bytes(m) bytes (0 for m <= 12). */
size_t zc_eq_expand_workspace_bytes(int32_t m);
zc_status zc_eq_expand(zc_field field, const uint32_t* z, int32_t m, uint32_t* out, void* workspace,
                       size_t workspace_bytes, void* stream);
/* Replaces eval_mle(mle, z, axis=0) (zorch/poly/multilinear.py:92-98) on w
 * base-field columns cols[w][2^m]: out[c] = sum_i eq(i, z) cols[c][i] (EF4). */
size_t zc_eval_mle_workspace_bytes(int32_t w, int32_t m);
zc_status zc_eval_mle(zc_field field, const uint32_t* cols, int32_t w, int32_t m,
                      const uint32_t* z, uint32_t* out, void* workspace, size_t workspace_bytes,
                      void* stream);
/* batch_staggered (zorch/pcs/basefold/batching.py:66-80) of one matrix's w base
 * columns cw[w][n] into the EF4 out[n]: weights eq(., r) over nbv <= 12 EF4
 * challenges (challenge 0 the most significant index bit), this matrix taking
 * weights offset .. offset+w-1; accumulate != 0 adds onto out. */
zc_status zc_rlc_columns_ex(zc_field field, const uint32_t* cw, int64_t n, int32_t w,
                            const uint32_t* challenges, int32_t nbv, int32_t offset,
                            int32_t accumulate, uint32_t* out, void* stream);
/* The same weights applied to w EF4 values (the batched claim): out (one EF4)
 * = [out +] sum_c weight[offset + c] values[c]. */
zc_status zc_rlc_values(zc_field field, const uint32_t* values, int32_t w,
                        const uint32_t* challenges, int32_t nbv, int32_t offset,
                        int32_t accumulate, uint32_t* out, void* stream);
/* Element-wise EF4 inverse of count values (16-byte aligned [count][4]
 * Montgomery words; in may equal out); zero maps to zero. The 1/z_i the
 * sumcheck message takes (Basefold's 1/z_last,
 * zorch/pcs/basefold/kernel.py:52-66), computed on the device. */
zc_status zc_ef4_inv(zc_field field, const uint32_t* in, uint32_t* out, int64_t count,
                     void* stream);
/* One interleaved-sumcheck message (SumcheckKernel.message,
 * zorch/pcs/basefold/kernel.py:52-66): the running MLE mle[2M] (EF4), the eq
 * table eq[M] of the unbound point prefix, the running claim and 1/z_last:
 * msg = (s0, s1), s0 = sum_j eq[j] mle[2j], s1 = (claim - s0) / z_last + s0.
 * workspace: zc_sumcheck_workspace_bytes() bytes. */
size_t zc_sumcheck_workspace_bytes(void);
zc_status zc_sumcheck_message(zc_field field, const uint32_t* mle, int64_t M, const uint32_t* eq,
                              const uint32_t* claim, const uint32_t* zinv, uint32_t* msg,
                              void* workspace, size_t workspace_bytes, void* stream);
/* The round's fold (SumcheckKernel.fold, :68-74; mle_fold,
 * zorch/poly/multilinear.py:101-109; contract_hypercube_step,
 * zorch/poly/eq.py:65-77): mle_out[j] = mle[2j] + beta mle[2j+1] (j < M),
 * eq_out[k] = eq[2k] + eq[2k+1] (k < M/2; skipped when eq_out is NULL),
 * claim = s0 + beta s1; beta has beta_limbs (1 or 4) device words. */
zc_status zc_sumcheck_fold(zc_field field, const uint32_t* mle, int64_t M, const uint32_t* beta,
                           int32_t beta_limbs, const uint32_t* msg, uint32_t* mle_out,
                           const uint32_t* eq, uint32_t* eq_out, uint32_t* claim, void* stream);

/* Staggered partial-Lagrange batching of a committed matrix's w base columns
 * (n words each) into one EF4 codeword [n, 4] (16-byte aligned): weights =
 * eq(., r) over nbv = ceil(log2 w) EF4 challenges (challenges: nbv x 4 words,
 * challenge 0 the most significant index bit), column c weighted by entry c
 * -- sample_rlc_coeffs_bits + batch_staggered (zorch/pcs/jagged/open.py:88-105,
 * zorch/pcs/basefold/batching.py:66-80). w <= 4096. */
zc_status zc_rlc_columns(zc_field field, const uint32_t* cw, int64_t n, int32_t w,
                         const uint32_t* challenges, uint32_t* out, void* stream);
/* out[i] = value for i < n, on the stream (zero through a memset): device
 * constants such as a zeroed transcript state or a round count to observe,
 * made without a host copy or a framework kernel, so fold loops stay free of
 * host synchronisation. No reference counterpart (the reference builds these
 * as jitted array constants). */
zc_status zc_fill_u32(uint32_t* out, int64_t n, uint32_t value, void* stream);
/* Device-to-device copy of `rows` rows of `row_bytes` bytes, row i from
 * src + i * src_pitch to dst + i * dst_pitch, as one 2D copy on the copy
 * engine (no kernel): gathers strided rows such as each tree's root out of a
 * stack of digest layers. Pitches >= row_bytes. No reference counterpart (the
 * reference slices jitted arrays). */
zc_status zc_copy_rows(void* dst, int64_t dst_pitch, const void* src, int64_t src_pitch,
                       int64_t row_bytes, int64_t rows, void* stream);
/* Synthetic benchmark data (no reference counterpart): out[i] =
 * SplitMix64(seed * 0x100000001B3 + i) mod p, canonical form. */
zc_status zc_fill_uniform(zc_field field, uint32_t* out, int64_t n, uint64_t seed, void* stream);

/* ---- Fiat-Shamir duplex (rate 8, width 16) ----------------------------- */
/* One observe-then-sample hop in the reference's host-FS FFI contract
 * (set_host_fs_ffi_target, zorch/transcript.py:1005-1035, _host_hop_ffi
 * :1056-1112): reads the five state operands and m values, writes the five
 * advanced operands and n challenge words. Inputs may alias outputs. The
 * device form runs on one GPU thread; the host form on the calling CPU thread
 * (all pointers host memory, stream ignored). */
zc_status zc_duplex_hop(const zc_poseidon2* p, const uint32_t* in_buf, const uint32_t* out_buf,
                        const uint32_t* sponge, const uint32_t* in_pos,
                        const uint32_t* out_pos, const uint32_t* values, int64_t m,
                        int32_t n, uint32_t* in_buf_o, uint32_t* out_buf_o,
                        uint32_t* sponge_o, uint32_t* in_pos_o, uint32_t* out_pos_o,
                        uint32_t* challenges, void* stream);
zc_status zc_duplex_hop_host(const zc_poseidon2* p, const uint32_t* in_buf,
                             const uint32_t* out_buf, const uint32_t* sponge,
                             const uint32_t* in_pos, const uint32_t* out_pos,
                             const uint32_t* values, int64_t m, int32_t n,
                             uint32_t* in_buf_o, uint32_t* out_buf_o, uint32_t* sponge_o,
                             uint32_t* in_pos_o, uint32_t* out_pos_o, uint32_t* challenges);
/* Proof-of-work grind (DuplexTranscript.grind / _grind_search,
 * zorch/transcript.py:439-481; grind_search, zorch/grind.py:66-93) on the
 * packed 34-word device state: writes to `witness` (one device word) the
 * lowest witness w in [0, p), as a Montgomery field element, whose challenge
 * -- observe w, sample once -- has pow_bits zero low canonical bits
 * (_pow_satisfied, :44-49); 0 when none passes (the reference's unchecked
 * fallback). pow_bits in [0, 32) else ZC_BAD_ARG. The state is read, not
 * advanced: observe the witness and sample once, as check_witness does. */
zc_status zc_duplex_grind(const zc_poseidon2* p, const uint32_t* state, int32_t pow_bits,
                          uint32_t* witness, void* stream);
/* Device-resident transcript step on a packed 34-word state: observe m values
 * then squeeze n words into `out`; if positions != NULL also write
 * positions[i] = out[i] mod block_len (sample_positions, zorch/pcs/fold.py:173-182). */
zc_status zc_duplex_step(const zc_poseidon2* p, uint32_t* state, const uint32_t* values,
                         int64_t m, int32_t n, uint32_t* out, int32_t* positions,
                         int64_t block_len, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ZORCH_GB300_ZC_H_ */
