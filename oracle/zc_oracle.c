/*
 * CPU ORACLE -- test infrastructure only (see zc_oracle.h). A plain-C
 * restatement of the reference algorithms; each function names the reference
 * file:line it follows. Compiled by oracle/build.py into oracle/_build/.
 */
#include "zc_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- field ---- */
/* zk_dtypes Montgomery form with R = 2^32 (zorch/commit/testing/sp1_koalabear16.py:16-18). */
typedef struct {
  uint32_t p, mu, r2, one, w; /* mu = p^-1 mod 2^32, r2 = 2^64 mod p, w = EF4 nonresidue (Mont) */
  uint32_t gen;               /* multiplicative generator (canonical) */
} fld;

static uint32_t inv_mod_2_32(uint32_t p) {
  uint32_t x = 1;
  for (int i = 0; i < 5; i++) x *= 2u - p * x;
  return x;
}

static uint32_t fmul(const fld* F, uint32_t a, uint32_t b) {
  uint64_t t = (uint64_t)a * b;
  uint32_t m = (uint32_t)t * F->mu;
  uint64_t mp = (uint64_t)m * F->p;
  int64_t r = (int64_t)(t >> 32) - (int64_t)(mp >> 32);
  return r < 0 ? (uint32_t)(r + F->p) : (uint32_t)r;
}
static uint32_t fadd(const fld* F, uint32_t a, uint32_t b) {
  uint32_t r = a + b;
  return r >= F->p ? r - F->p : r;
}
static uint32_t fsub(const fld* F, uint32_t a, uint32_t b) {
  return a >= b ? a - b : a + F->p - b;
}
static uint32_t fpow(const fld* F, uint32_t a, uint64_t e) {
  uint32_t r = F->one;
  while (e) {
    if (e & 1) r = fmul(F, r, a);
    a = fmul(F, a, a);
    e >>= 1;
  }
  return r;
}
static uint32_t finv(const fld* F, uint32_t a) { return fpow(F, a, F->p - 2); }

static fld FIELDS[2];
static int fields_ready = 0;

static void init_field(fld* F, uint32_t p, uint32_t gen, uint32_t w_canon) {
  F->p = p;
  F->mu = inv_mod_2_32(p);
  uint64_t r = ((uint64_t)1 << 32) % p;
  F->one = (uint32_t)r;
  F->r2 = (uint32_t)((r * r) % p);
  F->gen = gen;
  F->w = fmul(F, w_canon, F->r2);
}

static void init_fields(void) {
  if (!fields_ready) {
    /* BabyBear: p = 2^31 - 2^27 + 1, generator 31, EF4 = F[x]/(x^4 - 11). */
    init_field(&FIELDS[ORC_BABYBEAR], 2013265921u, 31u, 11u);
    /* KoalaBear: p = 2^31 - 2^24 + 1, generator 3, EF4 = F[x]/(x^4 - 3). */
    init_field(&FIELDS[ORC_KOALABEAR], 2130706433u, 3u, 3u);
    fields_ready = 1;
  }
}
/* Initialised at load time so OpenMP workers never race on the tables. */
__attribute__((constructor)) static void init_fields_at_load(void) { init_fields(); }
static const fld* FLD(int field) {
  init_fields();
  return &FIELDS[field ? 1 : 0];
}

static uint32_t to_m(const fld* F, uint32_t x) { return fmul(F, x % F->p, F->r2); }
static uint32_t from_m(const fld* F, uint32_t x) { return fmul(F, x, 1u); }

static int n_threads = 0;
void orc_set_threads(int n) { n_threads = n; }
int orc_get_threads(void) {
#ifdef _OPENMP
  return n_threads > 0 ? n_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

uint32_t orc_modulus(int field) { return FLD(field)->p; }
uint32_t orc_to_mont(int field, uint32_t x) { return to_m(FLD(field), x); }
uint32_t orc_from_mont(int field, uint32_t x) { return from_m(FLD(field), x); }
uint32_t orc_mul(int field, uint32_t a, uint32_t b) { return fmul(FLD(field), a, b); }
void orc_to_mont_vec(int field, const uint32_t* in, uint32_t* out, int64_t n) {
  const fld* F = FLD(field);
  for (int64_t i = 0; i < n; i++) out[i] = to_m(F, in[i]);
}
void orc_from_mont_vec(int field, const uint32_t* in, uint32_t* out, int64_t n) {
  const fld* F = FLD(field);
  for (int64_t i = 0; i < n; i++) out[i] = from_m(F, in[i]);
}

/* EF4 = F[x]/(x^4 - W), coefficients ascending (c0..c3). */
static void ef4_mul(const fld* F, const uint32_t* a, const uint32_t* b, uint32_t* c) {
  uint32_t t[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) t[i + j] = fadd(F, t[i + j], fmul(F, a[i], b[j]));
  for (int i = 0; i < 3; i++) t[i] = fadd(F, t[i], fmul(F, F->w, t[i + 4]));
  c[0] = t[0];
  c[1] = t[1];
  c[2] = t[2];
  c[3] = t[3];
}
void orc_ef4_mul(int field, const uint32_t* a, const uint32_t* b, uint32_t* out) {
  ef4_mul(FLD(field), a, b, out);
}

/* The order-2^log_n root the NTT uses: generator^((p-1)/n)
 * (zorch/coding/reed_solomon.py:57-59, 104-110). */
static uint32_t root_of_unity(const fld* F, int log_n, uint32_t gen_canon) {
  uint32_t g = to_m(F, gen_canon ? gen_canon : F->gen);
  return fpow(F, g, (uint64_t)(F->p - 1) >> log_n);
}
uint32_t orc_root_of_unity(int field, int log_n, uint32_t generator) {
  return root_of_unity(FLD(field), log_n, generator);
}

/* ------------------------------------------------------------ Poseidon2 ---- */
/* Width-16 Poseidon2 as hash-frx / Plonky3 compute it; the semantics are pinned
 * by the Plonky3 KoalaBear-16 root (zorch/commit/testing/merkle_test.py:51-63)
 * over the parameters at zorch/testkit/koalabear16.py:25-263. */
int orc_p2_size(void) { return (int)sizeof(orc_p2); }

static void ext_linear(const fld* F, uint32_t* s) {
  for (int c = 0; c < 16; c += 4) {
    uint32_t x0 = s[c], x1 = s[c + 1], x2 = s[c + 2], x3 = s[c + 3];
    uint32_t t01 = fadd(F, x0, x1), t23 = fadd(F, x2, x3);
    uint32_t t0123 = fadd(F, t01, t23);
    uint32_t t01123 = fadd(F, t0123, x1), t01233 = fadd(F, t0123, x3);
    s[c + 3] = fadd(F, t01233, fadd(F, x0, x0));       /* 3 1 1 2 */
    s[c + 1] = fadd(F, t01123, fadd(F, x2, x2));       /* 1 2 3 1 */
    s[c + 0] = fadd(F, t01123, t01);                   /* 2 3 1 1 */
    s[c + 2] = fadd(F, t01233, t23);                   /* 1 1 2 3 */
  }
  uint32_t sums[4];
  for (int k = 0; k < 4; k++)
    sums[k] = fadd(F, fadd(F, s[k], s[4 + k]), fadd(F, s[8 + k], s[12 + k]));
  for (int i = 0; i < 16; i++) s[i] = fadd(F, s[i], sums[i & 3]);
}

static uint32_t sbox(const fld* F, uint32_t x, int alpha) {
  if (alpha == 3) return fmul(F, fmul(F, x, x), x);
  if (alpha == 7) {
    uint32_t x2 = fmul(F, x, x), x3 = fmul(F, x2, x), x4 = fmul(F, x2, x2);
    return fmul(F, x3, x4);
  }
  return fpow(F, x, (uint64_t)alpha);
}

void orc_p2_permute(const orc_p2* P, uint32_t* s) {
  const fld* F = FLD(P->field);
  ext_linear(F, s);
  for (int r = 0; r < P->rounds_f_half; r++) {
    for (int i = 0; i < 16; i++) s[i] = sbox(F, fadd(F, s[i], P->ext_init[r][i]), P->alpha);
    ext_linear(F, s);
  }
  for (int r = 0; r < P->rounds_p; r++) {
    s[0] = sbox(F, fadd(F, s[0], P->int_rc[r]), P->alpha);
    uint32_t sum = 0;
    for (int i = 0; i < 16; i++) sum = fadd(F, sum, s[i]);
    uint32_t js = fmul(F, sum, P->j_scale);
    for (int i = 0; i < 16; i++) s[i] = fadd(F, js, fmul(F, P->diag[i], s[i]));
  }
  for (int r = 0; r < P->rounds_f_half; r++) {
    for (int i = 0; i < 16; i++) s[i] = sbox(F, fadd(F, s[i], P->ext_term[r][i]), P->alpha);
    ext_linear(F, s);
  }
}

void orc_p2_from_canonical(orc_p2* out, int field, int alpha, int rounds_f_half,
                           int rounds_p, const uint32_t* ext_init,
                           const uint32_t* ext_term, const uint32_t* int_rc,
                           const uint32_t* diag, uint32_t j_scale) {
  const fld* F = FLD(field);
  memset(out, 0, sizeof(*out));
  out->field = field;
  out->alpha = alpha;
  out->rounds_f_half = rounds_f_half;
  out->rounds_p = rounds_p;
  for (int r = 0; r < rounds_f_half; r++)
    for (int i = 0; i < 16; i++) {
      out->ext_init[r][i] = to_m(F, ext_init[r * 16 + i]);
      out->ext_term[r][i] = to_m(F, ext_term[r * 16 + i]);
    }
  for (int r = 0; r < rounds_p; r++) out->int_rc[r] = to_m(F, int_rc[r]);
  for (int i = 0; i < 16; i++) out->diag[i] = to_m(F, diag[i]);
  out->j_scale = to_m(F, j_scale);
}

void orc_p2_export_canonical(const orc_p2* P, uint32_t* ext_init, uint32_t* ext_term,
                             uint32_t* int_rc, uint32_t* diag) {
  const fld* F = FLD(P->field);
  for (int r = 0; r < P->rounds_f_half; r++)
    for (int i = 0; i < 16; i++) {
      ext_init[r * 16 + i] = from_m(F, P->ext_init[r][i]);
      ext_term[r * 16 + i] = from_m(F, P->ext_term[r][i]);
    }
  for (int r = 0; r < P->rounds_p; r++) int_rc[r] = from_m(F, P->int_rc[r]);
  for (int i = 0; i < 16; i++) diag[i] = from_m(F, P->diag[i]);
}

/* The Poseidon paper's Grain LFSR (eprint 2019/458), 80-bit state. */
typedef struct {
  uint8_t b[80];
} grain;
static int grain_clock(grain* g) {
  int nb = g->b[62] ^ g->b[51] ^ g->b[38] ^ g->b[23] ^ g->b[13] ^ g->b[0];
  memmove(g->b, g->b + 1, 79);
  g->b[79] = (uint8_t)nb;
  return nb;
}
static int grain_bit(grain* g) {
  int b = grain_clock(g);
  while (b == 0) {
    grain_clock(g);
    b = grain_clock(g);
  }
  return grain_clock(g);
}
static void grain_init(grain* g, int field, int sbox_t, int n, int t, int rf, int rp) {
  int k = 0;
  for (int i = 1; i >= 0; i--) g->b[k++] = (field >> i) & 1;
  for (int i = 3; i >= 0; i--) g->b[k++] = (sbox_t >> i) & 1;
  for (int i = 11; i >= 0; i--) g->b[k++] = (n >> i) & 1;
  for (int i = 11; i >= 0; i--) g->b[k++] = (t >> i) & 1;
  for (int i = 9; i >= 0; i--) g->b[k++] = (rf >> i) & 1;
  for (int i = 9; i >= 0; i--) g->b[k++] = (rp >> i) & 1;
  while (k < 80) g->b[k++] = 1;
  for (int i = 0; i < 160; i++) grain_clock(g);
}

/* Project-defined BabyBear-16 instance: x^7, 4+4 full, 13 partial rounds,
 * Grain-LFSR constants in round order, "shift friendly" internal diagonal.
 * Derived independently here; a test compares it with the CUDA header. */
void orc_p2_babybear16(orc_p2* out) {
  const fld* F = FLD(ORC_BABYBEAR);
  const uint32_t p = F->p;
  grain g;
  grain_init(&g, 1, 0, 31, 16, 8, 13);
  uint32_t rc[21][16];
  for (int r = 0; r < 21; r++)
    for (int i = 0; i < 16; i++) {
      uint32_t v;
      do {
        v = 0;
        for (int b = 0; b < 31; b++) v = (v << 1) | (uint32_t)grain_bit(&g);
      } while (v >= p);
      rc[r][i] = v;
    }
  uint32_t ext_init[64], ext_term[64], int_rc[13], diag[16];
  for (int r = 0; r < 4; r++)
    for (int i = 0; i < 16; i++) {
      ext_init[r * 16 + i] = rc[r][i];
      ext_term[r * 16 + i] = rc[17 + r][i];
    }
  for (int r = 0; r < 13; r++) int_rc[r] = rc[4 + r][0];
  /* -2, 1, 2, 1/2, 3, 4, -1/2, -3, -4, 1/2^8, 1/4, 1/8, 1/2^27, -1/2^8, -1/16, -1/2^27 */
  const int num[16] = {-2, 1, 2, 1, 3, 4, -1, -3, -4, 1, 1, 1, 1, -1, -1, -1};
  const int lg_den[16] = {0, 0, 0, 1, 0, 0, 1, 0, 0, 8, 2, 3, 27, 8, 4, 27};
  for (int i = 0; i < 16; i++) {
    uint32_t nm = to_m(F, num[i] < 0 ? p - (uint32_t)(-num[i]) : (uint32_t)num[i]);
    uint32_t den = to_m(F, 1u << lg_den[i]);
    diag[i] = from_m(F, fmul(F, nm, finv(F, den)));
  }
  orc_p2_from_canonical(out, ORC_BABYBEAR, 7, 4, 13, ext_init, ext_term, int_rc, diag, 1);
}

/* PaddingFreeSponge<16, rate 8, out 8>: overwrite the rate lanes block by
 * block, permute per block, a short tail overwrites only its prefix; the
 * digest is state[0:8] (hash-frx Sponge as fixed by
 * zorch/commit/testing/koalabear16.py:18-25 and the Plonky3 golden). */
void orc_sponge_hash(const orc_p2* P, const uint32_t* in, int64_t m, uint32_t* out8) {
  uint32_t s[16];
  memset(s, 0, sizeof(s));
  for (int64_t i = 0; i < m; i += 8) {
    int64_t blk = m - i < 8 ? m - i : 8;
    for (int64_t j = 0; j < blk; j++) s[j] = in[i + j];
    orc_p2_permute(P, s);
  }
  memcpy(out8, s, 32);
}

/* TruncatedPermutation<2, 8, 16>: permute(left || right)[0:8]
 * (Compression.compress, zorch/commit/merkle.py:183-185). */
void orc_compress(const orc_p2* P, const uint32_t* l8, const uint32_t* r8, uint32_t* out8) {
  uint32_t s[16];
  memcpy(s, l8, 32);
  memcpy(s + 8, r8, 32);
  orc_p2_permute(P, s);
  memcpy(out8, s, 32);
}

/* --------------------------------------------------------------- Merkle ---- */
static int is_pow2(int64_t x) { return x > 0 && (x & (x - 1)) == 0; }

/* j with its low `bits` bits reversed. */
static int64_t brev64(int64_t j, int bits) {
  int64_t r = 0;
  for (int b = 0; b < bits; b++) r |= ((j >> b) & 1) << (bits - 1 - b);
  return r;
}

static void gather_leaf(const uint32_t* base, int64_t p, int groups, int g,
                        int64_t gstride, uint32_t* row) {
  for (int q = 0; q < groups; q++)
    for (int e = 0; e < g; e++) row[q * g + e] = base[q * gstride + p * g + e];
}

/* MerkleTree.commit = hash_leaves + _fold_to_root (zorch/commit/merkle.py:118-202),
 * arity 2, every level stored leaf-first. */
int orc_merkle_commit(const orc_p2* P, const uint32_t* base, int64_t L, int groups,
                      int g, int64_t gstride, uint32_t* layers) {
  if (!is_pow2(L)) return 2;
  const int w = groups * g;
#pragma omp parallel num_threads(orc_get_threads())
  {
    uint32_t* row = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(w > 0 ? w : 1));
#pragma omp for schedule(static)
    for (int64_t p = 0; p < L; p++) {
      gather_leaf(base, p, groups, g, gstride, row);
      orc_sponge_hash(P, row, w, layers + 8 * p);
    }
    free(row);
  }
  int64_t off = 0, n = L;
  while (n > 1) {
    const uint32_t* cur = layers + 8 * off;
    uint32_t* nxt = layers + 8 * (off + n);
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
    for (int64_t i = 0; i < n / 2; i++) orc_compress(P, cur + 16 * i, cur + 16 * i + 8, nxt + 8 * i);
    off += n;
    n /= 2;
  }
  return 0;
}

/* MerkleTree.open per index (zorch/commit/merkle.py:204-235): the leaf row and
 * the sibling at each level, leaf first. paths: [level][query][8]. */
int orc_merkle_open(const uint32_t* base, int64_t L, int groups, int g, int64_t gstride,
                    const uint32_t* layers, const int32_t* idx, int q, uint32_t* rows,
                    uint32_t* paths) {
  int depth = 0;
  while (((int64_t)1 << depth) < L) depth++;
  const int w = groups * g;
  for (int k = 0; k < q; k++) {
    if (idx[k] < 0 || idx[k] >= L) return 3;
    gather_leaf(base, idx[k], groups, g, gstride, rows + (int64_t)k * w);
    int64_t i = idx[k], off = 0, n = L;
    for (int l = 0; l < depth; l++) {
      memcpy(paths + ((int64_t)l * q + k) * 8, layers + 8 * (off + (i ^ 1)), 32);
      off += n;
      n /= 2;
      i >>= 1;
    }
  }
  return 0;
}

/* StridedMerkleTree.commit (zorch/commit/strided_merkle.py:100-152): leaf
 * hashes of all `height` rows, then log2(rpq) query-strided levels
 * next[x s + y] = compress(prev[2x s + y], prev[(2x+1) s + y]) (s = height /
 * rpq, not stored), then the plain binary tree over the s query-layer nodes.
 * layers: (2s-1)*8 words, query layer first. */
int orc_strided_merkle_commit(const orc_p2* P, const uint32_t* base, int64_t height, int groups,
                              int g, int64_t gstride, int rpq, uint32_t* layers) {
  if (!is_pow2(height) || !is_pow2(rpq) || rpq > height) return 2;
  const int w = groups * g;
  const int64_t s = height / rpq;
  uint32_t* cur = (uint32_t*)malloc(sizeof(uint32_t) * 8 * (size_t)height);
#pragma omp parallel num_threads(orc_get_threads())
  {
    uint32_t* row = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(w > 0 ? w : 1));
#pragma omp for schedule(static)
    for (int64_t p = 0; p < height; p++) {
      gather_leaf(base, p, groups, g, gstride, row);
      orc_sponge_hash(P, row, w, cur + 8 * p);
    }
    free(row);
  }
  int64_t m = height;
  while (m > s) {
    uint32_t* nxt = (uint32_t*)malloc(sizeof(uint32_t) * 8 * (size_t)(m / 2));
    for (int64_t x = 0; x < m / (2 * s); x++)
      for (int64_t y = 0; y < s; y++)
        orc_compress(P, cur + 8 * ((2 * x) * s + y), cur + 8 * ((2 * x + 1) * s + y),
                     nxt + 8 * (x * s + y));
    free(cur);
    cur = nxt;
    m /= 2;
  }
  memcpy(layers, cur, sizeof(uint32_t) * 8 * (size_t)s);
  free(cur);
  int64_t off = 0, n = s;
  while (n > 1) {
    const uint32_t* a = layers + 8 * off;
    uint32_t* b = layers + 8 * (off + n);
    for (int64_t i = 0; i < n / 2; i++) orc_compress(P, a + 16 * i, a + 16 * i + 8, b + 8 * i);
    off += n;
    n /= 2;
  }
  return 0;
}

/* ------------------------------------------------------------------ NTT ---- */
static void ntt_inplace(const fld* F, uint32_t* a, int log_n, uint32_t omega) {
  const int64_t n = (int64_t)1 << log_n;
  for (int64_t i = 1, j = 0; i < n; i++) {
    int64_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      uint32_t t = a[i];
      a[i] = a[j];
      a[j] = t;
    }
  }
  uint32_t* tw = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n / 2 > 0 ? n / 2 : 1));
  for (int s = 1; s <= log_n; s++) {
    const int64_t len = (int64_t)1 << s, half = len >> 1;
    uint32_t wl = fpow(F, omega, (uint64_t)(n >> s));
    tw[0] = F->one;
    for (int64_t j = 1; j < half; j++) tw[j] = fmul(F, tw[j - 1], wl);
    for (int64_t i = 0; i < n; i += len)
      for (int64_t j = 0; j < half; j++) {
        uint32_t u = a[i + j], v = fmul(F, a[i + j + half], tw[j]);
        a[i + j] = fadd(F, u, v);
        a[i + j + half] = fsub(F, u, v);
      }
  }
  free(tw);
}

/* ReedSolomon.encode (zorch/coding/reed_solomon.py:177-188): zero-pad to
 * block_len, scale by the coset ramp [1,h,h^2,..] (:115-121,
 * zorch/poly/univariate.py:17-33), forward NTT natural in / natural out with
 * root generator^((p-1)/n). encode(m)[j] = sum_i m_i (h w^j)^i. */
int orc_rs_encode(int field, const uint32_t* coeffs, int64_t batch, int log_k,
                  int log_blowup, uint32_t shift_mont, uint32_t generator, uint32_t* out) {
  const fld* F = FLD(field);
  if (log_k < 0 || log_blowup < 0 || log_k + log_blowup > 27) return 1;
  const int log_n = log_k + log_blowup;
  const int64_t k = (int64_t)1 << log_k, n = (int64_t)1 << log_n;
  const uint32_t omega = root_of_unity(F, log_n, generator);
  uint32_t* ramp = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)k);
  ramp[0] = F->one;
  for (int64_t i = 1; i < k; i++) ramp[i] = shift_mont ? fmul(F, ramp[i - 1], shift_mont) : F->one;
  if (!shift_mont)
    for (int64_t i = 0; i < k; i++) ramp[i] = F->one;
#pragma omp parallel for num_threads(orc_get_threads()) schedule(dynamic, 1)
  for (int64_t b = 0; b < batch; b++) {
    uint32_t* a = out + b * n;
    for (int64_t i = 0; i < k; i++) a[i] = fmul(F, coeffs[b * k + i], ramp[i]);
    for (int64_t i = k; i < n; i++) a[i] = 0;
    ntt_inplace(F, a, log_n, omega);
  }
  free(ramp);
  return 0;
}

/* Independent check mirroring zorch/coding/testing/reed_solomon_test.py:48-60:
 * Horner-evaluate the message at every domain point. O(n k). */
int orc_rs_encode_horner(int field, const uint32_t* coeffs, int log_k, int log_blowup,
                         uint32_t shift_mont, uint32_t generator, uint32_t* out) {
  const fld* F = FLD(field);
  const int log_n = log_k + log_blowup;
  const int64_t k = (int64_t)1 << log_k, n = (int64_t)1 << log_n;
  uint32_t* dom = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
  orc_eval_domain(field, log_n, shift_mont, generator, dom);
  for (int64_t j = 0; j < n; j++) {
    uint32_t acc = 0;
    for (int64_t i = k - 1; i >= 0; i--) acc = fadd(F, fmul(F, acc, dom[j]), coeffs[i]);
    out[j] = acc;
  }
  free(dom);
  return 0;
}

/* BitReversedReedSolomon.encode (zorch/coding/reed_solomon.py:476-478): the
 * natural-order codeword of orc_rs_encode, then bit-reversed along the last
 * axis (out[b, brev(j)] = natural[b, j]). */
int orc_rs_encode_bitrev(int field, const uint32_t* coeffs, int64_t batch, int log_k,
                         int log_blowup, uint32_t shift_mont, uint32_t generator,
                         uint32_t* out) {
  const int rc = orc_rs_encode(field, coeffs, batch, log_k, log_blowup, shift_mont, generator, out);
  if (rc) return rc;
  const int log_n = log_k + log_blowup;
  const int64_t n = (int64_t)1 << log_n;
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
  for (int64_t b = 0; b < batch; b++) {
    uint32_t* a = out + b * n;
    for (int64_t j = 0; j < n; j++) {
      const int64_t r = brev64(j, log_n);
      if (j < r) {
        const uint32_t t = a[j];
        a[j] = a[r];
        a[r] = t;
      }
    }
  }
  return 0;
}

/* Horner evaluation of one polynomial at one point: sum_i c_i x^i. */
uint32_t orc_eval_poly(int field, const uint32_t* coeffs, int64_t k, uint32_t x) {
  const fld* F = FLD(field);
  uint32_t acc = 0;
  for (int64_t i = k - 1; i >= 0; i--) acc = fadd(F, fmul(F, acc, x), coeffs[i]);
  return acc;
}

/* The j-th point of the coset domain shift * w_n^j. */
uint32_t orc_domain_point(int field, int log_n, uint32_t shift_mont, uint32_t generator,
                          int64_t j) {
  const fld* F = FLD(field);
  uint32_t w = log_n ? root_of_unity(F, log_n, generator) : F->one;
  return fmul(F, shift_mont ? shift_mont : F->one, fpow(F, w, (uint64_t)j));
}

/* eval_domain (zorch/coding/reed_solomon.py:49-68): [shift * w^j]. */
void orc_eval_domain(int field, int log_n, uint32_t shift_mont, uint32_t generator,
                     uint32_t* out) {
  const fld* F = FLD(field);
  const int64_t n = (int64_t)1 << log_n;
  uint32_t w = log_n ? root_of_unity(F, log_n, generator) : F->one;
  uint32_t x = shift_mont ? shift_mont : F->one;
  for (int64_t j = 0; j < n; j++) {
    out[j] = x;
    x = fmul(F, x, w);
  }
}

/* ----------------------------------------------------------------- fold ---- */
/* fri_fold / fri_fold_values (zorch/coding/reed_solomon.py:543-548, 589-604):
 * g[j] = (f[j]+f[j+n/2])/2 + beta*(f[j]-f[j+n/2])/(2 x_j), x_j = shift*w_n^j,
 * shift = coset_shift^(2^level) (:331-339). */
int orc_fri_fold(int field, const uint32_t* cw, int64_t n, int ef_in, const uint32_t* beta,
                 int ef_beta, uint32_t shift_mont, uint32_t generator, uint32_t* out) {
  const fld* F = FLD(field);
  if (!is_pow2(n) || n < 2) return 2;
  int log_n = 0;
  while (((int64_t)1 << log_n) < n) log_n++;
  const int li = ef_in ? 4 : 1, lb = ef_beta ? 4 : 1, lo = (ef_in || ef_beta) ? 4 : 1;
  const int64_t half = n / 2;
  const uint32_t w = root_of_unity(F, log_n, generator);
  const uint32_t winv = finv(F, w);
  const uint32_t two = fadd(F, F->one, F->one);
  const uint32_t inv2 = finv(F, two);
  const uint32_t sh = shift_mont ? shift_mont : F->one;
  const uint32_t inv2s = fmul(F, inv2, finv(F, sh)); /* 1/(2 shift) */
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
  for (int64_t j = 0; j < half; j++) {
    uint32_t xinv = fmul(F, inv2s, fpow(F, winv, (uint64_t)j)); /* 1/(2 x_j) */
    uint32_t a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0}, sum[4], d[4], bt[4] = {0, 0, 0, 0};
    for (int e = 0; e < li; e++) {
      a[e] = cw[j * li + e];
      b[e] = cw[(j + half) * li + e];
    }
    for (int e = 0; e < lb; e++) bt[e] = beta[e];
    for (int e = 0; e < 4; e++) {
      sum[e] = fmul(F, fadd(F, a[e], b[e]), inv2);
      d[e] = fmul(F, fsub(F, a[e], b[e]), xinv);
    }
    uint32_t r[4];
    if (lo == 4) {
      ef4_mul(F, bt, d, r);
    } else {
      r[0] = fmul(F, bt[0], d[0]);
    }
    for (int e = 0; e < lo; e++) out[j * lo + e] = fadd(F, sum[e], r[e]);
  }
  return 0;
}

/* BitReversedReedSolomon.fold (zorch/coding/reed_solomon.py:484-492, 532-540)
 * on a bit-reversed layer: the pair (cw[2p], cw[2p+1]) = (f(x_p), f(-x_p)) with
 * x_p = shift * w_n^brev(p) (p read over log2(n/2) bits; x_0 = shift for n = 2),
 * folded by fri_fold_values (:543-548); the output is the next layer, again
 * bit-reversed. */
int orc_fri_fold_bitrev(int field, const uint32_t* cw, int64_t n, int ef_in, const uint32_t* beta,
                        int ef_beta, uint32_t shift_mont, uint32_t generator, uint32_t* out) {
  const fld* F = FLD(field);
  if (!is_pow2(n) || n < 2) return 2;
  int log_n = 0;
  while (((int64_t)1 << log_n) < n) log_n++;
  const int li = ef_in ? 4 : 1, lb = ef_beta ? 4 : 1, lo = (ef_in || ef_beta) ? 4 : 1;
  const int64_t half = n / 2;
  const uint32_t w = root_of_unity(F, log_n, generator);
  const uint32_t two = fadd(F, F->one, F->one);
  const uint32_t inv2 = finv(F, two);
  const uint32_t sh = shift_mont ? shift_mont : F->one;
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
  for (int64_t p = 0; p < half; p++) {
    const uint32_t x = fmul(F, sh, fpow(F, w, (uint64_t)brev64(p, log_n - 1)));
    const uint32_t xinv = finv(F, fmul(F, two, x)); /* 1/(2 x_p) */
    uint32_t a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0}, sum[4], d[4], bt[4] = {0, 0, 0, 0};
    for (int e = 0; e < li; e++) {
      a[e] = cw[(2 * p) * li + e];
      b[e] = cw[(2 * p + 1) * li + e];
    }
    for (int e = 0; e < lb; e++) bt[e] = beta[e];
    for (int e = 0; e < 4; e++) {
      sum[e] = fmul(F, fadd(F, a[e], b[e]), inv2);
      d[e] = fmul(F, fsub(F, a[e], b[e]), xinv);
    }
    uint32_t r[4];
    if (lo == 4) {
      ef4_mul(F, bt, d, r);
    } else {
      r[0] = fmul(F, bt[0], d[0]);
    }
    for (int e = 0; e < lo; e++) out[p * lo + e] = fadd(F, sum[e], r[e]);
  }
  return 0;
}

/* k-ary fold (ReedSolomon.fold_group, zorch/coding/reed_solomon.py:357-381,
 * fri_fold_k points= path :551-586, compute_lagrange_basis
 * zorch/poly/univariate.py:56-65): group p < n/k is
 * (cw[p], cw[p + n/k], ..., cw[p + (k-1)n/k]) on the points
 * x_m = shift w_n^(p + m n/k); out[p] = sum_m g_m L_m(beta), L_m the Lagrange
 * basis of the group's points. Values and beta EF4 or base; x base. */
int orc_fri_fold_k(int field, const uint32_t* cw, int64_t n, int ef_in, const uint32_t* beta,
                   int ef_beta, int log_k, uint32_t shift_mont, uint32_t generator,
                   uint32_t* out) {
  const fld* F = FLD(field);
  const int k = 1 << log_k;
  if (!is_pow2(n) || n < k || log_k < 1 || log_k > 6) return 2;
  int log_n = 0;
  while (((int64_t)1 << log_n) < n) log_n++;
  const int li = ef_in ? 4 : 1, lb = ef_beta ? 4 : 1, lo = (ef_in || ef_beta) ? 4 : 1;
  const int64_t sub = n / k;
  const uint32_t w = root_of_unity(F, log_n, generator);
  const uint32_t sh = shift_mont ? shift_mont : F->one;
  uint32_t bt[4] = {0, 0, 0, 0};
  for (int e = 0; e < lb; e++) bt[e] = beta[e];
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
  for (int64_t p = 0; p < sub; p++) {
    uint32_t x[64];
    for (int m = 0; m < k; m++) x[m] = fmul(F, sh, fpow(F, w, (uint64_t)(p + m * sub)));
    uint32_t acc[4] = {0, 0, 0, 0};
    for (int m = 0; m < k; m++) {
      /* L_m(beta) = prod_{j != m} (beta - x_j) / (x_m - x_j) */
      uint32_t num[4] = {F->one, 0, 0, 0};
      uint32_t den = F->one;
      for (int j = 0; j < k; j++) {
        if (j == m) continue;
        uint32_t d[4];
        memcpy(d, bt, 16);
        d[0] = fsub(F, d[0], x[j]);
        ef4_mul(F, num, d, num);
        den = fmul(F, den, fsub(F, x[m], x[j]));
      }
      const uint32_t dinv = finv(F, den);
      for (int e = 0; e < 4; e++) num[e] = fmul(F, num[e], dinv);
      uint32_t g[4] = {0, 0, 0, 0};
      for (int e = 0; e < li; e++) g[e] = cw[(p + m * sub) * li + e];
      uint32_t t[4];
      ef4_mul(F, g, num, t);
      for (int e = 0; e < 4; e++) acc[e] = fadd(F, acc[e], t[e]);
    }
    for (int e = 0; e < lo; e++) out[p * lo + e] = acc[e];
  }
  return 0;
}

/* SingleMatrixCommitmentScheme.bind_root (zorch/commit/smcs.py:118-140):
 * compress([raw_root, sponge([log_height, width])]), the two shape words as
 * field elements. */
void orc_smcs_bind_root(const orc_p2* P, const uint32_t* raw_root, uint32_t log_height,
                        uint32_t width, uint32_t* out8) {
  const fld* F = FLD(P->field);
  const uint32_t shape[2] = {to_m(F, log_height), to_m(F, width)};
  uint32_t params[8];
  orc_sponge_hash(P, shape, 2, params);
  orc_compress(P, raw_root, params, out8);
}

/* sample_rlc_coeffs_bits + batch_staggered (zorch/pcs/jagged/open.py:88-105,
 * zorch/pcs/basefold/batching.py:66-80): eq(., r) over nbv = ceil(log2 w) EF4
 * challenges expanded MSB-first (zorch/poly/eq.py:55-62, 92-115), column c
 * weighted by entry c of the table. */
void orc_rlc_columns(int field, const uint32_t* cw, int64_t n, int w, const uint32_t* chal,
                     uint32_t* out) {
  const fld* F = FLD(field);
  int nbv = 0;
  while ((1 << nbv) < w) nbv++;
  uint32_t* st = (uint32_t*)calloc((size_t)4 << nbv, sizeof(uint32_t));
  st[0] = F->one;
  for (int j = 0; j < nbv; j++) {
    uint32_t* nx = (uint32_t*)calloc((size_t)4 << (j + 1), sizeof(uint32_t));
    for (int i = 0; i < (1 << j); i++) {
      uint32_t hi[4], lo[4];
      ef4_mul(F, st + 4 * i, chal + 4 * j, hi);
      for (int e = 0; e < 4; e++) lo[e] = fsub(F, st[4 * i + e], hi[e]);
      memcpy(nx + 4 * (2 * i), lo, 16);
      memcpy(nx + 4 * (2 * i + 1), hi, 16);
    }
    memcpy(st, nx, sizeof(uint32_t) * ((size_t)4 << (j + 1)));
    free(nx);
  }
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
  for (int64_t j = 0; j < n; j++) {
    uint32_t r[4] = {0, 0, 0, 0};
    for (int c = 0; c < w; c++)
      for (int e = 0; e < 4; e++) r[e] = fadd(F, r[e], fmul(F, st[4 * c + e], cw[(int64_t)c * n + j]));
    memcpy(out + 4 * j, r, 16);
  }
  free(st);
}

/* ------------------------------------------------------------ sumcheck ---- */
static void ef4_add(const fld* F, const uint32_t* a, const uint32_t* b, uint32_t* c) {
  for (int e = 0; e < 4; e++) c[e] = fadd(F, a[e], b[e]);
}
static void ef4_sub(const fld* F, const uint32_t* a, const uint32_t* b, uint32_t* c) {
  for (int e = 0; e < 4; e++) c[e] = fsub(F, a[e], b[e]);
}

/* a^(p^4 - 2) = a^-1 in EF4 (a != 0). */
void orc_ef4_inv(int field, const uint32_t* a, uint32_t* out) {
  const fld* F = FLD(field);
  unsigned __int128 e = (unsigned __int128)F->p * F->p;
  e = e * F->p * F->p - 2;
  uint32_t r[4] = {F->one, 0, 0, 0}, b[4];
  memcpy(b, a, 16);
  while (e) {
    if (e & 1) ef4_mul(F, r, b, r);
    ef4_mul(F, b, b, b);
    e >>= 1;
  }
  memcpy(out, r, 16);
}

/* f(z) for an EF4 point z: Horner over the base coefficients
 * (_eval_poly, zorch/pcs/fri/prover.py:42-49, with z in the extension). */
void orc_eval_poly_ef4(int field, const uint32_t* coeffs, int64_t k, const uint32_t* z,
                       uint32_t* out) {
  const fld* F = FLD(field);
  uint32_t acc[4] = {0, 0, 0, 0};
  for (int64_t i = k - 1; i >= 0; i--) {
    ef4_mul(F, acc, z, acc);
    acc[0] = fadd(F, acc[0], coeffs[i]);
  }
  memcpy(out, acc, 16);
}

/* The DEEP quotient of _open_one (zorch/pcs/fri/prover.py:160-164):
 * out[j] = (cw[j] - v) / (x_j - z) with x_j = shift * w^j (natural order) or
 * shift * w^brev(j) (bit-reversed codeword), z and v of z_limbs (1 or 4)
 * limbs; out has z_limbs limbs per element. Inverses by blocks of 1024:
 * prefix products, one inversion per block (Fermat), back substitution; a zero
 * denominator gives a zero quotient. */
int orc_deep_quotient(int field, const uint32_t* cw, int64_t n, const uint32_t* z, int z_limbs,
                      const uint32_t* v, uint32_t shift_mont, uint32_t generator, int bitrev,
                      uint32_t* out) {
  const fld* F = FLD(field);
  if (!is_pow2(n) || (z_limbs != 1 && z_limbs != 4)) return 1;
  int log_n = 0;
  while (((int64_t)1 << log_n) < n) log_n++;
  const uint32_t w = log_n ? root_of_unity(F, log_n, generator) : F->one;
  const uint32_t sh = shift_mont ? shift_mont : F->one;
  const int64_t B = 1024;
  const int64_t nblocks = (n + B - 1) / B;
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
  for (int64_t b = 0; b < nblocks; b++) {
    uint32_t(*den)[4] = malloc(sizeof(uint32_t[4]) * (size_t)B);
    uint32_t(*pre)[4] = malloc(sizeof(uint32_t[4]) * (size_t)B);
    char* zero = malloc((size_t)B);
    const int64_t j0 = b * B;
    const int64_t m = n - j0 < B ? n - j0 : B;
    uint32_t acc[4] = {F->one, 0, 0, 0};
    for (int64_t i = 0; i < m; i++) {
      const int64_t j = j0 + i;
      const int64_t e = bitrev ? brev64(j, log_n) : j;
      const uint32_t x = fmul(F, sh, fpow(F, w, (uint64_t)e));
      uint32_t d[4] = {fsub(F, x, z[0]), 0, 0, 0};
      if (z_limbs == 4)
        for (int l = 1; l < 4; l++) d[l] = fsub(F, 0, z[l]);
      zero[i] = (d[0] | d[1] | d[2] | d[3]) == 0;
      if (zero[i]) d[0] = F->one;
      memcpy(den[i], d, 16);
      ef4_mul(F, acc, d, acc);
      memcpy(pre[i], acc, 16);
    }
    uint32_t inv[4];
    if (z_limbs == 1) {
      inv[0] = finv(F, acc[0]);
      inv[1] = inv[2] = inv[3] = 0;
    } else {
      orc_ef4_inv(field, acc, inv);
    }
    for (int64_t i = m - 1; i >= 0; i--) {
      uint32_t di[4];
      if (i) ef4_mul(F, inv, pre[i - 1], di);
      else memcpy(di, inv, 16);
      if (i) ef4_mul(F, inv, den[i], inv);
      uint32_t num[4] = {fsub(F, cw[j0 + i], v[0]), 0, 0, 0};
      if (z_limbs == 4)
        for (int l = 1; l < 4; l++) num[l] = fsub(F, 0, v[l]);
      uint32_t q[4];
      ef4_mul(F, num, di, q);
      if (zero[i]) q[0] = q[1] = q[2] = q[3] = 0;
      memcpy(out + (j0 + i) * z_limbs, q, sizeof(uint32_t) * (size_t)z_limbs);
    }
    free(den);
    free(pre);
    free(zero);
  }
  return 0;
}

/* expand_eq_to_hypercube(z, 1) (zorch/poly/eq.py:92-130, expand_hypercube_step
 * :55-62): eq(w, z) for w in {0,1}^m, z[0] on the most significant index bit;
 * each step splits an entry s into (s - s z_j, s z_j) at (2i, 2i+1). */
void orc_eq_expand(int field, const uint32_t* z, int m, uint32_t* out) {
  const fld* F = FLD(field);
  out[0] = F->one;
  out[1] = out[2] = out[3] = 0;
  for (int j = 0; j < m; j++) {
    for (int64_t i = ((int64_t)1 << j) - 1; i >= 0; i--) {
      uint32_t s[4], hi[4], lo[4];
      memcpy(s, out + 4 * i, 16);
      ef4_mul(F, s, z + 4 * j, hi);
      ef4_sub(F, s, hi, lo);
      memcpy(out + 4 * (2 * i), lo, 16);
      memcpy(out + 4 * (2 * i + 1), hi, 16);
    }
  }
}

/* eval_mle (zorch/poly/multilinear.py:92-98) of w base columns [w][2^m] at
 * the EF4 point z: out[c] = sum_i eq(i, z) cols[c][i]. */
void orc_eval_mle_base(int field, const uint32_t* cols, int w, int m, const uint32_t* z,
                       uint32_t* out) {
  const fld* F = FLD(field);
  const int64_t S = (int64_t)1 << m;
  uint32_t* eq = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (size_t)S);
  orc_eq_expand(field, z, m, eq);
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
  for (int c = 0; c < w; c++) {
    uint32_t acc[4] = {0, 0, 0, 0};
    for (int64_t i = 0; i < S; i++)
      for (int e = 0; e < 4; e++)
        acc[e] = fadd(F, acc[e], fmul(F, eq[4 * i + e], cols[(int64_t)c * S + i]));
    memcpy(out + 4 * c, acc, 16);
  }
  free(eq);
}

/* eval_mle of one EF4 MLE [2^m] at the EF4 point z (m = 0: mle[0]). */
void orc_eval_mle_ef4(int field, const uint32_t* mle, int m, const uint32_t* z, uint32_t* out) {
  const fld* F = FLD(field);
  const int64_t M = (int64_t)1 << m;
  uint32_t* eq = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (size_t)M);
  orc_eq_expand(field, z, m, eq);
  uint32_t acc[4] = {0, 0, 0, 0};
  for (int64_t i = 0; i < M; i++) {
    uint32_t t[4];
    ef4_mul(F, eq + 4 * i, mle + 4 * i, t);
    ef4_add(F, acc, t, acc);
  }
  memcpy(out, acc, 16);
  free(eq);
}

/* mle_fold (zorch/poly/multilinear.py:101-109): out[i] = mle[2i] + beta mle[2i+1],
 * EF4 entries, beta EF4 (a base beta as [b, 0, 0, 0]). */
void orc_mle_fold(int field, const uint32_t* mle, int64_t M, const uint32_t* beta,
                  uint32_t* out) {
  const fld* F = FLD(field);
  for (int64_t i = 0; i < M / 2; i++) {
    uint32_t t[4];
    ef4_mul(F, beta, mle + 4 * (2 * i + 1), t);
    ef4_add(F, mle + 4 * (2 * i), t, out + 4 * i);
  }
}

/* batch_staggered (zorch/pcs/basefold/batching.py:66-80) of one matrix's w
 * base columns [w][n] with partial_lagrange weights over nbv EF4 challenges,
 * the matrix taking weights offset .. offset+w-1; accumulate adds onto out. */
void orc_rlc_columns_ex(int field, const uint32_t* cw, int64_t n, int w, const uint32_t* chal,
                        int nbv, int offset, int accumulate, uint32_t* out) {
  const fld* F = FLD(field);
  uint32_t* wt = (uint32_t*)malloc(sizeof(uint32_t) * 4 * ((size_t)1 << nbv));
  orc_eq_expand(field, chal, nbv, wt);
#pragma omp parallel for num_threads(orc_get_threads()) schedule(static)
  for (int64_t j = 0; j < n; j++) {
    uint32_t r[4] = {0, 0, 0, 0};
    if (accumulate) memcpy(r, out + 4 * j, 16);
    for (int c = 0; c < w; c++)
      for (int e = 0; e < 4; e++)
        r[e] = fadd(F, r[e], fmul(F, wt[4 * (offset + c) + e], cw[(int64_t)c * n + j]));
    memcpy(out + 4 * j, r, 16);
  }
  free(wt);
}

/* ----------------------------------------------------------- transcript ---- */
/* DuplexTranscript (zorch/transcript.py:239-481), width 16, rate 8. */
void orc_duplex_init(orc_duplex* t) { memset(t, 0, sizeof(*t)); }

/* _observe_body (zorch/transcript.py:637-748): full rate blocks of the stream
 * in_buf[0:in_pos] ++ values overwrite sponge[0:8] and permute; the tail stays
 * pending; out_pos = rate (fresh output) iff no tail remains. */
void orc_duplex_observe(const orc_p2* P, orc_duplex* t, const uint32_t* v, int64_t m) {
  if (m == 0) return;
  int64_t pos = t->in_pos;
  int permuted = 0;
  uint32_t buf[8];
  memcpy(buf, t->in_buf, 32);
  for (int64_t i = 0; i < m; i++) {
    buf[pos++] = v[i];
    if (pos == 8) {
      memcpy(t->sponge, buf, 32);
      orc_p2_permute(P, t->sponge);
      pos = 0;
      permuted = 1;
    }
  }
  (void)permuted;
  for (int64_t i = pos; i < 8; i++) buf[i] = 0;
  memcpy(t->in_buf, buf, 32);
  t->in_pos = (int32_t)pos;
  if (pos == 0) {
    memcpy(t->out_buf, t->sponge, 32);
    t->out_pos = 8;
  } else {
    memset(t->out_buf, 0, 32);
    t->out_pos = 0;
  }
}

/* _sample_one (zorch/transcript.py:370-387) n times; _duplexing (:299-313)
 * merges the pending prefix over sponge[0:in_pos] (:154-163) and permutes. */
void orc_duplex_sample(const orc_p2* P, orc_duplex* t, int n, uint32_t* out) {
  for (int k = 0; k < n; k++) {
    if (t->in_pos > 0 || t->out_pos == 0) {
      for (int i = 0; i < t->in_pos; i++) t->sponge[i] = t->in_buf[i];
      orc_p2_permute(P, t->sponge);
      memset(t->in_buf, 0, 32);
      memcpy(t->out_buf, t->sponge, 32);
      t->in_pos = 0;
      t->out_pos = 8;
    }
    t->out_pos -= 1;
    out[k] = t->out_buf[t->out_pos];
  }
}

/* Proof-of-work grind (DuplexTranscript._grind_search / grind,
 * zorch/transcript.py:439-481, over grind_search, zorch/grind.py:66-93):
 * the lowest canonical witness w in [0, p) whose challenge -- observe w as a
 * field element, sample once -- has `pow_bits` zero low canonical bits
 * (_pow_satisfied, zorch/transcript.py:44-49). 0 when none passes (the
 * unchecked fallback). Each candidate replays the transcript literally: copy,
 * observe, sample. */
uint32_t orc_duplex_grind(const orc_p2* P, const orc_duplex* t, int pow_bits) {
  const uint32_t mask = (uint32_t)((1ull << pow_bits) - 1);
  const uint32_t mod = orc_modulus(P->field);
  for (uint32_t w = 0; w < mod; w++) {
    orc_duplex c = *t;
    const uint32_t v = orc_to_mont(P->field, w);
    uint32_t s;
    orc_duplex_observe(P, &c, &v, 1);
    orc_duplex_sample(P, &c, 1, &s);
    if ((orc_from_mont(P->field, s) & mask) == 0) return w;
  }
  return 0;
}

/* --------------------------------------------------- FRI commit phase ---- */
/* fold_rounds(PreFoldPairCommitRound) (zorch/prove.py:26-37,
 * zorch/pcs/fold.py:90-115) over the codeword, each round: pair_leaves
 * (zorch/coding/reed_solomon.py:303-307) -> to_base_field (zorch/pcs/fold.py:42-52)
 * -> Merkle commit -> observe(root) -> beta (one base squeeze, or an EF4
 * challenge of 4 squeezes as sample_challenge, zorch/transcript.py:122-137)
 * -> fold. Then observe(final layer), sample_positions (zorch/pcs/fold.py:173-182),
 * layer_positions (zorch/coding/reed_solomon.py:320-329) and open_rows
 * (zorch/pcs/fold.py:142-149) per layer, as in _open_one
 * (zorch/pcs/fri/prover.py:151-187).
 * rows: per layer [Q][2*limbs_i]; paths: per layer [depth_i][Q][8]. */
int orc_fri_commit_phase(const orc_p2* P, int field, const uint32_t* codeword, int log_n,
                         int ef_in, uint32_t shift_mont, uint32_t generator, int num_rounds,
                         int num_queries, int beta_limbs, orc_duplex* t, uint32_t* roots,
                         uint32_t* betas, uint32_t* final_layer, int32_t* positions,
                         uint32_t* rows, uint32_t* paths) {
  const fld* F = FLD(field);
  if (num_rounds < 0 || num_rounds >= log_n) return 1;
  const int64_t n0 = (int64_t)1 << log_n;
  uint32_t** cws = (uint32_t**)calloc((size_t)num_rounds + 1, sizeof(uint32_t*));
  uint32_t** lays = (uint32_t**)calloc((size_t)num_rounds + 1, sizeof(uint32_t*));
  int* limbs = (int*)calloc((size_t)num_rounds + 1, sizeof(int));
  limbs[0] = ef_in ? 4 : 1;
  cws[0] = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n0 * limbs[0]);
  memcpy(cws[0], codeword, sizeof(uint32_t) * (size_t)n0 * limbs[0]);
  uint32_t shift = shift_mont ? shift_mont : F->one;
  for (int r = 0; r < num_rounds; r++) {
    const int64_t n = n0 >> r, L = n / 2;
    lays[r] = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(2 * L - 1) * 8);
    /* pair leaf p = (cw[p], cw[p + n/2]) in base limbs: 2 groups of `limbs` */
    orc_merkle_commit(P, cws[r], L, 2, limbs[r], L * limbs[r], lays[r]);
    const uint32_t* root = lays[r] + (2 * L - 2) * 8;
    memcpy(roots + 8 * r, root, 32);
    orc_duplex_observe(P, t, root, 8);
    uint32_t beta[4] = {0, 0, 0, 0};
    orc_duplex_sample(P, t, beta_limbs, beta);
    memcpy(betas + 4 * r, beta, 16);
    limbs[r + 1] = (limbs[r] == 4 || beta_limbs == 4) ? 4 : 1;
    cws[r + 1] = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n / 2) * limbs[r + 1]);
    orc_fri_fold(field, cws[r], n, limbs[r] == 4, beta, beta_limbs == 4, shift, generator,
                 cws[r + 1]);
    shift = fmul(F, shift, shift);
  }
  const int64_t nf = n0 >> num_rounds;
  memcpy(final_layer, cws[num_rounds], sizeof(uint32_t) * (size_t)nf * limbs[num_rounds]);
  orc_duplex_observe(P, t, cws[num_rounds], nf * limbs[num_rounds]);
  uint32_t* raw = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(num_queries > 0 ? num_queries : 1));
  orc_duplex_sample(P, t, num_queries, raw);
  for (int q = 0; q < num_queries; q++) positions[q] = (int32_t)(raw[q] % (uint32_t)n0);
  free(raw);
  int32_t* a = (int32_t*)malloc(sizeof(int32_t) * (size_t)(num_queries > 0 ? num_queries : 1));
  for (int q = 0; q < num_queries; q++) a[q] = positions[q];
  int64_t row_off = 0, path_off = 0;
  for (int r = 0; r < num_rounds; r++) {
    const int64_t n = n0 >> r, L = n / 2;
    for (int q = 0; q < num_queries; q++) a[q] = (int32_t)(a[q] % L);
    orc_merkle_open(cws[r], L, 2, limbs[r], L * limbs[r], lays[r], a, num_queries,
                    rows + row_off, paths + path_off);
    int depth = 0;
    while (((int64_t)1 << depth) < L) depth++;
    row_off += (int64_t)num_queries * 2 * limbs[r];
    path_off += (int64_t)depth * num_queries * 8;
  }
  free(a);
  for (int r = 0; r <= num_rounds; r++) free(cws[r]);
  for (int r = 0; r < num_rounds; r++) free(lays[r]);
  free(cws);
  free(lays);
  free(limbs);
  return 0;
}
