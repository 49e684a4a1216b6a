/*
 * heu_gb300 — C-ABI of a GB300 (sm_103a) Paillier engine with HEU
 * `paillier_z` (ZPaillier, DJN-optimised Paillier) semantics.
 *
 * This is the device boundary a HEU schema adapter binds: plain pointers,
 * sizes and int status codes, no C++ or torch types.  It replaces the
 * reference's only device boundary, the CGBN C-ABI of `paillier_g`
 * (heu/library/algorithms/paillier_gpu/gpulib/gpupaillier.h:46-91), and is
 * called from the vectorized (span-of-pointers) SPI
 * (heu/library/algorithms/clean_template/vector_encryptor.h:24-33,
 *  vector_decryptor.h:25-31, vector_evaluator.h:24-66).
 *
 * Data formats (all little-endian 32-bit limbs, `k` = key bits = bitlen(n)):
 *   ciphertext  S = k/16 limbs (k/4 bytes), stored in Montgomery form
 *               c*R mod n^2 with R = 2^(32*S) — the representation HEU keeps
 *               in paillier_z `Ciphertext::c_` (encryptor.cc:46-49).
 *               hg_to_mont / hg_from_mont convert to and from the canonical
 *               Z-form c in [0, n^2).
 *   plaintext   int64_t, or (magnitude of k/32 limbs, sign byte) for the
 *               full range |m| <= n/2 (public_key.h:50-54).
 *   randomness  r of k/2 bits as k/64 limbs per ciphertext (the value
 *               `BigInt::RandomExactBits(k/2)` draws in encryptor.cc:26-31),
 *               injected by the caller so results are reproducible.
 *
 * Calls named hg_<op> take HOST pointers and are synchronous.  Calls named
 * hg_dev_<op> take DEVICE pointers and are asynchronous on `stream` (a
 * cudaStream_t passed as void*; NULL = the context's own stream).
 *
 * Every function returns HG_OK (0) or an HG_ERR_* code; hg_last_error()
 * gives the message of the calling thread's last failure.
 */
#ifndef HEU_GB300_H_
#define HEU_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HG_OK 0
#define HG_ERR_INVALID 1        /* bad argument (null pointer, unknown key, size) */
#define HG_ERR_CT_RANGE 2       /* a ciphertext >= n^2 (decryptor.cc:21-23) */
#define HG_ERR_PT_RANGE 3       /* plaintext |m| > n/2 (encryptor.cc:38-40) */
#define HG_ERR_NOMEM 4          /* device or host allocation failed */
#define HG_ERR_CUDA 5           /* CUDA runtime error */
#define HG_ERR_NOT_INVERTIBLE 6 /* gcd(c, n) != 1 in Negate/Sub/Mul(k<0) */
#define HG_ERR_NO_SECRET 7      /* decrypt on a key loaded without p, q */
#define HG_ERR_UNSUPPORTED 8    /* key size without a compiled variant */

typedef struct hg_ctx hg_ctx;

/* ---- context -------------------------------------------------------------
 * Replaces gpu_setcard / gpu_release_context (gpupaillier.h:47-48, declared
 * but never defined in the reference) and the per-call cudaSetDevice(0) +
 * cudaMalloc/cudaFree of paillier.cu:565-632.                               */
int hg_ctx_create(int device, hg_ctx** out);
int hg_ctx_destroy(hg_ctx* ctx);
const char* hg_last_error(void);
int hg_device_sm_count(hg_ctx* ctx);

/* ---- keys ----------------------------------------------------------------
 * hg_keygen follows paillier_zahlen/key_generator.cc:26-60 on the host with
 * every random draw taken from a seeded xoshiro256** stream (seed given) —
 * the reference draws from yacl's RNG instead.  Outputs: n (k/32 limbs),
 * p and q (k/64 limbs each), h_s = (-x^2)^n mod n^2 (k/16 limbs).          */
int hg_keygen(uint32_t key_bits, uint64_t seed, uint32_t* n_out, uint32_t* p_out, uint32_t* q_out,
              uint32_t* hs_out);

/* Loads a key and uploads its precompute: Montgomery constants mod n^2
 * (PublicKey::Init, public_key.cc:28-40), the fixed-base table of h_s
 * powers with `table_window` bits per digit (0 = default; the reference's
 * SetCacheTableDensity, public_key.cc:19-26, default 10), and, if p and q
 * are given, the CRT constants of SecretKey::Init (secret_key.cc:19-43).
 * p, q may be NULL for a public-key-only key.                              */
int hg_key_load(hg_ctx* ctx, uint32_t key_bits, const uint32_t* n, const uint32_t* h_s, const uint32_t* p,
                const uint32_t* q, int table_window, int* key_id);
int hg_key_free(hg_ctx* ctx, int key_id);

/* ---- Okamoto-Uchiyama keys ------------------------------------------------
 * No counterpart in HEU's GPU code: the engine also serves HEU's OU scheme
 * (heu/library/algorithms/ou).  hg_ou_keygen follows ou/key_generator.cc:
 * 26-96 with every random draw from a seeded xoshiro256** stream.  n = p^2 q,
 * G, H: S limbs (S = 64 for 1024-bit keys, 128 for 2048 / 3072); p, q, t
 * (the large prime factor of p - 1), gp_inv: S/2 limbs; max_pt_bits:
 * log2 of the plaintext bound (ou/key_generator.cc:86).
 * hg_ou_key_load uploads the fixed-base tables of H (randomness, < 2^128), G
 * and G^-1 (plaintexts) and, if the secret part is given, the decryption
 * constants.  The returned key id works with hg_encrypt / encrypt_bn /
 * encrypt_zero / randomize / decrypt / decrypt_bn / add / add_plain / sub /
 * sub_plain / plain_sub / mul / negate / sum / bucket_sum / matmul / to_mont /
 * from_mont and their hg_dev_ forms, with OU semantics (ou/encryptor.cc,
 * decryptor.cc, evaluator.cc): c = H^r G^m mod n in Montgomery form with
 * R = 2^(32 S); r < 2^80 / 2^110 / 2^128 by key size (4 limbs per r);
 * plaintexts |m| <= 2^max_pt_bits.  Batches, the server and the autotuner
 * serve ZPaillier keys only (HG_ERR_UNSUPPORTED otherwise).                */
int hg_ou_keygen(uint32_t key_bits, uint64_t seed, uint32_t* n_out, uint32_t* G_out, uint32_t* H_out,
                 uint32_t* p_out, uint32_t* q_out, uint32_t* t_out, uint32_t* gpinv_out, int* max_pt_bits);
int hg_ou_key_load(hg_ctx* ctx, uint32_t key_bits, const uint32_t* n, const uint32_t* G, const uint32_t* H,
                   int max_pt_bits, const uint32_t* p, const uint32_t* q, const uint32_t* t, const uint32_t* gp_inv,
                   int table_window, int* key_id);
/* limbs of one ciphertext (S) and of one r value for a loaded key */
int hg_key_shape(hg_ctx* ctx, int key_id, int* ct_limbs, int* r_limbs, int* pt_limbs);

/* ---- encryption (replaces gpu_paillier_enc, gpupaillier.h:50-52) ---------
 * c = (1 + m*n) * h_s^r mod n^2, output in Montgomery form
 * (paillier_zahlen/encryptor.cc:36-56).                                   */
int hg_encrypt(hg_ctx* ctx, int key_id, const int64_t* m, const uint32_t* r, uint32_t* ct_out, size_t count);
int hg_encrypt_bn(hg_ctx* ctx, int key_id, const uint32_t* m_mag, const uint8_t* m_neg, const uint32_t* r,
                  uint32_t* ct_out, size_t count);
/* EncryptZero: h_s^r (encryptor.cc:33; vector_encryptor.h:28)              */
int hg_encrypt_zero(hg_ctx* ctx, int key_id, const uint32_t* r, uint32_t* ct_out, size_t count);
/* Randomize: c * h_s^r in place (evaluator.cc:25-28)                        */
int hg_randomize(hg_ctx* ctx, int key_id, uint32_t* ct, const uint32_t* r, size_t count);

/* ---- decryption (replaces gpu_paillier_dec, gpupaillier.h:53-55) ---------
 * CRT over p^2 and q^2 (paillier_zahlen/decryptor.cc:32-53).  The int64
 * form sets overflow[i] = 1 where the plaintext does not fit in int64 (the
 * range check of numpy DecryptInRange, numpy/decryptor.cc:86-99).        */
int hg_decrypt(hg_ctx* ctx, int key_id, const uint32_t* ct, int64_t* m_out, uint8_t* overflow, size_t count);
int hg_decrypt_bn(hg_ctx* ctx, int key_id, const uint32_t* ct, uint32_t* m_mag, uint8_t* m_neg, size_t count);

/* Montgomery radix at the boundary.  Ciphertexts here are c * R mod n^2
 * with R = 2^(32 S) (S = 32-bit limbs of n^2), which is the radix of a
 * yacl BigInt backend with 32- or 64-bit limbs (OpenSSL, GMP: R =
 * 2^(64 * ceil(bits(n^2) / 64)), the same for key sizes that are multiples
 * of 64 bits).  A HEU build whose backend uses another radix (libtommath's
 * 60-bit digits: R = 2^(60 * ceil(bits(n^2) / 60))) converts its
 * ciphertexts with this call: to_external = 1 maps c * R to c * 2^radix_bits
 * mod n^2, 0 maps back (one Montgomery multiplication by a constant). */
int hg_convert_radix(hg_ctx* ctx, int key_id, const uint32_t* in, uint32_t* out, size_t count, uint32_t radix_bits,
                     int to_external);

/* ---- plaintext encodings on the device ----------------------------------
 * HEU's PlainEncoder (phe/encoding/plain_encoder.h:46-74, pylib's
 * IntegerEncoder / FloatEncoder) and BatchEncoder (phe/encoding/
 * batch_encoder.h:27-140) run inside the encryption and decryption kernels,
 * so raw int64 / double values go in and out with no host encode pass.
 *   HG_CODEC_PLAIN_I64: value * scale (exact 128-bit product); decode
 *     m / scale with C++ division (toward zero), flagged in `overflow` when
 *     it does not fit int64.
 *   HG_CODEC_PLAIN_F64: trunc(value * scale) as an integer of any size
 *     (non-finite values fail with HG_ERR_PT_RANGE); decode double(m)
 *     (nearest-even) / scale, flagged when beyond the double range.
 *   HG_CODEC_BATCH_I64 / _F64: two values per plaintext, (b * scale) <<
 *     (64 + padding_bits) | (a * scale) on 64-bit two's complement patterns
 *     (doubles: int64(trunc(x * scale))); decode slot s = the low 64 bits of
 *     m >> s * (64 + padding_bits) as int64, / scale (int64 division, or
 *     double division for _F64), slot 0 into `out`, slot 1 into `out2`.
 * `values` / `out` hold int64 or double per the codec (8 bytes each);
 * values2 / out2 are the second slots (batch codecs only).  Plaintexts above
 * n/2 fail with HG_ERR_PT_RANGE as in hg_encrypt.  ZPaillier keys only. */
#define HG_CODEC_PLAIN_I64 1
#define HG_CODEC_PLAIN_F64 2
#define HG_CODEC_BATCH_I64 3
#define HG_CODEC_BATCH_F64 4
int hg_encrypt_encoded(hg_ctx* ctx, int key_id, int codec, int64_t scale, int padding_bits, const void* values,
                       const void* values2, const uint32_t* r, uint32_t* ct_out, size_t count);
int hg_decrypt_decoded(hg_ctx* ctx, int key_id, int codec, int64_t scale, int padding_bits, const uint32_t* ct,
                       void* out, void* out2, uint8_t* overflow, size_t count);

/* ---- evaluator (replaces gpu_paillier_e_add / e_add_const / sub_ct /
 * sub_ctpt / sub_ptct / e_mul_const / e_inverse, gpupaillier.h:57-90) ---- */
int hg_add(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t count);
int hg_add_plain(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, uint32_t* out, size_t count);
int hg_sub(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t count);
int hg_sub_plain(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, uint32_t* out, size_t count);
int hg_plain_sub(hg_ctx* ctx, int key_id, const int64_t* p, const uint32_t* a, uint32_t* out, size_t count);
int hg_mul(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* k, uint32_t* out, size_t count);
/* Mul(ct, BigInt k) (paillier_zahlen/evaluator.cc:99-123, which takes a
 * scalar of any size: "ciphertext overflow is allowed"): k[i] = (k_neg[i] ?
 * -1 : 1) * the little-endian magnitude k_mag[i * k_limbs .. +k_limbs),
 * 1 <= k_limbs <= S (scalars up to the width of n^2).  Same results as
 * hg_mul where k fits int64. */
int hg_mul_bn(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* k_mag, const uint8_t* k_neg,
              size_t k_limbs, uint32_t* out, size_t count);
int hg_negate(hg_ctx* ctx, int key_id, const uint32_t* a, uint32_t* out, size_t count);

/* ---- heu.numpy reductions (numpy/evaluator.cc:355-373 Sum; the optional
 * vectorized ReduceSum hook numpy MatMul detects, evaluator.cc:250-260) --- */
int hg_sum(hg_ctx* ctx, int key_id, const uint32_t* a, size_t count, uint32_t* out);

/* FeatureWiseBucketSum (numpy/evaluator.cc:378-458; pylib
 * extension_functions.cc:80-98): x is rows x cols ciphertexts (row-major),
 * order_map rows x features bin ids (row-major), out (features*bucket_num) x
 * cols; row f*bucket_num+b of out is the product of x(i, col) over rows with
 * order_map(i, f) == b, or the Montgomery identity (GetZero,
 * numpy/evaluator.h:84-87) for an empty bucket; cumsum != 0 turns bucket b
 * into the product of buckets 0..b (evaluator.cc:444-449).  The reference's
 * order map is int8 (numpy/evaluator.h:21-23) and cannot hold bin ids >= 128;
 * this one is uint8 with bucket_num <= 256.                                 */
int hg_bucket_sum(hg_ctx* ctx, int key_id, const uint32_t* x, size_t rows, size_t cols, const uint8_t* order_map,
                  size_t features, int bucket_num, int cumsum, uint32_t* out);
/* MatMul of ciphertexts x (M x K, row-major) by int64 plaintexts y (K x N,
 * row-major): out(i,j) = prod_k x(i,k)^y(k,j) (numpy/evaluator.cc:208-353,
 * the vectorized Mul + ReduceSum path).  pt x ct is the transpose.        */
int hg_matmul(hg_ctx* ctx, int key_id, const uint32_t* x, size_t M, size_t K, const int64_t* y, size_t N,
              uint32_t* out);
/* MatMul with plaintexts of any size (numpy/evaluator.cc:208-353 takes any
 * PMatrix): y(k,j) = (y_neg ? -1 : 1) * magnitude of y_limbs little-endian
 * limbs at y_mag[(k * N + j) * y_limbs], 1 <= y_limbs <= S. */
int hg_matmul_bn(hg_ctx* ctx, int key_id, const uint32_t* x, size_t M, size_t K, const uint32_t* y_mag,
                 const uint8_t* y_neg, size_t y_limbs, size_t N, uint32_t* out);

/* ---- representation ----------------------------------------------------- */
int hg_to_mont(hg_ctx* ctx, int key_id, const uint32_t* z, uint32_t* mont, size_t count);
int hg_from_mont(hg_ctx* ctx, int key_id, const uint32_t* mont, uint32_t* z, size_t count);

/* ---- per-key tuning (no counterpart in the reference) --------------------
 * (threads per ciphertext, limbs per thread) variant and window widths.  The
 * results do not depend on the configuration, only the speed does.        */
typedef struct {
  int variant;     /* mod n^2 ops: 0 = default layout, 1 = alternative */
  int dec_variant; /* mod p^2 (CRT decryption): 0 or 1 */
  int mul_window;  /* sliding-window bits of scalar Mul, 2..6 */
  int dec_window;  /* sliding-window bits of CRT decryption, 2..7 */
} hg_key_config;
int hg_key_get_config(hg_ctx* ctx, int key_id, hg_key_config* out);
int hg_key_set_config(hg_ctx* ctx, int key_id, const hg_key_config* cfg);
/* Project autotuner: times encrypt and mul (both variants, mul windows 2..6)
 * and decrypt (both variants, windows 4..7) on `calib` random inputs
 * (0 = 65536; decryption uses enough of them for several full waves),
 * applies the fastest configuration and returns it; rates[0..2] receive
 * encrypt, mul and decrypt ops/s at that configuration.  Calibrate with at
 * least as many inputs as a production call fills the GPU with.          */
int hg_autotune(hg_ctx* ctx, int key_id, size_t calib, hg_key_config* best, double* rates);

/* ---- persistent multi-key batches (no counterpart in the reference) -----
 * A batch holds jobs of any loaded keys (1024/2048/3072 bits) and ops, all on
 * DEVICE pointers: ENCRYPT (in0 = int64 m, in1 = r limbs, out = ct),
 * DECRYPT (in0 = ct, out = int64 m, aux = overflow flags), ADD (in0, in1 =
 * ct, out = ct), MUL (in0 = ct, in1 = int64 k, out = ct; HG_JOB_NONNEG
 * promises k >= 0 and skips the inverse pass).  hg_batch_run executes every
 * job in ONE persistent kernel launch (warps take cost-ordered tiles from a
 * device queue), followed by the batch inverses of negative scalars; with
 * use_graph the whole sequence is captured once into a CUDA graph and
 * replayed on later runs (the host inversion becomes a host node).  Runs are
 * asynchronous on `stream`; hg_batch_wait synchronises and reports errors.
 * A batch keeps copies of its keys' constants: free no key it uses.      */
typedef struct hg_batch hg_batch;
#define HG_OP_ENCRYPT 0
#define HG_OP_DECRYPT 1
#define HG_OP_ADD 2
#define HG_OP_MUL 3
#define HG_JOB_NONNEG 1
int hg_batch_create(hg_ctx* ctx, hg_batch** out);
int hg_batch_destroy(hg_batch* b);
int hg_batch_add(hg_batch* b, int key_id, int op, size_t count, const void* in0, const void* in1, void* out,
                 void* aux, int flags);
int hg_batch_clear(hg_batch* b);
/* Layout variant set of the batch's kernel: 0 or 1 for every job (default
 * 0), or HG_BATCH_PER_KEY: every job in its key's tuned layout
 * (hg_key_config: dec_variant for decryptions, variant for the other ops),
 * run as one persistent launch per variant set in use, back to back.    */
#define HG_BATCH_PER_KEY (-1)
int hg_batch_set_variant(hg_batch* b, int variant);
int hg_batch_run(hg_batch* b, void* stream, int use_graph);
int hg_batch_wait(hg_batch* b, void* stream);

/* ---- continuous-batching server (no counterpart in the reference) --------
 * Keeps the loaded keys' tables and resident ciphertext vectors on the
 * device and serves requests submitted from any host thread.  A scheduler
 * thread admits queued requests into free slots (stream + device arena) as
 * long as their device bytes fit the slot and the server-wide budget, runs
 * each slot's requests as one persistent batch launch (sums as reduction
 * levels) and copies results back; requests arriving meanwhile are admitted
 * into the next free slot while earlier ones are still on the GPU, and
 * every pending request gets a slice of each micro-batch (processor
 * sharing).  Each result is bit-identical to the same request run alone.  Configure keys
 * (hg_key_set_config / hg_autotune) before creating the server.
 * Every slot's stream needs a hardware work queue of its own, or a slot
 * waits behind another slot's kernels: hg_ctx_create sets
 * CUDA_DEVICE_MAX_CONNECTIONS=32 unless it is set, which takes effect only
 * when that call creates the process's CUDA context (set it before the
 * first CUDA call otherwise).                                              */
typedef struct hg_server hg_server;
#define HG_OP_SUM 4
typedef struct {
  size_t budget_bytes;    /* device memory for in-flight requests (0 = 40 GiB) */
  int slots;              /* concurrent micro-batches (0 = 4); each owns budget/slots */
  size_t max_batch_elems; /* ciphertexts per micro-batch (0 = 2^20) */
  int variant;            /* layout variant of the batch kernel, 0 or 1 */
  double batch_us;        /* estimated GPU time per micro-batch (0 = 100000) */
  double slice_us;        /* most estimated GPU time one request gets per
                             micro-batch (0 = 50000); longer requests are cut
                             into slices so short ones are not stuck behind
                             them (sums are never cut) */
  int policy;             /* admission order: HG_POLICY_SHORTEST (0, pending
                             requests with the least estimated remaining work
                             first, arrival order among equals) or
                             HG_POLICY_FIFO (1, arrival order) */
  double express_us;      /* > 0: requests with at most this much estimated
                             GPU work run in an express slot (slot 0) that
                             keeps a share of every SM's blocks free for them,
                             so they do not wait for long batches; the other
                             batches then run on the remaining share
                             (0 or < 0 = no express slot; needs slots >= 2) */
  double express_share;   /* share of every SM's batch-kernel blocks kept for
                             the express slots (0 = 0.5 with express_len,
                             0.25 with express_us) */
  size_t express_len;     /* > 0: latency class by length instead of
                             express_us: requests of at most this many
                             elements run in the express slots, in the
                             latency layout of the batch kernel (a warp per
                             ciphertext), each batch as soon as a slot is
                             free; with slots >= 3 short decryptions get an
                             express slot of their own (slot 1), so the
                             other short requests never wait for a CRT
                             chain, and with slots >= 5 the other short
                             requests get two (slots 0 and 2), so one does
                             not wait for the batch before it; each express
                             slot has a scheduler thread of its own that
                             stages and launches its batches (and inverts a
                             Mul's negative scalars on that thread) */
} hg_server_config;
#define HG_POLICY_SHORTEST 0
#define HG_POLICY_FIFO 1
typedef struct {
  int key_id;
  int op;           /* HG_OP_ENCRYPT / DECRYPT / ADD / MUL / SUM */
  size_t count;
  const void* in0;  /* host: int64 m | ct | ct a | ct a | ct (unused when h0 != 0) */
  const void* in1;  /* host: r limbs | - | ct b | int64 k | - (ADD: unused when h1) */
  uint64_t h0, h1;  /* resident vector handles in place of in0 / in1, 0 = none */
  void* out;        /* host: ct | int64 m | ct | ct | one ct */
  void* aux;        /* host: - | overflow flags (may be NULL) | - | - | - */
} hg_request;
int hg_server_create(hg_ctx* ctx, const hg_server_config* cfg, hg_server** out);
int hg_server_destroy(hg_server* s);
int hg_server_store(hg_server* s, int key_id, const uint32_t* host_ct, size_t count, uint64_t* handle);
int hg_server_release(hg_server* s, uint64_t handle);
int hg_server_submit(hg_server* s, const hg_request* req, uint64_t* ticket);
/* Blocks until the request is done; returns its status and releases the ticket. */
int hg_server_wait(hg_server* s, uint64_t ticket, double* latency_s);
int hg_server_stats(hg_server* s, uint64_t* completed, uint64_t* batches, size_t* inflight_bytes, size_t* pending);

/* ---- device-pointer forms (asynchronous on `stream`) --------------------
 * Same semantics as the host forms above.  Range errors raised by kernels
 * are collected per context; hg_dev_check(ctx) synchronises and reports
 * them.  Negate / Sub / Mul with negative scalars synchronise `stream`
 * once per call (the root of the inversion tree is inverted on the host). */
int hg_dev_encrypt(hg_ctx* ctx, int key_id, const int64_t* m, const uint32_t* r, uint32_t* ct_out, size_t count,
                   void* stream);
int hg_dev_decrypt(hg_ctx* ctx, int key_id, const uint32_t* ct, int64_t* m_out, uint8_t* overflow, size_t count,
                   void* stream);
int hg_dev_add(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t count,
               void* stream);
int hg_dev_mul(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* k, uint32_t* out, size_t count,
               void* stream);
int hg_dev_encrypt_encoded(hg_ctx* ctx, int key_id, int codec, int64_t scale, int padding_bits, const void* values,
                           const void* values2, const uint32_t* r, uint32_t* ct_out, size_t count, void* stream);
int hg_dev_decrypt_decoded(hg_ctx* ctx, int key_id, int codec, int64_t scale, int padding_bits, const uint32_t* ct,
                           void* out, void* out2, uint8_t* overflow, size_t count, void* stream);
int hg_dev_mul_bn(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* k_mag, const uint8_t* k_neg,
                  size_t k_limbs, uint32_t* out, size_t count, void* stream);
int hg_dev_sum(hg_ctx* ctx, int key_id, const uint32_t* a, size_t count, uint32_t* out, void* stream);
/* EncryptZero / Randomize (encryptor.cc:26-33, evaluator.cc:25-28); ct is updated in place */
int hg_dev_encrypt_zero(hg_ctx* ctx, int key_id, const uint32_t* r, uint32_t* ct_out, size_t count, void* stream);
int hg_dev_randomize(hg_ctx* ctx, int key_id, uint32_t* ct, const uint32_t* r, size_t count, void* stream);
/* Add(ct, pt), Sub(ct, pt), Sub(pt, ct), Sub(ct, ct), Negate (evaluator.cc:46-97);
 * out may alias a */
int hg_dev_add_plain(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, uint32_t* out, size_t count,
                     void* stream);
int hg_dev_sub_plain(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, uint32_t* out, size_t count,
                     void* stream);
int hg_dev_plain_sub(hg_ctx* ctx, int key_id, const int64_t* p, const uint32_t* a, uint32_t* out, size_t count,
                     void* stream);
int hg_dev_sub(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t count,
               void* stream);
int hg_dev_negate(hg_ctx* ctx, int key_id, const uint32_t* a, uint32_t* out, size_t count, void* stream);
/* Allocation-free Sum.  No counterpart in the reference.  For callers that
 * cannot call cudaMalloc (device memory owned by another allocator or
 * reserved up front): same result as hg_dev_sum, but the partial products
 * live in a fixed 16 MiB device array inside the library, which every GPU
 * that loads the library holds until the process exits.  count is limited
 * to 128 * floor((16 MiB - 256) / (8 * S)) ciphertexts (S = limbs per
 * ciphertext: 4,194,176 / 2,097,024 / 1,398,016 for 1024 / 2048 / 3072-bit
 * keys); larger counts are rejected with HG_ERR_INVALID before any work.
 * Allocates no device memory and calls no cudaMalloc / cudaFree.  The first
 * call on a device resolves the array's address (cudaGetSymbolAddress), so
 * make that first call before any stream capture.  Calls share the array:
 * calls that overlap on the GPU race.  Synchronises `stream` before
 * returning, so range errors come back as HG_ERR_CT_RANGE.                */
int hg_dev_sum_noalloc(hg_ctx* ctx, int key_id, const uint32_t* a, size_t count, uint32_t* out, void* stream);
int hg_dev_bucket_sum(hg_ctx* ctx, int key_id, const uint32_t* x, size_t rows, size_t cols, const uint8_t* order_map,
                      size_t features, int bucket_num, int cumsum, uint32_t* out, void* stream);
/* y stays in HOST memory (it is small and is turned into bit-plane masks on
 * the host); x and out are device pointers. */
int hg_dev_matmul(hg_ctx* ctx, int key_id, const uint32_t* x, size_t M, size_t K, const int64_t* y, size_t N,
                  uint32_t* out, void* stream);
/* y_mag / y_neg stay in HOST memory, as for hg_dev_matmul. */
int hg_dev_matmul_bn(hg_ctx* ctx, int key_id, const uint32_t* x, size_t M, size_t K, const uint32_t* y_mag,
                     const uint8_t* y_neg, size_t y_limbs, size_t N, uint32_t* out, void* stream);
int hg_dev_check(hg_ctx* ctx);

/* ---- HEU wire format of ciphertext matrices ---------------------------------
 * Replaces DenseMatrix<Ciphertext>::Serialize / LoadFrom
 * (heu/library/numpy/matrix.h:221-310, bound to Python as serialize /
 * load_from and pickling in pylib/numpy_binding/bind_numpy.cc:42-59).
 * Layout: msgpack [rows, cols, ndim, [item_0 .. item_{n-1}]], items as msgpack
 * str; an item is msgpack [c] (MSGPACK_DEFINE(c_), paillier_zahlen/
 * ciphertext.h:38, ou/ciphertext.h:38) followed by the schema value as a
 * little-endian size_t (phe/base/serializable_types.cc:49-69): 4 = ZPaillier,
 * 1 = OU (phe/base/schema.h:47-51).  c is the ciphertext's Montgomery-form
 * value (the bytes the other calls exchange) as a msgpack bin of its
 * little-endian magnitude without leading zero bytes.
 * The items are in DenseMatrix's column-major order (matrix.h:159-162);
 * row_major = 1 says ct / ct_out hold the matrix in C (row-major) order, as
 * NumPy arrays do, and the kernels reorder; 0 = column-major as stored.
 * ndim is 0, 1 or 2 (a scalar is 1 x 1, a vector n x 1).
 * hg_serialize_bound gives an upper bound of the bytes; *len receives the
 * exact size, and when it exceeds cap the call fails with HG_ERR_INVALID
 * (nothing written) and *len still holds the size needed.
 * hg_deserialize checks the structure (matrix.h:280-292: a 4-element array,
 * inner array size = rows * cols) on the host, then unpacks the items on the
 * GPU; an item that does not parse, whose value needs more than S limbs or
 * whose schema value is not the key's fails with HG_ERR_INVALID.  When the
 * matrix holds more than cap_count ciphertexts the call fails with
 * HG_ERR_INVALID after setting *rows, *cols and *ndim (call with
 * cap_count = 0 to learn the shape).
 * The hg_dev_ forms take device ct / out (serialize) or a HOST buffer and a
 * device ct_out (deserialize, e.g. bytes received from a peer); both
 * synchronise `stream`; item errors of hg_dev_deserialize are reported by
 * hg_dev_check. */
int hg_serialize_bound(hg_ctx* ctx, int key_id, size_t count, size_t* bytes);
int hg_serialize(hg_ctx* ctx, int key_id, const uint32_t* ct, size_t rows, size_t cols, int ndim, int row_major,
                 uint8_t* out, size_t cap, size_t* len);
int hg_deserialize(hg_ctx* ctx, int key_id, const uint8_t* buf, size_t len, int row_major, uint32_t* ct_out,
                   size_t cap_count, size_t* rows, size_t* cols, int* ndim);
int hg_dev_serialize(hg_ctx* ctx, int key_id, const uint32_t* ct, size_t rows, size_t cols, int ndim, int row_major,
                     uint8_t* out, size_t cap, size_t* len, void* stream);
int hg_dev_deserialize(hg_ctx* ctx, int key_id, const uint8_t* buf, size_t len, int row_major, uint32_t* ct_out,
                       size_t cap_count, size_t* rows, size_t* cols, int* ndim, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HEU_GB300_H_ */
