// Kernel parameter blocks and launcher declarations shared by the kernels
// (paillier_kernels.cu) and the host engine (engine.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace hg {

// Error bits raised by kernels into a device word (atomicOr).
enum : uint32_t {
  kErrCtRange = 1u,      // a ciphertext >= n^2 reached a kernel
  kErrNotInvertible = 2u,
  kErrPtRange = 4u,      // a plaintext with |m| > n/2
  kErrBinRange = 8u,     // an order-map bin id >= bucket_num
  kErrFormat = 16u,      // a serialized ciphertext item that does not parse
};

// Public-key constants for arithmetic mod N = n^2 with R = 2^(32*S).
struct KeyConst {
  const uint32_t* N;    // n^2                         (S limbs)
  const uint32_t* R1;   // R mod N  (Montgomery one)  (S limbs)
  const uint32_t* R2;   // R^2 mod N                  (S limbs)
  const uint32_t* R3;   // R^3 mod N                  (S limbs)
  const uint32_t* nR2;  // n * R^2 mod N              (S limbs)
  const uint32_t* n;    // n                          (S/2 limbs)
  const uint32_t* nhalf;  // floor(n/2)              (S/2 limbs)
  const uint32_t* table;  // fixed-base table of h_s powers, Montgomery form
  uint32_t np;          // -N^-1 mod 2^32
  int S;                // 32-bit limbs of N
  int w;                // table window (bits per digit)
  int npos;             // digit positions = ceil(rbits / w)
  int rbits;            // bits of the encryption randomness r (k/2)
  int rlimbs;           // 32-bit limbs per r
  int variant;          // (threads per instance, limbs per thread) variant, 0 or 1
};

// Secret-key constants for CRT decryption.  Index 0 = p side, 1 = q side.
struct SecConst {
  const uint32_t* P2[2];    // p^2, q^2                    (Sp limbs)
  const uint32_t* P[2];     // p, q                        (Sp/2 limbs)
  const uint32_t* hR[2];    // hp*R1 mod p, hq*R1 mod q    (Sp/2 limbs), R1 = 2^(16*Sp)
  const uint32_t* inv2[2];  // p^-1, q^-1 mod 2^(16*Sp)    (Sp/2 limbs)
  const uint32_t* pinvqR;   // (p^-1 mod q)*R1 mod q       (Sp/2 limbs)
  const uint16_t* prog[2];  // exponent programs for p-1, q-1
  uint32_t np2[2];          // -(p^2)^-1, -(q^2)^-1 mod 2^32
  uint32_t np1[2];          // -p^-1, -q^-1 mod 2^32
  int start[2];             // first window's table index
  int prog_len;             // both programs padded to this many steps
  int wd;                   // decryption window bits
  int Sp;                   // 32-bit limbs of p^2
  int variant;              // (threads per unit side, limbs per thread) variant
};

// Okamoto-Uchiyama secret constants (ou/secret_key.h; decryptor.cc:27-45).
struct OuConst {
  const uint32_t* P2;     // p^2                                 (Sp limbs)
  const uint32_t* Kfix;   // R_p^3 * R_n^-1 mod p^2              (Sp limbs)
  const uint32_t* P;      // p                                   (Sp/2 limbs)
  const uint32_t* gpR;    // gp_inv * 2^(16*Sp) mod p            (Sp/2 limbs)
  const uint32_t* pinv;   // p^-1 mod 2^(16*Sp)                  (Sp/2 limbs)
  const uint32_t* phalf;  // p >> 1                              (Sp/2 limbs)
  const uint16_t* prog;   // sliding-window program of the exponent t
  uint32_t np2;           // -(p^2)^-1 mod 2^32
  uint32_t np1;           // -p^-1 mod 2^32
  int start;              // first window's table index
  int prog_len;
  int wd;                 // window bits
  int Sp;                 // 32-bit limbs of the p^2 arithmetic
};

// Exponent-program opcodes (one Montgomery multiplication per step).
constexpr uint16_t kOpSquare = 0xFFFFu;
constexpr uint16_t kOpNop = 0xFFFEu;

enum class EncMode : int { kEncrypt = 0, kZero = 1, kRandomize = 2 };

// Plaintext encodings applied inside the encryption and decryption kernels
// (HEU's PlainEncoder, phe/encoding/plain_encoder.h:46-74, and BatchEncoder,
// phe/encoding/batch_encoder.h:27-140).  Values match include/heu_gb300.h's
// HG_CODEC_*.
enum : int { kCodecNone = 0, kCodecPlainI64 = 1, kCodecPlainF64 = 2, kCodecBatchI64 = 3, kCodecBatchF64 = 4 };
struct Codec {
  int kind;         // kCodec*
  int padding;      // BatchEncoder padding bits between the two slots
  int64_t scale;    // > 0
  const void* in1;  // encryption: the second slot's values (batch kinds)
  void* out1;       // decryption: the second slot's values (batch kinds)
};

// Launchers.  All are asynchronous on `stream` and return cudaError_t of the
// launch.  `cfg` selects the (threads per instance, limbs per thread) variant.
// With cd.kind != kCodecNone (mode kEncrypt) `m` holds the values to encode
// (int64 or double, per cd.kind) and m_mag / m_neg are unused.
cudaError_t launch_encrypt(int S, const KeyConst& kc, EncMode mode, const int64_t* m, const uint32_t* m_mag,
                           const uint8_t* m_neg, const uint32_t* r, const uint32_t* ct_in, uint32_t* out,
                           size_t count, uint32_t* err, int grid, cudaStream_t st, const Codec& cd = Codec{});
cudaError_t launch_add(int S, const KeyConst& kc, const uint32_t* a, const uint32_t* b, uint32_t* out,
                       size_t count, uint32_t* err, cudaStream_t st);
cudaError_t launch_add_plain(int S, const KeyConst& kc, const uint32_t* a, const int64_t* p, int neg_p,
                             uint32_t* out, size_t count, uint32_t* err, cudaStream_t st);
// The persistent kernels (mul, decrypt, OU decrypt) take work from *ctr, a
// device counter that the launcher zeroes in stream order before the launch.
cudaError_t launch_mul(int S, const KeyConst& kc, const uint32_t* a, const int64_t* k, uint32_t* out,
                       size_t count, uint32_t* scratch, int wm, uint32_t* err, int grid, unsigned long long* ctr,
                       cudaStream_t st);
// Mul by multi-limb scalar magnitudes (el limbs each), window wb (1..8);
// persistent grid of `grid` blocks (resident_blocks_mul_bn) with a scratch of
// grid * instances_per_block(S, 0) * 2^(wb-1) * S limbs.
cudaError_t launch_mul_bn(int S, const KeyConst& kc, const uint32_t* a, const uint32_t* emag, int el,
                          uint32_t* out, size_t count, uint32_t* scratch, int wb, uint32_t* err, int grid,
                          unsigned long long* ctr, cudaStream_t st);
int resident_blocks_mul_bn(int S);
// sel[i] = neg[i] ? -1 : 1 (selector of the batch inverse)
cudaError_t launch_sel_from_neg(const uint8_t* neg, int64_t* sel, size_t count, cudaStream_t st);
// With cd.kind != kCodecNone out_i64 receives the decoded values (int64 or
// double, per cd.kind) and cd.out1 the second slot of batch kinds.
cudaError_t launch_decrypt(int Sp, const KeyConst& kc, const SecConst& sc, const uint32_t* ct, size_t count,
                           int64_t* out_i64, uint8_t* out_ovf, uint32_t* out_mag, uint8_t* out_neg,
                           uint32_t* scratch, uint32_t* err, int grid, unsigned long long* ctr, cudaStream_t st,
                           const Codec& cd = Codec{});
// OU decryption over S-limb ciphertexts with Sp-limb p^2 arithmetic
// (S, Sp) in {(64, 32), (128, 64), (128, 96)}.
cudaError_t launch_ou_decrypt(int S, const KeyConst& kc, const OuConst& oc, const uint32_t* ct, size_t count,
                              int64_t* out_i64, uint8_t* out_ovf, uint32_t* out_mag, uint8_t* out_neg,
                              uint32_t* scratch, uint32_t* err, int grid, unsigned long long* ctr,
                              cudaStream_t st);
cudaError_t ou_decrypt_geometry(int S, int Sp, int* grid, int* units_per_block);
// Signed plaintexts -> non-negative exponents for the G and G^-1 tables.
cudaError_t launch_ou_split_i64(const int64_t* p, int negate, uint32_t* ep, uint32_t* en, size_t count,
                                cudaStream_t st);
cudaError_t launch_ou_split_mag(const uint32_t* mag, const uint8_t* neg, int limbs, const uint32_t* maxpt,
                                uint32_t* ep, uint32_t* en, size_t count, uint32_t* err, cudaStream_t st);
// out[i] = MM(in[i], c) with one S-limb constant c in device memory
cudaError_t launch_mul_const(int S, const KeyConst& kc, const uint32_t* in, const uint32_t* c, uint32_t* out,
                             size_t count, uint32_t* err, cudaStream_t st);
cudaError_t launch_convert(int S, const KeyConst& kc, const uint32_t* in, uint32_t* out, size_t count,
                           int to_mont, uint32_t* err, cudaStream_t st);
// Sum as a tree: groups multiply chunks of `chunk` inputs, then combine by
// warp shuffles and shared memory into one ciphertext per block of the
// default layout; reduce_tree_outputs(S, count, chunk) blocks = outputs.
cudaError_t launch_reduce_tree(int S, const KeyConst& kc, const uint32_t* in, size_t count, int chunk,
                               uint32_t* out, uint32_t* err, cudaStream_t st);
size_t reduce_tree_outputs(int S, size_t count, int chunk);
// Chunk of one tree level over `count` inputs on `sms` multiprocessors: one
// full wave of groups while inputs outnumber the resident groups, one input
// per group below that, one block for the last few inputs.
int reduce_tree_chunk(int S, size_t count, int sms);
// The reduction and inversion-tree kernels prefer the largest shared-memory
// carveout, as the batch kernels do (serving loop).
void server_prefer_shared_carveout();
cudaError_t launch_reduce(int S, const KeyConst& kc, const uint32_t* in, size_t count, int chunk,
                          uint32_t* out, uint32_t* err, cudaStream_t st);
// product tree for batch inversion
cudaError_t launch_tree_leaves(int S, const KeyConst& kc, const uint32_t* in, const int64_t* sel, size_t count,
                               uint32_t* leaves, size_t padded, uint32_t* err, cudaStream_t st);
cudaError_t launch_tree_up(int S, const KeyConst& kc, const uint32_t* lower, uint32_t* upper, size_t upper_count,
                           cudaStream_t st);
cudaError_t launch_tree_down(int S, const KeyConst& kc, uint32_t* lower, const uint32_t* upper_inv,
                             size_t upper_count, cudaStream_t st);
cudaError_t launch_tree_apply(int S, const KeyConst& kc, const uint32_t* in, const int64_t* sel,
                              const uint32_t* leaves_inv, uint32_t* out, size_t count, cudaStream_t st);
// fixed-base table construction
cudaError_t launch_table_bases(int S, const KeyConst& kc, const uint32_t* hs_mont, uint32_t* bases,
                               cudaStream_t st);
cudaError_t launch_table_level(int S, const KeyConst& kc, uint32_t* table, const uint32_t* bases, int level,
                               cudaStream_t st);

// FeatureWiseBucketSum building blocks (reduce_kernels.cu)
cudaError_t launch_bin_sort(const uint8_t* om, size_t rows, int F, int B, uint32_t* cnt, uint32_t* offs,
                            uint32_t* cursor, uint32_t* idx, uint32_t* err, cudaStream_t st);
cudaError_t launch_seg_level(int S, const KeyConst& kc, const uint32_t* vals, size_t stride, size_t voff,
                             const uint32_t* idx, const uint32_t* offs_in, int nseg, int C, uint32_t* nch,
                             uint32_t* offs_out, uint32_t* out, size_t upper, uint32_t* err, cudaStream_t st);
cudaError_t launch_seg_finalize(int S, const uint32_t* vals, const uint32_t* offs, int nseg, const uint32_t* R1,
                                uint32_t* out, size_t ostride, size_t ooff, cudaStream_t st);
cudaError_t launch_bucket_cumsum(int S, const KeyConst& kc, uint32_t* out, int F, int B, size_t ostride,
                                 size_t ooff, cudaStream_t st);

// MatMul building blocks (matmul_kernels.cu)
cudaError_t launch_subset_tables(int S, const KeyConst& kc, const uint32_t* x, size_t r0, size_t rows, int K,
                                 uint32_t* T, uint32_t* err, cudaStream_t st);
cudaError_t launch_matmul_planes(int S, const KeyConst& kc, const uint32_t* T, const uint8_t* masks, size_t r0,
                                 size_t rows, int Ncols, int P, int K, uint32_t* out, cudaStream_t st);
cudaError_t launch_row_products(int S, const KeyConst& kc, const uint32_t* T, size_t rows, int K, uint32_t* prod,
                                cudaStream_t st);
cudaError_t launch_pow_shared(int S, const KeyConst& kc, uint32_t* v, size_t count, uint64_t e, cudaStream_t st);
// the same for one exponent of el limbs in device memory (nonzero)
cudaError_t launch_pow_shared_bn(int S, const KeyConst& kc, uint32_t* v, size_t count, const uint32_t* e, int el,
                                 cudaStream_t st);
cudaError_t launch_scale_rows(int S, const KeyConst& kc, uint32_t* out, const uint32_t* q, size_t r0, size_t rows,
                              int Ncols, cudaStream_t st);
size_t subset_table_bytes_per_row(int S, int K);

// Occupancy-derived grid sizes (blocks) for the persistent kernels.
int resident_blocks_mul(int S, int variant);
int resident_blocks_decrypt(int Sp, int variant);
int instances_per_block(int S, int variant);
int units_per_block_decrypt(int Sp, int variant);

bool supported_limbs(int S);
uint64_t launch_count();  // kernels launched by this process so far
void count_launches(uint64_t n);

// HEU wire format (wire_kernels.cu), over a rows x cols matrix whose items
// are written in column-major order; row_major says how ct / out hold the
// elements.  launch_wire_size fills mag_bytes (rows * cols words) and scratch
// (wire_scratch_words(rows * cols) uint64 words: item offsets, block totals)
// and copies the items' total bytes to *total_dev; launch_wire_write then
// writes the items at out + base.  Unpacking: item k is
// buf[offs[k] .. offs[k] + lens[k]).
size_t wire_scratch_words(size_t count);
cudaError_t launch_wire_size(const uint32_t* ct, size_t rows, size_t cols, int row_major, int S, uint32_t* mag_bytes,
                             uint64_t* scratch, uint64_t* total_dev, cudaStream_t st);
cudaError_t launch_wire_write(const uint32_t* ct, size_t rows, size_t cols, int row_major, int S, uint64_t schema,
                              const uint32_t* mag_bytes, const uint64_t* scratch, uint8_t* out, size_t base,
                              cudaStream_t st);
cudaError_t launch_wire_unpack(const uint8_t* buf, const uint64_t* offs, const uint64_t* lens, size_t rows,
                               size_t cols, int row_major, int S, uint64_t schema, uint32_t* out, uint32_t* err,
                               cudaStream_t st);

}  // namespace hg
