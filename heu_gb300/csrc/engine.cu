// Host engine behind the C-ABI (include/heu_gb300.h): contexts, key
// precompute and residency, device staging, and the multi-kernel sequences
// (product-tree inverse, reduction levels, fixed-base table build).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <random>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/heu_gb300.h"
#include "../../include/heu_gb300_probe.h"
#include "batch.cuh"
#include "engine_internal.hpp"
#include "host_bn.hpp"
#include "wire_host.hpp"
#include "paillier_kernels.cuh"

namespace {

using hg::BN;

thread_local std::string g_last_error;

struct HgError : std::runtime_error {
  int code;
  HgError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const std::string& msg) { throw HgError(code, msg); }

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    if (e == cudaErrorMemoryAllocation) fail(HG_ERR_NOMEM, std::string(what) + ": " + cudaGetErrorString(e));
    fail(HG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

// One NVTX range per C-ABI call (named after the entry point), so profilers
// show the engine's calls on the timeline; free when no tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

// The calling thread's current CUDA device, put back when a C-ABI call
// returns: the engine switches to its context's device, and a caller that
// works on another device must not find its own selection changed.
struct CurrentDeviceKeeper {
  int device = -1;
  CurrentDeviceKeeper() {
    if (cudaGetDevice(&device) != cudaSuccess) device = -1;
  }
  ~CurrentDeviceKeeper() {
    int now = -1;
    if (device >= 0 && cudaGetDevice(&now) == cudaSuccess && now != device) cudaSetDevice(device);
  }
};

template <typename F>
int guarded(const char* name, F&& f) {
  NvtxRange range(name);
  const CurrentDeviceKeeper keep;
  try {
    return f();
  } catch (const HgError& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return HG_ERR_NOMEM;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return HG_ERR_INVALID;
  }
}

// grow-only device buffer
// Device bytes held by engine buffers, and an optional cap on them (set by
// hg_probe_set_alloc_limit to make allocation failures happen on purpose,
// on the host, before cudaMalloc is called).
std::atomic<size_t> g_dev_bytes{0};
std::atomic<size_t> g_dev_limit{0};

struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() {
    if (p) {
      cudaFree(p);
      g_dev_bytes -= n;
    }
  }
  template <typename T = void>
  T* ensure(size_t bytes) {
    if (bytes > n) {
      const size_t limit = g_dev_limit.load();
      if (limit && g_dev_bytes.load() - n + bytes > limit)
        fail(HG_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes exceeds the set limit");
      if (p) {
        cudaFree(p);
        g_dev_bytes -= n;
      }
      p = nullptr;
      n = 0;
      cuda_check(cudaMalloc(&p, bytes), "cudaMalloc");
      n = bytes;
      g_dev_bytes += n;
    }
    return reinterpret_cast<T*>(p);
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

// Buffers of one product-tree inversion.
struct TreeBufs {
  DevBuf tree;
};

struct PinBuf {
  void* p = nullptr;
  size_t n = 0;
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
  ~PinBuf() {
    if (p) cudaFreeHost(p);
  }
  template <typename T = void>
  T* ensure(size_t bytes) {
    if (bytes > n) {
      if (p) cudaFreeHost(p);
      p = nullptr;
      n = 0;
      cuda_check(cudaMallocHost(&p, bytes), "cudaMallocHost");
      n = bytes;
    }
    return reinterpret_cast<T*>(p);
  }
};

uint32_t neg_inv32(uint32_t a) {
  uint32_t inv = 1;
  for (int i = 0; i < 5; ++i) inv *= 2u - a * inv;
  return 0u - inv;
}

// ---------------------------------------------------------------------------
// keys
// ---------------------------------------------------------------------------
struct KeyRec {
  int key_bits = 0;
  int S = 0, Sp = 0, H = 0;
  bool secret = false;
  BN n, N, hs, p, q;
  DevBuf consts, sconsts, table, progs;
  hg::KeyConst kc{};
  hg::SecConst sc{};
  int grid_mul = 0, grid_dec = 0;
  int grid_mul_bn = 0;  // persistent grid of the multi-limb scalar Mul (set on first use)
  int wm = 4;  // scalar-mul window
  // Okamoto-Uchiyama keys (scheme 1): kc is over n with the H table; kcG /
  // kcGi hold the G and G^-1 tables; oc the decryption constants
  int scheme = 0;
  hg::KeyConst kcG{}, kcGi{};
  DevBuf tableG, tableGi, oconsts, oprog;
  hg::OuConst oc{};
  int pt_limbs = 0, max_pt_bits = 0;
  int grid_oudec = 0, upb_oudec = 0;
  const uint32_t* d_maxpt = nullptr;  // max plaintext (pt_limbs), on the device
};

// Asynchronous inversion of the root of a product tree: the host function
// runs in stream order (and as a host node inside a captured CUDA graph).
struct InvTask {
  const BN* N = nullptr;
  int S = 0;
  uint32_t* root = nullptr;  // pinned: S limbs of the root, then the kernels' error word
  uint32_t* z = nullptr;     // pinned: S limbs of the root's inverse, Montgomery form
  volatile int status = 0;   // 0 ok, 1 not invertible, 2 range error upstream
};

// The status is sticky: a failure stays recorded until the caller resets it,
// so one task can serve several inversions enqueued in one stream.
void CUDART_CB inv_host_fn(void* p) {
  InvTask* t = static_cast<InvTask*>(p);
  const size_t S = (size_t)t->S;
  if (t->root[S] & (hg::kErrCtRange | hg::kErrPtRange)) {
    t->status = 2;
    for (size_t i = 0; i < S; ++i) t->z[i] = 0u;
    return;
  }
  // root = X*R; the tree's down-sweep wants X^-1 * R
  if (!hg::mont_root_inverse(t->root, *t->N, S, t->z)) {
    if (t->status == 0) t->status = 1;
    for (size_t i = 0; i < S; ++i) t->z[i] = 0u;
  }
}

// Sliding-window exponent program: first window index + one op per step.
void build_prog(const BN& e, int w, int* start, std::vector<uint16_t>* steps) {
  int i = (int)e.bitlen() - 1;
  bool first = true;
  *start = 0;
  while (i >= 0) {
    if (!e.bit((size_t)i)) {
      if (!first) steps->push_back(hg::kOpSquare);
      --i;
      continue;
    }
    int j = std::max(i - w + 1, 0);
    while (!e.bit((size_t)j)) ++j;
    uint32_t val = 0;
    for (int b = i; b >= j; --b) val = (val << 1) | (e.bit((size_t)b) ? 1u : 0u);
    const uint16_t idx = (uint16_t)((val - 1) >> 1);
    if (first) {
      *start = idx;
      first = false;
    } else {
      for (int s = 0; s < i - j + 1; ++s) steps->push_back(hg::kOpSquare);
      steps->push_back(idx);
    }
    i = j - 1;
  }
}

// ---------------------------------------------------------------------------
// per-call working state: stream, staging, scratch, error word
// ---------------------------------------------------------------------------
struct Work {
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  DevBuf io[6];
  DevBuf scratch, red[2];
  TreeBufs inv;
  DevBuf seg_cnt, seg_offs[3], seg_cursor, seg_idx, seg_nch, seg_part[2];
  DevBuf mm_tables, mm_masks, mm_prod, mm_exp;
  DevBuf sel;  // signs of multi-limb scalars as the inverse's selector
  DevBuf ou_e[2];
  DevBuf err;
  PinBuf pin_root, pin_err, pin_z, pin_wire;
  InvTask task;
  ~Work() {
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
  DevBuf ctr;  // work counter of the persistent kernels this lane launches
  uint32_t* errp() { return err.ensure<uint32_t>(sizeof(uint32_t)); }
  unsigned long long* ctrp() { return ctr.ensure<unsigned long long>(sizeof(unsigned long long)); }
};

}  // namespace

struct hg_ctx {
  int device = 0;
  int sm_count = 0;
  std::mutex mu;  // guards keys and the lane pool
  std::map<int, std::unique_ptr<KeyRec>> keys;
  int next_key = 1;
  std::vector<std::unique_ptr<Work>> lanes;
  std::vector<Work*> free_lanes;
  std::condition_variable lane_cv;
  std::mutex dev_mu;  // guards dev_work
  std::map<cudaStream_t, std::unique_ptr<Work>> dev_work;
  DevBuf dev_err;
};

namespace {

constexpr int kLanes = 4;

KeyRec* get_key(hg_ctx* ctx, int id) {
  if (!ctx) fail(HG_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->keys.find(id);
  if (it == ctx->keys.end()) fail(HG_ERR_INVALID, "unknown key id " + std::to_string(id));
  return it->second.get();
}

struct LaneGuard {
  hg_ctx* ctx;
  Work* w;
  explicit LaneGuard(hg_ctx* c) : ctx(c) {
    std::unique_lock<std::mutex> lk(ctx->mu);
    ctx->lane_cv.wait(lk, [&] { return !ctx->free_lanes.empty(); });
    w = ctx->free_lanes.back();
    ctx->free_lanes.pop_back();
  }
  ~LaneGuard() {
    {
      std::lock_guard<std::mutex> lk(ctx->mu);
      ctx->free_lanes.push_back(w);
    }
    ctx->lane_cv.notify_one();
  }
};

void set_device(hg_ctx* ctx) { cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice"); }

void reset_err(Work& w) { cuda_check(cudaMemsetAsync(w.errp(), 0, sizeof(uint32_t), w.stream), "memset err"); }

void raise_err_bits(uint32_t bits) {
  if (bits & hg::kErrCtRange) fail(HG_ERR_CT_RANGE, "Invalid ciphertext: value >= n^2");
  if (bits & hg::kErrBinRange) fail(HG_ERR_INVALID, "order map holds a bin id >= bucket_num");
  if (bits & hg::kErrFormat) fail(HG_ERR_INVALID, "Cannot parse inner_obj: buffer format error (ciphertext item)");
  if (bits & hg::kErrPtRange) fail(HG_ERR_PT_RANGE, "message number out of range: |m| > n/2");
  if (bits & hg::kErrNotInvertible) fail(HG_ERR_NOT_INVERTIBLE, "ciphertext not invertible mod n^2");
}

void finish(Work& w) {
  uint32_t* h = w.pin_err.ensure<uint32_t>(sizeof(uint32_t));
  cuda_check(cudaMemcpyAsync(h, w.errp(), sizeof(uint32_t), cudaMemcpyDeviceToHost, w.stream), "D2H err");
  cuda_check(cudaStreamSynchronize(w.stream), "stream sync");
  raise_err_bits(*h);
}

void h2d(void* d, const void* h, size_t bytes, Work& w) {
  if (bytes) cuda_check(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, w.stream), "H2D");
}
void d2h(void* h, const void* d, size_t bytes, Work& w) {
  if (bytes) cuda_check(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, w.stream), "D2H");
}

// Both lanes' error words, OR-ed: the same error a single lane would raise.
void finish_pair(Work& a, Work& b) {
  uint32_t* ha = a.pin_err.ensure<uint32_t>(sizeof(uint32_t));
  uint32_t* hb = b.pin_err.ensure<uint32_t>(sizeof(uint32_t));
  cuda_check(cudaMemcpyAsync(ha, a.errp(), sizeof(uint32_t), cudaMemcpyDeviceToHost, a.stream), "D2H err");
  cuda_check(cudaMemcpyAsync(hb, b.errp(), sizeof(uint32_t), cudaMemcpyDeviceToHost, b.stream), "D2H err");
  cuda_check(cudaStreamSynchronize(a.stream), "stream sync");
  cuda_check(cudaStreamSynchronize(b.stream), "stream sync");
  raise_err_bits(*ha | *hb);
}

// A second lane for one call, when one is free (never waits for one).
struct ExtraLane {
  hg_ctx* ctx;
  Work* w = nullptr;
  explicit ExtraLane(hg_ctx* c) : ctx(c) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->free_lanes.empty()) {
      w = ctx->free_lanes.back();
      ctx->free_lanes.pop_back();
    }
  }
  ~ExtraLane() {
    if (!w) return;
    {
      std::lock_guard<std::mutex> lk(ctx->mu);
      ctx->free_lanes.push_back(w);
    }
    ctx->lane_cv.notify_one();
  }
};

// Host-pointer calls over many elements run as up to kPipeMaxChunks chunks
// alternating between the caller's lane and a second free lane: each chunk is
// H2D -> kernels -> D2H in its own lane's stream order, so one lane's copies
// run while the other lane's kernels compute.  chunk(w, offset, count)
// enqueues one chunk; the call returns after both lanes drained.
constexpr size_t kPipeMinChunk = (size_t)1 << 16;
constexpr size_t kPipeMaxChunks = 8;

// prepare(w) runs on each lane before its first chunk, check(w) on each lane
// after both drained (the error words are raised first).  max_chunks bounds
// the chunks (signed-scalar Mul measured 0.516 s at 8 chunks and 0.532 s at 2
// for 2^20 ciphertexts, so every op uses the default).
template <class F, class Prep, class Check>
void run_chunked(hg_ctx* ctx, Work& w0, size_t count, F&& chunk, Prep&& prepare, Check&& check,
                 size_t max_chunks = kPipeMaxChunks) {
  if (count >= 2 * kPipeMinChunk && max_chunks >= 2) {
    ExtraLane extra(ctx);
    if (extra.w) {
      Work& w1 = *extra.w;
      reset_err(w1);
      prepare(w0);
      prepare(w1);
      const size_t nch = std::min(max_chunks, count / kPipeMinChunk);
      const size_t per = (count + nch - 1) / nch;
      Work* lanes[2] = {&w0, &w1};
      size_t c = 0;
      for (size_t off = 0; off < count; off += per, ++c) chunk(*lanes[c & 1], off, std::min(per, count - off));
      finish_pair(w0, w1);
      check(w0);
      check(w1);
      return;
    }
  }
  prepare(w0);
  chunk(w0, (size_t)0, count);
  finish(w0);
  check(w0);
}

template <class F>
void run_chunked(hg_ctx* ctx, Work& w0, size_t count, F&& chunk) {
  run_chunked(ctx, w0, count, std::forward<F>(chunk), [](Work&) {}, [](Work&) {});
}

// ---------------------------------------------------------------------------
// core device sequences (device pointers, asynchronous except the inverse)
// ---------------------------------------------------------------------------
size_t ct_bytes(const KeyRec& k) { return (size_t)k.S * 4; }

// OU: out = [ct_in or 1] * G^(m+) * (G^-1)^(m-) [* H^r]  (encryptor.cc:92-117,
// evaluator.cc:35-50), as three passes of the fixed-base kernel.
void ou_plain_pow(KeyRec& k, Work& w, const int64_t* m, int negate, const uint32_t* m_mag, const uint8_t* m_neg,
                  const uint32_t* r, const uint32_t* ct_in, uint32_t* out, size_t count) {
  const int el = m ? 2 : k.pt_limbs;  // exponent limbs
  uint32_t* ep = w.ou_e[0].ensure<uint32_t>(count * el * 4);
  uint32_t* en = w.ou_e[1].ensure<uint32_t>(count * el * 4);
  if (m)
    cuda_check(hg::launch_ou_split_i64(m, negate, ep, en, count, w.stream), "OU split");
  else
    cuda_check(hg::launch_ou_split_mag(m_mag, m_neg, el, k.d_maxpt, ep, en, count, w.errp(), w.stream),
               "OU split");
  hg::KeyConst g = k.kcG, gi = k.kcGi;
  g.rlimbs = gi.rlimbs = el;
  g.rbits = gi.rbits = m ? 64 : k.max_pt_bits;
  g.npos = gi.npos = (g.rbits + g.w - 1) / g.w;
  cuda_check(hg::launch_encrypt(k.S, g, ct_in ? hg::EncMode::kRandomize : hg::EncMode::kZero, nullptr, nullptr,
                                nullptr, ep, ct_in, out, count, w.errp(), 0, w.stream),
             "OU G pass");
  cuda_check(hg::launch_encrypt(k.S, gi, hg::EncMode::kRandomize, nullptr, nullptr, nullptr, en, out, out, count,
                                w.errp(), 0, w.stream),
             "OU G^-1 pass");
  if (r)
    cuda_check(hg::launch_encrypt(k.S, k.kc, hg::EncMode::kRandomize, nullptr, nullptr, nullptr, r, out, out, count,
                                  w.errp(), 0, w.stream),
               "OU H pass");
}

void core_encrypt(KeyRec& k, Work& w, hg::EncMode mode, const int64_t* m, const uint32_t* m_mag,
                  const uint8_t* m_neg, const uint32_t* r, const uint32_t* ct_in, uint32_t* out, size_t count) {
  if (k.scheme == 1 && mode == hg::EncMode::kEncrypt) {
    ou_plain_pow(k, w, m, 0, m_mag, m_neg, r, nullptr, out, count);
    return;
  }
  cuda_check(hg::launch_encrypt(k.S, k.kc, mode, m, m_mag, m_neg, r, ct_in, out, count, w.errp(), 0, w.stream),
             "encrypt launch");
}

// Device encodings (PlainEncoder / BatchEncoder) of the C-ABI's HG_CODEC_*.
hg::Codec make_codec(const KeyRec& k, int codec, int64_t scale, int padding, const void* in1, void* out1) {
  if (k.scheme != 0) fail(HG_ERR_UNSUPPORTED, "device encodings serve ZPaillier keys");
  if (codec < HG_CODEC_PLAIN_I64 || codec > HG_CODEC_BATCH_F64) fail(HG_ERR_INVALID, "unknown codec");
  if (scale <= 0) fail(HG_ERR_INVALID, "scale must be positive");
  const bool batch = codec == HG_CODEC_BATCH_I64 || codec == HG_CODEC_BATCH_F64;
  if (batch && (padding < 0 || 128 + padding > 16 * k.S))
    fail(HG_ERR_INVALID, "padding_bits must be >= 0 and leave both slots below the plaintext bound");
  hg::Codec cd{};
  cd.kind = codec;
  cd.padding = batch ? padding : 0;
  cd.scale = scale;
  cd.in1 = in1;
  cd.out1 = out1;
  return cd;
}

void core_encrypt_encoded(KeyRec& k, Work& w, const void* values, const uint32_t* r, uint32_t* out, size_t count,
                          const hg::Codec& cd) {
  cuda_check(hg::launch_encrypt(k.S, k.kc, hg::EncMode::kEncrypt, static_cast<const int64_t*>(values), nullptr,
                                nullptr, r, nullptr, out, count, w.errp(), 0, w.stream, cd),
             "encrypt launch");
}

void core_decrypt_decoded(KeyRec& k, Work& w, const uint32_t* ct, void* out, uint8_t* ovf, size_t count,
                          const hg::Codec& cd) {
  if (!k.secret) fail(HG_ERR_NO_SECRET, "key has no secret part");
  const size_t ntab = (size_t)1 << (k.sc.wd - 1);
  const size_t units = (size_t)k.grid_dec * hg::units_per_block_decrypt(k.Sp, k.sc.variant);
  uint32_t* scratch = w.scratch.ensure<uint32_t>(units * 2 * ntab * k.Sp * 4);
  cuda_check(hg::launch_decrypt(k.Sp, k.kc, k.sc, ct, count, static_cast<int64_t*>(out), ovf, nullptr, nullptr,
                                scratch, w.errp(), k.grid_dec, w.ctrp(), w.stream, cd),
             "decrypt launch");
}

// Add(ct, pt) / Sub(ct, pt) with int64 plaintexts, per scheme.
void core_add_plain(KeyRec& k, Work& w, const uint32_t* a, const int64_t* p, int neg, uint32_t* out, size_t count) {
  if (k.scheme == 1) {
    ou_plain_pow(k, w, p, neg, nullptr, nullptr, nullptr, a, out, count);
    return;
  }
  cuda_check(hg::launch_add_plain(k.S, k.kc, a, p, neg, out, count, w.errp(), w.stream), "add_plain launch");
}

void core_decrypt(KeyRec& k, Work& w, const uint32_t* ct, int64_t* m, uint8_t* ovf, uint32_t* mag, uint8_t* neg,
                  size_t count) {
  if (!k.secret) fail(HG_ERR_NO_SECRET, "key has no secret part");
  if (k.scheme == 1) {
    const size_t ntab = (size_t)1 << (k.oc.wd - 1);
    const size_t units = (size_t)k.grid_oudec * k.upb_oudec;
    uint32_t* scratch = w.scratch.ensure<uint32_t>(units * ntab * k.oc.Sp * 4);
    cuda_check(hg::launch_ou_decrypt(k.S, k.kc, k.oc, ct, count, m, ovf, mag, neg, scratch, w.errp(), k.grid_oudec,
                                     w.ctrp(), w.stream),
               "OU decrypt launch");
    return;
  }
  const size_t ntab = (size_t)1 << (k.sc.wd - 1);
  const size_t units = (size_t)k.grid_dec * hg::units_per_block_decrypt(k.Sp, k.sc.variant);
  uint32_t* scratch = w.scratch.ensure<uint32_t>(units * 2 * ntab * k.Sp * 4);
  cuda_check(hg::launch_decrypt(k.Sp, k.kc, k.sc, ct, count, m, ovf, mag, neg, scratch, w.errp(), k.grid_dec,
                                w.ctrp(), w.stream),
             "decrypt launch");
}

// out[i] = in[i]^-1 where sel == nullptr or sel[i] < 0, else in[i].
// out[i] = in[i]^-1 where sel == nullptr or sel[i] < 0, else in[i]; every
// step is in stream order (graph-capturable).  `task` must outlive the work.
void core_inverse_async_raw(KeyRec& k, const uint32_t* in, const int64_t* sel, uint32_t* out, size_t count,
                            uint32_t* tr, InvTask& task, uint32_t* errp, cudaStream_t st,
                            bool inline_host = false);

void core_inverse_async(KeyRec& k, const uint32_t* in, const int64_t* sel, uint32_t* out, size_t count,
                        TreeBufs& tb, InvTask& task, uint32_t* errp, cudaStream_t st) {
  if (count == 0) return;
  size_t padded = 1;
  while (padded < count) padded <<= 1;
  const size_t S = (size_t)k.S;
  uint32_t* tr = tb.tree.ensure<uint32_t>(2 * padded * S * 4);
  core_inverse_async_raw(k, in, sel, out, count, tr, task, errp, st);
}

// Same, on a caller-provided tree buffer of 2 * padded ciphertexts.  With
// inline_host the root is inverted by the calling thread after waiting for
// the stream (the latency class of the server does this on its own
// scheduler thread, so its batches never queue behind other streams' host
// functions on the runtime's callback thread); otherwise by a host function
// in stream order.
void core_inverse_async_raw(KeyRec& k, const uint32_t* in, const int64_t* sel, uint32_t* out, size_t count,
                            uint32_t* tr, InvTask& task, uint32_t* errp, cudaStream_t st, bool inline_host) {
  if (count == 0) return;
  size_t padded = 1;
  while (padded < count) padded <<= 1;
  const size_t S = (size_t)k.S;
  // level l occupies [off_l, off_l + padded >> l)
  std::vector<size_t> off;
  size_t total = 0;
  for (size_t sz = padded;; sz >>= 1) {
    off.push_back(total);
    total += sz;
    if (sz == 1) break;
  }
  task.N = &k.N;
  task.S = k.S;
  cuda_check(hg::launch_tree_leaves(k.S, k.kc, in, sel, count, tr, padded, errp, st), "tree leaves");
  for (size_t l = 0; l + 1 < off.size(); ++l) {
    const size_t up = padded >> (l + 1);
    cuda_check(hg::launch_tree_up(k.S, k.kc, tr + off[l] * S, tr + off[l + 1] * S, up, st), "tree up");
  }
  uint32_t* root = tr + off.back() * S;
  cuda_check(cudaMemcpyAsync(task.root, root, S * 4, cudaMemcpyDeviceToHost, st), "D2H root");
  cuda_check(cudaMemcpyAsync(task.root + S, errp, 4, cudaMemcpyDeviceToHost, st), "D2H err");
  if (inline_host) {
    cuda_check(cudaStreamSynchronize(st), "stream sync");
    inv_host_fn(&task);
  } else {
    cuda_check(cudaLaunchHostFunc(st, inv_host_fn, &task), "host inversion");
  }
  cuda_check(cudaMemcpyAsync(root, task.z, S * 4, cudaMemcpyHostToDevice, st), "H2D inverse");
  for (size_t l = off.size() - 1; l-- > 0;) {
    const size_t up = padded >> (l + 1);
    cuda_check(hg::launch_tree_down(k.S, k.kc, tr + off[l] * S, tr + off[l + 1] * S, up, st), "tree down");
  }
  cuda_check(hg::launch_tree_apply(k.S, k.kc, in, sel, tr, out, count, st), "tree apply");
}

void raise_task_status(const InvTask& t) {
  if (t.status == 2) fail(HG_ERR_CT_RANGE, "Invalid ciphertext: value >= n^2");
  if (t.status == 1) fail(HG_ERR_NOT_INVERTIBLE, "ciphertext not invertible mod n^2 (Negate/Sub/Mul with k<0)");
}

// The lane's inversion in stream order; w.task.status (reset by the caller)
// records a failure once the stream has run it.
void core_inverse_enqueue(KeyRec& k, Work& w, const uint32_t* in, const int64_t* sel, uint32_t* out,
                          size_t count) {
  if (count == 0) return;
  w.task.root = w.pin_root.ensure<uint32_t>((size_t)k.S * 4 + 4);
  w.task.z = w.pin_z.ensure<uint32_t>((size_t)k.S * 4);
  core_inverse_async(k, in, sel, out, count, w.inv, w.task, w.errp(), w.stream);
}

// Synchronous form used by the host-pointer and device-pointer calls.
void core_inverse(KeyRec& k, Work& w, const uint32_t* in, const int64_t* sel, uint32_t* out, size_t count) {
  if (count == 0) return;
  w.task.status = 0;
  core_inverse_enqueue(k, w, in, sel, out, count);
  cuda_check(cudaStreamSynchronize(w.stream), "stream sync");
  raise_task_status(w.task);
}

// sync_inverse = false leaves the inversion (k < 0) in stream order: the
// caller resets w.task.status first and checks it after the stream drained.
void core_mul(KeyRec& k, Work& w, const uint32_t* a, const int64_t* kk, const int64_t* host_k, uint32_t* out,
              size_t count, bool sync_inverse = true) {
  const size_t ntab = (size_t)1 << (k.wm - 1);
  const size_t inst = (size_t)k.grid_mul * hg::instances_per_block(k.S, k.kc.variant);
  uint32_t* scratch = w.scratch.ensure<uint32_t>(inst * ntab * k.S * 4);
  cuda_check(hg::launch_mul(k.S, k.kc, a, kk, out, count, scratch, k.wm, w.errp(), k.grid_mul, w.ctrp(), w.stream),
             "mul launch");
  bool any_neg = true;
  if (host_k) {
    any_neg = false;
    for (size_t i = 0; i < count && !any_neg; ++i) any_neg = host_k[i] < 0;
  }
  if (any_neg) {
    if (sync_inverse)
      core_inverse(k, w, out, kk, out, count);
    else
      core_inverse_enqueue(k, w, out, kk, out, count);
  }
}

// Sliding-window width for exponents of at most `bits` bits: the w in 1..8
// with the fewest multiplications, bits / (w + 1) window products plus the
// 2^(w-1) odd powers of the table.
int bn_window(size_t bits) {
  int best = 1;
  double cost = 1e300;
  for (int w = 1; w <= 8; ++w) {
    const double c = (double)bits / (w + 1) + (double)(1 << (w - 1));
    if (c < cost) {
      cost = c;
      best = w;
    }
  }
  return best;
}

// Mul(ct, k) for multi-limb scalars (evaluator.cc:99-123): magnitudes emag
// (el limbs each) and signs eneg on the device; max_bits bounds the
// magnitudes (it sets the window); any_neg = false skips the inverse.
void core_mul_bn(KeyRec& k, Work& w, const uint32_t* a, const uint32_t* emag, int el, const uint8_t* eneg,
                 size_t max_bits, bool any_neg, uint32_t* out, size_t count, bool sync_inverse = true) {
  if (el < 1 || el > k.S) fail(HG_ERR_INVALID, "scalar limbs must be in [1, S] (at most the width of n^2)");
  if (count == 0) return;
  const int wb = bn_window(std::max<size_t>(max_bits, 1));
  if (k.grid_mul_bn == 0) k.grid_mul_bn = hg::resident_blocks_mul_bn(k.S);
  const size_t inst = (size_t)k.grid_mul_bn * hg::instances_per_block(k.S, 0);
  uint32_t* scratch = w.scratch.ensure<uint32_t>(inst * ((size_t)1 << (wb - 1)) * k.S * 4);
  cuda_check(hg::launch_mul_bn(k.S, k.kc, a, emag, el, out, count, scratch, wb, w.errp(), k.grid_mul_bn, w.ctrp(),
                               w.stream),
             "mul_bn launch");
  if (any_neg) {
    int64_t* sel = w.sel.ensure<int64_t>(count * 8);
    cuda_check(hg::launch_sel_from_neg(eneg, sel, count, w.stream), "sign selector");
    if (sync_inverse)
      core_inverse(k, w, out, sel, out, count);
    else
      core_inverse_enqueue(k, w, out, sel, out, count);
  }
}

// Multiprocessors of the current device (the caller has selected it).
int current_sm_count() {
  int dev = 0, sms = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
  return sms;
}

void core_sum(KeyRec& k, Work& w, const uint32_t* a, size_t count, uint32_t* out) {
  if (count == 0) fail(HG_ERR_INVALID, "you cannot sum an empty tensor");
  const size_t S = (size_t)k.S;
  const int sms = current_sm_count();
  const uint32_t* cur = a;
  size_t n = count;
  int which = 0;
  if (n == 1) {
    cuda_check(cudaMemcpyAsync(out, a, S * 4, cudaMemcpyDeviceToDevice, w.stream), "copy");
    return;
  }
  // tree levels: groups multiply chunks, blocks combine their groups by warp
  // shuffles (one output per block); three levels for 2^20 inputs
  while (n > 1) {
    const int chunk = hg::reduce_tree_chunk(k.S, n, sms);
    const size_t outn = hg::reduce_tree_outputs(k.S, n, chunk);
    uint32_t* dst = (outn == 1) ? out : w.red[which].ensure<uint32_t>(outn * S * 4);
    cuda_check(hg::launch_reduce_tree(k.S, k.kc, cur, n, chunk, dst, w.errp(), w.stream), "reduce launch");
    cur = dst;
    n = outn;
    which ^= 1;
  }
}


// FeatureWiseBucketSum (numpy/evaluator.cc:378-458) over device arrays.
void core_bucket_sum(KeyRec& k, Work& w, const uint32_t* x, size_t rows, size_t cols, const uint8_t* om, int F,
                     int B, int cumsum, uint32_t* out) {
  if (rows == 0 || cols == 0) fail(HG_ERR_INVALID, "you cannot sum an empty tensor");
  if (F <= 0 || B <= 0 || B > 256) fail(HG_ERR_INVALID, "features must be > 0 and 0 < bucket_num <= 256");
  const size_t S = (size_t)k.S;
  const int nseg = F * B;
  if ((size_t)F * rows >= (1ull << 32)) fail(HG_ERR_INVALID, "features * rows must be < 2^32");
  uint32_t* cnt = w.seg_cnt.ensure<uint32_t>((size_t)nseg * 4);
  uint32_t* offs0 = w.seg_offs[0].ensure<uint32_t>(((size_t)nseg + 1) * 4);
  uint32_t* cursor = w.seg_cursor.ensure<uint32_t>((size_t)nseg * 4);
  uint32_t* idx = w.seg_idx.ensure<uint32_t>((size_t)F * rows * 4);
  uint32_t* nch = w.seg_nch.ensure<uint32_t>((size_t)nseg * 4);
  cuda_check(hg::launch_bin_sort(om, rows, F, B, cnt, offs0, cursor, idx, w.errp(), w.stream), "bin sort");
  const int C = 64;
  for (size_t col = 0; col < cols; ++col) {
    const uint32_t* vals = x;
    size_t stride = cols, voff = col;
    const uint32_t* vidx = idx;
    const uint32_t* offs_in = offs0;
    size_t total_in = (size_t)F * rows;  // elements across all segments
    size_t max_len = rows;
    int which = 0;
    do {
      const size_t upper = total_in / C + (size_t)nseg + 1;
      uint32_t* part = w.seg_part[which].ensure<uint32_t>(upper * S * 4);
      uint32_t* offs_out = w.seg_offs[1 + which].ensure<uint32_t>(((size_t)nseg + 1) * 4);
      cuda_check(hg::launch_seg_level(k.S, k.kc, vals, stride, voff, vidx, offs_in, nseg, C, nch, offs_out, part,
                                      upper, w.errp(), w.stream),
                 "segment level");
      vals = part;
      stride = 1;
      voff = 0;
      vidx = nullptr;
      offs_in = offs_out;
      total_in = upper;
      max_len = (max_len + C - 1) / C;
      which ^= 1;
    } while (max_len > 1);
    cuda_check(hg::launch_seg_finalize(k.S, vals, offs_in, nseg, k.kc.R1, out, cols, col, w.stream), "finalize");
    if (cumsum) cuda_check(hg::launch_bucket_cumsum(k.S, k.kc, out, F, B, cols, col, w.stream), "cumsum");
  }
}

// numpy MatMul of ciphertexts x (M x K) by int64 plaintexts y (K x N, host).
// MatMul over exponents given as bit planes: bit(kk, j, plane) is bit `plane`
// of y'(kk, j) = y(kk, j) + o >= 0 (P planes); o >= 0 is undone per row with
// (prod_k x(i,k))^-o.
template <typename Bit>
void core_matmul_planes(KeyRec& k, Work& w, const uint32_t* x, size_t M, size_t K, size_t N, int P, Bit&& bit,
                        const BN& o, uint32_t* out) {
  const int nch = (int)((K + 7) / 8);
  std::vector<uint8_t> hm((size_t)N * P * nch, 0);
  for (size_t j = 0; j < N; ++j)
    for (int plane = 0; plane < P; ++plane)
      for (int c = 0; c < nch; ++c) {
        uint8_t mk = 0;
        for (int b = 0; b < 8; ++b) {
          const size_t kk = (size_t)c * 8 + b;
          if (kk < K && bit(kk, j, plane)) mk |= (uint8_t)(1u << b);
        }
        hm[((size_t)j * P + plane) * nch + c] = mk;
      }
  uint8_t* dmask = w.mm_masks.ensure<uint8_t>(hm.size());
  cuda_check(cudaMemcpyAsync(dmask, hm.data(), hm.size(), cudaMemcpyHostToDevice, w.stream), "H2D masks");
  // o as exponent limbs on the device (only used when it does not fit 64 bits)
  const std::vector<uint32_t> ol = o.limbs(std::max<size_t>(1, (o.bitlen() + 31) / 32));
  uint32_t* dexp = nullptr;
  if (o.bitlen() > 64) {
    dexp = w.mm_exp.ensure<uint32_t>(ol.size() * 4);
    cuda_check(cudaMemcpyAsync(dexp, ol.data(), ol.size() * 4, cudaMemcpyHostToDevice, w.stream), "H2D exponent");
  }
  const size_t per_row = hg::subset_table_bytes_per_row(k.S, (int)K);
  const size_t budget = (size_t)8 << 30;
  const size_t Rb = std::max<size_t>(1, std::min(M, budget / per_row));
  uint32_t* T = w.mm_tables.ensure<uint32_t>(Rb * per_row);
  uint32_t* prod = w.mm_prod.ensure<uint32_t>(Rb * (size_t)k.S * 4);
  for (size_t r0 = 0; r0 < M; r0 += Rb) {
    const size_t rows = std::min(Rb, M - r0);
    cuda_check(hg::launch_subset_tables(k.S, k.kc, x, r0, rows, (int)K, T, w.errp(), w.stream), "subset tables");
    cuda_check(hg::launch_matmul_planes(k.S, k.kc, T, dmask, r0, rows, (int)N, P, (int)K, out, w.stream),
               "matmul planes");
    if (!o.is_zero()) {
      cuda_check(hg::launch_row_products(k.S, k.kc, T, rows, (int)K, prod, w.stream), "row products");
      core_inverse(k, w, prod, nullptr, prod, rows);
      if (dexp)
        cuda_check(hg::launch_pow_shared_bn(k.S, k.kc, prod, rows, dexp, (int)ol.size(), w.stream), "row power");
      else
        cuda_check(hg::launch_pow_shared(k.S, k.kc, prod, rows, o.low64(), w.stream), "row power");
      cuda_check(hg::launch_scale_rows(k.S, k.kc, out, prod, r0, rows, (int)N, w.stream), "scale rows");
    }
  }
  // keep the host mask and exponent arrays alive until their copies have run
  cuda_check(cudaStreamSynchronize(w.stream), "stream sync");
}

void check_matmul_dims(size_t M, size_t K, size_t N) {
  if (M == 0 || K == 0 || N == 0) fail(HG_ERR_INVALID, "HEU does not support empty tensor currently");
  if (K > (1u << 20) || N > (1u << 20)) fail(HG_ERR_INVALID, "matmul dimension too large");
}

void core_matmul(KeyRec& k, Work& w, const uint32_t* x, size_t M, size_t K, const int64_t* y, size_t N,
                 uint32_t* out) {
  check_matmul_dims(M, K, N);
  int64_t ymin = y[0], ymax = y[0];
  for (size_t i = 1; i < K * N; ++i) {
    ymin = std::min(ymin, y[i]);
    ymax = std::max(ymax, y[i]);
  }
  // shift to y' = y + o >= 0; undo with (prod_k x(i,k))^-o per row
  const uint64_t o = ymin < 0 ? (uint64_t)0 - (uint64_t)ymin : 0;
  const uint64_t ymax_s = (uint64_t)ymax + o;
  int P = 1;
  while (P < 64 && (ymax_s >> P) != 0) ++P;
  core_matmul_planes(k, w, x, M, K, N, P,
                     [&](size_t kk, size_t j, int plane) { return ((((uint64_t)y[kk * N + j] + o) >> plane) & 1ull) != 0; },
                     BN(o), out);
}

// MatMul with plaintext entries of any size (numpy/evaluator.cc:208-353 takes
// any PMatrix): y(kk, j) = (neg ? -1 : 1) * magnitude of yl limbs.
void core_matmul_bn(KeyRec& k, Work& w, const uint32_t* x, size_t M, size_t K, const uint32_t* y_mag,
                    const uint8_t* y_neg, size_t yl, size_t N, uint32_t* out) {
  check_matmul_dims(M, K, N);
  if (yl < 1 || yl > (size_t)k.S) fail(HG_ERR_INVALID, "plaintext limbs must be in [1, S]");
  const size_t cnt = K * N;
  std::vector<BN> mag(cnt);
  BN o(0);
  for (size_t i = 0; i < cnt; ++i) {
    mag[i] = BN::from_limbs(y_mag + i * yl, yl);
    if (y_neg[i] && !mag[i].is_zero() && mag[i] > o) o = mag[i];
  }
  // y' = y + o: o - |y| for negative entries, o + |y| otherwise
  std::vector<BN> ys(cnt);
  size_t P = 1;
  for (size_t i = 0; i < cnt; ++i) {
    ys[i] = (y_neg[i] && !mag[i].is_zero()) ? o - mag[i] : o + mag[i];
    P = std::max(P, ys[i].bitlen());
  }
  if (P > 32 * (size_t)k.S + 1) fail(HG_ERR_INVALID, "plaintext too wide");
  core_matmul_planes(k, w, x, M, K, N, (int)P,
                     [&](size_t kk, size_t j, int plane) { return ys[kk * N + j].bit((size_t)plane); }, o, out);
}

int load_key(hg_ctx* ctx, uint32_t key_bits, const uint32_t* n_l, const uint32_t* hs_l, const uint32_t* p_l,
                 const uint32_t* q_l, int window) {
  if (key_bits % 64 != 0) fail(HG_ERR_UNSUPPORTED, "key size must be a multiple of 64 bits");
  const int S = (int)key_bits / 16;
  if (!hg::supported_limbs(S)) fail(HG_ERR_UNSUPPORTED, "no compiled variant for " + std::to_string(key_bits) + "-bit keys");
  auto k = std::make_unique<KeyRec>();
  k->key_bits = (int)key_bits;
  k->S = S;
  k->Sp = S / 2;
  k->H = S / 4;
  k->n = BN::from_limbs(n_l, S / 2);
  if (!k->n.is_odd() || k->n.bitlen() < 16) fail(HG_ERR_INVALID, "n must be odd");
  k->N = k->n * k->n;
  k->hs = BN::from_limbs(hs_l, S);
  if (k->hs >= k->N) fail(HG_ERR_INVALID, "h_s must be < n^2");
  const BN R = BN(1).shl(32 * (size_t)S);
  const BN R1 = R % k->N, R2 = (R1 * R1) % k->N, R3 = (R2 * R1) % k->N;
  const BN nR2 = (k->n * R2) % k->N;
  const BN hsm = (k->hs * R1) % k->N;
  const BN nhalf = k->n.shr(1);
  const size_t key_size = k->n.bitlen();
  // device constants: N R1 R2 R3 nR2 hsm (S each), n nhalf (S/2 each)
  std::vector<uint32_t> hc(7 * (size_t)S);
  auto put = [&](size_t at, const BN& v, size_t limbs) { v.to_limbs(hc.data() + at, limbs); };
  put(0, k->N, S);
  put(S, R1, S);
  put(2 * S, R2, S);
  put(3 * S, R3, S);
  put(4 * S, nR2, S);
  put(5 * S, hsm, S);
  put(6 * S, k->n, S / 2);
  put(6 * S + S / 2, nhalf, S / 2);
  uint32_t* dc = k->consts.ensure<uint32_t>(hc.size() * 4);
  cuda_check(cudaMemcpy(dc, hc.data(), hc.size() * 4, cudaMemcpyHostToDevice), "upload consts");
  auto& kc = k->kc;
  kc.N = dc;
  kc.R1 = dc + S;
  kc.R2 = dc + 2 * S;
  kc.R3 = dc + 3 * S;
  kc.nR2 = dc + 4 * S;
  kc.n = dc + 6 * S;
  kc.nhalf = dc + 6 * S + S / 2;
  kc.np = neg_inv32(k->N.d[0]);
  kc.S = S;
  kc.w = window > 0 ? window : 12;
  if (kc.w > 20) fail(HG_ERR_INVALID, "table window must be <= 20");
  kc.rbits = (int)(key_size / 2);
  kc.rlimbs = (int)key_bits / 64;
  kc.npos = (kc.rbits + kc.w - 1) / kc.w;
  // fixed-base table on the device
  const size_t ent = ((size_t)1 << kc.w) - 1;
  uint32_t* tab = k->table.ensure<uint32_t>((size_t)kc.npos * ent * S * 4);
  kc.table = tab;
  {
    DevBuf bases;
    uint32_t* b = bases.ensure<uint32_t>((size_t)kc.npos * S * 4);
    cuda_check(hg::launch_table_bases(S, kc, dc + 5 * S, b, nullptr), "table bases");
    cuda_check(hg::launch_table_level(S, kc, tab, b, -1, nullptr), "table level");
    for (int lv = 0; lv < kc.w; ++lv) cuda_check(hg::launch_table_level(S, kc, tab, b, lv, nullptr), "table level");
    cuda_check(cudaDeviceSynchronize(), "table build");
  }
  kc.variant = 0;
  k->grid_mul = hg::resident_blocks_mul(S, 0);
  if (p_l && q_l) {
    const int Sp = S / 2, H = S / 4;
    k->p = BN::from_limbs(p_l, H);
    k->q = BN::from_limbs(q_l, H);
    if (k->p * k->q != k->n) fail(HG_ERR_INVALID, "pk and sk are not paired: p*q != n");
    if (!k->p.is_odd() || !k->q.is_odd()) fail(HG_ERR_INVALID, "p and q must be odd");
    k->secret = true;
    const BN p2 = k->p * k->p, q2 = k->q * k->q;
    const BN R1h = BN(1).shl(32 * (size_t)H);
    auto hfun = [&](const BN& pr, const BN& pr2) {
      // secret_key.cc:33-42: h = L((n+1)^(pr-1) mod pr^2)^-1 mod pr
      const BN g = k->n + BN(1);
      BN hv = hg::HostMont(pr2).pow(g, pr - BN(1));
      hv = (hv - BN(1)) / pr;
      return BN::invmod(hv, pr);
    };
    const BN hp = hfun(k->p, p2), hq = hfun(k->q, q2);
    const BN pinvq = BN::invmod(k->p, k->q);
    // p2 q2 (Sp) | p q hR_p hR_q inv2_p inv2_q pinvqR (H)
    std::vector<uint32_t> hs2(2 * (size_t)Sp + 7 * (size_t)H);
    auto put2 = [&](size_t at, const BN& v, size_t limbs) { v.to_limbs(hs2.data() + at, limbs); };
    put2(0, p2, Sp);
    put2(Sp, q2, Sp);
    size_t o = 2 * (size_t)Sp;
    put2(o, k->p, H);
    put2(o + H, k->q, H);
    put2(o + 2 * H, (hp * R1h) % k->p, H);
    put2(o + 3 * H, (hq * R1h) % k->q, H);
    put2(o + 4 * H, BN::invmod(k->p, R1h), H);
    put2(o + 5 * H, BN::invmod(k->q, R1h), H);
    put2(o + 6 * H, (pinvq * R1h) % k->q, H);
    uint32_t* ds = k->sconsts.ensure<uint32_t>(hs2.size() * 4);
    cuda_check(cudaMemcpy(ds, hs2.data(), hs2.size() * 4, cudaMemcpyHostToDevice), "upload secret consts");
    auto& sc = k->sc;
    sc.Sp = Sp;
    sc.P2[0] = ds;
    sc.P2[1] = ds + Sp;
    sc.P[0] = ds + o;
    sc.P[1] = ds + o + H;
    sc.hR[0] = ds + o + 2 * H;
    sc.hR[1] = ds + o + 3 * H;
    sc.inv2[0] = ds + o + 4 * H;
    sc.inv2[1] = ds + o + 5 * H;
    sc.pinvqR = ds + o + 6 * H;
    sc.np2[0] = neg_inv32(p2.d[0]);
    sc.np2[1] = neg_inv32(q2.d[0]);
    sc.np1[0] = neg_inv32(k->p.d[0]);
    sc.np1[1] = neg_inv32(k->q.d[0]);
    sc.wd = 5;
    std::vector<uint16_t> pp, pq;
    build_prog(k->p - BN(1), sc.wd, &sc.start[0], &pp);
    build_prog(k->q - BN(1), sc.wd, &sc.start[1], &pq);
    const size_t len = std::max(pp.size(), pq.size());
    pp.resize(len, hg::kOpNop);
    pq.resize(len, hg::kOpNop);
    sc.prog_len = (int)len;
    uint16_t* dp = k->progs.ensure<uint16_t>(std::max<size_t>(2 * len, 2) * 2);
    if (len) {
      cuda_check(cudaMemcpy(dp, pp.data(), len * 2, cudaMemcpyHostToDevice), "upload prog");
      cuda_check(cudaMemcpy(dp + len, pq.data(), len * 2, cudaMemcpyHostToDevice), "upload prog");
    }
    sc.prog[0] = dp;
    sc.prog[1] = dp + len;
    sc.variant = 0;
    k->grid_dec = hg::resident_blocks_decrypt(Sp, 0);
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  const int id = ctx->next_key++;
  ctx->keys[id] = std::move(k);
  return id;
}

// Fixed-base table of `base_mont` powers over the modulus of `t` (npos x
// (2^w - 1) entries, Montgomery form), the layout k_encrypt reads.
void build_fixed_base(int S, hg::KeyConst& t, DevBuf& buf, const uint32_t* base_mont, int exp_bits, int window) {
  t.w = window;
  t.rbits = exp_bits;
  t.npos = (exp_bits + window - 1) / window;
  const size_t ent = ((size_t)1 << window) - 1;
  t.table = buf.ensure<uint32_t>((size_t)t.npos * ent * S * 4);
  DevBuf bases;
  uint32_t* b = bases.ensure<uint32_t>((size_t)t.npos * S * 4);
  cuda_check(hg::launch_table_bases(S, t, base_mont, b, nullptr), "table bases");
  cuda_check(hg::launch_table_level(S, t, const_cast<uint32_t*>(t.table), b, -1, nullptr), "table level");
  for (int lv = 0; lv < window; ++lv)
    cuda_check(hg::launch_table_level(S, t, const_cast<uint32_t*>(t.table), b, lv, nullptr), "table level");
  cuda_check(cudaDeviceSynchronize(), "table build");
}

int ou_random_bits(size_t n_bits) {  // ou/encryptor.cc:12-20, public_key.h:27-31
  return n_bits >= 2560 ? 128 : n_bits >= 1536 ? 110 : 80;
}

void ou_sizes(uint32_t key_bits, int* S, int* Sp) {
  if (key_bits == 1024) {
    *S = 64;
    *Sp = 32;
  } else if (key_bits == 2048) {
    *S = 128;
    *Sp = 64;
  } else if (key_bits == 3072) {
    *S = 128;
    *Sp = 96;
  } else {
    fail(HG_ERR_UNSUPPORTED, "OU keys of 1024, 2048 or 3072 bits");
  }
}

// Okamoto-Uchiyama key (ou/public_key.cc:28-41, secret_key.h): tables for
// H (encryption randomness), G and G^-1 (plaintexts); CRT-free decryption
// constants mod p^2.
int load_ou_key(hg_ctx* ctx, uint32_t key_bits, const uint32_t* n_l, const uint32_t* G_l, const uint32_t* H_l,
                int max_pt_bits, const uint32_t* p_l, const uint32_t* q_l, const uint32_t* t_l,
                const uint32_t* gpinv_l, int window) {
  int S = 0, Sp = 0;
  ou_sizes(key_bits, &S, &Sp);
  const int Hh = Sp / 2;
  auto k = std::make_unique<KeyRec>();
  k->scheme = 1;
  k->key_bits = (int)key_bits;
  k->S = S;
  k->Sp = Sp;
  k->H = Hh;
  k->pt_limbs = Hh;
  k->n = BN::from_limbs(n_l, S);
  k->N = k->n;
  if (!k->n.is_odd() || k->n.bitlen() < 64) fail(HG_ERR_INVALID, "n must be odd");
  if (max_pt_bits < 2 || max_pt_bits > 32 * Hh) fail(HG_ERR_INVALID, "max plaintext bits out of range");
  k->max_pt_bits = max_pt_bits + 1;  // |m| <= 2^max_pt_bits has max_pt_bits + 1 bits
  const BN G = BN::from_limbs(G_l, S), Hb = BN::from_limbs(H_l, S);
  if (G >= k->N || Hb >= k->N) fail(HG_ERR_INVALID, "G and H must be < n");
  if (BN::gcd(G, k->N) != BN(1)) fail(HG_ERR_INVALID, "G is not invertible mod n");
  const BN Gi = BN::invmod(G, k->N);
  const BN R = BN(1).shl(32 * (size_t)S);
  const BN R1 = R % k->N, R2 = (R1 * R1) % k->N, R3 = (R2 * R1) % k->N;
  const BN maxpt = BN(1).shl((size_t)max_pt_bits);
  // N R1 R2 R3 nR2(0) Hm Gm Gim zeros(S) maxpt(Hh)
  std::vector<uint32_t> hc(9 * (size_t)S + Hh, 0u);
  auto put = [&](size_t at, const BN& v, size_t limbs) { v.to_limbs(hc.data() + at, limbs); };
  put(0, k->N, S);
  put(S, R1, S);
  put(2 * S, R2, S);
  put(3 * S, R3, S);
  put(5 * S, (Hb * R1) % k->N, S);
  put(6 * S, (G * R1) % k->N, S);
  put(7 * S, (Gi * R1) % k->N, S);
  put(9 * S, maxpt, Hh);
  uint32_t* dc = k->consts.ensure<uint32_t>(hc.size() * 4);
  cuda_check(cudaMemcpy(dc, hc.data(), hc.size() * 4, cudaMemcpyHostToDevice), "upload consts");
  auto& kc = k->kc;
  kc.N = dc;
  kc.R1 = dc + S;
  kc.R2 = dc + 2 * S;
  kc.R3 = dc + 3 * S;
  kc.nR2 = dc + 4 * S;
  kc.n = dc + 8 * S;
  kc.nhalf = dc + 8 * S;
  kc.np = neg_inv32(k->N.d[0]);
  kc.S = S;
  kc.variant = 0;
  k->d_maxpt = dc + 9 * S;
  const int w = window > 0 ? window : 12;
  if (w > 20) fail(HG_ERR_INVALID, "table window must be <= 20");
  k->kcG = kc;
  k->kcGi = kc;
  // H^r with r < 2^128 (the table covers kRandomBits3072, public_key.cc:38-39)
  build_fixed_base(S, kc, k->table, dc + 5 * S, 128, w);
  kc.rbits = ou_random_bits(k->n.bitlen());
  kc.npos = (kc.rbits + w - 1) / w;
  kc.rlimbs = 4;
  build_fixed_base(S, k->kcG, k->tableG, dc + 6 * S, k->max_pt_bits, w);
  build_fixed_base(S, k->kcGi, k->tableGi, dc + 7 * S, k->max_pt_bits, w);
  k->grid_mul = hg::resident_blocks_mul(S, 0);
  if (p_l && q_l && t_l && gpinv_l) {
    k->p = BN::from_limbs(p_l, S / 2);
    k->q = BN::from_limbs(q_l, S / 2);
    const BN t = BN::from_limbs(t_l, S / 2), gpinv = BN::from_limbs(gpinv_l, S / 2);
    const BN p2 = k->p * k->p;
    if (p2 * k->q != k->n) fail(HG_ERR_INVALID, "pk and sk are not paired: p^2 * q != n");
    if (p2.bitlen() > 32 * (size_t)Sp || k->p.bitlen() > 32 * (size_t)Hh) fail(HG_ERR_INVALID, "p too large");
    k->secret = true;
    const BN Rp = BN(1).shl(32 * (size_t)Sp), Rh = BN(1).shl(32 * (size_t)Hh);
    const BN Rp1 = Rp % p2;
    const BN Kfix = (((Rp1 * Rp1) % p2) * Rp1 % p2) * BN::invmod(R % p2, p2) % p2;
    // p2 Kfix (Sp) | p gpR pinv phalf (Hh)
    std::vector<uint32_t> hs2(2 * (size_t)Sp + 4 * (size_t)Hh, 0u);
    auto put2 = [&](size_t at, const BN& v, size_t limbs) { v.to_limbs(hs2.data() + at, limbs); };
    put2(0, p2, Sp);
    put2(Sp, Kfix, Sp);
    const size_t o = 2 * (size_t)Sp;
    put2(o, k->p, Hh);
    put2(o + Hh, (gpinv * (Rh % k->p)) % k->p, Hh);
    put2(o + 2 * Hh, BN::invmod(k->p, Rh), Hh);
    put2(o + 3 * Hh, k->p.shr(1), Hh);
    uint32_t* ds = k->oconsts.ensure<uint32_t>(hs2.size() * 4);
    cuda_check(cudaMemcpy(ds, hs2.data(), hs2.size() * 4, cudaMemcpyHostToDevice), "upload secret consts");
    auto& oc = k->oc;
    oc.Sp = Sp;
    oc.P2 = ds;
    oc.Kfix = ds + Sp;
    oc.P = ds + o;
    oc.gpR = ds + o + Hh;
    oc.pinv = ds + o + 2 * Hh;
    oc.phalf = ds + o + 3 * Hh;
    oc.np2 = neg_inv32(p2.d[0]);
    oc.np1 = neg_inv32(k->p.d[0]);
    oc.wd = 5;
    std::vector<uint16_t> prog;
    build_prog(t, oc.wd, &oc.start, &prog);
    oc.prog_len = (int)prog.size();
    uint16_t* dp = k->oprog.ensure<uint16_t>(std::max<size_t>(prog.size(), 1) * 2);
    if (!prog.empty()) cuda_check(cudaMemcpy(dp, prog.data(), prog.size() * 2, cudaMemcpyHostToDevice), "prog");
    oc.prog = dp;
    cuda_check(hg::ou_decrypt_geometry(S, Sp, &k->grid_oudec, &k->upb_oudec), "OU decrypt geometry");
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  const int id = ctx->next_key++;
  ctx->keys[id] = std::move(k);
  return id;
}

// key generation (key_generator.cc:26-60) from a seeded stream
std::vector<uint32_t> small_primes() {
  std::vector<uint32_t> out;
  std::vector<bool> sieve(2000, true);
  for (uint32_t i = 2; i < 2000; ++i) {
    if (!sieve[i]) continue;
    out.push_back(i);
    for (uint32_t j = i * i; j < 2000; j += i) sieve[j] = false;
  }
  return out;
}

bool is_probable_prime(const BN& c, const std::vector<uint32_t>& sp) {
  if (c < BN(2)) return false;
  for (uint32_t p : sp) {
    if (c == BN(p)) return true;
    if ((c % BN(p)).is_zero()) return false;
  }
  const BN cm1 = c - BN(1);
  BN d = cm1;
  size_t s = 0;
  while (!d.is_odd()) {
    d = d.shr(1);
    ++s;
  }
  hg::HostMont mont(c);
  for (size_t bi = 0; bi < 20; ++bi) {
    const BN a(sp[bi]);
    BN x = mont.pow(a, d);
    if (x == BN(1) || x == cm1) continue;
    bool comp = true;
    for (size_t r = 1; r < s; ++r) {
      x = (x * x) % c;
      if (x == cm1) {
        comp = false;
        break;
      }
    }
    if (comp) return false;
  }
  return true;
}

BN rand_prime_bbs(hg::Xoshiro& prg, size_t bits, const std::vector<uint32_t>& sp) {
  while (true) {
    BN c = prg.randbits(bits);
    if (c.d.size() < (bits + 31) / 32) c.d.resize((bits + 31) / 32, 0);
    c.d[(bits - 1) / 32] |= 1u << ((bits - 1) % 32);
    c.d[0] |= 3u;
    c.trim();
    if (is_probable_prime(c, sp)) return c;
  }
}

}  // namespace

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

const char* hg_last_error(void) { return g_last_error.c_str(); }

int hg_ctx_create(int device, hg_ctx** out) {
  return guarded(__func__, [&] {
    if (!out) fail(HG_ERR_INVALID, "null out pointer");
    auto ctx = std::make_unique<hg_ctx>();
    ctx->device = device;
    // Streams share the device's hardware work queues round-robin (8 by
    // default); a stream whose next command waits on its own kernel then
    // holds up every stream behind it in the same queue.  The server's slots
    // must not wait on one another that way, so ask for the most queues
    // unless the user has chosen a number; this takes effect when the
    // process's CUDA context is created by the call below.
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    hg::forget_noalloc_scratch(device);
    cuda_check(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device), "attr");
    for (int i = 0; i < kLanes; ++i) {
      auto w = std::make_unique<Work>();
      cuda_check(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking), "stream create");
      w->own_stream = true;
      ctx->free_lanes.push_back(w.get());
      ctx->lanes.push_back(std::move(w));
    }
    *out = ctx.release();
    return HG_OK;
  });
}

int hg_ctx_destroy(hg_ctx* ctx) {
  return guarded(__func__, [&] {
    if (!ctx) return HG_OK;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    delete ctx;
    return HG_OK;
  });
}

int hg_device_sm_count(hg_ctx* ctx) { return ctx ? ctx->sm_count : 0; }

int hg_keygen(uint32_t key_bits, uint64_t seed, uint32_t* n_out, uint32_t* p_out, uint32_t* q_out,
              uint32_t* hs_out) {
  return guarded(__func__, [&] {
    if (key_bits % 64 != 0 || key_bits < 128) fail(HG_ERR_INVALID, "Key size must be a multiple of 64");
    hg::Xoshiro prg(seed);
    const auto sp = small_primes();
    const size_t half = key_bits / 2;
    BN p, q, n;
    while (true) {
      p = rand_prime_bbs(prg, half, sp);
      while (true) {
        q = rand_prime_bbs(prg, half, sp);
        const BN c = BN::gcd(p - BN(1), q - BN(1));
        const BN diff = p > q ? p - q : q - p;
        if (c == BN(2) && diff.bitlen() >= half - 2) break;
      }
      n = p * q;
      if (n.bitlen() >= key_bits) break;
    }
    BN x;
    while (true) {
      x = prg.below(n);
      if (BN::gcd(x, n) == BN(1)) break;
    }
    const BN x2 = (x * x) % n;
    const BN N = n * n;
    // h = -x^2 mod n as a residue mod n^2; h_s = h^n mod n^2 (CRT in the
    // reference, secret_key.cc:45-62; the value is the same)
    const BN h = N - x2;
    const BN hs = hg::HostMont(N).pow(h, n);
    if (n_out) n.to_limbs(n_out, key_bits / 32);
    if (p_out) p.to_limbs(p_out, key_bits / 64);
    if (q_out) q.to_limbs(q_out, key_bits / 64);
    if (hs_out) hs.to_limbs(hs_out, key_bits / 16);
    return HG_OK;
  });
}

int hg_key_load(hg_ctx* ctx, uint32_t key_bits, const uint32_t* n, const uint32_t* h_s, const uint32_t* p,
                const uint32_t* q, int table_window, int* key_id) {
  return guarded(__func__, [&] {
    if (!ctx || !n || !h_s || !key_id) fail(HG_ERR_INVALID, "null argument");
    if ((p == nullptr) != (q == nullptr)) fail(HG_ERR_INVALID, "give both p and q or neither");
    set_device(ctx);
    *key_id = load_key(ctx, key_bits, n, h_s, p, q, table_window);
    return HG_OK;
  });
}

int hg_ou_keygen(uint32_t key_bits, uint64_t seed, uint32_t* n_out, uint32_t* G_out, uint32_t* H_out,
                 uint32_t* p_out, uint32_t* q_out, uint32_t* t_out, uint32_t* gpinv_out, int* max_pt_bits) {
  return guarded(__func__, [&] {
    int S = 0, Sp = 0;
    ou_sizes(key_bits, &S, &Sp);
    hg::Xoshiro prg(seed);
    const auto sp = small_primes();
    const size_t secret = (key_bits + 2) / 3;
    const size_t pf = key_bits >= 3072 ? 256 : key_bits >= 2048 ? 224 : 160;
    if (pf * 2 > secret) fail(HG_ERR_INVALID, "Key size too small");
    auto rand_prime = [&](size_t bits) {
      while (true) {
        BN c = prg.randbits(bits);
        c.d.resize((bits + 31) / 32, 0);
        c.d[(bits - 1) / 32] |= 1u << ((bits - 1) % 32);
        c.d[0] |= 1u;
        c.trim();
        if (is_probable_prime(c, sp)) return c;
      }
    };
    const size_t ub = secret - pf + 2;
    BN t, u, p;
    while (true) {
      t = rand_prime(pf);
      u = prg.randbits(ub);
      u.d.resize((ub + 31) / 32, 0);
      u.d[(ub - 1) / 32] |= 1u << ((ub - 1) % 32);
      u.trim();
      p = t * u + BN(1);
      if (is_probable_prime(p, sp)) break;
    }
    const BN q = rand_prime(secret + 1);
    const BN p2 = p * p, n = p2 * q;
    BN g, gp;
    while (true) {
      while (true) {
        g = prg.below(n);
        if (BN::gcd(g, p) == BN(1)) break;
      }
      gp = hg::HostMont(p2).pow(g % p2, p - BN(1));
      if (hg::HostMont(p2).pow(gp, p) == BN(1)) break;
    }
    const BN gpinv = BN::invmod((gp - BN(1)) / p, p);
    BN g2;
    while (true) {
      g2 = prg.below(n);
      if (!(g2 % p).is_zero()) break;
    }
    hg::HostMont mn(n);
    const BN G = mn.pow(g, u), Hb = mn.pow(g2, n * u);
    if (n_out) n.to_limbs(n_out, S);
    if (G_out) G.to_limbs(G_out, S);
    if (H_out) Hb.to_limbs(H_out, S);
    if (p_out) p.to_limbs(p_out, S / 2);
    if (q_out) q.to_limbs(q_out, S / 2);
    if (t_out) t.to_limbs(t_out, S / 2);
    if (gpinv_out) gpinv.to_limbs(gpinv_out, S / 2);
    if (max_pt_bits) *max_pt_bits = (int)p.shr(1).bitlen() - 1;
    return HG_OK;
  });
}

int hg_ou_key_load(hg_ctx* ctx, uint32_t key_bits, const uint32_t* n, const uint32_t* G, const uint32_t* H,
                   int max_pt_bits, const uint32_t* p, const uint32_t* q, const uint32_t* t, const uint32_t* gp_inv,
                   int table_window, int* key_id) {
  return guarded(__func__, [&] {
    if (!ctx || !n || !G || !H || !key_id) fail(HG_ERR_INVALID, "null argument");
    const bool any = p || q || t || gp_inv, all = p && q && t && gp_inv;
    if (any && !all) fail(HG_ERR_INVALID, "give all of p, q, t, gp_inv or none");
    set_device(ctx);
    *key_id = load_ou_key(ctx, key_bits, n, G, H, max_pt_bits, p, q, t, gp_inv, table_window);
    return HG_OK;
  });
}

int hg_key_free(hg_ctx* ctx, int key_id) {
  return guarded(__func__, [&] {
    if (!ctx) fail(HG_ERR_INVALID, "null context");
    set_device(ctx);
    cuda_check(cudaDeviceSynchronize(), "sync");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->keys.erase(key_id)) fail(HG_ERR_INVALID, "unknown key id");
    return HG_OK;
  });
}

int hg_key_shape(hg_ctx* ctx, int key_id, int* ct_limbs, int* r_limbs, int* pt_limbs) {
  return guarded(__func__, [&] {
    KeyRec* k = get_key(ctx, key_id);
    if (ct_limbs) *ct_limbs = k->S;
    if (r_limbs) *r_limbs = k->kc.rlimbs;
    if (pt_limbs) *pt_limbs = k->scheme == 1 ? k->pt_limbs : k->S / 2;
    return HG_OK;
  });
}

// ---- host-pointer API -------------------------------------------------------
#define HG_HOST_PROLOGUE                       \
  KeyRec* k = get_key(ctx, key_id);            \
  if (count == 0) return HG_OK;                \
  set_device(ctx);                             \
  LaneGuard lane(ctx);                         \
  Work& w = *lane.w;                           \
  reset_err(w);                                \
  const size_t cb = ct_bytes(*k);              \
  (void)cb;

int hg_encrypt(hg_ctx* ctx, int key_id, const int64_t* m, const uint32_t* r, uint32_t* ct_out, size_t count) {
  return guarded(__func__, [&] {
    if (!m || !r || !ct_out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    const size_t rb = (size_t)k->kc.rlimbs * 4;
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* dm = v.io[0].ensure<int64_t>(cnt * 8);
      auto* dr = v.io[1].ensure<uint32_t>(cnt * rb);
      auto* dout = v.io[2].ensure<uint32_t>(cnt * cb);
      h2d(dm, m + off, cnt * 8, v);
      h2d(dr, (const uint8_t*)r + off * rb, cnt * rb, v);
      core_encrypt(*k, v, hg::EncMode::kEncrypt, dm, nullptr, nullptr, dr, nullptr, dout, cnt);
      d2h((uint8_t*)ct_out + off * cb, dout, cnt * cb, v);
    });
    return HG_OK;
  });
}

int hg_convert_radix(hg_ctx* ctx, int key_id, const uint32_t* in, uint32_t* out, size_t count, uint32_t radix_bits,
                     int to_external) {
  return guarded(__func__, [&] {
    if (!in || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    if (radix_bits == 0 || radix_bits > 65536) fail(HG_ERR_INVALID, "radix_bits must be in [1, 65536]");
    // R = 2^(32 S) here, R_ext = 2^radix_bits there
    const BN Rin = BN(1).shl(32 * (size_t)k->S) % k->N;
    const BN Rext = BN(1).shl(radix_bits) % k->N;
    // MM(c R, R_ext) = c R_ext;  MM(c R_ext, R^2 / R_ext) = c R
    const BN K = to_external ? Rext : (((Rin * Rin) % k->N) * BN::invmod(Rext, k->N)) % k->N;
    const std::vector<uint32_t> kl = K.limbs((size_t)k->S);
    auto* dk = w.io[3].ensure<uint32_t>(cb);
    h2d(dk, kl.data(), cb, w);
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* di = v.io[0].ensure<uint32_t>(cnt * cb);
      auto* dout = v.io[1].ensure<uint32_t>(cnt * cb);
      uint32_t* kv = dk;
      if (&v != &w) {  // the other lane needs its own copy of the constant
        kv = v.io[3].ensure<uint32_t>(cb);
        h2d(kv, kl.data(), cb, v);
      }
      h2d(di, (const uint8_t*)in + off * cb, cnt * cb, v);
      cuda_check(hg::launch_mul_const(k->S, k->kc, di, kv, dout, cnt, v.errp(), v.stream), "radix launch");
      d2h((uint8_t*)out + off * cb, dout, cnt * cb, v);
    });
    return HG_OK;
  });
}

int hg_encrypt_encoded(hg_ctx* ctx, int key_id, int codec, int64_t scale, int padding_bits, const void* values,
                       const void* values2, const uint32_t* r, uint32_t* ct_out, size_t count) {
  return guarded(__func__, [&] {
    if (!values || !r || !ct_out) fail(HG_ERR_INVALID, "null argument");
    if ((codec == HG_CODEC_BATCH_I64 || codec == HG_CODEC_BATCH_F64) && !values2)
      fail(HG_ERR_INVALID, "batch encodings take two value arrays");
    HG_HOST_PROLOGUE
    make_codec(*k, codec, scale, padding_bits, nullptr, nullptr);  // validates before any work
    const size_t rb = (size_t)k->kc.rlimbs * 4;
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* dm = v.io[0].ensure<int64_t>(cnt * 8);
      auto* dr = v.io[1].ensure<uint32_t>(cnt * rb);
      auto* dout = v.io[2].ensure<uint32_t>(cnt * cb);
      int64_t* dm2 = nullptr;
      h2d(dm, static_cast<const uint8_t*>(values) + off * 8, cnt * 8, v);
      if (values2) {
        dm2 = v.io[3].ensure<int64_t>(cnt * 8);
        h2d(dm2, static_cast<const uint8_t*>(values2) + off * 8, cnt * 8, v);
      }
      h2d(dr, (const uint8_t*)r + off * rb, cnt * rb, v);
      core_encrypt_encoded(*k, v, dm, dr, dout, cnt, make_codec(*k, codec, scale, padding_bits, dm2, nullptr));
      d2h((uint8_t*)ct_out + off * cb, dout, cnt * cb, v);
    });
    return HG_OK;
  });
}

int hg_decrypt_decoded(hg_ctx* ctx, int key_id, int codec, int64_t scale, int padding_bits, const uint32_t* ct,
                       void* out, void* out2, uint8_t* overflow, size_t count) {
  return guarded(__func__, [&] {
    if (!ct || !out) fail(HG_ERR_INVALID, "null argument");
    const bool batch = codec == HG_CODEC_BATCH_I64 || codec == HG_CODEC_BATCH_F64;
    if (batch && !out2) fail(HG_ERR_INVALID, "batch decodings fill two output arrays");
    HG_HOST_PROLOGUE
    make_codec(*k, codec, scale, padding_bits, nullptr, nullptr);
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* dc = v.io[0].ensure<uint32_t>(cnt * cb);
      auto* dm = v.io[1].ensure<int64_t>(cnt * 8);
      auto* dov = v.io[2].ensure<uint8_t>(cnt);
      int64_t* dm2 = batch ? v.io[3].ensure<int64_t>(cnt * 8) : nullptr;
      h2d(dc, (const uint8_t*)ct + off * cb, cnt * cb, v);
      core_decrypt_decoded(*k, v, dc, dm, dov, cnt, make_codec(*k, codec, scale, padding_bits, nullptr, dm2));
      d2h(static_cast<uint8_t*>(out) + off * 8, dm, cnt * 8, v);
      if (batch) d2h(static_cast<uint8_t*>(out2) + off * 8, dm2, cnt * 8, v);
      if (overflow) d2h(overflow + off, dov, cnt, v);
    });
    return HG_OK;
  });
}

int hg_encrypt_bn(hg_ctx* ctx, int key_id, const uint32_t* m_mag, const uint8_t* m_neg, const uint32_t* r,
                  uint32_t* ct_out, size_t count) {
  return guarded(__func__, [&] {
    if (!m_mag || !m_neg || !r || !ct_out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    const size_t rb = (size_t)k->kc.rlimbs * 4, pb = (size_t)(k->scheme == 1 ? k->pt_limbs : k->S / 2) * 4;
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* dmag = v.io[0].ensure<uint32_t>(cnt * pb);
      auto* dneg = v.io[3].ensure<uint8_t>(cnt);
      auto* dr = v.io[1].ensure<uint32_t>(cnt * rb);
      auto* dout = v.io[2].ensure<uint32_t>(cnt * cb);
      h2d(dmag, (const uint8_t*)m_mag + off * pb, cnt * pb, v);
      h2d(dneg, m_neg + off, cnt, v);
      h2d(dr, (const uint8_t*)r + off * rb, cnt * rb, v);
      core_encrypt(*k, v, hg::EncMode::kEncrypt, nullptr, dmag, dneg, dr, nullptr, dout, cnt);
      d2h((uint8_t*)ct_out + off * cb, dout, cnt * cb, v);
    });
    return HG_OK;
  });
}

int hg_encrypt_zero(hg_ctx* ctx, int key_id, const uint32_t* r, uint32_t* ct_out, size_t count) {
  return guarded(__func__, [&] {
    if (!r || !ct_out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    const size_t rb = (size_t)k->kc.rlimbs * 4;
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* dr = v.io[1].ensure<uint32_t>(cnt * rb);
      auto* dout = v.io[2].ensure<uint32_t>(cnt * cb);
      h2d(dr, (const uint8_t*)r + off * rb, cnt * rb, v);
      core_encrypt(*k, v, hg::EncMode::kZero, nullptr, nullptr, nullptr, dr, nullptr, dout, cnt);
      d2h((uint8_t*)ct_out + off * cb, dout, cnt * cb, v);
    });
    return HG_OK;
  });
}

int hg_randomize(hg_ctx* ctx, int key_id, uint32_t* ct, const uint32_t* r, size_t count) {
  return guarded(__func__, [&] {
    if (!r || !ct) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    const size_t rb = (size_t)k->kc.rlimbs * 4;
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* dr = v.io[1].ensure<uint32_t>(cnt * rb);
      auto* dc = v.io[2].ensure<uint32_t>(cnt * cb);
      h2d(dr, (const uint8_t*)r + off * rb, cnt * rb, v);
      h2d(dc, (const uint8_t*)ct + off * cb, cnt * cb, v);
      core_encrypt(*k, v, hg::EncMode::kRandomize, nullptr, nullptr, nullptr, dr, dc, dc, cnt);
      d2h((uint8_t*)ct + off * cb, dc, cnt * cb, v);
    });
    return HG_OK;
  });
}

int hg_decrypt(hg_ctx* ctx, int key_id, const uint32_t* ct, int64_t* m_out, uint8_t* overflow, size_t count) {
  return guarded(__func__, [&] {
    if (!ct || !m_out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* dc = v.io[0].ensure<uint32_t>(cnt * cb);
      auto* dm = v.io[1].ensure<int64_t>(cnt * 8);
      auto* dov = v.io[2].ensure<uint8_t>(cnt);
      h2d(dc, (const uint8_t*)ct + off * cb, cnt * cb, v);
      core_decrypt(*k, v, dc, dm, dov, nullptr, nullptr, cnt);
      d2h(m_out + off, dm, cnt * 8, v);
      if (overflow) d2h(overflow + off, dov, cnt, v);
    });
    return HG_OK;
  });
}

int hg_decrypt_bn(hg_ctx* ctx, int key_id, const uint32_t* ct, uint32_t* m_mag, uint8_t* m_neg, size_t count) {
  return guarded(__func__, [&] {
    if (!ct || !m_mag || !m_neg) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    const size_t pb = (size_t)(k->scheme == 1 ? k->pt_limbs : k->S / 2) * 4;
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* dc = v.io[0].ensure<uint32_t>(cnt * cb);
      auto* dmag = v.io[1].ensure<uint32_t>(cnt * pb);
      auto* dneg = v.io[2].ensure<uint8_t>(cnt);
      h2d(dc, (const uint8_t*)ct + off * cb, cnt * cb, v);
      core_decrypt(*k, v, dc, nullptr, nullptr, dmag, dneg, cnt);
      d2h((uint8_t*)m_mag + off * pb, dmag, cnt * pb, v);
      d2h(m_neg + off, dneg, cnt, v);
    });
    return HG_OK;
  });
}

// The device address of page-locked host memory (cudaHostAlloc /
// cudaHostRegister, mapped into the device's address space), else nullptr.
void* mapped_host_ptr(const void* p) {
  cudaPointerAttributes pa{};
  if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return pa.type == cudaMemoryTypeHost ? pa.devicePointer : nullptr;
}

int hg_add(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t count) {
  return guarded(__func__, [&] {
    if (!a || !b || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    // Add is one multiplication per ciphertext, so copies would dominate it:
    // when all three buffers are page-locked host memory the kernel reads and
    // writes them in place over the host link instead.
    const auto* ma = static_cast<const uint32_t*>(mapped_host_ptr(a));
    const auto* mb = static_cast<const uint32_t*>(mapped_host_ptr(b));
    auto* mo = static_cast<uint32_t*>(mapped_host_ptr(out));
    if (ma && mb && mo) {
      cuda_check(hg::launch_add(k->S, k->kc, ma, mb, mo, count, w.errp(), w.stream), "add launch");
      finish(w);
      return HG_OK;
    }
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* da = v.io[0].ensure<uint32_t>(cnt * cb);
      auto* db = v.io[1].ensure<uint32_t>(cnt * cb);
      h2d(da, (const uint8_t*)a + off * cb, cnt * cb, v);
      h2d(db, (const uint8_t*)b + off * cb, cnt * cb, v);
      cuda_check(hg::launch_add(k->S, k->kc, da, db, da, cnt, v.errp(), v.stream), "add launch");
      d2h((uint8_t*)out + off * cb, da, cnt * cb, v);
    });
    return HG_OK;
  });
}

static int add_plain_impl(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, int neg, uint32_t* out,
                          size_t count) {
  return guarded(__func__, [&] {
    if (!a || !p || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* da = v.io[0].ensure<uint32_t>(cnt * cb);
      auto* dp = v.io[1].ensure<int64_t>(cnt * 8);
      h2d(da, (const uint8_t*)a + off * cb, cnt * cb, v);
      h2d(dp, p + off, cnt * 8, v);
      core_add_plain(*k, v, da, dp, neg, da, cnt);
      d2h((uint8_t*)out + off * cb, da, cnt * cb, v);
    });
    return HG_OK;
  });
}

int hg_add_plain(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, uint32_t* out, size_t count) {
  return add_plain_impl(ctx, key_id, a, p, 0, out, count);
}

int hg_sub_plain(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, uint32_t* out, size_t count) {
  return add_plain_impl(ctx, key_id, a, p, 1, out, count);
}

int hg_negate(hg_ctx* ctx, int key_id, const uint32_t* a, uint32_t* out, size_t count) {
  return guarded(__func__, [&] {
    if (!a || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    auto* da = w.io[0].ensure<uint32_t>(count * cb);
    h2d(da, a, count * cb, w);
    core_inverse(*k, w, da, nullptr, da, count);
    d2h(out, da, count * cb, w);
    finish(w);
    return HG_OK;
  });
}

int hg_sub(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t count) {
  return guarded(__func__, [&] {
    if (!a || !b || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    auto* da = w.io[0].ensure<uint32_t>(count * cb);
    auto* db = w.io[1].ensure<uint32_t>(count * cb);
    h2d(da, a, count * cb, w);
    h2d(db, b, count * cb, w);
    // evaluator.cc:66-68: Add(a, Negate(b))
    core_inverse(*k, w, db, nullptr, db, count);
    cuda_check(hg::launch_add(k->S, k->kc, da, db, da, count, w.errp(), w.stream), "add launch");
    d2h(out, da, count * cb, w);
    finish(w);
    return HG_OK;
  });
}

int hg_plain_sub(hg_ctx* ctx, int key_id, const int64_t* p, const uint32_t* a, uint32_t* out, size_t count) {
  return guarded(__func__, [&] {
    if (!a || !p || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    auto* da = w.io[0].ensure<uint32_t>(count * cb);
    auto* dp = w.io[1].ensure<int64_t>(count * 8);
    h2d(da, a, count * cb, w);
    h2d(dp, p, count * 8, w);
    // evaluator.cc:82-84: Add(Negate(a), p)
    core_inverse(*k, w, da, nullptr, da, count);
    core_add_plain(*k, w, da, dp, 0, da, count);
    d2h(out, da, count * cb, w);
    finish(w);
    return HG_OK;
  });
}

int hg_mul(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* kk, uint32_t* out, size_t count) {
  return guarded(__func__, [&] {
    if (!a || !kk || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* da = v.io[0].ensure<uint32_t>(cnt * cb);
      auto* dk = v.io[1].ensure<int64_t>(cnt * 8);
      auto* dout = v.io[2].ensure<uint32_t>(cnt * cb);
      h2d(da, (const uint8_t*)a + off * cb, cnt * cb, v);
      h2d(dk, kk + off, cnt * 8, v);
      core_mul(*k, v, da, dk, kk + off, dout, cnt, false);
      d2h((uint8_t*)out + off * cb, dout, cnt * cb, v);
    }, [](Work& v) { v.task.status = 0; }, [](Work& v) { raise_task_status(v.task); });
    return HG_OK;
  });
}

int hg_mul_bn(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* k_mag, const uint8_t* k_neg,
              size_t k_limbs, uint32_t* out, size_t count) {
  return guarded(__func__, [&] {
    if (!a || !k_mag || !k_neg || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    if (k_limbs < 1 || k_limbs > (size_t)k->S) fail(HG_ERR_INVALID, "scalar limbs must be in [1, S] (at most the width of n^2)");
    size_t max_bits = 0;
    bool any_neg = false;
    for (size_t i = 0; i < count; ++i) {
      const uint32_t* e = k_mag + i * k_limbs;
      size_t l = k_limbs;
      while (l > 0 && e[l - 1] == 0u) --l;
      if (l == 0) continue;
      size_t b = 32 * (l - 1);
      for (uint32_t t = e[l - 1]; t; t >>= 1) ++b;
      max_bits = std::max(max_bits, b);
      any_neg |= k_neg[i] != 0;
    }
    run_chunked(ctx, w, count, [&](Work& v, size_t off, size_t cnt) {
      auto* da = v.io[0].ensure<uint32_t>(cnt * cb);
      auto* dk = v.io[1].ensure<uint32_t>(cnt * k_limbs * 4);
      auto* dout = v.io[2].ensure<uint32_t>(cnt * cb);
      auto* dn = v.io[3].ensure<uint8_t>(cnt);
      h2d(da, (const uint8_t*)a + off * cb, cnt * cb, v);
      h2d(dk, k_mag + off * k_limbs, cnt * k_limbs * 4, v);
      h2d(dn, k_neg + off, cnt, v);
      core_mul_bn(*k, v, da, dk, (int)k_limbs, dn, max_bits, any_neg, dout, cnt, false);
      d2h((uint8_t*)out + off * cb, dout, cnt * cb, v);
    }, [](Work& v) { v.task.status = 0; }, [](Work& v) { raise_task_status(v.task); });
    return HG_OK;
  });
}

// ---------------------------------------------------------------------------
// HEU wire format for ciphertext matrices (numpy/matrix.h:221-310); the items
// are packed and unpacked by the kernels in wire_kernels.cu, the msgpack
// headers around them are written and walked here.
// ---------------------------------------------------------------------------
static Work& dev_work(hg_ctx* ctx, void* stream);

namespace {

using hg::wire::WireReader;
using hg::wire::WireShape;
using hg::wire::wire_header;
using hg::wire::wire_items;
using hg::wire::wire_prefix;

// SchemaType values (phe/base/schema.h:47-51) appended to every item.
uint64_t schema_value(const KeyRec& k) { return k.scheme == 1 ? 1u : 4u; }

void wire_pack(KeyRec& k, Work& w, const uint32_t* dct, size_t rows, size_t cols, int row_major,
               const std::vector<uint8_t>& prefix, uint8_t* host_out, uint8_t* dev_out, size_t cap, size_t* len) {
  const size_t count = rows * cols;
  auto* mag = w.io[1].ensure<uint32_t>(std::max<size_t>(count, 1) * 4);
  auto* scr = w.io[2].ensure<uint64_t>(hg::wire_scratch_words(count) * 8);
  auto* tot = w.io[3].ensure<uint64_t>(8);
  cuda_check(hg::launch_wire_size(dct, rows, cols, row_major, k.S, mag, scr, tot, w.stream), "wire size");
  uint64_t* htot = w.pin_err.ensure<uint64_t>(8);
  cuda_check(cudaMemcpyAsync(htot, tot, 8, cudaMemcpyDeviceToHost, w.stream), "D2H total");
  cuda_check(cudaStreamSynchronize(w.stream), "stream sync");
  const size_t need = prefix.size() + (size_t)*htot;
  *len = need;
  if (need > cap) fail(HG_ERR_INVALID, "output buffer too small: " + std::to_string(need) + " bytes needed");
  if (dev_out) {
    cuda_check(cudaMemcpyAsync(dev_out, prefix.data(), prefix.size(), cudaMemcpyHostToDevice, w.stream), "H2D prefix");
    cuda_check(hg::launch_wire_write(dct, rows, cols, row_major, k.S, schema_value(k), mag, scr, dev_out, prefix.size(),
                                     w.stream),
               "wire write");
  } else {
    std::memcpy(host_out, prefix.data(), prefix.size());
    auto* dbytes = w.io[4].ensure<uint8_t>(std::max<size_t>((size_t)*htot, 1));
    cuda_check(hg::launch_wire_write(dct, rows, cols, row_major, k.S, schema_value(k), mag, scr, dbytes, 0, w.stream),
               "wire write");
    d2h(host_out + prefix.size(), dbytes, (size_t)*htot, w);
  }
}

// Host bytes -> S limbs per item at dout (device).  The buffer's copy to the
// device is queued first, so the host walk over the item headers runs while
// it transfers; offsets and lengths go through pinned memory.  Synchronises
// the stream (also when the walk fails: the copy reads the caller's buffer).
WireShape wire_load(KeyRec& k, Work& w, const uint8_t* buf, size_t len, int row_major, uint32_t** dout_io,
                    uint32_t* dout_given, size_t cap_count) {
  WireReader r{buf, len};
  const WireShape sh = wire_header(r);
  if (sh.n > cap_count) {
    WireShape out = sh;
    out.n = (size_t)-1;  // tells the caller that the output is too small
    return out;
  }
  if (sh.n == 0) return sh;
  auto* dbuf = w.io[1].ensure<uint8_t>(len);
  h2d(dbuf, buf, len, w);
  auto* pin = w.pin_wire.ensure<uint64_t>(sh.n * 16);
  try {
    wire_items(r, sh.n, pin, pin + sh.n, (uint8_t)schema_value(k));
  } catch (...) {
    cudaStreamSynchronize(w.stream);
    throw;
  }
  auto* dmeta = w.io[2].ensure<uint64_t>(sh.n * 16);
  h2d(dmeta, pin, sh.n * 16, w);
  uint32_t* dout = dout_given ? dout_given : (*dout_io = w.io[0].ensure<uint32_t>(sh.n * ct_bytes(k)));
  cuda_check(hg::launch_wire_unpack(dbuf, dmeta, dmeta + sh.n, sh.rows, sh.cols, row_major, k.S, schema_value(k), dout,
                                     w.errp(), w.stream),
             "wire read");
  cuda_check(cudaStreamSynchronize(w.stream), "stream sync");
  return sh;
}

}  // namespace

int hg_serialize_bound(hg_ctx* ctx, int key_id, size_t count, size_t* bytes) {
  return guarded(__func__, [&] {
    if (!bytes) fail(HG_ERR_INVALID, "null argument");
    KeyRec* k = get_key(ctx, key_id);
    // header <= 1 + 3 * 9 + 5; item <= str32 + fixarray + bin32 + 4S + 8
    *bytes = 33 + count * (5 + 1 + 5 + (size_t)k->S * 4 + 8);
    return HG_OK;
  });
}

int hg_serialize(hg_ctx* ctx, int key_id, const uint32_t* ct, size_t rows, size_t cols, int ndim, int row_major,
                 uint8_t* out, size_t cap, size_t* len) {
  return guarded(__func__, [&] {
    if (!out || !len || (!ct && rows * cols)) fail(HG_ERR_INVALID, "null argument");
    if (ndim < 0 || ndim > 2) fail(HG_ERR_INVALID, "ndim must be 0, 1 or 2");
    if (cols && rows > SIZE_MAX / cols) fail(HG_ERR_INVALID, "rows * cols overflows");
    KeyRec* k = get_key(ctx, key_id);
    set_device(ctx);
    LaneGuard lane(ctx);
    Work& w = *lane.w;
    reset_err(w);
    const size_t count = rows * cols, cb = ct_bytes(*k);
    auto* dct = w.io[0].ensure<uint32_t>(std::max<size_t>(count, 1) * cb);
    h2d(dct, ct, count * cb, w);
    wire_pack(*k, w, dct, rows, cols, row_major, wire_prefix(rows, cols, ndim), out, nullptr, cap, len);
    finish(w);
    return HG_OK;
  });
}

int hg_dev_serialize(hg_ctx* ctx, int key_id, const uint32_t* ct, size_t rows, size_t cols, int ndim, int row_major,
                     uint8_t* out, size_t cap, size_t* len, void* stream) {
  return guarded(__func__, [&] {
    if (!out || !len || (!ct && rows * cols)) fail(HG_ERR_INVALID, "null argument");
    if (ndim < 0 || ndim > 2) fail(HG_ERR_INVALID, "ndim must be 0, 1 or 2");
    if (cols && rows > SIZE_MAX / cols) fail(HG_ERR_INVALID, "rows * cols overflows");
    KeyRec* k = get_key(ctx, key_id);
    set_device(ctx);
    Work& w = dev_work(ctx, stream);
    wire_pack(*k, w, ct, rows, cols, row_major, wire_prefix(rows, cols, ndim), nullptr, out, cap, len);
    cuda_check(cudaStreamSynchronize(w.stream), "stream sync");
    return HG_OK;
  });
}

int hg_deserialize(hg_ctx* ctx, int key_id, const uint8_t* buf, size_t len, int row_major, uint32_t* ct_out,
                   size_t cap_count, size_t* rows, size_t* cols, int* ndim) {
  return guarded(__func__, [&] {
    if (!buf || !rows || !cols || !ndim) fail(HG_ERR_INVALID, "null argument");
    KeyRec* k = get_key(ctx, key_id);
    set_device(ctx);
    LaneGuard lane(ctx);
    Work& w = *lane.w;
    reset_err(w);
    uint32_t* dout = nullptr;
    const WireShape sh = wire_load(*k, w, buf, len, row_major, &dout, nullptr, ct_out ? cap_count : 0);
    *rows = sh.rows;
    *cols = sh.cols;
    *ndim = sh.ndim;
    if (sh.n == (size_t)-1)
      fail(HG_ERR_INVALID, "output holds " + std::to_string(ct_out ? cap_count : 0) + " ciphertexts, " +
                               std::to_string(sh.rows * sh.cols) + " serialized");
    if (sh.n) d2h(ct_out, dout, sh.n * ct_bytes(*k), w);
    finish(w);
    return HG_OK;
  });
}

int hg_dev_deserialize(hg_ctx* ctx, int key_id, const uint8_t* buf, size_t len, int row_major, uint32_t* ct_out,
                       size_t cap_count, size_t* rows, size_t* cols, int* ndim, void* stream) {
  return guarded(__func__, [&] {
    if (!buf || !rows || !cols || !ndim) fail(HG_ERR_INVALID, "null argument");
    KeyRec* k = get_key(ctx, key_id);
    set_device(ctx);
    Work& w = dev_work(ctx, stream);
    const WireShape sh = wire_load(*k, w, buf, len, row_major, nullptr, ct_out, ct_out ? cap_count : 0);
    *rows = sh.rows;
    *cols = sh.cols;
    *ndim = sh.ndim;
    if (sh.n == (size_t)-1)
      fail(HG_ERR_INVALID, "output holds " + std::to_string(ct_out ? cap_count : 0) + " ciphertexts, " +
                               std::to_string(sh.rows * sh.cols) + " serialized");
    return HG_OK;
  });
}

int hg_sum(hg_ctx* ctx, int key_id, const uint32_t* a, size_t count, uint32_t* out) {
  return guarded(__func__, [&] {
    if (!a || !out) fail(HG_ERR_INVALID, "null argument");
    if (count == 0) fail(HG_ERR_INVALID, "you cannot sum an empty tensor");
    HG_HOST_PROLOGUE
    auto* da = w.io[0].ensure<uint32_t>(count * cb);
    auto* dout = w.io[1].ensure<uint32_t>(cb);
    h2d(da, a, count * cb, w);
    core_sum(*k, w, da, count, dout);
    d2h(out, dout, cb, w);
    finish(w);
    return HG_OK;
  });
}

static int convert_impl(hg_ctx* ctx, int key_id, const uint32_t* in, uint32_t* out, size_t count, int to_mont) {
  return guarded(__func__, [&] {
    if (!in || !out) fail(HG_ERR_INVALID, "null argument");
    HG_HOST_PROLOGUE
    auto* da = w.io[0].ensure<uint32_t>(count * cb);
    h2d(da, in, count * cb, w);
    cuda_check(hg::launch_convert(k->S, k->kc, da, da, count, to_mont, w.errp(), w.stream), "convert launch");
    d2h(out, da, count * cb, w);
    finish(w);
    return HG_OK;
  });
}

int hg_to_mont(hg_ctx* ctx, int key_id, const uint32_t* z, uint32_t* mont, size_t count) {
  return convert_impl(ctx, key_id, z, mont, count, 1);
}

int hg_from_mont(hg_ctx* ctx, int key_id, const uint32_t* mont, uint32_t* z, size_t count) {
  return convert_impl(ctx, key_id, mont, z, count, 0);
}

// ---- device-pointer API -----------------------------------------------------
static Work& dev_work(hg_ctx* ctx, void* stream) {
  std::lock_guard<std::mutex> lk(ctx->dev_mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->lanes[0]->stream;
  auto& slot = ctx->dev_work[st];
  if (!slot) {
    slot = std::make_unique<Work>();
    slot->stream = st;
    slot->own_stream = false;
    cuda_check(cudaMemsetAsync(slot->errp(), 0, sizeof(uint32_t), st), "memset err");
  }
  return *slot;
}

#define HG_DEV_PROLOGUE                   \
  KeyRec* k = get_key(ctx, key_id);       \
  if (count == 0) return HG_OK;           \
  set_device(ctx);                        \
  Work& w = dev_work(ctx, stream);

int hg_dev_encrypt(hg_ctx* ctx, int key_id, const int64_t* m, const uint32_t* r, uint32_t* ct_out, size_t count,
                   void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    core_encrypt(*k, w, hg::EncMode::kEncrypt, m, nullptr, nullptr, r, nullptr, ct_out, count);
    return HG_OK;
  });
}

int hg_dev_decrypt(hg_ctx* ctx, int key_id, const uint32_t* ct, int64_t* m_out, uint8_t* overflow, size_t count,
                   void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    core_decrypt(*k, w, ct, m_out, overflow, nullptr, nullptr, count);
    return HG_OK;
  });
}

int hg_dev_encrypt_encoded(hg_ctx* ctx, int key_id, int codec, int64_t scale, int padding_bits, const void* values,
                           const void* values2, const uint32_t* r, uint32_t* ct_out, size_t count, void* stream) {
  return guarded(__func__, [&] {
    if ((codec == HG_CODEC_BATCH_I64 || codec == HG_CODEC_BATCH_F64) && !values2)
      fail(HG_ERR_INVALID, "batch encodings take two value arrays");
    HG_DEV_PROLOGUE
    core_encrypt_encoded(*k, w, values, r, ct_out, count, make_codec(*k, codec, scale, padding_bits, values2, nullptr));
    return HG_OK;
  });
}

int hg_dev_decrypt_decoded(hg_ctx* ctx, int key_id, int codec, int64_t scale, int padding_bits, const uint32_t* ct,
                           void* out, void* out2, uint8_t* overflow, size_t count, void* stream) {
  return guarded(__func__, [&] {
    if ((codec == HG_CODEC_BATCH_I64 || codec == HG_CODEC_BATCH_F64) && !out2)
      fail(HG_ERR_INVALID, "batch decodings fill two output arrays");
    HG_DEV_PROLOGUE
    core_decrypt_decoded(*k, w, ct, out, overflow, count, make_codec(*k, codec, scale, padding_bits, nullptr, out2));
    return HG_OK;
  });
}

int hg_dev_add(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t count,
               void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    cuda_check(hg::launch_add(k->S, k->kc, a, b, out, count, w.errp(), w.stream), "add launch");
    return HG_OK;
  });
}

int hg_dev_mul(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* kk, uint32_t* out, size_t count,
               void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    core_mul(*k, w, a, kk, nullptr, out, count);
    return HG_OK;
  });
}

int hg_dev_mul_bn(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* k_mag, const uint8_t* k_neg,
                  size_t k_limbs, uint32_t* out, size_t count, void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    // the magnitudes stay on the device: the window follows their width and
    // the inverse runs with the signs as its selector
    core_mul_bn(*k, w, a, k_mag, (int)k_limbs, k_neg, 32 * k_limbs, true, out, count);
    return HG_OK;
  });
}

int hg_dev_encrypt_zero(hg_ctx* ctx, int key_id, const uint32_t* r, uint32_t* ct_out, size_t count, void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    core_encrypt(*k, w, hg::EncMode::kZero, nullptr, nullptr, nullptr, r, nullptr, ct_out, count);
    return HG_OK;
  });
}

int hg_dev_randomize(hg_ctx* ctx, int key_id, uint32_t* ct, const uint32_t* r, size_t count, void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    core_encrypt(*k, w, hg::EncMode::kRandomize, nullptr, nullptr, nullptr, r, ct, ct, count);
    return HG_OK;
  });
}

int hg_dev_add_plain(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, uint32_t* out, size_t count,
                     void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    core_add_plain(*k, w, a, p, 0, out, count);
    return HG_OK;
  });
}

int hg_dev_sub_plain(hg_ctx* ctx, int key_id, const uint32_t* a, const int64_t* p, uint32_t* out, size_t count,
                     void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    core_add_plain(*k, w, a, p, 1, out, count);
    return HG_OK;
  });
}

// out = a^-1: copy a into out (unless aliased), then invert in place
static void dev_negate_into(KeyRec& k, Work& w, const uint32_t* a, uint32_t* out, size_t count) {
  if (a != out)
    cuda_check(cudaMemcpyAsync(out, a, count * ct_bytes(k), cudaMemcpyDeviceToDevice, w.stream), "copy");
  core_inverse(k, w, out, nullptr, out, count);
}

int hg_dev_negate(hg_ctx* ctx, int key_id, const uint32_t* a, uint32_t* out, size_t count, void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    dev_negate_into(*k, w, a, out, count);
    return HG_OK;
  });
}

int hg_dev_plain_sub(hg_ctx* ctx, int key_id, const int64_t* p, const uint32_t* a, uint32_t* out, size_t count,
                     void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    // evaluator.cc:82-84: Add(Negate(a), p)
    dev_negate_into(*k, w, a, out, count);
    core_add_plain(*k, w, out, p, 0, out, count);
    return HG_OK;
  });
}

int hg_dev_sub(hg_ctx* ctx, int key_id, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t count,
               void* stream) {
  return guarded(__func__, [&] {
    HG_DEV_PROLOGUE
    // evaluator.cc:66-68: Add(a, Negate(b)); with out == a the inverse goes
    // through the context's staging buffer so a is not overwritten first
    uint32_t* nb = out;
    if (out == a) nb = w.io[5].ensure<uint32_t>(count * ct_bytes(*k));
    dev_negate_into(*k, w, b, nb, count);
    cuda_check(hg::launch_add(k->S, k->kc, a, nb, out, count, w.errp(), w.stream), "add launch");
    return HG_OK;
  });
}

int hg_dev_sum(hg_ctx* ctx, int key_id, const uint32_t* a, size_t count, uint32_t* out, void* stream) {
  return guarded(__func__, [&] {
    if (count == 0) fail(HG_ERR_INVALID, "you cannot sum an empty tensor");
    HG_DEV_PROLOGUE
    core_sum(*k, w, a, count, out);
    return HG_OK;
  });
}


int hg_bucket_sum(hg_ctx* ctx, int key_id, const uint32_t* x, size_t rows, size_t cols, const uint8_t* order_map,
                  size_t features, int bucket_num, int cumsum, uint32_t* out) {
  return guarded(__func__, [&] {
    if (!x || !order_map || !out) fail(HG_ERR_INVALID, "null argument");
    const size_t count = rows * cols;
    if (count == 0) fail(HG_ERR_INVALID, "you cannot sum an empty tensor");
    HG_HOST_PROLOGUE
    auto* dx = w.io[0].ensure<uint32_t>(count * cb);
    auto* dom = w.io[1].ensure<uint8_t>(rows * features);
    const size_t outn = features * (size_t)bucket_num * cols;
    auto* dout = w.io[2].ensure<uint32_t>(outn * cb);
    h2d(dx, x, count * cb, w);
    h2d(dom, order_map, rows * features, w);
    core_bucket_sum(*k, w, dx, rows, cols, dom, (int)features, bucket_num, cumsum, dout);
    d2h(out, dout, outn * cb, w);
    finish(w);
    return HG_OK;
  });
}

int hg_dev_bucket_sum(hg_ctx* ctx, int key_id, const uint32_t* x, size_t rows, size_t cols, const uint8_t* order_map,
                      size_t features, int bucket_num, int cumsum, uint32_t* out, void* stream) {
  return guarded(__func__, [&] {
    const size_t count = rows * cols;
    if (count == 0) fail(HG_ERR_INVALID, "you cannot sum an empty tensor");
    HG_DEV_PROLOGUE
    core_bucket_sum(*k, w, x, rows, cols, order_map, (int)features, bucket_num, cumsum, out);
    return HG_OK;
  });
}

int hg_matmul(hg_ctx* ctx, int key_id, const uint32_t* x, size_t M, size_t K, const int64_t* y, size_t N,
              uint32_t* out) {
  return guarded(__func__, [&] {
    if (!x || !y || !out) fail(HG_ERR_INVALID, "null argument");
    const size_t count = M * K;
    if (count == 0 || N == 0) fail(HG_ERR_INVALID, "HEU does not support empty tensor currently");
    HG_HOST_PROLOGUE
    auto* dx = w.io[0].ensure<uint32_t>(count * cb);
    auto* dout = w.io[1].ensure<uint32_t>(M * N * cb);
    h2d(dx, x, count * cb, w);
    core_matmul(*k, w, dx, M, K, y, N, dout);
    d2h(out, dout, M * N * cb, w);
    finish(w);
    return HG_OK;
  });
}

int hg_dev_matmul(hg_ctx* ctx, int key_id, const uint32_t* x, size_t M, size_t K, const int64_t* y, size_t N,
                  uint32_t* out, void* stream) {
  return guarded(__func__, [&] {
    if (!y) fail(HG_ERR_INVALID, "null argument");
    const size_t count = M * K;
    if (count == 0 || N == 0) fail(HG_ERR_INVALID, "HEU does not support empty tensor currently");
    HG_DEV_PROLOGUE
    core_matmul(*k, w, x, M, K, y, N, out);
    return HG_OK;
  });
}

int hg_matmul_bn(hg_ctx* ctx, int key_id, const uint32_t* x, size_t M, size_t K, const uint32_t* y_mag,
                 const uint8_t* y_neg, size_t y_limbs, size_t N, uint32_t* out) {
  return guarded(__func__, [&] {
    if (!x || !y_mag || !y_neg || !out) fail(HG_ERR_INVALID, "null argument");
    const size_t count = M * K;
    if (count == 0 || N == 0) fail(HG_ERR_INVALID, "HEU does not support empty tensor currently");
    HG_HOST_PROLOGUE
    auto* dx = w.io[0].ensure<uint32_t>(count * cb);
    auto* dout = w.io[1].ensure<uint32_t>(M * N * cb);
    h2d(dx, x, count * cb, w);
    core_matmul_bn(*k, w, dx, M, K, y_mag, y_neg, y_limbs, N, dout);
    d2h(out, dout, M * N * cb, w);
    finish(w);
    return HG_OK;
  });
}

int hg_dev_matmul_bn(hg_ctx* ctx, int key_id, const uint32_t* x, size_t M, size_t K, const uint32_t* y_mag,
                     const uint8_t* y_neg, size_t y_limbs, size_t N, uint32_t* out, void* stream) {
  return guarded(__func__, [&] {
    if (!y_mag || !y_neg) fail(HG_ERR_INVALID, "null argument");
    const size_t count = M * K;
    if (count == 0 || N == 0) fail(HG_ERR_INVALID, "HEU does not support empty tensor currently");
    HG_DEV_PROLOGUE
    core_matmul_bn(*k, w, x, M, K, y_mag, y_neg, y_limbs, N, out);
    return HG_OK;
  });
}

}  // extern "C"

namespace {

// ---- key configuration and autotuning ---------------------------------------
static void apply_config(KeyRec& k, const hg_key_config& c) {
  if (c.variant < 0 || c.variant > 1 || c.dec_variant < 0 || c.dec_variant > 1)
    fail(HG_ERR_INVALID, "variant must be 0 or 1");
  if (c.mul_window < 2 || c.mul_window > 6) fail(HG_ERR_INVALID, "mul_window must be in [2, 6]");
  if (c.dec_window < 2 || c.dec_window > 7) fail(HG_ERR_INVALID, "dec_window must be in [2, 7]");
  cuda_check(cudaDeviceSynchronize(), "sync");
  k.kc.variant = c.variant;
  k.grid_mul = hg::resident_blocks_mul(k.S, c.variant);
  k.wm = c.mul_window;
  if (k.secret) {
    if (c.dec_window != k.sc.wd) {
      std::vector<uint16_t> pp, pq;
      int st0 = 0, st1 = 0;
      build_prog(k.p - BN(1), c.dec_window, &st0, &pp);
      build_prog(k.q - BN(1), c.dec_window, &st1, &pq);
      const size_t len = std::max(pp.size(), pq.size());
      pp.resize(len, hg::kOpNop);
      pq.resize(len, hg::kOpNop);
      uint16_t* dp = k.progs.ensure<uint16_t>(std::max<size_t>(2 * len, 2) * 2);
      if (len) {
        cuda_check(cudaMemcpy(dp, pp.data(), len * 2, cudaMemcpyHostToDevice), "upload prog");
        cuda_check(cudaMemcpy(dp + len, pq.data(), len * 2, cudaMemcpyHostToDevice), "upload prog");
      }
      k.sc.prog[0] = dp;
      k.sc.prog[1] = dp + len;
      k.sc.prog_len = (int)len;
      k.sc.start[0] = st0;
      k.sc.start[1] = st1;
      k.sc.wd = c.dec_window;
    }
    k.sc.variant = c.dec_variant;
    k.grid_dec = hg::resident_blocks_decrypt(k.Sp, c.dec_variant);
  }
}

static hg_key_config current_config(const KeyRec& k) {
  hg_key_config c;
  c.variant = k.kc.variant;
  c.dec_variant = k.sc.variant;
  c.mul_window = k.wm;
  c.dec_window = k.secret ? k.sc.wd : 5;
  return c;
}

// ---- persistent multi-key batches ------------------------------------------
}  // namespace

struct hg_batch {
  struct Job {
    int key_id, op, flags;
    size_t count;
    const void* in0;
    const void* in1;
    void* out;
    void* aux;
  };
  hg_ctx* ctx = nullptr;
  std::vector<Job> jobs;
  bool dirty = true;
  int variant = 0;  // variant set of every job, or HG_BATCH_PER_KEY
  // one persistent launch per variant set in use (one unless per key)
  struct Group {
    int V = 0;
    DevBuf djobs, dtiles, dcounter;
    uint32_t ntiles = 0;
    size_t warp_words = 0;
    int grid = 0;
  };
  std::vector<std::unique_ptr<Group>> groups;
  DevBuf derr, dscratch;
  PinBuf pin_err;
  struct Inv {
    KeyRec* key;
    size_t job;
    TreeBufs bufs;
    PinBuf root, z;
    InvTask task;
  };
  std::vector<std::unique_ptr<Inv>> invs;
  std::vector<KeyRec*> keys;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  ~hg_batch() { drop_graph(); }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
};

namespace {

// Relative cost of one ciphertext of an op (Montgomery multiplications x S^2).
double job_cost(const KeyRec& k, int op) {
  const double s2 = (double)k.S * k.S;
  switch (op) {
    case hg::kBatchEncrypt: return (k.kc.npos + 2) * s2;
    case hg::kBatchDecrypt: return 2.0 * (k.key_bits / 2 + k.key_bits / 12) * (s2 / 4);
    case hg::kBatchMul: return 80.0 * s2;
    default: return s2;
  }
}

// One job of a persistent batch, resolved against its key.
struct JobSpec {
  KeyRec* k;
  int op, flags;
  size_t count;
  const void* in0;
  const void* in1;
  void* out;
  void* aux;
};

// Host-side plan of a batch: descriptors, cost-ordered tiles, scratch size.
struct BatchPlan {
  std::vector<hg::BatchJob> jobs;
  std::vector<hg::BatchTile> tiles;
  size_t warp_words = 1;
};

BatchPlan plan_batch(const std::vector<JobSpec>& specs, int V) {
  BatchPlan plan;
  struct T {
    hg::BatchTile t;
    double cost;
  };
  std::vector<T> tiles;
  for (size_t j = 0; j < specs.size(); ++j) {
    const JobSpec& J = specs[j];
    KeyRec* k = J.k;
    if (J.op == hg::kBatchDecrypt && !k->secret) fail(HG_ERR_NO_SECRET, "batch decrypt job on a public key");
    hg::BatchJob d{};
    d.op = J.op;
    d.S = k->S;
    d.wm = k->wm;
    d.kc = k->kc;
    d.sc = k->sc;
    d.in0 = J.in0;
    d.in1 = J.in1;
    d.out = J.out;
    d.aux = J.aux;
    d.count = J.count;
    plan.jobs.push_back(d);
    int per_pass;
    if (J.op == hg::kBatchDecrypt) {
      const int TP = hg::tp_for(k->Sp, V);
      per_pass = 32 / (2 * TP);
      plan.warp_words = std::max(plan.warp_words, (size_t)per_pass * 2 * ((size_t)1 << (k->sc.wd - 1)) * k->Sp);
    } else {
      const int TPI = hg::tpi_for(k->S, V);
      per_pass = 32 / TPI;
      if (J.op == hg::kBatchMul)
        plan.warp_words = std::max(plan.warp_words, (size_t)per_pass * ((size_t)1 << (k->wm - 1)) * k->S);
    }
    // a throughput tile is four passes of a warp (fewer trips to the
    // queue); a latency tile one pass, so a short batch spreads one chain
    // per warp instead of queueing four chains behind each other on a warp
    const size_t tile = (size_t)per_pass * (V == hg::kBatchLatencyVariant ? 1 : 4);
    const double c = job_cost(*k, J.op);
    for (size_t st = 0; st < J.count; st += tile) {
      const size_t cnt = std::min(tile, J.count - st);
      tiles.push_back({{(uint32_t)j, (uint32_t)st, (uint32_t)cnt, 0u}, c * (double)cnt});
    }
  }
  if (tiles.size() >= (1ull << 32)) fail(HG_ERR_INVALID, "batch too large");
  std::stable_sort(tiles.begin(), tiles.end(), [](const T& x, const T& y) { return x.cost > y.cost; });
  plan.tiles.reserve(tiles.size());
  for (auto& t : tiles) plan.tiles.push_back(t.t);
  return plan;
}

size_t padded_pow2(size_t n) {
  size_t p = 1;
  while (p < n) p <<= 1;
  return p;
}

void batch_build(hg_batch& b) {
  const int V = b.variant;
  std::vector<JobSpec> specs;
  b.keys.clear();
  b.invs.clear();
  for (size_t j = 0; j < b.jobs.size(); ++j) {
    const auto& J = b.jobs[j];
    KeyRec* k = get_key(b.ctx, J.key_id);
    specs.push_back({k, J.op, J.flags, J.count, J.in0, J.in1, J.out, J.aux});
    b.keys.push_back(k);
    if (J.op == hg::kBatchMul && !(J.flags & HG_JOB_NONNEG)) {
      auto inv = std::make_unique<hg_batch::Inv>();
      inv->key = k;
      inv->job = j;
      inv->task.root = inv->root.ensure<uint32_t>((size_t)k->S * 4 + 4);
      inv->task.z = inv->z.ensure<uint32_t>((size_t)k->S * 4);
      b.invs.push_back(std::move(inv));
    }
  }
  // the jobs of each variant set: all of them, or per key its tuned layout
  // (the decryption layout for decryptions, the mod n^2 layout otherwise)
  std::map<int, std::vector<JobSpec>> by_v;
  for (const JobSpec& J : specs) {
    const int jv = V >= 0 ? V : (J.op == hg::kBatchDecrypt ? J.k->sc.variant : J.k->kc.variant);
    by_v[jv].push_back(J);
  }
  b.groups.clear();
  size_t scratch_words = 1;
  for (auto& kv : by_v) {
    auto g = std::make_unique<hg_batch::Group>();
    g->V = kv.first;
    const BatchPlan plan = plan_batch(kv.second, g->V);
    auto* jd = g->djobs.ensure<hg::BatchJob>(std::max<size_t>(plan.jobs.size(), 1) * sizeof(hg::BatchJob));
    auto* td = g->dtiles.ensure<hg::BatchTile>(std::max<size_t>(plan.tiles.size(), 1) * sizeof(hg::BatchTile));
    if (!plan.jobs.empty())
      cuda_check(cudaMemcpy(jd, plan.jobs.data(), plan.jobs.size() * sizeof(hg::BatchJob), cudaMemcpyHostToDevice),
                 "jobs");
    if (!plan.tiles.empty())
      cuda_check(
          cudaMemcpy(td, plan.tiles.data(), plan.tiles.size() * sizeof(hg::BatchTile), cudaMemcpyHostToDevice),
          "tiles");
    g->ntiles = (uint32_t)plan.tiles.size();
    g->warp_words = plan.warp_words;
    g->grid = hg::batch_resident_blocks(g->V);
    g->dcounter.ensure<uint32_t>(4);
    scratch_words = std::max(scratch_words, (size_t)g->grid * hg::batch_warps_per_block() * plan.warp_words);
    b.groups.push_back(std::move(g));
  }
  // the launches run one after another on the stream, so they share scratch
  b.dscratch.ensure<uint32_t>(scratch_words * 4);
  b.derr.ensure<uint32_t>(4);
  b.pin_err.ensure<uint32_t>(4);
  // size the inversion trees now so nothing allocates during a capture
  for (auto& inv : b.invs) {
    const size_t padded = padded_pow2(b.jobs[inv->job].count);
    inv->bufs.tree.ensure<uint32_t>((2 * padded) * (size_t)inv->key->S * 4);
  }
  b.dirty = false;
}

void batch_enqueue(hg_batch& b, cudaStream_t st) {
  uint32_t* err = b.derr.as<uint32_t>();
  cuda_check(cudaMemsetAsync(err, 0, 4, st), "memset err");
  for (auto& g : b.groups) {
    cuda_check(cudaMemsetAsync(g->dcounter.p, 0, 4, st), "memset counter");
    cuda_check(hg::launch_batch(g->V, g->djobs.as<hg::BatchJob>(), g->dtiles.as<hg::BatchTile>(), g->ntiles,
                                g->dcounter.as<uint32_t>(), b.dscratch.as<uint32_t>(), g->warp_words, err, g->grid,
                                st),
               "batch launch");
  }
  for (auto& inv : b.invs) {
    const auto& J = b.jobs[inv->job];
    inv->task.status = 0;
    core_inverse_async(*inv->key, static_cast<const uint32_t*>(J.out), static_cast<const int64_t*>(J.in1),
                       static_cast<uint32_t*>(J.out), J.count, inv->bufs, inv->task, err, st);
  }
  cuda_check(cudaMemcpyAsync(b.pin_err.p, err, 4, cudaMemcpyDeviceToHost, st), "D2H err");
}

}  // namespace

#include "server_impl.hpp"

extern "C" {

int hg_key_get_config(hg_ctx* ctx, int key_id, hg_key_config* out) {
  return guarded(__func__, [&] {
    if (!out) fail(HG_ERR_INVALID, "null argument");
    *out = current_config(*get_key(ctx, key_id));
    return HG_OK;
  });
}

int hg_key_set_config(hg_ctx* ctx, int key_id, const hg_key_config* cfg) {
  return guarded(__func__, [&] {
    if (!cfg) fail(HG_ERR_INVALID, "null argument");
    KeyRec* k = get_key(ctx, key_id);
    if (k->scheme != 0) fail(HG_ERR_UNSUPPORTED, "this call serves ZPaillier keys only");
    set_device(ctx);
    apply_config(*k, *cfg);
    return HG_OK;
  });
}

int hg_autotune(hg_ctx* ctx, int key_id, size_t calib, hg_key_config* best, double* rates) {
  return guarded(__func__, [&] {
    KeyRec* k = get_key(ctx, key_id);
    if (k->scheme != 0) fail(HG_ERR_UNSUPPORTED, "this call serves ZPaillier keys only");
    set_device(ctx);
    const size_t n = calib ? calib : 65536;
    LaneGuard lane(ctx);
    Work& w = *lane.w;
    reset_err(w);
    std::mt19937_64 rng(12345);
    std::vector<int64_t> m(n), kk(n);
    std::vector<uint32_t> r(n * (size_t)k->kc.rlimbs);
    for (auto& v : m) v = (int64_t)(rng() >> 24) - (int64_t)(1ull << 39);
    for (auto& v : kk) v = (int64_t)(rng() >> 1);
    for (auto& v : r) v = (uint32_t)rng();
    const size_t cb = ct_bytes(*k);
    auto* dm = w.io[0].ensure<int64_t>(n * 8);
    auto* dk = w.io[1].ensure<int64_t>(n * 8);
    auto* dr = w.io[2].ensure<uint32_t>(r.size() * 4);
    auto* dct = w.io[3].ensure<uint32_t>(n * cb);
    auto* dout = w.io[4].ensure<uint32_t>(n * cb);
    auto* dm2 = w.io[5].ensure<int64_t>(n * 9);
    h2d(dm, m.data(), n * 8, w);
    h2d(dk, kk.data(), n * 8, w);
    h2d(dr, r.data(), r.size() * 4, w);
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    auto timed = [&](auto&& fn) {
      fn();  // warm
      cuda_check(cudaEventRecord(e0, w.stream), "event");
      fn();
      cuda_check(cudaEventRecord(e1, w.stream), "event");
      cuda_check(cudaEventSynchronize(e1), "event sync");
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      return (double)ms * 1e-3;
    };
    hg_key_config c = current_config(*k), bc = c;
    double best_nn = 1e300, t_enc = 0, t_mul = 0;
    for (int v = 0; v < 2; ++v) {
      c.variant = v;
      apply_config(*k, c);
      const double te = timed([&] { core_encrypt(*k, w, hg::EncMode::kEncrypt, dm, nullptr, nullptr, dr, nullptr, dct, n); });
      for (int wm = 2; wm <= 6; ++wm) {
        c.mul_window = wm;
        apply_config(*k, c);
        const double tm = timed([&] {
          const size_t inst = (size_t)k->grid_mul * hg::instances_per_block(k->S, k->kc.variant);
          uint32_t* scratch = w.scratch.ensure<uint32_t>(inst * ((size_t)1 << (k->wm - 1)) * k->S * 4);
          cuda_check(hg::launch_mul(k->S, k->kc, dct, dk, dout, n, scratch, k->wm, w.errp(), k->grid_mul, w.ctrp(),
                                    w.stream),
                     "mul launch");
        });
        if (te + tm < best_nn) {
          best_nn = te + tm;
          bc.variant = v;
          bc.mul_window = wm;
          t_enc = te;
          t_mul = tm;
        }
      }
    }
    c.variant = bc.variant;
    c.mul_window = bc.mul_window;
    apply_config(*k, c);
    double t_dec = 0;
    if (k->secret) {
      // fresh ciphertexts with the chosen variant
      core_encrypt(*k, w, hg::EncMode::kEncrypt, dm, nullptr, nullptr, dr, nullptr, dct, n);
      // enough ciphertexts for several waves of the widest layout, else the
      // layout with more lanes per ciphertext wins on a half-empty GPU
      const size_t wave = (size_t)hg::resident_blocks_decrypt(k->Sp, 0) * hg::units_per_block_decrypt(k->Sp, 0);
      const size_t nd = std::min(n, std::max<size_t>(n / 2, 4 * wave));
      double best_d = 1e300;
      for (int dv = 0; dv < 2; ++dv)
        for (int wd = 4; wd <= 7; ++wd) {
          c.dec_variant = dv;
          c.dec_window = wd;
          apply_config(*k, c);
          const double td = timed([&] {
            core_decrypt(*k, w, dct, dm2, reinterpret_cast<uint8_t*>(dm2 + nd), nullptr, nullptr, nd);
          });
          if (td < best_d) {
            best_d = td;
            bc.dec_variant = dv;
            bc.dec_window = wd;
          }
        }
      t_dec = best_d / (double)nd;
      c.dec_variant = bc.dec_variant;
      c.dec_window = bc.dec_window;
      apply_config(*k, c);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    finish(w);
    if (best) *best = current_config(*k);
    if (rates) {
      rates[0] = (double)n / t_enc;
      rates[1] = (double)n / t_mul;
      rates[2] = t_dec > 0 ? 1.0 / t_dec : 0.0;
    }
    return HG_OK;
  });
}

int hg_batch_create(hg_ctx* ctx, hg_batch** out) {
  return guarded(__func__, [&] {
    if (!ctx || !out) fail(HG_ERR_INVALID, "null argument");
    auto b = std::make_unique<hg_batch>();
    b->ctx = ctx;
    *out = b.release();
    return HG_OK;
  });
}

int hg_batch_destroy(hg_batch* b) {
  return guarded(__func__, [&] {
    if (b) {
      cudaSetDevice(b->ctx->device);
      cudaDeviceSynchronize();
      delete b;
    }
    return HG_OK;
  });
}

int hg_batch_add(hg_batch* b, int key_id, int op, size_t count, const void* in0, const void* in1, void* out,
                 void* aux, int flags) {
  return guarded(__func__, [&] {
    if (!b) fail(HG_ERR_INVALID, "null batch");
    if (op < hg::kBatchEncrypt || op > hg::kBatchMul) fail(HG_ERR_INVALID, "unknown batch op");
    if (count == 0) return HG_OK;
    if (!in0 || !out || (op != hg::kBatchDecrypt && !in1)) fail(HG_ERR_INVALID, "null job pointer");
    if (count >= (1ull << 31)) fail(HG_ERR_INVALID, "job too large");
    if (get_key(b->ctx, key_id)->scheme != 0) fail(HG_ERR_UNSUPPORTED, "batches serve ZPaillier keys only");
    b->jobs.push_back({key_id, op, flags, count, in0, in1, out, aux});
    b->dirty = true;
    b->drop_graph();
    return HG_OK;
  });
}

int hg_batch_clear(hg_batch* b) {
  return guarded(__func__, [&] {
    if (!b) fail(HG_ERR_INVALID, "null batch");
    b->jobs.clear();
    b->dirty = true;
    b->drop_graph();
    return HG_OK;
  });
}

int hg_batch_set_variant(hg_batch* b, int variant) {
  return guarded(__func__, [&] {
    if (!b || (variant != HG_BATCH_PER_KEY && (variant < 0 || variant > 1)))
      fail(HG_ERR_INVALID, "variant must be 0, 1 or HG_BATCH_PER_KEY");
    if (variant != b->variant) {
      b->variant = variant;
      b->dirty = true;
      b->drop_graph();
    }
    return HG_OK;
  });
}

int hg_batch_run(hg_batch* b, void* stream, int use_graph) {
  return guarded(__func__, [&] {
    if (!b) fail(HG_ERR_INVALID, "null batch");
    set_device(b->ctx);
    cudaStream_t st = stream ? (cudaStream_t)stream : b->ctx->lanes[0]->stream;
    if (b->dirty) batch_build(*b);
    if (!use_graph) {
      batch_enqueue(*b, st);
      return HG_OK;
    }
    if (!b->exec) {
      // every buffer is sized by batch_build; capture the whole sequence once
      cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
      try {
        batch_enqueue(*b, st);
      } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      cuda_check(cudaStreamEndCapture(st, &b->graph), "end capture");
      cuda_check(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
    }
    cuda_check(cudaGraphLaunch(b->exec, st), "graph launch");
    uint64_t per_run = 1;
    for (auto& inv : b->invs) {
      size_t padded = 1, levels = 0;
      while (padded < b->jobs[inv->job].count) {
        padded <<= 1;
        ++levels;
      }
      per_run += 2 * levels + 2;
    }
    hg::count_launches(per_run);
    return HG_OK;
  });
}

int hg_batch_wait(hg_batch* b, void* stream) {
  return guarded(__func__, [&] {
    if (!b) fail(HG_ERR_INVALID, "null batch");
    set_device(b->ctx);
    cudaStream_t st = stream ? (cudaStream_t)stream : b->ctx->lanes[0]->stream;
    cuda_check(cudaStreamSynchronize(st), "stream sync");
    raise_err_bits(*b->pin_err.as<uint32_t>());
    for (auto& inv : b->invs) raise_task_status(inv->task);
    return HG_OK;
  });
}



int hg_server_create(hg_ctx* ctx, const hg_server_config* cfg, hg_server** out) {
  return guarded(__func__, [&] {
    if (!ctx || !out) fail(HG_ERR_INVALID, "null argument");
    set_device(ctx);
    auto s = std::make_unique<hg_server>();
    s->ctx = ctx;
    hg_server_config c{};
    c.budget_bytes = (size_t)40 << 30;
    c.slots = 4;
    c.max_batch_elems = 1 << 20;
    c.variant = 0;
    if (cfg) {
      if (cfg->budget_bytes) c.budget_bytes = cfg->budget_bytes;
      if (cfg->slots > 0) c.slots = cfg->slots;
      if (cfg->max_batch_elems) c.max_batch_elems = cfg->max_batch_elems;
      c.variant = cfg->variant;
    }
    if (c.variant < 0 || c.variant > 1) fail(HG_ERR_INVALID, "variant must be 0 or 1");
    s->cfg = c;
    s->variant = c.variant;
    if (cfg && cfg->batch_us > 0) s->batch_us = cfg->batch_us;
    if (cfg && cfg->slice_us > 0) s->slice_us = cfg->slice_us;
    if (cfg && (cfg->policy < 0 || cfg->policy > 1)) fail(HG_ERR_INVALID, "policy must be 0 or 1");
    s->policy = cfg ? cfg->policy : 0;
    // every kernel the server launches asks for the same L1 / shared split,
    // so no SM has to drain to switch between them
    hg::batch_prefer_shared_carveout();
    hg::server_prefer_shared_carveout();
    const int resident = hg::batch_resident_blocks(c.variant);
    const int bps = hg::batch_blocks_per_sm(c.variant);
    const int sms = std::max(1, resident / std::max(1, bps));
    s->sms = current_sm_count();
    s->express_us = (cfg && cfg->express_us != 0.0) ? cfg->express_us : -1.0;
    s->express_len = cfg ? cfg->express_len : 0;
    if (s->express_len > 0) s->express_us = 0.0;  // the length rule replaces the cost rule
    // the length rule's two express slots keep half of every SM's blocks (one
    // each at four per SM); the cost rule's one slot a quarter
    const double share = (cfg && cfg->express_share > 0.0) ? cfg->express_share : s->express_len > 0 ? 0.5 : 0.25;
    if (share >= 1.0) fail(HG_ERR_INVALID, "express_share must be below 1");
    if (c.slots < 2 || bps < 2) {
      s->express_us = -1.0;
      s->express_len = 0;
    }
    s->regular_grid = resident;
    if (s->express_us >= 0.0) {
      // express: `eb` blocks on every SM; regular batches: the rest
      const int eb = std::min(bps - 1, std::max(1, (int)(share * bps + 0.5)));
      s->express_grid = eb * sms;
      s->regular_grid = (bps - eb) * sms;
      s->regular_smem = hg::batch_smem_cap(c.variant, bps - eb);
    }
    // batch-kernel scratch: the largest per-warp table over the loaded keys
    size_t warp_words = 1;
    {
      std::lock_guard<std::mutex> lk(ctx->mu);
      for (auto& kv : ctx->keys) {
        const KeyRec& k = *kv.second;
        if (k.scheme != 0) continue;  // the server serves ZPaillier keys only
        warp_words = std::max(warp_words, (size_t)(32 / hg::tpi_for(k.S, c.variant)) * ((size_t)1 << (k.wm - 1)) * k.S);
        if (k.secret)
          warp_words = std::max(warp_words, (size_t)(32 / (2 * hg::tp_for(k.Sp, c.variant))) * 2 *
                                                ((size_t)1 << (k.sc.wd - 1)) * k.Sp);
      }
    }
    const size_t scratch = (size_t)hg::batch_resident_blocks(c.variant) * hg::batch_warps_per_block() * warp_words * 4;
    const size_t arena = c.budget_bytes / (size_t)c.slots;
    for (int i = 0; i < c.slots; ++i) {
      auto sl = std::make_unique<Slot>();
      sl->express = (i == 0 && s->express_us >= 0.0);
      // the length rule: an express slot for short decryptions (slot 1), and
      // with five slots or more a second one for the other short requests
      // (slot 2), so a short request does not wait for the batch before it
      sl->express_dec = (i == 1 && s->express_len > 0 && c.slots >= 3);
      if (sl->express_dec) sl->express = true;
      if (i == 2 && s->express_len > 0 && c.slots >= 5) sl->express = true;
      int lo_prio = 0, hi_prio = 0;
      cuda_check(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio), "priority range");
      cuda_check(cudaStreamCreateWithPriority(&sl->st, cudaStreamNonBlocking, sl->express ? hi_prio : lo_prio),
                 "stream");
      cuda_check(cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming), "event");
      for (auto& e : sl->tev) cuda_check(cudaEventCreate(&e), "trace event");
      sl->dev.base = sl->dev_mem.ensure<uint8_t>(arena);
      sl->dev.cap = arena;
      sl->pin.base = sl->pin_mem.ensure<uint8_t>((size_t)16 << 20);
      sl->pin.cap = (size_t)16 << 20;
      sl->scratch.ensure<uint32_t>(scratch);
      sl->counter.ensure<uint32_t>(4);
      sl->err.ensure<uint32_t>(4);
      s->slots.push_back(std::move(sl));
    }
    hg_server* raw = s.get();
    if (s->express_len > 0) {
      s->sched = std::thread(scheduler, raw, kRegularSlots);
      for (size_t i = 0; i < s->slots.size(); ++i)
        if (s->slots[i]->express) s->sched_express.emplace_back(scheduler, raw, (int)i);
    } else {
      s->sched = std::thread(scheduler, raw, -1);
    }
    *out = s.release();
    return HG_OK;
  });
}

int hg_server_destroy(hg_server* s) {
  return guarded(__func__, [&] {
    if (!s) return HG_OK;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->sched.joinable()) s->sched.join();
    for (auto& t : s->sched_express)
      if (t.joinable()) t.join();
    cudaSetDevice(s->ctx->device);
    for (auto& sl : s->slots) {
      cudaStreamSynchronize(sl->st);
      cudaStreamDestroy(sl->st);
      cudaEventDestroy(sl->ev);
      for (auto& e : sl->tev)
        if (e) cudaEventDestroy(e);
    }
    if (s->trace_ref) cudaEventDestroy(s->trace_ref);
    delete s;
    return HG_OK;
  });
}

int hg_server_store(hg_server* s, int key_id, const uint32_t* host_ct, size_t count, uint64_t* handle) {
  return guarded(__func__, [&] {
    if (!s || !host_ct || !handle || count == 0) fail(HG_ERR_INVALID, "null argument");
    KeyRec* k = get_key(s->ctx, key_id);
    if (k->scheme != 0) fail(HG_ERR_UNSUPPORTED, "this call serves ZPaillier keys only");
    set_device(s->ctx);
    auto r = std::make_unique<Resident>();
    r->key_id = key_id;
    r->count = count;
    void* d = r->buf.ensure<void>(count * (size_t)k->S * 4);
    cuda_check(cudaMemcpy(d, host_ct, count * (size_t)k->S * 4, cudaMemcpyHostToDevice), "H2D resident");
    std::lock_guard<std::mutex> lk(s->mu);
    *handle = s->next_handle++;
    s->residents[*handle] = std::move(r);
    return HG_OK;
  });
}

int hg_server_release(hg_server* s, uint64_t handle) {
  return guarded(__func__, [&] {
    if (!s) fail(HG_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    // no request in flight may still read it
    s->cv_done.wait(lk, [&] { return s->pending.empty() && s->inflight == 0; });
    if (!s->residents.erase(handle)) fail(HG_ERR_INVALID, "unknown resident vector handle");
    return HG_OK;
  });
}

int hg_server_submit(hg_server* s, const hg_request* req, uint64_t* ticket) {
  return guarded(__func__, [&] {
    if (!s || !req || !ticket) fail(HG_ERR_INVALID, "null argument");
    if (req->op < hg::kBatchEncrypt || req->op > kOpSum) fail(HG_ERR_INVALID, "unknown request op");
    if (req->count == 0) fail(HG_ERR_INVALID, "empty request");
    if (!req->out) fail(HG_ERR_INVALID, "request without an output buffer");
    KeyRec* k = get_key(s->ctx, req->key_id);
    if (k->scheme != 0) fail(HG_ERR_UNSUPPORTED, "this call serves ZPaillier keys only");
    if (req->op == hg::kBatchDecrypt && !k->secret) fail(HG_ERR_NO_SECRET, "decrypt request on a public key");
    if ((req->op == hg::kBatchEncrypt || req->op == hg::kBatchMul) && (!req->in0 && !req->h0))
      fail(HG_ERR_INVALID, "request without input");
    if (req->op == hg::kBatchMul && !req->in1) fail(HG_ERR_INVALID, "mul request without scalars");
    if (req->op == hg::kBatchEncrypt && !req->in1) fail(HG_ERR_INVALID, "encrypt request without r");
    auto q = std::make_unique<Req>();
    q->r = *req;
    q->k = k;
    // the smallest slice must fit a slot (sums are never sliced)
    q->dev_bytes = slice_dev_bytes(*k, *req, req->op == kOpSum ? req->count : 1);
    if (q->dev_bytes > s->slots[0]->dev.cap) fail(HG_ERR_NOMEM, "request larger than a server slot");
    q->t_sub = std::chrono::steady_clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (req->h0 && !s->residents.count(req->h0)) fail(HG_ERR_INVALID, "unknown resident vector handle");
      if (req->h1 && !s->residents.count(req->h1)) fail(HG_ERR_INVALID, "unknown resident vector handle");
      q->id = s->next_id++;
      *ticket = q->id;
      s->pending.push_back(q.get());
      s->reqs[q->id] = std::move(q);
    }
    s->cv_work.notify_all();
    return HG_OK;
  });
}

namespace {

// hg_server_wait, with the request's phases (3 values, may be null).
int server_wait(hg_server* s, uint64_t ticket, double* latency_s, double* phases) {
  int status = HG_OK;
  const int rc = guarded("hg_server_wait", [&] {
    if (!s) fail(HG_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) fail(HG_ERR_INVALID, "unknown ticket");
    Req* q = it->second.get();
    s->cv_done.wait(lk, [&] { return q->done; });
    auto sec = [](std::chrono::steady_clock::duration d) { return std::chrono::duration<double>(d).count(); };
    if (latency_s) latency_s[0] = sec(q->t_done - q->t_sub);
    if (phases) {
      phases[0] = sec(q->t_admit - q->t_sub);
      phases[1] = sec(q->t_launch - q->t_admit);
      phases[2] = sec(q->t_done - q->t_launch);
    }
    status = q->status;
    s->reqs.erase(it);
    return HG_OK;
  });
  if (rc != HG_OK) return rc;
  if (status != HG_OK) g_last_error = "request failed";
  return status;
}

}  // namespace

int hg_server_wait(hg_server* s, uint64_t ticket, double* latency_s) {
  return server_wait(s, ticket, latency_s, nullptr);
}

int hg_server_stats(hg_server* s, uint64_t* completed, uint64_t* batches, size_t* inflight_bytes, size_t* pending) {
  return guarded(__func__, [&] {
    if (!s) fail(HG_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (completed) *completed = s->completed;
    if (batches) *batches = s->batches;
    if (inflight_bytes) *inflight_bytes = s->inflight;
    if (pending) *pending = s->pending.size();
    return HG_OK;
  });
}

int hg_probe_serve_load(hg_server* s, const hg_load_spec* spec, double* latencies, int* ops, uint64_t* lens,
                        double* wall_s) {
  return guarded(__func__, [&] {
    if (!s || !spec || !latencies) fail(HG_ERR_INVALID, "null argument");
    std::mt19937_64 rng(spec->seed);
    std::exponential_distribution<double> gap(spec->rate);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    std::discrete_distribution<int> opd(spec->op_weights, spec->op_weights + 5);
    const double lmin = std::log((double)spec->len_min), lmax = std::log((double)spec->len_max + 1.0);
    std::vector<uint64_t> tickets(spec->nreq);
    const auto t0 = std::chrono::steady_clock::now();
    double t_next = 0.0;
    static const int op_map[5] = {hg::kBatchEncrypt, hg::kBatchAdd, hg::kBatchMul, kOpSum, hg::kBatchDecrypt};
    for (size_t i = 0; i < spec->nreq; ++i) {
      t_next += gap(rng);
      while (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() < t_next) {
      }
      const int ki = (int)(rng() % (uint64_t)spec->nkeys);
      size_t len = (size_t)std::floor(std::exp(lmin + (lmax - lmin) * u01(rng)));
      len = std::min(std::max(len, spec->len_min), spec->len_max);
      const int op = op_map[opd(rng)];
      hg_request r{};
      r.key_id = spec->key_ids[ki];
      r.op = op;
      r.count = len;
      r.out = spec->sink;
      if (op == hg::kBatchEncrypt) {
        r.in0 = spec->m_host;
        r.in1 = spec->r_host;
      } else if (op == hg::kBatchMul) {
        r.h0 = spec->handles[ki];
        r.in1 = spec->k_host;
      } else if (op == hg::kBatchAdd) {
        r.h0 = spec->handles[ki];
        r.h1 = spec->handles[ki];
      } else {
        r.h0 = spec->handles[ki];
      }
      const int rc = hg_server_submit(s, &r, &tickets[i]);
      if (rc != HG_OK) fail(rc, g_last_error);
      if (ops) ops[i] = op;
      if (lens) lens[i] = len;
    }
    for (size_t i = 0; i < spec->nreq; ++i) {
      double ph[3];
      const int rc = server_wait(s, tickets[i], &latencies[i], spec->phases ? ph : nullptr);
      if (spec->phases)
        for (int k = 0; k < 3; ++k) spec->phases[3 * i + k] = ph[k];
      if (rc != HG_OK) fail(rc, "served request failed");
    }
    if (wall_s) *wall_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return HG_OK;
  });
}

int hg_probe_server_trace(hg_server* s, int enable, double* records, size_t cap, size_t* n) {
  return guarded(__func__, [&] {
    if (!s) fail(HG_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (enable) {
      set_device(s->ctx);
      if (!s->trace_ref) cuda_check(cudaEventCreate(&s->trace_ref), "trace event");
      s->traces.clear();
      // the reference event goes on an idle slot's stream, so the GPU takes
      // its time stamp when the host does
      cudaStream_t st = nullptr;
      for (auto& sl : s->slots)
        if (!sl->busy) st = sl->st;
      if (!st) fail(HG_ERR_INVALID, "trace enabled while every slot is busy");
      s->trace_t0 = std::chrono::steady_clock::now();
      cuda_check(cudaEventRecord(s->trace_ref, st), "trace event");
      s->trace = true;
      if (n) *n = 0;
      return HG_OK;
    }
    s->trace = false;
    if (n) *n = s->traces.size();
    if (records)
      for (size_t i = 0; i < std::min(cap, s->traces.size()); ++i)
        std::memcpy(records + i * kTraceFields, s->traces[i].data(), sizeof(double) * kTraceFields);
    return HG_OK;
  });
}

int hg_probe_set_alloc_limit(size_t bytes, size_t* held_bytes) {
  g_dev_limit = bytes;
  if (held_bytes) *held_bytes = g_dev_bytes.load();
  return HG_OK;
}

int hg_probe_launch_count(uint64_t* out) {
  if (!out) return HG_ERR_INVALID;
  *out = hg::launch_count();
  return HG_OK;
}

int hg_dev_check(hg_ctx* ctx) {
  return guarded(__func__, [&] {
    if (!ctx) fail(HG_ERR_INVALID, "null context");
    set_device(ctx);
    uint32_t bits = 0;
    std::lock_guard<std::mutex> lk(ctx->dev_mu);
    for (auto& kv : ctx->dev_work) {
      Work& w = *kv.second;
      uint32_t* h = w.pin_err.ensure<uint32_t>(sizeof(uint32_t));
      cuda_check(cudaMemcpyAsync(h, w.errp(), sizeof(uint32_t), cudaMemcpyDeviceToHost, w.stream), "D2H err");
      cuda_check(cudaStreamSynchronize(w.stream), "stream sync");
      bits |= *h;
      cuda_check(cudaMemsetAsync(w.errp(), 0, sizeof(uint32_t), w.stream), "memset err");
    }
    raise_err_bits(bits);
    return HG_OK;
  });
}

}  // extern "C"

namespace hg {

int key_view(hg_ctx* ctx, int key_id, KeyConst* kc, int* S, int* device, cudaStream_t* own_stream) {
  if (!ctx) return HG_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->keys.find(key_id);
  if (it == ctx->keys.end()) return HG_ERR_INVALID;
  *kc = it->second->kc;
  *S = it->second->S;
  *device = ctx->device;
  *own_stream = ctx->lanes[0]->stream;
  return HG_OK;
}

void set_last_error(const char* msg) { g_last_error = msg; }

}  // namespace hg
