// Continuous-batching request server (hg_server_* of the C-ABI).
//
// Included into engine.cu's translation unit: it uses the engine's key
// records, inversion tasks and batch planner.
//
// The server owns `slots` in-flight micro-batches, each with its own stream,
// a device arena, a pinned arena and a scratch buffer for the persistent
// batch kernel, all sized when the server starts so nothing is allocated
// while serving.  Requests wait in a queue; whenever a slot is free its
// scheduler thread admits requests while their device bytes fit the slot's
// arena and the server-wide budget, stages their host inputs, runs all their
// encrypt / decrypt / add / mul work in one persistent launch (sums as tree
// reduction levels, negative scalars as product trees with a host inversion),
// copies the results back and records an event.  Requests that arrive
// meanwhile are admitted into the next free slot while earlier slots are
// still on the GPU, so their work overlaps on the device.  With the length
// rule (express_len) short requests go to express slots: each has its own
// scheduler thread, runs the latency layout of the batch kernel and keeps a
// share of every SM that the padded regular batches cannot take.

namespace {

constexpr int kOpSum = 4;  // server-only op on top of the batch ops

struct Arena {
  uint8_t* base = nullptr;
  size_t cap = 0, off = 0;
  void reset() { off = 0; }
  bool fits(size_t bytes) const { return off + ((bytes + 255) & ~size_t(255)) <= cap; }
  template <typename T>
  T* take(size_t bytes) {
    const size_t a = (bytes + 255) & ~size_t(255);
    if (off + a > cap) fail(HG_ERR_NOMEM, "server arena exhausted");
    T* p = reinterpret_cast<T*>(base + off);
    off += a;
    return p;
  }
};

struct Resident {
  int key_id;
  size_t count;
  DevBuf buf;
};

struct Req {
  hg_request r;
  KeyRec* k = nullptr;
  uint64_t id = 0;
  size_t dev_bytes = 0;
  std::chrono::steady_clock::time_point t_sub, t_done;
  std::chrono::steady_clock::time_point t_admit, t_launch;  // first slice: admitted, its batch launched
  int status = HG_OK;
  bool done = false;
  InvTask* task = nullptr;
  const void* p0 = nullptr;  // resolved resident vectors (set at admission, under the lock)
  const void* p1 = nullptr;
  size_t next = 0;         // first element not yet handed to a micro-batch
  int outstanding = 0;     // slices on the GPU
  std::vector<std::unique_ptr<InvTask>> tasks;
};

// A contiguous slice [start, start + len) of one request.
struct Slice {
  Req* q;
  size_t start, len;
  size_t bytes;
  InvTask* task;
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  DevBuf dev_mem, scratch, counter, err;
  PinBuf pin_mem;
  Arena dev, pin;
  std::vector<Slice> slices;
  size_t bytes = 0;
  uint32_t* err_host = nullptr;
  bool busy = false;
  bool express = false;      // runs short requests on a reserved share of every SM
  bool express_dec = false;  // the express slot of short decryptions
  // per-batch trace (probe): timing events around the staged copies, the
  // kernels and the copies back, and the host times of the batch
  cudaEvent_t tev[4] = {nullptr, nullptr, nullptr, nullptr};
  bool traced = false;
  double tr[6] = {0, 0, 0, 0, 0, 0};  // class, slices, elems, op mask, formed, launched
  std::chrono::steady_clock::time_point t_launched;  // host time the batch was queued
};

// Fields of one trace record (hg_probe_server_trace).
constexpr int kTraceFields = 12;

size_t slice_dev_bytes(const KeyRec& k, const hg_request& r, size_t n) {
  const size_t cb = (size_t)k.S * 4, pad = 256;
  const size_t tree = 2 * padded_pow2(n) * cb + cb + pad;
  switch (r.op) {
    case hg::kBatchEncrypt: return n * 8 + n * (size_t)k.kc.rlimbs * 4 + n * cb + 3 * pad;
    case hg::kBatchDecrypt: return (r.h0 ? 0 : n * cb) + n * 9 + 3 * pad;
    case hg::kBatchAdd: return (r.h0 ? 0 : n * cb) + (r.h1 ? 0 : n * cb) + n * cb + 3 * pad;
    case hg::kBatchMul: return (r.h0 ? 0 : n * cb) + n * 8 + n * cb + tree + 3 * pad;
    case kOpSum: return (r.h0 ? 0 : n * cb) + 2 * ((n + 1) / 2) * cb + cb + 4 * pad;
    default: return 0;
  }
}

// Estimated GPU time of one element of an op, in microseconds (cost model
// used to size micro-batches; the kernels do not depend on it).
double elem_cost_us(const KeyRec& k, int op) {
  if (op == kOpSum) return (double)k.S * k.S / 3.11e6;
  return job_cost(k, op) / 3.11e6;
}

}  // namespace

struct hg_server {
  hg_ctx* ctx = nullptr;
  hg_server_config cfg{};
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req*> pending;
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
  std::unordered_map<uint64_t, std::unique_ptr<Resident>> residents;
  uint64_t next_id = 1, next_handle = 1;
  size_t inflight = 0;
  uint64_t completed = 0, batches = 0;
  bool stop = false;
  int variant = 0;
  double batch_us = 100000.0;  // target GPU time of one micro-batch
  double slice_us = 50000.0;   // most GPU time one request gets per micro-batch
  int policy = 0;              // HG_POLICY_SHORTEST or HG_POLICY_FIFO
  double express_us = -1.0;    // short-request threshold of the express slot (< 0: none)
  size_t express_len = 0;      // > 0: short = at most this many elements, run in the latency layout
  int express_grid = 0;        // batch-kernel blocks of all express slots together
  int regular_grid = 0;        // batch-kernel blocks of every other slot
  int sms = 1;                 // multiprocessors of the server's device
  size_t regular_smem = 0;     // dynamic shared memory that keeps regular batches
                               // off the express slots' blocks on every SM
  std::thread sched;                      // every slot, or the regular slots (length rule)
  std::vector<std::thread> sched_express;  // one per express slot (length rule)
  bool trace = false;              // record one trace record per retired batch
  std::chrono::steady_clock::time_point trace_t0;
  cudaEvent_t trace_ref = nullptr;  // GPU time zero of the trace
  std::vector<std::array<double, kTraceFields>> traces;
};

namespace {

const void* resident_ptr(hg_server& s, uint64_t h, const KeyRec& k, size_t count) {
  auto it = s.residents.find(h);
  if (it == s.residents.end()) fail(HG_ERR_INVALID, "unknown resident vector handle");
  if (it->second->count < count) fail(HG_ERR_INVALID, "request longer than its resident vector");
  if (it->second->key_id < 0 || get_key(s.ctx, it->second->key_id) != &k)
    fail(HG_ERR_INVALID, "resident vector belongs to another key");
  return it->second->buf.p;
}

// Stage and enqueue one micro-batch on its slot (scheduler thread, no lock).
void run_slot(hg_server& s, Slot& sl) {
  sl.dev.reset();
  sl.pin.reset();
  cudaStream_t st = sl.st;
  std::vector<JobSpec> specs;
  struct Post {
    Req* q;
    const void* dev_out;
    size_t bytes;
    const void* dev_aux;
    size_t aux_bytes;
    size_t out_off, aux_off;  // byte offsets of the slice in the host buffers
  };
  std::vector<Post> posts;
  struct SumJob {
    Req* q;
    const uint32_t* src;
    uint32_t* bufs[2];
    uint32_t* out;
  };
  std::vector<SumJob> sums;
  struct InvJob {
    Req* q;
    KeyRec* k;
    uint32_t* data;
    const int64_t* sel;
    size_t count;
    uint32_t* tree;
    InvTask* task;
  };
  std::vector<InvJob> invs;
  uint32_t* err = sl.err.as<uint32_t>();
  if (sl.traced) cuda_check(cudaEventRecord(sl.tev[0], st), "trace event");
  cuda_check(cudaMemsetAsync(err, 0, 4, st), "memset err");
  for (Slice& sc : sl.slices) {
    Req* q = sc.q;
    const hg_request& r = q->r;
    KeyRec& k = *q->k;
    const size_t n = sc.len, cb = (size_t)k.S * 4, s0 = sc.start;
    auto h2d_in = [&](const void* host, size_t bytes) {
      void* d = sl.dev.take<void>(bytes);
      cuda_check(cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, st), "H2D");
      return d;
    };
    auto at = [](const void* p, size_t off) -> const void* { return static_cast<const uint8_t*>(p) + off; };
    auto ct_in = [&](const void* resident, const void* host) -> const void* {
      return resident ? at(resident, s0 * cb) : h2d_in(at(host, s0 * cb), n * cb);
    };
    if (r.op == hg::kBatchEncrypt) {
      const void* m = h2d_in(at(r.in0, s0 * 8), n * 8);
      const size_t rb = (size_t)k.kc.rlimbs * 4;
      const void* rr = h2d_in(at(r.in1, s0 * rb), n * rb);
      void* out = sl.dev.take<void>(n * cb);
      specs.push_back({&k, r.op, 0, n, m, rr, out, nullptr});
      posts.push_back({q, out, n * cb, nullptr, 0, s0 * cb, 0});
    } else if (r.op == hg::kBatchDecrypt) {
      const void* c = ct_in(q->p0, r.in0);
      void* out = sl.dev.take<void>(n * 8);
      void* ovf = sl.dev.take<void>(n);
      specs.push_back({&k, r.op, 0, n, c, nullptr, out, ovf});
      posts.push_back({q, out, n * 8, r.aux ? ovf : nullptr, r.aux ? n : 0, s0 * 8, s0});
    } else if (r.op == hg::kBatchAdd) {
      const void* a = ct_in(q->p0, r.in0);
      const void* b = ct_in(q->p1, r.in1);
      void* out = sl.dev.take<void>(n * cb);
      specs.push_back({&k, r.op, 0, n, a, b, out, nullptr});
      posts.push_back({q, out, n * cb, nullptr, 0, s0 * cb, 0});
    } else if (r.op == hg::kBatchMul) {
      const void* a = ct_in(q->p0, r.in0);
      const int64_t* hk = static_cast<const int64_t*>(r.in1) + s0;
      bool neg = false;
      for (size_t i = 0; i < n && !neg; ++i) neg = hk[i] < 0;
      const void* kk = h2d_in(hk, n * 8);
      auto* out = sl.dev.take<uint32_t>(n * cb);
      specs.push_back({&k, r.op, neg ? 0 : HG_JOB_NONNEG, n, a, kk, out, nullptr});
      if (neg) {
        InvTask* task = sc.task;
        task->root = sl.pin.take<uint32_t>(cb + 4);
        task->z = sl.pin.take<uint32_t>(cb);
        const size_t padded = padded_pow2(n);
        invs.push_back({q, &k, out, static_cast<const int64_t*>(kk), n, sl.dev.take<uint32_t>(2 * padded * cb),
                        task});
      }
      posts.push_back({q, out, n * cb, nullptr, 0, s0 * cb, 0});
    } else {  // sum
      const auto* src = static_cast<const uint32_t*>(ct_in(q->p0, r.in0));
      const size_t half = (n + 1) / 2;
      SumJob sj{q, src, {sl.dev.take<uint32_t>(half * cb), sl.dev.take<uint32_t>(half * cb)},
                sl.dev.take<uint32_t>(cb)};
      sums.push_back(sj);
      posts.push_back({q, sj.out, cb, nullptr, 0, 0, 0});
    }
  }
  if (!specs.empty()) {
    // express batches of the length rule run in the latency layout
    const int V = (sl.express && s.express_len > 0) ? hg::kBatchLatencyVariant : s.variant;
    const BatchPlan plan = plan_batch(specs, V);
    const size_t jb = plan.jobs.size() * sizeof(hg::BatchJob), tb = plan.tiles.size() * sizeof(hg::BatchTile);
    auto* hj = sl.pin.take<uint8_t>(jb);
    auto* ht = sl.pin.take<uint8_t>(tb);
    std::memcpy(hj, plan.jobs.data(), jb);
    std::memcpy(ht, plan.tiles.data(), tb);
    auto* dj = sl.dev.take<hg::BatchJob>(jb);
    auto* dt = sl.dev.take<hg::BatchTile>(tb);
    cuda_check(cudaMemcpyAsync(dj, hj, jb, cudaMemcpyHostToDevice, st), "H2D jobs");
    cuda_check(cudaMemcpyAsync(dt, ht, tb, cudaMemcpyHostToDevice, st), "H2D tiles");
    cuda_check(cudaMemsetAsync(sl.counter.p, 0, 4, st), "memset counter");
    if (sl.traced) cuda_check(cudaEventRecord(sl.tev[1], st), "trace event");
    // the express slots split the reserved blocks, so none waits for
    // another's blocks to retire
    int n_express = 0;
    for (auto& o : s.slots) n_express += o->express ? 1 : 0;
    const int grid = sl.express ? std::max(1, s.express_grid / std::max(1, n_express)) : s.regular_grid;
    if ((size_t)grid * hg::batch_warps_per_block() * plan.warp_words * 4 > sl.scratch.n)
      fail(HG_ERR_NOMEM, "server scratch too small for this batch");
    // regular batches carry shared-memory padding that caps them below the
    // per-SM block limit, so however many overlap, every SM keeps room for
    // the express slots' blocks
    cuda_check(hg::launch_batch(V, dj, dt, (uint32_t)plan.tiles.size(), sl.counter.as<uint32_t>(),
                                sl.scratch.as<uint32_t>(), plan.warp_words, err, grid, st,
                                sl.express ? 0 : s.regular_smem),
               "batch launch");
  }
  // launched: the staged copies and the batch kernel are queued (the
  // inversions below may wait for the kernel on this thread)
  sl.t_launched = std::chrono::steady_clock::now();
  for (auto& iv : invs) {
    iv.task->status = 0;
    // express batches invert on their own scheduler thread (see
    // core_inverse_async_raw), regular ones through a stream host function
    core_inverse_async_raw(*iv.k, iv.data, iv.sel, iv.data, iv.count, iv.tree, *iv.task, err, st, sl.express);
  }
  for (auto& sj : sums) {
    KeyRec& k = *sj.q->k;
    size_t n = sj.q->r.count;  // sums are never sliced
    const uint32_t* cur = sj.src;
    int which = 0;
    if (n == 1) {
      cuda_check(cudaMemcpyAsync(sj.out, cur, (size_t)k.S * 4, cudaMemcpyDeviceToDevice, st), "copy");
    }
    while (n > 1) {
      const int chunk = hg::reduce_tree_chunk(k.S, n, s.sms);
      const size_t on = hg::reduce_tree_outputs(k.S, n, chunk);
      uint32_t* dst = on == 1 ? sj.out : sj.bufs[which];
      cuda_check(hg::launch_reduce_tree(k.S, k.kc, cur, n, chunk, dst, err, st), "reduce");
      cur = dst;
      n = on;
      which ^= 1;
    }
  }
  if (sl.traced) {
    if (specs.empty()) cuda_check(cudaEventRecord(sl.tev[1], st), "trace event");
    cuda_check(cudaEventRecord(sl.tev[2], st), "trace event");
  }
  for (auto& p : posts) {
    cuda_check(cudaMemcpyAsync(static_cast<uint8_t*>(p.q->r.out) + p.out_off, p.dev_out, p.bytes,
                               cudaMemcpyDeviceToHost, st),
               "D2H");
    if (p.dev_aux)
      cuda_check(cudaMemcpyAsync(static_cast<uint8_t*>(p.q->r.aux) + p.aux_off, p.dev_aux, p.aux_bytes,
                                 cudaMemcpyDeviceToHost, st),
                 "D2H");
  }
  sl.err_host = sl.pin.take<uint32_t>(4);
  cuda_check(cudaMemcpyAsync(sl.err_host, err, 4, cudaMemcpyDeviceToHost, st), "D2H err");
  if (sl.traced) cuda_check(cudaEventRecord(sl.tev[3], st), "trace event");
  cuda_check(cudaEventRecord(sl.ev, st), "event");
}

double since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// One trace record of a retired batch (under the lock): slot, class,
// slices, elements, op mask (bit per op), the host times at which the batch
// was formed, launched and retired (seconds since the trace started), the
// GPU time at which its stream started it (seconds since the trace's
// reference event), and the milliseconds its stream spent on staged copies,
// on the kernels and on the copies back.
void trace_retire(hg_server& s, Slot& sl) {
  std::array<double, kTraceFields> r{};
  int idx = 0;
  for (size_t i = 0; i < s.slots.size(); ++i)
    if (s.slots[i].get() == &sl) idx = (int)i;
  r[0] = idx;
  for (int i = 0; i < 4; ++i) r[1 + i] = sl.tr[i];
  r[5] = sl.tr[4];
  r[6] = sl.tr[5];
  r[7] = since(s.trace_t0);
  float ms = -1.0f;
  if (cudaEventElapsedTime(&ms, s.trace_ref, sl.tev[0]) != cudaSuccess) ms = -1.0f;
  r[8] = ms * 1e-3;
  for (int i = 0; i < 3; ++i) {
    if (cudaEventElapsedTime(&ms, sl.tev[i], sl.tev[i + 1]) != cudaSuccess) ms = -1.0f;
    r[9 + i] = ms;
  }
  if (s.traces.size() < ((size_t)1 << 20)) s.traces.push_back(r);
  sl.traced = false;
}

void finish_req(hg_server& s, Req* q) {
  q->done = true;
  q->t_done = std::chrono::steady_clock::now();
  ++s.completed;
  s.cv_done.notify_all();
}

// Class of a pending request: 0 regular, 1 express, 2 slow express.
// With express_len, short = at most express_len elements; short CRT
// decryptions (a chain of ~2,400 dependent Montgomery steps, several ms even
// on an idle GPU) get the second express slot when there is one, so a batch
// of the other short ops never waits for them.  Without express_len, short
// = estimated remaining work <= express_us.
int req_class(const hg_server& s, const Req* q) {
  if (s.express_len > 0) {
    if (q->r.count > s.express_len) return 0;
    bool dec_slot = false;
    for (auto& slp : s.slots) dec_slot |= slp->express_dec;
    return (dec_slot && q->r.op == hg::kBatchDecrypt) ? 2 : 1;
  }
  if (s.express_us < 0.0) return 0;
  const double rem = elem_cost_us(*q->k, q->r.op) * (double)(q->r.count - q->next);
  return rem <= s.express_us ? 1 : 0;
}

// Scheduler threads: which = -1 serves every slot (one thread, no length
// rule); with the length rule one thread serves the regular slots
// (which = kRegularSlots) and every express slot has a thread of its own
// (which = the slot's index), so a short batch is staged and launched
// without waiting for the host work (staging, planning, inversions) of
// another batch.
constexpr int kRegularSlots = -2;

bool serves(const hg_server& s, const Slot& sl, int which) {
  if (which == -1) return true;
  if (which == kRegularSlots) return !sl.express;
  return (size_t)which < s.slots.size() && s.slots[(size_t)which].get() == &sl;
}

// Request class a scheduler thread admits (-1: any).
int thread_class(const hg_server& s, int which) {
  if (which == -1) return -1;
  if (which == kRegularSlots) return 0;
  const Slot& sl = *s.slots[(size_t)which];
  return sl.express_dec ? 2 : 1;
}

void scheduler(hg_server* sp, int which) {
  hg_server& s = *sp;
  cudaSetDevice(s.ctx->device);
  std::unique_lock<std::mutex> lk(s.mu);
  while (true) {
    // retire finished slots
    for (auto& slp : s.slots) {
      Slot& sl = *slp;
      if (!sl.busy || !serves(s, sl, which)) continue;
      if (cudaEventQuery(sl.ev) != cudaSuccess) continue;
      const uint32_t bits = *sl.err_host;
      for (Slice& sc : sl.slices) {
        Req* q = sc.q;
        if (bits & hg::kErrCtRange) q->status = HG_ERR_CT_RANGE;
        if (sc.task && sc.task->status == 1 && q->status == HG_OK) q->status = HG_ERR_NOT_INVERTIBLE;
        if (sc.task && sc.task->status == 2) q->status = HG_ERR_CT_RANGE;
        if (--q->outstanding == 0 && q->next == q->r.count) finish_req(s, q);
      }
      s.inflight -= sl.bytes;
      if (sl.traced) trace_retire(s, sl);
      sl.slices.clear();
      sl.busy = false;
    }
    if (s.stop && s.pending.empty()) {
      bool any = false;
      for (auto& slp : s.slots) any |= slp->busy && serves(s, *slp, which);
      if (!any) break;
    }
    // admit: every pending request gets a slice of at most slice_us of work
    // per micro-batch (processor sharing), until the batch reaches batch_us;
    // with HG_POLICY_SHORTEST the requests with the least estimated remaining
    // work are offered first, so short requests do not queue behind long ones
    if (s.policy == HG_POLICY_SHORTEST && s.pending.size() > 1)
      std::stable_sort(s.pending.begin(), s.pending.end(), [](const Req* a, const Req* b) {
        const double ra = elem_cost_us(*a->k, a->r.op) * (double)(a->r.count - a->next);
        const double rb = elem_cost_us(*b->k, b->r.op) * (double)(b->r.count - b->next);
        return ra < rb;
      });
    bool launched = false;
    auto klass = [&](const Req* q) -> int { return req_class(s, q); };
    // short requests belong to the express slots unless their backlog
    // exceeds what those take per batch
    double short_backlog = 0.0;
    if (s.express_us >= 0.0)
      for (const Req* q : s.pending)
        if (klass(q) != 0) short_backlog += elem_cost_us(*q->k, q->r.op) * (double)(q->r.count - q->next);
    // an express batch of the length rule holds at most express_len
    // elements (one longest short request, or several shorter ones; a batch
    // lasts as long as its slowest chain, so small batches keep the tail
    // short); of the cost rule, 4 x express_us of work
    const double express_batch_us =
        s.express_len > 0 ? 1e300 : 4.0 * std::max(s.express_us, 1.0);
    const size_t express_batch_elems = s.express_len > 0 ? s.express_len : s.cfg.max_batch_elems;
    for (auto& slp : s.slots) {
      Slot& sl = *slp;
      if (sl.busy || s.pending.empty() || !serves(s, sl, which)) continue;
      size_t elems = 0, bytes = 0;
      double cost = 0.0;
      const double batch_cap = sl.express ? express_batch_us : s.batch_us;
      const size_t elem_cap = sl.express ? express_batch_elems : s.cfg.max_batch_elems;
      const int slot_class = sl.express_dec ? 2 : sl.express ? 1 : 0;
      for (auto it = s.pending.begin(); it != s.pending.end();) {
        Req* q = *it;
        if (s.express_us >= 0.0) {
          const int kq = klass(q);
          const bool overflow = s.express_len == 0 && short_backlog > express_batch_us;
          if ((sl.express && kq != slot_class) || (!sl.express && kq != 0 && !overflow)) {
            ++it;
            continue;
          }
        }
        if (q->next == 0 && q->outstanding == 0 && !q->p0 && !q->p1 && (q->r.h0 || q->r.h1)) {
          try {
            q->p0 = q->r.h0 ? resident_ptr(s, q->r.h0, *q->k, q->r.count) : nullptr;
            q->p1 = q->r.h1 ? resident_ptr(s, q->r.h1, *q->k, q->r.count) : nullptr;
          } catch (const HgError& e) {
            q->status = e.code;
            q->next = q->r.count;
            it = s.pending.erase(it);
            if (q->outstanding == 0) finish_req(s, q);
            continue;
          }
        }
        const double cpe = elem_cost_us(*q->k, q->r.op);
        const size_t remain = q->r.count - q->next;
        size_t len = remain;
        if (q->r.op != kOpSum) {
          const size_t cap = (size_t)std::max(1.0, s.slice_us / std::max(cpe, 1e-9));
          len = std::min(len, std::max<size_t>(cap, 1));
          len = std::min(len, s.cfg.max_batch_elems);
        }
        const size_t need = slice_dev_bytes(*q->k, q->r, len);
        const bool first = sl.slices.empty();
        if (!first && (elems + len > elem_cap || bytes + need > sl.dev.cap ||
                       s.inflight + bytes + need > s.cfg.budget_bytes || cost >= batch_cap))
          break;
        if (first && s.inflight + need > s.cfg.budget_bytes && s.inflight > 0) break;  // wait for memory
        std::unique_ptr<InvTask> task;
        InvTask* tp = nullptr;
        if (q->r.op == hg::kBatchMul) {
          task = std::make_unique<InvTask>();
          tp = task.get();
          q->tasks.push_back(std::move(task));
        }
        if (q->next == 0) q->t_admit = std::chrono::steady_clock::now();
        sl.slices.push_back({q, q->next, len, need, tp});
        q->next += len;
        q->outstanding++;
        elems += len;
        bytes += need;
        cost += cpe * (double)len;
        if (q->next == q->r.count)
          it = s.pending.erase(it);
        else
          ++it;
      }
      if (sl.slices.empty()) continue;
      s.inflight += bytes;
      sl.bytes = bytes;
      sl.busy = true;
      ++s.batches;
      sl.traced = s.trace && sl.tev[0];
      if (sl.traced) {
        int mask = 0;
        for (const Slice& sc : sl.slices) mask |= 1 << sc.q->r.op;
        sl.tr[0] = slot_class;
        sl.tr[1] = (double)sl.slices.size();
        sl.tr[2] = (double)elems;
        sl.tr[3] = mask;
        sl.tr[4] = since(s.trace_t0);
      }
      lk.unlock();
      try {
        run_slot(s, sl);
        if (sl.traced) sl.tr[5] = std::chrono::duration<double>(sl.t_launched - s.trace_t0).count();
        for (Slice& sc : sl.slices)
          if (sc.start == 0) sc.q->t_launch = sl.t_launched;
      } catch (const HgError& e) {
        cudaStreamSynchronize(sl.st);
        lk.lock();
        for (Slice& sc : sl.slices) {
          Req* q = sc.q;
          q->status = e.code;
          if (--q->outstanding == 0 && q->next == q->r.count) finish_req(s, q);
        }
        s.inflight -= bytes;
        sl.slices.clear();
        sl.busy = false;
        sl.traced = false;
        lk.unlock();
      }
      if (!lk.owns_lock()) lk.lock();
      launched = true;
    }
    if (!launched) {
      bool any_busy = false;
      for (auto& slp : s.slots) any_busy |= slp->busy && serves(s, *slp, which);
      // poll busy slots quickly; sleep when idle until work of this thread's
      // slots arrives (with the length rule each thread waits for its class)
      const int cls = thread_class(s, which);
      auto mine = [&] {
        if (s.stop) return true;
        if (cls < 0 || s.express_len == 0) return !s.pending.empty();
        for (const Req* q : s.pending)
          if (req_class(s, q) == cls) return true;
        return false;
      };
      if (any_busy)
        s.cv_work.wait_for(lk, std::chrono::microseconds(20));
      else
        s.cv_work.wait_for(lk, std::chrono::milliseconds(5), mine);
    }
  }
}

}  // namespace
