// Host side of HEU's wire format for ciphertext matrices
// (heu/library/numpy/matrix.h:221-310): the msgpack header written before the
// items, and the walk that finds every item in a received buffer.  Plain C++
// (no CUDA), so the walk is tested on the CPU alone.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace hg {
namespace wire {

struct FormatError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

inline void mp_uint(std::vector<uint8_t>& h, uint64_t v) {  // msgpack-c's smallest form of a non-negative int
  auto be = [&](int n) {
    for (int i = n - 1; i >= 0; --i) h.push_back((uint8_t)(v >> (8 * i)));
  };
  if (v < 128u) {
    h.push_back((uint8_t)v);
  } else if (v < 256u) {
    h.push_back(0xcc);
    be(1);
  } else if (v < 65536u) {
    h.push_back(0xcd);
    be(2);
  } else if (v < (1ull << 32)) {
    h.push_back(0xce);
    be(4);
  } else {
    h.push_back(0xcf);
    be(8);
  }
}

// fixarray(4), rows, cols, ndim, then the array header of the items
inline std::vector<uint8_t> wire_prefix(size_t rows, size_t cols, int ndim) {
  std::vector<uint8_t> h{0x94};
  mp_uint(h, rows);
  mp_uint(h, cols);
  mp_uint(h, (uint64_t)ndim);
  const uint64_t n = (uint64_t)rows * cols;
  if (n < 16u) {
    h.push_back((uint8_t)(0x90u | n));
  } else if (n < 65536u) {
    h.push_back(0xdc);
    h.push_back((uint8_t)(n >> 8));
    h.push_back((uint8_t)n);
  } else {
    h.push_back(0xdd);
    for (int i = 3; i >= 0; --i) h.push_back((uint8_t)(n >> (8 * i)));
  }
  return h;
}

struct WireReader {
  const uint8_t* p;
  size_t n, i = 0;
  [[noreturn]] void bad(const char* what) const {
    throw FormatError(std::string("Cannot parse: buffer format error (") + what + ")");
  }
  uint64_t be(int k) {
    if (n - i < (size_t)k) bad("truncated");
    uint64_t v = 0;
    for (int j = 0; j < k; ++j) v = (v << 8) | p[i++];
    return v;
  }
  uint8_t byte() { return (uint8_t)be(1); }
  int64_t integer() {
    const uint8_t t = byte();
    if (t < 0x80) return t;
    if (t >= 0xe0) return (int8_t)t;
    switch (t) {
      case 0xcc: return (int64_t)be(1);
      case 0xcd: return (int64_t)be(2);
      case 0xce: return (int64_t)be(4);
      case 0xcf: {
        const uint64_t v = be(8);
        if (v > (uint64_t)INT64_MAX) bad("integer");
        return (int64_t)v;
      }
      case 0xd0: return (int8_t)be(1);
      case 0xd1: return (int16_t)be(2);
      case 0xd2: return (int32_t)be(4);
      case 0xd3: return (int64_t)be(8);
      default: bad("integer");
    }
  }
  uint64_t array() {
    const uint8_t t = byte();
    if ((t & 0xf0) == 0x90) return t & 0x0f;
    if (t == 0xdc) return be(2);
    if (t == 0xdd) return be(4);
    bad("array");
  }
  // str or bin (msgpack-c's as<std::string_view> takes both)
  uint64_t bytes() {
    const uint8_t t = byte();
    if ((t & 0xe0) == 0xa0) return t & 0x1f;
    if (t == 0xd9 || t == 0xc4) return be(1);
    if (t == 0xda || t == 0xc5) return be(2);
    if (t == 0xdb || t == 0xc6) return be(4);
    bad("item");
  }
};

struct WireShape {
  size_t rows = 0, cols = 0, n = 0;
  int ndim = 0;
};

// The header checks of matrix.h:280-292 (a 4-element array, inner array
// size = rows * cols); leaves r at the first item.
inline WireShape wire_header(WireReader& r) {
  WireShape sh;
  if (r.array() != 4) r.bad("not a 4-element array");
  const int64_t rows = r.integer(), cols = r.integer(), ndim = r.integer();
  if (rows < 0 || cols < 0 || ndim < 0 || ndim > 2) r.bad("shape");
  const uint64_t n = r.array();
  if ((unsigned __int128)n != (unsigned __int128)(uint64_t)rows * (uint64_t)cols)
    r.bad("inner array size != rows * cols");
  if (n > r.n - r.i) r.bad("truncated");  // every item takes at least one byte
  sh.rows = (size_t)rows;
  sh.cols = (size_t)cols;
  sh.ndim = (int)ndim;
  sh.n = (size_t)n;
  return sh;
}

// The host walk over the items: offset and length of each.  Items of
// 256..65535 bytes (every ciphertext of a 1024..3072-bit key) have a str16
// header, read inline; other headers go through the general reader.
inline void wire_items_seq(WireReader& r, size_t n, uint64_t* offs, uint64_t* lens) {
  const uint8_t* p = r.p;
  const size_t len = r.n;
  size_t i = r.i;
  for (size_t k = 0; k < n; ++k) {
    uint64_t l;
    if (len - i >= 3 && p[i] == 0xda) {
      l = ((uint64_t)p[i + 1] << 8) | p[i + 2];
      i += 3;
    } else {
      r.i = i;
      l = r.bytes();
      i = r.i;
    }
    if (len - i < l) {
      r.i = i;
      r.bad("truncated item");
    }
    offs[k] = i;
    lens[k] = l;
    i += l;
  }
  r.i = i;
}

// Start of the next item at or after `from` if the bytes there look like one
// of this key's ciphertext items: a str16 header, fixarray(1), a bin8/bin16
// header whose length agrees with the str length, and the schema trailer
// (low byte = schema, seven zero bytes).  Returns len when none is found.
inline size_t wire_find_item(const uint8_t* p, size_t len, size_t from, size_t to, uint8_t schema) {
  for (size_t x = from; x < to && x + 12 <= len; ++x) {
    if (p[x] != 0xda || p[x + 3] != 0x91) continue;
    const uint64_t L = ((uint64_t)p[x + 1] << 8) | p[x + 2];
    uint64_t b, h;
    if (p[x + 4] == 0xc5) {
      b = ((uint64_t)p[x + 5] << 8) | p[x + 6];
      h = 3;
    } else if (p[x + 4] == 0xc4) {
      b = p[x + 5];
      h = 2;
    } else {
      continue;
    }
    if (L != 1 + h + b + 8 || x + 3 + L > len) continue;
    const uint8_t* tr = p + x + 3 + L - 8;
    bool ok = tr[0] == schema;
    for (int k = 1; k < 8 && ok; ++k) ok = tr[k] == 0;
    if (ok) return x;
  }
  return len;
}

// Walk from `at` over items while they start before `stop`: the count and
// the first item start at or after `stop` (or the end of the last item).
// With offs != nullptr the offsets and lengths are written as well.  Returns
// false on a malformed header or one that runs past the buffer.
inline bool wire_run(const uint8_t* p, size_t len, size_t at, size_t stop, size_t limit, size_t* count, size_t* end,
              uint64_t* offs, uint64_t* lens) {
  WireReader r{p, len};
  size_t i = at, k = 0;
  try {
    while (i < stop && k < limit) {
      uint64_t l;
      if (len - i >= 3 && p[i] == 0xda) {
        l = ((uint64_t)p[i + 1] << 8) | p[i + 2];
        i += 3;
      } else {
        r.i = i;
        l = r.bytes();
        i = r.i;
      }
      if (len - i < l) return false;
      if (offs) {
        offs[k] = i;
        lens[k] = l;
      }
      i += l;
      ++k;
    }
  } catch (...) {
    return false;
  }
  *count = k;
  *end = i;
  return true;
}

// The walk split over host threads.  The buffer is cut into segments; each
// thread finds the first item start in its segment (wire_find_item) and
// walks to the next segment.  The chain from the true first item is then
// followed segment by segment: where it lands exactly on a thread's start,
// that thread's items are the true ones; elsewhere (a false match, or an item
// of another shape) the segment is walked again from the true position.
// Every offset written comes from a walk that starts at a true item, so the
// result equals the sequential walk's.
// threads = 0: up to 16 host threads; walks of fewer than min_items items
// stay sequential.
inline void wire_items(WireReader& r, size_t n, uint64_t* offs, uint64_t* lens, uint8_t schema, unsigned threads = 0,
                       size_t min_items = (size_t)1 << 16) {
  const size_t body = r.n - r.i;
  const unsigned T = threads ? threads : std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (n < min_items || T == 1 || body < 2 * (size_t)T) {
    wire_items_seq(r, n, offs, lens);
    return;
  }
  std::vector<size_t> seg(T + 1), start(T), cnt(T), end(T);
  std::vector<char> valid(T);
  for (unsigned t = 0; t <= T; ++t) seg[t] = r.i + body * t / T;
  auto phase1 = [&](unsigned t) {
    start[t] = t == 0 ? r.i : wire_find_item(r.p, r.n, seg[t], seg[t + 1], schema);
    valid[t] = start[t] < seg[t + 1] &&
               wire_run(r.p, r.n, start[t], seg[t + 1], n, &cnt[t], &end[t], nullptr, nullptr);
  };
  {
    std::vector<std::thread> th;
    for (unsigned t = 1; t < T; ++t) th.emplace_back(phase1, t);
    phase1(0);
    for (auto& x : th) x.join();
  }
  // follow the true chain; bytes after the n-th item are not part of the
  // matrix (msgpack::unpack reads one object)
  std::vector<size_t> base(T), from(T);
  size_t pos = r.i, k = 0;
  for (unsigned t = 0; t < T; ++t) {
    base[t] = k;
    from[t] = pos;
    if (k == n || pos >= seg[t + 1]) {  // done, or an item longer than the segment
      cnt[t] = 0;
      continue;
    }
    if (!(valid[t] && start[t] == pos)) {
      if (!wire_run(r.p, r.n, pos, seg[t + 1], n - k, &cnt[t], &end[t], nullptr, nullptr)) {
        r.i = pos;
        wire_items_seq(r, n - k, offs + k, lens + k);  // raises the format error
        return;
      }
    }
    cnt[t] = std::min(cnt[t], n - k);
    k += cnt[t];
    pos = end[t];
  }
  if (k != n) {  // the buffer ended first
    r.i = pos;
    wire_items_seq(r, n - k, offs + k, lens + k);  // raises "truncated"
    return;
  }
  // write the offsets, every segment from its true first item
  auto phase3 = [&](unsigned t) {
    size_t c2, e2;
    if (cnt[t]) wire_run(r.p, r.n, from[t], seg[t + 1], cnt[t], &c2, &e2, offs + base[t], lens + base[t]);
  };
  {
    std::vector<std::thread> th;
    for (unsigned t = 1; t < T; ++t) th.emplace_back(phase3, t);
    phase3(0);
    for (auto& x : th) x.join();
  }
  r.i = pos;
}

}  // namespace wire
}  // namespace hg
