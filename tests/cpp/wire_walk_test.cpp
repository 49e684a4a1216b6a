// The host walk over HEU wire-format items (heu_gb300/csrc/wire_host.hpp):
// the threaded walk must give exactly the sequential walk's offsets on
// buffers with mixed item shapes, false item patterns planted inside
// payloads and trailing bytes, and both must reject truncated or miscounted
// buffers.  Built with g++ (no CUDA), under AddressSanitizer and
// UndefinedBehaviorSanitizer by tests/test_wire_walk.py.
#include <cstdio>
#include <random>
#include <vector>

#include "../../heu_gb300/csrc/wire_host.hpp"

using hg::wire::FormatError;
using hg::wire::WireReader;

namespace {

void put_str_header(std::vector<uint8_t>& b, size_t len) {
  if (len < 32) {
    b.push_back((uint8_t)(0xa0 | len));
  } else if (len < 256) {
    b.push_back(0xd9);
    b.push_back((uint8_t)len);
  } else {
    b.push_back(0xda);
    b.push_back((uint8_t)(len >> 8));
    b.push_back((uint8_t)len);
  }
}

// One item: fixarray(1), bin header, magnitude, schema trailer.
std::vector<uint8_t> item(std::mt19937_64& g, size_t mag, uint8_t schema, bool plant) {
  std::vector<uint8_t> it{0x91};
  if (mag < 256) {
    it.push_back(0xc4);
    it.push_back((uint8_t)mag);
  } else {
    it.push_back(0xc5);
    it.push_back((uint8_t)(mag >> 8));
    it.push_back((uint8_t)mag);
  }
  const size_t at = it.size();
  for (size_t i = 0; i < mag; ++i) it.push_back((uint8_t)g());
  if (plant && mag >= 300) {
    // a complete fake item inside the magnitude: header, lengths and trailer agree
    const size_t o = at + 5 + g() % 20, fb = 256 + g() % (mag - 300 < 40 ? 1 : 40);
    if (o + 15 + fb <= at + mag) {
      const size_t L = 1 + 3 + fb + 8;
      uint8_t* f = it.data() + o;
      f[0] = 0xda;
      f[1] = (uint8_t)(L >> 8);
      f[2] = (uint8_t)L;
      f[3] = 0x91;
      f[4] = 0xc5;
      f[5] = (uint8_t)(fb >> 8);
      f[6] = (uint8_t)fb;
      uint8_t* tr = f + 3 + L - 8;
      tr[0] = schema;
      for (int k = 1; k < 8; ++k) tr[k] = 0;
    }
  }
  it.push_back(schema);
  for (int k = 1; k < 8; ++k) it.push_back(0);
  return it;
}

std::vector<uint8_t> buffer(std::mt19937_64& g, size_t n, size_t declared, uint8_t schema, int trailing) {
  std::vector<uint8_t> b = hg::wire::wire_prefix(declared, 1, 1);
  for (size_t k = 0; k < n; ++k) {
    const unsigned kind = (unsigned)(g() % 100);
    const size_t mag = kind < 80 ? 512 : kind < 90 ? 256 + g() % 256 : kind < 97 ? g() % 256 : g() % 20;
    const auto it = item(g, mag, schema, g() % 4 == 0);
    put_str_header(b, it.size());
    b.insert(b.end(), it.begin(), it.end());
  }
  for (int t = 0; t < trailing; ++t) b.push_back((uint8_t)g());
  return b;
}

int failures = 0;

void check(bool ok, const char* what, size_t n, unsigned T) {
  if (!ok) {
    std::printf("FAIL %s n=%zu T=%u\n", what, n, T);
    ++failures;
  }
}

// Sequential and threaded walks of buf: both succeed with equal offsets, or
// both raise FormatError.
void compare(const std::vector<uint8_t>& buf, size_t n, unsigned T, bool expect_ok) {
  std::vector<uint64_t> o1(n), l1(n), o2(n), l2(n);
  bool ok1 = true, ok2 = true;
  try {
    WireReader r{buf.data(), buf.size()};
    const auto sh = hg::wire::wire_header(r);
    if (sh.n != n) throw FormatError("count");
    hg::wire::wire_items_seq(r, n, o1.data(), l1.data());
  } catch (const FormatError&) {
    ok1 = false;
  }
  try {
    WireReader r{buf.data(), buf.size()};
    const auto sh = hg::wire::wire_header(r);
    if (sh.n != n) throw FormatError("count");
    hg::wire::wire_items(r, n, o2.data(), l2.data(), 4, T, 1);
  } catch (const FormatError&) {
    ok2 = false;
  }
  check(ok1 == expect_ok, "sequential walk outcome", n, T);
  check(ok2 == expect_ok, "threaded walk outcome", n, T);
  if (ok1 && ok2) check(o1 == o2 && l1 == l2, "offsets differ", n, T);
}

}  // namespace

int main() {
  std::mt19937_64 g(12345);
  size_t cases = 0;
  for (size_t n : {1u, 2u, 3u, 17u, 100u, 1000u, 5000u}) {
    for (unsigned T : {2u, 3u, 4u, 7u, 16u}) {
      for (int trailing : {0, 5, 700}) {
        const auto buf = buffer(g, n, n, 4, trailing);
        compare(buf, n, T, true);
        ++cases;
      }
      // truncated inside an item
      auto buf = buffer(g, n, n, 4, 0);
      buf.resize(buf.size() - 1 - g() % 200);
      compare(buf, n, T, false);
      // the array claims one item more than there are
      const auto more = buffer(g, n, n + 1, 4, 0);
      compare(more, n + 1, T, false);
      cases += 2;
    }
  }
  // one long item spanning several segments
  {
    std::vector<uint8_t> b = hg::wire::wire_prefix(3, 1, 1);
    for (size_t mag : {512u, 60000u, 512u}) {
      const auto it = item(g, mag, 4, true);
      put_str_header(b, it.size());
      b.insert(b.end(), it.begin(), it.end());
    }
    for (unsigned T : {4u, 16u}) compare(b, 3, T, true);
    cases += 2;
  }
  if (failures) return 1;
  std::printf("%zu cases\nOK\n", cases);
  return 0;
}
