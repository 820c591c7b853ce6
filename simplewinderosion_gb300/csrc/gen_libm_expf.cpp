// Build-time generator: the arguments where this machine's C library expf
// differs from the correctly rounded exponential.
//
// The reference evaluates its boundary-layer factor with std::exp(float)
// (source/wind.hpp:50), i.e. the C library's expf. glibc's expf is accurate
// to about 0.502 ulp, so for roughly one argument in 10^4 it returns the
// neighbour of the correctly rounded value. The exact-semantics kernels
// compute the correctly rounded value and look the argument up in this list
// when the result lies near a rounding midpoint, which reproduces the C
// library bit for bit.
//
// Usage: gen_libm_expf <out.bin>
// Output: uint32 count, then count sorted uint32 argument bit patterns, then
// count int8 corrections (+1: next float up, -1: next float down).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

namespace {

float from_bits(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
uint32_t to_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

struct Hit {
  uint32_t x;
  int8_t d;
};

// Scans bit patterns [lo, hi); both finite exp results and their neighbours
// are compared as floats.
void scan(uint32_t lo, uint32_t hi, std::vector<Hit>* out) {
  for (uint32_t u = lo; u < hi; u++) {
    const float x = from_bits(u);
    const float a = std::exp(x);                  // C library expf
    const float b = (float)std::exp((double)x);   // correctly rounded
    if (a == b || (a != a && b != b)) continue;
    const int d = (a > b) ? 1 : -1;
    if (std::nextafter(b, d > 0 ? HUGE_VALF : -HUGE_VALF) != a) {
      std::fprintf(stderr, "expf differs from the rounded value by more than one ulp at %a\n", x);
      std::exit(2);
    }
    out->push_back(Hit{u, (int8_t)d});
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s out.bin\n", argv[0]);
    return 1;
  }
  // Arguments with a finite, non-zero result: [-104, 0] and [0, 88.8].
  const uint32_t neg_lo = 0x80000000u, neg_hi = to_bits(-104.0f) + 1;
  const uint32_t pos_lo = 0x00000000u, pos_hi = to_bits(88.8f) + 1;
  unsigned nt = std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > 64) nt = 64;
  std::vector<std::vector<Hit>> parts(2 * nt);
  std::vector<std::thread> th;
  auto split = [&](uint32_t lo, uint32_t hi, int base) {
    const uint64_t span = (uint64_t)hi - lo;
    for (unsigned t = 0; t < nt; t++) {
      const uint32_t a = (uint32_t)(lo + span * t / nt), b = (uint32_t)(lo + span * (t + 1) / nt);
      th.emplace_back(scan, a, b, &parts[base + t]);
    }
  };
  split(neg_lo, neg_hi, 0);
  split(pos_lo, pos_hi, nt);
  for (auto& t : th) t.join();
  std::vector<Hit> all;
  for (auto& p : parts) all.insert(all.end(), p.begin(), p.end());
  std::sort(all.begin(), all.end(), [](const Hit& a, const Hit& b) { return a.x < b.x; });
  FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 1;
  const uint32_t n = (uint32_t)all.size();
  std::fwrite(&n, 4, 1, f);
  for (const Hit& h : all) std::fwrite(&h.x, 4, 1, f);
  for (const Hit& h : all) std::fwrite(&h.d, 1, 1, f);
  std::fclose(f);
  std::printf("%u arguments where expf is not the correctly rounded value\n", n);
  return 0;
}
