// Host check of rocflu_gb300/csrc/convert.cuh (the mixed update's
// float<->double conversions done with integer instructions) against C
// casts: f2d on every float bit pattern, d2f on every double exponent with
// rounding-boundary mantissas (ties to even and odd, one unit either side,
// the extremes) and on random bit patterns.  NaNs must map to NaNs.  Built
// and run by tests/test_convert_cpu.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#include "convert.cuh"

namespace {

long long fails = 0;

void checkD2f(double d) {
  const float got = rflu::d2f(d), want = (float)d;
  if (std::isnan(want)) {
    if (!std::isnan(got)) ++fails;
  } else if (rflu::cvt::bits(got) != rflu::cvt::bits(want)) {
    if (fails < 10) std::printf("d2f %016llx: %08x, cast %08x\n", (unsigned long long)rflu::cvt::bits(d),
                                rflu::cvt::bits(got), rflu::cvt::bits(want));
    ++fails;
  }
}

}  // namespace

int main() {
  // f2d: all 2^32 floats
  long long n = 0;
  for (unsigned long long u = 0; u <= 0xFFFFFFFFull; ++u) {
    const float f = rflu::cvt::fromBits((unsigned)u);
    const double got = rflu::f2d(f), want = (double)f;
    if (std::isnan(want)) {
      if (!std::isnan(got)) ++fails;
    } else if (rflu::cvt::bits(got) != rflu::cvt::bits(want)) {
      if (fails < 10) std::printf("f2d %08x: %016llx, cast %016llx\n", (unsigned)u, rflu::cvt::bits(got),
                                  rflu::cvt::bits(want));
      ++fails;
    }
    ++n;
  }
  // d2f: every exponent, both signs, mantissas around the rounding points
  // of a normal float (bit 28 the half unit) and of every denormal shift
  std::vector<unsigned long long> mans = {0ull, 1ull, 0xFFFFFFFFFFFFFull, 0x8000000000000ull};
  for (int sh = 0; sh < 53; ++sh) {
    const unsigned long long h = 1ull << sh;
    for (unsigned long long base : {0ull, h, 2 * h, 3 * h, h << 1 | h})
      for (long long dlt : {-1ll, 0ll, 1ll}) {
        const unsigned long long m = (base + (unsigned long long)dlt) & 0xFFFFFFFFFFFFFull;
        mans.push_back(m);
        mans.push_back(m | 0x8000000000000ull);
        mans.push_back(m ^ 0xFFFFFFFFFFFFFull);
      }
  }
  long long nd = 0;
  for (unsigned long long e = 0; e < 2048; ++e)
    for (unsigned long long s : {0ull, 1ull})
      for (unsigned long long m : mans) {
        checkD2f(rflu::cvt::fromBits(s << 63 | e << 52 | m));
        ++nd;
      }
  std::mt19937_64 rng(7);
  for (int k = 0; k < 50000000; ++k) {
    checkD2f(rflu::cvt::fromBits((unsigned long long)rng()));
    ++nd;
  }
  // doubles near the float range's ends, densely
  for (int k = 0; k < 4000000; ++k) {
    const unsigned long long e = 860 + rng() % 40 + (rng() & 1 ? 0 : 150);  // denormal and overflow edges
    checkD2f(rflu::cvt::fromBits((rng() & 1) << 63 | (e & 0x7FF) << 52 | (rng() & 0xFFFFFFFFFFFFFull)));
    ++nd;
  }
  std::printf("f2d %lld floats, d2f %lld doubles, %lld mismatches\n", n, nd, fails);
  if (fails) return 1;
  std::printf("ok\n");
  return 0;
}
