// Compares ev::softfp::mul and ev::softfp::add (everett_gb300/csrc/
// ev_softfp.cuh) with the host's IEEE-754 multiplication and addition, bit
// for bit, over operand families that reach every rounding case: full random
// significands, short significands (exact results and exact ties),
// significands next to 1 and 2 (carries into the exponent), the edges of the
// fast-path exponent range, and for sums second operands that cancel the
// first (equal or nearly equal magnitudes of opposite sign) or sit at
// exponent gaps around the 53-bit significand and the 64-bit alignment.
//
// Usage: test_softfp COUNT_PER_FAMILY SEED
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "ev_softfp.cuh"

using ev::softfp::from_bits;
using ev::softfp::to_bits;

static uint64_t s_state;
static uint64_t next() {  // SplitMix64
  uint64_t z = (s_state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static double make(uint64_t sign, uint64_t exp, uint64_t frac) {
  return from_bits((sign << 63) | (exp << 52) | (frac & ((1ull << 52) - 1)));
}

static uint64_t rand_exp() { return 512 + next() % 1023; }  // [512, 1534]

static double family(int f) {
  const uint64_t s = next() & 1;
  switch (f) {
    case 0:  // any significand, any fast-path exponent
      return make(s, rand_exp(), next());
    case 1: {  // short significand: only the top k fraction bits random
      const int k = 1 + int(next() % 30);
      return make(s, rand_exp(), (next() >> (64 - k)) << (52 - k));
    }
    case 2: {  // 1 + small and 2 - small
      const uint64_t small = next() >> (12 + next() % 52);
      const uint64_t frac = (next() & 1) ? small : ((1ull << 52) - 1 - small);
      return make(s, rand_exp(), frac);
    }
    case 3: {  // exponent at the edges of the fast path
      const uint64_t edges[4] = {512, 513, 1533, 1534};
      return make(s, edges[next() & 3], (next() & 1) ? next() : ((1ull << 52) - 1));
    }
    default: {  // amplitude-like magnitudes: 2^-40 .. 2^0
      return make(s, 1023 - next() % 41, next());
    }
  }
}

int main(int argc, char** argv) {
  const long long count = argc > 1 ? atoll(argv[1]) : 1000000;
  s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  long long bad = 0, checked = 0;
  for (int fa = 0; fa < 5; ++fa) {
    for (int fb = 0; fb < 5; ++fb) {
      for (long long i = 0; i < count / 25 + 1; ++i) {
        const double a = family(fa), b = family(fb);
        const ev::softfp::Unpacked ua = ev::softfp::unpack(a), ub = ev::softfp::unpack(b);
        if (!ua.ok || !ub.ok) {
          std::printf("FAIL domain: %a %a reported outside the fast path\n", a, b);
          return 1;
        }
        volatile double want = a * b;
        const double got = ev::softfp::mul(ua, ub);
        ++checked;
        if (to_bits(got) != to_bits(want)) {
          if (++bad <= 10) std::printf("FAIL %a * %a: got %a want %a\n", a, b, got, (double)want);
        }
      }
    }
  }
  // sums: the same families for both operands, then second operands made
  // from the first (cancellation, exponent gaps at the alignment edges)
  long long bad_add = 0, checked_add = 0;
  for (int fa = 0; fa < 5; ++fa) {
    for (int fb = 0; fb < 8; ++fb) {
      for (long long i = 0; i < count / 40 + 1; ++i) {
        const double a = family(fa);
        double b;
        if (fb < 5) {
          b = family(fb);
        } else if (fb == 5) {  // opposite sign, low bits changed: cancellation
          const int k = int(next() % 53);  // fraction bits only
          const uint64_t flip = k ? (next() & ((1ull << k) - 1)) : 0;
          b = from_bits((to_bits(a) ^ flip) ^ (1ull << 63));
        } else {  // a gap of 50..66 exponents below a, either sign
          const uint64_t ua = to_bits(a);
          const uint64_t ea = (ua >> 52) & 0x7FF;
          const uint64_t gap = 50 + next() % 17;
          const uint64_t eb = ea - gap < 512 ? 512 : ea - gap;
          const uint64_t frac = fb == 6 ? next() : 0;  // fb 7: a power of two, exact ties
          b = make(next() & 1, eb, frac);
        }
        if (!ev::softfp::add_ok(a, b)) {
          std::printf("FAIL add domain: %a %a reported outside\n", a, b);
          return 1;
        }
        volatile double want = a + b;
        const double got = ev::softfp::add(a, b);
        const double got2 = ev::softfp::add(b, a);
        ++checked_add;
        if (to_bits(got) != to_bits(want) || to_bits(got2) != to_bits(want)) {
          if (++bad_add <= 10) std::printf("FAIL %a + %a: got %a / %a want %a\n", a, b, got, got2, (double)want);
        }
      }
    }
  }
  // exact cancellation is +0; the domain excludes zeros, subnormals, inf, NaN
  if (to_bits(ev::softfp::add(1.5, -1.5)) != to_bits(0.0)) {
    std::printf("FAIL 1.5 + -1.5 is not +0\n");
    return 1;
  }
  if (ev::softfp::add_ok(0.0, 1.0) || ev::softfp::add_ok(1.0, INFINITY) || ev::softfp::add_ok(NAN, 1.0)) {
    std::printf("FAIL add domain accepted a zero, an infinity or a NaN\n");
    return 1;
  }
  std::printf("%lld sums checked, %lld sum mismatches\n", checked_add, bad_add);
  bad += bad_add;
  // operands outside the domain are reported
  const double outside[] = {0.0, -0.0, 5e-324, 2.2250738585072014e-308, INFINITY, -INFINITY, NAN,
                            make(0, 511, 0), make(0, 1535, 0)};
  for (double x : outside) {
    if (ev::softfp::unpack(x).ok) {
      std::printf("FAIL domain: %a accepted\n", x);
      return 1;
    }
  }
  std::printf("%lld products checked, %lld mismatches\n", checked, bad);
  return bad == 0 ? 0 : 1;
}
