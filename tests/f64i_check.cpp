// Host check of the integer-pipe binary64 routines (diffrax_gb300/csrc/
// gbdx_f64i.cuh) against the host's IEEE-754 arithmetic: every result must be
// bit-identical.  Usage: f64i_check <n_random> <seed>; prints one line per
// routine with the number of cases and mismatches, exits 1 on any mismatch.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "gbdx_f64i.cuh"

using namespace gbdx;

static uint64_t g_state;
static uint64_t rnd() {  // splitmix64
  uint64_t z = (g_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double unif() { return double(rnd() >> 11) * 0x1.0p-53; }

static bool same_d(double x, double y) {
  if (isnan(x) || isnan(y)) return isnan(x) && isnan(y);
  return f64i_bits(x) == f64i_bits(y);
}
static bool same_f(float x, float y) {
  if (isnan(x) || isnan(y)) return isnan(x) && isnan(y);
  return f64i_fbits(x) == f64i_fbits(y);
}

// A double drawn from one of several families: raw bit patterns (every
// exponent, specials included), values near a given one (cancellation), and
// the times and step sizes of an integration.
static double draw(int fam, double near) {
  switch (fam) {
    case 0: return f64i_double(rnd());
    case 1: {  // exponents in the normal range, random significand and sign
      uint64_t u = rnd() & 0x800fffffffffffffull;
      uint64_t e = 1 + rnd() % 2046;
      return f64i_double(u | (e << 52));
    }
    case 2: {  // within a few ulp .. 2^-20 of `near`
      const int k = int(rnd() % 40);
      const double d = ldexp(unif() - 0.5, -k) * fabs(near);
      return (rnd() & 1) ? near + d : -(near + d);
    }
    case 3: return 100.0 * unif();                      // a time
    case 4: return exp2(-30.0 + 34.0 * unif());         // a step size
    case 5: return f64i_double(rnd() & 0x800fffffffffffffull);  // subnormal / zero
    default: {  // exponents at the edges of the normal range
      uint64_t e = (rnd() & 1) ? 1 + rnd() % 60 : 2046 - rnd() % 60;
      return f64i_double((rnd() & 0x800fffffffffffffull) | (e << 52));
    }
  }
}

static float draw_f(int fam) {
  switch (fam) {
    case 0: return f64i_float(uint32_t(rnd()));
    case 1: return float(0.2 + 9.8 * unif());  // a step-size factor
    case 2: return float(exp2(-20.0 + 40.0 * unif()));
    case 3: {  // few significant bits: products of such factors land on ties
      static const float m[] = {1.5f, 1.25f, 1.75f, 1.125f, 1.375f};
      const float v = ldexpf(m[rnd() % 5], int(rnd() % 21) - 10);
      return (rnd() & 1) ? v : -v;
    }
    default: {
      uint32_t e = (rnd() & 1) ? 1 + uint32_t(rnd() % 30) : 254 - uint32_t(rnd() % 30);
      return f64i_float((uint32_t(rnd()) & 0x807fffffu) | (e << 23));
    }
  }
}

int main(int argc, char **argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  g_state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
  long bad_add = 0, bad_mul = 0, bad_cvt = 0;
  // fixed edge cases
  const double ed[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, 0x1.0p-1022,
                       0x1.fffffffffffffp+1023, 0x1.0p-1074, 3.4028234663852886e38,
                       3.4028235677973366e38, 1.1754943508222875e-38, 1.1754942807573643e-38,
                       0x1.ffffffep+127, 0x1.000001p0, 0x1.0000018p0, 0x1.0000008p0};
  const int ne = sizeof ed / sizeof ed[0];
  for (int i = 0; i < ne; i++) {
    for (int j = 0; j < ne; j++) {
      bad_add += !same_d(f64i_add(ed[i], ed[j]), ed[i] + ed[j]);
      const float f = float(ed[j]);
      bad_mul += !same_d(f64i_mul_f32(ed[i], f), ed[i] * double(f));
    }
    bad_cvt += !same_f(f64i_to_f32(ed[i]), float(ed[i]));
    bad_cvt += !same_d(f64i_from_f32(float(ed[i])), double(float(ed[i])));
  }
  for (long it = 0; it < n; it++) {
    const int fa = int(rnd() % 7);
    const double a = draw(fa, 1.0);
    const double b = draw(int(rnd() % 7), a == a && a != 0 && !isinf(a) ? a : 1.0);
    if (!same_d(f64i_add(a, b), a + b)) {
      if (bad_add < 5) printf("add %a + %a: %a vs %a\n", a, b, f64i_add(a, b), a + b);
      bad_add++;
    }
    const float f = draw_f(int(rnd() % 5));
    if (!same_d(f64i_mul_f32(a, f), a * double(f))) {
      if (bad_mul < 5) printf("mul %a * %a: %a vs %a\n", a, double(f), f64i_mul_f32(a, f), a * double(f));
      bad_mul++;
    }
    // conversions: values near binary32 rounding boundaries and ties
    double c = a;
    if (rnd() & 1) {
      const float g = draw_f(int(rnd() % 4));
      const uint64_t t = f64i_bits(double(g)) + (rnd() & 1 ? 0x10000000ull : (rnd() & 0x3fffffffull));
      c = f64i_double(t);
    }
    const float w = draw_f(int(rnd() % 5));
    if (!same_d(f64i_from_f32(w), double(w))) {
      if (bad_cvt < 5) printf("widen %a: %a vs %a\n", double(w), f64i_from_f32(w), double(w));
      bad_cvt++;
    }
    if (!same_f(f64i_to_f32(c), float(c))) {
      if (bad_cvt < 5) printf("cvt %a: %a vs %a\n", c, double(f64i_to_f32(c)), double(float(c)));
      bad_cvt++;
    }
  }
  printf("add %ld cases, %ld mismatches\n", n + ne * ne, bad_add);
  printf("mul_f32 %ld cases, %ld mismatches\n", n + ne * ne, bad_mul);
  printf("to_f32 / from_f32 %ld cases, %ld mismatches\n", 2 * (n + ne), bad_cvt);
  return (bad_add || bad_mul || bad_cvt) ? 1 : 0;
}
